// C entry point over the programs' ABN writer (opsec_gpu/programs/progs.cpp) for
// tests/test_abn_parity.py: one comment, then one abn_write under options set in order.
#include <cstdio>

#include "../opsec_gpu/programs/progs.h"

extern "C" int chk_abn_write(const char* path, const char* comment, int nkeys, const char** keys,
                             const char** vals, const void* data, size_t n, const char* fmt) {
    FILE* f = std::fopen(path, "wb");
    if (!f) return 1;
    std::fputs(comment, f);
    progs::Config opts;
    for (int i = 0; i < nkeys; i++) opts.set(keys[i], vals[i]);
    progs::abn_write(f, data, n, fmt, &opts);
    std::fclose(f);
    return 0;
}
