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

// a configuration file read by the programs' reader, written back as an ABN header of
// n = 0 doubles (its options sorted, cfg_write's quoting)
extern "C" int chk_cfg_dump(const char* in, const char* out) {
    progs::Config c;
    if (!c.read_file(in)) return 1;
    FILE* f = std::fopen(out, "wb");
    if (!f) return 1;
    progs::abn_write_header(f, 0, "d", &c);
    std::fclose(f);
    return 0;
}
