// C entry point over the programs' ABN writer (opsec_gpu/programs/progs.cpp) for
// tests/test_abn_parity.py: one comment, then one abn_write under options set in order.
#include <algorithm>
#include <cstdio>
#include <cstring>
#include <vector>

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

// the first data block of an ABN file as the programs read it (host byte order); returns
// the byte count copied into out (at most cap), -1 when the file has no block
extern "C" long long chk_abn_read(const char* path, void* out, size_t cap) {
    FILE* f = std::fopen(path, "rb");
    if (!f) return -1;
    progs::AbnHeader h;
    std::vector<char> data;
    const bool ok = progs::abn_read(f, h, data);
    std::fclose(f);
    if (!ok) return -1;
    const size_t n = std::min(cap, data.size());
    std::memcpy(out, data.data(), n);
    return (long long)data.size();
}

// the first block through the programs' split-file reader: bytes copied, -1 on an error
extern "C" long long chk_abn_read_split(const char* path, void* out, size_t cap) {
    progs::AbnHeader h;
    std::vector<char> data;
    std::string err;
    if (!progs::abn_read_split(path, h, data, err)) return -1;
    std::memcpy(out, data.data(), std::min(cap, data.size()));
    return (long long)data.size();
}

// an integer option as the programs read it (cfg_get_int's "%i")
extern "C" int chk_get_int(const char* value) {
    progs::Config c;
    c.set("k", value);
    return c.get_int("k");
}

// the cells of a cell file as the programs accept them: their count, -1 when refused
extern "C" long long chk_read_cells(const char* path) {
    std::string err;
    std::vector<opsec_cell> cells = progs::read_cells(path, err);
    return err.empty() ? (long long)cells.size() : -1;
}

// the cell-file header the basis program writes, for a program configuration file
extern "C" int chk_survey_header(const char* cfgpath, int ncells, const char* outpath) {
    progs::Config c;
    if (!c.read_file(cfgpath)) return 1;
    const progs::Config opts = progs::survey_header(c, ncells);
    FILE* f = std::fopen(outpath, "wb");
    if (!f) return 1;
    progs::abn_write_header(f, (size_t)ncells, "4i8d", &opts);
    std::fclose(f);
    return 0;
}
