// progs.h -- shared pieces of the drop-in programs: command line and
// configuration handling (opsec.c:19-56 opsec_init: -h, -c FILE, then
// key=value arguments; later keys override earlier ones), annotated binary
// (ABN) files (abn.c:150-330) and cell files (Cell.cpp:16-61).
#pragma once

#include <cstdio>
#include <map>
#include <string>
#include <vector>

#include "../../include/opsec_gpu.h"

namespace progs {

struct Config {
    std::map<std::string, std::string> kv;
    std::vector<std::string> order;  // insertion order, for writing
    bool has(const std::string& k) const { return kv.count(k) > 0; }
    const std::string& get(const std::string& k) const;
    int get_int(const std::string& k) const;
    void set(const std::string& k, const std::string& v);
    bool read_line(const std::string& line);  // false (and a message) for an invalid line
    bool read_file(const std::string& path);
    std::string missing(const std::string& comma_keys) const;  // "" when all present
    std::string text() const;                                   // key = value lines
};

// opsec_init: exits(0) on -h, exits(1) on a bad switch or unreadable -c file
Config init(int argc, char** argv, const char* usage);

[[noreturn]] void die(const char* prog, const std::string& msg);

// ABN: a text header of key = value lines and comments ending in
// "#!Begin data block: n = N, size = S, endian = E, format = F", then N*S bytes.
struct AbnHeader {
    size_t n = 0, size = 0;
    char endian = 'L';
    std::string format;
    Config opts;
};
bool abn_read_header(FILE* f, AbnHeader& h);
// reads the whole data block (byte-swapped to host order for simple formats)
bool abn_read(FILE* f, AbnHeader& h, std::vector<char>& data);
// the first block of a file whose data may go on in split pieces (name.00, name.01, ...)
bool abn_read_split(const std::string& path, AbnHeader& h, std::vector<char>& data, std::string& err);
void abn_write_header(FILE* f, size_t n, const char* fmt, const Config* opts);
void abn_write(FILE* f, const void* data, size_t n, const char* fmt, const Config* opts);
int abn_calcsize(const std::string& fmt);
char host_endian();

// ReadCells: cellfile with format "4i8d" and header Ncells
std::vector<opsec_cell> read_cells(const std::string& path, std::string& err);
// Modes file: header Nmodes, Ncells; n = Nmodes * Ncells doubles (klt.cpp:209-248)
bool read_modes(const std::string& path, int& nmodes, int& ncells, std::vector<double>& modes, std::string& err);
// A data file of doubles (evalfile, pixfile, countfile)
bool read_doubles(const std::string& path, std::vector<double>& v, Config* opts, std::string& err);

// library context from the program's configuration; exits on error
// the survey options and Ncells that basis writes on its cell file (basis.cpp:195-199)
Config survey_header(const Config& cfg, int ncells);

opsec_gpu* make_context(const char* prog, const Config& cfg);

}  // namespace progs
