// progs.cpp -- configuration, ABN and cell-file handling for the programs.
#include "progs.h"

#include <unistd.h>

#include <algorithm>
#include <cctype>
#include <cerrno>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <sstream>

namespace progs {

const std::string& Config::get(const std::string& k) const {
    static const std::string empty;
    auto it = kv.find(k);
    return it == kv.end() ? empty : it->second;
}

// cfg_get_int (cfg.c:430-440): "%i", so octal and hex too, trailing text ignored
int Config::get_int(const std::string& k) const { return (int)std::strtol(get(k).c_str(), nullptr, 0); }

void Config::set(const std::string& k, const std::string& v) {
    if (!kv.count(k)) order.push_back(k);
    kv[k] = v;
}

// cfg_read_line (cfg.c:238-295): blank and '#' lines ignored, key = value, whitespace (C
// isspace) trimmed, one pair of surrounding quotes stripped; false for a line that is not
// key = value (no '=', or nothing before it)
static bool cspace(char c) { return std::isspace((unsigned char)c) != 0; }

bool Config::read_line(const std::string& line) {
    size_t p = 0, end = line.size();
    while (p < end && cspace(line[p])) p++;
    if (p == end || line[p] == '#') return true;
    const size_t eq = line.find('=', p);
    if (eq == std::string::npos || eq == p) {
        std::fprintf(stderr, "cfg_read_line: '%s' is not a valid configuration line\n", line.c_str());
        return false;
    }
    size_t ke = eq;
    while (ke > p && cspace(line[ke - 1])) ke--;
    size_t vb = eq + 1;
    while (vb < end && cspace(line[vb])) vb++;
    size_t ve = end;
    while (ve > vb && cspace(line[ve - 1])) ve--;
    if (ve - vb >= 2 && ((line[vb] == '"' && line[ve - 1] == '"') || (line[vb] == '\'' && line[ve - 1] == '\''))) {
        vb++;
        ve--;
    }
    set(line.substr(p, ke - p), line.substr(vb, ve - vb));
    return true;
}

// cfg_read (cfg.c:200-214): lines until the first one that is not key = value, which ends
// the file's reading (what was read before it is kept)
bool Config::read_file(const std::string& path) {
    std::ifstream in(path);
    if (!in) return false;
    std::string line;
    while (std::getline(in, line))
        if (!read_line(line)) break;
    return true;
}

std::string Config::missing(const std::string& keys) const {
    std::string out;
    std::stringstream ss(keys);
    std::string k;
    while (std::getline(ss, k, ','))
        if (!has(k)) out += (out.empty() ? "" : ",") + k;
    return out;
}

std::string Config::text() const {
    std::string t;
    for (const auto& k : order) t += k + " = " + kv.at(k) + "\n";
    return t;
}

Config init(int argc, char** argv, const char* usage) {
    Config cfg;
    int opt;
    opterr = 0;
    while ((opt = getopt(argc, argv, "hc:")) != -1) {
        switch (opt) {
        case 'h':
            std::fputs(usage, stdout);
            std::exit(0);
        case 'c':
            if (!cfg.read_file(optarg)) {
                std::fprintf(stderr, "cfg_read_file: could not read file '%s'\n", optarg);
                std::exit(1);
            }
            break;
        default:
            std::fputs(usage, stdout);
            std::exit(1);
        }
    }
    for (int i = optind; i < argc; i++) cfg.read_line(argv[i]);
    return cfg;
}

void die(const char* prog, const std::string& msg) {
    std::fprintf(stderr, "%s: %s\n", prog, msg.c_str());
    std::exit(1);
}

char host_endian() {
    const uint16_t one = 1;
    return *reinterpret_cast<const unsigned char*>(&one) ? 'L' : 'B';
}

// abn_calcsize (abn.c:16-82): struct-module codes with repeat counts
int abn_calcsize(const std::string& fmt) {
    int size = 0;
    size_t i = 0;
    while (i < fmt.size()) {
        while (i < fmt.size() && std::isspace((unsigned char)fmt[i])) i++;
        if (i >= fmt.size()) break;
        int num = 0;
        bool have = false;
        while (i < fmt.size() && std::isdigit((unsigned char)fmt[i])) {
            num = num * 10 + (fmt[i] - '0');
            i++;
            have = true;
        }
        if (!have) num = 1;
        if (i >= fmt.size()) return -1;
        switch (fmt[i]) {
        case 'x': case 'c': case 'b': case 'B': size += num; break;
        case 'h': case 'H': size += num * 2; break;
        case 'i': case 'I': size += num * 4; break;
        case 'l': case 'L': size += num * (int)sizeof(long); break;
        case 'q': case 'Q': size += num * 8; break;
        case 'f': size += num * 4; break;
        case 'd': size += num * 8; break;
        default: return -1;
        }
        i++;
    }
    return size;
}

static std::vector<int> field_sizes(const std::string& fmt) {
    std::vector<int> f;
    size_t i = 0;
    while (i < fmt.size()) {
        while (i < fmt.size() && std::isspace((unsigned char)fmt[i])) i++;  // as abn_byte_swap (abn.c:113-115)
        if (i >= fmt.size()) break;
        int num = 0;
        bool have = false;
        while (i < fmt.size() && std::isdigit((unsigned char)fmt[i])) {
            num = num * 10 + (fmt[i] - '0');
            i++;
            have = true;
        }
        if (!have) num = 1;
        if (i >= fmt.size()) break;
        int len = abn_calcsize(std::string(1, fmt[i]));
        for (int k = 0; k < num; k++) f.push_back(len);
        i++;
    }
    return f;
}

bool abn_read_header(FILE* f, AbnHeader& h) {
    char line[4096];
    while (std::fgets(line, sizeof line, f)) {
        unsigned long long n = 0, size = 0;
        char endian = 0;
        char fmt[256] = {0};
        if (std::sscanf(line, "#!Begin data block: n = %llu, size = %llu, endian = %c, format = %255s", &n, &size,
                        &endian, fmt) == 4) {
            h.n = (size_t)n;
            h.size = (size_t)size;
            h.endian = endian;
            h.format = fmt;
            return true;
        }
        h.opts.read_line(line);
    }
    return false;
}

// abn_byte_swap (abn.c:96-183): every field of every record reversed when the block's byte
// order is not the host's
static void swap_block(const AbnHeader& h, std::vector<char>& data) {
    if (h.endian == host_endian()) return;
    std::vector<int> fs = field_sizes(h.format);
    char* p = data.data();
    for (size_t e = 0; e < h.n; e++)
        for (int len : fs) {
            for (int k = 0; k < len / 2; k++) std::swap(p[k], p[len - 1 - k]);
            p += len;
        }
}

bool abn_read(FILE* f, AbnHeader& h, std::vector<char>& data) {
    if (!abn_read_header(f, h)) return false;
    data.resize(h.n * h.size);
    if (h.n && std::fread(data.data(), h.size, h.n, f) != h.n) return false;
    swap_block(h, data);
    return true;
}

// SplitFile (SplitFile.cpp:120-175): the data of a block may go on in the pieces of a file cut
// by `split -d` -- when one piece ends, the next is the name with its last two characters
// replaced by the two-digit index of the piece (cells.abn.00, cells.abn.01, ...).  The header
// is read from the first piece.  A complete file opens no other piece.
bool abn_read_split(const std::string& path, AbnHeader& h, std::vector<char>& data, std::string& err) {
    FILE* f = std::fopen(path.c_str(), "rb");
    if (!f) {
        err = "could not open '" + path + "'";
        return false;
    }
    if (!abn_read_header(f, h)) {
        std::fclose(f);
        err = "error reading '" + path + "'";
        return false;
    }
    data.resize(h.n * h.size);
    std::string name = path;
    size_t got = 0;
    for (int index = 0; got < data.size() && f;) {
        const size_t n = std::fread(data.data() + got, 1, data.size() - got, f);
        got += n;
        if (got < data.size()) {
            if (!std::feof(f) || name.size() < 2) break;
            index++;
            const char suf[3] = {char('0' + (index / 10) % 10), char('0' + index % 10), 0};
            name.replace(name.size() - 2, 2, suf);
            f = std::freopen(name.c_str(), "rb", f);  // null (and closed) when there is no such piece
        }
    }
    if (f) std::fclose(f);
    if (got != data.size()) {
        err = "error reading '" + path + "': " + std::to_string(got) + " of " + std::to_string(data.size()) +
              " data bytes";
        return false;
    }
    swap_block(h, data);
    return true;
}

void abn_write_header(FILE* f, size_t n, const char* fmt, const Config* opts) {
    std::fprintf(f, "\n");
    // keys in strcmp order: the reference's Config is a list kept sorted (cfg.c:49-132), and
    // cfg_write walks it (cfg.c:297-312), so its headers list their keys sorted
    std::vector<std::string> keys;
    if (opts) keys = opts->order;
    std::sort(keys.begin(), keys.end());
    if (opts)
        for (const auto& k : keys) {
            const std::string& v = opts->kv.at(k);
            bool quote = !v.empty() && (std::isspace((unsigned char)v.front()) || std::isspace((unsigned char)v.back()));
            std::fprintf(f, quote ? "%s = \"%s\"\n" : "%s = %s\n", k.c_str(), v.c_str());
        }
    std::fprintf(f, "#!Begin data block: n = %zu, size = %i, endian = %c, format = %s\n", n, abn_calcsize(fmt),
                 host_endian(), fmt);
}

void abn_write(FILE* f, const void* data, size_t n, const char* fmt, const Config* opts) {
    abn_write_header(f, n, fmt, opts);
    std::fwrite(data, abn_calcsize(fmt), n, f);
}

std::vector<opsec_cell> read_cells(const std::string& path, std::string& err) {
    std::vector<opsec_cell> cells;
    AbnHeader h;
    std::vector<char> data;
    if (!abn_read_split(path, h, data, err)) return cells;
    if (h.size != sizeof(opsec_cell)) {  // Cell.cpp:52-55 checks the record size, not the format
        err = "cell size mismatch in '" + path + "' (format " + h.format + ")";
        return cells;
    }
    if ((size_t)h.opts.get_int("Ncells") != h.n) {  // ReadCells (Cell.cpp:47-51): the header's Ncells is required
        err = "consistency check fail for Ncells in '" + path + "'";
        return cells;
    }
    cells.resize(h.n);
    std::memcpy(cells.data(), data.data(), data.size());
    return cells;
}

bool read_modes(const std::string& path, int& nmodes, int& ncells, std::vector<double>& modes, std::string& err) {
    AbnHeader h;
    std::vector<char> data;
    const bool ok = abn_read_split(path, h, data, err);
    if (!ok && err.rfind("could not open", 0) == 0) return false;
    nmodes = h.opts.get_int("Nmodes");
    ncells = h.opts.get_int("Ncells");
    if (!ok || nmodes <= 0 || ncells <= 0 || h.n != (size_t)nmodes * ncells || h.size != sizeof(double)) {
        err = "error reading '" + path + "'";  // ReadModesHeader (sig.cpp:617-641)
        return false;
    }
    modes.resize(h.n);
    std::memcpy(modes.data(), data.data(), data.size());
    return true;
}

bool read_doubles(const std::string& path, std::vector<double>& v, Config* opts, std::string& err) {
    AbnHeader h;
    std::vector<char> data;
    const bool ok = abn_read_split(path, h, data, err);
    if (!ok && err.rfind("could not open", 0) == 0) return false;
    if (!ok || h.size != sizeof(double)) {
        err = "error reading '" + path + "'";
        return false;
    }
    v.resize(h.n);
    std::memcpy(v.data(), data.data(), data.size());
    if (opts) *opts = h.opts;
    return true;
}

// The options basis writes on its cell file (basis.cpp:195-199): the survey's
// GetConfigurationOptions (Survey.cpp:103-129, BoxSurvey.cpp:135-141,
// SphericalSurvey.cpp:172-178) -- keys without the "survey." prefix, doubles printed "%g"
// (cfg_set_double), MuMin read from MuMuin (Survey.cpp:39; MuMin without it) -- and Ncells.
Config survey_header(const Config& cfg, int ncells) {
    auto key = [&](const std::string& k) { return "survey." + k; };
    auto dbl = [&](const std::string& k) {
        char buf[64];
        std::snprintf(buf, sizeof buf, "%g", std::strtod(cfg.get(key(k)).c_str(), nullptr));
        return std::string(buf);
    };
    auto num = [&](const std::string& k) { return std::to_string((int)std::strtol(cfg.get(key(k)).c_str(), nullptr, 0)); };
    Config o;
    if (cfg.get("survey.type") == "BoxSurvey") {
        o.set("coordsys", "cartesian");
        for (const char* k : {"XMin", "XMax", "YMin", "YMax", "ZMin", "ZMax"}) o.set(k, dbl(k));
        for (const char* k : {"Nx", "Ny", "Nz"}) o.set(k, num(k));
        o.set("galfile", cfg.get("survey.galfile"));
        o.set("nbar", dbl("nbar"));
        o.set("L", dbl("L"));
    } else {
        o.set("coordsys", "spherical");
        o.set("RMin", dbl("RMin"));
        o.set("RMax", dbl("RMax"));
        o.set("MuMin", dbl(cfg.has("survey.MuMuin") ? "MuMuin" : "MuMin"));
        o.set("MuMax", dbl("MuMax"));
        o.set("PhiMin", dbl("PhiMin"));
        o.set("PhiMax", dbl("PhiMax"));
        for (const char* k : {"Nr", "Nmu", "Nphi"}) o.set(k, num(k));
        o.set("galfile", cfg.get("survey.galfile"));
        o.set("maskfile", cfg.get("survey.maskfile"));
        o.set("radial", cfg.get("survey.radial"));
    }
    o.set("Ncells", std::to_string(ncells));
    return o;
}

opsec_gpu* make_context(const char* prog, const Config& cfg) {
    opsec_gpu* g = nullptr;
    int rc = opsec_gpu_create(&g, cfg.text().c_str());
    if (rc != OPSEC_OK) die(prog, std::string("configuration: ") + opsec_gpu_last_error(g));
    return g;
}

}  // namespace progs
