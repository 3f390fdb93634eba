// basis -- the cell list of a survey on the GPU: every grid cell with positive
// expected count Nbar, its bounds and effective volume, written as the
// reference program writes it (code/opsec/src/basis.cpp:145-201: cellfile in
// ABN format "4i8d" with the survey options and Ncells in its header).
//
// Selection: Cartesian grids the constant survey.nbar; spherical grids the
// radial file survey.radial (two columns r, nbar; linear between points) times
// an optional HEALPix completeness map.  The reference reads the map from a
// FITS file (survey.maskfile, through cfitsio); here the map is a file of
// 12 nside^2 little-endian float32 values, survey.mask.raw, with
// survey.mask.nside and survey.mask.ordering = RING | NESTED.
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <sstream>
#include <vector>

#include "progs.h"

static const char* usage =
    "Usage: basis [SWITCHES] [OPTIONS]\n"
    "Switches:\n"
    "  -h            Display this help\n"
    "  -c FILE       Read additional configuration options from FILE\n"
    "Configuration options:\n"
    "  cellfile=FILE          Write list of cells to FILE (required)\n"
    "  coordsys=TYPE          cartesian or spherical (required)\n"
    "  survey.*               Survey geometry (as klt), and its selection:\n"
    "  survey.nbar=NUM        Cartesian: constant number density\n"
    "  survey.radial=FILE     Spherical: radial selection, two columns r nbar\n"
    "  survey.mask.raw=FILE   Spherical, optional: HEALPix map, 12 nside^2 float32\n"
    "  survey.mask.nside=NUM  its nside\n"
    "  survey.mask.ordering=RING|NESTED\n"
    "  basis.quirk3=0|1       1: the reference's spherical Nbar (3x the expected count)\n";

int main(int argc, char** argv) {
    using namespace progs;
    Config cfg = init(argc, argv, usage);
    std::string miss = cfg.missing("cellfile,coordsys");
    if (!miss.empty()) {
        std::fputs(usage, stderr);
        die("basis", "missing configuration options " + miss);
    }
    // open the output first, as the reference does (basis.cpp:152-162)
    FILE* fcells = std::fopen(cfg.get("cellfile").c_str(), "wb");
    if (!fcells) die("basis", "cannot write to '" + cfg.get("cellfile") + "'");
    opsec_gpu* g = make_context("basis", cfg);
    if (cfg.get("coordsys") == "spherical") {
        if (!cfg.has("survey.radial")) die("basis", "missing configuration option survey.radial");
        std::ifstream in(cfg.get("survey.radial"));
        if (!in) die("basis", "cannot read '" + cfg.get("survey.radial") + "'");
        std::vector<double> r, n;
        std::string line;
        while (std::getline(in, line)) {
            if (line.empty() || line[0] == '#') continue;
            std::istringstream ss(line);
            double a, b;
            if (ss >> a >> b) {
                r.push_back(a);
                n.push_back(b);
            }
        }
        if (opsec_gpu_set_radial(g, (int)r.size(), r.data(), n.data()) != OPSEC_OK) die("basis", opsec_gpu_last_error(g));
        if (cfg.has("survey.mask.raw")) {
            const long long nside = std::atoll(cfg.get("survey.mask.nside").c_str());
            const std::string ord = cfg.has("survey.mask.ordering") ? cfg.get("survey.mask.ordering") : "RING";
            if (ord != "RING" && ord != "NESTED") die("basis", "survey.mask.ordering must be RING or NESTED");
            const size_t npix = (size_t)12 * nside * nside;
            std::vector<float> map(npix);
            FILE* fm = std::fopen(cfg.get("survey.mask.raw").c_str(), "rb");
            if (!fm || nside <= 0 || std::fread(map.data(), sizeof(float), npix, fm) != npix)
                die("basis", "cannot read " + std::to_string(npix) + " map values from '" + cfg.get("survey.mask.raw") + "'");
            std::fclose(fm);
            if (host_endian() == 'B')
                for (float& v : map) {
                    unsigned char* p = reinterpret_cast<unsigned char*>(&v);
                    std::swap(p[0], p[3]);
                    std::swap(p[1], p[2]);
                }
            if (opsec_gpu_set_mask(g, nside, ord == "NESTED", map.data()) != OPSEC_OK) die("basis", opsec_gpu_last_error(g));
        } else if (cfg.has("survey.maskfile") && cfg.get("survey.maskfile") != "none") {
            die("basis", "FITS maps (survey.maskfile) need cfitsio, which this build lacks: give the map as "
                         "survey.mask.raw with survey.mask.nside and survey.mask.ordering");
        }
    }
    int n = 0;
    if (opsec_gpu_basis(g, 0, nullptr, &n) != OPSEC_OK) die("basis", opsec_gpu_last_error(g));
    std::vector<opsec_cell> cells(n);
    if (n && opsec_gpu_basis(g, n, cells.data(), &n) != OPSEC_OK) die("basis", opsec_gpu_last_error(g));
    std::fprintf(stderr, "basis: got %d non-empty cells\n", n);
    const Config opts = survey_header(cfg, n);  // the reference's header, byte for byte
    abn_write(fcells, cells.data(), (size_t)n, "4i8d", &opts);
    std::fclose(fcells);
    opsec_gpu_destroy(g);
    return 0;
}
