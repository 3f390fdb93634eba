// dot -- pixel values y = B^T (N - Nbar)/sqrt(Nbar) on the GPU from weighted
// counts per cell (countfile: ABN doubles, one per cell); same pixfile as the
// reference program (code/opsec/src/dot.cpp:131-160).
#include <cstdio>
#include <vector>

#include "progs.h"

static const char* usage =
    "Usage: dot [SWITCHES] [OPTIONS]\n"
    "Switches:\n"
    "  -h            Display this help\n"
    "  -c FILE       Read additional configuration options from FILE\n"
    "Configuration options:\n"
    "  countfile=FILE Read (weighted) galaxy counts per cell from FILE (required)\n"
    "  pixfile=FILE  Write pixel values to FILE (required)\n"
    "  cellfile=FILE Read list of cells from FILE (required)\n"
    "  modefile=FILE Read KL mode coefficients from FILE (required)\n"
    "  Nmodes=NUM    Number of KL modes\n";

int main(int argc, char** argv) {
    using namespace progs;
    Config cfg = init(argc, argv, usage);
    std::string miss = cfg.missing("countfile,cellfile,modefile,pixfile,Nmodes");
    if (!miss.empty()) {
        std::fputs(usage, stderr);
        die("dot", "missing configuration options " + miss);
    }
    std::string err;
    std::vector<opsec_cell> cells = read_cells(cfg.get("cellfile"), err);
    if (cells.empty()) die("dot", err.empty() ? "no cells" : err);
    const int Ncells = (int)cells.size(), Nmodes = cfg.get_int("Nmodes");
    int nm = 0, nc = 0;
    std::vector<double> modes, counts;
    if (!read_modes(cfg.get("modefile"), nm, nc, modes, err)) die("dot", err);
    if (nm != Nmodes || nc != Ncells) die("dot", "inconsistent modes file");
    if (!read_doubles(cfg.get("countfile"), counts, nullptr, err)) die("dot", err);
    if ((int)counts.size() != Ncells) die("dot", "countfile must hold one value per cell");
    FILE* fpix = std::fopen(cfg.get("pixfile").c_str(), "wb");
    if (!fpix) die("dot", "could not open '" + cfg.get("pixfile") + "' for writing");
    opsec_gpu* g = make_context("dot", cfg);
    std::vector<double> y(Nmodes);
    if (opsec_gpu_dot(g, Ncells, cells.data(), counts.data(), Nmodes, modes.data(), y.data()) != OPSEC_OK)
        die("dot", opsec_gpu_last_error(g));
    std::fprintf(fpix, "# Pixel values\n");
    abn_write(fpix, y.data(), Nmodes, "d", nullptr);
    std::fclose(fpix);
    opsec_gpu_destroy(g);
    return 0;
}
