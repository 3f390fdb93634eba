// comma -- derivative matrices C_p = B^T S_p B of every band in the KL basis on
// the GPU; same options and covfile as the reference program
// (code/opsec/src/comma-scalapack.cpp:100-280).
#include <cstdio>
#include <vector>

#include "progs.h"

static const char* usage =
    "Usage: comma [SWITCHES] [OPTIONS]\n"
    "Switches:\n"
    "  -h             Display this help\n"
    "  -c FILE        Read additional configuration options from FILE\n"
    "Configuration options:\n"
    "  cellfile=FILE  Read list of cells from FILE (required)\n"
    "  modefile=FILE  Read KL modes from FILE (required)\n"
    "  covfile=FILE   Write covariance matrices to FILE (required)\n"
    "  Nmodes=NUM     Number of KL modes (required)\n"
    "  model=NAME     Use specified model (required)\n";

int main(int argc, char** argv) {
    using namespace progs;
    Config cfg = init(argc, argv, usage);
    std::string miss = cfg.missing("cellfile,modefile,covfile,Nmodes");
    if (!miss.empty()) {
        std::fputs(usage, stderr);
        die("comma", "missing configuration options " + miss);
    }
    std::string err;
    std::vector<opsec_cell> cells = read_cells(cfg.get("cellfile"), err);
    if (cells.empty()) die("comma", err.empty() ? "no cells" : err);
    const int Ncells = (int)cells.size(), Nmodes = cfg.get_int("Nmodes");
    int nm = 0, nc = 0;
    std::vector<double> modes;
    if (!read_modes(cfg.get("modefile"), nm, nc, modes, err)) die("comma", err);
    if (nc != Ncells || nm < Nmodes) die("comma", "inconsistent modes file");
    modes.resize((size_t)Nmodes * Ncells);  // the first Nmodes modes (ReadModes, comma-scalapack.cpp:84-94)
    FILE* fout = std::fopen(cfg.get("covfile").c_str(), "wb");
    if (!fout) die("comma", "could not open '" + cfg.get("covfile") + "' for writing");
    opsec_gpu* g = make_context("comma", cfg);
    int Nparams = 0;
    opsec_gpu_num_params(g, &Nparams);
    const size_t K = (size_t)Nmodes * (Nmodes + 1) / 2;
    std::vector<double> cov(K * Nparams);
    if (opsec_gpu_comma(g, Ncells, cells.data(), Nmodes, modes.data(), cov.data()) != OPSEC_OK)
        die("comma", opsec_gpu_last_error(g));
    // header as comma-scalapack.cpp:210-224
    std::fprintf(fout, "# Derivatives of the covariance matrix in KL basis, C_{ij,m}.\n");
    std::fprintf(fout, "# Binary data consists of %d consecutive symmetric %dx%d matrices\n", Nparams, Nmodes, Nmodes);
    std::fprintf(fout, "# in packed storage.  Each matrix consists of %zu elements.\n", K);
    Config opts;
    opts.set("Nmodes", std::to_string(Nmodes));
    opts.set("Nparams", std::to_string(Nparams));
    opts.set("packed", "1");
    abn_write(fout, cov.data(), cov.size(), "d", &opts);
    std::fclose(fout);
    opsec_gpu_destroy(g);
    return 0;
}
