// klt -- KL eigenmodes of the signal matrix on the GPU; same options and
// output files as the reference program (code/opsec/src/klt.cpp:100-267).
#include <cstdio>
#include <vector>

#include "progs.h"

static const char* usage =
    "Usage: klt [SWITCHES] [OPTIONS]\n"
    "Switches:\n"
    "  -h             Display this help\n"
    "  -c FILE        Read additional configuration options from FILE\n"
    "Configuration options:\n"
    "  cellfile=FILE  Read list of cells from FILE (required)\n"
    "  Nmodes=NUM     Compute NUM mode functions of greatest S/N (required)\n"
    "  modefile=FILE  Write mode function coefficients to FILE (required)\n"
    "  evalfile=FILE  Write S/N eigenvalues to FILE (required)\n"
    "  model=NAME     Use specified model (required)\n"
    "  solver=NAME    parpack or anasazi: accepted for the reference's configurations; the\n"
    "                 engine picks its eigensolver (klt.solver = auto|dense|chfsi)\n";

int main(int argc, char** argv) {
    using namespace progs;
    Config cfg = init(argc, argv, usage);
    std::string miss = cfg.missing("cellfile,Nmodes,modefile,evalfile");
    if (!miss.empty()) {
        std::fputs(usage, stderr);
        die("klt", "missing configuration options " + miss);
    }
    // klt.cpp:167-193 selects PARPACK or Anasazi by `solver`: both find the top Nmodes
    // eigenpairs, which the engine does by the azimuthal reduction, a dense solve or its own
    // iterative solver
    if (cfg.has("solver") && cfg.get("solver") != "parpack" && cfg.get("solver") != "anasazi")
        die("klt", "unrecognized solver: " + cfg.get("solver"));
    std::string err;
    std::vector<opsec_cell> cells = read_cells(cfg.get("cellfile"), err);
    if (cells.empty()) die("klt", err.empty() ? "no cells" : err);
    const int Ncells = (int)cells.size(), Nmodes = cfg.get_int("Nmodes");
    if (Nmodes > Ncells) die("klt", "requesting more modes than cells");
    FILE* fmode = std::fopen(cfg.get("modefile").c_str(), "wb");
    FILE* feval = std::fopen(cfg.get("evalfile").c_str(), "wb");
    if (!fmode || !feval) die("klt", "could not open output files");
    opsec_gpu* g = make_context("klt", cfg);
    std::vector<double> evals(Nmodes), modes((size_t)Nmodes * Ncells);
    int nconv = 0;
    if (opsec_gpu_klt(g, Ncells, cells.data(), Nmodes, evals.data(), modes.data(), &nconv) != OPSEC_OK)
        die("klt", opsec_gpu_last_error(g));
    double st[10];
    if (opsec_gpu_eig_stats(g, st) == OPSEC_OK) {  // in place of ParpackSolver.cpp:140-190's report
        static const char* names[] = {"dense", "azimuthal blocks", "subspace iteration"};
        std::fprintf(stderr, "klt: %d modes by the %s eigensolver", nconv, names[(int)st[0] % 3]);
        if ((int)st[0] == 2)
            std::fprintf(stderr, ", %d iterations, largest relative residual %.2e", (int)st[1], st[7]);
        std::fprintf(stderr, "\n");
    }
    // headers as klt.cpp:209-225
    Config opts;
    opts.set("cellfile", cfg.get("cellfile"));
    opts.set("Ncells", std::to_string(Ncells));
    opts.set("Nmodes", std::to_string(Nmodes));
    opts.set("nconv", std::to_string(nconv));
    std::fprintf(feval, "# Signal matrix eigenvalues\n");
    abn_write(feval, evals.data(), nconv, "d", &opts);
    std::fprintf(fmode, "# Signal matrix eigenmodes\n");
    std::fprintf(fmode, "# Each mode is stored consecutively, as below:\n");
    std::fprintf(fmode, "#   v_1,1   v_1,2   ... v_1,n\n");
    std::fprintf(fmode, "#   ...\n");
    std::fprintf(fmode, "#   v_m,1   v_m,2   ... v_m,n\n");
    abn_write(fmode, modes.data(), (size_t)nconv * Ncells, "d", &opts);
    std::fclose(feval);
    std::fclose(fmode);
    opsec_gpu_destroy(g);
    return 0;
}
