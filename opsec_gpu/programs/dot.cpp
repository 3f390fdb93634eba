// dot -- pixel values y = B^T (N - Nbar)/sqrt(Nbar) on the GPU; same pixfile as
// the reference program (code/opsec/src/dot.cpp:131-160).  The weighted counts
// per cell come from the survey's galaxy file (survey.galfile, ABN "4f", binned
// on the GPU as dot.cpp:95-130 does) or, given countfile, from a file of counts
// (ABN doubles, one per cell: the mockcounts program writes one).
#include <cstdio>
#include <vector>

#include "progs.h"

static const char* usage =
    "Usage: dot [SWITCHES] [OPTIONS]\n"
    "Switches:\n"
    "  -h            Display this help\n"
    "  -c FILE       Read additional configuration options from FILE\n"
    "Configuration options:\n"
    "  survey.galfile=FILE Read galaxies (ABN format 4f: x1 x2 x3 w) from FILE\n"
    "  countfile=FILE Without a galfile, read (weighted) counts per cell from FILE\n"
    "  pixfile=FILE  Write pixel values to FILE (required)\n"
    "  cellfile=FILE Read list of cells from FILE (required)\n"
    "  modefile=FILE Read KL mode coefficients from FILE (required)\n"
    "  Nmodes=NUM    Number of KL modes\n";

int main(int argc, char** argv) {
    using namespace progs;
    Config cfg = init(argc, argv, usage);
    std::string miss = cfg.missing("cellfile,modefile,pixfile,Nmodes");
    const bool galfile = cfg.has("survey.galfile") && cfg.get("survey.galfile") != "none";
    if (miss.empty() && !galfile && !cfg.has("countfile")) miss = "survey.galfile or countfile";
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
    opsec_gpu* g = make_context("dot", cfg);
    if (!galfile) {
        if (!read_doubles(cfg.get("countfile"), counts, nullptr, err)) die("dot", err);
        if ((int)counts.size() != Ncells) die("dot", "countfile must hold one value per cell");
    } else {
        // BoxSurvey.cpp:105-133 / SphericalSurvey.cpp:146-170: one ABN block of "4f" galaxies
        FILE* fg = std::fopen(cfg.get("survey.galfile").c_str(), "rb");
        if (!fg) die("dot", "could not open '" + cfg.get("survey.galfile") + "'");
        AbnHeader h;
        std::vector<char> data;
        const bool ok = abn_read(fg, h, data);
        std::fclose(fg);
        if (!ok || h.format != "4f" || h.size != 4 * sizeof(float) || h.n == 0)
            die("dot", "error reading galaxies from '" + cfg.get("survey.galfile") + "'");
        counts.resize(Ncells);
        double outside = 0;
        if (opsec_gpu_count_galaxies(g, Ncells, cells.data(), (long long)h.n, reinterpret_cast<const float*>(data.data()),
                                     counts.data(), &outside) != OPSEC_OK)
            die("dot", opsec_gpu_last_error(g));
        std::fprintf(stderr, "dot: %zu galaxies, weight %g outside the cells\n", h.n, outside);
    }
    FILE* fpix = std::fopen(cfg.get("pixfile").c_str(), "wb");
    if (!fpix) die("dot", "could not open '" + cfg.get("pixfile") + "' for writing");
    std::vector<double> y(Nmodes);
    if (opsec_gpu_dot(g, Ncells, cells.data(), counts.data(), Nmodes, modes.data(), y.data()) != OPSEC_OK)
        die("dot", opsec_gpu_last_error(g));
    std::fprintf(fpix, "# Pixel values\n");
    abn_write(fpix, y.data(), Nmodes, "d", nullptr);
    std::fclose(fpix);
    opsec_gpu_destroy(g);
    return 0;
}
