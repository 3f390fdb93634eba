// mockcounts -- counts per cell of a Gaussian-random-field mock on the GPU:
// the field of the configured P(k) at the cell centres, N_a ~ Poisson(Nbar_a
// max(0, 1 + b delta_a)).  Written as a countfile (ABN doubles, one per cell)
// for the dot program.  The reference draws mock galaxies instead
// (code/opsec/utils/gmock.cpp) and counts them per cell in dot
// (dot.cpp:123-129).
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "progs.h"

static const char* usage =
    "Usage: mockcounts [SWITCHES] [OPTIONS]\n"
    "Switches:\n"
    "  -h            Display this help\n"
    "  -c FILE       Read additional configuration options from FILE\n"
    "Configuration options:\n"
    "  cellfile=FILE    Read list of cells from FILE (required)\n"
    "  countfile=FILE   Write the counts to FILE (required)\n"
    "  RealModel.pkfile=FILE, model and survey options as for klt\n"
    "  mock.seed=NUM    Random seed (default 1)\n"
    "  mock.ngrid=NUM   Field mesh points per axis (even, default 64)\n"
    "  mock.bias=NUM    Linear bias b (default 1)\n";

int main(int argc, char** argv) {
    using namespace progs;
    Config cfg = init(argc, argv, usage);
    std::string miss = cfg.missing("cellfile,countfile");
    if (!miss.empty()) {
        std::fputs(usage, stderr);
        die("mockcounts", "missing configuration options " + miss);
    }
    std::string err;
    std::vector<opsec_cell> cells = read_cells(cfg.get("cellfile"), err);
    if (cells.empty()) die("mockcounts", err.empty() ? "no cells" : err);
    FILE* fout = std::fopen(cfg.get("countfile").c_str(), "wb");
    if (!fout) die("mockcounts", "could not open '" + cfg.get("countfile") + "' for writing");
    opsec_gpu* g = make_context("mockcounts", cfg);
    const unsigned long long seed = cfg.has("mock.seed") ? std::strtoull(cfg.get("mock.seed").c_str(), nullptr, 10) : 1;
    const int ngrid = cfg.has("mock.ngrid") ? cfg.get_int("mock.ngrid") : 64;
    const double bias = cfg.has("mock.bias") ? std::atof(cfg.get("mock.bias").c_str()) : 1.0;
    std::vector<double> counts(cells.size());
    if (opsec_gpu_mock_counts(g, (int)cells.size(), cells.data(), ngrid, seed, bias, counts.data(), nullptr) !=
        OPSEC_OK)
        die("mockcounts", opsec_gpu_last_error(g));
    Config opts;
    opts.set("Ncells", std::to_string(cells.size()));
    opts.set("mock.seed", std::to_string(seed));
    std::fprintf(fout, "# Mock counts per cell\n");
    abn_write(fout, counts.data(), counts.size(), "d", &opts);
    std::fclose(fout);
    opsec_gpu_destroy(g);
    return 0;
}
