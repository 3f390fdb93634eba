// estimate -- Fisher matrix, quadratic estimates and band powers on the GPU;
// same options and estfile as the reference program at one rank
// (code/opsec/src/estimate-mpi.cpp:340-660).
#include <cstdio>
#include <cstring>
#include <cmath>
#include <ctime>
#include <vector>

#include "progs.h"

static const char* usage =
    "Usage: estimate [SWITCHES] [OPTIONS]\n"
    "Switches:\n"
    "  -h             Display this help\n"
    "  -c FILE        Read additional configuration options from FILE\n"
    "Configuration options:\n"
    "  estfile=FILE   Write parameter estimates to FILE (required)\n"
    "  evalfile=FILE  Read S/N eigenvalues from FILE (required)\n"
    "  covfile=FILE   Read covariance matrix derivatives from FILE (required)\n"
    "  pixfile=FILE   Read pixel values from FILE (required)\n"
    "  mixing=MODE    Mixing matrix choice: inverse (default), inverse-sqrt, or identity\n";

int main(int argc, char** argv) {
    using namespace progs;
    Config cfg = init(argc, argv, usage);
    std::string miss = cfg.missing("estfile,evalfile,covfile,pixfile,Nmodes");
    if (!miss.empty()) {
        std::fputs(usage, stderr);
        die("estimate", "missing configuration options " + miss);
    }
    const int Nmodes = cfg.get_int("Nmodes");
    FILE* fest = std::fopen(cfg.get("estfile").c_str(), "wb");
    if (!fest) die("estimate", "cannot write to '" + cfg.get("estfile") + "'");
    int mixing = OPSEC_MIXING_INVERSE;
    if (cfg.has("mixing")) {
        // cfg_get_enum (cfg.c:486-501): the first tag the value is a prefix of; no match is inverse
        const std::string& m = cfg.get("mixing");
        const char* tags[] = {"inverse", "inverse-sqrt", "identity"};
        const int modes[] = {OPSEC_MIXING_INVERSE, OPSEC_MIXING_INVERSE_SQRT, OPSEC_MIXING_IDENTITY};
        for (int t = 0; t < 3; t++)
            if (m.size() <= std::strlen(tags[t]) && std::string(tags[t]).compare(0, m.size(), m) == 0) {
                mixing = modes[t];
                break;
            }
    }
    std::string err;
    std::vector<double> evals, cov, y;
    Config covopts;
    if (!read_doubles(cfg.get("evalfile"), evals, nullptr, err)) die("estimate", err);
    if ((int)evals.size() < Nmodes) die("estimate", "inconsistent evals length");
    evals.resize(Nmodes);
    if (!read_doubles(cfg.get("covfile"), cov, &covopts, err)) die("estimate", err);
    if (!read_doubles(cfg.get("pixfile"), y, nullptr, err)) die("estimate", err);
    if ((int)y.size() != Nmodes) die("estimate", "error reading pixel values");
    opsec_gpu* g = make_context("estimate", cfg);
    int Nparams = 0;
    opsec_gpu_num_params(g, &Nparams);
    const size_t K = (size_t)Nmodes * (Nmodes + 1) / 2;
    if (covopts.get_int("Nparams") != Nparams || covopts.get_int("Nmodes") != Nmodes)
        die("estimate", "inconsistent covfile");
    if (covopts.has("packed") && covopts.get_int("packed") == 0) {
        // full storage: keep the upper triangle column by column (ReadCovMatrix, estimate-mpi.cpp:226-260)
        std::vector<double> packed(K * Nparams);
        for (int p = 0; p < Nparams; p++)
            for (int j = 0; j < Nmodes; j++)
                for (int i = 0; i <= j; i++)
                    packed[p * K + (size_t)j * (j + 1) / 2 + i] = cov[(size_t)p * Nmodes * Nmodes + (size_t)j * Nmodes + i];
        cov.swap(packed);
    }
    if (cov.size() < K * Nparams) die("estimate", "covfile too short");
    const size_t n2 = (size_t)Nparams * Nparams;
    std::vector<double> phat(Nparams), pcov(n2), F(n2), W(n2), M(n2), q(Nparams), f(Nparams);
    if (opsec_gpu_estimate(g, Nmodes, evals.data(), cov.data(), y.data(), mixing, phat.data(), pcov.data(), F.data(),
                           W.data(), M.data(), q.data(), f.data()) != OPSEC_OK)
        die("estimate", opsec_gpu_last_error(g));
    std::printf("p_n          error\n");
    for (int n = 0; n < Nparams; n++) std::printf("%e %e\n", phat[n], std::sqrt(pcov[(size_t)n * Nparams + n]));
    // records as estimate-mpi.cpp:619-641
    std::fprintf(fest, "# Parameter estimates and associated matrices.\n");
    std::fprintf(fest, "# This file consists of several consecutive real-valued binary arrays:\n");
    std::fprintf(fest, "# - parameter estimates $\\hat{p}_n$ (vector of length Nparams)\n");
    std::fprintf(fest, "# - covariance matrix $Cov[\\hat{p}_m,\\hat{p}_n]$ (Nparams-by-Nparams matrix)\n");
    std::fprintf(fest, "# - Fisher matrix $F_{mn}$ (Nparams-by-Nparams matrix)\n");
    std::fprintf(fest, "# - window matrix $W_{mn}$ (Nparams-by-Nparams matrix)\n");
    std::fprintf(fest, "# - mixing matrix $M_{mn}$ (Nparams-by-Nparams matrix)\n");
    std::fprintf(fest, "# - quadratic combinations $q_n$ (vector of length Nparams)\n");
    std::fprintf(fest, "# - bias corrections $f_n$ (vector of length Nparams)\n");
    time_t now;
    time(&now);
    std::fprintf(fest, "# Generated %s\n", ctime(&now));
    Config opts;
    opts.set("Nparams", std::to_string(Nparams));
    abn_write(fest, phat.data(), Nparams, "d", &opts);
    abn_write(fest, pcov.data(), n2, "d", nullptr);
    abn_write(fest, F.data(), n2, "d", nullptr);
    abn_write(fest, W.data(), n2, "d", nullptr);
    abn_write(fest, M.data(), n2, "d", nullptr);
    abn_write(fest, q.data(), Nparams, "d", nullptr);
    abn_write(fest, f.data(), Nparams, "d", nullptr);
    std::fclose(fest);
    opsec_gpu_destroy(g);
    return 0;
}
