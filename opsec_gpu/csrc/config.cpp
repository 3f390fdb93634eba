// config.cpp -- the configuration text (cfg.c key = value rules) and the P(k) file into the context.
#include "context.h"

void load_pkfile(opsec_gpu* c, const std::string& path) {
    // Spline.cpp:48-90 LoadData: skip blank and '#' lines, columns 1 and 2
    FILE* fp = std::fopen(path.c_str(), "r");
    if (!fp) fail(OPSEC_ERR_FILE, "could not read pkfile '" + path + "'");
    char buf[4096];
    std::vector<double> k, P;
    while (std::fgets(buf, sizeof buf, fp)) {
        if (buf[0] == '\0' || buf[0] == '#' || buf[0] == '\n') continue;
        char* e1 = nullptr;
        double a = std::strtod(buf, &e1);
        char* e2 = nullptr;
        double b = std::strtod(e1, &e2);
        if (e1 == buf || e2 == e1) continue;
        k.push_back(a);
        P.push_back(b);
    }
    std::fclose(fp);
    if (k.size() < 2) fail(OPSEC_ERR_FILE, "pkfile '" + path + "' holds fewer than two points");
    c->pk_k = k;
    c->pk_P = P;
}

void configure(opsec_gpu* c, const std::map<std::string, std::string>& kv) {
    auto has = [&](const std::string& k) { return kv.count(k) > 0; };
    auto get = [&](const std::string& k) -> const std::string& {
        auto it = kv.find(k);
        if (it == kv.end()) fail(OPSEC_ERR_CONFIG, "missing configuration option " + k);
        return it->second;
    };
    // survey (Survey.cpp:12-60, InitializeSurvey Survey.cpp:140-165)
    std::string type = has("survey.type") ? get("survey.type") : "";
    std::string cs = has("coordsys") ? get("coordsys") : "";
    if (type == "BoxSurvey" || (type.empty() && cs == "cartesian")) {
        c->geo.coordsys = 1;
        const char* names[6] = {"XMin", "XMax", "YMin", "YMax", "ZMin", "ZMax"};
        const char* ns[3] = {"Nx", "Ny", "Nz"};
        for (int i = 0; i < 6; i++) c->geo.b[i] = to_double(names[i], get(std::string("survey.") + names[i]));
        for (int i = 0; i < 3; i++) c->geo.n[i] = to_int(ns[i], get(std::string("survey.") + ns[i]));
        // BoxSurvey separation is periodic with period L (BoxSurvey.cpp:19-37); L <= 0 = open box
        c->geo.L = has("survey.L") ? to_double("survey.L", get("survey.L")) : 0.0;
        if (has("survey.periodic") && get("survey.periodic") == "0") c->geo.L = 0.0;
    } else if (type == "SphericalSurvey" || (type.empty() && cs == "spherical")) {
        c->geo.coordsys = 2;
        c->geo.b[0] = to_double("RMin", get("survey.RMin"));
        c->geo.b[1] = to_double("RMax", get("survey.RMax"));
        // Survey.cpp:39 reads MuMin from the key "MuMuin"; it wins when present
        c->geo.b[2] = has("survey.MuMuin") ? to_double("MuMuin", get("survey.MuMuin"))
                                           : to_double("MuMin", get("survey.MuMin"));
        c->geo.b[3] = to_double("MuMax", get("survey.MuMax"));
        c->geo.b[4] = to_double("PhiMin", get("survey.PhiMin"));
        c->geo.b[5] = to_double("PhiMax", get("survey.PhiMax"));
        c->geo.n[0] = to_int("Nr", get("survey.Nr"));
        c->geo.n[1] = to_int("Nmu", get("survey.Nmu"));
        c->geo.n[2] = to_int("Nphi", get("survey.Nphi"));
    } else {
        fail(OPSEC_ERR_CONFIG, "survey.type must be BoxSurvey or SphericalSurvey (got '" + type + "')");
    }
    for (int i = 0; i < 3; i++) {
        if (c->geo.n[i] <= 0) fail(OPSEC_ERR_CONFIG, "survey grid sizes must be positive");
        if (!(c->geo.b[2 * i] < c->geo.b[2 * i + 1])) fail(OPSEC_ERR_CONFIG, "survey bounds must satisfy Min < Max");
    }
    if (c->geo.coordsys == 2 && (c->geo.b[0] < 0 || c->geo.b[2] < -1 || c->geo.b[3] > 1))
        fail(OPSEC_ERR_CONFIG, "spherical bounds need RMin >= 0 and -1 <= MuMin < MuMax <= 1");

    // model (Model.cpp:26-51, RealModel.cpp:33-79)
    if (has("model") && get("model") != "RealModel")
        fail(OPSEC_ERR_CONFIG, "model must be RealModel (got '" + get("model") + "')");
    if (has("RealModel.pkfile")) load_pkfile(c, get("RealModel.pkfile"));
    if (has("RealModel.bands")) {
        // whitespace- or comma-separated kmin kmax pairs (cfg_get_array_double, RealModel.cpp:44-48)
        std::string text = get("RealModel.bands");
        for (char& ch : text)
            if (ch == ',') ch = ' ';
        std::istringstream in(text);
        std::vector<double> v;
        std::string tok;
        while (in >> tok) v.push_back(to_double("RealModel.bands", tok));
        if (v.size() % 2) v.pop_back();  // RealModel.cpp:49-52 drops an odd trailing value
        for (size_t i = 0; i + 1 < v.size(); i += 2) {
            c->band_lo.push_back(v[i]);
            c->band_hi.push_back(v[i + 1]);
        }
    } else if (has("RealModel.Nbands")) {
        int nb = to_int("Nbands", get("RealModel.Nbands"));
        double kmin = to_double("kmin", get("RealModel.kmin"));
        double kmax = to_double("kmax", get("RealModel.kmax"));
        if (nb <= 0) fail(OPSEC_ERR_CONFIG, "RealModel.Nbands must be positive");
        for (int n = 0; n < nb; n++) {
            c->band_lo.push_back(kmin + n * (kmax - kmin) / nb);
            c->band_hi.push_back(kmin + (n + 1) * (kmax - kmin) / nb);
        }
    } else {
        fail(OPSEC_ERR_CONFIG, "k-bands not specified (RealModel.bands or RealModel.Nbands,kmin,kmax)");
    }
    if (c->band_lo.empty()) fail(OPSEC_ERR_CONFIG, "at least one k-band is required");
    for (size_t i = 0; i < c->band_lo.size(); i++)
        if (!(c->band_lo[i] < c->band_hi[i]) || c->band_lo[i] < 0)
            fail(OPSEC_ERR_CONFIG, "band " + std::to_string(i) + " has kmin >= kmax or kmin < 0");

    if (has("Nmodes")) c->nmodes_cfg = to_int("Nmodes", get("Nmodes"));
    if (has("mixing")) {
        // cfg_get_enum (cfg.c:486-501, estimate-mpi.cpp:369-372): the first of inverse,
        // inverse-sqrt, identity that the value is a prefix of; no match is inverse
        const std::string& m = get("mixing");
        static const std::pair<const char*, int> tags[] = {{"inverse", OPSEC_MIXING_INVERSE},
                                                          {"inverse-sqrt", OPSEC_MIXING_INVERSE_SQRT},
                                                          {"identity", OPSEC_MIXING_IDENTITY}};
        c->mixing = OPSEC_MIXING_INVERSE;
        for (const auto& t : tags)
            if (std::string(t.first).compare(0, m.size(), m) == 0 && m.size() <= std::strlen(t.first)) {
                c->mixing = t.second;
                break;
            }
    }
    if (has("xi.n1")) c->xl.n1 = to_int("xi.n1", get("xi.n1"));
    if (has("xi.n2")) c->xl.n2 = to_int("xi.n2", get("xi.n2"));
    if (has("xi.r1")) c->xl.r1 = to_double("xi.r1", get("xi.r1"));
    if (has("xi.r2")) c->xl.r2 = to_double("xi.r2", get("xi.r2"));
    if (c->xl.n1 < 1 || c->xl.n2 < 2 || !(c->xl.r1 > 0) || !(c->xl.r2 > c->xl.r1))
        fail(OPSEC_ERR_CONFIG, "xi table layout needs n1 >= 1, n2 >= 2, 0 < r1 < r2");
    if (has("sig.gauss")) c->ng = to_int("sig.gauss", get("sig.gauss"));
    if (c->ng < 1 || c->ng > 6) fail(OPSEC_ERR_CONFIG, "sig.gauss must be between 1 and 6");
    if (has("projection")) c->projection = get("projection");
    if (has("projection.wait_cycles")) {
        const std::string& v = get("projection.wait_cycles");
        char* end = nullptr;
        c->proj_wait = std::strtoll(v.c_str(), &end, 10);
        if (end == v.c_str() || c->proj_wait < 10000000LL)
            fail(OPSEC_ERR_CONFIG, "projection.wait_cycles must be an integer >= 10000000");
    }
    if (has("projection.arc_tables")) {
        const std::string& v = get("projection.arc_tables");
        if (v != "0" && v != "1") fail(OPSEC_ERR_CONFIG, "projection.arc_tables must be 0 or 1");
        c->proj_arcs = v == "1";
    }
    if (has("projection.chunk")) c->proj_chunk = to_int("projection.chunk", get("projection.chunk"));
    if (c->proj_chunk < 1) fail(OPSEC_ERR_CONFIG, "projection.chunk must be >= 1");
    if (has("azimuthal.gemm")) {
        const std::string& v = get("azimuthal.gemm");
        if (v == "f64" || v == "f32" || v == "tc") {
            c->az_gemm64 = v == "f64";
            c->az_tc = v == "tc";
        } else {
            fail(OPSEC_ERR_CONFIG, "azimuthal.gemm must be tc, f32 or f64");
        }
    }
    if (has("azimuthal.parity")) c->az_parity = get("azimuthal.parity") != "0";
    if (has("azimuthal.overlap")) c->az_overlap = to_int("azimuthal.overlap", get("azimuthal.overlap")) != 0;
    if (has("azimuthal.transform")) {
        const std::string& v = get("azimuthal.transform");
        if (v != "tiled" && v != "rows") fail(OPSEC_ERR_CONFIG, "azimuthal.transform must be tiled or rows");
        c->az_tiled = v == "tiled";
    }
    if (has("azimuthal.eig")) {
        const std::string& v = get("azimuthal.eig");
        if (v != "own" && v != "streams" && v != "batched")
            fail(OPSEC_ERR_CONFIG, "azimuthal.eig must be own, batched or streams");
        c->az_own = v == "own";
        c->az_batched = v != "streams";
    }
    if (has("klt.solver")) {
        c->eig_solver = get("klt.solver");
        if (c->eig_solver != "auto" && c->eig_solver != "dense" && c->eig_solver != "chfsi")
            fail(OPSEC_ERR_CONFIG, "klt.solver must be auto, dense or chfsi");
    }
    if (has("klt.tol")) c->chfsi.tol = to_double("klt.tol", get("klt.tol"));
    if (has("klt.degree")) c->chfsi.degree = to_int("klt.degree", get("klt.degree"));
    if (has("klt.maxit")) c->chfsi.maxit = to_int("klt.maxit", get("klt.maxit"));
    if (has("klt.guard")) {
        c->chfsi.guard = to_int("klt.guard", get("klt.guard"));
        c->chfsi_guard_set = true;
    }
    if (has("klt.refine")) c->chfsi.refine = to_int("klt.refine", get("klt.refine"));
    if (has("klt.cg")) c->chfsi.cg_steps = to_int("klt.cg", get("klt.cg"));
    if (c->chfsi.refine < 0 || c->chfsi.cg_steps < 1) fail(OPSEC_ERR_CONFIG, "klt.refine must be >= 0, klt.cg >= 1");
    if (has("klt.seed")) c->chfsi.seed = (unsigned long long)to_int("klt.seed", get("klt.seed"));
    if (has("klt.gemm")) {
        const std::string& v = get("klt.gemm");
        if (v != "tc" && v != "bf16x9" && v != "f32") fail(OPSEC_ERR_CONFIG, "klt.gemm must be tc, bf16x9 or f32");
        c->chfsi.tc = v == "tc";
        c->chfsi.emulate = v != "f32";
    }
    if (has("klt.fp64")) {
        const std::string& v = get("klt.fp64");
        if (v != "df32" && v != "native") fail(OPSEC_ERR_CONFIG, "klt.fp64 must be df32 or native");
        c->chfsi.df64 = v == "df32";
    }
    if (has("klt.qr")) {
        const std::string& v = get("klt.qr");
        if (v != "cholesky2" && v != "householder") fail(OPSEC_ERR_CONFIG, "klt.qr must be cholesky2 or householder");
        c->chfsi.cholqr = v == "cholesky2";
    }
    if (has("klt.tile")) {
        const std::string& v = get("klt.tile");
        if (v != "auto" && v != "128" && v != "256") fail(OPSEC_ERR_CONFIG, "klt.tile must be auto, 128 or 256");
        c->chfsi.tile = v == "auto" ? 0 : std::atoi(v.c_str());
    }
    if (!(c->chfsi.tol > 0) || c->chfsi.degree < 1 || c->chfsi.degree > 64 || c->chfsi.maxit < 1 || c->chfsi.guard < 0)
        fail(OPSEC_ERR_CONFIG, "klt.tol must be > 0, klt.degree in [1, 64], klt.maxit >= 1, klt.guard >= 0");
    if (has("survey.nbar")) c->sel_nbar = to_double("survey.nbar", get("survey.nbar"));
    if (has("basis.quirk3")) c->basis_quirk3 = to_int("basis.quirk3", get("basis.quirk3")) != 0;
    if (has("basis.samples")) {
        c->basis_samples = to_int("basis.samples", get("basis.samples"));
        if (c->basis_samples < 1 || c->basis_samples > 1024) fail(OPSEC_ERR_CONFIG, "basis.samples must be in [1, 1024]");
    }
    if (has("azimuthal.split")) {
        c->az_split = to_int("azimuthal.split", get("azimuthal.split"));
        if (c->az_split < 1 || c->az_split > opsec_gpu::kSide) fail(OPSEC_ERR_CONFIG, "azimuthal.split must be in [1, 16]");
    }
    if (has("azimuthal.streams")) {
        c->az_streams = to_int("azimuthal.streams", get("azimuthal.streams"));
        if (c->az_streams < 1 || c->az_streams > opsec_gpu::kSide) fail(OPSEC_ERR_CONFIG, "azimuthal.streams must be in [1, 16]");
    }
    if (has("surrogate")) c->surr_on = get("surrogate") == "1";
    if (has("surrogate.tol")) c->surr_tol = (float)to_double("surrogate.tol", get("surrogate.tol"));
    if (has("surrogate.far")) c->surr_far = (float)to_double("surrogate.far", get("surrogate.far"));
    if (!(c->surr_tol > 0) || !(c->surr_far >= 1)) fail(OPSEC_ERR_CONFIG, "surrogate.tol must be > 0 and surrogate.far >= 1");
    if (has("cubature.window")) c->cub_window = get("cubature.window") != "0";
    if (has("cubature.window_bins")) c->win_key = to_int("cubature.window_bins", get("cubature.window_bins"));
    if (c->win_key < 16 || c->win_key > 4096) fail(OPSEC_ERR_CONFIG, "cubature.window_bins must be in [16, 4096]");
    if (has("cubature.flush")) c->win_flush = to_int("cubature.flush", get("cubature.flush"));
    if (c->win_flush < 0) fail(OPSEC_ERR_CONFIG, "cubature.flush must be >= 0");
    if (has("cubature.dot")) c->win_dot64 = get("cubature.dot") != "f32";
    if (has("cubature.log_keys")) {
        const std::string& v = get("cubature.log_keys");
        if (v != "0" && v != "1") fail(OPSEC_ERR_CONFIG, "cubature.log_keys must be 0 or 1");
        c->win_logkeys = v == "1";
    }
    if (has("cubature.order")) {
        const std::string& v = get("cubature.order");
        if (v != "key" && v != "window") fail(OPSEC_ERR_CONFIG, "cubature.order must be key or window");
        c->win_keyorder = v == "key";
    }
    if (has("cubature.symmetry")) {
        const std::string& v = get("cubature.symmetry");
        if (v == "reflect")
            c->cub_reflect = true;
        else if (v == "none")
            c->cub_reflect = false;
        else
            fail(OPSEC_ERR_CONFIG, "cubature.symmetry must be reflect or none");
    }
    if (has("cubature.precision")) {
        const std::string& v = get("cubature.precision");
        if (v == "exact")
            c->cub_exact = 1;
        else if (v == "fast")
            c->cub_exact = 0;
        else
            fail(OPSEC_ERR_CONFIG, "cubature.precision must be exact or fast");
    }
    if (has("profile")) c->clock.on = get("profile") == "1";
}

void sync(opsec_gpu* c) { OPSEC_CUDA(cudaStreamSynchronize(c->stream)); }

// ---------------------------------------------------------------- stages
