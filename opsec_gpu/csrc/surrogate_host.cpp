// surrogate_host.cpp -- host side of the learned far-field surrogate: training set, training loop, use in a build.
#include "context.h"

void surr_tables(opsec_gpu* c) {
    std::vector<float4> ti(c->ntab());
    ti[0] = make_float4(0.f, 0.f, 0.02f, 0.f);  // the full xi table: scale of the peak of k^2 P(k)
    for (size_t p = 0; p < c->band_lo.size(); p++)
        ti[p + 1] = make_float4((float)(5 * c->band_lo[p]), (float)(5 * c->band_hi[p]),
                                (float)(0.5 * (c->band_lo[p] + c->band_hi[p])), 0.f);
    c->surr_tinfo.alloc(4 * ti.size());
    OPSEC_CUDA(cudaMemcpyAsync(c->surr_tinfo.p, ti.data(), sizeof(float4) * ti.size(), cudaMemcpyHostToDevice,
                               c->stream));
}

// env_t(r_i) = max |xi_t(r_j)| over r_j in [r_i / 1.25, 1.25 r_i]: the scale of
// the surrogate's target, so that its error follows the local size of a table
void surr_envelope(opsec_gpu* c) {
    const int n = c->xl.n(), ntab = c->ntab();
    std::vector<double> tab((size_t)ntab * n), env((size_t)ntab * n);
    OPSEC_CUDA(cudaMemcpyAsync(tab.data(), c->xi64.p, sizeof(double) * tab.size(), cudaMemcpyDeviceToHost, c->stream));
    std::vector<double> r(n);
    OPSEC_CUDA(cudaMemcpyAsync(r.data(), c->r_grid.p, sizeof(double) * n, cudaMemcpyDeviceToHost, c->stream));
    sync(c);
    for (int t = 0; t < ntab; t++) {
        const double* T = tab.data() + (size_t)t * n;
        int lo = 0, hi = 0;  // window [lo, hi) of r_j in [r_i / 1.25, 1.25 r_i]
        for (int i = 0; i < n; i++) {
            while (lo < i && r[lo] < r[i] / 1.25) lo++;
            if (hi < i + 1) hi = i + 1;
            while (hi < n && r[hi] <= 1.25 * r[i]) hi++;
            double m = 0;
            for (int j = lo; j < hi; j++) m = std::max(m, std::fabs(T[j]));
            env[(size_t)t * n + i] = m > 0 ? m : 1e-300;
        }
    }
    c->surr_env.alloc(env.size());
    OPSEC_CUDA(cudaMemcpyAsync(c->surr_env.p, env.data(), sizeof(double) * env.size(), cudaMemcpyHostToDevice,
                               c->stream));
    sync(c);
}

// key geometry and the canonical far keys; returns their number
long long surr_far_keys(opsec_gpu* c) {
    if (c->geo.coordsys != 2) fail(OPSEC_ERR_CONFIG, "the surrogate covers spherical grids only");
    const KeySpace& ks = c->ks;
    c->surr_kg.alloc((size_t)ks.nkeys * kSurrKeyStride);
    launch_surr_key_geometry(ks, surr_grid(c), c->surr_far, c->surr_kg.p, c->stream, &c->launches);
    c->surr_list.alloc((size_t)ks.nkeys);
    c->surr_cnt.alloc(4);
    OPSEC_CUDA(cudaMemsetAsync(c->surr_cnt.p, 0, sizeof(int) * 4, c->stream));
    launch_surr_far_list(ks, c->surr_kg.p, c->surr_list.p, c->surr_cnt.p, c->stream, &c->launches);
    int n = 0;
    OPSEC_CUDA(cudaMemcpyAsync(&n, c->surr_cnt.p, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
    sync(c);
    return n;
}

// Predict Q of the canonical far keys with the ensemble; keys it accepts are
// marked in surr_done and skipped by the cubature.
void surrogate_stage(opsec_gpu* c) {
    if (c->surr_w.size() != (size_t)opsec_gpu::kMembers * kSurrParams)
        fail(OPSEC_ERR_STATE, "surrogate = 1 but no trained weights: call opsec_gpu_surrogate_train or _weights");
    const KeySpace& ks = c->ks;
    const int ntab = c->ntab();
    surr_tables(c);
    surr_envelope(c);
    const long long nfar = surr_far_keys(c);
    c->surr_done.alloc((size_t)ks.nkeys);
    OPSEC_CUDA(cudaMemsetAsync(c->surr_done.p, 0, (size_t)ks.nkeys, c->stream));
    c->surr_counts[0] = c->surr_counts[1] = 0;
    c->surr_counts[2] = nfar;
    if (nfar == 0) return;
    const int nm = opsec_gpu::kMembers;
    c->surr_wdev.alloc(c->surr_w.size());
    OPSEC_CUDA(cudaMemcpyAsync(c->surr_wdev.p, c->surr_w.data(), sizeof(float) * c->surr_w.size(),
                               cudaMemcpyHostToDevice, c->stream));
    const long long nsamp = nfar * ntab;
    c->surr_pred.alloc((size_t)nm * nsamp);
    const float4* ti = reinterpret_cast<const float4*>(c->surr_tinfo.p);
    if (g_clock) g_clock->begin("surrogate", c->stream, 2.0 * nm * nsamp * (16.0 * 128 + 2 * 128.0 * 128 + 128));
    for (int m = 0; m < nm; m++)
        launch_surr_infer(nsamp, c->surr_list.p, ntab, c->surr_kg.p, ti, nullptr,
                          c->surr_wdev.p + (size_t)m * kSurrParams, c->surr_pred.p + (size_t)m * nsamp, c->stream,
                          &c->launches);
    launch_surr_combine(nfar, c->surr_list.p, ntab, nm, c->surr_pred.p, c->surr_kg.p, c->xl, c->xi64.p,
                        c->surr_env.p, c->surr_ysc, c->surr_tol, ks.nkeys, c->Q.p, c->surr_done.p, c->surr_cnt.p + 1,
                        c->stream, &c->launches);
    if (g_clock) g_clock->end(c->stream);
    int cnt[2] = {0, 0};
    OPSEC_CUDA(cudaMemcpyAsync(cnt, c->surr_cnt.p + 1, sizeof(int) * 2, cudaMemcpyDeviceToHost, c->stream));
    sync(c);
    c->surr_counts[0] = cnt[0];
    c->surr_counts[1] = cnt[1];
}

// Glorot-uniform weights (the first layer over its 12 used inputs), zero biases
void surr_init(std::vector<float>& w, unsigned seed) {
    w.assign(kSurrParams, 0.f);
    uint64_t st = 0x9E3779B97F4A7C15ull ^ ((uint64_t)seed * 0xBF58476D1CE4E5B9ull);
    auto uni = [&]() {  // splitmix64 -> [0, 1)
        st += 0x9E3779B97F4A7C15ull;
        uint64_t z = st;
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        z ^= z >> 31;
        return (double)(z >> 11) / 9007199254740992.0;
    };
    auto fill = [&](int off, int nout, int nin, int nin_used) {
        const double a = std::sqrt(6.0 / (nin_used + nout));
        for (int o = 0; o < nout; o++)
            for (int i = 0; i < nin; i++) w[off + o * nin + i] = i < nin_used ? (float)((2 * uni() - 1) * a) : 0.f;
    };
    fill(kSurrOffW1, kSurrHid, kSurrIn, 12);
    fill(kSurrOffW2, kSurrHid, kSurrHid, kSurrHid);
    fill(kSurrOffW3, kSurrHid, kSurrHid, kSurrHid);
    fill(kSurrOffW4, 1, kSurrHid, kSurrHid);
}

float bf16_round_host(float x) {
    uint32_t u;
    std::memcpy(&u, &x, 4);
    if ((u & 0x7f800000u) == 0x7f800000u) return x;
    u += 0x7fffu + ((u >> 16) & 1u);
    u &= 0xffff0000u;
    float r;
    std::memcpy(&r, &u, 4);
    return r;
}

long long gcd_ll(long long a, long long b) {
    while (b) {
        const long long t = a % b;
        a = b;
        b = t;
    }
    return a;
}

// Train the ensemble on this context's own survey: plain cubature Q of every key,
// then up to max_samples (canonical far key, table) samples, 2 % held out.
// stats: samples, validation rms error of y (mean over members), training seconds, ysc.
void surrogate_train(opsec_gpu* c, long long max_samples, int epochs, unsigned seed, double* stats) {
    const bool was_on = c->surr_on;
    c->surr_on = false;
    c->q_ok = c->qsq_ok = false;
    build_q(c);
    c->surr_on = was_on;
    c->q_ok = c->qsq_ok = false;  // the next build recomputes Q, with the surrogate when it is on
    const KeySpace& ks = c->ks;
    const int ntab = c->ntab();
    surr_tables(c);
    surr_envelope(c);
    const long long nfar = surr_far_keys(c);
    if (nfar < 16) fail(OPSEC_ERR_ARG, "too few far keys to train the surrogate");
    std::vector<long long> keys(nfar);
    OPSEC_CUDA(cudaMemcpyAsync(keys.data(), c->surr_list.p, sizeof(long long) * nfar, cudaMemcpyDeviceToHost,
                               c->stream));
    sync(c);
    std::sort(keys.begin(), keys.end());
    uint64_t st = 0x243F6A8885A308D3ull ^ seed;
    auto rnd = [&]() {  // xorshift64
        st ^= st << 13;
        st ^= st >> 7;
        st ^= st << 17;
        return st;
    };
    for (long long i = nfar - 1; i > 0; i--) std::swap(keys[i], keys[rnd() % (uint64_t)(i + 1)]);
    const long long nk = std::max<long long>(1, std::min<long long>(nfar, max_samples / ntab));
    keys.resize(nk);
    DevBuf<long long> dkeys;
    dkeys.alloc(nk);
    OPSEC_CUDA(cudaMemcpyAsync(dkeys.p, keys.data(), sizeof(long long) * nk, cudaMemcpyHostToDevice, c->stream));
    const long long S = nk * ntab;
    DevBuf<float> feat, y;
    feat.alloc((size_t)S * kSurrIn);
    y.alloc(S);
    launch_surr_samples(S, dkeys.p, ntab, c->surr_kg.p, reinterpret_cast<const float4*>(c->surr_tinfo.p), c->xl,
                        c->xi64.p, c->surr_env.p, c->Q.p, ks.nkeys, feat.p, y.p, c->stream, &c->launches);
    std::vector<float> hy(S);
    OPSEC_CUDA(cudaMemcpyAsync(hy.data(), y.p, sizeof(float) * S, cudaMemcpyDeviceToHost, c->stream));
    sync(c);
    float ysc = 0.f;
    for (float v : hy) ysc = std::max(ysc, std::fabs(v));
    if (!(ysc > 0)) ysc = 1.f;
    for (float& v : hy) v /= ysc;
    OPSEC_CUDA(cudaMemcpyAsync(y.p, hy.data(), sizeof(float) * S, cudaMemcpyHostToDevice, c->stream));
    const long long Sval = std::max<long long>(1, S / 50), Str = S - Sval;
    const int Bn = (int)std::min<long long>(2048, Str);
    DevBuf<float> xb, yb, w, wb, g, m1, v1, scratch, out;
    xb.alloc((size_t)Bn * kSurrIn);
    yb.alloc(Bn);
    w.alloc(kSurrParams);
    wb.alloc(kSurrParams);
    g.alloc(kSurrParams);
    m1.alloc(kSurrParams);
    v1.alloc(kSurrParams);
    scratch.alloc((size_t)7 * Bn * kSurrHid);
    out.alloc(Bn);
    DevBuf<double> loss;
    loss.alloc(1);
    std::vector<float> all((size_t)opsec_gpu::kMembers * kSurrParams);
    auto t0 = std::chrono::steady_clock::now();
    double val_sum = 0;
    for (int mem = 0; mem < opsec_gpu::kMembers; mem++) {
        std::vector<float> hw;
        surr_init(hw, seed * 7919u + 101u * (unsigned)mem + 1u);
        std::vector<float> hwb(hw.size());
        for (size_t i = 0; i < hw.size(); i++) hwb[i] = bf16_round_host(hw[i]);
        OPSEC_CUDA(cudaMemcpyAsync(w.p, hw.data(), sizeof(float) * kSurrParams, cudaMemcpyHostToDevice, c->stream));
        OPSEC_CUDA(cudaMemcpyAsync(wb.p, hwb.data(), sizeof(float) * kSurrParams, cudaMemcpyHostToDevice, c->stream));
        OPSEC_CUDA(cudaMemsetAsync(g.p, 0, sizeof(float) * kSurrParams, c->stream));
        OPSEC_CUDA(cudaMemsetAsync(m1.p, 0, sizeof(float) * kSurrParams, c->stream));
        OPSEC_CUDA(cudaMemsetAsync(v1.p, 0, sizeof(float) * kSurrParams, c->stream));
        const long long steps_per_epoch = std::max<long long>(1, Str / Bn);
        int step = 0;
        for (int ep = 0; ep < epochs; ep++) {
            long long stride = (long long)(rnd() % (uint64_t)Str) | 1;
            while (gcd_ll(stride, Str) != 1) stride += 2;
            const long long off = (long long)(rnd() % (uint64_t)Str);
            const float lr = 2e-3f * std::pow(0.05f, (float)ep / (float)std::max(1, epochs - 1));
            for (long long k = 0; k < steps_per_epoch; k++) {
                launch_surr_gather(Bn, Str, (off + (k * Bn % Str) * (stride % Str)) % Str, stride, feat.p, y.p, xb.p,
                                   yb.p, c->stream, &c->launches);
                surr_forward_backward(Bn, xb.p, yb.p, wb.p, g.p, nullptr, out.p, scratch.p, c->stream, &c->launches);
                launch_surr_adam(w.p, wb.p, g.p, m1.p, v1.p, lr, ++step, c->stream, &c->launches);
            }
        }
        // validation rms of y over the held-out tail
        double se = 0;
        long long nv = 0;
        for (long long i0 = Str; i0 < S; i0 += Bn) {
            const int nb = (int)std::min<long long>(Bn, S - i0);
            OPSEC_CUDA(cudaMemsetAsync(loss.p, 0, sizeof(double), c->stream));
            surr_forward_backward(nb, feat.p + (size_t)i0 * kSurrIn, y.p + i0, wb.p, g.p, loss.p, out.p, scratch.p,
                                  c->stream, &c->launches);
            double l = 0;
            OPSEC_CUDA(cudaMemcpyAsync(&l, loss.p, sizeof(double), cudaMemcpyDeviceToHost, c->stream));
            sync(c);
            se += l * nb;
            nv += nb;
        }
        val_sum += std::sqrt(se / std::max<long long>(nv, 1)) * ysc;
        OPSEC_CUDA(cudaMemcpyAsync(all.data() + (size_t)mem * kSurrParams, w.p, sizeof(float) * kSurrParams,
                                   cudaMemcpyDeviceToHost, c->stream));
        sync(c);
    }
    const double secs = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    c->surr_w = all;
    c->surr_ysc = ysc;
    if (stats) {
        stats[0] = (double)S;
        stats[1] = val_sum / opsec_gpu::kMembers;
        stats[2] = secs;
        stats[3] = ysc;
    }
}
