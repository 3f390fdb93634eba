// surrogate.cu -- the learned far-field surrogate of the cell-pair integrals.
//
// For a key whose two cells are at least `far` cell widths apart, a small MLP
// predicts the residual of Q_t(key) from the point value xi_t(d) at the
// centre separation d, in units of the table's local envelope env_t(d) =
// max |xi_t(r)| over r in [d / 1.25, 1.25 d]:
//
//   y_t(key) = (Q_t(key) - xi_t(d)) / env_t(d),   Q_t = xi_t(d) + env_t(d) ysc net(f)
//
// Inputs (12): d / 1000; k times the mean transverse path difference
// <|e_perp|^2> / 24 d; k times the six cell edges (dr, r dtheta, r sin(theta)
// dphi of both cells) projected on the separation, / 10; the band's k edges
// x 5 (both 0 for the full xi table); sin(k d) and cos(k d), with k the band
// centre (0.02 for the full xi table).  The phase features carry the
// oscillation of a table across the pair and the k-scaled extents its
// averaging over the cells, so the network learns a smooth map.
// Network: 12 (padded to 16) -> 128 -> 128 -> 128 -> 1, tanh-form GELU,
// BF16 weights and activations into every product, FP32 accumulation, FP32
// master weights trained by Adam.  Four members with different initial
// weights and sample orders form the ensemble; a key goes back to the
// cubature when any table's members spread by more than `tol` in y.
//
// Kernels:
//  * surr_key_geometry_kernel  per key: the 8 geometry features, d, far flag;
//  * surr_samples_kernel       training samples (features, target) from Q;
//  * surr_gemm_kernel          tiled FP32 GEMM with strides (training: the
//                              forward products, dX = dZ W, dW = dZ^T X) and
//                              fused bias/GELU/GELU' epilogues;
//  * surr_out_kernel, surr_colsum_kernel, surr_adam_kernel  the output layer,
//                              loss gradient, bias gradients and the update;
//  * surr_infer_kernel         the fused inference: one warp carries 16
//                              samples through all layers in registers with
//                              mma.sync m16n8k16 BF16 products;
//  * surr_combine_kernel       ensemble mean and spread, Q of accepted keys.
#include <cuda_bf16.h>

#include <algorithm>
#include <cmath>

#include "engine.h"

namespace opsec {
namespace {

__device__ __forceinline__ float bf16r(float x) { return __bfloat162float(__float2bfloat16_rn(x)); }

constexpr float kGeluC = 0.7978845608028654f;  // sqrt(2 / pi)

__device__ __forceinline__ float gelu(float z) {
    const float u = kGeluC * fmaf(0.044715f * z, z * z, z);
    return 0.5f * z * (1.f + tanhf(u));
}

__device__ __forceinline__ float gelu_grad(float z) {
    const float u = kGeluC * fmaf(0.044715f * z, z * z, z);
    const float th = tanhf(u);
    const float du = kGeluC * fmaf(3.f * 0.044715f, z * z, 1.f);
    return 0.5f * (1.f + th) + 0.5f * z * (1.f - th * th) * du;
}

// xi table value at r by the QSpline rule (linear in r below r1, in ln r above; QSpline.cpp:61-70)
__device__ double xi_at(const XiLayout& xl, const double* tab, double r) {
    const int n = xl.n();
    if (r < 0) return 0.0;
    if (r < xl.r1) {
        const double t = r * xl.n1 / xl.r1;
        const int i = min((int)t, xl.n1 - 1);
        const double fr = t - i;
        return tab[i] + fr * (tab[i + 1] - tab[i]);
    }
    if (r >= xl.r2) return tab[n - 1];
    const double du = log(xl.r2 / xl.r1) / (xl.n2 - 1);
    const double t = log(r / xl.r1) / du;
    const int j = min((int)t, xl.n2 - 2);
    const double fr = t - j;
    return tab[xl.n1 + j] + fr * (tab[xl.n1 + j + 1] - tab[xl.n1 + j]);
}

__device__ void tri_decode(int H, long long tri, int* ha, int* hb) {
    const double H2 = 2.0 * H + 1.0;
    int a = (int)floor((H2 - sqrt(H2 * H2 - 8.0 * (double)tri)) * 0.5);
    if (a < 0) a = 0;
    while (a > 0 && (long long)a * H - (long long)a * (a - 1) / 2 > tri) --a;
    while ((long long)(a + 1) * H - (long long)(a + 1) * a / 2 <= tri) ++a;
    *ha = a;
    *hb = a + (int)(tri - ((long long)a * H - (long long)a * (a - 1) / 2));
}

// ---------------------------------------------------------------- geometry and samples
__global__ void surr_key_geometry_kernel(KeySpace ks, SurrGrid g, float far_widths, float* kg) {
    for (long long key = blockIdx.x * (long long)blockDim.x + threadIdx.x; key < ks.nkeys;
         key += (long long)gridDim.x * blockDim.x) {
        const int df = (int)(key % ks.nf);
        int ha, hb;
        tri_decode(ks.H, key / ks.nf, &ha, &hb);
        const int ia[3] = {ha / ks.N2, ha % ks.N2, 0}, ib[3] = {hb / ks.N2, hb % ks.N2, df};
        double c[2][3], e[2][3];
        for (int s = 0; s < 2; s++) {
            const int* id = s ? ib : ia;
            const double r0 = g.b[0] + id[0] * g.d[0], r1 = r0 + g.d[0];
            const double m0 = g.b[2] + id[1] * g.d[1], m1 = m0 + g.d[1];
            const double p0 = g.b[4] + id[2] * g.d[2];
            const double r = 0.5 * (r0 + r1), mu = 0.5 * (m0 + m1), ph = p0 + 0.5 * g.d[2];
            const double st = sqrt(fmax(1.0 - mu * mu, 0.0));
            c[s][0] = r * st * cos(ph);
            c[s][1] = r * st * sin(ph);
            c[s][2] = r * mu;
            e[s][0] = r1 - r0;
            e[s][1] = r * (acos(fmax(fmin(m0, 1.0), -1.0)) - acos(fmax(fmin(m1, 1.0), -1.0)));
            e[s][2] = r * st * g.d[2];
        }
        double dv[3];
        for (int k = 0; k < 3; k++) dv[k] = c[1][k] - c[0][k];
        const double d = sqrt(dv[0] * dv[0] + dv[1] * dv[1] + dv[2] * dv[2]);
        double nh[3] = {0, 0, 1};
        if (d > 0)
            for (int k = 0; k < 3; k++) nh[k] = dv[k] / d;
        // edges of each cell along its local (r, theta, phi) frame, projected on the separation:
        // a = |e . n| (longitudinal spread), and the transverse spread sum |e|^2 - a^2
        double a[6], trans = 0, w = 0;
        for (int s = 0; s < 2; s++) {
            const double r = sqrt(c[s][0] * c[s][0] + c[s][1] * c[s][1] + c[s][2] * c[s][2]);
            const double ct = c[s][2] / r, st = sqrt(fmax(1.0 - ct * ct, 0.0));
            const double ph = atan2(c[s][1], c[s][0]);
            const double cp = cos(ph), sp = sin(ph);
            const double fr[3][3] = {{st * cp, st * sp, ct}, {ct * cp, ct * sp, -st}, {-sp, cp, 0.0}};
            for (int k = 0; k < 3; k++) {
                const double proj = e[s][k] * fabs(fr[k][0] * nh[0] + fr[k][1] * nh[1] + fr[k][2] * nh[2]);
                a[3 * s + k] = proj;
                trans += e[s][k] * e[s][k] - proj * proj;
                w = fmax(w, e[s][k]);
            }
        }
        float* o = kg + (size_t)key * kSurrKeyStride;
        o[0] = (float)(d / 1000);
        o[1] = (float)(d > 0 ? trans / (24.0 * d) : 0.0);  // mean transverse path difference, Mpc
        for (int k = 0; k < 6; k++) o[2 + k] = (float)a[k];
        o[8] = (float)d;
        o[9] = d >= far_widths * w ? 1.f : 0.f;
    }
}

// feature c of sample (key geometry kg, table info ti = (k_lo 5, k_hi 5, k mid, 0)):
// d / 1000, k <t^2> / 2d, k a_i / 10 for the six projected cell edges, the k edges, sin(k d), cos(k d)
__device__ __forceinline__ float surr_feature(const float* kg, float4 ti, int c) {
    switch (c) {
    case 0: return kg[0];
    case 1: return ti.z * kg[1];  // phase of the mean transverse path difference
    case 2: case 3: case 4: case 5: case 6: case 7: return 0.1f * ti.z * kg[c];  // k x projected extents
    case 8: return ti.x;
    case 9: return ti.y;
    case 10: return sinf(ti.z * kg[8]);
    case 11: return cosf(ti.z * kg[8]);
    default: return 0.f;
    }
}

// Training samples: sample s = (key list[s / ntab], table s % ntab): BF16-valued
// features [s][16] and target y = (Q - xi_t(d)) / env_t(d).
__global__ void surr_samples_kernel(long long nsamp, const long long* keys, int ntab, const float* kg,
                                    const float4* tinfo, XiLayout xl, const double* xi64, const double* env,
                                    const double* Q, long long nkeys, float* feat, float* y) {
    const int n = xl.n();
    for (long long s = blockIdx.x * (long long)blockDim.x + threadIdx.x; s < nsamp;
         s += (long long)gridDim.x * blockDim.x) {
        const long long key = keys[s / ntab];
        const int t = (int)(s % ntab);
        const float* g = kg + (size_t)key * kSurrKeyStride;
        const float4 ti = tinfo[t];
        for (int c = 0; c < kSurrIn; c++) feat[(size_t)s * kSurrIn + c] = bf16r(surr_feature(g, ti, c));
        const double* tab = xi64 + (size_t)t * n;
        y[s] = (float)((Q[(size_t)t * nkeys + key] - xi_at(xl, tab, g[8])) / xi_at(xl, env + (size_t)t * n, g[8]));
    }
}

// ---------------------------------------------------------------- training kernels
// C[m][n] = sum_k A(m,k) B(k,n), A(m,k) = A[m sam + k sak], B(k,n) = B[k sbk + n sbn];
// epilogue: 0 plain store, 1 Z = C + bias[n] and A = gelu(Z) (round to BF16 if `round`),
// 2 C *= gelu'(Zprev[m][n]) (the backward through the previous layer's GELU).
constexpr int kTM = 64, kTN = 64, kTK = 16;
__global__ void __launch_bounds__(256) surr_gemm_kernel(int M, int N, int K, const float* A, long long sam,
                                                        long long sak, const float* B, long long sbk, long long sbn,
                                                        float* C, int ldc, int epi, const float* bias, float* act,
                                                        int round, const float* zprev) {
    __shared__ float As[kTK][kTM + 4];
    __shared__ float Bs[kTK][kTN + 4];
    const int tx = threadIdx.x % 16, ty = threadIdx.x / 16;
    const int m0 = blockIdx.y * kTM, n0 = blockIdx.x * kTN;
    // split K over blockIdx.z (then the partial products are added into C, which starts at zero)
    const int kc = (K + gridDim.z - 1) / gridDim.z;
    const int kbeg = blockIdx.z * kc, kend = min(K, kbeg + kc);
    float acc[4][4] = {};
    for (int k0 = kbeg; k0 < kend; k0 += kTK) {
        for (int e = threadIdx.x; e < kTK * kTM; e += 256) {
            const int kk = e / kTM, mm = e % kTM;
            const int m = m0 + mm, k = k0 + kk;
            As[kk][mm] = (m < M && k < kend) ? A[m * sam + k * sak] : 0.f;
        }
        for (int e = threadIdx.x; e < kTK * kTN; e += 256) {
            const int kk = e / kTN, nn = e % kTN;
            const int n = n0 + nn, k = k0 + kk;
            Bs[kk][nn] = (n < N && k < kend) ? B[k * sbk + n * sbn] : 0.f;
        }
        __syncthreads();
#pragma unroll
        for (int kk = 0; kk < kTK; kk++) {
            float a[4], b[4];
#pragma unroll
            for (int i = 0; i < 4; i++) {
                a[i] = As[kk][ty * 4 + i];
                b[i] = Bs[kk][tx * 4 + i];
            }
#pragma unroll
            for (int i = 0; i < 4; i++)
#pragma unroll
                for (int j = 0; j < 4; j++) acc[i][j] = fmaf(a[i], b[j], acc[i][j]);
        }
        __syncthreads();
    }
#pragma unroll
    for (int i = 0; i < 4; i++)
#pragma unroll
        for (int j = 0; j < 4; j++) {
            const int m = m0 + ty * 4 + i, n = n0 + tx * 4 + j;
            if (m >= M || n >= N) continue;
            float v = acc[i][j];
            if (epi == 1) {
                v += bias[n];
                const float a = gelu(v);
                act[(size_t)m * ldc + n] = round ? bf16r(a) : a;
            } else if (epi == 2) {
                v *= gelu_grad(zprev[(size_t)m * ldc + n]);
            }
            if (gridDim.z > 1)
                atomicAdd(&C[(size_t)m * ldc + n], v);
            else
                C[(size_t)m * ldc + n] = v;
        }
}

// out[b] = a3[b] . w4 + b4; with targets: loss += mean (out - y)^2 and dZ3 = dout w4 gelu'(Z3),
// dout = 2 (out - y) / B
__global__ void surr_out_kernel(int Bn, const float* a3, const float* z3, const float* w, const float* y, float* out,
                                float* dz3, double* loss) {
    const int b = blockIdx.x * blockDim.y + threadIdx.y;
    const int lane = threadIdx.x;
    if (b >= Bn) return;
    const float* w4 = w + kSurrOffW4;
    float s = 0.f;
    for (int n = lane; n < kSurrHid; n += 32) s = fmaf(a3[(size_t)b * kSurrHid + n], w4[n], s);
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    const float o = s + w[kSurrOffB4];
    if (out && lane == 0) out[b] = o;
    if (!y) return;
    const float dout = 2.f * (o - y[b]) / Bn;
    if (lane == 0 && loss) atomicAdd(loss, (double)(o - y[b]) * (o - y[b]) / Bn);
    for (int n = lane; n < kSurrHid; n += 32)
        dz3[(size_t)b * kSurrHid + n] = dout * w4[n] * gelu_grad(z3[(size_t)b * kSurrHid + n]);
}

// output-layer gradients: dw4[n] = sum_b dout_b a3[b][n], db4 = sum_b dout_b
__global__ void surr_outgrad_kernel(int Bn, const float* a3, const float* out, const float* y, float* grad) {
    const int n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n > kSurrHid) return;
    double s = 0;
    for (int b = 0; b < Bn; b++) {
        const double dout = 2.0 * ((double)out[b] - y[b]) / Bn;
        s += dout * (n < kSurrHid ? a3[(size_t)b * kSurrHid + n] : 1.f);
    }
    grad[n < kSurrHid ? kSurrOffW4 + n : kSurrOffB4] = (float)s;
}

// bias gradient: column sums of dZ [B][N]
__global__ void surr_colsum_kernel(int Bn, int N, const float* dz, float* g) {
    const int n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= N) return;
    float s = 0.f;
    for (int b = 0; b < Bn; b++) s += dz[(size_t)b * N + n];
    g[n] = s;
}

// Adam on the FP32 master weights; wb = BF16-valued copy used by the products
__global__ void surr_adam_kernel(int np, float* w, float* wb, const float* g, float* m, float* v, float lr, float b1t,
                                 float b2t) {
    const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < np; i += gridDim.x * blockDim.x) {
        const float gi = g[i];
        m[i] = b1 * m[i] + (1 - b1) * gi;
        v[i] = b2 * v[i] + (1 - b2) * gi * gi;
        const float mh = m[i] / (1 - b1t), vh = v[i] / (1 - b2t);
        w[i] -= lr * mh / (sqrtf(vh) + eps);
        wb[i] = bf16r(w[i]);
    }
}

// minibatch gather: rows (off + i stride) mod S
__global__ void surr_gather_kernel(int Bn, long long S, long long off, long long stride, const float* feat,
                                   const float* y, float* xb, float* yb) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= Bn) return;
    const long long s = (off + (long long)i * stride) % S;
    for (int c = 0; c < kSurrIn; c++) xb[(size_t)i * kSurrIn + c] = feat[(size_t)s * kSurrIn + c];
    yb[i] = y[s];
}

// ---------------------------------------------------------------- fused inference (mma.sync BF16)
constexpr int kW1S = 24;   // shared-memory row strides (bf16) that keep the B-fragment loads conflict-free
constexpr int kW23S = 136;

__device__ __forceinline__ uint32_t pack2(float lo, float hi) {
    const __nv_bfloat162 p = __floats2bfloat162_rn(lo, hi);
    return *reinterpret_cast<const uint32_t*>(&p);
}

__device__ __forceinline__ void mma16816(float* c, const uint32_t* a, uint32_t b0, uint32_t b1) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};\n"
        : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

// Samples s = (keys[s / ntab], table s % ntab), or explicit features when feat != null.
// Fragment layout of m16n8k16 (g = lane / 4, t = lane % 4): A regs hold
// (row g, cols 2t..2t+1), (row g+8, 2t..), (row g, 2t+8..), (row g+8, 2t+8..);
// B regs (rows 2t..2t+1, col g), (rows 2t+8.., col g); C (row g, cols 2t..2t+1),
// (row g+8, cols 2t..).  Two neighbouring 8-column C tiles of one layer are
// one 16-wide A tile of the next.
__global__ void __launch_bounds__(256) surr_infer_kernel(long long nsamp, const long long* keys, int ntab,
                                                         const float* kg, const float4* tinfo, const float* feat,
                                                         const float* w, float* out) {
    extern __shared__ __align__(16) unsigned char surr_smem[];
    __nv_bfloat16* sW1 = reinterpret_cast<__nv_bfloat16*>(surr_smem);
    __nv_bfloat16* sW2 = sW1 + kSurrHid * kW1S;
    __nv_bfloat16* sW3 = sW2 + kSurrHid * kW23S;
    float* sB = reinterpret_cast<float*>(sW3 + kSurrHid * kW23S);  // b1, b2, b3, w4, b4
    for (int e = threadIdx.x; e < kSurrHid * kSurrIn; e += blockDim.x)
        sW1[(e / kSurrIn) * kW1S + e % kSurrIn] = __float2bfloat16_rn(w[kSurrOffW1 + e]);
    for (int e = threadIdx.x; e < kSurrHid * kSurrHid; e += blockDim.x) {
        sW2[(e / kSurrHid) * kW23S + e % kSurrHid] = __float2bfloat16_rn(w[kSurrOffW2 + e]);
        sW3[(e / kSurrHid) * kW23S + e % kSurrHid] = __float2bfloat16_rn(w[kSurrOffW3 + e]);
    }
    // every parameter enters as its BF16 value, as in training
    for (int e = threadIdx.x; e < kSurrHid; e += blockDim.x) {
        sB[e] = bf16r(w[kSurrOffB1 + e]);
        sB[kSurrHid + e] = bf16r(w[kSurrOffB2 + e]);
        sB[2 * kSurrHid + e] = bf16r(w[kSurrOffB3 + e]);
        sB[3 * kSurrHid + e] = bf16r(w[kSurrOffW4 + e]);
    }
    if (threadIdx.x == 0) sB[4 * kSurrHid] = bf16r(w[kSurrOffB4]);
    __syncthreads();
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
    const long long ntiles = (nsamp + 15) / 16;
    for (long long tile = (long long)blockIdx.x * 8 + warp; tile < ntiles; tile += (long long)gridDim.x * 8) {
        const long long s0 = tile * 16;
        // layer-1 A fragment: features of samples s0+g and s0+g+8, columns 2t,2t+1 and 2t+8,2t+9
        float f[2][4];
#pragma unroll
        for (int h = 0; h < 2; h++) {
            const long long s = s0 + g + 8 * h;
#pragma unroll
            for (int q = 0; q < 4; q++) {
                const int col = 2 * t + (q & 1) + 8 * (q >> 1);
                float v = 0.f;
                if (s < nsamp) {
                    if (feat) {
                        v = feat[(size_t)s * kSurrIn + col];
                    } else {
                        const float* kgs = kg + (size_t)keys[s / ntab] * kSurrKeyStride;
                        v = surr_feature(kgs, tinfo[s % ntab], col);
                    }
                }
                f[h][q] = v;
            }
        }
        uint32_t a[8][4];
        a[0][0] = pack2(f[0][0], f[0][1]);
        a[0][1] = pack2(f[1][0], f[1][1]);
        a[0][2] = pack2(f[0][2], f[0][3]);
        a[0][3] = pack2(f[1][2], f[1][3]);
        float c[16][4];
        // layer 1: K = 16
#pragma unroll
        for (int j = 0; j < 16; j++) {
            c[j][0] = c[j][1] = c[j][2] = c[j][3] = 0.f;
            const __nv_bfloat16* wr = sW1 + (8 * j + g) * kW1S + 2 * t;
            mma16816(c[j], a[0], *reinterpret_cast<const uint32_t*>(wr), *reinterpret_cast<const uint32_t*>(wr + 8));
        }
        // hidden layers 2 and 3
#pragma unroll
        for (int layer = 0; layer < 2; layer++) {
            const float* bl = sB + layer * kSurrHid;
#pragma unroll
            for (int kk = 0; kk < 8; kk++) {
                const int n0 = 16 * kk + 2 * t, n1 = n0 + 8;
                a[kk][0] = pack2(gelu(c[2 * kk][0] + bl[n0]), gelu(c[2 * kk][1] + bl[n0 + 1]));
                a[kk][1] = pack2(gelu(c[2 * kk][2] + bl[n0]), gelu(c[2 * kk][3] + bl[n0 + 1]));
                a[kk][2] = pack2(gelu(c[2 * kk + 1][0] + bl[n1]), gelu(c[2 * kk + 1][1] + bl[n1 + 1]));
                a[kk][3] = pack2(gelu(c[2 * kk + 1][2] + bl[n1]), gelu(c[2 * kk + 1][3] + bl[n1 + 1]));
            }
            const __nv_bfloat16* W = layer == 0 ? sW2 : sW3;
#pragma unroll
            for (int j = 0; j < 16; j++) {
                c[j][0] = c[j][1] = c[j][2] = c[j][3] = 0.f;
#pragma unroll
                for (int kk = 0; kk < 8; kk++) {
                    const __nv_bfloat16* wr = W + (8 * j + g) * kW23S + 16 * kk + 2 * t;
                    mma16816(c[j], a[kk], *reinterpret_cast<const uint32_t*>(wr),
                             *reinterpret_cast<const uint32_t*>(wr + 8));
                }
            }
        }
        // output: gelu(z3 + b3) . w4 + b4, FP32
        const float* b3 = sB + 2 * kSurrHid;
        const float* w4 = sB + 3 * kSurrHid;
        float o0 = 0.f, o1 = 0.f;
#pragma unroll
        for (int j = 0; j < 16; j++) {
            const int n = 8 * j + 2 * t;
            o0 = fmaf(gelu(c[j][0] + b3[n]), w4[n], fmaf(gelu(c[j][1] + b3[n + 1]), w4[n + 1], o0));
            o1 = fmaf(gelu(c[j][2] + b3[n]), w4[n], fmaf(gelu(c[j][3] + b3[n + 1]), w4[n + 1], o1));
        }
        o0 += __shfl_xor_sync(0xffffffffu, o0, 1);
        o0 += __shfl_xor_sync(0xffffffffu, o0, 2);
        o1 += __shfl_xor_sync(0xffffffffu, o1, 1);
        o1 += __shfl_xor_sync(0xffffffffu, o1, 2);
        if (t == 0) {
            const float b4 = sB[4 * kSurrHid];
            if (s0 + g < nsamp) out[s0 + g] = o0 + b4;
            if (s0 + g + 8 < nsamp) out[s0 + g + 8] = o1 + b4;
        }
    }
}

// Ensemble: per key of the list, every table's member mean and spread; a key
// whose spreads all stay within tol gets Q_t = xi_t(d) + env_t(d) ysc mean and
// is marked done; the others are left to the cubature.
__global__ void surr_combine_kernel(long long nlist, const long long* keys, int ntab, int nmem, const float* pred,
                                    const float* kg, XiLayout xl, const double* xi64, const double* env, float ysc,
                                    float tol, long long nkeys, double* Q, unsigned char* done, int* counts) {
    const int n = xl.n();
    const long long nsamp = nlist * ntab;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < nlist;
         i += (long long)gridDim.x * blockDim.x) {
        const long long key = keys[i];
        bool ok = true;
        for (int t = 0; t < ntab && ok; t++) {
            float lo = 1e30f, hi = -1e30f;
            for (int m = 0; m < nmem; m++) {
                const float p = pred[(size_t)m * nsamp + i * ntab + t];
                lo = fminf(lo, p);
                hi = fmaxf(hi, p);
            }
            if (!((hi - lo) * ysc <= tol)) ok = false;  // also rejects NaN
        }
        if (!ok) {
            atomicAdd(&counts[1], 1);
            continue;
        }
        const double d = kg[(size_t)key * kSurrKeyStride + 8];
        for (int t = 0; t < ntab; t++) {
            double s = 0;
            for (int m = 0; m < nmem; m++) s += pred[(size_t)m * nsamp + i * ntab + t];
            Q[(size_t)t * nkeys + key] =
                xi_at(xl, xi64 + (size_t)t * n, d) + xi_at(xl, env + (size_t)t * n, d) * ysc * (s / nmem);
        }
        done[key] = 1;
        atomicAdd(&counts[0], 1);
    }
}

// canonical keys (under the mu reflection) whose cells are far apart
__global__ void surr_far_list_kernel(KeySpace ks, const float* kg, long long* list, int* count) {
    for (long long key = blockIdx.x * (long long)blockDim.x + threadIdx.x; key < ks.nkeys;
         key += (long long)gridDim.x * blockDim.x) {
        if (kg[(size_t)key * kSurrKeyStride + 9] == 0.f) continue;
        if (ks.mu_reflect) {
            const int df = (int)(key % ks.nf);
            int ha, hb;
            tri_decode(ks.H, key / ks.nf, &ha, &hb);
            const int pa = (ha / ks.N2) * ks.N2 + (ks.N2 - 1 - ha % ks.N2);
            const int pb = (hb / ks.N2) * ks.N2 + (ks.N2 - 1 - hb % ks.N2);
            const int p1 = min(pa, pb), p2 = max(pa, pb);
            const long long pk = ((long long)p1 * ks.H - (long long)p1 * (p1 - 1) / 2 + (p2 - p1)) * ks.nf + df;
            if (pk < key) continue;
        }
        list[atomicAdd(count, 1)] = key;
    }
}

unsigned blocks_for(long long n, int threads = 256) {
    long long b = (n + threads - 1) / threads;
    if (b < 1) b = 1;
    if (b > 65535) b = 65535;
    return (unsigned)b;
}

}  // namespace

void launch_surr_key_geometry(const KeySpace& ks, const SurrGrid& g, float far_widths, float* kg, cudaStream_t s,
                              long long* l) {
    surr_key_geometry_kernel<<<blocks_for(ks.nkeys), 256, 0, s>>>(ks, g, far_widths, kg);
    OPSEC_CUDA(cudaGetLastError());
    ++*l;
}

void launch_surr_far_list(const KeySpace& ks, const float* kg, long long* list, int* count, cudaStream_t s,
                          long long* l) {
    surr_far_list_kernel<<<blocks_for(ks.nkeys), 256, 0, s>>>(ks, kg, list, count);
    OPSEC_CUDA(cudaGetLastError());
    ++*l;
}

void launch_surr_samples(long long nsamp, const long long* keys, int ntab, const float* kg, const float4* tinfo,
                         const XiLayout& xl, const double* xi64, const double* env, const double* Q, long long nkeys,
                         float* feat, float* y, cudaStream_t s, long long* l) {
    surr_samples_kernel<<<blocks_for(nsamp), 256, 0, s>>>(nsamp, keys, ntab, kg, tinfo, xl, xi64, env, Q, nkeys, feat,
                                                          y);
    OPSEC_CUDA(cudaGetLastError());
    ++*l;
}

void launch_surr_infer(long long nsamp, const long long* keys, int ntab, const float* kg, const float4* tinfo,
                       const float* feat, const float* w, float* out, cudaStream_t s, long long* l) {
    int dev = 0, nsm = 0;
    OPSEC_CUDA(cudaGetDevice(&dev));
    OPSEC_CUDA(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
    const long long tiles = (nsamp + 15) / 16;
    long long grid = std::min<long long>((tiles + 7) / 8, (long long)nsm * 4);
    if (grid < 1) grid = 1;
    const size_t smem = sizeof(__nv_bfloat16) * kSurrHid * (kW1S + 2 * kW23S) + sizeof(float) * (4 * kSurrHid + 1);
    OPSEC_CUDA(cudaFuncSetAttribute(surr_infer_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, max_dynamic_smem((const void*)surr_infer_kernel)));
    surr_infer_kernel<<<(unsigned)grid, 256, smem, s>>>(nsamp, keys, ntab, kg, tinfo, feat, w, out);
    OPSEC_CUDA(cudaGetLastError());
    ++*l;
}

void launch_surr_combine(long long nlist, const long long* keys, int ntab, int nmem, const float* pred,
                         const float* kg, const XiLayout& xl, const double* xi64, const double* env, float ysc,
                         float tol, long long nkeys, double* Q, unsigned char* done, int* counts, cudaStream_t s,
                         long long* l) {
    surr_combine_kernel<<<blocks_for(nlist), 256, 0, s>>>(nlist, keys, ntab, nmem, pred, kg, xl, xi64, env, ysc, tol,
                                                         nkeys, Q, done, counts);
    OPSEC_CUDA(cudaGetLastError());
    ++*l;
}

// One forward (+ backward when y != null) pass over a batch of Bn samples (x [Bn][16]) with
// the BF16-valued weights wb; gradients into grad [kSurrParams]; loss added to *loss.
// Scratch: 7 Bn 128 floats.
void surr_forward_backward(int Bn, const float* x, const float* y, const float* wb, float* grad, double* loss,
                           float* out, float* scratch, cudaStream_t s, long long* l) {
    const int H = kSurrHid;
    float* z1 = scratch;
    float* a1 = z1 + (size_t)Bn * H;
    float* z2 = a1 + (size_t)Bn * H;
    float* a2 = z2 + (size_t)Bn * H;
    float* z3 = a2 + (size_t)Bn * H;
    float* a3 = z3 + (size_t)Bn * H;
    float* dz = a3 + (size_t)Bn * H;
    const dim3 blk(256);
    auto grid = [&](int M, int N) { return dim3((N + kTN - 1) / kTN, (M + kTM - 1) / kTM); };
    // weight gradients sum over the batch: split it over 256-row slices, added atomically
    const int ks = std::max(1, std::min(32, Bn / 256));
    auto gridk = [&](int M, int N) { return dim3((N + kTN - 1) / kTN, (M + kTM - 1) / kTM, ks); };
    // forward: Z = X W^T + b, A = gelu(Z) (a1, a2 BF16-valued; a3 FP32 into the output layer)
    surr_gemm_kernel<<<grid(Bn, H), blk, 0, s>>>(Bn, H, kSurrIn, x, kSurrIn, 1, wb + kSurrOffW1, 1, kSurrIn, z1, H, 1,
                                                 wb + kSurrOffB1, a1, 1, nullptr);
    surr_gemm_kernel<<<grid(Bn, H), blk, 0, s>>>(Bn, H, H, a1, H, 1, wb + kSurrOffW2, 1, H, z2, H, 1,
                                                 wb + kSurrOffB2, a2, 1, nullptr);
    surr_gemm_kernel<<<grid(Bn, H), blk, 0, s>>>(Bn, H, H, a2, H, 1, wb + kSurrOffW3, 1, H, z3, H, 1,
                                                 wb + kSurrOffB3, a3, 0, nullptr);
    *l += 3;
    if (!y) {
        surr_out_kernel<<<(Bn + 7) / 8, dim3(32, 8), 0, s>>>(Bn, a3, z3, wb, nullptr, out, nullptr, nullptr);
        OPSEC_CUDA(cudaGetLastError());
        ++*l;
        return;
    }
    OPSEC_CUDA(cudaMemsetAsync(grad, 0, sizeof(float) * kSurrParams, s));
    surr_out_kernel<<<(Bn + 7) / 8, dim3(32, 8), 0, s>>>(Bn, a3, z3, wb, y, out, dz, loss);
    surr_outgrad_kernel<<<1, kSurrHid + 32, 0, s>>>(Bn, a3, out, y, grad);
    // layer 3: dW3 = dZ3^T A2, db3, dZ2 = (dZ3 W3) * gelu'(Z2) (into a3)
    surr_gemm_kernel<<<gridk(H, H), blk, 0, s>>>(H, H, Bn, dz, 1, H, a2, H, 1, grad + kSurrOffW3, H, 0, nullptr,
                                                nullptr, 0, nullptr);
    surr_colsum_kernel<<<1, H, 0, s>>>(Bn, H, dz, grad + kSurrOffB3);
    surr_gemm_kernel<<<grid(Bn, H), blk, 0, s>>>(Bn, H, H, dz, H, 1, wb + kSurrOffW3, H, 1, a3, H, 2, nullptr,
                                                 nullptr, 0, z2);
    // layer 2: dW2 = dZ2^T A1, db2, dZ1 = (dZ2 W2) * gelu'(Z1) (into dz)
    surr_gemm_kernel<<<gridk(H, H), blk, 0, s>>>(H, H, Bn, a3, 1, H, a1, H, 1, grad + kSurrOffW2, H, 0, nullptr,
                                                nullptr, 0, nullptr);
    surr_colsum_kernel<<<1, H, 0, s>>>(Bn, H, a3, grad + kSurrOffB2);
    surr_gemm_kernel<<<grid(Bn, H), blk, 0, s>>>(Bn, H, H, a3, H, 1, wb + kSurrOffW2, H, 1, dz, H, 2, nullptr,
                                                 nullptr, 0, z1);
    // layer 1: dW1 = dZ1^T X, db1
    surr_gemm_kernel<<<gridk(H, kSurrIn), blk, 0, s>>>(H, kSurrIn, Bn, dz, 1, H, x, kSurrIn, 1, grad + kSurrOffW1,
                                                      kSurrIn, 0, nullptr, nullptr, 0, nullptr);
    surr_colsum_kernel<<<1, H, 0, s>>>(Bn, H, dz, grad + kSurrOffB1);
    OPSEC_CUDA(cudaGetLastError());
    *l += 10;
}

void launch_surr_gather(int Bn, long long S, long long off, long long stride, const float* feat, const float* y,
                        float* xb, float* yb, cudaStream_t s, long long* l) {
    surr_gather_kernel<<<(Bn + 255) / 256, 256, 0, s>>>(Bn, S, off, stride, feat, y, xb, yb);
    OPSEC_CUDA(cudaGetLastError());
    ++*l;
}

void launch_surr_adam(float* w, float* wb, const float* g, float* m, float* v, float lr, int step, cudaStream_t s,
                      long long* l) {
    const float b1t = powf(0.9f, (float)step), b2t = powf(0.999f, (float)step);
    surr_adam_kernel<<<(kSurrParams + 255) / 256, 256, 0, s>>>(kSurrParams, w, wb, g, m, v, lr, b1t, b2t);
    OPSEC_CUDA(cudaGetLastError());
    ++*l;
}

}  // namespace opsec
