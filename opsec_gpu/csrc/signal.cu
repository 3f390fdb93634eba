// signal.cu -- signal-matrix assembly from the Q tables, the azimuthal block
// decomposition of full-sky spherical surveys, and the small FP64 helpers
// around them (mode scaling, pixel projection).
#include <cmath>

#include <type_traits>

#include "engine.h"

namespace opsec {
namespace {

__device__ __forceinline__ long long tri_index(int ha, int hb, int H) {
    return (long long)ha * H - (long long)ha * (ha - 1) / 2 + (hb - ha);
}

// Compact key of a cell pair (sig.cpp:99-119 Cartesian, :150-207 spherical).
__device__ __forceinline__ long long pair_key(const KeySpace& ks, int a1, int a2, int a3, int b1, int b2, int b3) {
    if (ks.coordsys == 1) {
        int kx = abs(a1 - b1), ky = abs(a2 - b2), kz = abs(a3 - b3);
        return ((long long)kx * ks.N2 + ky) * ks.N3 + kz;
    }
    int h1 = a1 * ks.N2 + a2, h2 = b1 * ks.N2 + b2;
    int ha = min(h1, h2), hb = max(h1, h2);
    int df = abs(a3 - b3);
    if (ks.fold && df > ks.N3 - df) df = ks.N3 - df;
    return tri_index(ha, hb, ks.H) * ks.nf + df;
}

__global__ void expand_q_kernel(KeySpace ks, int ntab, const double* Q, float* Qsq) {
    const long long total = (long long)ntab * ks.nsquare;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total;
         e += (long long)gridDim.x * blockDim.x) {
        const int t = (int)(e / ks.nsquare);
        const long long s = e % ks.nsquare;
        long long key;
        if (ks.coordsys == 1) {
            key = s;
        } else {
            const int df = (int)(s % ks.nf);
            const long long hh = s / ks.nf;
            const int h1 = (int)(hh / ks.H), h2 = (int)(hh % ks.H);
            key = tri_index(min(h1, h2), max(h1, h2), ks.H) * ks.nf + df;
        }
        Qsq[e] = (float)Q[(size_t)t * ks.nkeys + key];
    }
}

__global__ void signal_block_kernel(KeySpace ks, CellKeyInfo ci, const double* Qtab, int nrows, const int* rows,
                                    int ncols, const int* cols, double* s, int lld) {
    const long long total = (long long)nrows * ncols;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total;
         e += (long long)gridDim.x * blockDim.x) {
        const int i = (int)(e / ncols), j = (int)(e % ncols);
        const int a = rows[i], b = cols[j];
        const long long key = pair_key(ks, ci.d1[a], ci.d2[a], ci.d3[a], ci.d1[b], ci.d2[b], ci.d3[b]);
        s[(size_t)i * lld + j] = sqrt(ci.nbar[a] * ci.nbar[b]) * Qtab[key];  // sig.cpp:120,203
    }
}

// Azimuthal blocks of a full-sky S (or S_p): S(m)[h][h'] = D_h D_h' sum_d Q(h,h',|d|) cos(2 pi m d/Nphi).
// Folded form: sum over df = 0..Nphi/2 with weight 1 at df = 0 and df = Nphi/2, 2 between
// (cos(2 pi m (Nphi - df)/Nphi) = cos(2 pi m df/Nphi)); the weighted cosines sit in shared
// memory, computed with the angle reduced exactly on the integer lattice.
//
// npar = 2 (mu grid symmetric about 0, N_mu even, Nbar symmetric): the reflection
// P(i, j) = (i, N_mu-1-j) commutes with S(m), which splits into an even and an odd block
// over the half grid x = (i, j < N_mu/2):  S_+-(m)[x][y] = S(m)[h_x][h_y] +- S(m)[h_x][P h_y].
// Output block b = m npar + parity, Hb = H / npar, column-major [b][y][x].
template <typename T>
__global__ void azimuthal_blocks_kernel(KeySpace ks, const double* Q, const double* nbar_arc, int nm, int npar, T* Sm) {
    extern __shared__ double cw[];  // [nm][nf]
    const int H = ks.H, Nphi = ks.N3, nf = ks.nf, Nmu = ks.N2;
    for (int t = threadIdx.x; t < nm * nf; t += blockDim.x) {
        const int m = t / nf, df = t % nf;
        const int md = (int)(((long long)m * df) % Nphi);
        const double w = (df == 0 || 2 * df == Nphi) ? 1.0 : 2.0;
        cw[t] = w * cospi(2.0 * md / Nphi);
    }
    __syncthreads();
    const int Hb = H / npar, half = Nmu / npar;
    const long long HH = (long long)Hb * Hb;
    for (long long r = blockIdx.x * (long long)blockDim.x + threadIdx.x; r < HH; r += (long long)gridDim.x * blockDim.x) {
        const int y = (int)(r / Hb), x = (int)(r % Hb);
        const int ha = (x / half) * Nmu + x % half, hb = (y / half) * Nmu + y % half;
        const double* q1 = Q + tri_index(min(ha, hb), max(ha, hb), H) * nf;
        const int pb = (hb / Nmu) * Nmu + (Nmu - 1 - hb % Nmu);
        const double* q2 = Q + tri_index(min(ha, pb), max(ha, pb), H) * nf;
        const double d = sqrt(nbar_arc[ha] * nbar_arc[hb]);
        for (int m = blockIdx.y; m < nm; m += gridDim.y) {
            const double* c = cw + m * nf;
            double a1 = 0.0;
            for (int df = 0; df < nf; df++) a1 = fma(q1[df], c[df], a1);
            if (npar == 1) {
                Sm[(size_t)m * HH + r] = (T)(d * a1);
            } else {
                double a2 = 0.0;
                for (int df = 0; df < nf; df++) a2 = fma(q2[df], c[df], a2);
                Sm[(size_t)(2 * m) * HH + r] = (T)(d * (a1 + a2));
                Sm[(size_t)(2 * m + 1) * HH + r] = (T)(d * (a1 - a2));
            }
        }
    }
}

// Ucat[col][h] = U_m[h][idx] for the listed (m, idx) columns: the block
// eigenvectors the selected modes are built from, one copy per (m, idx).
template <typename T>
__global__ void gather_block_vectors_kernel(int H, int ncol, const int* col_m, const int* col_idx, const double* U,
                                            T* Ucat) {
    const long long total = (long long)ncol * H;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total;
         e += (long long)gridDim.x * blockDim.x) {
        const int c = (int)(e / H), h = (int)(e % H);
        Ucat[e] = (T)U[(size_t)col_m[c] * H * H + (size_t)col_idx[c] * H + h];
    }
}

// Packed C_p from the per-block products: modes i <= j of the same azimuthal
// order and the same trig class (cos-type or sin-type) take C_m[col_i][col_j];
// every other pair is zero by the orthogonality of the azimuthal factors.
// blockIdx.z = band, blockIdx.y strides over j, threads over i <= j.
template <typename T>
__global__ void azimuthal_scatter_kernel(int M, const int* mode_m, const int* mode_cls, const int* mode_col,
                                         const long long* blk_off, const int* blk_K, long long csize, const T* C,
                                         float* Dp) {
    const int p = blockIdx.z;
    const size_t K = (size_t)M * (M + 1) / 2;
    const T* Cp = C + (size_t)p * csize;
    float* out = Dp + (size_t)p * K;
    for (int j = blockIdx.y; j < M; j += gridDim.y) {
        const int mj = mode_m[j], cj = mode_cls[j], colj = mode_col[j];
        const T* Cj = Cp + blk_off[mj] + (size_t)colj * blk_K[mj];
        const size_t row = (size_t)j * (j + 1) / 2;
        for (int i = blockIdx.x * blockDim.x + threadIdx.x; i <= j; i += gridDim.x * blockDim.x) {
            float v = 0.f;
            if (mode_m[i] == mj && mode_cls[i] == cj) v = (float)Cj[mode_col[i]];
            out[row + i] = v;
        }
    }
}

// Weighted galaxy counts per cell (dot.cpp:105-130): each galaxy (x1, x2, x3, w) in the
// survey's coordinates goes to the grid cell of Survey::GetGridIndex (Survey.cpp:93-101,
// floor per axis in FP64), then through the map grid index -> cell.  Galaxies outside the
// grid or in a grid cell without a cell are summed into counts[ncells].  The reference
// sends the galaxies of grid index 0 there too (`e > 0`, dot.cpp:127) and indexes the
// counts with -1 for a galaxy in an empty cell; both are not reproduced.  FP64 atomics:
// integer weights sum exactly, others to the order of the additions.
__global__ void galaxy_counts_kernel(long long ngal, const float4* gal, GridBox g, const int* cellmap, int ncells,
                                     double* counts) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < ngal; i += (long long)gridDim.x * blockDim.x) {
        const float4 v = gal[i];
        // range tests on the FP64 floor before any conversion: NaN and far-away coordinates fail them
        const double t1 = floor(g.n[0] * ((double)v.x - g.lo[0]) / (g.hi[0] - g.lo[0]));
        const double t2 = floor(g.n[1] * ((double)v.y - g.lo[1]) / (g.hi[1] - g.lo[1]));
        const double t3 = floor(g.n[2] * ((double)v.z - g.lo[2]) / (g.hi[2] - g.lo[2]));
        int a = ncells;
        if (t1 >= 0.0 && t1 < g.n[0] && t2 >= 0.0 && t2 < g.n[1] && t3 >= 0.0 && t3 < g.n[2]) {
            const int m = cellmap[((long long)t1 * g.n[1] + (long long)t2) * g.n[2] + (long long)t3];
            if (m >= 0) a = m;
        }
        atomicAdd(&counts[a], (double)v.w);
    }
}

// modes[i][h*Nphi + f] = u_i(h) * trig_kind(m f), u_i the block eigenvector idx of block b = m npar + parity
// expanded to the full arc grid: u(h_x) = U_b[x][idx] / sqrt(npar), u(P h_x) = +-u(h_x) (even / odd)
__global__ void assemble_modes_kernel(int H, int Nphi, int Nmu, int npar, int nmodes, const int* sel_b,
                                      const int* sel_idx, const int* sel_kind, const double* U, double* modes) {
    extern __shared__ double trig[];  // cos, sin of 2 pi j / Nphi, j < Nphi
    for (int j = threadIdx.x; j < Nphi; j += blockDim.x) {
        trig[2 * j] = cospi(2.0 * j / Nphi);
        trig[2 * j + 1] = sinpi(2.0 * j / Nphi);
    }
    __syncthreads();
    const long long N = (long long)H * Nphi;
    const long long total = (long long)nmodes * N;
    const int Hb = H / npar, half = Nmu / npar;
    const double c0 = 1.0 / sqrt((double)Nphi), c1 = sqrt(2.0 / Nphi), cp = npar == 2 ? sqrt(0.5) : 1.0;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total;
         e += (long long)gridDim.x * blockDim.x) {
        const int i = (int)(e / N);
        const long long a = e % N;
        const int h = (int)(a / Nphi), f = (int)(a % Nphi);
        const int b = sel_b[i], m = b / npar;
        int j = h % Nmu;
        double sgn = cp;
        if (j >= half) {  // reflected half (npar = 2 only)
            j = Nmu - 1 - j;
            if (b % 2 == 1) sgn = -cp;
        }
        const int x = (h / Nmu) * half + j;
        const double u = sgn * U[(size_t)b * Hb * Hb + (size_t)sel_idx[i] * Hb + x];
        const int mf = (int)(((long long)m * f) % Nphi);
        double t;
        switch (sel_kind[i]) {
        case 0: t = c0; break;
        case 1: t = c1 * trig[2 * mf]; break;
        case 2: t = c1 * trig[2 * mf + 1]; break;
        default: t = (f & 1) ? -c0 : c0; break;
        }
        modes[e] = u * t;
    }
}

__global__ void scale_modes_kernel(int ncells, int nmodes, const double* modes, const double* nbar, double* Bs) {
    const long long total = (long long)ncells * nmodes;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total;
         e += (long long)gridDim.x * blockDim.x) {
        Bs[e] = sqrt(nbar[e % ncells]) * modes[e];
    }
}

// one warp per mode: y_i = sum_a B_ia (N_a - Nbar_a)/sqrt(Nbar_a)  (dot.cpp:131-152)
// x_a = (N_a - Nbar_a) / sqrt(Nbar_a), in place of the counts (dot.cpp:120-152)
__global__ void pixel_values_kernel(int ncells, double* counts, const double* nbar) {
    for (int a = blockIdx.x * blockDim.x + threadIdx.x; a < ncells; a += gridDim.x * blockDim.x)
        counts[a] = (counts[a] - nbar[a]) / sqrt(nbar[a]);
}

__global__ void dot_kernel(int ncells, int nmodes, const double* modes, const double* x, double* y) {
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    if (warp >= nmodes) return;
    const double* b = modes + (size_t)warp * ncells;
    double acc = 0.0;
    for (int a = lane; a < ncells; a += 32) acc = fma(b[a], x[a], acc);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if (lane == 0) y[warp] = acc;
}

// Pixel values on the azimuthal modes without forming them (dot.cpp:120-152 on the modes that
// assemble_modes_kernel would write): a mode is u_b[x] (the block eigenvector, + or - on the
// mu-reflected arcs) times cos or sin of order m over phi, so y_i = sum_h u(i, h) X(h, kind, m)
// with X the per-arc trig sums of the pixel values x = (N - Nbar)/sqrt(Nbar).
// Grid: one thread per (arc, order); X[h][m] = (cos sum, sin sum) with the modes' scales.
__global__ void arc_trig_sums_kernel(int H, int Nphi, const double* counts, const double* nbar, double2* X) {
    const int nm = Nphi / 2 + 1;
    const double c0 = 1.0 / sqrt((double)Nphi), c1 = sqrt(2.0 / Nphi);
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < H * nm; e += gridDim.x * blockDim.x) {
        const int h = e / nm, m = e % nm;
        double sc = 0.0, ss = 0.0;
        for (int f = 0; f < Nphi; f++) {
            const int a = h * Nphi + f;
            const double x = (counts[a] - nbar[a]) / sqrt(nbar[a]);
            const int mf = (int)(((long long)m * f) % Nphi);
            sc = fma(x, cospi(2.0 * mf / Nphi), sc);
            ss = fma(x, sinpi(2.0 * mf / Nphi), ss);
        }
        const bool edge = m == 0 || 2 * m == Nphi;
        X[e] = make_double2(sc * (edge ? c0 : c1), ss * c1);
    }
}

// One warp per mode: y_i = sum over the block's arcs x of u_b[x] (X(h1) +/- X(h2)) / sqrt 2 with
// h1, h2 the arc and its mu reflection (npar = 2), or sum_h u_b[h] X(h) (npar = 1).
__global__ void azimuthal_dot_kernel(int H, int Nphi, int Nmu, int npar, int nmodes, const int* sel_b,
                                     const int* sel_idx, const int* sel_kind, const double* U, const double2* X,
                                     double* y) {
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    if (warp >= nmodes) return;
    const int nm = Nphi / 2 + 1, Hb = H / npar, half = Nmu / npar;
    const int b = sel_b[warp], m = b / npar, kind = sel_kind[warp];
    const double* u = U + (size_t)b * Hb * Hb + (size_t)sel_idx[warp] * Hb;
    const double cp = npar == 2 ? sqrt(0.5) : 1.0, sg = (npar == 2 && (b & 1)) ? -1.0 : 1.0;
    double acc = 0.0;
    for (int x = lane; x < Hb; x += 32) {
        const int hr = x / half, j = x % half;
        const int h1 = hr * Nmu + j;
        const double2 a1 = X[(size_t)h1 * nm + m];
        double v = kind == 2 ? a1.y : a1.x;  // kinds 0, 1, 3 use the cos sum (order 0 and Nphi/2 included)
        if (npar == 2) {
            const double2 a2 = X[(size_t)(hr * Nmu + (Nmu - 1 - j)) * nm + m];
            v += sg * (kind == 2 ? a2.y : a2.x);
        }
        acc = fma(u[x] * cp, v, acc);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if (lane == 0) y[warp] = acc;
}

// modes[i][a] = A[(M-1-i)*lda + a], evals[i] = w[M-1-i]: syevdx returns ascending order
__global__ void reverse_modes_kernel(int n, int m, int lda, const double* A, const double* w, double* modes,
                                     double* evals) {
    const long long total = (long long)n * m;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total;
         e += (long long)gridDim.x * blockDim.x) {
        const int i = (int)(e / n), a = (int)(e % n);
        modes[e] = A[(size_t)(m - 1 - i) * lda + a];
        if (a == 0) evals[i] = w[m - 1 - i];
    }
}

__global__ void widen_kernel(size_t n, const float* in, double* out) {
    for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < n; e += (size_t)gridDim.x * blockDim.x)
        out[e] = (double)in[e];
}

unsigned grid_for(long long n, int threads = 256) {
    long long g = (n + threads - 1) / threads;
    if (g > 152LL * 64) g = 152LL * 64;
    if (g < 1) g = 1;
    return (unsigned)g;
}

}  // namespace

void launch_expand_q(const KeySpace& ks, int ntab, const double* Q, float* Qsq, cudaStream_t s, long long* l) {
    expand_q_kernel<<<grid_for((long long)ntab * ks.nsquare), 256, 0, s>>>(ks, ntab, Q, Qsq);
    OPSEC_CUDA(cudaGetLastError());
    ++*l;
}

void launch_signal_block(const KeySpace& ks, const CellKeyInfo& ci, const double* Qtab, int nrows, const int* rows,
                         int ncols, const int* cols, double* s, int lld, cudaStream_t st, long long* l) {
    signal_block_kernel<<<grid_for((long long)nrows * ncols), 256, 0, st>>>(ks, ci, Qtab, nrows, rows, ncols, cols,
                                                                           s, lld);
    OPSEC_CUDA(cudaGetLastError());
    ++*l;
}

// FP32 blocks for the band projection: the same transform with the 17 (for
// N_phi = 32) products per output in FP32 (the blocks are rounded to FP32
// anyway and feed FP32 GEMMs), each thread holding its two key rows in
// registers and producing every azimuthal order, so FP64 work (slow on this
// part) is only the conversion of the loaded Q values.
template <int NFM>
__global__ void azimuthal_blocks_f32_kernel(KeySpace ks, const double* Q, const double* nbar_arc, int nm, int npar,
                                            float* Sm) {
    extern __shared__ float cwf[];  // [nm][NFM], zero past nf
    const int H = ks.H, Nphi = ks.N3, nf = ks.nf, Nmu = ks.N2;
    for (int t = threadIdx.x; t < nm * NFM; t += blockDim.x) {
        const int m = t / NFM, df = t % NFM;
        const int md = (int)(((long long)m * df) % Nphi);
        const double w = (df == 0 || 2 * df == Nphi) ? 1.0 : 2.0;
        cwf[t] = df < nf ? (float)(w * cospi(2.0 * md / Nphi)) : 0.f;
    }
    __syncthreads();
    const int Hb = H / npar, half = Nmu / npar;
    const long long HH = (long long)Hb * Hb;
    for (long long r = blockIdx.x * (long long)blockDim.x + threadIdx.x; r < HH; r += (long long)gridDim.x * blockDim.x) {
        const int y = (int)(r / Hb), x = (int)(r % Hb);
        const int ha = (x / half) * Nmu + x % half, hb = (y / half) * Nmu + y % half;
        const double* p1 = Q + tri_index(min(ha, hb), max(ha, hb), H) * nf;
        const int pb = (hb / Nmu) * Nmu + (Nmu - 1 - hb % Nmu);
        const double* p2 = Q + tri_index(min(ha, pb), max(ha, pb), H) * nf;
        float q1[NFM], q2[NFM];
#pragma unroll
        for (int df = 0; df < NFM; df++) {
            q1[df] = df < nf ? (float)p1[df] : 0.f;
            q2[df] = (npar == 2 && df < nf) ? (float)p2[df] : 0.f;
        }
        const float d = sqrtf((float)nbar_arc[ha]) * sqrtf((float)nbar_arc[hb]);
        for (int m = 0; m < nm; m++) {
            const float* c = cwf + m * NFM;
            float a1 = 0.f, a2 = 0.f;
#pragma unroll
            for (int df = 0; df < NFM; df++) {
                a1 = fmaf(q1[df], c[df], a1);
                a2 = fmaf(q2[df], c[df], a2);
            }
            if (npar == 1) {
                Sm[(size_t)m * HH + r] = d * a1;
            } else {
                Sm[(size_t)(2 * m) * HH + r] = d * (a1 + a2);
                Sm[(size_t)(2 * m + 1) * HH + r] = d * (a1 - a2);
            }
        }
    }
}

// The same FP32 blocks by tiles of 16 (x) x 32 (y) outputs with y >= x, written at [x][y] and,
// mirrored through shared memory, at [y][x] (the blocks are symmetric).  In such a tile every
// key row the block needs -- (h_x, h_y) and (h_x, P h_y) -- has its smaller arc first (the arcs
// of the x half grow with x; P h_y lies in the upper mu half of h_y's shell), so for each x the
// rows of consecutive y are runs of consecutive keys: the tile's rows are staged in shared memory
// by coalesced loads (in the per-thread kernel above, one thread in two read a row of its own,
// ~H keys from its neighbour's).
constexpr int kTX = 16, kTY = 32;

template <int NFM>
__global__ void __launch_bounds__(256) azimuthal_blocks_tiled_kernel(KeySpace ks, const double* Q,
                                                                     const double* nbar_arc, int nm, int npar,
                                                                     float* Sm) {
    // tile (blockIdx.x, blockIdx.y); tiles entirely below the diagonal have nothing to do
    const int x0 = blockIdx.x * kTX, y0 = blockIdx.y * kTY;
    if (y0 + kTY - 1 < x0) return;
    extern __shared__ __align__(16) float tsm[];
    float* cwf = tsm;                     // [nm][NFM]
    float* q1s = cwf + nm * NFM;          // [kTX][kTY][NFM]
    float* q2s = q1s + kTX * kTY * NFM;   // [kTX][kTY][NFM]
    float* st = q2s + kTX * kTY * NFM;    // [2][kTY][kTX + 1]: one order's mirrored outputs
    const int H = ks.H, Nphi = ks.N3, nf = ks.nf, Nmu = ks.N2;
    const int Hb = H / npar, half = Nmu / npar;
    const long long HH = (long long)Hb * Hb;
    for (int t = threadIdx.x; t < nm * NFM; t += blockDim.x) {
        const int m = t / NFM, df = t % NFM;
        const int md = (int)(((long long)m * df) % Nphi);
        const double w = (df == 0 || 2 * df == Nphi) ? 1.0 : 2.0;
        cwf[t] = df < nf ? (float)(w * cospi(2.0 * md / Nphi)) : 0.f;
    }
    auto arc = [&](int v) { return (v / half) * Nmu + v % half; };
    auto refl = [&](int h) { return (h / Nmu) * Nmu + (Nmu - 1 - h % Nmu); };
    // stage the tile's key rows (pairs outside the block or below the diagonal: zeros)
    for (int e = threadIdx.x; e < kTX * kTY * NFM; e += blockDim.x) {
        const int xi = e / (kTY * NFM), r = e % (kTY * NFM), yi = r / NFM, df = r % NFM;
        const int x = x0 + xi, y = y0 + yi;
        float v1 = 0.f, v2 = 0.f;
        if (x < Hb && y < Hb && y >= x && df < nf) {
            const int ha = arc(x), hb = arc(y);
            v1 = (float)Q[tri_index(min(ha, hb), max(ha, hb), H) * nf + df];
            if (npar == 2) {
                const int pb = refl(hb);
                v2 = (float)Q[tri_index(min(ha, pb), max(ha, pb), H) * nf + df];
            }
        }
        q1s[e] = v1;
        q2s[e] = v2;
    }
    __syncthreads();
    // two pairs per thread, y fastest: p = threadIdx.x + 256 k -> (xi, yi) = (p / kTY, p % kTY)
    float q1[2][NFM], q2[2][NFM], dd[2];
    int xs[2], ys[2];
#pragma unroll
    for (int k = 0; k < 2; k++) {
        const int p = threadIdx.x + 256 * k, xi = p / kTY, yi = p % kTY;
        xs[k] = x0 + xi;
        ys[k] = y0 + yi;
#pragma unroll
        for (int df = 0; df < NFM; df++) {
            q1[k][df] = q1s[p * NFM + df];
            q2[k][df] = q2s[p * NFM + df];
        }
        const bool ok = xs[k] < Hb && ys[k] < Hb && ys[k] >= xs[k];
        dd[k] = ok ? sqrtf((float)nbar_arc[arc(xs[k])]) * sqrtf((float)nbar_arc[arc(ys[k])]) : 0.f;
    }
    for (int m = 0; m < nm; m++) {
        const float* c = cwf + m * NFM;
        float o[2][2];
#pragma unroll
        for (int k = 0; k < 2; k++) {
            float a1 = 0.f, a2 = 0.f;
#pragma unroll
            for (int df = 0; df < NFM; df++) {
                a1 = fmaf(q1[k][df], c[df], a1);
                a2 = fmaf(q2[k][df], c[df], a2);
            }
            o[k][0] = npar == 1 ? dd[k] * a1 : dd[k] * (a1 + a2);
            o[k][1] = dd[k] * (a1 - a2);
            const bool ok = xs[k] < Hb && ys[k] < Hb && ys[k] >= xs[k];
            if (ok) {
                if (npar == 1) {
                    Sm[(size_t)m * HH + (size_t)xs[k] * Hb + ys[k]] = o[k][0];
                } else {
                    Sm[(size_t)(2 * m) * HH + (size_t)xs[k] * Hb + ys[k]] = o[k][0];
                    Sm[(size_t)(2 * m + 1) * HH + (size_t)xs[k] * Hb + ys[k]] = o[k][1];
                }
            }
            const int p = threadIdx.x + 256 * k, xi = p / kTY, yi = p % kTY;
            st[yi * (kTX + 1) + xi] = o[k][0];
            st[kTY * (kTX + 1) + yi * (kTX + 1) + xi] = o[k][1];
        }
        __syncthreads();
        // mirror: [y][x] for y > x, x fastest
#pragma unroll
        for (int k = 0; k < 2; k++) {
            const int p = threadIdx.x + 256 * k, yi = p / kTX, xi = p % kTX;
            const int x = x0 + xi, y = y0 + yi;
            if (x < Hb && y < Hb && y > x) {
                if (npar == 1) {
                    Sm[(size_t)m * HH + (size_t)y * Hb + x] = st[yi * (kTX + 1) + xi];
                } else {
                    Sm[(size_t)(2 * m) * HH + (size_t)y * Hb + x] = st[yi * (kTX + 1) + xi];
                    Sm[(size_t)(2 * m + 1) * HH + (size_t)y * Hb + x] = st[kTY * (kTX + 1) + yi * (kTX + 1) + xi];
                }
            }
        }
        __syncthreads();
    }
}

template <int NFM>
void launch_azimuthal_f32(const KeySpace& ks, const double* Q, const double* nbar_arc, int nm, int npar, float* Sm,
                          cudaStream_t st, bool tiled) {
    const int Hb = ks.H / npar;
    if (tiled) {
        const size_t smem = sizeof(float) * ((size_t)nm * NFM + 2 * (size_t)kTX * kTY * NFM + 2 * kTY * (kTX + 1));
        OPSEC_CUDA(cudaFuncSetAttribute(azimuthal_blocks_tiled_kernel<NFM>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                        (int)smem));
        const dim3 grid((unsigned)((Hb + kTX - 1) / kTX), (unsigned)((Hb + kTY - 1) / kTY));
        azimuthal_blocks_tiled_kernel<NFM><<<grid, 256, smem, st>>>(ks, Q, nbar_arc, nm, npar, Sm);
        return;
    }
    const size_t smem = sizeof(float) * (size_t)nm * NFM;
    OPSEC_CUDA(cudaFuncSetAttribute(azimuthal_blocks_f32_kernel<NFM>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    max_dynamic_smem((const void*)azimuthal_blocks_f32_kernel<NFM>)));
    const long long HH = (long long)Hb * Hb;
    long long gx = (HH + 255) / 256;
    if (gx > 65535) gx = 65535;
    azimuthal_blocks_f32_kernel<NFM><<<(unsigned)gx, 256, smem, st>>>(ks, Q, nbar_arc, nm, npar, Sm);
}

template <typename T>
void launch_azimuthal_blocks_t(const KeySpace& ks, const double* Q, const double* nbar_arc, int nm, int npar, T* Sm,
                               cudaStream_t st, long long* l, bool tiled = false) {
    if (npar != 1 && !(npar == 2 && ks.N2 % 2 == 0)) fail(OPSEC_ERR_ARG, "parity split needs an even mu grid");
    if (!ks.fold) fail(OPSEC_ERR_CONFIG, "azimuthal blocks need a full-sky grid");
    if constexpr (std::is_same<T, float>::value) {
        if (ks.nf <= 33) {
            if (ks.nf <= 9)
                launch_azimuthal_f32<9>(ks, Q, nbar_arc, nm, npar, Sm, st, tiled);
            else if (ks.nf <= 17)
                launch_azimuthal_f32<17>(ks, Q, nbar_arc, nm, npar, Sm, st, tiled);
            else
                launch_azimuthal_f32<33>(ks, Q, nbar_arc, nm, npar, Sm, st, tiled);
            OPSEC_CUDA(cudaGetLastError());
            ++*l;
            return;
        }
    }
    const size_t smem = sizeof(double) * (size_t)nm * ks.nf;
    if (smem > 200 * 1024) fail(OPSEC_ERR_CONFIG, "too many phi cells for the azimuthal block transform");
    OPSEC_CUDA(cudaFuncSetAttribute(azimuthal_blocks_kernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, max_dynamic_smem((const void*)azimuthal_blocks_kernel<T>)));
    const long long HH = (long long)(ks.H / npar) * (ks.H / npar);
    const int gy = nm < 8 ? nm : 8;
    long long gx = (HH + 255) / 256;
    if (gx > 4096) gx = 4096;
    azimuthal_blocks_kernel<T><<<dim3((unsigned)gx, gy), 256, smem, st>>>(ks, Q, nbar_arc, nm, npar, Sm);
    OPSEC_CUDA(cudaGetLastError());
    ++*l;
}

void launch_azimuthal_blocks(const KeySpace& ks, const double* Q, const double* nbar_arc, int nm, int npar, double* Sm,
                             cudaStream_t st, long long* l) {
    launch_azimuthal_blocks_t(ks, Q, nbar_arc, nm, npar, Sm, st, l);
}

void launch_azimuthal_blocks(const KeySpace& ks, const double* Q, const double* nbar_arc, int nm, int npar, float* Sm,
                             cudaStream_t st, long long* l, bool tiled) {
    launch_azimuthal_blocks_t(ks, Q, nbar_arc, nm, npar, Sm, st, l, tiled);
}

template <typename T>
void launch_gather_t(int H, int ncol, const int* col_m, const int* col_idx, const double* U, T* Ucat, cudaStream_t st,
                     long long* l) {
    gather_block_vectors_kernel<T><<<grid_for((long long)ncol * H), 256, 0, st>>>(H, ncol, col_m, col_idx, U, Ucat);
    OPSEC_CUDA(cudaGetLastError());
    ++*l;
}

void launch_gather_block_vectors(int H, int ncol, const int* col_m, const int* col_idx, const double* U, double* Ucat,
                                 cudaStream_t st, long long* l) {
    launch_gather_t(H, ncol, col_m, col_idx, U, Ucat, st, l);
}

void launch_gather_block_vectors(int H, int ncol, const int* col_m, const int* col_idx, const double* U, float* Ucat,
                                 cudaStream_t st, long long* l) {
    launch_gather_t(H, ncol, col_m, col_idx, U, Ucat, st, l);
}

template <typename T>
void launch_scatter_t(int M, int nbands, const int* mode_m, const int* mode_cls, const int* mode_col,
                      const long long* blk_off, const int* blk_K, long long csize, const T* C, float* Dp,
                      cudaStream_t st, long long* l) {
    const int gy = M < 8192 ? M : 8192;
    const int gx = (M + 255) / 256 < 8 ? (M + 255) / 256 : 8;
    azimuthal_scatter_kernel<T><<<dim3(gx, gy, nbands), 256, 0, st>>>(M, mode_m, mode_cls, mode_col, blk_off, blk_K,
                                                                      csize, C, Dp);
    OPSEC_CUDA(cudaGetLastError());
    ++*l;
}

void launch_azimuthal_scatter(int M, int nbands, const int* mode_m, const int* mode_cls, const int* mode_col,
                              const long long* blk_off, const int* blk_K, long long csize, const double* C, float* Dp,
                              cudaStream_t st, long long* l) {
    launch_scatter_t(M, nbands, mode_m, mode_cls, mode_col, blk_off, blk_K, csize, C, Dp, st, l);
}

void launch_azimuthal_scatter(int M, int nbands, const int* mode_m, const int* mode_cls, const int* mode_col,
                              const long long* blk_off, const int* blk_K, long long csize, const float* C, float* Dp,
                              cudaStream_t st, long long* l) {
    launch_scatter_t(M, nbands, mode_m, mode_cls, mode_col, blk_off, blk_K, csize, C, Dp, st, l);
}

void launch_assemble_modes(int H, int Nphi, int Nmu, int npar, int nmodes, const int* sel_b, const int* sel_idx,
                           const int* sel_kind, const double* U, double* modes, cudaStream_t st, long long* l) {
    const size_t smem = sizeof(double) * 2 * Nphi;
    if (smem > 48 * 1024) fail(OPSEC_ERR_CONFIG, "too many phi cells for the mode assembly");
    assemble_modes_kernel<<<grid_for((long long)nmodes * H * Nphi), 256, smem, st>>>(H, Nphi, Nmu, npar, nmodes,
                                                                                    sel_b, sel_idx, sel_kind, U, modes);
    OPSEC_CUDA(cudaGetLastError());
    ++*l;
}

void launch_scale_modes(int ncells, int nmodes, const double* modes, const double* nbar, double* Bs, cudaStream_t s,
                        long long* l) {
    scale_modes_kernel<<<grid_for((long long)ncells * nmodes), 256, 0, s>>>(ncells, nmodes, modes, nbar, Bs);
    OPSEC_CUDA(cudaGetLastError());
    ++*l;
}

void launch_dot(int ncells, int nmodes, const double* modes, double* counts, const double* nbar, double* y,
                cudaStream_t s, long long* l) {
    pixel_values_kernel<<<grid_for(ncells), 256, 0, s>>>(ncells, counts, nbar);
    dot_kernel<<<(nmodes * 32 + 255) / 256, 256, 0, s>>>(ncells, nmodes, modes, counts, y);
    OPSEC_CUDA(cudaGetLastError());
    *l += 2;
}

void launch_dot_azimuthal(int H, int Nphi, int Nmu, int npar, int nmodes, const int* sel_b, const int* sel_idx,
                          const int* sel_kind, const double* U, const double* counts, const double* nbar, double* X,
                          double* y, cudaStream_t s, long long* l) {
    const int nm = Nphi / 2 + 1;
    double2* X2 = reinterpret_cast<double2*>(X);
    arc_trig_sums_kernel<<<grid_for((long long)H * nm), 256, 0, s>>>(H, Nphi, counts, nbar, X2);
    azimuthal_dot_kernel<<<(nmodes * 32 + 255) / 256, 256, 0, s>>>(H, Nphi, Nmu, npar, nmodes, sel_b, sel_idx,
                                                                     sel_kind, U, X2, y);
    OPSEC_CUDA(cudaGetLastError());
    *l += 2;
}

void launch_reverse_modes(int n, int m, int lda, const double* A, const double* w, double* modes, double* evals,
                          cudaStream_t s, long long* l) {
    reverse_modes_kernel<<<grid_for((long long)n * m), 256, 0, s>>>(n, m, lda, A, w, modes, evals);
    OPSEC_CUDA(cudaGetLastError());
    ++*l;
}

void launch_widen(size_t n, const float* in, double* out, cudaStream_t s, long long* l) {
    widen_kernel<<<grid_for((long long)n), 256, 0, s>>>(n, in, out);
    OPSEC_CUDA(cudaGetLastError());
    ++*l;
}

void launch_galaxy_counts(long long ngal, const float4* gal, const GridBox& g, const int* cellmap, int ncells,
                          double* counts, cudaStream_t st, long long* l) {
    OPSEC_CUDA(cudaMemsetAsync(counts, 0, sizeof(double) * (ncells + 1), st));
    if (ngal > 0) {
        galaxy_counts_kernel<<<grid_for(ngal), 256, 0, st>>>(ngal, gal, g, cellmap, ncells, counts);
        OPSEC_CUDA(cudaGetLastError());
        ++*l;
    }
}

}  // namespace opsec
