/* opsec_gpu.h -- C ABI of the GB300 Fisher-build engine.
 *
 * One context = one GPU (the current CUDA device at opsec_gpu_create), one
 * stream, device memory owned by the context.  Every entry point returns
 * OPSEC_OK (0) or a negative OPSEC_ERR_* code; opsec_gpu_last_error() gives
 * the message.  Calls are synchronous on return and not thread-safe on one
 * context.  All host arrays are owned by the caller; all outputs are double.
 *
 * Each entry point names the reference interface it replaces (paths inside
 * jwgcarlson/OPSEC, code/opsec/src/).
 */
#ifndef OPSEC_GPU_H
#define OPSEC_GPU_H

#ifdef __cplusplus
extern "C" {
#endif

#define OPSEC_OK 0
#define OPSEC_ERR_CONFIG (-1)  /* missing or invalid configuration option   */
#define OPSEC_ERR_ARG (-2)     /* invalid argument (size, pointer, index)    */
#define OPSEC_ERR_CUDA (-3)    /* CUDA runtime or library failure            */
#define OPSEC_ERR_NOMEM (-4)   /* device or host allocation failed           */
#define OPSEC_ERR_FILE (-5)    /* file missing, unreadable or malformed      */
#define OPSEC_ERR_NUMERIC (-6) /* non-finite input, eigensolver failure, singular Fisher matrix */
#define OPSEC_ERR_STATE (-7)   /* call made before its inputs exist          */

/* Mixing matrix choices of estimate-mpi.cpp:33-37. */
#define OPSEC_MIXING_INVERSE 0
#define OPSEC_MIXING_INVERSE_SQRT 1
#define OPSEC_MIXING_IDENTITY 2

/* A basis cell, byte-for-byte the reference's Cell ("4i8d", Cell.h:74-99). */
typedef struct opsec_cell {
    int a;          /* index within the list of cells   */
    int d1, d2, d3; /* grid index (x,y,z) or (r,mu,phi)  */
    double min1, max1, min2, max2, min3, max3;
    double Veff;
    double Nbar;
} opsec_cell;

typedef struct opsec_gpu opsec_gpu;

/* Parse key=value configuration text (the syntax of cfg.c:238-295; '#'
 * comments, optional quotes) and set up model and survey.  Replaces
 * opsec_init (opsec.c:19-56), InitializeModel (Model.cpp:26-51) and
 * InitializeSurvey (Survey.cpp:140-165).  Recognised keys: coordsys,
 * survey.type, survey.{XMin..ZMax,Nx,Ny,Nz,L} or survey.{RMin..PhiMax,
 * MuMuin,Nr,Nmu,Nphi}, model=RealModel, RealModel.pkfile,
 * RealModel.{Nbands,kmin,kmax} or RealModel.bands, Nmodes, mixing; and the
 * engine's own xi.{n1,n2,r1,r2} (xi-table layout, default 512,256,200,20000
 * as RealModel.cpp:99-102) and sig.gauss (Gauss points per cell axis, 1-6,
 * default 4). */
int opsec_gpu_create(opsec_gpu** ctx, const char* cfg_text);

/* Supply P(k) as arrays instead of RealModel.pkfile (RealModel.cpp:33-40:
 * CubicSpline(pkfile)). */
int opsec_gpu_set_pk(opsec_gpu* ctx, int n, const double* k, const double* P);

/* Model::NumParams and Model::GetParam for every band (RealModel.cpp:81-96). */
int opsec_gpu_num_params(opsec_gpu* ctx, int* nparams);
int opsec_gpu_get_params(opsec_gpu* ctx, double* params);

/* xi tables of RealModel::GetXi / GetXiDeriv (RealModel.cpp:98-127): row 0
 * is xi(r), row 1+p the derivative for band p, each xi_n1+xi_n2 values on the
 * r grid of QSpline::MakeArray (QSpline.cpp:6-17).  r_out (n) and xi_out
 * ((1+Nbands) x n) may be NULL. */
int opsec_gpu_xi_tables(opsec_gpu* ctx, int* n, double* r_out, double* xi_out);

/* Replace one xi table by caller values on the same r grid (n = xi.n1 +
 * xi.n2): the plug-in point of a custom correlation function, as an
 * XiFuncImpl subclass is in the reference (XiFunc.h:36-44).  table 0 is xi,
 * 1+p the derivative for band p.  Replaced tables persist until the next
 * opsec_gpu_set_pk. */
int opsec_gpu_set_xi_table(opsec_gpu* ctx, int table, int n, const double* values);

/* A block of the signal matrix, S_ab = sqrt(Nbar_a Nbar_b) Q_ab, written
 * row-major s[i*lld + j] for i < nrows, j < ncols (lld <= 0: lld = ncols).
 * table = 0 for xi (klt), 1+p for the derivative with respect to band p
 * (comma).  Replaces ComputeSignalMatrixBlock (sig.cpp:50-70). */
int opsec_gpu_signal_block(opsec_gpu* ctx, int ncells, const opsec_cell* cells, int nrows, const int* rows,
                           int ncols, const int* cols, double* s, int lld, int table);

/* Top-nmodes eigenpairs of the signal matrix, eigenvalues descending, modes
 * written mode-major (modes[i*ncells + a]).  *nconv = number of converged
 * modes.  Replaces klt's solve and write loop (klt.cpp:173-248). */
int opsec_gpu_klt(opsec_gpu* ctx, int ncells, const opsec_cell* cells, int nmodes, double* evals, double* modes,
                  int* nconv);

/* Packed derivative matrices C_p = B^T S_p B for every band, band after
 * band, each the upper triangle column by column (nmodes(nmodes+1)/2
 * values).  modes as written by opsec_gpu_klt.  Replaces the band loop of
 * comma (comma-scalapack.cpp:228-265). */
int opsec_gpu_comma(opsec_gpu* ctx, int ncells, const opsec_cell* cells, int nmodes, const double* modes,
                    double* cov_packed);

/* Pixel values y_i = sum_a B_ia (N_a - Nbar_a)/sqrt(Nbar_a) from weighted
 * counts per cell.  Replaces dot.cpp:131-152. */
int opsec_gpu_dot(opsec_gpu* ctx, int ncells, const opsec_cell* cells, const double* counts, int nmodes,
                  const double* modes, double* y);

/* Fisher matrix, bias, quadratic estimates and the estfile records of
 * estimate (estimate-mpi.cpp:480-641, one-rank semantics).  Outputs (any may
 * be NULL): phat (Nb), pcov, F, W, M (Nb x Nb, row-major), q (Nb; written as
 * q - f as the reference does), f (Nb). */
int opsec_gpu_estimate(opsec_gpu* ctx, int nmodes, const double* evals, const double* cov_packed, const double* y,
                       int mixing, double* phat, double* pcov, double* F, double* W, double* M, double* q,
                       double* f);

/* The whole path with every intermediate resident on the GPU: cells and
 * counts in, KL eigenvalues and estfile records out (klt -> comma -> dot ->
 * estimate).  evals (nmodes) and any output may be NULL. */
int opsec_gpu_fisher_build(opsec_gpu* ctx, int ncells, const opsec_cell* cells, const double* counts, int nmodes,
                           int mixing, double* evals, double* phat, double* pcov, double* F, double* W, double* M,
                           double* q, double* f);

/* Milliseconds spent in each stage of the last opsec_gpu_fisher_build
 * (CUDA events): xi tables, cubature, eigensolve, projection, Fisher.
 * times must hold 5 values. */
int opsec_gpu_stage_times(const opsec_gpu* ctx, double* times);

/* How the last eigensolve ran: stats[0] the solver (0 dense FP64 syevdx, 1 azimuthal
 * blocks, 2 Chebyshev-filtered subspace iteration -- klt.solver), then for the last:
 * [1] filter iterations, [2] final Chebyshev degree, [3] N x N x B GEMMs, [4] block
 * size B, [5] [6] the spectrum bounds used, [7] the largest relative residual
 * |S x - lambda x| / lambda of the returned modes (FP64), [8] FP64 Rayleigh-Ritz
 * rounds, [9] CG steps of the refinement.  stats must hold 10 values.  It replaces
 * ARPACK's iteration report (ParpackSolver.cpp:140-190). */
int opsec_gpu_eig_stats(const opsec_gpu* ctx, double* stats);

/* Per-kernel CUDA-event timing accumulated since creation when the
 * configuration sets profile = 1 (events on the launching stream around the
 * cubature, projection and Fisher kernels).  name: "cubature", "project_step1",
 * "project_step2", "fisher", and for the subspace-iteration eigensolver
 * "chfsi_filter", "chfsi_rayleigh_ritz", "chfsi_refine".  flops / bytes = algorithmic work attributed to
 * those launches.  No counterpart in the reference, which has no timers. */
int opsec_gpu_kernel_stats(const opsec_gpu* ctx, const char* name, long long* count, double* total_ms,
                           double* flops, double* bytes);

/* Number of kernels this context has launched since creation. */
long long opsec_gpu_launch_count(const opsec_gpu* ctx);

/* ---- learned far-field surrogate (no counterpart in the reference, whose
 * cell-pair integrals are all adaptive cubature).  A 4-member ensemble of MLPs
 * (12 geometry/band inputs -> 3 x 128 GELU -> 1, BF16 products, FP32
 * accumulation) predicts the integrals of key pairs at least `surrogate.far`
 * (default 2) cell widths apart on spherical grids; a key whose members
 * disagree by more than `surrogate.tol` (default 0.02, in units of the
 * table's largest magnitude within 25 % of the pair's centre separation)
 * and every nearer key are integrated by the cubature.  Enabled by
 * the configuration key `surrogate = 1` once weights are present. */

/* Train the ensemble on this context's own survey: every key integrated by
 * the cubature, then up to max_samples (far key, table) samples, 2% held out,
 * `epochs` passes of Adam.  stats (4, may be NULL): samples, validation rms of
 * the residual (units of the local table envelope), training seconds, output scale. */
int opsec_gpu_surrogate_train(opsec_gpu* ctx, long long max_samples, int epochs, unsigned seed, double* stats);
/* Floats in a weight buffer: 4 networks x 35336 FP32 parameters, then the output scale. */
int opsec_gpu_surrogate_size(void);
/* Copy the ensemble out (get = 1) or in (get = 0, e.g. weights trained on another survey). */
int opsec_gpu_surrogate_weights(opsec_gpu* ctx, float* buf, int get);
/* After a build with the surrogate: keys predicted, keys sent back to the cubature, far keys. */
int opsec_gpu_surrogate_stats(const opsec_gpu* ctx, long long* counts);
/* One network on explicit inputs (n x 16 floats, BF16-rounded on entry): out_tc from the
 * fused tensor-core inference kernel, out_simt from the training forward pass; with y
 * (n targets) also the mean squared error and its gradient (35336 floats). */
int opsec_gpu_surrogate_eval(opsec_gpu* ctx, const float* params, int n, const float* feats, const float* y,
                             float* out_tc, float* out_simt, double* loss, float* grad);

/* ---- batched mocks (no counterpart in the reference, which runs one survey per
 * program invocation).  One full-sky spherical survey per mock: the shell
 * r in [rmin, rmax] on an nr x nmu x nphi grid (mu in [-1, 1], phi in
 * [0, 2 pi)), its cells in grid order and its counts, built to nmodes modes. */
typedef struct {
    double rmin, rmax;
    int nr, nmu, nphi;
    int ncells; /* nr * nmu * nphi */
    const opsec_cell* cells;
    const double* counts;
    int nmodes;
} opsec_mock;

/* Fisher builds of many mocks with the bands, xi layout, Gauss rule and P(k) of
 * `ctx`: worker contexts (each with its own stream, solver handles and xi
 * tables, computed once) take mocks in turn from host threads, so that the
 * builds of small surveys overlap on the GPU.  workers = 1 runs them one after
 * the other; workers <= 0 autotunes the count on the first mocks (1, 2, 4, 8, 12
 * and 16 workers, two mocks each) and runs the rest with the fastest.  Outputs
 * per mock i (mixing = inverse): F + i nb^2, phat + i nb, pcov + i nb^2 (any may
 * be NULL).  stats (8, may be NULL): seconds, workers used, then the rate of
 * each candidate while autotuning, in mocks of the batch's mean cost per second
 * (a mock's cost taken as ncells^1.5: the largest mocks run first). */
int opsec_gpu_batch_fisher(opsec_gpu* ctx, int nmocks, const opsec_mock* mocks, int workers, double* F,
                           double* phat, double* pcov, double* stats);

/* Weighted galaxy counts per cell (dot.cpp:95-130): gals holds ngal records
 * (x1, x2, x3, w) as float32 -- the survey's galaxy file, ABN format "4f"
 * (Survey.h:14-19) -- in the survey's coordinates (x, y, z or r, mu, phi);
 * each goes to its grid cell (Survey::GetGridIndex, Survey.cpp:93-101).
 * counts[a] (ncells) receives the weight in cell a; *outside (may be NULL) the
 * weight of galaxies outside the grid or in grid cells without a listed cell.
 * Unlike the reference, galaxies in the cell at grid index 0 are counted there
 * (dot.cpp:127 tests e > 0). */
int opsec_gpu_count_galaxies(opsec_gpu* ctx, int ncells, const opsec_cell* cells, long long ngal, const float* gals,
                             double* counts, double* outside);

/* The cell builder (replaces basis.cpp:89-128, 160-201 with FinalizeCell's
 * adaptive cubature): every cell of the configured grid whose expected count
 * Nbar is positive, numbered in grid order (d1, d2, d3), with its bounds
 * (Survey::CreateEmptyCell, Survey.cpp:80-97), Veff and Nbar.  Cartesian
 * grids: the constant selection survey.nbar (BoxSurvey.cpp:61-75), Nbar =
 * nbar Veff.  Spherical grids: the radial linear spline of
 * opsec_gpu_set_radial times the HEALPix map of opsec_gpu_set_mask
 * (SphericalSurvey.cpp:51-80); the radial integral is exact (closed form per
 * spline segment), the map's by basis.samples^2 points per cell (default
 * 16^2).  The reference's spherical Nbar is 3x the expected count (it
 * integrates over r^3 without the 1/3); configuration basis.quirk3 = 1
 * reproduces that.  With capacity 0 only *ncells is set. */
int opsec_gpu_basis(opsec_gpu* ctx, int capacity, opsec_cell* cells, int* ncells);
/* The radial selection nbar(r) (the `radial` file of SphericalSurvey.cpp:126-131):
 * linear between the n points, zero outside [r_0, r_{n-1}). */
int opsec_gpu_set_radial(opsec_gpu* ctx, int n, const double* r, const double* nbar);
/* The angular completeness map (the FITS `maskfile` of SphericalSurvey.cpp:100-118,
 * as 12 nside^2 floats; nest = 1 for NESTED ordering, 0 for RING).  nside 0
 * removes it (completeness 1). */
int opsec_gpu_set_mask(opsec_gpu* ctx, long long nside, int nest, const float* mask);
/* HEALPix pixel of each (theta, phi) (chealpix.c ang2pix_ring / ang2pix_nest). */
int opsec_gpu_ang2pix(opsec_gpu* ctx, long long nside, int nest, int n, const double* theta, const double* phi,
                      long long* pix);

/* Mock counts for the context's P(k) (replaces the mock generator of
 * code/opsec/utils/gmock.cpp:1-40 and the counting of dot.cpp:123-129 for
 * Gaussian-random-field mocks): a Gaussian random field of P(k) on a periodic
 * ngrid^3 mesh enclosing the cell centres (side 1.25 x their span), sampled at
 * each centre's mesh point, then counts[a] ~ Poisson(Nbar_a max(0, 1 + bias
 * delta_a)).  Deterministic in seed (Philox4x64-10 streams; see the engine
 * sources).  delta (may be NULL) receives delta_a.  ngrid even, 4..1024. */
int opsec_gpu_mock_counts(opsec_gpu* ctx, int ncells, const opsec_cell* cells, int ngrid, unsigned long long seed,
                          double bias, double* counts, double* delta);

/* Failure handling.  The reference stops the whole job on any error (opsec_abort
 * and MPI_Abort, opsec.c:88-116); here every call returns a status and leaves the
 * context usable.  These two entry points exercise that without a GPU fault; they
 * have no counterpart in the reference.
 *
 * opsec_gpu_fail_alloc: host-side fault injection.  With after >= 0 the device
 * allocation after `after` more successful ones fails as if cudaMalloc had
 * (OPSEC_ERR_NOMEM, message "... injected ..."); the call that meets it returns
 * that status, forgets the context's cached device state, and the next call
 * rebuilds it.  after = -1 switches injection off.
 *
 * opsec_gpu_wait_probe: the bounded mbarrier wait of the tensor-core projection
 * kernels, run on a barrier that one thread completes after delay_cycles
 * (arrive = 1) or that nothing completes (arrive = 0).  *timed_out = 1 when the
 * wait gave up after limit_cycles; the kernel then returns normally (no copy is
 * in flight), so the context stays usable.  Cycles in [1, 4e9]. */
int opsec_gpu_fail_alloc(opsec_gpu* ctx, long long after);

/* The block product of the iterative eigensolver (klt.solver = chfsi): the product
 * of the signal matrix with a block of vectors that replaces the reference's one
 * matrix-vector product per ARPACK step (y = A x of the reverse-communication
 * loop, ParpackSolver.cpp:116-122), on the engine's tcgen05 kernel:
 *   C = alpha S X + beta C + gamma D
 * S: N x N symmetric (FP64, both triangles); X, C, D: N x ncols FP32, column-major
 * (leading dimension N); host buffers.  S and X are split into FP16 hi + lo after
 * a power-of-two scaling (~22 significant bits); the result is accurate to a few
 * 1e-7 of sum_k |S_ik X_kj|.  D may be null when gamma = 0; C is not read when
 * beta = 0.  The kernel's output tiles follow the configuration's klt.tile. */
int opsec_gpu_block_product(opsec_gpu* ctx, int N, int ncols, const double* S, const float* X, float alpha,
                            float beta, float* C, float gamma, const float* D);
int opsec_gpu_wait_probe(opsec_gpu* ctx, long long limit_cycles, int arrive, long long delay_cycles, int* timed_out);

/* Largest band count opsec_gpu_fisher_noalloc accepts. */
#define OPSEC_NOALLOC_MAX_BANDS 64

/* Fisher matrix, bias and quadratic estimates from device-resident inputs,
 * with no memory allocation -- for callers that cannot call cudaMalloc: code
 * whose device memory is all handed out by its own pool allocator, or a
 * latency-critical loop where an allocation or free could synchronize the
 * device.  No counterpart in the reference (its estimate allocates freely).
 *
 * All pointers are device memory owned by the caller: cov_packed = FP32
 * packed upper triangles, band after band (nbands x nmodes(nmodes+1)/2),
 * evals (nmodes), y (nmodes), prior band powers (nbands); out receives
 * F (nbands x nbands, row-major), then f (nbands), then q (nbands, the raw
 * quadratic estimate).  Kernels are queued on `stream` (a cudaStream_t, NULL
 * for the legacy stream) and the call returns without waiting.
 *
 * Scratch: one file-scope device array of 2.7 MB (152 x 2208 doubles) that
 * every GPU which loads this library holds until the process exits.  The
 * first call on a device, with that device current, looks up the array's
 * device address (first calls from several host threads at once are safe);
 * make that first call before any stream capture.  Every call shares the
 * array and overwrites all of it that it reads, so no clearing is needed --
 * but calls that overlap on the GPU (different streams, or different host
 * threads, running at once) race on it.  The result equals the allocating
 * path (opsec_gpu_estimate) within rounding, not bit for bit: the two sum
 * their per-CTA partials over different CTA counts.
 *
 * Returns OPSEC_ERR_ARG for nbands > OPSEC_NOALLOC_MAX_BANDS (64), non-positive
 * sizes or null pointers; OPSEC_ERR_CUDA, without launching, when a CUDA error
 * is already pending on the calling thread (it is left for its owner), and
 * when a launch fails. */
int opsec_gpu_fisher_noalloc(int nmodes, int nbands, const float* cov_packed, const double* evals, const double* y,
                             const double* prior, double* out, void* stream);

const char* opsec_gpu_last_error(const opsec_gpu* ctx);
void opsec_gpu_destroy(opsec_gpu* ctx);

#ifdef __cplusplus
}
#endif
#endif /* OPSEC_GPU_H */
