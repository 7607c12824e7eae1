/*
 * ffs_reml.h -- C ABI of the GB300 ARMA(1,1) REML voxelwise GLM library
 * (libffs_reml.so).
 *
 * Every entry point takes plain device pointers and sizes, launches on the
 * caller's CUDA stream (cudaStream_t passed as void*), allocates nothing and
 * never synchronises the device. Buffers are owned by the caller; their layouts
 * are stated below. Each call returns an ffs_status; on failure a message for
 * the calling thread is available from ffs_last_error().
 *
 * The reference is Python (fastfuncstuff/glm/arma.py, fastfuncstuff/glm/whiten.py);
 * each entry point names the reference function whose work it replaces. The
 * Python package fastfuncstuff_gb300 binds these through ctypes and exposes the
 * reference's own API (fit_glm_arma11, fit_glm_arma11_grouped, ...).
 *
 * Notation: V voxels, T retained time points, K design columns, P valid (a,b)
 * pairs, R runs. "time-major" = [T][V] (voxel index fastest), "voxel-major" =
 * [V][T]. Every K x T matrix (U, G, Q0, Xt) is stored with row stride
 * ld_t = T rounded up to a multiple of 4 (16-byte rows), the padding zero.
 */
#ifndef FFS_REML_H
#define FFS_REML_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
  FFS_OK = 0,
  FFS_ERR_INVALID = 1,     /* bad argument or shape (Python: ValueError)          */
  FFS_ERR_CUDA = 2,        /* CUDA runtime error                                  */
  FFS_ERR_UNSUPPORTED = 3, /* shape outside what the kernels were built for       */
  FFS_ERR_WORKSPACE = 4,   /* workspace smaller than required (Python: MemoryError)*/
  FFS_ERR_TIMEOUT = 5      /* a bounded device-side wait expired                  */
} ffs_status;

/* Library version, (major << 16) | minor. */
int ffs_version(void);

/* Static description of a status code. */
const char* ffs_status_string(int status);

/* Message of the last failing call on this thread ("" if none). */
const char* ffs_last_error(void);

/* ------------------------------------------------------------------------ grid
 * Replaces fastfuncstuff/glm/whiten.py:197-271 (arma11_whiteners) and
 * fastfuncstuff/glm/arma.py:1371-1531 (precompute_reml_grid), plus the
 * per-group GLS constants of fastfuncstuff/glm/arma.py:4853-4905.
 *
 * For each valid pair p (a_p, b_p) the ARMA(1,1) correlation of every run is
 * factorised exactly in FP64 through its AR-filtered tridiagonal form
 * (R = A^-1 L~ D L~^T A^-T, so the Cholesky factor is A^-1 L~ D^1/2), giving:
 *   coef[p][t]   = (c_t, m_t, 1/D_t, 1/sqrt(D_t)) as float4:
 *                  z_t = y_t - c_t y_{t-1};  v_t = z_t - m_t v_{t-1};
 *                  (L^-1 y)_t = v_t / sqrt(D_t);  y'R^-1 y = sum v_t^2 / D_t.
 *                  c_t = m_t = 0 at every run start.
 *   logdet_R[p]  = 2 sum_t log(sqrt(D_t) + 1e-10)          (FP64)
 *   logdet_XtX[p]= 2 sum_j log(|L_xtx,jj| + 1e-10)          (FP64)
 *   U[p]         = L^-T Q, Q = X_w L_xtx^-T, stored [P][K][ld_t] fp32:
 *                  ||Q' L^-1 y||^2 = ||U' y||^2 for any series y.
 *   U_hi/U_lo    = the same as an fp16 split of U * 2^uexp[p] (hi + lo carry
 *                  about 22 significant bits; the power of two puts each
 *                  pair's largest entry in [128, 256)), rows p*K+j of length
 *                  ld_u (>= T, multiple of 8, zero padded): the B operand of
 *                  the projection GEMM.
 *   pairs with lambda == 0 have R = I exactly; their coefficients are the
 *   identity (c = m = 0, D = 1), so ties between them stay exact ties.
 *   G[p]         = U L_xtx^-1 = R^-1 X (X'R^-1 X)^-1, [P][K][ld_t] fp32:
 *                  GLS betas b = G' y.
 *   Adiag[p][K]  = diag((X_w'X_w)^-1);  XtX[p][K][K] = X_w'X_w (fp32).
 *   Ftask[p]     = inv(A_task + 1e-8 I) for the task-column F statistic
 *                  (fastfuncstuff/glm/arma.py:4891-4898), A = (X_w'X_w)^-1.
 *   glt_var[p][c]= c A c' for each single-row GLT c (arma.py:5455-5466).
 *   Fsets[p]     = inv(A_SS + 1e-8 I) of every column set S (the column_sets
 *                  Wald F, arma.py:3542-3561), the sets' q_S x q_S blocks one
 *                  after another ([P][sum q_S^2]).
 *   info[p]      = 0 Cholesky of X_w'X_w, 1 QR fallback used (the design is
 *                  rank deficient at this pair), 2 a pivot of R's factor was
 *                  not positive.
 */
#define FFS_BAND_MAX_W 129 /* widest band row (128 off-diagonals) of the banded R */

typedef struct {
  int T, K, P, n_runs;
  const int* run_start; /* device [n_runs + 1], run_start[n_runs] == T           */
  const int* tau;       /* device [T], within-run time index (censoring gaps)    */
  const float* a;       /* device [P]                                            */
  const float* b;       /* device [P]                                            */
  const float* X;       /* device [T][K] row-major design                        */
  int lambda_fp32;      /* 1: lambda in float32 op order (float32 fits),
                           0: in float64 (use_double fits)                        */
  int ld_u;             /* row length of U_hi / U_lo (>= T, multiple of 8)       */
  int n_task;           /* task columns for the F statistic (0: full model)      */
  const int* task_idx;  /* device [n_task]                                       */
  int n_glt;            /* single-row GLT contrasts                              */
  const float* glt;     /* device [n_glt][K]                                     */
  int n_sets;           /* column sets for Fsets (0: none)                       */
  const int* set_ptr;   /* device [n_sets + 1]: set s is set_idx[set_ptr[s] ..]  */
  const int* set_idx;   /* device [set_ptr[n_sets]] column indices (< K)         */
  /* AFNI-faithful banded R (fastfuncstuff/glm/arma.py:95-109, :1075-1089):
   * with band, correlations at |tau_i - tau_j| > band[p] are zero and R is
   * factored as a band (band_L, band_coef below; coef is then the identity
   * and unused). band_w = max band[p] + 1 <= FFS_BAND_MAX_W; NULL band: the
   * exact ARMA(1,1) R. */
  int band_w;
  const int* band;      /* device [P] or NULL                                    */
} ffs_grid_desc;

typedef struct {
  float* coef;          /* [P][T][4]                                              */
  double* logdet_R;     /* [P]                                                    */
  double* logdet_XtX;   /* [P]                                                    */
  float* U;             /* [P][K][ld_t]                                           */
  uint16_t* U_hi;       /* [P*K][ld_u] fp16 bits (may be NULL)                    */
  uint16_t* U_lo;       /* [P*K][ld_u] fp16 bits (may be NULL)                    */
  int* uexp;            /* [P] power-of-two scale of U_hi/U_lo (with U_hi)        */
  float* G;             /* [P][K][ld_t]                                           */
  float* Adiag;         /* [P][K]                                                 */
  float* XtX;           /* [P][K][K]                                              */
  int* info;            /* [P]                                                    */
  float* Ftask;         /* [P][n_task][n_task] inv(A_task + 1e-8 I), or NULL      */
  float* glt_var;       /* [P][n_glt] c A c', or NULL                             */
  float* Gsum;          /* [P][K] G' 1: the betas of the constant series          */
  double* work;         /* scratch, ffs_grid_work_bytes() bytes                   */
  float* Fsets;         /* [P][sum q_S^2] (with n_sets), or NULL                  */
  float* Afull;         /* [P][K][K] (X_w'X_w)^-1 (fp32), or NULL                 */
  /* with d->band: the Cholesky factor of each run of the banded R, row t of
   * pair p at [p][t][0 .. band_w): band_L[.][t][j] = L(t, t - j) (FP64, j = 0
   * the diagonal, zero past the row's band), and band_coef[.][t][0] =
   * 1 / L(t, t), band_coef[.][t][j] = L(t, t - j) / L(t, t) (fp32): the
   * whitening w_t = y_t band_coef[t][0] - sum_j band_coef[t][j] w_{t-j}. */
  double* band_L;
  float* band_coef;
} ffs_grid_out;

size_t ffs_grid_work_bytes(int T, int K, int P);
int ffs_grid_build(const ffs_grid_desc* d, const ffs_grid_out* o, void* stream);

/* ffs_grid_build for n_designs designs of one shape at once (the per-group
 * designs of fastfuncstuff/glm/arma.py:2836-3183, which the reference fits one
 * group after another): d->X is [n_designs][T][K]. coef and logdet_R depend on
 * the pair only and keep their [P] layout; every other output is indexed by
 * pd = design * P + pair (U [n_designs * P][K][T], logdet_XtX [n_designs * P],
 * U_hi rows pd * K + j, ...). One launch walks the n_designs * P items with
 * at most max_ctas CTAs (0 or more than FFS_GRID_MAX_SLOTS: that limit) --
 * fewer CTAs leave SMs to kernels running beside the build on other streams;
 * work: ffs_grid_work_bytes_designs with the same max_ctas. With more than one
 * design a first launch factors R once per pair (it depends on the pair
 * only) and the items of every design read that factor; with the banded R
 * (d->band) that launch also writes band_L and band_coef ([P] layout). */
#define FFS_GRID_MAX_SLOTS 2048
size_t ffs_grid_work_bytes_designs(int T, int K, int P, int n_designs, int max_ctas);
int ffs_grid_build_designs(const ffs_grid_desc* d, int n_designs, int max_ctas, const ffs_grid_out* o, void* stream);

/* ffs_grid_build without a workspace argument: this variant has no counterpart
 * in the reference. It is for callers that cannot allocate device memory where
 * they build the grid -- code whose device memory is already owned by a
 * framework's allocator, or a foreign-language embedding that is handed only
 * its input and output buffers. The FP64 scratch is instead a file-scope
 * device array of FFS_GRID_STATIC_SCRATCH_BYTES (16 MiB) that every GPU
 * loading the library holds until the process exits; o->work is ignored.
 * - Sizes whose ffs_grid_work_bytes(T, K, P) exceeds the limit are rejected
 *   with FFS_ERR_WORKSPACE and a message.
 * - The first call on a device resolves the array's device address (with that
 *   device current); make that first call before any stream capture. The
 *   address is cached per device for the life of the process: after a
 *   cudaDeviceReset the cached address is stale, so a process that resets a
 *   device must not call this entry point on that device again.
 * - All calls share the one array: calls whose kernels overlap on the GPU
 *   (different streams, or different host threads on one device) race and
 *   must be serialised by the caller. Nothing in the array needs clearing
 *   between calls.
 * It calls no cudaMalloc, cudaFree or allocating library routine. */
#define FFS_GRID_STATIC_SCRATCH_BYTES ((size_t)16 << 20)
int ffs_grid_build_noalloc(const ffs_grid_desc* d, const ffs_grid_out* o, void* stream);

/* Orthonormal basis of the design's columns, Q0 [K][ld_t] fp32 (no reference
 * counterpart as a separate step: it is U of the pair (0, 0), which
 * ffs_grid_build also writes). Q0 = X Lx^-T with Lx the FP64 Cholesky factor of
 * X'X, or modified Gram-Schmidt (twice) when X'X is not positive definite
 * (*info = 1). Needing only X, it lets the residualisation (ffs_reml_prep) run
 * while the grid build is still in flight; Q0 equals the grid build's U of
 * (0, 0) bit for bit. Two kernel launches (the Gram entries of [X | 1] over
 * several CTAs, then one CTA for the factor). work: ffs_design_basis_work_bytes.
 * With const_flag / const_coef (both or neither) it also decides whether the
 * constant series lies in span(X): c = (X'X)^-1 X'1 from the same FP64
 * factor, *const_flag = 1 and const_coef[K] = c when ||X c - 1|| <= 1e-6
 * sqrt(T), else 0 and zeros (the centring test of ffs_reml_prep and the GLS). */
size_t ffs_design_basis_work_bytes(int T, int K);
int ffs_design_basis(int T, int K, const float* X, void* work, float* Q0, int* info, int* const_flag,
                     float* const_coef, void* stream);

/* The device address of host_ptr: pinned host memory mapped into the device's
 * address space (cudaHostAlloc / cudaHostRegister), or device memory (returned
 * as it is). FFS_ERR_INVALID for pageable or unregistered host memory, which
 * kernels must not read (no reference counterpart: the reference copies its
 * batches to the device). */
int ffs_device_view(const void* host_ptr, const void** dev_ptr);

/* ---------------------------------------------------------------- search data
 * Replaces the per-voxel scaling of fastfuncstuff/glm/arma.py:3952-3954,
 * 4685-4686 and _residualize_reml_search_data (arma.py:1554-1571).
 *   scale[v] = max(std(Y[v]) (N-1 divisor), 1e-8);
 *   Y_r[v]   = Y[v]/scale[v] - Q0 Q0' (Y[v]/scale[v]), Q0 an orthonormal basis
 *              of the design's columns (U of the pair (0,0) is that basis).
 * Outputs Y_r time-major fp32 and, when yr_hi/yr_lo are given, voxel-major fp16
 * hi/lo splits of Y_r * 2^yexp[v] (largest entry in [128, 256)) with row length
 * ld_y (>= T, multiple of 8, zero padded).
 * With do_scale == 0 the data are used as given (scale = 1). With center != 0
 * (only valid when the constant series lies in the design's span) each voxel's
 * mean is subtracted first: the criterion is unchanged, and the float32
 * residualisation no longer rounds against a large baseline.
 */
typedef struct {
  int V, T, K;
  const float* Y;       /* device [V][T] voxel-major input                       */
  const float* Q0;      /* device [K][ld_t]: orthonormal basis of the design columns */
  int do_scale;
  int center;
  int ld_y;
  float* scale;         /* [V]                                                    */
  float* yr_t;          /* [T][V] time-major residualised data                    */
  uint16_t* yr_hi;      /* [V][ld_y] fp16 bits or NULL                            */
  uint16_t* yr_lo;      /* [V][ld_y] fp16 bits or NULL                            */
  int* yexp;            /* [V] power-of-two scale of yr_hi/yr_lo (with yr_hi)     */
  /* Extensions for the learned-seeded refine (no reference counterpart):
   * idx   NULL, or [V] rows of Y to process: output row i is Y row idx[i]
   *       (scale is still written at idx[i]; every other output at i);
   * feats NULL, or [V][9]: lag 1..8 autocorrelations of each residualised row
   *       within runs (sum y_t y_t+k / sum y_t^2, 0 for a zero row) and T/1000,
   *       with run boundaries run_start[0..n_runs] (run_start[n_runs] = T).
   * yr_t may be NULL when only feats are wanted. */
  const int* idx;
  float* feats;
  int n_runs;
  const int* run_start;
  float* yr_rows;       /* NULL, or [V][T] the residualised rows, voxel-major    */
  const int* center_dev;/* NULL, or a device int that replaces `center` (set by
                           the caller's stream, so deciding needs no host sync) */
  /* Grouped fits (one design per voxel group): with tile_design, Q0 is
   * [n_designs][K][T] and tile v / 32 of the output rows uses design
   * tile_design[v / 32]; idx[i] < 0 marks an empty (padding) output row,
   * whose outputs are zero and which writes no scale. */
  const int* tile_design;
  /* End-to-end input without a staging copy (no reference counterpart; the
   * tiled prep only, T % 4 == 0, idx == NULL, no tile_design):
   * Y_ref  NULL, or a device pointer to the input's address (device memory):
   *        the rows are read from *Y_ref instead of Y (Y is then ignored; it
   *        may be NULL), staged by asynchronous copies. Being read on the
   *        device, the address can change between replays of a captured
   *        launch.
   * Y_copy NULL, or [V][T]: the input rows as read, written out (the later
   *        stages then read device memory). */
  const float* const* Y_ref;
  float* Y_copy;
} ffs_prep_args;

int ffs_reml_prep(const ffs_prep_args* a, void* stream);

/* ------------------------------------------------------------------ projection
 * The ||Q'Y_w||^2 term of fastfuncstuff/glm/arma.py:1992-1995 for every voxel
 * and pair: proj[p][v] = sum_j (sum_t U[p][j][t] Y_r[v][t])^2.
 * ffs_reml_project_tc runs it as a TMA-fed tcgen05 GEMM on fp16 hi/lo splits
 * (hi*hi + hi*lo + lo*hi, fp32 accumulation in TMEM) with the square-and-sum
 * epilogue on chip, which also removes the power-of-two scales. ffs_reml_project_simt is the CUDA-core form of the same
 * contraction (fp32), used for small or per-voxel-window problems.
 */
typedef struct {
  int V, T, K, P;
  int ld_y, ld_u;
  const uint16_t* yr_hi; const uint16_t* yr_lo;   /* [V][ld_y]  fp16 bits */
  const uint16_t* u_hi;  const uint16_t* u_lo;    /* [P*K][ld_u] fp16 bits */
  const int* yexp;      /* [V] */
  const int* uexp;      /* [P] */
  const float* yr_t;    /* [T][V] (simt form)                                    */
  const float* U;       /* [P][K][ld_t] (simt form)                              */
  float* proj;          /* [P][V]                                                 */
  int* flag;            /* device int, 0 on entry; set non-zero if a bounded
                           device-side wait expired (tc form)                    */
  const int* V_dev;     /* NULL, or a device count: only the operand rows
                           v < min(V, *V_dev) are projected (tc grid form; V
                           stays the row stride of proj)                         */
} ffs_project_args;

int ffs_reml_project_tc(const ffs_project_args* a, void* stream);

/* Tile shape of ffs_reml_project_tc for designs of K columns: the pairs that
 * share one B tile (pairs x K <= 256 columns of the MMA's N; 0 restores the
 * widest tile, 256 / K pairs). Process-wide, thread-safe; the results do not
 * depend on it (every pair's sums are formed in the same order), only the
 * speed. The Python autotuner (fastfuncstuff_gb300.autotune_projection) times
 * the candidates on the fit's shape and sets the fastest. */
int ffs_reml_tune_tc_pairs(int K, int pairs);
int ffs_reml_project_simt(const ffs_project_args* a, void* stream);

/* Work-list form of ffs_reml_project_tc (no reference counterpart: the
 * learned-seeded refine evaluates each voxel's 5 x 5 window only, and the
 * grouped fit walks (design, pair block, voxel tile) items in one launch).
 * Item i projects the 128 operand rows v0 .. v0+127 (nv of them real) onto the
 * np consecutive pairs whose U rows start at row_b (= first pair * K) and
 * writes, for ld_out > 0,
 *   proj[(out0 + r) * ld_out + slot0 + j] = ||U_{p+j}' y_{v0+r}||^2
 * or, for ld_out == 0, pair-major proj[(slot0 + j) * a->V + out0 + r].
 * The item count is read on the device from *n_items (<= max_items); every
 * item has np <= max_pairs and max_pairs * K <= 256. a->V is the number of
 * operand rows, a->P the number of U row blocks (pairs, or designs x pairs:
 * uexp[row_b / K + j] scales pair j), a->proj the output. */
typedef struct {
  int v0, nv;     /* first operand row, real rows (<= 128)                       */
  int row_b, np;  /* first U row, pairs                                          */
  int out0;       /* output row of operand row v0                                */
  int slot0;      /* output column of the first pair                             */
} ffs_tc_item;

int ffs_reml_project_tc_list(const ffs_project_args* a, const ffs_tc_item* items, const int* n_items,
                             int max_items, int max_pairs, int ld_out, void* stream);

/* --------------------------------------------------------------------- surface
 * The REML criterion of every voxel at every pair
 * (fastfuncstuff/glm/arma.py:1983-2002):
 *   crit = logdet_R + logdet_XtX + (T-K) log(RSS + 1e-10),
 *   RSS  = y'R^-1 y - proj, y'R^-1 y by the O(T) recurrence of coef.
 * The criterion is formed relative to the pair (0,0) (index p0) so that the
 * float32 arithmetic resolves differences between neighbouring pairs:
 *   d[p][v] = (const_p - const_p0) + (T-K) log1p((RSS_p - RSS_p0)/(RSS_p0+1e-10))
 * and crit = crit0[v] + d[p][v], crit0 = const_p0 + (T-K) log(RSS_p0 + 1e-10)
 * evaluated in FP64. Pairs are walked in chunks of 4 quarters (work list below).
 */
typedef struct {
  int V, T, K, P;
  int p0;                 /* index of the pair (0, 0)                             */
  const float* yr_t;      /* [T][V]                                               */
  const float* coef;      /* [P][T][4]                                            */
  const double* logdet_R; const double* logdet_XtX;  /* [P]                      */
  const float* proj;      /* [P][V]                                               */
  const int* chunk_start; /* device [n_chunks+1]: the (at most 16) pair slots of */
  int n_chunks;           /*   chunk c are chunk_pairs[chunk_start[c] ..         */
  const int* chunk_pairs; /*   chunk_start[c+1]), -1 an empty slot; slots 4q..4q+3 */
                          /*   (quarter q) share one AR filter: one a, or all    */
                          /*   lambda == 0 (identity)                            */
  float* surf;            /* [P][V] d[p][v]                                       */
  double* crit0;          /* [V]                                                  */
  const int* tile_design; /* NULL, or [ceil(V / 256)]: the design of each tile of */
                          /*   256 voxels (grouped fits); logdet_XtX is then      */
                          /*   [n_designs][P] and read at design * P + pair       */
  /* AFNI-faithful banded R (ffs_grid_desc.band): y'R^-1 y by the band's
   * forward substitution (band_coef, row stride band_w, band[p] terms per
   * step) instead of coef's recursion; every pair of the grid is evaluated
   * and the chunks are not read. NULL band_coef: the exact ARMA(1,1) R. */
  const float* band_coef;
  int band_w;
  const int* band;
} ffs_surface_args;

int ffs_reml_surface(const ffs_surface_args* a, void* stream);

/* ---------------------------------------------------------------------- select
 * Exhaustive global argmin (fastfuncstuff/glm/arma.py:2004-2009: strict '<',
 * the first pair in list order wins ties) or AFNI's power-of-2 hierarchical
 * descent from (0,0) on the lattice (select_arma_params_hierarchical_from_surface,
 * fastfuncstuff/glm/arma.py:2224-2322).
 * lattice[ai*n_b + bi] = pair index or -1 for a filtered point.
 */
typedef struct {
  int V, P;
  const float* surf;      /* [P][V]                                               */
  const double* crit0;    /* [V]                                                  */
  int hierarchical;       /* 0 exhaustive, 1 hierarchical                         */
  int n_a, n_b, ltop, za, zb;
  const int* lattice;     /* device [n_a*n_b]                                     */
  int* best;              /* [V] pair index                                       */
  float* best_crit;       /* [V] crit0 + d (float32, the reported likelihood)     */
} ffs_select_args;

int ffs_reml_select(const ffs_select_args* a, void* stream);

/* ---------------------------------------------------------------------- GLS
 * The GLS refit at each voxel's chosen pair (fastfuncstuff/glm/arma.py:4784-5590):
 * betas by G' y with one refinement step on the unwhitened residual, sigma2 from
 * the whitened residual (float64-style blocked accumulation), t, F (full model
 * or task columns), R^2 (unwhitened), GLT contrasts, lambda, and optional
 * residuals / whitened residuals / predicted series, all unscaled by scale[v].
 * Voxels are processed in the order of `order` (sorted by pair) so that a
 * warp reads one pair's matrices.
 */
typedef struct {
  int V, T, K;
  int dof;
  int center;             /* subtract the voxel mean first and add its betas
                             (mean/scale * Gsum) back; constant must be in span(X)*/
  const float* Gsum;      /* [P][K] (used with center)                            */
  const float* Y;         /* [V][T] voxel-major input data (unscaled)             */
  const float* scale;     /* [V]                                                  */
  const float* Xt;        /* [K][ld_t] the design, transposed                     */
  const int* best;        /* [V] pair per voxel                                   */
  const int* order;       /* [V] voxel permutation (grouped by pair) or NULL      */
  const float* coef; const float* G; const float* Adiag; const float* XtX;
  const float* a; const float* b;                    /* [P] grid values          */
  int lambda_fp32;        /* output lambda in float32 (1) or float64 rounded (0)  */
  int n_task; const int* task_idx;                   /* task columns (device)    */
  const float* Ftask;     /* [P][n_task][n_task] inv(A_task + 1e-8 I), or NULL    */
  int n_glt; const float* glt;                       /* [n_glt][K]                */
  const float* glt_var;   /* [P][n_glt] c A c'                                    */
  float* betas;           /* [V][K] every column; task selection is the caller's  */
  float* tstats;          /* [V][K]                                               */
  float* sigma2; float* fstats; float* r2; float* lam;   /* [V]                  */
  float* cbeta; float* ct;                           /* [V][n_glt] or NULL        */
  float* resid; float* resid_w; float* pred;         /* [V][T] or NULL            */
  const int* center_dev; /* NULL, or a device int that replaces `center`        */
  int n_pairs;            /* 0: one design, best[] / the groups are pairs.        */
                          /* > 0 (grouped fits): they are keys design * n_pairs + */
                          /*   pair; G, Adiag, XtX, Gsum, Ftask and glt_var are   */
                          /*   read at the key, coef, a, b at the pair and Xt is  */
                          /*   [n_designs][K][T], read at the design              */
  /* AFNI-faithful banded R (ffs_grid_desc.band): the whitening of the
   * residual is w_t = r_t c[t][0] - sum_{1 <= j <= band[p]} c[t][j] w_{t-j}
   * with c = band_coef of the pair (row stride band_w) instead of coef's
   * recursion; NULL band_coef: the exact ARMA(1,1) R. */
  const float* band_coef;
  int band_w;
  const int* band;
} ffs_gls_args;

int ffs_reml_gls(const ffs_gls_args* a, void* stream);

/* Column-set statistics of every voxel after the GLS (the reference's
 * -nuisance_summary sets, fastfuncstuff/glm/arma.py:3564-3586, unscaled at
 * :5845-5848): with b the betas of the scaled series (betas / scale[v]) and
 * s2 = sigma2 / scale[v]^2,
 *   F    = b_S' Fsets b_S / (q_S s2 + 1e-30),
 *   sd   = sqrt(max(b_S' Csets b_S, 0)) * scale[v]  (temporal SD of X_S b_S),
 *   coef = betas[v][S_0] for a one-column set, else NaN.
 * Set s writes column set_col[s] of the [V][n_out] outputs; the caller fills
 * the other columns (sets naming a column outside the design) with NaN.
 */
typedef struct {
  int V, K, n_sets, n_out;
  const int* set_ptr;     /* device [n_sets + 1]                                  */
  const int* set_idx;     /* device [set_ptr[n_sets]]                             */
  const int* set_col;     /* device [n_sets] output column of each set            */
  int msum;               /* sum of q_S^2                                         */
  const float* Fsets;     /* [keys][msum] from the grid build                     */
  const float* Csets;     /* [n_designs][msum] Xc_S' Xc_S / T, Xc the column-     */
                          /*   centred design                                     */
  const int* best;        /* [V] pair of each voxel                               */
  const int* design;      /* [V] design of each voxel (grouped fits) or NULL:     */
                          /*   key = design * n_pairs + pair                      */
  int n_pairs;
  const float* betas;     /* [V][K] every column, unscaled (ffs_reml_gls)         */
  const float* sigma2;    /* [V] unscaled                                         */
  const float* scale;     /* [V]                                                  */
  float* set_fstats; float* set_sd; float* set_coef;  /* [V][n_out]              */
} ffs_set_stats_args;

int ffs_reml_set_stats(const ffs_set_stats_args* a, void* stream);

/* -dsort: the GLS of every voxel with the extended design [X | D_v] at its
 * pair, D_v its q voxelwise regressors (fastfuncstuff/glm/arma.py:3248-3539,
 * after the constant guard and any per-run expansion, which the caller does).
 * Block elimination against the pair's factors: with b0 = G'y, H = G'D,
 * P_y = U'y, P_D = U'D (U'x = Q'L^-1 x) and the whitened D_w, y_w,
 *   S   = D_w'D_w - P_D'P_D + 1e-8 I,   b_D = S^-1 (D_w'y_w - P_D'P_y),
 *   b_X = b0 - H b_D,   cov / sigma2 = [[A + H S^-1 H', -H S^-1], [., S^-1]]
 * (A = (X_w'X_w)^-1), then sigma2 = ||L^-1 r||^2 / dof of the unwhitened
 * residual r, t, F over the task (or all base) columns through the Woodbury
 * form of inv(cov_task + 1e-8 I) with Ftask (or X_w'X_w), R^2, GLT on the
 * base block, column sets over [X | D] (indices >= K are D columns; needs
 * Afull) and Ljung-Box of the whitened residual; all unscaled by scale[v].
 * The data are divided by scale[v]; D stays in its own units.
 */
typedef struct {
  int V, T, K, q;
  int dof;                /* max(1, T - K - q)                                    */
  const float* Y;         /* [V][T] data (unscaled)                               */
  const float* scale;     /* [V]                                                  */
  const float* D;         /* [V][q][T] voxelwise regressors                       */
  const float* Xt;        /* [n_designs][K][ld_t] the design(s), transposed       */
  const float* xmean;     /* [n_designs][K] column means of the design(s) (sets)  */
  const int* best;        /* [V] pair, or key design * n_pairs + pair             */
  int n_pairs;            /* 0: one design                                        */
  const float* coef;      /* [P][T] float4 (indexed by pair)                      */
  const float* G; const float* U;   /* [keys][K][ld_t]                            */
  const float* Adiag;     /* [keys][K]                                            */
  const float* XtX;       /* [keys][K][K]                                         */
  const float* Afull;     /* [keys][K][K] or NULL (needed with column sets)       */
  int n_task; const int* task_idx; const float* Ftask;  /* [keys][n_task]^2       */
  int n_glt; const float* glt; const float* glt_var;    /* [n_glt][K], [keys][n_glt] */
  int n_sets; const int* set_ptr; const int* set_idx; const int* set_col; int n_set_out;
  int lj_h; const int* lj_tau; const float* lj_w;
  float* betas; float* tstats;      /* [V][K] every base column                   */
  float* dbetas; float* dtstats;    /* [V][q]                                     */
  float* sigma2; float* fstats; float* r2;             /* [V]                     */
  float* cbeta; float* ct;          /* [V][n_glt] or NULL                         */
  float* resid; float* resid_w; float* pred;           /* [V][T] or NULL          */
  float* ljung_box;                 /* [V] or NULL                                */
  float* set_fstats; float* set_sd; float* set_coef;   /* [V][n_set_out] or NULL  */
  int* status;            /* device int: set to 1 if some voxel's S had a pivot   */
                          /*   <= 0 (D in the span of X); NULL to skip            */
  /* AFNI-faithful banded R (ffs_grid_desc.band): y, D and the residual are
   * whitened by the pair's band (band_coef, row stride band_w, band[p] terms)
   * instead of coef's recursion; NULL band_coef: the exact ARMA(1,1) R. */
  const float* band_coef;
  int band_w;
  const int* band;
} ffs_dsort_args;

#define FFS_DSORT_QMAX 16
int ffs_reml_gls_dsort(const ffs_dsort_args* a, void* stream);

/* ffs_reml_gls plus the Ljung-Box statistic of each voxel's whitened residual
 * (fastfuncstuff/glm/arma.py:6058-6141, AFNI ljung_box_uneven): lj_h is the
 * resolved max lag (<= T/2), lj_tau the pseudo-time of every retained point
 * (NULL: plain index lags), lj_w[k] = 1/n_k for bins with n_k > 1 else 0. */
int ffs_reml_gls_ex(const ffs_gls_args* a, int lj_h, const int* lj_tau, const float* lj_w,
                    float* ljung_box, void* stream);

/* ffs_reml_gls_ex for voxels grouped by pair (after ffs_reml_group): group_end
 * is ffs_reml_group's work array (group_end[g] = end of pair g's voxels in
 * order), tile_start a [P + 1] int scratch. Tiles of up to 32 same-pair voxels
 * share one staging of the pair's G and of the design in shared memory. */
int ffs_reml_gls_grouped(const ffs_gls_args* a, int lj_h, const int* lj_tau, const float* lj_w,
                         float* ljung_box, int P, const int* group_end, int* tile_start, void* stream);

/* Counting sort of voxels by pair: order[] lists voxel ids grouped by best[].
 * Replaces the torch.unique / sort grouping of fastfuncstuff/glm/arma.py:4794-4811.
 * work: int[P + 1]; on return work[g] is the end of pair g's voxels in order.
 * Keys outside [0, P) are left out (order then holds work[P - 1] entries). */
int ffs_reml_group(int V, int P, const int* best, int* work, int* order, void* stream);

/* --------------------------------------------------------- learned proposal
 * No counterpart in the reference: this build's learned seed for the grid
 * search. A 9 -> 64 -> 64 -> 2 GELU MLP maps each voxel's OLS-residual
 * autocorrelations (lags 1-8) and T/1000 to a proposed (a, b); only the 5 x 5
 * lattice window around it is evaluated, and voxels whose best pair sits on
 * the window edge (a valid lattice neighbour outside the window) fall back to
 * the full grid.
 * Parameters are one float32 vector of ffs_mlp_param_count() entries:
 * W1[64][9], b1[64], W2[64][64], b2[64], W3[2][64], b3[2].
 */
int ffs_mlp_param_count(void);

/* Training voxels: per run y_t = a y_{t-1} + e_t + b e_{t-1} (200 burn-in
 * samples, standardised), Y[v] = X beta + sigma noise, beta ~ N(0,1),
 * sigma ~ U(0.5, 2); Philox4x32-10 counter-based normals (seed, voxel). */
int ffs_arma_simulate(int V, int T, int K, int n_runs, const int* run_start, const float* X, const float* a,
                      const float* b, uint64_t seed, float* Y, void* stream);

/* Features come from ffs_reml_prep (ffs_prep_args.feats). */

int ffs_mlp_forward(const float* params, const float* x, int B, float* out, void* stream);

/* grad += d/dparams of sum_b (out_b - y_b)^2 / (2 n_total) over the B samples
 * idx[0..B) (or 0..B when idx is NULL); loss += the same sum. */
int ffs_mlp_grad(const float* params, const float* x, const float* y, const int* idx, int B, int n_total,
                 float* grad, float* loss, void* stream);

/* One bias-corrected Adam step (step >= 1); consumes and zeroes grad. */
int ffs_mlp_adam(float* params, float* grad, float* m, float* v, int n, float lr, float beta1, float beta2,
                 float eps, int step, void* stream);

/* center[v] = ai * n_b + bi of the lattice point nearest the proposal prop[v]. */
int ffs_reml_centers(int V, const float* prop, const float* a_axis, int n_a, const float* b_axis, int n_b,
                     int* center, void* stream);

/* Rows of the prep outputs in the order idx[0..n): out_hi/out_lo[i] =
 * yr_hi/yr_lo[idx[i]] ([.][ld_y] fp16 bits) -- or, with yr_hi = yr_lo = NULL,
 * the same split formed here from yr_rows[idx[i]] and yexp (so the prep need
 * not store every voxel's split) --, out_exp[i] = yexp[idx[i]] and,
 * when out_t is given, out_t[t][i] = yr_rows[idx[i]][t] ([T][n], time-major)
 * for the windowed refine's sorted operands. With n_dev (device int) only the
 * rows i < min(n, *n_dev) are written. */
int ffs_reml_gather(int n, const int* n_dev, int T, int ld_y, const int* idx, const uint16_t* yr_hi,
                    const uint16_t* yr_lo, const int* yexp, const float* yr_rows, uint16_t* out_hi, uint16_t* out_lo,
                    int* out_exp, float* out_t, void* stream);

/* Work list of the windowed refine for voxels sorted by window centre
 * (cell = ai * n_b + bi; cell c's sorted rows end at cell_end[c], as
 * ffs_reml_group leaves them): one ffs_tc_item per 128-row tile of a cell and
 * run of at most max_pairs consecutive valid pairs of one window row, with
 * slot0 = 5 * window row + window column, and one tile (v0, nv) = tiles[2t],
 * tiles[2t+1] per 128-row tile of a cell for ffs_reml_window. The counts go to
 * *n_items and *n_tiles (clamped to max_items, max_tiles; *overflow = 1 if
 * anything was dropped). With P > 0 (grouped designs) the sort keys are
 * cell * n_designs + design (ncell = n_designs * n_a n_b): the items' U rows
 * are those of the key's design, (design * P + pair) * K, and the tiles span
 * a cell's rows of every design. */
int ffs_reml_window_items(int ncell, const int* cell_end, int n_a, int n_b, const int* lattice, int K,
                          int max_pairs, ffs_tc_item* items, int* n_items, int max_items, int* tiles,
                          int* n_tiles, int max_tiles, int* overflow, int P, void* stream);

/* The windowed refine's criterion over the tiles of ffs_reml_window_items
 * (launched for max_tiles, *n_tiles of them real), one sorted row i < n (voxel
 * idx[i], window centre center[idx[i]]): y'R^-1 y of each non-identity window pair by the O(T)
 * recurrence of coef over rows[idx[i]] (rows: [V][T] residualised series,
 * voxel-major, 16-byte aligned: ffs_reml_prep's yr_rows), its
 * projection from winproj[i][slot] (ffs_reml_project_tc_list), the criterion
 * relative to (0, 0) with dcf[p] = (logdet_R + logdet_XtX)[p] - that of (0, 0)
 * (*c_p0, a device scalar),
 * and the argmin. Identity pairs (ident[p] = 1 when lambda == 0) all have
 * d = 0 and the full grid picks the first of them, p_id: a window holding one
 * competes with (p_id, 0), and a win by it is final. Writes at voxel idx[i]:
 * best, dbest (criterion relative to (0, 0)), crit0 (as ffs_reml_surface),
 * fallback = 1 when the full grid must decide (the best non-identity pair has
 * a valid lattice neighbour outside the window, or the window holds no
 * identity pair and nothing below d = 0), best_cell (the lattice cell of the
 * best non-identity pair, -1 if none) and, when next_center is given, the
 * voxel's centre for a re-centred round: best_cell when fallback = 1 and
 * best_cell >= 0, else n_a * n_b (no window). With design (grouped designs,
 * [V] each voxel's design), dcf is [n_designs][P] and c_p0 [n_designs], each
 * read at the row's design. With ssw_pre ([n][25], AFNI's banded R:
 * ffs_reml_band_sums) y'R^-1 y of each window slot is read from it instead
 * of the recurrence of coef. */
int ffs_reml_window(int n, int T, int K, int n_a, int n_b, const int* lattice, const int* idx, const int* center,
                    const int* tiles, const int* n_tiles, int max_tiles, const float* rows, const float* coef,
                    const float* winproj, const float* dcf, const unsigned char* ident, int p_id,
                    const double* c_p0, int* best, float* dbest, double* crit0, int* fallback, int* best_cell,
                    int* next_center, const int* design, int P, const float* ssw_pre, void* stream);

/* y'R^-1 y of sorted rows under AFNI's banded R (ffs_grid_desc.band) for the
 * learned-seeded refine, by the band's forward substitution of band_coef
 * (row stride band_w, band[p] terms) over rows[idx[i]] (T samples, voxel-
 * major). Window mode (tiles given, as ffs_reml_window_items leaves them):
 * the rows of tile x, each pair of the 5 x 5 window of the tile's centre
 * cell center[idx[first row]] that is valid and not an identity pair
 * (ident), into out[i][slot] (25 slots, 5 * window row + window column).
 * Strip mode (tiles NULL): the rows i < min(n, *n_dev) against the n_pairs
 * pairs[q], into out[q][i] (row stride n). No reference counterpart. */
int ffs_reml_band_sums(int n, const int* n_dev, int T, const int* idx, const float* rows, const float* band_coef,
                       int band_w, const int* band, const int* tiles, const int* n_tiles, int max_tiles,
                       const int* center, const int* lattice, int n_a, int n_b, const unsigned char* ident,
                       const int* pairs, int n_pairs, float* out, void* stream);

/* The strip next to the identity line in the learned-seeded refine (no
 * reference counterpart: the reference searches every pair). Near lambda = 0
 * the criterion is nearly flat along the line a = -b and can have minima at
 * several a, so a window holding one of them proves nothing about the others.
 * n_pairs <= 64 pairs (pair indices pairs[]) are evaluated for the sorted rows
 * i < min(n, *n_dev) (n_dev may be NULL) of the voxels idx[i]: the window
 * kernel's recurrence over rows[idx[i]] (16-byte aligned, T samples each) and
 * the projections proj[q][i] (row stride n: ffs_reml_project_tc of the
 * gathered rows against the pairs' U rows), giving each pair's criterion
 * relative to (0, 0) as ffs_reml_window forms it. A voxel v whose least strip
 * criterion lies below its window answer dbest[v] by more than
 * 1e-6 |crit0[v]| gets fallback[v] = 1 and best_cell[v] = -1 (the full grid
 * decides); nothing else is written. With design (grouped designs, [V] each
 * voxel's design, P pairs per design) dcf is [n_designs][P], read at the
 * voxel's design; otherwise dcf is [P] and P is ignored. With ssw_pre
 * ([n_pairs][n], AFNI's banded R: ffs_reml_band_sums in strip mode) y'R^-1 y
 * of each pair is read from it instead of the recurrence of coef. */
int ffs_reml_strip(int n, const int* n_dev, int T, int K, int n_pairs, const int* pairs, const int* idx,
                   const float* rows, const float* coef, const float* proj, const float* dcf, const float* dbest,
                   const double* crit0, int* fallback, int* best_cell, const int* design, int P,
                   const float* ssw_pre, void* stream);

/* Work list of ffs_reml_project_tc_list for rows sorted into n_seg segments
 * (segment s: sorted rows [seg_end[s-1], seg_end[s]), seg_end[-1] = 0, as
 * ffs_reml_group leaves them) that each project onto their own n_pairs pairs:
 * one ffs_tc_item per 128-row tile of a segment and block of at most
 * max_pairs (max_pairs * K <= 256) of its pairs, U rows from
 * (s * n_pairs + first pair) * K, output slot = the pair's rank (pair-major,
 * ld_out = 0). The strip next to the identity line of a grouped fit uses one
 * segment per design against the strip pairs' U rows of every design
 * ([n_designs][n_pairs][K][ld]). The count goes to *n_items (clamped to
 * max_items; *overflow = 1 if items were dropped). No reference counterpart. */
int ffs_reml_segment_items(int n_seg, const int* seg_end, int n_pairs, int K, int max_pairs, ffs_tc_item* items,
                           int* n_items, int max_items, int* overflow, void* stream);

/* The voxels v < V whose pair best[v] lies within k0 lattice steps of an
 * identity pair (dist[p]: the Manhattan lattice distance of pair p to the
 * nearest lambda = 0 pair) and, when fallback is given, fallback[v] == 0, into
 * ids[0 .. *count), in no particular order: the learned-seeded refine
 * evaluates the strip next to the identity line for these voxels (no
 * reference counterpart). */
int ffs_reml_near_line(int V, const int* best, const int* dist, int k0, const int* fallback, int* ids, int* count,
                       void* stream);

/* The end of the learned-seeded refine's window rounds: best_crit[v] =
 * crit0[v] + dbest[v] (FP64 sum rounded to float) for v < V, small[0] = the
 * number of voxels with fallback[v] != 0, small[1 + i] = *extra[i] for the
 * n_extra <= 8 device ints named by the host array extra (the wait flag and
 * the work lists' overflow flags): the few numbers the host reads back (no
 * reference counterpart). */
int ffs_reml_window_finish(int V, const double* crit0, const float* dbest, const int* fallback, float* best_crit,
                           int* small, int n_extra, const int* const* extra, void* stream);

/* The voxels v < V with flag[v] != 0 into ids[0 .. *count), in no particular
 * order, with ids[*count .. n_pad) = 0 and pos[v] = the slot of voxel v in ids
 * or -1: the list of the voxels the full grid takes after the learned-seeded
 * refine, padded to a captured size (no reference counterpart: the reference
 * searches every pair). A flagged voxel past n_pad keeps pos -1; size n_pad
 * from the same flags. */
int ffs_reml_compact(int V, const int* flag, int n_pad, int* ids, int* pos, int* count, void* stream);

/* One output field of ffs_merge_rows: V rows of row_bytes (a multiple of 4)
 * each. */
typedef struct {
  void* dst;            /* [V] rows written */
  const void* src;      /* [V] rows: every voxel's value, or NULL: dst's other rows stay */
  const void* src_sub;  /* NULL, or [n] rows that replace src's for the voxels with pos[v] >= 0 */
  int row_bytes;
} ffs_merge_field;

/* dst[v] = src_sub[pos[v]] if pos (may be NULL) gives pos[v] >= 0 and the
 * field has src_sub, else src[v] (nothing, for a field without src), for up
 * to 32 fields in one launch: the fit's outputs from the windows' answers and
 * the full grid's answers for the voxels it took (no reference counterpart).
 * dst may be pinned host memory mapped into the device's address space. */
int ffs_merge_rows(int V, const int* pos, int n_fields, const ffs_merge_field* fields, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* FFS_REML_H */
