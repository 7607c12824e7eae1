// GLS refit at each voxel's chosen (a, b), one warp per voxel.
//
// Follows fastfuncstuff/glm/arma.py:4784-5590 (X'X path):
//   betas   b = (X_w'X_w)^-1 X_w' L^-1 y = G' y, then one refinement step
//           b += G' (y - X b) on the unwhitened residual;
//   sigma2  = ||L^-1 (y - X b)||^2 / dof (whitened residual, fastfuncstuff
//             accumulates it in float64; here fp32 in blocks of 32 terms);
//   t       = b / (sqrt(sigma2 diag A) + 1e-10);
//   F       = b'Mb / (sigma2 q + 1e-10), M = X_w'X_w (full model, q = K) or
//             inv(A_task + 1e-8 I) (task columns, q = n_task);
//   R^2     = 1 - SS_res/SS_tot on the unwhitened scaled data (xval.py:564-593);
//   GLT     c'b and c'b / (sqrt(max(sigma2 c A c', 0)) + 1e-10);
//   Ljung-Box of the whitened residual (arma.py:6058-6141);
// then unscaled by the voxel's std (arma.py:5827-5862).
#include "common.cuh"
#include "tile.cuh"

namespace ffsk {
namespace {

constexpr int GLS_WARPS = 4;

struct GlsExtra {
  int lj_h;             // Ljung-Box max lag (0: off)
  const int* lj_tau;    // [T] pseudo-time or NULL (plain index lags)
  const float* lj_w;    // [lj_h + 1] 1 / n_k for good bins, 0 otherwise
  float* ljung_box;     // [V]
};

// A group key g is the pair itself (one design) or design * n_pairs + pair.
__device__ __forceinline__ int pair_of(const ffs_gls_args& a, int g) { return a.n_pairs > 0 ? g % a.n_pairs : g; }
__device__ __forceinline__ int design_of(const ffs_gls_args& a, int g) { return a.n_pairs > 0 ? g / a.n_pairs : 0; }

__device__ void gls_finish(const ffs_gls_args& a, const GlsExtra& x, int v, int g, float* beta, const float* w,
                           float ssr, float sst, float ssw, float m, float sc, float* bins, const float* Mq);

// The F statistic's matrix of group g: inv(A_task + 1e-8 I) for task columns,
// X_w'X_w for the full model.
__device__ __forceinline__ const float* quad_matrix(const ffs_gls_args& a, int g) {
  return a.n_task > 0 ? a.Ftask + (size_t)g * a.n_task * a.n_task : a.XtX + (size_t)g * a.K * a.K;
}

// Whitening against AFNI's banded R: w_t = r_t c[t][0] - sum_j c[t][j] w_{t-j}
// for j up to the pair's band (rows past a run start or a censoring gap have
// zero coefficients there), by one thread over the whole series; r and w may
// be the same array (w_{t-j} is then read where it was written).
__device__ __forceinline__ void band_whiten_rows(const float* cb, int W, int bw, const float* r, float* w, int T) {
  for (int t = 0; t < T; ++t) {
    const float* c = cb + (size_t)t * W;
    float acc = r[t] * c[0];
    const int jm = min(bw, t);
    for (int j = 1; j <= jm; ++j) acc = fmaf(-c[j], w[t - j], acc);
    w[t] = acc;
  }
}

__device__ __forceinline__ void band_whiten(const ffs_gls_args& a, int p, const float* r, float* w, int T) {
  band_whiten_rows(a.band_coef + (size_t)p * T * a.band_w, a.band_w, a.band[p], r, w, T);
}

// GLS of one voxel v at pair g, executed by one warp. Gp = G of pair g and Xt
// (the transposed design) may live in shared or global memory; ys, r, beta and
// bins are this warp's shared scratch.
__device__ void gls_voxel(const ffs_gls_args& a, const GlsExtra& x, const int v, const int g, const float* Gp,
                          const float* Xt, float* ys, float* r, float* beta, float* bins) {
  const int lane = threadIdx.x & 31;
  const int T = a.T, K = a.K;
  const float sc = a.scale[v];
  const float* y = a.Y + (size_t)v * T;

  // optional centring: fit (y - m)/s, then add (m/s) * G'1 to the betas; the
  // residuals, sigma2, R^2 and the t of every column but the constant's are
  // unchanged because the constant lies in span(X)
  float m = 0.f;
  if (a.center_dev ? (*a.center_dev != 0) : (a.center != 0)) {
    float sm_ = 0.f;
    for (int t = lane; t < T; t += 32) sm_ += y[t];
    m = warp_sum(sm_) / (float)T;
  }
  for (int t = lane; t < T; t += 32) ys[t] = __fdiv_rn(__fsub_rn(y[t], m), sc);
  __syncwarp();

  // b0 = G' y
  for (int j = 0; j < K; ++j) {
    const float* gj = Gp + (size_t)j * ld_t(T);
    float s = 0.f;
    for (int t = lane; t < T; t += 32) s = fmaf(gj[t], ys[t], s);
    s = warp_sum(s);
    if (lane == 0) beta[j] = s;
  }
  __syncwarp();
  // refinement: b += G' (y - X b)
  for (int t = lane; t < T; t += 32) {
    float acc = ys[t];
    for (int j = 0; j < K; ++j) acc = fmaf(-Xt[(size_t)j * ld_t(T) + t], beta[j], acc);
    r[t] = acc;
  }
  __syncwarp();
  for (int j = 0; j < K; ++j) {
    const float* gj = Gp + (size_t)j * ld_t(T);
    float s = 0.f;
    for (int t = lane; t < T; t += 32) s = fmaf(gj[t], r[t], s);
    s = warp_sum(s);
    if (lane == 0) beta[j] += s;
  }
  __syncwarp();
  // final unwhitened residual, SS_res and SS_tot
  float ssr = 0.f, sy = 0.f;
  for (int t = lane; t < T; t += 32) {
    float acc = ys[t];
    for (int j = 0; j < K; ++j) acc = fmaf(-Xt[(size_t)j * ld_t(T) + t], beta[j], acc);
    r[t] = acc;
    ssr = fmaf(acc, acc, ssr);
    sy += ys[t];
  }
  ssr = warp_sum(ssr);
  const float mean = warp_sum(sy) / (float)T;
  float sst = 0.f;
  for (int t = lane; t < T; t += 32) {
    const float dlt = ys[t] - mean;
    sst = fmaf(dlt, dlt, sst);
  }
  sst = warp_sum(sst);
  __syncwarp();
  if (a.pred) {
    for (int t = lane; t < T; t += 32) a.pred[(size_t)v * T + t] = (ys[t] - r[t]) * sc + m;
  }
  if (a.resid) {
    for (int t = lane; t < T; t += 32) a.resid[(size_t)v * T + t] = r[t] * sc;
  }
  __syncwarp();
  // whitened residual r_w = L^-1 r (serial recurrence on lane 0), into ys
  const float4* cf = reinterpret_cast<const float4*>(a.coef) + (size_t)pair_of(a, g) * T;
  if (a.band_coef) {
    if (lane == 0) band_whiten(a, pair_of(a, g), r, ys, T);
  } else if (lane == 0) {
    float rp = 0.f, vp = 0.f;
    for (int t = 0; t < T; ++t) {
      const float4 q = cf[t];
      const float rt = r[t];
      const float z = fmaf(-q.x, rp, rt);
      const float vt = fmaf(-q.y, vp, z);
      ys[t] = vt * q.w;
      rp = rt;
      vp = vt;
    }
  }
  __syncwarp();
  float ssw = 0.f;
  for (int t = lane; t < T; t += 32) ssw = fmaf(ys[t], ys[t], ssw);
  ssw = warp_sum(ssw);
  gls_finish(a, x, v, g, beta, ys, ssr, sst, ssw, m, sc, bins, quad_matrix(a, g));
}

// Ljung-Box statistic of one series ys[T] (shared memory) with sum of squares
// ssw, by one warp: c_k = sum r_j r_{j+k} / ssw binned by time lag (plain
// index lags without tau), LB = T (T + 2) sum_k c_k^2 w_k, clamped at 1e10;
// 0 when T < 10 or ssw < 1e-10 (fastfuncstuff/glm/arma.py:6058-6141). bins:
// [h + 1] floats of shared memory. The value is returned on lane 0.
__device__ float ljung_box_warp(int h, const int* tau, const float* w, const float* ys, int T, float ssw,
                                float* bins) {
  const int lane = threadIdx.x & 31;
  for (int k = lane; k <= h; k += 32) bins[k] = 0.f;
  __syncwarp();
  for (int k = 1; k <= h; ++k) {
    if (!tau) {
      float part = 0.f;
      for (int t = lane; t + k < T; t += 32) part = fmaf(ys[t], ys[t + k], part);
      part = warp_sum(part);
      if (lane == 0) bins[k] += part;
    } else {
      for (int t = lane; t + k < T; t += 32) {
        const int dj = tau[t + k] - tau[t];
        if (dj > 0 && dj <= h) atomicAdd(bins + dj, ys[t] * ys[t + k]);
      }
    }
  }
  __syncwarp();
  float lb = 0.f;
  if (lane == 0 && ssw >= 1e-10f && T >= 10) {
    double acc = 0.0;
    for (int k = 1; k <= h; ++k) {
      const double ck = (double)bins[k] / (double)ssw;
      acc += ck * ck * (double)w[k];
    }
    acc *= (double)T * ((double)T + 2.0);
    lb = (float)fmin(acc, 1.0e10);
  }
  return lb;
}

// The statistics of voxel v at pair g from its betas (of the centred, scaled
// series: beta, shared memory), whitened residual w (shared memory, [T]) and
// sums of squares; executed by one warp.
__device__ void gls_finish(const ffs_gls_args& a, const GlsExtra& x, const int v, const int g, float* beta,
                           const float* w, const float ssr, const float sst, const float ssw, const float m,
                           const float sc, float* bins, const float* Mq) {
  const int lane = threadIdx.x & 31;
  const int T = a.T, K = a.K;
  const float* ys = w;
  if (a.resid_w) {
    for (int t = lane; t < T; t += 32) a.resid_w[(size_t)v * T + t] = ys[t] * sc;
  }
  const float sigma2 = ssw / (float)a.dof;

  // betas of the uncentred data: add (m/s) * G'1
  if (a.center_dev ? (*a.center_dev != 0) : (a.center != 0)) {
    const float ms = m / sc;
    for (int j = lane; j < K; j += 32) beta[j] = fmaf(ms, a.Gsum[(size_t)g * K + j], beta[j]);
  }
  __syncwarp();
  // t statistics and betas of every column (task selection is the caller's)
  for (int j = lane; j < K; j += 32) {
    const float se = sqrtf(sigma2 * a.Adiag[(size_t)g * K + j]);
    a.betas[(size_t)v * K + j] = beta[j] * sc;
    a.tstats[(size_t)v * K + j] = beta[j] / (se + 1e-10f);
  }
  float quad = 0.f;
  if (a.n_task > 0) {
    const float* M = Mq;
    for (int k = lane; k < a.n_task; k += 32) {
      float s = 0.f;
      for (int l = 0; l < a.n_task; ++l) s = fmaf(M[k * a.n_task + l], beta[a.task_idx[l]], s);
      quad = fmaf(beta[a.task_idx[k]], s, quad);
    }
  } else {
    const float* M = Mq;
    for (int k = lane; k < K; k += 32) {
      float s = 0.f;
      for (int l = 0; l < K; ++l) s = fmaf(M[k * K + l], beta[l], s);
      quad = fmaf(beta[k], s, quad);
    }
  }
  quad = warp_sum(quad);
  for (int c = lane; c < a.n_glt; c += 32) {
    const float* gc = a.glt + (size_t)c * K;
    float cb = 0.f;
    for (int j = 0; j < K; ++j) cb = fmaf(gc[j], beta[j], cb);
    const float var = a.glt_var[(size_t)g * a.n_glt + c] * sigma2;
    a.cbeta[(size_t)v * a.n_glt + c] = cb * sc;
    a.ct[(size_t)v * a.n_glt + c] = cb / (sqrtf(fmaxf(var, 0.f)) + 1e-10f);
  }

  if (x.lj_h > 0 && x.ljung_box) {
    const float lb = ljung_box_warp(x.lj_h, x.lj_tau, x.lj_w, ys, T, ssw, bins);
    if (lane == 0) x.ljung_box[v] = lb;
  }

  if (lane == 0) {
    const float q = a.n_task > 0 ? (float)a.n_task : (float)K;
    a.fstats[v] = quad / (sigma2 * q + 1e-10f);
    a.sigma2[v] = sigma2 * sc * sc;
    const bool deg = sst <= 1e-10f;
    const float r2 = 1.0f - ssr / fmaxf(sst, 1e-10f);
    a.r2[v] = deg ? 0.f : fminf(r2, 1.0f);
    const float af = a.a[pair_of(a, g)], bf = a.b[pair_of(a, g)];
    if (a.lambda_fp32) {
      a.lam[v] = lambda_out_f32(af, bf);
    } else {
      const double ad = af, bd = bf;
      a.lam[v] = (float)((bd + ad) * (1.0 + ad * bd) / (1.0 + 2.0 * ad * bd + bd * bd + 1e-10));
    }
  }
}

// One warp per voxel, matrices read from global memory (any shape).
__global__ void __launch_bounds__(GLS_WARPS * 32) gls_kernel(ffs_gls_args a, GlsExtra x, int ld_s,
                                                              int kp, int hb) {
  extern __shared__ float sm[];
  const int wid = threadIdx.x >> 5;
  float* ys = sm + (size_t)wid * (2 * ld_s + kp + hb);
  const int i = blockIdx.x * GLS_WARPS + wid;
  if (i >= a.V) return;
  const int v = a.order ? a.order[i] : i;
  const int g = a.best[v];
  gls_voxel(a, x, v, g, a.G + (size_t)g * a.K * ld_t(a.T), a.Xt + (size_t)design_of(a, g) * a.K * ld_t(a.T), ys, ys + ld_s,
            ys + 2 * ld_s, ys + 2 * ld_s + kp);
}

// Tiles of up to GLS_TILE voxels that share one pair (voxels grouped by pair:
// order[end[g-1] .. end[g]) are pair g's, end[-1] = 0); tile_start[g] numbers
// the tiles of pair g and blocks past the last tile exit. T % 4 == 0.
//
// The tile's 32 series sit in shared memory, one voxel per lane (tile.cuh):
//   b0 = G'y and r = y - X b0, then the refinement d = G'r (b = b0 + d): the
//   projections as register-blocked CUDA-core passes (tile_project), the
//   update r = y - X b0 as warp-level tensor-core MMAs of tf32 hi/lo splits
//   (tile_subtract_any). The residual statistics use r: the refined
//   residual r - X d differs from it by X d, which changes the whitened
//   residual sum of squares only to second order (L^-1 r is orthogonal to
//   L^-1 X up to d), so the update is not formed. The whitened residual
//   L^-1 r is computed by 8 segments of
//   the time axis (one per warp): each warp runs v_t = z_t - m_t v_{t-1} from
//   v = 0 over its segment, the true state entering segment k is carried
//   across the segment ends, and each sample adds its term prod(-m) * v_in.
// The per-voxel statistics (gls_finish) then run one warp per voxel.
constexpr int GLS_TILE = TILE_V;

// gls_finish for the n <= 32 voxels of a tile at once (no Ljung-Box): b =
// C0 + C1 (in C0) with the constant's betas added back, then t, F, R^2,
// sigma2, lambda and the GLT contrasts, spread over the CTA's threads instead
// of one warp per voxel. st holds m, sc, mean, ssr, sst, ssw per voxel; red
// (>= 8 x 32 floats) is scratch. Ends with the outputs written.
__device__ void gls_finish_tile(const ffs_gls_args& a, int g, int j0, int n, float* C0, const float* C1,
                                const float* Ys, int ld, const float* st, float* red, const float* Mq) {
  const int K = a.K, T = a.T, tid = threadIdx.x, nth = blockDim.x;
  const bool centre = a.center_dev ? (*a.center_dev != 0) : (a.center != 0);
  for (int idx = tid; idx < K * TILE_V; idx += nth) {
    const int j = idx / TILE_V, l = idx % TILE_V;
    float bj = C0[idx] + C1[idx];
    // betas of the uncentred data: add (m/s) * G'1
    if (centre) bj = fmaf(st[l] / st[TILE_V + l], a.Gsum[(size_t)g * K + j], bj);
    C0[idx] = bj;
  }
  __syncthreads();
  // betas and t statistics, voxel-major stores
  for (int idx = tid; idx < n * K; idx += nth) {
    const int l = idx / K, j = idx % K;
    const int v = a.order[j0 + l];
    const float sc = st[TILE_V + l], sigma2 = st[5 * TILE_V + l] / (float)a.dof;
    const float bj = C0[j * TILE_V + l];
    const float se = sqrtf(sigma2 * a.Adiag[(size_t)g * K + j]);
    a.betas[(size_t)v * K + j] = bj * sc;
    a.tstats[(size_t)v * K + j] = bj / (se + 1e-10f);
  }
  // whitened residual output
  if (a.resid_w) {
    for (int l = tid >> 5; l < n; l += nth >> 5) {
      const int v = a.order[j0 + l];
      const float sc = st[TILE_V + l];
      for (int t = tid & 31; t < T; t += 32) a.resid_w[(size_t)v * T + t] = Ys[(size_t)l * ld + t] * sc;
    }
  }
  // F: quad = b' M b over the model's (or the task) columns, 8 slices of the
  // rows k summed in order
  const int nk = a.n_task > 0 ? a.n_task : K;
  {
    const int l = tid & 31, ks = tid >> 5;
    float part = 0.f;
    if (l < n) {
      for (int k = ks; k < nk; k += TILE_WARPS) {
        const int ck = a.n_task > 0 ? a.task_idx[k] : k;
        float s = 0.f;
        for (int c = 0; c < nk; ++c) {
          const int cl = a.n_task > 0 ? a.task_idx[c] : c;
          s = fmaf(Mq[k * nk + c], C0[cl * TILE_V + l], s);
        }
        part = fmaf(C0[ck * TILE_V + l], s, part);
      }
    }
    red[ks * TILE_V + l] = part;
  }
  // GLT contrasts c'b and their t
  for (int idx = tid; idx < n * a.n_glt; idx += nth) {
    const int l = idx / a.n_glt, c = idx % a.n_glt;
    const int v = a.order[j0 + l];
    const float* gc = a.glt + (size_t)c * K;
    float cb = 0.f;
    for (int j = 0; j < K; ++j) cb = fmaf(gc[j], C0[j * TILE_V + l], cb);
    const float sigma2 = st[5 * TILE_V + l] / (float)a.dof;
    const float var = a.glt_var[(size_t)g * a.n_glt + c] * sigma2;
    a.cbeta[(size_t)v * a.n_glt + c] = cb * st[TILE_V + l];
    a.ct[(size_t)v * a.n_glt + c] = cb / (sqrtf(fmaxf(var, 0.f)) + 1e-10f);
  }
  __syncthreads();
  if (tid < n) {
    const int l = tid;
    const int v = a.order[j0 + l];
    float quad = 0.f;
    for (int w = 0; w < TILE_WARPS; ++w) quad += red[w * TILE_V + l];
    const float sc = st[TILE_V + l], ssr = st[3 * TILE_V + l], sst = st[4 * TILE_V + l];
    const float sigma2 = st[5 * TILE_V + l] / (float)a.dof;
    const float q = a.n_task > 0 ? (float)a.n_task : (float)K;
    a.fstats[v] = quad / (sigma2 * q + 1e-10f);
    a.sigma2[v] = sigma2 * sc * sc;
    const bool deg = sst <= 1e-10f;
    const float r2 = 1.0f - ssr / fmaxf(sst, 1e-10f);
    a.r2[v] = deg ? 0.f : fminf(r2, 1.0f);
    const int p = pair_of(a, g);
    const float af = a.a[p], bf = a.b[p];
    if (a.lambda_fp32) {
      a.lam[v] = lambda_out_f32(af, bf);
    } else {
      const double ad = af, bd = bf;
      a.lam[v] = (float)((bd + ad) * (1.0 + ad * bd) / (1.0 + 2.0 * ad * bd + bd * bd + 1e-10));
    }
  }
}

__global__ void __launch_bounds__(TILE_WARPS * 32, 3) gls_tile_kernel(ffs_gls_args a, GlsExtra x, const int* end,
                                                                   const int* tile_start, int P, int ld, int kp,
                                                                   int hb, int msz) {
  extern __shared__ float4 sm4[];
  const int T = a.T, K = a.K, LT = ld_t(T), nq = LT >> 2;
  const bool vec = (T & 3) == 0;  // 16-byte rows of the [V][T] outputs
  float* Ys = reinterpret_cast<float*>(sm4);        // [32][ld]
  float* C0 = Ys + (size_t)TILE_V * ld;             // [K][32] b0
  float* C1 = C0 + (size_t)K * TILE_V;              // [K][32] d
  float* red = C1 + (size_t)K * TILE_V;             // [8][32] SS_w partials
  float* vend = red + TILE_WARPS * TILE_V;          // [8][32]
  float* carry = vend + TILE_WARPS * TILE_V;        // [8][32]
  float* Hs = carry + TILE_WARPS * TILE_V;          // [32]
  float* st = Hs + TILE_V;                          // [6][32] m, sc, mean, ssr, sst, ssw
  float* betas = st + 6 * TILE_V;                   // [8][kp]
  float* bins = betas + (size_t)TILE_WARPS * kp;    // [8][hb]
  float* Ms = bins + (size_t)TILE_WARPS * hb;       // [msz] the F matrix of the tile's group (msz > 0)

  const int tile = blockIdx.x;
  if (tile >= tile_start[P]) return;
  int lo = 0, hi = P;  // largest g with tile_start[g] <= tile
  while (hi - lo > 1) {
    const int mid = (lo + hi) >> 1;
    if (tile_start[mid] <= tile) lo = mid; else hi = mid;
  }
  const int g = lo;
  const int g0 = g ? end[g - 1] : 0;
  const int j0 = g0 + (tile - tile_start[g]) * GLS_TILE;
  const int n = min(GLS_TILE, end[g] - j0);
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;

  // stage (y - m) / s of each voxel; empty slots of a short tile are zero
  __shared__ int src_row[TILE_V];
  if (threadIdx.x < TILE_V) src_row[threadIdx.x] = (int)threadIdx.x < n ? a.order[j0 + threadIdx.x] : -1;
  const float* Mq = quad_matrix(a, g);
  if (msz > 0) {  // read by every voxel's F statistic
    for (int i = threadIdx.x; i < msz; i += blockDim.x) Ms[i] = Mq[i];
    Mq = Ms;
  }
  __syncthreads();
  tile_stage_rows(a.Y, T, nq, src_row, Ys, ld);
  const bool centre = a.center_dev ? (*a.center_dev != 0) : (a.center != 0);
  {
    // the warp's rows wid + 8k together, so their reductions overlap; a row
    // past the tile's voxels keeps m = 0, sc = 1 and mean 0
    constexpr int RW = TILE_V / TILE_WARPS;
    bool on[RW];
    float sc[RW], m[RW], inv[RW], sy[RW];
#pragma unroll
    for (int k = 0; k < RW; ++k) {
      const int i = wid + TILE_WARPS * k;
      on[k] = i < n;
      sc[k] = on[k] ? a.scale[src_row[i]] : 1.f;
      m[k] = 0.f;
      sy[k] = 0.f;
      inv[k] = __frcp_rn(sc[k]);  // one reciprocal per voxel, then products
    }
    if (centre) {
#pragma unroll
      for (int k = 0; k < RW; ++k) {
        if (!on[k]) continue;  // warp-uniform
        const float4* row4 = reinterpret_cast<const float4*>(Ys + (size_t)(wid + TILE_WARPS * k) * ld);
        for (int q = lane; q < nq; q += 32) {
          const float4 y = row4[q];
          m[k] += ((y.x + y.y) + y.z) + y.w;
        }
      }
      warp_sum_n(m);
#pragma unroll
      for (int k = 0; k < RW; ++k) m[k] = on[k] ? m[k] / (float)T : 0.f;
    }
#pragma unroll
    for (int k = 0; k < RW; ++k) {
      if (!on[k]) continue;
      float4* row4 = reinterpret_cast<float4*>(Ys + (size_t)(wid + TILE_WARPS * k) * ld);
      const float mk = m[k], ik = inv[k];
      for (int q = lane; q < nq; q += 32) {
        const float4 y = row4[q];
        const int t = 4 * q;
        float4 r;  // whole quads when T % 4 == 0: no padding inside the row
        r.x = __fmul_rn(__fsub_rn(y.x, mk), ik);
        r.y = (vec || t + 1 < T) ? __fmul_rn(__fsub_rn(y.y, mk), ik) : 0.f;
        r.z = (vec || t + 2 < T) ? __fmul_rn(__fsub_rn(y.z, mk), ik) : 0.f;
        r.w = (vec || t + 3 < T) ? __fmul_rn(__fsub_rn(y.w, mk), ik) : 0.f;
        row4[q] = r;
        sy[k] += ((r.x + r.y) + r.z) + r.w;
      }
    }
    warp_sum_n(sy);
    if (lane == 0) {
#pragma unroll
      for (int k = 0; k < RW; ++k) {
        const int i = wid + TILE_WARPS * k;
        st[i] = m[k];
        st[TILE_V + i] = sc[k];
        st[2 * TILE_V + i] = on[k] ? sy[k] / (float)T : 0.f;
      }
    }
  }
  __syncthreads();

  const float* Gg = a.G + (size_t)g * K * LT;
  const float* Xt = a.Xt + (size_t)design_of(a, g) * K * LT;
  // b0 = G'y; SS_tot; r = y - X b0. Warp w takes the rows 4w .. 4w+3 in the
  // row passes, lanes over quads.
  tile_project(Gg, LT, Ys, ld, K, C0);
#pragma unroll
  for (int i = 0; i < TILE_SUB_VB; ++i) {
    const int l = TILE_SUB_VB * wid + i;
    const float mu = st[2 * TILE_V + l];
    const float4* r4 = reinterpret_cast<const float4*>(Ys + (size_t)l * ld);
    float sst = 0.f;
    for (int q = lane; q < nq; q += 32) {
      const float4 r = r4[q];
      const int t = 4 * q;
      float d = r.x - mu;
      sst = fmaf(d, d, sst);
      d = (vec || t + 1 < T) ? r.y - mu : 0.f;
      sst = fmaf(d, d, sst);
      d = (vec || t + 2 < T) ? r.z - mu : 0.f;
      sst = fmaf(d, d, sst);
      d = (vec || t + 3 < T) ? r.w - mu : 0.f;
      sst = fmaf(d, d, sst);
    }
    sst = warp_sum(sst);
    if (lane == 0) st[4 * TILE_V + l] = sst;
  }
  tile_subtract_any(Xt, LT, C0, Ys, ld, K);
  // the refinement d = G'r; SS_res and the unwhitened outputs
  tile_project(Gg, LT, Ys, ld, K, C1);
#pragma unroll
  for (int i = 0; i < TILE_SUB_VB; ++i) {
    const int l = TILE_SUB_VB * wid + i;
    const float4* r4 = reinterpret_cast<const float4*>(Ys + (size_t)l * ld);
    float ssr = 0.f;
    for (int q = lane; q < nq; q += 32) {
      const float4 r = r4[q];
      ssr = fmaf(r.x, r.x, ssr);
      ssr = fmaf(r.y, r.y, ssr);
      ssr = fmaf(r.z, r.z, ssr);
      ssr = fmaf(r.w, r.w, ssr);
    }
    ssr = warp_sum(ssr);
    if (lane == 0) st[3 * TILE_V + l] = ssr;
    if (l < n && (a.resid || a.pred)) {  // warp-uniform
      const int v = a.order[j0 + l];
      const float m = st[l], sc = st[TILE_V + l];
      // [V][T] rows: 16-byte words when T % 4 == 0, single samples otherwise
      auto put = [&](float* row, int q, float4 x) {
        if (vec) {
          reinterpret_cast<float4*>(row)[q] = x;
          return;
        }
        const int t = 4 * q;
        row[t] = x.x;
        if (t + 1 < T) row[t + 1] = x.y;
        if (t + 2 < T) row[t + 2] = x.z;
        if (t + 3 < T) row[t + 3] = x.w;
      };
      for (int q = lane; q < nq; q += 32) {
        if (a.resid) {
          const float4 r = r4[q];
          put(a.resid + (size_t)v * T, q, make_float4(r.x * sc, r.y * sc, r.z * sc, r.w * sc));
        }
        if (a.pred) {  // X b, b = b0 + d
          float4 p = make_float4(0.f, 0.f, 0.f, 0.f);
          for (int j = 0; j < K; ++j) {
            const float bj = C0[j * TILE_V + l] + C1[j * TILE_V + l];
            const float4 xj = __ldg(reinterpret_cast<const float4*>(Xt + (size_t)j * LT) + q);
            p.x = fmaf(xj.x, bj, p.x);
            p.y = fmaf(xj.y, bj, p.y);
            p.z = fmaf(xj.z, bj, p.z);
            p.w = fmaf(xj.w, bj, p.w);
          }
          put(a.pred + (size_t)v * T, q, make_float4(fmaf(p.x, sc, m), fmaf(p.y, sc, m), fmaf(p.z, sc, m),
                                                     fmaf(p.w, sc, m)));
        }
      }
    }
  }
  __syncthreads();
  float4* rr = reinterpret_cast<float4*>(Ys + (size_t)lane * ld);

  if (a.band_coef) {
    // the banded R's whitening: one lane per voxel over the whole series, in
    // place, and the whitened sum of squares
    if (wid == 0) {
      float* row = Ys + (size_t)lane * ld;
      band_whiten(a, pair_of(a, g), row, row, T);
      float ssw = 0.f;
      for (int t = 0; t < T; ++t) ssw = fmaf(row[t], row[t], ssw);
      st[5 * TILE_V + lane] = ssw;
    }
    __syncthreads();
  } else {
  // whitened residual by segments of the time axis
  const int SQ = (nq + TILE_WARPS - 1) / TILE_WARPS;
  const int s0 = min(T, wid * SQ * 4), s1 = min(T, (wid + 1) * SQ * 4);
  const float4* cf = reinterpret_cast<const float4*>(a.coef) + (size_t)pair_of(a, g) * T;
  float rp = s0 > 0 ? Ys[(size_t)lane * ld + s0 - 1] : 0.f;
  __syncthreads();
  {
    float vp = 0.f, H = 1.f;
    for (int t = s0; t < s1; t += 4) {
      const float4 r = rr[t >> 2];
      const float rv[4] = {r.x, r.y, r.z, r.w};
      float o[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        if (t + k < s1) {  // s1 = T ends the last segment inside a quad
          const float4 q = __ldg(cf + t + k);
          const float z = fmaf(-q.x, rp, rv[k]);
          const float vt = fmaf(-q.y, vp, z);
          o[k] = vt;
          rp = rv[k];
          vp = vt;
          H *= -q.y;
        }
      }
      rr[t >> 2] = make_float4(o[0], o[1], o[2], o[3]);
    }
    vend[wid * TILE_V + lane] = vp;
    if (lane == 0) Hs[wid] = H;
  }
  __syncthreads();
  if (wid == 0) {
    float vin = 0.f;
    for (int k = 0; k < TILE_WARPS; ++k) {
      carry[k * TILE_V + lane] = vin;
      vin = fmaf(Hs[k], vin, vend[k * TILE_V + lane]);
    }
  }
  __syncthreads();
  {
    const float cin = carry[wid * TILE_V + lane];
    float h = 1.f, ssw = 0.f;
    for (int t = s0; t < s1; t += 4) {
      const float4 r = rr[t >> 2];
      const float rv[4] = {r.x, r.y, r.z, r.w};
      float o[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        if (t + k < s1) {
          const float4 q = __ldg(cf + t + k);
          h *= -q.y;
          const float wt = fmaf(h, cin, rv[k]) * q.w;
          ssw = fmaf(wt, wt, ssw);
          o[k] = wt;
        }
      }
      rr[t >> 2] = make_float4(o[0], o[1], o[2], o[3]);
    }
    red[wid * TILE_V + lane] = ssw;
  }
  __syncthreads();
  if (wid == 0) {
    float s = 0.f;
    for (int w = 0; w < TILE_WARPS; ++w) s += red[w * TILE_V + lane];
    st[5 * TILE_V + lane] = s;
  }
  __syncthreads();
  }

  if (x.lj_h > 0 && x.ljung_box) {
    // per-voxel statistics with the Ljung-Box lags: warp w takes voxels w, w + 8, ...
    float* b = betas + (size_t)wid * kp;
    for (int i = wid; i < n; i += TILE_WARPS) {
      const int v = a.order[j0 + i];
      for (int j = lane; j < K; j += 32) b[j] = C0[j * TILE_V + i] + C1[j * TILE_V + i];
      __syncwarp();
      gls_finish(a, x, v, g, b, Ys + (size_t)i * ld, st[3 * TILE_V + i], st[4 * TILE_V + i], st[5 * TILE_V + i],
                 st[i], st[TILE_V + i], bins + (size_t)wid * hb, Mq);
      __syncwarp();
    }
    return;
  }
  gls_finish_tile(a, g, j0, n, C0, C1, Ys, ld, st, red, Mq);
}

// Column-set statistics, one thread per voxel (the sets are a few small
// blocks; betas and sigma2 come back to the scaled series' units first, as
// the reference computes them before its unscale step)
__global__ void __launch_bounds__(256) set_stats_kernel(ffs_set_stats_args a) {
  const int v = blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= a.V) return;
  const int p = a.best[v];
  const int dsg = a.design ? a.design[v] : 0;
  const size_t key = a.design ? (size_t)dsg * a.n_pairs + p : (size_t)p;
  const float* Fm = a.Fsets + key * a.msum;
  const float* Cm = a.Csets + (size_t)dsg * a.msum;
  const float sc = a.scale[v];
  const float* bv = a.betas + (size_t)v * a.K;
  const float s2 = __fdiv_rn(a.sigma2[v], sc * sc);
  size_t off = 0;
  for (int g = 0; g < a.n_sets; ++g) {
    const int b0 = a.set_ptr[g], q = a.set_ptr[g + 1] - b0;
    const int* ix = a.set_idx + b0;
    float quad = 0.f, cq = 0.f;
    for (int i = 0; i < q; ++i) {
      float fi = 0.f, ci = 0.f;
      for (int j = 0; j < q; ++j) {
        const float bj = __fdiv_rn(bv[ix[j]], sc);
        fi = fmaf(Fm[off + (size_t)i * q + j], bj, fi);
        ci = fmaf(Cm[off + (size_t)i * q + j], bj, ci);
      }
      const float bi = __fdiv_rn(bv[ix[i]], sc);
      quad = fmaf(bi, fi, quad);
      cq = fmaf(bi, ci, cq);
    }
    const size_t o = (size_t)v * a.n_out + a.set_col[g];
    a.set_fstats[o] = quad / ((float)q * s2 + 1e-30f);
    a.set_sd[o] = sqrtf(fmaxf(cq, 0.f)) * sc;
    a.set_coef[o] = q == 1 ? bv[ix[0]] : __int_as_float(0x7fc00000);
    off += (size_t)q * q;
  }
}

// ------------------------------------------------------------------ -dsort
// One warp per voxel. Per-warp shared memory (floats): the scaled series ys,
// the residual r, the whitened series / residual w [T] each; D and D_w
// [q][T] each; then the small arrays of ds_layout.
constexpr int DS_WARPS = 4;

struct DsLayout {
  int ys, r, w, D, Dw, b0, Py, bx, H, PD, HS, S, Si, bd, e, u, FH, W, blk, bins, total;
};

__host__ __device__ inline DsLayout ds_layout(int T, int K, int q, int n_f, int ns_max, int h) {
  DsLayout l;
  int o = 0;
  auto take = [&](int n) { const int at = o; o += (n + 3) & ~3; return at; };
  l.ys = take(T); l.r = take(T); l.w = take(T); l.D = take(q * T); l.Dw = take(q * T);
  l.b0 = take(K); l.Py = take(K); l.bx = take(K); l.H = take(K * q); l.PD = take(K * q); l.HS = take(K * q);
  l.S = take(q * q); l.Si = take(q * q); l.bd = take(q); l.e = take(q); l.u = take(n_f > q ? n_f : q);
  const int blk = ns_max * ns_max + 2 * ns_max;  // a column set's block, b_S and the solve; q for the F step
  l.FH = take(n_f * q); l.W = take(q * q); l.blk = take(blk > q ? blk : q); l.bins = take(h + 1);
  l.total = o;
  return l;
}

// In-place Cholesky of the n x n matrix M (one thread), L in the lower
// triangle; false if a pivot is not positive.
__device__ bool chol_small(float* M, int n) {
  for (int k = 0; k < n; ++k) {
    float d = M[k * n + k];
    for (int j = 0; j < k; ++j) d = fmaf(-M[k * n + j], M[k * n + j], d);
    if (!(d > 0.f)) return false;
    const float lk = sqrtf(d);
    M[k * n + k] = lk;
    for (int i = k + 1; i < n; ++i) {
      float x = M[i * n + k];
      for (int j = 0; j < k; ++j) x = fmaf(-M[i * n + j], M[k * n + j], x);
      M[i * n + k] = x / lk;
    }
  }
  return true;
}

// x := (L L')^-1 x for the factor L of chol_small (one thread)
__device__ void chol_solve_small(const float* L, int n, float* x) {
  for (int i = 0; i < n; ++i) {
    float v = x[i];
    for (int j = 0; j < i; ++j) v = fmaf(-L[i * n + j], x[j], v);
    x[i] = v / L[i * n + i];
  }
  for (int i = n - 1; i >= 0; --i) {
    float v = x[i];
    for (int j = i + 1; j < n; ++j) v = fmaf(-L[j * n + i], x[j], v);
    x[i] = v / L[i * n + i];
  }
}

// L^-1 x of one series by the whole warp: out[t] = (z_t - m_t v_{t-1}) /
// sqrt(D_t), z_t = x_t - c_t x_{t-1} (coef (c, m, ., 1/sqrt D), c = m = 0 at
// run starts). Lane l takes the segment [l S, (l + 1) S) of the time axis:
// it runs the recursion from v = 0 (z needs only x of the previous sample),
// the warp composes the segments' affine maps v_out = E + H v_in (H the
// product of -m over the segment) in a shuffle scan, and a second pass adds
// each segment's carry-in times the running product. x and out do not overlap.
__device__ void whiten_warp(const float4* __restrict__ cf, const float* x, float* out, int T) {
  const int lane = threadIdx.x & 31;
  const int seg = (T + 31) >> 5;
  const int s0 = min(T, lane * seg), s1 = min(T, s0 + seg);
  float xp = s0 > 0 ? x[s0 - 1] : 0.f;
  float vp = 0.f, H = 1.f;
  for (int t = s0; t < s1; ++t) {
    const float4 q = __ldg(cf + t);
    const float xt = x[t];
    const float v = fmaf(-q.y, vp, fmaf(-q.x, xp, xt));
    out[t] = v;
    xp = xt;
    vp = v;
    H *= -q.y;
  }
  float E = vp;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const float Hp = __shfl_up_sync(0xffffffffu, H, o), Ep = __shfl_up_sync(0xffffffffu, E, o);
    if (lane >= o) {
      E = fmaf(H, Ep, E);
      H *= Hp;
    }
  }
  float vin = __shfl_up_sync(0xffffffffu, E, 1);
  if (lane == 0) vin = 0.f;
  float h = 1.f;
  for (int t = s0; t < s1; ++t) {
    const float4 q = __ldg(cf + t);
    h *= -q.y;
    out[t] = fmaf(h, vin, out[t]) * q.w;
  }
  __syncwarp();
}

// L^-1 x of one series for the dsort GLS: the exact R's recurrence by the
// whole warp (whiten_warp), or AFNI's banded R by lane 0 (band_whiten_rows).
// x and out do not overlap.
__device__ void whiten_dsort(const ffs_dsort_args& a, int p, const float4* __restrict__ cf, const float* x,
                             float* out, int T) {
  if (a.band_coef) {
    __syncwarp();  // x was written by every lane
    if ((threadIdx.x & 31) == 0)
      band_whiten_rows(a.band_coef + (size_t)p * T * a.band_w, a.band_w, a.band[p], x, out, T);
    __syncwarp();
  } else {
    whiten_warp(cf, x, out, T);
  }
}

// QB: the projection loop's unrolled bound on q (q itself for 1..4, the
// maximum otherwise), so that small q issues no predicated-off work
template <int QB>
__global__ void __launch_bounds__(DS_WARPS * 32) gls_dsort_kernel(ffs_dsort_args a, int n_f, int ns_max) {
  extern __shared__ float dsm[];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int v = blockIdx.x * DS_WARPS + wid;
  if (v >= a.V) return;  // warp-uniform
  const int T = a.T, K = a.K, q = a.q, LT = ld_t(T);
  const DsLayout L = ds_layout(T, K, q, n_f, ns_max, a.lj_h);
  float* sm = dsm + (size_t)wid * L.total;
  float *ys = sm + L.ys, *r = sm + L.r, *w = sm + L.w, *Ds = sm + L.D, *Dw = sm + L.Dw;
  float *b0 = sm + L.b0, *Py = sm + L.Py, *bx = sm + L.bx, *H = sm + L.H, *PD = sm + L.PD, *HS = sm + L.HS;
  float *S = sm + L.S, *Si = sm + L.Si, *bd = sm + L.bd, *ev = sm + L.e, *u = sm + L.u, *FH = sm + L.FH;
  float *W = sm + L.W, *blk = sm + L.blk, *bins = sm + L.bins;
  const int g = a.best[v];
  const int p = a.n_pairs > 0 ? g % a.n_pairs : g;
  const int dsg = a.n_pairs > 0 ? g / a.n_pairs : 0;
  const float* Gg = a.G + (size_t)g * K * LT;
  const float* Ug = a.U + (size_t)g * K * LT;
  const float* Xt = a.Xt + (size_t)dsg * K * LT;
  const float4* cf = reinterpret_cast<const float4*>(a.coef) + (size_t)p * T;
  const float sc = a.scale[v];

  // scaled series and the voxel's regressors
  float sy = 0.f;
  for (int t = lane; t < T; t += 32) {
    const float y = __fdiv_rn(a.Y[(size_t)v * T + t], sc);
    ys[t] = y;
    sy += y;
  }
  for (int i = lane; i < q * T; i += 32) Ds[i] = a.D[(size_t)v * q * T + i];
  const float mean = warp_sum(sy) / (float)T;
  __syncwarp();

  // G'y, U'y, G'D, U'D (lanes over t)
  for (int j = 0; j < K; ++j) {
    const float* gr = Gg + (size_t)j * LT;
    const float* ur = Ug + (size_t)j * LT;
    float ag = 0.f, au = 0.f;
    float hg[QB], hu[QB];
#pragma unroll
    for (int k = 0; k < QB; ++k) hg[k] = hu[k] = 0.f;
#pragma unroll 4
    for (int t = lane; t < T; t += 32) {
      const float gt = gr[t], ut = ur[t];
      ag = fmaf(gt, ys[t], ag);
      au = fmaf(ut, ys[t], au);
#pragma unroll
      for (int k = 0; k < QB; ++k)
        if (k < q) {
          hg[k] = fmaf(gt, Ds[k * T + t], hg[k]);
          hu[k] = fmaf(ut, Ds[k * T + t], hu[k]);
        }
    }
    ag = warp_sum(ag);
    au = warp_sum(au);
    if (lane == 0) {
      b0[j] = ag;
      Py[j] = au;
    }
#pragma unroll
    for (int k = 0; k < QB; ++k)
      if (k < q) {
        const float x = warp_sum(hg[k]), y = warp_sum(hu[k]);
        if (lane == 0) {
          H[j * q + k] = x;
          PD[j * q + k] = y;
        }
      }
  }
  // whitened y (into w) and D
  whiten_dsort(a, p, cf, ys, w, T);
  for (int k = 0; k < q; ++k) whiten_dsort(a, p, cf, Ds + k * T, Dw + k * T, T);
  // D_w'D_w and D_w'y_w
  for (int k = 0; k < q; ++k) {
    for (int l = 0; l <= k; ++l) {
      float acc = 0.f;
      for (int t = lane; t < T; t += 32) acc = fmaf(Dw[k * T + t], Dw[l * T + t], acc);
      acc = warp_sum(acc);
      if (lane == 0) {
        float x = acc;
        for (int j = 0; j < K; ++j) x = fmaf(-PD[j * q + k], PD[j * q + l], x);
        S[k * q + l] = S[l * q + k] = x + (k == l ? 1e-8f : 0.f);
      }
    }
    float acc = 0.f;
    for (int t = lane; t < T; t += 32) acc = fmaf(Dw[k * T + t], w[t], acc);
    acc = warp_sum(acc);
    if (lane == 0) {
      float x = acc;
      for (int j = 0; j < K; ++j) x = fmaf(-PD[j * q + k], Py[j], x);
      ev[k] = x;
    }
  }
  __syncwarp();
  // S^-1 (Cholesky on lane 0), b_D = S^-1 e
  if (lane == 0) {
    for (int i = 0; i < q * q; ++i) W[i] = S[i];
    if (!chol_small(W, q)) {
      if (a.status) *a.status = 1;
      for (int i = 0; i < q * q; ++i) W[i] = 0.f;
      for (int i = 0; i < q; ++i) W[i * q + i] = 1.f;  // identity factor: b_D = e, finite
    }
    for (int c = 0; c < q; ++c) {
      for (int i = 0; i < q; ++i) u[i] = (i == c) ? 1.f : 0.f;
      chol_solve_small(W, q, u);
      for (int i = 0; i < q; ++i) Si[i * q + c] = u[i];
    }
    for (int i = 0; i < q; ++i) {
      float x = 0.f;
      for (int k = 0; k < q; ++k) x = fmaf(Si[i * q + k], ev[k], x);
      bd[i] = x;
    }
  }
  __syncwarp();
  // b_X = b0 - H b_D; HS = H S^-1 (lanes over columns)
  for (int j = lane; j < K; j += 32) {
    float x = b0[j];
    for (int k = 0; k < q; ++k) x = fmaf(-H[j * q + k], bd[k], x);
    bx[j] = x;
    for (int k = 0; k < q; ++k) {
      float y = 0.f;
      for (int l = 0; l < q; ++l) y = fmaf(H[j * q + l], Si[l * q + k], y);
      HS[j * q + k] = y;
    }
  }
  __syncwarp();
  // unwhitened residual, R^2 sums
  float ssr = 0.f, sst = 0.f;
#pragma unroll 2
  for (int t = lane; t < T; t += 32) {
    float x = ys[t];
    for (int j = 0; j < K; ++j) x = fmaf(-Xt[(size_t)j * LT + t], bx[j], x);
    for (int k = 0; k < q; ++k) x = fmaf(-Ds[k * T + t], bd[k], x);
    r[t] = x;
    ssr = fmaf(x, x, ssr);
    const float dy = ys[t] - mean;
    sst = fmaf(dy, dy, sst);
  }
  ssr = warp_sum(ssr);
  sst = warp_sum(sst);
  __syncwarp();
  // whitened residual and its sum of squares (blocks of 32 terms)
  whiten_dsort(a, p, cf, r, w, T);
  double ssw_d = 0.0;
  for (int t0 = 0; t0 < T; t0 += 32) {
    const float x = t0 + lane < T ? w[t0 + lane] : 0.f;
    ssw_d += (double)warp_sum(x * x);
  }
  const float ssw = (float)ssw_d;
  const float s2 = ssw / (float)a.dof;

  // t of the base and the D columns
  for (int j = lane; j < K; j += 32) {
    float c = a.Adiag[(size_t)g * K + j];
    for (int k = 0; k < q; ++k) c = fmaf(HS[j * q + k], H[j * q + k], c);
    const float se = sqrtf(s2 * c);
    a.betas[(size_t)v * K + j] = bx[j] * sc;
    a.tstats[(size_t)v * K + j] = bx[j] / (se + 1e-10f);
  }
  for (int k = lane; k < q; k += 32) {
    const float se = sqrtf(s2 * Si[k * q + k]);
    a.dbetas[(size_t)v * q + k] = bd[k] * sc;
    a.dtstats[(size_t)v * q + k] = bd[k] / (se + 1e-10f);
  }
  // F over the task (or all base) columns: inv(A_t + H_t S^-1 H_t' + 1e-8 I)
  // by the Woodbury identity around Fm = inv(A_t + 1e-8 I) (X_w'X_w for the
  // full model): quad = b'Fm b - u'(S + H_t'Fm H_t)^-1 u, u = H_t'Fm b
  const float* Fm = a.n_task > 0 ? a.Ftask + (size_t)g * n_f * n_f : a.XtX + (size_t)g * K * K;
  float quad0 = 0.f;
  for (int i = lane; i < n_f; i += 32) {
    float fb = 0.f;
    for (int l = 0; l < n_f; ++l) fb = fmaf(Fm[i * n_f + l], bx[a.n_task > 0 ? a.task_idx[l] : l], fb);
    quad0 = fmaf(bx[a.n_task > 0 ? a.task_idx[i] : i], fb, quad0);
    for (int k = 0; k < q; ++k) {
      float fh = 0.f;
      for (int l = 0; l < n_f; ++l) fh = fmaf(Fm[i * n_f + l], H[(a.n_task > 0 ? a.task_idx[l] : l) * q + k], fh);
      FH[i * q + k] = fh;
    }
  }
  quad0 = warp_sum(quad0);
  __syncwarp();
  if (lane == 0) {
    for (int k = 0; k < q; ++k) {
      float uk = 0.f;
      for (int i = 0; i < n_f; ++i) uk = fmaf(FH[i * q + k], bx[a.n_task > 0 ? a.task_idx[i] : i], uk);
      u[k] = uk;
      for (int l = 0; l < q; ++l) {
        float x = S[k * q + l];
        for (int i = 0; i < n_f; ++i) x = fmaf(H[(a.n_task > 0 ? a.task_idx[i] : i) * q + k], FH[i * q + l], x);
        W[k * q + l] = x;
      }
    }
    float quad = quad0;
    for (int k = 0; k < q; ++k) blk[k] = u[k];
    if (chol_small(W, q)) {
      chol_solve_small(W, q, blk);
      for (int k = 0; k < q; ++k) quad = fmaf(-u[k], blk[k], quad);
    }
    a.fstats[v] = quad / (s2 * (float)n_f + 1e-30f);
    a.sigma2[v] = s2 * sc * sc;
    const bool deg = sst <= 1e-10f;
    a.r2[v] = deg ? 0.f : fminf(1.0f - ssr / fmaxf(sst, 1e-10f), 1.0f);
  }
  // GLT on the base block: var = s2 (c A c' + (H'c)' S^-1 (H'c))
  for (int c = lane; c < a.n_glt; c += 32) {
    const float* gc = a.glt + (size_t)c * K;
    float cb = 0.f;
    for (int j = 0; j < K; ++j) cb = fmaf(gc[j], bx[j], cb);
    float hc[FFS_DSORT_QMAX];
    for (int k = 0; k < q; ++k) {
      float x = 0.f;
      for (int j = 0; j < K; ++j) x = fmaf(H[j * q + k], gc[j], x);
      hc[k] = x;
    }
    float var = a.glt_var[(size_t)g * a.n_glt + c];
    for (int k = 0; k < q; ++k)
      for (int l = 0; l < q; ++l) var = fmaf(hc[k] * Si[k * q + l], hc[l], var);
    var *= s2;
    a.cbeta[(size_t)v * a.n_glt + c] = cb * sc;
    a.ct[(size_t)v * a.n_glt + c] = cb / (sqrtf(fmaxf(var, 0.f)) + 1e-10f);
  }
  // series outputs
  if (a.resid || a.resid_w || a.pred) {
    for (int t = lane; t < T; t += 32) {
      if (a.resid) a.resid[(size_t)v * T + t] = r[t] * sc;
      if (a.resid_w) a.resid_w[(size_t)v * T + t] = w[t] * sc;
      if (a.pred) a.pred[(size_t)v * T + t] = (ys[t] - r[t]) * sc;
    }
  }
  // column sets over [X | D]: the voxel's block of the covariance, + 1e-8 I
  for (int sg = 0; sg < a.n_sets; ++sg) {
    const int b0i = a.set_ptr[sg], ns = a.set_ptr[sg + 1] - b0i;
    const int* ix = a.set_idx + b0i;
    float* B = blk;
    float* bs = blk + ns * ns;
    for (int e = lane; e < ns * ns; e += 32) {
      const int i = ix[e / ns], j = ix[e % ns];
      float x;
      if (i < K && j < K) {
        x = a.Afull[(size_t)g * K * K + i * K + j];
        for (int k = 0; k < q; ++k) x = fmaf(HS[i * q + k], H[j * q + k], x);
      } else if (i < K) {
        x = -HS[i * q + (j - K)];
      } else if (j < K) {
        x = -HS[j * q + (i - K)];
      } else {
        x = Si[(i - K) * q + (j - K)];
      }
      B[e] = x + (e / ns == e % ns ? 1e-8f : 0.f);
    }
    for (int i = lane; i < ns; i += 32) bs[i] = ix[i] < K ? bx[ix[i]] : bd[ix[i] - K];
    __syncwarp();
    // SD over time of the centred [X | D]_S b_S (two passes)
    float sum = 0.f;
    for (int t = lane; t < T; t += 32) {
      float x = 0.f;
      for (int i = 0; i < ns; ++i) {
        const int c = ix[i];
        const float col = c < K ? Xt[(size_t)c * LT + t] - a.xmean[(size_t)dsg * K + c] : Ds[(c - K) * T + t];
        x = fmaf(col, bs[i], x);
      }
      r[t] = x;  // the residual is no longer needed
      sum += x;
    }
    const float mu = warp_sum(sum) / (float)T;
    float ss = 0.f;
    for (int t = lane; t < T; t += 32) {
      const float d = r[t] - mu;
      ss = fmaf(d, d, ss);
    }
    ss = warp_sum(ss);
    __syncwarp();
    if (lane == 0) {
      const size_t o = (size_t)v * a.n_set_out + a.set_col[sg];
      float* x = bs + ns;
      for (int i = 0; i < ns; ++i) x[i] = bs[i];
      float quad = 0.f;
      if (chol_small(B, ns)) {
        chol_solve_small(B, ns, x);
        for (int i = 0; i < ns; ++i) quad = fmaf(bs[i], x[i], quad);
      } else {
        quad = __int_as_float(0x7fc00000);
      }
      a.set_fstats[o] = quad / ((float)ns * s2 + 1e-30f);
      a.set_sd[o] = sqrtf(ss / (float)T) * sc;
      a.set_coef[o] = ns == 1 ? bs[0] * sc : __int_as_float(0x7fc00000);
    }
    __syncwarp();
  }
  // Ljung-Box of the whitened residual
  if (a.lj_h > 0 && a.ljung_box) {
    const float lb = ljung_box_warp(a.lj_h, a.lj_tau, a.lj_w, w, T, ssw, bins);
    if (lane == 0) a.ljung_box[v] = lb;
  }
}

// tile_start[g] = sum over g' < g of ceil(count[g'] / GLS_TILE)
__global__ void gls_tile_scan(int P, const int* end, int* tile_start) {
  __shared__ int part[1024];
  // counts per thread-strided block, then a serial scan over 1024 partials
  const int tid = threadIdx.x;
  const int per = (P + blockDim.x - 1) / blockDim.x;
  int acc = 0;
  for (int g = tid * per; g < min(P, (tid + 1) * per); ++g)
    acc += (end[g] - (g ? end[g - 1] : 0) + GLS_TILE - 1) / GLS_TILE;
  part[tid] = acc;
  __syncthreads();
  if (tid == 0) {
    int run = 0;
    for (int i = 0; i < (int)blockDim.x; ++i) {
      const int c = part[i];
      part[i] = run;
      run += c;
    }
    tile_start[P] = run;
  }
  __syncthreads();
  int run = part[tid];
  for (int g = tid * per; g < min(P, (tid + 1) * per); ++g) {
    tile_start[g] = run;
    run += (end[g] - (g ? end[g - 1] : 0) + GLS_TILE - 1) / GLS_TILE;
  }
}

}  // namespace
}  // namespace ffsk

using namespace ffsk;

extern "C" int ffs_reml_gls_ex(const ffs_gls_args* a, int lj_h, const int* lj_tau, const float* lj_w,
                               float* ljung_box, void* stream) {
  clear_error();
  FFS_REQUIRE(a && a->V > 0 && a->T > 0 && a->K > 0 && a->dof > 0, "ffs_reml_gls: bad sizes");
  FFS_REQUIRE(a->Y && a->scale && a->Xt && a->best && a->coef && a->G && a->Adiag && a->XtX &&
                  a->a && a->b && a->betas && a->tstats && a->sigma2 && a->fstats && a->r2 && a->lam,
              "ffs_reml_gls: null buffer");
  FFS_REQUIRE(a->n_task == 0 || (a->task_idx && a->Ftask), "ffs_reml_gls: task columns need Ftask");
  FFS_REQUIRE((!a->center && !a->center_dev) || a->Gsum, "ffs_reml_gls: centring needs Gsum");
  FFS_REQUIRE(a->n_glt == 0 || (a->glt && a->glt_var && a->cbeta && a->ct), "ffs_reml_gls: GLT buffers");
  FFS_REQUIRE(lj_h >= 0 && lj_h <= a->T / 2, "ffs_reml_gls: Ljung-Box lag %d out of range", lj_h);
  FFS_REQUIRE(lj_h == 0 || (lj_w && ljung_box), "ffs_reml_gls: Ljung-Box buffers");
  const int ld_s = a->T + 1;
  const int kp = (a->K + 3) & ~3;
  const int hb = (lj_h + 4) & ~3;
  const size_t smem = sizeof(float) * GLS_WARPS * (size_t)(2 * ld_s + kp + hb);
  FFS_REQUIRE(smem <= 227 * 1024, "ffs_reml_gls: T=%d too long", a->T);
  FFS_CUDA(ensure_dyn_smem(reinterpret_cast<const void*>(gls_kernel), smem));
  GlsExtra x{lj_h, lj_tau, lj_w, ljung_box};
  gls_kernel<<<ceil_div(a->V, GLS_WARPS), GLS_WARPS * 32, smem, (cudaStream_t)stream>>>(*a, x, ld_s, kp, hb);
  return check_launch("gls_kernel");
}

extern "C" int ffs_reml_gls_grouped(const ffs_gls_args* a, int lj_h, const int* lj_tau, const float* lj_w,
                                    float* ljung_box, int P, const int* group_end, int* tile_start, void* stream) {
  clear_error();
  FFS_REQUIRE(a && a->V > 0 && a->T > 0 && a->K > 0 && a->dof > 0 && P > 0, "ffs_reml_gls_grouped: bad sizes");
  FFS_REQUIRE(a->order && group_end && tile_start, "ffs_reml_gls_grouped: needs order, group_end, tile_start");
  FFS_REQUIRE(a->Y && a->scale && a->Xt && a->best && a->coef && a->G && a->Adiag && a->XtX && a->a && a->b &&
                  a->betas && a->tstats && a->sigma2 && a->fstats && a->r2 && a->lam,
              "ffs_reml_gls_grouped: null buffer");
  FFS_REQUIRE(a->n_task == 0 || (a->task_idx && a->Ftask), "ffs_reml_gls_grouped: task columns need Ftask");
  FFS_REQUIRE((!a->center && !a->center_dev) || a->Gsum, "ffs_reml_gls_grouped: centring needs Gsum");
  FFS_REQUIRE(a->n_glt == 0 || (a->glt && a->glt_var && a->cbeta && a->ct), "ffs_reml_gls_grouped: GLT buffers");
  FFS_REQUIRE(lj_h >= 0 && lj_h <= a->T / 2, "ffs_reml_gls_grouped: Ljung-Box lag %d out of range", lj_h);
  FFS_REQUIRE(lj_h == 0 || (lj_w && ljung_box), "ffs_reml_gls_grouped: Ljung-Box buffers");
  const int ld = tile_ld(a->T);
  const int kp = (a->K + 3) & ~3;
  const int hb = (lj_h + 4) & ~3;
  const int nm = a->n_task > 0 ? a->n_task : a->K;
  const int msz = nm * nm <= 4096 ? nm * nm : 0;  // F matrix staged per tile when it is small
  const size_t smem = sizeof(float) * ((size_t)TILE_V * ld + 2 * (size_t)a->K * TILE_V +
                                       (1 + 2) * TILE_WARPS * TILE_V + TILE_V + 6 * TILE_V +
                                       (size_t)TILE_WARPS * (kp + hb) + msz);
  if (smem > 200 * 1024) {  // the tile does not fit: one warp per voxel
    return ffs_reml_gls_ex(a, lj_h, lj_tau, lj_w, ljung_box, stream);
  }
  cudaStream_t st = (cudaStream_t)stream;
  GlsExtra x{lj_h, lj_tau, lj_w, ljung_box};
  gls_tile_scan<<<1, 1024, 0, st>>>(P, group_end, tile_start);
  FFS_CUDA(ensure_dyn_smem(reinterpret_cast<const void*>(gls_tile_kernel), smem));
  const int max_tiles = ceil_div(a->V, GLS_TILE) + P;
  gls_tile_kernel<<<max_tiles, TILE_WARPS * 32, smem, st>>>(*a, x, group_end, tile_start, P, ld, kp, hb, msz);
  return check_launch("gls_tile_kernel");
}

extern "C" int ffs_reml_gls(const ffs_gls_args* a, void* stream) {
  return ffs_reml_gls_ex(a, 0, nullptr, nullptr, nullptr, stream);
}

extern "C" int ffs_reml_set_stats(const ffs_set_stats_args* a, void* stream) {
  clear_error();
  FFS_REQUIRE(a, "ffs_reml_set_stats: null args");
  FFS_REQUIRE(a->V >= 0 && a->K > 0 && a->n_sets >= 0 && a->n_out >= a->n_sets && a->msum >= 0,
              "ffs_reml_set_stats: V=%d K=%d n_sets=%d n_out=%d msum=%d", a->V, a->K, a->n_sets, a->n_out,
              a->msum);
  if (a->V == 0 || a->n_sets == 0) return FFS_OK;
  FFS_REQUIRE(a->set_ptr && a->set_idx && a->set_col && a->Fsets && a->Csets && a->best && a->betas &&
                  a->sigma2 && a->scale && a->set_fstats && a->set_sd && a->set_coef,
              "ffs_reml_set_stats: null buffer");
  FFS_REQUIRE(!a->design || a->n_pairs > 0, "ffs_reml_set_stats: design needs n_pairs");
  set_stats_kernel<<<ceil_div(a->V, 256), 256, 0, (cudaStream_t)stream>>>(*a);
  return check_launch("set_stats_kernel");
}

extern "C" int ffs_reml_gls_dsort(const ffs_dsort_args* a, void* stream) {
  clear_error();
  FFS_REQUIRE(a, "ffs_reml_gls_dsort: null args");
  FFS_REQUIRE(a->V >= 0 && a->T > 0 && a->K > 0 && a->q > 0 && a->q <= FFS_DSORT_QMAX && a->dof > 0,
              "ffs_reml_gls_dsort: V=%d T=%d K=%d q=%d (1..%d) dof=%d", a->V, a->T, a->K, a->q, FFS_DSORT_QMAX,
              a->dof);
  if (a->V == 0) return FFS_OK;
  FFS_REQUIRE(a->Y && a->scale && a->D && a->Xt && a->best && a->coef && a->G && a->U && a->Adiag && a->XtX &&
                  a->betas && a->tstats && a->dbetas && a->dtstats && a->sigma2 && a->fstats && a->r2,
              "ffs_reml_gls_dsort: null buffer");
  FFS_REQUIRE(a->n_task == 0 || (a->task_idx && a->Ftask), "ffs_reml_gls_dsort: task columns need task_idx, Ftask");
  FFS_REQUIRE(a->n_glt == 0 || (a->glt && a->glt_var && a->cbeta && a->ct), "ffs_reml_gls_dsort: GLT buffers");
  FFS_REQUIRE(a->n_sets == 0 || (a->set_ptr && a->set_idx && a->set_col && a->Afull && a->xmean && a->set_fstats &&
                                 a->set_sd && a->set_coef),
              "ffs_reml_gls_dsort: column sets need set_ptr, set_idx, set_col, Afull, xmean and outputs");
  FFS_REQUIRE(a->lj_h == 0 || (a->lj_w && a->ljung_box), "ffs_reml_gls_dsort: Ljung-Box buffers");
  FFS_REQUIRE(!a->band_coef || (a->band && a->band_w >= 1 && a->band_w <= FFS_BAND_MAX_W),
              "ffs_reml_gls_dsort: the banded R needs band and 1 <= band_w=%d <= %d", a->band_w, FFS_BAND_MAX_W);
  // the set sizes live on the device; a set of distinct columns of [X | D]
  // has at most K + q of them (the caller removes repeats)
  const int ns_max = a->n_sets > 0 ? a->K + a->q : 0;
  const int n_f = a->n_task > 0 ? a->n_task : a->K;
  const DsLayout L = ds_layout(a->T, a->K, a->q, n_f, ns_max, a->lj_h);
  const size_t per_warp = sizeof(float) * (size_t)L.total;
  FFS_REQUIRE(per_warp * DS_WARPS <= 200 * 1024, "ffs_reml_gls_dsort: T=%d K=%d q=%d need %zu bytes of shared memory",
              a->T, a->K, a->q, per_warp * DS_WARPS);
  const size_t smem = per_warp * DS_WARPS;
  const int nb = ceil_div(a->V, DS_WARPS);
  cudaStream_t st = (cudaStream_t)stream;
  switch (a->q) {
#define FFS_DSORT_LAUNCH(QB)                                                                  \
  FFS_CUDA(ensure_dyn_smem(reinterpret_cast<const void*>(gls_dsort_kernel<QB>), smem));      \
  gls_dsort_kernel<QB><<<nb, DS_WARPS * 32, smem, st>>>(*a, n_f, ns_max);                     \
  break;
    case 1: FFS_DSORT_LAUNCH(1)
    case 2: FFS_DSORT_LAUNCH(2)
    case 3: FFS_DSORT_LAUNCH(3)
    case 4: FFS_DSORT_LAUNCH(4)
    default: FFS_DSORT_LAUNCH(FFS_DSORT_QMAX)
#undef FFS_DSORT_LAUNCH
  }
  return check_launch("gls_dsort_kernel");
}
