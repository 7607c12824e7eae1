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

namespace ffsk {
namespace {

constexpr int GLS_WARPS = 4;

struct GlsExtra {
  int lj_h;             // Ljung-Box max lag (0: off)
  const int* lj_tau;    // [T] pseudo-time or NULL (plain index lags)
  const float* lj_w;    // [lj_h + 1] 1 / n_k for good bins, 0 otherwise
  float* ljung_box;     // [V]
};

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
  if (a.center) {
    float sm_ = 0.f;
    for (int t = lane; t < T; t += 32) sm_ += y[t];
    m = warp_sum(sm_) / (float)T;
  }
  for (int t = lane; t < T; t += 32) ys[t] = __fdiv_rn(__fsub_rn(y[t], m), sc);
  __syncwarp();

  // b0 = G' y
  for (int j = 0; j < K; ++j) {
    const float* gj = Gp + (size_t)j * T;
    float s = 0.f;
    for (int t = lane; t < T; t += 32) s = fmaf(gj[t], ys[t], s);
    s = warp_sum(s);
    if (lane == 0) beta[j] = s;
  }
  __syncwarp();
  // refinement: b += G' (y - X b)
  for (int t = lane; t < T; t += 32) {
    float acc = ys[t];
    for (int j = 0; j < K; ++j) acc = fmaf(-Xt[(size_t)j * T + t], beta[j], acc);
    r[t] = acc;
  }
  __syncwarp();
  for (int j = 0; j < K; ++j) {
    const float* gj = Gp + (size_t)j * T;
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
    for (int j = 0; j < K; ++j) acc = fmaf(-Xt[(size_t)j * T + t], beta[j], acc);
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
  const float4* cf = reinterpret_cast<const float4*>(a.coef) + (size_t)g * T;
  if (lane == 0) {
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
  if (a.resid_w) {
    for (int t = lane; t < T; t += 32) a.resid_w[(size_t)v * T + t] = ys[t] * sc;
  }
  const float sigma2 = ssw / (float)a.dof;

  // betas of the uncentred data: add (m/s) * G'1
  if (a.center) {
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
    const float* M = a.Ftask + (size_t)g * a.n_task * a.n_task;
    for (int k = lane; k < a.n_task; k += 32) {
      float s = 0.f;
      for (int l = 0; l < a.n_task; ++l) s = fmaf(M[k * a.n_task + l], beta[a.task_idx[l]], s);
      quad = fmaf(beta[a.task_idx[k]], s, quad);
    }
  } else {
    const float* M = a.XtX + (size_t)g * K * K;
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

  // Ljung-Box: c_k = sum r_j r_{j+k} / sum r^2, binned by time lag
  float lb = 0.f;
  if (x.lj_h > 0 && x.ljung_box) {
    const int h = x.lj_h;
    for (int k = lane; k <= h; k += 32) bins[k] = 0.f;
    __syncwarp();
    for (int k = 1; k <= h; ++k) {
      float part = 0.f;
      if (!x.lj_tau) {
        for (int t = lane; t + k < T; t += 32) part = fmaf(ys[t], ys[t + k], part);
        part = warp_sum(part);
        if (lane == 0) bins[k] += part;
      } else {
        for (int t = lane; t + k < T; t += 32) {
          const int dj = x.lj_tau[t + k] - x.lj_tau[t];
          if (dj > 0 && dj <= h) atomicAdd(bins + dj, ys[t] * ys[t + k]);
        }
      }
    }
    __syncwarp();
    if (lane == 0) {
      if (ssw >= 1e-10f && T >= 10) {
        double acc = 0.0;
        for (int k = 1; k <= h; ++k) {
          const double ck = (double)bins[k] / (double)ssw;
          acc += ck * ck * (double)x.lj_w[k];
        }
        acc *= (double)T * ((double)T + 2.0);
        lb = (float)fmin(acc, 1.0e10);
      }
      x.ljung_box[v] = lb;
    }
  }

  if (lane == 0) {
    const float q = a.n_task > 0 ? (float)a.n_task : (float)K;
    a.fstats[v] = quad / (sigma2 * q + 1e-10f);
    a.sigma2[v] = sigma2 * sc * sc;
    const bool deg = sst <= 1e-10f;
    const float r2 = 1.0f - ssr / fmaxf(sst, 1e-10f);
    a.r2[v] = deg ? 0.f : fminf(r2, 1.0f);
    const float af = a.a[g], bf = a.b[g];
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
  gls_voxel(a, x, v, g, a.G + (size_t)g * a.K * a.T, a.Xt, ys, ys + ld_s, ys + 2 * ld_s, ys + 2 * ld_s + kp);
}

// Tiles of up to GLS_TILE voxels that share one pair (voxels grouped by pair:
// order[end[g-1] .. end[g]) are pair g's, end[-1] = 0). The pair's G and the
// transposed design are staged in shared memory once per tile; tile_start[g]
// numbers the tiles of pair g. Blocks past the last tile exit.
constexpr int GLS_TILE = 32;
constexpr int GLS_TWARPS = 8;

__global__ void __launch_bounds__(GLS_TWARPS * 32) gls_tile_kernel(ffs_gls_args a, GlsExtra x, const int* end,
                                                                   const int* tile_start, int P, int ld_s, int kp,
                                                                   int hb) {
  extern __shared__ float sm[];
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
  const int KT = a.K * a.T;
  float* Gs = sm;
  float* Xs = sm + KT;
  const float* Gg = a.G + (size_t)g * KT;
  for (int i = threadIdx.x; i < KT; i += blockDim.x) {
    Gs[i] = Gg[i];
    Xs[i] = a.Xt[i];
  }
  __syncthreads();
  const int wid = threadIdx.x >> 5;
  float* ys = sm + 2 * (size_t)KT + (size_t)wid * (2 * ld_s + kp + hb);
  for (int i = wid; i < n; i += GLS_TWARPS) {
    const int v = a.order[j0 + i];
    gls_voxel(a, x, v, g, Gs, Xs, ys, ys + ld_s, ys + 2 * ld_s, ys + 2 * ld_s + kp);
    __syncwarp();
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
  FFS_REQUIRE(!a->center || a->Gsum, "ffs_reml_gls: centring needs Gsum");
  FFS_REQUIRE(a->n_glt == 0 || (a->glt && a->glt_var && a->cbeta && a->ct), "ffs_reml_gls: GLT buffers");
  FFS_REQUIRE(lj_h >= 0 && lj_h <= a->T / 2, "ffs_reml_gls: Ljung-Box lag %d out of range", lj_h);
  FFS_REQUIRE(lj_h == 0 || (lj_w && ljung_box), "ffs_reml_gls: Ljung-Box buffers");
  const int ld_s = a->T + 1;
  const int kp = (a->K + 3) & ~3;
  const int hb = (lj_h + 4) & ~3;
  const size_t smem = sizeof(float) * GLS_WARPS * (size_t)(2 * ld_s + kp + hb);
  FFS_REQUIRE(smem <= 227 * 1024, "ffs_reml_gls: T=%d too long", a->T);
  FFS_CUDA(cudaFuncSetAttribute(gls_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
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
  FFS_REQUIRE(!a->center || a->Gsum, "ffs_reml_gls_grouped: centring needs Gsum");
  FFS_REQUIRE(a->n_glt == 0 || (a->glt && a->glt_var && a->cbeta && a->ct), "ffs_reml_gls_grouped: GLT buffers");
  FFS_REQUIRE(lj_h >= 0 && lj_h <= a->T / 2, "ffs_reml_gls_grouped: Ljung-Box lag %d out of range", lj_h);
  FFS_REQUIRE(lj_h == 0 || (lj_w && ljung_box), "ffs_reml_gls_grouped: Ljung-Box buffers");
  const int ld_s = a->T + 1;
  const int kp = (a->K + 3) & ~3;
  const int hb = (lj_h + 4) & ~3;
  const size_t mats = sizeof(float) * 2 * (size_t)a->K * a->T;
  const size_t smem = mats + sizeof(float) * GLS_TWARPS * (size_t)(2 * ld_s + kp + hb);
  if (smem > 200 * 1024) {  // the pair's matrices do not fit: read them from global memory
    return ffs_reml_gls_ex(a, lj_h, lj_tau, lj_w, ljung_box, stream);
  }
  cudaStream_t st = (cudaStream_t)stream;
  GlsExtra x{lj_h, lj_tau, lj_w, ljung_box};
  gls_tile_scan<<<1, 1024, 0, st>>>(P, group_end, tile_start);
  FFS_CUDA(cudaFuncSetAttribute(gls_tile_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  const int max_tiles = ceil_div(a->V, GLS_TILE) + P;
  gls_tile_kernel<<<max_tiles, GLS_TWARPS * 32, smem, st>>>(*a, x, group_end, tile_start, P, ld_s, kp, hb);
  return check_launch("gls_tile_kernel");
}

extern "C" int ffs_reml_gls(const ffs_gls_args* a, void* stream) {
  return ffs_reml_gls_ex(a, 0, nullptr, nullptr, nullptr, stream);
}
