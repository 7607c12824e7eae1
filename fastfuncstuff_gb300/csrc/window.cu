// Learned-seeded refine: each voxel evaluates only the 5 x 5 lattice window
// around its proposed (a, b), with the same criterion as the full grid
// (fastfuncstuff/glm/arma.py:1983-2002, relative to the pair (0, 0)), and is
// flagged for the full-grid search when its best pair touches a valid lattice
// neighbour outside the window.
//
// One thread per voxel, voxels in the order given (grouped by window centre so
// that a warp reads the same pairs' coefficients). A window row (5 pairs with
// one a) is one pass over the voxel's series: per time point and pair, the AR
// filter, the recurrence, the sum of squares and the K-column projection.
#include "common.cuh"

namespace ffsk {
namespace {

constexpr int WIN = 5;

struct WinArgs {
  int V, T, K, P, p0;
  int n_a, n_b;
  const int* lattice;     // [n_a][n_b]
  const int* center;      // [V] ai * n_b + bi
  const int* order;       // [V] or NULL
  const float* yr_t;      // [T][V]
  const float4* coef;     // [P][T]
  const float* Ut;        // [P][T][K]
  const double* logdet_R;
  const double* logdet_XtX;
  int* best;
  float* dbest;
  double* crit0;
  int* fallback;
};

template <int KMAX>
__device__ void eval_row(const WinArgs& w, int v, const int* pr, int npr, float* rss_out, float& yy_out,
                         bool want_yy) {
  float vv[WIN], sb[WIN], st[WIN], acc[WIN][KMAX];
#pragma unroll
  for (int g = 0; g < WIN; ++g) {
    vv[g] = sb[g] = st[g] = 0.f;
#pragma unroll
    for (int j = 0; j < KMAX; ++j) acc[g][j] = 0.f;
  }
  float yp = 0.f, yyb = 0.f, yyt = 0.f;
  const int T = w.T, K = w.K;
  for (int t0 = 0; t0 < T; t0 += 32) {
    const int t1 = min(T, t0 + 32);
    for (int t = t0; t < t1; ++t) {
      const float y = w.yr_t[(size_t)t * w.V + v];
      yyb = fmaf(y, y, yyb);
#pragma unroll
      for (int g = 0; g < WIN; ++g) {
        if (g < npr) {
          const int p = pr[g];
          const float4 q = w.coef[(size_t)p * T + t];
          const float z = fmaf(-q.x, yp, y);
          vv[g] = fmaf(-q.y, vv[g], z);
          sb[g] = fmaf(vv[g] * q.z, vv[g], sb[g]);
          const float* u = w.Ut + ((size_t)p * T + t) * K;
#pragma unroll
          for (int j = 0; j < KMAX; ++j)
            if (j < K) acc[g][j] = fmaf(u[j], y, acc[g][j]);
        }
      }
      yp = y;
    }
#pragma unroll
    for (int g = 0; g < WIN; ++g) {
      st[g] += sb[g];
      sb[g] = 0.f;
    }
    yyt += yyb;
    yyb = 0.f;
  }
#pragma unroll
  for (int g = 0; g < WIN; ++g) {
    if (g < npr) {
      float pj = 0.f;
#pragma unroll
      for (int j = 0; j < KMAX; ++j) pj = fmaf(acc[g][j], acc[g][j], pj);
      rss_out[g] = fmaxf(st[g] - pj, 0.f);
    }
  }
  if (want_yy) yy_out = yyt;
}

template <int KMAX>
__global__ void __launch_bounds__(128) window_kernel(WinArgs w) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= w.V) return;
  const int v = w.order ? w.order[i] : i;
  const int c = w.center[v];
  const int ca = c / w.n_b, cb = c % w.n_b;
  const int wa = min(WIN, w.n_a), wb = min(WIN, w.n_b);
  const int a0 = min(max(ca - WIN / 2, 0), w.n_a - wa);
  const int b0 = min(max(cb - WIN / 2, 0), w.n_b - wb);
  const int Tk = w.T - w.K;
  const double c_p0 = w.logdet_R[w.p0] + w.logdet_XtX[w.p0];

  // reference pair (0, 0): y'y - ||Q0'y||^2
  float rss[WIN], yy = 0.f;
  int pr[WIN];
  pr[0] = w.p0;
  eval_row<KMAX>(w, v, pr, 1, rss, yy, true);
  const float rss0 = rss[0];
  const float den = rss0 + 1e-10f;

  int best = w.p0, ba = -1, bb = -1;
  float bl = INFINITY;
  for (int ra = 0; ra < wa; ++ra) {
    int npr = 0, col[WIN];
    for (int rb = 0; rb < wb; ++rb) {
      const int p = w.lattice[(a0 + ra) * w.n_b + b0 + rb];
      if (p >= 0) {
        col[npr] = b0 + rb;
        pr[npr++] = p;
      }
    }
    if (npr == 0) continue;
    eval_row<KMAX>(w, v, pr, npr, rss, yy, false);
    for (int g = 0; g < npr; ++g) {  // lattice order = pair order within the window
      const int p = pr[g];
      const float dc = (float)((w.logdet_R[p] + w.logdet_XtX[p]) - c_p0);
      const float d = dc + (float)Tk * log1pf((rss[g] - rss0) / den);
      if (d < bl) {
        bl = d;
        best = p;
        ba = a0 + ra;
        bb = col[g];
      }
    }
  }
  // edge test: a valid lattice neighbour of the best pair outside the window
  int fb = (ba < 0) ? 1 : 0;
  for (int da = -1; da <= 1 && !fb; ++da)
    for (int db = -1; db <= 1; ++db) {
      const int na = ba + da, nb = bb + db;
      if ((da == 0 && db == 0) || na < 0 || nb < 0 || na >= w.n_a || nb >= w.n_b) continue;
      const bool inside = na >= a0 && na < a0 + wa && nb >= b0 && nb < b0 + wb;
      if (!inside && w.lattice[na * w.n_b + nb] >= 0) {
        fb = 1;
        break;
      }
    }
  w.best[v] = best;
  w.dbest[v] = bl;
  w.crit0[v] = c_p0 + (double)Tk * log((double)rss0 + 1e-10);
  w.fallback[v] = fb;
}

// nearest lattice point of each proposal: centre index ai * n_b + bi
__global__ void center_kernel(int V, const float* prop, const float* a_axis, int n_a, const float* b_axis, int n_b,
                              int* center) {
  const int v = blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= V) return;
  const float pa = prop[2 * v], pb = prop[2 * v + 1];
  int ia = 0, ib = 0;
  float da = INFINITY, db = INFINITY;
  for (int i = 0; i < n_a; ++i) {
    const float d = fabsf(a_axis[i] - pa);
    if (d < da) { da = d; ia = i; }
  }
  for (int i = 0; i < n_b; ++i) {
    const float d = fabsf(b_axis[i] - pb);
    if (d < db) { db = d; ib = i; }
  }
  center[v] = ia * n_b + ib;
}

// U [P][K][T] -> Ut [P][T][K]
__global__ void transpose_u_kernel(int P, int K, int T, const float* U, float* Ut) {
  const size_t n = (size_t)P * K * T;
  for (size_t idx = blockIdx.x * (size_t)blockDim.x + threadIdx.x; idx < n; idx += (size_t)gridDim.x * blockDim.x) {
    const size_t p = idx / ((size_t)K * T), r = idx % ((size_t)K * T);
    const int j = (int)(r / T), t = (int)(r % T);
    Ut[(p * T + t) * K + j] = U[idx];
  }
}

}  // namespace
}  // namespace ffsk

using namespace ffsk;

extern "C" int ffs_reml_window(int V, int T, int K, int P, int p0, int n_a, int n_b, const int* lattice,
                               const int* center, const int* order, const float* yr_t, const float* coef,
                               const float* Ut, const double* logdet_R, const double* logdet_XtX, int* best,
                               float* dbest, double* crit0, int* fallback, void* stream) {
  clear_error();
  FFS_REQUIRE(V > 0 && T > 0 && K > 0 && P > 0 && n_a > 0 && n_b > 0, "ffs_reml_window: bad sizes");
  FFS_REQUIRE(p0 >= 0 && p0 < P, "ffs_reml_window: p0 out of range");
  FFS_REQUIRE(lattice && center && yr_t && coef && Ut && logdet_R && logdet_XtX && best && dbest && crit0 &&
                  fallback,
              "ffs_reml_window: null buffer");
  WinArgs w{V, T, K, P, p0, n_a, n_b, lattice, center, order, yr_t, reinterpret_cast<const float4*>(coef), Ut,
            logdet_R, logdet_XtX, best, dbest, crit0, fallback};
  cudaStream_t st = (cudaStream_t)stream;
  if (K <= 8) {
    window_kernel<8><<<ceil_div(V, 128), 128, 0, st>>>(w);
  } else if (K <= 24) {
    window_kernel<24><<<ceil_div(V, 128), 128, 0, st>>>(w);
  } else if (K <= 32) {
    window_kernel<32><<<ceil_div(V, 128), 128, 0, st>>>(w);
  } else {
    set_error("ffs_reml_window: K=%d above the 32 columns the windowed refine supports", K);
    return FFS_ERR_UNSUPPORTED;
  }
  return check_launch("window_kernel");
}

extern "C" int ffs_reml_centers(int V, const float* prop, const float* a_axis, int n_a, const float* b_axis, int n_b,
                                int* center, void* stream) {
  clear_error();
  FFS_REQUIRE(V > 0 && prop && a_axis && b_axis && center && n_a > 0 && n_b > 0, "ffs_reml_centers: bad arguments");
  center_kernel<<<ceil_div(V, 256), 256, 0, (cudaStream_t)stream>>>(V, prop, a_axis, n_a, b_axis, n_b, center);
  return check_launch("center_kernel");
}

extern "C" int ffs_transpose_u(int P, int K, int T, const float* U, float* Ut, void* stream) {
  clear_error();
  FFS_REQUIRE(P > 0 && K > 0 && T > 0 && U && Ut, "ffs_transpose_u: bad arguments");
  transpose_u_kernel<<<1024, 256, 0, (cudaStream_t)stream>>>(P, K, T, U, Ut);
  return check_launch("transpose_u_kernel");
}
