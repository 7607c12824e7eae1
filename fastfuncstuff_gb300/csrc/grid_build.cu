// K1: FP64 factorisation of the REML grid, one CTA per (a, b) pair.
//
// The ARMA(1,1) correlation of a run, R_ij = rho(|tau_i - tau_j|) with
// rho(0) = 1, rho(k) = lambda a^(k-1), becomes tridiagonal after the AR filter
// z_t = y_t - c_t y_{t-1}, c_t = a^(tau_t - tau_{t-1}) (c = 0 at a run start):
//   T_tt      = 1 + c_t^2 - 2 c_t rho(g_t)      (1 at a run start)
//   T_t,t-1   = rho(g_t) - c_t                  (g_t = tau_t - tau_{t-1})
// and every other entry is zero, censoring gaps included. Its LDL' factor
// (unit bidiagonal L~ with sub-diagonal m_t, diagonal D_t) gives the Cholesky
// factor of R exactly: chol(R) = A^-1 L~ D^1/2, A the unit bidiagonal AR filter.
// So diag(chol(R)) = sqrt(D_t) and log|R| = 2 sum log(sqrt(D_t) + 1e-10), the
// same quantity fastfuncstuff/glm/whiten.py:219-223 takes from a dense
// Cholesky, at O(T) cost instead of O(T^3).
//
// The design-dependent part follows fastfuncstuff/glm/arma.py:1459-1506:
// X_w = L^-1 X, Cholesky of X_w'X_w (QR when it is not positive definite),
// Q = X_w L_xtx^-T, logdet = 2 sum log(|diag| + 1e-10). On top of that the
// kernel emits U = L^-T Q (the projection that lets the search skip the
// whitening GEMM) and G = U L_xtx^-1 (the GLS solve), and the per-pair GLS
// constants of fastfuncstuff/glm/arma.py:4853-4905.
#include <mutex>

#include "common.cuh"

namespace ffsk {

namespace {

constexpr int GB_PF = 4;  // samples loaded ahead in the sequential recursions
// Threads per CTA (one (design, pair) item at a time); 128 measured no faster
// at K = 20 and slower at K = 130, where the Gram matrix and the O(K^3)
// phases use every thread.
constexpr int GB_THREADS = 256;

struct PairScratch {
  double* cm;  // [T][4]  c, m, D, 1/sqrt(D)
  double* Xw;  // [K][T]  whitened design, later U = L^-T Q
  double* Qm;  // [K][T]  Q
  double* Lx;  // [K][K]  Cholesky factor of X_w'X_w (lower, row-major)
  double* Li;  // [K][K]  its inverse
  double* A;   // [K][K]  (X_w'X_w)^-1
  double* S;   // [K][K]  scratch for the task block
};

__host__ __device__ inline size_t pair_doubles(int T, int K) {
  return (size_t)4 * T + (size_t)2 * K * T + (size_t)4 * K * K;
}

__device__ PairScratch scratch_of(double* work, int p, int T, int K) {
  PairScratch s;
  double* w = work + (size_t)p * pair_doubles(T, K);
  s.cm = w;
  s.Xw = s.cm + 4 * T;
  s.Qm = s.Xw + (size_t)K * T;
  s.Lx = s.Qm + (size_t)K * T;
  s.Li = s.Lx + (size_t)K * K;
  s.A = s.Li + (size_t)K * K;
  s.S = s.A + (size_t)K * K;
  return s;
}

__device__ double block_sum(double v, double* red) {
  v = warp_sum_d(v);
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  __syncthreads();
  if (lane == 0) red[wid] = v;
  __syncthreads();
  double t = 0.0;
  if (threadIdx.x < 32) {
    t = (threadIdx.x < (blockDim.x >> 5)) ? red[threadIdx.x] : 0.0;
    t = warp_sum_d(t);
    if (threadIdx.x == 0) red[0] = t;
  }
  __syncthreads();
  return red[0];
}

// 1/sqrt(d) by the Newton-Raphson iteration r <- r + r (1 - d r^2) / 2 from
// the fp32 estimate (relative error about 2^-22; each step squares it, so two
// steps reach FP64 rounding). On this GPU an FP64 square root or division
// takes about ten dependent FMAs' time; the factorisations below have one of
// each per column on their critical path. Outside the range where the fp32
// estimate is a normal number, the plain expression.
__device__ __forceinline__ double rsqrt_newton(double d) {
  if (!(d > 1e-30 && d < 1e30)) return 1.0 / sqrt(d);
  double r = (double)rsqrtf((float)d);
#pragma unroll
  for (int k = 0; k < 2; ++k) {
    const double h = d * r;
    r = fma(0.5 * r, fma(-h, r, 1.0), r);
  }
  return r;
}

// Exact float -> double by its bit fields (sign, exponent rebiased by
// 1023 - 127 = 896, mantissa shifted into place), on the integer pipe;
// zeros, subnormals, infinities and NaNs take the hardware conversion.
__device__ __forceinline__ double f2d_exact(float x) {
  const uint32_t u = __float_as_uint(x);
  const uint32_t ax = u & 0x7fffffffu;
  if (ax - 0x00800000u >= 0x7f000000u) return (double)x;
  const uint32_t hi = (u & 0x80000000u) | ((ax >> 3) + (896u << 20));
  return __hiloint2double((int)hi, (int)(ax << 29));
}

// (i, j), j <= i, of the packed lower-triangle index e = i (i + 1) / 2 + j
__device__ __forceinline__ void tri_index(int e, int& i, int& j) {
  int r = (int)((sqrtf(8.f * (float)e + 1.f) - 1.f) * 0.5f);
  while (r > 0 && r * (r + 1) / 2 > e) --r;
  while ((r + 1) * (r + 2) / 2 <= e) ++r;
  i = r;
  j = e - r * (r + 1) / 2;
}

// A Gram entry sum_t x_i[t] x_j[t] as four interleaved FP64 chains (t mod 4),
// added pairwise at the end: a quarter of the dependent-FMA latency of one
// chain, and a fixed operation order, so every kernel that forms a Gram entry
// through Dot4 gets the same bits. run() continues the chains over n further
// samples; every run but the last must cover a multiple of 4 samples.
struct Dot4 {
  double s0 = 0.0, s1 = 0.0, s2 = 0.0, s3 = 0.0;
  __device__ __forceinline__ void run(const double* xi, const double* xj, int n) {
    int t = 0;
    for (; t + 4 <= n; t += 4) {
      s0 = fma(xi[t], xj[t], s0);
      s1 = fma(xi[t + 1], xj[t + 1], s1);
      s2 = fma(xi[t + 2], xj[t + 2], s2);
      s3 = fma(xi[t + 3], xj[t + 3], s3);
    }
    if (t < n) s0 = fma(xi[t], xj[t], s0);
    if (t + 1 < n) s1 = fma(xi[t + 1], xj[t + 1], s1);
    if (t + 2 < n) s2 = fma(xi[t + 2], xj[t + 2], s2);
  }
  __device__ __forceinline__ double sum() const { return (s0 + s1) + (s2 + s3); }
};

// In-place right-looking Cholesky of the leading n x n block of M (row stride
// ld, lower triangle used): the pivot's reciprocal square root by
// rsqrt_newton, the column scaled by it, L_kk = d / sqrt(d). rdiag (optional)
// receives 1 / L_kk. Returns false if a pivot is not positive (LAPACK potrf's
// failure test).
__device__ bool block_cholesky(double* M, int n, int ld, int* flag, double* rdiag = nullptr) {
  __shared__ double rk;
  if (threadIdx.x == 0) *flag = 0;
  __syncthreads();
  for (int k = 0; k < n; ++k) {
    if (threadIdx.x == 0) {
      const double d = M[k * ld + k];
      const bool pos = d > 0.0;
      if (!pos) *flag = 1;
      const double r = pos ? rsqrt_newton(d) : 1.0;
      M[k * ld + k] = pos ? d * r : 1.0;
      rk = r;
      if (rdiag) rdiag[k] = r;
    }
    __syncthreads();
    if (*flag) return false;
    const double r = rk;
    for (int i = k + 1 + threadIdx.x; i < n; i += blockDim.x) M[i * ld + k] *= r;
    __syncthreads();
    const int m = n - k - 1;
    for (int idx = threadIdx.x; idx < m * m; idx += blockDim.x) {
      const int i = k + 1 + idx / m, j = k + 1 + idx % m;
      if (j <= i) M[i * ld + j] -= M[i * ld + k] * M[j * ld + k];
    }
    __syncthreads();
  }
  return true;
}

// Li = L^-1 for lower-triangular L (n x n, row stride ld); column-parallel.
// With rdiag (1 / L_ii from block_cholesky) the diagonal divisions of the
// column recursions become products.
__device__ void block_tri_inverse(const double* L, double* Li, int n, int ld, const double* rdiag = nullptr) {
  for (int c = threadIdx.x; c < n; c += blockDim.x) {
    for (int i = 0; i < c; ++i) Li[i * ld + c] = 0.0;
    for (int i = c; i < n; ++i) {
      double s = (i == c) ? 1.0 : 0.0;
      for (int k = c; k < i; ++k) s -= L[i * ld + k] * Li[k * ld + c];
      const double d = L[i * ld + i];
      Li[i * ld + c] = rdiag ? s * rdiag[i] : (d != 0.0 ? s / d : 0.0);
    }
  }
  __syncthreads();
}

// out[n][n] = inv(A_SS + 1e-8 I) for the columns idx[0 .. n) of A = Li' Li
// = (X_w'X_w)^-1: S = A_SS + 1e-8 I (the S slot), its Cholesky factor, that
// factor's inverse (the A slot) and out = inverse' inverse, in FP64. Ends
// with a barrier.
__device__ __forceinline__ void sub_block_inverse(const PairScratch& s, int K, const int* idx, int n, int* flag, float* out) {
  for (int e = threadIdx.x; e < n * n; e += blockDim.x) {
    const int i = e / n, j = e % n;
    const int ti = idx[i], tj = idx[j];
    double acc = 0.0;
    for (int k = max(ti, tj); k < K; ++k) acc += s.Li[k * K + ti] * s.Li[k * K + tj];
    s.S[i * n + j] = acc + (i == j ? 1e-8 : 0.0);
  }
  __syncthreads();
  block_cholesky(s.S, n, n, flag);
  block_tri_inverse(s.S, s.A, n, n);
  for (int e = threadIdx.x; e < n * n; e += blockDim.x) {
    const int i = e / n, j = e % n;
    double acc = 0.0;
    for (int k = max(i, j); k < n; ++k) acc += s.A[k * n + i] * s.A[k * n + j];
    out[e] = (float)acc;
  }
  __syncthreads();
}

struct BuildArgs {
  ffs_grid_desc d;
  ffs_grid_out o;
};

// Phase 1 of an item: the per-run LDL' of pair p's AR-filtered tridiagonal
// correlation, the serial recursion m_t = T_t,t-1 / D_t-1, D_t = T_tt - m_t
// T_t,t-1 (one thread per run; unit gaps need no pow: a^1 = a and a^0 = 1
// exactly), then sqrt, log and the reciprocals of every sample in parallel:
// cms[t] = (c, m, D, 1/sqrt(D)) in shared memory, coef[p] and logdet_R[p].
// *bad_r = 1 if a pivot D_t was not positive. Ends with a barrier.
__device__ __forceinline__ void ldl_of_pair(const ffs_grid_desc& d, const ffs_grid_out& o, int p, double* cms, double* red,
                            int* bad_r) {
  const int T = d.T;
  const float af = d.a[p], bf = d.b[p];
  const double a = (double)af;
  const double lam = d.lambda_fp32 ? (double)lambda_f32(af, bf) : lambda_f64(a, (double)bf);
  if (threadIdx.x == 0) *bad_r = 0;
  __syncthreads();
  for (int r = threadIdx.x; r < d.n_runs; r += blockDim.x) {
    const int t0 = d.run_start[r], t1 = d.run_start[r + 1];
    double Dprev = 1.0, mprev = 0.0;
    int prev_gap = 0;
    for (int t = t0; t < t1; ++t) {
      double c = 0.0, m = 0.0, D = 1.0;
      // lambda == 0: every lag correlation is zero, R = I exactly
      if (t > t0 && lam != 0.0) {
        const int gap = d.tau[t] - d.tau[t - 1];
        double rho;
        if (gap == 1) {
          c = a;
          rho = lam;
        } else {
          // a^gap and a^(gap - 1) of small integer gaps by products
          double ag1 = 1.0;
          if (gap <= 16) {
            for (int k = 1; k < gap; ++k) ag1 *= a;
          } else {
            ag1 = pow(a, (double)(gap - 1));
          }
          c = ag1 * a;
          rho = lam * ag1;
        }
        const double Ttt = 1.0 + c * c - 2.0 * c * rho;
        const double Toff = rho - c;
        if (gap == 1 && prev_gap == 1 && Dprev == cms[4 * (t - 1) - 4 + 2]) {
          // the previous step left D unchanged: the recursion has reached
          // its fixed point, and every step of this stretch of unit gaps
          // repeats it
          m = mprev;
          D = Dprev;
        } else {
          // 1/D_{t-1}: fp32 estimate refined by two Newton steps r (2 - D r)
          // (error ~2^-24 -> ~2^-48 -> below 2^-53), cheaper than a
          // correctly rounded FP64 division in this serial chain
          if (Dprev > 1e-30 && Dprev < 1e30) {
            double r = (double)__frcp_rn((float)Dprev);
            r = r * fma(-Dprev, r, 2.0);
            r = r * fma(-Dprev, r, 2.0);
            m = Toff * r;
          } else {
            m = Toff / Dprev;
          }
          D = Ttt - m * Toff;
        }
        prev_gap = gap;
      }
      if (!(D > 0.0)) {
        *bad_r = 1;
        D = 1.0;
      }
      double* cm = cms + 4 * t;
      cm[0] = c; cm[1] = m; cm[2] = D;
      Dprev = D;
      mprev = m;
    }
  }
  __syncthreads();
  {
    double ld = 0.0;
    for (int t = threadIdx.x; t < T; t += blockDim.x) {
      double* cm = cms + 4 * t;
      const double D = cm[2];
      const double sD = sqrt(D);
      const double rsD = 1.0 / sD;
      ld += 2.0 * log(sD + 1e-10);
      cm[3] = rsD;
      reinterpret_cast<float4*>(o.coef)[(size_t)p * T + t] =
          make_float4((float)cm[0], (float)cm[1], (float)(1.0 / D), (float)rsD);
    }
    ld = block_sum(ld, red);
    if (threadIdx.x == 0) o.logdet_R[p] = ld;
  }
  __syncthreads();
}

// Phase 1 of an item with AFNI's banded R (d.band): the Cholesky factor of
// each run's block of R, where R(t, k) = lam a^(g-1) for 1 <= g = tau_t -
// tau_k <= band[p] and 0 beyond. One warp per run, rows in order; row t has
// J_t earlier rows of its run within the band (zero at a run start), and its
// off-diagonal entries L(t, t - j) solve the triangular system of those rows
// against R(t, t - j): the lanes hold the right-hand side (lane l the terms
// j = l + 1 + 32 q), each solved entry is broadcast and taken off the terms
// not yet solved. The diagonal is sqrt(1 - sum_j L(t, t - j)^2); a pivot that
// is not positive flags the pair (bad_r) and is replaced by 1. FP64
// throughout; band_L keeps the factor, band_coef its fp32 whitening
// coefficients, invdiag and Jrow (shared memory) the reciprocal diagonal and
// each row's band for phases 2 and 6. logdet_R = 2 sum log(L(t, t) + 1e-10)
// as the reference takes it from its dense factor; coef is the identity.
__device__ void band_chol_of_pair(const ffs_grid_desc& d, const ffs_grid_out& o, int p, double* invdiag, int* Jrow,
                                  double* apow, double* red, int* bad_r) {
  const int T = d.T, W = d.band_w, bw = d.band[p];
  const float af = d.a[p], bf = d.b[p];
  const double a = (double)af;
  const double lam = d.lambda_fp32 ? (double)lambda_f32(af, bf) : lambda_f64(a, (double)bf);
  double* Lb = o.band_L + (size_t)p * T * W;
  float* Cb = o.band_coef + (size_t)p * T * W;
  if (threadIdx.x == 0) {
    *bad_r = 0;
    double x = 1.0;
    for (int k = 0; k < W; ++k) {  // a^k: corr(g) = lam a^(g - 1), 1 <= g < W
      apow[k] = x;
      x *= a;
    }
  }
  __syncthreads();
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  for (int r = warp; r < d.n_runs; r += nw) {
    const int t0 = d.run_start[r], t1 = d.run_start[r + 1];
    for (int t = t0; t < t1; ++t) {
      const int tt = d.tau[t];
      int J = 0;
      while (J < t - t0 && J < W - 1 && tt - d.tau[t - J - 1] <= bw) ++J;
      double rj[4], own = 0.0;
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        const int j = lane + 1 + 32 * q;
        rj[q] = (j <= J && lam != 0.0) ? lam * apow[tt - d.tau[t - j] - 1] : 0.0;
      }
      for (int j = J; j >= 1; --j) {
        const int q = (j - 1) >> 5, owner = (j - 1) & 31;
        const double mine = q == 0 ? rj[0] : q == 1 ? rj[1] : q == 2 ? rj[2] : rj[3];
        const double ell = __shfl_sync(0xffffffffu, mine, owner) * invdiag[t - j];
        if (lane == owner) {
          Lb[(size_t)t * W + j] = ell;
          own = fma(ell, ell, own);
        }
#pragma unroll
        for (int qq = 0; qq < 4; ++qq) {
          const int jp = lane + 1 + 32 * qq;  // the term of row t - jp, column t - j
          if (jp < j && j - jp <= Jrow[t - jp]) rj[qq] -= ell * Lb[(size_t)(t - jp) * W + (j - jp)];
        }
      }
      __syncwarp();  // the row's entries, written by their owner lanes, are read below
      double d2 = 1.0 - warp_sum_d(own);
      if (!(d2 > 0.0)) {
        if (lane == 0) *bad_r = 1;
        d2 = 1.0;
      }
      const double ltt = sqrt(d2);
      const double inv = 1.0 / ltt;
      for (int j = lane; j < W; j += 32) {
        const double v = j == 0 ? ltt : (j <= J ? Lb[(size_t)t * W + j] : 0.0);
        if (j > J) Lb[(size_t)t * W + j] = 0.0;
        if (j == 0) Lb[(size_t)t * W] = ltt;
        Cb[(size_t)t * W + j] = (float)(j == 0 ? inv : v * inv);
      }
      if (lane == 0) {
        invdiag[t] = inv;
        Jrow[t] = J;
      }
      __syncwarp();
    }
  }
  __syncthreads();
  double ld = 0.0;
  for (int t = threadIdx.x; t < T; t += blockDim.x) {
    ld += 2.0 * log(Lb[(size_t)t * W] + 1e-10);
    reinterpret_cast<float4*>(o.coef)[(size_t)p * T + t] = make_float4(0.f, 0.f, 1.f, 1.f);
  }
  ld = block_sum(ld, red);
  if (threadIdx.x == 0) o.logdet_R[p] = ld;
  __syncthreads();
}

// Phase 1 of every pair once, for the items of all designs (coef and
// logdet_R depend on the pair only): cm [P][T][4] and bad [P] in the
// workspace, read back by grid_build_kernel. With the banded R the pair's
// band_L, band_coef, coef and logdet_R are written here, and cm keeps the
// reciprocal diagonal and each row's band (the first 1.5 T doubles).
__global__ void __launch_bounds__(GB_THREADS) pair_ldl_kernel(BuildArgs args, double* cm, int* bad) {
  __shared__ double red[32];
  __shared__ int bad_r;
  extern __shared__ double cms[];  // [T][4], or with the band as band_chol_of_pair lays it out
  const int T = args.d.T;
  if (args.d.band)
    band_chol_of_pair(args.d, args.o, blockIdx.x, cms, reinterpret_cast<int*>(cms + T), cms + T + (T + 1) / 2, red,
                      &bad_r);
  else
    ldl_of_pair(args.d, args.o, blockIdx.x, cms, red, &bad_r);
  double2* dst = reinterpret_cast<double2*>(cm + (size_t)blockIdx.x * 4 * T);
  for (int i = threadIdx.x; i < 2 * T; i += blockDim.x) dst[i] = reinterpret_cast<const double2*>(cms)[i];
  if (threadIdx.x == 0) bad[blockIdx.x] = bad_r;
}

// Items are (design, pair) = (item / P, item % P); a CTA takes items
// blockIdx.x, blockIdx.x + gridDim.x, ... with scratch slot blockIdx.x.
// Design-dependent outputs sit at pd = design * P + pair. With SHARED_LDL
// (more than one design) phase 1 comes from pair_ldl_kernel (pair_cm,
// pair_bad), which also wrote coef and logdet_R; without it every item
// factors its pair's R itself. Capped at 64 registers (4 CTAs per SM): left
// free, the compiler takes 80 to 126 of them.
template <bool SHARED_LDL>
__global__ void __launch_bounds__(GB_THREADS, 4) grid_build_kernel(BuildArgs args, int n_designs,
                                                                                  const double* pair_cm,
                                                                                  const int* pair_bad) {
  const ffs_grid_desc& d = args.d;
  const ffs_grid_out& o = args.o;
  const int T = d.T, K = d.K, LT = ld_t(T);
  PairScratch s = scratch_of(o.work, blockIdx.x, T, K);

  __shared__ double red[32];
  __shared__ int flag, bad_r;
  extern __shared__ double cms[];  // [T][4] c, m, D, 1/sqrt(D) of the current pair

  for (int item = blockIdx.x; item < d.P * n_designs; item += gridDim.x) {
    const int p = item % d.P, pd = item;
    const float* Xd = d.X + (size_t)(item / d.P) * T * K;
    if constexpr (SHARED_LDL) {
      // the pre-pass factored R for every pair once: copy this pair's rows
      const double2* src = reinterpret_cast<const double2*>(pair_cm + (size_t)p * 4 * T);
      for (int i = threadIdx.x; i < 2 * T; i += blockDim.x) reinterpret_cast<double2*>(cms)[i] = src[i];
      if (threadIdx.x == 0) bad_r = pair_bad[p];
      __syncthreads();
    } else if (d.band) {
      band_chol_of_pair(d, o, p, cms, reinterpret_cast<int*>(cms + T), cms + T + (T + 1) / 2, red, &bad_r);
    } else {
      ldl_of_pair(d, o, p, cms, red, &bad_r);
    }

    // ---- 2. X_w = L^-1 X, one column per thread; the design samples of
    // GB_PF steps are loaded ahead of the recursion that needs them (with the
    // banded R: forward substitution against the band of each row)
    if (d.band) {
      const int W = d.band_w;
      const double* Lb = o.band_L + (size_t)p * T * W;
      const int* Jrow = reinterpret_cast<const int*>(cms + T);
      for (int j = threadIdx.x; j < K; j += blockDim.x) {
        double* xw = s.Xw + (size_t)j * T;
        for (int t = 0; t < T; ++t) {
          double acc = f2d_exact(__ldg(Xd + (size_t)t * K + j));
          const double* row = Lb + (size_t)t * W;
          for (int i = 1; i <= Jrow[t]; ++i) acc = fma(-row[i], xw[t - i], acc);
          xw[t] = acc * cms[t];
        }
      }
    }
    for (int j = threadIdx.x; j < K && !d.band; j += blockDim.x) {
      double xp = 0.0, vp = 0.0;
      for (int t0 = 0; t0 < T; t0 += GB_PF) {
        float xb[GB_PF];
#pragma unroll
        for (int k = 0; k < GB_PF; ++k) xb[k] = t0 + k < T ? __ldg(Xd + (size_t)(t0 + k) * K + j) : 0.f;
#pragma unroll
        for (int k = 0; k < GB_PF; ++k) {
          const int t = t0 + k;
          if (t < T) {
            const double* cm = cms + 4 * t;
            const double x = f2d_exact(xb[k]);
            const double z = x - cm[0] * xp;
            const double v = z - cm[1] * vp;
            s.Xw[(size_t)j * T + t] = v * cm[3];
            xp = x;
            vp = v;
          }
        }
      }
    }
    __syncthreads();

    // ---- 3. X_w'X_w (full symmetric) into Lx, and the fp32 copy: one thread
    // per lower-triangle entry (full warps), four chains each
    for (int e = threadIdx.x; e < K * (K + 1) / 2; e += blockDim.x) {
      int i, j;
      tri_index(e, i, j);
      Dot4 acc;
      acc.run(s.Xw + (size_t)i * T, s.Xw + (size_t)j * T, T);
      const double v = acc.sum();
      s.Lx[i * K + j] = v;
      s.Lx[j * K + i] = v;
      o.XtX[(size_t)pd * K * K + i * K + j] = (float)v;
      o.XtX[(size_t)pd * K * K + j * K + i] = (float)v;
    }
    __syncthreads();

    // ---- 4. Cholesky of X_w'X_w, QR (modified Gram-Schmidt, twice) otherwise
    // 1 / diag(Lx) goes to the A slot, free until phase 9
    int info = 0;
    const bool chol = block_cholesky(s.Lx, K, K, &flag, s.A);
    if (!chol) {
      info = 1;
      // Q and R from X_w; Lx := R' (lower), so that X_w'X_w = Lx Lx'.
      for (int idx = threadIdx.x; idx < K * K; idx += blockDim.x) s.Lx[idx] = 0.0;
      __syncthreads();
      for (int j = 0; j < K; ++j) {
        double* q = s.Qm + (size_t)j * T;
        for (int t = threadIdx.x; t < T; t += blockDim.x) q[t] = s.Xw[(size_t)j * T + t];
        __syncthreads();
        for (int pass = 0; pass < 2; ++pass) {
          for (int i = 0; i < j; ++i) {
            const double* qi = s.Qm + (size_t)i * T;
            double part = 0.0;
            for (int t = threadIdx.x; t < T; t += blockDim.x) part += qi[t] * q[t];
            const double rij = block_sum(part, red);
            for (int t = threadIdx.x; t < T; t += blockDim.x) q[t] -= rij * qi[t];
            if (threadIdx.x == 0) s.Lx[j * K + i] += rij;
            __syncthreads();
          }
        }
        double part = 0.0;
        for (int t = threadIdx.x; t < T; t += blockDim.x) part += q[t] * q[t];
        const double nrm = sqrt(block_sum(part, red));
        const double inv = nrm > 0.0 ? 1.0 / nrm : 0.0;
        for (int t = threadIdx.x; t < T; t += blockDim.x) q[t] *= inv;
        if (threadIdx.x == 0) s.Lx[j * K + j] = nrm;
        __syncthreads();
      }
    }
    if (bad_r) info = 2;
    __syncthreads();

    if (threadIdx.x == 0) {
      double ld = 0.0;
      for (int j = 0; j < K; ++j) ld += 2.0 * log(fabs(s.Lx[j * K + j]) + 1e-10);
      o.logdet_XtX[pd] = ld;
      o.info[pd] = info;
    }

    // ---- 5. Q = X_w Lx^-T in fp32 (Q, U and G only leave as fp32 or fp16
    // splits; the factorisation and the logdets above stay FP64). The two [K][T]
    // FP64 slots are reused as fp32 arrays; the QR fallback converts its Q.
    float* const xw_f = reinterpret_cast<float*>(s.Xw);
    float* const qm_f = reinterpret_cast<float*>(s.Qm);
    float* const lx_f = reinterpret_cast<float*>(s.S);  // [K][K] Lx, then Li in lx_f + K*K
    float* qf;
    float* uf;
    for (int idx = threadIdx.x; idx < K * K; idx += blockDim.x) lx_f[idx] = (float)s.Lx[idx];
    __syncthreads();
    if (info != 1) {
      for (int t = threadIdx.x; t < T; t += blockDim.x) {
        for (int j = 0; j < K; ++j) {
          float acc = (float)s.Xw[(size_t)j * T + t];
          for (int i = 0; i < j; ++i) acc = fmaf(-lx_f[j * K + i], qm_f[(size_t)i * T + t], acc);
          qm_f[(size_t)j * T + t] = acc / lx_f[j * K + j];
        }
      }
      qf = qm_f;
      uf = xw_f;
    } else {
      for (int idx = threadIdx.x; idx < K * T; idx += blockDim.x) xw_f[idx] = (float)s.Qm[idx];
      qf = xw_f;
      uf = qm_f;
    }
    __syncthreads();

    // ---- 6. U = L^-T Q = A' L~^-T D^-1/2 Q (backward recursions) in fp32, with
    // the fp32 coefficients of phase 1
    const float4* cf = reinterpret_cast<const float4*>(o.coef) + (size_t)p * T;
    float umax_local = 0.f;
    if (d.band) {
      // back substitution against the band: u_t = (q_t - sum_i L(t + i, t)
      // u_{t+i}) / L(t, t), the rows t + i of t's run within the band
      const int W = d.band_w;
      const double* Lb = o.band_L + (size_t)p * T * W;
      const int* Jrow = reinterpret_cast<const int*>(cms + T);
      for (int j = threadIdx.x; j < K; j += blockDim.x) {
        const float* q = qf + (size_t)j * T;
        float* u = uf + (size_t)j * T;
        for (int t = T - 1; t >= 0; --t) {
          double acc = (double)q[t];
          for (int i = 1; t + i < T && i <= Jrow[t + i]; ++i) acc = fma(-Lb[(size_t)(t + i) * W + i], (double)u[t + i], acc);
          const float ut = (float)(acc * cms[t]);
          u[t] = ut;
          o.U[((size_t)pd * K + j) * LT + t] = ut;
          umax_local = fmaxf(umax_local, fabsf(ut));
        }
        for (int t = T; t < LT; ++t) o.U[((size_t)pd * K + j) * LT + t] = 0.f;
      }
    }
    for (int j = threadIdx.x; j < K && !d.band; j += blockDim.x) {
      const float* q = qf + (size_t)j * T;
      float* u = uf + (size_t)j * T;
      float xn = 0.f, mn = 0.f, cn = 0.f;  // x_{t+1}, m_{t+1}, c_{t+1}
      for (int t1 = T - 1; t1 >= 0; t1 -= GB_PF) {  // GB_PF steps of q and coef loaded ahead
        float qb[GB_PF];
        float4 cb[GB_PF];
#pragma unroll
        for (int k = 0; k < GB_PF; ++k) {
          const int t = t1 - k;
          qb[k] = t >= 0 ? q[t] : 0.f;
          cb[k] = t >= 0 ? cf[t] : make_float4(0.f, 0.f, 0.f, 0.f);
        }
#pragma unroll
        for (int k = 0; k < GB_PF; ++k) {
          const int t = t1 - k;
          if (t >= 0) {
            const float4 c4 = cb[k];  // (c, m, 1/D, 1/sqrt(D))
            const float x = fmaf(-mn, xn, qb[k] * c4.w);
            const float ut = fmaf(-cn, xn, x);
            u[t] = ut;
            o.U[((size_t)pd * K + j) * LT + t] = ut;
            umax_local = fmaxf(umax_local, fabsf(ut));
            xn = x;
            mn = c4.y;
            cn = c4.x;
          }
        }
      }
      for (int t = T; t < LT; ++t) o.U[((size_t)pd * K + j) * LT + t] = 0.f;
    }
    __syncthreads();
    if (o.U_hi) {
      // fp16 hi/lo split of U * 2^e, e placing max|U| in [128, 256)
      double um = umax_local;
      for (int off = 16; off > 0; off >>= 1) um = fmax(um, __shfl_xor_sync(0xffffffffu, um, off));
      if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = um;
      __syncthreads();
      if (threadIdx.x == 0) {
        double mx = 0.0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) mx = fmax(mx, red[w]);
        red[0] = mx;
      }
      __syncthreads();
      const int e = scale_exp((float)red[0]);
      if (threadIdx.x == 0) o.uexp[pd] = e;
      for (int idx = threadIdx.x; idx < K * d.ld_u; idx += blockDim.x) {
        const int j = idx / d.ld_u, t = idx % d.ld_u;
        uint16_t hi = 0, lo = 0;
        if (t < T) split_fp16(ldexpf(uf[(size_t)j * T + t], e), hi, lo);
        const size_t at = ((size_t)pd * K + j) * d.ld_u + t;
        o.U_hi[at] = hi;
        o.U_lo[at] = lo;
      }
    }
    __syncthreads();

    // ---- 7. Lx^-1 and diag(A), A = Lx^-T Lx^-1 = (X_w'X_w)^-1 (only the
    // entries the statistics read are formed: the diagonal here, the task
    // block and c A c' in phase 9)
    block_tri_inverse(s.Lx, s.Li, K, K, chol ? s.A : nullptr);
    for (int j = threadIdx.x; j < K; j += blockDim.x) {
      double acc = 0.0;
      for (int k = j; k < K; ++k) acc += s.Li[k * K + j] * s.Li[k * K + j];
      o.Adiag[(size_t)pd * K + j] = (float)acc;
    }
    if (o.Afull) {  // all of A, for the per-voxel blocks of the -dsort fit
      for (int e = threadIdx.x; e < K * K; e += blockDim.x) {
        const int i = e / K, j = e % K;
        double acc = 0.0;
        for (int k = max(i, j); k < K; ++k) acc += s.Li[k * K + i] * s.Li[k * K + j];
        o.Afull[(size_t)pd * K * K + e] = (float)acc;
      }
    }
    __syncthreads();

    // ---- 8. G = U Lx^-1 in fp32 (row t of G solves g Lx = u_t); Gsum = G' 1
    // accumulated in FP64
    float* const li_f = lx_f + (size_t)K * K;
    for (int idx = threadIdx.x; idx < K * K; idx += blockDim.x) li_f[idx] = (float)s.Li[idx];
    __syncthreads();
    for (int t = threadIdx.x; t < LT; t += blockDim.x) {
      for (int j = 0; j < K; ++j) {
        float acc = 0.f;
        if (t < T)
          for (int i = j; i < K; ++i) acc = fmaf(uf[(size_t)i * T + t], li_f[i * K + j], acc);
        o.G[((size_t)pd * K + j) * LT + t] = acc;
      }
    }
    __syncthreads();
    if (o.Gsum) {
      for (int j = threadIdx.x; j < K; j += blockDim.x) {
        double acc = 0.0;
        for (int t = 0; t < T; ++t) acc += (double)o.G[((size_t)pd * K + j) * LT + t];
        o.Gsum[(size_t)pd * K + j] = (float)acc;
      }
    }

    // ---- 9. task-column F matrix inv(A_task + 1e-8 I) and GLT variances c A c'
    const int nt = d.n_task;
    if (d.n_glt > 0 && o.glt_var) {  // c A c' = ||Lx^-1 c||^2
      for (int c = 0; c < d.n_glt; ++c) {
        const float* gc = d.glt + (size_t)c * K;
        double part = 0.0;
        for (int k = threadIdx.x; k < K; k += blockDim.x) {
          double w = 0.0;
          for (int j = 0; j <= k; ++j) w += s.Li[k * K + j] * (double)gc[j];
          part += w * w;
        }
        const double v = block_sum(part, red);
        if (threadIdx.x == 0) o.glt_var[(size_t)pd * d.n_glt + c] = (float)v;
      }
    }
    // the task block, then the column sets' blocks one after another
    const int has_task = nt > 0 && o.Ftask ? 1 : 0;
    const int nsets = o.Fsets ? d.n_sets : 0;
    size_t msum = 0, off = 0;
    for (int g = 0; g < nsets; ++g) {
      const size_t q = (size_t)(d.set_ptr[g + 1] - d.set_ptr[g]);
      msum += q * q;
    }
    for (int bk = 0; bk < has_task + nsets; ++bk) {
      const bool task = bk < has_task;
      const int g = bk - has_task;
      const int n = task ? nt : d.set_ptr[g + 1] - d.set_ptr[g];
      const int* idx = task ? d.task_idx : d.set_idx + d.set_ptr[g];
      float* out = task ? o.Ftask + (size_t)pd * nt * nt : o.Fsets + (size_t)pd * msum + off;
      sub_block_inverse(s, K, idx, n, &flag, out);
      if (!task) off += (size_t)n * n;
    }
    __syncthreads();  // the next item reuses the scratch slot and the shared state
  }
}

// ---- Design basis: Q0 = X Lx^-T, Lx the FP64 Cholesky factor of X'X (Q0 is
// U of the pair (0, 0), where R = I and X_w = X, and comes out bit for bit
// equal to the grid build's: the same Dot4 entries, block_cholesky and fp32
// recursion), and the centring test c = (X'X)^-1 X'1. Two launches: the Gram
// entries of [X | 1] spread over CTAs (each entry a chain of FP64 FMAs whose
// latency, not the FP64 rate, bounds it), then one CTA for the factor, Q0 and
// c. work: [NE] Gram entries of [X | 1] (packed lower triangle), [K][T]
// doubles (QR fallback), then K x K doubles when K > DB_SMEM_K.

constexpr int DB_ENTRIES = 32;   // Gram entries per CTA: one warp's lanes
constexpr int DB_SMEM_K = 64;    // the factor stays in shared memory up to this K
constexpr int DB_THREADS = 256;  // the finishing CTA (its MGS fallback's sums depend on it)

__host__ __device__ inline int db_entries(int K) { return (K + 1) * (K + 2) / 2; }

// Samples of the design staged per pass: a multiple of 4 (the Dot4 chains
// continue across passes), with (K + 1) columns of (chunk + 1) doubles within
// 96 KB of shared memory.
inline int db_chunk(int T, int K) {
  const int fit = (96 * 1024 / (8 * (K + 1)) - 1) & ~3;
  const int t4 = (T + 3) & ~3;
  return fit < t4 ? fit : t4;
}

__global__ void __launch_bounds__(256) design_gram_kernel(int T, int K, int chunk, const float* __restrict__ Xg,
                                                          double* __restrict__ gram) {
  extern __shared__ double xt[];  // [ncol][chunk + 1]: the columns this CTA reads, FP64, odd row stride
  const int ne = db_entries(K);
  const int e0 = blockIdx.x * DB_ENTRIES;
  const int e1 = min(e0 + DB_ENTRIES, ne);
  int ihi, jhi;
  tri_index(e1 - 1, ihi, jhi);
  const int ncol = ihi + 1;  // the entries' rows i <= ihi read columns 0..ihi (column K is the constant)
  const int ld = chunk + 1;
  const int e = e0 + (int)threadIdx.x;
  int i = 0, j = 0;
  if (threadIdx.x < 32 && e < e1) tri_index(e, i, j);
  Dot4 acc;
  for (int t0 = 0; t0 < T; t0 += chunk) {
    const int n = min(chunk, T - t0);
    __syncthreads();
    for (int idx = threadIdx.x; idx < n * ncol; idx += blockDim.x) {
      const int t = idx / ncol, c = idx % ncol;
      xt[c * ld + t] = c < K ? f2d_exact(Xg[(size_t)(t0 + t) * K + c]) : 1.0;
    }
    __syncthreads();
    if (threadIdx.x < 32 && e < e1) acc.run(xt + i * ld, xt + j * ld, n);
  }
  if (threadIdx.x < 32 && e < e1) gram[e] = acc.sum();
}

__global__ void __launch_bounds__(DB_THREADS) design_basis_kernel(int T, int K, const float* __restrict__ X,
                                                                  const double* __restrict__ gram, double* work,
                                                                  float* Q0, int* info, int* const_flag,
                                                                  float* const_coef) {
  __shared__ double red[32];
  __shared__ int flag;
  extern __shared__ double sm[];  // rd [K], cv [K]; K <= DB_SMEM_K: M [K][K], mf [K][K] fp32, q [K][DB_THREADS] fp32
  const int LT = ld_t(T);
  const bool small = K <= DB_SMEM_K;
  double* rd = sm;
  double* cv = rd + K;
  double* Qd = work + db_entries(K);  // [K][T] (QR fallback)
  double* M = small ? cv + K : Qd + (size_t)K * T;
  // the fp32 factor: in shared memory, else in the QR slot (unused once the
  // Cholesky factor exists)
  float* mf = small ? reinterpret_cast<float*>(M + (size_t)K * K) : reinterpret_cast<float*>(Qd);
  float* qs = small ? mf + (size_t)K * K : nullptr;
  for (int idx = threadIdx.x; idx < K * (LT - T); idx += blockDim.x)
    Q0[(size_t)(idx / (LT - T)) * LT + T + idx % (LT - T)] = 0.f;
  for (int e = threadIdx.x; e < K * (K + 1) / 2; e += blockDim.x) {
    int i, j;
    tri_index(e, i, j);
    M[i * K + j] = gram[e];
    M[j * K + i] = gram[e];
  }
  for (int j = threadIdx.x; j < K; j += blockDim.x) cv[j] = gram[K * (K + 1) / 2 + j];  // row K: X'1
  __syncthreads();
  if (block_cholesky(M, K, K, &flag, rd)) {
    for (int idx = threadIdx.x; idx < K * K; idx += blockDim.x) mf[idx] = (float)M[idx];
    __syncthreads();
    // Q0 row by row, the grid build's fp32 recursion; a row's earlier entries
    // are read back from shared memory (from Q0 itself when K is large)
    for (int t = threadIdx.x; t < T; t += blockDim.x) {
      float* q = small ? qs + threadIdx.x : Q0 + t;
      const size_t qst = small ? DB_THREADS : LT;
      for (int j = 0; j < K; ++j) {
        float acc = X[(size_t)t * K + j];
        for (int i = 0; i < j; ++i) acc = fmaf(-mf[j * K + i], q[i * qst], acc);
        const float v = acc / mf[j * K + j];
        q[j * qst] = v;
        if (small) Q0[(size_t)j * LT + t] = v;
      }
    }
    if (const_flag) {
      // c = (X'X)^-1 X'1 from the same factor (one warp: forward and back
      // substitution, a column of updates per step), accepted when
      // ||X c - 1||^2 <= 1e-12 T
      if (threadIdx.x < 32) {
        const int lane = threadIdx.x;
        for (int j = 0; j < K; ++j) {
          const double yj = cv[j] * rd[j];
          __syncwarp();
          for (int i = j + 1 + lane; i < K; i += 32) cv[i] = fma(-M[i * K + j], yj, cv[i]);
          if (lane == 0) cv[j] = yj;
          __syncwarp();
        }
        for (int j = K - 1; j >= 0; --j) {
          const double cj = cv[j] * rd[j];
          __syncwarp();
          for (int i = lane; i < j; i += 32) cv[i] = fma(-M[j * K + i], cj, cv[i]);
          if (lane == 0) cv[j] = cj;
          __syncwarp();
        }
      }
      __syncthreads();
      double part = 0.0;
      for (int t = threadIdx.x; t < T; t += blockDim.x) {
        double r = -1.0;
        for (int j = 0; j < K; ++j) r = fma(f2d_exact(X[(size_t)t * K + j]), cv[j], r);
        part = fma(r, r, part);
      }
      const double ss = block_sum(part, red);
      const bool ok = ss <= 1e-12 * (double)T;
      for (int j = threadIdx.x; j < K; j += blockDim.x) const_coef[j] = ok ? (float)cv[j] : 0.f;
      if (threadIdx.x == 0) *const_flag = ok ? 1 : 0;
    }
    if (threadIdx.x == 0) *info = 0;
    return;
  }
  if (const_flag) {  // X'X not positive definite: no centring
    for (int j = threadIdx.x; j < K; j += blockDim.x) const_coef[j] = 0.f;
    if (threadIdx.x == 0) *const_flag = 0;
  }
  // QR of X by modified Gram-Schmidt (twice) in FP64, the grid build's
  // fallback on X_w = X
  for (int j = 0; j < K; ++j) {
    double* q = Qd + (size_t)j * T;
    for (int t = threadIdx.x; t < T; t += blockDim.x) q[t] = (double)X[(size_t)t * K + j];
    __syncthreads();
    for (int pass = 0; pass < 2; ++pass) {
      for (int i = 0; i < j; ++i) {
        const double* qi = Qd + (size_t)i * T;
        double part = 0.0;
        for (int t = threadIdx.x; t < T; t += blockDim.x) part += qi[t] * q[t];
        const double rij = block_sum(part, red);
        for (int t = threadIdx.x; t < T; t += blockDim.x) q[t] -= rij * qi[t];
        __syncthreads();
      }
    }
    double part = 0.0;
    for (int t = threadIdx.x; t < T; t += blockDim.x) part += q[t] * q[t];
    const double nrm = sqrt(block_sum(part, red));
    const double inv = nrm > 0.0 ? 1.0 / nrm : 0.0;
    for (int t = threadIdx.x; t < T; t += blockDim.x) {
      q[t] *= inv;
      Q0[(size_t)j * LT + t] = (float)q[t];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) *info = 1;
}

}  // namespace

}  // namespace ffsk

extern "C" size_t ffs_design_basis_work_bytes(int T, int K) {
  const size_t kk = K > ffsk::DB_SMEM_K ? (size_t)K * K : 0;
  return sizeof(double) * ((size_t)ffsk::db_entries(K) + (size_t)K * T + kk);
}

extern "C" int ffs_design_basis(int T, int K, const float* X, void* work, float* Q0, int* info, int* const_flag,
                                float* const_coef, void* stream) {
  using namespace ffsk;
  clear_error();
  FFS_REQUIRE(T > 0 && K > 0 && K <= T, "ffs_design_basis: T=%d K=%d", T, K);
  FFS_REQUIRE(X && work && Q0 && info, "ffs_design_basis: null buffer");
  FFS_REQUIRE(!const_flag == !const_coef, "ffs_design_basis: const_flag and const_coef go together");
  double* gram = static_cast<double*>(work);
  const int chunk = db_chunk(T, K);
  FFS_REQUIRE(chunk >= 4, "ffs_design_basis: K=%d too wide", K);
  const size_t gsm = sizeof(double) * (size_t)(K + 1) * (chunk + 1);
  FFS_CUDA(ensure_dyn_smem(reinterpret_cast<const void*>(design_gram_kernel), gsm));
  const int nb = ceil_div(db_entries(K), DB_ENTRIES);
  design_gram_kernel<<<nb, 256, gsm, (cudaStream_t)stream>>>(T, K, chunk, X, gram);
  if (const int rc = check_launch("design_gram_kernel")) return rc;
  const size_t fsm = K <= DB_SMEM_K ? sizeof(double) * 2 * K + sizeof(double) * (size_t)K * K +
                                          sizeof(float) * (size_t)K * K + sizeof(float) * (size_t)K * DB_THREADS
                                    : sizeof(double) * 2 * K;
  FFS_CUDA(ensure_dyn_smem(reinterpret_cast<const void*>(design_basis_kernel), fsm));
  design_basis_kernel<<<1, DB_THREADS, fsm, (cudaStream_t)stream>>>(T, K, X, gram, gram, Q0, info, const_flag,
                                                                   const_coef);
  return check_launch("design_basis_kernel");
}

extern "C" size_t ffs_grid_work_bytes(int T, int K, int P) {
  return sizeof(double) * ffsk::pair_doubles(T, K) * (size_t)P;
}

// Per-slot scratch of the CTAs, then (more than one design) the pre-pass's
// factors of R: cm [P][T][4] doubles and bad [P] ints.
static size_t designs_slot_doubles(int T, int K, int P, int n_designs, int max_ctas) {
  const long long items = (long long)P * (n_designs > 0 ? n_designs : 1);
  const long long cap = max_ctas > 0 && max_ctas < FFS_GRID_MAX_SLOTS ? max_ctas : FFS_GRID_MAX_SLOTS;
  return (ffsk::pair_doubles(T, K) * (size_t)(items < cap ? items : cap) + 1) & ~(size_t)1;  // 16-byte aligned end
}

extern "C" size_t ffs_grid_work_bytes_designs(int T, int K, int P, int n_designs, int max_ctas) {
  size_t n = designs_slot_doubles(T, K, P, n_designs, max_ctas);
  if (n_designs > 1) n += (size_t)P * 4 * T + ((size_t)P + 1) / 2;
  return sizeof(double) * n;
}

// n_sets needs its index arrays and the Fsets output
static int check_sets(const ffs_grid_desc* d, const ffs_grid_out* o, const char* who) {
  FFS_REQUIRE(d->n_sets >= 0, "%s: n_sets=%d", who, d->n_sets);
  FFS_REQUIRE(d->n_sets == 0 || (d->set_ptr && d->set_idx && o->Fsets), "%s: column sets need set_ptr, set_idx and Fsets",
              who);
  return FFS_OK;
}

extern "C" int ffs_grid_build(const ffs_grid_desc* d, const ffs_grid_out* o, void* stream) {
  using namespace ffsk;
  clear_error();
  FFS_REQUIRE(d && o, "ffs_grid_build: null descriptor");
  FFS_REQUIRE(d->T > 0 && d->K > 0 && d->P > 0 && d->n_runs > 0,
              "ffs_grid_build: T=%d K=%d P=%d n_runs=%d must be positive", d->T, d->K, d->P,
              d->n_runs);
  FFS_REQUIRE(d->K <= d->T, "ffs_grid_build: K=%d exceeds T=%d", d->K, d->T);
  FFS_REQUIRE(d->n_task >= 0 && d->n_task <= d->K, "ffs_grid_build: bad n_task=%d", d->n_task);
  if (const int rc = check_sets(d, o, "ffs_grid_build")) return rc;
  FFS_REQUIRE(!o->U_hi || (o->U_lo && o->uexp), "ffs_grid_build: U_hi needs U_lo and uexp");
  FFS_REQUIRE(!o->U_hi || (d->ld_u >= d->T && d->ld_u % 8 == 0),
              "ffs_grid_build: ld_u=%d must be >= T and a multiple of 8", d->ld_u);
  FFS_REQUIRE(d->run_start && d->tau && d->a && d->b && d->X, "ffs_grid_build: null input");
  FFS_REQUIRE(o->coef && o->logdet_R && o->logdet_XtX && o->U && o->G && o->Adiag && o->XtX &&
                  o->info && o->work,
              "ffs_grid_build: null output");
  FFS_REQUIRE(!d->band || (d->band_w >= 1 && d->band_w <= FFS_BAND_MAX_W && o->band_L && o->band_coef),
              "ffs_grid_build: the banded R needs 1 <= band_w=%d <= %d, band_L and band_coef", d->band_w,
              FFS_BAND_MAX_W);
  BuildArgs args{*d, *o};
  // shared memory: [T][4] doubles, or with the band invdiag [T], Jrow [T]
  // (ints) and the powers of a [band_w]
  size_t smem = sizeof(double) * 4 * (size_t)d->T;
  if (d->band)
    smem = std::max(smem, sizeof(double) * ((size_t)d->T + (d->T + 1) / 2 + (size_t)d->band_w + 1));
  FFS_REQUIRE(smem <= 200 * 1024, "ffs_grid_build: T=%d too long", d->T);
  FFS_CUDA(ensure_dyn_smem(reinterpret_cast<const void*>(grid_build_kernel<false>), smem));
  grid_build_kernel<false><<<d->P, GB_THREADS, smem, (cudaStream_t)stream>>>(args, 1, nullptr, nullptr);
  return check_launch("grid_build_kernel");
}

extern "C" int ffs_grid_build_designs(const ffs_grid_desc* d, int n_designs, int max_ctas, const ffs_grid_out* o,
                                      void* stream) {
  using namespace ffsk;
  clear_error();
  FFS_REQUIRE(d && o, "ffs_grid_build_designs: null descriptor");
  FFS_REQUIRE(n_designs > 0, "ffs_grid_build_designs: n_designs=%d must be positive", n_designs);
  FFS_REQUIRE(d->T > 0 && d->K > 0 && d->P > 0 && d->n_runs > 0,
              "ffs_grid_build_designs: T=%d K=%d P=%d n_runs=%d must be positive", d->T, d->K, d->P, d->n_runs);
  FFS_REQUIRE((long long)d->P * n_designs < (1LL << 31), "ffs_grid_build_designs: too many items");
  FFS_REQUIRE(!d->band || (d->band_w >= 1 && d->band_w <= FFS_BAND_MAX_W && o->band_L && o->band_coef),
              "ffs_grid_build_designs: the banded R needs 1 <= band_w=%d <= %d, band_L and band_coef", d->band_w,
              FFS_BAND_MAX_W);
  FFS_REQUIRE(d->K <= d->T, "ffs_grid_build_designs: K=%d exceeds T=%d", d->K, d->T);
  FFS_REQUIRE(d->n_task >= 0 && d->n_task <= d->K, "ffs_grid_build_designs: bad n_task=%d", d->n_task);
  if (const int rc = check_sets(d, o, "ffs_grid_build_designs")) return rc;
  FFS_REQUIRE(!o->U_hi || (o->U_lo && o->uexp), "ffs_grid_build_designs: U_hi needs U_lo and uexp");
  FFS_REQUIRE(!o->U_hi || (d->ld_u >= d->T && d->ld_u % 8 == 0),
              "ffs_grid_build_designs: ld_u=%d must be >= T and a multiple of 8", d->ld_u);
  FFS_REQUIRE(d->run_start && d->tau && d->a && d->b && d->X, "ffs_grid_build_designs: null input");
  FFS_REQUIRE(o->coef && o->logdet_R && o->logdet_XtX && o->U && o->G && o->Adiag && o->XtX && o->info && o->work,
              "ffs_grid_build_designs: null output");
  const long long items = (long long)d->P * n_designs;
  const long long cap = max_ctas > 0 && max_ctas < FFS_GRID_MAX_SLOTS ? max_ctas : FFS_GRID_MAX_SLOTS;
  const int grid = (int)(items < cap ? items : cap);
  BuildArgs args{*d, *o};
  const size_t smem = sizeof(double) * 4 * (size_t)d->T;
  // phase 1 of the banded R also holds the powers of a (band_chol_of_pair)
  const size_t smem1 = d->band ? std::max(smem, sizeof(double) * ((size_t)d->T + (d->T + 1) / 2 +
                                                                  (size_t)d->band_w + 1))
                               : smem;
  FFS_REQUIRE(smem1 <= 200 * 1024, "ffs_grid_build_designs: T=%d too long", d->T);
  FFS_CUDA(ensure_dyn_smem(reinterpret_cast<const void*>(grid_build_kernel<false>), smem1));
  FFS_CUDA(ensure_dyn_smem(reinterpret_cast<const void*>(grid_build_kernel<true>), smem));
  FFS_CUDA(ensure_dyn_smem(reinterpret_cast<const void*>(pair_ldl_kernel), smem1));
  double* pair_cm = nullptr;
  int* pair_bad = nullptr;
  if (n_designs > 1) {
    pair_cm = o->work + designs_slot_doubles(d->T, d->K, d->P, n_designs, max_ctas);
    pair_bad = reinterpret_cast<int*>(pair_cm + (size_t)d->P * 4 * d->T);
    pair_ldl_kernel<<<d->P, GB_THREADS, smem1, (cudaStream_t)stream>>>(args, pair_cm, pair_bad);
    if (const int rc = check_launch("pair_ldl_kernel")) return rc;
  }
  if (pair_cm)
    grid_build_kernel<true><<<grid, GB_THREADS, smem, (cudaStream_t)stream>>>(args, n_designs, pair_cm, pair_bad);
  else
    grid_build_kernel<false><<<grid, GB_THREADS, smem1, (cudaStream_t)stream>>>(args, n_designs, nullptr, nullptr);
  return check_launch("grid_build_kernel (designs)");
}

// ---------------------------------------------------------------------------
// Allocation-free variant of ffs_grid_build.
//
// Some callers cannot allocate device memory at the point where they build the
// grid factors: code running under a framework allocator that already owns
// the device's memory, or an embedding (for example a foreign-language binding
// driving the library from inside a larger pipeline) that is handed only its
// input and output buffers and has no allocator of its own. For them the FP64
// scratch lives in this file-scope device array instead of a caller-provided
// workspace. Every GPU that loads the library holds the array until the
// process exits.
namespace ffsk {
namespace {

constexpr size_t kStaticGridScratchBytes = (size_t)16 << 20;  // 16 MiB
static __device__ __align__(256) double g_grid_scratch[kStaticGridScratchBytes / sizeof(double)];

// Device address of g_grid_scratch, resolved once per device with that device
// current (host code may only pass this address to kernels, never the symbol).
// The cache lives as long as the process; a cudaDeviceReset would leave it
// stale (documented in the header).
double* static_grid_scratch(int* status) {
  static std::mutex mu;
  static double* addr[256] = {nullptr};
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess || dev < 0 || dev >= 256) {
    set_error("ffs_grid_build_noalloc: cudaGetDevice failed (%s)", cudaGetErrorString(e));
    *status = FFS_ERR_CUDA;
    return nullptr;
  }
  std::lock_guard<std::mutex> lock(mu);
  if (!addr[dev]) {
    double* ptr = nullptr;
    e = cudaGetSymbolAddress((void**)&ptr, g_grid_scratch);
    if (e != cudaSuccess || !ptr) {
      set_error("ffs_grid_build_noalloc: cudaGetSymbolAddress failed on device %d (%s)", dev,
                cudaGetErrorString(e));
      *status = FFS_ERR_CUDA;
      return nullptr;
    }
    addr[dev] = ptr;
  }
  *status = FFS_OK;
  return addr[dev];
}

}  // namespace
}  // namespace ffsk

extern "C" int ffs_grid_build_noalloc(const ffs_grid_desc* d, const ffs_grid_out* o, void* stream) {
  using namespace ffsk;
  clear_error();
  FFS_REQUIRE(d && o, "ffs_grid_build_noalloc: null descriptor");
  FFS_REQUIRE(d->T > 0 && d->K > 0 && d->P > 0 && d->n_runs > 0,
              "ffs_grid_build_noalloc: T=%d K=%d P=%d n_runs=%d must be positive", d->T, d->K, d->P, d->n_runs);
  FFS_REQUIRE(d->K <= d->T, "ffs_grid_build_noalloc: K=%d exceeds T=%d", d->K, d->T);
  FFS_REQUIRE(d->n_task >= 0 && d->n_task <= d->K, "ffs_grid_build_noalloc: bad n_task=%d", d->n_task);
  if (const int rc = check_sets(d, o, "ffs_grid_build_noalloc")) return rc;
  FFS_REQUIRE(!o->U_hi || (o->U_lo && o->uexp), "ffs_grid_build_noalloc: U_hi needs U_lo and uexp");
  FFS_REQUIRE(!o->U_hi || (d->ld_u >= d->T && d->ld_u % 8 == 0),
              "ffs_grid_build_noalloc: ld_u=%d must be >= T and a multiple of 8", d->ld_u);
  FFS_REQUIRE(d->run_start && d->tau && d->a && d->b && d->X, "ffs_grid_build_noalloc: null input");
  FFS_REQUIRE(o->coef && o->logdet_R && o->logdet_XtX && o->U && o->G && o->Adiag && o->XtX && o->info,
              "ffs_grid_build_noalloc: null output");
  FFS_REQUIRE(!d->band || (d->band_w >= 1 && d->band_w <= FFS_BAND_MAX_W && o->band_L && o->band_coef),
              "ffs_grid_build_noalloc: the banded R needs 1 <= band_w=%d <= %d, band_L and band_coef", d->band_w,
              FFS_BAND_MAX_W);
  const size_t need = sizeof(double) * pair_doubles(d->T, d->K) * (size_t)d->P;
  if (need > kStaticGridScratchBytes) {
    set_error("ffs_grid_build_noalloc: T=%d K=%d P=%d needs %zu bytes of scratch, above the %zu-byte static "
              "scratch; use ffs_grid_build with a caller-provided workspace",
              d->T, d->K, d->P, need, kStaticGridScratchBytes);
    return FFS_ERR_WORKSPACE;
  }
  int st = FFS_OK;
  double* scratch = static_grid_scratch(&st);
  if (!scratch) return st;
  // every scratch entry the kernel reads it writes first in the same launch, so
  // the previous call's contents need no clearing
  BuildArgs args{*d, *o};
  args.o.work = scratch;
  size_t smem = sizeof(double) * 4 * (size_t)d->T;  // as ffs_grid_build
  if (d->band)
    smem = std::max(smem, sizeof(double) * ((size_t)d->T + (d->T + 1) / 2 + (size_t)d->band_w + 1));
  FFS_REQUIRE(smem <= 200 * 1024, "ffs_grid_build_noalloc: T=%d too long", d->T);
  FFS_CUDA(ensure_dyn_smem(reinterpret_cast<const void*>(grid_build_kernel<false>), smem));
  grid_build_kernel<false><<<d->P, GB_THREADS, smem, (cudaStream_t)stream>>>(args, 1, nullptr, nullptr);
  return check_launch("grid_build_kernel (static scratch)");
}
