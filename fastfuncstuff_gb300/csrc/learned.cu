// The learned (a, b) proposal: simulation of training voxels and a
// 9 -> 64 -> 64 -> 2 GELU MLP with hand-written forward, backward and Adam
// kernels (the features come from the prep kernel, search.cu).
//
//   simulate  y_t = a y_{t-1} + e_t + b e_{t-1} per run (200 burn-in samples,
//             standardised per run), Y = X beta + sigma * noise, beta ~ N(0,1),
//             sigma ~ U(0.5, 2); normals from Philox4x32-10 (Salmon et al.,
//             SC'11) through Box-Muller.
//   MLP       exact-erf GELU; loss sum (out - y)^2 / (2 B); Adam.
#include "common.cuh"

namespace ffsk {
namespace {

// ------------------------------------------------------------------ Philox
struct Philox {
  uint32_t c0, c1, c2, c3, k0, k1;
  float cache[4];
  int left;

  __device__ Philox(uint64_t seed, uint32_t stream) {
    c0 = 0; c1 = 0; c2 = stream; c3 = 0;
    k0 = (uint32_t)seed;
    k1 = (uint32_t)(seed >> 32);
    left = 0;
  }

  __device__ void block(uint32_t r[4]) {
    uint32_t x0 = c0, x1 = c1, x2 = c2, x3 = c3, a = k0, b = k1;
#pragma unroll
    for (int i = 0; i < 10; ++i) {
      const uint32_t hi0 = __umulhi(0xD2511F53u, x0), lo0 = 0xD2511F53u * x0;
      const uint32_t hi1 = __umulhi(0xCD9E8D57u, x2), lo1 = 0xCD9E8D57u * x2;
      x0 = hi1 ^ x1 ^ a;
      x1 = lo1;
      x2 = hi0 ^ x3 ^ b;
      x3 = lo0;
      a += 0x9E3779B9u;
      b += 0xBB67AE85u;
    }
    r[0] = x0; r[1] = x1; r[2] = x2; r[3] = x3;
    if (++c0 == 0) ++c1;
  }

  // uniform in (0, 1]
  __device__ static float u01(uint32_t x) { return ((float)(x >> 8) + 1.0f) * (1.0f / 16777216.0f); }

  __device__ float normal() {
    if (left == 0) {
      uint32_t r[4];
      block(r);
      float rad0 = sqrtf(-2.0f * logf(u01(r[0])));
      float th0 = 6.28318530717958647692f * u01(r[1]);
      float rad1 = sqrtf(-2.0f * logf(u01(r[2])));
      float th1 = 6.28318530717958647692f * u01(r[3]);
      cache[0] = rad0 * cosf(th0);
      cache[1] = rad0 * sinf(th0);
      cache[2] = rad1 * cosf(th1);
      cache[3] = rad1 * sinf(th1);
      left = 4;
    }
    return cache[--left];
  }

  __device__ float uniform() {
    uint32_t r[4];
    block(r);
    return u01(r[0]);
  }
};

struct SimArgs {
  int V, T, K, n_runs;
  const int* run_start;
  const float* X;       // [T][K]
  const float* a;       // [V]
  const float* b;       // [V]
  uint64_t seed;
  float* Y;             // [V][T]
};

__global__ void simulate_kernel(SimArgs s) {
  const int v = blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= s.V) return;
  Philox rng(s.seed, (uint32_t)v);
  const float a = s.a[v], b = s.b[v];
  float* y = s.Y + (size_t)v * s.T;
  for (int r = 0; r < s.n_runs; ++r) {
    const int t0 = s.run_start[r], t1 = s.run_start[r + 1];
    float e_prev = rng.normal();
    float yt = e_prev;
    for (int i = 1; i < 200 + (t1 - t0); ++i) {
      const float e = rng.normal();
      yt = a * yt + e + b * e_prev;
      e_prev = e;
      if (i >= 200) y[t0 + i - 200] = yt;
    }
    double m = 0.0, q = 0.0;
    for (int t = t0; t < t1; ++t) m += y[t];
    m /= (double)(t1 - t0);
    for (int t = t0; t < t1; ++t) q += ((double)y[t] - m) * ((double)y[t] - m);
    const double sd = (t1 - t0 > 1) ? sqrt(q / (double)(t1 - t0 - 1)) : 1.0;
    const float inv = sd > 0.0 ? (float)(1.0 / sd) : 0.f;
    for (int t = t0; t < t1; ++t) y[t] = (float)(((double)y[t] - m) * inv);
  }
  const float sigma = 0.5f + 1.5f * rng.uniform();
  float beta[64];
  const int K = s.K;
  for (int j0 = 0; j0 < K; j0 += 64) {
    const int nj = min(64, K - j0);
    for (int j = 0; j < nj; ++j) beta[j] = rng.normal();
    for (int t = 0; t < s.T; ++t) {
      float acc = (j0 == 0) ? sigma * y[t] : y[t];
      for (int j = 0; j < nj; ++j) acc = fmaf(s.X[(size_t)t * K + j0 + j], beta[j], acc);
      y[t] = acc;
    }
  }
}

// --------------------------------------------------------------------- MLP
constexpr int NI = 9, NH = 64, NO = 2;
constexpr int OFF_W1 = 0, OFF_B1 = OFF_W1 + NH * NI, OFF_W2 = OFF_B1 + NH, OFF_B2 = OFF_W2 + NH * NH,
              OFF_W3 = OFF_B2 + NH, OFF_B3 = OFF_W3 + NO * NH, N_PARAMS = OFF_B3 + NO;

__device__ __forceinline__ float gelu(float z) { return 0.5f * z * (1.0f + erff(z * 0.70710678118654752f)); }
__device__ __forceinline__ float gelu_grad(float z) {
  return 0.5f * (1.0f + erff(z * 0.70710678118654752f)) + z * expf(-0.5f * z * z) * 0.3989422804014327f;
}

// Two samples per thread: every weight read from shared memory serves both,
// and the two dependent FMA chains of a unit interleave.
constexpr int FWD_PER_THREAD = 2;

__global__ void __launch_bounds__(128) mlp_forward_kernel(const float* __restrict__ prm, const float* __restrict__ x,
                                                          int B, float* __restrict__ out) {
  __shared__ float P[N_PARAMS];
  for (int i = threadIdx.x; i < N_PARAMS; i += blockDim.x) P[i] = prm[i];
  __syncthreads();
  const int s0 = (blockIdx.x * blockDim.x + threadIdx.x) * FWD_PER_THREAD;
  if (s0 >= B) return;
  const bool two = s0 + 1 < B;
  float xa[NI], xb[NI], ha[NH], hb[NH];
#pragma unroll
  for (int i = 0; i < NI; ++i) {
    xa[i] = x[(size_t)s0 * NI + i];
    xb[i] = two ? x[(size_t)(s0 + 1) * NI + i] : 0.f;
  }
#pragma unroll
  for (int u = 0; u < NH; ++u) {
    float za = P[OFF_B1 + u], zb = za;
#pragma unroll
    for (int i = 0; i < NI; ++i) {
      const float w = P[OFF_W1 + u * NI + i];
      za = fmaf(w, xa[i], za);
      zb = fmaf(w, xb[i], zb);
    }
    ha[u] = gelu(za);
    hb[u] = gelu(zb);
  }
  float oa0 = P[OFF_B3], oa1 = P[OFF_B3 + 1], ob0 = oa0, ob1 = oa1;
  for (int u = 0; u < NH; ++u) {
    float za = P[OFF_B2 + u], zb = za;
#pragma unroll
    for (int k = 0; k < NH; ++k) {
      const float w = P[OFF_W2 + u * NH + k];
      za = fmaf(w, ha[k], za);
      zb = fmaf(w, hb[k], zb);
    }
    const float ga = gelu(za), gb = gelu(zb);
    const float w0 = P[OFF_W3 + u], w1 = P[OFF_W3 + NH + u];
    oa0 = fmaf(w0, ga, oa0);
    oa1 = fmaf(w1, ga, oa1);
    ob0 = fmaf(w0, gb, ob0);
    ob1 = fmaf(w1, gb, ob1);
  }
  out[(size_t)s0 * NO] = oa0;
  out[(size_t)s0 * NO + 1] = oa1;
  if (two) {
    out[(size_t)(s0 + 1) * NO] = ob0;
    out[(size_t)(s0 + 1) * NO + 1] = ob1;
  }
}

// One CTA = TILE samples. Forward, loss, backward into shared memory, then the
// tile's parameter gradients are summed over its samples and added to grad.
constexpr int TILE = 16;  // keeps the CTA's static shared memory under 48 KB

__global__ void __launch_bounds__(256) mlp_grad_kernel(const float* __restrict__ prm, const float* __restrict__ x,
                                                       const float* __restrict__ y, const int* __restrict__ idx,
                                                       int B, float inv_n, float* __restrict__ grad,
                                                       float* __restrict__ loss) {
  __shared__ float P[N_PARAMS];
  __shared__ float X[TILE][NI];
  __shared__ float Z1[TILE][NH], H1[TILE][NH], Z2[TILE][NH], H2[TILE][NH], D1[TILE][NH], D2[TILE][NH];
  __shared__ float DO[TILE][NO];
  __shared__ float lsum;
  const int tid = threadIdx.x, nt = blockDim.x;
  const int s0 = blockIdx.x * TILE;
  const int ns = min(TILE, B - s0);
  for (int i = tid; i < N_PARAMS; i += nt) P[i] = prm[i];
  for (int i = tid; i < TILE * NI; i += nt) {
    const int s = i / NI, k = i % NI;
    X[s][k] = s < ns ? x[(size_t)(idx ? idx[s0 + s] : s0 + s) * NI + k] : 0.f;
  }
  if (tid == 0) lsum = 0.f;
  __syncthreads();
  for (int i = tid; i < TILE * NH; i += nt) {
    const int s = i / NH, u = i % NH;
    float z = P[OFF_B1 + u];
#pragma unroll
    for (int k = 0; k < NI; ++k) z = fmaf(P[OFF_W1 + u * NI + k], X[s][k], z);
    Z1[s][u] = z;
    H1[s][u] = gelu(z);
  }
  __syncthreads();
  for (int i = tid; i < TILE * NH; i += nt) {
    const int s = i / NH, u = i % NH;
    float z = P[OFF_B2 + u];
    for (int k = 0; k < NH; ++k) z = fmaf(P[OFF_W2 + u * NH + k], H1[s][k], z);
    Z2[s][u] = z;
    H2[s][u] = gelu(z);
  }
  __syncthreads();
  for (int i = tid; i < TILE * NO; i += nt) {
    const int s = i / NO, o = i % NO;
    float z = P[OFF_B3 + o];
    for (int k = 0; k < NH; ++k) z = fmaf(P[OFF_W3 + o * NH + k], H2[s][k], z);
    float e = 0.f;
    if (s < ns) e = z - y[(size_t)(idx ? idx[s0 + s] : s0 + s) * NO + o];
    DO[s][o] = e * inv_n;
    atomicAdd(&lsum, 0.5f * e * e * inv_n);
  }
  __syncthreads();
  for (int i = tid; i < TILE * NH; i += nt) {
    const int s = i / NH, k = i % NH;
    const float dh = P[OFF_W3 + k] * DO[s][0] + P[OFF_W3 + NH + k] * DO[s][1];
    D2[s][k] = dh * gelu_grad(Z2[s][k]);
  }
  __syncthreads();
  for (int i = tid; i < TILE * NH; i += nt) {
    const int s = i / NH, k = i % NH;
    float dh = 0.f;
    for (int u = 0; u < NH; ++u) dh = fmaf(P[OFF_W2 + u * NH + k], D2[s][u], dh);
    D1[s][k] = dh * gelu_grad(Z1[s][k]);
  }
  __syncthreads();
  for (int pi = tid; pi < N_PARAMS; pi += nt) {
    float g = 0.f;
    if (pi < OFF_B1) {
      const int u = pi / NI, k = pi % NI;
      for (int s = 0; s < ns; ++s) g = fmaf(D1[s][u], X[s][k], g);
    } else if (pi < OFF_W2) {
      const int u = pi - OFF_B1;
      for (int s = 0; s < ns; ++s) g += D1[s][u];
    } else if (pi < OFF_B2) {
      const int u = (pi - OFF_W2) / NH, k = (pi - OFF_W2) % NH;
      for (int s = 0; s < ns; ++s) g = fmaf(D2[s][u], H1[s][k], g);
    } else if (pi < OFF_W3) {
      const int u = pi - OFF_B2;
      for (int s = 0; s < ns; ++s) g += D2[s][u];
    } else if (pi < OFF_B3) {
      const int o = (pi - OFF_W3) / NH, k = (pi - OFF_W3) % NH;
      for (int s = 0; s < ns; ++s) g = fmaf(DO[s][o], H2[s][k], g);
    } else {
      const int o = pi - OFF_B3;
      for (int s = 0; s < ns; ++s) g += DO[s][o];
    }
    atomicAdd(grad + pi, g);
  }
  if (tid == 0 && loss) atomicAdd(loss, lsum);
}

// Adam with bias correction; consumes and zeroes the gradient.
__global__ void adam_kernel(float* prm, float* grad, float* m, float* v, int n, float lr, float b1, float b2,
                            float eps, float c1, float c2) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float g = grad[i];
  const float mi = b1 * m[i] + (1.f - b1) * g;
  const float vi = b2 * v[i] + (1.f - b2) * g * g;
  m[i] = mi;
  v[i] = vi;
  prm[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
  grad[i] = 0.f;
}

}  // namespace
}  // namespace ffsk

using namespace ffsk;

extern "C" int ffs_mlp_param_count(void) { return N_PARAMS; }

extern "C" int ffs_arma_simulate(int V, int T, int K, int n_runs, const int* run_start, const float* X,
                                 const float* a, const float* b, uint64_t seed, float* Y, void* stream) {
  clear_error();
  FFS_REQUIRE(V > 0 && T > 0 && K >= 0 && n_runs > 0, "ffs_arma_simulate: bad sizes");
  FFS_REQUIRE(run_start && a && b && Y && (K == 0 || X), "ffs_arma_simulate: null buffer");
  SimArgs s{V, T, K, n_runs, run_start, X, a, b, seed, Y};
  simulate_kernel<<<ceil_div(V, 128), 128, 0, (cudaStream_t)stream>>>(s);
  return check_launch("simulate_kernel");
}

extern "C" int ffs_mlp_forward(const float* params, const float* x, int B, float* out, void* stream) {
  clear_error();
  FFS_REQUIRE(params && x && out && B > 0, "ffs_mlp_forward: bad arguments");
  mlp_forward_kernel<<<ceil_div(B, 128 * FWD_PER_THREAD), 128, 0, (cudaStream_t)stream>>>(params, x, B, out);
  return check_launch("mlp_forward_kernel");
}

extern "C" int ffs_mlp_grad(const float* params, const float* x, const float* y, const int* idx, int B, int n_total,
                            float* grad, float* loss, void* stream) {
  clear_error();
  FFS_REQUIRE(params && x && y && grad && B > 0 && n_total > 0, "ffs_mlp_grad: bad arguments");
  mlp_grad_kernel<<<ceil_div(B, TILE), 256, 0, (cudaStream_t)stream>>>(params, x, y, idx, B, 1.0f / (float)n_total,
                                                                       grad, loss);
  return check_launch("mlp_grad_kernel");
}

extern "C" int ffs_mlp_adam(float* params, float* grad, float* m, float* v, int n, float lr, float beta1, float beta2,
                            float eps, int step, void* stream) {
  clear_error();
  FFS_REQUIRE(params && grad && m && v && n > 0 && step > 0, "ffs_mlp_adam: bad arguments");
  const float c1 = 1.0f - powf(beta1, (float)step), c2 = 1.0f - powf(beta2, (float)step);
  adam_kernel<<<ceil_div(n, 256), 256, 0, (cudaStream_t)stream>>>(params, grad, m, v, n, lr, beta1, beta2, eps, c1,
                                                                  c2);
  return check_launch("adam_kernel");
}
