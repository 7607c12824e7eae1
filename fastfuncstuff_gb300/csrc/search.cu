// Search-side kernels of the REML grid search:
//   prep     per-voxel std scaling + residualisation against the design
//   surface  y'R^-1 y by the O(T) recurrence for every (voxel, pair) and the
//            REML criterion, relative to the pair (0, 0)
//   select   exhaustive argmin or AFNI's hierarchical descent
//   group    counting sort of voxels by their chosen pair
//   project  (CUDA-core form) ||U'y||^2 for every (voxel, pair)
#include "common.cuh"
#include "tile.cuh"

namespace ffsk {

namespace {

// ------------------------------------------------------------------------ prep
__device__ __forceinline__ bool centre_on(const ffs_prep_args& a) {
  return a.center_dev ? (*a.center_dev != 0) : (a.center != 0);
}

// Lag 1..8 autocorrelations of one residualised row within runs (products
// never cross a run boundary) and T/1000, by one warp; lane 0 writes out[9].
// Each lane walks a contiguous stretch of every run backwards, keeping the 8
// following samples in registers, so a sample is read once.
__device__ void row_features(const float* row, int T, int n_runs, const int* run_start, float* out) {
  const int lane = threadIdx.x & 31;
  float acc[8], s0 = 0.f;
#pragma unroll
  for (int k = 0; k < 8; ++k) acc[k] = 0.f;
  for (int r = 0; r < n_runs; ++r) {
    const int t0 = run_start[r], t1 = run_start[r + 1];
    const int len = (t1 - t0 + 31) / 32;
    const int a = min(t1, t0 + lane * len), b = min(t1, a + len);
    float w[8];  // w[k] = y_{t+1+k} (0 past the run's end)
#pragma unroll
    for (int k = 0; k < 8; ++k) w[k] = b + k < t1 ? row[b + k] : 0.f;
    for (int t = b - 1; t >= a; --t) {
      const float y = row[t];
      s0 = fmaf(y, y, s0);
#pragma unroll
      for (int k = 0; k < 8; ++k) acc[k] = fmaf(y, w[k], acc[k]);
#pragma unroll
      for (int k = 7; k > 0; --k) w[k] = w[k - 1];
      w[0] = y;
    }
  }
  s0 = warp_sum(s0);
#pragma unroll
  for (int k = 0; k < 8; ++k) acc[k] = warp_sum(acc[k]);
  if (lane == 0) {
#pragma unroll
    for (int k = 0; k < 8; ++k) out[k] = s0 > 0.f ? acc[k] / s0 : 0.f;
    out[8] = (float)T / 1000.0f;
  }
}

// 8 warps, 32 voxels per CTA (4 per warp). The residualised rows are staged in
// shared memory and written out time-major in coalesced 128-byte rows.
constexpr int PREP_VOX = 32;

__global__ void __launch_bounds__(256) prep_kernel(ffs_prep_args a, int ld_s) {
  extern __shared__ float sm[];  // [PREP_VOX][ld_s]
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int T = a.T, K = a.K;
  const int v0 = blockIdx.x * PREP_VOX;
  const int LT = ld_t(T);
  const float* Q0 = a.Q0 + (a.tile_design ? (size_t)a.tile_design[blockIdx.x] * K * LT : 0);
  for (int k = 0; k < PREP_VOX / 8; ++k) {
    const int lv = wid * (PREP_VOX / 8) + k;
    const int v = v0 + lv;
    if (v >= a.V) break;  // warp-uniform
    const int vs = a.idx ? a.idx[v] : v;  // source row (< 0: an empty row)
    float* row = sm + (size_t)lv * ld_s;
    const float* y = vs >= 0 ? a.Y + (size_t)vs * T : nullptr;
    // mean and (N-1) variance, two passes for accuracy
    float s = 0.f;
    for (int t = lane; t < T; t += 32) {
      const float x = y ? y[t] : 0.f;
      row[t] = x;
      s += x;
    }
    const float mean = warp_sum(s) / (float)T;
    float q = 0.f;
    for (int t = lane; t < T; t += 32) {
      const float dlt = row[t] - mean;
      q += dlt * dlt;
    }
    q = warp_sum(q);
    float sc = 1.0f;
    if (a.do_scale) {
      sc = T > 1 ? sqrtf(q / (float)(T - 1)) : 0.f;
      sc = fmaxf(sc, 1e-8f);
    }
    // centring is one subtraction per sample, rounded relative to its (small)
    // result; the criterion ignores the constant when it lies in span(X)
    const float m = centre_on(a) ? mean : 0.f;
    for (int t = lane; t < T; t += 32) row[t] = __fdiv_rn(__fsub_rn(row[t], m), sc);
    __syncwarp();
    // residualise: row -= Q0 (Q0' row)
    for (int j = 0; j < K; ++j) {
      const float* qj = Q0 + (size_t)j * LT;
      float c = 0.f;
      for (int t = lane; t < T; t += 32) c += qj[t] * row[t];
      c = warp_sum(c);
      for (int t = lane; t < T; t += 32) row[t] -= c * qj[t];
      __syncwarp();
    }
    if (lane == 0 && vs >= 0) a.scale[vs] = sc;
    if (a.feats) row_features(row, T, a.n_runs, a.run_start, a.feats + (size_t)v * 9);
    if (a.yr_hi || a.yexp) {
      float amax = 0.f;
      for (int t = lane; t < T; t += 32) amax = fmaxf(amax, fabsf(row[t]));
      for (int off = 16; off > 0; off >>= 1) amax = fmaxf(amax, __shfl_xor_sync(0xffffffffu, amax, off));
      const int e = scale_exp(amax);
      if (lane == 0) a.yexp[v] = e;
      if (!a.yr_hi) continue;
      uint16_t* hi = a.yr_hi + (size_t)v * a.ld_y;
      uint16_t* lo = a.yr_lo + (size_t)v * a.ld_y;
      for (int t = lane; t < a.ld_y; t += 32) {
        uint16_t h = 0, l = 0;
        if (t < T) split_fp16(ldexpf(row[t], e), h, l);
        hi[t] = h;
        lo[t] = l;
      }
    }
  }
  __syncthreads();
  // time-major store: warp w writes rows t = w, w+8, ...; lane = voxel
  const int nv = min(PREP_VOX, a.V - v0);
  if (a.yr_rows) {
    for (int k = 0; k < PREP_VOX / 8; ++k) {
      const int lv = wid * (PREP_VOX / 8) + k;
      if (lv >= nv) break;
      for (int t = lane; t < T; t += 32) a.yr_rows[(size_t)(v0 + lv) * T + t] = sm[(size_t)lv * ld_s + t];
    }
  }
  if (!a.yr_t) return;
  for (int t = wid; t < T; t += 8) {
    if (lane < nv) a.yr_t[(size_t)t * a.V + v0 + lane] = sm[(size_t)lane * ld_s + t];
  }
}

// Tiled form: 32 voxels per CTA, the projection c = Q0 y and the update
// y -= Q0' c as register-blocked passes over the tile (tile.cuh), i.e.
// y - Q0'(Q0 y) in one step as the reference's Y - (Y pinv(X)') X'
// (fastfuncstuff/glm/arma.py:1554-1571). Rows of Y are read as 16-byte words
// when T % 4 == 0 and as single samples otherwise; the tile's samples
// T .. ld_t(T) stay zero.
__global__ void __launch_bounds__(TILE_WARPS * 32, 3) prep_tile_kernel(ffs_prep_args a, int ld) {
  extern __shared__ float4 sm4[];
  float* Ys = reinterpret_cast<float*>(sm4);       // [32][ld]
  float* Cq = Ys + (size_t)TILE_V * ld;            // [K][32]
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int T = a.T, K = a.K, LT = ld_t(T), nq = LT >> 2;
  const bool vec = (T & 3) == 0;  // 16-byte rows of the [V][T] outputs
  const int v0 = blockIdx.x * TILE_V;
  const int nv = min(TILE_V, a.V - v0);
  __shared__ int src_row[TILE_V];  // source row of each tile row (-1: zero row)
  if (threadIdx.x < TILE_V) {
    const int i = threadIdx.x;
    src_row[i] = i >= nv ? -1 : (a.idx ? a.idx[v0 + i] : v0 + i);
  }
  __syncthreads();
  if (a.Y_ref) {
    // the input through its address held on the device (device memory): the
    // tile's rows staged by asynchronous copies, all in flight at once, then
    // written out from shared memory as read for the later stages (T % 4 == 0)
    tile_stage_rows(*a.Y_ref, T, nq, src_row, Ys, ld);
    if (a.Y_copy) {
      for (int i = wid; i < nv; i += TILE_WARPS) {
        const int v = src_row[i];
        if (v < 0) continue;  // warp-uniform
        const float4* row4 = reinterpret_cast<const float4*>(Ys + (size_t)i * ld);
        float4* cpy = reinterpret_cast<float4*>(a.Y_copy + (size_t)v * T);
        for (int q = lane; q < nq; q += 32) cpy[q] = row4[q];
      }
    }
  } else {
    tile_stage_rows(a.Y, T, nq, src_row, Ys, ld);
  }
  for (int i = wid; i < nv; i += TILE_WARPS) {
    const int vs = src_row[i];
    if (vs < 0) continue;  // warp-uniform: an empty (padding) row stays zero
    float* row = Ys + (size_t)i * ld;
    const float4* row4 = reinterpret_cast<const float4*>(row);
    // mean and (N-1) variance, two passes for accuracy
    float s = 0.f;
    for (int q = lane; q < nq; q += 32) {
      const float4 x = row4[q];
      s += ((x.x + x.y) + x.z) + x.w;
    }
    const float mean = warp_sum(s) / (float)T;
    float sq = 0.f;
    if (vec) {  // whole quads: no padding inside the row
      for (int q = lane; q < nq; q += 32) {
        const float4 x = row4[q];
        const float d0 = x.x - mean, d1 = x.y - mean, d2 = x.z - mean, d3 = x.w - mean;
        sq += ((d0 * d0 + d1 * d1) + d2 * d2) + d3 * d3;
      }
    } else {
      for (int t = lane; t < T; t += 32) {
        const float dlt = row[t] - mean;
        sq += dlt * dlt;
      }
    }
    sq = warp_sum(sq);
    float sc = 1.0f;
    if (a.do_scale) {
      sc = sqrtf(sq / (float)(T - 1));
      sc = fmaxf(sc, 1e-8f);
    }
    const float m = centre_on(a) ? mean : 0.f;
    if (vec) {
      float4* rw4 = reinterpret_cast<float4*>(row);
      for (int q = lane; q < nq; q += 32) {
        const float4 x = rw4[q];
        rw4[q] = make_float4(__fdiv_rn(__fsub_rn(x.x, m), sc), __fdiv_rn(__fsub_rn(x.y, m), sc),
                             __fdiv_rn(__fsub_rn(x.z, m), sc), __fdiv_rn(__fsub_rn(x.w, m), sc));
      }
    } else {
      for (int t = lane; t < T; t += 32) row[t] = __fdiv_rn(__fsub_rn(row[t], m), sc);
    }
    if (lane == 0) a.scale[vs] = sc;
  }
  __syncthreads();
  if (K > 0) {
    const float* Q0 = a.Q0 + (a.tile_design ? (size_t)a.tile_design[blockIdx.x] * K * LT : 0);
    tile_project(Q0, LT, Ys, ld, K, Cq);
    tile_subtract_any(Q0, LT, Cq, Ys, ld, K);
  }
  __syncthreads();
  if (a.feats) {
    for (int i = wid; i < nv; i += TILE_WARPS)
      row_features(Ys + (size_t)i * ld, T, a.n_runs, a.run_start, a.feats + (size_t)(v0 + i) * 9);
  }
  if (a.yr_hi || a.yexp) {  // the split's exponent; the split itself with yr_hi
    for (int i = wid; i < nv; i += TILE_WARPS) {
      const float* row = Ys + (size_t)i * ld;
      const int v = v0 + i;
      float amax = 0.f;
      for (int q = lane; q < nq; q += 32) {
        const float4 x = reinterpret_cast<const float4*>(row)[q];
        amax = fmaxf(fmaxf(amax, fabsf(x.x)), fmaxf(fabsf(x.y), fmaxf(fabsf(x.z), fabsf(x.w))));
      }
      for (int off = 16; off > 0; off >>= 1) amax = fmaxf(amax, __shfl_xor_sync(0xffffffffu, amax, off));
      const int e = scale_exp(amax);
      if (lane == 0) a.yexp[v] = e;
      if (!a.yr_hi) continue;
      // two samples per lane: 32-bit stores of (hi_t, hi_t+1)
      uint32_t* hi = reinterpret_cast<uint32_t*>(a.yr_hi + (size_t)v * a.ld_y);
      uint32_t* lo = reinterpret_cast<uint32_t*>(a.yr_lo + (size_t)v * a.ld_y);
      // x * 2^e as one product when 2^e is a normal float (then the same
      // correctly rounded value as ldexpf)
      const bool pw = e >= -126 && e <= 127;
      const float p2 = pw ? __int_as_float((e + 127) << 23) : 0.f;
      for (int t2 = lane; t2 < (a.ld_y >> 1); t2 += 32) {
        uint16_t h0 = 0, l0 = 0, h1 = 0, l1 = 0;
        const int t = 2 * t2;
        if (t < T) split_fp16(pw ? __fmul_rn(row[t], p2) : ldexpf(row[t], e), h0, l0);
        if (t + 1 < T) split_fp16(pw ? __fmul_rn(row[t + 1], p2) : ldexpf(row[t + 1], e), h1, l1);
        hi[t2] = (uint32_t)h0 | ((uint32_t)h1 << 16);
        lo[t2] = (uint32_t)l0 | ((uint32_t)l1 << 16);
      }
    }
  }
  if (a.yr_rows) {  // voxel-major rows, a warp per row
    for (int i = wid; i < nv; i += TILE_WARPS) {
      const float* r = Ys + (size_t)i * ld;
      float* o = a.yr_rows + (size_t)(v0 + i) * T;
      if (vec) {
        for (int q = lane; q < nq; q += 32) reinterpret_cast<float4*>(o)[q] = reinterpret_cast<const float4*>(r)[q];
      } else {
        for (int t = lane; t < T; t += 32) o[t] = r[t];
      }
    }
  }
  // time-major store: lane = voxel (coalesced 128-byte rows), warp w takes
  // quads w, w + 8, ...
  if (a.yr_t && lane < nv) {
    const float4* r4 = reinterpret_cast<const float4*>(Ys + (size_t)lane * ld);
    float* out = a.yr_t + v0 + lane;
    const size_t V = (size_t)a.V;
    for (int q = wid; q < nq; q += TILE_WARPS) {
      const float4 r = r4[q];
      const int t = 4 * q;
      out[(size_t)t * V] = r.x;
      if (t + 1 < T) out[(size_t)(t + 1) * V] = r.y;
      if (t + 2 < T) out[(size_t)(t + 2) * V] = r.z;
      if (t + 3 < T) out[(size_t)(t + 3) * V] = r.w;
    }
  }
}

// --------------------------------------------------------------------- surface
// One thread per voxel, one CTA per (chunk of 16 pair slots, voxel tile). A
// chunk is 4 quarters of up to 4 pairs; the pairs of a quarter share one AR
// filter c_t (one a, or lambda == 0), so each step forms z = y_t - c_t y_{t-1}
// once per quarter. For each pair: v_t = z_t - m_t v_{t-1}, s += v_t^2 / D_t.
// The chunk's coefficient table is staged in shared memory as (-m, 1/D) of
// pair couples, so each couple advances with packed fma.rn.f32x2 /
// mul.rn.f32x2 instructions. A step whose coefficients equal the previous
// step's for every pair of the chunk (the LDL' factor of a Toeplitz run
// converges to a constant, so most steps after a short transient are such
// "steady" steps) reuses the registers instead of reloading them. Each thread
// prefetches 16 samples of its voxel at a time so the loads overlap; a block of
// 16 steady steps sums v_t^2 alone and multiplies the block's sum by the
// common 1/D once (two packed instructions per pair couple and step). A chunk
// of identity pairs only (R = I) sums y_t^2 once for all of them.
constexpr int SURF_G = 16;
constexpr int SURF_G2 = SURF_G / 2;
constexpr int SURF_THREADS = 256;
constexpr int SURF_TB = 16;  // time steps per prefetch block

__global__ void __launch_bounds__(SURF_THREADS, 2) surface_kernel(ffs_surface_args a) {
  extern __shared__ float4 cf4[];  // [T][SURF_G2] (-m_2k, -m_2k+1, 1/D_2k, 1/D_2k+1)
  float4* cs4 = cf4 + (size_t)a.T * SURF_G2;                        // [T] c_t of the 4 quarters
  float* dcs = reinterpret_cast<float*>(cs4 + a.T);                 // [SURF_G] const_p - const_p0
  uint8_t* steady = reinterpret_cast<uint8_t*>(dcs + SURF_G);       // [T]
  uint8_t* bsteady = steady + a.T;                                  // [ceil(T / SURF_TB)]
  // chunks are the fast grid dimension: the CTAs of one voxel tile run together
  // and its samples stay in L2 across the chunks
  const int chunk = blockIdx.x;
  const int c0 = a.chunk_start[chunk], c1 = a.chunk_start[chunk + 1];
  const int ng = c1 - c0;
  const int T = a.T;
  const float4* coef = reinterpret_cast<const float4*>(a.coef);
  auto pair_of = [&](int slot) { return slot < ng ? a.chunk_pairs[c0 + slot] : -1; };
  // coefficient table; an empty slot keeps m = 0, 1/D = 0 (its sum stays 0).
  // ident: every filled slot is the identity (lambda == 0: c = m = 0, D = 1)
  int ident = 1;
  for (int idx = threadIdx.x; idx < T * SURF_G2; idx += blockDim.x) {
    const int t = idx / SURF_G2, k = idx % SURF_G2;
    float4 val = make_float4(0.f, 0.f, 0.f, 0.f);
    const int p0 = pair_of(2 * k), p1 = pair_of(2 * k + 1);
    if (p0 >= 0) {
      const float4 q = coef[(size_t)p0 * T + t];
      val.x = -q.y;
      val.z = q.z;
      ident &= q.x == 0.f && q.y == 0.f && q.z == 1.f;
    }
    if (p1 >= 0) {
      const float4 q = coef[(size_t)p1 * T + t];
      val.y = -q.y;
      val.w = q.z;
      ident &= q.x == 0.f && q.y == 0.f && q.z == 1.f;
    }
    cf4[idx] = val;
  }
  for (int t = threadIdx.x; t < T; t += blockDim.x) {
    float cq[4];
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      // the quarter's first filled slot carries its AR filter
      int p = -1;
      for (int s2 = 4 * q; s2 < 4 * q + 4 && p < 0; ++s2) p = pair_of(s2);
      cq[q] = p >= 0 ? coef[(size_t)p * T + t].x : 0.f;
    }
    cs4[t] = make_float4(cq[0], cq[1], cq[2], cq[3]);
  }
  const double* ldx = a.logdet_XtX + (a.tile_design ? (size_t)a.tile_design[blockIdx.y] * a.P : 0);
  if (threadIdx.x < SURF_G) {
    const double c_p0 = a.logdet_R[a.p0] + ldx[a.p0];
    const int p = pair_of(threadIdx.x);
    dcs[threadIdx.x] = p >= 0 ? (float)((a.logdet_R[p] + ldx[p]) - c_p0) : 0.f;
  }
  ident = __syncthreads_and(ident);
  for (int t = threadIdx.x; t < T; t += blockDim.x) {
    bool same = false;
    if (t > 0) {
      const float4 u = cs4[t], w = cs4[t - 1];
      same = u.x == w.x && u.y == w.y && u.z == w.z && u.w == w.w;
    }
    for (int k = 0; k < SURF_G2 && same; ++k) {
      const float4 x = cf4[t * SURF_G2 + k], y = cf4[(t - 1) * SURF_G2 + k];
      same = x.x == y.x && x.y == y.y && x.z == y.z && x.w == y.w;
    }
    steady[t] = same ? 1 : 0;
  }
  __syncthreads();
  // a block is steady when all its SURF_TB steps are (a partial last block never is)
  for (int bk = threadIdx.x; bk * SURF_TB < T; bk += blockDim.x) {
    bool all = bk * SURF_TB + SURF_TB <= T;
    for (int t = bk * SURF_TB; t < bk * SURF_TB + SURF_TB && all; ++t) all = steady[t] != 0;
    bsteady[bk] = all ? 1 : 0;
  }
  __syncthreads();

  const int v = blockIdx.y * SURF_THREADS + threadIdx.x;
  if (v >= a.V) return;
  const float* yc = a.yr_t + v;
  float yy = 0.f;
  float sg[SURF_G];
  if (ident) {
    // R = I for every pair of the chunk: y'R^-1 y = sum y^2, accumulated in
    // the same blocks and order as the recurrence (bit-identical to it)
    for (int t0 = 0; t0 < T; t0 += SURF_TB) {
      float yy_b = 0.f;
#pragma unroll 8
      for (int k = 0; k < SURF_TB; ++k) {
        if (t0 + k < T) {
          const float y = yc[(size_t)(t0 + k) * a.V];
          yy_b = fmaf(y, y, yy_b);
        }
      }
      yy += yy_b;
    }
#pragma unroll
    for (int g = 0; g < SURF_G; ++g) sg[g] = yy;
  } else {
    uint64_t vv[SURF_G2], sb[SURF_G2], st[SURF_G2], nm[SURF_G2], id[SURF_G2];
    const uint64_t zero2 = pack2(0.f, 0.f);
#pragma unroll
    for (int k = 0; k < SURF_G2; ++k) vv[k] = sb[k] = st[k] = nm[k] = id[k] = zero2;
    float4 c = make_float4(0.f, 0.f, 0.f, 0.f);
    float yy_b = 0.f, yp = 0.f;
    for (int t0 = 0; t0 < T; t0 += SURF_TB) {
      float yb[SURF_TB];
#pragma unroll
      for (int k = 0; k < SURF_TB; ++k) yb[k] = (t0 + k < T) ? yc[(size_t)(t0 + k) * a.V] : 0.f;
      if (bsteady[t0 / SURF_TB]) {
        // SURF_TB steady steps: the coefficients in registers hold for all of them
#pragma unroll
        for (int k = 0; k < SURF_TB; ++k) {
          const float y = yb[k];
          uint64_t z2[4];
          z2[0] = pack2(fmaf(-c.x, yp, y), fmaf(-c.x, yp, y));
          z2[1] = pack2(fmaf(-c.y, yp, y), fmaf(-c.y, yp, y));
          z2[2] = pack2(fmaf(-c.z, yp, y), fmaf(-c.z, yp, y));
          z2[3] = pack2(fmaf(-c.w, yp, y), fmaf(-c.w, yp, y));
          yp = y;
          yy_b = fmaf(y, y, yy_b);
#pragma unroll
          for (int j = 0; j < SURF_G2; ++j) vv[j] = fma2(nm[j], vv[j], z2[j >> 1]);
#pragma unroll
          for (int j = 0; j < SURF_G2; ++j) sb[j] = fma2(vv[j], vv[j], sb[j]);
        }
#pragma unroll
        for (int j = 0; j < SURF_G2; ++j) {
          st[j] = fma2(sb[j], id[j], st[j]);
          sb[j] = zero2;
        }
      } else {
#pragma unroll
        for (int k = 0; k < SURF_TB; ++k) {
          const int t = t0 + k;
          if (t < T) {
            if (!steady[t]) {
              c = cs4[t];
              const float4* row = cf4 + (size_t)t * SURF_G2;
#pragma unroll
              for (int j = 0; j < SURF_G2; ++j) {
                const float4 q = row[j];
                nm[j] = pack2(q.x, q.y);
                id[j] = pack2(q.z, q.w);
              }
            }
            const float y = yb[k];
            uint64_t z2[4];
            z2[0] = pack2(fmaf(-c.x, yp, y), fmaf(-c.x, yp, y));
            z2[1] = pack2(fmaf(-c.y, yp, y), fmaf(-c.y, yp, y));
            z2[2] = pack2(fmaf(-c.z, yp, y), fmaf(-c.z, yp, y));
            z2[3] = pack2(fmaf(-c.w, yp, y), fmaf(-c.w, yp, y));
            yp = y;
            yy_b = fmaf(y, y, yy_b);
#pragma unroll
            for (int j = 0; j < SURF_G2; ++j) {
              vv[j] = fma2(nm[j], vv[j], z2[j >> 1]);
              sb[j] = fma2(mul2(vv[j], id[j]), vv[j], sb[j]);
            }
          }
        }
#pragma unroll
        for (int j = 0; j < SURF_G2; ++j) {
          st[j] = add2(st[j], sb[j]);
          sb[j] = zero2;
        }
      }
      yy += yy_b;
      yy_b = 0.f;
    }
#pragma unroll
    for (int j = 0; j < SURF_G2; ++j) unpack2(st[j], sg[2 * j], sg[2 * j + 1]);
  }
  const int Tk = a.T - a.K;
  const float rss0 = fmaxf(yy - a.proj[(size_t)a.p0 * a.V + v], 0.f);
  const float den = rss0 + 1e-10f;
#pragma unroll
  for (int g = 0; g < SURF_G; ++g) {
    const int p = pair_of(g);
    if (p >= 0) {
      const float rss = fmaxf(sg[g] - a.proj[(size_t)p * a.V + v], 0.f);
      const float dv = dcs[g] + (float)Tk * log1pf((rss - rss0) / den);
      a.surf[(size_t)p * a.V + v] = dv;
    }
  }
  if (chunk == 0) a.crit0[v] = (a.logdet_R[a.p0] + ldx[a.p0]) + (double)Tk * log((double)rss0 + 1e-10);
}

// ------------------------------------------------------------- banded surface
// AFNI's banded R: one CTA per (pair, tile of SB_THREADS voxels), one thread
// per voxel. Each step forms w_t = y_t c[t][0] - sum_{j <= band} c[t][j] w_{t-j}
// against the last band_w - 1 values of w, kept per thread in a ring in
// shared memory ([slot][thread], so a warp's accesses fall in distinct banks);
// the coefficients of SB_STEPS steps are staged in shared memory at a time
// and read by every thread (broadcast). y'R^-1 y = sum w_t^2, and the
// criterion as the surface kernel forms it.
constexpr int SB_THREADS = 128;
static_assert(256 % SB_THREADS == 0, "a CTA's voxels lie in one 256-voxel design tile");
constexpr int SB_STEPS = 32;

__global__ void __launch_bounds__(SB_THREADS) surface_band_kernel(ffs_surface_args a) {
  extern __shared__ float sbm[];
  const int W = a.band_w, T = a.T;
  float* ring = sbm;                                  // [W][SB_THREADS]
  float* cs = ring + (size_t)W * SB_THREADS;          // [SB_STEPS][W]
  const int p = blockIdx.x, bw = a.band[p];
  const int tid = threadIdx.x;
  const int v = blockIdx.y * SB_THREADS + tid;
  const bool live = v < a.V;
  const float* cb = a.band_coef + (size_t)p * T * W;
  for (int i = tid; i < W * SB_THREADS; i += blockDim.x) ring[i] = 0.f;
  float yy = 0.f, ssw = 0.f;
  int pos = 0;  // the ring slot of step t
  for (int c0 = 0; c0 < T; c0 += SB_STEPS) {
    const int cn = min(SB_STEPS, T - c0);
    __syncthreads();  // the previous chunk's coefficients are no longer read
    for (int i = tid; i < cn * W; i += blockDim.x) cs[i] = cb[(size_t)c0 * W + i];
    __syncthreads();
    for (int s = 0; s < cn; ++s) {
      const int t = c0 + s;
      const float y = live ? a.yr_t[(size_t)t * a.V + v] : 0.f;
      const float* c = cs + (size_t)s * W;
      float acc = y * c[0];
      const int jm = min(bw, t);
      int q = pos;
      for (int j = 1; j <= jm; ++j) {
        q = q == 0 ? W - 1 : q - 1;
        acc = fmaf(-c[j], ring[(size_t)q * SB_THREADS + tid], acc);
      }
      ring[(size_t)pos * SB_THREADS + tid] = acc;
      pos = pos + 1 == W ? 0 : pos + 1;
      yy = fmaf(y, y, yy);
      ssw = fmaf(acc, acc, ssw);
    }
  }
  if (!live) return;
  const int Tk = a.T - a.K;
  // grouped fits: the design of this CTA's 256-voxel tile
  const double* ldx = a.logdet_XtX + (a.tile_design ? (size_t)a.tile_design[blockIdx.y * SB_THREADS / 256] * a.P : 0);
  const double c_p0 = a.logdet_R[a.p0] + ldx[a.p0];
  const float rss0 = fmaxf(yy - a.proj[(size_t)a.p0 * a.V + v], 0.f);
  const float den = rss0 + 1e-10f;
  const float rss = fmaxf(ssw - a.proj[(size_t)p * a.V + v], 0.f);
  const float dc = (float)((a.logdet_R[p] + ldx[p]) - c_p0);
  a.surf[(size_t)p * a.V + v] = dc + (float)Tk * log1pf((rss - rss0) / den);
  if (p == 0) a.crit0[v] = c_p0 + (double)Tk * log((double)rss0 + 1e-10);
}

// ---------------------------------------------------------------------- select
__global__ void select_kernel(ffs_select_args a) {
  const int v = blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= a.V) return;
  const float* s = a.surf + v;
  const size_t V = (size_t)a.V;
  int best = a.lattice[a.za * a.n_b + a.zb];
  float bl;
  if (!a.hierarchical) {
    bl = INFINITY;
    for (int p = 0; p < a.P; ++p) {
      const float d = s[(size_t)p * V];
      if (d < bl) {
        bl = d;
        best = p;
      }
    }
  } else {
    // AFNI power-of-2 descent from (0, 0) on the (a, b) lattice
    auto at = [&](int ai, int bi) -> float {
      const int p = a.lattice[ai * a.n_b + bi];
      return p < 0 ? INFINITY : s[(size_t)p * V];
    };
    int ba = a.za, bb = a.zb;
    bl = at(ba, bb);
    for (int lev = a.ltop; lev >= 0; --lev) {
      const int step = 1 << lev;
      float mn = INFINITY;
      int sa = -1, sb = -1;
      if (lev == a.ltop) {
        for (int bi = 0; bi < a.n_b; bi += step)
          for (int ai = 0; ai < a.n_a; ai += step) {
            const float d = at(ai, bi);
            if (sa < 0 || d < mn) {
              mn = d;
              sa = ai;
              sb = bi;
            }
          }
      } else {
        for (int ob = -1; ob <= 1; ++ob) {
          const int bi = min(max(bb + ob * step, 0), a.n_b - 1);
          for (int oa = -1; oa <= 1; ++oa) {
            const int ai = min(max(ba + oa * step, 0), a.n_a - 1);
            const float d = at(ai, bi);
            if (sa < 0 || d < mn) {
              mn = d;
              sa = ai;
              sb = bi;
            }
          }
        }
      }
      if (mn < bl) {
        bl = mn;
        ba = sa;
        bb = sb;
      }
    }
    best = a.lattice[ba * a.n_b + bb];
  }
  a.best[v] = best;
  a.best_crit[v] = (float)(a.crit0[v] + (double)bl);
}

// ----------------------------------------------------------------------- group
// Counting with warp-aggregated atomics: the lanes of a warp holding the same
// key add their count once (neighbouring voxels of a smooth parameter map
// mostly share a pair, so a popular bin sees one atomic per warp, not 32).
// Keys outside [0, P) are not counted (nor placed by group_scatter).
__global__ void group_hist(int V, const int* best, int P, int* cnt) {
  const int v = blockIdx.x * blockDim.x + threadIdx.x;
  const int key = v < V ? best[v] : -1;
  const bool ok = (unsigned)key < (unsigned)P;
  const unsigned act = __ballot_sync(0xffffffffu, ok);
  if (!ok) return;
  const unsigned same = __match_any_sync(act, key);
  if ((threadIdx.x & 31) == __ffs(same) - 1) atomicAdd(cnt + key, __popc(same));
}

__global__ void group_scan(int P, int* cnt) {
  // single CTA exclusive scan of cnt[0..P) in place; cnt[P] = total
  __shared__ int carry;
  if (threadIdx.x == 0) carry = 0;
  __syncthreads();
  for (int base = 0; base < P; base += blockDim.x) {
    const int i = base + threadIdx.x;
    const int x = i < P ? cnt[i] : 0;
    // block inclusive scan by warps
    int incl = x;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    for (int o = 1; o < 32; o <<= 1) {
      const int y = __shfl_up_sync(0xffffffffu, incl, o);
      if (lane >= o) incl += y;
    }
    __shared__ int wsum[32];
    if (lane == 31) wsum[wid] = incl;
    __syncthreads();
    if (wid == 0) {
      int w = lane < (int)(blockDim.x >> 5) ? wsum[lane] : 0;
      for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, w, o);
        if (lane >= o) w += y;
      }
      wsum[lane] = w;
    }
    __syncthreads();
    const int before = (wid > 0 ? wsum[wid - 1] : 0) + carry;
    if (i < P) cnt[i] = before + incl - x;
    __syncthreads();
    if (threadIdx.x == blockDim.x - 1) carry = before + incl;
    __syncthreads();
  }
  if (threadIdx.x == 0) cnt[P] = carry;
}

// Keys up to GROUP_BLOCK_KEYS: each CTA counts a contiguous chunk of the
// voxels in shared memory (warp-aggregated), then adds each key's count to the
// global histogram once, so a popular key takes one global atomic per CTA
// instead of one per warp. Keys lie in [0, P); others are not counted.
constexpr int GROUP_BLOCK_KEYS = 6144;
constexpr int GROUP_BLOCK_THREADS = 256;

__device__ __forceinline__ void group_chunk(int V, int& v0, int& v1) {
  const int chunk = (V + gridDim.x - 1) / gridDim.x;
  v0 = min(V, (int)blockIdx.x * chunk);
  v1 = min(V, v0 + chunk);
}

// the CTA's chunk counted into h[P] (shared memory, zeroed by the caller)
__device__ __forceinline__ void group_count_chunk(int v0, int v1, const int* best, int P, int* h) {
  for (int b0 = v0; b0 < v1; b0 += blockDim.x) {  // uniform over the CTA
    const int v = b0 + threadIdx.x;
    const bool on = v < v1;
    const int key = on ? best[v] : -1;
    const bool ok = on && (unsigned)key < (unsigned)P;
    const unsigned act = __ballot_sync(0xffffffffu, ok);
    if (ok) {
      const unsigned same = __match_any_sync(act, key);
      if ((threadIdx.x & 31) == __ffs(same) - 1) atomicAdd(h + key, __popc(same));
    }
  }
}

__global__ void __launch_bounds__(GROUP_BLOCK_THREADS) group_hist_block(int V, const int* best, int P, int* cnt) {
  extern __shared__ float sm[];
  int* h = reinterpret_cast<int*>(sm);  // [P]
  for (int i = threadIdx.x; i < P; i += blockDim.x) h[i] = 0;
  __syncthreads();
  int v0, v1;
  group_chunk(V, v0, v1);
  group_count_chunk(v0, v1, best, P, h);
  __syncthreads();
  for (int i = threadIdx.x; i < P; i += blockDim.x)
    if (h[i]) atomicAdd(cnt + i, h[i]);
}

// The CTA reserves each key's slots for its chunk with one global atomic,
// then every voxel takes the next slot of its key within them (warp leaders
// claim a run of slots for the lanes of equal key).
__global__ void __launch_bounds__(GROUP_BLOCK_THREADS) group_scatter_block(int V, const int* best, int P,
                                                                           int* cursor, int* order) {
  extern __shared__ float sm[];
  int* h = reinterpret_cast<int*>(sm);  // [P] the chunk's count, then its running slot
  int* base = h + P;                    // [P] the chunk's first slot of each key
  for (int i = threadIdx.x; i < P; i += blockDim.x) h[i] = 0;
  __syncthreads();
  int v0, v1;
  group_chunk(V, v0, v1);
  group_count_chunk(v0, v1, best, P, h);
  __syncthreads();
  for (int i = threadIdx.x; i < P; i += blockDim.x) {
    const int c = h[i];
    base[i] = c ? atomicAdd(cursor + i, c) : 0;
    h[i] = 0;
  }
  __syncthreads();
  const int lane = threadIdx.x & 31;
  for (int b0 = v0; b0 < v1; b0 += blockDim.x) {
    const int v = b0 + threadIdx.x;
    const bool on = v < v1;
    const int key = on ? best[v] : -1;
    const bool ok = on && (unsigned)key < (unsigned)P;
    const unsigned act = __ballot_sync(0xffffffffu, ok);
    if (ok) {
      const unsigned same = __match_any_sync(act, key);
      const int leader = __ffs(same) - 1;
      int r = 0;
      if (lane == leader) r = atomicAdd(h + key, __popc(same));
      r = __shfl_sync(same, r, leader);
      order[base[key] + r + __popc(same & ((1u << lane) - 1u))] = v;
    }
  }
}

// The leader of each set of equal keys reserves the set's slots with one
// atomic; every lane takes the slot of its rank within the set.
__global__ void group_scatter(int V, const int* best, int P, int* cursor, int* order) {
  const int v = blockIdx.x * blockDim.x + threadIdx.x;
  const int key = v < V ? best[v] : -1;
  const bool ok = (unsigned)key < (unsigned)P;
  const unsigned act = __ballot_sync(0xffffffffu, ok);
  if (!ok) return;
  const int lane = threadIdx.x & 31;
  const unsigned same = __match_any_sync(act, key);
  const int leader = __ffs(same) - 1;
  int base = 0;
  if (lane == leader) base = atomicAdd(cursor + key, __popc(same));
  base = __shfl_sync(same, base, leader);
  order[base + __popc(same & ((1u << lane) - 1u))] = v;
}

// --------------------------------------------------------- projection (CUDA cores)
// proj[p][v] = sum_j (sum_t U[p][j][t] y_t)^2 with y time-major. CTA = 128
// voxels x one pair; U columns are staged through shared memory 16 at a time.
constexpr int PJ_COLS = 16;
constexpr int PJ_TT = 128;

__global__ void __launch_bounds__(128) project_simt_kernel(ffs_project_args a) {
  __shared__ float us[PJ_COLS][PJ_TT];
  const int p = blockIdx.y;
  const int v = blockIdx.x * 128 + threadIdx.x;
  const int T = a.T, K = a.K;
  float total = 0.f;
  for (int c0 = 0; c0 < K; c0 += PJ_COLS) {
    const int nc = min(PJ_COLS, K - c0);
    float acc[PJ_COLS];
#pragma unroll
    for (int j = 0; j < PJ_COLS; ++j) acc[j] = 0.f;
    for (int t0 = 0; t0 < T; t0 += PJ_TT) {
      const int nt = min(PJ_TT, T - t0);
      __syncthreads();
      for (int idx = threadIdx.x; idx < PJ_COLS * PJ_TT; idx += 128) {
        const int j = idx / PJ_TT, t = idx % PJ_TT;
        us[j][t] = (j < nc && t < nt) ? a.U[((size_t)p * K + c0 + j) * ld_t(T) + t0 + t] : 0.f;
      }
      __syncthreads();
      if (v < a.V) {
        const float* yc = a.yr_t + (size_t)t0 * a.V + v;
        for (int t = 0; t < nt; ++t) {
          const float y = yc[(size_t)t * a.V];
#pragma unroll
          for (int j = 0; j < PJ_COLS; ++j) acc[j] = fmaf(us[j][t], y, acc[j]);
        }
      }
    }
#pragma unroll
    for (int j = 0; j < PJ_COLS; ++j) total = fmaf(acc[j], acc[j], total);
  }
  if (v < a.V) a.proj[(size_t)p * a.V + v] = total;
}

}  // namespace

}  // namespace ffsk

using namespace ffsk;

extern "C" int ffs_reml_prep(const ffs_prep_args* a, void* stream) {
  clear_error();
  FFS_REQUIRE(a && a->V > 0 && a->T > 1 && a->K >= 0, "ffs_reml_prep: bad sizes");
  FFS_REQUIRE((a->Y || a->Y_ref) && a->scale && (a->K == 0 || a->Q0), "ffs_reml_prep: null buffer");
  FFS_REQUIRE((!a->Y_ref && !a->Y_copy) || (a->T % 4 == 0 && !a->idx && !a->tile_design && a->Y_ref),
              "ffs_reml_prep: Y_ref / Y_copy need T %% 4 == 0, no idx and no tile_design (T=%d)", a->T);
  FFS_REQUIRE(!a->feats || (a->n_runs > 0 && a->run_start), "ffs_reml_prep: features need the run layout");
  FFS_REQUIRE(!a->yr_hi || (a->yr_lo && a->yexp && a->ld_y >= a->T && a->ld_y % 8 == 0),
              "ffs_reml_prep: ld_y=%d must be >= T and a multiple of 8", a->ld_y);
  {
    const int ld = tile_ld(a->T);
    const size_t smem = sizeof(float) * ((size_t)TILE_V * ld + (size_t)a->K * TILE_V);
    FFS_REQUIRE(smem <= 200 * 1024 || !a->Y_ref, "ffs_reml_prep: Y_ref needs the tiled prep (T=%d too long)", a->T);
    if (smem <= 200 * 1024) {
      FFS_CUDA(ensure_dyn_smem(reinterpret_cast<const void*>(prep_tile_kernel), smem));
      prep_tile_kernel<<<ceil_div(a->V, TILE_V), TILE_WARPS * 32, smem, (cudaStream_t)stream>>>(*a, ld);
      return check_launch("prep_tile_kernel");
    }
  }
  const int ld_s = a->T + ((a->T & 1) ? 2 : 1);  // odd stride: conflict-free transposed reads
  const size_t smem = sizeof(float) * PREP_VOX * ld_s;
  FFS_REQUIRE(smem <= 227 * 1024, "ffs_reml_prep: T=%d too long for one tile", a->T);
  FFS_CUDA(ensure_dyn_smem(reinterpret_cast<const void*>(prep_kernel), smem));
  prep_kernel<<<ceil_div(a->V, PREP_VOX), 256, smem, (cudaStream_t)stream>>>(*a, ld_s);
  return check_launch("prep_kernel");
}

extern "C" int ffs_reml_surface(const ffs_surface_args* a, void* stream) {
  clear_error();
  if (a && a->band_coef) {
    FFS_REQUIRE(a->V > 0 && a->T > a->K && a->P > 0 && a->band_w >= 1 && a->band_w <= FFS_BAND_MAX_W,
                "ffs_reml_surface: bad sizes for the banded R");
    FFS_REQUIRE(a->p0 >= 0 && a->p0 < a->P, "ffs_reml_surface: p0=%d out of range", a->p0);
    FFS_REQUIRE(a->yr_t && a->band && a->logdet_R && a->logdet_XtX && a->proj && a->surf && a->crit0,
                "ffs_reml_surface: null buffer");
    FFS_REQUIRE(ceil_div(a->V, SB_THREADS) <= 65535, "ffs_reml_surface: V=%d exceeds one launch", a->V);
    const size_t smem = sizeof(float) * (size_t)a->band_w * (SB_THREADS + SB_STEPS);
    FFS_CUDA(ensure_dyn_smem(reinterpret_cast<const void*>(surface_band_kernel), smem));
    surface_band_kernel<<<dim3(a->P, ceil_div(a->V, SB_THREADS)), SB_THREADS, smem, (cudaStream_t)stream>>>(*a);
    return check_launch("surface_band_kernel");
  }
  FFS_REQUIRE(a && a->V > 0 && a->T > 0 && a->P > 0 && a->n_chunks > 0, "ffs_reml_surface: bad sizes");
  FFS_REQUIRE(a->p0 >= 0 && a->p0 < a->P, "ffs_reml_surface: p0=%d out of range", a->p0);
  FFS_REQUIRE(a->yr_t && a->coef && a->logdet_R && a->logdet_XtX && a->proj && a->chunk_start &&
                  a->chunk_pairs && a->surf && a->crit0,
              "ffs_reml_surface: null buffer");
  const size_t smem = (sizeof(float4) * (SURF_G2 + 1) + 1) * (size_t)a->T + sizeof(float) * SURF_G +
                      ceil_div(a->T, SURF_TB);
  FFS_REQUIRE(smem <= 227 * 1024, "ffs_reml_surface: T=%d too long", a->T);
  FFS_CUDA(ensure_dyn_smem(reinterpret_cast<const void*>(surface_kernel), smem));
  FFS_REQUIRE(ceil_div(a->V, SURF_THREADS) <= 65535, "ffs_reml_surface: V=%d exceeds one launch", a->V);
  dim3 grid(a->n_chunks, ceil_div(a->V, SURF_THREADS));
  surface_kernel<<<grid, SURF_THREADS, smem, (cudaStream_t)stream>>>(*a);
  return check_launch("surface_kernel");
}

extern "C" int ffs_reml_select(const ffs_select_args* a, void* stream) {
  clear_error();
  FFS_REQUIRE(a && a->V > 0 && a->P > 0, "ffs_reml_select: bad sizes");
  FFS_REQUIRE(a->surf && a->crit0 && a->lattice && a->best && a->best_crit, "ffs_reml_select: null buffer");
  FFS_REQUIRE(a->za >= 0 && a->za < a->n_a && a->zb >= 0 && a->zb < a->n_b,
              "ffs_reml_select: (0,0) index outside the lattice");
  select_kernel<<<ceil_div(a->V, 256), 256, 0, (cudaStream_t)stream>>>(*a);
  return check_launch("select_kernel");
}

extern "C" int ffs_reml_group(int V, int P, const int* best, int* work, int* order, void* stream) {
  clear_error();
  FFS_REQUIRE(V > 0 && P > 0 && best && work && order, "ffs_reml_group: bad arguments");
  cudaStream_t st = (cudaStream_t)stream;
  FFS_CUDA(cudaMemsetAsync(work, 0, sizeof(int) * (P + 1), st));
  if (P <= GROUP_BLOCK_KEYS) {
    // a contiguous chunk of the voxels per CTA, counted in shared memory
    const int grid = std::min(ceil_div(V, GROUP_BLOCK_THREADS), 2 * 152);
    group_hist_block<<<grid, GROUP_BLOCK_THREADS, sizeof(int) * P, st>>>(V, best, P, work);
    group_scan<<<1, 1024, 0, st>>>(P, work);
    group_scatter_block<<<grid, GROUP_BLOCK_THREADS, 2 * sizeof(int) * P, st>>>(V, best, P, work, order);
  } else {
    group_hist<<<ceil_div(V, 256), 256, 0, st>>>(V, best, P, work);
    group_scan<<<1, 1024, 0, st>>>(P, work);
    group_scatter<<<ceil_div(V, 256), 256, 0, st>>>(V, best, P, work, order);
  }
  return check_launch("group kernels");
}

extern "C" int ffs_reml_project_simt(const ffs_project_args* a, void* stream) {
  clear_error();
  FFS_REQUIRE(a && a->V > 0 && a->T > 0 && a->K > 0 && a->P > 0, "ffs_reml_project_simt: bad sizes");
  FFS_REQUIRE(a->yr_t && a->U && a->proj, "ffs_reml_project_simt: null buffer");
  dim3 grid(ceil_div(a->V, 128), a->P);
  project_simt_kernel<<<grid, 128, 0, (cudaStream_t)stream>>>(*a);
  return check_launch("project_simt_kernel");
}
