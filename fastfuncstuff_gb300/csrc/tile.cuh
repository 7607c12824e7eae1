// Tiles of 32 voxel series in shared memory, worked on by a CTA of 8 warps:
// the K x T products of the residualisation (prep) and of the GLS refit run
// as register-blocked passes over the tile (projections) and as warp-level
// tensor-core MMAs (updates, tile_subtract_any) instead of one warp reduction
// per design column.
//
// Layout: Ys[l][t] (l < 32 voxels, row stride tile_ld(T)), zero for t >= T;
// K x T matrices stay in global memory (row stride lm = ld_t(T), a multiple
// of 4, zero padded) and are read through the L1 cache, which every CTA
// working on the same matrix shares. The passes run over nq = lm / 4 quads of
// samples; the zero padding adds nothing to the products.
//
// Cost model. The L1 / shared-memory data path delivers 128 bytes per cycle
// to the registers of a warp, whether the 32 lanes read one address or 32;
// a 16-byte load of the whole warp is 4 such cycles even when every lane
// reads the same float4. A product whose operands are both loaded for every
// FMA is therefore bound by that path, not by the FMA pipe. Each thread here
// keeps a block of operands in registers instead: in the projection 8 voxels
// x up to 5 columns (every loaded matrix entry serves 8 voxels, every loaded
// sample up to 5 columns), in the update 4 voxels x up to 10 columns.
#pragma once
#include "common.cuh"

namespace ffsk {

constexpr int TILE_V = 32;       // voxels per tile
constexpr int TILE_WARPS = 8;    // warps per CTA
constexpr int TILE_SLICES = 16;  // time slices of tile_project (lane bits 0..3)
constexpr int TILE_VB = 8;       // voxels per thread in tile_project
constexpr int TILE_KB_MAX = 5;   // columns per thread and pass in tile_project
constexpr int TILE_SUB_VB = 4;   // voxels per warp in tile_subtract (warp w: 4w .. 4w+3)
constexpr int TILE_SUB_KC = 10;  // columns per pass in tile_subtract

// Row stride (floats) of a tile: a multiple of 4 with ld / 4 odd, so 128-bit
// loads of 8 lanes from 8 different rows fall in distinct banks.
__host__ __device__ inline int tile_ld(int T) {
  int ld = (T + 3) & ~3;
  if (((ld >> 2) & 1) == 0) ld += 4;
  return ld;
}

// Copies the series rows[l] of Y ([V][T], l < 32; rows[l] < 0: a zero row)
// into Ys[l][0 .. 4 nq) with asynchronous copies, all in flight at once (16
// bytes each when T % 4 == 0, single samples otherwise; samples T .. 4 nq are
// zero), then waits for them and ends with a barrier. rows is in shared
// memory.
__device__ __forceinline__ void tile_stage_rows(const float* __restrict__ Y, int T, int nq, const int* rows,
                                                float* Ys, int ld) {
  if ((T & 3) == 0) {
    for (int idx = threadIdx.x; idx < TILE_V * nq; idx += blockDim.x) {
      const int l = idx / nq, q = idx % nq;
      const int v = rows[l];
      const float* src = v >= 0 ? Y + (size_t)v * T + 4 * q : Y;
      const uint32_t dst = static_cast<uint32_t>(__cvta_generic_to_shared(Ys + (size_t)l * ld + 4 * q));
      asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;" ::"r"(dst), "l"(src), "r"(v >= 0 ? 16 : 0)
                   : "memory");
    }
  } else {
    const int n4 = 4 * nq;
    for (int idx = threadIdx.x; idx < TILE_V * n4; idx += blockDim.x) {
      const int l = idx / n4, t = idx % n4;
      const int v = rows[l];
      const bool in = v >= 0 && t < T;
      const float* src = in ? Y + (size_t)v * T + t : Y;
      const uint32_t dst = static_cast<uint32_t>(__cvta_generic_to_shared(Ys + (size_t)l * ld + t));
      asm volatile("cp.async.ca.shared.global [%0], [%1], 4, %2;" ::"r"(dst), "l"(src), "r"(in ? 4 : 0)
                   : "memory");
    }
  }
  asm volatile("cp.async.commit_group;" ::: "memory");
  asm volatile("cp.async.wait_group 0;" ::: "memory");
  __syncthreads();
}

// C[j][l] = sum_t M[j][t] Ys[l][t] for j < K, l < 32 with KB columns per
// thread and pass. Thread layout: s = lane & 15 is the time slice (quads
// q = s, s + 16, ...), unit u = 2 * warp + (lane >> 4) is voxel group
// u & 3 (voxels 8 (u & 3) + i, i < 8) and column group u >> 2 (columns
// j0 + KB (u >> 2) + k, k < KB, of the pass starting at j0). The 16 slice
// partials are summed by recursive halving across lane bits 3, 2, 1 (each
// exchange ships half of the remaining values) and a final exchange across
// bit 0; lanes s and s ^ 1 then hold the KB sums of voxel s >> 1.
template <int KB>
__device__ __forceinline__ void tile_project_kb(const float* __restrict__ M, int lm, const float* Ys, int ld, int K,
                                                float* C) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int s = lane & 15;
  const int u = 2 * w + (lane >> 4);
  const int vg = u & 3, cg = u >> 2;  // cg is warp-uniform
  const int nq = lm >> 2, ld4 = ld >> 2;
  const float4* y4 = reinterpret_cast<const float4*>(Ys) + (size_t)(vg * TILE_VB) * ld4;
  for (int j0 = 0; j0 < K; j0 += 4 * KB) {
    const int jb = j0 + cg * KB;
    float acc[TILE_VB * KB];
#pragma unroll
    for (int i = 0; i < TILE_VB * KB; ++i) acc[i] = 0.f;
    const float4* mb = reinterpret_cast<const float4*>(M + (size_t)min(jb, K - 1) * lm);  // row jb, stride nq
    for (int q = s; q < nq; q += TILE_SLICES) {
      float4 m[KB];
#pragma unroll
      for (int k = 0; k < KB; ++k)
        m[k] = (jb + k < K) ? __ldg(mb + (size_t)k * nq + q) : make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
      for (int i = 0; i < TILE_VB; ++i) {
        const float4 y = y4[(size_t)i * ld4 + q];
#pragma unroll
        for (int k = 0; k < KB; ++k) {
          float a = acc[i * KB + k];
          a = fmaf(m[k].x, y.x, a);
          a = fmaf(m[k].y, y.y, a);
          a = fmaf(m[k].z, y.z, a);
          a = fmaf(m[k].w, y.w, a);
          acc[i * KB + k] = a;
        }
      }
    }
    // recursive halving over lane bits 3, 2, 1: the lane whose bit is set
    // keeps the upper half of its values, its partner the lower half
#pragma unroll
    for (int b = 8, n = TILE_VB * KB; b >= 2; b >>= 1, n >>= 1) {
      const bool up = (lane & b) != 0;
#pragma unroll
      for (int i = 0; i < n / 2; ++i) {
        const float send = up ? acc[i] : acc[i + n / 2];
        const float keep = up ? acc[i + n / 2] : acc[i];
        acc[i] = keep + __shfl_xor_sync(0xffffffffu, send, b);
      }
    }
#pragma unroll
    for (int k = 0; k < KB; ++k) acc[k] += __shfl_xor_sync(0xffffffffu, acc[k], 1);
    if ((lane & 1) == 0) {
      const int l = vg * TILE_VB + (s >> 1);
#pragma unroll
      for (int k = 0; k < KB; ++k)
        if (jb + k < K) C[(size_t)(jb + k) * TILE_V + l] = acc[k];
    }
  }
}

// C[j][l] = sum_t M[j][t] Ys[l][t] for j < K, l < 32 (C is [K][32]; M has
// row stride lm). Ends with a barrier.
__device__ __forceinline__ void tile_project(const float* __restrict__ M, int lm, const float* Ys, int ld, int K,
                                             float* C) {
  const int passes = (K + 4 * TILE_KB_MAX - 1) / (4 * TILE_KB_MAX);
  const int kb = (K + 4 * passes - 1) / (4 * passes);  // columns per thread and pass, <= TILE_KB_MAX
  switch (kb) {
    case 1: tile_project_kb<1>(M, lm, Ys, ld, K, C); break;
    case 2: tile_project_kb<2>(M, lm, Ys, ld, K, C); break;
    case 3: tile_project_kb<3>(M, lm, Ys, ld, K, C); break;
    case 4: tile_project_kb<4>(M, lm, Ys, ld, K, C); break;
    default: tile_project_kb<5>(M, lm, Ys, ld, K, C); break;
  }
  __syncthreads();
}

// Ys[l][t] -= sum_j N[j][t] C[j][l] (N has row stride lm). Warp w updates the rows 4w .. 4w+3
// (lanes over quads), so a thread's later reads of those rows need no
// barrier; rows of other warps do. No barrier.
__device__ __forceinline__ void tile_subtract(const float* __restrict__ N, int lm, const float* C, float* Ys, int ld,
                                              int K) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int nq = lm >> 2, ld4 = ld >> 2;
  float4* r4 = reinterpret_cast<float4*>(Ys) + (size_t)(TILE_SUB_VB * w) * ld4;
  for (int j0 = 0; j0 < K; j0 += TILE_SUB_KC) {
    float c[TILE_SUB_VB][TILE_SUB_KC];
#pragma unroll
    for (int k = 0; k < TILE_SUB_KC; ++k) {
#pragma unroll
      for (int i = 0; i < TILE_SUB_VB; ++i)
        c[i][k] = (j0 + k < K) ? C[(size_t)(j0 + k) * TILE_V + TILE_SUB_VB * w + i] : 0.f;
    }
    for (int q = lane; q < nq; q += 32) {
      float4 r[TILE_SUB_VB];
#pragma unroll
      for (int i = 0; i < TILE_SUB_VB; ++i) r[i] = r4[(size_t)i * ld4 + q];
#pragma unroll
      for (int k = 0; k < TILE_SUB_KC; ++k) {
        if (j0 + k < K) {
          const float4 n = __ldg(reinterpret_cast<const float4*>(N + (size_t)(j0 + k) * lm) + q);
#pragma unroll
          for (int i = 0; i < TILE_SUB_VB; ++i) {
            r[i].x = fmaf(-n.x, c[i][k], r[i].x);
            r[i].y = fmaf(-n.y, c[i][k], r[i].y);
            r[i].z = fmaf(-n.z, c[i][k], r[i].z);
            r[i].w = fmaf(-n.w, c[i][k], r[i].w);
          }
        }
      }
#pragma unroll
      for (int i = 0; i < TILE_SUB_VB; ++i) r4[(size_t)i * ld4 + q] = r[i];
    }
  }
}

// ------------------------------------------------------------ tensor-core forms
// The update on the tensor cores, as warp-level tf32 MMAs (m16n8k8, fp32
// accumulation) of hi/lo splits: x = hi + lo with hi = tf32(x) and
// lo = tf32(x - hi) (about 22 significant bits, fp32's exponent range, so no
// per-row scaling), each product formed as hi*hi + (lo*hi + hi*lo) (the lo*lo
// term is below fp32 rounding). A tile of 32 voxels is two 16-row MMA tiles;
// time is the MMA's n. The update wins here because every output element is
// written once with its series value as the accumulator; the projection onto
// K columns reduces over time instead, and stays on the CUDA cores
// (tile_project), whose wide loads hide the latency of the matrix reads. Fragment layouts of mma.m16n8k8 with .tf32 operands, lane = 4 g + q:
// A (16 x 8, row-major): a0 (g, q), a1 (g + 8, q), a2 (g, q + 4), a3 (g + 8, q + 4);
// B (8 x 8, column-major): b0 (q, g), b1 (q + 4, g);
// C/D (16 x 8, fp32): c0 (g, 2q), c1 (g, 2q + 1), c2 (g + 8, 2q), c3 (g + 8, 2q + 1).

__device__ __forceinline__ void split_tf32(float x, uint32_t& hi, uint32_t& lo) {
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(hi) : "f"(x));
  const float r = __fsub_rn(x, __uint_as_float(hi));
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(lo) : "f"(r));
}

__device__ __forceinline__ void mma_tf32(float (&d)[4], uint32_t a0, uint32_t a1, uint32_t a2, uint32_t a3,
                                         uint32_t b0, uint32_t b1) {
  asm("mma.sync.aligned.m16n8k8.row.col.f32.tf32.tf32.f32 {%0, %1, %2, %3}, {%4, %5, %6, %7}, {%8, %9}, "
      "{%0, %1, %2, %3};"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a0), "r"(a1), "r"(a2), "r"(a3), "r"(b0), "r"(b1));
}

// d += a_hi b_hi and e += a_lo b_hi + a_hi b_lo (a and b as hi/lo splits):
// two accumulators, so the three products form two short dependency chains
__device__ __forceinline__ void mma_tf32x3(float (&d)[4], float (&e)[4], const uint32_t (&ah)[4],
                                           const uint32_t (&al)[4], const uint32_t (&bh)[2], const uint32_t (&bl)[2]) {
  mma_tf32(e, al[0], al[1], al[2], al[3], bh[0], bh[1]);
  mma_tf32(d, ah[0], ah[1], ah[2], ah[3], bh[0], bh[1]);
  mma_tf32(e, ah[0], ah[1], ah[2], ah[3], bl[0], bl[1]);
}

// Ys[l][t] -= sum_j N[j][t] C[j][l] (N has row stride lm, C is [K][32]) on
// the tensor cores, for K <= 8 * KS: warp w updates the 16 rows of m tile
// (w & 1) at the n tiles of 8 samples i = (w >> 1) + 4u, t < lm, each output
// element once (the series value enters as the accumulator of the hi*hi
// products, the cross terms are summed apart and added last). Starts
// with a barrier (other warps may still read the rows); no barrier at the end.
template <int KS>
__device__ __forceinline__ void tile_subtract_tc(const float* __restrict__ N, int lm, const float* C, float* Ys,
                                                 int ld, int K) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int g = lane >> 2, q = lane & 3;
  const int mt = w & 1, np = w >> 1;
  const int r0 = 16 * mt + g, r1 = r0 + 8;
  // A = -C' (rows: voxels, k: design columns), split once
  uint32_t ah[KS][4], al[KS][4];
#pragma unroll
  for (int k = 0; k < KS; ++k) {
    const int ja = 8 * k + q, jb = ja + 4;
    split_tf32(ja < K ? -C[(size_t)ja * TILE_V + r0] : 0.f, ah[k][0], al[k][0]);
    split_tf32(ja < K ? -C[(size_t)ja * TILE_V + r1] : 0.f, ah[k][1], al[k][1]);
    split_tf32(jb < K ? -C[(size_t)jb * TILE_V + r0] : 0.f, ah[k][2], al[k][2]);
    split_tf32(jb < K ? -C[(size_t)jb * TILE_V + r1] : 0.f, ah[k][3], al[k][3]);
  }
  __syncthreads();
  float* y0 = Ys + (size_t)r0 * ld;
  float* y1 = Ys + (size_t)r1 * ld;
  const int S = (lm + 7) >> 3;
  for (int i0 = np; i0 < S; i0 += 8) {  // n tiles i0 and i0 + 4
    float d[2][4], e[2][4];
#pragma unroll
    for (int u = 0; u < 2; ++u) {
      const int t = 8 * (i0 + 4 * u) + 2 * q;  // this lane's two columns of the n tile
      d[u][0] = d[u][1] = d[u][2] = d[u][3] = 0.f;
      e[u][0] = e[u][1] = e[u][2] = e[u][3] = 0.f;
      if (t < lm) {  // lm % 4 == 0: t and t + 1 both in or both out
        const float2 a = *reinterpret_cast<const float2*>(y0 + t);
        const float2 b = *reinterpret_cast<const float2*>(y1 + t);
        d[u][0] = a.x;
        d[u][1] = a.y;
        d[u][2] = b.x;
        d[u][3] = b.y;
      }
    }
#pragma unroll
    for (int k = 0; k < KS; ++k) {
      const int ja = 8 * k + q, jb = ja + 4;
#pragma unroll
      for (int u = 0; u < 2; ++u) {
        const int tb = 8 * (i0 + 4 * u) + g;  // the B column this lane feeds
        uint32_t bh[2], bl[2];
        split_tf32((ja < K && tb < lm) ? __ldg(N + (size_t)ja * lm + tb) : 0.f, bh[0], bl[0]);
        split_tf32((jb < K && tb < lm) ? __ldg(N + (size_t)jb * lm + tb) : 0.f, bh[1], bl[1]);
        mma_tf32x3(d[u], e[u], ah[k], al[k], bh, bl);
      }
    }
#pragma unroll
    for (int u = 0; u < 2; ++u) {
      const int t = 8 * (i0 + 4 * u) + 2 * q;
      if (t < lm) {
        *reinterpret_cast<float2*>(y0 + t) = make_float2(d[u][0] + e[u][0], d[u][1] + e[u][1]);
        *reinterpret_cast<float2*>(y1 + t) = make_float2(d[u][2] + e[u][2], d[u][3] + e[u][3]);
      }
    }
  }
}

// Ys -= (N C)' with the tensor cores for K <= 32 and the register-blocked
// CUDA-core pass otherwise. Starts with a barrier and ends with one.
__device__ __forceinline__ void tile_subtract_any(const float* __restrict__ N, int lm, const float* C, float* Ys,
                                                  int ld, int K) {
  switch ((K + 7) >> 3) {
    case 1: tile_subtract_tc<1>(N, lm, C, Ys, ld, K); break;
    case 2: tile_subtract_tc<2>(N, lm, C, Ys, ld, K); break;
    case 3: tile_subtract_tc<3>(N, lm, C, Ys, ld, K); break;
    case 4: tile_subtract_tc<4>(N, lm, C, Ys, ld, K); break;
    default:
      __syncthreads();
      tile_subtract(N, lm, C, Ys, ld, K);
      break;
  }
  __syncthreads();
}

}  // namespace ffsk
