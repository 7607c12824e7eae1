// Tiles of 32 voxel series in shared memory, worked on by a CTA of 8 warps:
// the K x T products of the residualisation (prep) and of the GLS refit run
// as register-blocked passes over the tile instead of one warp reduction per
// design column.
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

}  // namespace ffsk
