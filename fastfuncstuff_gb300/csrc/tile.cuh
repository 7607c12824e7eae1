// Tiles of 32 voxel series in shared memory, one voxel per lane, worked on by
// a CTA of 8 warps: the K x T products of the residualisation (prep) and of
// the GLS refit run as register-blocked passes over the tile instead of one
// warp reduction per design column.
//
// Layout: Ys[l][t] (l < 32 voxels, t < T, row stride tile_ld(T)); K x T
// matrices stay in global memory ([K][T], rows 16-byte aligned, T % 4 == 0)
// and are read as warp-uniform float4 loads that the L1 cache serves to every
// warp of the CTA.
#pragma once
#include "common.cuh"

namespace ffsk {

constexpr int TILE_V = 32;      // voxels per tile (one per lane)
constexpr int TILE_WARPS = 8;   // warps per CTA
constexpr int TILE_PROJ_KC = 12; // columns a thread accumulates per pass in tile_project
constexpr int TILE_JG = 2;       // column groups of tile_project (warps = TILE_JG x TILE_TS)
constexpr int TILE_TS = TILE_WARPS / TILE_JG;  // time splits of tile_project
constexpr int TILE_SUB_KC = 16; // coefficients a thread holds per pass in tile_subtract

// Row stride (floats) of a tile: a multiple of 4 with ld / 4 odd, so the
// 128-bit loads of 8 consecutive lanes from 8 rows fall in distinct banks.
__host__ __device__ inline int tile_ld(int T) {
  int ld = (T + 3) & ~3;
  if (((ld >> 2) & 1) == 0) ld += 4;
  return ld;
}

// Quads [q0, q1) of every row owned by warp w in the row-update passes; the
// same thread always owns the same samples, so consecutive passes over them
// need no barrier.
__device__ __forceinline__ void tile_qrange(int T, int w, int& q0, int& q1) {
  const int nq = T >> 2;
  q0 = w * nq / TILE_WARPS;
  q1 = (w + 1) * nq / TILE_WARPS;
}

// C[j][l] = sum_t M[j][t] Ys[l][t] for j < K, l < 32; part is [TILE_TS][K][32]
// scratch. Warp w takes the columns j = (w % TILE_JG) + TILE_JG u and one of
// TILE_TS slices of the time range (w / TILE_JG); the slices are added in
// order at the end. Ends with a barrier.
__device__ __forceinline__ void tile_project(const float* __restrict__ M, const float* Ys, int T, int ld, int K,
                                             float* C, float* part) {
  const int l = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int jg = w % TILE_JG, ts = w / TILE_JG;
  const int nq = T >> 2;
  const int q0 = ts * nq / TILE_TS, q1 = (ts + 1) * nq / TILE_TS;
  const float4* yr = reinterpret_cast<const float4*>(Ys + (size_t)l * ld);
  for (int u0 = jg; u0 < K; u0 += TILE_JG * TILE_PROJ_KC) {
    float acc[TILE_PROJ_KC];
#pragma unroll
    for (int k = 0; k < TILE_PROJ_KC; ++k) acc[k] = 0.f;
    for (int q = q0; q < q1; ++q) {
      const float4 y = yr[q];
#pragma unroll
      for (int k = 0; k < TILE_PROJ_KC; ++k) {
        const int j = u0 + TILE_JG * k;
        if (j < K) {
          const float4 m = __ldg(reinterpret_cast<const float4*>(M + (size_t)j * T) + q);
          acc[k] = fmaf(m.x, y.x, acc[k]);
          acc[k] = fmaf(m.y, y.y, acc[k]);
          acc[k] = fmaf(m.z, y.z, acc[k]);
          acc[k] = fmaf(m.w, y.w, acc[k]);
        }
      }
    }
#pragma unroll
    for (int k = 0; k < TILE_PROJ_KC; ++k) {
      const int j = u0 + TILE_JG * k;
      if (j < K) part[((size_t)ts * K + j) * 32 + l] = acc[k];
    }
  }
  __syncthreads();
  for (int i = threadIdx.x; i < K * 32; i += blockDim.x) {
    float c = part[i];
#pragma unroll
    for (int k = 1; k < TILE_TS; ++k) c += part[(size_t)k * K * 32 + i];
    C[i] = c;
  }
  __syncthreads();
}

// Ys[l][t] -= sum_j N[j][t] C[j][l] over the quads this thread owns
// (tile_qrange). No barrier.
__device__ __forceinline__ void tile_subtract(const float* __restrict__ N, const float* C, float* Ys, int T, int ld,
                                              int K) {
  const int l = threadIdx.x & 31, w = threadIdx.x >> 5;
  int q0, q1;
  tile_qrange(T, w, q0, q1);
  float4* rr = reinterpret_cast<float4*>(Ys + (size_t)l * ld);
  for (int j0 = 0; j0 < K; j0 += TILE_SUB_KC) {
    float c[TILE_SUB_KC];
#pragma unroll
    for (int k = 0; k < TILE_SUB_KC; ++k) c[k] = (j0 + k < K) ? C[(size_t)(j0 + k) * 32 + l] : 0.f;
    for (int q = q0; q < q1; ++q) {
      float4 r = rr[q];
#pragma unroll
      for (int k = 0; k < TILE_SUB_KC; ++k) {
        if (j0 + k < K) {
          const float4 n = __ldg(reinterpret_cast<const float4*>(N + (size_t)(j0 + k) * T) + q);
          r.x = fmaf(-n.x, c[k], r.x);
          r.y = fmaf(-n.y, c[k], r.y);
          r.z = fmaf(-n.z, c[k], r.z);
          r.w = fmaf(-n.w, c[k], r.w);
        }
      }
      rr[q] = r;
    }
  }
}

}  // namespace ffsk
