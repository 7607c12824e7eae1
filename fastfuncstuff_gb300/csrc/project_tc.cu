// Projection GEMM on the 5th-generation tensor cores.
//
//   proj[p][v] = sum_{j<K} ( sum_t Y_r[v][t] U[p*K + j][t] )^2
//
// is the ||Q'Y_w||^2 term of the REML criterion (fastfuncstuff/glm/arma.py:
// 1992-1995) for every voxel and every pair at once, since Q'L^-1 y = U'y with
// U = L^-T Q. Operands are fp16 hi/lo splits of Y_r (voxel-major) and U, each
// scaled by a power of two that puts its largest entry in [128, 256), so the
// contraction runs as three tcgen05.mma products per k-step (hi*hi, hi*lo,
// lo*hi) accumulating in fp32 in tensor memory, with a relative error near
// 2^-22 per product; the epilogue removes the scales exactly.
//
// Work item: 128 voxels x N columns (g whole pairs, N = roundup16(g*K) <= 256).
// Warp 0 issues TMA loads (128B-swizzled boxes of 64 k-elements), warp 1 owns
// TMEM and issues the MMAs from one thread, warps 2-5 square and sum each
// pair's K columns straight out of TMEM and store proj. Nothing but proj
// returns to global memory. All mbarrier waits are bounded: on expiry a flag is
// raised and the CTA winds down instead of spinning.
#include <cuda.h>
#include <cudaTypedefs.h>

#include <mutex>

#include "common.cuh"

namespace ffsk {
namespace {

constexpr int BM = 128;         // voxels per tile (TMEM lanes)
constexpr int BK = 64;          // k elements per stage (one 128-byte swizzle row)
constexpr int STAGES = 2;
constexpr int A_TILE = BM * BK * 2;  // bytes of one A box (hi or lo, fp16)
constexpr uint32_t WAIT_LIMIT = 1u << 22;

struct TcParams {
  int V, K, P, ld, T;  // ld: padded k extent (multiple of BK); T: real extent
  int g, N;            // grid mode: pairs per column tile, MMA N
  int NB;              // rows of every B box (>= the N of any item)
  int n_col_tiles, n_vox_tiles;
  const ffs_tc_item* items;  // work-list mode: items[0 .. *n_items)
  const int* n_items;
  int s_vox;           // work-list mode: proj[(out0 + r) * s_vox + slot0 + j], or with
                       // s_vox == 0 pair-major proj[(slot0 + j) * V + out0 + r]
  const int* yexp;
  const int* uexp;
  float* proj;
  int* flag;
  const int* v_dev;    // grid mode: device count of the operand rows to project (or NULL: V)
};

// One work item: BM operand rows from v0 (nv of them real) against the np
// pairs whose U rows start at row_b.
struct Item {
  int v0, nv, row_b, np, out0, slot0, N;
};

template <bool LIST>
__device__ __forceinline__ Item item_at(const TcParams& prm, int item, int Vd) {
  Item it;
  if (LIST) {
    const ffs_tc_item w = prm.items[item];
    it.v0 = w.v0;
    it.nv = w.nv;
    it.row_b = w.row_b;
    it.np = w.np;
    it.out0 = w.out0;
    it.slot0 = w.slot0;
    it.N = (w.np * prm.K + 15) / 16 * 16;
  } else {
    const int col = item % prm.n_col_tiles;
    it.v0 = (item / prm.n_col_tiles) * BM;
    it.nv = min(BM, Vd - it.v0);
    it.row_b = col * prm.g * prm.K;
    it.np = min(prm.g, prm.P - col * prm.g);
    it.out0 = it.v0;
    it.slot0 = col * prm.g;
    it.N = prm.N;
  }
  return it;
}

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count));
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
               : "memory");
}

// Bounded parity wait; returns false if the limit expired.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity) {
  const uint32_t addr = smem_u32(bar);
  for (uint32_t i = 0; i < WAIT_LIMIT; ++i) {
    uint32_t ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(ok)
        : "r"(addr), "r"(parity)
        : "memory");
    if (ok) return true;
  }
  return false;
}

__device__ __forceinline__ void tma_load_2d(void* dst, const CUtensorMap* map, uint64_t* bar, int c0, int c1) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%3, %4}], [%2];"
      ::"r"(smem_u32(dst)), "l"(reinterpret_cast<uint64_t>(map)), "r"(smem_u32(bar)), "r"(c0), "r"(c1)
      : "memory");
}

// UMMA shared-memory descriptor: K-major, 128-byte swizzle, 8-row atoms of
// 1024 bytes (stride byte offset 1024), descriptor version 1.
__device__ __forceinline__ uint64_t sdesc(uint32_t saddr) {
  uint64_t d = 0;
  d |= (uint64_t)((saddr & 0x3FFFFu) >> 4);
  d |= (uint64_t)1 << 16;              // leading byte offset (unused for swizzled K-major)
  d |= (uint64_t)(1024 >> 4) << 32;    // stride byte offset
  d |= (uint64_t)1 << 46;              // version
  d |= (uint64_t)2 << 61;              // SWIZZLE_128B
  return d;
}

// kind::f16 instruction descriptor: fp32 accumulator (bits 4-5 = 1), fp16 A
// and B (format fields 0), both K-major, N >> 3 at bit 17, M >> 4 at bit 24.
__host__ __device__ constexpr uint32_t idesc_f16(int M, int N) {
  return (1u << 4) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

__device__ __forceinline__ void mma_f16(uint32_t tmem_d, uint64_t a, uint64_t b, uint32_t idesc, uint32_t acc) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem_d),
      "l"(a), "l"(b), "r"(idesc), "r"(acc));
}

__device__ __forceinline__ void mma_commit(uint64_t* bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
               : "memory");
}

// Persistent kernel: CTA b walks work items b, b + gridDim.x, ... where item
// = vox_tile * n_col_tiles + col_tile (column tiles fastest, so the CTAs that
// run together share voxel tiles in L2). The TMA ring of STAGES k-blocks runs
// across items; TMEM holds two 256-column accumulators so the epilogue warps
// drain item i while the MMA warp accumulates item i + 1.
template <bool LIST>
__global__ void __launch_bounds__(192, 1)
    project_tc_kernel(const __grid_constant__ CUtensorMap ta_hi, const __grid_constant__ CUtensorMap ta_lo,
                      const __grid_constant__ CUtensorMap tb_hi, const __grid_constant__ CUtensorMap tb_lo,
                      TcParams prm) {
  extern __shared__ uint8_t smem_raw[];
  uint8_t* smem = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  const int b_tile = prm.NB * BK * 2;
  const int stage_bytes = 2 * A_TILE + 2 * b_tile;
  uint64_t* full = reinterpret_cast<uint64_t*>(smem + STAGES * stage_bytes);
  uint64_t* empty = full + STAGES;
  uint64_t* acc_full = empty + STAGES;    // [2] MMA -> epilogue
  uint64_t* acc_empty = acc_full + 2;     // [2] epilogue -> MMA
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(acc_empty + 2);

  // a CTA that finds an earlier CTA's wait expired does nothing
  if (*reinterpret_cast<volatile int*>(prm.flag) != 0) return;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  // grid mode: the rows to project (a device count when given)
  const int Vd = (!LIST && prm.v_dev) ? min(prm.V, max(0, *prm.v_dev)) : prm.V;
  const int n_items = LIST ? *prm.n_items : prm.n_col_tiles * ((Vd + BM - 1) / BM);
  const int nk = prm.ld / BK;

  if (threadIdx.x == 0) {
    for (int s = 0; s < STAGES; ++s) {
      mbar_init(full + s, 1);
      mbar_init(empty + s, 1);
    }
    for (int b = 0; b < 2; ++b) {
      mbar_init(acc_full + b, 1);
      mbar_init(acc_empty + b, 128);
    }
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  }
  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], 512;" ::"r"(smem_u32(tmem_slot)));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = *tmem_slot;

  if (warp == 0 && lane == 0) {
    // ---- TMA producer: k-blocks of every item of this CTA through the ring
    int kc = 0;
    bool ok = true;
    for (int item = blockIdx.x; item < n_items && ok; item += gridDim.x) {
      const Item it = item_at<LIST>(prm, item, Vd);
      const int v0 = it.v0, row_b = it.row_b;
      for (int kb = 0; kb < nk; ++kb, ++kc) {
        const int s = kc % STAGES;
        if (kc >= STAGES && !mbar_wait(empty + s, ((kc / STAGES) - 1) & 1)) {
          atomicExch(prm.flag, 1);
          ok = false;
          break;
        }
        uint8_t* st = smem + s * stage_bytes;
        mbar_expect_tx(full + s, (uint32_t)stage_bytes);
        const int k0 = kb * BK;
        tma_load_2d(st, &ta_hi, full + s, k0, v0);
        tma_load_2d(st + A_TILE, &ta_lo, full + s, k0, v0);
        tma_load_2d(st + 2 * A_TILE, &tb_hi, full + s, k0, row_b);
        tma_load_2d(st + 2 * A_TILE + b_tile, &tb_lo, full + s, k0, row_b);
      }
    }
  } else if (warp == 1 && lane == 0) {
    // ---- MMA issuer
    int kc = 0, local = 0;
    bool ok = true;
    for (int item = blockIdx.x; item < n_items && ok; item += gridDim.x, ++local) {
      const uint32_t idesc = idesc_f16(BM, item_at<LIST>(prm, item, Vd).N);
      const int buf = local & 1;
      const uint32_t acc = tmem + (uint32_t)(buf * 256);
      if (local >= 2 && !mbar_wait(acc_empty + buf, ((local >> 1) - 1) & 1)) {
        atomicExch(prm.flag, 4);
        ok = false;
        break;
      }
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      for (int kb = 0; kb < nk; ++kb, ++kc) {
        const int s = kc % STAGES;
        if (!mbar_wait(full + s, (kc / STAGES) & 1)) {
          atomicExch(prm.flag, 2);
          ok = false;
          break;
        }
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        uint8_t* st = smem + s * stage_bytes;
        const uint64_t a_hi = sdesc(smem_u32(st));
        const uint64_t a_lo = sdesc(smem_u32(st + A_TILE));
        const uint64_t b_hi = sdesc(smem_u32(st + 2 * A_TILE));
        const uint64_t b_lo = sdesc(smem_u32(st + 2 * A_TILE + b_tile));
        // k-steps past T multiply zero padding: skip them
        const int nkk = min(BK / 16, (prm.T - kb * BK + 15) / 16);
        for (int kk = 0; kk < nkk; ++kk) {
          const uint64_t off = (uint64_t)((kk * 32) >> 4);  // 16 fp16 = 32 bytes along k
          const uint32_t acc0 = (kb > 0 || kk > 0) ? 1u : 0u;
          mma_f16(acc, a_hi + off, b_hi + off, idesc, acc0);
          mma_f16(acc, a_hi + off, b_lo + off, idesc, 1u);
          mma_f16(acc, a_lo + off, b_hi + off, idesc, 1u);
        }
        mma_commit(empty + s);
      }
      mma_commit(acc_full + buf);
    }
  } else if (warp >= 2) {
    // ---- epilogue: square and sum each pair's K columns from TMEM
    const int q = warp & 3;  // TMEM lane quarter this warp may access
    const int row = q * 32 + lane;
    int local = 0;
    for (int item = blockIdx.x; item < n_items; item += gridDim.x, ++local) {
      const int buf = local & 1;
      const bool ok = __all_sync(0xffffffffu, mbar_wait(acc_full + buf, (local >> 1) & 1));
      if (!ok) {
        if (lane == 0) atomicExch(prm.flag, 3);
        break;
      }
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      // grid mode keeps the exact form whose timing was measured best; the
      // work-list mode differs in where the result goes
      int v, p_first, ncols, nmax, out_row, out_slot = 0;
      if (LIST) {
        const Item it = item_at<LIST>(prm, item, Vd);
        v = row < it.nv ? it.v0 + row : prm.V;
        p_first = it.row_b / prm.K;
        ncols = it.np * prm.K;
        nmax = it.N;
        out_row = prm.s_vox > 0 ? (it.out0 + row) * prm.s_vox + it.slot0 : it.out0 + row;
        out_slot = it.slot0;
      } else {
        v = (item / prm.n_col_tiles) * BM + row;
        if (v >= Vd) v = prm.V;  // rows past the device count are not written
        p_first = (item % prm.n_col_tiles) * prm.g;
        ncols = prm.g * prm.K;
        nmax = prm.N;
        out_row = 0;
      }
      const int ey = v < prm.V ? prm.yexp[v] : 0;
      int j = 0, pl = 0;
      float run = 0.f;
      for (int c0 = 0; c0 < nmax; c0 += 16) {
        uint32_t r[16];
        const uint32_t taddr = tmem + (uint32_t)(buf * 256) + ((uint32_t)(q * 32) << 16) + (uint32_t)c0;
        asm volatile(
            "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
            : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
              "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]),
              "=r"(r[15])
            : "r"(taddr));
        asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
        for (int i = 0; i < 16; ++i) {
          if (c0 + i < ncols) {
            const float x = __uint_as_float(r[i]);
            run = fmaf(x, x, run);
            if (++j == prm.K) {
              const int p = p_first + pl;
              if (p < prm.P && v < prm.V) {
                const float val = ldexpf(run, -2 * (ey + prm.uexp[p]));
                if (LIST && prm.s_vox > 0)
                  prm.proj[(size_t)out_row + pl] = val;
                else if (LIST)
                  prm.proj[(size_t)(out_slot + pl) * prm.V + out_row] = val;
                else
                  prm.proj[(size_t)p * prm.V + v] = val;
              }
              run = 0.f;
              j = 0;
              ++pl;
            }
          }
        }
      }
      // this accumulator may be overwritten now
      asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
      asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(acc_empty + buf)) : "memory");
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 1) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, 512;" ::"r"(tmem));
  }
}

PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  if (!fn) {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
            cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
  }
  return fn;
}

int make_map(CUtensorMap* m, const void* base, int inner, int rows, int box_rows) {
  auto fn = encode_fn();
  if (!fn) {
    set_error("cuTensorMapEncodeTiled is not available from the driver");
    return FFS_ERR_CUDA;
  }
  cuuint64_t dims[2] = {(cuuint64_t)inner, (cuuint64_t)rows};
  cuuint64_t strides[1] = {(cuuint64_t)inner * 2};
  cuuint32_t box[2] = {(cuuint32_t)BK, (cuuint32_t)box_rows};
  cuuint32_t estr[2] = {1, 1};
  CUresult r = fn(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT16, 2, const_cast<void*>(base), dims, strides, box, estr,
                  CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                  CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) {
    set_error("cuTensorMapEncodeTiled failed (%d) for a %d x %d fp16 operand", (int)r, rows, inner);
    return FFS_ERR_CUDA;
  }
  return FFS_OK;
}

// Maps of both operands (B boxes of prm.NB rows) and the persistent launch:
// one CTA per SM, at most max_items CTAs.
int launch_tc(const ffs_project_args* a, const TcParams& prm, int max_items, void* stream) {
  CUtensorMap ta_hi, ta_lo, tb_hi, tb_lo;
  int st;
  if ((st = make_map(&ta_hi, a->yr_hi, a->ld_y, a->V, BM))) return st;
  if ((st = make_map(&ta_lo, a->yr_lo, a->ld_y, a->V, BM))) return st;
  if ((st = make_map(&tb_hi, a->u_hi, a->ld_u, a->P * a->K, prm.NB))) return st;
  if ((st = make_map(&tb_lo, a->u_lo, a->ld_u, a->P * a->K, prm.NB))) return st;
  const int stage_bytes = 2 * A_TILE + 2 * prm.NB * BK * 2;
  const size_t smem = (size_t)STAGES * stage_bytes + 1024 + 128;
  FFS_REQUIRE(smem <= 227 * 1024, "project_tc: tile needs %zu bytes of shared memory", smem);
  auto kern = prm.items ? project_tc_kernel<true> : project_tc_kernel<false>;
  FFS_CUDA(ensure_dyn_smem(reinterpret_cast<const void*>(kern), smem));
  int n_sm = 0;
  FFS_CUDA(sm_count(&n_sm));
  if (max_items <= 0) return FFS_OK;
  kern<<<min(max_items, n_sm), 192, smem, (cudaStream_t)stream>>>(ta_hi, ta_lo, tb_hi, tb_lo, prm);
  return check_launch("project_tc_kernel");
}

// Pairs per B tile of the grid-mode projection, per K (0: the widest tile,
// 256 / K pairs); set by the autotuner through ffs_reml_tune_tc_pairs.
std::mutex g_tune_mu;
int g_tune_pairs[257] = {0};

int tc_pairs_for(int K, int P) {
  int g = 0;
  {
    std::lock_guard<std::mutex> lock(g_tune_mu);
    g = g_tune_pairs[K];
  }
  if (g <= 0 || g * K > 256) g = 256 / K;
  return g < P ? g : P;
}

}  // namespace
}  // namespace ffsk

using namespace ffsk;

extern "C" int ffs_reml_tune_tc_pairs(int K, int pairs) {
  clear_error();
  FFS_REQUIRE(K > 0 && K <= 256 && pairs >= 0 && pairs * K <= 256,
              "ffs_reml_tune_tc_pairs: K=%d pairs=%d (pairs x K <= 256; 0 resets)", K, pairs);
  std::lock_guard<std::mutex> lock(g_tune_mu);
  g_tune_pairs[K] = pairs;
  return FFS_OK;
}

extern "C" int ffs_reml_project_tc(const ffs_project_args* a, void* stream) {
  clear_error();
  FFS_REQUIRE(a && a->V > 0 && a->T > 0 && a->K > 0 && a->P > 0, "ffs_reml_project_tc: bad sizes");
  FFS_REQUIRE(a->yr_hi && a->yr_lo && a->u_hi && a->u_lo && a->yexp && a->uexp && a->proj && a->flag,
              "ffs_reml_project_tc: null buffer");
  FFS_REQUIRE(a->ld_y == a->ld_u && a->ld_y % BK == 0 && a->ld_y >= a->T,
              "ffs_reml_project_tc: ld_y=%d and ld_u=%d must be equal multiples of %d", a->ld_y, a->ld_u, BK);
  if (a->K > 256) {
    set_error("ffs_reml_project_tc: K=%d exceeds one 256-column MMA tile", a->K);
    return FFS_ERR_UNSUPPORTED;
  }
  for (const void* ptr : {(const void*)a->yr_hi, (const void*)a->yr_lo, (const void*)a->u_hi, (const void*)a->u_lo})
    FFS_REQUIRE(((uintptr_t)ptr & 15) == 0, "ffs_reml_project_tc: operands must be 16-byte aligned");
  TcParams prm;
  prm.V = a->V;
  prm.K = a->K;
  prm.P = a->P;
  prm.ld = a->ld_y;
  prm.g = tc_pairs_for(a->K, a->P);
  prm.N = ((prm.g * a->K) + 15) / 16 * 16;
  prm.n_col_tiles = ceil_div(a->P, prm.g);
  prm.n_vox_tiles = ceil_div(a->V, BM);
  prm.NB = prm.N;
  prm.T = a->T;
  prm.items = nullptr;
  prm.n_items = nullptr;
  prm.s_vox = 0;
  prm.yexp = a->yexp;
  prm.uexp = a->uexp;
  prm.proj = a->proj;
  prm.flag = a->flag;
  prm.v_dev = a->V_dev;
  return launch_tc(a, prm, prm.n_col_tiles * prm.n_vox_tiles, stream);
}

extern "C" int ffs_reml_project_tc_list(const ffs_project_args* a, const ffs_tc_item* items, const int* n_items,
                                        int max_items, int max_pairs, int ld_out, void* stream) {
  clear_error();
  FFS_REQUIRE(a && a->V > 0 && a->T > 0 && a->K > 0 && a->P > 0, "ffs_reml_project_tc_list: bad sizes");
  FFS_REQUIRE(a->yr_hi && a->yr_lo && a->u_hi && a->u_lo && a->yexp && a->uexp && a->proj && a->flag && items &&
                  n_items,
              "ffs_reml_project_tc_list: null buffer");
  FFS_REQUIRE(a->ld_y == a->ld_u && a->ld_y % BK == 0 && a->ld_y >= a->T,
              "ffs_reml_project_tc_list: ld_y=%d and ld_u=%d must be equal multiples of %d", a->ld_y, a->ld_u, BK);
  FFS_REQUIRE(max_pairs > 0 && max_pairs * a->K <= 256 && max_items > 0 && ld_out >= 0,
              "ffs_reml_project_tc_list: max_pairs=%d x K=%d must fit one 256-column tile", max_pairs, a->K);
  for (const void* ptr : {(const void*)a->yr_hi, (const void*)a->yr_lo, (const void*)a->u_hi, (const void*)a->u_lo})
    FFS_REQUIRE(((uintptr_t)ptr & 15) == 0, "ffs_reml_project_tc_list: operands must be 16-byte aligned");
  TcParams prm;
  prm.V = a->V;
  prm.K = a->K;
  prm.P = a->P;
  prm.ld = a->ld_y;
  prm.T = a->T;
  prm.g = max_pairs;
  prm.N = (max_pairs * a->K + 15) / 16 * 16;
  prm.NB = prm.N;
  prm.n_col_tiles = 1;
  prm.n_vox_tiles = 0;
  prm.items = items;
  prm.n_items = n_items;
  prm.s_vox = ld_out;
  prm.yexp = a->yexp;
  prm.uexp = a->uexp;
  prm.proj = a->proj;
  prm.flag = a->flag;
  prm.v_dev = nullptr;
  return launch_tc(a, prm, max_items, stream);
}
