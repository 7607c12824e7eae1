// Voxel bookkeeping of the learned-seeded fit on the device: the list of the
// voxels the full grid takes (compacted from their flags) and the merge of
// two result sets (every voxel's window answer and the full grid's answers
// for the listed voxels) into fresh output rows in one launch, so that the
// host never reads the flags and no per-field copy is launched.
#include "common.cuh"

namespace ffsk {

namespace {

// ids[slot] = v for the voxels with flag[v] != 0 (slots taken by warp-wide
// atomics, so in no particular order: each voxel's later results depend on
// its own row alone), pos[v] = its slot or -1. Slots at or past n_pad are
// not written (the voxel then keeps pos -1: the caller sizes n_pad from the
// same flags, so this does not happen).
__global__ void compact_kernel(int V, const int* __restrict__ flag, int n_pad, int* __restrict__ ids,
                               int* __restrict__ pos, int* __restrict__ count) {
  const int v = blockIdx.x * blockDim.x + threadIdx.x;
  const bool take = v < V && flag[v] != 0;
  const unsigned mk = __ballot_sync(0xffffffffu, take);
  int slot = -1;
  if (mk) {
    const int lane = threadIdx.x & 31;
    const int first = __ffs(mk) - 1;
    int base = 0;
    if (lane == first) base = atomicAdd(count, __popc(mk));
    base = __shfl_sync(0xffffffffu, base, first);
    if (take) {
      const int s = base + __popc(mk & ((1u << lane) - 1));
      if (s < n_pad) {
        ids[s] = v;
        slot = s;
      }
    }
  }
  if (v < V) pos[v] = slot;
}

constexpr int MERGE_MAX = 32;

struct MergeFields {
  ffs_merge_field f[MERGE_MAX];
};

// dst[v] = src_sub[pos[v]] when pos[v] >= 0 and the field has src_sub, else
// src[v] (a field without src leaves those rows as they are); blockIdx.y is
// the field, 16-byte words when the field's rows and pointers allow, 4-byte
// words otherwise
__global__ void __launch_bounds__(256) merge_kernel(int V, const int* __restrict__ pos, MergeFields m) {
  const ffs_merge_field fd = m.f[blockIdx.y];
  const bool vec = (fd.row_bytes & 15) == 0 && (((uintptr_t)fd.dst | (uintptr_t)fd.src |
                                                   (uintptr_t)fd.src_sub) & 15) == 0;
  const int wb = vec ? 16 : 4;
  const int nw = fd.row_bytes / wb;
  const long long total = (long long)V * nw;
  for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < total;
       e += (long long)gridDim.x * blockDim.x) {
    const int v = (int)(e / nw), k = (int)(e % nw);
    const int p = (pos && fd.src_sub) ? pos[v] : -1;
    if (p < 0 && !fd.src) continue;
    const char* s = p >= 0 ? static_cast<const char*>(fd.src_sub) + (size_t)p * fd.row_bytes
                           : static_cast<const char*>(fd.src) + (size_t)v * fd.row_bytes;
    char* d = static_cast<char*>(fd.dst) + (size_t)v * fd.row_bytes;
    if (vec) {
      reinterpret_cast<uint4*>(d)[k] = reinterpret_cast<const uint4*>(s)[k];
    } else {
      reinterpret_cast<uint32_t*>(d)[k] = reinterpret_cast<const uint32_t*>(s)[k];
    }
  }
}

constexpr int FINISH_EXTRA = 8;

struct FinishExtra {
  const int* p[FINISH_EXTRA];
};

// best_crit[v] = crit0[v] + dbest[v] in FP64, rounded to float; small[0] +=
// the flagged voxels of each block (small[0] is zeroed before the launch);
// block 0 copies the n_extra device ints into small[1 ..]
__global__ void __launch_bounds__(256) window_finish_kernel(int V, const double* __restrict__ crit0,
                                                            const float* __restrict__ dbest,
                                                            const int* __restrict__ fallback,
                                                            float* __restrict__ best_crit, int* small, int n_extra,
                                                            FinishExtra ex) {
  __shared__ int part[8];
  int cnt = 0;
  for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < V; v += gridDim.x * blockDim.x) {
    best_crit[v] = (float)(crit0[v] + (double)dbest[v]);
    cnt += fallback[v] != 0;
  }
  cnt = __reduce_add_sync(0xffffffffu, cnt);
  if ((threadIdx.x & 31) == 0) part[threadIdx.x >> 5] = cnt;
  __syncthreads();
  if (threadIdx.x == 0) {
    int s = 0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) s += part[w];
    if (s) atomicAdd(small, s);
    if (blockIdx.x == 0)
      for (int i = 0; i < n_extra; ++i) small[1 + i] = *ex.p[i];
  }
}

}  // namespace
}  // namespace ffsk

using namespace ffsk;

extern "C" int ffs_reml_compact(int V, const int* flag, int n_pad, int* ids, int* pos, int* count, void* stream) {
  clear_error();
  FFS_REQUIRE(V > 0 && n_pad >= 0 && flag && pos && count && (ids || n_pad == 0),
              "ffs_reml_compact: bad arguments (V=%d n_pad=%d)", V, n_pad);
  cudaStream_t st = (cudaStream_t)stream;
  FFS_CUDA(cudaMemsetAsync(count, 0, sizeof(int), st));
  if (n_pad > 0) FFS_CUDA(cudaMemsetAsync(ids, 0, sizeof(int) * (size_t)n_pad, st));
  compact_kernel<<<ceil_div(V, 256), 256, 0, st>>>(V, flag, n_pad, ids, pos, count);
  return check_launch("compact_kernel");
}

extern "C" int ffs_merge_rows(int V, const int* pos, int n_fields, const ffs_merge_field* fields, void* stream) {
  clear_error();
  FFS_REQUIRE(V > 0 && n_fields > 0 && n_fields <= MERGE_MAX && fields,
              "ffs_merge_rows: bad arguments (V=%d, %d fields, at most %d)", V, n_fields, MERGE_MAX);
  MergeFields m{};
  long long most = 0;
  for (int i = 0; i < n_fields; ++i) {
    const ffs_merge_field& f = fields[i];
    FFS_REQUIRE(f.dst && (f.src || (f.src_sub && pos)) && f.row_bytes > 0 && f.row_bytes % 4 == 0 &&
                    (((uintptr_t)f.dst | (uintptr_t)f.src | (uintptr_t)f.src_sub) & 3) == 0,
                "ffs_merge_rows: field %d: null buffer, or rows or pointers not 4-byte aligned", i);
    m.f[i] = f;
    most = std::max(most, (long long)V * f.row_bytes / 4);
  }
  const int blocks = (int)std::min<long long>(ceil_div(most, 256 * 4), 1184);
  merge_kernel<<<dim3(std::max(blocks, 1), n_fields), 256, 0, (cudaStream_t)stream>>>(V, pos, m);
  return check_launch("merge_kernel");
}

extern "C" int ffs_reml_window_finish(int V, const double* crit0, const float* dbest, const int* fallback,
                                      float* best_crit, int* small, int n_extra, const int* const* extra,
                                      void* stream) {
  clear_error();
  FFS_REQUIRE(V > 0 && crit0 && dbest && fallback && best_crit && small && n_extra >= 0 &&
                  n_extra <= FINISH_EXTRA && (n_extra == 0 || extra),
              "ffs_reml_window_finish: bad arguments (V=%d, %d extra, at most %d)", V, n_extra, FINISH_EXTRA);
  FinishExtra ex{};
  for (int i = 0; i < n_extra; ++i) {
    FFS_REQUIRE(extra[i], "ffs_reml_window_finish: null extra pointer %d", i);
    ex.p[i] = extra[i];
  }
  cudaStream_t st = (cudaStream_t)stream;
  FFS_CUDA(cudaMemsetAsync(small, 0, sizeof(int), st));
  window_finish_kernel<<<std::min(ceil_div(V, 256), 4 * 152), 256, 0, st>>>(V, crit0, dbest, fallback, best_crit,
                                                                            small, n_extra, ex);
  return check_launch("window_finish_kernel");
}
