// Learned-seeded refine: each voxel evaluates only the 5 x 5 lattice window
// around its proposed (a, b) (clamped to the lattice), with the same
// criterion as the full grid (fastfuncstuff/glm/arma.py:1983-2002, relative
// to the pair (0, 0)), and is flagged for the full-grid search when its best
// pair is not an identity pair and has a valid lattice neighbour outside the
// window.
//
// The voxels arrive sorted by window centre (rows of the sorted operands).
//   window_items   one work item per (128-row tile of a centre, run of
//                  consecutive valid pairs of one window row): the tcgen05
//                  projection kernel's work list (||U'y||^2 per window slot);
//   window_crit    one thread per sorted voxel: y'R^-1 y of every window pair
//                  by the O(T) recurrence, the criterion, the argmin and the
//                  edge test.
// Pairs with lambda == 0 (R = I, the identity) all have the criterion of the
// pair (0, 0) exactly (d = 0), and the full grid breaks that tie towards the
// first identity pair in pair order, p_id. Window identity pairs are not
// evaluated: a window holding one competes with (p_id, d = 0) instead.
#include <algorithm>

#include "common.cuh"

namespace ffsk {
namespace {

constexpr int WIN = 5;
constexpr int WSLOTS = WIN * WIN;
constexpr int WTILE = 128;  // operand rows per projection item

__device__ __forceinline__ void window_of(int c, int n_a, int n_b, int& a0, int& wa, int& b0, int& wb) {
  const int ca = c / n_b, cb = c % n_b;
  wa = min(WIN, n_a);
  wb = min(WIN, n_b);
  a0 = min(max(ca - WIN / 2, 0), n_a - wa);
  b0 = min(max(cb - WIN / 2, 0), n_b - wb);
}

// one thread per lattice cell; cell c's voxels are sorted rows
// [end[c-1], end[c]) (end[-1] = 0)
__global__ void window_items_kernel(int ncell, const int* end, int n_a, int n_b, const int* lattice, int K,
                                    int max_pairs, ffs_tc_item* items, int* n_items, int max_items, int2* tiles,
                                    int* n_tiles, int max_tiles, int* overflow, int P) {
  const int key = blockIdx.x * blockDim.x + threadIdx.x;
  if (key >= ncell) return;
  // with designs (P > 0) the key is cell * n_designs + design: the work items
  // of a key read its design's U rows, (design * P + pair) * K, and the
  // criterion tiles of a cell span the rows of all its designs (the window
  // is the cell's), emitted by the key of the cell's first design
  const int D = P > 0 ? ncell / (n_a * n_b) : 1;
  const int c = key / D, dsg = key % D;
  const int row0 = dsg * P * K;
  const int s0 = key ? end[key - 1] : 0, n = end[key] - s0;
  if (dsg == 0) {
    const int cn = end[key + D - 1] - s0;
    const int ntile = (cn + WTILE - 1) / WTILE;
    const int tt = ntile > 0 ? atomicAdd(n_tiles, ntile) : 0;
    for (int t = 0; t < ntile; ++t) {
      if (tt + t >= max_tiles) {
        atomicExch(overflow, 1);
        break;
      }
      tiles[tt + t] = make_int2(s0 + t * WTILE, min(WTILE, cn - t * WTILE));
    }
  }
  if (n <= 0) return;
  int a0, wa, b0, wb;
  window_of(c, n_a, n_b, a0, wa, b0, wb);
  const int ntile = (n + WTILE - 1) / WTILE;
  // the window's runs of consecutive valid pairs (at most one per pair)
  int seg_p[WSLOTS], seg_np[WSLOTS], seg_slot[WSLOTS], nseg = 0;
  for (int ra = 0; ra < wa; ++ra) {
    int rb = 0;
    while (rb < wb) {
      const int p = lattice[(a0 + ra) * n_b + b0 + rb];
      if (p < 0) {
        ++rb;
        continue;
      }
      int np = 1;
      while (rb + np < wb && np < max_pairs && lattice[(a0 + ra) * n_b + b0 + rb + np] == p + np) ++np;
      seg_p[nseg] = p;
      seg_np[nseg] = np;
      seg_slot[nseg++] = ra * WIN + rb;
      rb += np;
    }
  }
  // tile-major: the segments of one operand tile are consecutive items, so
  // the CTAs that take them at the same time share the tile in L2
  const int at = atomicAdd(n_items, ntile * nseg);
  for (int t = 0; t < ntile; ++t) {
    for (int sg = 0; sg < nseg; ++sg) {
      const int k = at + t * nseg + sg;
      if (k >= max_items) {
        atomicExch(overflow, 1);
        return;
      }
      ffs_tc_item it;
      it.v0 = s0 + t * WTILE;
      it.nv = min(WTILE, n - t * WTILE);
      it.row_b = row0 + seg_p[sg] * K;
      it.np = seg_np[sg];
      it.out0 = it.v0;
      it.slot0 = seg_slot[sg];
      items[k] = it;
    }
  }
}

// one thread per segment s of the sorted rows [end[s-1], end[s]) (end[-1] =
// 0): an item per 128-row tile and block of at most max_pairs of the
// segment's n_pairs pairs, U rows from (s * n_pairs + first pair) * K
__global__ void segment_items_kernel(int n_seg, const int* end, int n_pairs, int K, int max_pairs,
                                     ffs_tc_item* items, int* n_items, int max_items, int* overflow) {
  const int sg = blockIdx.x * blockDim.x + threadIdx.x;
  if (sg >= n_seg) return;
  const int s0 = sg ? end[sg - 1] : 0, n = end[sg] - s0;
  if (n <= 0) return;
  const int ntile = (n + WTILE - 1) / WTILE, nblk = (n_pairs + max_pairs - 1) / max_pairs;
  const int at = atomicAdd(n_items, ntile * nblk);
  for (int t = 0; t < ntile; ++t) {
    for (int bk = 0; bk < nblk; ++bk) {
      const int k = at + t * nblk + bk;
      if (k >= max_items) {
        atomicExch(overflow, 1);
        return;
      }
      ffs_tc_item it;
      it.v0 = s0 + t * WTILE;
      it.nv = min(WTILE, n - t * WTILE);
      it.row_b = (sg * n_pairs + bk * max_pairs) * K;
      it.np = min(max_pairs, n_pairs - bk * max_pairs);
      it.out0 = it.v0;
      it.slot0 = bk * max_pairs;
      items[k] = it;
    }
  }
}

__global__ void clamp_count_kernel(int* n_items, int max_items, int* n_tiles, int max_tiles) {
  if (*n_items > max_items) *n_items = max_items;
  if (*n_tiles > max_tiles) *n_tiles = max_tiles;
}

struct CritArgs {
  int n, T, K, n_a, n_b;
  const int* lattice;       // [n_a][n_b]
  const int* idx;           // [n] voxel of each sorted row
  const int* center;        // [V] window centre cell of each voxel (read at idx[i])
  const float* rows;        // [V][T] residualised rows, voxel-major (read at idx[i])
  const float4* coef;       // [P][T]
  const float* winproj;     // [n][25]
  const float* dcf;         // [P] (logdet_R + logdet_XtX)[p] - that of (0, 0)
  const uint8_t* ident;     // [P]
  int p_id;
  const double* c_p0;       // device scalar: logdet_R + logdet_XtX of (0, 0)
  int* best;                // outputs at idx[i]
  float* dbest;
  double* crit0;
  int* fallback;
  int* best_cell;
  int* next_center;         // NULL, or [V]: the next round's centre of each voxel taken
  const int* design;        // NULL, or [V]: each voxel's design; dcf then [n_designs][P], c_p0 [n_designs]
  int P;
  const float* ssw_pre;     // NULL, or [n][WSLOTS]: y'R^-1 y of each row and window slot (the banded R)
};

constexpr int CRIT_TB = 16;  // steps per partial sum and sample prefetch

// One CTA per tile of WTILE sorted rows that share a window centre, one thread
// per row, one pass over each series: the time axis is walked in chunks of
// WCH steps, for which the coefficients (-m, 1/D) of every window row's <= 5
// non-identity pairs and the row's AR filter c_t (its pairs share a) are
// staged in shared memory; each 16-sample block of the series is loaded once
// and advances the recurrences of all window rows, whose per-thread states
// (v_{t-1} and the running sum of v^2 / D of each pair) live in shared memory
// between blocks. As in the surface kernel, a step whose coefficients equal
// the previous step's (for every pair of that window row) reuses the
// registers, and a block of 16 such steps sums v^2 alone and scales the block
// sum by 1/D once; each row keeps its own steady flags, so a pair's
// arithmetic does not depend on the other rows. y'y is summed on the way.
constexpr int WCH = 64;  // steps per staged chunk (a multiple of CRIT_TB)
constexpr int WCP = (WIN + 1) / 2;  // pair couples of a window row
constexpr int WCB = WCH / CRIT_TB;

__host__ __device__ inline size_t crit_smem_bytes() {
  return sizeof(float2) * WIN * WIN * (WCH + 1) + sizeof(float) * WIN * (WCH + 1) +
         2 * sizeof(float) * WIN * WIN * WTILE + WIN * WCH + WIN * WCB;
}

__global__ void __launch_bounds__(WTILE, 4) window_crit_kernel(CritArgs w, const int2* tiles, const int* n_tiles) {
  extern __shared__ float2 tab[];  // [WIN rows][WIN pairs][WCH + 1]: steps c0 - 1 .. c0 + WCH - 1
  float* cs = reinterpret_cast<float*>(tab + WIN * WIN * (WCH + 1));  // [WIN][WCH + 1] AR filter c_t
  float* svv = cs + WIN * (WCH + 1);                                   // [WIN * WIN][WTILE] v_{t-1}
  float* sst = svv + WIN * WIN * WTILE;                                // [WIN * WIN][WTILE] sum of v^2 / D
  uint8_t* steady = reinterpret_cast<uint8_t*>(sst + WIN * WIN * WTILE);  // [WIN][WCH]
  uint8_t* bsteady = steady + WIN * WCH;                                   // [WIN][WCB]
  __shared__ int s_pr[WIN][WIN], s_col[WIN][WIN], s_np[WIN], s_ident;
  if ((int)blockIdx.x >= *n_tiles) return;
  const int2 tl = tiles[blockIdx.x];
  const int tid = threadIdx.x;
  const int i = tl.x + tid;
  const bool live = tid < tl.y;
  const int c = w.center[w.idx[tl.x]];  // every row of the tile has this centre
  // the row's design (grouped designs: a tile's rows share the cell, not
  // necessarily the design) and its criterion constants
  const int dsg = w.design ? w.design[w.idx[live ? i : tl.x]] : 0;
  const float* dcf = w.dcf + (size_t)dsg * w.P;
  int a0, wa, b0, wb;
  window_of(c, w.n_a, w.n_b, a0, wa, b0, wb);
  const int T = w.T, Tk = w.T - w.K;
  // this thread's residualised series, voxel-major: 16 samples per block as
  // four 16-byte loads when T % 4 == 0
  const float* yrow = w.rows + (size_t)w.idx[live ? i : tl.x] * w.T;
  const bool vec = (w.T & 3) == 0;

  // the window's non-identity pairs by row (compacted), and whether it holds
  // an identity pair (R = I: criterion d = 0)
  if (tid == 0) {
    int hid = 0;
    for (int ra = 0; ra < WIN; ++ra) {
      int n = 0;
      for (int rb = 0; rb < WIN; ++rb) {
        s_pr[ra][rb] = -1;
        s_col[ra][rb] = 0;
      }
      for (int rb = 0; rb < WIN; ++rb) {
        const int p = (ra < wa && rb < wb) ? w.lattice[(a0 + ra) * w.n_b + b0 + rb] : -1;
        if (p < 0) continue;
        if (w.ident[p]) {
          hid = 1;
        } else {
          s_pr[ra][n] = p;
          s_col[ra][n] = rb;
          ++n;
        }
      }
      s_np[ra] = n;
    }
    s_ident = hid;
  }
  for (int e = tid; e < WIN * WIN * WTILE; e += blockDim.x) {
    svv[e] = 0.f;
    sst[e] = 0.f;
  }
  __syncthreads();
  const bool has_ident = s_ident != 0;

  float yy = 0.f;  // y'y in the full grid's blocks (the identity chunk of the surface kernel)
  float yp = 0.f;
  // 16 samples of this thread's series from t0 (zero past T); each block's
  // samples are requested one block ahead, so the loads overlap the work
  auto load_block = [&](float (&dst)[CRIT_TB], int t0) {
    if (vec) {
#pragma unroll
      for (int k = 0; k < CRIT_TB; k += 4) {
        const float4 q = t0 + k < T ? *reinterpret_cast<const float4*>(yrow + t0 + k)
                                    : make_float4(0.f, 0.f, 0.f, 0.f);
        dst[k] = q.x;
        dst[k + 1] = q.y;
        dst[k + 2] = q.z;
        dst[k + 3] = q.w;
      }
    } else {
#pragma unroll
      for (int k = 0; k < CRIT_TB; ++k) dst[k] = (t0 + k < T) ? yrow[t0 + k] : 0.f;
    }
  };
  float yb[CRIT_TB];
  load_block(yb, 0);
  // a warp holding no row of the tile (a partly filled tile: the re-centred
  // rounds' tiles often hold a few rows) stages the tables but skips the
  // recurrences
  const bool warp_live = (tid & ~31) < tl.y;
  if (w.ssw_pre && live) {
    // the banded R's sums come from band_sums_kernel: y'y alone here, in the
    // recurrence path's blocks
    for (int t0 = 0; t0 < T; t0 += CRIT_TB) {
      float yq[CRIT_TB];
      load_block(yq, t0);
      float yy_b = 0.f;
#pragma unroll
      for (int k = 0; k < CRIT_TB; ++k) yy_b = fmaf(yq[k], yq[k], yy_b);
      yy += yy_b;
    }
  }
  for (int c0 = 0; c0 < T && !w.ssw_pre; c0 += WCH) {
    const int cn = min(WCH, T - c0);
    __syncthreads();  // the previous chunk's tables are no longer read
    for (int e = tid; e < WIN * WIN * (cn + 1); e += blockDim.x) {
      const int rg = e / (cn + 1), s = e % (cn + 1);
      const int r = rg / WIN, g = rg % WIN;
      const int t = c0 - 1 + s;
      const int p = s_pr[r][g];
      float2 v2 = make_float2(0.f, 0.f);
      float cv = 0.f;
      if (p >= 0 && t >= 0) {
        const float4 q = w.coef[(size_t)p * T + t];
        v2 = make_float2(-q.y, q.z);
        cv = q.x;
      }
      tab[(size_t)rg * (WCH + 1) + s] = v2;
      if (g == 0) cs[(size_t)r * (WCH + 1) + s] = cv;
    }
    __syncthreads();
    // steady steps of each row: every pair's coefficients (and c) equal the
    // previous step's
    for (int e = tid; e < WIN * cn; e += blockDim.x) {
      const int r = e / cn, s = e % cn;
      const float* cr = cs + (size_t)r * (WCH + 1);
      bool same = c0 + s > 0 && cr[s + 1] == cr[s];
      for (int g = 0; g < s_np[r] && same; ++g) {
        const float2 x = tab[(size_t)(r * WIN + g) * (WCH + 1) + s + 1];
        const float2 y = tab[(size_t)(r * WIN + g) * (WCH + 1) + s];
        same = x.x == y.x && x.y == y.y;
      }
      steady[r * WCH + s] = same ? 1 : 0;
    }
    __syncthreads();
    for (int e = tid; e < WIN * WCB; e += blockDim.x) {
      const int r = e / WCB, bk = e % WCB;
      bool all = bk * CRIT_TB + CRIT_TB <= cn;
      for (int s = bk * CRIT_TB; s < bk * CRIT_TB + CRIT_TB && all; ++s) all = steady[r * WCH + s] != 0;
      bsteady[e] = all ? 1 : 0;
    }
    __syncthreads();
    for (int bs = 0; bs < cn && warp_live; bs += CRIT_TB) {
      const int t0 = c0 + bs;
      float yn[CRIT_TB];
      load_block(yn, t0 + CRIT_TB);
      {
        float yy_b = 0.f;
#pragma unroll
        for (int k = 0; k < CRIT_TB; ++k) yy_b = fmaf(yb[k], yb[k], yy_b);
        yy += yy_b;
      }
      for (int r = 0; r < WIN; ++r) {
        const int npr = s_np[r];
        if (npr == 0) continue;  // uniform over the CTA
        const float2* tr = tab + (size_t)r * WIN * (WCH + 1);
        const float* crr = cs + (size_t)r * (WCH + 1);
        // the row's pairs as couples (2c, 2c + 1) in 64-bit registers, advanced
        // with packed f32x2 instructions (two fmaf each, so the same values)
        uint64_t vv[WCP], st[WCP], sq[WCP], nm[WCP], id[WCP];
        // the coefficients at the block's first step: the table's value there
        // equals what a step-by-step walk holds in its registers
        float cc = crr[bs + 1];
#pragma unroll
        for (int c = 0; c < WCP; ++c) {
          const bool on0 = 2 * c < npr, on1 = 2 * c + 1 < npr;
          const int e0 = (r * WIN + 2 * c) * WTILE + tid, e1 = e0 + WTILE;
          vv[c] = pack2(on0 ? svv[e0] : 0.f, on1 ? svv[e1] : 0.f);
          st[c] = pack2(on0 ? sst[e0] : 0.f, on1 ? sst[e1] : 0.f);
          const float2 q0 = on0 ? tr[(size_t)(2 * c) * (WCH + 1) + bs + 1] : make_float2(0.f, 0.f);
          const float2 q1 = on1 ? tr[(size_t)(2 * c + 1) * (WCH + 1) + bs + 1] : make_float2(0.f, 0.f);
          nm[c] = pack2(q0.x, q1.x);
          id[c] = pack2(q0.y, q1.y);
          sq[c] = pack2(0.f, 0.f);
        }
        float ypr = yp;
        if (bsteady[r * WCB + bs / CRIT_TB]) {
          // CRIT_TB steady steps: coefficients in registers, sum of v^2 alone
#pragma unroll
          for (int k = 0; k < CRIT_TB; ++k) {
            const float z = fmaf(-cc, ypr, yb[k]);
            ypr = yb[k];
            const uint64_t z2 = pack2(z, z);
#pragma unroll
            for (int c = 0; c < WCP; ++c) {
              vv[c] = fma2(nm[c], vv[c], z2);
              sq[c] = fma2(vv[c], vv[c], sq[c]);
            }
          }
#pragma unroll
          for (int c = 0; c < WCP; ++c) st[c] = fma2(sq[c], id[c], st[c]);
        } else {
          const uint8_t* sr = steady + r * WCH;
#pragma unroll
          for (int k = 0; k < CRIT_TB; ++k) {
            if (t0 + k < T) {
              if (!sr[bs + k]) {
                cc = crr[bs + k + 1];
#pragma unroll
                for (int c = 0; c < WCP; ++c) {
                  const bool on0 = 2 * c < npr, on1 = 2 * c + 1 < npr;
                  const float2 q0 = on0 ? tr[(size_t)(2 * c) * (WCH + 1) + bs + k + 1] : make_float2(0.f, 0.f);
                  const float2 q1 = on1 ? tr[(size_t)(2 * c + 1) * (WCH + 1) + bs + k + 1] : make_float2(0.f, 0.f);
                  nm[c] = pack2(q0.x, q1.x);
                  id[c] = pack2(q0.y, q1.y);
                }
              }
              const float z = fmaf(-cc, ypr, yb[k]);
              ypr = yb[k];
              const uint64_t z2 = pack2(z, z);
#pragma unroll
              for (int c = 0; c < WCP; ++c) {
                vv[c] = fma2(nm[c], vv[c], z2);
                sq[c] = fma2(mul2(vv[c], id[c]), vv[c], sq[c]);
              }
            }
          }
#pragma unroll
          for (int c = 0; c < WCP; ++c) st[c] = add2(st[c], sq[c]);
        }
#pragma unroll
        for (int c = 0; c < WCP; ++c) {
          float v0, v1, s0, s1;
          unpack2(vv[c], v0, v1);
          unpack2(st[c], s0, s1);
          const int e0 = (r * WIN + 2 * c) * WTILE + tid, e1 = e0 + WTILE;
          if (2 * c < npr) {
            svv[e0] = v0;
            sst[e0] = s0;
          }
          if (2 * c + 1 < npr) {
            svv[e1] = v1;
            sst[e1] = s1;
          }
        }
      }
      yp = yb[CRIT_TB - 1];
#pragma unroll
      for (int k = 0; k < CRIT_TB; ++k) yb[k] = yn[k];
    }
  }

  // best non-identity window pair
  int best = -1, bcell = -1;
  float bd = INFINITY;
  for (int ra = 0; ra < WIN; ++ra) {
    for (int g = 0; g < s_np[ra]; ++g) {
      if (!live) break;
      const int p = s_pr[ra][g];
      const float stv = w.ssw_pre ? w.ssw_pre[(size_t)i * WSLOTS + ra * WIN + s_col[ra][g]]
                                  : sst[(ra * WIN + g) * WTILE + tid];
      const float rss = fmaxf(stv - w.winproj[(size_t)i * WSLOTS + ra * WIN + s_col[ra][g]], 0.f);
      const float d = dcf[p] + (float)Tk * log1pf((rss - yy) / (yy + 1e-10f));
      if (d < bd || (d == bd && p < best) || best < 0) {
        bd = d;
        best = p;
        bcell = (a0 + ra) * w.n_b + b0 + s_col[ra][g];
      }
    }
  }
  const float rss0 = yy;  // ||Q0'y_r||^2 of the residualised series is zero to rounding
  if (!live) return;
  // The identity pairs (d = 0) take part when the window holds one of them,
  // and then a win by them is final. A window without them whose best is not
  // below 0 goes to the full grid (the identity pairs outside it are at least
  // as good); otherwise the edge test decides.
  int fb = 0;
  if (has_ident && (bd > 0.f || (bd == 0.f && w.p_id < best) || best < 0)) {
    best = w.p_id;
    bd = 0.f;
    bcell = -1;
  } else if (best < 0 || bd >= 0.f) {
    fb = 1;
    if (best < 0) {
      best = w.p_id;
      bd = 0.f;
    }
  } else {
    const int ba = bcell / w.n_b, bb = bcell % w.n_b;
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
  }
  const int v = w.idx[i];
  w.best[v] = best;
  w.dbest[v] = bd;
  w.crit0[v] = w.c_p0[dsg] + (double)Tk * log((double)rss0 + 1e-10);
  w.fallback[v] = fb;
  w.best_cell[v] = bcell;
  // a voxel on its window's edge is re-centred on its best pair; the rest
  // (and those without a non-identity candidate) skip the next round
  if (w.next_center) w.next_center[v] = (fb && bcell >= 0) ? bcell : w.n_a * w.n_b;
}

// ---------------------------------------------------------------------- strip
// The strip next to the identity line: pairs of distinct a (each its own AR
// filter), evaluated for the sorted rows i < min(n, *n_dev) of the voxels
// idx[i] after the window rounds, to find a second basin of the criterion
// that the windows could not see. One thread per row, STRIP_TILE rows per
// CTA and STRIP_G pairs per CTA (blockIdx.y: the group of pairs). Per chunk
// of WCH steps the pairs' (c_t, -m_t, 1/D_t) are staged in shared memory with
// per-couple steady flags; each thread keeps its pairs' states as couples in
// 64-bit registers advanced with packed f32x2 instructions, in the window
// kernel's operation order (z = y_t - c_t y_{t-1}, v = z - m v, and in a
// block of 16 steady steps the sum of v^2 scaled by 1/D once), so a strip
// pair that is also a window pair gets the window's criterion up to the
// steady/non-steady split of its couple. A voxel whose least strip criterion
// lies below its window answer dbest[v] by more than 1e-6 of |crit0[v]| is
// sent to the full grid: fallback[v] = 1, best_cell[v] = -1 (several CTAs may
// store the same values).
constexpr int STRIP_TILE = 128;
constexpr int STRIP_G = 16;
constexpr int STRIP_G2 = STRIP_G / 2;
constexpr int STRIP_MAX = 64;  // pairs per call

struct StripArgs {
  int n, T, K, n_pairs;
  const int* n_dev;      // device count of real sorted rows (or NULL: n)
  const int* pairs;      // [n_pairs] pair indices
  const int* idx;        // [n] voxel of each sorted row
  const float* rows;     // [V][T] residualised rows (read at idx[i])
  const float4* coef;    // [P][T] (c, m, 1/D, -)
  const float* proj;     // [n_pairs][n] ||U'y||^2 of each strip pair and sorted row
  const float* dcf;      // [P] (logdet_R + logdet_XtX)[p] - that of (0, 0)
  const float* dbest;    // [V] the window rounds' criterion (relative to (0, 0))
  const double* crit0;   // [V] the criterion at (0, 0)
  int* fallback;         // [V]
  int* best_cell;        // [V]
  const int* design;     // [V] each voxel's design (dcf [n_designs][P]), or NULL (dcf [P])
  int P;                 // pairs per design
  const float* ssw_pre;  // NULL, or [n_pairs][n]: y'R^-1 y of each pair and row (the banded R)
};

__global__ void __launch_bounds__(STRIP_TILE) strip_crit_kernel(StripArgs w) {
  __shared__ float4 tab[STRIP_G][WCH + 1];  // (-c, -m, 1/D, 0) at steps c0 - 1 .. c0 + WCH - 1
  __shared__ uint8_t steady[STRIP_G2][WCH];
  __shared__ uint8_t bsteady[STRIP_G2][WCB];
  const int m = w.n_dev ? min(w.n, *w.n_dev) : w.n;
  const int r0 = blockIdx.x * STRIP_TILE;
  if (r0 >= m) return;  // uniform over the CTA
  const int q0 = blockIdx.y * STRIP_G;
  const int nq = min(STRIP_G, w.n_pairs - q0);
  const int tid = threadIdx.x;
  const int i = r0 + tid;
  const bool live = i < m;
  const int T = w.T;
  const float* yrow = w.rows + (size_t)w.idx[live ? i : r0] * T;
  const bool vec = (T & 3) == 0;
  const uint64_t zero2 = pack2(0.f, 0.f);
  uint64_t vv[STRIP_G2], st[STRIP_G2];
#pragma unroll
  for (int j = 0; j < STRIP_G2; ++j) vv[j] = st[j] = zero2;
  float yy = 0.f, yp = 0.f;
  if (w.ssw_pre && live) {
    // the banded R's sums come from band_sums_kernel: y'y alone here
    for (int t0 = 0; t0 < T; t0 += CRIT_TB) {
      float yy_b = 0.f;
      for (int k = 0; k < CRIT_TB; ++k) {
        const float y = t0 + k < T ? yrow[t0 + k] : 0.f;
        yy_b = fmaf(y, y, yy_b);
      }
      yy += yy_b;
    }
  }
  for (int c0 = 0; c0 < T && !w.ssw_pre; c0 += WCH) {
    const int cn = min(WCH, T - c0);
    __syncthreads();  // the previous chunk's tables are no longer read
    for (int e = tid; e < STRIP_G * (cn + 1); e += blockDim.x) {
      const int q = e / (cn + 1), s = e % (cn + 1);
      const int t = c0 - 1 + s;
      float4 c = make_float4(0.f, 0.f, 0.f, 0.f);  // an empty slot: nothing summed
      if (q < nq && t >= 0) {
        const float4 r = w.coef[(size_t)w.pairs[q0 + q] * T + t];
        c = make_float4(-r.x, -r.y, r.z, 0.f);
      }
      tab[q][s] = c;
    }
    __syncthreads();
    for (int e = tid; e < STRIP_G2 * cn; e += blockDim.x) {
      const int j = e / cn, s = e % cn;
      bool same = c0 + s > 0;
      for (int h = 0; h < 2 && same; ++h) {
        const float4 x = tab[2 * j + h][s + 1], y = tab[2 * j + h][s];
        same = x.x == y.x && x.y == y.y && x.z == y.z;
      }
      steady[j][s] = same ? 1 : 0;
    }
    __syncthreads();
    for (int e = tid; e < STRIP_G2 * WCB; e += blockDim.x) {
      const int j = e / WCB, bk = e % WCB;
      bool all = bk * CRIT_TB + CRIT_TB <= cn;
      for (int s = bk * CRIT_TB; s < bk * CRIT_TB + CRIT_TB && all; ++s) all = steady[j][s] != 0;
      bsteady[j][bk] = all ? 1 : 0;
    }
    __syncthreads();
    for (int bs = 0; bs < cn; bs += CRIT_TB) {
      const int t0 = c0 + bs;
      float yb[CRIT_TB];
      if (vec) {
#pragma unroll
        for (int k = 0; k < CRIT_TB; k += 4) {
          const float4 q4 = t0 + k < T ? *reinterpret_cast<const float4*>(yrow + t0 + k)
                                       : make_float4(0.f, 0.f, 0.f, 0.f);
          yb[k] = q4.x;
          yb[k + 1] = q4.y;
          yb[k + 2] = q4.z;
          yb[k + 3] = q4.w;
        }
      } else {
#pragma unroll
        for (int k = 0; k < CRIT_TB; ++k) yb[k] = (t0 + k < T) ? yrow[t0 + k] : 0.f;
      }
      {
        float yy_b = 0.f;
#pragma unroll
        for (int k = 0; k < CRIT_TB; ++k) yy_b = fmaf(yb[k], yb[k], yy_b);
        yy += yy_b;
      }
#pragma unroll
      for (int j = 0; j < STRIP_G2; ++j) {
        if (2 * j < nq) {  // uniform over the CTA
          float4 ca = tab[2 * j][bs + 1], cb = tab[2 * j + 1][bs + 1];
          uint64_t nc = pack2(ca.x, cb.x), nm = pack2(ca.y, cb.y), id = pack2(ca.z, cb.z);
          uint64_t v2 = vv[j], sq = zero2;
          float ypr = yp;
          if (bsteady[j][bs / CRIT_TB]) {
#pragma unroll
            for (int k = 0; k < CRIT_TB; ++k) {
              const uint64_t z = fma2(nc, pack2(ypr, ypr), pack2(yb[k], yb[k]));
              ypr = yb[k];
              v2 = fma2(nm, v2, z);
              sq = fma2(v2, v2, sq);
            }
            st[j] = fma2(sq, id, st[j]);
          } else {
#pragma unroll
            for (int k = 0; k < CRIT_TB; ++k) {
              if (t0 + k < T) {
                if (!steady[j][bs + k]) {
                  ca = tab[2 * j][bs + k + 1];
                  cb = tab[2 * j + 1][bs + k + 1];
                  nc = pack2(ca.x, cb.x);
                  nm = pack2(ca.y, cb.y);
                  id = pack2(ca.z, cb.z);
                }
                const uint64_t z = fma2(nc, pack2(ypr, ypr), pack2(yb[k], yb[k]));
                ypr = yb[k];
                v2 = fma2(nm, v2, z);
                sq = fma2(mul2(v2, id), v2, sq);
              }
            }
            st[j] = add2(st[j], sq);
          }
          vv[j] = v2;
        }
      }
      yp = yb[CRIT_TB - 1];
    }
  }
  if (!live) return;
  const float Tk = (float)(T - w.K);
  const int v = w.idx[i];
  const float* dcf = w.dcf + (w.design ? (size_t)w.design[v] * w.P : 0);
  float bd = INFINITY;
#pragma unroll
  for (int j = 0; j < STRIP_G2; ++j) {
    float s2[2];
    unpack2(st[j], s2[0], s2[1]);
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      const int q = 2 * j + h;
      if (q < nq) {
        const float ssw = w.ssw_pre ? w.ssw_pre[(size_t)(q0 + q) * w.n + i] : s2[h];
        const float rss = fmaxf(ssw - w.proj[(size_t)(q0 + q) * w.n + i], 0.f);
        bd = fminf(bd, dcf[w.pairs[q0 + q]] + Tk * log1pf((rss - yy) / (yy + 1e-10f)));
      }
    }
  }
  if (bd < w.dbest[v] - 1e-6f * fabsf((float)w.crit0[v])) {
    w.fallback[v] = 1;
    w.best_cell[v] = -1;
  }
}

// y'R^-1 y under AFNI's banded R for the learned refine: one CTA per (tile
// of sorted rows, pair), one thread per row, the band's forward substitution
// w_t = y_t c[t][0] - sum_{j <= band} c[t][j] w_{t-j} with the last band
// values of w in a shared-memory ring and the coefficients staged per chunk
// of BS_STEPS steps (as the full grid's surface_band_kernel forms it). With
// tiles (the window rounds) CTA (x, s) takes tile x and window slot s of the
// tile's centre (no work for an empty slot or an identity pair) and writes
// out[i][s]; without them CTA (x, q) takes rows 128 x .. and pair pairs[q] and
// writes out[q][i] (row stride n).
constexpr int BS_STEPS = 32;

struct BandSumArgs {
  int n;
  const int* n_dev;        // device count of real rows (strip mode), or NULL
  int T;
  const int* idx;          // [n] voxel of each sorted row
  const float* rows;       // [V][T] residualised rows (read at idx[i])
  const float* band_coef;  // [P][T][band_w]
  int band_w;
  const int* band;         // [P]
  const int2* tiles;       // window mode: (first row, rows) per tile, *n_tiles of them
  const int* n_tiles;
  const int* center;       // [V] window centre cell
  const int* lattice;
  int n_a, n_b;
  const uint8_t* ident;    // [P] lambda == 0
  const int* pairs;        // strip mode: [n_pairs]
  float* out;
};

__global__ void __launch_bounds__(WTILE) band_sums_kernel(BandSumArgs a) {
  extern __shared__ float bsm[];
  const int W = a.band_w, T = a.T;
  int r0, nrow, p;
  if (a.tiles) {
    if ((int)blockIdx.x >= *a.n_tiles) return;
    const int2 tl = a.tiles[blockIdx.x];
    r0 = tl.x;
    nrow = tl.y;
    int a0, wa, b0, wb;
    window_of(a.center[a.idx[r0]], a.n_a, a.n_b, a0, wa, b0, wb);
    const int ra = blockIdx.y / WIN, rb = blockIdx.y % WIN;
    if (ra >= wa || rb >= wb) return;
    p = a.lattice[(a0 + ra) * a.n_b + b0 + rb];
    if (p < 0 || a.ident[p]) return;
  } else {
    const int m = a.n_dev ? min(a.n, *a.n_dev) : a.n;
    r0 = blockIdx.x * WTILE;
    if (r0 >= m) return;
    nrow = min(WTILE, m - r0);
    p = a.pairs[blockIdx.y];
  }
  float* ring = bsm;                     // [W][WTILE]
  float* cs = ring + (size_t)W * WTILE;  // [BS_STEPS][W]
  const int bw = a.band[p];
  const int tid = threadIdx.x;
  const bool live = tid < nrow;
  const int i = r0 + (live ? tid : 0);
  const float* yrow = a.rows + (size_t)a.idx[i] * T;
  const float* cb = a.band_coef + (size_t)p * T * W;
  for (int e = tid; e < W * WTILE; e += blockDim.x) ring[e] = 0.f;
  float ssw = 0.f;
  int pos = 0;
  for (int c0 = 0; c0 < T; c0 += BS_STEPS) {
    const int cn = min(BS_STEPS, T - c0);
    __syncthreads();  // the previous chunk's coefficients are no longer read
    for (int e = tid; e < cn * W; e += blockDim.x) cs[e] = cb[(size_t)c0 * W + e];
    __syncthreads();
    for (int s = 0; s < cn; ++s) {
      const int t = c0 + s;
      const float* c = cs + (size_t)s * W;
      float acc = yrow[t] * c[0];
      const int jm = min(bw, t);
      int q = pos;
      for (int j = 1; j <= jm; ++j) {
        q = q == 0 ? W - 1 : q - 1;
        acc = fmaf(-c[j], ring[(size_t)q * WTILE + tid], acc);
      }
      ring[(size_t)pos * WTILE + tid] = acc;
      pos = pos + 1 == W ? 0 : pos + 1;
      ssw = fmaf(acc, acc, ssw);
    }
  }
  if (!live) return;
  if (a.tiles)
    a.out[(size_t)i * WSLOTS + blockIdx.y] = ssw;
  else
    a.out[(size_t)blockIdx.y * a.n + i] = ssw;
}

// The voxels v < V whose pair best[v] lies within k0 lattice steps of an
// identity pair (dist[p] per pair) and that the full grid does not take
// anyway (fallback[v] == 0, when given), compacted into ids[0 .. *count) (in
// no particular order; each voxel's later results depend on it alone).
__global__ void near_line_kernel(int V, const int* best, const int* dist, int k0, const int* fallback, int* ids,
                                 int* count) {
  const int v = blockIdx.x * blockDim.x + threadIdx.x;
  const bool take = v < V && dist[best[v]] <= k0 && !(fallback && fallback[v]);
  const unsigned mk = __ballot_sync(0xffffffffu, take);
  if (!mk) return;
  const int lane = threadIdx.x & 31;
  const int first = __ffs(mk) - 1;
  int base = 0;
  if (lane == first) base = atomicAdd(count, __popc(mk));
  base = __shfl_sync(0xffffffffu, base, first);
  if (take) ids[base + __popc(mk & ((1u << lane) - 1))] = v;
}

// fp16 operand rows and exponents in the order idx: a warp per row, 16-byte words
__global__ void __launch_bounds__(256) gather_rows_kernel(int n, const int* n_dev, int ld_y, const int* __restrict__ idx,
                                                          const uint4* __restrict__ hi, const uint4* __restrict__ lo,
                                                          const int* __restrict__ yexp, uint4* __restrict__ out_hi,
                                                          uint4* __restrict__ out_lo, int* __restrict__ out_exp) {
  // one 16-byte word of one row per thread, grid-stride over rows x words:
  // consecutive threads copy consecutive words, every copy independent
  const int m = n_dev ? min(n, *n_dev) : n;
  const int nw = ld_y / 8;  // 8 fp16 per 16-byte word
  const long long total = (long long)m * nw;
  for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < total;
       e += (long long)gridDim.x * blockDim.x) {
    const int i = (int)(e / nw), k = (int)(e % nw);
    const int v = idx[i];
    const uint4 h = hi[(size_t)v * nw + k], l = lo[(size_t)v * nw + k];
    out_hi[(size_t)i * nw + k] = h;
    out_lo[(size_t)i * nw + k] = l;
    if (k == 0) out_exp[i] = yexp[v];
  }
}

// The same gathered fp16 rows formed from the fp32 rows: each thread one
// 16-byte output word (8 samples) of one row, split as the prep kernel splits
// (fp16 hi/lo of x * 2^yexp), so the prep need not store the split of every
// voxel when only the windows' rows are gathered. Samples past T are zero.
__global__ void __launch_bounds__(256) gather_split_kernel(int n, const int* n_dev, int T, int ld_y,
                                                           const int* __restrict__ idx, const float* __restrict__ rows,
                                                           const int* __restrict__ yexp, uint4* __restrict__ out_hi,
                                                           uint4* __restrict__ out_lo, int* __restrict__ out_exp) {
  const int m = n_dev ? min(n, *n_dev) : n;
  const int nw = ld_y / 8;
  const bool vec = (T & 3) == 0;
  const long long total = (long long)m * nw;
  for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < total;
       e += (long long)gridDim.x * blockDim.x) {
    const int i = (int)(e / nw), k = (int)(e % nw);
    const int v = idx[i];
    const int ex = yexp[v];
    const float* src = rows + (size_t)v * T;
    const int t0 = 8 * k;
    float x[8];
    if (vec) {
      const float4 a = t0 < T ? *reinterpret_cast<const float4*>(src + t0) : make_float4(0.f, 0.f, 0.f, 0.f);
      const float4 b = t0 + 4 < T ? *reinterpret_cast<const float4*>(src + t0 + 4) : make_float4(0.f, 0.f, 0.f, 0.f);
      x[0] = a.x; x[1] = a.y; x[2] = a.z; x[3] = a.w; x[4] = b.x; x[5] = b.y; x[6] = b.z; x[7] = b.w;
    } else {
#pragma unroll
      for (int j = 0; j < 8; ++j) x[j] = t0 + j < T ? src[t0 + j] : 0.f;
    }
    uint32_t hw[4], lw[4];
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      uint16_t h0 = 0, l0 = 0, h1 = 0, l1 = 0;
      if (t0 + 2 * j < T) split_fp16(ldexpf(x[2 * j], ex), h0, l0);
      if (t0 + 2 * j + 1 < T) split_fp16(ldexpf(x[2 * j + 1], ex), h1, l1);
      hw[j] = (uint32_t)h0 | ((uint32_t)h1 << 16);
      lw[j] = (uint32_t)l0 | ((uint32_t)l1 << 16);
    }
    out_hi[(size_t)i * nw + k] = make_uint4(hw[0], hw[1], hw[2], hw[3]);
    out_lo[(size_t)i * nw + k] = make_uint4(lw[0], lw[1], lw[2], lw[3]);
    if (k == 0) out_exp[i] = ex;
  }
}

// out_t[t][i] = rows[idx[i]][t]: 32 rows x 64 samples per CTA through shared
// memory (eight loads in flight per thread)
__global__ void gather_transpose_kernel(int n, const int* n_dev, int T, const int* __restrict__ idx,
                                        const float* __restrict__ rows, float* __restrict__ out_t) {
  __shared__ float tile[64][33];
  const int i0 = blockIdx.x * 32, t0 = blockIdx.y * 64;
  // rows taken: i < m (n stays the row stride of out_t)
  const int m = n_dev ? min(n, *n_dev) : n;
  if (i0 >= m) return;  // uniform over the CTA
  const int tx = threadIdx.x, ty = threadIdx.y;  // 32 x 8
  float x[8];
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    const int r = ty + 8 * k, i = i0 + r;
    const float* src = rows + (size_t)(i < m ? idx[i] : 0) * T;
    const int ta = t0 + tx, tb = t0 + 32 + tx;
    x[2 * k] = (i < m && ta < T) ? src[ta] : 0.f;
    x[2 * k + 1] = (i < m && tb < T) ? src[tb] : 0.f;
  }
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    const int r = ty + 8 * k;
    tile[tx][r] = x[2 * k];
    tile[32 + tx][r] = x[2 * k + 1];
  }
  __syncthreads();
#pragma unroll
  for (int k = 0; k < 8; ++k) {
    const int tt = ty + 8 * k, t = t0 + tt, i = i0 + tx;
    if (t < T && i < m) out_t[(size_t)t * n + i] = tile[tt][tx];
  }
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

}  // namespace
}  // namespace ffsk

using namespace ffsk;

extern "C" int ffs_reml_gather(int n, const int* n_dev, int T, int ld_y, const int* idx, const uint16_t* yr_hi,
                               const uint16_t* yr_lo, const int* yexp, const float* yr_rows, uint16_t* out_hi,
                               uint16_t* out_lo, int* out_exp, float* out_t, void* stream) {
  clear_error();
  FFS_REQUIRE(n > 0 && T > 0 && ld_y >= T && ld_y % 8 == 0, "ffs_reml_gather: bad sizes");
  FFS_REQUIRE(idx && yexp && out_hi && out_lo && out_exp && (!out_t || yr_rows), "ffs_reml_gather: null buffer");
  FFS_REQUIRE((yr_hi && yr_lo) || (!yr_hi && !yr_lo && yr_rows),
              "ffs_reml_gather: yr_hi and yr_lo, or (both NULL) the fp32 rows to split");
  for (const void* ptr : {(const void*)yr_hi, (const void*)yr_lo, (const void*)out_hi, (const void*)out_lo})
    FFS_REQUIRE(((uintptr_t)ptr & 15) == 0, "ffs_reml_gather: fp16 rows must be 16-byte aligned");
  FFS_REQUIRE(yr_hi || ((uintptr_t)yr_rows & 15) == 0, "ffs_reml_gather: fp32 rows must be 16-byte aligned");
  cudaStream_t st = (cudaStream_t)stream;
  int sms = 0;
  FFS_CUDA(sm_count(&sms));
  const int blocks = (int)std::min<long long>(ceil_div((long long)n * (ld_y / 8), 256), (long long)sms * 8);
  if (yr_hi) {
    gather_rows_kernel<<<blocks, 256, 0, st>>>(n, n_dev, ld_y, idx, reinterpret_cast<const uint4*>(yr_hi),
                                                        reinterpret_cast<const uint4*>(yr_lo), yexp,
                                                        reinterpret_cast<uint4*>(out_hi),
                                                        reinterpret_cast<uint4*>(out_lo), out_exp);
  } else {
    gather_split_kernel<<<blocks, 256, 0, st>>>(n, n_dev, T, ld_y, idx, yr_rows, yexp, reinterpret_cast<uint4*>(out_hi),
                                                reinterpret_cast<uint4*>(out_lo), out_exp);
  }
  if (out_t) {
    FFS_REQUIRE(ceil_div(T, 64) <= 65535, "ffs_reml_gather: T=%d too long", T);
    gather_transpose_kernel<<<dim3(ceil_div(n, 32), ceil_div(T, 64)), dim3(32, 8), 0, st>>>(n, n_dev, T, idx,
                                                                                            yr_rows, out_t);
  }
  return check_launch("gather kernels");
}

extern "C" int ffs_reml_window_items(int ncell, const int* cell_end, int n_a, int n_b, const int* lattice, int K,
                                     int max_pairs, ffs_tc_item* items, int* n_items, int max_items, int* tiles,
                                     int* n_tiles, int max_tiles, int* overflow, int P, void* stream) {
  clear_error();
  FFS_REQUIRE(ncell > 0 && n_a > 0 && n_b > 0 && K > 0 && max_pairs > 0 && max_items > 0 && max_tiles > 0 &&
                  P >= 0 && (P == 0 || ncell % (n_a * n_b) == 0),
              "ffs_reml_window_items: bad sizes");
  FFS_REQUIRE(cell_end && lattice && items && n_items && tiles && n_tiles && overflow,
              "ffs_reml_window_items: null buffer");
  cudaStream_t st = (cudaStream_t)stream;
  FFS_CUDA(cudaMemsetAsync(n_items, 0, sizeof(int), st));
  FFS_CUDA(cudaMemsetAsync(n_tiles, 0, sizeof(int), st));
  FFS_CUDA(cudaMemsetAsync(overflow, 0, sizeof(int), st));
  window_items_kernel<<<ceil_div(ncell, 128), 128, 0, st>>>(ncell, cell_end, n_a, n_b, lattice, K, max_pairs, items,
                                                             n_items, max_items, reinterpret_cast<int2*>(tiles),
                                                             n_tiles, max_tiles, overflow, P);
  clamp_count_kernel<<<1, 1, 0, st>>>(n_items, max_items, n_tiles, max_tiles);
  return check_launch("window_items_kernel");
}

extern "C" int ffs_reml_segment_items(int n_seg, const int* seg_end, int n_pairs, int K, int max_pairs,
                                      ffs_tc_item* items, int* n_items, int max_items, int* overflow, void* stream) {
  clear_error();
  FFS_REQUIRE(n_seg > 0 && n_pairs > 0 && K > 0 && max_pairs > 0 && max_pairs * K <= 256 && max_items > 0,
              "ffs_reml_segment_items: bad sizes");
  FFS_REQUIRE(seg_end && items && n_items && overflow, "ffs_reml_segment_items: null buffer");
  cudaStream_t st = (cudaStream_t)stream;
  FFS_CUDA(cudaMemsetAsync(n_items, 0, sizeof(int), st));
  FFS_CUDA(cudaMemsetAsync(overflow, 0, sizeof(int), st));
  segment_items_kernel<<<ceil_div(n_seg, 128), 128, 0, st>>>(n_seg, seg_end, n_pairs, K, max_pairs, items, n_items,
                                                              max_items, overflow);
  clamp_count_kernel<<<1, 1, 0, st>>>(n_items, max_items, n_items, max_items);
  return check_launch("segment_items_kernel");
}

extern "C" int ffs_reml_window(int n, int T, int K, int n_a, int n_b, const int* lattice, const int* idx,
                               const int* center, const int* tiles, const int* n_tiles, int max_tiles,
                               const float* rows, const float* coef, const float* winproj, const float* dcf,
                               const unsigned char* ident, int p_id, const double* c_p0, int* best, float* dbest,
                               double* crit0, int* fallback, int* best_cell, int* next_center, const int* design,
                               int P, const float* ssw_pre, void* stream) {
  clear_error();
  FFS_REQUIRE(n > 0 && T > K && K > 0 && n_a > 0 && n_b > 0 && p_id >= 0 && max_tiles > 0 && (!design || P > 0),
              "ffs_reml_window: bad sizes");
  FFS_REQUIRE(lattice && idx && center && tiles && n_tiles && rows && coef && winproj && dcf && ident && c_p0 &&
                  best && dbest && crit0 && fallback && best_cell,
              "ffs_reml_window: null buffer");
  const size_t smem = crit_smem_bytes();
  FFS_CUDA(ensure_dyn_smem(reinterpret_cast<const void*>(window_crit_kernel), smem));
  FFS_REQUIRE(((uintptr_t)rows & 15) == 0, "ffs_reml_window: rows must be 16-byte aligned");
  CritArgs w{n, T, K, n_a, n_b, lattice, idx, center, rows, reinterpret_cast<const float4*>(coef), winproj, dcf,
             ident, p_id, c_p0, best, dbest, crit0, fallback, best_cell, next_center, design, P, ssw_pre};
  window_crit_kernel<<<max_tiles, WTILE, smem, (cudaStream_t)stream>>>(w, reinterpret_cast<const int2*>(tiles),
                                                                        n_tiles);
  return check_launch("window_crit_kernel");
}

extern "C" int ffs_reml_centers(int V, const float* prop, const float* a_axis, int n_a, const float* b_axis, int n_b,
                                int* center, void* stream) {
  clear_error();
  FFS_REQUIRE(V > 0 && prop && a_axis && b_axis && center && n_a > 0 && n_b > 0, "ffs_reml_centers: bad arguments");
  center_kernel<<<ceil_div(V, 256), 256, 0, (cudaStream_t)stream>>>(V, prop, a_axis, n_a, b_axis, n_b, center);
  return check_launch("center_kernel");
}

extern "C" int ffs_reml_strip(int n, const int* n_dev, int T, int K, int n_pairs, const int* pairs, const int* idx,
                              const float* rows, const float* coef, const float* proj, const float* dcf,
                              const float* dbest, const double* crit0, int* fallback, int* best_cell,
                              const int* design, int P, const float* ssw_pre, void* stream) {
  clear_error();
  FFS_REQUIRE(!design || P > 0, "ffs_reml_strip: designs need P > 0");
  FFS_REQUIRE(n > 0 && T > K && K > 0 && n_pairs > 0 && n_pairs <= STRIP_MAX,
              "ffs_reml_strip: bad sizes (n=%d T=%d K=%d n_pairs=%d, at most %d pairs)", n, T, K, n_pairs,
              STRIP_MAX);
  FFS_REQUIRE(pairs && idx && rows && coef && proj && dcf && dbest && crit0 && fallback && best_cell,
              "ffs_reml_strip: null buffer");
  FFS_REQUIRE(((uintptr_t)rows & 15) == 0 && ((uintptr_t)coef & 15) == 0,
              "ffs_reml_strip: rows and coef must be 16-byte aligned");
  StripArgs w{n, T, K, n_pairs, n_dev, pairs, idx, rows, reinterpret_cast<const float4*>(coef), proj, dcf, dbest,
              crit0, fallback, best_cell, design, P, ssw_pre};
  const dim3 grid(ceil_div(n, STRIP_TILE), ceil_div(n_pairs, STRIP_G));
  strip_crit_kernel<<<grid, STRIP_TILE, 0, (cudaStream_t)stream>>>(w);
  return check_launch("strip_crit_kernel");
}

extern "C" int ffs_reml_band_sums(int n, const int* n_dev, int T, const int* idx, const float* rows,
                                  const float* band_coef, int band_w, const int* band, const int* tiles,
                                  const int* n_tiles, int max_tiles, const int* center, const int* lattice, int n_a,
                                  int n_b, const unsigned char* ident, const int* pairs, int n_pairs, float* out,
                                  void* stream) {
  clear_error();
  FFS_REQUIRE(n > 0 && T > 0 && band_w >= 1 && band_w <= FFS_BAND_MAX_W, "ffs_reml_band_sums: bad sizes");
  FFS_REQUIRE(idx && rows && band_coef && band && out, "ffs_reml_band_sums: null buffer");
  FFS_REQUIRE(tiles ? (n_tiles && max_tiles > 0 && center && lattice && ident && n_a > 0 && n_b > 0)
                    : (pairs && n_pairs > 0 && n_pairs <= 65535),
              "ffs_reml_band_sums: window mode needs tiles, n_tiles, centre, lattice and ident; strip mode pairs");
  const size_t smem = sizeof(float) * (size_t)band_w * (WTILE + BS_STEPS);
  FFS_CUDA(ensure_dyn_smem(reinterpret_cast<const void*>(band_sums_kernel), smem));
  BandSumArgs a{n, n_dev, T, idx, rows, band_coef, band_w, band, reinterpret_cast<const int2*>(tiles), n_tiles,
                center, lattice, n_a, n_b, ident, pairs, out};
  const dim3 grid = tiles ? dim3(max_tiles, WSLOTS) : dim3(ceil_div(n, WTILE), n_pairs);
  band_sums_kernel<<<grid, WTILE, smem, (cudaStream_t)stream>>>(a);
  return check_launch("band_sums_kernel");
}

extern "C" int ffs_reml_near_line(int V, const int* best, const int* dist, int k0, const int* fallback, int* ids,
                                  int* count, void* stream) {
  clear_error();
  FFS_REQUIRE(V > 0 && best && dist && ids && count, "ffs_reml_near_line: bad arguments");
  cudaStream_t st = (cudaStream_t)stream;
  FFS_CUDA(cudaMemsetAsync(count, 0, sizeof(int), st));
  near_line_kernel<<<ceil_div(V, 256), 256, 0, st>>>(V, best, dist, k0, fallback, ids, count);
  return check_launch("near_line_kernel");
}
