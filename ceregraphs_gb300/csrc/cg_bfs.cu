// Per-root direction-optimizing BFS: one persistent cooperative kernel that
// runs every round of a search on the device.
//
// Reference mapping (bfs/implementation/src/bool_pe.csl):
//   start_spmv (:673-729)          -> phase 0 of bfs_persistent (state reset, seed)
//   compute_topdown (:865-887)     -> push_round: frontier queue, out-lists,
//                                     atomicOr into the next-frontier bitmap
//   compute_bottomup (:899-921)    -> pull_round: unvisited vertices scan their
//                                     ascending in-lists, stop at the first
//                                     frontier source
//   reduce_or + reduce_done        -> the shared bitmaps make the OR-reduce
//     (:923-1004, collectives_2d     implicit; update_round applies
//      pe.csl:319-349)                 visited |= next, frontier = next, and the
//                                     per-round counters give nf = popcount
//   termination relay (:1003-1046)  -> every block reads nf from the round
//                                     record after a grid-wide wait; nf == 0 ends
//   direction switch (:1078-1088)   -> next_direction(): Beamer's alpha/beta rule,
//                                     or the reference's one-way tau rule
//   reduce_select_any (:1145-1154)  -> not needed: every parent is final when it
//                                     is written (lowest-index rule below)
//
// Parent rule: the lowest-numbered in-neighbour one level closer
// (bfs/README.md:208-224).  A push round applies atomicMin over every
// frontier source of a newly reached vertex (the visited bitmap is frozen
// during the round, so all of them are seen); a pull round takes the first
// frontier source of an ascending in-list, which is the minimum.  Parents
// start at 0xFFFFFFFF, the reference's PARENT_NONE (device_io.py:157), which
// reads back as -1 through int32 without a conversion pass.
#include <cuda_runtime.h>

#include "cg_internal.cuh"

namespace cg {

constexpr unsigned kFull = 0xffffffffu;
constexpr int kPush = 0, kPull = 1;
constexpr int kBfsBlock = 512;
// In-degree above which a pull-round in-list is scanned by a whole warp.
constexpr int kPullLight = 32;

struct Acc {
  unsigned long long nf = 0, mf = 0, visdeg = 0;
};

// Pushes the discoveries of one warp-wide step into the next frontier's queue
// (light: front, medium: back, heavy: separate list).  All 32 lanes call it.
__device__ __forceinline__ void enqueue_claims(const BfsParams &p, bool claimed, int32_t v,
                                               int64_t deg, int next_parity, RoundRec *Rn,
                                               Acc &acc) {
  const int lane = lane_id();
  unsigned any = __ballot_sync(kFull, claimed);
  if (!any) return;
  int cls = !claimed ? -1 : (deg <= kLightMax ? 0 : (deg <= kMediumMax ? 1 : 2));
  int32_t *q = next_parity ? p.queue1 : p.queue0;
  int32_t *h = next_parity ? p.heavy1 : p.heavy0;
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    unsigned m = __ballot_sync(kFull, cls == c);
    if (!m) continue;
    int leader = __ffs(m) - 1;
    unsigned base = 0;
    if (lane == leader) {
      unsigned *ctr = c == 0 ? &Rn->nlight : (c == 1 ? &Rn->nmedium : &Rn->nheavy);
      base = atomicAdd(ctr, (unsigned)__popc(m));
    }
    base = __shfl_sync(kFull, base, leader);
    if (cls == c) {
      unsigned pos = base + __popc(m & ((1u << lane) - 1u));
      if (c == 0)
        q[pos] = v;
      else if (c == 1)
        q[p.n - 1 - (int64_t)pos] = v;
      else
        h[pos] = v;
    }
  }
  if (claimed) {
    acc.nf += 1;
    acc.mf += (unsigned long long)deg;
    acc.visdeg += (unsigned long long)deg;
  }
}

// Edge u -> v of a push round.  Returns true for the one thread that claims v.
__device__ __forceinline__ bool relax_push(const BfsParams &p, int32_t u, int32_t v,
                                           int next_level) {
  const uint32_t w = (uint32_t)v >> 5, bit = 1u << (v & 31);
  if (p.vis[w] & bit) return false;
  atomicMin(reinterpret_cast<unsigned *>(p.parents) + v, (unsigned)u);
  if (p.nxt[w] & bit) return false;
  unsigned old = atomicOr(p.nxt + w, bit);
  if (old & bit) return false;
  p.levels[v] = next_level;
  return true;
}

__device__ __forceinline__ void push_step(const BfsParams &p, bool valid, int32_t u, int64_t e,
                                          int L, int next_parity, RoundRec *Rn, Acc &acc) {
  bool claimed = false;
  int32_t v = 0;
  int64_t deg = 0;
  if (valid) {
    v = __ldg(p.out_idx + e);
    claimed = relax_push(p, u, v, L + 1);
    if (claimed) deg = __ldg(p.out_off + v + 1) - __ldg(p.out_off + v);
  }
  enqueue_claims(p, claimed, v, deg, next_parity, Rn, acc);
}

// Expands frontier F_L (queue parity L & 1) top-down.
__device__ void push_round(const BfsParams &p, int L, RoundRec *Rc, RoundRec *Rn, Acc &acc) {
  __shared__ int32_t s_u[kBfsBlock / 32][32];
  __shared__ int64_t s_s[kBfsBlock / 32][32];
  __shared__ int32_t s_x[kBfsBlock / 32][32];
  const int lane = lane_id();
  const int wib = threadIdx.x >> 5;
  const int gw = warp_id_global();
  const int nwarps = (gridDim.x * blockDim.x) >> 5;
  const int parity = L & 1, next_parity = parity ^ 1;
  const int32_t *q = parity ? p.queue1 : p.queue0;
  const int32_t *h = parity ? p.heavy1 : p.heavy0;

  // heavy vertices: each adjacency list is split over every warp of the grid
  const unsigned nheavy = *(volatile unsigned *)&Rc->nheavy;
  for (unsigned b = 0; b < nheavy; ++b) {
    const int32_t u = h[b];
    const int64_t s = __ldg(p.out_off + u), e = __ldg(p.out_off + u + 1);
    for (int64_t base = s + (int64_t)gw * 32; base < e; base += (int64_t)nwarps * 32) {
      const int64_t i = base + lane;
      push_step(p, i < e, u, i, L, next_parity, Rn, acc);
    }
  }

  // medium vertices (one warp each), then light vertices 32 to a warp with the
  // warp's combined edge list spread evenly over its lanes
  const unsigned nmed = *(volatile unsigned *)&Rc->nmedium;
  const unsigned nlight = *(volatile unsigned *)&Rc->nlight;
  const unsigned nitems = nmed + (nlight + 31u) / 32u;
  while (true) {
    unsigned item = 0;
    if (lane == 0) item = atomicAdd(&Rc->work, 1u);
    item = __shfl_sync(kFull, item, 0);
    if (item >= nitems) break;
    if (item < nmed) {
      const int32_t u = q[p.n - 1 - (int64_t)item];
      const int64_t s = __ldg(p.out_off + u), e = __ldg(p.out_off + u + 1);
      for (int64_t base = s; base < e; base += 32) {
        const int64_t i = base + lane;
        push_step(p, i < e, u, i, L, next_parity, Rn, acc);
      }
    } else {
      const unsigned idx = (item - nmed) * 32u + lane;
      int32_t u = 0;
      int64_t s = 0;
      int d = 0;
      if (idx < nlight) {
        u = q[idx];
        s = __ldg(p.out_off + u);
        d = (int)(__ldg(p.out_off + u + 1) - s);
      }
      int incl = d;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        int t = __shfl_up_sync(kFull, incl, o);
        if (lane >= o) incl += t;
      }
      const int total = __shfl_sync(kFull, incl, 31);
      s_u[wib][lane] = u;
      s_s[wib][lane] = s;
      s_x[wib][lane] = incl - d;
      __syncwarp();
      for (int base = 0; base < total; base += 32) {
        const int t = base + lane;
        bool valid = t < total;
        int32_t uu = 0;
        int64_t e = 0;
        if (valid) {
          int lo = 0, hi = 31;
          while (lo < hi) {
            int mid = (lo + hi + 1) >> 1;
            if (s_x[wib][mid] <= t)
              lo = mid;
            else
              hi = mid - 1;
          }
          uu = s_u[wib][lo];
          e = s_s[wib][lo] + (t - s_x[wib][lo]);
        }
        push_step(p, valid, uu, e, L, next_parity, Rn, acc);
      }
      __syncwarp();
    }
  }
}

// Bottom-up round: every unvisited vertex scans its ascending in-list and
// stops at the first source in frontier F_L.  One warp owns one bitmap word,
// so the next-frontier word is written whole, without atomics.
__device__ void pull_round(const BfsParams &p, int L, Acc &acc) {
  const int lane = lane_id();
  const int gw = warp_id_global();
  const int nwarps = (gridDim.x * blockDim.x) >> 5;
  for (int64_t w = gw; w < p.words; w += nwarps) {
    const uint32_t vw = p.vis[w];
    const int64_t v = w * 32 + lane;
    const bool active = v < p.n && !((vw >> lane) & 1u);
    if (__ballot_sync(kFull, active) == 0) continue;
    bool found = false;
    int64_t s = 0, e = 0;
    if (active) {
      s = __ldg(p.in_off + v);
      e = __ldg(p.in_off + v + 1);
    }
    const bool heavy = active && (e - s) > kPullLight;
    if (active && !heavy) {
      for (int64_t i = s; i < e; ++i) {
        const int32_t u = __ldg(p.in_idx + i);
        if ((p.cur[(uint32_t)u >> 5] >> (u & 31)) & 1u) {
          p.parents[v] = u;
          p.levels[v] = L + 1;
          found = true;
          break;
        }
      }
    }
    // long in-lists: the whole warp scans one at a time, 32 sources per step;
    // the lowest lane with a frontier source holds the smallest one
    unsigned hm = __ballot_sync(kFull, heavy);
    while (hm) {
      const int j = __ffs(hm) - 1;
      hm &= hm - 1;
      const int64_t sj = __shfl_sync(kFull, s, j), ej = __shfl_sync(kFull, e, j);
      const int64_t vj = w * 32 + j;
      for (int64_t base = sj; base < ej; base += 32) {
        const int64_t i = base + lane;
        int32_t u = 0;
        bool hit = false;
        if (i < ej) {
          u = __ldg(p.in_idx + i);
          hit = (p.cur[(uint32_t)u >> 5] >> (u & 31)) & 1u;
        }
        const unsigned who = __ballot_sync(kFull, hit);
        if (who) {
          if (lane == __ffs(who) - 1) {
            p.parents[vj] = u;
            p.levels[vj] = L + 1;
          }
          if (lane == j) found = true;
          break;
        }
      }
    }
    const unsigned m = __ballot_sync(kFull, found);
    if (lane == 0 && m) p.nxt[w] = m;
    if (found) {
      acc.nf += 1;
      acc.visdeg += (unsigned long long)(e - s);
    }
  }
}

// visited |= next; frontier = next; next = 0.  When the next round pushes
// after a pull round, the new frontier's queue is built here as well.
__device__ void update_round(const BfsParams &p, int L, bool build_queue, RoundRec *Rn,
                             Acc &acc) {
  const int lane = lane_id();
  const int gw = warp_id_global();
  const int nwarps = (gridDim.x * blockDim.x) >> 5;
  const int next_parity = (L + 1) & 1;
  for (int64_t w0 = (int64_t)gw * 32; w0 < p.words; w0 += (int64_t)nwarps * 32) {
    const int64_t w = w0 + lane;
    uint32_t bits = 0;
    if (w < p.words) {
      bits = p.nxt[w];
      if (bits) {
        p.vis[w] |= bits;
        p.nxt[w] = 0;
      }
      p.cur[w] = bits;
    }
    if (build_queue) {
      uint32_t rest = bits;
      while (__ballot_sync(kFull, rest != 0)) {
        bool claimed = rest != 0;
        int32_t v = 0;
        int64_t deg = 0;
        if (claimed) {
          const int b = __ffs(rest) - 1;
          rest &= rest - 1u;
          v = (int32_t)(w * 32 + b);
          deg = __ldg(p.out_off + v + 1) - __ldg(p.out_off + v);
        }
        Acc scratch;  // counts of this frontier were taken in the pull round
        enqueue_claims(p, claimed, v, deg, next_parity, Rn, scratch);
      }
    }
  }
  (void)acc;
}

__device__ __forceinline__ unsigned long long warp_sum(unsigned long long x) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(kFull, x, o);
  return x;
}

// Adds the block's per-thread counters into round record Rn (one atomic per
// counter per block, skipped when zero).
__device__ void flush_acc(Acc &acc, RoundRec *Rn) {
  __shared__ unsigned long long s_red[3][kBfsBlock / 32];
  const int lane = lane_id(), wib = threadIdx.x >> 5;
  unsigned long long a = warp_sum(acc.nf), b = warp_sum(acc.mf), c = warp_sum(acc.visdeg);
  if (lane == 0) {
    s_red[0][wib] = a;
    s_red[1][wib] = b;
    s_red[2][wib] = c;
  }
  __syncthreads();
  if (wib == 0) {
    const int nw = blockDim.x >> 5;
    a = lane < nw ? s_red[0][lane] : 0ull;
    b = lane < nw ? s_red[1][lane] : 0ull;
    c = lane < nw ? s_red[2][lane] : 0ull;
    a = warp_sum(a);
    b = warp_sum(b);
    c = warp_sum(c);
    if (lane == 0) {
      if (a) atomicAdd(&Rn->nf, a);
      if (b) atomicAdd(&Rn->mf, b);
      if (c) atomicAdd(&Rn->visdeg, c);
    }
  }
  acc = Acc();
}

__device__ __forceinline__ int next_direction(const BfsParams &p, int dir, unsigned long long nf,
                                              unsigned long long prev_nf,
                                              unsigned long long mf,
                                              unsigned long long explored) {
  switch (p.direction) {
    case CG_DIR_TOPDOWN:
      return kPush;
    case CG_DIR_BOTTOMUP:
      return kPull;
    case CG_DIR_TAU:
      // bool_pe.csl:1078-1088: one way only, once nf exceeds tau
      return (dir == kPull || (long long)nf > p.tau) ? kPull : kPush;
    default: {
      if (dir == kPush) {
        const double unexplored = (double)p.nnz - (double)explored;
        return ((double)mf > unexplored / (double)p.alpha) ? kPull : kPush;
      }
      const bool shrinking = nf < prev_nf;
      return (shrinking && (double)nf < (double)p.n / (double)p.beta) ? kPush : kPull;
    }
  }
}

__global__ void __launch_bounds__(kBfsBlock) bfs_persistent(BfsParams p) {
  BfsCtl *ctl = p.ctl;
  const int64_t gtid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t nthreads = (int64_t)gridDim.x * blockDim.x;
  const int32_t root = (int32_t)p.root;
  const bool leader = blockIdx.x == 0 && threadIdx.x == 0;
  const long long t_start = leader ? global_ns() : 0;

  // ---- phase 0: start_spmv -- reset outputs and bitmaps, seed the root ----
  for (int64_t i = gtid; i < p.n; i += nthreads) {
    p.levels[i] = (i == root) ? 0 : -1;
    p.parents[i] = (i == root) ? root : -1;
  }
  for (int64_t w = gtid; w < p.words; w += nthreads) {
    const uint32_t bit = (w == (root >> 5)) ? (1u << (root & 31)) : 0u;
    p.vis[w] = bit;
    p.cur[w] = bit;
    p.nxt[w] = 0;
  }
  if (leader) {
    const int64_t deg = p.out_off[root + 1] - p.out_off[root];
    RoundRec *R0 = &ctl->rec[0];
    R0->nf = 1;
    R0->mf = deg;
    R0->visdeg = deg;
    if (deg <= kLightMax) {
      p.queue0[0] = root;
      R0->nlight = 1;
    } else if (deg <= kMediumMax) {
      p.queue0[p.n - 1] = root;
      R0->nmedium = 1;
    } else {
      p.heavy0[0] = root;
      R0->nheavy = 1;
    }
  }
  bool ok = grid_wait(&ctl->wait, &ctl->status, p.timeout_ns, p.unmatched_wait ? 1u : 0u);

  int dir = kPush;
  int L = 0;
  int pull_rounds = 0, switches = 0;
  unsigned long long prev_nf = 1, visited = 1;
  unsigned long long explored = (unsigned long long)(p.out_off[root + 1] - p.out_off[root]);
  Acc acc;
  long long t_round = leader ? global_ns() : 0;
  if (leader) p.stats->setup_ns = t_round - t_start;
  while (ok) {
    RoundRec *Rc = &ctl->rec[L % kRing];
    RoundRec *Rn = &ctl->rec[(L + 1) % kRing];
    if (leader && L > 0 && L - 1 < CG_HISTORY) {
      const long long now = global_ns();
      p.stats->round_ns[L - 1] = now - t_round;
      t_round = now;
    }
    if (dir == kPush)
      push_round(p, L, Rc, Rn, acc);
    else
      pull_round(p, L, acc);
    flush_acc(acc, Rn);
    if (!(ok = grid_wait(&ctl->wait, &ctl->status, p.timeout_ns))) break;

    const unsigned long long nf = *(volatile unsigned long long *)&Rn->nf;
    const unsigned long long mf = *(volatile unsigned long long *)&Rn->mf;
    const unsigned long long vd = *(volatile unsigned long long *)&Rn->visdeg;
    if (leader && L < CG_HISTORY) {
      p.stats->nf_history[L] = (int64_t)nf;
      p.stats->direction_history[L] = dir;
    }
    if (dir == kPull) ++pull_rounds;
    visited += nf;
    if (nf == 0) {
      L += 1;
      break;
    }
    if (L + 1 >= p.level_cap) {
      if (leader) atomicCAS(&ctl->status, 0, (int)CG_ERR_LEVEL_CAP);
      L += 1;
      ok = false;
      break;
    }
    const int next = next_direction(p, dir, nf, prev_nf, mf, explored);
    explored += vd;
    update_round(p, L, next == kPush && dir == kPull, Rn, acc);
    if (leader) {
      RoundRec *Rz = &ctl->rec[(L + 2) % kRing];
      Rz->nf = Rz->mf = Rz->visdeg = 0;
      Rz->nlight = Rz->nmedium = Rz->nheavy = Rz->work = 0;
    }
    if (!(ok = grid_wait(&ctl->wait, &ctl->status, p.timeout_ns))) break;
    if (next != dir) ++switches;
    prev_nf = nf;
    dir = next;
    ++L;
  }
  if (leader) {
    cg_stats *st = p.stats;
    if (L > 0 && L - 1 < CG_HISTORY) st->round_ns[L - 1] = global_ns() - t_round;
    st->finish_ns = 0;
    st->status = *(volatile int *)&ctl->status;
    st->rounds = L;
    st->visited = (int64_t)visited;
    st->pull_rounds = pull_rounds;
    st->switches = switches;
    st->history_len = L < CG_HISTORY ? L : CG_HISTORY;
    st->device_ms = 0.f;
  }
}

// Graph500 m per search (bfs_timing.py:379-398), lane = blockIdx.y.
__global__ void count_edges_kernel(int64_t n, int symmetric, const int64_t *__restrict__ in_off,
                                   const int32_t *__restrict__ in_idx,
                                   const int64_t *__restrict__ out_off,
                                   const int32_t *__restrict__ levels,
                                   unsigned long long *m_out) {
  const int64_t lane_base = (int64_t)blockIdx.y * n;
  unsigned long long local = 0;
  for (int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; v < n;
       v += (int64_t)gridDim.x * blockDim.x) {
    if (levels[lane_base + v] < 0) continue;
    if (symmetric) {
      // row v of A is ascending: count its entries c <= v (binary search)
      int64_t lo = in_off[v], hi = in_off[v + 1];
      while (lo < hi) {
        const int64_t mid = (lo + hi) >> 1;
        if (in_idx[mid] <= v)
          lo = mid + 1;
        else
          hi = mid;
      }
      local += (unsigned long long)(lo - in_off[v]);
    } else {
      local += (unsigned long long)(out_off[v + 1] - out_off[v]);
    }
  }
  local = warp_sum(local);
  if ((threadIdx.x & 31) == 0 && local) atomicAdd(m_out + blockIdx.y, local);
}

int bfs_prepare(cg_graph *g) {
  if (g->bitmaps) return CG_OK;
  int dev_coop = 0;
  CG_CUDA(cudaDeviceGetAttribute(&dev_coop, cudaDevAttrCooperativeLaunch, g->device));
  if (!dev_coop) return CG_ERR_NOT_SUPPORTED;
  g->words = (g->n + 31) / 32;
  g->hcap = g->nnz / (kMediumMax + 1) + 1;
  if (g->hcap > g->n) g->hcap = g->n;
  size_t bytes_bm = sizeof(uint32_t) * 3 * (size_t)g->words;
  size_t bytes_q = sizeof(int32_t) * 2 * (size_t)g->n;
  size_t bytes_h = sizeof(int32_t) * 2 * (size_t)g->hcap;
  if (cudaMalloc(&g->bitmaps, bytes_bm) != cudaSuccess) return CG_ERR_OUT_OF_MEMORY;
  if (cudaMalloc(&g->queue, bytes_q) != cudaSuccess) return CG_ERR_OUT_OF_MEMORY;
  if (cudaMalloc(&g->heavy, bytes_h) != cudaSuccess) return CG_ERR_OUT_OF_MEMORY;
  if (cudaMalloc(&g->ctl, sizeof(BfsCtl)) != cudaSuccess) return CG_ERR_OUT_OF_MEMORY;
  if (cudaMalloc(&g->d_stats, sizeof(cg_stats)) != cudaSuccess) return CG_ERR_OUT_OF_MEMORY;
  g->device_bytes += bytes_bm + bytes_q + bytes_h + sizeof(BfsCtl) + sizeof(cg_stats);
  CG_CUDA(cudaMemsetAsync(g->ctl, 0, sizeof(BfsCtl), g->stream));
  CG_CUDA(cudaMemsetAsync(g->d_stats, 0, sizeof(cg_stats), g->stream));
  return CG_OK;
}

static int bfs_grid(cg_graph *g) {
  int block = g->opt.block_size > 0 ? g->opt.block_size : kBfsBlock;
  if (block > kBfsBlock) block = kBfsBlock;
  block = (block / 32) * 32;
  if (block < 64) block = 64;
  int per_sm = 0;
  CG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, bfs_persistent, block, 0));
  if (per_sm <= 0) return CG_ERR_NOT_SUPPORTED;
  if (g->opt.blocks_per_sm > 0 && g->opt.blocks_per_sm < per_sm) per_sm = g->opt.blocks_per_sm;
  g->bfs_grid = per_sm * g->num_sms;
  g->bfs_block = block;
  return CG_OK;
}

int bfs_launch(cg_graph *g, int64_t root, int32_t *d_levels, int32_t *d_parents) {
  int rc = bfs_prepare(g);
  if (rc) return rc;
  if ((rc = bfs_grid(g))) return rc;
  BfsParams p;
  p.n = g->n;
  p.nnz = g->nnz;
  p.words = g->words;
  p.in_off = g->in_off;
  p.in_idx = g->in_idx;
  p.out_off = g->out_off;
  p.out_idx = g->out_idx;
  p.vis = g->bitmaps;
  p.cur = g->bitmaps + g->words;
  p.nxt = g->bitmaps + 2 * g->words;
  p.queue0 = g->queue;
  p.queue1 = g->queue + g->n;
  p.heavy0 = g->heavy;
  p.heavy1 = g->heavy + g->hcap;
  p.levels = d_levels;
  p.parents = d_parents;
  p.ctl = g->ctl;
  p.stats = g->d_stats;
  p.root = root;
  p.direction = g->opt.direction;
  p.alpha = g->opt.alpha > 0 ? g->opt.alpha : 15.f;
  p.beta = g->opt.beta > 0 ? g->opt.beta : 18.f;
  p.tau = g->opt.tau_switch_count;
  p.level_cap = g->opt.level_cap > 0 ? g->opt.level_cap
                                     : (int)((g->n + 1) < 0x7fffffff ? g->n + 1 : 0x7fffffff);
  p.timeout_ns = (long long)(g->opt.wait_timeout_ms > 0 ? g->opt.wait_timeout_ms : 1000) * 1000000ll;
  p.unmatched_wait = g->opt.test_unmatched_wait;
  // every launch starts from a clean control block (round records, wait counter)
  CG_CUDA(cudaMemsetAsync(g->ctl, 0, sizeof(BfsCtl), g->stream));
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(g->bfs_grid);
  cfg.blockDim = dim3(g->bfs_block);
  cfg.dynamicSmemBytes = 0;
  cfg.stream = g->stream;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeCooperative;  // all blocks co-resident (grid waits)
  attr[0].val.cooperative = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  CG_CUDA(cudaLaunchKernelEx(&cfg, bfs_persistent, p));
  return CG_OK;
}

int count_edges_launch(cg_graph *g, const int32_t *d_levels, int32_t k,
                       unsigned long long *d_m) {
  CG_CUDA(cudaMemsetAsync(d_m, 0, sizeof(unsigned long long) * (size_t)k, g->stream));
  int blocks = (int)((g->n + 255) / 256);
  const int cap = g->num_sms * 8;
  if (blocks > cap) blocks = cap;
  if (blocks < 1) blocks = 1;
  count_edges_kernel<<<dim3(blocks, k), 256, 0, g->stream>>>(
      g->n, g->symmetric ? 1 : 0, g->in_off, g->in_idx, g->out_off, d_levels, d_m);
  CG_CUDA(cudaGetLastError());
  return CG_OK;
}

}  // namespace cg
