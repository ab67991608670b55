// Multi-source BFS: up to 64 * W searches advance together, one bit lane per
// search in a W-word mask per vertex -- a boolean SpMM, Y = A (AND, OR) X with
// X the n x (64 W) frontier bit matrix, iterated round by round in one
// persistent cooperative launch.
//
// There is no batched kernel in the reference (its f_spmv_iter, bool_pe.csl
// :742-1161, runs one root per launch and run_graph500.py:321-440 loops over
// roots on the host); every lane here reproduces that single-root search
// exactly: level = round of first discovery, parent = lowest-numbered
// in-neighbour one level closer (bfs/README.md:208-224), -1 when unreached.
//
// State per vertex (HBM, W uint64 words each):
//   vis          lanes that have reached the vertex
//   fr[3]        frontier masks: round L reads fr[L % 3] (F_L), writes
//                fr[(L+1) % 3] (F_{L+1}) and clears fr[(L+2) % 3] (F_{L-1})
//   touched[2]   1 bit per vertex: "already queued this round" (push rounds)
//   queue[2]     vertex queues of the frontier (any lane set), light from the
//                front, medium from the back; heavy[2] for grid-split lists
//
// Pull round: every vertex with unvisited lanes scans its ascending in-list
// and takes, per lane, the first frontier source (the minimum); it stops once
// every wanted lane is found.  Push round: frontier vertices OR their masks
// into their out-neighbours' next masks (atomicOr), then a resolve phase
// scans each newly reached vertex's ascending in-list for its parents -- no
// atomics on the per-lane parent arrays in either direction.
#include <cuda_runtime.h>

#include "cg_internal.cuh"

namespace cg {

constexpr unsigned kMsFull = 0xffffffffu;
constexpr int kMsBlock = 512;
constexpr int kMsMaxLanes = 128;

struct MsRound {
  unsigned long long nf;      // vertices with a nonzero frontier mask
  unsigned long long visits;  // lane discoveries
  unsigned long long mf;      // sum of out-degrees over the frontier vertices
  unsigned int nlight, nmedium, nheavy, work;
  unsigned long long lanes[2];  // lanes whose frontier is non-empty
  unsigned long long pad;
};

// In-degree above which a vertex's in-list is scanned by a whole warp.
constexpr int kPullLight = 32;

struct MsCtl {
  GridWait wait;
  int status;
  int pad[31];
  MsRound rec[kRing];
};

struct MsParams {
  int64_t n, nnz, words;
  const int64_t *__restrict__ in_off;
  const int32_t *__restrict__ in_idx;
  const int64_t *__restrict__ out_off;
  const int32_t *__restrict__ out_idx;
  uint64_t *vis, *fr0, *fr1, *fr2;
  uint32_t *touched0, *touched1;
  int32_t *queue0, *queue1, *heavy0, *heavy1;
  int32_t *levels, *parents;  // root-major, k x n
  MsCtl *ctl;
  cg_stats *stats;
  int k;
  int direction;
  float ms_alpha;
  int level_cap;
  long long timeout_ns;
  int32_t roots[kMsMaxLanes];
};

template <int W>
struct Mask {
  uint64_t w[W];
  __device__ __forceinline__ static Mask zero() {
    Mask m;
#pragma unroll
    for (int i = 0; i < W; ++i) m.w[i] = 0;
    return m;
  }
  __device__ __forceinline__ bool any() const {
    uint64_t a = 0;
#pragma unroll
    for (int i = 0; i < W; ++i) a |= w[i];
    return a != 0;
  }
  __device__ __forceinline__ int popc() const {
    int c = 0;
#pragma unroll
    for (int i = 0; i < W; ++i) c += __popcll(w[i]);
    return c;
  }
  __device__ __forceinline__ Mask operator&(const Mask &o) const {
    Mask m;
#pragma unroll
    for (int i = 0; i < W; ++i) m.w[i] = w[i] & o.w[i];
    return m;
  }
  __device__ __forceinline__ Mask operator|(const Mask &o) const {
    Mask m;
#pragma unroll
    for (int i = 0; i < W; ++i) m.w[i] = w[i] | o.w[i];
    return m;
  }
  __device__ __forceinline__ Mask andnot(const Mask &o) const {  // this & ~o
    Mask m;
#pragma unroll
    for (int i = 0; i < W; ++i) m.w[i] = w[i] & ~o.w[i];
    return m;
  }
  __device__ __forceinline__ bool operator==(const Mask &o) const {
    bool e = true;
#pragma unroll
    for (int i = 0; i < W; ++i) e = e && (w[i] == o.w[i]);
    return e;
  }
};

template <int W>
__device__ __forceinline__ Mask<W> ld_mask(const uint64_t *base, int64_t v) {
  Mask<W> m;
  if (W == 2) {
    const ulonglong2 x = *reinterpret_cast<const ulonglong2 *>(base + v * 2);
    m.w[0] = x.x;
    m.w[W - 1] = x.y;
  } else {
#pragma unroll
    for (int i = 0; i < W; ++i) m.w[i] = base[v * W + i];
  }
  return m;
}

template <int W>
__device__ __forceinline__ void st_mask(uint64_t *base, int64_t v, const Mask<W> &m) {
  if (W == 2) {
    *reinterpret_cast<ulonglong2 *>(base + v * 2) = make_ulonglong2(m.w[0], m.w[W - 1]);
  } else {
#pragma unroll
    for (int i = 0; i < W; ++i) base[v * W + i] = m.w[i];
  }
}

template <int W>
__device__ __forceinline__ Mask<W> lane_mask(int k) {
  Mask<W> m;
#pragma unroll
  for (int i = 0; i < W; ++i) {
    const int lo = i * 64;
    m.w[i] = k >= lo + 64 ? ~0ull : (k <= lo ? 0ull : ((1ull << (k - lo)) - 1ull));
  }
  return m;
}

// Writes level and parent of vertex v for every lane in `m`.
template <int W>
__device__ __forceinline__ void write_lanes(const MsParams &p, int64_t v, const Mask<W> &m,
                                            int32_t parent, int level) {
#pragma unroll
  for (int i = 0; i < W; ++i) {
    uint64_t bits = m.w[i];
    while (bits) {
      const int b = __ffsll((long long)bits) - 1;
      bits &= bits - 1;
      const int64_t at = (int64_t)(i * 64 + b) * p.n + v;
      p.levels[at] = level;
      p.parents[at] = parent;
    }
  }
}

struct MsAcc {
  unsigned long long nf = 0, visits = 0, mf = 0;
  unsigned long long lanes[2] = {0ull, 0ull};
};

// Appends claimed vertices to the next frontier's queue (all lanes call).
__device__ __forceinline__ void ms_enqueue(const MsParams &p, bool claimed, int32_t v,
                                           int64_t deg, int next_parity, MsRound *Rn,
                                           MsAcc &acc) {
  const int lane = lane_id();
  if (!__ballot_sync(kMsFull, claimed)) return;
  const int cls = !claimed ? -1 : (deg <= kLightMax ? 0 : (deg <= kMediumMax ? 1 : 2));
  int32_t *q = next_parity ? p.queue1 : p.queue0;
  int32_t *h = next_parity ? p.heavy1 : p.heavy0;
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    const unsigned m = __ballot_sync(kMsFull, cls == c);
    if (!m) continue;
    const int leader = __ffs(m) - 1;
    unsigned base = 0;
    if (lane == leader) {
      unsigned *ctr = c == 0 ? &Rn->nlight : (c == 1 ? &Rn->nmedium : &Rn->nheavy);
      base = atomicAdd(ctr, (unsigned)__popc(m));
    }
    base = __shfl_sync(kMsFull, base, leader);
    if (cls == c) {
      const unsigned pos = base + __popc(m & ((1u << lane) - 1u));
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
  }
}

__device__ __forceinline__ unsigned long long ms_warp_sum(unsigned long long x) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(kMsFull, x, o);
  return x;
}

__device__ void ms_flush(MsAcc &acc, MsRound *Rn) {
  __shared__ unsigned long long s_red[3][kMsBlock / 32];
  __shared__ unsigned long long s_lanes[2];
  const int lane = lane_id(), wib = threadIdx.x >> 5;
  if (threadIdx.x < 2) s_lanes[threadIdx.x] = 0ull;
  unsigned long long a = ms_warp_sum(acc.nf), b = ms_warp_sum(acc.visits),
                     c = ms_warp_sum(acc.mf);
  unsigned long long l0 = acc.lanes[0], l1 = acc.lanes[1];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    l0 |= __shfl_xor_sync(kMsFull, l0, o);
    l1 |= __shfl_xor_sync(kMsFull, l1, o);
  }
  if (lane == 0) {
    s_red[0][wib] = a;
    s_red[1][wib] = b;
    s_red[2][wib] = c;
  }
  __syncthreads();
  if (lane == 0) {
    if (l0) atomicOr(&s_lanes[0], l0);
    if (l1) atomicOr(&s_lanes[1], l1);
  }
  __syncthreads();
  if (wib == 0) {
    const int nw = blockDim.x >> 5;
    a = ms_warp_sum(lane < nw ? s_red[0][lane] : 0ull);
    b = ms_warp_sum(lane < nw ? s_red[1][lane] : 0ull);
    c = ms_warp_sum(lane < nw ? s_red[2][lane] : 0ull);
    if (lane == 0) {
      if (a) atomicAdd(&Rn->nf, a);
      if (b) atomicAdd(&Rn->visits, b);
      if (c) atomicAdd(&Rn->mf, c);
      if (s_lanes[0]) atomicOr(&Rn->lanes[0], s_lanes[0]);
      if (s_lanes[1]) atomicOr(&Rn->lanes[1], s_lanes[1]);
    }
  }
  __syncthreads();
  acc = MsAcc();
}

template <int W>
__device__ __forceinline__ void acc_lanes(MsAcc &acc, const Mask<W> &m) {
#pragma unroll
  for (int i = 0; i < W; ++i) acc.lanes[i] |= m.w[i];
}

// Warp-cooperative scan of vertex v's ascending in-list (all 32 lanes call
// with the same v and want): 32 sources per step; for each lane bit found in
// a step, the lowest warp lane holding it -- the smallest source -- is the
// parent.  Stops once every wanted bit is found.  Returns the found bits.
template <int W>
__device__ Mask<W> warp_scan_in_list(const MsParams &p, int64_t v, const Mask<W> &want,
                                     const uint64_t *cur, int level) {
  const int lane = lane_id();
  Mask<W> got = Mask<W>::zero();
  const int64_t s = __ldg(p.in_off + v), e = __ldg(p.in_off + v + 1);
  for (int64_t base = s; base < e; base += 32) {
    const int64_t i = base + lane;
    Mask<W> f = Mask<W>::zero();
    int32_t u = 0;
    if (i < e) {
      u = __ldg(p.in_idx + i);
      f = (ld_mask<W>(cur, u) & want).andnot(got);
    }
    Mask<W> F = f;
#pragma unroll
    for (int j = 0; j < W; ++j)
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) F.w[j] |= __shfl_xor_sync(kMsFull, F.w[j], o);
    if (F.any()) {
#pragma unroll
      for (int j = 0; j < W; ++j) {
        uint64_t bits = F.w[j];
        while (bits) {
          const int b = __ffsll((long long)bits) - 1;
          bits &= bits - 1;
          const unsigned who = __ballot_sync(kMsFull, (f.w[j] >> b) & 1ull);
          if (lane == __ffs(who) - 1) {
            const int64_t at = (int64_t)(j * 64 + b) * p.n + v;
            p.levels[at] = level;
            p.parents[at] = u;
          }
        }
      }
      got = got | F;
      if (got == want) break;
    }
  }
  return got;
}

// Thread-level scan of the same kind, for short in-lists.
template <int W>
__device__ __forceinline__ Mask<W> thread_scan_in_list(const MsParams &p, int64_t v,
                                                       const Mask<W> &want,
                                                       const uint64_t *cur, int level) {
  Mask<W> got = Mask<W>::zero();
  const int64_t s = __ldg(p.in_off + v), e = __ldg(p.in_off + v + 1);
  for (int64_t i = s; i < e; ++i) {
    const int32_t u = __ldg(p.in_idx + i);
    const Mask<W> f = (ld_mask<W>(cur, u) & want).andnot(got);
    if (f.any()) {
      write_lanes<W>(p, v, f, u, level);
      got = got | f;
      if (got == want) break;
    }
  }
  return got;
}

// Scans a warp's 32 vertices: short lists one per thread, long ones by the
// whole warp in turn.  want must be zero for vertices that need no scan.
template <int W>
__device__ __forceinline__ Mask<W> scan_group(const MsParams &p, int64_t v, const Mask<W> &want,
                                              const uint64_t *cur, int level) {
  const bool need = want.any();
  const int64_t deg = need ? (__ldg(p.in_off + v + 1) - __ldg(p.in_off + v)) : 0;
  const bool heavy = need && deg > kPullLight;
  Mask<W> got = Mask<W>::zero();
  if (need && !heavy) got = thread_scan_in_list<W>(p, v, want, cur, level);
  unsigned hm = __ballot_sync(kMsFull, heavy);
  while (hm) {
    const int j = __ffs(hm) - 1;
    hm &= hm - 1;
    const int64_t vj = __shfl_sync(kMsFull, v, j);
    Mask<W> wj;
#pragma unroll
    for (int i = 0; i < W; ++i) wj.w[i] = __shfl_sync(kMsFull, want.w[i], j);
    const Mask<W> gj = warp_scan_in_list<W>(p, vj, wj, cur, level);
    if (lane_id() == j) got = gj;
  }
  return got;
}

// Pull round over every vertex with unvisited lanes whose frontier is not
// empty (`active`: lanes whose search has ended cannot be found any more).
template <int W>
__device__ void ms_pull(const MsParams &p, int L, const uint64_t *cur, uint64_t *nxt,
                        const Mask<W> &active, MsRound *Rn, MsAcc &acc) {
  const int64_t nthreads = (int64_t)gridDim.x * blockDim.x;
  const int next_parity = (L + 1) & 1;
  for (int64_t base = (int64_t)blockIdx.x * blockDim.x + (threadIdx.x & ~31);
       base < p.n; base += nthreads) {
    const int64_t v = base + lane_id();
    Mask<W> want = Mask<W>::zero();
    Mask<W> seen = Mask<W>::zero();
    if (v < p.n) {
      seen = ld_mask<W>(p.vis, v);
      want = active.andnot(seen);
    }
    if (!__ballot_sync(kMsFull, want.any())) continue;
    const Mask<W> got = scan_group<W>(p, v, want, cur, L + 1);
    bool claimed = false;
    int64_t deg = 0;
    if (got.any()) {
      st_mask<W>(nxt, v, got);
      st_mask<W>(p.vis, v, seen | got);
      claimed = true;
      acc.visits += (unsigned long long)got.popc();
      acc_lanes<W>(acc, got);
      deg = __ldg(p.out_off + v + 1) - __ldg(p.out_off + v);
    }
    ms_enqueue(p, claimed, (int32_t)v, deg, next_parity, Rn, acc);
  }
}

// Edge u -> v of a push round; true for the one thread that queues v.
template <int W>
__device__ __forceinline__ bool ms_relax(const MsParams &p, const Mask<W> &fu, int32_t v,
                                         uint64_t *nxt, uint32_t *touched) {
  const Mask<W> f = fu.andnot(ld_mask<W>(p.vis, v));
  if (!f.any()) return false;
  const Mask<W> have = ld_mask<W>(nxt, v);
  const Mask<W> add = f.andnot(have);
  if (add.any()) {
#pragma unroll
    for (int i = 0; i < W; ++i)
      if (add.w[i])
        atomicOr(reinterpret_cast<unsigned long long *>(nxt + (int64_t)v * W + i),
                 (unsigned long long)add.w[i]);
  }
  const uint32_t tb = 1u << (v & 31);
  if (touched[v >> 5] & tb) return false;
  return (atomicOr(touched + (v >> 5), tb) & tb) == 0;
}

template <int W>
__device__ __forceinline__ void ms_push_step(const MsParams &p, bool valid, const Mask<W> &fu,
                                             int64_t e, uint64_t *nxt, uint32_t *touched,
                                             int next_parity, MsRound *Rn, MsAcc &acc) {
  bool claimed = false;
  int32_t v = 0;
  int64_t deg = 0;
  if (valid) {
    v = __ldg(p.out_idx + e);
    claimed = ms_relax<W>(p, fu, v, nxt, touched);
    if (claimed) deg = __ldg(p.out_off + v + 1) - __ldg(p.out_off + v);
  }
  ms_enqueue(p, claimed, v, deg, next_parity, Rn, acc);
}

template <int W>
__device__ void ms_push(const MsParams &p, int L, const uint64_t *cur, uint64_t *nxt,
                        uint32_t *touched, MsRound *Rc, MsRound *Rn, MsAcc &acc) {
  __shared__ int32_t s_u[kMsBlock / 32][32];
  __shared__ int64_t s_s[kMsBlock / 32][32];
  __shared__ int32_t s_x[kMsBlock / 32][32];
  const int lane = lane_id();
  const int wib = threadIdx.x >> 5;
  const int gw = warp_id_global();
  const int nwarps = (gridDim.x * blockDim.x) >> 5;
  const int parity = L & 1, next_parity = parity ^ 1;
  const int32_t *q = parity ? p.queue1 : p.queue0;
  const int32_t *h = parity ? p.heavy1 : p.heavy0;

  const unsigned nheavy = *(volatile unsigned *)&Rc->nheavy;
  for (unsigned b = 0; b < nheavy; ++b) {
    const int32_t u = h[b];
    const Mask<W> fu = ld_mask<W>(cur, u);
    const int64_t s = __ldg(p.out_off + u), e = __ldg(p.out_off + u + 1);
    for (int64_t base = s + (int64_t)gw * 32; base < e; base += (int64_t)nwarps * 32) {
      const int64_t i = base + lane;
      ms_push_step<W>(p, i < e, fu, i, nxt, touched, next_parity, Rn, acc);
    }
  }
  const unsigned nmed = *(volatile unsigned *)&Rc->nmedium;
  const unsigned nlight = *(volatile unsigned *)&Rc->nlight;
  const unsigned nitems = nmed + (nlight + 31u) / 32u;
  while (true) {
    unsigned item = 0;
    if (lane == 0) item = atomicAdd(&Rc->work, 1u);
    item = __shfl_sync(kMsFull, item, 0);
    if (item >= nitems) break;
    if (item < nmed) {
      const int32_t u = q[p.n - 1 - (int64_t)item];
      const Mask<W> fu = ld_mask<W>(cur, u);
      const int64_t s = __ldg(p.out_off + u), e = __ldg(p.out_off + u + 1);
      for (int64_t base = s; base < e; base += 32) {
        const int64_t i = base + lane;
        ms_push_step<W>(p, i < e, fu, i, nxt, touched, next_parity, Rn, acc);
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
        const int t = __shfl_up_sync(kMsFull, incl, o);
        if (lane >= o) incl += t;
      }
      const int total = __shfl_sync(kMsFull, incl, 31);
      s_u[wib][lane] = u;
      s_s[wib][lane] = s;
      s_x[wib][lane] = incl - d;
      __syncwarp();
      for (int base = 0; base < total; base += 32) {
        const int t = base + lane;
        const bool valid = t < total;
        int64_t e = 0;
        Mask<W> fu = Mask<W>::zero();
        if (valid) {
          int lo = 0, hi = 31;
          while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (s_x[wib][mid] <= t)
              lo = mid;
            else
              hi = mid - 1;
          }
          fu = ld_mask<W>(cur, s_u[wib][lo]);
          e = s_s[wib][lo] + (t - s_x[wib][lo]);
        }
        ms_push_step<W>(p, valid, fu, e, nxt, touched, next_parity, Rn, acc);
      }
      __syncwarp();
    }
  }
}

// After a push round: for every newly reached vertex, merge its lanes into
// vis and resolve each lane's parent by scanning the ascending in-list.
template <int W>
__device__ void ms_resolve(const MsParams &p, int L, const uint64_t *cur, const uint64_t *nxt,
                           const MsRound *Rn, MsAcc &acc) {
  const int64_t nthreads = (int64_t)gridDim.x * blockDim.x;
  const int next_parity = (L + 1) & 1;
  const int32_t *q = next_parity ? p.queue1 : p.queue0;
  const int32_t *h = next_parity ? p.heavy1 : p.heavy0;
  const int64_t nl = *(volatile unsigned *)&Rn->nlight;
  const int64_t nm = *(volatile unsigned *)&Rn->nmedium;
  const int64_t nh = *(volatile unsigned *)&Rn->nheavy;
  const int64_t total = nl + nm + nh;
  for (int64_t base = (int64_t)blockIdx.x * blockDim.x + (threadIdx.x & ~31); base < total;
       base += nthreads) {
    const int64_t j = base + lane_id();
    int64_t v = 0;
    Mask<W> nw = Mask<W>::zero();
    if (j < total) {
      if (j < nl)
        v = q[j];
      else if (j < nl + nm)
        v = q[p.n - 1 - (j - nl)];
      else
        v = h[j - nl - nm];
      nw = ld_mask<W>(nxt, v);
      st_mask<W>(p.vis, v, ld_mask<W>(p.vis, v) | nw);
      acc.visits += (unsigned long long)nw.popc();
      acc_lanes<W>(acc, nw);
    }
    // every lane of nw has a frontier source in v's in-list: the scan ends
    scan_group<W>(p, v, nw, cur, L + 1);
  }
}

template <int W>
__global__ void __launch_bounds__(kMsBlock) msbfs_persistent(MsParams p) {
  MsCtl *ctl = p.ctl;
  const int64_t gtid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t nthreads = (int64_t)gridDim.x * blockDim.x;
  const bool leader = blockIdx.x == 0 && threadIdx.x == 0;
  const long long t_start = leader ? global_ns() : 0;
  uint64_t *fr[3] = {p.fr0, p.fr1, p.fr2};

  // phase 0: clear the lane state
  for (int64_t i = gtid; i < p.n * W; i += nthreads) {
    p.vis[i] = 0;
    p.fr0[i] = 0;
    p.fr1[i] = 0;
    p.fr2[i] = 0;
  }
  for (int64_t w = gtid; w < p.words; w += nthreads) {
    p.touched0[w] = 0;
    p.touched1[w] = 0;
  }
  bool ok = grid_wait(&ctl->wait, &ctl->status, p.timeout_ns);
  // seed: lane i starts at roots[i] (block 0)
  if (ok && blockIdx.x == 0) {
    if (threadIdx.x < p.k) {
      const int i = threadIdx.x;
      const int32_t r = p.roots[i];
      const unsigned long long bit = 1ull << (i & 63);
      atomicOr(reinterpret_cast<unsigned long long *>(p.vis + (int64_t)r * W + (i >> 6)), bit);
      atomicOr(reinterpret_cast<unsigned long long *>(p.fr0 + (int64_t)r * W + (i >> 6)), bit);
      p.levels[(int64_t)i * p.n + r] = 0;
      p.parents[(int64_t)i * p.n + r] = r;
      bool first = true;
      for (int j = 0; j < i; ++j) first = first && (p.roots[j] != r);
      if (first) {
        const int64_t deg = p.out_off[r + 1] - p.out_off[r];
        MsRound *R0 = &ctl->rec[0];
        if (deg <= kLightMax)
          p.queue0[atomicAdd(&R0->nlight, 1u)] = r;
        else if (deg <= kMediumMax)
          p.queue0[p.n - 1 - (int64_t)atomicAdd(&R0->nmedium, 1u)] = r;
        else
          p.heavy0[atomicAdd(&R0->nheavy, 1u)] = r;
        atomicAdd(&R0->nf, 1ull);
        atomicAdd(&R0->mf, (unsigned long long)deg);
      }
      if (i == 0) {
        const Mask<W> a0 = lane_mask<W>(p.k);
        ctl->rec[0].lanes[0] = a0.w[0];
        ctl->rec[0].lanes[1] = W == 2 ? a0.w[W - 1] : 0ull;
      }
    }
  }
  if (ok) ok = grid_wait(&ctl->wait, &ctl->status, p.timeout_ns);

  int dir = 0;  // 0 push, 1 pull
  int L = 0, pull_rounds = 0, switches = 0;
  unsigned long long visited = (unsigned long long)p.k;
  MsAcc acc;
  long long t_round = leader ? global_ns() : 0;
  if (leader) p.stats->setup_ns = t_round - t_start;
  while (ok) {
    if (leader && L > 0 && L - 1 < CG_HISTORY) {
      const long long now = global_ns();
      p.stats->round_ns[L - 1] = now - t_round;
      t_round = now;
    }
    const uint64_t *cur = fr[L % 3];
    uint64_t *nxt = fr[(L + 1) % 3];
    uint64_t *old = fr[(L + 2) % 3];
    uint32_t *touched = (L & 1) ? p.touched1 : p.touched0;
    uint32_t *touched_next = (L & 1) ? p.touched0 : p.touched1;
    MsRound *Rc = &ctl->rec[L % kRing];
    MsRound *Rn = &ctl->rec[(L + 1) % kRing];
    // F_{L-1}, last round's touched bits and the record of round L-1 are no
    // longer read by anyone; the record is next appended to in round L + 2
    if (leader) {
      MsRound *Rz = &ctl->rec[(L + 3) % kRing];
      Rz->nf = Rz->visits = Rz->mf = 0;
      Rz->nlight = Rz->nmedium = Rz->nheavy = Rz->work = 0;
      Rz->lanes[0] = Rz->lanes[1] = 0;
    }
    for (int64_t i = gtid; i < p.n * W; i += nthreads) old[i] = 0;
    for (int64_t w = gtid; w < p.words; w += nthreads) touched_next[w] = 0;
    if (dir == 1) {
      Mask<W> active;
#pragma unroll
      for (int i = 0; i < W; ++i) active.w[i] = *(volatile unsigned long long *)&Rc->lanes[i];
      ms_pull<W>(p, L, cur, nxt, active, Rn, acc);
      ms_flush(acc, Rn);
      if (!(ok = grid_wait(&ctl->wait, &ctl->status, p.timeout_ns))) break;
    } else {
      ms_push<W>(p, L, cur, nxt, touched, Rc, Rn, acc);
      if (!(ok = grid_wait(&ctl->wait, &ctl->status, p.timeout_ns))) break;
      ms_resolve<W>(p, L, cur, nxt, Rn, acc);
      ms_flush(acc, Rn);
      if (!(ok = grid_wait(&ctl->wait, &ctl->status, p.timeout_ns))) break;
    }
    const unsigned long long nf = *(volatile unsigned long long *)&Rn->nf;
    const unsigned long long visits = *(volatile unsigned long long *)&Rn->visits;
    const unsigned long long mf = *(volatile unsigned long long *)&Rn->mf;
    if (leader && L < CG_HISTORY) {
      p.stats->nf_history[L] = (int64_t)visits;
      p.stats->direction_history[L] = dir;
    }
    if (dir == 1) ++pull_rounds;
    visited += visits;
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
    int next;
    if (p.direction == CG_DIR_TOPDOWN)
      next = 0;
    else if (p.direction == CG_DIR_BOTTOMUP)
      next = 1;
    else
      next = ((double)mf * (double)p.ms_alpha > (double)p.nnz) ? 1 : 0;
    if (next != dir) ++switches;
    dir = next;
    ++L;
  }
  long long t_finish = 0;
  if (leader) {
    t_finish = global_ns();
    if (L > 0 && L - 1 < CG_HISTORY) p.stats->round_ns[L - 1] = t_finish - t_round;
  }
  // unreached lanes: level and parent -1 (each (lane, vertex) is written once)
  if (ok) {
    for (int64_t v = gtid; v < p.n; v += nthreads) {
      const Mask<W> m = ld_mask<W>(p.vis, v);
      for (int l = 0; l < p.k; ++l) {
        if (!((m.w[l >> 6] >> (l & 63)) & 1ull)) {
          p.levels[(int64_t)l * p.n + v] = -1;
          p.parents[(int64_t)l * p.n + v] = -1;
        }
      }
    }
  }
  if (leader) {
    cg_stats *st = p.stats;
    st->finish_ns = global_ns() - t_finish;
    st->status = *(volatile int *)&ctl->status;
    st->rounds = L;
    st->visited = (int64_t)visited;
    st->pull_rounds = pull_rounds;
    st->switches = switches;
    st->history_len = L < CG_HISTORY ? L : CG_HISTORY;
    st->device_ms = 0.f;
  }
}

// ---------------------------------------------------------------------------
struct MsState {
  uint64_t *bits;
  uint32_t *touched;
  int32_t *queue;
  int32_t *heavy;
  MsCtl *ctl;
  int64_t hcap;
};

void msbfs_release(cg_graph *g) {
  MsState *s = reinterpret_cast<MsState *>(g->ms_ctl);
  if (s) {
    cudaFree(s->bits);
    cudaFree(s->touched);
    cudaFree(s->queue);
    cudaFree(s->heavy);
    cudaFree(s->ctl);
    delete s;
  }
  g->ms_ctl = nullptr;
  cudaFree(g->ms_levels);
  cudaFree(g->ms_parents);
  g->ms_levels = g->ms_parents = nullptr;
  g->ms_out_cap = 0;
  g->ms_lane_words = 0;
}

static int ms_alloc_state(cg_graph *g, int lane_words) {
  if (g->ms_ctl && g->ms_lane_words == lane_words) return CG_OK;
  if (g->ms_ctl) {
    MsState *s = reinterpret_cast<MsState *>(g->ms_ctl);
    cudaFree(s->bits);
    cudaFree(s->touched);
    cudaFree(s->queue);
    cudaFree(s->heavy);
    cudaFree(s->ctl);
    delete s;
    g->ms_ctl = nullptr;
  }
  MsState *s = new MsState();
  s->hcap = g->nnz / (kMediumMax + 1) + 1;
  if (s->hcap > g->n) s->hcap = g->n;
  const size_t bits = sizeof(uint64_t) * 4 * (size_t)g->n * lane_words;
  const size_t words = (size_t)((g->n + 31) / 32);
  if (cudaMalloc(&s->bits, bits) != cudaSuccess ||
      cudaMalloc(&s->touched, sizeof(uint32_t) * 2 * words) != cudaSuccess ||
      cudaMalloc(&s->queue, sizeof(int32_t) * 2 * (size_t)g->n) != cudaSuccess ||
      cudaMalloc(&s->heavy, sizeof(int32_t) * 2 * (size_t)s->hcap) != cudaSuccess ||
      cudaMalloc(&s->ctl, sizeof(MsCtl)) != cudaSuccess) {
    g->ms_ctl = s;
    msbfs_release(g);
    return CG_ERR_OUT_OF_MEMORY;
  }
  g->ms_ctl = s;
  g->ms_lane_words = lane_words;
  g->device_bytes += bits + sizeof(uint32_t) * 2 * words + sizeof(int32_t) * 2 * g->n +
                     sizeof(int32_t) * 2 * s->hcap + sizeof(MsCtl);
  return CG_OK;
}

int msbfs_prepare(cg_graph *g, int lane_words, int64_t out_elems) {
  int rc = ms_alloc_state(g, lane_words);
  if (rc) return rc;
  if (out_elems > g->ms_out_cap) {
    cudaFree(g->ms_levels);
    cudaFree(g->ms_parents);
    g->ms_levels = g->ms_parents = nullptr;
    if (cudaMalloc(&g->ms_levels, sizeof(int32_t) * (size_t)out_elems) != cudaSuccess ||
        cudaMalloc(&g->ms_parents, sizeof(int32_t) * (size_t)out_elems) != cudaSuccess) {
      cudaFree(g->ms_levels);
      g->ms_levels = nullptr;
      g->ms_out_cap = 0;
      return CG_ERR_OUT_OF_MEMORY;
    }
    g->device_bytes += 2 * sizeof(int32_t) * (out_elems - g->ms_out_cap);
    g->ms_out_cap = out_elems;
  }
  return CG_OK;
}

template <int W>
static int ms_launch_pass(cg_graph *g, MsState *s, const int64_t *roots, int k,
                          int32_t *d_levels, int32_t *d_parents) {
  int block = g->opt.block_size > 0 ? g->opt.block_size : kMsBlock;
  if (block > kMsBlock) block = kMsBlock;
  block = (block / 32) * 32;
  if (block < 128) block = 128;  // seeding uses threads 0..k-1 of block 0
  int per_sm = 0;
  CG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, msbfs_persistent<W>, block, 0));
  if (per_sm <= 0) return CG_ERR_NOT_SUPPORTED;
  if (g->opt.blocks_per_sm > 0 && g->opt.blocks_per_sm < per_sm) per_sm = g->opt.blocks_per_sm;
  MsParams p;
  p.n = g->n;
  p.nnz = g->nnz;
  p.words = (g->n + 31) / 32;
  p.in_off = g->in_off;
  p.in_idx = g->in_idx;
  p.out_off = g->out_off;
  p.out_idx = g->out_idx;
  const size_t plane = (size_t)g->n * W;
  p.vis = s->bits;
  p.fr0 = s->bits + plane;
  p.fr1 = s->bits + 2 * plane;
  p.fr2 = s->bits + 3 * plane;
  p.touched0 = s->touched;
  p.touched1 = s->touched + p.words;
  p.queue0 = s->queue;
  p.queue1 = s->queue + g->n;
  p.heavy0 = s->heavy;
  p.heavy1 = s->heavy + s->hcap;
  p.levels = d_levels;
  p.parents = d_parents;
  p.ctl = s->ctl;
  p.stats = g->d_stats;
  p.k = k;
  p.direction = g->opt.direction == CG_DIR_TAU ? CG_DIR_AUTO : g->opt.direction;
  p.ms_alpha = g->opt.ms_alpha > 0 ? g->opt.ms_alpha : 4.f;
  p.level_cap = g->opt.level_cap > 0 ? g->opt.level_cap
                                     : (int)((g->n + 1) < 0x7fffffff ? g->n + 1 : 0x7fffffff);
  p.timeout_ns = (long long)(g->opt.wait_timeout_ms > 0 ? g->opt.wait_timeout_ms : 1000) * 1000000ll;
  for (int i = 0; i < kMsMaxLanes; ++i) p.roots[i] = i < k ? (int32_t)roots[i] : 0;
  CG_CUDA(cudaMemsetAsync(s->ctl, 0, sizeof(MsCtl), g->stream));
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(per_sm * g->num_sms);
  cfg.blockDim = dim3(block);
  cfg.dynamicSmemBytes = 0;
  cfg.stream = g->stream;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeCooperative;
  attr[0].val.cooperative = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  CG_CUDA(cudaLaunchKernelEx(&cfg, msbfs_persistent<W>, p));
  return CG_OK;
}

int msbfs_launch(cg_graph *g, const int64_t *roots, int32_t k, int32_t *d_levels,
                 int32_t *d_parents) {
  const int W = g->opt.lane_words == 2 ? 2 : 1;
  int rc = ms_alloc_state(g, W);
  if (rc) return rc;
  MsState *s = reinterpret_cast<MsState *>(g->ms_ctl);
  const int lanes = 64 * W;
  for (int32_t b = 0; b < k; b += lanes) {
    const int kk = (k - b) < lanes ? (k - b) : lanes;
    int32_t *lv = d_levels + (int64_t)b * g->n;
    int32_t *pa = d_parents + (int64_t)b * g->n;
    rc = W == 2 ? ms_launch_pass<2>(g, s, roots + b, kk, lv, pa)
                : ms_launch_pass<1>(g, s, roots + b, kk, lv, pa);
    if (rc) return rc;
  }
  return CG_OK;
}

}  // namespace cg
