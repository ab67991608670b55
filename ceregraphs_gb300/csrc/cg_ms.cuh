// Shared pieces of the multi-source kernels (cg_msbfs.cu: outputs written
// during the rounds, serving pools; cg_msledger.cu: rounds on frontier masks
// only, outputs from the round history in one coalesced pass).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "cg_internal.cuh"

namespace cg {

constexpr unsigned kMsFull = 0xffffffffu;
constexpr int kMsBlock = 512;
constexpr int kMsMaxLanes = 128;
constexpr int kPullLight = 32;    // in-degree <= this: one thread scans the in-list
constexpr int kHubDeg = 1024;     // in-degree > this: hub
constexpr int kHubChunk = 1024;   // in-list entries of a hub per work item
constexpr int kPairs = 4;         // first-hit records a light vertex's pull rounds may take,
                                  // unless the light vertices hold under half of the edges
                                  // (then all kRecords: see MsState::pull_records)
constexpr int kRecords = 8;       // records per light vertex in all (pull rounds + scan pass)

struct MsRound {
  unsigned long long nf[kCounterShards];      // vertices with a nonzero frontier mask
  unsigned long long visits[kCounterShards];  // lane discoveries
  unsigned long long mf[kCounterShards];      // sum of out-degrees over the frontier
  unsigned long long big;       // queue: (count << 32) | edges of its big vertices
  unsigned int nlight, work;
  unsigned int res_light, res_big;  // queue counts a push round's resolve phase covers
  unsigned long long lanes[2];  // lanes whose frontier is non-empty
  unsigned long long pad[2];
};

// Lane table of a serving pool: where each lane's outputs go and the round at
// which its search started (its level = round + 1 - start).
struct LaneTable {
  int32_t *levels[kMsMaxLanes];
  int32_t *parents[kMsMaxLanes];
  int32_t start[kMsMaxLanes];
};

// Only the block that arrives last at a round's grid-wide wait touches the
// round bookkeeping (L .. t_round); the waits order those accesses.  L and
// dir persist between launches, so a serving pool resumes where it stopped.
struct MsCtl {
  GridWait wait;
  int status;
  int L;                          // next round to run
  int dir;                        // its direction (0 push, 1 pull)
  int pull_rounds;
  int switches;
  unsigned exited;                // blocks past the final pass (finish time)
  unsigned nover;                 // light vertices whose records ran out (scan pass)
  unsigned scan_work;             // scan pass: chunks of scanmap handed out
  unsigned long long visited;
  unsigned long long done[2];     // lanes whose search ended (cleared by the host)
  long long t_start;
  long long t_round;
  unsigned long long pad[8];
  MsRound rec[kRing];
};

struct MsParams {
  int64_t n, nnz, words;
  const int64_t *__restrict__ in_off;
  const int32_t *__restrict__ in_idx;
  const int64_t *__restrict__ out_off;
  const int32_t *__restrict__ out_idx;
  uint64_t *vis, *fr0, *fr1, *fr2;
  uint32_t *touched0, *touched1, *touched2;
  uint32_t *scanmap;  // light vertices with lanes their records leave open (ledger)
  const uint32_t *dead;  // vertices without in-edges (never reached after round 0)
  // ledger batches: vertices of in-degree 1 .. kPullLight (static), and those
  // of them a batch has finished -- every running lane visited (no lane can
  // reach them again), so later pull rounds skip them
  const uint32_t *light;
  uint32_t *fin;
  int pull_records;    // ledger: records a light vertex's pull rounds may take (<= kRecords)
  int32_t *queue0, *queue1;
  uint32_t *bigoff0, *bigoff1;
  const int32_t *hub_slot;   // [n], -1 for non-hubs
  const int32_t *hub_vtx;    // [nhub]
  const int32_t *med_vtx;    // [nmed] vertices of in-degree in (kPullLight, kHubDeg]
  int64_t nmed;
  const uint32_t *hub_choff; // [nhub + 1] prefix of in-list chunks
  const uint32_t *hub_of_chunk; // [chunks] the hub each in-list chunk belongs to
  const uint32_t *hub_chunk_order; // [chunks] chunk ids by rank within their hub, then hub
  uint32_t *hub_cand;        // [nhub][64 W] parent candidates (0xFFFFFFFF = none)
  uint64_t *hub_found;       // [nhub][W] lanes found this round
  // [nhub] lowest chunk that found every wanted lane, per round (ledger pull):
  // ((round + 1) << 24) | (0xFFFFFF - chunk), combined with atomicMax; ledger
  // rounds stay below 255 and chunks below 2^24 (nnz < 2^32, 1024 per chunk)
  unsigned *hub_done;
  int nhub;
  int32_t *levels, *parents;  // batch mode: lane l at levels + l * n (start round 0)
  const LaneTable *lanes;     // serving pool: per-lane outputs and start rounds
  MsCtl *ctl;
  cg_stats *stats;
  int k;
  int direction;
  float ms_alpha;
  int level_cap;
  long long timeout_ns;
  int resume;                 // continue from ctl->L instead of clearing and seeding
  int max_rounds;             // stop after this many rounds in this launch
  int stop_on_finish;         // stop after a round in which some lane's search ended
  int finish_all;             // write -1 for every unreached (lane, vertex) at the end
  // round history (cg_msledger.cu): F_L of round L at hist + L * n * W
  uint64_t *hist;
  int hist_planes;            // F_0 .. F_{hist_planes - 1}
  int *flag;                  // set when a search outgrows the history
  // parent candidates of the output pass: vertices of in-degree > kPullLight
  const int32_t *cand_slot;   // [n], -1 for light vertices
  const int32_t *cand_vtx;    // [ncand]
  const uint32_t *cand_choff; // [ncand + 1] prefix of in-list chunks
  uint32_t *cand;             // [ncand][64 W], 0xFFFFFFFF = none yet
  int ncand;
  // (source, lanes) records of light vertices: the first hits of their
  // pull-round scans (up to kPairs), then those of the scan pass after the
  // rounds (up to kRecords in all); record q at [q * n + v]
  int32_t *pair_u;
  uint64_t *pair_m;           // W words per record
  uint8_t *pair_n;            // [n] records used
  int gate;                   // run only if *flag is set (the fallback launch)
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

// OR over the warp: one redux.sync per 32-bit half (a shuffle tree would be
// five dependent shuffle round trips per half).
__device__ __forceinline__ uint64_t warp_or64(uint64_t x) {
  const unsigned lo = __reduce_or_sync(kMsFull, (unsigned)x);
  const unsigned hi = __reduce_or_sync(kMsFull, (unsigned)(x >> 32));
  return ((uint64_t)hi << 32) | lo;
}

template <int W>
__device__ __forceinline__ Mask<W> warp_or(Mask<W> m) {
#pragma unroll
  for (int j = 0; j < W; ++j) m.w[j] = warp_or64(m.w[j]);
  return m;
}

struct MsAcc {
  unsigned long long nf = 0, visits = 0, mf = 0;
  unsigned long long lanes[2] = {0ull, 0ull};
};

template <int W>
__device__ __forceinline__ void acc_lanes(MsAcc &acc, const Mask<W> &m) {
#pragma unroll
  for (int i = 0; i < W; ++i) acc.lanes[i] |= m.w[i];
}

// Appends claimed vertices to a frontier list: light ones at the front of
// `q` (unless LightQ is false: the ledger kernel finds them in a claim
// bitmap), big ones (out-degree > kLightMax) at the back with the prefix
// offset of their edge lists (one packed atomic per warp: count << 32 |
// edges).  All 32 lanes call.
template <bool LightQ = true>
__device__ __forceinline__ void ms_enqueue(bool claimed, int32_t v, int64_t deg, int32_t *q,
                                           int64_t qcap, uint32_t *boff, unsigned *nlight,
                                           unsigned long long *big, MsAcc &acc) {
  const int lane = lane_id();
  if (!__ballot_sync(kMsFull, claimed)) return;
  const bool light = claimed && deg <= kLightMax;
  const bool heavy = claimed && deg > kLightMax;
  const unsigned below = (1u << lane) - 1u;
  const unsigned ml = __ballot_sync(kMsFull, light);
  if (LightQ && ml) {
    const int leader = __ffs(ml) - 1;
    unsigned base = 0;
    if (lane == leader) base = atomicAdd(nlight, (unsigned)__popc(ml));
    base = __shfl_sync(kMsFull, base, leader);
    if (light) q[base + __popc(ml & below)] = v;
  }
  const unsigned mb = __ballot_sync(kMsFull, heavy);
  if (mb) {
    const unsigned d = heavy ? (unsigned)deg : 0u;
    unsigned incl = d;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const unsigned t = __shfl_up_sync(kMsFull, incl, o);
      if (lane >= o) incl += t;
    }
    const unsigned total = __shfl_sync(kMsFull, incl, 31);
    unsigned long long old = 0;
    if (lane == 0) old = atomicAdd(big, ((unsigned long long)__popc(mb) << 32) | total);
    old = __shfl_sync(kMsFull, old, 0);
    if (heavy) {
      const unsigned idx = (unsigned)(old >> 32) + __popc(mb & below);
      q[qcap - 1 - (int64_t)idx] = v;
      boff[idx] = (unsigned)(old & 0xffffffffu) + incl - d;
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

// Lanes of m held by no lower warp lane: an exclusive prefix OR over the warp.
template <int W>
__device__ __forceinline__ Mask<W> first_holder(const Mask<W> &m) {
  const int lane = lane_id();
  Mask<W> below = Mask<W>::zero();
  Mask<W> run = m;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
#pragma unroll
    for (int j = 0; j < W; ++j) {
      const uint64_t t = __shfl_up_sync(kMsFull, run.w[j], o);
      if (lane >= o) run.w[j] |= t;
    }
  }
#pragma unroll
  for (int j = 0; j < W; ++j) {
    below.w[j] = __shfl_up_sync(kMsFull, run.w[j], 1);
    if (lane == 0) below.w[j] = 0ull;
  }
  return m.andnot(below);
}

// Edge u -> v of a push round of the direct kernel (outputs written during
// the rounds).  Targets get their new lanes ORed into the next mask, and the
// one thread that first touches v this round queues it; hub targets take
// parent candidates by atomicMin instead.
template <int W>
__device__ __forceinline__ bool ms_relax(const MsParams &p, const Mask<W> &fu, int32_t u,
                                         int32_t v, uint64_t *nxt, uint32_t *touched) {
  const Mask<W> f = fu.andnot(ld_mask<W>(p.vis, v));
  if (!f.any()) return false;
  const int h = p.hub_slot[v];
  if (h >= 0) {
    const Mask<W> have = ld_mask<W>(p.hub_found, h);
#pragma unroll
    for (int j = 0; j < W; ++j) {
      uint64_t bits = f.w[j];
      while (bits) {
        const int b = __ffsll((long long)bits) - 1;
        bits &= bits - 1;
        atomicMin(p.hub_cand + (int64_t)h * (64 * W) + j * 64 + b, (unsigned)u);
      }
      const uint64_t add = f.w[j] & ~have.w[j];
      if (add)
        atomicOr(reinterpret_cast<unsigned long long *>(p.hub_found + (int64_t)h * W + j),
                 (unsigned long long)add);
    }
    return false;
  }
  const Mask<W> add = f.andnot(ld_mask<W>(nxt, v));
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
                                             int32_t u, int64_t e, uint64_t *nxt,
                                             uint32_t *touched, int32_t *q, uint32_t *boff,
                                             MsRound *Rn, MsAcc &acc) {
  bool claimed = false;
  int32_t v = 0;
  int64_t deg = 0;
  if (valid) {
    v = __ldg(p.out_idx + e);
    claimed = ms_relax<W>(p, fu, u, v, nxt, touched);
    if (claimed) deg = __ldg(p.out_off + v + 1) - __ldg(p.out_off + v);
  }
  ms_enqueue(claimed, v, deg, q, p.n, boff, &Rn->nlight, &Rn->big, acc);
}

// Walks edge positions [x0, x1) of a big-vertex list (vertices q[cap-1-j],
// prefix offsets boff[j], all of out-degree > 32).
template <int W>
__device__ void ms_push_chunk(const MsParams &p, const uint64_t *cur, uint64_t *nxt,
                              uint32_t *touched, const int32_t *bq, int64_t cap,
                              const uint32_t *boff, unsigned nbig, unsigned x0, unsigned x1,
                              int32_t *q, uint32_t *qoff, MsRound *Rn, MsAcc &acc) {
  const int lane = lane_id();
  unsigned lo = 0, hi = nbig - 1;
  while (lo < hi) {
    const unsigned mid = (lo + hi + 1) >> 1;
    if (boff[mid] <= x0)
      lo = mid;
    else
      hi = mid - 1;
  }
  unsigned j = lo;
  int32_t vj = bq[cap - 1 - (int64_t)j];
  int64_t sj = __ldg(p.out_off + vj);
  unsigned oj = boff[j];
  unsigned endj = oj + (unsigned)(__ldg(p.out_off + vj + 1) - sj);
  Mask<W> fj = ld_mask<W>(cur, vj);
  for (unsigned base = x0; base < x1; base += 32) {
    while (base >= endj) {
      ++j;
      vj = bq[cap - 1 - (int64_t)j];
      sj = __ldg(p.out_off + vj);
      oj = boff[j];
      endj = oj + (unsigned)(__ldg(p.out_off + vj + 1) - sj);
      fj = ld_mask<W>(cur, vj);
    }
    const unsigned x = base + lane;
    const bool valid = x < x1;
    int32_t u = vj;
    int64_t e = sj + (int64_t)(x - oj);
    Mask<W> fu = fj;
    if (__ballot_sync(kMsFull, valid && x >= endj)) {
      const int32_t vn = bq[cap - 1 - (int64_t)(j + 1)];
      if (valid && x >= endj) {
        u = vn;
        e = __ldg(p.out_off + vn) + (int64_t)(x - endj);
        fu = ld_mask<W>(cur, vn);
      }
    }
    ms_push_step<W>(p, valid, fu, u, e, nxt, touched, q, qoff, Rn, acc);
  }
}

template <int W>
__device__ void ms_push(const MsParams &p, int L, const uint64_t *cur, uint64_t *nxt,
                        uint32_t *touched, MsRound *Rc, MsRound *Rn, MsAcc &acc) {
  __shared__ int32_t s_u[kMsBlock / 32][32];
  __shared__ int64_t s_s[kMsBlock / 32][32];
  __shared__ int64_t s_x[kMsBlock / 32][32];
  const int lane = lane_id();
  const int wib = threadIdx.x >> 5;
  const int nwarps = (gridDim.x * blockDim.x) >> 5;
  const int parity = L & 1, next_parity = parity ^ 1;
  const int32_t *qc = parity ? p.queue1 : p.queue0;
  const uint32_t *bc = parity ? p.bigoff1 : p.bigoff0;
  int32_t *qn = next_parity ? p.queue1 : p.queue0;
  uint32_t *bn = next_parity ? p.bigoff1 : p.bigoff0;

  const unsigned long long bigw = *(volatile unsigned long long *)&Rc->big;
  const unsigned nbig = (unsigned)(bigw >> 32), big_edges = (unsigned)bigw;
  const unsigned nlight = *(volatile unsigned *)&Rc->nlight;
  // chunks of 32 .. kPushChunk edges: small frontiers still spread over the grid
  unsigned chunk = ((big_edges / (unsigned)nwarps) + 31u) & ~31u;
  chunk = chunk < 32u ? 32u : (chunk > (unsigned)kPushChunk ? (unsigned)kPushChunk : chunk);
  const unsigned nb = (big_edges + chunk - 1) / chunk;
  const unsigned nitems = nb + (nlight + 31u) / 32u;
  unsigned item = (unsigned)warp_id_global();
  while (item < nitems) {
    if (item < nb) {
      const unsigned x0 = item * chunk;
      ms_push_chunk<W>(p, cur, nxt, touched, qc, p.n, bc, nbig, x0, min(x0 + chunk, big_edges),
                       qn, bn, Rn, acc);
    } else {
      const unsigned idx = (item - nb) * 32u + lane;
      int32_t u = -1;
      int64_t s = 0, d = 0;
      if (idx < nlight) {
        u = qc[idx];
        s = __ldg(p.out_off + u);
        d = __ldg(p.out_off + u + 1) - s;
      }
      int64_t incl = d;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const int64_t t = __shfl_up_sync(kMsFull, incl, o);
        if (lane >= o) incl += t;
      }
      const int64_t total = __shfl_sync(kMsFull, incl, 31);
      s_u[wib][lane] = u;
      s_s[wib][lane] = s;
      s_x[wib][lane] = incl - d;
      __syncwarp();
      for (int64_t base = 0; base < total; base += 32) {
        const int64_t t = base + lane;
        const bool valid = t < total;
        int64_t e = 0;
        int32_t uu = 0;
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
          uu = s_u[wib][lo];
          fu = ld_mask<W>(cur, uu);
          e = s_s[wib][lo] + (t - s_x[wib][lo]);
        }
        ms_push_step<W>(p, valid, fu, uu, e, nxt, touched, qn, bn, Rn, acc);
      }
      __syncwarp();
    }
    unsigned nextitem = 0;
    if (lane == 0) nextitem = (unsigned)nwarps + atomicAdd(&Rc->work, 1u);
    item = __shfl_sync(kMsFull, nextitem, 0);
  }
}

// Block totals of the per-thread counters (thread 0 gets them) -- the one
// __syncthreads of a round's end before the grid-wide wait.
__device__ __forceinline__ void ms_block_totals(MsAcc &acc, MsAcc &tot) {
  __shared__ unsigned long long s_red[5][kMsBlock / 32];
  const int lane = lane_id(), wib = threadIdx.x >> 5;
  const unsigned long long a = ms_warp_sum(acc.nf), b = ms_warp_sum(acc.visits),
                           c = ms_warp_sum(acc.mf);
  const unsigned long long l0 = warp_or64(acc.lanes[0]), l1 = warp_or64(acc.lanes[1]);
  if (lane == 0) {
    s_red[0][wib] = a;
    s_red[1][wib] = b;
    s_red[2][wib] = c;
    s_red[3][wib] = l0;
    s_red[4][wib] = l1;
  }
  __syncthreads();
  tot = MsAcc();
  if (threadIdx.x == 0) {
    for (int i = 0; i < (int)(blockDim.x >> 5); ++i) {
      tot.nf += s_red[0][i];
      tot.visits += s_red[1][i];
      tot.mf += s_red[2][i];
      tot.lanes[0] |= s_red[3][i];
      tot.lanes[1] |= s_red[4][i];
    }
  }
  acc = MsAcc();
}

// kMsSparse (ledger): the next round's frontier has under n/1024 vertices
constexpr unsigned kMsStop = 1u, kMsNextPull = 2u, kMsSparse = 4u;

struct MsState {
  uint64_t *bits = nullptr;
  uint32_t *touched = nullptr;
  int32_t *queue = nullptr;
  uint32_t *bigoff = nullptr;
  int32_t *hub_slot = nullptr;
  int32_t *hub_vtx = nullptr;
  int32_t *med_vtx = nullptr;
  int64_t nmed = 0;
  uint32_t *hub_choff = nullptr;
  uint32_t *hub_of_chunk = nullptr;
  uint32_t *hub_chunk_order = nullptr;
  uint32_t *hub_cand = nullptr;
  uint64_t *hub_found = nullptr;
  unsigned *hub_done = nullptr;
  MsCtl *ctl = nullptr;
  int *flag = nullptr;        // history overflow flag of the last batch
  int32_t *cand_slot = nullptr;
  int32_t *cand_vtx = nullptr;
  uint32_t *cand_choff = nullptr;
  uint32_t *cand = nullptr;
  int ncand = 0;
  int32_t *pair_u = nullptr;
  uint64_t *pair_m = nullptr;
  uint8_t *pair_n = nullptr;
  uint32_t *lightfin = nullptr;  // [2][words]: the light map, then the finished map
  int pull_records = kPairs;     // records a light vertex's pull rounds may take
  int64_t bcap = 0;
  int nhub = 0;
  int lane_words = 0;
  int hist_planes = 0;        // frontier planes after vis: 3, or the round history
  int hist_opt = 0;           // the ms_history option the state was sized for
};

// Fields of a launch shared by batches and serving pools.
template <int W>
inline MsParams ms_params(const cg_graph *g, const MsState *s) {
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
  p.hist = s->bits + plane;
  p.hist_planes = s->hist_planes;
  p.flag = s->flag;
  p.gate = 0;
  p.cand_slot = s->cand_slot;
  p.cand_vtx = s->cand_vtx;
  p.cand_choff = s->cand_choff;
  p.cand = s->cand;
  p.ncand = s->ncand;
  p.pair_u = s->pair_u;
  p.pair_m = s->pair_m;
  p.pair_n = s->pair_n;
  p.light = s->lightfin;
  p.fin = s->lightfin ? s->lightfin + p.words : nullptr;
  p.pull_records = s->pull_records;
  p.touched0 = s->touched;
  p.scanmap = s->touched + 3 * p.words;
  p.dead = g->dead;
  p.touched1 = s->touched + p.words;
  p.touched2 = s->touched + 2 * p.words;
  p.queue0 = s->queue;
  p.queue1 = s->queue + g->n;
  p.bigoff0 = s->bigoff;
  p.bigoff1 = s->bigoff + s->bcap;
  const int64_t nh = s->nhub > 0 ? s->nhub : 1;
  p.hub_slot = s->hub_slot;
  p.hub_vtx = s->hub_vtx;
  p.med_vtx = s->med_vtx;
  p.nmed = s->nmed;
  p.hub_choff = s->hub_choff;
  p.hub_of_chunk = s->hub_of_chunk;
  p.hub_chunk_order = s->hub_chunk_order;
  p.hub_cand = s->hub_cand;
  p.hub_found = s->hub_found;
  p.hub_done = s->hub_done;
  p.nhub = s->nhub;
  p.levels = p.parents = nullptr;
  p.lanes = nullptr;
  p.ctl = s->ctl;
  p.stats = g->d_stats;
  p.k = 0;
  p.resume = 0;
  p.max_rounds = 0x7fffffff;
  p.stop_on_finish = 0;
  p.finish_all = 0;
  p.direction = g->opt.direction == CG_DIR_TAU ? CG_DIR_AUTO : g->opt.direction;
  p.ms_alpha = g->opt.ms_alpha > 0 ? g->opt.ms_alpha : 4.f;
  p.level_cap = g->opt.level_cap > 0 ? g->opt.level_cap
                                     : (int)((g->n + 1) < 0x7fffffff ? g->n + 1 : 0x7fffffff);
  p.timeout_ns = (long long)(g->opt.wait_timeout_ms > 0 ? g->opt.wait_timeout_ms : 1000) * 1000000ll;
  for (int i = 0; i < kMsMaxLanes; ++i) p.roots[i] = 0;
  return p;
}

// Clean control block and hub candidates for a fresh launch on `s`.
template <int W>
inline int ms_reset(const MsState *s, cudaStream_t stream) {
  const int64_t nh = s->nhub > 0 ? s->nhub : 1;
  CG_CUDA(cudaMemsetAsync(s->ctl, 0, sizeof(MsCtl), stream));
  CG_CUDA(cudaMemsetAsync(s->flag, 0, sizeof(int), stream));
  if (s->cand)
    CG_CUDA(cudaMemsetAsync(s->cand, 0xff,
                            sizeof(uint32_t) * (size_t)(s->ncand > 0 ? s->ncand : 1) * 64 * W,
                            stream));
  CG_CUDA(cudaMemsetAsync(s->hub_cand, 0xff, sizeof(uint32_t) * (size_t)nh * 64 * W, stream));
  CG_CUDA(cudaMemsetAsync(s->hub_found, 0, sizeof(uint64_t) * (size_t)nh * W, stream));
  CG_CUDA(cudaMemsetAsync(s->hub_done, 0, sizeof(unsigned) * (size_t)nh, stream));
  return CG_OK;
}

// History launch of one batch (cg_msledger.cu): the rounds, then the scan,
// output and fix-up passes; sets *s->flag instead if the search outgrows the
// history.
int ms_ledger_pass(cg_graph *g, MsState *s, const int64_t *roots, int k, int32_t *d_levels,
                   int32_t *d_parents);

}  // namespace cg
