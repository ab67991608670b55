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
//   queue[2]     frontier vertices (any lane set): light from the front, big
//                (out-degree > kLightMax) from the back with edge prefix offsets
// Hubs (in-degree > kHubDeg; a fixed list per graph) never have their in-list
// walked by one warp: each round their in-list is cut into kHubChunk pieces
// scanned by different warps, which combine per-lane parent candidates with
// atomicMin in a small per-hub buffer; a finalize phase then writes the hub's
// outputs and queues it after the round's other discoveries.
//
// Pull round: every non-hub vertex with unvisited lanes whose search is still
// running scans its ascending in-list and takes, per lane, the first frontier
// source (the minimum), stopping once every wanted lane is found; hubs go
// through the chunks.  Push round: frontier vertices OR their masks into
// their out-neighbours' next masks (atomicOr); hub targets get parent
// candidates by atomicMin instead; a resolve phase scans each newly reached
// non-hub vertex's ascending in-list for its parents.
#include <cuda_runtime.h>
#include <string.h>

#include <new>

#include <vector>

#include "cg_ms.cuh"

namespace cg {

// Output of lane l for vertex v discovered in round `round` (level round + 1
// for a batch; relative to the lane's start round in a serving pool).
__device__ __forceinline__ void write_lane(const MsParams &p, int l, int64_t v, int32_t parent,
                                           int round) {
  if (p.lanes) {
    p.lanes->levels[l][v] = round + 1 - p.lanes->start[l];
    p.lanes->parents[l][v] = parent;
  } else {
    const int64_t at = (int64_t)l * p.n + v;
    p.levels[at] = round + 1;
    p.parents[at] = parent;
  }
}

// Writes level and parent of vertex v for every lane in `m`.
template <int W>
__device__ __forceinline__ void write_lanes(const MsParams &p, int64_t v, const Mask<W> &m,
                                            int32_t parent, int round) {
#pragma unroll
  for (int i = 0; i < W; ++i) {
    uint64_t bits = m.w[i];
    while (bits) {
      const int b = __ffsll((long long)bits) - 1;
      bits &= bits - 1;
      write_lane(p, i * 64 + b, v, parent, round);
    }
  }
}

// Warp-cooperative scan of in-list entries [s, e) of vertex v (all lanes call
// with the same arguments): 4 x 32 sources per step, their index and mask
// loads in flight together, taken 32 at a time in ascending order; for each
// lane bit found among 32 sources the lowest warp lane holding it -- the
// smallest source -- wins.  Stops once every wanted bit is found.  With
// hub >= 0 the winners go to the hub's candidate buffer by atomicMin;
// otherwise they are written as outputs.
template <int W>
__device__ Mask<W> warp_scan(const MsParams &p, int64_t v, int64_t s, int64_t e,
                             const Mask<W> &want, const uint64_t *cur, int level, int hub) {
  constexpr int G = 4;
  const int lane = lane_id();
  Mask<W> got = Mask<W>::zero();
  for (int64_t base = s; base < e; base += 32 * G) {
    int32_t u[G];
    Mask<W> f[G];
#pragma unroll
    for (int k = 0; k < G; ++k) {
      const int64_t i = base + 32 * k + lane;
      u[k] = i < e ? __ldg(p.in_idx + i) : -1;
    }
#pragma unroll
    for (int k = 0; k < G; ++k) f[k] = u[k] >= 0 ? ld_mask<W>(cur, u[k]) : Mask<W>::zero();
    bool done = false;
#pragma unroll
    for (int k = 0; k < G; ++k) {
      if (!done) {
        const Mask<W> fk = (f[k] & want).andnot(got);
        const Mask<W> F = warp_or<W>(fk);
        if (F.any()) {
          const Mask<W> mine = first_holder<W>(fk);
#pragma unroll
          for (int j = 0; j < W; ++j) {
            uint64_t bits = mine.w[j];
            while (bits) {
              const int b = __ffsll((long long)bits) - 1;
              bits &= bits - 1;
              if (hub >= 0)
                atomicMin(p.hub_cand + (int64_t)hub * (64 * W) + j * 64 + b, (unsigned)u[k]);
              else
                write_lane(p, j * 64 + b, v, u[k], level);
            }
          }
          got = got | F;
          done = got == want;
        }
      }
    }
    if (done) break;
  }
  return got;
}

// Thread-level scan of the same kind, for short in-lists.
template <int W>
__device__ __forceinline__ Mask<W> thread_scan(const MsParams &p, int64_t v, int64_t s, int64_t e,
                                               const Mask<W> &want, const uint64_t *cur,
                                               int level) {
  // four sources at a time: their index and mask loads are all in flight
  // together; the four are then taken in ascending order
  constexpr int G = 4;
  Mask<W> got = Mask<W>::zero();
  for (int64_t i0 = s; i0 < e; i0 += G) {
    int32_t u[G];
    Mask<W> m[G];
#pragma unroll
    for (int k = 0; k < G; ++k) u[k] = i0 + k < e ? __ldg(p.in_idx + i0 + k) : -1;
#pragma unroll
    for (int k = 0; k < G; ++k) m[k] = u[k] >= 0 ? ld_mask<W>(cur, u[k]) : Mask<W>::zero();
    bool done = false;
#pragma unroll
    for (int k = 0; k < G; ++k) {
      const Mask<W> f = (m[k] & want).andnot(got);
      if (f.any()) {
        write_lanes<W>(p, v, f, u[k], level);
        got = got | f;
        if (got == want) done = true;
      }
    }
    if (done) break;
  }
  return got;
}

// Scans a warp's 32 non-hub vertices: short in-lists one per thread, the
// others by the whole warp in turn.  want must be zero where no scan is due.
template <int W>
__device__ __forceinline__ Mask<W> scan_group(const MsParams &p, int64_t v, int64_t s, int64_t e,
                                              const Mask<W> &want, const uint64_t *cur,
                                              int level) {
  const bool need = want.any();
  const bool longer = need && (e - s) > kPullLight;
  Mask<W> got = Mask<W>::zero();
  if (need && !longer) got = thread_scan<W>(p, v, s, e, want, cur, level);
  unsigned hm = __ballot_sync(kMsFull, longer);
  while (hm) {
    const int j = __ffs(hm) - 1;
    hm &= hm - 1;
    const int64_t vj = __shfl_sync(kMsFull, v, j);
    const int64_t sj = __shfl_sync(kMsFull, s, j), ej = __shfl_sync(kMsFull, e, j);
    Mask<W> wj;
#pragma unroll
    for (int i = 0; i < W; ++i) wj.w[i] = __shfl_sync(kMsFull, want.w[i], j);
    const Mask<W> gj = warp_scan<W>(p, vj, sj, ej, wj, cur, level, -1);
    if (lane_id() == j) got = gj;
  }
  return got;
}

// Hub in-list chunks of a round: chunk c of hub h scans its slice for the
// wanted lanes (frozen for the round: nothing writes a hub's vis before its
// finalize), min-combining winners into the candidate buffer.
template <int W>
__device__ void hub_chunks(const MsParams &p, const uint64_t *cur, const Mask<W> &active,
                           int level) {
  const int nwarps = (gridDim.x * blockDim.x) >> 5;
  const unsigned nchunks = p.hub_choff[p.nhub];
  for (unsigned c = (unsigned)warp_id_global(); c < nchunks; c += (unsigned)nwarps) {
    const int h = (int)p.hub_of_chunk[c];
    const int32_t v = p.hub_vtx[h];
    const Mask<W> want = active.andnot(ld_mask<W>(p.vis, v));
    if (!want.any()) continue;
    const int64_t s = __ldg(p.in_off + v) + (int64_t)(c - p.hub_choff[h]) * kHubChunk;
    const int64_t e = min(s + (int64_t)kHubChunk, __ldg(p.in_off + v + 1));
    const Mask<W> got = warp_scan<W>(p, v, s, e, want, cur, level, h);
    if (lane_id() == 0) {
#pragma unroll
      for (int j = 0; j < W; ++j)
        if (got.w[j])
          atomicOr(reinterpret_cast<unsigned long long *>(p.hub_found + (int64_t)h * W + j),
                   (unsigned long long)got.w[j]);
    }
  }
}

// Hubs reached this round: outputs from the candidates, next mask, vis,
// queue (hub list of the next frontier); candidates reset for the next round.
template <int W>
__device__ void hub_finalize(const MsParams &p, int L, uint64_t *nxt, MsRound *Rn, MsAcc &acc) {
  const int lane = lane_id();
  const int nwarps = (gridDim.x * blockDim.x) >> 5;
  const int next_parity = (L + 1) & 1;
  int32_t *q = next_parity ? p.queue1 : p.queue0;
  uint32_t *boff = next_parity ? p.bigoff1 : p.bigoff0;
  for (int h = warp_id_global(); h < p.nhub; h += nwarps) {
    const Mask<W> found = ld_mask<W>(p.hub_found, h);
    if (!found.any()) continue;
    const int32_t v = p.hub_vtx[h];
#pragma unroll
    for (int j = 0; j < W; ++j) {
#pragma unroll
      for (int half = 0; half < 2; ++half) {
        const int b = lane + 32 * half;
        if ((found.w[j] >> b) & 1ull) {
          uint32_t *cand = p.hub_cand + (int64_t)h * (64 * W) + j * 64 + b;
          write_lane(p, j * 64 + b, v, (int32_t)*cand, L);
          *cand = 0xffffffffu;
        }
      }
    }
    int64_t deg = 0;
    if (lane == 0) {
      st_mask<W>(nxt, v, found);
      st_mask<W>(p.vis, v, ld_mask<W>(p.vis, v) | found);
      st_mask<W>(p.hub_found, h, Mask<W>::zero());
      acc.visits += (unsigned long long)found.popc();
      acc_lanes<W>(acc, found);
      deg = __ldg(p.out_off + v + 1) - __ldg(p.out_off + v);
    }
    // queued after every other vertex of the next frontier (a push round's
    // resolve phase only walks the queue as it stood before this phase)
    ms_enqueue(lane == 0, v, deg, q, p.n, boff, &Rn->nlight, &Rn->big, acc);
  }
}

// Pull round over every non-hub vertex with unvisited lanes whose search is
// still running (`active`), and over the hub chunks.
template <int W>
__device__ void ms_pull(const MsParams &p, int L, const uint64_t *cur, uint64_t *nxt,
                        const Mask<W> &active, MsRound *Rn, MsAcc &acc) {
  const int64_t nthreads = (int64_t)gridDim.x * blockDim.x;
  const int next_parity = (L + 1) & 1;
  int32_t *q = next_parity ? p.queue1 : p.queue0;
  uint32_t *boff = next_parity ? p.bigoff1 : p.bigoff0;
  // light vertices (in-degree <= kPullLight): one thread each
  for (int64_t base = (int64_t)blockIdx.x * blockDim.x + (threadIdx.x & ~31);
       base < p.n; base += nthreads) {
    const int64_t v = base + lane_id();
    Mask<W> want = Mask<W>::zero();
    Mask<W> seen = Mask<W>::zero();
    int64_t s = 0, e = 0;
    if (v < p.n) {
      seen = ld_mask<W>(p.vis, v);
      want = active.andnot(seen);
      if (want.any()) {
        s = __ldg(p.in_off + v);
        e = __ldg(p.in_off + v + 1);
        if (e - s > kPullLight) want = Mask<W>::zero();  // medium list or hub chunks
      }
    }
    if (!__ballot_sync(kMsFull, want.any())) continue;
    Mask<W> got = Mask<W>::zero();
    if (want.any()) got = thread_scan<W>(p, v, s, e, want, cur, L);
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
    ms_enqueue(claimed, (int32_t)v, deg, q, p.n, boff, &Rn->nlight, &Rn->big, acc);
  }
  // medium vertices (kPullLight < in-degree <= kHubDeg, a fixed list): one warp each
  const int nwarps = (gridDim.x * blockDim.x) >> 5;
  for (int64_t j = warp_id_global(); j < p.nmed; j += nwarps) {
    const int32_t v = p.med_vtx[j];
    const Mask<W> seen = ld_mask<W>(p.vis, v);
    const Mask<W> want = active.andnot(seen);
    if (!want.any()) continue;
    const Mask<W> got = warp_scan<W>(p, v, __ldg(p.in_off + v), __ldg(p.in_off + v + 1), want,
                                     cur, L, -1);
    const bool claimed = lane_id() == 0 && got.any();
    int64_t deg = 0;
    if (claimed) {
      st_mask<W>(nxt, v, got);
      st_mask<W>(p.vis, v, seen | got);
      acc.visits += (unsigned long long)got.popc();
      acc_lanes<W>(acc, got);
      deg = __ldg(p.out_off + v + 1) - __ldg(p.out_off + v);
    }
    ms_enqueue(claimed, v, deg, q, p.n, boff, &Rn->nlight, &Rn->big, acc);
  }
  if (p.nhub > 0) hub_chunks<W>(p, cur, active, L);
}

// After a push round: every newly reached non-hub vertex merges its lanes
// into vis and finds each lane's parent by scanning its ascending in-list
// (it ends: every lane has a frontier source there).  Hubs are finalized from
// their candidates.
template <int W>
__device__ void ms_resolve(const MsParams &p, int L, const uint64_t *cur, uint64_t *nxt,
                           MsRound *Rn, MsAcc &acc) {
  const int64_t nthreads = (int64_t)gridDim.x * blockDim.x;
  const int next_parity = (L + 1) & 1;
  const int32_t *q = next_parity ? p.queue1 : p.queue0;
  const int64_t nl = *(volatile unsigned *)&Rn->res_light;
  const int64_t nbg = *(volatile unsigned *)&Rn->res_big;
  const int64_t total = nl + nbg;
  // every entry: merge into vis; short in-lists scanned by their thread
  for (int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; j < total; j += nthreads) {
    const int64_t v = j < nl ? q[j] : q[p.n - 1 - (j - nl)];
    const Mask<W> nw = ld_mask<W>(nxt, v);
    st_mask<W>(p.vis, v, ld_mask<W>(p.vis, v) | nw);
    acc.visits += (unsigned long long)nw.popc();
    acc_lanes<W>(acc, nw);
    const int64_t s = __ldg(p.in_off + v), e = __ldg(p.in_off + v + 1);
    if (e - s <= kPullLight) thread_scan<W>(p, v, s, e, nw, cur, L);
  }
  // longer in-lists: one warp per entry
  const int nwarps = (gridDim.x * blockDim.x) >> 5;
  for (int64_t j = warp_id_global(); j < total; j += nwarps) {
    const int64_t v = j < nl ? q[j] : q[p.n - 1 - (j - nl)];
    const int64_t s = __ldg(p.in_off + v), e = __ldg(p.in_off + v + 1);
    if (e - s <= kPullLight) continue;
    warp_scan<W>(p, v, s, e, ld_mask<W>(nxt, v), cur, L, -1);
  }
  if (p.nhub > 0) hub_finalize<W>(p, L, nxt, Rn, acc);
}

// End of round L, run by the block that arrives last: termination (no lane
// has a frontier), lanes whose search ended this round, the direction of the
// next round, statistics, and the reset of the record round L + 1 fills.
template <int W>
__device__ unsigned ms_decide(const MsParams &p, int L, int dir, int ran) {
  MsCtl *ctl = p.ctl;
  const MsRound *Rc = &ctl->rec[L % kRing];
  const MsRound *Rn = &ctl->rec[(L + 1) % kRing];
  unsigned long long nf = 0, visits = 0, mf = 0;
#pragma unroll
  for (int i = 0; i < kCounterShards; ++i) {
    nf += *(volatile const unsigned long long *)&Rn->nf[i];
    visits += *(volatile const unsigned long long *)&Rn->visits[i];
    mf += *(volatile const unsigned long long *)&Rn->mf[i];
  }
  bool finished = false;
#pragma unroll
  for (int i = 0; i < 2; ++i) {
    const unsigned long long ended = *(volatile const unsigned long long *)&Rc->lanes[i] &
                                     ~*(volatile const unsigned long long *)&Rn->lanes[i];
    if (ended) {
      ctl->done[i] |= ended;
      finished = true;
    }
  }
  cg_stats *st = p.stats;
  const long long now = global_ns();
  if (ran < CG_HISTORY) {
    st->nf_history[ran] = (int64_t)visits;
    st->direction_history[ran] = dir;
    st->round_ns[ran] = now - ctl->t_round;
  }
  ctl->t_round = now;
  if (dir == 1) ctl->pull_rounds += 1;
  ctl->visited += visits;
  bool stop = nf == 0 || ran + 1 >= p.max_rounds || (p.stop_on_finish && finished);
  if (nf != 0 && L + 1 >= p.level_cap) {
    atomicCAS(&ctl->status, 0, (int)CG_ERR_LEVEL_CAP);
    stop = true;
  }
  int next;
  if (p.direction == CG_DIR_TOPDOWN)
    next = 0;
  else if (p.direction == CG_DIR_BOTTOMUP)
    next = 1;
  else
    next = ((double)mf * (double)p.ms_alpha > (double)p.nnz) ? 1 : 0;
  if (next != dir) ctl->switches += 1;
  ctl->L = L + 1;
  ctl->dir = next;
  MsRound *Rz = &ctl->rec[(L + 2) % kRing];  // last used in round L - 2
  for (int i = 0; i < kCounterShards; ++i) Rz->nf[i] = Rz->visits[i] = Rz->mf[i] = 0;
  Rz->big = 0;
  Rz->res_light = Rz->res_big = 0;
  Rz->nlight = Rz->work = 0;
  Rz->lanes[0] = Rz->lanes[1] = 0;
  if (stop) {
    const int rounds = ran + 1;
    st->status = *(volatile int *)&ctl->status;
    st->rounds = rounds;
    st->visited = (int64_t)ctl->visited;
    st->pull_rounds = ctl->pull_rounds;
    st->switches = ctl->switches;
    st->history_len = rounds < CG_HISTORY ? rounds : CG_HISTORY;
    st->device_ms = 0.f;
  }
  return (stop ? kMsStop : 0u) | (next ? kMsNextPull : 0u);
}

template <int W>
struct MsRoundDecision {
  const MsParams *p;
  int L, dir, ran;
  __device__ unsigned operator()() const { return ms_decide<W>(*p, L, dir, ran); }
};

// At the wait between a push round's push and resolve phases: the queue as
// it stands then (hubs finalized during resolve are appended after it).
struct ResolveSnapshot {
  MsRound *R;
  __device__ unsigned operator()() const {
    R->res_light = *(volatile unsigned *)&R->nlight;
    R->res_big = (unsigned)(*(volatile unsigned long long *)&R->big >> 32);
    return 0u;
  }
};

struct MsSetupDecision {
  MsCtl *ctl;
  cg_stats *st;
  __device__ unsigned operator()() const {
    const long long now = global_ns();
    st->setup_ns = now - ctl->t_start;
    ctl->t_round = now;
    ctl->pull_rounds = 0;
    ctl->switches = 0;
    ctl->exited = 0u;
    return 0u;
  }
};

// One launch runs rounds until every lane's search has ended, or max_rounds
// rounds, or (stop_on_finish) a round in which some lane's search ended.
// A fresh launch clears the lane state and seeds roots[0..k); a resumed one
// (a serving pool) continues at round ctl->L with the lanes admitted since.
template <int W>
__global__ void __launch_bounds__(kMsBlock, 2) msbfs_persistent(MsParams p) {
  __shared__ unsigned s_payload;
  if (p.gate && *(volatile int *)p.flag == 0) return;  // the ledger pass succeeded
  MsCtl *ctl = p.ctl;
  const int64_t gtid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t nthreads = (int64_t)gridDim.x * blockDim.x;
  const bool leader = blockIdx.x == 0 && threadIdx.x == 0;
  if (leader) ctl->t_start = global_ns();
  uint64_t *fr[3] = {p.fr0, p.fr1, p.fr2};

  bool ok = true;
  if (!p.resume) {
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
    ok = grid_wait(&ctl->wait, &ctl->status, p.timeout_ns);
    // seed: lane i starts at roots[i] (block 0)
    if (ok && blockIdx.x == 0 && threadIdx.x < p.k) {
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
        if (deg <= kLightMax) {
          p.queue0[atomicAdd(&R0->nlight, 1u)] = r;
        } else {
          // roots are queued one by one: a 64-bit add keeps index and offset paired
          const unsigned long long old =
              atomicAdd(&R0->big, (1ull << 32) | (unsigned long long)deg);
          p.queue0[p.n - 1 - (int64_t)(old >> 32)] = r;
          p.bigoff0[old >> 32] = (unsigned)old;
        }
        atomicAdd(&R0->nf[0], 1ull);
        atomicAdd(&R0->mf[0], (unsigned long long)deg);
      }
      if (i == 0) {
        const Mask<W> a0 = lane_mask<W>(p.k);
        ctl->rec[0].lanes[0] = a0.w[0];
        ctl->rec[0].lanes[1] = W == 2 ? a0.w[W - 1] : 0ull;
        ctl->visited = (unsigned long long)p.k;
        ctl->L = 0;
        ctl->dir = 0;
      }
    }
  }
  if (ok) {
    __syncthreads();
    if (threadIdx.x == 0)
      s_payload = arrive_and_wait(&ctl->wait, &ctl->status, p.timeout_ns, 0u,
                                  MsSetupDecision{ctl, p.stats});
    __syncthreads();
    ok = s_payload != kWaitFailed;
  }

  int L = ctl->L, dir = ctl->dir;  // ordered by the wait above
  int ran = 0;
  MsAcc acc, tot;
  while (ok) {
    const uint64_t *cur = fr[L % 3];
    uint64_t *nxt = fr[(L + 1) % 3];
    uint64_t *old = fr[(L + 2) % 3];
    uint32_t *touched = (L & 1) ? p.touched1 : p.touched0;
    uint32_t *touched_next = (L & 1) ? p.touched0 : p.touched1;
    MsRound *Rc = &ctl->rec[L % kRing];
    MsRound *Rn = &ctl->rec[(L + 1) % kRing];
    // F_{L-1} and last round's touched bits are no longer read by anyone
    for (int64_t i = gtid; i < p.n * W; i += nthreads) old[i] = 0;
    for (int64_t w = gtid; w < p.words; w += nthreads) touched_next[w] = 0;
    if (dir == 1) {
      Mask<W> active;
#pragma unroll
      for (int i = 0; i < W; ++i) active.w[i] = *(volatile unsigned long long *)&Rc->lanes[i];
      ms_pull<W>(p, L, cur, nxt, active, Rn, acc);
      if (p.nhub > 0) {
        if (!(ok = grid_wait(&ctl->wait, &ctl->status, p.timeout_ns))) break;
        hub_finalize<W>(p, L, nxt, Rn, acc);
      }
    } else {
      ms_push<W>(p, L, cur, nxt, touched, Rc, Rn, acc);
      __syncthreads();
      if (threadIdx.x == 0)
        s_payload = arrive_and_wait(&ctl->wait, &ctl->status, p.timeout_ns, 0u,
                                    ResolveSnapshot{Rn});
      __syncthreads();
      if (s_payload == kWaitFailed) {
        ok = false;
        break;
      }
      ms_resolve<W>(p, L, cur, nxt, Rn, acc);
    }
    ms_block_totals(acc, tot);
    if (threadIdx.x == 0) {
      const int sh = blockIdx.x % kCounterShards;
      if (tot.nf) atomicAdd(&Rn->nf[sh], tot.nf);
      if (tot.visits) atomicAdd(&Rn->visits[sh], tot.visits);
      if (tot.mf) atomicAdd(&Rn->mf[sh], tot.mf);
      if (tot.lanes[0]) atomicOr(&Rn->lanes[0], tot.lanes[0]);
      if (tot.lanes[1]) atomicOr(&Rn->lanes[1], tot.lanes[1]);
      s_payload = arrive_and_wait(&ctl->wait, &ctl->status, p.timeout_ns, 0u,
                                  MsRoundDecision<W>{&p, L, dir, ran});
    }
    __syncthreads();
    const unsigned payload = s_payload;
    if (payload == kWaitFailed) {
      ok = false;
      break;
    }
    if (payload & kMsStop) break;
    dir = (payload & kMsNextPull) ? 1 : 0;
    ++L;
    ++ran;
  }
  // batch: unreached lanes get level and parent -1 (each (lane, vertex) is
  // written once); a serving pool does this per lane when the lane is done
  if (ok && p.finish_all) {
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
  if (leader && !ok) p.stats->status = *(volatile int *)&ctl->status;
  // the last block out records the time from the end of the last round
  if (ok) {
    __syncthreads();
    if (threadIdx.x == 0 && atomicAdd(&ctl->exited, 1u) + 1u == gridDim.x)
      p.stats->finish_ns = global_ns() - *(volatile long long *)&ctl->t_round;
  }
}

// ---------------------------------------------------------------------------
// per-graph hub list: vertices of in-degree > kHubDeg, their chunk prefix
// per-graph vertex lists by in-degree: hubs (> kHubDeg) with their slot map,
// and medium vertices (kPullLight, kHubDeg]
__global__ void hub_mark_kernel(int64_t n, const int64_t *__restrict__ in_off, int32_t *hub_slot,
                                int32_t *hub_vtx, int32_t *med_vtx, unsigned *count) {
  for (int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; v < n;
       v += (int64_t)gridDim.x * blockDim.x) {
    const int64_t d = in_off[v + 1] - in_off[v];
    int32_t slot = -1;
    if (d > kHubDeg) {
      slot = (int32_t)atomicAdd(count, 1u);
      hub_vtx[slot] = (int32_t)v;
    } else if (d > kPullLight) {
      med_vtx[atomicAdd(count + 1, 1u)] = (int32_t)v;
    }
    hub_slot[v] = slot;
  }
}

__global__ void hub_chunks_kernel(int nhub, const int64_t *__restrict__ in_off,
                                  const int32_t *__restrict__ hub_vtx, uint32_t *chunks) {
  for (int h = blockIdx.x * blockDim.x + threadIdx.x; h < nhub; h += gridDim.x * blockDim.x) {
    const int32_t v = hub_vtx[h];
    chunks[h] = (uint32_t)((in_off[v + 1] - in_off[v] + kHubChunk - 1) / kHubChunk);
  }
}

static void ms_free_state(MsState *s) {
  if (!s) return;
  cudaFree(s->bits);
  cudaFree(s->touched);
  cudaFree(s->queue);
  cudaFree(s->bigoff);
  cudaFree(s->hub_slot);
  cudaFree(s->hub_vtx);
  cudaFree(s->med_vtx);
  cudaFree(s->hub_choff);
  cudaFree(s->hub_of_chunk);
  cudaFree(s->hub_chunk_order);
  cudaFree(s->hub_cand);
  cudaFree(s->hub_found);
  cudaFree(s->hub_done);
  cudaFree(s->ctl);
  cudaFree(s->flag);
  cudaFree(s->cand_slot);
  cudaFree(s->cand_vtx);
  cudaFree(s->cand_choff);
  cudaFree(s->cand);
  cudaFree(s->pair_u);
  cudaFree(s->pair_m);
  cudaFree(s->pair_n);
  cudaFree(s->lightfin);
  delete s;
}

void msbfs_release(cg_graph *g) {
  ms_free_state(reinterpret_cast<MsState *>(g->ms_ctl));
  g->ms_ctl = nullptr;
  cudaFree(g->ms_levels);
  cudaFree(g->ms_parents);
  g->ms_levels = g->ms_parents = nullptr;
  g->ms_out_cap = 0;
  g->ms_lane_words = 0;
}

int64_t bfs_big_capacity(int64_t n, int64_t nnz);

static int ms_build_hubs(cg_graph *g, MsState *s) {
  const int64_t cap = g->nnz / (kHubDeg + 1) + 1;
  int64_t mcap = g->nnz / (kPullLight + 1) + 1;
  if (mcap > g->n) mcap = g->n;
  unsigned *d_count = nullptr;
  if (cudaMalloc(&s->hub_slot, sizeof(int32_t) * (size_t)g->n) != cudaSuccess ||
      cudaMalloc(&s->hub_vtx, sizeof(int32_t) * (size_t)cap) != cudaSuccess ||
      cudaMalloc(&s->med_vtx, sizeof(int32_t) * (size_t)mcap) != cudaSuccess ||
      cudaMalloc(&d_count, 2 * sizeof(unsigned)) != cudaSuccess) {
    cudaFree(d_count);
    return CG_ERR_OUT_OF_MEMORY;
  }
  int rc = CG_OK;
  do {
    cudaError_t e = cudaMemsetAsync(d_count, 0, 2 * sizeof(unsigned), g->stream);
    if (e != cudaSuccess) { rc = cuda_fail(e, "hub count"); break; }
    int blocks = (int)((g->n + 255) / 256);
    if (blocks > g->num_sms * 16) blocks = g->num_sms * 16;
    hub_mark_kernel<<<blocks, 256, 0, g->stream>>>(g->n, g->in_off, s->hub_slot, s->hub_vtx,
                                                    s->med_vtx, d_count);
    unsigned counts[2] = {0u, 0u};
    e = cudaMemcpyAsync(counts, d_count, 2 * sizeof(unsigned), cudaMemcpyDeviceToHost, g->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(g->stream);
    if (e != cudaSuccess) { rc = cuda_fail(e, "hub mark"); break; }
    const unsigned nhub = counts[0];
    s->nhub = (int)nhub;
    s->nmed = counts[1];
    const size_t nh = nhub > 0 ? nhub : 1;
    if (cudaMalloc(&s->hub_choff, sizeof(uint32_t) * (nh + 1)) != cudaSuccess ||
        cudaMalloc(&s->hub_cand, sizeof(uint32_t) * nh * 64 * s->lane_words) != cudaSuccess ||
        cudaMalloc(&s->hub_found, sizeof(uint64_t) * nh * s->lane_words) != cudaSuccess ||
        cudaMalloc(&s->hub_done, sizeof(unsigned) * nh) != cudaSuccess) {
      rc = CG_ERR_OUT_OF_MEMORY;
      break;
    }
    uint32_t *chunks = nullptr;
    if (cudaMalloc(&chunks, sizeof(uint32_t) * nh) != cudaSuccess) {
      rc = CG_ERR_OUT_OF_MEMORY;
      break;
    }
    if (nhub) hub_chunks_kernel<<<(nhub + 255) / 256, 256, 0, g->stream>>>(nhub, g->in_off,
                                                                          s->hub_vtx, chunks);
    uint32_t *h_chunks = new uint32_t[nh + 1];
    h_chunks[0] = 0;
    e = cudaMemcpyAsync(h_chunks + 1, chunks, sizeof(uint32_t) * nhub, cudaMemcpyDeviceToHost,
                        g->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(g->stream);
    uint32_t *h_owner = nullptr;
    size_t nchunks = 0;
    if (e == cudaSuccess) {
      for (unsigned h = 0; h < nhub; ++h) h_chunks[h + 1] += h_chunks[h];
      // chunk -> hub, so a work item finds its hub with one load
      nchunks = h_chunks[nhub];
      h_owner = new uint32_t[2 * (nchunks ? nchunks : 1)];
      uint32_t *h_order = h_owner + (nchunks ? nchunks : 1);
      for (unsigned h = 0; h < nhub; ++h)
        for (uint32_t c = h_chunks[h]; c < h_chunks[h + 1]; ++c) h_owner[c] = h;
      // every hub's first chunk, then every hub's second, ...: a pull round's
      // later chunks mostly start after a hub's earlier ones are done
      // (counting sort of the chunks by their rank within the hub)
      uint32_t maxr = 0;
      for (unsigned h = 0; h < nhub; ++h)
        maxr = h_chunks[h + 1] - h_chunks[h] > maxr ? h_chunks[h + 1] - h_chunks[h] : maxr;
      std::vector<uint32_t> at((size_t)maxr + 1, 0u);
      for (size_t c = 0; c < nchunks; ++c) ++at[c - h_chunks[h_owner[c]] + 1];
      for (uint32_t r = 1; r <= maxr; ++r) at[r] += at[r - 1];
      for (size_t c = 0; c < nchunks; ++c) h_order[at[c - h_chunks[h_owner[c]]]++] = (uint32_t)c;
      if (cudaMalloc(&s->hub_of_chunk, sizeof(uint32_t) * (nchunks ? nchunks : 1)) != cudaSuccess ||
          cudaMalloc(&s->hub_chunk_order, sizeof(uint32_t) * (nchunks ? nchunks : 1)) !=
              cudaSuccess)
        rc = CG_ERR_OUT_OF_MEMORY;
      if (!rc) e = cudaMemcpyAsync(s->hub_choff, h_chunks, sizeof(uint32_t) * (nhub + 1),
                                   cudaMemcpyHostToDevice, g->stream);
      if (!rc && e == cudaSuccess && nchunks)
        e = cudaMemcpyAsync(s->hub_of_chunk, h_owner, sizeof(uint32_t) * nchunks,
                            cudaMemcpyHostToDevice, g->stream);
      if (!rc && e == cudaSuccess && nchunks)
        e = cudaMemcpyAsync(s->hub_chunk_order, h_order, sizeof(uint32_t) * nchunks,
                            cudaMemcpyHostToDevice, g->stream);
      if (!rc && e == cudaSuccess) e = cudaStreamSynchronize(g->stream);
    }
    delete[] h_chunks;
    delete[] h_owner;
    if (rc) {
      cudaFree(chunks);
      break;
    }
    g->device_bytes += 2 * sizeof(uint32_t) * nchunks;
    cudaFree(chunks);
    if (e != cudaSuccess) { rc = cuda_fail(e, "hub chunks"); break; }
    g->device_bytes += sizeof(int32_t) * g->n + sizeof(int32_t) * (cap + mcap) +
                       nh * (sizeof(uint32_t) * (1 + 64 * s->lane_words + 4 + 1) +
                             sizeof(uint64_t) * s->lane_words);
  } while (0);
  cudaFree(d_count);
  return rc;
}

__global__ void slot_map_kernel(int count, const int32_t *__restrict__ vtx, int32_t *slot) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < count; i += gridDim.x * blockDim.x)
    slot[vtx[i]] = i;
}

// Bit v of light[w]: vertex v = 32 w + b has in-degree 1 .. kPullLight (the
// vertices a ledger pull round scans one thread each); *light_edges sums
// their in-degrees.
__global__ void light_map_kernel(int64_t n, int64_t words, const int64_t *__restrict__ in_off,
                                 uint32_t *light, unsigned long long *light_edges) {
  unsigned long long e = 0;
  for (int64_t w = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; w < words;
       w += (int64_t)gridDim.x * blockDim.x) {
    uint32_t m = 0;
    for (int b = 0; b < 32; ++b) {
      const int64_t v = w * 32 + b;
      if (v >= n) break;
      const int64_t d = in_off[v + 1] - in_off[v];
      if (d >= 1 && d <= kPullLight) {
        m |= 1u << b;
        e += (unsigned long long)d;
      }
    }
    light[w] = m;
  }
  if (e) atomicAdd(light_edges, e);
}

// Parent-candidate slots of the output pass of a ledger batch: every vertex of
// in-degree > kPullLight (the medium list, then the hubs) gets a slot of 64 W
// candidates and its in-list is cut into kHubChunk-entry chunks.
static int ms_build_cands(cg_graph *g, MsState *s) {
  const int64_t ncand = s->nmed + s->nhub;
  s->ncand = (int)ncand;
  const size_t nc = ncand > 0 ? (size_t)ncand : 1;
  if (cudaMalloc(&s->cand_slot, sizeof(int32_t) * (size_t)g->n) != cudaSuccess ||
      cudaMalloc(&s->cand_vtx, sizeof(int32_t) * nc) != cudaSuccess ||
      cudaMalloc(&s->cand_choff, sizeof(uint32_t) * (nc + 1)) != cudaSuccess ||
      cudaMalloc(&s->cand, sizeof(uint32_t) * nc * 64 * s->lane_words) != cudaSuccess ||
      cudaMalloc(&s->pair_u, sizeof(int32_t) * kRecords * (size_t)g->n) != cudaSuccess ||
      cudaMalloc(&s->pair_m, sizeof(uint64_t) * kRecords * (size_t)g->n * s->lane_words) !=
          cudaSuccess ||
      cudaMalloc(&s->pair_n, (size_t)((g->n + 3) / 4) * 4) != cudaSuccess ||
      cudaMalloc(&s->lightfin, sizeof(uint32_t) * 2 * (size_t)((g->n + 31) / 32)) != cudaSuccess)
    return CG_ERR_OUT_OF_MEMORY;
  g->device_bytes += (sizeof(int32_t) + sizeof(uint64_t) * s->lane_words) * kRecords * g->n + g->n +
                     sizeof(uint32_t) * 2 * ((g->n + 31) / 32);
  {
    // pull rounds may take all kRecords records where light vertices hold
    // under half of the edges (their parents are a few hubs: R-MAT), else
    // kPairs, leaving room for the scan pass to merge later hits into
    // records of the same source (graphs of light vertices only: each is
    // reached over many rounds, from the same few in-neighbours)
    const int64_t words = (g->n + 31) / 32;
    const int64_t blocks = (words + 255) / 256;
    unsigned long long *d_le = nullptr, le = 0;
    CG_CUDA(cudaMalloc(&d_le, sizeof(unsigned long long)));
    cudaError_t e = cudaMemsetAsync(d_le, 0, sizeof(unsigned long long), g->stream);
    if (e == cudaSuccess) {
      light_map_kernel<<<(unsigned)(blocks < 4096 ? blocks : 4096), 256, 0, g->stream>>>(
          g->n, words, g->in_off, s->lightfin, d_le);
      e = cudaGetLastError();
    }
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(&le, d_le, sizeof(le), cudaMemcpyDeviceToHost, g->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(g->stream);
    cudaFree(d_le);
    if (e != cudaSuccess) return cuda_fail(e, "light-vertex map");
    s->pull_records = 2 * le < (unsigned long long)g->nnz ? kRecords : kPairs;
  }
  CG_CUDA(cudaMemsetAsync(s->cand_slot, 0xff, sizeof(int32_t) * (size_t)g->n, g->stream));
  if (s->nmed)
    CG_CUDA(cudaMemcpyAsync(s->cand_vtx, s->med_vtx, sizeof(int32_t) * (size_t)s->nmed,
                            cudaMemcpyDeviceToDevice, g->stream));
  if (s->nhub)
    CG_CUDA(cudaMemcpyAsync(s->cand_vtx + s->nmed, s->hub_vtx, sizeof(int32_t) * (size_t)s->nhub,
                            cudaMemcpyDeviceToDevice, g->stream));
  uint32_t *chunks = nullptr;
  CG_CUDA(cudaMalloc(&chunks, sizeof(uint32_t) * nc));
  int rc = CG_OK;
  uint32_t *h = new (std::nothrow) uint32_t[nc + 1];
  do {
    if (!h) { rc = CG_ERR_OUT_OF_MEMORY; break; }
    h[0] = 0;
    if (ncand > 0) {
      const int blocks = (int)((ncand + 255) / 256 < g->num_sms * 16 ? (ncand + 255) / 256
                                                                      : g->num_sms * 16);
      slot_map_kernel<<<blocks, 256, 0, g->stream>>>((int)ncand, s->cand_vtx, s->cand_slot);
      hub_chunks_kernel<<<blocks, 256, 0, g->stream>>>((int)ncand, g->in_off, s->cand_vtx, chunks);
      cudaError_t e = cudaMemcpyAsync(h + 1, chunks, sizeof(uint32_t) * (size_t)ncand,
                                      cudaMemcpyDeviceToHost, g->stream);
      if (e == cudaSuccess) e = cudaStreamSynchronize(g->stream);
      if (e != cudaSuccess) { rc = cuda_fail(e, "candidate chunks"); break; }
      for (int64_t i = 0; i < ncand; ++i) h[i + 1] += h[i];
    }
    cudaError_t e = cudaMemcpyAsync(s->cand_choff, h, sizeof(uint32_t) * (size_t)(ncand + 1),
                                    cudaMemcpyHostToDevice, g->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(g->stream);
    if (e != cudaSuccess) { rc = cuda_fail(e, "candidate chunks"); break; }
    g->device_bytes += sizeof(int32_t) * (g->n + nc) + sizeof(uint32_t) * (nc + 1) +
                       sizeof(uint32_t) * nc * 64 * s->lane_words;
  } while (0);
  delete[] h;
  cudaFree(chunks);
  return rc;
}

// Lane state for one batched search stream (a graph's batch state or a pool).
static int ms_create_state(cg_graph *g, int lane_words, int hist_planes, MsState **out) {
  MsState *s = new MsState();
  s->lane_words = lane_words;
  s->bcap = bfs_big_capacity(g->n, g->nnz);
  s->hist_planes = hist_planes > 3 ? hist_planes : 3;
  const size_t bits = sizeof(uint64_t) * (1 + (size_t)s->hist_planes) * (size_t)g->n * lane_words;
  const size_t words = (size_t)((g->n + 31) / 32);
  if (cudaMalloc(&s->bits, bits) != cudaSuccess ||
      cudaMalloc(&s->touched, sizeof(uint32_t) * 4 * words) != cudaSuccess ||
      cudaMalloc(&s->queue, sizeof(int32_t) * 2 * (size_t)g->n) != cudaSuccess ||
      cudaMalloc(&s->bigoff, sizeof(uint32_t) * 2 * (size_t)s->bcap) != cudaSuccess ||
      cudaMalloc(&s->ctl, sizeof(MsCtl)) != cudaSuccess ||
      cudaMalloc(&s->flag, sizeof(int)) != cudaSuccess) {
    ms_free_state(s);
    return CG_ERR_OUT_OF_MEMORY;
  }
  int rc = ms_build_hubs(g, s);
  if (!rc && s->hist_planes >= 4) rc = ms_build_cands(g, s);
  if (rc) {
    ms_free_state(s);
    return rc;
  }
  g->device_bytes += bits + sizeof(uint32_t) * 4 * words + sizeof(int32_t) * 2 * g->n +
                     sizeof(uint32_t) * 2 * s->bcap + sizeof(MsCtl);
  *out = s;
  return CG_OK;
}

// Frontier planes of a graph's batch state: the round history F_0 .. F_D of
// the ledger kernel when the option allows it and memory holds at least four
// planes (D = 64 at most, within a quarter of free memory and 16 GiB), else
// the three rotating planes of the direct kernel.
static int ms_history_planes(const cg_graph *g, int lane_words) {
  const int want = g->opt.ms_history;
  if (want < 0) return 3;
  const size_t plane = sizeof(uint64_t) * (size_t)g->n * (size_t)lane_words;
  size_t free_b = 0, total_b = 0;
  if (cudaMemGetInfo(&free_b, &total_b) != cudaSuccess) return 3;
  size_t budget = free_b / 4;
  const size_t cap = (size_t)16 << 30;
  if (budget > cap) budget = cap;
  long long planes = (long long)(budget / plane);
  // at most CG_HISTORY + 1 planes: the output pass reads each level's round
  // direction from the statistics' history
  const long long most = want > 0 && want < CG_HISTORY ? (long long)want + 1 : CG_HISTORY + 1;
  if (planes > most) planes = most;
  return planes >= 4 ? (int)planes : 3;
}

static int ms_alloc_state(cg_graph *g, int lane_words) {
  int rc0 = dead_prepare(g);
  if (rc0) return rc0;
  MsState *old = reinterpret_cast<MsState *>(g->ms_ctl);
  if (old && g->ms_lane_words == lane_words && old->hist_opt == g->opt.ms_history) return CG_OK;
  rc0 = refuse_setup_in_capture(g);
  if (rc0) return rc0;
  ms_free_state(old);
  g->ms_ctl = nullptr;
  MsState *s = nullptr;
  int rc = ms_create_state(g, lane_words, ms_history_planes(g, lane_words), &s);
  if (rc) return rc;
  s->hist_opt = g->opt.ms_history;
  g->ms_ctl = s;
  g->ms_lane_words = lane_words;
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
static int ms_launch(const cg_graph *g, const MsParams &p, cudaStream_t stream) {
  int block = g->opt.block_size > 0 ? g->opt.block_size : kMsBlock;
  if (block > kMsBlock) block = kMsBlock;
  block = (block / 32) * 32;
  if (block < 128) block = 128;  // seeding uses threads 0..k-1 of block 0
  int per_sm = 0;
  CG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, msbfs_persistent<W>, block, 0));
  if (per_sm <= 0) return CG_ERR_NOT_SUPPORTED;
  if (g->opt.blocks_per_sm > 0 && g->opt.blocks_per_sm < per_sm) per_sm = g->opt.blocks_per_sm;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(per_sm * g->num_sms);
  cfg.blockDim = dim3(block);
  cfg.dynamicSmemBytes = 0;
  cfg.stream = stream;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeCooperative;
  attr[0].val.cooperative = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  CG_CUDA(cudaLaunchKernelEx(&cfg, msbfs_persistent<W>, p));
  return CG_OK;
}

template <int W>
static int ms_launch_pass(cg_graph *g, MsState *s, const int64_t *roots, int k,
                          int32_t *d_levels, int32_t *d_parents) {
  MsParams p = ms_params<W>(g, s);
  p.levels = d_levels;
  p.parents = d_parents;
  p.k = k;
  p.finish_all = 1;
  for (int i = 0; i < kMsMaxLanes; ++i) p.roots[i] = i < k ? (int32_t)roots[i] : 0;
  int rc = ms_reset<W>(s, g->stream);
  if (rc) return rc;
  return ms_launch<W>(g, p, g->stream);
}

// The direct kernel as the fallback of a ledger pass: it returns at once
// unless the ledger kernel set the overflow flag (the output pass has then
// cleared the control block).
template <int W>
static int ms_launch_gated(cg_graph *g, MsState *s, const int64_t *roots, int k,
                           int32_t *d_levels, int32_t *d_parents) {
  MsParams p = ms_params<W>(g, s);
  p.levels = d_levels;
  p.parents = d_parents;
  p.k = k;
  p.finish_all = 1;
  p.gate = 1;
  for (int i = 0; i < kMsMaxLanes; ++i) p.roots[i] = i < k ? (int32_t)roots[i] : 0;
  return ms_launch<W>(g, p, g->stream);
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
    if (s->hist_planes >= 4) {
      // rounds on masks, then the scan, output and fix-up passes; the direct
      // kernel runs only if the search outgrew the history
      rc = ms_ledger_pass(g, s, roots + b, kk, lv, pa);
      if (!rc) rc = W == 2 ? ms_launch_gated<2>(g, s, roots + b, kk, lv, pa)
                           : ms_launch_gated<1>(g, s, roots + b, kk, lv, pa);
    } else {
      rc = W == 2 ? ms_launch_pass<2>(g, s, roots + b, kk, lv, pa)
                  : ms_launch_pass<1>(g, s, roots + b, kk, lv, pa);
    }
    if (rc) return rc;
  }
  return CG_OK;
}


// ---------------------------------------------------------------------------
// Serving pools: continuous batching over the lanes of one resumable launch.
struct Admission {
  int count;
  int32_t lane[kMsMaxLanes];
  int32_t root[kMsMaxLanes];
};

// Seeds admitted lanes into the frontier of the next round (ctl->L): visited
// and frontier bit, level 0 / parent root, the root queued once for a push
// round, the lane marked active.  One thread, in order, so roots shared by
// several admissions are queued once.
template <int W>
__global__ void pool_admit_kernel(MsParams p, Admission a) {
  if (blockIdx.x != 0 || threadIdx.x != 0) return;
  MsCtl *ctl = p.ctl;
  const int L = ctl->L;
  uint64_t *fr[3] = {p.fr0, p.fr1, p.fr2};
  uint64_t *cur = fr[L % 3];
  MsRound *Rc = &ctl->rec[L % kRing];
  int32_t *q = (L & 1) ? p.queue1 : p.queue0;
  uint32_t *boff = (L & 1) ? p.bigoff1 : p.bigoff0;
  for (int i = 0; i < a.count; ++i) {
    const int l = a.lane[i];
    const int32_t r = a.root[i];
    const Mask<W> before = ld_mask<W>(cur, r);
    p.vis[(int64_t)r * W + (l >> 6)] |= 1ull << (l & 63);
    cur[(int64_t)r * W + (l >> 6)] |= 1ull << (l & 63);
    p.lanes->levels[l][r] = 0;
    p.lanes->parents[l][r] = r;
    Rc->lanes[l >> 6] |= 1ull << (l & 63);
    if (!before.any()) {
      const int64_t deg = p.out_off[r + 1] - p.out_off[r];
      if (deg <= kLightMax) {
        q[Rc->nlight++] = r;
      } else {
        const unsigned long long old = Rc->big;
        Rc->big = old + ((1ull << 32) | (unsigned long long)deg);
        q[p.n - 1 - (int64_t)(old >> 32)] = r;
        boff[old >> 32] = (unsigned)old;
      }
    }
  }
}

// Lanes whose search ended (ctl->done): level and parent -1 for the vertices
// they never reached, and their bits cleared from the visited masks so the
// lanes can be admitted again.  The mask is copied to done_out.
template <int W>
__global__ void pool_finish_kernel(MsParams p, unsigned long long *done_out) {
  const MsCtl *ctl = p.ctl;
  Mask<W> done;
#pragma unroll
  for (int i = 0; i < W; ++i) done.w[i] = ctl->done[i];
  const int64_t gtid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (gtid == 0) {
    done_out[0] = ctl->done[0];
    done_out[1] = ctl->done[1];
    done_out[2] = (unsigned long long)(unsigned)ctl->L;
    done_out[3] = (unsigned long long)(unsigned)ctl->status;
  }
  if (!done.any()) return;
  for (int64_t v = gtid; v < p.n; v += (int64_t)gridDim.x * blockDim.x) {
    const Mask<W> m = ld_mask<W>(p.vis, v);
    const Mask<W> missed = done.andnot(m);
#pragma unroll
    for (int i = 0; i < W; ++i) {
      uint64_t bits = missed.w[i];
      while (bits) {
        const int b = __ffsll((long long)bits) - 1;
        bits &= bits - 1;
        p.lanes->levels[i * 64 + b][v] = -1;
        p.lanes->parents[i * 64 + b][v] = -1;
      }
    }
    if ((m & done).any()) st_mask<W>(p.vis, v, m.andnot(done));
  }
}

}  // namespace cg

struct cg_pool {
  cg_graph *g = nullptr;
  int W = 1;
  cg::MsState *s = nullptr;
  cg::LaneTable *d_lanes = nullptr;
  cg::LaneTable h_lanes{};
  unsigned long long busy[2] = {0ull, 0ull};
  cg::Admission pending{};
  unsigned long long *d_out = nullptr;  // done[2], L, status
  unsigned long long *h_out = nullptr;  // page-locked copy
  int next_round = 0;
};

namespace cg {

template <int W>
static int pool_start(cg_pool *pl) {
  MsParams p = ms_params<W>(pl->g, pl->s);
  p.lanes = pl->d_lanes;
  p.level_cap = 0x7fffffff;
  p.max_rounds = 1;
  int rc = ms_reset<W>(pl->s, pl->g->stream);
  if (rc) return rc;
  return ms_launch<W>(pl->g, p, pl->g->stream);  // k = 0: clears the lane state
}

template <int W>
static int pool_step(cg_pool *pl, int max_rounds, int stop_on_finish) {
  cg_graph *g = pl->g;
  MsParams p = ms_params<W>(g, pl->s);
  p.lanes = pl->d_lanes;
  p.level_cap = 0x7fffffff;
  p.resume = 1;
  p.k = 64 * W;
  p.max_rounds = max_rounds > 0 ? max_rounds : 0x7fffffff;
  p.stop_on_finish = stop_on_finish;
  if (pl->pending.count) {
    CG_CUDA(cudaMemcpyAsync(pl->d_lanes, &pl->h_lanes, sizeof(LaneTable), cudaMemcpyHostToDevice,
                            g->stream));
    pool_admit_kernel<W><<<1, 32, 0, g->stream>>>(p, pl->pending);
    CG_CUDA(cudaGetLastError());
    pl->pending.count = 0;
  }
  int rc = ms_launch<W>(g, p, g->stream);
  if (rc) return rc;
  int blocks = (int)((g->n + 255) / 256);
  if (blocks > g->num_sms * 8) blocks = g->num_sms * 8;
  if (blocks < 1) blocks = 1;
  pool_finish_kernel<W><<<blocks, 256, 0, g->stream>>>(p, pl->d_out);
  CG_CUDA(cudaGetLastError());
  CG_CUDA(cudaMemsetAsync(&pl->s->ctl->done, 0, sizeof(unsigned long long) * 2, g->stream));
  CG_CUDA(cudaMemcpyAsync(pl->h_out, pl->d_out, sizeof(unsigned long long) * 4,
                          cudaMemcpyDeviceToHost, g->stream));
  CG_CUDA(cudaStreamSynchronize(g->stream));
  return CG_OK;
}

}  // namespace cg

using namespace cg;

extern "C" {

int cg_pool_create(cg_graph *g, int32_t lane_words, cg_pool **out) {
  if (g) {
    if (int r = refuse_reordered(g, "cg_pool_create")) return r;
  }
  if (!g || !out || (lane_words != 1 && lane_words != 2)) return CG_ERR_INVALID_ARG;
  *out = nullptr;
  cg_pool *pl = new (std::nothrow) cg_pool();
  if (!pl) return CG_ERR_OUT_OF_MEMORY;
  pl->g = g;
  pl->W = lane_words;
  int rc = ms_create_state(g, lane_words, 0, &pl->s);
  if (!rc && (cudaMalloc(&pl->d_lanes, sizeof(LaneTable)) != cudaSuccess ||
              cudaMalloc(&pl->d_out, sizeof(unsigned long long) * 4) != cudaSuccess ||
              cudaHostAlloc(&pl->h_out, sizeof(unsigned long long) * 4, cudaHostAllocDefault) !=
                  cudaSuccess))
    rc = CG_ERR_OUT_OF_MEMORY;
  if (!rc) {
    memset(&pl->h_lanes, 0, sizeof(LaneTable));
    cudaMemsetAsync(pl->d_lanes, 0, sizeof(LaneTable), g->stream);
    rc = lane_words == 2 ? pool_start<2>(pl) : pool_start<1>(pl);
    if (!rc) {
      cudaError_t e = cudaStreamSynchronize(g->stream);
      if (e != cudaSuccess) rc = cuda_fail(e, "cg_pool_create");
    }
  }
  int L0 = 0;
  if (!rc && cudaMemcpy(&L0, &pl->s->ctl->L, sizeof(int), cudaMemcpyDeviceToHost) != cudaSuccess)
    rc = CG_ERR_CUDA;
  if (rc) {
    cg_pool_destroy(pl);
    return rc;
  }
  pl->next_round = L0;
  *out = pl;
  return CG_OK;
}

int cg_pool_destroy(cg_pool *pl) {
  if (!pl) return CG_ERR_INVALID_ARG;
  if (pl->g && pl->g->stream) cudaStreamSynchronize(pl->g->stream);
  ms_free_state(pl->s);
  cudaFree(pl->d_lanes);
  cudaFree(pl->d_out);
  if (pl->h_out) cudaFreeHost(pl->h_out);
  delete pl;
  return CG_OK;
}

int cg_pool_admit(cg_pool *pl, int64_t root, int32_t *d_levels, int32_t *d_parents,
                  int32_t *lane_out) {
  if (!pl || !d_levels || !d_parents || root < 0 || root >= pl->g->n) return CG_ERR_INVALID_ARG;
  const int lanes = 64 * pl->W;
  int l = -1;
  for (int i = 0; i < lanes; ++i)
    if (!((pl->busy[i >> 6] >> (i & 63)) & 1ull)) {
      l = i;
      break;
    }
  if (l < 0) return CG_ERR_ADMISSION;
  pl->busy[l >> 6] |= 1ull << (l & 63);
  pl->h_lanes.levels[l] = d_levels;
  pl->h_lanes.parents[l] = d_parents;
  pl->h_lanes.start[l] = pl->next_round;
  Admission &a = pl->pending;
  a.lane[a.count] = l;
  a.root[a.count] = (int32_t)root;
  a.count += 1;
  if (lane_out) *lane_out = l;
  return CG_OK;
}

int cg_pool_step(cg_pool *pl, int32_t max_rounds, int32_t stop_on_finish, uint64_t *done_out,
                 int32_t *next_round) {
  if (!pl) return CG_ERR_INVALID_ARG;
  int rc = pl->W == 2 ? pool_step<2>(pl, max_rounds, stop_on_finish)
                      : pool_step<1>(pl, max_rounds, stop_on_finish);
  if (rc) return rc;
  pl->next_round = (int)pl->h_out[2];
  if (done_out) {
    done_out[0] = pl->h_out[0];
    done_out[1] = pl->h_out[1];
  }
  if (next_round) *next_round = pl->next_round;
  return (int)pl->h_out[3];
}

int cg_pool_release(cg_pool *pl, int32_t lane) {
  if (!pl || lane < 0 || lane >= 64 * pl->W) return CG_ERR_INVALID_ARG;
  pl->busy[lane >> 6] &= ~(1ull << (lane & 63));
  return CG_OK;
}

int cg_pool_info(const cg_pool *pl, int32_t *lanes, int32_t *busy) {
  if (!pl) return CG_ERR_INVALID_ARG;
  if (lanes) *lanes = 64 * pl->W;
  if (busy) *busy = __builtin_popcountll(pl->busy[0]) + __builtin_popcountll(pl->busy[1]);
  return CG_OK;
}

}  // extern "C"
