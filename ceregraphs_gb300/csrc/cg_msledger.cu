// Multi-source BFS with the outputs written after the search ("ledger"
// mode).  The rounds advance the W-word lane masks -- vis, and the frontier
// F_L of every round, kept as a history F_0 .. F_D in HBM -- and write no
// per-(lane, vertex) output.  One output pass after the last round writes
// every (lane, vertex) output exactly once:
//   level(l, v)  = the round L whose F_L[v] holds bit l      (-1 if none)
//   parent(l, v) = v at level 0, roots[l] at level 1, else the lowest
//                  in-neighbour u of v with bit l in F_{level - 1}[u]
// which is the lowest-index rule of the per-root search and of the direct
// batched kernel (bfs/README.md:208-224), so the outputs are identical.
//
// Why: written during the rounds, every discovery is a 4-byte store into one
// of 64 rows -- 32 scattered stores per warp instruction, each a separate L1
// wavefront and L2 transaction, and sectors completed across rounds (partial
// sector writes).  Here the output pass writes, lane by lane, the 32 values of
// a warp's 32 consecutive vertices as one 128-byte row.
//
// Parents: vertices of in-degree > kPullLight have a slot of 64 W parent
// candidates.  A push round relaxing u -> v takes atomicMin(slot[l], u) for
// each new lane l (ms_relax); a pull round scans such a vertex's ascending
// in-list with one warp (or its chunks, for hubs, with several) and records
// each lane's first hit (or_warp_first).  Vertices of smaller in-degree are
// resolved in the output pass by their thread's scan of their short in-list.
//
// Rounds: a pull round ORs the frontier masks of a vertex's in-neighbours
// until every wanted lane is found; a push round ORs frontier masks into
// out-neighbours' next masks with atomicOr, then merges them into vis.  Hubs'
// in-lists are split into chunks across warps as in the direct kernel.
//
// A search that needs more rounds than the history holds sets a flag and
// stops; the output pass then only clears the control block, and the direct
// kernel, launched after it gated on the flag, runs the batch from scratch.
#include <cuda_runtime.h>
#include <stdint.h>

#include "cg_ms.cuh"

namespace cg {
namespace {

constexpr int kOutBlock = 128;                 // output pass: 4 warps a block
constexpr int kOutWarps = kOutBlock / 32;
constexpr int kOutLevels = 4;                  // levels resolved per in-list scan
constexpr int kParStride = 65;                 // shared row strides (bank-conflict free)
constexpr int kLvlStride = 68;
constexpr int kOutWarpBytes = 32 * kParStride * 4 + 32 * kLvlStride;

template <int W>
__device__ __forceinline__ uint64_t *plane(const MsParams &p, int L) {
  return p.hist + (int64_t)L * p.n * W;
}

// OR of the frontier masks of in-list entries [s, e) restricted to `want`,
// one thread, four entries' loads in flight; stops once all of want is found.
template <int W>
__device__ __forceinline__ Mask<W> or_thread(const MsParams &p, int64_t s, int64_t e,
                                             const Mask<W> &want, const uint64_t *cur) {
  constexpr int G = 4;
  Mask<W> got = Mask<W>::zero();
  for (int64_t i0 = s; i0 < e; i0 += G) {
    int32_t u[G];
#pragma unroll
    for (int k = 0; k < G; ++k) u[k] = i0 + k < e ? __ldg(p.in_idx + i0 + k) : -1;
#pragma unroll
    for (int k = 0; k < G; ++k)
      if (u[k] >= 0) got = got | (ld_mask<W>(cur, u[k]) & want);
    if (got == want) break;
  }
  return got;
}

// 32 x 32 bit-matrix transpose across the warp: lane r holds row r (bit c =
// entry (r, c)); afterwards lane t holds column t (bit r = entry (r, t)).
// Five butterfly steps, each swapping off-diagonal blocks with the partner
// lane t ^ j.
__device__ __forceinline__ uint32_t warp_transpose32(uint32_t x) {
  const int lane = lane_id();
#pragma unroll
  for (int j = 16; j > 0; j >>= 1) {
    const uint32_t m = j == 16 ? 0x0000ffffu
                     : j == 8  ? 0x00ff00ffu
                     : j == 4  ? 0x0f0f0f0fu
                     : j == 2  ? 0x33333333u
                               : 0x55555555u;
    const uint32_t y = __shfl_xor_sync(kMsFull, x, j);
    x = (lane & j) ? ((x & ~m) | ((y & ~m) >> j)) : ((x & m) | ((y & m) << j));
  }
  return x;
}

// or_warp that also records, per lane of `want`, the first in-list entry
// holding it -- the lowest-index parent -- into row[lane] (plain stores when
// the warp scans the whole in-list, atomicMin when other warps scan other
// chunks of it).  The hits of 32 entries form a 32 x 64 W bit matrix that is
// transposed a word at a time, so warp lane t resolves lanes t and t + 32 of
// each word at once.
template <int W>
__device__ __forceinline__ Mask<W> or_warp_first(const MsParams &p, int64_t s, int64_t e,
                                                 const Mask<W> &want, const uint64_t *cur,
                                                 uint32_t *row, bool atomic) {
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
    {
      // nothing new among these 4 x 32 entries (the common case late in a
      // list that some lanes only reach in a later round): one reduction
      Mask<W> any = Mask<W>::zero();
#pragma unroll
      for (int k = 0; k < G; ++k) any = any | f[k];
      if (!warp_or<W>(any & want).andnot(got).any()) continue;
    }
#pragma unroll
    for (int k = 0; k < G; ++k) {
      const Mask<W> fk = (f[k] & want).andnot(got);
      const Mask<W> F = warp_or<W>(fk);
      if (!F.any()) continue;
#pragma unroll
      for (int j = 0; j < W; ++j) {
        if (!F.w[j]) continue;
        uint32_t *r = row + 64 * j;
        if (__popcll(F.w[j]) <= 6) {
          // few lanes: one ballot each
          uint64_t bits = F.w[j];
          while (bits) {
            const int b = __ffsll((long long)bits) - 1;
            bits &= bits - 1;
            const unsigned who = __ballot_sync(kMsFull, (fk.w[j] >> b) & 1ull);
            if (lane == __ffs(who) - 1) {
              if (atomic)
                atomicMin(r + b, (unsigned)u[k]);
              else
                r[b] = (uint32_t)u[k];
            }
          }
          continue;
        }
        const uint32_t lo = warp_transpose32((uint32_t)fk.w[j]);
        const uint32_t hi = warp_transpose32((uint32_t)(fk.w[j] >> 32));
        const int32_t plo = __shfl_sync(kMsFull, u[k], lo ? __ffs(lo) - 1 : 0);
        const int32_t phi = __shfl_sync(kMsFull, u[k], hi ? __ffs(hi) - 1 : 0);
        if (atomic) {
          if (lo) atomicMin(r + lane, (unsigned)plo);
          if (hi) atomicMin(r + lane + 32, (unsigned)phi);
        } else {
          if (lo) r[lane] = (uint32_t)plo;
          if (hi) r[lane + 32] = (uint32_t)phi;
        }
      }
      got = got | F;
      if (got == want) return got;
    }
  }
  return got;
}

// Pull round: light vertices one thread each, medium vertices one warp each,
// hub in-lists by chunks (ORed into hub_found, merged after the wait).
template <int W>
__device__ void lg_pull(const MsParams &p, int L, const uint64_t *cur, uint64_t *nxt,
                        const Mask<W> &active, MsRound *Rn, MsAcc &acc) {
  const int64_t nthreads = (int64_t)gridDim.x * blockDim.x;
  const int next_parity = (L + 1) & 1;
  int32_t *q = next_parity ? p.queue1 : p.queue0;
  uint32_t *boff = next_parity ? p.bigoff1 : p.bigoff0;
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
    if (want.any()) got = or_thread<W>(p, s, e, want, cur);
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
  const int nwarps = (int)(nthreads >> 5);
  for (int64_t j = warp_id_global(); j < p.nmed; j += nwarps) {
    const int32_t v = p.med_vtx[j];
    const Mask<W> seen = ld_mask<W>(p.vis, v);
    const Mask<W> want = active.andnot(seen);
    if (!want.any()) continue;
    // medium vertex j has candidate slot j: its parents of this round go there
    const Mask<W> got = or_warp_first<W>(p, __ldg(p.in_off + v), __ldg(p.in_off + v + 1), want,
                                         cur, p.cand + j * (64 * W), false);
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
  if (p.nhub == 0) return;
  const unsigned nchunks = p.hub_choff[p.nhub];
  for (unsigned c = (unsigned)warp_id_global(); c < nchunks; c += (unsigned)nwarps) {
    unsigned lo = 0, hi = (unsigned)p.nhub - 1;
    while (lo < hi) {
      const unsigned mid = (lo + hi + 1) >> 1;
      if (p.hub_choff[mid] <= c)
        lo = mid;
      else
        hi = mid - 1;
    }
    const int h = (int)lo;
    const int32_t v = p.hub_vtx[h];
    const Mask<W> want = active.andnot(ld_mask<W>(p.vis, v));
    if (!want.any()) continue;
    const int64_t s = __ldg(p.in_off + v) + (int64_t)(c - p.hub_choff[h]) * kHubChunk;
    const int64_t e = min(s + (int64_t)kHubChunk, __ldg(p.in_off + v + 1));
    // hub h has candidate slot nmed + h; several warps scan its chunks
    const Mask<W> got = or_warp_first<W>(p, s, e, want, cur,
                                         p.cand + (p.nmed + h) * (64 * W), true);
    if (lane_id() == 0) {
#pragma unroll
      for (int j = 0; j < W; ++j)
        if (got.w[j])
          atomicOr(reinterpret_cast<unsigned long long *>(p.hub_found + (int64_t)h * W + j),
                   (unsigned long long)got.w[j]);
    }
  }
}

// After the wait that ends a pull round's scans: hubs found this round get
// their next mask and vis, and are queued after the round's other vertices.
template <int W>
__device__ void lg_hub_merge(const MsParams &p, int L, uint64_t *nxt, MsRound *Rn, MsAcc &acc) {
  const int lane = lane_id();
  const int nwarps = (gridDim.x * blockDim.x) >> 5;
  const int next_parity = (L + 1) & 1;
  int32_t *q = next_parity ? p.queue1 : p.queue0;
  uint32_t *boff = next_parity ? p.bigoff1 : p.bigoff0;
  for (int64_t h0 = (int64_t)warp_id_global() * 32; h0 < p.nhub; h0 += (int64_t)nwarps * 32) {
    const int64_t h = h0 + lane;
    bool claimed = false;
    int32_t v = 0;
    int64_t deg = 0;
    if (h < p.nhub) {
      const Mask<W> found = ld_mask<W>(p.hub_found, h);
      if (found.any()) {
        v = p.hub_vtx[h];
        st_mask<W>(nxt, v, found);
        st_mask<W>(p.vis, v, ld_mask<W>(p.vis, v) | found);
        st_mask<W>(p.hub_found, h, Mask<W>::zero());
        acc.visits += (unsigned long long)found.popc();
        acc_lanes<W>(acc, found);
        deg = __ldg(p.out_off + v + 1) - __ldg(p.out_off + v);
        claimed = true;
      }
    }
    ms_enqueue(claimed, v, deg, q, p.n, boff, &Rn->nlight, &Rn->big, acc);
  }
}

// After a push round: the vertices it queued merge their new lanes into vis.
template <int W>
__device__ void lg_push_merge(const MsParams &p, int L, const uint64_t *nxt, MsRound *Rn,
                              MsAcc &acc) {
  const int64_t nthreads = (int64_t)gridDim.x * blockDim.x;
  const int next_parity = (L + 1) & 1;
  const int32_t *q = next_parity ? p.queue1 : p.queue0;
  const int64_t nl = *(volatile unsigned *)&Rn->res_light;
  const int64_t nbg = *(volatile unsigned *)&Rn->res_big;
  for (int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; j < nl + nbg; j += nthreads) {
    const int64_t v = j < nl ? q[j] : q[p.n - 1 - (j - nl)];
    const Mask<W> nw = ld_mask<W>(nxt, v);
    st_mask<W>(p.vis, v, ld_mask<W>(p.vis, v) | nw);
    acc.visits += (unsigned long long)nw.popc();
    acc_lanes<W>(acc, nw);
  }
}

// End of round L (last block to arrive): as the direct kernel's, plus the
// history bound -- round L + 1 writes F_{L+2}, which must be a plane.
template <int W>
__device__ unsigned lg_decide(const MsParams &p, int L, int dir, int ran) {
  MsCtl *ctl = p.ctl;
  const MsRound *Rn = &ctl->rec[(L + 1) % kRing];
  unsigned long long nf = 0, visits = 0, mf = 0;
#pragma unroll
  for (int i = 0; i < kCounterShards; ++i) {
    nf += *(volatile const unsigned long long *)&Rn->nf[i];
    visits += *(volatile const unsigned long long *)&Rn->visits[i];
    mf += *(volatile const unsigned long long *)&Rn->mf[i];
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
  bool stop = nf == 0;
  if (!stop && L + 1 >= p.level_cap) {
    atomicCAS(&ctl->status, 0, (int)CG_ERR_LEVEL_CAP);
    stop = true;
  }
  if (!stop && L + 2 >= p.hist_planes) {
    *(volatile int *)p.flag = 1;  // outgrew the history: the direct kernel takes over
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
struct LgRoundDecision {
  const MsParams *p;
  int L, dir, ran;
  __device__ unsigned operator()() const { return lg_decide<W>(*p, L, dir, ran); }
};

struct LgResolveSnapshot {
  MsRound *R;
  __device__ unsigned operator()() const {
    R->res_light = *(volatile unsigned *)&R->nlight;
    R->res_big = (unsigned)(*(volatile unsigned long long *)&R->big >> 32);
    return 0u;
  }
};

struct LgSetupDecision {
  MsCtl *ctl;
  cg_stats *st;
  __device__ unsigned operator()() const {
    const long long now = global_ns();
    st->setup_ns = now - ctl->t_start;
    st->finish_ns = 0;
    ctl->t_round = now;
    return 0u;
  }
};

// The rounds of one batch (cooperative, persistent): roots[0..k) seeded in
// F_0; round L reads F_L, writes F_{L+1} and clears F_{L+2}.
template <int W>
__global__ void __launch_bounds__(kMsBlock, 2) msbfs_ledger(MsParams p) {
  __shared__ unsigned s_payload;
  MsCtl *ctl = p.ctl;
  const int64_t gtid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t nthreads = (int64_t)gridDim.x * blockDim.x;
  if (blockIdx.x == 0 && threadIdx.x == 0) ctl->t_start = global_ns();
  uint64_t *f0 = plane<W>(p, 0), *f1 = plane<W>(p, 1);
  for (int64_t i = gtid; i < p.n * W; i += nthreads) {
    p.vis[i] = 0;
    f0[i] = 0;
    f1[i] = 0;
  }
  for (int64_t w = gtid; w < p.words; w += nthreads) {
    p.touched0[w] = 0;
    p.touched1[w] = 0;
  }
  bool ok = grid_wait(&ctl->wait, &ctl->status, p.timeout_ns);
  if (ok && blockIdx.x == 0 && threadIdx.x < p.k) {
    const int i = threadIdx.x;
    const int32_t r = p.roots[i];
    const unsigned long long bit = 1ull << (i & 63);
    atomicOr(reinterpret_cast<unsigned long long *>(p.vis + (int64_t)r * W + (i >> 6)), bit);
    atomicOr(reinterpret_cast<unsigned long long *>(f0 + (int64_t)r * W + (i >> 6)), bit);
    bool first = true;
    for (int j = 0; j < i; ++j) first = first && (p.roots[j] != r);
    if (first) {
      const int64_t deg = p.out_off[r + 1] - p.out_off[r];
      MsRound *R0 = &ctl->rec[0];
      if (deg <= kLightMax) {
        p.queue0[atomicAdd(&R0->nlight, 1u)] = r;
      } else {
        const unsigned long long old = atomicAdd(&R0->big, (1ull << 32) | (unsigned long long)deg);
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
    }
  }
  if (ok) {
    __syncthreads();
    if (threadIdx.x == 0)
      s_payload = arrive_and_wait(&ctl->wait, &ctl->status, p.timeout_ns, 0u,
                                  LgSetupDecision{ctl, p.stats});
    __syncthreads();
    ok = s_payload != kWaitFailed;
  }
  int L = 0, dir = 0, ran = 0;
  MsAcc acc, tot;
  while (ok) {
    const uint64_t *cur = plane<W>(p, L);
    uint64_t *nxt = plane<W>(p, L + 1);
    uint32_t *touched = (L & 1) ? p.touched1 : p.touched0;
    uint32_t *touched_next = (L & 1) ? p.touched0 : p.touched1;
    MsRound *Rc = &ctl->rec[L % kRing];
    MsRound *Rn = &ctl->rec[(L + 1) % kRing];
    if (L + 2 < p.hist_planes) {
      uint64_t *clr = plane<W>(p, L + 2);
      for (int64_t i = gtid; i < p.n * W; i += nthreads) clr[i] = 0;
    }
    for (int64_t w = gtid; w < p.words; w += nthreads) touched_next[w] = 0;
    if (dir == 1) {
      Mask<W> active;
#pragma unroll
      for (int i = 0; i < W; ++i) active.w[i] = *(volatile unsigned long long *)&Rc->lanes[i];
      lg_pull<W>(p, L, cur, nxt, active, Rn, acc);
      if (p.nhub > 0) {
        if (!(ok = grid_wait(&ctl->wait, &ctl->status, p.timeout_ns))) break;
        lg_hub_merge<W>(p, L, nxt, Rn, acc);
      }
    } else {
      ms_push<W, true>(p, L, cur, nxt, touched, Rc, Rn, acc);
      __syncthreads();
      if (threadIdx.x == 0)
        s_payload = arrive_and_wait(&ctl->wait, &ctl->status, p.timeout_ns, 0u,
                                    LgResolveSnapshot{Rn});
      __syncthreads();
      if (s_payload == kWaitFailed) {
        ok = false;
        break;
      }
      lg_push_merge<W>(p, L, nxt, Rn, acc);
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
                                  LgRoundDecision<W>{&p, L, dir, ran});
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
  if (blockIdx.x == 0 && threadIdx.x == 0 && !ok)
    p.stats->status = *(volatile int *)&ctl->status;
}

// ---- output pass ----------------------------------------------------------

// Up to kOutLevels levels >= `from` holding lanes of `todo` at vertex v (half
// h of the lanes), ascending: Ls[k] the level, Ms[k] its lanes.  Advances
// `from` past the last one taken; returns the lanes taken.
template <int W>
__device__ __forceinline__ uint64_t collect_levels(const MsParams &p, int64_t v, int h, int rounds,
                                                   uint64_t todo, int &from, int (&Ls)[kOutLevels],
                                                   uint64_t (&Ms)[kOutLevels]) {
#pragma unroll
  for (int k = 0; k < kOutLevels; ++k) {
    Ls[k] = 1;
    Ms[k] = 0;
  }
  uint64_t covered = 0;
  int nl = 0;
  for (int L = from; L < rounds && nl < kOutLevels && todo; ++L) {
    const uint64_t m = plane<W>(p, L)[v * W + h] & todo;
    if (m) {
#pragma unroll
      for (int k = 0; k < kOutLevels; ++k)
        if (k == nl) {
          Ls[k] = L;
          Ms[k] = m;
        }
      covered |= m;
      todo &= ~m;
      ++nl;
    }
    from = L + 1;
  }
  return covered;
}

// Lanes of `want` for which u is one level closer to the root than v: bit l
// of Ms[k] is a lane with v at level Ls[k]; u qualifies if F_{Ls[k]-1}[u] has l.
template <int W>
__device__ __forceinline__ uint64_t parent_hits(const MsParams &p, int32_t u, int h,
                                                const int (&Ls)[kOutLevels],
                                                const uint64_t (&Ms)[kOutLevels], uint64_t want) {
  uint64_t b = 0;
#pragma unroll
  for (int k = 0; k < kOutLevels; ++k)
    if (Ms[k] & want) b |= Ms[k] & plane<W>(p, Ls[k] - 1)[(int64_t)u * W + h];
  return b & want;
}

// Output pass.  Each warp takes 32 consecutive vertices (one per thread).  Per
// 64-lane half of the batch a thread reads its vertex's history masks once
// and records each lane's level as a byte of a shared tile row (0xFF =
// unreached); parents of levels >= 2 go to a second tile: the slot's
// candidates (in-degree > kPullLight, copied by the warp) or the first hit of
// the thread's scan of its own short in-list.  Then, lane by lane, the warp
// writes the tile's 32 levels and 32 parents as two 128-byte rows; parents of
// levels 0 and 1 are the vertex and the lane's root.
template <int W>
__global__ void __launch_bounds__(kOutBlock) msbfs_outputs(MsParams p) {
  extern __shared__ __align__(16) unsigned char s_tile[];
  constexpr int kPre = 8;     // history planes loaded together
  constexpr int kScanG = 8;   // in-list entries loaded together
  MsCtl *ctl = p.ctl;
  if (*(volatile int *)p.flag) {
    // the gated direct launch that follows needs a clean control block
    if (blockIdx.x == 0) {
      unsigned long long *c = reinterpret_cast<unsigned long long *>(ctl);
      for (int i = threadIdx.x; i < (int)(sizeof(MsCtl) / 8); i += blockDim.x) c[i] = 0ull;
    }
    return;
  }
  if (*(volatile int *)&ctl->status != 0) return;  // timed out or over the level cap
  int rounds = *(volatile int *)&ctl->L;           // F_0 .. F_rounds, F_rounds empty
  if (rounds > p.hist_planes) rounds = p.hist_planes;
  const int lane = lane_id();
  const int wib = threadIdx.x >> 5;
  int32_t *par = reinterpret_cast<int32_t *>(s_tile + wib * kOutWarpBytes);
  uint8_t *lvl = s_tile + wib * kOutWarpBytes + 32 * kParStride * 4;
  int32_t *my_par = par + lane * kParStride;
  uint8_t *my_lvl = lvl + lane * kLvlStride;
  const int64_t nwarps = (int64_t)gridDim.x * kOutWarps;
  for (int64_t tile = (int64_t)blockIdx.x * kOutWarps + wib; tile * 32 < p.n; tile += nwarps) {
    const int64_t v = tile * 32 + lane;
    const bool valid = v < p.n;
    int64_t s = 0, e = 0;
    int slot = -1;
    if (valid) {
      s = __ldg(p.in_off + v);
      e = __ldg(p.in_off + v + 1);
      slot = p.cand_slot[v];
    }
#pragma unroll 1
    for (int h = 0; h < W && 64 * h < p.k; ++h) {
      // parents of levels >= 2 of the tile's slotted vertices: the warp copies
      // each slot's 256-byte candidate row into the vertex's tile row, four
      // rows' loads in flight
      {
        unsigned pend = __ballot_sync(kMsFull, slot >= 0);
        while (pend) {
          int src[4];
          uint2 x[4];
#pragma unroll
          for (int r = 0; r < 4; ++r) {
            src[r] = pend ? __ffs(pend) - 1 : -1;
            if (pend) pend &= pend - 1;
          }
#pragma unroll
          for (int r = 0; r < 4; ++r) {
            const int ss = src[r] >= 0 ? __shfl_sync(kMsFull, slot, src[r]) : -1;
            x[r] = ss >= 0 ? __ldg(reinterpret_cast<const uint2 *>(p.cand + (int64_t)ss * (64 * W) +
                                                                  64 * h) + lane)
                           : make_uint2(0u, 0u);
          }
#pragma unroll
          for (int r = 0; r < 4; ++r) {
            if (src[r] >= 0) {
              par[src[r] * kParStride + 2 * lane] = (int32_t)x[r].x;
              par[src[r] * kParStride + 2 * lane + 1] = (int32_t)x[r].y;
            }
          }
        }
      }
      // level bytes; the first kOutLevels levels >= 2 of a light vertex for its
      // scan, any further ones (rare) through collect_levels below
      uint32_t *lw = reinterpret_cast<uint32_t *>(my_lvl);
#pragma unroll
      for (int i = 0; i < 16; ++i) lw[i] = 0xffffffffu;
      int Ls[kOutLevels];
      uint64_t Ms[kOutLevels];
      int nl = 0;
      uint64_t gtodo = 0, rest = 0;
      int last = 1;
#pragma unroll
      for (int k = 0; k < kOutLevels; ++k) {
        Ls[k] = 1;
        Ms[k] = 0;
      }
      if (valid) {
        for (int L0 = 0; L0 < rounds; L0 += kPre) {
          uint64_t pm[kPre];
#pragma unroll
          for (int j = 0; j < kPre; ++j)
            pm[j] = L0 + j < rounds ? plane<W>(p, L0 + j)[v * W + h] : 0ull;
#pragma unroll
          for (int j = 0; j < kPre; ++j) {
            uint64_t m = pm[j];
            const int L = L0 + j;
            if (m && L >= 2 && slot < 0) {
              if (nl < kOutLevels) {
#pragma unroll
                for (int k = 0; k < kOutLevels; ++k)
                  if (k == nl) {
                    Ls[k] = L;
                    Ms[k] = m;
                  }
                ++nl;
                gtodo |= m;
                last = L;
              } else {
                rest |= m;
              }
            }
            while (m) {
              const int b = __ffsll((long long)m) - 1;
              m &= m - 1;
              my_lvl[b] = (uint8_t)L;
            }
          }
        }
      }
      // light vertices: the whole in-list (<= kPullLight entries), kScanG
      // entries' loads in flight, kOutLevels levels per pass
      int from = last + 1;
      while (gtodo) {
        for (int64_t j0 = s; j0 < e && gtodo; j0 += kScanG) {
          int32_t u[kScanG];
          uint64_t b[kScanG];
#pragma unroll
          for (int k = 0; k < kScanG; ++k) u[k] = j0 + k < e ? __ldg(p.in_idx + j0 + k) : -1;
#pragma unroll
          for (int k = 0; k < kScanG; ++k)
            b[k] = u[k] >= 0 ? parent_hits<W>(p, u[k], h, Ls, Ms, gtodo) : 0;
#pragma unroll
          for (int k = 0; k < kScanG; ++k) {
            uint64_t bk = b[k] & gtodo;
            gtodo &= ~bk;
            while (bk) {
              const int bit = __ffsll((long long)bk) - 1;
              bk &= bk - 1;
              my_par[bit] = u[k];
            }
          }
        }
        gtodo = 0;
        if (rest) {  // more than kOutLevels levels at this vertex
          gtodo = collect_levels<W>(p, v, h, rounds, rest, from, Ls, Ms);
          rest &= ~gtodo;
          if (!gtodo) rest = 0;
        }
      }
      __syncwarp();
      // rows: lane l of this half, vertices tile*32 .. tile*32 + 31
      const int lanes = min(64, p.k - 64 * h);
#pragma unroll 4
      for (int l = 0; l < lanes; ++l) {
        const uint8_t lv = my_lvl[l];
        const int32_t pv = lv == 0 ? (int32_t)v : (lv == 1 ? p.roots[64 * h + l] : my_par[l]);
        const int64_t at = (int64_t)(64 * h + l) * p.n + v;
        if (valid) {
          p.levels[at] = lv == 0xff ? -1 : (int32_t)lv;
          p.parents[at] = lv == 0xff ? -1 : pv;
        }
      }
      __syncwarp();
    }
  }
  // the last block out records the time since the last round ended
  __syncthreads();
  if (threadIdx.x == 0 && atomicAdd(&ctl->exited, 1u) + 1u == gridDim.x)
    p.stats->finish_ns = global_ns() - *(volatile long long *)&ctl->t_round;
}

template <int W>
int ledger_pass(cg_graph *g, MsState *s, const int64_t *roots, int k, int32_t *d_levels,
                int32_t *d_parents) {
  MsParams p = ms_params<W>(g, s);
  p.levels = d_levels;
  p.parents = d_parents;
  p.k = k;
  for (int i = 0; i < kMsMaxLanes; ++i) p.roots[i] = i < k ? (int32_t)roots[i] : 0;
  int rc = ms_reset<W>(s, g->stream);
  if (rc) return rc;
  int block = g->opt.block_size > 0 ? g->opt.block_size : kMsBlock;
  if (block > kMsBlock) block = kMsBlock;
  block = (block / 32) * 32;
  if (block < 128) block = 128;  // seeding uses threads 0..k-1 of block 0
  int per_sm = 0;
  CG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, msbfs_ledger<W>, block, 0));
  if (per_sm <= 0) return CG_ERR_NOT_SUPPORTED;
  if (g->opt.blocks_per_sm > 0 && g->opt.blocks_per_sm < per_sm) per_sm = g->opt.blocks_per_sm;
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
  CG_CUDA(cudaLaunchKernelEx(&cfg, msbfs_ledger<W>, p));
  const int smem = kOutWarps * kOutWarpBytes;
  CG_CUDA(cudaFuncSetAttribute(msbfs_outputs<W>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               smem));
  int out_per_sm = 0;
  CG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&out_per_sm, msbfs_outputs<W>, kOutBlock,
                                                        smem));
  if (out_per_sm <= 0) return CG_ERR_NOT_SUPPORTED;
  const int64_t tiles = (g->n + 31) / 32;
  int64_t blocks = (tiles + kOutWarps - 1) / kOutWarps;
  const int64_t cap = (int64_t)out_per_sm * g->num_sms;
  if (blocks > cap) blocks = cap;
  msbfs_outputs<W><<<(unsigned)blocks, kOutBlock, smem, g->stream>>>(p);
  CG_CUDA(cudaGetLastError());
  return CG_OK;
}

}  // namespace

int ms_ledger_pass(cg_graph *g, MsState *s, const int64_t *roots, int k, int32_t *d_levels,
                   int32_t *d_parents) {
  return s->lane_words == 2 ? ledger_pass<2>(g, s, roots, k, d_levels, d_parents)
                            : ledger_pass<1>(g, s, roots, k, d_levels, d_parents);
}

}  // namespace cg
