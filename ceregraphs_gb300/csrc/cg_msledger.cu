// Multi-source BFS with the outputs written after the search ("ledger"
// mode).  The rounds advance the W-word lane masks -- vis, and the frontier
// F_L of every round, kept as a history F_0 .. F_D in HBM -- and write no
// per-(lane, vertex) output.  After the last round a scan pass resolves the
// parents the rounds left open, one output pass writes every (lane, vertex)
// output exactly once, and a fix-up pass rewrites the few parents that did
// not fit the per-vertex records:
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
// each lane's first hit (or_warp_first).  Vertices of smaller in-degree keep
// (source, lanes) records: a pull round's thread scan records each entry that
// brings new lanes (the lowest-index parent of those lanes, the in-list being
// ascending); the lanes pushes gave them, and those past the pull rounds'
// records, are resolved by the scan pass (scan_in_list), which appends
// records; lanes past all records go to the fix-up pass.
//
// Rounds: a pull round ORs the frontier masks of a vertex's in-neighbours
// until every wanted lane is found; a push round ORs frontier masks into
// out-neighbours' next masks with atomicOr.  Hubs' in-lists are split into
// chunks across warps as in the direct kernel.  The frontier set of round L is
// a claim bitmap T_L (one bit per vertex, set by whoever first gives the
// vertex a lane): push rounds find their light frontier vertices there and
// only big ones (out-degree > kLightMax) go through a queue, so no per-vertex
// atomic on a shared queue counter.  vis is merged lazily: round L folds F_L
// into vis for its frontier vertices and tests "visited" as vis | F_L, so a
// push round needs no second phase.
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
// A warp's shared tile: one parent table of kTab words per thread -- 64
// parents of its vertex (lane l at column (l - 8 t) mod 64 for thread t: the
// 32 threads reading the same lane hit 32 different banks, the stride being
// 9 mod 32), then the sources of its kRecords records at kTabRec + q, and -1
// (unreached) at kTabNone.  A lane's parent is one table read at a byte index.
constexpr int kTabRec = 64;
constexpr int kTabNone = kTabRec + 8;
constexpr int kTab = kTabNone + 1;
constexpr int kOutWarpBytes = 32 * kTab * 4;
static_assert(kRecords <= 8, "record indices are 3 bit slices");
constexpr int kSlices = 7;                     // bit slices of a level (levels 0..64)

// Bits 0..3 of x moved to bit 0 of bytes 0..3 (the four shifted copies do not
// overlap, so the product has no carries).
__device__ __forceinline__ uint32_t spread4(uint32_t x) { return (x * 0x00204081u) & 0x01010101u; }

template <bool B>
struct Flag {
  static constexpr bool value = B;
};

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

// or_thread that also records, for light vertex v, each in-list entry that
// brings new lanes -- their lowest-index parent, the scan being ascending --
// as a (source, lanes) pair, up to p.pull_records per vertex over all pull rounds.
// `want1`, after a push round: the lanes that push gave v at this round's
// level L, whose parents are the first entries holding them in F_{L-1}
// (`prev`) -- found in the same pass and recorded alike, so the scan pass
// need not rescan v.  Lanes found after the records run out (`over`) are
// left to the scan pass.  Returns the lanes of `want` found.
template <int W>
__device__ __forceinline__ Mask<W> or_thread_rec(const MsParams &p, int64_t v, int64_t s,
                                                 int64_t e, const Mask<W> &want,
                                                 const uint64_t *cur, const uint64_t *prev,
                                                 const Mask<W> &want1, bool &over) {
  constexpr int G = 4;
  Mask<W> got = Mask<W>::zero(), got1 = Mask<W>::zero();
  const bool two = want1.any();
  int used = p.pair_n[v];
  const int first = used;
  for (int64_t i0 = s; i0 < e; i0 += G) {
    int32_t u[G];
    Mask<W> m[G], m1[G];
#pragma unroll
    for (int k = 0; k < G; ++k) u[k] = i0 + k < e ? __ldg(p.in_idx + i0 + k) : -1;
#pragma unroll
    for (int k = 0; k < G; ++k) {
      m[k] = u[k] >= 0 ? ld_mask<W>(cur, u[k]) : Mask<W>::zero();
      m1[k] = two && u[k] >= 0 ? ld_mask<W>(prev, u[k]) : Mask<W>::zero();
    }
#pragma unroll
    for (int k = 0; k < G; ++k) {
      const Mask<W> nb = (m[k] & want).andnot(got);
      const Mask<W> nb1 = (m1[k] & want1).andnot(got1);
      const Mask<W> r = nb | nb1;  // disjoint: want1 lanes are visited, want lanes are not
      if (r.any()) {
        if (used < p.pull_records) {
          const int64_t at = (int64_t)used * p.n + v;
          p.pair_u[at] = u[k];
          st_mask<W>(p.pair_m, at, r);
          ++used;
        } else {
          over = true;
        }
        got = got | nb;
        got1 = got1 | nb1;
      }
    }
    if (got == want && got1 == want1) break;
  }
  if (used != first) p.pair_n[v] = (uint8_t)used;
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

// Claim bitmap T_L: one bit per vertex with a nonzero frontier mask F_L --
// round L's frontier set.  Round L reads T_L (push rounds enumerate light
// frontier vertices from it), sets T_{L+1}, and clears T_{L+2}; three rotate.
__device__ __forceinline__ uint32_t *claims(const MsParams &p, int L) {
  const int r = L % 3;
  return r == 0 ? p.touched0 : (r == 1 ? p.touched1 : p.touched2);
}

// vis is merged lazily: a vertex's frontier lanes F_L[v] join vis[v] during
// round L (pull rounds for every vertex, push rounds for every frontier
// vertex), so round L tests "visited" as vis | F_L.

// Pull round: light vertices one thread each, medium vertices one warp each,
// hub in-lists by chunks (ORed into hub_found, merged after the wait).
template <int W>
__device__ void lg_pull(const MsParams &p, int L, const uint64_t *cur, uint64_t *nxt,
                        const Mask<W> &active, bool after_push, MsRound *Rc, MsRound *Rn,
                        MsAcc &acc) {
  // after a push round of level >= 1, light vertices also resolve the
  // parents of the lanes that push gave them (F_L) against F_{L-1} (64
  // lanes; with 128 the registers would spill, and the scan pass does it)
  after_push = after_push && W == 1;
  const uint64_t *prev = after_push ? plane<W>(p, L - 1) : cur;
  const int64_t nthreads = (int64_t)gridDim.x * blockDim.x;
  const int next_parity = (L + 1) & 1;
  int32_t *q = next_parity ? p.queue1 : p.queue0;
  uint32_t *boff = next_parity ? p.bigoff1 : p.bigoff0;
  uint32_t *tnext = claims(p, L + 1);
  const int lane = lane_id();
  // a symmetric graph stores one list per vertex: out-degree = in-degree
  const bool sym = p.out_off == p.in_off;
  // light vertex groups (kLightGrab x 32 vertices), then medium vertices
  // (groups of kMedGrab), then hub chunks (groups of kHubGrab), handed out
  // dynamically -- one item per warp, then a counter -- so that the round's
  // last warps are not the ones with the longest lists
  constexpr unsigned kLightGrab = 8, kMedGrab = 8, kHubGrab = 4;
  const unsigned nwarps = (unsigned)(nthreads >> 5);
  const unsigned nlg = (unsigned)((p.n + 32 * kLightGrab - 1) / (32 * kLightGrab));
  const unsigned nmg = (unsigned)((p.nmed + kMedGrab - 1) / kMedGrab);
  const unsigned nchunks = p.nhub > 0 ? p.hub_choff[p.nhub] : 0u;
  const unsigned nhg = (nchunks + kHubGrab - 1) / kHubGrab;
  unsigned item = (unsigned)warp_id_global();
  while (item < nlg + nmg + nhg) {
    // the next item is claimed before this one is worked, hiding the atomic
    unsigned nextitem = 0;
    if (lane == 0) nextitem = nwarps + atomicAdd(&Rc->work, 1u);
    if (item < nlg) {
      // the light vertices of kLightGrab words not yet finished, compacted 32
      // at a time (vertices without in-edges are not light: none can reach
      // them).  Lane j < kLightGrab holds word j; the t-th vertex is the
      // (t - prefix)-th set bit of the first word whose inclusive count
      // exceeds t.  Only this warp touches these words of fin this round.
      const int64_t w0 = (int64_t)item * kLightGrab;
      uint32_t finw = 0, mine = 0;
      if (lane < kLightGrab && w0 + lane < p.words) {
        finw = p.fin[w0 + lane];
        mine = __ldg(p.light + w0 + lane) & ~finw;
      }
      const uint32_t fin0 = finw;
      const int cnt = __popc(mine);
      int incl = cnt;
#pragma unroll
      for (int o = 1; o < kLightGrab; o <<= 1) {
        const int t = __shfl_up_sync(kMsFull, incl, o);
        if (lane >= o) incl += t;
      }
      const int total = __shfl_sync(kMsFull, incl, kLightGrab - 1);
      for (int b0 = 0; b0 < total; b0 += 32) {
        const int t = b0 + lane;
        int wsel = 0;
#pragma unroll
        for (int step = kLightGrab / 2; step > 0; step >>= 1)
          if (__shfl_sync(kMsFull, incl, wsel + step - 1) <= t) wsel += step;
        const uint32_t wbits = __shfl_sync(kMsFull, mine, wsel);
        const int before = __shfl_sync(kMsFull, incl - cnt, wsel);
        const bool has = t < total;
        int64_t v = 0;
        Mask<W> want = Mask<W>::zero(), want1 = Mask<W>::zero();
        int64_t s = 0, e = 0;
        if (has) {
          v = (w0 + wsel) * 32 + (__fns(wbits, 0, t - before + 1) & 31);
          const Mask<W> fv = ld_mask<W>(cur, v);
          const Mask<W> seen = ld_mask<W>(p.vis, v) | fv;
          if (fv.any()) st_mask<W>(p.vis, v, seen);
          want = active.andnot(seen);
          if (after_push) want1 = fv;
          if (want.any() || want1.any()) {
            s = __ldg(p.in_off + v);
            e = __ldg(p.in_off + v + 1);
          }
        }
        // every running lane visited: no lane can reach v again (finished
        // lanes never run again), so later rounds skip it
        const bool done = has && !want.any();
        bool claimed = false, over = false;
        int64_t deg = 0;
        const bool scan = want.any() || want1.any();
        if (__ballot_sync(kMsFull, scan)) {
          Mask<W> got = Mask<W>::zero();
          if (scan) got = or_thread_rec<W>(p, v, s, e, want, cur, prev, want1, over);
          claimed = got.any();
          if (claimed) {
            st_mask<W>(nxt, v, got);
            acc_lanes<W>(acc, got);
            deg = sym ? e - s : __ldg(p.out_off + v + 1) - __ldg(p.out_off + v);
          }
        }
        // per word of the batch: claim bits (T_{L+1}), records overflow
        // (scanmap), finished bits
        const unsigned mybit = 1u << (unsigned)(v & 31);
        const int wlo = __shfl_sync(kMsFull, wsel, 0);
        const int whi = __shfl_sync(kMsFull, wsel, min(31, total - 1 - b0));
        for (int j = wlo; j <= whi; ++j) {  // uniform: the whole warp
          const bool inj = has && wsel == j;
          const unsigned cb = __reduce_or_sync(kMsFull, inj && claimed ? mybit : 0u);
          const unsigned ob = __reduce_or_sync(kMsFull, inj && over ? mybit : 0u);
          const unsigned db = __reduce_or_sync(kMsFull, inj && done ? mybit : 0u);
          if (lane == j) {
            finw |= db;
            if (cb) atomicOr(tnext + w0 + j, cb);
            if (ob) atomicOr(p.scanmap + w0 + j, ob);
          }
        }
        ms_enqueue<false>(claimed, (int32_t)v, deg, q, p.n, boff, &Rn->nlight, &Rn->big, acc);
      }
      if (finw != fin0) p.fin[w0 + lane] = finw;
    } else if (item < nlg + nmg) {
      const unsigned mi = item - nlg;
      const int64_t j0 = (int64_t)mi * kMedGrab;
      const int64_t j1 = min(j0 + kMedGrab, p.nmed);
      // 64 lanes: lanes 0 .. kMedGrab-1 look at the group's vertices at once
      // (the lanes each still wants and its in-list) and the warp then scans
      // those wanting any; 128 lanes (more registers): one vertex at a time
      int32_t vq = 0;
      Mask<W> wq = Mask<W>::zero();
      int64_t sq = 0, eq = 0;
      bool cq = false;  // 64 lanes: lane t's vertex was claimed (queued once, at the end)
      if (W == 1 && lane < j1 - j0) {
        vq = p.med_vtx[j0 + lane];
        // F_L joins vis here for medium vertices (the light loop does it
        // for light ones, the hub merge for hubs)
        const Mask<W> fq = ld_mask<W>(cur, vq);
        const Mask<W> sq0 = ld_mask<W>(p.vis, vq) | fq;
        if (fq.any()) st_mask<W>(p.vis, vq, sq0);
        wq = active.andnot(sq0);
        sq = __ldg(p.in_off + vq);
        eq = __ldg(p.in_off + vq + 1);
      }
      unsigned pend = W == 1 ? __ballot_sync(kMsFull, wq.any())
                             : (1u << (unsigned)(j1 - j0)) - 1u;
      while (pend) {
        const int t = __ffs(pend) - 1;
        pend &= pend - 1;
        const int64_t j = j0 + t;
        int32_t v;
        Mask<W> want;
        int64_t s, e;
        if (W == 1) {
          v = __shfl_sync(kMsFull, vq, t);
#pragma unroll
          for (int w = 0; w < W; ++w) want.w[w] = __shfl_sync(kMsFull, wq.w[w], t);
          s = __shfl_sync(kMsFull, sq, t);
          e = __shfl_sync(kMsFull, eq, t);
        } else {
          v = p.med_vtx[j];
          const Mask<W> fvm = ld_mask<W>(cur, v);
          const Mask<W> svm = ld_mask<W>(p.vis, v) | fvm;
          __syncwarp();
          if (lane == 0 && fvm.any()) st_mask<W>(p.vis, v, svm);
          want = active.andnot(svm);
          if (!want.any()) continue;
          s = __ldg(p.in_off + v);
          e = __ldg(p.in_off + v + 1);
        }
        // medium vertex j has candidate slot j: its parents of this round go there
        const Mask<W> got = or_warp_first<W>(p, s, e, want, cur, p.cand + j * (64 * W), false);
        const bool claimed = lane == 0 && got.any();
        int64_t deg = 0;
        if (claimed) {
          st_mask<W>(nxt, v, got);
          atomicOr(tnext + (v >> 5), 1u << (v & 31));
          acc_lanes<W>(acc, got);
          if (W != 1) deg = __ldg(p.out_off + v + 1) - __ldg(p.out_off + v);
        }
        if (W == 1) {
          if (lane == t && got.any()) cq = true;
        } else {
          ms_enqueue<false>(claimed, v, deg, q, p.n, boff, &Rn->nlight, &Rn->big, acc);
        }
      }
      // the group's claimed vertices queued together: one atomic, not one each
      if (W == 1) {
        const int64_t dq =
            !cq ? 0 : (sym ? eq - sq : __ldg(p.out_off + vq + 1) - __ldg(p.out_off + vq));
        ms_enqueue<false>(cq, vq, dq, q, p.n, boff, &Rn->nlight, &Rn->big, acc);
      }
    } else {
      const unsigned hi_item = item - nlg - nmg;
      const unsigned c1 = min((hi_item + 1) * kHubGrab, nchunks);
      // a hub whose chunk c' < c found every wanted lane: chunk c holds only
      // higher-index entries, which could not be parents (known to this item
      // at once, to others through hub_done, tagged with the round)
      const unsigned tag = (unsigned)(L + 1) << 24;
      int done_h = -1;
      for (unsigned ci = hi_item * kHubGrab; ci < c1; ++ci) {
        const unsigned c = p.hub_chunk_order[ci];  // by rank within the hub, then hub
        const int h = (int)p.hub_of_chunk[c];
        if (h == done_h) continue;
        const unsigned d = *(volatile unsigned *)(p.hub_done + h);
        if ((d & 0xFF000000u) == tag && 0xFFFFFFu - (d & 0xFFFFFFu) < c) continue;
        const int32_t v = p.hub_vtx[h];
        const Mask<W> want = active.andnot(ld_mask<W>(p.vis, v) | ld_mask<W>(cur, v));
        if (!want.any()) continue;
        const int64_t s = __ldg(p.in_off + v) + (int64_t)(c - p.hub_choff[h]) * kHubChunk;
        const int64_t e = min(s + (int64_t)kHubChunk, __ldg(p.in_off + v + 1));
        // hub h has candidate slot nmed + h; several warps scan its chunks
        const Mask<W> got = or_warp_first<W>(p, s, e, want, cur,
                                             p.cand + (p.nmed + h) * (64 * W), true);
        if (got == want) {
          done_h = h;
          if (lane == 0) atomicMax(p.hub_done + h, tag | (0xFFFFFFu - c));
        }
        if (lane == 0) {
#pragma unroll
          for (int w = 0; w < W; ++w)
            if (got.w[w])
              atomicOr(reinterpret_cast<unsigned long long *>(p.hub_found + (int64_t)h * W + w),
                       (unsigned long long)got.w[w]);
        }
      }
    }
    item = __shfl_sync(kMsFull, nextitem, 0);
  }
}

// After the wait that ends a pull round's scans: hubs found this round get
// their next mask and claim bit, and are queued if big.
template <int W>
__device__ void lg_hub_merge(const MsParams &p, int L, const uint64_t *cur, uint64_t *nxt,
                             MsRound *Rn, MsAcc &acc) {
  const int lane = lane_id();
  const int nwarps = (gridDim.x * blockDim.x) >> 5;
  const int next_parity = (L + 1) & 1;
  int32_t *q = next_parity ? p.queue1 : p.queue0;
  uint32_t *boff = next_parity ? p.bigoff1 : p.bigoff0;
  uint32_t *tnext = claims(p, L + 1);
  for (int64_t h0 = (int64_t)warp_id_global() * 32; h0 < p.nhub; h0 += (int64_t)nwarps * 32) {
    const int64_t h = h0 + lane;
    bool claimed = false;
    int32_t v = 0;
    int64_t deg = 0;
    if (h < p.nhub) {
      // F_L joins vis for the hubs (their chunk scans have ended)
      const int32_t vh = p.hub_vtx[h];
      const Mask<W> fh = ld_mask<W>(cur, vh);
      if (fh.any()) st_mask<W>(p.vis, vh, ld_mask<W>(p.vis, vh) | fh);
      const Mask<W> found = ld_mask<W>(p.hub_found, h);
      if (found.any()) {
        v = vh;
        st_mask<W>(nxt, v, found);
        st_mask<W>(p.hub_found, h, Mask<W>::zero());
        atomicOr(tnext + (v >> 5), 1u << (v & 31));
        acc_lanes<W>(acc, found);
        deg = __ldg(p.out_off + v + 1) - __ldg(p.out_off + v);
        claimed = true;
      }
    }
    ms_enqueue<false>(claimed, v, deg, q, p.n, boff, &Rn->nlight, &Rn->big, acc);
  }
}

// Edge u -> v of a push round: the lanes of u's frontier that v has neither
// visited nor in its own frontier of this round are ORed into v's next mask
// (after a read, so hot targets see few atomics); a vertex with a candidate
// slot also takes u as a parent candidate per lane (atomicMin).  The loads
// that depend only on v go out together; with a sparse frontier (`tfront`,
// its claim bitmap) v's own frontier mask is read only if v is in it.
// Returns whether this thread claimed v (set its bit in the next claim
// bitmap first).
template <int W>
__device__ __forceinline__ bool lg_relax(const MsParams &p, const Mask<W> &fu, int32_t u,
                                         int32_t v, const uint64_t *cur, uint64_t *nxt,
                                         uint32_t *tnext, const uint32_t *tfront, MsAcc &acc) {
  const Mask<W> seen = ld_mask<W>(p.vis, v);
  const Mask<W> have = ld_mask<W>(nxt, v);
  const int slot = p.cand_slot[v];
  const uint32_t tw = tnext[v >> 5];
  Mask<W> now = Mask<W>::zero();
  if (!tfront || ((tfront[v >> 5] >> (v & 31)) & 1u)) now = ld_mask<W>(cur, v);
  const Mask<W> f = fu.andnot(seen | now);
  if (!f.any()) return false;
  acc_lanes<W>(acc, f);
  if (slot >= 0) {
    // lowest source per new lane: read first (a lower one is often there
    // already), four lanes' reads in flight at a time
    uint32_t *cand = p.cand + (int64_t)slot * (64 * W);
#pragma unroll
    for (int j = 0; j < W; ++j) {
      uint64_t bits = f.w[j];
      while (bits) {
        int b[4];
        uint32_t c[4];
#pragma unroll
        for (int k = 0; k < 4; ++k) {
          b[k] = bits ? __ffsll((long long)bits) - 1 : -1;
          bits &= bits ? bits - 1 : 0ull;
        }
#pragma unroll
        for (int k = 0; k < 4; ++k) c[k] = b[k] >= 0 ? cand[j * 64 + b[k]] : 0u;
#pragma unroll
        for (int k = 0; k < 4; ++k)
          if (b[k] >= 0 && (unsigned)u < c[k]) atomicMin(cand + j * 64 + b[k], (unsigned)u);
      }
    }
  }
  const Mask<W> add = f.andnot(have);
#pragma unroll
  for (int i = 0; i < W; ++i)
    if (add.w[i])
      atomicOr(reinterpret_cast<unsigned long long *>(nxt + (int64_t)v * W + i),
               (unsigned long long)add.w[i]);
  const uint32_t tb = 1u << (v & 31);
  if (tw & tb) return false;
  return (atomicOr(tnext + (v >> 5), tb) & tb) == 0;
}

template <int W>
__device__ __forceinline__ void lg_step(const MsParams &p, bool valid, const Mask<W> &fu,
                                        int32_t u, int64_t e, const uint64_t *cur, uint64_t *nxt,
                                        uint32_t *tnext, const uint32_t *tfront, int32_t *q,
                                        uint32_t *boff, MsRound *Rn, MsAcc &acc) {
  bool claimed = false;
  int32_t v = 0;
  int64_t deg = 0;
  if (valid) {
    v = __ldg(p.out_idx + e);
    claimed = lg_relax<W>(p, fu, u, v, cur, nxt, tnext, tfront, acc);
    if (claimed) deg = __ldg(p.out_off + v + 1) - __ldg(p.out_off + v);
  }
  ms_enqueue<false>(claimed, v, deg, q, p.n, boff, &Rn->nlight, &Rn->big, acc);
}

// Edge positions [x0, x1) of the big-vertex edge space (queue entries
// q[cap-1-j] with prefix offsets boff[j], all of out-degree > kLightMax).
template <int W>
__device__ void lg_push_chunk(const MsParams &p, const uint64_t *cur, uint64_t *nxt,
                              uint32_t *tnext, const int32_t *bq, const uint32_t *boff,
                              unsigned nbig, unsigned x0, unsigned x1, const uint32_t *tfront,
                              int32_t *q, uint32_t *qoff, MsRound *Rn, MsAcc &acc) {
  const int lane = lane_id();
  const int64_t cap = p.n;
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
    lg_step<W>(p, valid, fu, u, e, cur, nxt, tnext, tfront, q, qoff, Rn, acc);
  }
}

// Push round.  Work items: the big vertices' edges in chunks (from the
// queue, as in the direct kernel), then groups of 32 claim words (1024
// vertices): the frontier vertices there merge their lanes into vis, and the
// light ones (out-degree <= kLightMax) spread their edges over the warp.
template <int W>
__device__ void lg_push(const MsParams &p, int L, const uint64_t *cur, uint64_t *nxt,
                        bool sparse, MsRound *Rc, MsRound *Rn, MsAcc &acc) {
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
  const uint32_t *tcur = claims(p, L);
  uint32_t *tnext = claims(p, L + 1);
  // a frontier of under n/1024 vertices (few targets are in it): its claim
  // bitmap (1/64 of a mask plane, cache-resident) is tested before a
  // target's frontier mask is read
  const uint32_t *tfront = sparse ? tcur : nullptr;

  const unsigned long long bigw = *(volatile unsigned long long *)&Rc->big;
  const unsigned nbig = (unsigned)(bigw >> 32), big_edges = (unsigned)bigw;
  unsigned chunk = ((big_edges / (unsigned)nwarps) + 31u) & ~31u;
  chunk = chunk < 32u ? 32u : (chunk > (unsigned)kPushChunk ? (unsigned)kPushChunk : chunk);
  const unsigned nb = (big_edges + chunk - 1) / chunk;
  const unsigned ngroups = (unsigned)((p.words + 31) / 32);
  const unsigned nitems = nb + ngroups;
  unsigned item = (unsigned)warp_id_global();
  while (item < nitems) {
    if (item < nb) {
      const unsigned x0 = item * chunk;
      lg_push_chunk<W>(p, cur, nxt, tnext, qc, bc, nbig, x0, min(x0 + chunk, big_edges), tfront,
                       qn, bn, Rn, acc);
    } else {
      // the group's frontier vertices, compacted 32 at a time: lane j holds
      // word j; the t-th frontier vertex is the (t - prefix)-th set bit of the
      // word whose prefix count covers t
      const int64_t w0 = (int64_t)(item - nb) * 32;
      const uint32_t mine = w0 + lane < p.words ? tcur[w0 + lane] : 0u;
      const int cnt = __popc(mine);
      int incl_c = cnt;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const int t = __shfl_up_sync(kMsFull, incl_c, o);
        if (lane >= o) incl_c += t;
      }
      const int total_v = __shfl_sync(kMsFull, incl_c, 31);
      for (int b0 = 0; b0 < total_v; b0 += 32) {
        const int t = b0 + lane;
        int32_t u = -1;
        int64_t s = 0, d = 0;
        // word holding the t-th vertex: the first lane whose inclusive count
        // exceeds t (the counts never decrease)
        int wsel = 0;
#pragma unroll
        for (int step = 16; step > 0; step >>= 1)
          if (__shfl_sync(kMsFull, incl_c, wsel + step - 1) <= t) wsel += step;
        const uint32_t wbits = __shfl_sync(kMsFull, mine, wsel);
        const int before = __shfl_sync(kMsFull, incl_c - cnt, wsel);
        if (t < total_v) {
          const int bit = __fns(wbits, 0, t - before + 1);
          const int64_t v = (w0 + wsel) * 32 + bit;
          const Mask<W> fv = ld_mask<W>(cur, v);
          st_mask<W>(p.vis, v, ld_mask<W>(p.vis, v) | fv);
          s = __ldg(p.out_off + v);
          d = __ldg(p.out_off + v + 1) - s;
          if (d > kLightMax)
            d = 0;  // big: its edges are in the chunks above
          else
            u = (int32_t)v;
        }
        int64_t incl = d;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
          const int64_t tt = __shfl_up_sync(kMsFull, incl, o);
          if (lane >= o) incl += tt;
        }
        const int64_t total = __shfl_sync(kMsFull, incl, 31);
        s_u[wib][lane] = u;
        s_s[wib][lane] = s;
        s_x[wib][lane] = incl - d;
        __syncwarp();
        for (int64_t base = 0; base < total; base += 32) {
          const int64_t t2 = base + lane;
          const bool valid = t2 < total;
          int64_t e = 0;
          int32_t uu = 0;
          Mask<W> fu = Mask<W>::zero();
          if (valid) {
            int lo = 0, hi = 31;
            while (lo < hi) {
              const int mid = (lo + hi + 1) >> 1;
              if (s_x[wib][mid] <= t2)
                lo = mid;
              else
                hi = mid - 1;
            }
            uu = s_u[wib][lo];
            fu = ld_mask<W>(cur, uu);
            e = s_s[wib][lo] + (t2 - s_x[wib][lo]);
          }
          lg_step<W>(p, valid, fu, uu, e, cur, nxt, tnext, tfront, qn, bn, Rn, acc);
        }
        __syncwarp();
      }
    }
    unsigned nextitem = 0;
    if (lane == 0) nextitem = (unsigned)nwarps + atomicAdd(&Rc->work, 1u);
    item = __shfl_sync(kMsFull, nextitem, 0);
  }
}

// End of round L (last block to arrive): termination, the next direction,
// statistics, the history bound -- round L + 1 writes F_{L+2}, which must be
// a plane -- and the reset of the record round L + 1 fills.  Lane discoveries
// per round are counted by the output pass, from the history.
template <int W>
__device__ unsigned lg_decide(const MsParams &p, int L, int dir, int ran) {
  MsCtl *ctl = p.ctl;
  const MsRound *Rn = &ctl->rec[(L + 1) % kRing];
  unsigned long long nf = 0, mf = 0;
#pragma unroll
  for (int i = 0; i < kCounterShards; ++i) {
    nf += *(volatile const unsigned long long *)&Rn->nf[i];
    mf += *(volatile const unsigned long long *)&Rn->mf[i];
  }
  cg_stats *st = p.stats;
  const long long now = global_ns();
  if (ran < CG_HISTORY) {
    st->direction_history[ran] = dir;
    st->round_ns[ran] = now - ctl->t_round;
  }
  ctl->t_round = now;
  if (dir == 1) ctl->pull_rounds += 1;
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
    st->pull_rounds = ctl->pull_rounds;
    st->switches = ctl->switches;
    st->history_len = rounds < CG_HISTORY ? rounds : CG_HISTORY;
    st->device_ms = 0.f;
  }
  return (stop ? kMsStop : 0u) | (next ? kMsNextPull : 0u) |
         (nf * 1024 < (unsigned long long)p.n ? kMsSparse : 0u);
}

template <int W>
struct LgRoundDecision {
  const MsParams *p;
  int L, dir, ran;
  __device__ unsigned operator()() const { return lg_decide<W>(*p, L, dir, ran); }
};

struct LgSetupDecision {
  MsCtl *ctl;
  cg_stats *st;
  __device__ unsigned operator()() const {
    const long long now = global_ns();
    st->setup_ns = now - ctl->t_start;
    st->finish_ns = 0;
    st->visited = 0;
    for (int i = 0; i < CG_HISTORY; ++i) st->nf_history[i] = 0;
    ctl->t_round = now;
    return 0u;
  }
};

// The rounds of one batch (cooperative, persistent): roots[0..k) seeded in
// F_0 and T_0; round L reads F_L and T_L, writes F_{L+1} and T_{L+1}, clears
// F_{L+2} and T_{L+2}.
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
    p.touched2[w] = 0;
    p.scanmap[w] = 0;
    p.fin[w] = 0;
  }
  uint32_t *pn = reinterpret_cast<uint32_t *>(p.pair_n);
  for (int64_t w = gtid; w < (p.n + 3) / 4; w += nthreads) pn[w] = 0;
  bool ok = grid_wait(&ctl->wait, &ctl->status, p.timeout_ns);
  if (ok && blockIdx.x == 0 && threadIdx.x < p.k) {
    const int i = threadIdx.x;
    const int32_t r = p.roots[i];
    const unsigned long long bit = 1ull << (i & 63);
    atomicOr(reinterpret_cast<unsigned long long *>(f0 + (int64_t)r * W + (i >> 6)), bit);
    atomicOr(p.touched0 + (r >> 5), 1u << (r & 31));
    bool first = true;
    for (int j = 0; j < i; ++j) first = first && (p.roots[j] != r);
    if (first) {
      const int64_t deg = p.out_off[r + 1] - p.out_off[r];
      MsRound *R0 = &ctl->rec[0];
      if (deg > kLightMax) {
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
  int L = 0, dir = 0, pdir = 0, ran = 0;
  bool sparse = false;  // this round's frontier has under n/1024 vertices (round 0: not tested)
  MsAcc acc, tot;
  while (ok) {
    const uint64_t *cur = plane<W>(p, L);
    uint64_t *nxt = plane<W>(p, L + 1);
    MsRound *Rc = &ctl->rec[L % kRing];
    MsRound *Rn = &ctl->rec[(L + 1) % kRing];
    if (L + 2 < p.hist_planes) {
      uint64_t *clr = plane<W>(p, L + 2);
      for (int64_t i = gtid; i < p.n * W; i += nthreads) clr[i] = 0;
    }
    uint32_t *tclr = claims(p, L + 2);
    for (int64_t w = gtid; w < p.words; w += nthreads) tclr[w] = 0;
    if (L >= 2 && pdir == 0 && (dir == 0 || W != 1)) {
      // a push round gave these vertices lanes at level L >= 2 and this
      // round is a push too (or 128 lanes): the scan pass resolves their
      // parents (else this pull round's light scans do, or_thread_rec)
      const uint32_t *tcur = claims(p, L);
      for (int64_t w = gtid; w < p.words; w += nthreads) {
        const uint32_t t = tcur[w];
        if (t) atomicOr(p.scanmap + w, t);
      }
    }
    if (dir == 1) {
      Mask<W> active;
#pragma unroll
      for (int i = 0; i < W; ++i) active.w[i] = *(volatile unsigned long long *)&Rc->lanes[i];
      lg_pull<W>(p, L, cur, nxt, active, L >= 2 && pdir == 0, Rc, Rn, acc);
      if (p.nhub > 0) {
        if (!(ok = grid_wait(&ctl->wait, &ctl->status, p.timeout_ns))) break;
        lg_hub_merge<W>(p, L, cur, nxt, Rn, acc);
      }
    } else {
      lg_push<W>(p, L, cur, nxt, sparse, Rc, Rn, acc);
    }
    ms_block_totals(acc, tot);
    if (threadIdx.x == 0) {
      const int sh = blockIdx.x % kCounterShards;
      if (tot.nf) atomicAdd(&Rn->nf[sh], tot.nf);
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
    pdir = dir;
    dir = (payload & kMsNextPull) ? 1 : 0;
    sparse = (payload & kMsSparse) != 0;
    ++L;
    ++ran;
  }
  if (blockIdx.x == 0 && threadIdx.x == 0 && !ok)
    p.stats->status = *(volatile int *)&ctl->status;
}

// ---- scan pass, output pass, fix-up pass ------------------------------------

constexpr int kScanBlock = 256;  // scan and fix-up passes: threads a block
constexpr int kScanWords = 4;    // scan pass: scanmap words a warp takes at a time
constexpr int kScanG = 2;        // in-list entries loaded together (most lanes resolve at the first)
constexpr int kPre = 8;          // history planes loaded together (the output pass needs 8)

// The planes the rounds filled: F_0 .. F_{rounds - 1} (F_rounds is empty).
__device__ __forceinline__ int history_rounds(const MsParams &p) {
  int rounds = *(volatile int *)&p.ctl->L;
  if (rounds > p.hist_planes) rounds = p.hist_planes;
  if (rounds > CG_HISTORY + 1) rounds = CG_HISTORY + 1;
  return rounds;
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

// The lanes of `todo` (half h) that light vertex v reached at a level >= 2,
// resolved by scans of v's ascending in-list: the first entry u holding the
// lane in F_{level - 1}[u] is the lane's parent, the lowest-index rule.  One
// pass over the list resolves up to kOutLevels levels; hit(u, lanes) gets
// each entry that resolves lanes.
template <int W, int G, class Hit>
__device__ __forceinline__ void scan_in_list(const MsParams &p, int64_t v, int h, int rounds,
                                             int64_t s, int64_t e, uint64_t todo, Hit &&hit) {
  int L = 2;
  while (todo && L < rounds) {
    int Ls[kOutLevels];
    uint64_t Ms[kOutLevels];
#pragma unroll
    for (int k = 0; k < kOutLevels; ++k) {
      Ls[k] = 1;
      Ms[k] = 0;
    }
    int nl = 0;
    uint64_t gtodo = 0;
    while (nl < kOutLevels && L < rounds && todo) {
      uint64_t pm[kPre];
#pragma unroll
      for (int j = 0; j < kPre; ++j)
        pm[j] = L + j < rounds ? plane<W>(p, L + j)[v * W + h] : 0ull;
      int taken = 0;
#pragma unroll
      for (int j = 0; j < kPre; ++j) {
        if (nl < kOutLevels) {
          const uint64_t m = pm[j] & todo;
          if (m) {
#pragma unroll
            for (int k = 0; k < kOutLevels; ++k)
              if (k == nl) {
                Ls[k] = L + j;
                Ms[k] = m;
              }
            ++nl;
            todo &= ~m;
            gtodo |= m;
          }
          taken = j + 1;
        }
      }
      L += taken;
    }
    for (int64_t j0 = s; j0 < e && gtodo; j0 += G) {
      int32_t u[G];
      uint64_t b[G];
#pragma unroll
      for (int k = 0; k < G; ++k) u[k] = j0 + k < e ? __ldg(p.in_idx + j0 + k) : -1;
#pragma unroll
      for (int k = 0; k < G; ++k)
        b[k] = u[k] >= 0 ? parent_hits<W>(p, u[k], h, Ls, Ms, gtodo) : 0;
#pragma unroll
      for (int k = 0; k < G; ++k) {
        const uint64_t bk = b[k] & gtodo;
        if (bk) {
          gtodo &= ~bk;
          hit(u[k], bk);
        }
      }
    }
  }
}

// OR of the masks of records [0, np) of vertex v, half h (np <= kRecords).
template <int W>
__device__ __forceinline__ uint64_t records_mask(const MsParams &p, int64_t v, int h, int np) {
  uint64_t m = 0;
#pragma unroll
  for (int q = 0; q < kRecords; ++q)
    if (q < np) m |= p.pair_m[((int64_t)q * p.n + v) * W + h];
  return m;
}

// Scan pass, between the rounds and the output pass, over the light vertices
// (in-degree 1 .. kPullLight; heavier ones have candidate slots) that the
// rounds marked in scanmap: reached by a push round at a level >= 2, or with
// more pull-round first hits than records.  A warp takes kScanWords words of
// the map at a time (the first by its index, the next from a counter, claimed
// before the current chunk is worked), compacts their marked vertices in
// shared memory, and gives each thread one.
// The lanes a vertex's records leave open are resolved by scan_in_list and
// appended as records; a vertex that runs out of records goes on a list
// (queue0, free once the rounds are over) for the fix-up pass.
template <int W>
__global__ void __launch_bounds__(kScanBlock) msbfs_scan(MsParams p) {
  __shared__ int32_t s_list[kScanBlock / 32][kScanWords * 32];
  __shared__ int32_t s_ru[kScanBlock][kRecords + 1];  // a thread's record sources
  if (*(volatile int *)p.flag || *(volatile int *)&p.ctl->status != 0) return;
  const int rounds = history_rounds(p);
  if (rounds <= 2) return;
  const int lane = lane_id();
  int32_t *list = s_list[threadIdx.x >> 5];
  const unsigned nwarps = gridDim.x * (kScanBlock / 32);
  const unsigned nchunks = (unsigned)((p.words + kScanWords - 1) / kScanWords);
  unsigned chunk = (unsigned)warp_id_global();
  while (chunk < nchunks) {
    unsigned next = 0;
    if (lane == 0) next = nwarps + atomicAdd(&p.ctl->scan_work, 1u);
    const int64_t w0 = (int64_t)chunk * kScanWords;
    const int64_t wi = w0 + lane;
    uint32_t bits = lane < kScanWords && wi < p.words ? p.scanmap[wi] : 0u;
    const int c = __popc(bits);
    int incl = c;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
      const int y = __shfl_up_sync(kMsFull, incl, d);
      if (lane >= d) incl += y;
    }
    const int total = __shfl_sync(kMsFull, incl, 31);
    for (int at = incl - c; bits; bits &= bits - 1) list[at++] = (int32_t)(wi * 32 + __ffs(bits) - 1);
    __syncwarp();
    for (int i = lane; i < total; i += 32) {
      const int64_t v = list[i];
      const int64_t s = __ldg(p.in_off + v), e = __ldg(p.in_off + v + 1);
      if (e == s || e - s > kPullLight) continue;
      const int np0 = p.pair_n[v];
      int np = np0;
      bool over = false;
      // the records' sources: a hit from a source already recorded joins its
      // record (pull rounds record a source again in each round it serves)
      int32_t *ru = s_ru[threadIdx.x];
      for (int q = 0; q < np0; ++q) ru[q] = p.pair_u[(int64_t)q * p.n + v];
      for (int h = 0; h < W && 64 * h < p.k; ++h) {
        const uint64_t covered = records_mask<W>(p, v, h, np0);
        scan_in_list<W, kScanG>(p, v, h, rounds, s, e, ~covered, [&](int32_t u, uint64_t m) {
          int found = -1;
          for (int q = 0; q < np && found < 0; ++q)
            if (ru[q] == u) found = q;
          if (found >= 0) {
            p.pair_m[((int64_t)found * p.n + v) * W + h] |= m;
          } else if (np < kRecords) {
            const int64_t at = (int64_t)np * p.n + v;
            p.pair_u[at] = u;
#pragma unroll
            for (int w = 0; w < W; ++w) p.pair_m[at * W + w] = w == h ? m : 0ull;
            ru[np] = u;
            ++np;
          } else {
            over = true;
          }
        });
      }
      if (np != np0) p.pair_n[v] = (uint8_t)np;
      if (over) p.queue0[atomicAdd(&p.ctl->nover, 1u)] = (int32_t)v;
    }
    __syncwarp();
    chunk = __shfl_sync(kMsFull, next, 0);
  }
}

// Fix-up pass, after the output pass: the lanes of the listed vertices that
// no record covers (a vertex with more distinct parents than kRecords) get
// their parents written one by one.  One warp a vertex, 32 in-list entries
// at a time in ascending order: lane j holds entry j of the chunk and gathers
// that entry's history masks for up to kPre levels at once; the 32 x 64 hit
// matrix is transposed a 32-lane word at a time (warp_transpose32), so warp
// lane b finds the chunk's first entry -- the lowest-index parent, earlier
// chunks having had no hit -- of lane b of that word.
template <int W>
__global__ void __launch_bounds__(kScanBlock, W == 1 ? 6 : 4) msbfs_fixup(MsParams p) {
  if (*(volatile int *)p.flag || *(volatile int *)&p.ctl->status != 0) return;
  const unsigned cnt = *(volatile unsigned *)&p.ctl->nover;
  if (cnt == 0) return;
  const int rounds = history_rounds(p);
  const int lane = lane_id();
  const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t i = warp_id_global(); i < cnt; i += nwarps) {
    const int64_t v = p.queue0[i];
    const int64_t s = __ldg(p.in_off + v), e = __ldg(p.in_off + v + 1);
    const int np = min((int)p.pair_n[v], kRecords);
    for (int h = 0; h < W && 64 * h < p.k; ++h) {
      // the lanes no record covers; those reached at a level >= 2 get parents
      uint64_t todo = ~records_mask<W>(p, v, h, np);
      for (int64_t c0 = s; c0 < e && todo; c0 += 32) {  // uniform: the whole warp
        const bool has = c0 + lane < e;
        const int32_t u = has ? __ldg(p.in_idx + c0 + lane) : 0;
        for (int L0 = 2; L0 < rounds && todo; L0 += kPre) {
          uint64_t pm[kPre];
#pragma unroll
          for (int j = 0; j < kPre; ++j)
            pm[j] = L0 + j < rounds ? plane<W>(p, L0 + j)[v * W + h] & todo : 0ull;
          uint64_t hit = 0, batch = 0;
#pragma unroll
          for (int j = 0; j < kPre; ++j) {
            batch |= pm[j];
            if (pm[j] && has) hit |= pm[j] & plane<W>(p, L0 + j - 1)[(int64_t)u * W + h];
          }
          if (!batch) continue;
          uint64_t found = 0;
#pragma unroll
          for (int half = 0; half < 2; ++half) {
            const uint32_t t = warp_transpose32((uint32_t)(hit >> (32 * half)));
            const int first = t ? __ffs(t) - 1 : 0;
            const int32_t par = __shfl_sync(kMsFull, u, first);
            if (t) p.parents[(int64_t)(64 * h + 32 * half + lane) * p.n + v] = par;
            found |= (uint64_t)__ballot_sync(kMsFull, t != 0) << (32 * half);
          }
          todo &= ~found;
        }
      }
    }
  }
}

// Output pass.  Each warp takes 32 consecutive vertices (one per thread).  Per
// 64-lane half of the batch a thread reads its vertex's history masks once
// and keeps each lane's level as bit slices in registers; parents of levels
// >= 2 come from the slot's candidates (in-degree > kPullLight), copied by
// the warp into the parent row of the vertex's shared table, or from the
// vertex's (source, lanes) records: their sources in the same table, each
// lane's record index as bit slices like the levels.  Then, lane by lane,
// the warp writes the tile's 32 levels and 32 parents as two 128-byte rows,
// each parent one table read; parents of levels 0 and 1 are the vertex and
// the lane's root.
template <int W>
__global__ void __launch_bounds__(kOutBlock) msbfs_outputs(MsParams p) {
  extern __shared__ __align__(16) unsigned char s_tile[];
  __shared__ unsigned s_cnt[CG_HISTORY + 1];  // lane discoveries per level
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
  const int rounds = history_rounds(p);
  for (int i = threadIdx.x; i <= CG_HISTORY; i += blockDim.x) s_cnt[i] = 0;
  __syncthreads();
  const int lane = lane_id();
  const int wib = threadIdx.x >> 5;
  int32_t *tab = reinterpret_cast<int32_t *>(s_tile + wib * kOutWarpBytes);
  int32_t *my_tab = tab + lane * kTab;  // lane l at my_tab[(l - 8 * lane) & 63]
  my_tab[kTabNone] = -1;
  int nsl = 1;  // bit slices needed for levels 0 .. rounds - 1
  while (nsl < kSlices && (rounds - 1) >> nsl) ++nsl;
  const int64_t nwarps = (int64_t)gridDim.x * kOutWarps;
  // a tile's slot and record count are loaded one tile ahead: the tile's
  // history, candidate and record loads then all go out at its start
  int64_t tile = (int64_t)blockIdx.x * kOutWarps + wib;
  int next_slot = -1, next_np = 0;
  if (tile * 32 + lane < p.n) {
    next_slot = p.cand_slot[tile * 32 + lane];
    next_np = p.pair_n[tile * 32 + lane];
  }
  for (; tile * 32 < p.n; tile += nwarps) {
    const int64_t v = tile * 32 + lane;
    const bool valid = v < p.n;
    const int slot = next_slot;
    const int np = slot < 0 ? min(next_np, kRecords) : 0;
    const int64_t vn = (tile + nwarps) * 32 + lane;
    next_slot = -1;
    next_np = 0;
    if (vn < p.n) {
      next_slot = p.cand_slot[vn];
      next_np = p.pair_n[vn];
    }
#pragma unroll 1
    for (int h = 0; h < W && 64 * h < p.k; ++h) {
      // the first kPre history planes: independent of the slot and record
      // loads below, so they are issued first and their latency overlaps
      uint64_t pm0[kPre];
#pragma unroll
      for (int j = 0; j < kPre; ++j)
        pm0[j] = valid && j < rounds ? plane<W>(p, j)[v * W + h] : 0ull;
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
              int32_t *t = tab + src[r] * kTab + ((2 * lane - 8 * src[r]) & 63);
              t[0] = (int32_t)x[r].x;
              t[1] = (int32_t)x[r].y;
            }
          }
        }
      }
      // a light vertex's records (pull rounds, then the scan pass), four
      // records' loads in flight: sources into the thread's table, each
      // lane's record index as three bit slices rq (the masks are disjoint)
      uint64_t rq[3] = {0ull, 0ull, 0ull}, cov = 0;
      for (int q0 = 0; q0 < np; q0 += 4) {
        int32_t pu[4];
        uint64_t pmk[4];
#pragma unroll
        for (int r = 0; r < 4; ++r) {
          pu[r] = 0;
          pmk[r] = 0;
          if (q0 + r < np) {
            const int64_t at = (int64_t)(q0 + r) * p.n + v;
            pu[r] = p.pair_u[at];
            pmk[r] = p.pair_m[at * W + h];
          }
        }
#pragma unroll
        for (int r = 0; r < 4; ++r)
          if (q0 + r < np) my_tab[kTabRec + q0 + r] = pu[r];
        const uint64_t all4 = pmk[0] | pmk[1] | pmk[2] | pmk[3];
        cov |= all4;
        rq[0] |= pmk[1] | pmk[3];
        rq[1] |= pmk[2] | pmk[3];
        if (q0 & 4) rq[2] |= all4;
      }
      // each lane's level as bit slices: bit l of S[b] = bit b of lane l's level
      uint64_t S[kSlices], reached = 0, m01[2] = {0ull, 0ull};
#pragma unroll
      for (int b = 0; b < kSlices; ++b) S[b] = 0;
      m01[0] = pm0[0];
      m01[1] = pm0[1];
      for (int L0 = 0; L0 < rounds; L0 += kPre) {  // uniform: the whole warp
        uint64_t pm[kPre];
#pragma unroll
        for (int j = 0; j < kPre; ++j)
          pm[j] = L0 == 0 ? pm0[j]
                          : (valid && L0 + j < rounds ? plane<W>(p, L0 + j)[v * W + h] : 0ull);
        // L0 is a multiple of kPre = 8: bits 0..2 of level L0 + j are those
        // of j, known at compile time; bits 3.. those of L0, the same for the
        // whole batch
        uint64_t batch = 0;
#pragma unroll
        for (int j = 0; j < kPre; ++j) {
          const uint64_t m = pm[j];
          const unsigned c = __reduce_add_sync(kMsFull, (unsigned)__popcll(m));
          if (lane == 0 && c) atomicAdd(&s_cnt[L0 + j], c);
          batch |= m;
#pragma unroll
          for (int b = 0; b < 3; ++b)
            if ((j >> b) & 1) S[b] |= m;
        }
        reached |= batch;
#pragma unroll
        for (int b = 3; b < kSlices; ++b)
          if ((L0 >> b) & 1) S[b] |= batch;
      }
      __syncwarp();  // the candidate rows copied by the warp are in place
      // levels 0 and 1 (rare): the vertex itself, the lane's root
      for (uint64_t x = m01[0]; x; x &= x - 1)
        my_tab[(__ffsll((long long)x) - 1 - 8 * lane) & 63] = (int32_t)v;
      for (uint64_t x = m01[1]; x; x &= x - 1) {
        const int b = __ffsll((long long)x) - 1;
        my_tab[(b - 8 * lane) & 63] = p.roots[64 * h + b];
      }
      __syncwarp();
      // rows: lane l of this half, vertices tile*32 .. tile*32 + 31, a 32-lane
      // word of the masks at a time; four lanes' levels are built as the
      // bytes of a word (0xFF unreached, which sign-extends to -1)
      const int lanes = min(64, p.k - 64 * h);
      const int64_t n = p.n;
#pragma unroll 1
      for (int hw = 0; hw < 2 && 32 * hw < lanes; ++hw) {
        uint32_t sl[kSlices];
#pragma unroll
        for (int b = 0; b < kSlices; ++b) sl[b] = (uint32_t)(S[b] >> (32 * hw));
        const uint32_t rw = (uint32_t)(reached >> (32 * hw));
        const uint32_t cw = (uint32_t)(cov >> (32 * hw));
        uint32_t qs[3];
#pragma unroll
        for (int b = 0; b < 3; ++b) qs[b] = (uint32_t)(rq[b] >> (32 * hw));
        const int lend = min(32, lanes - 32 * hw);
        // rows of lane 64 h + 32 hw, advanced one row per lane written
        int32_t *pl = p.levels + (int64_t)(64 * h + 32 * hw) * n + v;
        int32_t *pp = p.parents + (int64_t)(64 * h + 32 * hw) * n + v;
        auto group = [&](int l4, auto checked) {
          // bytes of four lanes: 0xFF where unreached (um), where a record
          // covers the lane (cm), its level (0xFF unreached sign-extends to -1)
          const uint32_t um = spread4(~(rw >> l4) & 0xFu) * 0xFFu;
          const uint32_t cm = spread4((cw >> l4) & 0xFu) * 0xFFu;
          uint32_t word = um;
#pragma unroll
          for (int b = 0; b < kSlices; ++b)
            if (b < nsl) word |= spread4((sl[b] >> l4) & 0xFu) << b;
          // each lane's table index: its record's source, -1 when unreached,
          // else its column of the parent row ((l - 8 lane) mod 64 never
          // wraps inside an aligned group of four)
          const uint32_t qw = spread4((qs[0] >> l4) & 0xFu) | (spread4((qs[1] >> l4) & 0xFu) << 1) |
                              (spread4((qs[2] >> l4) & 0xFu) << 2);
          const uint32_t col = ((uint32_t)((32 * hw + l4 - 8 * lane) & 63) * 0x01010101u) | 0x03020100u;
          const uint32_t idx = (col & ~(cm | um)) | ((qw | (0x01010101u * kTabRec)) & cm) |
                               ((0x01010101u * kTabNone) & um);
#pragma unroll
          for (int i = 0; i < 4; ++i) {
            if (!decltype(checked)::value || l4 + i < lend) {
              const int32_t lv = (int32_t)(int8_t)(uint8_t)(word >> (8 * i));
              const int32_t pv = my_tab[(idx >> (8 * i)) & 0xFFu];
              if (valid) {  // written once, never read here: evict-first
                __stcs(pl, lv);
                __stcs(pp, pv);
              }
              pl += n;
              pp += n;
            }
          }
        };
        if (lend == 32) {
#pragma unroll
          for (int l4 = 0; l4 < 32; l4 += 4) group(l4, Flag<false>{});
        } else {
          for (int l4 = 0; l4 < lend; l4 += 4) group(l4, Flag<true>{});
        }
      }
      __syncwarp();
    }
  }
  // the statistics: lane discoveries per round (level L came from round
  // L - 1) and in all; the last block out records the time since the last
  // round ended
  __syncthreads();
  for (int i = threadIdx.x; i < rounds; i += blockDim.x) {
    const unsigned long long c = s_cnt[i];  // widened for the global sums
    if (!c) continue;
    atomicAdd(reinterpret_cast<unsigned long long *>(&p.stats->visited), c);
    if (i >= 1)
      atomicAdd(reinterpret_cast<unsigned long long *>(&p.stats->nf_history[i - 1]), c);
  }
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
  int scan_per_sm = 0;
  CG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&scan_per_sm, msbfs_scan<W>, kScanBlock, 0));
  if (scan_per_sm <= 0) return CG_ERR_NOT_SUPPORTED;
  const int64_t chunks = ((g->n + 31) / 32 + kScanWords - 1) / kScanWords;
  int64_t scan_blocks = (chunks + kScanBlock / 32 - 1) / (kScanBlock / 32);
  if (scan_blocks > (int64_t)scan_per_sm * g->num_sms) scan_blocks = (int64_t)scan_per_sm * g->num_sms;
  msbfs_scan<W><<<(unsigned)scan_blocks, kScanBlock, 0, g->stream>>>(p);
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
  int fix_per_sm = 0;
  CG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&fix_per_sm, msbfs_fixup<W>, kScanBlock, 0));
  if (fix_per_sm <= 0) return CG_ERR_NOT_SUPPORTED;
  msbfs_fixup<W><<<(unsigned)(fix_per_sm * g->num_sms), kScanBlock, 0, g->stream>>>(p);
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
