// Per-root direction-optimizing BFS: one persistent cooperative kernel that
// runs every round of a search on the device, with one grid-wide wait per round.
//
// Reference mapping (bfs/implementation/src/bool_pe.csl):
//   start_spmv (:673-729)          -> phase 0 of bfs_persistent (state reset, seed)
//   compute_topdown (:865-887)     -> push_round_*: frontier queue (or bitmap),
//                                     out-lists, atomicOr into the next frontier
//   compute_bottomup (:899-921)    -> pull_round: unvisited vertices scan their
//                                     ascending in-lists, stop at the first
//                                     frontier source
//   reduce_or + reduce_done        -> the shared bitmaps make the OR-reduce
//     (:923-1004, collectives_2d     implicit; the visited set is vis | F_L, and
//      pe.csl:319-349)                 vis |= F_L is folded into round L's work;
//                                     per-round counters give nf = popcount
//   termination relay (:1003-1046)  -> every block reads nf from the round
//                                     record after the grid-wide wait; nf == 0 ends
//   direction switch (:1078-1088)   -> next_direction(): Beamer's alpha/beta rule,
//                                     or the reference's one-way tau rule
//   reduce_select_any (:1145-1154)  -> not needed: every parent is final when it
//                                     is written (lowest-index rule below)
//
// Parent rule: the lowest-numbered in-neighbour one level closer
// (bfs/README.md:208-224).  A push round applies atomicMin over every
// frontier source of a newly reached vertex (the visited set is frozen during
// the round, so all of them are seen); a pull round takes the first frontier
// source of an ascending in-list, which is the minimum.  Parents start at
// 0xFFFFFFFF, the reference's PARENT_NONE (device_io.py:157), which reads back
// as -1 through int32 without a conversion pass.
//
// Bitmaps: vis holds the vertices of F_0 .. F_{L-1}, the frontier F_L is
// fr[L % 3], the next frontier is written into fr[(L+1) % 3] and fr[(L+2) % 3]
// (F_{L-1}) is cleared during round L.  "Visited" is tested as vis | F_L, so
// merging F_L into vis during round L races with nothing.
#include <cuda_runtime.h>

#include "cg_internal.cuh"

namespace cg {

constexpr unsigned kFull = 0xffffffffu;
constexpr int kPush = 0, kPull = 1;
constexpr int kBfsBlock = 512;
// Pull rounds: in-list entries a thread loads at once (all in flight before
// any is tested), and how many entries of its vertex's list a thread scans
// before the whole warp takes over the rest of it.
#ifndef CG_PULL_CHUNK
#define CG_PULL_CHUNK 4
#endif
#ifndef CG_PULL_LANE_MAX
#define CG_PULL_LANE_MAX 32
#endif
constexpr int kPullThreadScan = CG_PULL_CHUNK;
constexpr unsigned kPullLaneMax = CG_PULL_LANE_MAX;
constexpr int kBfsWarps = kBfsBlock / 32;

// Per-warp shared memory of the bitmap-wide rounds: a staged tile (its words
// and the exclusive prefix of their popcounts, so that a lane can select the
// k-th set bit) and the tile's next-frontier words found by a pull round.
struct __align__(16) WarpTile {  // 16-byte vector accesses to every member
  uint32_t m[kTileWords];
  uint32_t pre[kTileWords];
  uint32_t found[kTileWords];
};
static_assert(sizeof(WarpTile) % 16 == 0 && kTileWords % 4 == 0, "16-byte tile rows");
// Per-warp shared memory of a push round's edge spreading (gather_expand).
struct WarpExpand {
  int32_t u[32];
  int64_t s[32];
  int64_t x[32];
};
__shared__ WarpTile s_tiles[kBfsWarps];
__shared__ WarpExpand s_expand[kBfsWarps];

__device__ __forceinline__ uint4 ld4(const uint32_t *a) {
  return *reinterpret_cast<const uint4 *>(a);
}
// Non-coherent (read-only path) load: only for data no thread writes while
// the kernel runs (the dead-vertex map).  Bitmaps that earlier rounds wrote are
// read with ordinary loads, which the grid waits' acquire makes current.
__device__ __forceinline__ uint4 ldg4(const uint32_t *a) {
  return __ldg(reinterpret_cast<const uint4 *>(a));
}
__device__ __forceinline__ void st4(uint32_t *a, uint4 v) { *reinterpret_cast<uint4 *>(a) = v; }
__device__ __forceinline__ bool any4(uint4 v) { return (v.x | v.y | v.z | v.w) != 0u; }

// Original id of resident vertex v (the identity unless the graph was
// relabelled): the output position and the parent value outputs use.
__device__ __forceinline__ int32_t orig_id(const BfsParams &p, int64_t v) {
  return p.orig ? __ldg(p.orig + v) : (int32_t)v;
}

// Bits of word `wi` that stand for vertices < n.
__device__ __forceinline__ uint32_t valid_bits(int64_t wi, int64_t n) {
  const int64_t lo = wi * 32;
  if (lo + 32 <= n) return kFull;
  if (lo >= n) return 0u;
  return (1u << (unsigned)(n - lo)) - 1u;
}

// Stages the tile's 128 words (4 per lane, lane order) in shared memory with
// the exclusive prefix of their popcounts; returns the tile's total number of
// set bits (the same in every lane).  All 32 lanes call.
__device__ __forceinline__ unsigned stage_tile(uint4 m, WarpTile &T) {
  const int lane = lane_id();
  const unsigned c0 = __popc(m.x), c1 = __popc(m.y), c2 = __popc(m.z), c3 = __popc(m.w);
  const unsigned cnt = c0 + c1 + c2 + c3;
  unsigned incl = cnt;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const unsigned t = __shfl_up_sync(kFull, incl, o);
    if (lane >= o) incl += t;
  }
  const unsigned base = incl - cnt;
  st4(T.m + 4 * lane, m);
  st4(T.pre + 4 * lane, make_uint4(base, base + c0, base + c0 + c1, base + c0 + c1 + c2));
  __syncwarp();
  return __shfl_sync(kFull, incl, 31);
}

// The k-th set bit (k below the staged total) of the staged tile: word j of
// the tile and bit b of that word.  The last word whose prefix is <= k holds it.
__device__ __forceinline__ void select_bit(const WarpTile &T, unsigned k, int &j, int &b) {
  int lo = 0;
#pragma unroll
  for (int step = kTileWords / 2; step > 0; step >>= 1)
    if (T.pre[lo + step] <= k) lo += step;
  j = lo;
  b = (int)__fns(T.m[lo], 0, (int)(k - T.pre[lo]) + 1);
}

// A thread's discoveries in one round: vertices, and the sum of their
// out-degrees / in-degrees.  32 bits suffice: a round discovers at most n
// vertices and their degrees sum to at most nnz < 2^32 (checked at upload).
struct Acc {
  unsigned nf = 0, mf = 0, visdeg = 0;
};

// Appends the discoveries of one warp-wide step to the next frontier's queue:
// light vertices at the front; big ones at the back, each with the prefix
// offset of its edge list among the big vertices (one packed 64-bit atomic per
// warp: count in the high word, edges in the low word).  All 32 lanes call.
__device__ __forceinline__ void enqueue_claims(const BfsParams &p, bool claimed, int32_t v,
                                               int64_t deg, int next_parity, RoundRec *Rn,
                                               Acc &acc) {
  const int lane = lane_id();
  if (!__ballot_sync(kFull, claimed)) return;
  int32_t *q = next_parity ? p.queue1 : p.queue0;
  const bool light = claimed && deg <= kLightMax;
  const bool big = claimed && deg > kLightMax;
  const unsigned below = (1u << lane) - 1u;
  const unsigned ml = __ballot_sync(kFull, light);
  if (ml) {
    const int leader = __ffs(ml) - 1;
    unsigned base = 0;
    if (lane == leader) base = atomicAdd(&Rn->nlight, (unsigned)__popc(ml));
    base = __shfl_sync(kFull, base, leader);
    if (light) q[base + __popc(ml & below)] = v;
  }
  const unsigned mb = __ballot_sync(kFull, big);
  if (mb) {
    const unsigned d = big ? (unsigned)deg : 0u;
    unsigned incl = d;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const unsigned t = __shfl_up_sync(kFull, incl, o);
      if (lane >= o) incl += t;
    }
    const unsigned total = __shfl_sync(kFull, incl, 31);
    unsigned long long old = 0;
    if (lane == 0)
      old = atomicAdd(&Rn->big, ((unsigned long long)__popc(mb) << 32) | total);
    old = __shfl_sync(kFull, old, 0);
    if (big) {
      const unsigned idx = (unsigned)(old >> 32) + __popc(mb & below);
      q[p.n - 1 - (int64_t)idx] = v;
      (next_parity ? p.bigoff1 : p.bigoff0)[idx] = (unsigned)(old & 0xffffffffu) + incl - d;
    }
  }
  if (claimed) {
    acc.nf += 1;
    acc.mf += (unsigned)deg;
    acc.visdeg += (unsigned)deg;
  }
}

// Edge u -> v of a push round.  Returns true for the one thread that claims
// v, with v's out-degree in deg (its offsets are loaded with the claim, so the
// claimer does not wait for them afterwards).
__device__ __forceinline__ bool relax_push(const BfsParams &p, const uint32_t *cur,
                                           uint32_t *nxt, int32_t u, int32_t v, int next_level,
                                           int64_t &deg) {
  const uint32_t w = (uint32_t)v >> 5, bit = 1u << (v & 31);
  // the three words in one round trip: a claim bit seen set stays set
  const uint32_t seen = p.vis[w] | cur[w], claimed = nxt[w];
  if (seen & bit) return false;
  const int32_t ov = orig_id(p, v);
  atomicMin(reinterpret_cast<unsigned *>(p.parents) + ov, (unsigned)orig_id(p, u));
  if (claimed & bit) return false;
  const int64_t o0 = __ldg(p.out_off + v), o1 = __ldg(p.out_off + v + 1);
  const unsigned old = atomicOr(nxt + w, bit);
  if (old & bit) return false;
  p.levels[ov] = next_level;
  deg = o1 - o0;
  return true;
}

__device__ __forceinline__ void push_step(const BfsParams &p, const uint32_t *cur, uint32_t *nxt,
                                          bool valid, int32_t u, int64_t e, int L,
                                          int next_parity, RoundRec *Rn, Acc &acc) {
  bool claimed = false;
  int32_t v = 0;
  int64_t deg = 0;
  if (valid) {
    v = __ldg(p.out_idx + e);
    claimed = relax_push(p, cur, nxt, u, v, L + 1, deg);
  }
  enqueue_claims(p, claimed, v, deg, next_parity, Rn, acc);
}

// Expands up to 32 frontier vertices (one per lane, u < 0 for none) with the
// warp's combined edge list spread evenly over its lanes.
__device__ __forceinline__ void gather_expand(const BfsParams &p, const uint32_t *cur,
                                              uint32_t *nxt, int32_t u, int L, int next_parity,
                                              RoundRec *Rn, Acc &acc, int32_t *s_u, int64_t *s_s,
                                              int64_t *s_x) {
  const int lane = lane_id();
  int64_t s = 0, d = 0;
  if (u >= 0) {
    s = __ldg(p.out_off + u);
    d = __ldg(p.out_off + u + 1) - s;
  }
  int64_t incl = d;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int64_t t = __shfl_up_sync(kFull, incl, o);
    if (lane >= o) incl += t;
  }
  const int64_t total = __shfl_sync(kFull, incl, 31);
  if (total == 0) return;
  s_u[lane] = u;
  s_s[lane] = s;
  s_x[lane] = incl - d;
  __syncwarp();
  for (int64_t base = 0; base < total; base += 32) {
    const int64_t t = base + lane;
    const bool valid = t < total;
    int32_t uu = 0;
    int64_t e = 0;
    if (valid) {
      int lo = 0, hi = 31;
      while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (s_x[mid] <= t)
          lo = mid;
        else
          hi = mid - 1;
      }
      uu = s_u[lo];
      e = s_s[lo] + (t - s_x[lo]);
    }
    push_step(p, cur, nxt, valid, uu, e, L, next_parity, Rn, acc);
  }
  __syncwarp();
}

// Expands frontier F_L from its queue (parity L & 1): edge-balanced chunks of
// the big vertices' combined edge list, then the light vertices 32 to a warp.
// Item i goes to warp i first; warps that finish take the rest from a counter.
// bigw / nlight: F_L's queue sizes ((big count << 32) | big edges, light
// count), handed over with the barrier that ended round L - 1.
__device__ void push_round_queue(const BfsParams &p, const uint32_t *cur, uint32_t *nxt, int L,
                                 RoundRec *Rc, RoundRec *Rn, unsigned long long bigw,
                                 unsigned nlight, Acc &acc) {
  const int lane = lane_id();
  const int wib = threadIdx.x >> 5;
  const int nwarps = (gridDim.x * blockDim.x) >> 5;
  const int parity = L & 1, next_parity = parity ^ 1;
  const int32_t *q = parity ? p.queue1 : p.queue0;
  const uint32_t *boff = parity ? p.bigoff1 : p.bigoff0;

  const unsigned nbig = (unsigned)(bigw >> 32);
  const unsigned big_edges = (unsigned)(bigw & 0xffffffffu);
  // chunks of 32 .. kPushChunk edges: small frontiers still spread over the grid
  unsigned chunk = ((big_edges / (unsigned)nwarps) + 31u) & ~31u;
  chunk = chunk < 32u ? 32u : (chunk > (unsigned)kPushChunk ? (unsigned)kPushChunk : chunk);
  const unsigned nchunks = (big_edges + chunk - 1) / chunk;
  const unsigned nitems = nchunks + (nlight + 31u) / 32u;
  unsigned item = (unsigned)warp_id_global();
  while (item < nitems) {
    // the next item is claimed before this one is worked, hiding the atomic
    unsigned nextitem = 0;
    if (lane == 0) nextitem = (unsigned)nwarps + atomicAdd(&Rc->work, 1u);
    if (item < nchunks) {
      const unsigned x0 = item * chunk;
      const unsigned x1 = min(x0 + chunk, big_edges);
      // big vertex j holding edge position x0: the last j with boff[j] <= x0
      unsigned lo = 0, hi = nbig - 1;
      while (lo < hi) {
        const unsigned mid = (lo + hi + 1) >> 1;
        if (boff[mid] <= x0)
          lo = mid;
        else
          hi = mid - 1;
      }
      unsigned j = lo;
      int32_t vj = q[p.n - 1 - (int64_t)j];
      int64_t sj = __ldg(p.out_off + vj);
      unsigned oj = boff[j];
      unsigned endj = oj + (unsigned)(__ldg(p.out_off + vj + 1) - sj);
      for (unsigned base = x0; base < x1; base += 32) {
        while (base >= endj) {  // the next big vertex (degrees exceed 32)
          ++j;
          vj = q[p.n - 1 - (int64_t)j];
          sj = __ldg(p.out_off + vj);
          oj = boff[j];
          endj = oj + (unsigned)(__ldg(p.out_off + vj + 1) - sj);
        }
        const unsigned x = base + lane;
        const bool valid = x < x1;
        int32_t u = vj;
        int64_t e = sj + (int64_t)(x - oj);
        if (__ballot_sync(kFull, valid && x >= endj)) {  // lanes past vertex j's end
          const int32_t vn = q[p.n - 1 - (int64_t)(j + 1)];
          if (valid && x >= endj) {
            u = vn;
            e = __ldg(p.out_off + vn) + (int64_t)(x - endj);
          }
        }
        push_step(p, cur, nxt, valid, u, e, L, next_parity, Rn, acc);
      }
    } else {
      const unsigned idx = (item - nchunks) * 32u + lane;
      WarpExpand &X = s_expand[wib];
      gather_expand(p, cur, nxt, idx < nlight ? q[idx] : -1, L, next_parity, Rn, acc, X.u, X.s,
                    X.x);
    }
    item = __shfl_sync(kFull, nextitem, 0);
  }
}

// Work items of a bitmap-wide round: (tile, slot) pairs; a tile holds 4096
// vertices (there are fewer tiles than warps below ~30M vertices) and its S
// slots split its set bits into S even ranges.  A heavy round (enough work for
// every warp) hands out about two items per warp, item i to warp i first and
// the rest from the round record's counter: its work crowds into the low
// tiles, where the unvisited vertices with in-edges are.  A light round takes
// S = warps / tiles and item i to warp i, with no counter for the grid's warps
// to queue on when they all finish at once.
__device__ __forceinline__ unsigned tile_slots(int64_t tiles, int nwarps, bool heavy) {
  const int64_t s = heavy ? (2 * (int64_t)nwarps + tiles - 1) / tiles : (int64_t)nwarps / tiles;
  return (unsigned)(s < 1 ? 1 : (s > 64 ? 64 : s));
}

__device__ __forceinline__ int64_t next_item(int64_t item, int nwarps, RoundRec *Rc, bool heavy) {
  if (!heavy) return item + nwarps;
  unsigned nextitem = 0;
  if (lane_id() == 0) nextitem = (unsigned)nwarps + atomicAdd(&Rc->work, 1u);
  return (int64_t)__shfl_sync(kFull, nextitem, 0);
}

// Push round right after a pull round: the frontier is only in the bitmap, so
// warps stage it a tile at a time (one 16-byte load per lane) and expand its
// set bits 32 at a time (lane i takes the i-th bit of its batch).
__device__ void push_round_bitmap(const BfsParams &p, const uint32_t *cur, uint32_t *nxt, int L,
                                  RoundRec *Rc, RoundRec *Rn, bool heavy, Acc &acc) {
  const int lane = lane_id();
  const int wib = threadIdx.x >> 5;
  const int nwarps = (gridDim.x * blockDim.x) >> 5;
  const int next_parity = (L + 1) & 1;
  WarpTile &T = s_tiles[wib];
  WarpExpand &X = s_expand[wib];
  const unsigned S = tile_slots(p.tiles, nwarps, heavy);
  const int64_t items = p.tiles * S;
  for (int64_t item = warp_id_global(); item < items; item = next_item(item, nwarps, Rc, heavy)) {
    const int64_t t = item % p.tiles;
    const unsigned slot = (unsigned)(item / p.tiles);
    const uint4 c = ld4(cur + t * kTileWords + 4 * lane);
    const unsigned total = stage_tile(c, T);
    const unsigned k1 = (unsigned)((unsigned long long)total * (slot + 1) / S);
    for (unsigned b = (unsigned)((unsigned long long)total * slot / S); b < k1; b += 32) {
      int32_t u = -1;
      if (b + lane < k1) {
        int j, bit;
        select_bit(T, b + lane, j, bit);
        u = (int32_t)((t * kTileWords + j) * 32 + bit);
      }
      gather_expand(p, cur, nxt, u, L, next_parity, Rn, acc, X.u, X.s, X.x);
    }
    __syncwarp();  // T is restaged by the next item
  }
}

// Bottom-up round: every unvisited vertex scans its ascending in-list and
// stops at the first source in F_L, which is its lowest-index parent.
// Work items are (tile, slot) pairs of 4096-vertex bitmap tiles: one 16-byte
// load per lane of each of vis, F_L and the map of vertices without in-edges
// gives the tile's unvisited set, staged in shared memory, and the slot takes
// an even range of it.  Each lane works on one vertex of the range at a time,
// kPullThreadScan entries of its list a step (all loads in flight before any
// test); a lane whose vertex is done (found, or its list exhausted) takes the
// range's next vertex at once, so lanes do not wait for the slowest list of a
// batch.  A list still unresolved after kPullLaneMax entries is finished by
// the whole warp, 32 entries a step.  Found vertices set their bit in the
// warp's shared copy of the tile's next-frontier words, ORed into F_{L+1} at
// the end of the item.  Slot 0 of each tile also merges F_L into vis (the
// union vis | F_L that other slots test is unchanged by it) and clears F_{L-1}
// (the next round's output bitmap), so pull rounds need no sweep.
__device__ void pull_round(const BfsParams &p, const uint32_t *cur, uint32_t *nxt, uint32_t *old,
                           int L, RoundRec *Rc, bool heavy, Acc &acc) {
  const int lane = lane_id();
  const unsigned lt_mask = (1u << lane) - 1u;
  const int wib = threadIdx.x >> 5;
  const int nwarps = (gridDim.x * blockDim.x) >> 5;
  WarpTile &T = s_tiles[wib];
  const unsigned S = tile_slots(p.tiles, nwarps, heavy);
  const int64_t items = p.tiles * S;
  for (int64_t item = warp_id_global(); item < items; item = next_item(item, nwarps, Rc, heavy)) {
    const int64_t t = item % p.tiles;
    const unsigned slot = (unsigned)(item / p.tiles);
    const int64_t w0 = t * kTileWords + 4 * lane;
    const uint4 vi = ld4(p.vis + w0);
    const uint4 cu = ld4(cur + w0);
    uint4 dd;
    if (p.dead) {
      dd = ldg4(p.dead + w0);
    } else {
      dd = make_uint4(~valid_bits(w0, p.n), ~valid_bits(w0 + 1, p.n), ~valid_bits(w0 + 2, p.n),
                      ~valid_bits(w0 + 3, p.n));
    }
    if (slot == 0) {
      if (any4(cu))
        st4(p.vis + w0, make_uint4(vi.x | cu.x, vi.y | cu.y, vi.z | cu.z, vi.w | cu.w));
      st4(old + w0, make_uint4(0u, 0u, 0u, 0u));
    }
    const uint4 un = make_uint4(~(vi.x | cu.x | dd.x), ~(vi.y | cu.y | dd.y),
                                ~(vi.z | cu.z | dd.z), ~(vi.w | cu.w | dd.w));
    st4(T.found + 4 * lane, make_uint4(0u, 0u, 0u, 0u));
    const unsigned total = stage_tile(un, T);
    const unsigned k1 = (unsigned)((unsigned long long)total * (slot + 1) / S);
    unsigned cursor = (unsigned)((unsigned long long)total * slot / S);
    // lane state: the vertex it works on (v, word j / bit of the tile), its
    // list [s, s + deg) and the next entry to scan
    bool has = false;
    int j = 0, bit = 0;
    int64_t s = 0;
    unsigned deg = 0, pos = 0;
    const int64_t v0 = t * kTileWords * 32;  // the tile's first vertex
    bool refill = true;  // some lane has no vertex (warp-uniform)
    while (true) {
      if (refill) {
        const unsigned need = __ballot_sync(kFull, !has);
        if (!has) {
          const unsigned k = cursor + __popc(need & lt_mask);
          if (k < k1) {
            has = true;
            select_bit(T, k, j, bit);
            const int64_t v = v0 + j * 32 + bit;
            s = __ldg(p.in_off + v);
            deg = (unsigned)(__ldg(p.in_off + v + 1) - s);
            pos = 0;
          }
        }
        cursor += __popc(need);
      }
      if (!__any_sync(kFull, has)) break;
      bool found = false;
      if (has && pos < kPullLaneMax) {
        int32_t u[kPullThreadScan];
#pragma unroll
        for (int k = 0; k < kPullThreadScan; ++k)
          u[k] = pos + k < deg ? __ldg(p.in_idx + s + pos + k) : -1;
        uint32_t hit = 0;
#pragma unroll
        for (int k = 0; k < kPullThreadScan; ++k)
          if (u[k] >= 0 && ((cur[(uint32_t)u[k] >> 5] >> (u[k] & 31)) & 1u)) hit |= 1u << k;
        if (hit) {
          const int k = __ffs(hit) - 1;  // ascending list: the lowest hit is the minimum
          int32_t uk = u[0];
#pragma unroll
          for (int q = 1; q < kPullThreadScan; ++q)
            if (q == k) uk = u[q];
          const int32_t ov = orig_id(p, v0 + j * 32 + bit);
          p.parents[ov] = orig_id(p, uk);
          p.levels[ov] = L + 1;
          found = true;
        }
        pos += kPullThreadScan;
      }
      // lists still open after kPullLaneMax entries: the whole warp scans the
      // rest, one vertex at a time
      unsigned rest = __ballot_sync(kFull, has && !found && pos >= kPullLaneMax && pos < deg);
      while (rest) {
        const int jl = __ffs(rest) - 1;
        rest &= rest - 1;
        const int64_t sj = __shfl_sync(kFull, s, jl);
        const unsigned pj = __shfl_sync(kFull, pos, jl);
        const unsigned dj = __shfl_sync(kFull, deg, jl);
        const int64_t vj = v0 + __shfl_sync(kFull, j * 32 + bit, jl);
        bool got = false;
        for (unsigned base = pj; base < dj; base += 32) {
          const unsigned i = base + lane;
          int32_t u = 0;
          bool hit = false;
          if (i < dj) {
            u = __ldg(p.in_idx + sj + i);
            hit = (cur[(uint32_t)u >> 5] >> (u & 31)) & 1u;
          }
          const unsigned who = __ballot_sync(kFull, hit);
          if (who) {
            if (lane == __ffs(who) - 1) {
              const int32_t ovj = orig_id(p, vj);
              p.parents[ovj] = orig_id(p, u);
              p.levels[ovj] = L + 1;
            }
            got = true;
            break;
          }
        }
        if (lane == jl) {
          found = got;
          pos = deg;  // scanned to the end (or found)
        }
      }
      if (found) {
        atomicOr(&T.found[j], 1u << bit);
        acc.nf += 1;
        acc.visdeg += deg;
      }
      const bool done = has && (found || pos >= deg);
      if (done) has = false;
      refill = __any_sync(kFull, done) && cursor < k1;
    }
    __syncwarp();
    const uint4 f = ld4(T.found + 4 * lane);
    if (f.x) atomicOr(nxt + w0, f.x);
    if (f.y) atomicOr(nxt + w0 + 1, f.y);
    if (f.z) atomicOr(nxt + w0 + 2, f.z);
    if (f.w) atomicOr(nxt + w0 + 3, f.w);
    __syncwarp();  // T is restaged by the next item
  }
}

__device__ __forceinline__ unsigned long long warp_sum(unsigned long long x) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(kFull, x, o);
  return x;
}

// Block totals of the per-thread counters (all threads call; thread 0 gets
// the sums) -- the one __syncthreads of a round's end before the wait.
__device__ void block_totals(Acc &acc, unsigned long long &a, unsigned long long &b,
                             unsigned long long &c) {
  __shared__ unsigned long long s_red[3][kBfsBlock / 32];
  const int lane = lane_id(), wib = threadIdx.x >> 5;
  a = warp_sum(acc.nf);
  b = warp_sum(acc.mf);
  c = warp_sum(acc.visdeg);
  if (lane == 0) {
    s_red[0][wib] = a;
    s_red[1][wib] = b;
    s_red[2][wib] = c;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    const int nw = blockDim.x >> 5;
    a = b = c = 0;
    for (int i = 0; i < nw; ++i) {
      a += s_red[0][i];
      b += s_red[1][i];
      c += s_red[2][i];
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
        // Beamer's rule, plus a floor: a pull round walks every vertex's
        // visited word, so a frontier whose edges are fewer than n / 8 stays
        // push (near the end "unexplored" counts only unreachable edges)
        const double unexplored = (double)p.nnz - (double)explored;
        return ((double)mf > unexplored / (double)p.alpha && (double)mf > (double)p.n / 8.0)
                   ? kPull
                   : kPush;
      }
      const bool shrinking = nf < prev_nf;
      return (shrinking && (double)nf < (double)p.n / (double)p.beta) ? kPush : kPull;
    }
  }
}

// Payload of a round's grid-wide barrier: the search ended; the next round
// pulls; the next round is heavy (enough work for every warp of the grid).
constexpr unsigned kDone = 1u, kNextPull = 2u, kHeavy = 4u;

// Flat grid-wide barrier of the per-root kernel, called by thread 0 of each
// block after a __syncthreads: one fire-and-forget release add on the launch's
// 64-bit arrival count, relaxed polls until the count reaches `target` (the
// b-th barrier of a launch waits for (b + 1) * gridDim.x arrivals; the count is
// zeroed before every launch), then one acquire fence, which makes every
// block's writes before its arrival visible.  Relaxed polls leave the SM's L1
// alone (an acquire load invalidates it while blocks of the same SM may still
// be working).  Bounded: after timeout_ns, or once another block has flagged
// an error, the thread records CG_ERR_TIMEOUT and returns false, so a barrier
// that cannot complete ends the kernel instead of spinning.
__device__ __forceinline__ bool flat_barrier(unsigned long long *count, unsigned long long target,
                                             int *status, long long timeout_ns) {
  asm volatile("red.release.gpu.global.add.u64 [%0], 1;" ::"l"(count) : "memory");
  long long t0 = 0;
  unsigned spins = 0;
  while (true) {
    unsigned long long c;
    asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];" : "=l"(c) : "l"(count) : "memory");
    if (c >= target) break;
    if ((++spins & 255u) == 0) {
      if (t0 == 0) t0 = global_ns();
      if (*(volatile int *)status != 0 || global_ns() - t0 > timeout_ns) {
        atomicCAS(status, 0, (int)CG_ERR_TIMEOUT);
        return false;
      }
    }
  }
  asm volatile("fence.acq_rel.gpu;" ::: "memory");
  return true;
}

// The search-wide bookkeeping of bool_pe.csl:947-1100 (visited total,
// explored edges, previous frontier size, pull rounds, direction switches).
// Every block keeps its own copy (thread 0) and updates it from the same round
// totals, so all blocks take the same decision without a second barrier.
struct SearchState {
  unsigned long long visited, prev_nf, explored;
  int pull_rounds, switches;
  long long t_mark;  // block 0: end of the previous round on the device clock
  unsigned long long next_big;  // the next frontier's queue sizes (record big, nlight)
  unsigned next_light;
};

// End of round L in warp 0 of every block, after the round's barrier: the
// termination test of bool_pe.csl:1048-1100 (nf == 0 ends the search) and the
// direction of round L + 1.  Lanes 0-23 each load one sharded counter of the
// round record (one L2 round trip), lane 0 takes the decision and block 0's
// lane 0 records the round's statistics.  All 32 lanes call; lane 0's return
// value is the payload.
__device__ unsigned round_decision(const BfsParams &p, int L, int dir, SearchState &ss) {
  BfsCtl *ctl = p.ctl;
  const RoundRec *Rn = &ctl->rec[(L + 1) % kRing];
  const int lane = lane_id();
  const int g = lane >> 3, sh = lane & (kCounterShards - 1);
  static_assert(kCounterShards == 8, "three groups of eight lanes");
  unsigned long long x = 0, q = 0;
  if (g == 0) x = __ldcg(&Rn->nf[sh]);
  else if (g == 1) x = __ldcg(&Rn->mf[sh]);
  else if (g == 2) x = __ldcg(&Rn->visdeg[sh]);
  // F_{L+1}'s queue sizes, for the next push round (same round trip)
  if (lane == 24) q = __ldcg(&Rn->big);
  else if (lane == 25) q = __ldcg(&Rn->nlight);
  const unsigned long long qbig = __shfl_sync(kFull, q, 24);
  const unsigned long long qlight = __shfl_sync(kFull, q, 25);
#pragma unroll
  for (int o = 1; o < kCounterShards; o <<= 1) x += __shfl_xor_sync(kFull, x, o);
  const unsigned long long nf = __shfl_sync(kFull, x, 0);
  const unsigned long long mf = __shfl_sync(kFull, x, 8);
  const unsigned long long vd = __shfl_sync(kFull, x, 16);
  if (lane != 0) return 0u;
  ss.next_big = qbig;
  ss.next_light = (unsigned)qlight;
  const bool block0 = blockIdx.x == 0;
  ss.pull_rounds += dir == kPull ? 1 : 0;
  ss.visited += nf;
  bool done = nf == 0;
  bool capped = false;
  if (!done && L + 1 >= p.level_cap) {
    capped = true;
    done = true;
  }
  const int next = next_direction(p, dir, nf, ss.prev_nf, mf, ss.explored);
  ss.explored += vd;
  ss.prev_nf = nf;
  ss.switches += (!done && next != dir) ? 1 : 0;
  if (block0) {
    cg_stats *st = p.stats;
    const long long now = global_ns();
    if (L < CG_HISTORY) {
      st->nf_history[L] = (int64_t)nf;
      st->direction_history[L] = dir;
      st->round_ns[L] = now - ss.t_mark;
    }
    ss.t_mark = now;
    if (capped) atomicCAS(&ctl->status, 0, (int)CG_ERR_LEVEL_CAP);
    if (done) {
      const int rounds = L + 1;
      const int stat = *(volatile int *)&ctl->status;
      st->status = stat != 0 ? stat : (capped ? (int)CG_ERR_LEVEL_CAP : 0);
      st->rounds = rounds;
      st->visited = (int64_t)ss.visited;
      st->pull_rounds = ss.pull_rounds;
      st->switches = ss.switches;
      st->history_len = rounds < CG_HISTORY ? rounds : CG_HISTORY;
      st->finish_ns = 0;
      st->device_ms = 0.f;
    }
  }
  // a pull round's work is the unvisited vertices with in-edges, a push
  // round's (from the bitmap) its frontier
  const unsigned long long work =
      next == kPull ? (p.live > (int64_t)ss.visited ? (unsigned long long)p.live - ss.visited : 0ull)
                    : nf;
  const bool heavy = work >= 32ull * (unsigned long long)((gridDim.x * blockDim.x) >> 5);
  return (done ? kDone : 0u) | (next == kPull ? kNextPull : 0u) | (heavy ? kHeavy : 0u);
}

// A host caller's outputs, copied by every block into the page-locked
// buffers (16 bytes a thread when n allows).  Kept out of line so the search
// loop's registers are not shared with it.
__device__ __noinline__ void copy_to_host(const BfsParams &p) {
  const int64_t t0 = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t step = (int64_t)gridDim.x * blockDim.x;
  for (int a = 0; a < 2; ++a) {
    const int32_t *src = a ? p.parents : p.levels;
    int32_t *dst = a ? p.host_parents : p.host_levels;
    if (!dst) continue;
    if ((p.n & 3) == 0) {
      const int4 *s4 = reinterpret_cast<const int4 *>(src);
      int4 *d4 = reinterpret_cast<int4 *>(dst);
      for (int64_t i = t0; i < (p.n >> 2); i += step) d4[i] = s4[i];
    } else {
      for (int64_t i = t0; i < p.n; i += step) dst[i] = src[i];
    }
  }
}

__global__ void __launch_bounds__(kBfsBlock, 3) bfs_persistent(BfsParams p) {
  __shared__ unsigned s_payload;
  BfsCtl *ctl = p.ctl;
  const int64_t gtid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t nthreads = (int64_t)gridDim.x * blockDim.x;
  // the root in original ids (output positions) and as a resident vertex
  const int32_t root_out = (int32_t)p.root;
  const int32_t root = p.perm ? __ldg(p.perm + p.root) : root_out;
  const bool leader = blockIdx.x == 0 && threadIdx.x == 0;

  // ---- phase 0: start_spmv -- reset outputs and bitmaps, seed the root ----
  __shared__ SearchState ss;  // thread 0's copy of the search-wide bookkeeping
  if (leader) ss.t_mark = global_ns();
  for (int64_t i = gtid; i < p.n; i += nthreads) {
    p.levels[i] = (i == root_out) ? 0 : -1;
    p.parents[i] = (i == root_out) ? root_out : -1;
  }
  // whole tiles (the padding past `words` too: a bitmap-wide round reads it)
  const uint4 zero4 = make_uint4(0u, 0u, 0u, 0u);
  const int64_t root_word = root >> 5;
  for (int64_t i = gtid; i < p.tiles * (kTileWords / 4); i += nthreads) {
    st4(p.vis + 4 * i, zero4);
    uint4 f0 = zero4;
    if (i == (root_word >> 2)) {  // F_0 = {root}, seeded by the thread that clears its word
      const uint32_t bit = 1u << (root & 31);
      const int c = (int)(root_word & 3);
      f0 = make_uint4(c == 0 ? bit : 0u, c == 1 ? bit : 0u, c == 2 ? bit : 0u, c == 3 ? bit : 0u);
    }
    st4(p.fr0 + 4 * i, f0);
    st4(p.fr1 + 4 * i, zero4);
    st4(p.fr2 + 4 * i, zero4);
  }
  if (leader) {
    const int64_t deg = p.out_off[root + 1] - p.out_off[root];
    RoundRec *R0 = &ctl->rec[0];
    R0->nf[0] = 1;
    R0->mf[0] = deg;
    R0->visdeg[0] = deg;
    if (deg <= kLightMax) {
      p.queue0[0] = root;
      R0->nlight = 1;
    } else {
      p.queue0[p.n - 1] = root;
      p.bigoff0[0] = 0;
      R0->big = (1ull << 32) | (unsigned long long)deg;
    }
  }
  // barrier b of this launch completes at (b + 1) * gridDim.x arrivals
  __shared__ unsigned long long s_target;
  __syncthreads();
  if (threadIdx.x == 0) {
    const unsigned long long target = gridDim.x;
    s_target = target;
    // the test hook expects one arrival more than the grid has: it must time out
    const bool ok0 = flat_barrier(&ctl->arrive, target + (p.unmatched_wait ? 1u : 0u),
                                  &ctl->status, p.timeout_ns);
    ss.visited = 1;
    ss.prev_nf = 1;
    ss.explored = (unsigned long long)(__ldg(p.out_off + root + 1) - __ldg(p.out_off + root));
    ss.pull_rounds = 0;
    ss.switches = 0;
    // F_0 = {root}: queued light or big by its degree (phase 0 above)
    ss.next_big = ss.explored > (unsigned long long)kLightMax ? ((1ull << 32) | ss.explored) : 0ull;
    ss.next_light = ss.explored > (unsigned long long)kLightMax ? 0u : 1u;
    if (blockIdx.x == 0 && ok0) {
      const long long now = global_ns();
      p.stats->setup_ns = now - ss.t_mark;
      ss.t_mark = now;
    }
    s_payload = ok0 ? 0u : kWaitFailed;
  }
  __syncthreads();
  bool ok = s_payload != kWaitFailed;

  uint32_t *fr0 = p.fr0, *fr1 = p.fr1, *fr2 = p.fr2;
  int dir = kPush;
  bool heavy = false;
  bool queued = true;  // F_L is in a queue (a pull round leaves it in the bitmap only)
  int L = 0;
  Acc acc;
  while (ok) {
    RoundRec *Rc = &ctl->rec[L % kRing];
    RoundRec *Rn = &ctl->rec[(L + 1) % kRing];
    const uint32_t *cur = fr0;  // F_L
    uint32_t *nxt = fr1;        // F_{L+1}
    uint32_t *old = fr2;        // F_{L-1}
    if (dir == kPush) {
      if (queued)
        push_round_queue(p, cur, nxt, L, Rc, Rn, ss.next_big, ss.next_light, acc);
      else
        push_round_bitmap(p, cur, nxt, L, Rc, Rn, heavy, acc);
      // vis |= F_L (readers test vis | F_L, so this races with nothing) and
      // clear F_{L-1}, which becomes the next round's output bitmap; a pull
      // round does both in its own tile pass
      for (int64_t i = gtid; i < p.tiles * (kTileWords / 4); i += nthreads) {
        const uint4 c = ld4(cur + 4 * i), vv = ld4(p.vis + 4 * i);
        if (any4(c))
          st4(p.vis + 4 * i, make_uint4(vv.x | c.x, vv.y | c.y, vv.z | c.z, vv.w | c.w));
        st4(old + 4 * i, zero4);
      }
    } else {
      pull_round(p, cur, nxt, old, L, Rc, heavy, acc);
    }
    unsigned long long a, b, c;
    block_totals(acc, a, b, c);
    if (threadIdx.x < 32) {
      bool arrived = false;
      if (threadIdx.x == 0) {
        const int sh = blockIdx.x % kCounterShards;
        if (a) atomicAdd(&Rn->nf[sh], a);
        if (b) atomicAdd(&Rn->mf[sh], b);
        if (c) atomicAdd(&Rn->visdeg[sh], c);
        if (blockIdx.x == 0) {
          // the record round L + 1 accumulates into next: its last readers were
          // done before the barrier of round L - 2 (ordered by this arrival)
          RoundRec *Rz = &ctl->rec[(L + 2) % kRing];
          for (int i = 0; i < kCounterShards; ++i) Rz->nf[i] = Rz->mf[i] = Rz->visdeg[i] = 0;
          Rz->big = 0;
          Rz->nlight = Rz->work = 0;
        }
        const unsigned long long target = s_target + gridDim.x;
        s_target = target;
        arrived = flat_barrier(&ctl->arrive, target, &ctl->status, p.timeout_ns);
      }
      // lane 0's acquire fence, then this warp barrier, order the other lanes'
      // counter loads after every block's arrival
      arrived = __shfl_sync(kFull, arrived, 0);
      const unsigned payload = arrived ? round_decision(p, L, dir, ss) : kWaitFailed;
      if (threadIdx.x == 0) s_payload = payload;
    }
    __syncthreads();
    const unsigned payload = s_payload;
    if (payload == kWaitFailed || (payload & kDone)) break;
    queued = dir == kPush;  // a push round queued F_{L+1}; a pull round did not
    dir = (payload & kNextPull) ? kPull : kPush;
    heavy = (payload & kHeavy) != 0;
    uint32_t *t = fr2;  // rotate: F_{L+1} becomes the frontier
    fr2 = fr0;
    fr0 = fr1;
    fr1 = t;
    ++L;
  }
  if (leader && s_payload == kWaitFailed) p.stats->status = *(volatile int *)&ctl->status;
  // after the last wait every output is final
  if (s_payload != kWaitFailed && (p.host_levels || p.host_parents)) copy_to_host(p);
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

int64_t bfs_big_capacity(int64_t n, int64_t nnz) {
  const int64_t c = nnz / (kLightMax + 1) + 1;
  return c < n ? c : n;
}

// Vertices with in-edges: n minus the dead bits below n.
__global__ void live_count_kernel(int64_t n, int64_t words, const uint32_t *__restrict__ dead,
                                  unsigned long long *live) {
  unsigned long long c = 0;
  for (int64_t w = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; w < words;
       w += (int64_t)gridDim.x * blockDim.x)
    c += (unsigned long long)__popc(~dead[w] & valid_bits(w, n));
  c = warp_sum(c);
  if (lane_id() == 0 && c) atomicAdd(live, c);
}

// Bit v of dead[v / 32]: vertex v has no in-edges, so no round reaches it
// (bits past n are set too, through the tile padding: `words` = stride).
__global__ void dead_map_kernel(int64_t n, int64_t words, const int64_t *__restrict__ in_off,
                                uint32_t *dead) {
  for (int64_t w = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; w < words;
       w += (int64_t)gridDim.x * blockDim.x) {
    uint32_t m = 0;
    int64_t prev = w * 32 < n ? in_off[w * 32] : 0;
    for (int b = 0; b < 32; ++b) {
      const int64_t v = w * 32 + b;
      if (v >= n) {
        m |= 1u << b;
        continue;
      }
      const int64_t next = in_off[v + 1];
      if (next == prev) m |= 1u << b;
      prev = next;
    }
    dead[w] = m;
  }
}

int refuse_setup_in_capture(cg_graph *g) {
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  CG_CUDA(cudaStreamIsCapturing(g->stream, &cs));
  if (cs == cudaStreamCaptureStatusNone) return CG_OK;
  set_error_text("a handle's first batched search sets up state: run it outside a capture");
  return CG_ERR_NOT_SUPPORTED;
}

// A handle's one-time per-root set-up runs on a private stream and is waited
// for, so it is done once and at once even when the first search is issued
// inside a capture of the handle's stream (which would only record it).  Work
// still queued on the handle's stream (the graph upload) is waited for first.
static int setup_stream(cg_graph *g, cudaStream_t *s) {
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  CG_CUDA(cudaStreamIsCapturing(g->stream, &cs));
  if (cs == cudaStreamCaptureStatusNone) CG_CUDA(cudaStreamSynchronize(g->stream));
  CG_CUDA(cudaStreamCreateWithFlags(s, cudaStreamNonBlocking));
  return CG_OK;
}

static int setup_wait(cudaStream_t s) {
  const cudaError_t e = cudaStreamSynchronize(s);
  cudaStreamDestroy(s);
  return e == cudaSuccess ? CG_OK : cuda_fail(e, "search state set-up");
}

int dead_prepare(cg_graph *g) {
  if (g->dead) return CG_OK;
  const int64_t words = bitmap_stride(g->n);
  uint32_t *dead = nullptr;
  unsigned long long *d_live = nullptr;  // the live count, read back once
  if (cudaMalloc(&dead, sizeof(uint32_t) * (size_t)words) != cudaSuccess ||
      cudaMalloc(&d_live, sizeof(unsigned long long)) != cudaSuccess) {
    cudaFree(dead);
    return CG_ERR_OUT_OF_MEMORY;
  }
  unsigned long long live = 0;
  cudaStream_t s = nullptr;
  int rc = setup_stream(g, &s);
  if (!rc) {
    const int64_t blocks = (words + 255) / 256;
    const unsigned grid = (unsigned)(blocks < 4096 ? blocks : 4096);
    cudaError_t e = cudaMemsetAsync(d_live, 0, sizeof(unsigned long long), s);
    dead_map_kernel<<<grid, 256, 0, s>>>(g->n, words, g->in_off, dead);
    live_count_kernel<<<grid, 256, 0, s>>>(g->n, words, dead, d_live);
    if (e == cudaSuccess) e = cudaGetLastError();
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(&live, d_live, sizeof(live), cudaMemcpyDeviceToHost, s);
    rc = setup_wait(s);
    if (!rc && e != cudaSuccess) rc = cuda_fail(e, "dead-vertex map");
  }
  cudaFree(d_live);
  if (rc) {
    cudaFree(dead);
    return rc;
  }
  g->dead = dead;
  g->live = (int64_t)live;
  g->device_bytes += sizeof(uint32_t) * words;
  return CG_OK;
}

int bfs_prepare(cg_graph *g) {
  if (g->d_stats) return CG_OK;  // the last of the buffers below: all are in place
  int rc = dead_prepare(g);
  if (rc) return rc;
  int dev_coop = 0;
  CG_CUDA(cudaDeviceGetAttribute(&dev_coop, cudaDevAttrCooperativeLaunch, g->device));
  if (!dev_coop) return CG_ERR_NOT_SUPPORTED;
  const int64_t words = (g->n + 31) / 32;
  const int64_t bcap = bfs_big_capacity(g->n, g->nnz);
  const size_t bytes_bm = sizeof(uint32_t) * 4 * (size_t)bitmap_stride(g->n);
  const size_t bytes_q = sizeof(int32_t) * 2 * (size_t)g->n;
  const size_t bytes_b = sizeof(uint32_t) * 2 * (size_t)bcap;
  uint32_t *bitmaps = nullptr, *bigoff = nullptr;
  int32_t *queue = nullptr;
  BfsCtl *ctl = nullptr;
  cg_stats *stats = nullptr;
  if (cudaMalloc(&bitmaps, bytes_bm) != cudaSuccess || cudaMalloc(&queue, bytes_q) != cudaSuccess ||
      cudaMalloc(&bigoff, bytes_b) != cudaSuccess || cudaMalloc(&ctl, sizeof(BfsCtl)) != cudaSuccess ||
      cudaMalloc(&stats, sizeof(cg_stats)) != cudaSuccess) {
    cudaFree(bitmaps);
    cudaFree(queue);
    cudaFree(bigoff);
    cudaFree(ctl);
    cudaFree(stats);
    return CG_ERR_OUT_OF_MEMORY;
  }
  cudaStream_t s = nullptr;
  rc = setup_stream(g, &s);
  cudaError_t e = cudaSuccess;
  if (!rc) {
    e = cudaMemsetAsync(ctl, 0, sizeof(BfsCtl), s);
    if (e == cudaSuccess) e = cudaMemsetAsync(stats, 0, sizeof(cg_stats), s);
    rc = setup_wait(s);
    if (!rc && e != cudaSuccess) rc = cuda_fail(e, "search state reset");
  }
  if (rc) {
    cudaFree(bitmaps);
    cudaFree(queue);
    cudaFree(bigoff);
    cudaFree(ctl);
    cudaFree(stats);
    return rc;
  }
  g->words = words;
  g->bcap = bcap;
  g->bitmaps = bitmaps;
  g->queue = queue;
  g->bigoff = bigoff;
  g->ctl = ctl;
  g->d_stats = stats;
  g->device_bytes += bytes_bm + bytes_q + bytes_b + sizeof(BfsCtl) + sizeof(cg_stats);
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

int bfs_launch(cg_graph *g, int64_t root, int32_t *d_levels, int32_t *d_parents,
               int32_t *host_levels, int32_t *host_parents) {
  int rc = bfs_prepare(g);
  if (rc) return rc;
  if ((rc = bfs_grid(g))) return rc;
  BfsParams p;
  p.n = g->n;
  p.nnz = g->nnz;
  p.words = g->words;
  const int64_t stride = bitmap_stride(g->n);
  p.tiles = stride / kTileWords;
  p.in_off = g->in_off;
  p.in_idx = g->in_idx;
  p.out_off = g->out_off;
  p.out_idx = g->out_idx;
  p.vis = g->bitmaps;
  p.fr0 = g->bitmaps + stride;
  p.fr1 = g->bitmaps + 2 * stride;
  p.fr2 = g->bitmaps + 3 * stride;
  p.dead = g->dead;
  p.live = g->live;
  p.orig = g->orig;
  p.perm = g->perm;
  p.queue0 = g->queue;
  p.queue1 = g->queue + g->n;
  p.bigoff0 = g->bigoff;
  p.bigoff1 = g->bigoff + g->bcap;
  p.levels = d_levels;
  p.parents = d_parents;
  p.host_levels = host_levels;
  p.host_parents = host_parents;
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
