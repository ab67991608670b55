// FIFO parents: the parent rule of scipy's breadth_first_order, the host BFS
// the reference's driver checks its searches against (run_graph500.py:383-395,
// run_bfs.py:517-527).  That search pops its queue in order and gives every
// out-neighbour it has not seen yet (in ascending id order) the popped vertex
// as predecessor.  So the parent of a vertex at level L+1 is its level-L
// in-neighbour of smallest queue rank, and level L+1 is queued in order of
// (rank of the parent, vertex id).
//
// Given the levels of a finished search, this pass recomputes the parents
// level by level: one warp per level-(L+1) vertex takes the minimum of
// (rank, id) over its level-L in-neighbours; a radix sort of the resulting
// (parent rank, vertex id) keys is the queue order of level L+1, i.e. the
// next level's ranks.  The level sizes steer the sorts from the host, so the
// pass synchronises with the stream (and is refused inside a graph capture).
#include <cuda_runtime.h>
#include <stdint.h>

#include <vector>

#include <cub/block/block_scan.cuh>
#include <cub/device/device_radix_sort.cuh>

#include "cg_internal.cuh"

namespace cg {

struct FifoState {
  int64_t n = 0;
  int32_t *rank = nullptr;              // [n] queue rank within the vertex's level
  // [n] (level << 32) | rank and (level << 32) | FIFO parent of the vertices
  // ranked so far in this pass (-1 elsewhere): one load tells a list entry's
  // level and rank, or whether an out-neighbour is a given parent's child
  unsigned long long *lr = nullptr, *pl = nullptr;
  int32_t *order = nullptr;             // [n] vertices of levels >= 1, grouped by level
  unsigned long long *keys = nullptr;   // [n] (parent rank, vertex) of one level
  unsigned long long *sorted = nullptr; // [n]
  unsigned *counts = nullptr;           // [n + 1] vertices per level
  unsigned *cursor = nullptr;           // [n + 1] scatter cursors
  unsigned *offs = nullptr;             // [n + 1] first slot of each level in order
  int *maxlevel = nullptr;
  void *temp = nullptr;                 // radix sort scratch
  size_t temp_bytes = 0;
};

namespace {

constexpr int kFifoBlock = 256;
constexpr int kFifoSmemLevels = 64;

// Vertices per level (levels >= 0) and the deepest level.
__global__ void fifo_hist_kernel(int64_t n, const int32_t *__restrict__ levels, unsigned *counts,
                                 int *maxlevel) {
  __shared__ unsigned s[kFifoSmemLevels];
  for (int i = threadIdx.x; i < kFifoSmemLevels; i += blockDim.x) s[i] = 0;
  __syncthreads();
  int mx = -1;
  for (int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; v < n;
       v += (int64_t)gridDim.x * blockDim.x) {
    const int L = levels[v];
    if (L < 0) continue;
    mx = L > mx ? L : mx;
    if (L < kFifoSmemLevels)
      atomicAdd(&s[L], 1u);
    else
      atomicAdd(&counts[L], 1u);
  }
  mx = __reduce_max_sync(0xffffffffu, mx);
  if ((threadIdx.x & 31) == 0 && mx >= 0) atomicMax(maxlevel, mx);
  __syncthreads();
  for (int i = threadIdx.x; i < kFifoSmemLevels; i += blockDim.x)
    if (s[i]) atomicAdd(&counts[i], s[i]);
}

// order[offs[L] ..] = the vertices of level L >= 1 (in no particular order;
// each level is sorted later).  One atomic per level present in a warp.
__global__ void fifo_scatter_kernel(int64_t n, const int32_t *__restrict__ levels,
                                    const unsigned *__restrict__ offs, unsigned *cursor,
                                    int32_t *order) {
  const int lane = threadIdx.x & 31;
  for (int64_t base = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) & ~31ll; base < n;
       base += (int64_t)gridDim.x * blockDim.x) {
    const int64_t v = base + lane;
    const int L = v < n ? levels[v] : -1;
    const unsigned peers = __match_any_sync(0xffffffffu, L);
    if (L >= 1) {
      const int leader = __ffs(peers) - 1;
      unsigned at = 0;
      if (lane == leader) at = atomicAdd(&cursor[L], (unsigned)__popc(peers));
      at = __shfl_sync(peers, at, leader);
      order[offs[L] + at + __popc(peers & ((1u << lane) - 1u))] = (int32_t)v;
    }
  }
}

// One warp per vertex v of level L+1 (order[0 .. count)): its level-L
// in-neighbour of smallest rank is its parent (ranks are unique within a
// level); keys[i] = (that rank << vbits) | v, the sort key of level L+1's
// queue order (v < 2^vbits).
__global__ void fifo_pick_kernel(const int64_t *__restrict__ in_off,
                                 const int32_t *__restrict__ in_idx,
                                 const int32_t *__restrict__ levels,
                                 const int32_t *__restrict__ rank,
                                 const int32_t *__restrict__ order, unsigned count, int L,
                                 int vbits, unsigned long long *keys, int32_t *parents) {
  const int lane = threadIdx.x & 31;
  const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t i = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; i < count;
       i += nwarps) {
    const int32_t v = order[i];
    const int64_t s = __ldg(in_off + v), e = __ldg(in_off + v + 1);
    unsigned long long best = ~0ull;
    for (int64_t j = s + lane; j < e; j += 32) {
      const int32_t u = __ldg(in_idx + j);
      if (levels[u] == L) {
        const unsigned long long k = ((unsigned long long)(uint32_t)rank[u] << 32) | (uint32_t)u;
        best = k < best ? k : best;
      }
    }
#pragma unroll
    for (int d = 16; d > 0; d >>= 1) {
      const unsigned long long o = __shfl_xor_sync(0xffffffffu, best, d);
      best = o < best ? o : best;
    }
    if (lane == 0) {
      parents[v] = best == ~0ull ? -1 : (int32_t)(uint32_t)best;
      keys[i] = ((best >> 32) << vbits) | (uint32_t)v;
    }
  }
}

__global__ void fifo_rank_kernel(const unsigned long long *__restrict__ sorted, unsigned count,
                                 int vbits, int level, int32_t *rank, unsigned long long *lr) {
  const unsigned long long vmask = (1ull << vbits) - 1ull;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < count;
       i += (int64_t)gridDim.x * blockDim.x) {
    const unsigned long long v = sorted[i] & vmask;
    rank[v] = (int32_t)i;
    lr[v] = ((unsigned long long)level << 32) | (unsigned long long)i;
  }
}

// Levels of at most kSmallLevel vertices are handled by one block, many
// levels to a launch, with no sort: level L+1's queue is level L's queue in
// order with each vertex's children (the out-neighbours whose FIFO parent it
// is) appended in out-list order, which is ascending -- the same order the
// sort of (parent rank, id) gives.  Per level: (1) every child picks its
// parent, the level-L in-neighbour of smallest rank (one 8-byte load of
// (level, rank) per in-list entry), records (level + 1, parent) for the
// parent's scan and counts itself in its parent's shared-memory counter;
// (2) a block scan of the counts in rank order gives each parent its first
// child's rank; (3) every parent with children walks its out-list handing
// out ranks to the entries recorded as its children.  Long lists go to a
// warp.  One SM's load pipeline bounds this, so each list entry costs one
// load.  On deep graphs launches would otherwise dominate (a 4096 x 4096 grid
// has ~8000 levels).
constexpr int kSmallThreads = 1024;
constexpr int kSmallPer = 8;                                // counts a thread scans
constexpr int kSmallLevel = kSmallThreads * kSmallPer;     // vertices per level, at most
constexpr int kHeavyList = 64;  // list length above which a warp scans
using SmallScan = cub::BlockScan<unsigned, kSmallThreads>;
struct SmallSmem {
  int32_t queue[2][kSmallLevel];     // levels L and L+1 in queue (rank) order
  unsigned cnt[kSmallLevel + 1];     // children per parent rank, then first ranks
  int32_t heavy[kSmallLevel];        // positions whose lists a warp scans
  unsigned nheavy;
  typename SmallScan::TempStorage scan;
};

__device__ __forceinline__ unsigned long long warp_min64(unsigned long long x) {
#pragma unroll
  for (int d = 16; d > 0; d >>= 1) {
    const unsigned long long o = __shfl_xor_sync(0xffffffffu, x, d);
    x = o < x ? o : x;
  }
  return x;
}

// Over in-list entries [s, e) (lanes lane, lane + step, ...), the smallest
// (rank << 32) | u of a level-L in-neighbour u; lr is written by this block at
// earlier levels, so it is read with ordinary loads, never the read-only path.
__device__ __forceinline__ unsigned long long fifo_best(const int32_t *__restrict__ in_idx,
                                                        const unsigned long long *lr, int64_t s,
                                                        int64_t e, int L, int lane, int step) {
  unsigned long long best = ~0ull;
  for (int64_t j = s + lane; j < e; j += step) {
    const int32_t u = __ldg(in_idx + j);
    const unsigned long long x = lr[u];
    if ((unsigned)(x >> 32) == (unsigned)L) {
      const unsigned long long k = ((x & 0xffffffffull) << 32) | (uint32_t)u;
      best = k < best ? k : best;
    }
  }
  return best;
}

// Level L+1 vertex w takes parent u (rank r among level L).
__device__ __forceinline__ void fifo_adopt(int32_t w, unsigned long long best, int L,
                                           int32_t *parents, unsigned long long *pl,
                                           unsigned *cnt) {
  if (best == ~0ull) return;  // no level-L in-neighbour: not a level-(L+1) vertex
  const int32_t u = (int32_t)(uint32_t)best;
  parents[w] = u;
  pl[w] = ((unsigned long long)(L + 1) << 32) | (uint32_t)u;
  atomicAdd(&cnt[best >> 32], 1u);
}

// One block: levels L0 .. L1-1 in turn; for each, level L has counts[L] and
// level L+1 counts[L+1] vertices, both at most kSmallLevel; order[offs[L+1] ..]
// lists level L+1 in no particular order.
__global__ void __launch_bounds__(kSmallThreads) fifo_small_levels_kernel(
    const int64_t *__restrict__ in_off, const int32_t *__restrict__ in_idx,
    const int64_t *__restrict__ out_off, const int32_t *__restrict__ out_idx, int32_t *rank,
    unsigned long long *lr, unsigned long long *pl, const int32_t *__restrict__ order,
    const unsigned *__restrict__ counts, const unsigned *__restrict__ offs, int L0, int L1,
    int32_t root, int32_t *parents) {
  extern __shared__ __align__(16) unsigned char s_raw[];
  SmallSmem &S = *reinterpret_cast<SmallSmem *>(s_raw);
  const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
  constexpr int kWarps = kSmallThreads / 32;
  int cur = 0;
  // level L0 in queue order, from the ranks already assigned (level 0 is the
  // root alone; order[] lists levels >= 1)
  if (L0 == 0) {
    if (t == 0) S.queue[0][0] = root;
  } else {
    for (unsigned i = t; i < counts[L0]; i += kSmallThreads) {
      const int32_t u = order[offs[L0] + i];
      S.queue[0][rank[u]] = u;
    }
  }
  for (int L = L0; L < L1; ++L) {
    const unsigned c = counts[L + 1], p = counts[L];
    const unsigned base = offs[L + 1];
    int32_t *qL = S.queue[cur];
    int32_t *qN = S.queue[cur ^ 1];
    for (unsigned r = t; r < p; r += kSmallThreads) S.cnt[r] = 0;
    if (t == 0) S.nheavy = 0;
    __syncthreads();
    // (1) parents of level L+1
    for (unsigned pos = t; pos < c; pos += kSmallThreads) {
      const int32_t w = order[base + pos];
      const int64_t s = __ldg(in_off + w), e = __ldg(in_off + w + 1);
      if (e - s > kHeavyList)
        S.heavy[atomicAdd(&S.nheavy, 1u)] = w;
      else
        fifo_adopt(w, fifo_best(in_idx, lr, s, e, L, 0, 1), L, parents, pl, S.cnt);
    }
    __syncthreads();
    for (unsigned h = warp; h < S.nheavy; h += kWarps) {
      const int32_t w = S.heavy[h];
      const unsigned long long best =
          warp_min64(fifo_best(in_idx, lr, __ldg(in_off + w), __ldg(in_off + w + 1), L, lane, 32));
      if (lane == 0) fifo_adopt(w, best, L, parents, pl, S.cnt);
    }
    __syncthreads();  // every warp is done with the list before it is reset
    // (2) first rank of each parent's children: exclusive scan in rank order
    {
      unsigned v[kSmallPer], sum = 0;
#pragma unroll
      for (int i = 0; i < kSmallPer; ++i) {
        const unsigned r = t * kSmallPer + i;
        v[i] = r < p ? S.cnt[r] : 0u;
        sum += v[i];
      }
      unsigned before = 0;
      SmallScan(S.scan).ExclusiveSum(sum, before);
      __syncthreads();
#pragma unroll
      for (int i = 0; i < kSmallPer; ++i) {
        const unsigned r = t * kSmallPer + i;
        if (r < p) S.cnt[r] = before;
        before += v[i];
      }
      if (t == 0) {
        S.cnt[p] = c;
        S.nheavy = 0;
      }
    }
    __syncthreads();
    // (3) ranks of level L+1: parents with children walk their out-lists
    const unsigned long long tag = (unsigned long long)(L + 1) << 32;
    for (unsigned r = t; r < p; r += kSmallThreads) {
      unsigned at = S.cnt[r];
      const unsigned end = S.cnt[r + 1];
      if (at == end) continue;
      const int32_t u = qL[r];
      const int64_t s = __ldg(out_off + u), e = __ldg(out_off + u + 1);
      if (e - s > kHeavyList) {
        S.heavy[atomicAdd(&S.nheavy, 1u)] = (int32_t)r;
        continue;
      }
      const unsigned long long mine = tag | (uint32_t)u;
      for (int64_t j = s; j < e && at < end; ++j) {
        const int32_t w = __ldg(out_idx + j);
        if (pl[w] == mine) {
          rank[w] = (int32_t)at;
          lr[w] = tag | at;
          qN[at++] = w;
        }
      }
    }
    __syncthreads();
    for (unsigned h = warp; h < S.nheavy; h += kWarps) {
      const unsigned r = (unsigned)S.heavy[h];
      const int32_t u = qL[r];
      const unsigned long long mine = tag | (uint32_t)u;
      const int64_t s = __ldg(out_off + u), e = __ldg(out_off + u + 1);
      unsigned at = S.cnt[r];
      for (int64_t j0 = s; j0 < e; j0 += 32) {
        const int64_t j = j0 + lane;
        int32_t w = 0;
        bool child = false;
        if (j < e) {
          w = __ldg(out_idx + j);
          child = pl[w] == mine;
        }
        const unsigned m = __ballot_sync(0xffffffffu, child);
        if (child) {
          const unsigned k = at + __popc(m & ((1u << lane) - 1u));
          rank[w] = (int32_t)k;
          lr[w] = tag | k;
          qN[k] = w;
        }
        at += __popc(m);
      }
    }
    __syncthreads();
    cur ^= 1;
  }
}

// Bits needed for the values 0 .. x (at least 1).
int bits_for(uint64_t x) {
  int b = 1;
  while (b < 64 && (x >> b)) ++b;
  return b;
}

unsigned grid_for(int64_t items, int per_block, int sms) {
  int64_t b = (items + per_block - 1) / per_block;
  const int64_t cap = (int64_t)sms * 16;
  if (b > cap) b = cap;
  return (unsigned)(b > 0 ? b : 1);
}

int fifo_state(cg_graph *g, FifoState **out) {
  if (g->fifo) {
    *out = g->fifo;
    return CG_OK;
  }
  FifoState *f = new FifoState();
  f->n = g->n;
  const size_t n = (size_t)g->n;
  bool ok = cudaMalloc(&f->rank, sizeof(int32_t) * n) == cudaSuccess &&
            cudaMalloc(&f->lr, sizeof(unsigned long long) * n) == cudaSuccess &&
            cudaMalloc(&f->pl, sizeof(unsigned long long) * n) == cudaSuccess &&
            cudaMalloc(&f->order, sizeof(int32_t) * n) == cudaSuccess &&
            cudaMalloc(&f->keys, sizeof(unsigned long long) * n) == cudaSuccess &&
            cudaMalloc(&f->sorted, sizeof(unsigned long long) * n) == cudaSuccess &&
            cudaMalloc(&f->counts, sizeof(unsigned) * (n + 1)) == cudaSuccess &&
            cudaMalloc(&f->cursor, sizeof(unsigned) * (n + 1)) == cudaSuccess &&
            cudaMalloc(&f->offs, sizeof(unsigned) * (n + 1)) == cudaSuccess &&
            cudaMalloc(&f->maxlevel, sizeof(int)) == cudaSuccess;
  if (ok)
    ok = cudaFuncSetAttribute(fifo_small_levels_kernel,
                              cudaFuncAttributeMaxDynamicSharedMemorySize,
                              (int)sizeof(SmallSmem)) == cudaSuccess;
  if (ok) {
    cub::DeviceRadixSort::SortKeys(nullptr, f->temp_bytes, f->keys, f->sorted, (int)n, 0, 64,
                                   g->stream);
    ok = cudaMalloc(&f->temp, f->temp_bytes ? f->temp_bytes : 16) == cudaSuccess;
  }
  if (!ok) {
    fifo_free(f);
    return CG_ERR_OUT_OF_MEMORY;
  }
  g->device_bytes += (int64_t)((sizeof(int32_t) * 2 + sizeof(unsigned long long) * 4) * n +
                               sizeof(unsigned) * 3 * (n + 1) + f->temp_bytes);
  g->fifo = f;
  *out = f;
  return CG_OK;
}

}  // namespace

void fifo_free(FifoState *f) {
  if (!f) return;
  cudaFree(f->rank);
  cudaFree(f->lr);
  cudaFree(f->pl);
  cudaFree(f->order);
  cudaFree(f->keys);
  cudaFree(f->sorted);
  cudaFree(f->counts);
  cudaFree(f->cursor);
  cudaFree(f->offs);
  cudaFree(f->maxlevel);
  cudaFree(f->temp);
  delete f;
}

int fifo_parents(cg_graph *g, int64_t root, const int32_t *d_levels, int32_t *d_parents) {
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  CG_CUDA(cudaStreamIsCapturing(g->stream, &cs));
  if (cs != cudaStreamCaptureStatusNone) {
    set_error_text("the FIFO parent rule synchronises with the stream: not capturable");
    return CG_ERR_NOT_SUPPORTED;
  }
  FifoState *f = nullptr;
  int rc = fifo_state(g, &f);
  if (rc) return rc;
  const int64_t n = g->n;
  cudaStream_t st = g->stream;
  CG_CUDA(cudaMemsetAsync(f->counts, 0, sizeof(unsigned) * (size_t)(n + 1), st));
  CG_CUDA(cudaMemsetAsync(f->maxlevel, 0xff, sizeof(int), st));
  fifo_hist_kernel<<<grid_for(n, kFifoBlock, g->num_sms), kFifoBlock, 0, st>>>(n, d_levels,
                                                                               f->counts,
                                                                               f->maxlevel);
  CG_CUDA(cudaGetLastError());
  int maxlevel = -1;
  CG_CUDA(cudaMemcpyAsync(&maxlevel, f->maxlevel, sizeof(int), cudaMemcpyDeviceToHost, st));
  CG_CUDA(cudaStreamSynchronize(st));
  if (maxlevel <= 0) return CG_OK;  // only the root: its parent is itself already
  std::vector<unsigned> counts((size_t)maxlevel + 1), offs((size_t)maxlevel + 2, 0u);
  CG_CUDA(cudaMemcpyAsync(counts.data(), f->counts, sizeof(unsigned) * counts.size(),
                          cudaMemcpyDeviceToHost, st));
  CG_CUDA(cudaStreamSynchronize(st));
  for (int L = 1; L <= maxlevel; ++L) offs[L + 1] = offs[L] + counts[L];
  CG_CUDA(cudaMemcpyAsync(f->offs, offs.data(), sizeof(unsigned) * offs.size(),
                          cudaMemcpyHostToDevice, st));
  CG_CUDA(cudaMemsetAsync(f->cursor, 0, sizeof(unsigned) * (size_t)(maxlevel + 1), st));
  fifo_scatter_kernel<<<grid_for(n, kFifoBlock, g->num_sms), kFifoBlock, 0, st>>>(
      n, d_levels, f->offs, f->cursor, f->order);
  CG_CUDA(cudaMemsetAsync(f->rank + root, 0, sizeof(int32_t), st));
  CG_CUDA(cudaMemsetAsync(f->lr, 0xff, sizeof(unsigned long long) * (size_t)n, st));
  CG_CUDA(cudaMemsetAsync(f->pl, 0xff, sizeof(unsigned long long) * (size_t)n, st));
  CG_CUDA(cudaMemsetAsync(f->lr + root, 0, sizeof(unsigned long long), st));  // level 0, rank 0
  // keys (parent rank << vbits) | v: only the bits in use are sorted
  const int vbits = bits_for((uint64_t)(n - 1));
  for (int L = 0; L < maxlevel; ++L) {
    const unsigned c = counts[(size_t)L + 1];
    if (c == 0) break;
    if (c <= (unsigned)kSmallLevel && counts[(size_t)L] <= (unsigned)kSmallLevel) {
      // a run of small levels: one launch of one block
      int L1 = L + 1;
      while (L1 < maxlevel && counts[(size_t)L1 + 1] > 0 &&
             counts[(size_t)L1 + 1] <= (unsigned)kSmallLevel &&
             counts[(size_t)L1] <= (unsigned)kSmallLevel)
        ++L1;
      fifo_small_levels_kernel<<<1, kSmallThreads, sizeof(SmallSmem), st>>>(
          g->in_off, g->in_idx, g->out_off, g->out_idx, f->rank, f->lr, f->pl, f->order,
          f->counts, f->offs, L, L1, (int32_t)root, d_parents);
      CG_CUDA(cudaGetLastError());
      L = L1 - 1;
      continue;
    }
    const unsigned parents_c = counts[(size_t)L];  // ranks of level L: 0 .. parents_c - 1
    const int end_bit = vbits + bits_for(parents_c ? parents_c - 1 : 0);
    fifo_pick_kernel<<<grid_for((int64_t)c * 32, kFifoBlock, g->num_sms), kFifoBlock, 0, st>>>(
        g->in_off, g->in_idx, d_levels, f->rank, f->order + offs[(size_t)L + 1], c, L, vbits,
        f->keys, d_parents);
    size_t tb = f->temp_bytes;
    CG_CUDA(cub::DeviceRadixSort::SortKeys(f->temp, tb, f->keys, f->sorted, (int)c, 0,
                                           end_bit, st));
    fifo_rank_kernel<<<grid_for(c, kFifoBlock, g->num_sms), kFifoBlock, 0, st>>>(
        f->sorted, c, vbits, L + 1, f->rank, f->lr);
  }
  CG_CUDA(cudaGetLastError());
  return CG_OK;
}

}  // namespace cg
