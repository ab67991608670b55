// Internal definitions shared by the engine's translation units.
//
// Layout in HBM of one resident graph (cg_graph):
//   in_off  int64[n+1], in_idx  int32[nnz]   CSR of A (row r = sources of edges c -> r)
//   out_off int64[n+1], out_idx int32[nnz]   CSC of A (column c = targets of c);
//                                             aliases of in_* when A is symmetric
// Per-root search state (allocated once per handle, reused by every search):
//   vis, fr[3]     uint32[stride] packed bitmaps: visited-before-the-frontier and three
//                                 rotating frontier bitmaps (round L reads fr[L%3] = F_L,
//                                 writes fr[(L+1)%3] and clears fr[(L+2)%3]); a vertex
//                                 counts as visited when its bit is in vis | F_L.  These
//                                 are the reference's visited_bitmap / x_bitmap / y_bitmap
//                                 (bool_pe.csl) over all n vertices instead of per PE.
//                                 stride = words rounded up to whole tiles of kTileWords
//                                 (16-byte vector loads; the padding stays zero)
//   queue[2]       int32[n]       push-round frontier queues: light vertices (out-degree
//                                 <= kLightMax) from the front, big ones from the back
//   bigoff[2]      uint32[bcap]   prefix offsets of the big vertices' edge lists, in
//                                 queue order (edge-balanced chunking)
//   ctl            BfsCtl         per-round records, grid-wait counter, status
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/ceregraphs.h"

namespace cg {

// Grid-wide wait state: blocks arrive on one of kWaitGroups group counters
// (blockIdx % kWaitGroups), the last of each group on the top counter, the
// last group releases the sync word: generation in the low 32 bits and a
// 32-bit payload (the decision the last arrival took for everyone) in the
// high bits.  Each counter has its own 128-byte line so arrivals of
// different groups do not serialise.
constexpr int kWaitGroups = 16;
struct GridWaitGroup {
  unsigned int count;
  unsigned int pad[31];
};
struct GridWait {
  unsigned int top;
  unsigned int pad0;
  unsigned long long sync;
  unsigned int pad[28];
  GridWaitGroup group[kWaitGroups];
};

// Round counters are sharded over kCounterShards addresses (blockIdx % shards)
// so that block flushes do not all land on one address.
constexpr int kCounterShards = 8;

// Degree classes of a push-round frontier vertex.
constexpr int kLightMax = 64;     // <= this: 32 vertices share one warp (edge-balanced)
constexpr int kMediumMax = 4096;  // multi-source push: <= this one warp, above: whole grid
constexpr int kPushChunk = 1024;  // edges of big frontier vertices per work item

constexpr int kRing = 4;          // per-round record ring (rounds L .. L+3)

// Bitmap words a warp stages per tile of a bitmap-wide round (4 per lane, one
// 16-byte load each): 4096 vertices.  Bitmaps are allocated in whole tiles.
constexpr int kTileWords = 128;
__host__ __device__ constexpr int64_t bitmap_stride(int64_t n) {
  return ((n + 31) / 32 + kTileWords - 1) / kTileWords * kTileWords;
}

// Statistics of frontier F_k (the vertices at level k) and the queue holding it.
struct RoundRec {
  unsigned long long nf[kCounterShards];      // |F_k|
  unsigned long long mf[kCounterShards];      // sum of out-degrees over F_k
  unsigned long long visdeg[kCounterShards];  // sum of degrees over F_k (unexplored edges)
  unsigned long long big;      // (count << 32) | total edges of the big vertices of F_k
  unsigned int nlight;         // light vertices, queue front
  unsigned int work;           // dynamic work counter used while F_k is expanded
  unsigned long long pad[6];
};

// Control block of one per-root search, zeroed before every launch.  The
// search-wide bookkeeping (visited total, explored edges, ...) is not here:
// every block keeps its own copy, updated from the same round totals.
struct BfsCtl {
  unsigned long long arrive;   // flat grid barrier: arrivals so far in this launch
  unsigned long long pad0[15];
  int status;                  // first error (CG_ERR_TIMEOUT, CG_ERR_LEVEL_CAP), else 0
  int pad1[31];
  RoundRec rec[kRing];
};

struct BfsParams {
  int64_t n, nnz, words;
  int64_t tiles;         // bitmap tiles: stride / kTileWords
  const int64_t *__restrict__ in_off;
  const int32_t *__restrict__ in_idx;
  const int64_t *__restrict__ out_off;
  const int32_t *__restrict__ out_idx;
  uint32_t *vis, *fr0, *fr1, *fr2;
  const uint32_t *dead;  // vertices without in-edges (never reached), or null; bits
                         // past n are set, `stride` words
  int64_t live;          // vertices with in-edges (n when `dead` is null)
  // Relabelled graph (cg_graph_reorder), or null: orig[v] is the original id
  // of resident vertex v and perm its inverse.  Roots come in original ids;
  // outputs are written at original positions with original parent ids.
  const int32_t *orig, *perm;
  int32_t *queue0, *queue1;
  uint32_t *bigoff0, *bigoff1;
  int32_t *levels, *parents;
  // page-locked host buffers the finished search is copied into by the
  // kernel itself (device-visible addresses; NULL = none)
  int32_t *host_levels, *host_parents;
  BfsCtl *ctl;
  cg_stats *stats;
  int64_t root;
  int direction;
  float alpha, beta;
  int64_t tau;
  int level_cap;
  long long timeout_ns;
  int unmatched_wait;
};

}  // namespace cg

namespace cg {
struct FifoState;
}

struct cg_graph {
  int device = 0;
  int num_sms = 0;
  int64_t n = 0, nnz = 0;
  bool symmetric = false;
  int64_t *in_off = nullptr;
  int32_t *in_idx = nullptr;
  int64_t *out_off = nullptr;
  int32_t *out_idx = nullptr;
  cudaStream_t stream = nullptr;
  cg_options opt{};
  // per-root search state
  int64_t words = 0;            // ceil(n / 32)
  uint32_t *bitmaps = nullptr;  // vis | fr0 | fr1 | fr2, 4 * bitmap_stride(n)
  uint32_t *dead = nullptr;     // 1 bit per vertex: no in-edges (dead_prepare),
                                // bitmap_stride(n) words
  int64_t live = 0;             // vertices with in-edges
  // cg_graph_reorder: resident vertex v is original vertex orig[v]; perm is
  // the inverse (both int32[n], null for a graph in its original order)
  int32_t *orig = nullptr;
  int32_t *perm = nullptr;
  int32_t reorder = 0;          // CG_ORDER_* the handle was built with
  int32_t *queue = nullptr;     // 2 * n
  uint32_t *bigoff = nullptr;   // 2 * bcap
  int64_t bcap = 0;
  cg::BfsCtl *ctl = nullptr;
  cg_stats *d_stats = nullptr;
  int32_t *tmp_levels = nullptr;   // host-output searches land here first
  int32_t *tmp_parents = nullptr;
  int bfs_grid = 0, bfs_block = 0;
  // multi-source state (allocated on first use)
  int ms_lane_words = 0;
  uint64_t *ms_bits = nullptr;     // vis | cur | nxt, 3 * n * lane_words
  int32_t *ms_levels = nullptr;    // host-output batches land here first
  int32_t *ms_parents = nullptr;
  int64_t ms_out_cap = 0;          // elements of ms_levels / ms_parents
  void *ms_ctl = nullptr;
  int ms_grid = 0, ms_block = 0;
  int64_t device_bytes = 0;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  cg_stats *h_stats = nullptr;     // page-locked copy target of d_stats
  cg::FifoState *fifo = nullptr;   // FIFO parent pass scratch (first use)
};

namespace cg {
// Records a CUDA error for cg_last_error_string and returns CG_ERR_CUDA.
int cuda_fail(cudaError_t e, const char *what);
// Sets the text cg_last_error_string returns (a reason, not a CUDA error).
void set_error_text(const char *text);
int bfs_prepare(cg_graph *g);
int dead_prepare(cg_graph *g);
// CG_ERR_NOT_SUPPORTED (with a reason) while the handle's stream is being
// captured: for set-up that has to synchronise the handle's stream.
int refuse_setup_in_capture(cg_graph *g);
int msbfs_prepare(cg_graph *g, int lane_words, int64_t out_elems);
// CG_ERR_NOT_SUPPORTED (with a reason naming `what`) on a graph made by
// cg_graph_reorder, whose relabelled arrays only the per-root search maps back.
int refuse_reordered(const cg_graph *g, const char *what);
void msbfs_release(cg_graph *g);
// Rewrites the parents of a finished search (d_levels final) by the FIFO rule
// of scipy's breadth_first_order; synchronises with the handle's stream.
int fifo_parents(cg_graph *g, int64_t root, const int32_t *d_levels, int32_t *d_parents);
void fifo_free(FifoState *f);
}  // namespace cg

#define CG_CUDA(call)                                    \
  do {                                                   \
    cudaError_t _e = (call);                             \
    if (_e != cudaSuccess) return cg::cuda_fail(_e, #call); \
  } while (0)

// ---------------------------------------------------------------------------
// device helpers
// ---------------------------------------------------------------------------
namespace cg {

__device__ __forceinline__ long long global_ns() {
  long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

__device__ __forceinline__ unsigned ld_acquire(const unsigned *p) {
  unsigned v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

__device__ __forceinline__ unsigned atom_add_acq_rel(unsigned *p, unsigned v) {
  unsigned old;
  asm volatile("atom.acq_rel.gpu.global.add.u32 %0, [%1], %2;"
               : "=r"(old) : "l"(p), "r"(v) : "memory");
  return old;
}

__device__ __forceinline__ unsigned long long ld_acquire64(const unsigned long long *p) {
  unsigned long long v;
  asm volatile("ld.acquire.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
  return v;
}

constexpr unsigned kWaitFailed = 0xffffffffu;

// Grid-wide wait for a cooperative launch (all blocks co-resident), called by
// thread 0 of each block after a __syncthreads.  The thread arrives on its
// group counter with an acquire-release add (releasing the block's writes,
// ordered before it by the __syncthreads); the last arrival of a group resets
// that counter and arrives on the top counter the same way; the last group
// resets the top counter, runs `decide()` (it sees every block's writes) and
// releases the sync word with the next generation and decide()'s payload.
// Everyone else polls the sync word with acquire loads and gets the payload.
// Every wait is bounded: after `timeout_ns` (or once another block has
// flagged an error) the thread records CG_ERR_TIMEOUT and returns
// kWaitFailed, so a wait that can never complete ends the kernel instead of
// spinning.  `extra` > 0 makes the top counter expect that many arrivals that
// never come (the test hook behind cg_options.test_unmatched_wait).
// arrive_and_wait for a caller that knows the generation g of the sync word
// (the value before this wait; each completed wait adds one), saving the load
// of it from the arrival's critical path.
template <class Decide>
__device__ __forceinline__ unsigned arrive_and_wait_gen(GridWait *w, unsigned g, int *status,
                                                        long long timeout_ns, unsigned extra,
                                                        Decide decide) {
  const unsigned groups = gridDim.x < (unsigned)kWaitGroups ? gridDim.x : kWaitGroups;
  const unsigned grp = blockIdx.x % kWaitGroups;
  const unsigned members = (gridDim.x - grp + kWaitGroups - 1) / kWaitGroups;
  if (atom_add_acq_rel(&w->group[grp].count, 1u) + 1u == members) {
    asm volatile("st.relaxed.gpu.global.u32 [%0], 0;" ::"l"(&w->group[grp].count) : "memory");
    if (atom_add_acq_rel(&w->top, 1u) + 1u == groups + extra) {
      asm volatile("st.relaxed.gpu.global.u32 [%0], 0;" ::"l"(&w->top) : "memory");
      const unsigned payload = decide();
      const unsigned long long word =
          (unsigned long long)(g + 1u) | ((unsigned long long)payload << 32);
      asm volatile("st.release.gpu.global.u64 [%0], %1;" ::"l"(&w->sync), "l"(word) : "memory");
      return payload;
    }
  }
  long long t0 = 0;
  unsigned spins = 0;
  while (true) {
    const unsigned long long s1 = ld_acquire64(&w->sync);
    if ((unsigned)s1 != g) return (unsigned)(s1 >> 32);
    if ((++spins & 255u) == 0) {
      if (t0 == 0) t0 = global_ns();
      if (*(volatile int *)status != 0 || global_ns() - t0 > timeout_ns) {
        atomicCAS(status, 0, (int)CG_ERR_TIMEOUT);
        return kWaitFailed;
      }
    }
  }
}

template <class Decide>
__device__ __forceinline__ unsigned arrive_and_wait(GridWait *w, int *status,
                                                    long long timeout_ns, unsigned extra,
                                                    Decide decide) {
  const unsigned g = (unsigned)ld_acquire64(&w->sync);
  return arrive_and_wait_gen(w, g, status, timeout_ns, extra, decide);
}

struct NoDecision {
  __device__ unsigned operator()() const { return 0u; }
};

// Block-wide form without a decision: all threads call; false on timeout.
__device__ __forceinline__ bool grid_wait(GridWait *w, int *status, long long timeout_ns,
                                          unsigned extra = 0) {
  __shared__ int s_ok;
  __syncthreads();
  if (threadIdx.x == 0)
    s_ok = arrive_and_wait(w, status, timeout_ns, extra, NoDecision()) != kWaitFailed;
  __syncthreads();
  return s_ok != 0;
}

__device__ __forceinline__ int warp_id_global() {
  return (int)((blockIdx.x * blockDim.x + threadIdx.x) >> 5);
}
__device__ __forceinline__ int lane_id() { return (int)(threadIdx.x & 31); }

}  // namespace cg
