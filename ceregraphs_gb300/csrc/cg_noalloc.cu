// cg_bfs_noalloc: the per-root search for callers that cannot let the library
// allocate device memory.
//
// Some callers own every byte of device memory they use and forbid anyone else
// from calling cudaMalloc: runtimes that reserve the GPU up front in their own
// pool (a JVM or Go service that binds this library over JNI/cgo and budgets
// HBM itself), or real-time loops where an allocation's implicit device-wide
// synchronisation would stall other work.  The handle API cannot serve them:
// cg_graph_create allocates the graph copy and the search state.  This entry
// point takes the caller's device CSR/CSC and output arrays as they are, and
// keeps its search state (bitmaps, frontier queues, round records, statistics)
// in one file-scope __device__ array of fixed size, which exists in every GPU
// that loads the library until the process exits.  It calls no cudaMalloc,
// cudaFree or allocating library routine; the search is the same persistent
// kernel the handle API launches.
#include <cuda_runtime.h>
#include <stdio.h>

#include <mutex>

#include "cg_internal.cuh"

namespace cg {

__global__ void bfs_persistent(BfsParams p);
void set_error_text(const char *text);

int64_t bfs_big_capacity(int64_t n, int64_t nnz);

constexpr int64_t kNoAllocMaxVertices = CG_NOALLOC_MAX_VERTICES;
constexpr int64_t kNoAllocMaxBig = CG_NOALLOC_MAX_BIG;
constexpr int64_t kNoAllocWords = bitmap_stride(kNoAllocMaxVertices);

constexpr size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }
constexpr size_t kOffCtl = 0;
constexpr size_t kOffStats = align256(kOffCtl + sizeof(BfsCtl));
constexpr size_t kOffBitmaps = align256(kOffStats + sizeof(cg_stats));
constexpr size_t kOffQueue = align256(kOffBitmaps + sizeof(uint32_t) * 4 * kNoAllocWords);
constexpr size_t kOffBig = align256(kOffQueue + sizeof(int32_t) * 2 * kNoAllocMaxVertices);
constexpr size_t kScratchBytes = align256(kOffBig + sizeof(uint32_t) * 2 * kNoAllocMaxBig);

// The search state of every cg_bfs_noalloc call on this GPU (about 25 MiB).
static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

constexpr int kMaxDevices = 64;
static std::mutex g_setup_mu;
static int g_grid[kMaxDevices] = {};

// With the device current: the device address of the scratch array (host code
// cannot use the symbol itself, whose host-side name is only a stand-in) and
// the grid size.  The address is looked up on every call -- the lookup is a
// host-side table read -- so a cudaDeviceReset between calls, which reloads
// the module and may move the array, leaves no stale address behind.  The
// grid size (SM count times resident blocks per SM) is fixed per device and
// computed once.
static int noalloc_setup(int dev, void **scratch, int *grid) {
  void *addr = nullptr;
  cudaError_t e = cudaGetSymbolAddress(&addr, g_noalloc_scratch);
  if (e != cudaSuccess) return cuda_fail(e, "cudaGetSymbolAddress(g_noalloc_scratch)");
  std::lock_guard<std::mutex> lock(g_setup_mu);
  if (!g_grid[dev]) {
    int sms = 0, per_sm = 0;
    e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess) return cuda_fail(e, "cudaDeviceGetAttribute");
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, bfs_persistent, 512, 0);
    if (e != cudaSuccess) return cuda_fail(e, "cudaOccupancyMaxActiveBlocksPerMultiprocessor");
    if (per_sm <= 0) return CG_ERR_NOT_SUPPORTED;
    g_grid[dev] = per_sm * sms;
  }
  *scratch = addr;
  *grid = g_grid[dev];
  return CG_OK;
}

// True when `p` is page-locked host memory the GPU can write (cudaHostAlloc,
// cudaHostRegister, cg_host_alloc); false for pageable memory.
static bool page_locked(const void *p) {
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();  // pageable pointers may set a non-sticky error
    return false;
  }
  return a.type == cudaMemoryTypeHost;
}

}  // namespace cg

using namespace cg;

extern "C" int cg_bfs_noalloc(int64_t n, int64_t nnz, const int64_t *d_in_off,
                              const int32_t *d_in_idx, const int64_t *d_out_off,
                              const int32_t *d_out_idx, int64_t root, int32_t *d_levels,
                              int32_t *d_parents, cg_stats *stats, void *stream) {
  if (n <= 0 || nnz < 0 || !d_in_off || (nnz > 0 && !d_in_idx) || !d_levels || !d_parents ||
      root < 0 || root >= n || ((d_out_off == nullptr) != (d_out_idx == nullptr)))
    return CG_ERR_INVALID_ARG;
  if (n > kNoAllocMaxVertices || bfs_big_capacity(n, nnz) > kNoAllocMaxBig) {
    char msg[200];
    snprintf(msg, sizeof(msg),
             "cg_bfs_noalloc: graph exceeds the fixed scratch capacity (n = %lld > %lld "
             "vertices, or nnz / %d + 1 > %lld vertices of out-degree > %d)",
             (long long)n, (long long)kNoAllocMaxVertices, kLightMax + 1,
             (long long)kNoAllocMaxBig, kLightMax);
    set_error_text(msg);
    return CG_ERR_INVALID_ARG;
  }
  int dev = 0;
  CG_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= kMaxDevices) return CG_ERR_NOT_SUPPORTED;
  void *scratch = nullptr;
  int grid = 0;
  int rc = noalloc_setup(dev, &scratch, &grid);
  if (rc) return rc;
  unsigned char *base = static_cast<unsigned char *>(scratch);
  const int64_t words = (n + 31) / 32;
  cudaStream_t st = (cudaStream_t)stream;

  BfsParams p;
  p.n = n;
  p.nnz = nnz;
  p.words = words;
  const int64_t stride = bitmap_stride(n);  // <= kNoAllocWords
  p.tiles = stride / kTileWords;
  p.in_off = d_in_off;
  p.in_idx = d_in_idx;
  p.out_off = d_out_off ? d_out_off : d_in_off;
  p.out_idx = d_out_idx ? d_out_idx : d_in_idx;
  uint32_t *bitmaps = reinterpret_cast<uint32_t *>(base + kOffBitmaps);
  p.vis = bitmaps;
  p.fr0 = bitmaps + stride;
  p.fr1 = bitmaps + 2 * stride;
  p.fr2 = bitmaps + 3 * stride;
  // No per-graph state is kept here, so the map of vertices without in-edges
  // that the handle API builds once is absent: pull rounds load the in-list
  // offsets of those vertices too (about 10 us more per late pull round at
  // R-MAT scale 21 than cg_bfs; results are the same).
  p.dead = nullptr;
  p.live = n;
  p.orig = p.perm = nullptr;
  int32_t *queue = reinterpret_cast<int32_t *>(base + kOffQueue);
  p.queue0 = queue;
  p.queue1 = queue + n;
  uint32_t *bigoff = reinterpret_cast<uint32_t *>(base + kOffBig);
  p.bigoff0 = bigoff;
  p.bigoff1 = bigoff + kNoAllocMaxBig;
  p.levels = d_levels;
  p.host_levels = nullptr;
  p.host_parents = nullptr;
  p.parents = d_parents;
  p.ctl = reinterpret_cast<BfsCtl *>(base + kOffCtl);
  p.stats = reinterpret_cast<cg_stats *>(base + kOffStats);
  p.root = root;
  p.direction = CG_DIR_AUTO;
  p.alpha = 15.f;
  p.beta = 18.f;
  p.tau = (int64_t)(0.15 * (double)n + 0.5);
  p.level_cap = (int)((n + 1) < 0x7fffffff ? n + 1 : 0x7fffffff);
  p.timeout_ns = 1000ll * 1000000ll;
  p.unmatched_wait = 0;
  // The array keeps the previous call's contents: the round records and the
  // grid-wait counter must start at zero (bitmaps and outputs are reset by the
  // kernel itself); the memset is enqueued below, after the argument checks.
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(grid);
  cfg.blockDim = dim3(512);
  cfg.dynamicSmemBytes = 0;
  cfg.stream = st;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeCooperative;
  attr[0].val.cooperative = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  // A call that would wait for the stream cannot run inside a stream capture:
  // refuse it before anything is enqueued.
  const bool async_stats = stats && page_locked(stats);
  if (stats && !async_stats) {
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    CG_CUDA(cudaStreamIsCapturing(st, &cs));
    if (cs != cudaStreamCaptureStatusNone) {
      set_error_text("cg_bfs_noalloc: pageable stats make the call wait for the stream, and "
                     "the stream is being captured");
      return CG_ERR_NOT_SUPPORTED;
    }
  }
  CG_CUDA(cudaMemsetAsync(p.ctl, 0, sizeof(BfsCtl), st));
  CG_CUDA(cudaLaunchKernelEx(&cfg, bfs_persistent, p));
  if (!stats) return CG_OK;
  CG_CUDA(cudaMemcpyAsync(stats, p.stats, sizeof(cg_stats), cudaMemcpyDeviceToHost, st));
  if (async_stats) return CG_OK;  // valid once the stream has reached this point
  CG_CUDA(cudaStreamSynchronize(st));
  return stats->status;
}
