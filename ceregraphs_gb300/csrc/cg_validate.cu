// Graph500 result validation on the device: the five tree checks for k
// searches in two passes over the resident graph, instead of the host-side
// scipy cross-check and invalid_parents walk the reference runs per search
// (run_graph500.py:383-395, bfs/plots/bfs_tree_plot.py:140-152), which
// dominates wall time for 64 searches at scale 23 and above.
//
// Checks (each search has a root, levels[n] and parents[n]; -1 = unreached):
//   ROOT       parent[root] == root and level[root] == 0
//   TREE       every reached v != root has a parent p in [0, n), level[v] >= 1
//              and level[p] == level[v] - 1 (levels fall by one along every
//              parent pointer, so the pointers form a tree into the root)
//   EDGES      every stored edge u -> v with u reached has v reached and
//              level[v] <= level[u] + 1 (for symmetric graphs both
//              orientations are stored, giving |level[u] - level[v]| <= 1)
//   SPAN       level[v] >= 0 exactly when parent[v] >= 0; with TREE and EDGES
//              the reached set is closed under out-edges and every reached
//              vertex leads to the root, so it is the reachable set
//   TREE_EDGE  parent[v] -> v is an edge (parent[v] is in v's in-list)
//   LOWEST     parent[v] is the lowest-index in-neighbour at level[v] - 1
//              (this engine's parent rule; not a Graph500 requirement)
// Inputs are treated as untrusted: a parent outside [0, n) is counted, never
// dereferenced.
#include <cuda_runtime.h>
#include <stdint.h>

#include <new>

#include "cg_internal.cuh"

namespace cg {
namespace {

constexpr int kChecks = CG_CHECKS;
constexpr int kBlock = 256;
constexpr int kEdgesPerWarp = 32 * 64;

struct Tally {  // per search, device side
  unsigned long long fail[kChecks];
  unsigned long long first[kChecks];  // lowest failing vertex, ~0 if none
};

__device__ __forceinline__ void flag(Tally *t, int check, int64_t v) {
  atomicAdd(&t->fail[check], 1ull);
  atomicMin(&t->first[check], (unsigned long long)v);
}

// Binary search for u in the sorted list idx[b, e).
__device__ __forceinline__ bool contains(const int32_t *__restrict__ idx, int64_t b, int64_t e,
                                         int32_t u) {
  while (b < e) {
    const int64_t mid = (b + e) >> 1;
    const int32_t x = idx[mid];
    if (x == u) return true;
    if (x < u)
      b = mid + 1;
    else
      e = mid;
  }
  return false;
}

// Per-vertex checks (ROOT, TREE, SPAN, TREE_EDGE, LOWEST).  Each warp takes 32
// consecutive vertices; a lane scans its own in-list for the lowest parent
// when it is short, and the warp scans the long ones together.
__global__ void __launch_bounds__(kBlock) vertex_checks_kernel(
    int64_t n, const int64_t *__restrict__ in_off, const int32_t *__restrict__ in_idx,
    const int64_t *__restrict__ roots, const int32_t *__restrict__ levels_all,
    const int32_t *__restrict__ parents_all, Tally *tallies) {
  const int s = blockIdx.y;
  const int32_t *__restrict__ level = levels_all + (int64_t)s * n;
  const int32_t *__restrict__ parent = parents_all + (int64_t)s * n;
  const int64_t root = roots[s];
  Tally *t = tallies + s;
  const int lane = threadIdx.x & 31;
  const int64_t warps = (int64_t)gridDim.x * (kBlock / 32);
  for (int64_t base = ((int64_t)blockIdx.x * (kBlock / 32) + (threadIdx.x >> 5)) * 32; base < n;
       base += warps * 32) {
    const int64_t v = base + lane;
    bool long_scan = false;
    int32_t want_level = 0, p = -1;
    int64_t b = 0, e = 0;
    if (v < n) {
      const int32_t lv = level[v];
      p = parent[v];
      if ((lv >= 0) != (p >= 0)) flag(t, CG_CHECK_SPAN, v);
      if (v == root) {
        if (p != (int32_t)root || lv != 0) flag(t, CG_CHECK_ROOT, v);
      } else if (p >= 0) {
        if (p >= n || lv < 1 || level[p] != lv - 1) {
          flag(t, CG_CHECK_TREE, v);
        } else {
          b = in_off[v];
          e = in_off[v + 1];
          if (!contains(in_idx, b, e, p)) flag(t, CG_CHECK_TREE_EDGE, v);
          want_level = lv - 1;
          if (e - b <= 32) {
            int32_t low = -1;
            for (int64_t j = b; j < e; ++j) {
              const int32_t u = in_idx[j];
              if (level[u] == want_level) {
                low = u;
                break;
              }
            }
            if (low != p) flag(t, CG_CHECK_LOWEST, v);
          } else {
            long_scan = true;
          }
        }
      } else if (p < -1) {
        flag(t, CG_CHECK_TREE, v);
      }
    }
    // long in-lists: the whole warp scans one list at a time, 32 entries per step
    unsigned pending = __ballot_sync(0xffffffffu, long_scan);
    while (pending) {
      const int src = __ffs(pending) - 1;
      pending &= pending - 1;
      const int64_t sb = __shfl_sync(0xffffffffu, b, src);
      const int64_t se = __shfl_sync(0xffffffffu, e, src);
      const int32_t sl = __shfl_sync(0xffffffffu, want_level, src);
      int32_t low = -1;
      for (int64_t j = sb; j < se; j += 32) {
        const int64_t jj = j + lane;
        const bool hit = jj < se && level[in_idx[jj]] == sl;
        const unsigned m = __ballot_sync(0xffffffffu, hit);
        if (m) {
          low = __shfl_sync(0xffffffffu, jj < se ? in_idx[jj] : -1, __ffs(m) - 1);
          break;
        }
      }
      if (lane == src && low != p) flag(t, CG_CHECK_LOWEST, v);
    }
  }
}

// EDGES over every stored entry, balanced by entries: each warp owns
// kEdgesPerWarp consecutive entries, lanes stride by 32 and track their row.
__global__ void __launch_bounds__(kBlock) edge_checks_kernel(
    int64_t n, int64_t nnz, const int64_t *__restrict__ in_off, const int32_t *__restrict__ in_idx,
    const int32_t *__restrict__ levels_all, Tally *tallies) {
  const int s = blockIdx.y;
  const int32_t *__restrict__ level = levels_all + (int64_t)s * n;
  Tally *t = tallies + s;
  const int lane = threadIdx.x & 31;
  const int64_t warps = (int64_t)gridDim.x * (kBlock / 32);
  for (int64_t w0 = ((int64_t)blockIdx.x * (kBlock / 32) + (threadIdx.x >> 5)) * kEdgesPerWarp;
       w0 < nnz; w0 += warps * kEdgesPerWarp) {
    int64_t e = w0 + lane;
    if (e >= nnz) continue;
    // row r with in_off[r] <= e < in_off[r + 1]
    int64_t lo = 0, hi = n;
    while (lo < hi) {
      const int64_t mid = (lo + hi + 1) >> 1;
      if (in_off[mid] <= e)
        lo = mid;
      else
        hi = mid - 1;
    }
    int64_t r = lo, r_end = in_off[r + 1];
    int32_t lr = level[r];
    const int64_t stop = min(w0 + (int64_t)kEdgesPerWarp, nnz);
    for (; e < stop; e += 32) {
      while (e >= r_end) {
        ++r;
        r_end = in_off[r + 1];
        lr = level[r];
      }
      const int32_t lu = level[in_idx[e]];
      if (lu >= 0 && (lr < 0 || (int64_t)lr > (int64_t)lu + 1)) flag(t, CG_CHECK_EDGES, r);
    }
  }
}

__global__ void tally_init_kernel(Tally *t, int k) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < k * kChecks) {
    t[i / kChecks].fail[i % kChecks] = 0ull;
    t[i / kChecks].first[i % kChecks] = ~0ull;
  }
}

}  // namespace
}  // namespace cg

using namespace cg;

extern "C" int cg_validate_device(cg_graph *g, const int64_t *roots, int32_t k,
                                  const int32_t *d_levels, const int32_t *d_parents,
                                  cg_validation *out) {
  if (g) {
    if (int r = refuse_reordered(g, "cg_validate_device")) return r;
  }
  if (!g || !roots || k <= 0 || k > 65535 || !d_levels || !d_parents || !out)
    return CG_ERR_INVALID_ARG;
  for (int32_t i = 0; i < k; ++i)
    if (roots[i] < 0 || roots[i] >= g->n) return CG_ERR_INVALID_ARG;
  CG_CUDA(cudaSetDevice(g->device));
  Tally *d_t = nullptr;
  int64_t *d_roots = nullptr;
  if (cudaMallocAsync((void **)&d_t, sizeof(Tally) * (size_t)k, g->stream) != cudaSuccess)
    return CG_ERR_OUT_OF_MEMORY;
  if (cudaMallocAsync((void **)&d_roots, sizeof(int64_t) * (size_t)k, g->stream) != cudaSuccess) {
    cudaFreeAsync(d_t, g->stream);
    return CG_ERR_OUT_OF_MEMORY;
  }
  int rc = CG_OK;
  Tally *h_t = new (std::nothrow) Tally[k];
  do {
    if (!h_t) { rc = CG_ERR_OUT_OF_MEMORY; break; }
    cudaError_t e = cudaMemcpyAsync(d_roots, roots, sizeof(int64_t) * (size_t)k,
                                    cudaMemcpyHostToDevice, g->stream);
    if (e != cudaSuccess) { rc = cuda_fail(e, "validate roots"); break; }
    tally_init_kernel<<<(k * kChecks + 255) / 256, 256, 0, g->stream>>>(d_t, k);
    // about 8 warps' worth of work per SM for each search
    const int64_t vblocks = (g->n + kBlock - 1) / kBlock;
    const int64_t cap = (int64_t)g->num_sms * 8;
    dim3 vg((unsigned)(vblocks < cap ? (vblocks > 0 ? vblocks : 1) : cap), (unsigned)k);
    vertex_checks_kernel<<<vg, kBlock, 0, g->stream>>>(g->n, g->in_off, g->in_idx, d_roots,
                                                        d_levels, d_parents, d_t);
    if (g->nnz > 0) {
      const int64_t eblocks = (g->nnz + (int64_t)kEdgesPerWarp * (kBlock / 32) - 1) /
                              ((int64_t)kEdgesPerWarp * (kBlock / 32));
      dim3 eg((unsigned)(eblocks < cap ? eblocks : cap), (unsigned)k);
      edge_checks_kernel<<<eg, kBlock, 0, g->stream>>>(g->n, g->nnz, g->in_off, g->in_idx,
                                                        d_levels, d_t);
    }
    e = cudaGetLastError();
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(h_t, d_t, sizeof(Tally) * (size_t)k, cudaMemcpyDeviceToHost, g->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(g->stream);
    if (e != cudaSuccess) { rc = cuda_fail(e, "cg_validate_device"); break; }
    for (int32_t i = 0; i < k; ++i) {
      for (int c = 0; c < kChecks; ++c) {
        out[i].failures[c] = (int64_t)h_t[i].fail[c];
        out[i].first[c] = h_t[i].first[c] == ~0ull ? -1 : (int64_t)h_t[i].first[c];
      }
    }
  } while (0);
  cudaFreeAsync(d_t, g->stream);
  cudaFreeAsync(d_roots, g->stream);
  cudaStreamSynchronize(g->stream);
  delete[] h_t;
  return rc;
}
