// cg_graph_reorder: a degree-ordered copy of a resident graph for per-root
// searches -- the one-GPU counterpart of the reference's balancing step,
// util/analyze.cpp:226-372, which reassigns vertices so that each PE of a P x P
// grid gets a similar share of the edges, keeping vertex identity for the
// results (--operm, util/analyze.cpp:431-437).  One GPU has no PE grid to
// balance; what a relabelling can buy here is locality: vertices of high
// in-degree (the ones pull rounds find parents among and push rounds expand)
// get the lowest resident ids, so their frontier bits and list offsets share
// cache lines, and the vertices without in-edges end up together at the top,
// where whole bitmap tiles of them are skipped at once.
//
// Identity is kept as in --operm: searches on the copy take roots in original
// ids and write levels and parents at original positions with original parent
// ids (the kernel maps through orig[]), and every in-list stays in ascending
// ORIGINAL id order, so "first frontier entry of the in-list" and the push
// rounds' atomicMin (taken over original ids) still give the lowest-index
// parent: results are bit-identical to the original graph's.
#include <cuda_runtime.h>
#include <stdint.h>
#include <stdio.h>

#include <cub/cub.cuh>

#include "cg_internal.cuh"

namespace cg {
namespace {

// Sort key of vertex v: descending in-degree, then ascending id.
__global__ void degree_keys_kernel(int64_t n, const int64_t *__restrict__ off, uint64_t *keys) {
  for (int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; v < n;
       v += (int64_t)gridDim.x * blockDim.x) {
    const uint64_t deg = (uint64_t)(off[v + 1] - off[v]);
    keys[v] = ((0xffffffffull - (deg < 0xffffffffull ? deg : 0xffffffffull)) << 32) |
              (uint64_t)v;
  }
}

// orig[i] = the vertex at sorted position i, perm its inverse; len[i] = the
// in-degree of orig[i] (len[n] = 0, for the exclusive scan into offsets).
__global__ void permutation_kernel(int64_t n, const uint64_t *__restrict__ sorted,
                                   const int64_t *__restrict__ off, int32_t *orig, int32_t *perm,
                                   int64_t *len) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i <= n;
       i += (int64_t)gridDim.x * blockDim.x) {
    if (i == n) {
      len[n] = 0;
      continue;
    }
    const int32_t o = (int32_t)(sorted[i] & 0xffffffffull);
    orig[i] = o;
    perm[o] = (int32_t)i;
    len[i] = off[o + 1] - off[o];
  }
}

// Lengths of a second list family (the out-lists of a directed graph) in the
// new order.
__global__ void lengths_kernel(int64_t n, const int32_t *__restrict__ orig,
                               const int64_t *__restrict__ off, int64_t *len) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i <= n;
       i += (int64_t)gridDim.x * blockDim.x) {
    if (i == n) {
      len[n] = 0;
      continue;
    }
    const int32_t o = orig[i];
    len[i] = off[o + 1] - off[o];
  }
}

// One warp per new vertex i: copies the list of orig[i], entries renamed to
// new ids, in the same (ascending original id) order.
__global__ void relabel_lists_kernel(int64_t n, const int32_t *__restrict__ orig,
                                     const int32_t *__restrict__ perm,
                                     const int64_t *__restrict__ off,
                                     const int32_t *__restrict__ idx,
                                     const int64_t *__restrict__ off2, int32_t *idx2) {
  const int lane = threadIdx.x & 31;
  const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t i = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; i < n; i += nwarps) {
    const int32_t o = orig[i];
    const int64_t s = off[o], e = off[o + 1], d = off2[i];
    for (int64_t j = s + lane; j < e; j += 32) idx2[d + (j - s)] = perm[idx[j]];
  }
}

unsigned grid_for(int64_t work, int sms) {
  const int64_t b = (work + 255) / 256;
  const int64_t cap = (int64_t)sms * 16;
  return (unsigned)(b < 1 ? 1 : (b > cap ? cap : b));
}

// Offsets (exclusive sum of len[0..n]) into off2.
int scan_offsets(const int64_t *len, int64_t *off2, int64_t n, cudaStream_t st) {
  size_t tb = 0;
  CG_CUDA(cub::DeviceScan::ExclusiveSum(nullptr, tb, len, off2, n + 1, st));
  void *temp = nullptr;
  if (cudaMalloc(&temp, tb ? tb : 16) != cudaSuccess) return CG_ERR_OUT_OF_MEMORY;
  cudaError_t e = cub::DeviceScan::ExclusiveSum(temp, tb, len, off2, n + 1, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  cudaFree(temp);
  if (e != cudaSuccess) return cuda_fail(e, "offset scan");
  return CG_OK;
}

}  // namespace

int refuse_reordered(const cg_graph *g, const char *what) {
  if (!g->orig) return CG_OK;
  char msg[160];
  snprintf(msg, sizeof(msg), "%s: not supported on a reordered graph (per-root searches only)",
           what);
  set_error_text(msg);
  return CG_ERR_NOT_SUPPORTED;
}

}  // namespace cg

using namespace cg;

extern "C" int cg_graph_reorder(const cg_graph *g, int32_t order, cg_graph **out) {
  if (!g || !out || order != CG_ORDER_DEGREE) return CG_ERR_INVALID_ARG;
  *out = nullptr;
  if (g->orig) {
    set_error_text("cg_graph_reorder: the graph is already a reordered copy");
    return CG_ERR_NOT_SUPPORTED;
  }
  int prev = 0;
  CG_CUDA(cudaGetDevice(&prev));
  CG_CUDA(cudaSetDevice(g->device));
  CG_CUDA(cudaStreamSynchronize(g->stream));  // the graph's upload has landed
  const int64_t n = g->n, nnz = g->nnz;
  cudaStream_t st = nullptr;
  CG_CUDA(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
  uint64_t *keys = nullptr, *sorted = nullptr;
  int32_t *orig = nullptr, *perm = nullptr, *in_idx = nullptr, *out_idx = nullptr;
  int64_t *len = nullptr, *in_off = nullptr, *out_off = nullptr;
  void *temp = nullptr;
  cg_graph *g2 = nullptr;
  int rc = CG_OK;
  do {
    if (cudaMalloc(&keys, sizeof(uint64_t) * n) != cudaSuccess ||
        cudaMalloc(&sorted, sizeof(uint64_t) * n) != cudaSuccess ||
        cudaMalloc(&orig, sizeof(int32_t) * n) != cudaSuccess ||
        cudaMalloc(&perm, sizeof(int32_t) * n) != cudaSuccess ||
        cudaMalloc(&len, sizeof(int64_t) * (n + 1)) != cudaSuccess ||
        cudaMalloc(&in_off, sizeof(int64_t) * (n + 1)) != cudaSuccess ||
        cudaMalloc(&in_idx, sizeof(int32_t) * (nnz > 0 ? nnz : 1)) != cudaSuccess) {
      rc = CG_ERR_OUT_OF_MEMORY;
      break;
    }
    degree_keys_kernel<<<grid_for(n, g->num_sms), 256, 0, st>>>(n, g->in_off, keys);
    size_t tb = 0;
    cudaError_t e = cub::DeviceRadixSort::SortKeys(nullptr, tb, keys, sorted, n, 0, 64, st);
    if (e != cudaSuccess) { rc = cuda_fail(e, "degree sort"); break; }
    if (cudaMalloc(&temp, tb ? tb : 16) != cudaSuccess) { rc = CG_ERR_OUT_OF_MEMORY; break; }
    e = cub::DeviceRadixSort::SortKeys(temp, tb, keys, sorted, n, 0, 64, st);
    if (e != cudaSuccess) { rc = cuda_fail(e, "degree sort"); break; }
    permutation_kernel<<<grid_for(n + 1, g->num_sms), 256, 0, st>>>(n, sorted, g->in_off, orig,
                                                                    perm, len);
    if ((rc = scan_offsets(len, in_off, n, st))) break;
    relabel_lists_kernel<<<grid_for(32 * n, g->num_sms), 256, 0, st>>>(n, orig, perm, g->in_off,
                                                                       g->in_idx, in_off, in_idx);
    if (!g->symmetric) {
      if (cudaMalloc(&out_off, sizeof(int64_t) * (n + 1)) != cudaSuccess ||
          cudaMalloc(&out_idx, sizeof(int32_t) * (nnz > 0 ? nnz : 1)) != cudaSuccess) {
        rc = CG_ERR_OUT_OF_MEMORY;
        break;
      }
      lengths_kernel<<<grid_for(n + 1, g->num_sms), 256, 0, st>>>(n, orig, g->out_off, len);
      if ((rc = scan_offsets(len, out_off, n, st))) break;
      relabel_lists_kernel<<<grid_for(32 * n, g->num_sms), 256, 0, st>>>(
          n, orig, perm, g->out_off, g->out_idx, out_off, out_idx);
    }
    if ((e = cudaGetLastError()) != cudaSuccess || (e = cudaStreamSynchronize(st)) != cudaSuccess) {
      rc = cuda_fail(e, "cg_graph_reorder");
      break;
    }
    rc = cg_graph_create(n, nnz, in_off, in_idx, out_off, out_idx,
                         CG_GRAPH_DEVICE_PTRS | (g->symmetric ? CG_GRAPH_SYMMETRIC : 0), &g2);
    if (rc) break;
    g2->opt = g->opt;
    g2->orig = orig;
    g2->perm = perm;
    g2->reorder = order;
    g2->device_bytes += 2 * sizeof(int32_t) * n;
    orig = perm = nullptr;  // owned by g2
  } while (0);
  cudaStreamSynchronize(st);
  cudaFree(keys);
  cudaFree(sorted);
  cudaFree(temp);
  cudaFree(len);
  cudaFree(in_off);
  cudaFree(in_idx);
  cudaFree(out_off);
  cudaFree(out_idx);
  cudaFree(orig);
  cudaFree(perm);
  cudaStreamDestroy(st);
  cudaSetDevice(prev);
  if (rc) return rc;
  *out = g2;
  return CG_OK;
}
