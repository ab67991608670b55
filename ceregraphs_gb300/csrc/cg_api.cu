// C ABI entry points (include/ceregraphs.h): handle lifecycle, Kernel-1 upload,
// Kernel-2 searches with host or device outputs, the Graph500 edge count.
#include <cuda_runtime.h>
#include <stdio.h>
#include <string.h>

#include <new>

#include "cg_internal.cuh"

namespace cg {
int bfs_launch(cg_graph *g, int64_t root, int32_t *d_levels, int32_t *d_parents,
               int32_t *host_levels = nullptr, int32_t *host_parents = nullptr);
int count_edges_launch(cg_graph *g, const int32_t *d_levels, int32_t k, unsigned long long *d_m);
int msbfs_launch(cg_graph *g, const int64_t *roots, int32_t k, int32_t *d_levels,
                 int32_t *d_parents);

static thread_local char t_last_error[256] = {0};

int cuda_fail(cudaError_t e, const char *what) {
  snprintf(t_last_error, sizeof(t_last_error), "%s: %s (%d)", what, cudaGetErrorString(e), (int)e);
  return CG_ERR_CUDA;
}

void set_error_text(const char *text) { snprintf(t_last_error, sizeof(t_last_error), "%s", text); }

static void free_graph(cg_graph *g) {
  if (!g) return;
  int prev = 0;
  cudaGetDevice(&prev);
  cudaSetDevice(g->device);
  if (g->stream) cudaStreamSynchronize(g->stream);
  msbfs_release(g);
  fifo_free(g->fifo);
  if (g->out_off && g->out_off != g->in_off) cudaFree(g->out_off);
  if (g->out_idx && g->out_idx != g->in_idx) cudaFree(g->out_idx);
  cudaFree(g->in_off);
  cudaFree(g->in_idx);
  cudaFree(g->bitmaps);
  cudaFree(g->dead);
  cudaFree(g->queue);
  cudaFree(g->bigoff);
  cudaFree(g->ctl);
  cudaFree(g->d_stats);
  cudaFree(g->tmp_levels);
  cudaFree(g->tmp_parents);
  cudaFree(g->orig);
  cudaFree(g->perm);
  if (g->ev0) cudaEventDestroy(g->ev0);
  if (g->ev1) cudaEventDestroy(g->ev1);
  if (g->h_stats) cudaFreeHost(g->h_stats);
  if (g->stream) cudaStreamDestroy(g->stream);
  cudaSetDevice(prev);
  delete g;
}

// Checks CSR structure on the host: monotone offsets within [0, nnz], indices
// in [0, n).  (Device-pointer inputs are trusted: checking them would need a
// kernel and a copy back.)
static bool valid_host_csr(int64_t n, int64_t nnz, const int64_t *off, const int32_t *idx) {
  if (off[0] != 0 || off[n] != nnz) return false;
  for (int64_t i = 0; i < n; ++i)
    if (off[i + 1] < off[i]) return false;
  for (int64_t e = 0; e < nnz; ++e)
    if (idx[e] < 0 || idx[e] >= n) return false;
  return true;
}

static int upload(const void *src, size_t bytes, bool device_src, void **dst, cg_graph *g) {
  if (cudaMalloc(dst, bytes ? bytes : 16) != cudaSuccess) return CG_ERR_OUT_OF_MEMORY;
  g->device_bytes += (int64_t)bytes;
  if (bytes) CG_CUDA(cudaMemcpyAsync(*dst, src, bytes, device_src ? cudaMemcpyDeviceToDevice
                                                                  : cudaMemcpyHostToDevice,
                                     g->stream));
  return CG_OK;
}

}  // namespace cg

using namespace cg;

extern "C" {

int cg_version(void) { return 10100; }

const char *cg_strerror(int status) {
  switch (status) {
    case CG_OK: return "ok";
    case CG_ERR_INVALID_ARG: return "invalid argument";
    case CG_ERR_OUT_OF_MEMORY: return "out of device memory";
    case CG_ERR_CUDA: return "CUDA error";
    case CG_ERR_LEVEL_CAP: return "round cap reached before the frontier emptied";
    case CG_ERR_TIMEOUT: return "device-side wait timed out";
    case CG_ERR_NOT_SUPPORTED: return "not supported on this device";
    case CG_ERR_ADMISSION: return "request exceeds the HBM budget";
    case CG_ERR_PARSE: return "malformed graph file";
    case CG_ERR_IO: return "graph file could not be read";
    default: return "unknown status";
  }
}

const char *cg_last_error_string(void) { return t_last_error; }

void cg_default_options(cg_options *opt) {
  if (!opt) return;
  memset(opt, 0, sizeof(*opt));
  opt->direction = CG_DIR_AUTO;
  opt->alpha = 15.f;
  opt->beta = 18.f;
  opt->tau_switch_count = -1;
  opt->block_size = 512;
  opt->blocks_per_sm = 0;
  opt->level_cap = 0;
  opt->wait_timeout_ms = 1000;
  opt->lane_words = 1;
  opt->ms_alpha = 4.f;
  opt->test_unmatched_wait = 0;
  opt->ms_history = 0;
}

int cg_graph_create(int64_t n, int64_t nnz, const int64_t *in_off, const int32_t *in_idx,
                    const int64_t *out_off, const int32_t *out_idx, int32_t flags,
                    cg_graph **out) {
  if (!out) return CG_ERR_INVALID_ARG;
  *out = nullptr;
  const bool dev = (flags & CG_GRAPH_DEVICE_PTRS) != 0;
  const bool sym = (flags & CG_GRAPH_SYMMETRIC) != 0;
  if (n <= 0 || n > 0x7fffffffLL || nnz < 0 || !in_off || (nnz > 0 && !in_idx))
    return CG_ERR_INVALID_ARG;
  // frontier edge counts are 32-bit in the push rounds' chunking
  if (nnz >= (1ll << 32) - (1ll << 16)) return CG_ERR_NOT_SUPPORTED;
  if (!sym && (!out_off || (nnz > 0 && !out_idx))) return CG_ERR_INVALID_ARG;
  if (!dev) {
    if (!valid_host_csr(n, nnz, in_off, in_idx)) return CG_ERR_INVALID_ARG;
    if (!sym && !valid_host_csr(n, nnz, out_off, out_idx)) return CG_ERR_INVALID_ARG;
  }
  cg_graph *g = new (std::nothrow) cg_graph();
  if (!g) return CG_ERR_OUT_OF_MEMORY;
  int rc = CG_OK;
  do {
    if (cudaGetDevice(&g->device) != cudaSuccess) { rc = CG_ERR_CUDA; break; }
    if (cudaDeviceGetAttribute(&g->num_sms, cudaDevAttrMultiProcessorCount, g->device) !=
        cudaSuccess) { rc = CG_ERR_CUDA; break; }
    if (cudaStreamCreateWithFlags(&g->stream, cudaStreamNonBlocking) != cudaSuccess) {
      rc = CG_ERR_CUDA;
      break;
    }
    cudaEventCreate(&g->ev0);
    cudaEventCreate(&g->ev1);
    g->n = n;
    g->nnz = nnz;
    g->symmetric = sym;
    cg_default_options(&g->opt);
    g->opt.tau_switch_count = (int64_t)(0.15 * (double)n + 0.5);
    rc = upload(in_off, sizeof(int64_t) * (size_t)(n + 1), dev, (void **)&g->in_off, g);
    if (rc) break;
    rc = upload(in_idx, sizeof(int32_t) * (size_t)nnz, dev, (void **)&g->in_idx, g);
    if (rc) break;
    if (sym) {
      g->out_off = g->in_off;
      g->out_idx = g->in_idx;
    } else {
      rc = upload(out_off, sizeof(int64_t) * (size_t)(n + 1), dev, (void **)&g->out_off, g);
      if (rc) break;
      rc = upload(out_idx, sizeof(int32_t) * (size_t)nnz, dev, (void **)&g->out_idx, g);
      if (rc) break;
    }
    rc = bfs_prepare(g);
    if (rc) break;
    cudaError_t e = cudaStreamSynchronize(g->stream);
    if (e != cudaSuccess) { rc = cuda_fail(e, "cg_graph_create"); break; }
  } while (0);
  if (rc) {
    free_graph(g);
    return rc;
  }
  *out = g;
  return CG_OK;
}

int cg_graph_destroy(cg_graph *g) {
  if (!g) return CG_ERR_INVALID_ARG;
  free_graph(g);
  return CG_OK;
}

int cg_graph_set_options(cg_graph *g, const cg_options *opt) {
  if (!g || !opt) return CG_ERR_INVALID_ARG;
  if (opt->direction < CG_DIR_AUTO || opt->direction > CG_DIR_TAU) return CG_ERR_INVALID_ARG;
  if (opt->block_size < 0 || (opt->block_size % 32) != 0 || opt->block_size > 512)
    return CG_ERR_INVALID_ARG;
  if (opt->lane_words != 1 && opt->lane_words != 2) return CG_ERR_INVALID_ARG;
  if (opt->parent_rule != CG_PARENT_LOWEST && opt->parent_rule != CG_PARENT_FIFO)
    return CG_ERR_INVALID_ARG;
  if (opt->alpha < 0 || opt->beta < 0 || opt->ms_alpha < 0 || opt->level_cap < 0 ||
      opt->wait_timeout_ms < 0)
    return CG_ERR_INVALID_ARG;
  g->opt = *opt;
  if (g->opt.tau_switch_count < 0) g->opt.tau_switch_count = (int64_t)(0.15 * (double)g->n + 0.5);
  return CG_OK;
}

int cg_graph_get_options(const cg_graph *g, cg_options *opt) {
  if (!g || !opt) return CG_ERR_INVALID_ARG;
  *opt = g->opt;
  return CG_OK;
}

int cg_graph_info(const cg_graph *g, int64_t *n, int64_t *nnz, int32_t *symmetric,
                  int64_t *device_bytes) {
  if (!g) return CG_ERR_INVALID_ARG;
  if (n) *n = g->n;
  if (nnz) *nnz = g->nnz;
  if (symmetric) *symmetric = g->symmetric ? 1 : 0;
  if (device_bytes) *device_bytes = g->device_bytes;
  return CG_OK;
}

void *cg_graph_stream(const cg_graph *g) { return g ? (void *)g->stream : nullptr; }

int cg_bfs_device(cg_graph *g, int64_t root, int32_t *d_levels, int32_t *d_parents) {
  if (!g || !d_levels || !d_parents || root < 0 || root >= g->n) return CG_ERR_INVALID_ARG;
  if (g->opt.parent_rule == CG_PARENT_FIFO) {
    const int r = refuse_reordered(g, "the FIFO parent rule");
    if (r) return r;
  }
  const int rc = bfs_launch(g, root, d_levels, d_parents);
  if (rc || g->opt.parent_rule != CG_PARENT_FIFO) return rc;
  return fifo_parents(g, root, d_levels, d_parents);
}

int cg_graph_last_stats(cg_graph *g, cg_stats *stats) {
  if (!g || !stats || !g->d_stats) return CG_ERR_INVALID_ARG;
  CG_CUDA(cudaMemcpyAsync(stats, g->d_stats, sizeof(cg_stats), cudaMemcpyDeviceToHost, g->stream));
  CG_CUDA(cudaStreamSynchronize(g->stream));
  return CG_OK;
}

// Device-visible address of a page-locked host buffer, or NULL for pageable
// memory (which is then filled by an ordinary copy).
static int32_t *pinned_device_ptr(int32_t *host) {
  if (!host) return nullptr;
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, host) != cudaSuccess) {
    cudaGetLastError();  // not a CUDA pointer: clear the sticky-free error
    return nullptr;
  }
  if (a.type != cudaMemoryTypeHost || !a.devicePointer) return nullptr;
  return static_cast<int32_t *>(a.devicePointer);
}

int cg_bfs(cg_graph *g, int64_t root, int32_t *levels, int32_t *parents, cg_stats *stats) {
  if (!g || root < 0 || root >= g->n) return CG_ERR_INVALID_ARG;
  if (g->opt.parent_rule == CG_PARENT_FIFO) {
    const int r = refuse_reordered(g, "the FIFO parent rule");
    if (r) return r;
  }
  if (!g->tmp_levels) {
    if (cudaMalloc(&g->tmp_levels, sizeof(int32_t) * (size_t)g->n) != cudaSuccess)
      return CG_ERR_OUT_OF_MEMORY;
    if (cudaMalloc(&g->tmp_parents, sizeof(int32_t) * (size_t)g->n) != cudaSuccess)
      return CG_ERR_OUT_OF_MEMORY;
    g->device_bytes += 2 * sizeof(int32_t) * g->n;
  }
  if (!g->h_stats) {
    void *h = nullptr;
    if (cudaHostAlloc(&h, sizeof(cg_stats), cudaHostAllocDefault) != cudaSuccess)
      return CG_ERR_OUT_OF_MEMORY;
    g->h_stats = static_cast<cg_stats *>(h);
  }
  // page-locked outputs are written by the search kernel itself at its end
  // (the GPU's own SMs over the host link); pageable ones by a copy after it
  const bool fifo = g->opt.parent_rule == CG_PARENT_FIFO;
  int32_t *hl = pinned_device_ptr(levels), *hp = fifo ? nullptr : pinned_device_ptr(parents);
  CG_CUDA(cudaEventRecord(g->ev0, g->stream));
  int rc = bfs_launch(g, root, g->tmp_levels, g->tmp_parents, hl, hp);
  if (rc) return rc;
  if (fifo && (rc = fifo_parents(g, root, g->tmp_levels, g->tmp_parents))) return rc;
  CG_CUDA(cudaEventRecord(g->ev1, g->stream));
  const size_t bytes = sizeof(int32_t) * (size_t)g->n;
  if (levels && !hl)
    CG_CUDA(cudaMemcpyAsync(levels, g->tmp_levels, bytes, cudaMemcpyDeviceToHost, g->stream));
  if (parents && !hp)
    CG_CUDA(cudaMemcpyAsync(parents, g->tmp_parents, bytes, cudaMemcpyDeviceToHost, g->stream));
  CG_CUDA(cudaMemcpyAsync(g->h_stats, g->d_stats, sizeof(cg_stats), cudaMemcpyDeviceToHost,
                          g->stream));
  CG_CUDA(cudaStreamSynchronize(g->stream));
  cg_stats local = *g->h_stats;
  float ms = 0.f;
  cudaEventElapsedTime(&ms, g->ev0, g->ev1);
  local.device_ms = ms;
  if (stats) *stats = local;
  return local.status;
}

// FIFO parents for each of k finished searches (rows of k x n outputs); a
// search that failed on the device keeps its status for the caller.
static int fifo_all(cg_graph *g, const int64_t *roots, int32_t k, const int32_t *d_levels,
                    int32_t *d_parents) {
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  CG_CUDA(cudaStreamIsCapturing(g->stream, &cs));
  if (cs != cudaStreamCaptureStatusNone) {
    set_error_text("the FIFO parent rule synchronises with the stream: not capturable");
    return CG_ERR_NOT_SUPPORTED;
  }
  cg_stats st;
  CG_CUDA(cudaMemcpyAsync(&st, g->d_stats, sizeof(cg_stats), cudaMemcpyDeviceToHost, g->stream));
  CG_CUDA(cudaStreamSynchronize(g->stream));
  if (st.status) return CG_OK;
  for (int32_t i = 0; i < k; ++i) {
    const int rc = fifo_parents(g, roots[i], d_levels + (int64_t)i * g->n,
                                d_parents + (int64_t)i * g->n);
    if (rc) return rc;
  }
  return CG_OK;
}

int cg_msbfs_device(cg_graph *g, const int64_t *roots, int32_t k, int32_t *d_levels,
                    int32_t *d_parents) {
  if (!g || !roots || k <= 0 || !d_levels || !d_parents) return CG_ERR_INVALID_ARG;
  if (int r = refuse_reordered(g, "cg_msbfs_device")) return r;
  for (int32_t i = 0; i < k; ++i)
    if (roots[i] < 0 || roots[i] >= g->n) return CG_ERR_INVALID_ARG;
  int rc = msbfs_launch(g, roots, k, d_levels, d_parents);
  if (rc || g->opt.parent_rule != CG_PARENT_FIFO) return rc;
  return fifo_all(g, roots, k, d_levels, d_parents);
}

int cg_msbfs(cg_graph *g, const int64_t *roots, int32_t k, int32_t *levels, int32_t *parents,
             cg_stats *stats) {
  if (!g || !roots || k <= 0) return CG_ERR_INVALID_ARG;
  if (int r = refuse_reordered(g, "cg_msbfs")) return r;
  for (int32_t i = 0; i < k; ++i)
    if (roots[i] < 0 || roots[i] >= g->n) return CG_ERR_INVALID_ARG;
  const int64_t elems = (int64_t)k * g->n;
  // Both outputs page-locked (and the lowest-index rule, whose passes write
  // each output once): the batch's passes store straight into host memory, so
  // the transfer runs with the output pass instead of after it.  Otherwise
  // the batch lands in device buffers and is copied afterwards.
  const bool fifo = g->opt.parent_rule == CG_PARENT_FIFO;
  int32_t *hl = fifo ? nullptr : pinned_device_ptr(levels);
  int32_t *hp = fifo ? nullptr : pinned_device_ptr(parents);
  const bool to_host = hl && hp;
  int rc = msbfs_prepare(g, g->opt.lane_words, to_host ? 0 : elems);
  if (rc) return rc;
  CG_CUDA(cudaEventRecord(g->ev0, g->stream));
  rc = msbfs_launch(g, roots, k, to_host ? hl : g->ms_levels, to_host ? hp : g->ms_parents);
  if (rc) return rc;
  if (fifo && (rc = fifo_all(g, roots, k, g->ms_levels, g->ms_parents))) return rc;
  CG_CUDA(cudaEventRecord(g->ev1, g->stream));
  const size_t bytes = sizeof(int32_t) * (size_t)elems;
  if (levels && !to_host)
    CG_CUDA(cudaMemcpyAsync(levels, g->ms_levels, bytes, cudaMemcpyDeviceToHost, g->stream));
  if (parents && !to_host)
    CG_CUDA(cudaMemcpyAsync(parents, g->ms_parents, bytes, cudaMemcpyDeviceToHost, g->stream));
  cg_stats local;
  CG_CUDA(cudaMemcpyAsync(&local, g->d_stats, sizeof(cg_stats), cudaMemcpyDeviceToHost, g->stream));
  CG_CUDA(cudaStreamSynchronize(g->stream));
  float ms = 0.f;
  cudaEventElapsedTime(&ms, g->ev0, g->ev1);
  local.device_ms = ms;
  if (stats) *stats = local;
  return local.status;
}

int cg_count_edges(cg_graph *g, const int32_t *d_levels, int32_t k, int64_t *m_out) {
  if (!g || !d_levels || k <= 0 || k > 65535 || !m_out) return CG_ERR_INVALID_ARG;
  if (int r = refuse_reordered(g, "cg_count_edges")) return r;
  unsigned long long *d_m = nullptr;
  if (cudaMallocAsync((void **)&d_m, sizeof(unsigned long long) * (size_t)k, g->stream) !=
      cudaSuccess)
    return CG_ERR_OUT_OF_MEMORY;
  int rc = count_edges_launch(g, d_levels, k, d_m);
  if (rc == CG_OK) {
    cudaError_t e = cudaMemcpyAsync(m_out, d_m, sizeof(int64_t) * (size_t)k,
                                    cudaMemcpyDeviceToHost, g->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(g->stream);
    if (e != cudaSuccess) rc = cuda_fail(e, "cg_count_edges");
  }
  cudaFreeAsync(d_m, g->stream);
  cudaStreamSynchronize(g->stream);
  return rc;
}

int cg_host_alloc(void **ptr, int64_t bytes) {
  if (!ptr || bytes <= 0) return CG_ERR_INVALID_ARG;
  if (cudaHostAlloc(ptr, (size_t)bytes, cudaHostAllocDefault) != cudaSuccess) {
    *ptr = nullptr;
    return CG_ERR_OUT_OF_MEMORY;
  }
  return CG_OK;
}

int cg_host_free(void *ptr) {
  if (!ptr) return CG_ERR_INVALID_ARG;
  CG_CUDA(cudaFreeHost(ptr));
  return CG_OK;
}

struct cg_exec {
  cg_graph *g;
  cudaGraph_t graph;
  cudaGraphExec_t exec;
};

int cg_capture_begin(cg_graph *g) {
  if (!g) return CG_ERR_INVALID_ARG;
  CG_CUDA(cudaStreamBeginCapture(g->stream, cudaStreamCaptureModeRelaxed));
  return CG_OK;
}

int cg_capture_end(cg_graph *g, cg_exec **out) {
  if (!g || !out) return CG_ERR_INVALID_ARG;
  *out = nullptr;
  cudaGraph_t graph = nullptr;
  CG_CUDA(cudaStreamEndCapture(g->stream, &graph));
  cudaGraphExec_t exec = nullptr;
  cudaError_t e = cudaGraphInstantiate(&exec, graph, 0);
  if (e != cudaSuccess) {
    cudaGraphDestroy(graph);
    return cuda_fail(e, "cudaGraphInstantiate");
  }
  cg_exec *x = new (std::nothrow) cg_exec{g, graph, exec};
  if (!x) {
    cudaGraphExecDestroy(exec);
    cudaGraphDestroy(graph);
    return CG_ERR_OUT_OF_MEMORY;
  }
  *out = x;
  return CG_OK;
}

int cg_exec_launch(cg_exec *x) {
  if (!x) return CG_ERR_INVALID_ARG;
  CG_CUDA(cudaGraphLaunch(x->exec, x->g->stream));
  return CG_OK;
}

int cg_exec_destroy(cg_exec *x) {
  if (!x) return CG_ERR_INVALID_ARG;
  cudaGraphExecDestroy(x->exec);
  cudaGraphDestroy(x->graph);
  delete x;
  return CG_OK;
}

}  // extern "C"
