/*
 * ceregraphs.h -- C ABI of the GB300 (sm_103a) BFS engine.
 *
 * This is the drop-in boundary for CereGraphs' on-device BFS.  The reference
 * exposes its kernel through the Cerebras SdkRuntime symbol table of
 * bfs/implementation/src/layout_bool.csl:84-122 (buffers x_bitmap,
 * parent_local_buf, rounds_completed, mat_* ... and the function f_spmv_iter),
 * driven by bfs/scripts/run_graph500.py:248-375 through memcpy_h2d / launch /
 * memcpy_d2h.  Each entry point below names the reference step it replaces.
 *
 * Matrix convention (as in the reference, docs/GRAPH500_BENCHMARK.md:126-128):
 * A[r, c] != 0 means an edge c -> r.  A search from `root` follows out-edges.
 *   in_off / in_idx   = CSR of A: row r lists the sources c of edges c -> r,
 *                       ascending (the reference's A_csr, run_graph500.py:165-168)
 *   out_off / out_idx = CSC of A: column c lists the targets of c, ascending
 *                       (the reference's A_csc, run_graph500.py:185-187);
 *                       pass NULL for a symmetric A.
 *
 * Outputs are int32 per vertex: level (-1 = unreached, root = 0) and parent
 * (-1 = unreached, parent[root] = root), the reference's readback convention
 * (device_io.py:157-205, run_graph500.py:377-380).  The parent of v is the
 * lowest-numbered in-neighbour one level closer to the root (the rule of
 * bfs/README.md:208-224), so results do not depend on scheduling.
 *
 * All functions return 0 (CG_OK) or a positive cg_status code.  A handle is
 * used by one host thread at a time; each handle owns one CUDA stream.
 */
#ifndef CEREGRAPHS_H
#define CEREGRAPHS_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum cg_status {
  CG_OK = 0,
  CG_ERR_INVALID_ARG = 1,   /* bad pointer, size or root (run_graph500.py:111 asserts) */
  CG_ERR_OUT_OF_MEMORY = 2, /* device allocation failed */
  CG_ERR_CUDA = 3,          /* a CUDA runtime call failed; see cg_last_error_string */
  CG_ERR_LEVEL_CAP = 4,     /* the search ran more rounds than the cap allows */
  CG_ERR_TIMEOUT = 5,       /* a device-side wait ran out; the context stays usable */
  CG_ERR_NOT_SUPPORTED = 6, /* e.g. cooperative launch unavailable */
  CG_ERR_ADMISSION = 7,     /* refused: the request does not fit the HBM budget */
  CG_ERR_PARSE = 8,         /* malformed graph file; the line is in cg_last_error_string */
  CG_ERR_IO = 9             /* a graph file could not be read */
} cg_status;

typedef struct cg_graph cg_graph;

/* Direction policy of the per-root search. */
enum {
  CG_DIR_AUTO = 0,          /* direction-optimizing (Beamer): alpha / beta switches */
  CG_DIR_TOPDOWN = 1,       /* push only: what run_graph500.py runs (tau = 0xFFFFFFFF) */
  CG_DIR_BOTTOMUP = 2,      /* pull from round 1 on (round 0 is always push) */
  CG_DIR_TAU = 3            /* one-way switch when nf > tau_switch_count
                               (bool_pe.csl:1078-1088, run_bfs.py:239-243) */
};

/* Graph flags for cg_graph_create. */
enum {
  CG_GRAPH_DEVICE_PTRS = 1, /* the CSR/CSC arrays are device pointers (copied) */
  CG_GRAPH_SYMMETRIC = 2    /* A == A^T: out_off/out_idx are ignored */
};

typedef struct cg_options {
  int32_t direction;        /* CG_DIR_* */
  float alpha;              /* push->pull when frontier edges > unexplored edges / alpha */
  float beta;               /* pull->push when frontier vertices < n / beta (and shrinking) */
  int64_t tau_switch_count; /* CG_DIR_TAU threshold; the reference uses round(0.15 n) */
  int32_t block_size;       /* threads per block of the persistent kernel (multiple of 32) */
  int32_t blocks_per_sm;    /* 0 = as many as fit */
  int32_t level_cap;        /* stop with CG_ERR_LEVEL_CAP after this many rounds (0 = n + 1) */
  int32_t wait_timeout_ms;  /* bound on each grid-wide wait (default 1000) */
  int32_t lane_words;       /* multi-source: 1 = 64 lanes, 2 = 128 lanes per pass */
  float ms_alpha;           /* multi-source: pull when frontier edges > nnz / ms_alpha */
  int32_t test_unmatched_wait; /* test hook: 1 makes the first grid-wide wait wait for an
                                  arrival that never comes, so it must time out */
  int32_t ms_history;       /* multi-source: rounds of frontier history for the output
                               pass (0 = as memory allows, at most 64; < 0 = none: outputs
                               are written during the rounds) */
  int32_t parent_rule;      /* CG_PARENT_LOWEST (default) or CG_PARENT_FIFO */
} cg_options;

/* Parent of a vertex at level L+1 (cg_options.parent_rule):
 *  LOWEST: its lowest-index in-neighbour at level L -- the documented rule of
 *          the reference's kernel (bfs/README.md:208-224);
 *  FIFO:   the in-neighbour scipy's breadth_first_order, the reference's host
 *          check (run_graph500.py:383-395), assigns: the first one dequeued.
 *          A pass after the search (cg_bfs, cg_bfs_device, cg_msbfs,
 *          cg_msbfs_device); it synchronises with the handle's stream, so it is
 *          refused (CG_ERR_NOT_SUPPORTED) while the stream is being captured. */
#define CG_PARENT_LOWEST 0
#define CG_PARENT_FIFO 1

#define CG_HISTORY 64

typedef struct cg_stats {
  int32_t status;           /* cg_status of the device run */
  int32_t rounds;           /* rounds_completed: max level + 1 (bool_pe.csl:989) */
  int64_t visited;          /* vertices reached, root included */
  int32_t pull_rounds;      /* rounds run bottom-up */
  int32_t switches;         /* direction changes */
  float device_ms;          /* device time of the search (CUDA events), 0 if not timed */
  int32_t history_len;      /* min(rounds, CG_HISTORY) */
  int64_t nf_history[CG_HISTORY];      /* new vertices found per round (nf_history) */
  int32_t direction_history[CG_HISTORY]; /* 0 push, 1 pull (direction_history) */
  int64_t round_ns[CG_HISTORY]; /* device time of each round, grid waits included
                                   (the reference's per-round ts_buf, bool_pe.csl:226-285) */
  int64_t setup_ns;             /* state reset + seed, before round 0 */
  int64_t finish_ns;            /* after the last round (output finishing) */
} cg_stats;

/* ---- library ---------------------------------------------------------- */
/* 10000 * major + 100 * minor: 1.1 (10100) added cg_options.parent_rule at the
 * end of cg_options -- a caller with the 1.0 struct must allocate the new size. */
int cg_version(void);
const char *cg_strerror(int status);
/* Text of the last error seen by this thread: a CUDA error, or why a size was
 * rejected (empty if none). */
const char *cg_last_error_string(void);
void cg_default_options(cg_options *opt);

/* ---- Kernel 1: construction ------------------------------------------
 * Replaces the matrix upload of run_graph500.py:284-315 (seven memcpy_h2d
 * of mat_rows/col_idx/col_loc/col_len/local_nnz*) and the 2-D partition of
 * preprocess_bool.py:29-229: the whole CSR (and CSC if directed) becomes
 * device-resident once and serves every later search. */
int cg_graph_create(int64_t n, int64_t nnz, const int64_t *in_off, const int32_t *in_idx,
                    const int64_t *out_off, const int32_t *out_idx, int32_t flags,
                    cg_graph **out);
int cg_graph_destroy(cg_graph *g);
int cg_graph_set_options(cg_graph *g, const cg_options *opt);
int cg_graph_get_options(const cg_graph *g, cg_options *opt);
/* n, nnz, symmetric flag and device bytes held by the handle (graph + state). */
int cg_graph_info(const cg_graph *g, int64_t *n, int64_t *nnz, int32_t *symmetric,
                  int64_t *device_bytes);
/* The handle's CUDA stream (a cudaStream_t), for callers that order work on it. */
void *cg_graph_stream(const cg_graph *g);

/* ---- Kernel 2: one search --------------------------------------------
 * Replaces single_source_seed_pe + memcpy_h2d(x_bitmap) (device_io.py:119-148,
 * run_graph500.py:325-335), launch("f_spmv_iter") (run_graph500.py:339,
 * bool_pe.csl:742-744 and the round loop :673-1161) and memcpy_d2h of
 * parent_local_buf (run_graph500.py:347-358) plus extract_parent_result
 * (device_io.py:160-178).  Host output buffers of n int32 each; either may be
 * NULL.  Blocks until the outputs are in host memory. */
int cg_bfs(cg_graph *g, int64_t root, int32_t *levels, int32_t *parents, cg_stats *stats);

/* Same search with device output pointers (n int32 each, both required),
 * enqueued on the handle's stream; returns without waiting.  Read the
 * outcome with cg_graph_last_stats. */
int cg_bfs_device(cg_graph *g, int64_t root, int32_t *d_levels, int32_t *d_parents);

/* Waits for the handle's stream, then reports the last search's device
 * statistics (rounds_completed, nf_history, direction_history, status). */
int cg_graph_last_stats(cg_graph *g, cg_stats *stats);

/* ---- Kernel 2, batched: k searches in one pass ------------------------
 * Multi-source BFS: roots packed as bit lanes per vertex (64 or 128 lanes a
 * pass, cg_options.lane_words), a boolean SpMM per round.  No reference
 * counterpart as one call: it replaces run_graph500.py:321-440's per-root
 * loop of seed/launch/readback.  Outputs are root-major: levels[i * n + v].
 * Host buffers of k * n int32 each (either may be NULL); blocks.  When both are
 * page-locked (cg_host_alloc) and the parent rule is CG_PARENT_LOWEST, the
 * batch's kernels store the outputs straight into them (the transfer runs
 * during the output pass); otherwise they are copied after the batch. */
int cg_msbfs(cg_graph *g, const int64_t *roots, int32_t k, int32_t *levels, int32_t *parents,
             cg_stats *stats);
/* Device-pointer form (both outputs required), enqueued on the handle's
 * stream.  d_roots is a HOST array of k roots. */
int cg_msbfs_device(cg_graph *g, const int64_t *roots, int32_t k, int32_t *d_levels,
                    int32_t *d_parents);

/* ---- metric ------------------------------------------------------------
 * Graph500 edges traversed per search, compute_m_and_gteps
 * (bfs_timing.py:379-398): symmetric A counts (r, c) with r visited and
 * c <= r; directed A counts entries whose source c is visited.  d_levels are
 * k device arrays of n int32 laid out root-major; m_out receives k counts. */
int cg_count_edges(cg_graph *g, const int32_t *d_levels, int32_t k, int64_t *m_out);

/* ---- CUDA graphs -----------------------------------------------------------
 * Capture the searches enqueued on a handle's stream (cg_bfs_device,
 * cg_msbfs_device) between begin and end into one executable CUDA graph, and
 * replay it with one launch.  The captured searches keep the roots and
 * output pointers they were given.  Refused with CG_ERR_NOT_SUPPORTED while
 * capturing: a handle's first batched search at a lane width (its state is
 * set up with stream synchronisations; run one outside the capture first) and
 * searches under CG_PARENT_FIFO. */
typedef struct cg_exec cg_exec;
int cg_capture_begin(cg_graph *g);
int cg_capture_end(cg_graph *g, cg_exec **out);
int cg_exec_launch(cg_exec *e);
int cg_exec_destroy(cg_exec *e);

/* ---- serving: continuous batching ----------------------------------------
 * A pool keeps up to 64 * lane_words searches in flight on one resident graph,
 * as bit lanes of one resumable batched launch.  cg_pool_admit puts a query
 * (root + device outputs of n int32 each) into a free lane; cg_pool_step runs
 * up to max_rounds rounds for every lane in flight (stop_on_finish: stop after
 * a round in which some lane's search ended), finishes the lanes that ended
 * (their outputs are then complete) and returns them in done (2 words of lane
 * bits) -- queries admitted between steps join the lanes already running.
 * cg_pool_release frees a finished lane.  Every lane's result equals the
 * single-root search (cg_bfs) of its root.  No reference counterpart: this is
 * the query loop around the kernel that run_graph500.py:321-440 runs one root
 * at a time.  CG_ERR_ADMISSION: no free lane. */
typedef struct cg_pool cg_pool;
int cg_pool_create(cg_graph *g, int32_t lane_words, cg_pool **out);
int cg_pool_destroy(cg_pool *pool);
int cg_pool_admit(cg_pool *pool, int64_t root, int32_t *d_levels, int32_t *d_parents,
                  int32_t *lane);
int cg_pool_step(cg_pool *pool, int32_t max_rounds, int32_t stop_on_finish, uint64_t *done,
                 int32_t *next_round);
int cg_pool_release(cg_pool *pool, int32_t lane);
int cg_pool_info(const cg_pool *pool, int32_t *lanes, int32_t *busy);

/* ---- construction on the device -------------------------------------------
 * Synthetic inputs and the edge-list -> CSR/CSC build run on the GPU.
 *
 * cg_rmat_edges: the R-MAT endpoints of datasets/gen_rmat.py:15-44, bit for
 * bit: m = 2^scale * edgefactor pairs (u[e], v[e]) written to device arrays.
 * gen_state = {state_hi, state_lo, inc_hi, inc_lo} of the PCG64 generator
 * that np.random.default_rng(seed) starts from; thresholds = ceil(t * 2^53)
 * for t = A, A+B, A+B+C.  `stream` is a cudaStream_t (NULL = default). */
int cg_rmat_edges(int32_t scale, int64_t m, const uint64_t *gen_state,
                  const uint64_t *thresholds, uint32_t *d_u, uint32_t *d_v, void *stream);
/* floor(r * 2^bits) for the doubles r number first .. first+count-1 of the
 * same generator stream (the directed Erdos-Renyi inputs). */
int cg_uniform_bits(const uint64_t *gen_state, uint64_t first, int64_t count, int32_t bits,
                    uint32_t *d_out, void *stream);

/* Edge-list flags for cg_graph_from_edges. */
enum {
  CG_EDGES_SYMMETRIZE = 1,  /* store both directions (gen_rmat.py:34-36) */
  CG_EDGES_DROP_LOOPS = 2,  /* drop self-loops (gen_rmat.py:37-38) */
  CG_EDGES_DETECT_SYMMETRIC = 4 /* keep one copy when A == A^T (run_graph500.py:179) */
};

/* Kernel 1 from a device edge list src[e] -> dst[e] (entries A[dst, src]):
 * sort, merge duplicates, build the CSR (and the CSC when not symmetrised)
 * on the device and create the handle.  Replaces load_graph + tocsr +
 * sorted_indices + tocsc (run_graph500.py:165-187) for generated inputs. */
int cg_graph_from_edges(int64_t n, int64_t m, const uint32_t *d_src, const uint32_t *d_dst,
                        int32_t flags, cg_graph **out);
/* Copies the resident arrays to host buffers (any may be NULL): CSR offsets
 * (n+1 int64) and indices (nnz int32), CSC likewise. */
int cg_graph_export(const cg_graph *g, int64_t *in_off, int32_t *in_idx, int64_t *out_off,
                    int32_t *out_idx);

/* ---- graph files -----------------------------------------------------------
 * Replaces graph_loader.load_graph (bfs/implementation/graph_loader.py:27-95)
 * with the reference's format detection and direction rule:
 *  - Matrix Market (first line starts with "%%MatrixMarket"), coordinate
 *    storage: entry (i, j), 1-based, is A[i-1, j-1], the edge j-1 -> i-1;
 *    symmetric / skew-symmetric / hermitian storage is mirrored off the
 *    diagonal (scipy.io.mmread); values are ignored (the reference consumes
 *    indptr/indices only); rows must equal cols.
 *  - otherwise a SNAP edge list: "u v" per line (whitespace separated, extra
 *    columns ignored) is the edge u -> v, i.e. A[v, u] (graph_loader.py:78-93);
 *    '#' lines are comments, except that "Nodes: N" in one declares the vertex
 *    count; n = max(N, max id + 1).
 * Compressed files are decompressed by the caller (the Python loader handles
 * .gz and .bz2). */
enum { CG_FORMAT_MTX = 1, CG_FORMAT_EDGELIST = 2 };
typedef struct cg_edge_list {
  int64_t n;             /* vertices */
  int64_t m;             /* edges, symmetric storage expanded, duplicates kept */
  uint32_t *src;         /* host arrays of m, owned by the library */
  uint32_t *dst;
  int32_t format;        /* CG_FORMAT_* */
  int32_t mtx_symmetry;  /* 0 general, 1 symmetric, 2 skew-symmetric, 3 hermitian */
} cg_edge_list;
/* Parses `len` bytes of text with up to `threads` host threads (<= 0: all
 * cores).  Host-only: needs no GPU.  Free the result with cg_edge_list_free. */
int cg_parse_edges(const char *text, int64_t len, int32_t threads, cg_edge_list *out);
int cg_edge_list_free(cg_edge_list *el);
/* Kernel 1 from graph text: parse on the host, then the device build of
 * cg_graph_from_edges with CG_EDGES_DETECT_SYMMETRIC added to `flags`. */
int cg_graph_from_text(const char *text, int64_t len, int32_t flags, cg_graph **out);
/* The same from an uncompressed file (CG_ERR_IO if it cannot be read). */
int cg_graph_load(const char *path, int32_t flags, cg_graph **out);

/* ---- result validation on the device --------------------------------------
 * The Graph500 tree checks for k searches whose levels and parents (k x n,
 * search-major, -1 = unreached) are in device memory, in two passes over the
 * resident graph.  Replaces the per-search host cross-check of
 * run_graph500.py:383-395 and bfs/plots/bfs_tree_plot.py:140-152.  out[i]
 * counts the failing vertices of search i per check, and the lowest one
 * (-1 if none).  Values are treated as untrusted (never dereferenced out of
 * range). */
enum {
  CG_CHECK_ROOT = 0,      /* parent[root] == root, level[root] == 0 */
  CG_CHECK_TREE = 1,      /* reached v != root: level[parent[v]] == level[v] - 1 */
  CG_CHECK_EDGES = 2,     /* edge u -> v, u reached: v reached, level[v] <= level[u] + 1 */
  CG_CHECK_SPAN = 3,      /* level[v] >= 0 exactly when parent[v] >= 0 */
  CG_CHECK_TREE_EDGE = 4, /* parent[v] -> v is an input edge */
  CG_CHECK_LOWEST = 5,    /* parent[v] is the lowest in-neighbour one level up */
  CG_CHECKS = 6
};
typedef struct cg_validation {
  int64_t failures[CG_CHECKS];
  int64_t first[CG_CHECKS];
} cg_validation;
int cg_validate_device(cg_graph *g, const int64_t *roots, int32_t k, const int32_t *d_levels,
                       const int32_t *d_parents, cg_validation *out);

/* ---- degree-aware reordering ----------------------------------------------
 * The one-GPU counterpart of the reference's vertex balancing
 * (util/analyze.cpp:226-372), keeping vertex identity as its --operm option
 * does (util/analyze.cpp:431-437).  cg_graph_reorder builds a second resident
 * handle whose vertices are numbered by descending in-degree (ties by id) --
 * hubs first, vertices without in-edges last -- for locality of the frontier
 * bits and list offsets a search touches.  Each in-list keeps ascending
 * ORIGINAL id order.  Per-root searches on it (cg_bfs, cg_bfs_device and
 * captures of them) take roots in original ids and return levels and parents
 * at original positions with original parent ids, bit-identical to the
 * original handle's (lowest-index rule).  Everything else is refused with
 * CG_ERR_NOT_SUPPORTED on the reordered handle: batched searches, pools, the
 * FIFO parent rule, cg_count_edges, cg_validate_device, cg_graph_export --
 * run those on the original handle.  The original handle stays valid; each
 * is destroyed separately. */
enum { CG_ORDER_DEGREE = 1 };
int cg_graph_reorder(const cg_graph *g, int32_t order, cg_graph **out);

/* ---- one search without any library allocation --------------------------
 * No counterpart in the reference.  For callers that cannot let this library
 * allocate device memory: runtimes that reserve and budget the GPU's memory
 * themselves (a JVM or Go server binding this ABI over JNI/cgo, a framework
 * whose pool owns the device), and loops that cannot afford the device-wide
 * synchronisation a cudaMalloc or cudaFree implies.  The caller passes its own
 * device CSR (and CSC, or NULL for a symmetric A) and device outputs of n
 * int32 each; the search state lives in one fixed __device__ array of this
 * library (about 25 MiB, present on every GPU that loads the library until
 * the process exits).  Nothing is allocated: no cudaMalloc, cudaFree or
 * allocating library routine is called.
 * Limits: n <= CG_NOALLOC_MAX_VERTICES and min(n, nnz / 65 + 1) (the bound on
 * vertices of out-degree > 64) <= CG_NOALLOC_MAX_BIG; larger graphs are
 * rejected with CG_ERR_INVALID_ARG and a message in cg_last_error_string.
 * Every call on a GPU shares the array and it keeps the last call's contents:
 * calls that overlap on that GPU (other streams or threads) race and give
 * wrong results.  The first call on each device computes the grid size; the
 * array's device address is looked up on every call.  Direction policy:
 * Beamer's alpha = 15, beta = 18.  Unlike the handle API it keeps no map of
 * vertices without in-edges, so late pull rounds are a little slower (about
 * 10 us per such round at R-MAT scale 21); results are identical.
 * Outcome of the search (status, rounds, ...):
 *  - stats in pageable memory: the call waits for `stream` and returns the
 *    search's status (CG_ERR_NOT_SUPPORTED, before anything is enqueued, if
 *    the stream is being captured: a wait is not allowed then);
 *  - stats in page-locked memory (cg_host_alloc, cudaHostAlloc,
 *    cudaHostRegister): the call returns CG_OK once the work is queued and the
 *    statistics land in *stats when the stream reaches them -- read
 *    stats->status after synchronising;
 *  - stats == NULL: the call returns once the work is queued and a failed
 *    search (CG_ERR_TIMEOUT, CG_ERR_LEVEL_CAP) is not reported anywhere. */
#define CG_NOALLOC_MAX_VERTICES (1 << 21)
#define CG_NOALLOC_MAX_BIG (1 << 20)
int cg_bfs_noalloc(int64_t n, int64_t nnz, const int64_t *d_in_off, const int32_t *d_in_idx,
                   const int64_t *d_out_off, const int32_t *d_out_idx, int64_t root,
                   int32_t *d_levels, int32_t *d_parents, cg_stats *stats, void *stream);

/* ---- host memory ----------------------------------------------------------
 * Page-locked host buffers, so that the parent/level readback of cg_bfs runs
 * at full link speed (the reference's d2h of parent_local_buf,
 * run_graph500.py:347-358, is part of each search's time). */
int cg_host_alloc(void **ptr, int64_t bytes);
int cg_host_free(void *ptr);

#ifdef __cplusplus
}
#endif
#endif /* CEREGRAPHS_H */
