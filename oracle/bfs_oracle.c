/*
 * ORACLE -- test infrastructure only. Nothing in the ceregraphs_gb300 package
 * links, loads or calls this file; only tests/, __graft_entry__.smoke() and
 * bench.py's CPU-baseline leg do, as the checker.
 *
 * Plain-C restatement of CereGraphs' level-synchronous boolean-semiring BFS
 * (the Cerebras CSL kernel bfs/implementation/src/bool_pe.csl), written for a
 * single address space:
 *
 *   - start_spmv           bool_pe.csl:673-729  visited := seed, parent := NONE,
 *                                               rounds := 0
 *   - compute_topdown      bool_pe.csl:865-887  y = OR_j(A[i,j] AND x[j]) by
 *                                               walking the out-lists of the
 *                                               frontier columns
 *   - reduce_done          bool_pe.csl:947-1004 newly = y & ~visited;
 *                                               visited |= newly; x = newly;
 *                                               nf = popcount(newly)
 *   - termination relay    bool_pe.csl:1048-1100 stop iff nf == 0; rounds
 *                                               counts the empty last round
 *   - parent resolution    bool_pe.csl:1145-1154 + the lowest-global-index rule
 *                          stated in bfs/README.md:208-224: the parent of v is
 *                          the smallest vertex id u with an edge u->v and
 *                          level[u] == level[v] - 1
 *   - output conventions   device_io.py:157-205 and run_graph500.py:377-380:
 *                          parent NONE -> -1, parent[root] = root,
 *                          level[root] = 0, unreached level = -1
 *
 * Matrix convention (docs/GRAPH500_BENCHMARK.md:126-128, graph_loader.py:76-90):
 * A[r, c] != 0 means an edge c -> r.  The arrays handed in here are:
 *   out_off/out_idx : CSC of A  (column c lists the vertices c points to)
 *   in_off/in_idx   : CSR of A  (row r lists the vertices pointing to r),
 *                     sorted ascending within each row
 * For a symmetric graph both pairs are the same arrays.
 *
 * The edge count m follows bfs/implementation/bfs_timing.py:379-398:
 *   symmetric : m = #{(r, c) in A : visited[r] and c <= r}
 *   directed  : m = #{(r, c) in A : visited[c]}
 */
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

/* Level-synchronous BFS from `root`.  Returns the number of rounds the
 * reference kernel would report in rounds_completed (max level + 1, the last
 * round being the one that finds nothing, bool_pe.csl:989 and :1068), or a
 * negative value on bad arguments. */
int64_t oracle_bfs(int64_t n, const int64_t *out_off, const int32_t *out_idx,
                   const int64_t *in_off, const int32_t *in_idx, int64_t root,
                   int32_t *levels, int32_t *parents) {
  if (n <= 0 || root < 0 || root >= n) return -1;
  for (int64_t v = 0; v < n; v++) {
    levels[v] = -1;
    parents[v] = -1;
  }
  int32_t *queue = (int32_t *)malloc(sizeof(int32_t) * (size_t)n);
  if (!queue) return -2;
  int64_t head = 0, tail = 0;
  queue[tail++] = (int32_t)root;
  levels[root] = 0;
  int64_t rounds = 0;
  int32_t level = 0;
  /* one iteration of this loop = one round of f_spmv_iter */
  while (head < tail) {
    int64_t level_end = tail;
    for (int64_t q = head; q < level_end; q++) {
      int32_t u = queue[q];
      for (int64_t e = out_off[u]; e < out_off[u + 1]; e++) {
        int32_t v = out_idx[e];
        if (levels[v] < 0) {
          levels[v] = level + 1;
          queue[tail++] = v;
        }
      }
    }
    head = level_end;
    rounds++;
    level++;
  }
  /* Lowest-index parent among the in-neighbours one level closer.  The
   * in-lists are ascending, so the first hit is the minimum. */
  for (int64_t v = 0; v < n; v++) {
    int32_t lv = levels[v];
    if (lv <= 0) continue;
    for (int64_t e = in_off[v]; e < in_off[v + 1]; e++) {
      int32_t u = in_idx[e];
      if (levels[u] == lv - 1) {
        parents[v] = u;
        break;
      }
    }
  }
  parents[root] = (int32_t)root;
  free(queue);
  return rounds;
}

/* Graph500 m for one search, bfs_timing.py:379-398.  `rows_off/rows_idx` is
 * the CSR of A (row r lists its columns c).  `levels[v] >= 0` marks visited. */
int64_t oracle_count_m(int64_t n, const int64_t *rows_off, const int32_t *rows_idx,
                       const int32_t *levels, int symmetric) {
  int64_t m = 0;
  for (int64_t r = 0; r < n; r++) {
    for (int64_t e = rows_off[r]; e < rows_off[r + 1]; e++) {
      int64_t c = rows_idx[e];
      if (symmetric) {
        if (levels[r] >= 0 && c <= r) m++;
      } else {
        if (levels[c] >= 0) m++;
      }
    }
  }
  return m;
}

/* Multi-source form: k independent searches, outputs laid out root-major
 * (levels[i * n + v]).  By definition each lane equals a single-root search;
 * this is what the batched GPU path has to reproduce bit for bit. */
int64_t oracle_msbfs(int64_t n, const int64_t *out_off, const int32_t *out_idx,
                     const int64_t *in_off, const int32_t *in_idx, const int64_t *roots,
                     int64_t k, int32_t *levels, int32_t *parents) {
  int64_t max_rounds = 0;
  for (int64_t i = 0; i < k; i++) {
    int64_t r = oracle_bfs(n, out_off, out_idx, in_off, in_idx, roots[i], levels + i * n,
                           parents + i * n);
    if (r < 0) return r;
    if (r > max_rounds) max_rounds = r;
  }
  return max_rounds;
}
