// Graph files -> edge lists on the host cores, then the device CSR build.
//
// Replaces bfs/implementation/graph_loader.py:27-95 (load_graph: Matrix
// Market through scipy.io.mmread, SNAP edge lists through a Python line loop)
// and the tocsr/tocsc that follows it (run_graph500.py:165-187).  The text is
// cut into pieces at line ends, one host thread parses each piece into its
// own edge arrays, and the pieces are concatenated; sorting, merging
// duplicates and the CSR/CSC come from cg_graph_from_edges on the device.
//
// Direction rule (graph_loader.py:78-93): the reference's matrix is
// row = dst, col = src.  An edge-list line "u v" is the entry A[v, u], the
// edge u -> v; a Matrix Market entry (i, j) is A[i-1, j-1], the edge
// j-1 -> i-1.
#include <cuda_runtime.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <new>
#include <system_error>
#include <thread>
#include <vector>

#include "cg_internal.cuh"

namespace cg {
void set_error_text(const char *text);

namespace {

constexpr int64_t kMaxId = 0x7ffffffeLL;  // vertex ids must fit int32 with n <= 2^31 - 1
constexpr int64_t kMinPiece = 1 << 20;    // bytes of text per thread, at least

enum Symmetry { kGeneral = 0, kSymmetric = 1, kSkew = 2, kHermitian = 3 };

inline bool blank(char c) { return c == ' ' || c == '\t' || c == '\r' || c == '\v' || c == '\f'; }

// End of the line starting at p: the next '\n' or '\r' (Python's universal
// newlines, which the reference's line loop reads with), or e.
inline const char *line_end(const char *p, const char *e) {
  while (p < e && *p != '\n' && *p != '\r') ++p;
  return p;
}

inline char lower(char c) { return (c >= 'A' && c <= 'Z') ? (char)(c - 'A' + 'a') : c; }

// Case-insensitive comparison of [p, e) with a lower-case word.
bool word_is(const char *p, const char *e, const char *w) {
  const size_t n = strlen(w);
  if ((size_t)(e - p) != n) return false;
  for (size_t i = 0; i < n; ++i)
    if (lower(p[i]) != w[i]) return false;
  return true;
}

// Next whitespace-separated token of [*p, e); false when none is left.
bool next_token(const char **p, const char *e, const char **tb, const char **te) {
  const char *q = *p;
  while (q < e && blank(*q)) ++q;
  if (q == e) return false;
  *tb = q;
  while (q < e && !blank(*q)) ++q;
  *te = q;
  *p = q;
  return true;
}

// A decimal integer token with an optional sign.  0 = ok, 1 = not an
// integer, 2 = negative, 3 = too large for a vertex id.
int parse_int(const char *b, const char *e, int64_t *out) {
  bool neg = false;
  if (b < e && (*b == '+' || *b == '-')) {
    neg = *b == '-';
    ++b;
  }
  if (b == e) return 1;
  int64_t v = 0;
  for (const char *q = b; q < e; ++q) {
    if (*q < '0' || *q > '9') return 1;
    v = v * 10 + (*q - '0');
    if (v > (int64_t)1 << 40) return 3;
  }
  if (neg && v != 0) return 2;
  *out = v;
  return 0;
}

struct Piece {
  const char *b = nullptr, *e = nullptr;
  std::vector<uint32_t> src, dst;
  int64_t max_id = -1;      // edge lists: largest id seen
  int64_t declared = -1;    // edge lists: last "Nodes: N" in this piece
  int64_t entries = 0;      // Matrix Market: entries read (before mirroring)
  const char *err_at = nullptr;
  const char *why = nullptr;
  bool oom = false;
};

// "Nodes:" followed by optional blanks and digits anywhere in a comment line
// (graph_loader.py:23 NODES_DECLARED_RE, first match in the line).
bool declared_nodes(const char *b, const char *e, int64_t *n) {
  static const char kKey[] = "Nodes:";
  const size_t kl = sizeof(kKey) - 1;
  for (const char *p = b; p + kl <= e; ++p) {
    if (memcmp(p, kKey, kl) != 0) continue;
    const char *q = p + kl;
    while (q < e && (blank(*q))) ++q;
    const char *d = q;
    int64_t v = 0;
    while (q < e && *q >= '0' && *q <= '9' && v < ((int64_t)1 << 50)) v = v * 10 + (*q++ - '0');
    if (q > d) {
      *n = v;
      return true;
    }
  }
  return false;
}

void parse_edge_list(Piece *pc) {
  const char *p = pc->b;
  while (p < pc->e) {
    const char *eol = line_end(p, pc->e);
    const char *lb = p, *le = eol;
    p = eol + 1;
    while (lb < le && blank(*lb)) ++lb;
    while (le > lb && blank(le[-1])) --le;
    if (lb == le) continue;
    if (*lb == '#') {
      int64_t n = 0;
      if (declared_nodes(lb, le, &n)) pc->declared = n;
      continue;
    }
    const char *q = lb, *ub, *ue, *vb, *ve;
    if (!next_token(&q, le, &ub, &ue) || !next_token(&q, le, &vb, &ve)) {
      pc->err_at = lb;
      pc->why = "expected two vertex ids";
      return;
    }
    int64_t u = 0, v = 0;
    const int ru = parse_int(ub, ue, &u), rv = ru ? ru : parse_int(vb, ve, &v);
    if (ru || rv || u > kMaxId || v > kMaxId) {
      const int r = ru ? ru : rv;
      pc->err_at = lb;
      pc->why = r == 2 ? "negative vertex id" : r == 1 ? "vertex id is not an integer"
                                                       : "vertex id does not fit int32";
      return;
    }
    pc->src.push_back((uint32_t)u);
    pc->dst.push_back((uint32_t)v);
    pc->max_id = std::max(pc->max_id, std::max(u, v));
  }
}

void parse_mtx_entries(Piece *pc, int64_t rows, int64_t cols, int symmetry) {
  const char *p = pc->b;
  while (p < pc->e) {
    const char *eol = line_end(p, pc->e);
    const char *lb = p, *le = eol;
    p = eol + 1;
    while (lb < le && blank(*lb)) ++lb;
    if (lb == le || *lb == '%') continue;
    const char *q = lb, *ib, *ie, *jb, *je;
    if (!next_token(&q, le, &ib, &ie) || !next_token(&q, le, &jb, &je)) {
      pc->err_at = lb;
      pc->why = "expected a row and a column index";
      return;
    }
    int64_t i = 0, j = 0;
    if (parse_int(ib, ie, &i) || parse_int(jb, je, &j) || i < 1 || i > rows || j < 1 ||
        j > cols) {
      pc->err_at = lb;
      pc->why = "index out of range or not an integer";
      return;
    }
    ++pc->entries;
    // A[i-1, j-1]: edge (j-1) -> (i-1)
    pc->src.push_back((uint32_t)(j - 1));
    pc->dst.push_back((uint32_t)(i - 1));
    if (symmetry != kGeneral && i != j) {
      pc->src.push_back((uint32_t)(i - 1));
      pc->dst.push_back((uint32_t)(j - 1));
    }
  }
}

// Splits [b, e) into up to `threads` pieces that end at line ends.
std::vector<Piece> split(const char *b, const char *e, int threads) {
  std::vector<Piece> out;
  const int64_t len = e - b;
  int64_t want = std::max<int64_t>(1, std::min<int64_t>(threads, len / kMinPiece));
  const char *p = b;
  for (int64_t k = 0; k < want && p < e; ++k) {
    const char *q = (k == want - 1) ? e : b + (len * (k + 1)) / want;
    if (q < p) q = p;
    if (q < e) {
      const char *nl = (const char *)memchr(q, '\n', (size_t)(e - q));
      q = nl ? nl + 1 : e;
    }
    Piece pc;
    pc.b = p;
    pc.e = q;
    out.push_back(std::move(pc));
    p = q;
  }
  return out;
}

// Runs f on every piece, one thread each; a piece whose thread cannot be
// started runs on the calling thread.  Host memory running out inside f marks
// the piece instead of escaping the thread.
template <class F>
void run_pieces(std::vector<Piece> &pieces, F f) {
  auto guarded = [&f](Piece *pc) {
    try {
      f(pc);
    } catch (const std::bad_alloc &) {
      pc->oom = true;
    }
  };
  std::vector<std::thread> th;
  size_t started = 1;
  try {
    th.reserve(pieces.size());
    for (; started < pieces.size(); ++started) th.emplace_back(guarded, &pieces[started]);
  } catch (const std::exception &) {
  }
  for (size_t k = started; k < pieces.size(); ++k) guarded(&pieces[k]);
  if (!pieces.empty()) guarded(&pieces[0]);
  for (auto &t : th) t.join();
}

int64_t line_number(const char *text, const char *at) {
  int64_t n = 1;
  for (const char *p = text; p < at; ++p) n += *p == '\n' || (*p == '\r' && p[1] != '\n');
  return n;
}

int fail_at(const char *text, const Piece &pc) {
  char msg[200];
  snprintf(msg, sizeof(msg), "graph text line %lld: %s", (long long)line_number(text, pc.err_at),
           pc.why);
  set_error_text(msg);
  return CG_ERR_PARSE;
}

int fail(const char *why) {
  set_error_text(why);
  return CG_ERR_PARSE;
}

// First error among the pieces (they are in text order), as a status.
int check_pieces(const char *text, const std::vector<Piece> &pieces) {
  for (const auto &pc : pieces) {
    if (pc.oom) {
      set_error_text("host memory while parsing");
      return CG_ERR_OUT_OF_MEMORY;
    }
    if (pc.err_at) return fail_at(text, pc);
  }
  return CG_OK;
}

int gather(std::vector<Piece> &pieces, int64_t n, int format, int symmetry, cg_edge_list *out) {
  int64_t m = 0;
  std::vector<int64_t> at(pieces.size());
  for (size_t k = 0; k < pieces.size(); ++k) {
    at[k] = m;
    m += (int64_t)pieces[k].src.size();
  }
  const size_t bytes = sizeof(uint32_t) * (size_t)(m > 0 ? m : 1);
  uint32_t *src = (uint32_t *)malloc(bytes), *dst = (uint32_t *)malloc(bytes);
  if (!src || !dst) {
    free(src);
    free(dst);
    set_error_text("host memory for the edge list");
    return CG_ERR_OUT_OF_MEMORY;
  }
  Piece *first = pieces.data();
  run_pieces(pieces, [&](Piece *pc) {
    const int64_t o = at[(size_t)(pc - first)];
    if (!pc->src.empty()) {
      memcpy(src + o, pc->src.data(), sizeof(uint32_t) * pc->src.size());
      memcpy(dst + o, pc->dst.data(), sizeof(uint32_t) * pc->dst.size());
    }
    std::vector<uint32_t>().swap(pc->src);
    std::vector<uint32_t>().swap(pc->dst);
  });
  out->n = n;
  out->m = m;
  out->src = src;
  out->dst = dst;
  out->format = format;
  out->mtx_symmetry = symmetry;
  return CG_OK;
}

int parse_mtx(const char *text, const char *end, int threads, cg_edge_list *out) {
  // banner: %%MatrixMarket matrix coordinate <field> <symmetry>
  const char *eol = line_end(text, end);
  const char *q = text + 14, *tb, *te;
  const char *tok[4][2];
  for (int k = 0; k < 4; ++k) {
    if (!next_token(&q, eol, &tb, &te)) return fail("Matrix Market banner: too few fields");
    tok[k][0] = tb;
    tok[k][1] = te;
  }
  if (!word_is(tok[0][0], tok[0][1], "matrix")) return fail("Matrix Market: object is not matrix");
  if (word_is(tok[1][0], tok[1][1], "array")) {
    set_error_text("Matrix Market: dense array storage is not a graph");
    return CG_ERR_NOT_SUPPORTED;
  }
  if (!word_is(tok[1][0], tok[1][1], "coordinate"))
    return fail("Matrix Market: unknown storage format");
  const char *fb = tok[2][0], *fe = tok[2][1];
  if (!word_is(fb, fe, "real") && !word_is(fb, fe, "double") && !word_is(fb, fe, "complex") &&
      !word_is(fb, fe, "integer") && !word_is(fb, fe, "unsigned-integer") &&
      !word_is(fb, fe, "pattern"))
    return fail("Matrix Market: unknown field");
  int symmetry;
  const char *sb = tok[3][0], *se = tok[3][1];
  if (word_is(sb, se, "general"))
    symmetry = kGeneral;
  else if (word_is(sb, se, "symmetric"))
    symmetry = kSymmetric;
  else if (word_is(sb, se, "skew-symmetric"))
    symmetry = kSkew;
  else if (word_is(sb, se, "hermitian"))
    symmetry = kHermitian;
  else
    return fail("Matrix Market: unknown symmetry");
  // comments, then the size line "rows cols entries"
  const char *p = eol < end ? eol + 1 : end;
  int64_t dims[3] = {0, 0, 0};
  bool have_size = false;
  while (p < end && !have_size) {
    const char *le = line_end(p, end);
    const char *lb = p;
    p = le < end ? le + 1 : end;
    while (lb < le && blank(*lb)) ++lb;
    if (lb == le || *lb == '%') continue;
    const char *r = lb;
    for (int k = 0; k < 3; ++k) {
      if (!next_token(&r, le, &tb, &te) || parse_int(tb, te, &dims[k]))
        return fail("Matrix Market: bad size line");
    }
    have_size = true;
  }
  if (!have_size) return fail("Matrix Market: no size line");
  if (dims[0] != dims[1]) return fail("Matrix Market: BFS needs a square matrix");
  if (dims[0] < 1 || dims[0] > kMaxId + 1) return fail("Matrix Market: vertex count out of range");
  std::vector<Piece> pieces = split(p, end, threads);
  const int64_t rows = dims[0], cols = dims[1];
  run_pieces(pieces, [&](Piece *pc) { parse_mtx_entries(pc, rows, cols, symmetry); });
  if (int rc = check_pieces(text, pieces)) return rc;
  int64_t entries = 0;
  for (const auto &pc : pieces) entries += pc.entries;
  if (entries != dims[2]) {
    char msg[160];
    snprintf(msg, sizeof(msg), "Matrix Market: header declares %lld entries, file holds %lld",
             (long long)dims[2], (long long)entries);
    set_error_text(msg);
    return CG_ERR_PARSE;
  }
  return gather(pieces, rows, CG_FORMAT_MTX, symmetry, out);
}

int parse_edge_text(const char *text, const char *end, int threads, cg_edge_list *out) {
  std::vector<Piece> pieces = split(text, end, threads);
  run_pieces(pieces, parse_edge_list);
  if (int rc = check_pieces(text, pieces)) return rc;
  int64_t declared = -1, max_id = -1;
  for (const auto &pc : pieces) {
    if (pc.declared >= 0) declared = pc.declared;  // the last declaration wins
    max_id = std::max(max_id, pc.max_id);
  }
  // graph_loader.py:69-73: n = max(declared or 0, max id + 1)
  const int64_t n = std::max<int64_t>(declared > 0 ? declared : 0, max_id + 1);
  if (n > kMaxId + 1) return fail("edge list: declared vertex count does not fit int32");
  return gather(pieces, n, CG_FORMAT_EDGELIST, kGeneral, out);
}

int hw_threads(int requested) {
  if (requested > 0) return requested;
  const unsigned h = std::thread::hardware_concurrency();
  return h ? (int)std::min(h, 64u) : 4;
}

}  // namespace
}  // namespace cg

using namespace cg;

extern "C" {

int cg_parse_edges(const char *text, int64_t len, int32_t threads, cg_edge_list *out) {
  if (!out || len < 0 || (len > 0 && !text)) return CG_ERR_INVALID_ARG;
  memset(out, 0, sizeof(*out));
  set_error_text("");
  const char *end = text + len;
  try {
    if (len >= 14 && memcmp(text, "%%MatrixMarket", 14) == 0)
      return parse_mtx(text, end, hw_threads(threads), out);
    return parse_edge_text(text, end, hw_threads(threads), out);
  } catch (const std::bad_alloc &) {
    set_error_text("host memory while parsing");
    return CG_ERR_OUT_OF_MEMORY;
  } catch (const std::system_error &) {
    set_error_text("could not start parser threads");
    return CG_ERR_NOT_SUPPORTED;
  }
}

int cg_edge_list_free(cg_edge_list *el) {
  if (!el) return CG_ERR_INVALID_ARG;
  free(el->src);
  free(el->dst);
  el->src = el->dst = nullptr;
  el->m = 0;
  return CG_OK;
}

int cg_graph_from_text(const char *text, int64_t len, int32_t flags, cg_graph **out) {
  if (!out) return CG_ERR_INVALID_ARG;
  *out = nullptr;
  cg_edge_list el;
  int rc = cg_parse_edges(text, len, 0, &el);
  if (rc) return rc;
  if (el.n < 1) {
    cg_edge_list_free(&el);
    set_error_text("graph text holds no vertices");
    return CG_ERR_PARSE;
  }
  uint32_t *d_src = nullptr, *d_dst = nullptr;
  const size_t bytes = sizeof(uint32_t) * (size_t)(el.m > 0 ? el.m : 1);
  do {
    if (cudaMalloc(&d_src, bytes) != cudaSuccess || cudaMalloc(&d_dst, bytes) != cudaSuccess) {
      rc = CG_ERR_OUT_OF_MEMORY;
      break;
    }
    if (el.m > 0) {
      cudaError_t e = cudaMemcpy(d_src, el.src, bytes, cudaMemcpyHostToDevice);
      if (e == cudaSuccess) e = cudaMemcpy(d_dst, el.dst, bytes, cudaMemcpyHostToDevice);
      if (e != cudaSuccess) {
        rc = cuda_fail(e, "edge upload");
        break;
      }
    }
    rc = cg_graph_from_edges(el.n, el.m, d_src, d_dst, flags | CG_EDGES_DETECT_SYMMETRIC, out);
  } while (0);
  cudaFree(d_src);
  cudaFree(d_dst);
  cg_edge_list_free(&el);
  return rc;
}

int cg_graph_load(const char *path, int32_t flags, cg_graph **out) {
  if (!path || !out) return CG_ERR_INVALID_ARG;
  *out = nullptr;
  FILE *f = fopen(path, "rb");
  if (!f) {
    char msg[256];
    snprintf(msg, sizeof(msg), "cannot open %s", path);
    set_error_text(msg);
    return CG_ERR_IO;
  }
  int rc = CG_OK;
  char *buf = nullptr;
  do {
    if (fseek(f, 0, SEEK_END) != 0) { rc = CG_ERR_IO; break; }
    const long size = ftell(f);
    if (size < 0 || fseek(f, 0, SEEK_SET) != 0) { rc = CG_ERR_IO; break; }
    buf = (char *)malloc((size_t)size + 1);
    if (!buf) {
      set_error_text("host memory for the graph file");
      rc = CG_ERR_OUT_OF_MEMORY;
      break;
    }
    if (size > 0 && fread(buf, 1, (size_t)size, f) != (size_t)size) { rc = CG_ERR_IO; break; }
    const unsigned char *u = (const unsigned char *)buf;
    if ((size >= 2 && u[0] == 0x1f && u[1] == 0x8b) ||
        (size >= 3 && u[0] == 'B' && u[1] == 'Z' && u[2] == 'h')) {
      set_error_text("compressed graph file: decompress it first (the Python loader does)");
      rc = CG_ERR_NOT_SUPPORTED;
      break;
    }
    rc = cg_graph_from_text(buf, (int64_t)size, flags, out);
  } while (0);
  if (rc == CG_ERR_IO) set_error_text("graph file read failed");
  free(buf);
  fclose(f);
  return rc;
}

}  // extern "C"
