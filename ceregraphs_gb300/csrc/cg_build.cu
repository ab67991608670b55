// Kernel-1 construction on the device: synthetic edge generation and the
// edge-list -> CSR/CSC build, so that graphs at scale 23-26 are built in
// seconds instead of the reference's tens of host seconds
// (docs/ERRORS.md:121-136 reports ~20 s for the s17 upload alone).
//
// R-MAT (datasets/gen_rmat.py:15-44) draws one double per edge per level
// from np.random.default_rng(seed) -- a PCG64 stream (128-bit LCG, XSL-RR
// output) consumed level by level, rng.random(m) each.  Each thread here owns
// R consecutive edges: it jumps its generator to the first of them once, draws
// its R doubles of a level, then jumps by m - R to the same edges of the next
// level.  Jump-ahead is Brown's arbitrary-stride LCG method ("Random number
// generation with arbitrary strides", 1994): the affine map s -> a s + c
// applied d times, by square-and-multiply.  A double is (x >> 11) * 2^-53, so
// every quadrant test "r >= t" is done exactly on the 53-bit integer against
// ceil(t * 2^53), computed on the host.
//
// CSR build: one 64-bit key (row << 32 | col) per stored entry, a CUB radix
// sort, CUB unique, and a binary search per row for the offsets.
#include <cuda_runtime.h>
#include <stdint.h>

#include <cub/cub.cuh>
#include <new>

#include "cg_internal.cuh"

namespace cg {

typedef unsigned __int128 u128;

__host__ __device__ __forceinline__ u128 mk128(uint64_t hi, uint64_t lo) {
  return ((u128)hi << 64) | (u128)lo;
}

static constexpr uint64_t kPcgMulHi = 0x2360ED051FC65DA4ull;
static constexpr uint64_t kPcgMulLo = 0x4385DF649FCCF645ull;

struct Affine {  // s -> mul * s + add (mod 2^128)
  u128 mul, add;
};

__host__ __device__ inline Affine lcg_jump(u128 inc, uint64_t delta) {
  u128 cur_mul = mk128(kPcgMulHi, kPcgMulLo), cur_add = inc;
  u128 acc_mul = 1, acc_add = 0;
  while (delta) {
    if (delta & 1) {
      acc_mul *= cur_mul;
      acc_add = acc_add * cur_mul + cur_add;
    }
    cur_add = (cur_mul + 1) * cur_add;
    cur_mul *= cur_mul;
    delta >>= 1;
  }
  return Affine{acc_mul, acc_add};
}

__device__ __forceinline__ uint64_t pcg_next(u128 &s, u128 inc) {
  s = s * mk128(kPcgMulHi, kPcgMulLo) + inc;
  const uint64_t x = (uint64_t)(s >> 64) ^ (uint64_t)s;
  const unsigned rot = (unsigned)(s >> 122);
  return (x >> rot) | (x << ((64u - rot) & 63u));
}

struct RmatParams {
  uint64_t st_hi, st_lo, inc_hi, inc_lo;  // generator state after seeding
  uint64_t t_a, t_ab, t_abc;              // ceil(t * 2^53) of A, A+B, A+B+C
  uint64_t skip_mul_hi, skip_mul_lo, skip_add_hi, skip_add_lo;  // jump by m - R
  int64_t m;
  int scale;
};

template <int R>
__global__ void rmat_kernel(RmatParams p, uint32_t *__restrict__ u_out,
                            uint32_t *__restrict__ v_out) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t e0 = t * R;
  if (e0 >= p.m) return;
  const u128 inc = mk128(p.inc_hi, p.inc_lo);
  const int64_t cnt = (p.m - e0) < R ? (p.m - e0) : R;
  Affine j0 = lcg_jump(inc, (uint64_t)e0);
  u128 s = j0.mul * mk128(p.st_hi, p.st_lo) + j0.add;
  Affine skip;
  if (cnt == R)
    skip = Affine{mk128(p.skip_mul_hi, p.skip_mul_lo), mk128(p.skip_add_hi, p.skip_add_lo)};
  else
    skip = lcg_jump(inc, (uint64_t)(p.m - cnt));
  uint32_t u[R], v[R];
#pragma unroll
  for (int j = 0; j < R; ++j) u[j] = v[j] = 0;
  for (int level = 0; level < p.scale; ++level) {
    const uint32_t bit = 1u << (p.scale - 1 - level);
#pragma unroll
    for (int j = 0; j < R; ++j) {
      if (j < cnt) {
        const uint64_t k = pcg_next(s, inc) >> 11;
        const bool ub = k >= p.t_ab;
        const bool vb = (k >= p.t_a && k < p.t_ab) || k >= p.t_abc;
        u[j] |= ub ? bit : 0u;
        v[j] |= vb ? bit : 0u;
      }
    }
    s = skip.mul * s + skip.add;
  }
#pragma unroll
  for (int j = 0; j < R; ++j)
    if (j < cnt) {
      u_out[e0 + j] = u[j];
      v_out[e0 + j] = v[j];
    }
}

// k-th double of the stream -> floor(r * 2^bits), k = first + e
__global__ void uniform_bits_kernel(uint64_t st_hi, uint64_t st_lo, uint64_t inc_hi,
                                    uint64_t inc_lo, uint64_t first, int64_t count, int bits,
                                    uint32_t *__restrict__ out) {
  constexpr int R = 16;
  const int64_t e0 = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) * R;
  if (e0 >= count) return;
  const u128 inc = mk128(inc_hi, inc_lo);
  Affine j0 = lcg_jump(inc, first + (uint64_t)e0);
  u128 s = j0.mul * mk128(st_hi, st_lo) + j0.add;
  for (int j = 0; j < R && e0 + j < count; ++j)
    out[e0 + j] = (uint32_t)((pcg_next(s, inc) >> 11) >> (53 - bits));
}

// one key per stored entry: row = dst, col = src (A[dst, src] = edge src -> dst)
__global__ void edge_keys_kernel(int64_t m, const uint32_t *__restrict__ src,
                                 const uint32_t *__restrict__ dst, int symmetrize,
                                 int drop_loops, uint64_t sentinel, uint64_t *__restrict__ keys) {
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < m;
       e += (int64_t)gridDim.x * blockDim.x) {
    const uint64_t s = src[e], d = dst[e];
    const bool loop = drop_loops && s == d;
    keys[e] = loop ? sentinel : ((d << 32) | s);
    if (symmetrize) keys[m + e] = loop ? sentinel : ((s << 32) | d);
  }
}

__global__ void swap_halves_kernel(int64_t nnz, const uint64_t *__restrict__ in,
                                   uint64_t *__restrict__ out) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < nnz;
       i += (int64_t)gridDim.x * blockDim.x) {
    const uint64_t k = in[i];
    out[i] = (k << 32) | (k >> 32);
  }
}

__global__ void csr_from_keys_kernel(int64_t n, int64_t nnz, const uint64_t *__restrict__ keys,
                                     int64_t *__restrict__ off, int32_t *__restrict__ idx) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  const int64_t t0 = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  for (int64_t i = t0; i < nnz; i += stride) idx[i] = (int32_t)(keys[i] & 0xffffffffull);
  for (int64_t r = t0; r <= n; r += stride) {
    const uint64_t target = (uint64_t)r << 32;
    int64_t lo = 0, hi = nnz;
    while (lo < hi) {
      const int64_t mid = (lo + hi) >> 1;
      if (keys[mid] < target)
        lo = mid + 1;
      else
        hi = mid;
    }
    off[r] = lo;
  }
}

// A == A^T exactly when the CSR and the CSC of the same entries coincide.
__global__ void same_arrays_kernel(int64_t n, int64_t nnz, const int64_t *__restrict__ a_off,
                                   const int32_t *__restrict__ a_idx,
                                   const int64_t *__restrict__ b_off,
                                   const int32_t *__restrict__ b_idx, unsigned *differ) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  const int64_t t0 = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  bool d = false;
  for (int64_t i = t0; i < nnz; i += stride) d |= a_idx[i] != b_idx[i];
  for (int64_t r = t0; r <= n; r += stride) d |= a_off[r] != b_off[r];
  if (__any_sync(0xffffffffu, d) && (threadIdx.x & 31) == 0) atomicOr(differ, 1u);
}

static int grid_for(int64_t work, int num_sms) {
  int64_t b = (work + 255) / 256;
  const int64_t cap = (int64_t)num_sms * 32;
  if (b > cap) b = cap;
  if (b < 1) b = 1;
  return (int)b;
}

// Sorts `count` keys in place (using `tmp` of the same size), removes
// duplicates and sentinel keys; returns the number kept in *kept and the
// buffer holding them in *result (keys or tmp).
static int sort_unique(uint64_t *keys, uint64_t *tmp, int64_t count, int end_bit,
                       uint64_t sentinel, cudaStream_t stream, uint64_t **result,
                       int64_t *kept) {
  size_t tb_sort = 0, tb_uniq = 0;
  cub::DoubleBuffer<uint64_t> db(keys, tmp);
  CG_CUDA(cub::DeviceRadixSort::SortKeys(nullptr, tb_sort, db, count, 0, end_bit, stream));
  int64_t *d_num = nullptr;
  CG_CUDA(cub::DeviceSelect::Unique(nullptr, tb_uniq, keys, tmp, d_num, count, stream));
  size_t tb = tb_sort > tb_uniq ? tb_sort : tb_uniq;
  void *temp = nullptr;
  if (cudaMallocAsync(&temp, tb + 16, stream) != cudaSuccess) return CG_ERR_OUT_OF_MEMORY;
  if (cudaMallocAsync((void **)&d_num, sizeof(int64_t), stream) != cudaSuccess) {
    cudaFreeAsync(temp, stream);
    return CG_ERR_OUT_OF_MEMORY;
  }
  int rc = CG_OK;
  do {
    cudaError_t e = cub::DeviceRadixSort::SortKeys(temp, tb_sort, db, count, 0, end_bit, stream);
    if (e != cudaSuccess) { rc = cuda_fail(e, "SortKeys"); break; }
    uint64_t *sorted = db.Current();
    uint64_t *other = db.Alternate();
    e = cub::DeviceSelect::Unique(temp, tb_uniq, sorted, other, d_num, count, stream);
    if (e != cudaSuccess) { rc = cuda_fail(e, "Unique"); break; }
    int64_t nu = 0;
    e = cudaMemcpyAsync(&nu, d_num, sizeof(int64_t), cudaMemcpyDeviceToHost, stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(stream);
    if (e != cudaSuccess) { rc = cuda_fail(e, "Unique count"); break; }
    if (nu > 0) {
      uint64_t last = 0;
      e = cudaMemcpyAsync(&last, other + nu - 1, sizeof(uint64_t), cudaMemcpyDeviceToHost, stream);
      if (e == cudaSuccess) e = cudaStreamSynchronize(stream);
      if (e != cudaSuccess) { rc = cuda_fail(e, "Unique last"); break; }
      if (last == sentinel) --nu;
    }
    *result = other;
    *kept = nu;
  } while (0);
  cudaFreeAsync(temp, stream);
  cudaFreeAsync(d_num, stream);
  return rc;
}

}  // namespace cg

using namespace cg;

extern "C" {

int cg_rmat_edges(int32_t scale, int64_t m, const uint64_t *gen_state,
                  const uint64_t *thresholds, uint32_t *d_u, uint32_t *d_v, void *stream) {
  if (scale < 1 || scale > 31 || m <= 0 || !gen_state || !thresholds || !d_u || !d_v)
    return CG_ERR_INVALID_ARG;
  constexpr int R = 16;
  RmatParams p;
  p.st_hi = gen_state[0];
  p.st_lo = gen_state[1];
  p.inc_hi = gen_state[2];
  p.inc_lo = gen_state[3];
  p.t_a = thresholds[0];
  p.t_ab = thresholds[1];
  p.t_abc = thresholds[2];
  const Affine skip = lcg_jump(mk128(p.inc_hi, p.inc_lo), (uint64_t)(m - R));
  p.skip_mul_hi = (uint64_t)(skip.mul >> 64);
  p.skip_mul_lo = (uint64_t)skip.mul;
  p.skip_add_hi = (uint64_t)(skip.add >> 64);
  p.skip_add_lo = (uint64_t)skip.add;
  p.m = m;
  p.scale = scale;
  const int64_t threads = (m + R - 1) / R;
  const int block = 128;
  rmat_kernel<R><<<(unsigned)((threads + block - 1) / block), block, 0, (cudaStream_t)stream>>>(
      p, d_u, d_v);
  CG_CUDA(cudaGetLastError());
  return CG_OK;
}

int cg_uniform_bits(const uint64_t *gen_state, uint64_t first, int64_t count, int32_t bits,
                    uint32_t *d_out, void *stream) {
  if (!gen_state || count <= 0 || bits < 1 || bits > 32 || !d_out) return CG_ERR_INVALID_ARG;
  const int64_t threads = (count + 15) / 16;
  uniform_bits_kernel<<<(unsigned)((threads + 127) / 128), 128, 0, (cudaStream_t)stream>>>(
      gen_state[0], gen_state[1], gen_state[2], gen_state[3], first, count, bits, d_out);
  CG_CUDA(cudaGetLastError());
  return CG_OK;
}

int cg_graph_from_edges(int64_t n, int64_t m, const uint32_t *d_src, const uint32_t *d_dst,
                        int32_t flags, cg_graph **out) {
  if (!out || n <= 0 || n > 0x7fffffffLL || m < 0 || (m > 0 && (!d_src || !d_dst)))
    return CG_ERR_INVALID_ARG;
  *out = nullptr;
  const bool sym = (flags & CG_EDGES_SYMMETRIZE) != 0;
  const bool drop = (flags & CG_EDGES_DROP_LOOPS) != 0;
  const bool detect = (flags & CG_EDGES_DETECT_SYMMETRIC) != 0;
  bool found_sym = false;
  int dev = 0, sms = 0;
  CG_CUDA(cudaGetDevice(&dev));
  CG_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  cudaStream_t st = nullptr;
  CG_CUDA(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
  const int64_t count = sym ? 2 * m : m;
  const uint64_t sentinel = (uint64_t)n << 32;
  int end_bit = 33;
  while ((1ll << (end_bit - 32)) <= n) ++end_bit;
  uint64_t *keys = nullptr, *tmp = nullptr, *res = nullptr;
  int64_t *in_off = nullptr, *out_off = nullptr;
  int32_t *in_idx = nullptr, *out_idx = nullptr;
  int64_t nnz = 0;
  int rc = CG_OK;
  do {
    const size_t kb = sizeof(uint64_t) * (size_t)(count > 0 ? count : 1);
    if (cudaMalloc(&keys, kb) != cudaSuccess || cudaMalloc(&tmp, kb) != cudaSuccess) {
      rc = CG_ERR_OUT_OF_MEMORY;
      break;
    }
    if (count > 0) {
      edge_keys_kernel<<<grid_for(m, sms), 256, 0, st>>>(m, d_src, d_dst, sym ? 1 : 0,
                                                         drop ? 1 : 0, sentinel, keys);
      cudaError_t e = cudaGetLastError();
      if (e != cudaSuccess) { rc = cuda_fail(e, "edge_keys"); break; }
      rc = sort_unique(keys, tmp, count, end_bit, sentinel, st, &res, &nnz);
      if (rc) break;
    }
    if (cudaMalloc(&in_off, sizeof(int64_t) * (size_t)(n + 1)) != cudaSuccess ||
        cudaMalloc(&in_idx, sizeof(int32_t) * (size_t)(nnz > 0 ? nnz : 1)) != cudaSuccess) {
      rc = CG_ERR_OUT_OF_MEMORY;
      break;
    }
    if (count > 0) {
      csr_from_keys_kernel<<<grid_for(nnz > n ? nnz : n + 1, sms), 256, 0, st>>>(n, nnz, res,
                                                                                in_off, in_idx);
    } else {
      cudaMemsetAsync(in_off, 0, sizeof(int64_t) * (size_t)(n + 1), st);
    }
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) { rc = cuda_fail(e, "csr_from_keys"); break; }
    if (!sym && nnz > 0) {
      // CSC of A: the same entries keyed (col, row)
      uint64_t *other = res == keys ? tmp : keys;
      swap_halves_kernel<<<grid_for(nnz, sms), 256, 0, st>>>(nnz, res, other);
      uint64_t *res2 = nullptr;
      int64_t nnz2 = 0;
      rc = sort_unique(other, res, nnz, 64, ~0ull, st, &res2, &nnz2);
      if (rc) break;
      if (cudaMalloc(&out_off, sizeof(int64_t) * (size_t)(n + 1)) != cudaSuccess ||
          cudaMalloc(&out_idx, sizeof(int32_t) * (size_t)nnz) != cudaSuccess) {
        rc = CG_ERR_OUT_OF_MEMORY;
        break;
      }
      csr_from_keys_kernel<<<grid_for(nnz > n ? nnz : n + 1, sms), 256, 0, st>>>(n, nnz2, res2,
                                                                                out_off, out_idx);
      e = cudaGetLastError();
      if (e != cudaSuccess) { rc = cuda_fail(e, "csc_from_keys"); break; }
      if (detect) {
        // the key buffers are free now: borrow one word of `keys` for the flag
        unsigned *differ = reinterpret_cast<unsigned *>(keys);
        e = cudaMemsetAsync(differ, 0, sizeof(unsigned), st);
        if (e == cudaSuccess) {
          same_arrays_kernel<<<grid_for(nnz > n ? nnz : n + 1, sms), 256, 0, st>>>(
              n, nnz, in_off, in_idx, out_off, out_idx, differ);
          e = cudaGetLastError();
        }
        unsigned h_differ = 1u;
        if (e == cudaSuccess)
          e = cudaMemcpyAsync(&h_differ, differ, sizeof(unsigned), cudaMemcpyDeviceToHost, st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(st);
        if (e != cudaSuccess) { rc = cuda_fail(e, "symmetry check"); break; }
        found_sym = h_differ == 0u;
      }
    }
    e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) { rc = cuda_fail(e, "cg_graph_from_edges"); break; }
    cudaFree(keys);
    cudaFree(tmp);
    keys = tmp = nullptr;
    const bool out_sym = sym || nnz == 0 || found_sym;
    rc = cg_graph_create(n, nnz, in_off, in_idx, out_sym ? nullptr : out_off,
                         out_sym ? nullptr : out_idx,
                         CG_GRAPH_DEVICE_PTRS | (out_sym ? CG_GRAPH_SYMMETRIC : 0), out);
  } while (0);
  cudaFree(keys);
  cudaFree(tmp);
  cudaFree(in_off);
  cudaFree(in_idx);
  cudaFree(out_off);
  cudaFree(out_idx);
  cudaStreamDestroy(st);
  return rc;
}

int cg_graph_export(const cg_graph *g, int64_t *in_off, int32_t *in_idx, int64_t *out_off,
                    int32_t *out_idx) {
  if (g) {
    if (int r = refuse_reordered(g, "cg_graph_export")) return r;
  }
  if (!g) return CG_ERR_INVALID_ARG;
  const size_t ob = sizeof(int64_t) * (size_t)(g->n + 1), ib = sizeof(int32_t) * (size_t)g->nnz;
  if (in_off) CG_CUDA(cudaMemcpyAsync(in_off, g->in_off, ob, cudaMemcpyDeviceToHost, g->stream));
  if (in_idx && ib)
    CG_CUDA(cudaMemcpyAsync(in_idx, g->in_idx, ib, cudaMemcpyDeviceToHost, g->stream));
  if (out_off)
    CG_CUDA(cudaMemcpyAsync(out_off, g->out_off, ob, cudaMemcpyDeviceToHost, g->stream));
  if (out_idx && ib)
    CG_CUDA(cudaMemcpyAsync(out_idx, g->out_idx, ib, cudaMemcpyDeviceToHost, g->stream));
  CG_CUDA(cudaStreamSynchronize(g->stream));
  return CG_OK;
}

}  // extern "C"
