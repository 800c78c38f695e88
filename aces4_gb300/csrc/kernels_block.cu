// HBM-bound block kernels: element-wise ops, permute (tensor_block_copy_),
// permuted add/subtract, slice/insert, deterministic dot/norm reductions,
// orbital-energy denominators and the scalar cases of tensor_block_contract_.
//
// Arithmetic follows the reference's operation order with explicit
// round-to-nearest intrinsics (__dmul_rn/__dadd_rn/__dsub_rn), so no multiply
// and add are fused and element-wise results match the reference bit for bit.
#include <algorithm>
#include <cstring>

#include "a4g_internal.h"
#include "exact_fp.h"

namespace a4g {

namespace {

constexpr int kThreads = 256;

int grid_for(int64_t n, int per_thread = 4) {
  const int sms = ctx()->num_sms > 0 ? ctx()->num_sms : 152;
  int64_t want = (n + int64_t(kThreads) * per_thread - 1) / (int64_t(kThreads) * per_thread);
  want = std::max<int64_t>(1, std::min<int64_t>(want, int64_t(sms) * 8));
  return int(want);
}

bool aligned16(const void* p) { return (reinterpret_cast<uintptr_t>(p) & 15) == 0; }

// ---------------------------------------------------------------- element-wise
enum class EwOp { kFill, kScale, kScaleCopy, kIncrement, kAddScaled, kAdd, kAxpy };

template <EwOp OP>
__device__ __forceinline__ double ew(double d, double s, double a) {
  if constexpr (OP == EwOp::kFill) return a;
  else if constexpr (OP == EwOp::kScale) return __dmul_rn(d, a);
  else if constexpr (OP == EwOp::kScaleCopy) return __dmul_rn(s, a);
  else if constexpr (OP == EwOp::kIncrement) return __dadd_rn(d, a);
  else if constexpr (OP == EwOp::kAddScaled) return __dadd_rn(d, __dmul_rn(s, a));
  else if constexpr (OP == EwOp::kAdd) return __dadd_rn(d, s);
  else return fma(a, s, d);  // _gpu_axpy: cuBLAS daxpy semantics
}

template <EwOp OP, bool VEC>
__global__ void __launch_bounds__(kThreads) ew_kernel(double* __restrict__ d,
                                                      const double* __restrict__ s, int64_t n,
                                                      double a) {
  const int64_t stride = int64_t(gridDim.x) * blockDim.x;
  int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  constexpr bool kReadD = !(OP == EwOp::kFill || OP == EwOp::kScaleCopy);
  constexpr bool kReadS = (OP == EwOp::kScaleCopy || OP == EwOp::kAddScaled || OP == EwOp::kAdd ||
                           OP == EwOp::kAxpy);
  if constexpr (VEC) {
    const int64_t n2 = n / 2;
    double2* d2 = reinterpret_cast<double2*>(d);
    const double2* s2 = reinterpret_cast<const double2*>(s);
    for (int64_t k = i; k < n2; k += stride) {
      double2 dv = kReadD ? d2[k] : make_double2(0.0, 0.0);
      double2 sv = kReadS ? __ldg(&s2[k]) : make_double2(0.0, 0.0);
      dv.x = ew<OP>(dv.x, sv.x, a);
      dv.y = ew<OP>(dv.y, sv.y, a);
      d2[k] = dv;
    }
    if (i == 0 && (n & 1)) {
      const int64_t k = n - 1;
      d[k] = ew<OP>(kReadD ? d[k] : 0.0, kReadS ? s[k] : 0.0, a);
    }
  } else {
    for (int64_t k = i; k < n; k += stride) d[k] = ew<OP>(kReadD ? d[k] : 0.0, kReadS ? s[k] : 0.0, a);
  }
}

template <EwOp OP>
int launch_ew(double* d, const double* s, int64_t n, double a, cudaStream_t st) {
  if (n < 0) return fail(A4G_ERR_ARG, "negative element count");
  if (n == 0) return A4G_OK;
  if (!d) return fail(A4G_ERR_ARG, "null block pointer");
  const bool vec = aligned16(d) && (s == nullptr || aligned16(s));
  const int g = grid_for(vec ? n / 2 + 1 : n);
  if (vec) ew_kernel<OP, true><<<g, kThreads, 0, st>>>(d, s, n, a);
  else ew_kernel<OP, false><<<g, kThreads, 0, st>>>(d, s, n, a);
  A4G_CUDA(cudaGetLastError());
  return A4G_OK;
}

// ---------------------------------------------------------------- permute
constexpr int kPermMax = kMaxRank;

struct PermParams {
  int rank;           // after merging
  int a_dim, b_dim;   // input dim 0 (read-contiguous), input dim that is output dim 0
  int ext[kPermMax];  // input-order extents
  int64_t sin[kPermMax], sout[kPermMax];  // strides of each input dim in input / output
  int rest_dims[kPermMax];                // input dims other than a_dim, b_dim
  int n_rest;
  int64_t n_rest_total;
};

// Describes a permute after dropping unit extents and merging runs of input
// dims that stay adjacent and in order in the output (input dim i and i+1 merge
// when their output positions are consecutive).  o2n is 0-based.
void make_perm(int rank, const int* ext, const int* o2n, PermParams* p) {
  int e[kPermMax], o[kPermMax], r = 0;
  for (int i = 0; i < rank; ++i)
    if (ext[i] != 1) {
      e[r] = ext[i];
      o[r] = o2n[i];
      ++r;
    }
  int dense[kPermMax];
  for (int i = 0; i < r; ++i) {
    int c = 0;
    for (int j = 0; j < r; ++j) c += o[j] < o[i];
    dense[i] = c;
  }
  int ge[kPermMax], gpos[kPermMax], m = 0;
  for (int i = 0; i < r; ++i) {
    if (i > 0 && dense[i] == dense[i - 1] + 1) {
      ge[m - 1] *= e[i];
      continue;
    }
    ge[m] = e[i];
    gpos[m] = dense[i];
    ++m;
  }
  int ord[kPermMax];
  for (int i = 0; i < m; ++i) ord[i] = i;
  std::sort(ord, ord + m, [&](int x, int y) { return gpos[x] < gpos[y]; });
  int64_t so = 1;
  for (int q = 0; q < m; ++q) {
    p->sout[ord[q]] = so;
    so *= ge[ord[q]];
  }
  int64_t si = 1;
  for (int i = 0; i < m; ++i) {
    p->ext[i] = ge[i];
    p->sin[i] = si;
    si *= ge[i];
  }
  p->rank = m;
  p->a_dim = 0;
  p->b_dim = m > 0 ? ord[0] : 0;
  p->n_rest = 0;
  p->n_rest_total = 1;
  for (int i = 0; i < m; ++i)
    if (i != p->a_dim && i != p->b_dim) {
      p->rest_dims[p->n_rest++] = i;
      p->n_rest_total *= ge[i];
    }
}

// Element op of the permute family: OP 0 out = r (permute), 1 out = l + r,
// 2 out = l - r (block add/subtract with a permuted right operand).
template <int OP>
__device__ __forceinline__ double perm_op(const double* l, int64_t o, double rv) {
  if constexpr (OP == 0) return rv;
  else if constexpr (OP == 1) return __dadd_rn(l[o], rv);
  else return __dsub_rn(l[o], rv);
}

// Input dim 0 is also output dim 0: runs of dim 0 are contiguous on both
// sides; a block takes several runs and decodes each run's output offset once.
template <int OP>
__global__ void __launch_bounds__(kThreads) perm_direct_kernel(PermParams p, const double* __restrict__ in,
                                                               double* out, const double* l, int64_t nruns,
                                                               int runs_per_block) {
  const int E0 = p.ext[0];
  const int64_t r0 = int64_t(blockIdx.x) * runs_per_block;
  const int64_t r1 = r0 + runs_per_block < nruns ? r0 + runs_per_block : nruns;
  for (int64_t run = r0; run < r1; ++run) {
    int64_t rem = run, base_out = 0;
    for (int q = 1; q < p.rank; ++q) {
      const int64_t x = rem % p.ext[q];
      rem /= p.ext[q];
      base_out += x * p.sout[q];
    }
    const int64_t base_in = run * E0;
    for (int e = threadIdx.x; e < E0; e += blockDim.x)
      out[base_out + e] = perm_op<OP>(l, base_out + e, __ldg(&in[base_in + e]));
  }
}

// Shared-memory tiled transpose between input dim a (contiguous reads) and
// input dim b (contiguous writes); the remaining dims index the grid, several
// of them per block (a block moves 16 KB per slice, so one slice per block
// would be bound by block scheduling, not by HBM).
constexpr int kTile = 32;
template <int OP>
__global__ void __launch_bounds__(kTile * 8) perm_tiled_kernel(PermParams p, const double* __restrict__ in,
                                                               double* out, const double* l,
                                                               int rest_per_block) {
  __shared__ double tile[2][kTile][kTile + 1];
  const int Ea = p.ext[p.a_dim], Eb = p.ext[p.b_dim];
  const int ta = (Ea + kTile - 1) / kTile, tb = (Eb + kTile - 1) / kTile;
  const int64_t tiles = int64_t(ta) * tb;
  const int64_t t = blockIdx.x % tiles;
  const int ia = int(t % ta), ib = int(t / ta);
  const int64_t rest0 = (blockIdx.x / tiles) * rest_per_block;
  const int64_t rest1 = rest0 + rest_per_block < p.n_rest_total ? rest0 + rest_per_block : p.n_rest_total;
  const int tx = threadIdx.x, ty = threadIdx.y;
  const int a0 = ia * kTile, b0 = ib * kTile;
  const int64_t sb_in = p.sin[p.b_dim], sa_out = p.sout[p.a_dim];
  // two slices per iteration: eight loads in flight per thread before the
  // first shared-memory write
  for (int64_t rest = rest0; rest < rest1; rest += 2) {
    int64_t bin[2], bout[2];
    bool have[2];
#pragma unroll
    for (int u = 0; u < 2; ++u) {
      have[u] = rest + u < rest1;
      int64_t rem = rest + u, bi = 0, bo = 0;
      for (int q = 0; q < p.n_rest; ++q) {
        const int d = p.rest_dims[q];
        const int64_t x = rem % p.ext[d];
        rem /= p.ext[d];
        bi += x * p.sin[d];
        bo += x * p.sout[d];
      }
      bin[u] = bi;
      bout[u] = bo;
    }
    double v[2][kTile / 8];
    double lv[2][kTile / 8];  // add/subtract: the left operand at this thread's store positions
#pragma unroll
    for (int u = 0; u < 2; ++u)
#pragma unroll
      for (int k = 0; k < kTile / 8; ++k) {
        const int a = a0 + tx, b = b0 + ty + 8 * k;
        v[u][k] = (have[u] && a < Ea && b < Eb) ? __ldg(&in[bin[u] + a + int64_t(b) * sb_in]) : 0.0;
        if constexpr (OP != 0) {
          const int bs = b0 + tx, as = a0 + ty + 8 * k;
          lv[u][k] = (have[u] && as < Ea && bs < Eb) ? l[bout[u] + bs + int64_t(as) * sa_out] : 0.0;
        }
      }
    __syncthreads();  // the previous iteration's stores have read the tiles
#pragma unroll
    for (int u = 0; u < 2; ++u)
#pragma unroll
      for (int k = 0; k < kTile / 8; ++k) tile[u][ty + 8 * k][tx] = v[u][k];
    __syncthreads();
#pragma unroll
    for (int u = 0; u < 2; ++u) {
      if (!have[u]) continue;
#pragma unroll
      for (int k = 0; k < kTile / 8; ++k) {
        const int b = b0 + tx, a = a0 + ty + 8 * k;
        if (a < Ea && b < Eb) {
          const int64_t o = bout[u] + b + int64_t(a) * sa_out;
          const double rv = tile[u][tx][ty + 8 * k];
          if constexpr (OP == 0) out[o] = rv;
          else out[o] = OP == 1 ? __dadd_rn(lv[u][k], rv) : __dsub_rn(lv[u][k], rv);
        }
      }
    }
  }
}

// Launches the permute family for a described permute (make_perm) of
// `total` elements: OP 0 permute in -> out; 1 / 2: out = l +/- permute(in).
template <int OP>
int launch_perm_op(const PermParams& p, const double* in, double* out, const double* l, int64_t total,
                   cudaStream_t s) {
  const int sms = ctx()->num_sms > 0 ? ctx()->num_sms : 152;
  const int64_t want = int64_t(sms) * 16;  // blocks to aim for
  if (p.rank <= 1 || p.b_dim == p.a_dim) {
    const int E0 = p.rank >= 1 ? p.ext[0] : 1;
    const int64_t nruns = total / E0;
    const int threads = E0 >= kThreads ? kThreads : (E0 + 31) / 32 * 32;
    const int rpb = int(std::max<int64_t>(1, std::min<int64_t>(64, nruns / want)));
    const int64_t blocks = (nruns + rpb - 1) / rpb;
    if (blocks > 0x7fffffffLL) return fail(A4G_ERR_RANGE, "permute grid too large");
    if (blocks > 0) perm_direct_kernel<OP><<<unsigned(blocks), threads, 0, s>>>(p, in, out, l, nruns, rpb);
  } else {
    const int Ea = p.ext[p.a_dim], Eb = p.ext[p.b_dim];
    const int64_t tiles = int64_t((Ea + kTile - 1) / kTile) * ((Eb + kTile - 1) / kTile);
    const int rpb = 2 * int(std::max<int64_t>(1, std::min<int64_t>(8, p.n_rest_total * tiles / (2 * want))));
    const int64_t blocks = tiles * ((p.n_rest_total + rpb - 1) / rpb);
    if (blocks > 0x7fffffffLL) return fail(A4G_ERR_RANGE, "permute grid too large");
    perm_tiled_kernel<OP><<<unsigned(blocks), dim3(kTile, 8), 0, s>>>(p, in, out, l, rpb);
  }
  A4G_CUDA(cudaGetLastError());
  return A4G_OK;
}

// ---------------------------------------------------------------- dot / norm
constexpr int kDotBlocks = 1024;
__global__ void __launch_bounds__(kThreads) dot_partial_kernel(const double* __restrict__ a,
                                                               const double* __restrict__ b,
                                                               const int64_t* __restrict__ offA,
                                                               const int64_t* __restrict__ offB,
                                                               int64_t n, double* partial) {
  double acc = 0.0;
  const int64_t stride = int64_t(gridDim.x) * blockDim.x;
  for (int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += stride) {
    const double x = a[offA ? offA[i] : i];
    const double y = b[offB ? offB[i] : i];
    acc = fma(x, y, acc);
  }
  __shared__ double red[kThreads / 32];
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    double s = 0.0;
    for (int w = 0; w < kThreads / 32; ++w) s += red[w];
    partial[blockIdx.x] = s;
  }
}

__global__ void dot_final_kernel(const double* partial, int np, double* out, int beta) {
  // fixed-order sum of the partials: deterministic for a fixed grid size
  __shared__ double red[kThreads];
  double acc = 0.0;
  for (int i = threadIdx.x; i < np; i += blockDim.x) acc += partial[i];
  red[threadIdx.x] = acc;
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) red[threadIdx.x] += red[threadIdx.x + s];
    __syncthreads();
  }
  if (threadIdx.x == 0) *out = beta ? *out + red[0] : red[0];
}

// ---------------------------------------------------------------- slice/insert
struct SliceParams {
  int rank;
  int sext[kPermMax];
  int64_t tstride[kPermMax];
  int64_t tbase;
};

__global__ void __launch_bounds__(kThreads) slice_insert_kernel(SliceParams p, int insert,
                                                                double* tens, double* slice,
                                                                int64_t n) {
  const int64_t stride = int64_t(gridDim.x) * blockDim.x;
  for (int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += stride) {
    int64_t rem = i, o = p.tbase;
    for (int q = 0; q < p.rank; ++q) {
      const int64_t x = rem % p.sext[q];
      rem /= p.sext[q];
      o += x * p.tstride[q];
    }
    if (insert) tens[o] = slice[i];
    else slice[i] = tens[o];
  }
}

// ---------------------------------------------------------------- denominator
struct DenParams {
  int rank0, rank1, ld1;
  int ext[6];  // extents in storage order
  int off[6];  // first orbital of each storage dimension's segment
  int pos[6];  // storage dimension holding denominator position q
  int poff[6];  // off[pos[q]]: first orbital of the segment at position q
};

// x[k] for a run-time k without indexing a register array (which would put
// it in local memory)
__device__ __forceinline__ int pick6(const int (&x)[6], int k) {
  return k == 0 ? x[0] : k == 1 ? x[1] : k == 2 ? x[2] : k == 3 ? x[3] : k == 4 ? x[4] : x[5];
}

__device__ __forceinline__ double eps_at(const DenParams& p, const double* e, int orb) {
  return p.rank1 == 2 ? e[int64_t(orb) + int64_t(orb) * p.ld1] : e[orb];
}

// Denominator of the element with storage coordinates x, in the reference's
// order of additions (energy_denominator_rhf.F do_rhf_den2/4/6): positions
// 0, 2, 4 are virtual (subtracted), 1, 3, 5 occupied (added).
// div_rn (a / b rounded to the nearest double: integer arithmetic for normal
// operands and results, the FP64 divide otherwise) and nonzero come from
// exact_fp.h.

__device__ __forceinline__ double den_eps(const DenParams& p, const double* e, const int (&x)[6]) {
  const double ea = eps_at(p, e, pick6(x, p.pos[0]) + p.poff[0]);
  const double eb = eps_at(p, e, pick6(x, p.pos[1]) + p.poff[1]);
  if (p.rank0 == 2) return __dsub_rn(eb, ea);  // epsb - epsa
  const double ec = eps_at(p, e, pick6(x, p.pos[2]) + p.poff[2]);
  const double ed = eps_at(p, e, pick6(x, p.pos[3]) + p.poff[3]);
  if (p.rank0 == 4) return __dsub_rn(__dsub_rn(__dadd_rn(eb, ed), ea), ec);  // epsb + epsd - epsa - epsc
  const double e5 = eps_at(p, e, pick6(x, p.pos[4]) + p.poff[4]);
  const double e6 = eps_at(p, e, pick6(x, p.pos[5]) + p.poff[5]);
  return __dsub_rn(__dsub_rn(__dsub_rn(__dadd_rn(__dadd_rn(eb, ed), e6), ea), ec), e5);
}

__device__ __forceinline__ void den_coords(const DenParams& p, int64_t i, int (&x)[6]) {
#pragma unroll
  for (int q = 0; q < 6; ++q) {
    if (q < p.rank0) {
      x[q] = int(i % p.ext[q]);
      i /= p.ext[q];
    } else {
      x[q] = 0;
    }
  }
}

// Four consecutive elements per thread: the coordinates are decoded once
// (64-bit divisions are dear) and stepped along dimension 0 with carries.
constexpr int kDenRun = 4;

__global__ void __launch_bounds__(kThreads) denominator_kernel(DenParams p, double* data,
                                                               const double* __restrict__ e,
                                                               int64_t n) {
  const int64_t stride = int64_t(gridDim.x) * blockDim.x * kDenRun;
  for (int64_t i0 = (int64_t(blockIdx.x) * blockDim.x + threadIdx.x) * kDenRun; i0 < n; i0 += stride) {
    int x[6];
    den_coords(p, i0, x);
    double v[kDenRun];
#pragma unroll
    for (int u = 0; u < kDenRun; ++u) v[u] = i0 + u < n ? data[i0 + u] : 0.0;
#pragma unroll
    for (int u = 0; u < kDenRun; ++u) {
      if (i0 + u >= n) break;
      data[i0 + u] = div_rn(v[u], den_eps(p, e, x));
#pragma unroll
      for (int q = 0; q < 6; ++q) {  // next element: x[0] + 1 with carries
        if (q >= p.rank0) break;
        if (++x[q] < p.ext[q]) break;
        x[q] = 0;
      }
    }
  }
}

// ---------------------------------------------------------------- (T) energy
// The (T)-energy pattern of rccsdpt_aaa.sialx:2163-2172 on one block of W:
// divide by the orbital-energy denominators (energy_denominator_rhf), then
// contract the divided block with the undivided one to a scalar:
//     partial += w(x) * fl(w(x) / eps(x))
// in FP64 throughout: eps summed in the reference's order (do_rhf_den2/4/6:
// the occupied positions 1, 3, 5 added left to right, then the virtual
// positions 0, 2, 4 subtracted), the quotient rounded to nearest exactly as
// the FP64 divide rounds it (div_rn), and the products accumulated in FP64
// (one fused multiply-add per element).  Each CTA writes one partial sum; the
// partials are added in a fixed order, so a GPU gives the same bits every run.

// Deterministic CTA sum of acc into partial[slot].
__device__ __forceinline__ void block_sum_to(double acc, double* partial, int64_t slot) {
  __shared__ double red[32];
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    double sum = 0.0;
    for (int q = 0; q < int(blockDim.x + 31) / 32; ++q) sum += red[q];
    partial[slot] = sum;
  }
}

// Storage in the denominator's order (position q = storage dimension q), rank
// 4 or 6: eps = ((((e1 + e3) + e5) - e0) - e2) - e4, or ((e1 + e3) - e0) - e2.
// The chain's prefix is formed where its terms are fixed: a thread owns one
// (x0, x1) position of the block and a work unit fixes the occupied
// coordinates x3 (and x5), so (e1 + e3) (+ e5) - e0 is formed once per unit,
// - e2 once per x2, and (rank 6) - e4 per element: one FP64 subtraction per
// element instead of five, the same roundings in the same order.  The
// division runs in integer arithmetic (div_rn, the same bits as the FP64
// divide).  (An integer form of the subtraction, exact as well, ran slower
// than the FP64 one.)  Units (x3 [x5], a range of x2) are spread over
// gridDim.y CTAs in a fixed order.
constexpr int kEnLoads = 4;  // loads in flight per thread
constexpr int kEnThreads = 512;
// DIVIDE: the denominator drop-in on the same walk, in place: each element
// becomes fl(w / eps) (zeros included: 0 / eps keeps the IEEE sign), nothing
// is summed.
template <bool DIVIDE>
__global__ void __launch_bounds__(kEnThreads, 2) energy_chain_kernel(DenParams p, double* w,
                                                            const double* __restrict__ e, int x2_per_unit,
                                                            int64_t nunits, double* partial) {
  extern __shared__ double en[];  // e2 energies [ext2], then e4 energies [ext4]
  const int n0 = p.ext[0], n1 = p.ext[1], n2 = p.ext[2], n3 = p.ext[3];
  const bool r6 = p.rank0 == 6;
  const int n4 = r6 ? p.ext[4] : 1;
  for (int t = threadIdx.x; t < n2; t += blockDim.x) en[t] = eps_at(p, e, t + p.off[2]);
  if (r6)
    for (int t = threadIdx.x; t < n4; t += blockDim.x) en[n2 + t] = eps_at(p, e, t + p.off[4]);
  __syncthreads();
  const int64_t n01 = int64_t(n0) * n1;
  const int64_t pp = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  const int x2_chunks = (n2 + x2_per_unit - 1) / x2_per_unit;
  // the energy form only reads w (read-only cache); the divide form writes it
  auto load = [](const double* q) -> double {
    if constexpr (DIVIDE) return *q;
    else return __ldg(q);
  };
  double acc = 0.0;
  if (pp < n01) {
    const int x0 = int(pp % n0), x1 = int(pp / n0);
    const double e1v = eps_at(p, e, x1 + p.off[1]), e0v = eps_at(p, e, x0 + p.off[0]);
    for (int64_t u = blockIdx.y; u < nunits; u += gridDim.y) {
      const int chunk = int(u % x2_chunks);
      const int64_t occ = u / x2_chunks;  // x3 + n3 * x5
      const int x3 = int(occ % n3), x5 = int(occ / n3);
      double t = __dadd_rn(e1v, eps_at(p, e, x3 + p.off[3]));
      if (r6) t = __dadd_rn(t, eps_at(p, e, x5 + p.off[5]));
      t = __dsub_rn(t, e0v);
      const int x2b = chunk * x2_per_unit, x2e = min(n2, x2b + x2_per_unit);
      if (!r6) {
        double* base = w + pp + n01 * (int64_t(n2) * x3);
        for (int x2 = x2b; x2 < x2e; x2 += kEnLoads) {
          double v[kEnLoads];
#pragma unroll
          for (int k = 0; k < kEnLoads; ++k) v[k] = x2 + k < x2e ? load(base + n01 * (x2 + k)) : 0.0;
#pragma unroll
          for (int k = 0; k < kEnLoads; ++k) {
            if constexpr (DIVIDE) {
              if (x2 + k < x2e) base[n01 * (x2 + k)] = div_rn(v[k], __dsub_rn(t, en[x2 + k]));
            } else if (nonzero(v[k])) {
              acc = fma(v[k], div_rn(v[k], __dsub_rn(t, en[x2 + k])), acc);
            }
          }
        }
      } else {
        const int64_t s4 = n01 * int64_t(n2) * n3;  // stride of x4
        for (int x2 = x2b; x2 < x2e; ++x2) {
          const double t2 = __dsub_rn(t, en[x2]);
          double* base = w + pp + n01 * (x2 + int64_t(n2) * x3) + s4 * int64_t(n4) * x5;
          for (int x4 = 0; x4 < n4; x4 += kEnLoads) {
            double v[kEnLoads];
#pragma unroll
            for (int k = 0; k < kEnLoads; ++k) v[k] = x4 + k < n4 ? load(base + s4 * (x4 + k)) : 0.0;
#pragma unroll
            for (int k = 0; k < kEnLoads; ++k) {
              if constexpr (DIVIDE) {
                if (x4 + k < n4) base[s4 * (x4 + k)] = div_rn(v[k], __dsub_rn(t2, en[n2 + x4 + k]));
              } else if (nonzero(v[k])) {
                acc = fma(v[k], div_rn(v[k], __dsub_rn(t2, en[n2 + x4 + k])), acc);
              }
            }
          }
        }
      }
    }
  }
  if constexpr (!DIVIDE) block_sum_to(acc, partial, int64_t(blockIdx.y) * gridDim.x + blockIdx.x);
}

// Any other storage order or rank: the whole chain per element (den_eps, the
// same additions as energy_denominator_rhf), coordinates stepped as in the
// denominator kernel; a fixed grid, one partial per CTA.
__global__ void __launch_bounds__(kThreads) energy_generic_kernel(DenParams p, const double* __restrict__ w,
                                                                  const double* __restrict__ e, int64_t n,
                                                                  double* partial) {
  const int64_t stride = int64_t(gridDim.x) * blockDim.x * kDenRun;
  double acc = 0.0;
  for (int64_t i0 = (int64_t(blockIdx.x) * blockDim.x + threadIdx.x) * kDenRun; i0 < n; i0 += stride) {
    int x[6];
    den_coords(p, i0, x);
    double v[kDenRun];
#pragma unroll
    for (int u = 0; u < kDenRun; ++u) v[u] = i0 + u < n ? __ldg(w + i0 + u) : 0.0;
#pragma unroll
    for (int u = 0; u < kDenRun; ++u) {
      if (i0 + u >= n) break;
      if (nonzero(v[u])) acc = fma(v[u], div_rn(v[u], den_eps(p, e, x)), acc);
#pragma unroll
      for (int q = 0; q < 6; ++q) {
        if (q >= p.rank0) break;
        if (++x[q] < p.ext[q]) break;
        x[q] = 0;
      }
    }
  }
  block_sum_to(acc, partial, blockIdx.x);
}

// ---------------------------------------------------------------- amplitude update
// updatet2 of rlccd_rhf.sialx:557-600 for one block (a,i,b,j), both pardo
// passes fused into one read of the four input blocks:
//   t  = T2new[b,j,a,i] + T2new[a,i,b,j]        (the partner block in its own storage)
//   t1 = T2old[b,j,a,i] + T2old[a,i,b,j]
//   E(a,i,b,j)      = -0.5 * (t1 - t / eps)      (DIIS error vector)
//   T2old'(a,i,b,j) = (0.5 * t) / eps            (next amplitudes, a separate buffer:
//                                                 the partner block still reads T2old)
//   partial[block] = sum of E^2                  (its residual norm, deterministic)
// eps = ((e_i + e_j) - e_a) - e_b, energy_denominator_rhf's rank-4 order.  Each
// CTA handles a 32x32 (a,b) tile at fixed (i,j); the partner tiles are read
// along b and transposed through shared memory so all loads coalesce.
// (0.5 t)/eps is formed as 0.5 (t/eps): both are t/(2 eps) correctly rounded
// while the quotient is a normal number; below that the division is redone.
struct UpdParams {
  int ea, ei, eb, ej;   // extents
  int oa, oi, ob, oj;   // first orbitals
  int rank1, ld1;
};

__device__ __forceinline__ double eps_at_upd(const UpdParams& p, const double* e, int orb) {
  return p.rank1 == 2 ? e[int64_t(orb) + int64_t(orb) * p.ld1] : e[orb];
}

// x / 2 without the FP64 pipe where that is an exponent decrement (normal x
// whose half is normal); the FP64 multiply otherwise (the same bits either way)
__device__ __forceinline__ double half_of(double x) {
  const unsigned long long b = bits_of(x);
  const unsigned f = unsigned(b >> 52) & 0x7FFu;
  return f >= 2u && f != 0x7FFu ? double_of(b - (1ull << 52)) : __dmul_rn(x, 0.5);
}

__global__ void __launch_bounds__(256) update_t2_kernel(UpdParams p, const double* __restrict__ xn,
                                                        const double* __restrict__ xnp,
                                                        const double* __restrict__ xo,
                                                        const double* __restrict__ xop, double* __restrict__ err,
                                                        double* __restrict__ next, const double* __restrict__ e,
                                                        double* partial) {
  __shared__ double pn[32][33], po[32][33];  // [a][b] of the partner tiles
  const int tiles_a = (p.ea + 31) / 32;
  const int ta = blockIdx.x % tiles_a, tb = blockIdx.x / tiles_a;
  const int i = blockIdx.y % p.ei, j = blockIdx.y / p.ei;
  const int a0 = ta * 32, b0 = tb * 32;
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
  // partner block (b,j,a,i): element (b, j, a, i) at b + eb*(j + ej*(a + ea*i))
  for (int k = ty; k < 32; k += 8) {
    const int b = b0 + tx, a = a0 + k;
    double vn = 0.0, vo = 0.0;
    if (a < p.ea && b < p.eb) {
      const int64_t q = b + int64_t(p.eb) * (j + int64_t(p.ej) * (a + int64_t(p.ea) * i));
      vn = __ldg(xnp + q);
      vo = __ldg(xop + q);
    }
    pn[k][tx] = vn;
    po[k][tx] = vo;
  }
  __syncthreads();
  // (e_i + e_j) - e_a once per thread (a is fixed per thread), - e_b per element
  const int a = a0 + tx;
  const double eija = a < p.ea ? __dsub_rn(__dadd_rn(eps_at_upd(p, e, p.oi + i), eps_at_upd(p, e, p.oj + j)),
                                           eps_at_upd(p, e, p.oa + a))
                               : 0.0;
  double acc = 0.0;
  for (int k = ty; k < 32; k += 8) {
    const int b = b0 + k;
    if (a >= p.ea || b >= p.eb) continue;
    const int64_t q = a + int64_t(p.ea) * (i + int64_t(p.ei) * (b + int64_t(p.eb) * j));
    const double t = __dadd_rn(pn[tx][k], __ldg(xn + q));
    const double t1 = __dadd_rn(po[tx][k], __ldg(xo + q));
    const double eps = __dsub_rn(eija, eps_at_upd(p, e, p.ob + b));
    const double td = div_rn(t, eps);
    const double ev = double_of(bits_of(half_of(__dsub_rn(t1, td))) ^ (1ull << 63));  // -0.5 (t1 - td)
    if (err) err[q] = ev;
    next[q] = fabs(td) >= 0x1p-1021 ? half_of(td) : __ddiv_rn(__dmul_rn(t, 0.5), eps);
    acc = fma(ev, ev, acc);
  }
  __shared__ double red[8];
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    double sum = 0.0;
    for (int q = 0; q < 8; ++q) sum += red[q];
    partial[int64_t(blockIdx.y) * gridDim.x + blockIdx.x] = sum;
  }
}

// *out += fixed-order sum of the partials (out may be null: nothing)
__global__ void sum_partials_kernel(const double* partial, int64_t np, double* out) {
  __shared__ double red[kThreads];
  double acc = 0.0;
  for (int64_t q = threadIdx.x; q < np; q += blockDim.x) acc += partial[q];
  red[threadIdx.x] = acc;
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) red[threadIdx.x] += red[threadIdx.x + s];
    __syncthreads();
  }
  if (threadIdx.x == 0 && out) *out = __dadd_rn(*out, red[0]);
}

// *esum += efact * (fixed-order sum of the partials)
__global__ void energy_final_kernel(const double* partial, int np, double efact, double* esum) {
  __shared__ double red[kThreads];
  double acc = 0.0;
  for (int i = threadIdx.x; i < np; i += blockDim.x) acc += partial[i];
  red[threadIdx.x] = acc;
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) red[threadIdx.x] += red[threadIdx.x + s];
    __syncthreads();
  }
  if (threadIdx.x == 0) *esum = __dadd_rn(*esum, __dmul_rn(red[0], efact));
}

// ---------------------------------------------------------------- scalar cases
// tensor_block_contract_ with a rank-0 operand (tensor_dil_omp.F90:770-778):
// the zeroed destination receives tensor*scalar through tensor_block_add_,
// whose factor rule (|s-1| <= 1e-13 means 1) applies; scalar*scalar is a plain
// product.  Results land in D through the destination offsets.
__global__ void __launch_bounds__(kThreads) scalar_case_kernel(
    const double* __restrict__ t, const double* __restrict__ sc, const int64_t* __restrict__ offT,
    const int64_t* __restrict__ offD, double* D, int64_t n, int beta) {
  const double s = *sc;
  const bool unit = fabs(s - 1.0) <= 1e-13;
  const int64_t stride = int64_t(gridDim.x) * blockDim.x;
  for (int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += stride) {
    const double x = t[offT[i]];
    const double v = __dadd_rn(0.0, unit ? x : __dmul_rn(x, s));
    const int64_t o = offD[i];
    D[o] = beta ? __dadd_rn(D[o], v) : v;
  }
}

__global__ void scalar_scalar_kernel(const double* l, const double* r, double* d, int beta) {
  const double v = __dmul_rn(*l, *r);
  *d = beta ? __dadd_rn(*d, v) : v;
}

}  // namespace

// ============================================================== launchers
int launch_fill(double* d, int64_t n, double v, cudaStream_t s) {
  return launch_ew<EwOp::kFill>(d, nullptr, n, v, s);
}
int launch_scale(double* d, int64_t n, double f, cudaStream_t s) {
  return launch_ew<EwOp::kScale>(d, nullptr, n, f, s);
}
int launch_scale_copy(double* d, const double* src, int64_t n, double f, cudaStream_t s) {
  if (!src) return fail(A4G_ERR_ARG, "null source block");
  return launch_ew<EwOp::kScaleCopy>(d, src, n, f, s);
}
int launch_increment(double* d, int64_t n, double delta, cudaStream_t s) {
  return launch_ew<EwOp::kIncrement>(d, nullptr, n, delta, s);
}
int launch_add_scaled(double* t0, const double* t1, int64_t n, double scale, cudaStream_t s) {
  if (!t1) return fail(A4G_ERR_ARG, "null source block");
  if (fabs(scale - 1.0) > 1e-13) return launch_ew<EwOp::kAddScaled>(t0, t1, n, scale, s);
  return launch_ew<EwOp::kAdd>(t0, t1, n, 1.0, s);
}
int launch_axpy(double* y, const double* x, int64_t n, double alpha, cudaStream_t s) {
  if (!x) return fail(A4G_ERR_ARG, "null source block");
  return launch_ew<EwOp::kAxpy>(y, x, n, alpha, s);
}

int launch_permute(int rank, const int* ext, const int* o2n_1based, const double* in, double* out,
                   cudaStream_t s) {
  if (rank < 0 || rank > kMaxRank) return fail(A4G_ERR_ARG, "rank out of range");
  if (!in || !out) return fail(A4G_ERR_ARG, "null block pointer");
  if (rank == 0) {
    A4G_CUDA(cudaMemcpyAsync(out, in, sizeof(double), cudaMemcpyDeviceToDevice, s));
    return A4G_OK;
  }
  int o2n[kPermMax];
  bool seen[kPermMax] = {false};
  int64_t total = 1;
  for (int i = 0; i < rank; ++i) {
    o2n[i] = o2n_1based[i] - 1;
    if (o2n[i] < 0 || o2n[i] >= rank || seen[o2n[i]]) return fail(A4G_ERR_ARG, "invalid permutation");
    seen[o2n[i]] = true;
    if (ext[i] <= 0) return fail(A4G_ERR_ARG, "non-positive extent");
    total *= ext[i];
  }
  PermParams p;
  make_perm(rank, ext, o2n, &p);
  if (p.rank <= 1) {
    A4G_CUDA(cudaMemcpyAsync(out, in, total * sizeof(double), cudaMemcpyDeviceToDevice, s));
    return A4G_OK;
  }
  return launch_perm_op<0>(p, in, out, nullptr, total, s);
}

int launch_add_sub_permuted(int subtract, int rank, const int* r_ext, const int* o2n_1based,
                            double* d, const double* l, const double* r, cudaStream_t s) {
  if (rank < 0 || rank > kMaxRank) return fail(A4G_ERR_ARG, "rank out of range");
  if (!d || !l || !r) return fail(A4G_ERR_ARG, "null block pointer");
  int64_t total = 1;
  int o2n[kPermMax];
  for (int i = 0; i < rank; ++i) {
    total *= r_ext[i];
    o2n[i] = o2n_1based[i] - 1;
  }
  if (total == 0) return A4G_OK;
  PermParams p{};
  if (rank == 0) {
    p.rank = 1;
    p.ext[0] = 1;
    p.sin[0] = p.sout[0] = 1;
  } else {
    make_perm(rank, r_ext, o2n, &p);
  }
  if (p.rank == 0) {  // every extent is 1
    p.rank = 1;
    p.ext[0] = 1;
    p.sin[0] = p.sout[0] = 1;
  }
  return subtract ? launch_perm_op<2>(p, r, d, l, total, s) : launch_perm_op<1>(p, r, d, l, total, s);
}

int dot_scratch_len() { return kDotBlocks; }

int launch_dot(const double* a, const double* b, const int64_t* offA, const int64_t* offB,
               int64_t n, double* d_out, double* d_scratch, int64_t scratch_len, cudaStream_t s) {
  return launch_dot_beta(a, b, offA, offB, n, d_out, d_scratch, scratch_len, 0, s);
}

int launch_dot_beta(const double* a, const double* b, const int64_t* offA, const int64_t* offB,
                    int64_t n, double* d_out, double* d_scratch, int64_t scratch_len, int beta,
                    cudaStream_t s) {
  if (scratch_len < kDotBlocks) return fail(A4G_ERR_ARG, "dot scratch too small");
  const int g = std::min<int>(kDotBlocks, grid_for(n, 8));
  dot_partial_kernel<<<g, kThreads, 0, s>>>(a, b, offA, offB, n, d_scratch);
  dot_final_kernel<<<1, kThreads, 0, s>>>(d_scratch, g, d_out, beta);
  A4G_CUDA(cudaGetLastError());
  return A4G_OK;
}

int launch_slice_insert(int insert, int rank, double* tens, const int* tens_ext, double* slice,
                        const int* slice_ext, const int* ext_beg, cudaStream_t s) {
  if (rank < 0 || rank > kMaxRank) return fail(A4G_ERR_ARG, "rank out of range");
  if (!tens || !slice) return fail(A4G_ERR_ARG, "null block pointer");
  SliceParams p{};
  p.rank = rank;
  int64_t n = 1, st = 1;
  p.tbase = 0;
  for (int q = 0; q < rank; ++q) {
    if (ext_beg[q] < 0 || slice_ext[q] <= 0 || ext_beg[q] + slice_ext[q] > tens_ext[q])
      return fail(A4G_ERR_ARG, "slice outside the block");
    p.sext[q] = slice_ext[q];
    p.tstride[q] = st;
    p.tbase += int64_t(ext_beg[q]) * st;
    st *= tens_ext[q];
    n *= slice_ext[q];
  }
  slice_insert_kernel<<<grid_for(n), kThreads, 0, s>>>(p, insert, tens, slice, n);
  A4G_CUDA(cudaGetLastError());
  return A4G_OK;
}

static DenParams den_params(int rank0, const int* off, const int* ext0, const int* pos, int rank1, int ld1,
                            int64_t* n) {
  DenParams p{};
  p.rank0 = rank0;
  p.rank1 = rank1;
  p.ld1 = ld1;
  *n = 1;
  for (int q = 0; q < rank0; ++q) {
    p.ext[q] = ext0[q];
    p.off[q] = off[q];
    p.pos[q] = pos ? pos[q] : q;
    *n *= ext0[q];
  }
  for (int q = 0; q < rank0; ++q) p.poff[q] = p.off[p.pos[q]];
  return p;
}

// Grid of the chain walk (rank 4 or 6 in the denominator's order): a thread
// per (x0, x1) position (the positions split evenly over gx CTAs of at most
// 512 threads); units (x3 [x5], an x2 range) spread over enough CTAs to fill
// the GPU a few times, at most max_ctas in all.
struct ChainGrid {
  int64_t gx = 0, gy = 0, nunits = 0;
  int threads = 0, per = 0;
  size_t smem = 0;
};
ChainGrid chain_grid(int rank0, const int* ext0, int64_t max_ctas) {
  ChainGrid g;
  const int sms = ctx()->num_sms > 0 ? ctx()->num_sms : 152;
  const int64_t n01 = int64_t(ext0[0]) * ext0[1];
  g.gx = (n01 + kEnThreads - 1) / kEnThreads;
  g.threads = int(((n01 + g.gx - 1) / g.gx + 31) / 32 * 32);
  const int64_t nocc = rank0 == 6 ? int64_t(ext0[3]) * ext0[5] : ext0[3];
  const int64_t want = 16LL * sms;  // CTAs
  const int chunks = int(std::max<int64_t>(1, std::min<int64_t>(ext0[2], (want / g.gx + nocc - 1) / nocc)));
  g.per = (ext0[2] + chunks - 1) / chunks;
  g.nunits = nocc * ((ext0[2] + g.per - 1) / g.per);
  g.gy = std::max<int64_t>(1, std::min<int64_t>({g.nunits, std::max<int64_t>(1, want / g.gx), max_ctas / g.gx}));
  g.smem = size_t(ext0[2] + (rank0 == 6 ? ext0[4] : 0)) * sizeof(double);
  return g;
}

int launch_denominator(int rank0, const int* off, const int* ext0, double* data, int rank1,
                       int ld1, const double* e_or_fock, cudaStream_t s) {
  int64_t n = 0;
  const DenParams p = den_params(rank0, off, ext0, nullptr, rank1, ld1, &n);
  if (n == 0) return A4G_OK;
  if (rank0 == 4 || rank0 == 6) {
    // the chain's prefix formed once per unit: one FP64 subtraction per element
    const ChainGrid g = chain_grid(rank0, ext0, 0x7fffffffLL);
    if (g.smem <= 48 * 1024 && g.gx <= 0x7fffffffLL && g.gy <= 65535) {
      energy_chain_kernel<true><<<dim3(unsigned(g.gx), unsigned(g.gy)), g.threads, g.smem, s>>>(
          p, data, e_or_fock, g.per, g.nunits, nullptr);
      A4G_CUDA(cudaGetLastError());
      return A4G_OK;
    }
  }
  denominator_kernel<<<grid_for((n + kDenRun - 1) / kDenRun), kThreads, 0, s>>>(p, data, e_or_fock, n);
  A4G_CUDA(cudaGetLastError());
  return A4G_OK;
}

int launch_update_t2(const int* off, const int* ext, const double* t2new, const double* t2new_pair,
                     const double* t2old, const double* t2old_pair, double* err, double* next, int rank1, int ld1,
                     const double* e_or_fock, double* norm2, double* d_scratch, int64_t scratch_len,
                     cudaStream_t s) {
  UpdParams p{};
  p.ea = ext[0], p.ei = ext[1], p.eb = ext[2], p.ej = ext[3];
  p.oa = off[0], p.oi = off[1], p.ob = off[2], p.oj = off[3];
  p.rank1 = rank1, p.ld1 = ld1;
  const int64_t gx = int64_t((p.ea + 31) / 32) * ((p.eb + 31) / 32), gy = int64_t(p.ei) * p.ej;
  if (gx * gy == 0) return A4G_OK;
  if (gx > 0x7fffffffLL || gy > 65535) return fail(A4G_ERR_RANGE, "amplitude update: block too large");
  double* partial = d_scratch;
  bool own = false;
  if (gx * gy > scratch_len) {  // more CTAs than the reduction scratch holds
    if (const int rc_ = async_alloc(reinterpret_cast<void**>(&partial), size_t(gx * gy) * sizeof(double), s)) return rc_;
    own = true;
  }
  update_t2_kernel<<<dim3(unsigned(gx), unsigned(gy)), 256, 0, s>>>(p, t2new, t2new_pair, t2old, t2old_pair, err,
                                                                     next, e_or_fock, partial);
  sum_partials_kernel<<<1, kThreads, 0, s>>>(partial, gx * gy, norm2);
  if (own) A4G_CUDA(cudaFreeAsync(partial, s));
  A4G_CUDA(cudaGetLastError());
  return A4G_OK;
}

int launch_energy_contract(int rank0, const int* off, const int* ext0, const int* pos, const double* w,
                           int rank1, int ld1, const double* e_or_fock, double efact, double* esum,
                           double* d_scratch, int scratch_len, cudaStream_t s) {
  int64_t n = 0;
  const DenParams p = den_params(rank0, off, ext0, pos, rank1, ld1, &n);
  if (n == 0) return A4G_OK;
  bool identity = true;
  for (int q = 0; q < rank0; ++q) identity &= p.pos[q] == q;
  const int sms = ctx()->num_sms > 0 ? ctx()->num_sms : 152;
  const int64_t n01 = rank0 >= 2 ? int64_t(ext0[0]) * ext0[1] : n;
  if (identity && (rank0 == 4 || rank0 == 6) && n01 <= kEnThreads * int64_t(scratch_len)) {
    // at most scratch_len partials (one per CTA)
    const ChainGrid g = chain_grid(rank0, ext0, scratch_len);
    if (g.smem > 48 * 1024) return fail(A4G_ERR_RANGE, "energy contraction: segments too large");
    energy_chain_kernel<false><<<dim3(unsigned(g.gx), unsigned(g.gy)), g.threads, g.smem, s>>>(
        p, const_cast<double*>(w), e_or_fock, g.per, g.nunits, d_scratch);
    energy_final_kernel<<<1, kThreads, 0, s>>>(d_scratch, int(g.gx * g.gy), efact, esum);
  } else {
    const int g = int(std::min<int64_t>({int64_t(scratch_len), 8LL * sms,
                                         std::max<int64_t>(1, (n + kThreads * kDenRun - 1) / (kThreads * kDenRun))}));
    energy_generic_kernel<<<g, kThreads, 0, s>>>(p, w, e_or_fock, n, d_scratch);
    energy_final_kernel<<<1, kThreads, 0, s>>>(d_scratch, g, efact, esum);
  }
  A4G_CUDA(cudaGetLastError());
  return A4G_OK;
}

int launch_scalar_cases(const DevPlan* p, const double* L, const double* R, double* D, int beta,
                        double* d_scratch, cudaStream_t s) {
  const GemmPlan& h = p->host;
  switch (h.kind) {
    case ContractKind::kFull:
      return launch_dot_beta(L, R, p->offLk, p->offRk, h.K, D, d_scratch, kDotBlocks, beta, s);
    case ContractKind::kRightScalar:
      scalar_case_kernel<<<grid_for(h.M), kThreads, 0, s>>>(L, R, p->offLm, p->offDm, D, h.M, beta);
      break;
    case ContractKind::kLeftScalar:
      scalar_case_kernel<<<grid_for(h.N), kThreads, 0, s>>>(R, L, p->offRn, p->offDn, D, h.N, beta);
      break;
    case ContractKind::kScalarScalar:
      scalar_scalar_kernel<<<1, 1, 0, s>>>(L, R, D, beta);
      break;
    default:
      return fail(A4G_ERR_ARG, "not a scalar contraction");
  }
  A4G_CUDA(cudaGetLastError());
  return A4G_OK;
}

}  // namespace a4g
