// Plain FP64 block contraction on the FP64 tensor path (DMMA, mma.sync f64),
// with the operand and result permutes folded into the tile loads/stores.
//
// Matrix view (planner):  D[offDm[m]+offDn[n]] (=|+=) sum_k L[offLm[m]+offLk[k]] * R[offRk[k]+offRn[n]]
// so no transposed copy of L, R or D is ever written (the reference allocates
// and fills transposed temporaries, tensor_dil_omp.F90:729-751, 782-785).
//
// CTA tile 64x64, k-step 16, 128 threads (2x2 warps, 32x32 per warp = 4x4
// m8n8k4 DMMA tiles).  Tiles are gathered through the offset tables into
// registers, then staged in double-buffered shared memory.  FP64 throughput on
// GB300 is ~2 FMA/clk/SM, so the kernel is bound by the FP64 pipe; the gather
// traffic is small in comparison.
#include "a4g_internal.h"

namespace a4g {
namespace {

constexpr int BM = 64, BN = 64, BK = 16, LDS = BM + 4;  // +4 doubles: conflict-free fragment reads
constexpr int kThreadsF64 = 128;

__device__ __forceinline__ void dmma_8x8x4(double (&c)[2], double a, double b) {
  asm volatile("mma.sync.aligned.m8n8k4.row.col.f64.f64.f64.f64 {%0,%1}, {%2}, {%3}, {%0,%1};\n"
               : "+d"(c[0]), "+d"(c[1])
               : "d"(a), "d"(b));
}

// Gathers one BMxBK (or BKxBN) operand tile into 8 registers per thread.
// KFAST: the operand is unit-stride along k, so threads walk k fastest.
template <bool KFAST>
__device__ __forceinline__ void gather_tile(double (&reg)[8], const double* __restrict__ X,
                                            const int64_t* __restrict__ offRow,  // per m (or n), smem
                                            const int64_t* __restrict__ offK,    // global, per k
                                            int row0, int rows, int k0, int K) {
  const int t = threadIdx.x;
#pragma unroll
  for (int i = 0; i < 8; ++i) {
    int r, kk;
    if (KFAST) {
      kk = t & (BK - 1);
      r = (t >> 4) + 8 * i;
    } else {
      r = t & (BM - 1);
      kk = (t >> 6) + 2 * i;
    }
    const int k = k0 + kk;
    reg[i] = (row0 + r < rows && k < K) ? __ldg(&X[offRow[r] + __ldg(&offK[k])]) : 0.0;
  }
}

template <bool KFAST>
__device__ __forceinline__ void store_tile(double (*S)[LDS], const double (&reg)[8]) {
  const int t = threadIdx.x;
#pragma unroll
  for (int i = 0; i < 8; ++i) {
    int r, kk;
    if (KFAST) {
      kk = t & (BK - 1);
      r = (t >> 4) + 8 * i;
    } else {
      r = t & (BM - 1);
      kk = (t >> 6) + 2 * i;
    }
    S[kk][r] = reg[i];
  }
}

template <bool A_KFAST, bool B_KFAST>
__global__ void __launch_bounds__(kThreadsF64) contract_f64_kernel(
    const double* __restrict__ L, const double* __restrict__ R, double* __restrict__ D,
    const int64_t* __restrict__ offLm, const int64_t* __restrict__ offLk,
    const int64_t* __restrict__ offRk, const int64_t* __restrict__ offRn,
    const int64_t* __restrict__ offDm, const int64_t* __restrict__ offDn, int M, int N, int K,
    int tiles_m, int beta) {
  __shared__ __align__(16) double As[2][BK][LDS];
  __shared__ __align__(16) double Bs[2][BK][LDS];
  __shared__ int64_t sLm[BM], sRn[BN];

  const int tm = blockIdx.x % tiles_m, tn = blockIdx.x / tiles_m;
  const int m0 = tm * BM, n0 = tn * BN;
  const int t = threadIdx.x;
  if (t < BM) sLm[t] = (m0 + t < M) ? offLm[m0 + t] : 0;
  else sRn[t - BM] = (n0 + t - BM < N) ? offRn[n0 + t - BM] : 0;
  __syncthreads();

  const int warp = t >> 5, lane = t & 31;
  const int g = lane >> 2, tig = lane & 3;
  const int wm = (warp & 1) * 32, wn = (warp >> 1) * 32;

  double acc[4][4][2];
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) acc[i][j][0] = acc[i][j][1] = 0.0;

  double ra[8], rb[8];
  const int ksteps = (K + BK - 1) / BK;
  gather_tile<A_KFAST>(ra, L, sLm, offLk, m0, M, 0, K);
  gather_tile<B_KFAST>(rb, R, sRn, offRk, n0, N, 0, K);
  store_tile<A_KFAST>(As[0], ra);
  store_tile<B_KFAST>(Bs[0], rb);
  __syncthreads();

  for (int ks = 0; ks < ksteps; ++ks) {
    const int cur = ks & 1;
    if (ks + 1 < ksteps) {
      gather_tile<A_KFAST>(ra, L, sLm, offLk, m0, M, (ks + 1) * BK, K);
      gather_tile<B_KFAST>(rb, R, sRn, offRk, n0, N, (ks + 1) * BK, K);
    }
#pragma unroll
    for (int kk = 0; kk < BK; kk += 4) {
      double af[4], bf[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) af[i] = As[cur][kk + tig][wm + i * 8 + g];
#pragma unroll
      for (int j = 0; j < 4; ++j) bf[j] = Bs[cur][kk + tig][wn + j * 8 + g];
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) dmma_8x8x4(acc[i][j], af[i], bf[j]);
    }
    if (ks + 1 < ksteps) {
      store_tile<A_KFAST>(As[cur ^ 1], ra);
      store_tile<B_KFAST>(Bs[cur ^ 1], rb);
    }
    __syncthreads();
  }

  // Epilogue: scatter into D through the destination offset tables.
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const int m = m0 + wm + i * 8 + g;
    if (m >= M) continue;
    const int64_t om = offDm[m];
#pragma unroll
    for (int j = 0; j < 4; ++j) {
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        const int n = n0 + wn + j * 8 + 2 * tig + h;
        if (n >= N) continue;
        double* p = &D[om + offDn[n]];
        *p = beta ? *p + acc[i][j][h] : acc[i][j][h];
      }
    }
  }
}

}  // namespace

int launch_contract_f64(const DevPlan* p, const double* L, const double* R, double* D, int beta,
                        cudaStream_t s) {
  const GemmPlan& h = p->host;
  if (h.M > 0x7fffffff || h.N > 0x7fffffff || h.K > 0x7fffffff)
    return fail(A4G_ERR_RANGE, "matrix dimension exceeds 2^31");
  const int M = int(h.M), N = int(h.N), K = int(h.K);
  const int64_t tiles_m = (M + BM - 1) / BM, tiles_n = (N + BN - 1) / BN;
  const int64_t grid = tiles_m * tiles_n;
  if (grid > 0x7fffffffLL) return fail(A4G_ERR_RANGE, "contraction grid too large");
  auto args = [&](auto kern) {
    kern<<<unsigned(grid), kThreadsF64, 0, s>>>(L, R, D, p->offLm, p->offLk, p->offRk, p->offRn,
                                                p->offDm, p->offDn, M, N, K, int(tiles_m), beta);
  };
  if (h.a_kfast && h.b_kfast) args(contract_f64_kernel<true, true>);
  else if (h.a_kfast) args(contract_f64_kernel<true, false>);
  else if (h.b_kfast) args(contract_f64_kernel<false, true>);
  else args(contract_f64_kernel<false, false>);
  A4G_CUDA(cudaGetLastError());
  return A4G_OK;
}

}  // namespace a4g
