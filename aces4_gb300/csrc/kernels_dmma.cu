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
//
// The grouped form runs a whole pardo step: one CTA owns one 64x64 tile of one
// destination block and sums the products of every block pair that feeds that
// block (the contract-accumulate the interpreter lacks), then writes D once.
#include "a4g_internal.h"
#include "grouped.h"

namespace a4g {
namespace {

constexpr int BM = 64, BN = 64, BK = 16, LDS = BM + 4;  // +4 doubles: conflict-free fragment reads
constexpr int kThreadsF64 = 128;

__device__ __forceinline__ void dmma_8x8x4(double (&c)[2], double a, double b) {
  asm volatile("mma.sync.aligned.m8n8k4.row.col.f64.f64.f64.f64 {%0,%1}, {%2}, {%3}, {%0,%1};\n"
               : "+d"(c[0]), "+d"(c[1])
               : "d"(a), "d"(b));
}

// Gathers one 64x16 operand tile (rows x k) into 8 registers per thread.
// KFAST: the operand is unit-stride along k, so threads walk k fastest.
__device__ __forceinline__ void gather_tile(bool kfast, double (&reg)[8], const double* __restrict__ X,
                                            const int64_t* __restrict__ offRow,  // smem, per row
                                            const int64_t* __restrict__ offK,    // global, per k
                                            int rows_left, int k0, int K) {
  const int t = threadIdx.x;
#pragma unroll
  for (int i = 0; i < 8; ++i) {
    const int kk = kfast ? (t & (BK - 1)) : ((t >> 6) + 2 * i);
    const int r = kfast ? ((t >> 4) + 8 * i) : (t & (BM - 1));
    const int k = k0 + kk;
    reg[i] = (r < rows_left && k < K) ? __ldg(&X[offRow[r] + __ldg(&offK[k])]) : 0.0;
  }
}

__device__ __forceinline__ void store_tile(bool kfast, double (*S)[LDS], const double (&reg)[8]) {
  const int t = threadIdx.x;
#pragma unroll
  for (int i = 0; i < 8; ++i) {
    const int kk = kfast ? (t & (BK - 1)) : ((t >> 6) + 2 * i);
    const int r = kfast ? ((t >> 4) + 8 * i) : (t & (BM - 1));
    S[kk][r] = reg[i];
  }
}

struct Smem {
  double As[2][BK][LDS];
  double Bs[2][BK][LDS];
  int64_t sLm[BM], sRn[BN];
};

// acc += L_tile * R_tile over all K of one block pair.
__device__ void accumulate_pair(Smem& sm, double (&acc)[4][4][2], const double* __restrict__ L,
                                const double* __restrict__ R, const int64_t* __restrict__ offLm,
                                const int64_t* __restrict__ offLk, const int64_t* __restrict__ offRk,
                                const int64_t* __restrict__ offRn, int M, int N, int K, int m0, int n0,
                                bool a_kfast, bool b_kfast) {
  const int t = threadIdx.x;
  __syncthreads();  // previous pair done with the tables / tiles
  if (t < BM) sm.sLm[t] = (m0 + t < M) ? offLm[m0 + t] : 0;
  else sm.sRn[t - BM] = (n0 + t - BM < N) ? offRn[n0 + t - BM] : 0;
  __syncthreads();

  const int warp = t >> 5, lane = t & 31;
  const int g = lane >> 2, tig = lane & 3;
  const int wm = (warp & 1) * 32, wn = (warp >> 1) * 32;
  double ra[8], rb[8];
  const int ksteps = (K + BK - 1) / BK;
  gather_tile(a_kfast, ra, L, sm.sLm, offLk, M - m0, 0, K);
  gather_tile(b_kfast, rb, R, sm.sRn, offRk, N - n0, 0, K);
  store_tile(a_kfast, sm.As[0], ra);
  store_tile(b_kfast, sm.Bs[0], rb);
  __syncthreads();
  for (int ks = 0; ks < ksteps; ++ks) {
    const int cur = ks & 1;
    if (ks + 1 < ksteps) {
      gather_tile(a_kfast, ra, L, sm.sLm, offLk, M - m0, (ks + 1) * BK, K);
      gather_tile(b_kfast, rb, R, sm.sRn, offRk, N - n0, (ks + 1) * BK, K);
    }
#pragma unroll
    for (int kk = 0; kk < BK; kk += 4) {
      double af[4], bf[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) af[i] = sm.As[cur][kk + tig][wm + i * 8 + g];
#pragma unroll
      for (int j = 0; j < 4; ++j) bf[j] = sm.Bs[cur][kk + tig][wn + j * 8 + g];
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) dmma_8x8x4(acc[i][j], af[i], bf[j]);
    }
    if (ks + 1 < ksteps) {
      store_tile(a_kfast, sm.As[cur ^ 1], ra);
      store_tile(b_kfast, sm.Bs[cur ^ 1], rb);
    }
    __syncthreads();
  }
}

// mode bit 0: accumulate into D (beta = 1), bit 1: store the negated sum.
__device__ void write_tile(const double (&acc)[4][4][2], double* __restrict__ D,
                           const int64_t* __restrict__ offDm, const int64_t* __restrict__ offDn,
                           int M, int N, int m0, int n0, int mode) {
  const int t = threadIdx.x, warp = t >> 5, lane = t & 31;
  const int g = lane >> 2, tig = lane & 3;
  const int wm = (warp & 1) * 32, wn = (warp >> 1) * 32;
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
        const double v = (mode & 2) ? -acc[i][j][h] : acc[i][j][h];
        *p = (mode & 1) ? *p + v : v;
      }
    }
  }
}

__global__ void __launch_bounds__(kThreadsF64) contract_f64_kernel(
    const double* __restrict__ L, const double* __restrict__ R, double* __restrict__ D,
    const int64_t* __restrict__ offLm, const int64_t* __restrict__ offLk,
    const int64_t* __restrict__ offRk, const int64_t* __restrict__ offRn,
    const int64_t* __restrict__ offDm, const int64_t* __restrict__ offDn, int M, int N, int K,
    int tiles_m, int mode, int a_kfast, int b_kfast) {
  __shared__ __align__(16) Smem sm;
  const int tm = blockIdx.x % tiles_m, tn = blockIdx.x / tiles_m;
  const int m0 = tm * BM, n0 = tn * BN;
  double acc[4][4][2];
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) acc[i][j][0] = acc[i][j][1] = 0.0;
  accumulate_pair(sm, acc, L, R, offLm, offLk, offRk, offRn, M, N, K, m0, n0, a_kfast, b_kfast);
  write_tile(acc, D, offDm, offDn, M, N, m0, n0, mode);
}

// One CTA per (destination block, 64x64 tile, share of its pairs); the pairs
// are summed and the tile stored into D, or into a workspace slot when the
// tile's pairs are spread over several CTAs (few tiles, many pairs).
__global__ void __launch_bounds__(kThreadsF64) grouped_f64_kernel(const GroupedF64Tile* __restrict__ tiles,
                                                                  const GroupedPair* __restrict__ pairs,
                                                                  const PlanRef* __restrict__ plans,
                                                                  int mode, double* __restrict__ ws) {
  __shared__ __align__(16) Smem sm;
  const GroupedF64Tile tl = tiles[blockIdx.x];
  double acc[4][4][2];
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) acc[i][j][0] = acc[i][j][1] = 0.0;
  for (int q = tl.pair_begin; q < tl.pair_end; ++q) {
    const GroupedPair pr = pairs[q];
    const PlanRef pl = plans[pr.plan];
    accumulate_pair(sm, acc, pr.l, pr.r, pl.offLm, pl.offLk, pl.offRk, pl.offRn, pl.M, pl.N, pl.K,
                    tl.m0, tl.n0, pl.a_kfast, pl.b_kfast);
  }
  if (tl.slot >= 0) {  // partial tile, column-major 64x64 in its slot
    double* w = ws + size_t(tl.slot) * BM * BN;
    const int t = threadIdx.x, warp = t >> 5, lane = t & 31;
    const int g = lane >> 2, tig = lane & 3;
    const int wm = (warp & 1) * 32, wn = (warp >> 1) * 32;
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
      for (int j = 0; j < 4; ++j)
#pragma unroll
        for (int h = 0; h < 2; ++h) w[(wn + j * 8 + 2 * tig + h) * BM + wm + i * 8 + g] = acc[i][j][h];
    return;
  }
  const PlanRef dp = plans[tl.dplan];
  write_tile(acc, tl.d, dp.offDm, dp.offDn, dp.M, dp.N, tl.m0, tl.n0, mode);
}

// Sums a spread tile's partials in slot order (deterministic) and stores it.
__global__ void __launch_bounds__(256) grouped_f64_reduce_kernel(const GroupedF64Reduce* __restrict__ reds,
                                                                 const PlanRef* __restrict__ plans,
                                                                 const double* __restrict__ ws, int mode) {
  const GroupedF64Reduce rd = reds[blockIdx.x];
  const PlanRef dp = plans[rd.dplan];
  for (int e = threadIdx.x; e < BM * BN; e += blockDim.x) {
    const int ml = e % BM, nl = e / BM;
    const int m = rd.m0 + ml, n = rd.n0 + nl;
    if (m >= dp.M || n >= dp.N) continue;
    double v = 0.0;
    for (int q = 0; q < rd.nparts; ++q) v += ws[size_t(rd.slot0 + q) * BM * BN + e];
    if (mode & 2) v = -v;
    double* p = rd.d + dp.offDm[m] + dp.offDn[n];
    *p = (mode & 1) ? *p + v : v;
  }
}

}  // namespace

int launch_contract_f64(const DevPlan* p, const double* L, const double* R, double* D, int mode,
                        cudaStream_t s) {
  const GemmPlan& h = p->host;
  if (h.M > 0x7fffffff || h.N > 0x7fffffff || h.K > 0x7fffffff)
    return fail(A4G_ERR_RANGE, "matrix dimension exceeds 2^31");
  const int M = int(h.M), N = int(h.N), K = int(h.K);
  const int64_t tiles_m = (M + BM - 1) / BM, tiles_n = (N + BN - 1) / BN;
  const int64_t grid = tiles_m * tiles_n;
  if (grid > 0x7fffffffLL) return fail(A4G_ERR_RANGE, "contraction grid too large");
  contract_f64_kernel<<<unsigned(grid), kThreadsF64, 0, s>>>(L, R, D, p->offLm, p->offLk, p->offRk,
                                                            p->offRn, p->offDm, p->offDn, M, N, K,
                                                            int(tiles_m), mode, h.a_kfast, h.b_kfast);
  A4G_CUDA(cudaGetLastError());
  return A4G_OK;
}

int launch_grouped_f64(const GroupedF64Tile* tiles, int ntiles, const GroupedPair* pairs,
                       const PlanRef* plans, int mode, double* ws, const GroupedF64Reduce* reds, int nreds,
                       cudaStream_t s) {
  if (ntiles <= 0) return A4G_OK;
  grouped_f64_kernel<<<ntiles, kThreadsF64, 0, s>>>(tiles, pairs, plans, mode, ws);
  if (nreds > 0) grouped_f64_reduce_kernel<<<nreds, 256, 0, s>>>(reds, plans, ws, mode);
  A4G_CUDA(cudaGetLastError());
  return A4G_OK;
}

int grouped_f64_tile_m() { return BM; }
int grouped_f64_tile_n() { return BN; }

}  // namespace a4g
