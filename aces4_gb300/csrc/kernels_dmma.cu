// Plain FP64 block contraction on the FP64 tensor path (DMMA, mma.sync f64),
// with the operand and result permutes folded into the tile loads/stores.
//
// Matrix view (planner):  D[offDm[m]+offDn[n]] (=|+=) sum_k L[offLm[m]+offLk[k]] * R[offRk[k]+offRn[n]]
// so no transposed copy of L, R or D is ever written (the reference allocates
// and fills transposed temporaries, tensor_dil_omp.F90:729-751, 782-785).
//
// CTA tile 64 or 48 rows x 64 or 32 columns (the smaller forms for small or
// narrow destinations), k-step 16, 128 threads (2x2 warps, BM/16 x BN/16
// m8n8k4 DMMA tiles per warp).  Tiles are gathered through the offset tables into
// registers, then staged in double-buffered shared memory.  FP64 throughput on
// GB300 is ~2 FMA/clk/SM, so the kernel is bound by the FP64 pipe; the gather
// traffic is small in comparison.
//
// The grouped form runs a whole pardo step: one CTA owns one 64x64 tile of one
// destination block and sums the products of every block pair that feeds that
// block (the contract-accumulate the interpreter lacks), then writes D once.
#include <algorithm>

#include "a4g_internal.h"
#include "grouped.h"

namespace a4g {
namespace {

constexpr int BK = 16;
constexpr int kThreadsF64 = 128;

__device__ __forceinline__ void dmma_8x8x4(double (&c)[2], double a, double b) {
  asm volatile("mma.sync.aligned.m8n8k4.row.col.f64.f64.f64.f64 {%0,%1}, {%2}, {%3}, {%0,%1};\n"
               : "+d"(c[0]), "+d"(c[1])
               : "d"(a), "d"(b));
}

// Element e = threadIdx.x + 128 i of a ROWS x 16 operand tile: with the
// operand unit-stride along k (kfast) threads walk k fastest, else the rows.
template <int ROWS>
__device__ __forceinline__ void tile_coord(bool kfast, int e, int& r, int& kk) {
  if (kfast) kk = e & (BK - 1), r = e >> 4;
  else r = e % ROWS, kk = e / ROWS;
}

// Gathers one ROWS x 16 operand tile (rows x k) into ROWS/8 registers per thread.
template <int ROWS>
__device__ __forceinline__ void gather_tile(bool kfast, double (&reg)[ROWS / 8], const double* __restrict__ X,
                                            const int64_t* __restrict__ offRow,  // smem, per row
                                            const int64_t* __restrict__ offK,    // global, per k
                                            int rows_left, int k0, int K) {
#pragma unroll
  for (int i = 0; i < ROWS / 8; ++i) {
    int r, kk;
    tile_coord<ROWS>(kfast, int(threadIdx.x) + kThreadsF64 * i, r, kk);
    const int k = k0 + kk;
    reg[i] = (r < rows_left && k < K) ? __ldg(&X[offRow[r] + __ldg(&offK[k])]) : 0.0;
  }
}

template <int ROWS, int LD>
__device__ __forceinline__ void store_tile(bool kfast, double (*S)[LD], const double (&reg)[ROWS / 8]) {
#pragma unroll
  for (int i = 0; i < ROWS / 8; ++i) {
    int r, kk;
    tile_coord<ROWS>(kfast, int(threadIdx.x) + kThreadsF64 * i, r, kk);
    S[kk][r] = reg[i];
  }
}

// Tile BM x BN: BM 64 or 48 rows (48 when it cuts the row padding: the small
// ladder's 144 rows are three 48-row tiles, 75 % of three 64-row ones), BN
// 64 or 32 columns (32 for narrow destinations: the ladder's i,j extent of 25
// fills 78 % of a 32-column tile, 39 % of a 64-column one).  4 warps as 2 x 2,
// each (BM/2) x (BN/2) = BM/16 x BN/16 m8n8k4 DMMA tiles.
template <int BM, int BN>
struct Smem {
  double As[2][BK][BM + 4];  // +4 doubles: conflict-free fragment reads
  double Bs[2][BK][BN + 4];
  int64_t sLm[BM], sRn[BN];
};

template <int BM, int BN>
struct Acc {
  double v[BM / 16][BN / 16][2];
  __device__ __forceinline__ void zero() {
#pragma unroll
    for (int i = 0; i < BM / 16; ++i)
#pragma unroll
      for (int j = 0; j < BN / 16; ++j) v[i][j][0] = v[i][j][1] = 0.0;
  }
};

// acc += L_tile * R_tile over the k steps [ks0, ks1) (16 k each) of one pair.
template <int BM, int BN>
__device__ void accumulate_pair(Smem<BM, BN>& sm, Acc<BM, BN>& acc, const double* __restrict__ L,
                                const double* __restrict__ R, const int64_t* __restrict__ offLm,
                                const int64_t* __restrict__ offLk, const int64_t* __restrict__ offRk,
                                const int64_t* __restrict__ offRn, int M, int N, int K, int m0, int n0,
                                bool a_kfast, bool b_kfast, int ks0, int ks1) {
  const int t = threadIdx.x;
  __syncthreads();  // previous pair done with the tables / tiles
  if (t < BM) sm.sLm[t] = (m0 + t < M) ? offLm[m0 + t] : 0;
  if (t < BN) sm.sRn[t] = (n0 + t < N) ? offRn[n0 + t] : 0;
  __syncthreads();
  if (ks0 >= ks1) return;

  const int warp = t >> 5, lane = t & 31;
  const int g = lane >> 2, tig = lane & 3;
  const int wm = (warp & 1) * (BM / 2), wn = (warp >> 1) * (BN / 2);
  double ra[BM / 8], rb[BN / 8];
  gather_tile<BM>(a_kfast, ra, L, sm.sLm, offLk, M - m0, ks0 * BK, K);
  gather_tile<BN>(b_kfast, rb, R, sm.sRn, offRk, N - n0, ks0 * BK, K);
  store_tile<BM, BM + 4>(a_kfast, sm.As[0], ra);
  store_tile<BN, BN + 4>(b_kfast, sm.Bs[0], rb);
  __syncthreads();
  for (int ks = ks0; ks < ks1; ++ks) {
    const int cur = (ks - ks0) & 1;
    if (ks + 1 < ks1) {
      gather_tile<BM>(a_kfast, ra, L, sm.sLm, offLk, M - m0, (ks + 1) * BK, K);
      gather_tile<BN>(b_kfast, rb, R, sm.sRn, offRk, N - n0, (ks + 1) * BK, K);
    }
#pragma unroll
    for (int kk = 0; kk < BK; kk += 4) {
      double af[BM / 16], bf[BN / 16];
#pragma unroll
      for (int i = 0; i < BM / 16; ++i) af[i] = sm.As[cur][kk + tig][wm + i * 8 + g];
#pragma unroll
      for (int j = 0; j < BN / 16; ++j) bf[j] = sm.Bs[cur][kk + tig][wn + j * 8 + g];
#pragma unroll
      for (int i = 0; i < BM / 16; ++i)
#pragma unroll
        for (int j = 0; j < BN / 16; ++j) dmma_8x8x4(acc.v[i][j], af[i], bf[j]);
    }
    if (ks + 1 < ks1) {
      store_tile<BM, BM + 4>(a_kfast, sm.As[cur ^ 1], ra);
      store_tile<BN, BN + 4>(b_kfast, sm.Bs[cur ^ 1], rb);
    }
    __syncthreads();
  }
}

// mode bit 0: accumulate into D (beta = 1), bit 1: store the negated sum.
template <int BM, int BN>
__device__ void write_tile(const Acc<BM, BN>& acc, double* __restrict__ D, const int64_t* __restrict__ offDm,
                           const int64_t* __restrict__ offDn, int M, int N, int m0, int n0, int mode) {
  const int t = threadIdx.x, warp = t >> 5, lane = t & 31;
  const int g = lane >> 2, tig = lane & 3;
  const int wm = (warp & 1) * (BM / 2), wn = (warp >> 1) * (BN / 2);
#pragma unroll
  for (int i = 0; i < BM / 16; ++i) {
    const int m = m0 + wm + i * 8 + g;
    if (m >= M) continue;
    const int64_t om = offDm[m];
#pragma unroll
    for (int j = 0; j < BN / 16; ++j) {
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        const int n = n0 + wn + j * 8 + 2 * tig + h;
        if (n >= N) continue;
        double* p = &D[om + offDn[n]];
        const double v = (mode & 2) ? -acc.v[i][j][h] : acc.v[i][j][h];
        *p = (mode & 1) ? *p + v : v;
      }
    }
  }
}

// A partial tile, column-major BM x BN, into workspace slot `slot`.
template <int BM, int BN>
__device__ void write_partial(const Acc<BM, BN>& acc, double* __restrict__ ws, int64_t slot) {
  double* w = ws + slot * BM * BN;
  const int t = threadIdx.x, warp = t >> 5, lane = t & 31;
  const int g = lane >> 2, tig = lane & 3;
  const int wm = (warp & 1) * (BM / 2), wn = (warp >> 1) * (BN / 2);
#pragma unroll
  for (int i = 0; i < BM / 16; ++i)
#pragma unroll
    for (int j = 0; j < BN / 16; ++j)
#pragma unroll
      for (int h = 0; h < 2; ++h) w[(wn + j * 8 + 2 * tig + h) * BM + wm + i * 8 + g] = acc.v[i][j][h];
}

// One block pair.  CTA x = tile + tiles * split: with nsplit == 1 each CTA
// computes a whole tile and stores it; otherwise each computes the tile over
// its share of the k steps and writes a partial tile to the workspace, which
// contract_f64_reduce_kernel sums in split order.  FP64 runs at a few FMA per
// clock per SM on this GPU, so a small block (the ladder's 144 x 25 x 144)
// needs its k range spread over many SMs to finish in microseconds.
template <int BM, int BN>
__global__ void __launch_bounds__(kThreadsF64) contract_f64_kernel(
    const double* __restrict__ L, const double* __restrict__ R, double* __restrict__ D,
    const int64_t* __restrict__ offLm, const int64_t* __restrict__ offLk,
    const int64_t* __restrict__ offRk, const int64_t* __restrict__ offRn,
    const int64_t* __restrict__ offDm, const int64_t* __restrict__ offDn, int M, int N, int K,
    int tiles_m, int tiles, int nsplit, int mode, int a_kfast, int b_kfast, double* __restrict__ ws) {
  __shared__ __align__(16) Smem<BM, BN> sm;
  const int tile = blockIdx.x % tiles, split = blockIdx.x / tiles;
  const int tm = tile % tiles_m, tn = tile / tiles_m;
  const int m0 = tm * BM, n0 = tn * BN;
  const int ksteps = (K + BK - 1) / BK;
  const int ks0 = int(int64_t(ksteps) * split / nsplit), ks1 = int(int64_t(ksteps) * (split + 1) / nsplit);
  Acc<BM, BN> acc;
  acc.zero();
  accumulate_pair<BM, BN>(sm, acc, L, R, offLm, offLk, offRk, offRn, M, N, K, m0, n0, a_kfast, b_kfast, ks0,
                          ks1);
  if (nsplit > 1) write_partial<BM, BN>(acc, ws, blockIdx.x);
  else write_tile<BM, BN>(acc, D, offDm, offDn, M, N, m0, n0, mode);
}

// Sums tile `blockIdx.x`'s nsplit partials (slots tile + tiles * split) in
// split order and stores it: the same bits on every run.
template <int BM, int BN>
__global__ void __launch_bounds__(256) contract_f64_reduce_kernel(const double* __restrict__ ws, int tiles,
                                                                  int nsplit, int tiles_m, double* __restrict__ D,
                                                                  const int64_t* __restrict__ offDm,
                                                                  const int64_t* __restrict__ offDn, int M, int N,
                                                                  int mode) {
  const int tile = blockIdx.x, tm = tile % tiles_m, tn = tile / tiles_m;
  for (int e = threadIdx.x; e < BM * BN; e += blockDim.x) {
    const int ml = e % BM, nl = e / BM;
    const int m = tm * BM + ml, n = tn * BN + nl;
    if (m >= M || n >= N) continue;
    double v = 0.0;
    for (int q = 0; q < nsplit; ++q) v += ws[(int64_t(tile) + int64_t(tiles) * q) * BM * BN + e];
    if (mode & 2) v = -v;
    double* p = D + offDm[m] + offDn[n];
    *p = (mode & 1) ? *p + v : v;
  }
}

// One CTA per (destination block, tile, share of its pairs); the pairs are
// summed and the tile stored into D, or into a workspace slot when the tile's
// pairs are spread over several CTAs (few tiles, many pairs).
template <int BM, int BN>
__global__ void __launch_bounds__(kThreadsF64) grouped_f64_kernel(const GroupedF64Tile* __restrict__ tiles,
                                                                  const GroupedPair* __restrict__ pairs,
                                                                  const PlanRef* __restrict__ plans,
                                                                  int mode, double* __restrict__ ws) {
  __shared__ __align__(16) Smem<BM, BN> sm;
  const GroupedF64Tile tl = tiles[blockIdx.x];
  Acc<BM, BN> acc;
  acc.zero();
  for (int q = tl.pair_begin; q < tl.pair_end; ++q) {
    const GroupedPair pr = pairs[q];
    const PlanRef pl = plans[pr.plan];
    accumulate_pair<BM, BN>(sm, acc, pr.l, pr.r, pl.offLm, pl.offLk, pl.offRk, pl.offRn, pl.M, pl.N, pl.K,
                            tl.m0, tl.n0, pl.a_kfast, pl.b_kfast, 0, (pl.K + BK - 1) / BK);
  }
  if (tl.slot >= 0) {
    write_partial<BM, BN>(acc, ws, tl.slot);
    return;
  }
  const PlanRef dp = plans[tl.dplan];
  write_tile<BM, BN>(acc, tl.d, dp.offDm, dp.offDn, dp.M, dp.N, tl.m0, tl.n0, mode);
}

// Sums a spread tile's partials in slot order (deterministic) and stores it.
template <int BM, int BN>
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

template <int BM, int BN>
void launch_single(const DevPlan* p, const double* L, const double* R, double* D, int M, int N, int K, int mode,
                   int tiles_m, int64_t tiles, int nsplit, double* ws, cudaStream_t s) {
  const GemmPlan& h = p->host;
  contract_f64_kernel<BM, BN><<<unsigned(tiles * nsplit), kThreadsF64, 0, s>>>(
      L, R, D, p->offLm, p->offLk, p->offRk, p->offRn, p->offDm, p->offDn, M, N, K, tiles_m, int(tiles), nsplit, mode,
      h.a_kfast, h.b_kfast, ws);
  if (nsplit > 1)
    contract_f64_reduce_kernel<BM, BN><<<unsigned(tiles), 256, 0, s>>>(ws, int(tiles), nsplit, tiles_m, D, p->offDm,
                                                                      p->offDn, M, N, mode);
}

template <int BM, int BN>
void launch_grouped(const GroupedF64Tile* tiles, int ntiles, const GroupedPair* pairs, const PlanRef* plans, int mode,
                    double* ws, const GroupedF64Reduce* reds, int nreds, cudaStream_t s) {
  grouped_f64_kernel<BM, BN><<<ntiles, kThreadsF64, 0, s>>>(tiles, pairs, plans, mode, ws);
  if (nreds > 0) grouped_f64_reduce_kernel<BM, BN><<<nreds, 256, 0, s>>>(reds, plans, ws, mode);
}

}  // namespace

// Tile rows for destination rows m: 48 when it pads less than 64 by a tenth.
int f64_tile_m_for(int64_t padded64, int64_t padded48) { return padded48 * 10 < padded64 * 9 ? 48 : 64; }

int launch_contract_f64(const DevPlan* p, const double* L, const double* R, double* D, int mode,
                        cudaStream_t s) {
  const GemmPlan& h = p->host;
  if (h.M > 0x7fffffff || h.N > 0x7fffffff || h.K > 0x7fffffff)
    return fail(A4G_ERR_RANGE, "matrix dimension exceeds 2^31");
  const int M = int(h.M), N = int(h.N), K = int(h.K);
  const int bn = N <= 32 ? 32 : 64;
  const int bm = f64_tile_m_for((M + 63) / 64 * 64, (M + 47) / 48 * 48);
  const int64_t tiles_m = (M + bm - 1) / bm, tiles_n = (N + bn - 1) / bn;
  const int64_t tiles = tiles_m * tiles_n;
  if (tiles > 0x3fffffffLL) return fail(A4G_ERR_RANGE, "contraction grid too large");
  // split the k steps when the tiles alone would leave most SMs idle (about
  // two CTAs per SM, at most 64 splits of at least one k step)
  const int sms = ctx()->num_sms > 0 ? ctx()->num_sms : 152;
  const int64_t ksteps = (K + BK - 1) / BK;
  int nsplit = int(std::max<int64_t>(1, std::min<int64_t>({64, ksteps, (2LL * sms + tiles - 1) / tiles})));
  if (tiles * nsplit > 0x7fffffffLL) nsplit = 1;
  double* ws = nullptr;
  if (nsplit > 1)
    if (const int rc_ = async_alloc(reinterpret_cast<void**>(&ws), size_t(tiles * nsplit) * bm * bn * sizeof(double), s))
      return rc_;
  if (bm == 48 && bn == 32) launch_single<48, 32>(p, L, R, D, M, N, K, mode, int(tiles_m), tiles, nsplit, ws, s);
  else if (bm == 48) launch_single<48, 64>(p, L, R, D, M, N, K, mode, int(tiles_m), tiles, nsplit, ws, s);
  else if (bn == 32) launch_single<64, 32>(p, L, R, D, M, N, K, mode, int(tiles_m), tiles, nsplit, ws, s);
  else launch_single<64, 64>(p, L, R, D, M, N, K, mode, int(tiles_m), tiles, nsplit, ws, s);
  if (nsplit > 1) A4G_CUDA(cudaFreeAsync(ws, s));
  A4G_CUDA(cudaGetLastError());
  return A4G_OK;
}

int launch_grouped_f64(const GroupedF64Tile* tiles, int ntiles, const GroupedPair* pairs, const PlanRef* plans,
                       int mode, double* ws, const GroupedF64Reduce* reds, int nreds, int tile_m, int tile_n,
                       cudaStream_t s) {
  if (ntiles <= 0) return A4G_OK;
  if (tile_m == 48 && tile_n == 32) launch_grouped<48, 32>(tiles, ntiles, pairs, plans, mode, ws, reds, nreds, s);
  else if (tile_m == 48) launch_grouped<48, 64>(tiles, ntiles, pairs, plans, mode, ws, reds, nreds, s);
  else if (tile_n == 32) launch_grouped<64, 32>(tiles, ntiles, pairs, plans, mode, ws, reds, nreds, s);
  else launch_grouped<64, 64>(tiles, ntiles, pairs, plans, mode, ws, reds, nreds, s);
  A4G_CUDA(cudaGetLastError());
  return A4G_OK;
}

int grouped_f64_tile_m(int64_t padded64, int64_t padded48) { return f64_tile_m_for(padded64, padded48); }
int grouped_f64_tile_n(int max_n) { return max_n <= 32 ? 32 : 64; }

}  // namespace a4g
