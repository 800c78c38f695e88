// Split-precision (Ozaki scheme) block contraction on the tcgen05 tensor cores.
//
// Each FP64 operand row (left blocks) / column (right blocks) is scaled by a
// power of two with |x| < 2^E over the whole row of the pardo step, rounded to
// the integer n = round(x * 2^(8*slices - E - 1)) (|n| <= 2^(8*slices-1)) and
// cut into `slices` balanced base-256 digits:
//     x ~= sum_i d_i * 2^(E + 1 - 8(i+1)),   d_0 in [-128, 128], d_i in [-128, 127].
// Digits are exact BF16 values and every digit product is at most 2^14.  The
// product of two slices is an integer matrix, so
//     L*R ~= sum_t 2^(E_m + F_n + 2 - 8(t+2)) * S_t,   S_t = sum_{i+j=t} A_i B_j
// over levels t < slices (triangular truncation).  Each S_t is computed on the
// tensor cores (kind::f16, BF16 x BF16 -> FP32) in chunks of k short enough
// that every FP32 partial sum is an integer below 2^24 and therefore exact;
// the epilogue warps fold each chunk into an exact running sum (an FP32 (hi,
// lo) TwoSum pair kept in TMEM for 128-column tiles, int32 registers for
// 256-column tiles).  A final FP64 kernel applies the powers of two and
// writes D.
//
// Published method: Ozaki, Ogita, Oishi, Rump, "Error-free transformations of
// matrix multiplication by using fast routines of matrix multiplication and
// its applications", Numer. Algorithms 59 (2012); Mukunoki, Ozaki, Ogita,
// Imamura, "DGEMM using Tensor Cores, and Its Accurate and Reproducible
// Versions", ISC 2020 (slices on tensor cores with exact FP32 accumulation).
//
// Kernels:
//   oz_exp_*_kernel     max exponent per panel row          (HBM: 8 B/elem read)
//   oz_split_*_kernel   FP64 -> BF16 digit slices, K-major   (HBM: 8 B read + 2*slices B write)
//                       with the block's index permute folded into the gather
//   oz_gemm_kernel<PAIR, BN, DIRECT, ENERGY>
//                       persistent warp-specialised tcgen05 GEMM: TMA (SW128)
//                       -> smem ring -> tcgen05.mma into TMEM (2 accumulators)
//                       -> epilogue warps fold each exact chunk into the level
//                       sum.  Four forms: one SM or a CTA pair (cta_group::2)
//                       per tile, 128 or 256 columns per MMA; the batch
//                       autotunes among them.
//   oz_recombine_kernel int64 sum over split-K units, FP64 combination of the
//                       levels, scaled store into D
#include <cuda.h>
#include <cuda_bf16.h>
#include <cudaTypedefs.h>

#include <algorithm>
#include <atomic>
#include <type_traits>

#include "a4g_internal.h"
#include "exact_fp.h"
#include "grouped.h"
#include "ozaki.h"

namespace a4g {
namespace {

constexpr int kDigitBits = 8;
constexpr int kThreadsOz = 320;  // warp 0 TMA, warp 1 MMA, warps 2..9 epilogue
// Direct forms: warps 2..17 epilogue (four per TMEM lane quadrant, 32 columns
// each): their epilogue also rounds and stores every result.
constexpr int kThreadsOzDirect = 576;
constexpr uint32_t kTileBytes = kOzBM * kOzBK * 2;  // 16 KB per operand tile
// TMEM columns, 128-column forms: [0,128) and [128,256) are the two FP32 MMA
// accumulators; [256,384) and [384,512) hold the running exact (hi, lo) sums of
// the current level.  256-column forms: [0,256) and [256,512) are the two
// accumulators; the level sums live in the epilogue threads' registers.
constexpr uint32_t kTmemCols = 512;
constexpr uint32_t kTmemHi = 256, kTmemLo = 384;
// Direct form: the same two regions hold the low and high 32-bit words of the
// exact 64-bit running sum over levels.
constexpr uint32_t kTmemW0 = 256, kTmemW1 = 384;
constexpr unsigned long long kWaitLimitNs = 20ull * 1000 * 1000 * 1000;  // 20 s

// tcgen05 instruction descriptor, kind::f16: D F32 (bits 4-5 = 1), A BF16
// (bits 7-9 = 1), B BF16 (bits 10-12 = 1), both K-major (bits 15/16 = 0),
// N>>3 at bits 17-22, M>>4 at bits 24-28.
template <int M, int N>
constexpr uint32_t idesc_bf16() {
  return (1u << 4) | (1u << 7) | (1u << 10) | (uint32_t(N >> 3) << 17) | (uint32_t(M >> 4) << 24);
}

// Shared memory of the tensor-core kernel, per form (PAIR: a CTA pair computes
// one tile with cta_group::2; BN: tile columns).  Each CTA stages its 128 rows
// of A and its BN (1-SM) or BN/2 (pair) rows of B per 64-wide k block:
//   1-SM BN=128: 32 KB x 6 stages   pair BN=128: 24 KB x 9
//   1-SM BN=256: 48 KB x 4 stages   pair BN=256: 32 KB x 6
template <bool PAIR, int BN>
struct __align__(1024) OzSmemT {
  static constexpr uint32_t kBBytes = uint32_t(PAIR ? BN / 2 : BN) * kOzBK * 2;
  static constexpr int kSt = int((216u * 1024u) / (kTileBytes + kBBytes)) > 9 ? 9
                                                                               : int((216u * 1024u) / (kTileBytes + kBBytes));
  uint8_t a[kSt][kTileBytes];
  uint8_t b[kSt][kBBytes];
  uint64_t full[kSt], empty[kSt];
  uint64_t acc_full[2], acc_empty[2];
  uint64_t drain;
  uint32_t tmem_base;
  volatile int abort;
};

// ------------------------------------------------------------------ PTX helpers
__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}
__device__ __forceinline__ unsigned long long now_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %globaltimer;" : "=l"(t));
  return t;
}
__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count));
}
__device__ __forceinline__ void fence_mbar_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
               : "memory");
}
__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}\n"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
// Bounded wait: gives up after kWaitLimitNs or when another role aborted.
template <class SM>
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, SM& sm, int* err, int code) {
  if (mbar_try_wait(bar, parity)) return true;
  const unsigned long long t0 = now_ns();
#pragma unroll 1
  for (uint32_t it = 1;; ++it) {
    if (mbar_try_wait(bar, parity)) return true;
    if ((it & 255) == 0) {
      if (sm.abort) return false;
      if (now_ns() - t0 > kWaitLimitNs) {
        sm.abort = 1;
        atomicExch(err, code);
        return false;
      }
    }
  }
}
__device__ __forceinline__ void tma_load_2d(void* dst, const void* map, uint64_t* bar, int c0, int c1) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%3, %4}], [%2];" ::"r"(
          smem_u32(dst)),
      "l"(map), "r"(smem_u32(bar)), "r"(c0), "r"(c1)
      : "memory");
}
__device__ __forceinline__ void tc_fence_before() {
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void tc_fence_after() {
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void tc_commit(uint64_t* bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                   smem_u32(bar))
               : "memory");
}
template <int N>
__device__ __forceinline__ void tc_mma(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc, uint32_t accum) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(d_tmem),
      "l"(adesc), "l"(bdesc), "r"(idesc_bf16<128, N>()), "r"(accum));
}
// --- CTA-pair (cta_group::2) forms
__device__ __forceinline__ uint32_t cluster_rank() {
  uint32_t r;
  asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
  return r;
}
// shared::cluster address of the same shared variable in CTA `rank` of the cluster
__device__ __forceinline__ uint32_t mapa_shared(const void* p, uint32_t rank) {
  uint32_t out;
  asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(out) : "r"(smem_u32(p)), "r"(rank));
  return out;
}
__device__ __forceinline__ void cluster_sync() {
  asm volatile("barrier.cluster.arrive.release.aligned;\n\tbarrier.cluster.wait.acquire.aligned;" ::: "memory");
}
__device__ __forceinline__ void mbar_arrive_cluster(uint32_t bar_cluster) {
  asm volatile("mbarrier.arrive.shared::cluster.b64 _, [%0];" ::"r"(bar_cluster) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx_cluster(uint32_t bar_cluster, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cluster.b64 _, [%0], %1;" ::"r"(bar_cluster), "r"(bytes)
               : "memory");
}
// TMA load into this CTA's shared memory that signals an mbarrier which may
// live in either CTA of the pair
__device__ __forceinline__ void tma_load_2d_pair(void* dst, const void* map, uint32_t bar_cluster, int c0,
                                                 int c1) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes.cta_group::2 [%0], [%1, {%3, %4}], [%2];" ::"r"(
          smem_u32(dst)),
      "l"(map), "r"(bar_cluster), "r"(c0), "r"(c1)
      : "memory");
}
template <int N>
__device__ __forceinline__ void tc_mma_pair(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc, uint32_t accum) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::2.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(d_tmem),
      "l"(adesc), "l"(bdesc), "r"(idesc_bf16<256, N>()), "r"(accum));
}
// arrive on the mbarrier at the same offset in both CTAs of the pair once
// this thread's tcgen05 operations complete
__device__ __forceinline__ void tc_commit_pair(uint64_t* bar) {
  asm volatile(
      "tcgen05.commit.cta_group::2.mbarrier::arrive::one.shared::cluster.multicast::cluster.b64 [%0], %1;" ::"r"(
          smem_u32(bar)),
      "h"(uint16_t(3))
      : "memory");
}

// Shared-memory matrix descriptor: K-major, 128-byte swizzle, rows of 128 B,
// 8-row core groups 1024 B apart (SBO), descriptor version 1 (bits 46-48).
__device__ __forceinline__ uint64_t sw128_desc(const void* tile) {
  const uint32_t addr = smem_u32(tile);
  uint64_t d = uint64_t((addr & 0x3FFFF) >> 4);
  d |= uint64_t(1) << 16;            // leading byte offset (unused for SW128 K-major)
  d |= uint64_t(1024 >> 4) << 32;    // stride byte offset
  d |= uint64_t(1) << 46;
  d |= uint64_t(2) << 61;            // SWIZZLE_128B
  return d;
}
__device__ __forceinline__ void tc_wait_ld() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }
__device__ __forceinline__ void tc_wait_st() { asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory"); }
// 32 consecutive TMEM columns of this thread's lane; completes at tc_wait_ld().
__device__ __forceinline__ void tc_ld32_nowait(uint32_t taddr, uint32_t (&r)[32]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 "
      "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
      "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
        "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),
        "=r"(r[14]), "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]),
        "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]), "=r"(r[25]),
        "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
      : "r"(taddr));
}
__device__ __forceinline__ void tc_ld16_nowait(uint32_t taddr, uint32_t (&r)[16]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 "
      "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
        "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),
        "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
}
// Exact accumulation of an integer-valued float x (|x| < 2^24) into hi + lo.
__device__ __forceinline__ void two_sum_acc(float& hi, float& lo, float x) {
  const float s = __fadd_rn(hi, x);
  const float bp = __fsub_rn(s, hi);
  const float e = __fadd_rn(__fsub_rn(hi, __fsub_rn(s, bp)), __fsub_rn(x, bp));
  hi = s;
  lo = __fadd_rn(lo, e);
}

// A row or column exponent of 2047 (the field of Inf and NaN) marks a panel
// row that holds a non-finite value: digits cannot carry it, so every result
// that row or column feeds is stored as NaN (in FP64 a NaN or an infinity in
// an operand makes the whole row or column of the product NaN or infinite).
constexpr int kNonFiniteExp = 2047;

// ------------------------------------------------------------------ roles
// Walks the k blocks of one unit: calls f(koff_a, koff_b, kb) per 64-wide
// block (the panels are zero beyond the end of every stretch of pairs up to
// the next 64-column boundary, so whole blocks are always multiplied).
template <class F>
__device__ __forceinline__ void for_unit_kblocks(const OzGemmArgs& a, const OzUnit& un, const OzTile& tl,
                                                 F&& f) {
  int kb = un.kb_begin;
  int q = un.trip_first, j = un.kb_in_trip;
  while (kb < un.kb_end && q < tl.trip_end) {
    const OzTrip tr = a.trips[q];
    for (; j < tr.nkb && kb < un.kb_end; ++j, ++kb)
      if (!f(int(tr.koff_a) + j * kOzBK, int(tr.koff_b) + j * kOzBK, kb)) return;
    ++q;
    j = 0;
  }
}

// Units are distributed over CTAs (1-SM form) or over CTA pairs (2-SM form:
// both CTAs of a pair walk the same units).
template <bool PAIR>
__device__ __forceinline__ int unit_first() { return PAIR ? int(blockIdx.x >> 1) : int(blockIdx.x); }
template <bool PAIR>
__device__ __forceinline__ int unit_stride() { return PAIR ? int(gridDim.x >> 1) : int(gridDim.x); }

// This CTA's (pair's) units in run order; f(u) returns false to stop.  The
// direct form hands out whole tiles: units (tile, 0..slices-1) in a row.
template <bool PAIR, class F>
__device__ __forceinline__ void for_units(const OzGemmArgs& a, F&& f) {
  if (a.direct) {
    const int groups = a.n_units / a.slices;
    for (int g = unit_first<PAIR>(); g < groups; g += unit_stride<PAIR>())
      for (int lv = 0; lv < a.slices; ++lv)
        if (!f(g * a.slices + lv)) return;
  } else {
    for (int u = unit_first<PAIR>(); u < a.n_units; u += unit_stride<PAIR>())
      if (!f(u)) return;
  }
}

template <bool PAIR, int BN>
__device__ void producer(const OzGemmArgs& a, OzSmemT<PAIR, BN>& sm, uint32_t rank) {
  using SM = OzSmemT<PAIR, BN>;
  constexpr uint32_t kBytes = kTileBytes + SM::kBBytes;
  uint32_t it = 0;
  for_units<PAIR>(a, [&](int u) {
    const OzUnit un = a.units[u];
    const OzTile tl = a.tiles[un.tile];
    const int level = un.level;
    const void* ma = static_cast<const uint8_t*>(a.maps_a) + size_t(tl.panel_a) * 128;
    const void* mb = static_cast<const uint8_t*>(a.maps_b) + size_t(tl.panel_b) * 128;
    const int rpa = a.panels_a[tl.panel_a].rows_pad, rpb = a.panels_b[tl.panel_b].rows_pad;
    const int arow = tl.m0 + int(rank) * kOzBM;          // this CTA's 128 rows of A
    const int brow = tl.n0 + int(rank) * (BN / 2);       // this CTA's half of B (pair form)
    bool ok = true;
    for_unit_kblocks(a, un, tl, [&](int ka, int kb, int) {
      for (int i = 0; i <= level; ++i) {
        const int s = it % SM::kSt;
        const uint32_t ph = (it / SM::kSt) & 1;
        if (!mbar_wait(&sm.empty[s], ph ^ 1, sm, a.err_flag, 1)) return ok = false;
        if constexpr (PAIR) {
          const uint32_t fb = mapa_shared(&sm.full[s], 0);  // the leader CTA's barrier
          mbar_expect_tx_cluster(fb, kBytes);
          tma_load_2d_pair(sm.a[s], ma, fb, ka, i * rpa + arow);
          tma_load_2d_pair(sm.b[s], mb, fb, kb, (level - i) * rpb + brow);
        } else {
          mbar_expect_tx(&sm.full[s], kBytes);
          tma_load_2d(sm.a[s], ma, &sm.full[s], ka, i * rpa + arow);
          tma_load_2d(sm.b[s], mb, &sm.full[s], kb, (level - i) * rpb + tl.n0);
        }
        ++it;
      }
      return true;
    });
    return ok;
  });
}

// One thread issues every MMA (the leader CTA's in the pair form).
template <bool PAIR, int BN>
__device__ void mma_issuer(const OzGemmArgs& a, OzSmemT<PAIR, BN>& sm, uint32_t tmem) {
  using SM = OzSmemT<PAIR, BN>;
  uint32_t it = 0, chunk = 0;
  for_units<PAIR>(a, [&](int u) {
    const OzUnit un = a.units[u];
    const OzTile tl = a.tiles[un.tile];
    const int level = un.level;
    const int ckb = a.chunk_kb[level];
    int in_chunk = 0;
    uint32_t buf = 0;
    bool ok = true;
    for_unit_kblocks(a, un, tl, [&](int, int, int kb) {
      if (in_chunk == 0) {
        buf = chunk & 1;
        if (!mbar_wait(&sm.acc_empty[buf], ((chunk >> 1) & 1) ^ 1, sm, a.err_flag, 2)) return ok = false;
        tc_fence_after();
      }
      const uint32_t d_tmem = tmem + buf * BN;
      for (int i = 0; i <= level; ++i) {
        const int s = it % SM::kSt;
        const uint32_t ph = (it / SM::kSt) & 1;
        if (!mbar_wait(&sm.full[s], ph, sm, a.err_flag, 3)) return ok = false;
        tc_fence_after();
        const uint64_t ad = sw128_desc(sm.a[s]), bd = sw128_desc(sm.b[s]);
#pragma unroll
        for (int kk = 0; kk < kOzBK / 16; ++kk) {
          const uint32_t acc = (in_chunk == 0 && i == 0 && kk == 0) ? 0u : 1u;
          if constexpr (PAIR) tc_mma_pair<BN>(d_tmem, ad + 2 * kk, bd + 2 * kk, acc);
          else tc_mma<BN>(d_tmem, ad + 2 * kk, bd + 2 * kk, acc);
        }
        if constexpr (PAIR) tc_commit_pair(&sm.empty[s]);
        else tc_commit(&sm.empty[s]);
        ++it;
      }
      ++in_chunk;
      if (in_chunk == ckb || kb + 1 == un.kb_end) {
        if constexpr (PAIR) tc_commit_pair(&sm.acc_full[buf]);
        else tc_commit(&sm.acc_full[buf]);
        ++chunk;
        in_chunk = 0;
      }
      return true;
    });
    return ok;
  });
}

__device__ __forceinline__ void tc_st32(uint32_t taddr, const uint32_t (&r)[32]) {
  asm volatile(
      "tcgen05.st.sync.aligned.32x32b.x32.b32 [%0], "
      "{%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16,"
      "%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31,%32};" ::"r"(taddr),
      "r"(r[0]), "r"(r[1]), "r"(r[2]), "r"(r[3]), "r"(r[4]), "r"(r[5]), "r"(r[6]), "r"(r[7]),
      "r"(r[8]), "r"(r[9]), "r"(r[10]), "r"(r[11]), "r"(r[12]), "r"(r[13]), "r"(r[14]),
      "r"(r[15]), "r"(r[16]), "r"(r[17]), "r"(r[18]), "r"(r[19]), "r"(r[20]), "r"(r[21]),
      "r"(r[22]), "r"(r[23]), "r"(r[24]), "r"(r[25]), "r"(r[26]), "r"(r[27]), "r"(r[28]),
      "r"(r[29]), "r"(r[30]), "r"(r[31])
      : "memory");
}

__device__ __forceinline__ void tc_st8(uint32_t taddr, const uint32_t (&r)[8]) {
  asm volatile("tcgen05.st.sync.aligned.32x32b.x8.b32 [%0], {%1,%2,%3,%4,%5,%6,%7,%8};" ::"r"(taddr),
      "r"(r[0]), "r"(r[1]), "r"(r[2]), "r"(r[3]), "r"(r[4]), "r"(r[5]), "r"(r[6]), "r"(r[7]) : "memory");
}
__device__ __forceinline__ void tc_ld8_nowait(uint32_t taddr, uint32_t (&r)[8]) {
  asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7])
               : "r"(taddr));
}

// Direct form: what a thread needs to store its part of a tile (its row,
// columns col0..col0+31), gathered once when the tile starts (while the
// tensor cores work on the tile's first level): the row's D offset and
// scale; the 32 columns' D bases and scales go to the warp's table in shared
// memory (read back as broadcasts).
struct DirectCol {
  double* colp;  // column base in D; null: column outside D
  int F;         // biased column exponent (at least 1)
  int pad;
};
// Energy form: a second per-warp table (only that kernel declares it, so the
// store forms keep their shared memory).
struct EnergyCol {
  double ec;  // the column's last-term orbital energy (when the last term is a column index)
  int ck;     // the column's index into the prefix table (-1: outside D)
  int pad;
};
struct DirectTile {
  long long roff;   // the row's offset from a column base
  DirectCol* cols;  // this warp's 32 entries
  int ebase;        // row scale and constant part of the result's exponent
  bool mlive;
  bool nonfinite;   // the row holds a non-finite operand value
  // energy form
  EnergyCol* ecols;    // this warp's 32 entries
  const double* prow;  // the row's prefix-table row
  double er;           // the row's last-term orbital energy (when the last term is a row index)
  bool last_row;
};

template <bool ENERGY>
__device__ __forceinline__ void direct_tile(DirectTile& t, const OzGemmArgs& a, const OzTile& tl, int row,
                                            int col0, int lane) {
  const OzDBlock db = a.dblocks[tl.dblock];
  const int m = tl.m0 + row, n = tl.n0 + col0 + lane;
  t.mlive = m < db.M;
  int Em = 1;
  t.roff = 0;
  t.nonfinite = false;
  [[maybe_unused]] OzEnergyBlock eb{};
  if constexpr (ENERGY) {
    eb = a.eblocks[tl.dblock];
    t.last_row = eb.last_row != 0;
    t.prow = eb.ptab;
    t.er = 0.0;
  }
  if (t.mlive) {
    const int e = a.panels_a[tl.panel_a].exps[m];
    Em = e ? e : 1;
    t.nonfinite = e == kNonFiniteExp;
    if constexpr (ENERGY) {
      t.prow = eb.ptab + int64_t(eb.rk[m]) * eb.ckn;
      if (t.last_row) t.er = eb.elast[m];
    } else {
      t.roff = db.rowoff[m];
    }
  }
  t.ebase = Em - 1022 - 1022 + 2 - kDigitBits * (a.slices + 1);
  DirectCol c{nullptr, 1, 0};
  [[maybe_unused]] EnergyCol ec{0.0, -1, 0};
  if (n < db.N) {
    const int f = a.panels_b[tl.panel_b].exps[n];
    c.F = f ? f : 1;
    if constexpr (ENERGY) {
      ec.ck = eb.ck[n];
      if (!eb.last_row) ec.ec = eb.elast[n];
    } else {
      c.colp = db.colptr[n];
    }
  }
  __syncwarp();  // the previous tile's entries are read
  t.cols[lane] = c;
  if constexpr (ENERGY) t.ecols[lane] = ec;
  __syncwarp();
}

// Accumulate mode: asks L2 for the thread's 32 D elements when the tile
// starts, so that the loads after its last chunk find them there.
__device__ __forceinline__ void prefetch_direct(const DirectTile& t) {
  if (!t.mlive) return;
#pragma unroll 8
  for (int j = 0; j < 32; ++j) {
    double* cp = t.cols[j].colp;
    if (cp) asm volatile("prefetch.global.L2 [%0];" ::"l"(cp + t.roff));
  }
}

__device__ __forceinline__ void load_d8(const DirectTile& t, int c0, bool acc, double (&d)[8]) {
#pragma unroll
  for (int j = 0; j < 8; ++j) {
    double* cp = t.cols[c0 + j].colp;
    d[j] = 0.0;
    if (acc && t.mlive && cp) d[j] = cp[t.roff];
  }
}

// Direct form, after the last chunk of a tile's last level: rounds the 32
// exact 64-bit sums of this thread's row held in TMEM (low words at w0addr,
// high words kTmemW1 - kTmemW0 columns further) to FP64 with the row and
// column scales and stores (or adds) them into D, 8 columns at a time; in the
// accumulate mode the next 8 D loads are in flight while 8 are added.
__device__ __forceinline__ void store_direct(const OzGemmArgs& a, const DirectTile& t, uint32_t w0addr) {
  if (a.dry) return;
  const bool acc = a.mode & 1;
  double dn[8];
  load_d8(t, 0, acc, dn);
#pragma unroll 1
  for (int p = 0; p < 4; ++p) {
    double dc[8];
#pragma unroll
    for (int j = 0; j < 8; ++j) dc[j] = dn[j];
    if (p < 3) load_d8(t, 8 * (p + 1), acc, dn);
    uint32_t w0[8], w1[8];
    tc_ld8_nowait(w0addr + 8 * p, w0);
    tc_ld8_nowait(w0addr + (kTmemW1 - kTmemW0) + 8 * p, w1);
    tc_wait_ld();
#pragma unroll
    for (int j = 0; j < 8; ++j) {
      const DirectCol c = t.cols[8 * p + j];
      const long long v = (long long)(((unsigned long long)w1[j] << 32) | w0[j]);
      double x = i64_scaled_to_double(v, t.ebase + c.F, a.mode & 2);
      if (t.nonfinite || c.F == kNonFiniteExp) x = __longlong_as_double(0x7FF8000000000000ll);
      if (t.mlive && c.colp) c.colp[t.roff] = acc ? dc[j] + x : x;
    }
  }
}

// Energy form, after the last chunk of a tile's last level: the same rounding
// of the 32 exact sums as store_direct, then per element (nothing stored)
//     acc += x * fl(x / eps),   eps = fl(prefix - e_last)
// in FP64: the prefix is the denominator chain without its last term, formed
// on the host in the reference's order; the quotient is the exactly rounded
// FP64 quotient (div_rn); zeros add nothing and skip the division.  A
// non-finite operand value in the row or column makes x (and the sum) NaN.
// Every lane of the warp runs the TMEM loads (.sync.aligned: the whole warp
// together); rows outside the block are skipped per element.
__device__ __forceinline__ void energy_direct(const OzGemmArgs& a, const DirectTile& t, uint32_t w0addr,
                                              double& acc) {
#pragma unroll 1
  for (int p = 0; p < 4; ++p) {
    uint32_t w0[8], w1[8];
    tc_ld8_nowait(w0addr + 8 * p, w0);
    tc_ld8_nowait(w0addr + (kTmemW1 - kTmemW0) + 8 * p, w1);
    tc_wait_ld();
#pragma unroll
    for (int j = 0; j < 8; ++j) {
      const EnergyCol ec = t.ecols[8 * p + j];
      if (!t.mlive || ec.ck < 0) continue;
      const int F = t.cols[8 * p + j].F;
      const long long v = (long long)(((unsigned long long)w1[j] << 32) | w0[j]);
      double x = i64_scaled_to_double(v, t.ebase + F, false);
      if (t.nonfinite || F == kNonFiniteExp) x = __longlong_as_double(0x7FF8000000000000ll);
      if (!nonzero(x)) continue;
      const double eps = __dsub_rn(t.prow[ec.ck], t.last_row ? t.er : ec.ec);
      acc = fma(x, div_rn(x, eps), acc);
    }
  }
}

// Eight warps, two per TMEM lane quadrant (warp % 4); each thread owns one
// accumulator row and 64 of its 128 columns, in two groups of 32.  The three
// TMEM loads of a group (chunk, hi, lo) are issued before one wait.  In the
// pair form each CTA drains its own 128 rows and signals the leader.
//
// Direct form: the running sum of a tile is the exact integer
//     sum_t S_t * 256^(slices-1-t)
// (Horner over the levels t, which arrive in order), kept as two 32-bit
// TMEM words per element; the host admits a batch to this form only when the
// sum stays below 2^63.  The last chunk of the last level is rounded once and
// stored into D.
template <bool PAIR, bool DIRECT, bool ENERGY = false>
__device__ void epilogue(const OzGemmArgs& a, OzSmemT<PAIR, 128>& sm, uint32_t tmem, int warp, int lane,
                         uint32_t rank) {
  constexpr int kRows = PAIR ? 2 * kOzBM : kOzBM;  // rows of a tile
  constexpr int kCols = DIRECT ? 32 : 64;          // columns of a thread
  const int q = warp & 3, h = (warp - 2) >> 2;
  const int row = int(rank) * kOzBM + 32 * q + lane;
  const uint32_t lane_addr = tmem + (uint32_t(32 * q) << 16) + uint32_t(kCols * h);
  uint32_t empty_bar[2];
  for (int b = 0; b < 2; ++b) empty_bar[b] = PAIR ? mapa_shared(&sm.acc_empty[b], 0) : smem_u32(&sm.acc_empty[b]);
  uint32_t chunk = 0;
  [[maybe_unused]] DirectTile dt{};
  [[maybe_unused]] double eacc = 0.0;
  if constexpr (DIRECT) {
    __shared__ DirectCol direct_cols[kThreadsOzDirect / 32 - 2][32];  // one table per epilogue warp
    dt.cols = direct_cols[warp - 2];
    if constexpr (ENERGY) {
      __shared__ EnergyCol energy_cols[kThreadsOzDirect / 32 - 2][32];
      dt.ecols = energy_cols[warp - 2];
    }
  }
  auto release = [&](uint32_t buf) {
    tc_fence_before();
    __syncwarp();
    if (lane == 0) {
      if constexpr (PAIR) mbar_arrive_cluster(empty_bar[buf]);
      else mbar_arrive(&sm.acc_empty[buf]);
    }
  };
  for_units<PAIR>(a, [&](int u) {
    const OzUnit un = a.units[u];
    const int ckb = a.chunk_kb[un.level];
    const int nchunks = (un.kb_end - un.kb_begin + ckb - 1) / ckb;
    if constexpr (DIRECT) {
      const bool last_level = un.level == a.slices - 1;
      if (un.level == 0) {
        direct_tile<ENERGY>(dt, a, a.tiles[un.tile], row, kCols * h, lane);
        if constexpr (!ENERGY)
          if ((a.mode & 1) && !a.dry) prefetch_direct(dt);
      }
      for (int c = 0; c < nchunks; ++c) {
        const uint32_t buf = chunk & 1;
        if (!mbar_wait(&sm.acc_full[buf], (chunk >> 1) & 1, sm, a.err_flag, 4)) return false;
        tc_fence_after();
        const bool fresh = c == 0 && un.level == 0;  // no running sum yet
        const uint32_t mul = c == 0 ? 256u : 1u;     // a new level: running sum * 256
        const bool final = last_level && c == nchunks - 1;
#pragma unroll 1
        for (int g = 0; g < 4; ++g) {
          uint32_t x[8], w0[8], w1[8];
          tc_ld8_nowait(lane_addr + buf * kOzBN + 8 * g, x);
          if (!fresh) {
            tc_ld8_nowait(lane_addr + kTmemW0 + 8 * g, w0);
            tc_ld8_nowait(lane_addr + kTmemW1 + 8 * g, w1);
          } else {
#pragma unroll
            for (int j = 0; j < 8; ++j) w0[j] = w1[j] = 0u;
          }
          tc_wait_ld();
#pragma unroll
          for (int j = 0; j < 8; ++j) {
            // (w1:w0) * mul + x modulo 2^64 in 32-bit multiply-adds (x is an
            // integer below 2^24, exact in FP32): low word with its carry, then
            // the high word
            const unsigned long long lo =
                (unsigned long long)w0[j] * mul + (unsigned long long)(long long)__float2int_rz(__uint_as_float(x[j]));
            w0[j] = uint32_t(lo);
            w1[j] = w1[j] * mul + uint32_t(lo >> 32);
          }
          tc_st8(lane_addr + kTmemW0 + 8 * g, w0);
          tc_st8(lane_addr + kTmemW1 + 8 * g, w1);
        }
        tc_wait_st();
        release(buf);  // the next MMAs may start while this thread stores D
        ++chunk;
        if (final) {
          if constexpr (ENERGY) energy_direct(a, dt, lane_addr + kTmemW0, eacc);
          else store_direct(a, dt, lane_addr + kTmemW0);
        }
      }
      return true;
    } else {
    int* w = a.ws + ((size_t(un.tile) * a.slices + un.level) * a.nsplit + un.split) * kOzBN * kRows +
             size_t(64 * h) * kRows + row;
    if (nchunks == 0) {  // empty k range: its partial sum is zero
#pragma unroll 8
      for (int j = 0; j < 64; ++j) w[size_t(j) * kRows] = 0;
      return true;
    }
    for (int c = 0; c < nchunks; ++c) {
      const uint32_t buf = chunk & 1;
      if (!mbar_wait(&sm.acc_full[buf], (chunk >> 1) & 1, sm, a.err_flag, 4)) return false;
      tc_fence_after();
      const bool first = c == 0, last = c == nchunks - 1;
#pragma unroll 1
      for (int g = 0; g < 2; ++g) {
        uint32_t x[32], hi[32], lo[32];
        tc_ld32_nowait(lane_addr + buf * kOzBN + 32 * g, x);
        if (!first) {
          tc_ld32_nowait(lane_addr + kTmemHi + 32 * g, hi);
          tc_ld32_nowait(lane_addr + kTmemLo + 32 * g, lo);
        }
        tc_wait_ld();
        if (first) {
#pragma unroll
          for (int j = 0; j < 32; ++j) hi[j] = x[j], lo[j] = 0u;
        } else {
#pragma unroll
          for (int j = 0; j < 32; ++j) {
            float hv = __uint_as_float(hi[j]), lv = __uint_as_float(lo[j]);
            two_sum_acc(hv, lv, __uint_as_float(x[j]));
            hi[j] = __float_as_uint(hv), lo[j] = __float_as_uint(lv);
          }
        }
        if (!last) {
          tc_st32(lane_addr + kTmemHi + 32 * g, hi);
          tc_st32(lane_addr + kTmemLo + 32 * g, lo);
        } else {
          // hi + lo is the unit's exact level sum, an integer below 2^31 (the
          // host sizes units for that), stored as int32
#pragma unroll
          for (int j = 0; j < 32; ++j)
            w[size_t(32 * g + j) * kRows] =
                int(static_cast<long long>(__uint_as_float(hi[j])) + static_cast<long long>(__uint_as_float(lo[j])));
        }
      }
      if (!last) tc_wait_st();
      release(buf);
      ++chunk;
    }
    return true;
    }
  });
  if constexpr (ENERGY) a.epart[(size_t(blockIdx.x) * 16 + size_t(warp - 2)) * 32 + lane] = eacc;
}

// 256-column tiles: the two FP32 accumulators use all 512 TMEM columns, so the
// exact running level sum of a unit lives in registers as int32 (a unit's
// level sum is an integer below 2^31 and every chunk value below 2^24, so the
// conversion and the additions are exact).  Eight warps, two per lane
// quadrant; each thread owns one row and 128 columns, read 16 at a time.
template <bool PAIR>
__device__ void epilogue_int(const OzGemmArgs& a, OzSmemT<PAIR, 256>& sm, uint32_t tmem, int warp, int lane,
                             uint32_t rank) {
  constexpr int BN = 256;
  constexpr int kRows = PAIR ? 2 * kOzBM : kOzBM;
  const int q = warp & 3, h = (warp - 2) >> 2;
  const int row = int(rank) * kOzBM + 32 * q + lane;
  const uint32_t lane_addr = tmem + (uint32_t(32 * q) << 16) + uint32_t(128 * h);
  uint32_t empty_bar[2];
  for (int b = 0; b < 2; ++b) empty_bar[b] = PAIR ? mapa_shared(&sm.acc_empty[b], 0) : smem_u32(&sm.acc_empty[b]);
  uint32_t chunk = 0;
  for_units<PAIR>(a, [&](int u) {
    const OzUnit un = a.units[u];
    const int ckb = a.chunk_kb[un.level];
    const int nchunks = (un.kb_end - un.kb_begin + ckb - 1) / ckb;
    int* w = a.ws + ((size_t(un.tile) * a.slices + un.level) * a.nsplit + un.split) * BN * kRows +
             size_t(128 * h) * kRows + row;
    int sum[128];
#pragma unroll
    for (int j = 0; j < 128; ++j) sum[j] = 0;
    for (int c = 0; c < nchunks; ++c) {
      const uint32_t buf = chunk & 1;
      if (!mbar_wait(&sm.acc_full[buf], (chunk >> 1) & 1, sm, a.err_flag, 4)) return false;
      tc_fence_after();
#pragma unroll
      for (int g = 0; g < 8; ++g) {
        uint32_t x[16];
        tc_ld16_nowait(lane_addr + buf * BN + 16 * g, x);
        tc_wait_ld();
#pragma unroll
        for (int j = 0; j < 16; ++j) sum[16 * g + j] += __float2int_rz(__uint_as_float(x[j]));
      }
      tc_fence_before();
      __syncwarp();
      if (lane == 0) {
        if constexpr (PAIR) mbar_arrive_cluster(empty_bar[buf]);
        else mbar_arrive(&sm.acc_empty[buf]);
      }
      ++chunk;
    }
#pragma unroll
    for (int j = 0; j < 128; ++j) w[size_t(j) * kRows] = sum[j];
    return true;
  });
}

template <bool PAIR, int BN, bool DIRECT = false, bool ENERGY = false>
__global__ void __launch_bounds__(DIRECT ? kThreadsOzDirect : kThreadsOz, 1)
    oz_gemm_kernel(const __grid_constant__ OzGemmArgs a) {
  using SM = OzSmemT<PAIR, BN>;
  extern __shared__ uint8_t smem_raw[];
  SM& sm = *reinterpret_cast<SM*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const uint32_t rank = PAIR ? cluster_rank() : 0u;
  if (threadIdx.x == 0) {
    for (int s = 0; s < SM::kSt; ++s) {
      mbar_init(&sm.full[s], PAIR ? 2 : 1);  // pair form: one expect_tx arrive from each CTA
      mbar_init(&sm.empty[s], 1);
    }
    for (int b = 0; b < 2; ++b) {
      mbar_init(&sm.acc_full[b], 1);
      // one arrive per epilogue warp (of both CTAs)
      mbar_init(&sm.acc_empty[b], (DIRECT ? 16 : 8) * (PAIR ? 2 : 1));
    }
    mbar_init(&sm.drain, 1);
    sm.abort = 0;
    fence_mbar_init();
  }
  if (warp == 1) {
    if constexpr (PAIR) {
      asm volatile("tcgen05.alloc.cta_group::2.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                       smem_u32(&sm.tmem_base)),
                   "r"(kTmemCols));
      asm volatile("tcgen05.relinquish_alloc_permit.cta_group::2.sync.aligned;");
    } else {
      asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                       smem_u32(&sm.tmem_base)),
                   "r"(kTmemCols));
      asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
  }
  tc_fence_before();
  __syncthreads();
  if constexpr (PAIR) cluster_sync();  // the peer's barriers exist before anyone signals them
  tc_fence_after();
  const uint32_t tmem = sm.tmem_base;

  if (warp == 0) {
    if (lane == 0) producer<PAIR, BN>(a, sm, rank);
  } else if (warp == 1) {
    if (lane == 0 && rank == 0) {
      mma_issuer<PAIR, BN>(a, sm, tmem);
      // all MMAs this thread issued have completed before TMEM is released
      if constexpr (PAIR) tc_commit_pair(&sm.drain);
      else tc_commit(&sm.drain);
      mbar_wait(&sm.drain, 0, sm, a.err_flag, 5);
    }
  } else {
    if constexpr (BN == 256) epilogue_int<PAIR>(a, sm, tmem, warp, lane, rank);
    else epilogue<PAIR, DIRECT, ENERGY>(a, sm, tmem, warp, lane, rank);
  }
  tc_fence_before();
  __syncthreads();
  if constexpr (PAIR) cluster_sync();  // the leader's MMAs have read this CTA's smem and TMEM
  if (warp == 1) {
    tc_fence_after();
    if constexpr (PAIR)
      asm volatile("tcgen05.dealloc.cta_group::2.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kTmemCols));
    else
      asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kTmemCols));
  }
}

// ------------------------------------------------------------------ all levels at once
// Form of the direct GEMM for sub-problems whose k range fits one exact FP32
// flush per level (at most 5 slices, k at most 320): every level accumulator
// of a 128 x 64 tile lives in TMEM at once (levels 0-2 one each; levels 3 and
// 4, whose sums over 320 k could pass 2^24, one per half of the k range:
// 7 x 64 = 448 columns).  Each 32-wide k block of the tile's S A-slices and S
// B-slices is then loaded once for all S (S + 1) / 2 slice pairs, where the
// level-by-level form loads two tiles per pair.  When the tile's MMAs
// complete, the epilogue reads each accumulator once, forms the exact sum
// over levels (the same 64-bit integer as the level-by-level Horner sum) in
// registers and releases TMEM before it rounds and divides, sums or stores:
// the tensor cores run the next tile meanwhile.
constexpr int kLvBN = 64, kLvBK = 32, kLvMaxS = 5, kLvSt = 3, kLvAcc = 7;
constexpr uint32_t kLvATile = kOzBM * kLvBK * 2;  // 8 KB: 128 rows x 32 k
constexpr uint32_t kLvBTile = kLvBN * kLvBK * 2;  // 4 KB: 64 columns x 32 k
struct __align__(1024) LvSmem {
  uint8_t a[kLvSt][kLvMaxS][kLvATile];
  uint8_t b[kLvSt][kLvMaxS][kLvBTile];
  uint64_t full[kLvSt], empty[kLvSt];
  uint64_t acc_full, acc_empty, drain;
  uint32_t tmem_base;
  volatile int abort;
};
static_assert(kLvBN == kOzLevelsTileCols, "tile columns of the all-levels form");
// TMEM accumulator (in 64-column units) of level t; levels 3 and 4: of k half h.
__device__ __forceinline__ int lv_acc(int t, int h) { return t < 3 ? t : 2 * t - 3 + h; }

// Shared-memory matrix descriptor: K-major, 64-byte swizzle, rows of 64 B,
// 8-row core groups 512 B apart.
__device__ __forceinline__ uint64_t sw64_desc(const void* tile) {
  const uint32_t addr = smem_u32(tile);
  uint64_t d = uint64_t((addr & 0x3FFFF) >> 4);
  d |= uint64_t(1) << 16;          // leading byte offset (unused for swizzled K-major)
  d |= uint64_t(512 >> 4) << 32;   // stride byte offset
  d |= uint64_t(1) << 46;
  d |= uint64_t(4) << 61;          // SWIZZLE_64B
  return d;
}

// Per 32-wide k block of a tile, one stage: the S A-slices (rows m0..m0+127)
// and the S B-slices (columns n0..n0+63).
__device__ void lv_producer(const OzGemmArgs& a, LvSmem& sm) {
  const int S = a.slices;
  const uint32_t bytes = uint32_t(S) * (kLvATile + kLvBTile);
  uint32_t it = 0;
  for (int g = int(blockIdx.x); g < a.n_tiles; g += int(gridDim.x)) {
    const OzTile tl = a.tiles[g];
    const void* ma = static_cast<const uint8_t*>(a.maps_a) + size_t(tl.panel_a) * 128;
    const void* mb = static_cast<const uint8_t*>(a.maps_b) + size_t(tl.panel_b) * 128;
    const int rpa = a.panels_a[tl.panel_a].rows_pad, rpb = a.panels_b[tl.panel_b].rows_pad;
    for (int q = tl.trip_begin; q < tl.trip_end; ++q) {
      const OzTrip tr = a.trips[q];
      for (int j = 0; j < 2 * tr.nkb; ++j) {
        const int s = int(it % kLvSt);
        const uint32_t ph = (it / kLvSt) & 1;
        if (!mbar_wait(&sm.empty[s], ph ^ 1, sm, a.err_flag, 1)) return;
        mbar_expect_tx(&sm.full[s], bytes);
        const int ka = int(tr.koff_a) + j * kLvBK, kb = int(tr.koff_b) + j * kLvBK;
        for (int i = 0; i < S; ++i) {
          tma_load_2d(sm.a[s][i], ma, &sm.full[s], ka, i * rpa + tl.m0);
          tma_load_2d(sm.b[s][i], mb, &sm.full[s], kb, i * rpb + tl.n0);
        }
        ++it;
      }
    }
  }
}

// One thread issues every MMA: per stage, slice pair (i, j) with i + j < S
// into the accumulator of level i + j (k half h for levels 3 and 4: the
// tile's 2 kb_total 32-wide blocks split in two equal halves, at most 160 k
// each).  The first MMA into an accumulator overwrites it.
__device__ void lv_mma(const OzGemmArgs& a, LvSmem& sm, uint32_t tmem) {
  const int S = a.slices;
  uint32_t it = 0, nt = 0;
  for (int g = int(blockIdx.x); g < a.n_tiles; g += int(gridDim.x), ++nt) {
    const OzTile tl = a.tiles[g];
    const int half = tl.kb_total;
    if (!mbar_wait(&sm.acc_empty, (nt & 1) ^ 1, sm, a.err_flag, 2)) return;
    tc_fence_after();
    int kb = 0;
    for (int q = tl.trip_begin; q < tl.trip_end; ++q) {
      const int nk = 2 * a.trips[q].nkb;
      for (int j = 0; j < nk; ++j, ++kb) {
        const int s = int(it % kLvSt);
        const uint32_t ph = (it / kLvSt) & 1;
        if (!mbar_wait(&sm.full[s], ph, sm, a.err_flag, 3)) return;
        tc_fence_after();
        // one issue slot per MMA: the slices' descriptors are the stage's first
        // plus the tile offset (in 16-byte units), the accumulator columns and
        // the overwrite flags fixed per stage
        const uint32_t h64 = kb >= half ? uint32_t(kLvBN) : 0u;  // levels 3, 4: second k half
        const uint32_t acc_lo = kb == 0 ? 0u : 1u;                // levels 0-2: overwrite at the first block
        const uint32_t acc_hi = kb == 0 || kb == half ? 0u : 1u;  // levels 3, 4: at the first block of a half
        const uint64_t ad0 = sw64_desc(sm.a[s][0]), bd0 = sw64_desc(sm.b[s][0]);
#pragma unroll
        for (int i = 0; i < kLvMaxS; ++i) {
#pragma unroll
          for (int jj = 0; jj < kLvMaxS - i; ++jj) {
            const int t = i + jj;
            if (t >= S) continue;
            const uint32_t d = tmem + uint32_t(kLvBN * lv_acc(t, 0)) + (t >= 3 ? h64 : 0u);
            const uint32_t acc = i > 0 ? 1u : (t < 3 ? acc_lo : acc_hi);
            const uint64_t ad = ad0 + uint64_t(i) * (kLvATile >> 4), bd = bd0 + uint64_t(jj) * (kLvBTile >> 4);
            tc_mma<kLvBN>(d, ad, bd, acc);
            tc_mma<kLvBN>(d, ad + 2, bd + 2, 1u);  // the block's second 16 k: 32 B further
          }
        }
        tc_commit(&sm.empty[s]);
        ++it;
      }
    }
    tc_commit(&sm.acc_full);
  }
}

// What a thread needs of one of its warp's 16 columns (a table per warp in
// shared memory, filled while the tensor cores work on the tile).
struct LvCol {
  double* colp;  // store form: column base in D (null: outside D)
  double ec;     // energy form: the column's last-term orbital energy
  int F;         // biased column exponent (at least 1)
  int ck;        // energy form: prefix-table column (-1: outside D)
};

// Sixteen warps, four per TMEM lane quadrant; a thread owns one row and 16
// columns.  Per tile: the row's scale and tables, the 16 columns' table, the
// wait for the tile's MMAs, the exact sums (two groups of 8 columns, each
// accumulator read once), TMEM released, then per element the rounding to
// FP64 with the row and column scales and
//   energy form: acc += x * fl(x / eps), eps = fl(prefix - e_last)
//   (the chain without its last term tabulated in the reference's order; the
//   quotient exactly rounded; zeros add nothing);
//   store form: D = x or D += x.
// A non-finite operand value in the row or column makes x NaN.
template <bool ENERGY>
__device__ void lv_epilogue(const OzGemmArgs& a, LvSmem& sm, uint32_t tmem, int warp, int lane) {
  __shared__ LvCol lv_cols[kThreadsOzDirect / 32 - 2][16];
  LvCol* tab = lv_cols[warp - 2];
  const int q = warp & 3, h = (warp - 2) >> 2;
  const int row = 32 * q + lane;
  const uint32_t lane_addr = tmem + (uint32_t(32 * q) << 16) + uint32_t(16 * h);
  const int S = a.slices;
  [[maybe_unused]] double eacc = 0.0;
  uint32_t nt = 0;
  for (int g = int(blockIdx.x); g < a.n_tiles; g += int(gridDim.x), ++nt) {
    const OzTile tl = a.tiles[g];
    const OzDBlock db = a.dblocks[tl.dblock];
    const int m = tl.m0 + row;
    const bool mlive = m < db.M;
    int Em = 1;
    bool nonfinite = false;
    [[maybe_unused]] long long roff = 0;
    [[maybe_unused]] const double* prow = nullptr;
    [[maybe_unused]] double er = 0.0;
    [[maybe_unused]] bool last_row = false;
    [[maybe_unused]] OzEnergyBlock eb{};
    if constexpr (ENERGY) {
      eb = a.eblocks[tl.dblock];
      last_row = eb.last_row != 0;
    }
    if (mlive) {
      const int e = a.panels_a[tl.panel_a].exps[m];
      Em = e ? e : 1;
      nonfinite = e == kNonFiniteExp;
      if constexpr (ENERGY) {
        prow = eb.ptab + int64_t(eb.rk[m]) * eb.ckn;
        if (last_row) er = eb.elast[m];
      } else {
        roff = db.rowoff[m];
      }
    }
    const int ebase = Em - 1022 - 1022 + 2 - kDigitBits * (S + 1);
    __syncwarp();  // the previous tile's entries are read
    if (lane < 16) {
      const int n = tl.n0 + 16 * h + lane;
      LvCol c{nullptr, 0.0, 1, -1};
      if (n < db.N) {
        const int f = a.panels_b[tl.panel_b].exps[n];
        c.F = f ? f : 1;
        if constexpr (ENERGY) {
          c.ck = eb.ck[n];
          if (!last_row) c.ec = eb.elast[n];
        } else {
          c.colp = db.colptr[n];
        }
      }
      tab[lane] = c;
    }
    __syncwarp();
    if (!mbar_wait(&sm.acc_full, nt & 1, sm, a.err_flag, 4)) break;
    tc_fence_after();
    long long sum[16];
#pragma unroll
    for (int gg = 0; gg < 2; ++gg) {
      uint32_t v[kLvAcc][8];
#pragma unroll
      for (int c = 0; c < kLvAcc; ++c) tc_ld8_nowait(lane_addr + uint32_t(kLvBN * c + 8 * gg), v[c]);
      tc_wait_ld();
#pragma unroll
      for (int j = 0; j < 8; ++j) {
        // sum_t S_t 256^(S-1-t), S_t an integer below 2^24 in FP32 (levels
        // 3 and 4: the sum of the two halves)
        long long r = 0;
#pragma unroll
        for (int t = 0; t < kLvMaxS; ++t)
          if (t < S) {
            long long st = __float2int_rz(__uint_as_float(v[lv_acc(t, 0)][j]));
            if (t >= 3) st += __float2int_rz(__uint_as_float(v[lv_acc(t, 1)][j]));
            r = r * 256 + st;
          }
        sum[8 * gg + j] = r;
      }
    }
    tc_fence_before();
    __syncwarp();
    if (lane == 0) mbar_arrive(&sm.acc_empty);  // the next tile's MMAs may start
    if constexpr (ENERGY) {
#pragma unroll
      for (int j = 0; j < 16; ++j) {
        const LvCol c = tab[j];
        if (!mlive || c.ck < 0) continue;
        double x = i64_scaled_to_double(sum[j], ebase + c.F, false);
        if (nonfinite || c.F == kNonFiniteExp) x = __longlong_as_double(0x7FF8000000000000ll);
        if (!nonzero(x)) continue;
        const double eps = __dsub_rn(prow[c.ck], last_row ? er : c.ec);
        eacc = fma(x, div_rn(x, eps), eacc);
      }
    } else {
      const bool acc = a.mode & 1;
#pragma unroll
      for (int j = 0; j < 16; ++j) {
        const LvCol c = tab[j];
        if (!mlive || !c.colp) continue;
        double x = i64_scaled_to_double(sum[j], ebase + c.F, a.mode & 2);
        if (nonfinite || c.F == kNonFiniteExp) x = __longlong_as_double(0x7FF8000000000000ll);
        double* p = c.colp + roff;
        *p = acc ? *p + x : x;
      }
    }
  }
  if constexpr (ENERGY) a.epart[(size_t(blockIdx.x) * 16 + size_t(warp - 2)) * 32 + lane] = eacc;
}

template <bool ENERGY>
__global__ void __launch_bounds__(kThreadsOzDirect, 1) oz_levels_kernel(const __grid_constant__ OzGemmArgs a) {
  extern __shared__ uint8_t smem_raw[];
  LvSmem& sm = *reinterpret_cast<LvSmem*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (threadIdx.x == 0) {
    for (int s = 0; s < kLvSt; ++s) {
      mbar_init(&sm.full[s], 1);
      mbar_init(&sm.empty[s], 1);
    }
    mbar_init(&sm.acc_full, 1);
    mbar_init(&sm.acc_empty, 16);  // one arrive per epilogue warp
    mbar_init(&sm.drain, 1);
    sm.abort = 0;
    fence_mbar_init();
  }
  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&sm.tmem_base)),
                 "r"(kTmemCols));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = sm.tmem_base;
  if (warp == 0) {
    if (lane == 0) lv_producer(a, sm);
  } else if (warp == 1) {
    if (lane == 0) {
      lv_mma(a, sm, tmem);
      tc_commit(&sm.drain);  // all MMAs this thread issued have completed before TMEM is released
      mbar_wait(&sm.drain, 0, sm, a.err_flag, 5);
    }
  } else {
    lv_epilogue<ENERGY>(a, sm, tmem, warp, lane);
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 1) {
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kTmemCols));
  }
}

// ------------------------------------------------------------------ split side
// Tiles of 64 rows x 64 k over the jobs; job_tiles[j] is the prefix count.
__device__ __forceinline__ int find_job(const int64_t* prefix, int njobs, int64_t t) {
  int lo = 0, hi = njobs;  // prefix[lo] <= t < prefix[hi]
  while (hi - lo > 1) {
    const int mid = (lo + hi) >> 1;
    if (prefix[mid] <= t) lo = mid;
    else hi = mid;
  }
  return lo;
}

constexpr int kSplitT = 64;

// Loads one 64x64 (row, k) tile of a job into shared memory as raw bits.
__device__ __forceinline__ void load_job_tile(const OzSplitJob& jb, int r0, int k0,
                                              unsigned long long (*tile)[kSplitT + 1]) {
  const int t = threadIdx.x;  // 256 threads
  for (int p = 0; p < 16; ++p) {
    int r, k;
    if (jb.kfast) {
      k = t & 63;
      r = (t >> 6) + 4 * p;
    } else {
      r = t & 63;
      k = (t >> 6) + 4 * p;
    }
    unsigned long long v = 0;
    if (r0 + r < jb.rows && k0 + k < jb.K)
      v = __double_as_longlong(__ldg(&jb.src[__ldg(&jb.offRow[r0 + r]) + __ldg(&jb.offK[k0 + k])]));
    tile[r][k] = v ^ (jb.negate ? (1ull << 63) : 0ull);  // -x: the sign bit (exponents unchanged)
  }
}

__global__ void __launch_bounds__(256) oz_exp_kernel(const OzSplitJob* __restrict__ jobs,
                                                     const int64_t* __restrict__ prefix, int njobs,
                                                     const OzPanel* __restrict__ panels) {
  __shared__ unsigned long long tile[kSplitT][kSplitT + 1];
  const int64_t t = blockIdx.x;
  const int j = find_job(prefix, njobs, t);
  const OzSplitJob jb = jobs[j];
  const int64_t local = t - prefix[j];
  const int ktiles = (jb.K + kSplitT - 1) / kSplitT;
  const int r0 = int(local / ktiles) * kSplitT, k0 = int(local % ktiles) * kSplitT;
  load_job_tile(jb, r0, k0, tile);
  __syncthreads();
  // 4 threads per row, 16 k each
  const int r = threadIdx.x >> 2, part = threadIdx.x & 3;
  int m = 0;
  for (int k = part * 16; k < part * 16 + 16; ++k) m = max(m, int((tile[r][k] >> 52) & 0x7FF));
  m = max(m, __shfl_xor_sync(0xffffffffu, m, 1));
  m = max(m, __shfl_xor_sync(0xffffffffu, m, 2));
  if (part == 0 && r0 + r < jb.rows && m > 0) atomicMax(&panels[jb.panel].exps[r0 + r], m);
}

// Signed fixed-point value of one double against its row exponent (biased
// max exponent mx, |x| < 2^E with E = mx - 1022):
//     n = round_half_away(x * 2^(8*slices - E - 1)),   |n| <= 2^(8*slices - 1).
__device__ __forceinline__ long long quantize(unsigned long long bits, int mx, int slices) {
  const int be = int((bits >> 52) & 0x7FF);
  const unsigned long long frac = bits & ((1ull << 52) - 1);
  const unsigned long long mant = be ? (frac | (1ull << 52)) : frac;
  const int ex = be ? be : 1;
  const int E = (mx ? mx : 1) - 1022;
  const int sh = ex - 1076 + kDigitBits * slices - E;  // |x| * 2^(8s-E-1) = mant * 2^sh
  unsigned long long m;
  if (sh >= 0) m = mant << sh;  // only for 7 slices: sh <= 2, mant << 2 < 2^55
  else if (-sh >= 63) m = 0ull;
  else m = (mant + (1ull << (-sh - 1))) >> (-sh);
  return (bits >> 63) ? -static_cast<long long>(m) : static_cast<long long>(m);
}

// Balanced base-256 digits of n, most significant first: d[0] in [-128, 128],
// the others in [-128, 127]; sum_i d[i] * 256^(S-1-i) == n.  The low 24 bits
// give up to three digits with 32-bit arithmetic; the rest (|n| < 2^47 for up
// to 6 slices) also stays in 32 bits, only 7 slices need 64-bit steps.  S is
// a compile-time constant so every digit lives in a register.
template <int S>
__device__ __forceinline__ void balanced_digits(long long n, int (&d)[S]) {
  constexpr int K = S - 1 < 3 ? S - 1 : 3;  // digits taken from the low 24 bits
  int x = int(n & 0xFFFFFF);
  const long long hi = n >> 24;  // arithmetic shift: n == hi * 2^24 + x
#pragma unroll
  for (int t = 0; t < K; ++t) {
    const int r = ((x + 128) & 255) - 128;
    d[S - 1 - t] = r;
    x = (x - r) >> 8;
  }
  if constexpr (S <= 6) {
    int rem = int(hi << (24 - 8 * K)) + x;
#pragma unroll
    for (int t = K; t < S - 1; ++t) {
      const int r = ((rem + 128) & 255) - 128;
      d[S - 1 - t] = r;
      rem = (rem - r) >> 8;
    }
    d[0] = rem;
  } else {
    long long rem = (hi << (24 - 8 * K)) + x;
#pragma unroll
    for (int t = K; t < S - 1; ++t) {
      const long long r = ((rem + 128) & 255) - 128;
      d[S - 1 - t] = int(r);
      rem = (rem - r) >> 8;
    }
    d[0] = int(rem);
  }
}

// Exact BF16 bits of two digits in [-128, 128]: float(d) is formed exactly as
// (2^23 + 256 + d) - (2^23 + 256); one cvt.rn.bf16x2.f32 packs the pair (exact,
// at most 8 significant bits).
__device__ __forceinline__ uint32_t digits_bf16x2(int d0, int d1) {
  const float f0 = __fsub_rn(__uint_as_float(0x4B000000u + uint32_t(d0 + 256)), 8388864.0f);
  const float f1 = __fsub_rn(__uint_as_float(0x4B000000u + uint32_t(d1 + 256)), 8388864.0f);
  __nv_bfloat162 h = __floats2bfloat162_rn(f0, f1);
  return *reinterpret_cast<uint32_t*>(&h);
}

template <int S>
__global__ void __launch_bounds__(256) oz_split_kernel(const OzSplitJob* __restrict__ jobs,
                                                       const int64_t* __restrict__ prefix, int njobs,
                                                       const OzPanel* __restrict__ panels) {
  __shared__ unsigned long long tile[kSplitT][kSplitT + 1];
  const int64_t t = blockIdx.x;
  const int j = find_job(prefix, njobs, t);
  const OzSplitJob jb = jobs[j];
  const int64_t local = t - prefix[j];
  const int ktiles = (jb.K + kSplitT - 1) / kSplitT;
  const int r0 = int(local / ktiles) * kSplitT, k0 = int(local % ktiles) * kSplitT;
  load_job_tile(jb, r0, k0, tile);
  __syncthreads();
  const OzPanel pn = panels[jb.panel];
  // each thread: one row, two consecutive k -> one bf16x2 store per slice
  const int kp = threadIdx.x & 31;
  for (int p = 0; p < 8; ++p) {
    const int r = (threadIdx.x >> 5) + 8 * p;
    if (r0 + r >= jb.rows) continue;
    const int k = 2 * kp;
    if (k0 + k >= jb.K) continue;
    const int mx = pn.exps[r0 + r];
    const unsigned long long b0 = tile[r][k], b1 = (k0 + k + 1 < jb.K) ? tile[r][k + 1] : 0ull;
    int d0[S], d1[S];
    balanced_digits<S>(quantize(b0, mx, S), d0);
    balanced_digits<S>(quantize(b1, mx, S), d1);
    uint32_t* dst = reinterpret_cast<uint32_t*>(pn.base + (size_t(r0 + r) * pn.kpad + jb.koff + k0 + k));
    const size_t slice_stride = size_t(pn.rows_pad) * pn.kpad / 2;
#pragma unroll
    for (int i = 0; i < S; ++i) dst[i * slice_stride] = digits_bf16x2(d0[i], d1[i]);
  }
}

// ------------------------------------------------------------------ fast split paths
// Row maxima of a column-major [rows x K] block (rows contiguous): each thread
// owns two rows (one 16-byte load per k) over a 64-wide k range.
__global__ void __launch_bounds__(256) oz_exp_rows_kernel(const OzSplitJob* __restrict__ jobs,
                                                          const int64_t* __restrict__ prefix, int njobs,
                                                          const OzPanel* __restrict__ panels) {
  const int j = find_job(prefix, njobs, blockIdx.x);
  const OzSplitJob jb = jobs[j];
  const int64_t local = int64_t(blockIdx.x) - prefix[j];
  const int ktiles = (jb.K + 63) / 64;
  const int r = int(local / ktiles) * 512 + 2 * threadIdx.x;
  const int k0 = int(local % ktiles) * 64;
  if (r >= jb.rows) return;
  const int k1 = min(jb.K, k0 + 64);
  const bool pair = r + 1 < jb.rows && (jb.rows & 1) == 0;
  unsigned long long m0 = 0, m1 = 0;
  const double* base = jb.src + r;
  if (pair) {
#pragma unroll 8
    for (int k = k0; k < k1; ++k) {
      const double2 v = __ldg(reinterpret_cast<const double2*>(base + size_t(k) * jb.rows));
      m0 = max(m0, __double_as_longlong(v.x) & 0x7FF0000000000000ull);
      m1 = max(m1, __double_as_longlong(v.y) & 0x7FF0000000000000ull);
    }
  } else {
    for (int k = k0; k < k1; ++k) {
      m0 = max(m0, __double_as_longlong(__ldg(base + size_t(k) * jb.rows)) & 0x7FF0000000000000ull);
      if (r + 1 < jb.rows)
        m1 = max(m1, __double_as_longlong(__ldg(base + 1 + size_t(k) * jb.rows)) & 0x7FF0000000000000ull);
    }
  }
  int* e = panels[jb.panel].exps;
  if (m0) atomicMax(&e[r], int(m0 >> 52));
  if (m1 && r + 1 < jb.rows) atomicMax(&e[r + 1], int(m1 >> 52));
}

// Row maxima of a [K x rows] block (k contiguous): one warp per row.
__global__ void __launch_bounds__(256) oz_exp_kmaj_kernel(const OzSplitJob* __restrict__ jobs,
                                                          const int64_t* __restrict__ prefix, int njobs,
                                                          const OzPanel* __restrict__ panels) {
  const int j = find_job(prefix, njobs, blockIdx.x);
  const OzSplitJob jb = jobs[j];
  const int64_t local = int64_t(blockIdx.x) - prefix[j];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  int* e = panels[jb.panel].exps;
  const bool vec = (jb.K & 1) == 0;
  for (int rr = 0; rr < 4; ++rr) {
    const int r = int(local) * 32 + warp * 4 + rr;
    if (r >= jb.rows) return;
    const double* row = jb.src + size_t(r) * jb.K;
    unsigned long long m = 0;
    if (vec) {
      const double2* row2 = reinterpret_cast<const double2*>(row);
#pragma unroll 4
      for (int k = lane; k < jb.K / 2; k += 32) {
        const double2 v = __ldg(row2 + k);
        m = max(m, max(__double_as_longlong(v.x) & 0x7FF0000000000000ull,
                       __double_as_longlong(v.y) & 0x7FF0000000000000ull));
      }
    } else {
      for (int k = lane; k < jb.K; k += 32)
        m = max(m, __double_as_longlong(__ldg(row + k)) & 0x7FF0000000000000ull);
    }
    for (int o = 16; o > 0; o >>= 1) m = max(m, __shfl_xor_sync(0xffffffffu, m, o));
    if (lane == 0 && m) atomicMax(&e[r], int(m >> 52));
  }
}

// Slices of a [K x rows] block: one warp per row, each lane four consecutive k
// (two 16-byte loads, one 8-byte store per slice).
template <int S>
__global__ void __launch_bounds__(256) oz_split_kmaj_kernel(const OzSplitJob* __restrict__ jobs,
                                                            const int64_t* __restrict__ prefix, int njobs,
                                                            const OzPanel* __restrict__ panels) {
  const int j = find_job(prefix, njobs, blockIdx.x);
  const OzSplitJob jb = jobs[j];
  const int64_t local = int64_t(blockIdx.x) - prefix[j];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int r = int(local) * 8 + warp;
  if (r >= jb.rows) return;
  const OzPanel pn = panels[jb.panel];
  const int mx = pn.exps[r];
  const double* row = jb.src + size_t(r) * jb.K;
  uint2* dst = reinterpret_cast<uint2*>(pn.base + (size_t(r) * pn.kpad + jb.koff));
  const size_t slice_stride = size_t(pn.rows_pad) * pn.kpad / 4;  // in uint2 (4 bf16)
  const bool vec = (jb.K & 3) == 0;
  for (int k = 4 * lane; k < jb.K; k += 128) {
    unsigned long long b[4];
    if (vec) {
      const double2 v0 = __ldg(reinterpret_cast<const double2*>(row + k));
      const double2 v1 = __ldg(reinterpret_cast<const double2*>(row + k + 2));
      b[0] = __double_as_longlong(v0.x), b[1] = __double_as_longlong(v0.y);
      b[2] = __double_as_longlong(v1.x), b[3] = __double_as_longlong(v1.y);
    } else {
#pragma unroll
      for (int t = 0; t < 4; ++t) b[t] = k + t < jb.K ? __double_as_longlong(__ldg(row + k + t)) : 0ull;
    }
    int d[4][S];
#pragma unroll
    for (int t = 0; t < 4; ++t) balanced_digits<S>(quantize(b[t], mx, S), d[t]);
#pragma unroll
    for (int i = 0; i < S; ++i) {
      uint2 o;
      o.x = digits_bf16x2(d[0][i], d[1][i]);
      o.y = digits_bf16x2(d[2][i], d[3][i]);
      dst[i * slice_stride + (k >> 2)] = o;
    }
  }
}

// Column of k inside a row of the transpose tile: within each 16-column group
// the low two bits are rotated by the group index, so that the store phase's
// half-warp (one row, columns 4 kq + u for kq = 0..15) hits 16 distinct bank
// pairs instead of 4 (k = 16 b + 4 a + u is kept at 16 b + 4 a + (u + b) mod 4).
__device__ __forceinline__ int rows_tile_col(int k) { return (k & ~3) | (((k & 3) + (k >> 4)) & 3); }

// Slices of a column-major [rows x K] block: 64x64 tiles transposed through
// shared memory (16-byte loads along rows, 8-byte stores along k).
template <int S>
__global__ void __launch_bounds__(256) oz_split_rows_kernel(const OzSplitJob* __restrict__ jobs,
                                                            const int64_t* __restrict__ prefix, int njobs,
                                                            const OzPanel* __restrict__ panels) {
  __shared__ unsigned long long tile[64][65];
  const int j = find_job(prefix, njobs, blockIdx.x);
  const OzSplitJob jb = jobs[j];
  const int64_t local = int64_t(blockIdx.x) - prefix[j];
  const int ktiles = (jb.K + 63) / 64;
  const int r0 = int(local / ktiles) * 64, k0 = int(local % ktiles) * 64;
  const int t = threadIdx.x;
  // load: thread -> (row pair, k): 32 row pairs x 8 k per pass, 8 passes
  const bool vec = (jb.rows & 1) == 0;
#pragma unroll
  for (int p = 0; p < 8; ++p) {
    const int rp = t & 31, k = (t >> 5) + 8 * p;
    const int r = r0 + 2 * rp;
    unsigned long long x0 = 0, x1 = 0;
    if (k0 + k < jb.K && r < jb.rows) {
      const double* src = jb.src + size_t(k0 + k) * jb.rows + r;
      if (vec) {
        const double2 v = __ldg(reinterpret_cast<const double2*>(src));
        x0 = __double_as_longlong(v.x), x1 = __double_as_longlong(v.y);
      } else {
        x0 = __double_as_longlong(__ldg(src));
        if (r + 1 < jb.rows) x1 = __double_as_longlong(__ldg(src + 1));
      }
    }
    tile[2 * rp][rows_tile_col(k)] = x0;
    tile[2 * rp + 1][rows_tile_col(k)] = x1;
  }
  __syncthreads();
  // store: thread -> (row, 4 consecutive k): 16 k-quads x 16 rows per pass, 4 passes
  const OzPanel pn = panels[jb.panel];
  const size_t slice_stride = size_t(pn.rows_pad) * pn.kpad / 4;
#pragma unroll 1
  for (int p = 0; p < 4; ++p) {
    const int kq = t & 15, r = (t >> 4) + 16 * p;
    if (r0 + r >= jb.rows || k0 + 4 * kq >= jb.K) continue;
    const int mx = pn.exps[r0 + r];
    int d[4][S];
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      const unsigned long long b = (k0 + 4 * kq + u < jb.K) ? tile[r][rows_tile_col(4 * kq + u)] : 0ull;
      balanced_digits<S>(quantize(b, mx, S), d[u]);
    }
    uint2* dst = reinterpret_cast<uint2*>(pn.base + (size_t(r0 + r) * pn.kpad + jb.koff + k0 + 4 * kq));
#pragma unroll
    for (int i = 0; i < S; ++i) {
      uint2 o;
      o.x = digits_bf16x2(d[0][i], d[1][i]);
      o.y = digits_bf16x2(d[2][i], d[3][i]);
      dst[i * slice_stride] = o;
    }
  }
}

// ------------------------------------------------------------------ recombine
// One block of 256 threads per 32-column strip of a tile, walked as 32x32
// pieces (four elements per thread): every level's split partials of a piece
// are loaded before any is used (20 loads in flight per thread at 5 slices),
// summed exactly (int64), the levels combined exactly (64-bit when the top
// level allows it, else 128-bit) and rounded once to FP64 with the row/column
// scales.  Reads run along rows (the workspace order); strips whose D is
// unit-stride along n transpose through shared memory so the stores run
// along n.
template <int S>
__global__ void __launch_bounds__(256) oz_recombine_kernel(const OzTile* __restrict__ tiles,
                                                           const OzDBlock* __restrict__ dblocks,
                                                           const OzPanel* __restrict__ pa,
                                                           const OzPanel* __restrict__ pb,
                                                           const int* __restrict__ ws, int log_rows, int log_cols,
                                                           int nsplit, int mode) {
  constexpr int kSub = 32, kPer = kSub * kSub / 256;
  __shared__ double sm[kSub][kSub + 1];
  const int strips_log = log_cols - 5;
  const int tile = blockIdx.x >> strips_log;
  const int sc = (blockIdx.x & ((1 << strips_log) - 1)) * kSub;
  const OzTile tl = tiles[tile];
  const OzDBlock db = dblocks[tl.dblock];
  const int* ea = pa[tl.panel_a].exps;
  const int* eb = pb[tl.panel_b].exps;
  const size_t plane = size_t(1) << (log_rows + log_cols);     // one split's [cols][rows]
  const int* wtile = ws + size_t(tile) * S * nsplit * plane;
  const int rows_here = min(1 << log_rows, db.M - tl.m0);
  for (int sr = 0; sr < rows_here; sr += kSub) {
    long long lev[kPer][S];
#pragma unroll
    for (int p = 0; p < kPer; ++p)
#pragma unroll
      for (int lv = 0; lv < S; ++lv) lev[p][lv] = 0;
    for (int sp = 0; sp < nsplit; ++sp) {
      int raw[kPer][S];
#pragma unroll
      for (int p = 0; p < kPer; ++p) {
        const int e = p * 256 + threadIdx.x;
        const int row = sr + (e & (kSub - 1)), col = sc + (e >> 5);
        const int* q = wtile + (size_t(sp) << (log_rows + log_cols)) + (size_t(col) << log_rows) + row;
#pragma unroll
        for (int lv = 0; lv < S; ++lv) raw[p][lv] = __ldg(q + size_t(lv) * nsplit * plane);
      }
#pragma unroll
      for (int p = 0; p < kPer; ++p)
#pragma unroll
        for (int lv = 0; lv < S; ++lv) lev[p][lv] += raw[p][lv];
    }
#pragma unroll
    for (int p = 0; p < kPer; ++p) {
      const int e = p * 256 + threadIdx.x;
      const int row = sr + (e & (kSub - 1)), col = sc + (e >> 5);
      const int m = tl.m0 + row, n = tl.n0 + col;
      double v = 0.0;
      const bool live = m < db.M && n < db.N;
      if (live) {
        // value = sum_t lev[t] 2^(8(S-1-t)) * 2^(E + F + 2 - 8(S+1))
        const int E = (ea[m] ? ea[m] : 1) - 1022, F = (eb[n] ? eb[n] : 1) - 1022;
        const int e2 = E + F + 2 - kDigitBits * (S + 1);
        const long long top = lev[p][0] < 0 ? -lev[p][0] : lev[p][0];
        if (top < (1ll << (62 - kDigitBits * (S - 1)))) {  // the 64-bit sum cannot overflow
          long long acc = 0;
#pragma unroll
          for (int lv = 0; lv < S; ++lv) acc += lev[p][lv] * (1ll << (kDigitBits * (S - 1 - lv)));
          v = i64_scaled_to_double(acc, e2, false);
        } else {
          unsigned __int128 acc = 0;  // two's complement, wrapping (exact: |sum| < 2^101)
#pragma unroll
          for (int lv = 0; lv < S; ++lv)
            acc += (unsigned __int128)(__int128)lev[p][lv] << (kDigitBits * (S - 1 - lv));
          v = i128_scaled_to_double((__int128)acc, e2);
        }
        if (mode & 2) v = -v;  // negated term
        if (ea[m] == kNonFiniteExp || eb[n] == kNonFiniteExp) v = __longlong_as_double(0x7FF8000000000000ll);
      }
      if (db.col_fast) {
        sm[e & (kSub - 1)][e >> 5] = v;
      } else if (live) {
        double* dst = db.colptr[n] + db.rowoff[m];
        *dst = (mode & 1) ? *dst + v : v;
      }
    }
    if (!db.col_fast) continue;
    __syncthreads();
#pragma unroll
    for (int p = 0; p < kPer; ++p) {
      const int e = p * 256 + threadIdx.x;
      const int col = sc + (e & (kSub - 1)), row = sr + (e >> 5);
      const int m = tl.m0 + row, n = tl.n0 + col;
      if (m < db.M && n < db.N) {
        const double v = sm[e >> 5][e & (kSub - 1)];
        double* dst = db.colptr[n] + db.rowoff[m];
        *dst = (mode & 1) ? *dst + v : v;
      }
    }
    __syncthreads();
  }
}

// Single-split form of the recombine (every level sum already complete, e.g.
// the short-k triples): a persistent CTA per SM walks pieces of 4096 elements
// (16 KB per level: one whole column run of the tile's int32 plane per
// level, 16 or 32 columns; 1024 threads, four elements each), each level's
// piece fetched by one bulk async copy
// into a double-buffered shared-memory stage, so the next piece streams in
// while this one is combined and stored.  Waits are bounded (error flag, then
// a bounded drain of the copy still in flight).
constexpr int kRecPiece = 4096;  // int32 elements per level per piece (16 KB)
// Pieces in flight: one ahead of the one being combined.  (Four stages of
// 2048-element pieces were measured slower: 14 instead of 11 ms on the
// triples' term 1, the per-piece overhead doubling.)
constexpr int kRecStages = 2;

template <int S>
struct __align__(128) RecSmem {
  int lev[kRecStages][S][kRecPiece];
  double val[kRecPiece + 64];  // [col][rows + 1] transpose buffer
  uint64_t full[kRecStages];
};

__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                   smem_u32(dst)),
               "l"(src), "r"(bytes), "r"(smem_u32(bar))
               : "memory");
}

__device__ __forceinline__ bool wait_bounded(uint64_t* bar, uint32_t parity) {
  if (mbar_try_wait(bar, parity)) return true;
  const unsigned long long t0 = now_ns();
#pragma unroll 1
  for (uint32_t it = 1;; ++it) {
    if (mbar_try_wait(bar, parity)) return true;
    if ((it & 255) == 0 && now_ns() - t0 > kWaitLimitNs) return false;
  }
}

template <int S>
__global__ void __launch_bounds__(1024, 1) oz_recombine_bulk_kernel(const OzTile* __restrict__ tiles,
                                                                  const OzDBlock* __restrict__ dblocks,
                                                                         const OzPanel* __restrict__ pa,
                                                                  const OzPanel* __restrict__ pb,
                                                                  const int* __restrict__ ws, int log_rows,
                                                                  int log_cols, int n_tiles, int mode, int* err) {
  extern __shared__ __align__(128) unsigned char rec_smem_raw[];
  RecSmem<S>& sm = *reinterpret_cast<RecSmem<S>*>(rec_smem_raw);
  const int rows = 1 << log_rows;
  const int cols_pp = kRecPiece >> log_rows;                    // columns per piece
  const int pieces_per_tile = 1 << (log_rows + log_cols - 12);  // 4096 = 2^12
  const int npieces = n_tiles * pieces_per_tile;
  const size_t plane = size_t(1) << (log_rows + log_cols);
  if (threadIdx.x == 0) {
    for (int st = 0; st < kRecStages; ++st) mbar_init(&sm.full[st], 1);
    fence_mbar_init();
  }
  __syncthreads();
  auto issue = [&](int q, int st) {
    const int tile = q / pieces_per_tile, pc = q % pieces_per_tile;
    mbar_expect_tx(&sm.full[st], uint32_t(S) * kRecPiece * 4);
#pragma unroll
    for (int lv = 0; lv < S; ++lv)
      bulk_g2s(sm.lev[st][lv], ws + (size_t(tile) * S + lv) * plane + size_t(pc) * kRecPiece, kRecPiece * 4,
               &sm.full[st]);
  };
  int q = blockIdx.x;
  const int G = gridDim.x;
  if (threadIdx.x == 0)
    for (int i = 0; i < kRecStages - 1; ++i)
      if (q + i * G < npieces) issue(q + i * G, i);
  for (int it = 0; q < npieces; q += G, ++it) {
    const int st = it % kRecStages;
    // the stage of piece it + kRecStages - 1 was combined in iteration it - 1
    // (the barrier at the end of that iteration freed it)
    const int ahead = q + (kRecStages - 1) * G;
    if (threadIdx.x == 0 && ahead < npieces) issue(ahead, (it + kRecStages - 1) % kRecStages);
    if (!wait_bounded(&sm.full[st], uint32_t(it / kRecStages) & 1u)) {
      atomicExch(err, 5);
      // drain the later pieces' copies (those issued) before this CTA's memory is released
      if (threadIdx.x == 0)
        for (int i = 1; i < kRecStages && q + i * G < npieces; ++i)
          wait_bounded(&sm.full[(it + i) % kRecStages], uint32_t((it + i) / kRecStages) & 1u);
      return;
    }
    const int tile = q / pieces_per_tile, pc = q % pieces_per_tile;
    const OzTile tl = tiles[tile];
    const OzDBlock db = dblocks[tl.dblock];
    const int* ea = pa[tl.panel_a].exps;
    const int* eb = pb[tl.panel_b].exps;
    const int sc = pc * cols_pp;
    constexpr int kPerT = kRecPiece / 1024;
    double vals[kPerT];
    double* dsts[kPerT];
#pragma unroll
    for (int p = 0; p < kPerT; ++p) {
      const int e = p * 1024 + threadIdx.x;
      const int row = e & (rows - 1), cl = e >> log_rows;
      const int m = tl.m0 + row, n = tl.n0 + sc + cl;
      double v = 0.0;
      const bool live = m < db.M && n < db.N;
      if (live) {
        const int E = (ea[m] ? ea[m] : 1) - 1022, F = (eb[n] ? eb[n] : 1) - 1022;
        const int e2 = E + F + 2 - kDigitBits * (S + 1);
        long long acc = 0;  // a unit's level-t sum is below (t+1) 2^31 / S: the 64-bit sum is exact
#pragma unroll
        for (int lv = 0; lv < S; ++lv) acc += (long long)sm.lev[st][lv][e] * (1ll << (kDigitBits * (S - 1 - lv)));
        v = i64_scaled_to_double(acc, e2, mode & 2);  // negated term: the sign folded into the rounding
        if (ea[m] == kNonFiniteExp || eb[n] == kNonFiniteExp) v = __longlong_as_double(0x7FF8000000000000ll);
      }
      vals[p] = v;
      dsts[p] = nullptr;
      if (db.col_fast) sm.val[cl * (rows + 1) + row] = v;
      else if (live) dsts[p] = db.colptr[n] + db.rowoff[m];
    }
    if (!db.col_fast) {
      double old[kPerT];  // accumulate mode: the old values' loads in flight together
#pragma unroll
      for (int p = 0; p < kPerT; ++p) old[p] = (dsts[p] && (mode & 1)) ? *dsts[p] : 0.0;
#pragma unroll
      for (int p = 0; p < kPerT; ++p)
        if (dsts[p]) *dsts[p] = (mode & 1) ? old[p] + vals[p] : vals[p];
    }
    if (db.col_fast) {
      __syncthreads();
      constexpr int kPer = kRecPiece / 1024;
      double* dst[kPer];
      double old[kPer];
#pragma unroll
      for (int p = 0; p < kPer; ++p) {  // addresses and (beta) the old values first: loads in flight together
        const int e = p * 1024 + threadIdx.x;
        const int cl = e % cols_pp, row = e / cols_pp;
        const int m = tl.m0 + row, n = tl.n0 + sc + cl;
        dst[p] = (m < db.M && n < db.N) ? db.colptr[n] + db.rowoff[m] : nullptr;
        old[p] = (dst[p] && (mode & 1)) ? *dst[p] : 0.0;
      }
#pragma unroll
      for (int p = 0; p < kPer; ++p) {
        const int e = p * 1024 + threadIdx.x;
        const int cl = e % cols_pp, row = e / cols_pp;
        if (dst[p]) *dst[p] = (mode & 1) ? old[p] + sm.val[cl * (rows + 1) + row] : sm.val[cl * (rows + 1) + row];
      }
    }
    __syncthreads();  // stage st and the transpose buffer are free again
  }
}

// Self-test of the bounded-wait path every pipeline wait uses: one thread
// waits on an mbarrier that nothing arrives at, gives up after limit_ns, and
// reports through the device error flag exactly as a stalled pipeline would.
__global__ void wait_timeout_selftest_kernel(unsigned long long limit_ns, int* err, int* waited_ms) {
  __shared__ uint64_t bar;
  if (threadIdx.x != 0) return;
  mbar_init(&bar, 1);
  fence_mbar_init();
  const unsigned long long t0 = now_ns();
  bool done = mbar_try_wait(&bar, 0);
#pragma unroll 1
  for (uint32_t it = 1; !done; ++it) {
    done = mbar_try_wait(&bar, 0);
    if (!done && (it & 255) == 0 && now_ns() - t0 > limit_ns) break;
  }
  *waited_ms = int((now_ns() - t0) / 1000000ull);
  if (!done) atomicExch(err, 6);
}

// Self-tests of the one-rounding helpers exactly as the kernels run them: the
// integer-to-FP64 rounding of every split-precision epilogue and the exact
// division of the denominator and energy passes, one element per thread.
__global__ void round_selftest_kernel(int n, const long long* __restrict__ v, const int* __restrict__ e2,
                                      const int* __restrict__ neg, double* __restrict__ out) {
  const int i = int(blockIdx.x) * int(blockDim.x) + int(threadIdx.x);
  if (i < n) out[i] = i64_scaled_to_double(v[i], e2[i], neg[i] != 0);
}
__global__ void div_selftest_kernel(int n, const double* __restrict__ a, const double* __restrict__ b,
                                    double* __restrict__ out) {
  const int i = int(blockIdx.x) * int(blockDim.x) + int(threadIdx.x);
  if (i < n) out[i] = div_rn(a[i], b[i]);
}

// esum += efact * (sum of the n partial energies), the partials added in a
// fixed order (one CTA: strided per-thread sums, then a fixed tree), so a GPU
// gives the same bits every run.
__global__ void __launch_bounds__(1024) oz_energy_reduce_kernel(const double* __restrict__ part, int n,
                                                                double efact, double* esum) {
  __shared__ double red[1024];
  double acc = 0.0;
  for (int i = threadIdx.x; i < n; i += 1024) acc += part[i];
  red[threadIdx.x] = acc;
  __syncthreads();
  for (int w = 512; w > 0; w >>= 1) {
    if (int(threadIdx.x) < w) red[threadIdx.x] += red[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) *esum += efact * red[0];
}

using EncodeTiled = PFN_cuTensorMapEncodeTiled_v12000;
EncodeTiled get_encoder() {
  static EncodeTiled fn = nullptr;
  if (!fn) {
    cudaDriverEntryPointQueryResult q;
    void* p = nullptr;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
            cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<EncodeTiled>(p);
  }
  return fn;
}

}  // namespace

int oz_chunk_kb(int level) {
  // largest multiple of 64 k such that (level+1) * 128^2 * k < 2^24: every
  // FP32 partial sum of the chunk is an integer below 2^24, hence exact
  const long long per = (long long)(level + 1) * 128 * 128;
  const long long k = ((1LL << 24) - 1) / per;
  return int(k / kOzBK);
}

int oz_make_tensor_map(void* map128, const void* base, int64_t kpad, int64_t rows_total, int box_rows) {
  return oz_make_tensor_map_k(map128, base, kpad, rows_total, box_rows, kOzBK);
}

int oz_make_tensor_map_k(void* map128, const void* base, int64_t kpad, int64_t rows_total, int box_rows, int box_k) {
  EncodeTiled enc = get_encoder();
  if (!enc) return fail(A4G_ERR_CUDA, "cuTensorMapEncodeTiled unavailable");
  if (box_k != kOzBK && box_k != kLvBK) return fail(A4G_ERR_ARG, "tensor map: k box of 64 or 32");
  if (kpad % kOzBK != 0 || (reinterpret_cast<uintptr_t>(base) & 15) != 0)
    return fail(A4G_ERR_ARG, "panel not aligned for TMA");
  cuuint64_t dims[2] = {cuuint64_t(kpad), cuuint64_t(rows_total)};
  cuuint64_t strides[1] = {cuuint64_t(kpad) * 2};
  cuuint32_t box[2] = {cuuint32_t(box_k), cuuint32_t(box_rows)};
  cuuint32_t estr[2] = {1, 1};
  // rows of 128 B (64 k) with the 128-byte swizzle, of 64 B (32 k) with the 64-byte one
  CUresult r = enc(reinterpret_cast<CUtensorMap*>(map128), CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2,
                   const_cast<void*>(base), dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                   box_k == kOzBK ? CU_TENSOR_MAP_SWIZZLE_128B : CU_TENSOR_MAP_SWIZZLE_64B,
                   CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) return fail(A4G_ERR_CUDA, "cuTensorMapEncodeTiled failed: " + std::to_string(int(r)));
  return A4G_OK;
}

int64_t oz_exp_tiles(int layout, int rows, int K) {
  if (layout == kOzRowsMajor) return int64_t((rows + 511) / 512) * ((K + 63) / 64);
  if (layout == kOzKMajor) return (rows + 31) / 32;
  return int64_t((rows + 63) / 64) * ((K + 63) / 64);
}

int64_t oz_split_tiles(int layout, int rows, int K) {
  if (layout == kOzKMajor) return (rows + 7) / 8;
  return int64_t((rows + 63) / 64) * ((K + 63) / 64);
}

int oz_launch_exp(int layout, const OzSplitJob* jobs, const int64_t* prefix, int njobs, int64_t ntiles,
                  const OzPanel* panels, cudaStream_t s) {
  if (ntiles <= 0) return A4G_OK;
  if (ntiles > 0x7fffffffLL) return fail(A4G_ERR_RANGE, "too many split tiles");
  if (layout == kOzRowsMajor) oz_exp_rows_kernel<<<unsigned(ntiles), 256, 0, s>>>(jobs, prefix, njobs, panels);
  else if (layout == kOzKMajor) oz_exp_kmaj_kernel<<<unsigned(ntiles), 256, 0, s>>>(jobs, prefix, njobs, panels);
  else oz_exp_kernel<<<unsigned(ntiles), 256, 0, s>>>(jobs, prefix, njobs, panels);
  A4G_CUDA(cudaGetLastError());
  return A4G_OK;
}

int oz_launch_split(int layout, const OzSplitJob* jobs, const int64_t* prefix, int njobs, int64_t ntiles,
                    const OzPanel* panels, int slices, cudaStream_t s) {
  if (ntiles <= 0) return A4G_OK;
  if (ntiles > 0x7fffffffLL) return fail(A4G_ERR_RANGE, "too many split tiles");
  auto go = [&](auto sc) {
    constexpr int S = decltype(sc)::value;
    if (layout == kOzRowsMajor) oz_split_rows_kernel<S><<<unsigned(ntiles), 256, 0, s>>>(jobs, prefix, njobs, panels);
    else if (layout == kOzKMajor) oz_split_kmaj_kernel<S><<<unsigned(ntiles), 256, 0, s>>>(jobs, prefix, njobs, panels);
    else oz_split_kernel<S><<<unsigned(ntiles), 256, 0, s>>>(jobs, prefix, njobs, panels);
  };
  switch (slices) {
    case 1: go(std::integral_constant<int, 1>()); break;
    case 2: go(std::integral_constant<int, 2>()); break;
    case 3: go(std::integral_constant<int, 3>()); break;
    case 4: go(std::integral_constant<int, 4>()); break;
    case 5: go(std::integral_constant<int, 5>()); break;
    case 6: go(std::integral_constant<int, 6>()); break;
    case 7: go(std::integral_constant<int, 7>()); break;
    default: return fail(A4G_ERR_ARG, "slices must be 1..7");
  }
  A4G_CUDA(cudaGetLastError());
  return A4G_OK;
}

template <bool PAIR, int BN, bool DIRECT = false, bool ENERGY = false>
int set_smem_attr() {
  A4G_CUDA(cudaFuncSetAttribute(oz_gemm_kernel<PAIR, BN, DIRECT, ENERGY>,
                                cudaFuncAttributeMaxDynamicSharedMemorySize, int(sizeof(OzSmemT<PAIR, BN>)) + 1024));
  return A4G_OK;
}

template <bool ENERGY>
int set_levels_attr() {
  A4G_CUDA(cudaFuncSetAttribute(oz_levels_kernel<ENERGY>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                int(sizeof(LvSmem)) + 1024));
  return A4G_OK;
}

// Function attributes are set once per device (they belong to the device's
// instance of the kernel).
bool first_on_device(std::atomic<unsigned long long>& mask) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return true;
  const unsigned long long bit = 1ull << dev;
  return (mask.fetch_or(bit) & bit) == 0;
}

int oz_prepare() {
  static std::atomic<unsigned long long> done{0};
  if (first_on_device(done)) {
    int rc;
    if ((rc = set_smem_attr<false, 128>()) || (rc = set_smem_attr<true, 128>()) ||
        (rc = set_smem_attr<false, 256>()) || (rc = set_smem_attr<true, 256>()) ||
        (rc = set_smem_attr<false, 128, true>()) || (rc = set_smem_attr<true, 128, true>()) ||
        (rc = set_smem_attr<false, 128, true, true>()) || (rc = set_levels_attr<false>()) ||
        (rc = set_levels_attr<true>())) {
      done.store(0);
      return rc;
    }
  }
  return A4G_OK;
}

int oz_max_pairs(int* pairs) {
  int rc = oz_prepare();
  if (rc) return rc;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(2 * 76, 1, 1);
  cfg.blockDim = dim3(kThreadsOz, 1, 1);
  cfg.dynamicSmemBytes = sizeof(OzSmemT<true, 128>) + 1024;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = 2, attr[0].val.clusterDim.y = 1, attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  int n = 0, n2 = 0;
  A4G_CUDA(cudaOccupancyMaxActiveClusters(&n, oz_gemm_kernel<true, 128>, &cfg));
  cfg.dynamicSmemBytes = sizeof(OzSmemT<true, 256>) + 1024;
  A4G_CUDA(cudaOccupancyMaxActiveClusters(&n2, oz_gemm_kernel<true, 256>, &cfg));
  *pairs = std::min(n, n2);
  return A4G_OK;
}

template <bool PAIR, int BN, bool DIRECT = false, bool ENERGY = false>
int launch_form(const OzGemmArgs& args, int grid, cudaStream_t s) {
  const size_t smem = sizeof(OzSmemT<PAIR, BN>) + 1024;
  if constexpr (!PAIR) {
    oz_gemm_kernel<false, BN, DIRECT, ENERGY><<<grid, DIRECT ? kThreadsOzDirect : kThreadsOz, smem, s>>>(args);
  } else {
    if (grid % 2) return fail(A4G_ERR_ARG, "CTA-pair grid must be even");
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(grid, 1, 1);
    cfg.blockDim = dim3(DIRECT ? kThreadsOzDirect : kThreadsOz, 1, 1);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = 2, attr[0].val.clusterDim.y = 1, attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    A4G_CUDA(cudaLaunchKernelEx(&cfg, oz_gemm_kernel<true, BN, DIRECT>, args));
  }
  A4G_CUDA(cudaGetLastError());
  return A4G_OK;
}

int oz_launch_gemm(const OzGemmArgs& args, int grid, bool pair, int tile_cols, cudaStream_t s) {
  if (args.slices > kOzMaxUsableSlices) return fail(A4G_ERR_ARG, "at most 7 slices");
  int rc = oz_prepare();
  if (rc) return rc;
  if (args.n_units <= 0) return A4G_OK;
  if (args.direct) {
    if (tile_cols != 128 || args.nsplit != 1 || args.n_units % args.slices)
      return fail(A4G_ERR_ARG, "direct form: 128-column tiles, one split, whole tiles");
    if (args.energy) {
      if (pair || !args.eblocks || !args.epart) return fail(A4G_ERR_ARG, "energy form: one SM per tile, tables");
      return launch_form<false, 128, true, true>(args, grid, s);
    }
    return pair ? launch_form<true, 128, true>(args, grid, s) : launch_form<false, 128, true>(args, grid, s);
  }
  if (tile_cols == 256) return pair ? launch_form<true, 256>(args, grid, s) : launch_form<false, 256>(args, grid, s);
  return pair ? launch_form<true, 128>(args, grid, s) : launch_form<false, 128>(args, grid, s);
}

bool oz_levels_fit(int slices, int kb_total) { return slices >= 1 && slices <= kLvMaxS && kb_total <= 5; }

int oz_launch_levels(const OzGemmArgs& args, int grid, cudaStream_t s) {
  if (!oz_levels_fit(args.slices, 0) || !args.direct) return fail(A4G_ERR_ARG, "all-levels form: 1..5 slices, direct");
  int rc = oz_prepare();
  if (rc) return rc;
  if (args.n_tiles <= 0) return A4G_OK;
  const size_t smem = sizeof(LvSmem) + 1024;
  if (args.energy) {
    if (!args.eblocks || !args.epart) return fail(A4G_ERR_ARG, "energy form: tables");
    oz_levels_kernel<true><<<grid, kThreadsOzDirect, smem, s>>>(args);
  } else {
    oz_levels_kernel<false><<<grid, kThreadsOzDirect, smem, s>>>(args);
  }
  A4G_CUDA(cudaGetLastError());
  return A4G_OK;
}

int oz_launch_recombine(const OzTile* tiles, int ntiles, int tile_rows, int tile_cols, const OzDBlock* dblocks,
                        const OzPanel* pa, const OzPanel* pb, const int* ws, int slices,
                        int nsplit, int mode, cudaStream_t s) {
  if (ntiles <= 0) return A4G_OK;
  if ((tile_rows != 128 && tile_rows != 256) || (tile_cols != 128 && tile_cols != 256))
    return fail(A4G_ERR_ARG, "recombine: unsupported tile shape");
  const int lr = tile_rows == 256 ? 8 : 7, lc = tile_cols == 256 ? 8 : 7;
  if (nsplit == 1 && slices <= 5) {
    // single split: the bulk-copy pipelined form (one CTA per SM)
    const int npieces = ntiles * (tile_rows * tile_cols / kRecPiece);
    const int grid = std::min(npieces, ctx()->num_sms > 0 ? ctx()->num_sms : 152);
    int* err = ctx()->d_error_flag;
    switch (slices) {
#define A4G_RECOMBINE_BULK(SL)                                                                                   \
  case SL: {                                                                                                     \
    static std::atomic<unsigned long long> attr{0};                                                             \
    if (first_on_device(attr))                                                                                   \
      A4G_CUDA(cudaFuncSetAttribute(oz_recombine_bulk_kernel<SL>, cudaFuncAttributeMaxDynamicSharedMemorySize,  \
                                    int(sizeof(RecSmem<SL>))));                                                 \
    oz_recombine_bulk_kernel<SL><<<grid, 1024, sizeof(RecSmem<SL>), s>>>(tiles, dblocks, pa, pb, ws, lr, lc, \
                                                                       ntiles, mode, err);                       \
    break;                                                                                                       \
  }
      A4G_RECOMBINE_BULK(1) A4G_RECOMBINE_BULK(2) A4G_RECOMBINE_BULK(3) A4G_RECOMBINE_BULK(4) A4G_RECOMBINE_BULK(5)
#undef A4G_RECOMBINE_BULK
    }
    A4G_CUDA(cudaGetLastError());
    return A4G_OK;
  }
  const int per = tile_cols / 32;  // 32-column strips per tile
  if (int64_t(ntiles) * per > 0x7fffffffLL) return fail(A4G_ERR_RANGE, "too many tiles");
  const unsigned g = unsigned(ntiles * per);
  switch (slices) {
#define A4G_RECOMBINE(SL) \
  case SL: oz_recombine_kernel<SL><<<g, 256, 0, s>>>(tiles, dblocks, pa, pb, ws, lr, lc, nsplit, mode); break;
    A4G_RECOMBINE(1) A4G_RECOMBINE(2) A4G_RECOMBINE(3) A4G_RECOMBINE(4) A4G_RECOMBINE(5) A4G_RECOMBINE(6)
    A4G_RECOMBINE(7)
#undef A4G_RECOMBINE
    default: return fail(A4G_ERR_ARG, "recombine: slices must be 1..7");
  }
  A4G_CUDA(cudaGetLastError());
  return A4G_OK;
}

int oz_launch_energy_reduce(const double* part, int n, double efact, double* esum, cudaStream_t s) {
  oz_energy_reduce_kernel<<<1, 1024, 0, s>>>(part, n, efact, esum);
  A4G_CUDA(cudaGetLastError());
  return A4G_OK;
}

int oz_wait_timeout_selftest(int limit_ms, int* waited_ms, cudaStream_t s) {
  int* d_ms = nullptr;
  if (const int rc_ = async_alloc(reinterpret_cast<void**>(&d_ms), sizeof(int), s)) return rc_;
  wait_timeout_selftest_kernel<<<1, 32, 0, s>>>((unsigned long long)limit_ms * 1000000ull, ctx()->d_error_flag, d_ms);
  A4G_CUDA(cudaGetLastError());
  A4G_CUDA(cudaMemcpyAsync(waited_ms, d_ms, sizeof(int), cudaMemcpyDeviceToHost, s));
  A4G_CUDA(cudaFreeAsync(d_ms, s));
  return A4G_OK;
}

int oz_round_selftest(int n, const long long* v, const int* e2, const int* neg, double* out, cudaStream_t s) {
  if (n <= 0) return A4G_OK;
  round_selftest_kernel<<<unsigned((n + 255) / 256), 256, 0, s>>>(n, v, e2, neg, out);
  A4G_CUDA(cudaGetLastError());
  return A4G_OK;
}

int oz_div_selftest(int n, const double* a, const double* b, double* out, cudaStream_t s) {
  if (n <= 0) return A4G_OK;
  div_selftest_kernel<<<unsigned((n + 255) / 256), 256, 0, s>>>(n, a, b, out);
  A4G_CUDA(cudaGetLastError());
  return A4G_OK;
}

}  // namespace a4g
