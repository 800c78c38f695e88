// Host launchers of the split-precision (Ozaki) contraction kernels.
#pragma once

#include "grouped.h"

namespace a4g {

constexpr int kOzMaxUsableSlices = 7;  // 7 digits x 7 bits = 49 bits <= the 53-bit FP64 mantissa

int oz_prepare();  // one-time kernel attributes (call outside stream capture)
int oz_chunk_kb(int level);  // 64-wide k blocks per exact FP32 flush at a level
int oz_make_tensor_map(void* map128, const void* base, int64_t kpad, int64_t rows_total, int box_rows);
// the same with a k box of 64 (128-byte swizzle) or 32 (64-byte swizzle, the all-levels form)
int oz_make_tensor_map_k(void* map128, const void* base, int64_t kpad, int64_t rows_total, int box_rows, int box_k);
int oz_max_pairs(int* pairs);  // CTA pairs of the 2-SM kernel that fit on the GPU at once
// CTA counts of the exponent / split kernels for one job of a given layout.
int64_t oz_exp_tiles(int layout, int rows, int K);
int64_t oz_split_tiles(int layout, int rows, int K);
int oz_launch_exp(int layout, const OzSplitJob* jobs, const int64_t* prefix, int njobs, int64_t ntiles,
                  const OzPanel* panels, cudaStream_t s);
int oz_launch_split(int layout, const OzSplitJob* jobs, const int64_t* prefix, int njobs, int64_t ntiles,
                    const OzPanel* panels, int slices, cudaStream_t s);
// pair = false: 1-SM kernel, 128 x tile_cols tiles; pair = true: CTA-pair
// kernel (cluster of 2, cta_group::2), 256 x tile_cols tiles, grid even.
// tile_cols: 128 (exact sums kept in TMEM) or 256 (exact sums in registers).
int oz_launch_gemm(const OzGemmArgs& args, int grid, bool pair, int tile_cols, cudaStream_t s);
// All-levels form of the direct GEMM (128 x 64 tiles, every level accumulator
// in TMEM at once; maps with a k box of 32): fits when slices <= 5 and every
// tile's k range is at most 5 blocks of 64.
constexpr int kOzLevelsTileCols = 64;
bool oz_levels_fit(int slices, int kb_total);
int oz_launch_levels(const OzGemmArgs& args, int grid, cudaStream_t s);
int oz_wait_timeout_selftest(int limit_ms, int* waited_ms, cudaStream_t s);
// device runs of the one-rounding helpers (exact_fp.h) over device arrays
int oz_round_selftest(int n, const long long* v, const int* e2, const int* neg, double* out, cudaStream_t s);
int oz_div_selftest(int n, const double* a, const double* b, double* out, cudaStream_t s);
// esum (device) += efact * the sum of the energy form's n partials, in a fixed order.
int oz_launch_energy_reduce(const double* part, int n, double efact, double* esum, cudaStream_t s);
int oz_launch_recombine(const OzTile* tiles, int ntiles, int tile_rows, int tile_cols, const OzDBlock* dblocks,
                        const OzPanel* pa, const OzPanel* pb, const int* ws, int slices,
                        int nsplit, int mode, cudaStream_t s);  // mode: bit 0 accumulate, bit 1 negate

}  // namespace a4g
