// Device-visible descriptors of a planned pardo step (batched contraction):
// the FP64 grouped kernel and the split-precision (Ozaki) pipeline.
#pragma once

#include <cuda_bf16.h>
#include <stdint.h>

namespace a4g {

// Device copy of one contraction plan's address tables (see GemmPlan).
struct PlanRef {
  const int64_t *offLm, *offLk, *offRk, *offRn, *offDm, *offDn;
  int M, N, K;
  int a_kfast, b_kfast;
};

// ------------------------------------------------------------ FP64 grouped
struct GroupedPair {
  const double* l;
  const double* r;
  int plan;
  int pad;
};
struct GroupedF64Tile {
  double* d;
  int m0, n0;
  int pair_begin, pair_end;  // pairs summed into this tile
  int dplan;                 // plan giving D's tables and M, N
  int slot;                  // -1: store into D; else the partial-tile slot in the workspace
};
// Destination tiles whose pairs were spread over several CTAs: the partial
// tiles in slots [slot0, slot0 + nparts) are summed in order and stored.
struct GroupedF64Reduce {
  double* d;
  int m0, n0;
  int dplan;
  int slot0, nparts;
  int pad;
};
// mode: bit 0 accumulate, bit 1 negate; tile_m: 64 or 48 (grouped_f64_tile_m), tile_n: 64 or 32
// (grouped_f64_tile_n)
int launch_grouped_f64(const GroupedF64Tile* tiles, int ntiles, const GroupedPair* pairs, const PlanRef* plans,
                       int mode, double* ws, const GroupedF64Reduce* reds, int nreds, int tile_m, int tile_n,
                       cudaStream_t s);
// tile rows given the destination rows padded to 64- and to 48-row tiles (summed over the blocks)
int grouped_f64_tile_m(int64_t padded64, int64_t padded48);
int grouped_f64_tile_n(int max_n);  // tile columns for destination blocks of at most max_n columns

// ------------------------------------------------------------ split precision
// A panel holds the BF16 slices of every left block that feeds one group of
// destination rows, K-major: slice i, row m, column k at
//   base[(i * rows_pad + m) * kpad + k];
// the same layout with n for right-operand (B) panels.  Row exponents E (|x| <
// 2^E over the whole row of the panel) are kept per row.
struct OzPanel {
  __nv_bfloat16* base;
  int* exps;   // biased max exponent per row (atomicMax target)
  int rows;    // live rows
  int rows_pad;
  int64_t kpad;
};

// One operand block to slice into a panel (left blocks into A panels, right
// blocks into B panels).  Element (row, k) of the block is
//   src[offRow[row] + offK[k]].
struct OzSplitJob {
  const double* src;
  const int64_t* offRow;
  const int64_t* offK;
  int rows, K;
  int kfast;  // src is unit-stride along k
  int panel;
  int64_t koff;  // first k column of this block inside the panel (multiple of 16)
  int negate;    // slice -x instead of x (a term subtracted in a fused two-term step); generic layout only
  int pad;
};

// Memory layout of a split job's source block, detected on the host from the
// address tables: a plain column-major [rows x K] matrix (rows contiguous), a
// [K x rows] matrix (k contiguous), or anything else (gathered through the
// tables).
enum OzLayout { kOzGeneric = 0, kOzRowsMajor = 1, kOzKMajor = 2 };

// One output tile (the GEMM form's tile_rows x tile_cols) of one destination block.
struct OzTile {
  int dblock;
  int m0, n0;
  int panel_a, panel_b;
  int trip_begin, trip_end;  // range of OzTrip (one per block pair feeding the tile)
  int kb_total;              // sum of the pairs' 64-wide k blocks
};
// k position of one stretch of block pairs (back to back in both panels)
// inside the A and B panels.
struct OzTrip {
  int64_t koff_a, koff_b;
  int nkb;
  int pad;
};
// Destination of a tile grid: one destination block, or a stack of blocks
// that share the rows (the same left blocks, the same row addressing) laid
// side by side along n.  Element (m, n) lives at colptr[n] + rowoff[m].
struct OzDBlock {
  double* d;
  int plan;  // PlanRef index of the (first) block
  int panel_a, panel_b;
  int col_fast;  // D is unit-stride along n, not along m: store by columns
  int M, N;      // rows; columns of all stacked blocks
  const int64_t* rowoff;  // [M] row offsets (the blocks' common offDm)
  double* const* colptr;  // [N] column bases (block + offDn of its column)
};

constexpr int kOzBM = 128, kOzBN = 128, kOzBK = 64, kOzK16 = 16, kOzMaxSlices = 8;
constexpr int kOzMaxPipelineParts = 8;  // GEMM launches per pardo step when the right split pipelines

// Work unit of the tensor-core kernel: one level of one tile over a range of
// its k blocks (split-K).  Units are ordered (level, split, tile) so that the
// CTAs running at the same time stream the same k window of the panels; in
// the direct form (no split-K) they are ordered (tile, level) and one CTA (or
// CTA pair) runs all levels of a tile in a row.
struct OzUnit {
  int tile, level, split;
  int kb_begin, kb_end;  // range in the tile's concatenated k-block list
  int trip_first;        // first trip overlapping kb_begin
  int kb_in_trip;        // k-block offset inside that trip
  int pad;
};

// Energy form of the direct GEMM (fused two-term step): per destination
// sub-block, what the epilogue needs to form the orbital-energy denominator of
// element (m, n) in the reference's order of additions: the chain without its
// last term, precomputed per sub-block as ptab[rk[m] * ckn + ck[n]], then the
// last term (a row or a column index) subtracted:
//     eps(m, n) = ptab[rk[m] * ckn + ck[n]] - elast[last_row ? m : n]
struct OzEnergyBlock {
  const double* ptab;
  const int* rk;        // [M]
  const int* ck;        // [N]
  const double* elast;  // [M] or [N]
  int ckn;
  int last_row;
};

struct OzGemmArgs {
  const void* maps_a;  // CUtensorMap[n_panels_a], 64-byte aligned, device memory
  const void* maps_b;
  const OzPanel* panels_a;
  const OzPanel* panels_b;
  const OzTile* tiles;
  const OzTrip* trips;
  const OzUnit* units;
  int n_units;
  int n_tiles;
  int slices;
  int nsplit;
  int chunk_kb[kOzMaxSlices];  // k blocks per exact flush at each level
  int* ws;                     // [tile][level][split][col 128][row 128] exact integer level sums
  int* err_flag;
  // Direct form (128-column tiles, one split): the levels of a tile are folded
  // exactly in TMEM (64-bit Horner sum over levels) and the epilogue rounds
  // once and stores D; no workspace, no recombine kernel.
  int direct;
  int mode;  // direct: bit 0 accumulate into D, bit 1 negate
  int dry;   // direct: compute everything but store nothing (timing)
  const OzDBlock* dblocks;
  // Energy form (direct, one SM per tile): nothing is stored; each epilogue
  // thread accumulates sum D(x) * fl(D(x) / eps(x)) over its elements in FP64
  // and writes it to epart[(blockIdx.x * 16 + epilogue warp) * 32 + lane].
  int energy;
  const OzEnergyBlock* eblocks;  // one per destination sub-block (tile.dblock)
  double* epart;
};

}  // namespace a4g
