// Batched contraction of one pardo step (a4g_batch_*): planning on the host,
// one grouped kernel (FP64) or the split-precision pipeline (Ozaki, BF16
// tcgen05) on the device, optionally captured once into a CUDA graph.
//
// The reference runs one tensor_block_contract__ per block pair from the
// interpreter loop (src/sip/worker/interpreter.cpp:734-742, one pardo
// iteration at a time, loop_manager.cpp:289-314) and accumulates partial
// results with a separate += (rlccd_rhf.sialx:408-412).  Here the whole step
// is one call: pairs that feed the same destination block are summed in the
// kernel, zero blocks (NULL operand) are never touched.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <deque>
#include <limits>
#include <map>
#include <memory>
#include <mutex>
#include <set>
#include <unordered_map>
#include <unordered_set>
#include <vector>

#include "a4g_internal.h"
#include "grouped.h"
#include "ozaki.h"

using namespace a4g;

struct a4g_batch {
  int precision = A4G_PREC_FP64;
  int slices = 5;
  int beta = 0;
  int negate = 0;
  // store mode of the writing kernels: bit 0 accumulate into D, bit 1 negate
  int store_mode() const { return beta | (negate << 1); }
  int variant = 0;  // tensor-core GEMM form: 0 autotuned, else 1 + index into forms
  int pipeline = 0;  // requested GEMM parts (0/1: one launch)
  int64_t pairs = 0;
  double flops = 0.0;
  int64_t device_bytes = 0;
  std::vector<void*> allocs;
  std::vector<std::pair<double*, int64_t>> zero_blocks;  // D blocks with no live pair (beta = 0)
  PlanRef* d_plans = nullptr;
  // The triples as given at creation (or at the last rebind): a rebind maps
  // their block pointers to the new ones and rewrites every device table that
  // holds a block pointer from its host copy below.
  int drank = 0, lrank = 0, rrank = 0;
  std::vector<a4g_triple> bound;
  // FP64 grouped
  GroupedF64Tile* d_f64_tiles = nullptr;
  GroupedPair* d_f64_pairs = nullptr;
  int n_f64_tiles = 0;
  double* d_f64_ws = nullptr;           // partial tiles when tiles are spread
  GroupedF64Reduce* d_f64_reds = nullptr;
  int n_f64_reds = 0;
  int f64_tile_m = 64, f64_tile_n = 64;  // rows (64 or 48) and columns (64 or 32) of a grouped FP64 tile
  std::vector<GroupedF64Tile> h_f64_tiles;
  std::vector<GroupedPair> h_f64_pairs;
  std::vector<GroupedF64Reduce> h_f64_reds;
  // split precision
  OzPanel* d_pa = nullptr;
  OzPanel* d_pb = nullptr;
  OzPanel* d_pb_view = nullptr;  // the split kernels' views of the B panels (stacked panels: one per member)
  int* d_exps = nullptr;
  size_t exps_bytes = 0;
  size_t exps_a_bytes = 0;  // the A panels' exponents come first in d_exps, then the B panels'
  // Held operand sides (0: A panels, 1: B panels, after any role exchange):
  // their digits were sliced by a4g_batch_hold and runs do not slice them again.
  bool held[2] = {false, false};
  // Per destination block, what the certified error bound needs: the block,
  // where its rows' and columns' exponents sit in d_exps, and the length of
  // its k sum (the same for all of its elements).
  struct ErrGroup {
    double* d;
    int64_t size;
    int64_t rows, cols;
    size_t exp_rows, exp_cols;  // element offsets into d_exps
    double K;
  };
  std::vector<ErrGroup> err_groups;
  std::vector<OzDBlock> h_dblocks;
  double** d_colptr = nullptr;
  std::vector<double*> h_colptr;        // column bases: block + offDn of the column
  std::vector<double*> h_colptr_block;  // the block each column base lies in
  // Autotuning: taken from the process's tuning cache (keyed by the batch's
  // structure), and the host time the autotuner spent at creation.
  uint64_t signature = 0;
  bool tuned_from_cache = false;
  float autotune_ms = 0.f;
  // A rebind's tables travel through a ring of pinned, mapped host slots and
  // are put in place by a kernel (see copy_tables_kernel).
  static constexpr int kStageRing = 4;
  char* h_stage = nullptr;
  char* d_stage = nullptr;  // the same memory as the device sees it
  size_t stage_bytes = 0;
  int stage_next = 0;
  cudaEvent_t stage_ev[kStageRing] = {};
  bool stage_busy[kStageRing] = {};
  // split jobs grouped by operand side (A: left blocks, B: right blocks) and
  // source layout; each set has its own CTA prefix sums for both passes
  struct JobSet {
    bool left;
    int layout;
    int group = 0;  // split pipeline group: 0 before the GEMM, g > 0 with GEMM part g-1
    OzSplitJob* d_jobs = nullptr;
    int64_t* d_prefix_exp = nullptr;
    int64_t* d_prefix_split = nullptr;
    int njobs = 0;
    int64_t tiles_exp = 0, tiles_split = 0;
    std::vector<OzSplitJob> h_jobs;  // host copy (a rebind rewrites the source pointers)
  };
  std::vector<JobSet> jobsets;
  OzDBlock* d_dblocks = nullptr;
  // Tensor-core GEMM forms: [0] 1-SM 128x128 tiles, [1] CTA-pair 256x128,
  // [2] 1-SM 128x256, [3] CTA-pair 256x256 (level sums to the workspace, then
  // the recombine kernel); [4] 1-SM 128x128 and [5] CTA-pair 256x128 direct
  // (levels folded in TMEM, FP64 stored by the GEMM's epilogue).
  static constexpr int kForms = 6;
  struct GemmForm {
    bool pair = false;
    bool direct = false;
    bool built = false;
    int tile_rows = 128;
    int tile_cols = 128;
    OzTile* d_tiles = nullptr;
    int n_tiles = 0;
    int nsplit = 1;
    int grid = 0;
    OzGemmArgs args{};
    float tuned_ms = -1.f;  // GEMM time measured at creation (direct: without its D stores)
    float score_ms = -1.f;  // tuned_ms + modelled workspace read and D traffic
  };
  GemmForm forms[kForms];
  int form = 0;  // the form run() uses (chosen by the autotuner or the caller)
  // split-count tuning of the chosen form: candidates and their scores (ms)
  int split_candidates[2] = {0, 0};
  // D = L R computed as D = R L with the operands' roles exchanged (so that
  // D's unit-stride index runs along the tile rows)
  bool swapped = false;
  std::deque<DevPlan> own_plans;
  float split_cost_ms[2] = {-1.f, -1.f};
  // Split/GEMM pipeline of the chosen form: the GEMM runs as `parts` launches
  // over consecutive split-K ranges; the right-operand split jobs that only
  // later parts read run on `side` while earlier parts multiply.
  int parts = 1;
  std::vector<OzGemmArgs> part_args;
  std::vector<int> part_grid;
  cudaStream_t side = nullptr;
  std::vector<cudaEvent_t> part_ev;  // [0]: fork after split group 0; [g]: split group g done
  int* d_ws = nullptr;
  cudaGraphExec_t graph = nullptr;
  cudaStream_t capture = nullptr;  // private stream the graph is captured on (any caller stream may replay it)
  // phase timing: events[run][6] recorded by a4g_batch_run_timed
  std::vector<std::vector<cudaEvent_t>> events;
  int timed_runs = 0;

  ~a4g_batch() {
    for (int i = 0; i < kStageRing; ++i)
      if (stage_ev[i]) cudaEventSynchronize(stage_ev[i]), cudaEventDestroy(stage_ev[i]);
    if (h_stage) cudaFreeHost(h_stage);
    for (auto& ev : events)
      for (cudaEvent_t e : ev) cudaEventDestroy(e);
    for (cudaEvent_t e : part_ev) cudaEventDestroy(e);
    if (side) cudaStreamDestroy(side);
    if (capture) cudaStreamDestroy(capture);
    if (graph) cudaGraphExecDestroy(graph);
    for (void* p : allocs) cudaFree(p);
  }
};

namespace {

// ------------------------------------------------------------ tuning cache
// The autotuner's choice (GEMM form and split-K count) for one batch
// structure, kept for the life of the process (and optionally saved to and
// loaded from a file), so that a batch built again for the same structure (the
// next iteration of the same contraction, a batch rebuilt per step) skips the
// timing runs.
struct TuneRecord {
  int form = -1;
  int nsplit = 0;
  float score_ms[a4g_batch::kForms];
  int split_candidates[2] = {0, 0};
  float split_cost_ms[2] = {-1.f, -1.f};
};
std::mutex g_tune_mu;
std::unordered_map<uint64_t, TuneRecord> g_tune;

bool tune_get(uint64_t key, TuneRecord* out) {
  std::lock_guard<std::mutex> lock(g_tune_mu);
  auto it = g_tune.find(key);
  if (it == g_tune.end()) return false;
  *out = it->second;
  return true;
}

void tune_put(uint64_t key, const TuneRecord& r) {
  std::lock_guard<std::mutex> lock(g_tune_mu);
  g_tune[key] = r;
}

// 64-bit FNV-1a over the bytes that decide the tuning.
struct Fnv {
  uint64_t h = 1469598103934665603ull;
  void add(const void* p, size_t n) {
    const unsigned char* c = static_cast<const unsigned char*>(p);
    for (size_t i = 0; i < n; ++i) h = (h ^ c[i]) * 1099511628211ull;
  }
  template <class T>
  void put(const T& v) {
    add(&v, sizeof(v));
  }
};

// Structure of a batch as the autotuner sees it: the options, the pattern,
// every triple's extents, which triples share a block (blocks numbered in
// order of first appearance, NULL as -1), the 16-byte alignment of each
// operand block (it selects the split kernels' vector loads) and the GPU.
uint64_t batch_signature(const a4g_batch* b, const int* ptrn, const a4g_triple* t, int64_t n) {
  Fnv f;
  f.put(uint32_t(0x41344731));  // format tag
  f.put(ctx()->num_sms);
  f.put(b->precision), f.put(b->slices), f.put(b->beta), f.put(b->negate), f.put(b->pipeline);
  f.put(b->drank), f.put(b->lrank), f.put(b->rrank);
  f.add(ptrn, sizeof(int) * size_t(b->lrank + b->rrank));
  f.put(n);
  std::unordered_map<const void*, int> id;
  auto ident = [&](const void* p) -> int {
    if (!p) return -1;
    return id.emplace(p, int(id.size())).first->second;
  };
  for (int64_t i = 0; i < n; ++i) {
    const a4g_triple& x = t[i];
    f.add(x.dext, sizeof(int) * size_t(b->drank));
    f.add(x.lext, sizeof(int) * size_t(b->lrank));
    f.add(x.rext, sizeof(int) * size_t(b->rrank));
    const int ids[3] = {ident(x.d), ident(x.l), ident(x.r)};
    f.put(ids);
    const int al = ((reinterpret_cast<uintptr_t>(x.l) & 15) == 0) | (((reinterpret_cast<uintptr_t>(x.r) & 15) == 0) << 1);
    f.put(al);
  }
  return f.h;
}

template <class T>
int upload(a4g_batch* b, const std::vector<T>& v, T** out) {
  *out = nullptr;
  if (v.empty()) return A4G_OK;
  const size_t bytes = v.size() * sizeof(T);
  void* p = nullptr;
  A4G_CUDA(cudaMalloc(&p, bytes));
  b->allocs.push_back(p);
  b->device_bytes += int64_t(bytes);
  A4G_CUDA(cudaMemcpy(p, v.data(), bytes, cudaMemcpyHostToDevice));
  *out = static_cast<T*>(p);
  return A4G_OK;
}

int device_alloc(a4g_batch* b, size_t bytes, void** out, bool zero) {
  void* p = nullptr;
  A4G_CUDA(cudaMalloc(&p, std::max<size_t>(bytes, 256)));
  b->allocs.push_back(p);
  b->device_bytes += int64_t(bytes);
  if (zero) A4G_CUDA(cudaMemset(p, 0, bytes));
  *out = p;
  return A4G_OK;
}

// Frees one allocation made by upload/device_alloc before the batch ends.
void release(a4g_batch* b, void* p, size_t bytes) {
  if (!p) return;
  auto it = std::find(b->allocs.begin(), b->allocs.end(), p);
  if (it == b->allocs.end()) return;
  b->allocs.erase(it);
  b->device_bytes -= int64_t(bytes);
  cudaFree(p);
}

PlanRef ref_of(const DevPlan* p) {
  PlanRef r;
  r.offLm = p->offLm, r.offLk = p->offLk, r.offRk = p->offRk, r.offRn = p->offRn;
  r.offDm = p->offDm, r.offDn = p->offDn;
  r.M = int(p->host.M), r.N = int(p->host.N), r.K = int(p->host.K);
  r.a_kfast = p->host.a_kfast, r.b_kfast = p->host.b_kfast;
  return r;
}

struct Pair {
  const double* l;
  const double* r;
  int plan;
};
struct DGroup {
  double* d;
  std::vector<Pair> pairs;
  int plan = -1;  // any pair's plan: D-side tables are identical for all
};

int64_t ceil_to(int64_t x, int64_t m) { return (x + m - 1) / m * m; }

struct alignas(64) MapBytes {  // host image of one CUtensorMap (128 bytes, 64-byte aligned)
  uint8_t b[128];
};

// Panel of one operand side: the distinct blocks feeding a set of destination
// rows (A) or columns (B), each with its k offset inside the panel.  Blocks
// are packed at a 16-column granularity (32-byte aligned TMA coordinates,
// zero padded to it), so pairs that sit back to back in both panels run as
// one stretch of k.  In the A panel every stretch starts on a 64-column
// boundary and its last block is zero padded to the next one, so the last
// 64-wide k block of a stretch multiplies A's zeros beyond it.
struct PanelBuild {
  std::vector<const double*> key;    // sorted block pointers
  std::vector<const double*> order;  // blocks in panel order
  std::map<const double*, int64_t> koff;
  std::map<const double*, int> plan;
  std::set<const double*> pad_before, pad_after;  // stretch starts / ends (A panels)
  int rows = 0;
  int64_t kpad = 0;
  // A stacked B panel: the rows of other panels (first row, panel index) one
  // after another, each with its own blocks at its own k offsets.
  std::vector<std::pair<int, int>> members;
  bool used = true;  // some tile reads it (stacked member panels are not read themselves)
};

// (Re)assign the k offsets of a panel's blocks in panel order.
void layout_panel(PanelBuild& pb, const std::vector<DevPlan const*>& plans) {
  pb.kpad = 0;
  for (const double* blk : pb.order) {
    if (pb.pad_before.count(blk)) pb.kpad = ceil_to(pb.kpad, kOzBK);
    pb.koff[blk] = pb.kpad;
    pb.kpad += ceil_to(plans[pb.plan.at(blk)]->host.K, kOzK16);
    if (pb.pad_after.count(blk)) pb.kpad = ceil_to(pb.kpad, kOzBK);
  }
  pb.kpad = ceil_to(pb.kpad, kOzBK);  // whole 64-column boxes
}

int find_or_add_panel(std::vector<PanelBuild>& panels, std::map<std::vector<const double*>, int>& index,
                      const std::vector<std::pair<const double*, int>>& blocks, int rows,
                      const std::vector<DevPlan const*>& plans) {
  std::vector<const double*> key;
  for (auto& b : blocks) key.push_back(b.first);
  std::sort(key.begin(), key.end());
  key.erase(std::unique(key.begin(), key.end()), key.end());
  auto it = index.find(key);
  if (it != index.end()) return it->second;
  PanelBuild pb;
  pb.key = key;
  pb.rows = rows;
  for (auto& b : blocks) {
    if (pb.plan.count(b.first)) continue;
    pb.order.push_back(b.first);
    pb.plan[b.first] = b.second;
  }
  layout_panel(pb, plans);
  panels.push_back(pb);
  index[key] = int(panels.size()) - 1;
  return int(panels.size()) - 1;
}

// Stretches of a destination block's pairs: maximal runs of consecutive
// pairs whose blocks sit back to back in both panels.  f(first, last) per
// stretch (pair indices, inclusive).
template <class F>
void for_stretches(const DGroup& g, const PanelBuild& pa, const PanelBuild& pb,
                   const std::vector<DevPlan const*>& plans, F&& f) {
  int first = -1;
  int64_t ka = 0, kb = 0, kk = 0;
  for (int q = 0; q < int(g.pairs.size()); ++q) {
    const Pair& p = g.pairs[q];
    const int64_t K = ceil_to(plans[p.plan]->host.K, kOzK16);
    const int64_t a = pa.koff.at(p.l), b = pb.koff.at(p.r);
    if (first >= 0 && a == ka + kk && b == kb + kk) {
      kk += K;
      continue;
    }
    if (first >= 0) f(first, q - 1, ka, kb, kk);
    first = q, ka = a, kb = b, kk = K;
  }
  if (first >= 0) f(first, int(g.pairs.size()) - 1, ka, kb, kk);
}

int build_f64(a4g_batch* b, const std::vector<DGroup>& groups, const std::vector<const DevPlan*>& plans) {
  std::vector<GroupedF64Tile> tiles;
  std::vector<GroupedPair> pairs;
  int64_t max_n = 0, pad64 = 0, pad48 = 0;
  for (const DGroup& g : groups) {
    const int64_t M = plans[g.plan]->host.M;
    max_n = std::max(max_n, plans[g.plan]->host.N);
    pad64 += (M + 63) / 64 * 64, pad48 += (M + 47) / 48 * 48;
  }
  const int TM = grouped_f64_tile_m(pad64, pad48), TN = grouped_f64_tile_n(int(std::min<int64_t>(max_n, 1 << 30)));
  b->f64_tile_m = TM, b->f64_tile_n = TN;
  for (const DGroup& g : groups) {
    const int begin = int(pairs.size());
    for (const Pair& p : g.pairs) pairs.push_back({p.l, p.r, p.plan, 0});
    const int end = int(pairs.size());
    const GemmPlan& h = plans[g.plan]->host;
    for (int64_t n0 = 0; n0 < h.N; n0 += TN)
      for (int64_t m0 = 0; m0 < h.M; m0 += TM)
        tiles.push_back({g.d, int(m0), int(n0), begin, end, g.plan, -1});
  }
  // Few tiles with many pairs each (small blocks, long sums): spread each
  // tile's pairs over G CTAs writing partial tiles, summed in order after.
  const int sms = ctx()->num_sms > 0 ? ctx()->num_sms : 152;
  const int64_t want = 4LL * sms;
  int min_pairs = 1 << 30;
  for (const auto& t : tiles) min_pairs = std::min(min_pairs, t.pair_end - t.pair_begin);
  const int G = tiles.empty() ? 1
                              : int(std::max<int64_t>(1, std::min<int64_t>({16, int64_t(min_pairs),
                                                                            (want + int64_t(tiles.size()) - 1) /
                                                                                int64_t(tiles.size())})));
  if (G > 1) {
    std::vector<GroupedF64Tile> spread;
    std::vector<GroupedF64Reduce> reds;
    int slot = 0;
    for (const auto& t : tiles) {
      const int np = t.pair_end - t.pair_begin;
      reds.push_back({t.d, t.m0, t.n0, t.dplan, slot, G, 0});
      for (int q = 0; q < G; ++q)
        spread.push_back({t.d, t.m0, t.n0, t.pair_begin + np * q / G, t.pair_begin + np * (q + 1) / G, t.dplan,
                          slot++});
    }
    void* ws = nullptr;
    int rc = device_alloc(b, size_t(slot) * TM * TN * sizeof(double), &ws, false);
    if (rc) return rc;
    b->d_f64_ws = static_cast<double*>(ws);
    if ((rc = upload(b, reds, &b->d_f64_reds))) return rc;
    b->n_f64_reds = int(reds.size());
    b->h_f64_reds = reds;
    tiles.swap(spread);
  }
  if (tiles.size() > 0x7fffffffu) return fail(A4G_ERR_RANGE, "too many tiles");
  b->n_f64_tiles = int(tiles.size());
  int rc = upload(b, tiles, &b->d_f64_tiles);
  if (!rc) rc = upload(b, pairs, &b->d_f64_pairs);
  b->h_f64_tiles = tiles;
  b->h_f64_pairs = pairs;
  return rc;
}

int build_ozaki(a4g_batch* b, const std::vector<DGroup>& groups, const std::vector<const DevPlan*>& plans) {
  std::vector<PanelBuild> pa, pb;
  std::map<std::vector<const double*>, int> ia, ib;
  std::vector<OzDBlock> dblocks;
  std::vector<OzTile> dinfo;  // one per destination block: m0 = M, n0 = N (tiles are cut per form)
  std::vector<OzTrip> trips;
  std::vector<int> ga(groups.size()), gb(groups.size());
  for (size_t gi = 0; gi < groups.size(); ++gi) {
    const DGroup& g = groups[gi];
    const GemmPlan& h = plans[g.plan]->host;
    std::vector<std::pair<const double*, int>> ls, rs;
    for (const Pair& p : g.pairs) ls.push_back({p.l, p.plan}), rs.push_back({p.r, p.plan});
    ga[gi] = find_or_add_panel(pa, ia, ls, int(h.M), plans);
    gb[gi] = find_or_add_panel(pb, ib, rs, int(h.N), plans);
  }
  // In the A panels, align the first block of every stretch to 64 columns and
  // pad after its last block; padding only splits stretches, so repeat until
  // every stretch starts and ends on marked blocks (marks only grow).
  for (bool changed = true; changed;) {
    changed = false;
    for (size_t gi = 0; gi < groups.size(); ++gi) {
      PanelBuild& A = pa[ga[gi]];
      for_stretches(groups[gi], A, pb[gb[gi]], plans, [&](int first, int last, int64_t, int64_t, int64_t) {
        changed |= A.pad_before.insert(groups[gi].pairs[first].l).second;
        changed |= A.pad_after.insert(groups[gi].pairs[last].l).second;
      });
    }
    if (changed)
      for (auto& p : pa) layout_panel(p, plans);
  }
  // Stacks: destination blocks whose pairs multiply the same left blocks at
  // the same k positions of one A panel, whose B panels lay their pairs out
  // alike, and whose rows are addressed alike (equal offDm) are laid side by
  // side along n: one tile grid over all their columns, so that only the
  // stack's last tile column is ragged instead of every block's (the ring's
  // 480..800-column blocks left ~30 % of the 256-column tiles empty).
  std::map<std::vector<int64_t>, int> offdm_ids;
  std::map<std::vector<int64_t>, int> stack_index;
  std::vector<std::vector<int>> stacks;
  for (size_t gi = 0; gi < groups.size(); ++gi) {
    const DGroup& g = groups[gi];
    const GemmPlan& h = plans[g.plan]->host;
    const int od = offdm_ids.emplace(h.offDm, int(offdm_ids.size())).first->second;
    std::vector<int64_t> sig = {ga[gi], h.M, od, pb[gb[gi]].kpad};
    for (const Pair& p : g.pairs) {
      sig.push_back(int64_t(reinterpret_cast<uintptr_t>(p.l)));
      sig.push_back(plans[p.plan]->host.K);
      sig.push_back(pa[ga[gi]].koff.at(p.l));
      sig.push_back(pb[gb[gi]].koff.at(p.r));
    }
    auto it = stack_index.find(sig);
    if (it == stack_index.end()) {
      stack_index.emplace(sig, int(stacks.size()));
      stacks.push_back({int(gi)});
    } else {
      stacks[it->second].push_back(int(gi));
    }
  }
  for (auto& p : pb) p.used = false;
  std::vector<std::pair<int, int>> col_panel(groups.size());  // (B panel read, first row in it) per group
  std::map<std::vector<int>, int> stacked_index;  // member panels -> stacked panel
  std::vector<double*> colptr_host;  // every destination's column bases, concatenated
  std::vector<size_t> colptr_at;
  for (const std::vector<int>& st : stacks) {
    const int g0 = st[0];
    const DGroup& g = groups[g0];
    const GemmPlan& h = plans[g.plan]->host;
    const int a = ga[g0];
    int c = gb[g0];
    int64_t ncols = 0;
    colptr_at.push_back(colptr_host.size());
    for (int gm : st) {
      const GemmPlan& hm = plans[groups[gm].plan]->host;
      for (int64_t n = 0; n < hm.N; ++n) {
        colptr_host.push_back(groups[gm].d + hm.offDn[n]);
        b->h_colptr_block.push_back(groups[gm].d);
      }
      ncols += hm.N;
    }
    if (ncols > 0x7fffffffLL) return fail(A4G_ERR_RANGE, "stacked destination too wide");
    if (st.size() > 1) {
      // stacks over the same member panels (the ring: every (a,i) row block
      // over all (b,j) columns) share one stacked panel, split once
      std::vector<int> key;
      for (int gm : st) key.push_back(gb[gm]);
      auto it = stacked_index.find(key);
      if (it != stacked_index.end()) {
        c = it->second;
      } else {
        PanelBuild sp;
        sp.rows = int(ncols);
        sp.kpad = pb[c].kpad;
        int row0 = 0;
        for (int gm : st) {
          sp.members.push_back({row0, gb[gm]});
          row0 += pb[gb[gm]].rows;
        }
        pb.push_back(sp);
        c = int(pb.size()) - 1;
        stacked_index.emplace(key, c);
      }
    }
    pb[c].used = true;
    {
      int row0 = 0;
      for (int gm : st) {
        col_panel[size_t(gm)] = {c, row0};
        row0 += pb[gb[gm]].rows;
      }
    }
    const int db = int(dblocks.size());
    const bool col_fast = h.N > 1 && h.offDn[1] - h.offDn[0] == 1 && !(h.M > 1 && h.offDm[1] - h.offDm[0] == 1);
    OzDBlock od{};
    od.d = g.d, od.plan = g.plan, od.panel_a = a, od.panel_b = c, od.col_fast = col_fast ? 1 : 0;
    od.M = int(h.M), od.N = int(ncols);
    od.rowoff = plans[g.plan]->offDm;
    dblocks.push_back(od);
    const int tb = int(trips.size());
    int kb_total = 0;
    for_stretches(g, pa[a], pb[gb[g0]], plans, [&](int, int, int64_t ka, int64_t kbo, int64_t kk) {
      const int nkb = int(ceil_to(kk, kOzBK) / kOzBK);
      trips.push_back({ka, kbo, nkb, 0});
      kb_total += nkb;
    });
    const int te = int(trips.size());
    dinfo.push_back({db, int(h.M), int(ncols), a, c, tb, te, kb_total});
  }
  {
    double** d_colptr = nullptr;
    int r = upload(b, colptr_host, &d_colptr);
    if (r) return r;
    for (size_t i = 0; i < dblocks.size(); ++i) dblocks[i].colptr = d_colptr + colptr_at[i];
    b->d_colptr = d_colptr;
    b->h_colptr = colptr_host;
    b->h_dblocks = dblocks;
  }
  const int S = b->slices;
  int rc0 = oz_prepare();
  if (rc0) return rc0;
  // panels: slices (BF16, zero padded), exponents, tensor maps
  std::vector<OzPanel> hpa, hpb;
  // one A descriptor (128-row boxes); B descriptors with 64-, 128- and
  // 256-row boxes for the forms' B halves / tiles
  std::vector<MapBytes> maps_a(pa.size()), maps_b64(pb.size()), maps_b128(pb.size()), maps_b256(pb.size());
  size_t exps_total = 0;
  for (auto& p : pa) exps_total += ceil_to(p.rows, 2 * kOzBM);
  b->exps_a_bytes = exps_total * sizeof(int);
  for (auto& p : pb)
    if (p.used) exps_total += ceil_to(p.rows, 2 * kOzBN);
  void* exps = nullptr;
  int rc = device_alloc(b, exps_total * sizeof(int), &exps, true);
  if (rc) return rc;
  b->d_exps = static_cast<int*>(exps);
  b->exps_bytes = exps_total * sizeof(int);
  size_t eoff = 0;
  // A and B panels are padded to 256 rows (every tile form fits).
  auto make_panels = [&](std::vector<PanelBuild>& src, std::vector<OzPanel>& dst, std::vector<MapBytes>& maps,
                         std::vector<MapBytes>* maps2, std::vector<MapBytes>* maps3, int rows_tile) -> int {
    for (size_t i = 0; i < src.size(); ++i) {
      OzPanel p{};
      if (!src[i].used) {  // read by no tile: no memory, no tensor map
        dst.push_back(p);
        continue;
      }
      p.rows = src[i].rows;
      p.rows_pad = int(ceil_to(src[i].rows, rows_tile));
      p.kpad = src[i].kpad;
      const size_t bytes = size_t(S) * p.rows_pad * size_t(p.kpad) * 2;
      void* mem = nullptr;
      int r = device_alloc(b, bytes, &mem, true);
      if (r) return r;
      p.base = static_cast<__nv_bfloat16*>(mem);
      p.exps = b->d_exps + eoff;
      eoff += p.rows_pad;
      r = oz_make_tensor_map(maps[i].b, mem, p.kpad, int64_t(S) * p.rows_pad, kOzBM);
      if (r) return r;
      if (maps2 && (r = oz_make_tensor_map((*maps2)[i].b, mem, p.kpad, int64_t(S) * p.rows_pad, 64))) return r;
      if (maps3 && (r = oz_make_tensor_map((*maps3)[i].b, mem, p.kpad, int64_t(S) * p.rows_pad, 256))) return r;
      dst.push_back(p);
    }
    return A4G_OK;
  };
  if ((rc = make_panels(pa, hpa, maps_a, nullptr, nullptr, 2 * kOzBM))) return rc;
  if ((rc = make_panels(pb, hpb, maps_b128, &maps_b64, &maps_b256, 2 * kOzBN))) return rc;
  for (size_t gi = 0; gi < groups.size(); ++gi) {
    const DGroup& g = groups[gi];
    const GemmPlan& h = plans[g.plan]->host;
    a4g_batch::ErrGroup eg{};
    eg.d = g.d;
    eg.rows = h.M, eg.cols = h.N, eg.size = h.M * h.N;
    eg.exp_rows = size_t(hpa[size_t(ga[gi])].exps - b->d_exps);
    eg.exp_cols = size_t(hpb[size_t(col_panel[gi].first)].exps - b->d_exps) + size_t(col_panel[gi].second);
    for (const Pair& p : g.pairs) eg.K += double(plans[p.plan]->host.K);
    b->err_groups.push_back(eg);
  }
  for (auto& p : hpa)
    if (p.kpad > 0x7fffffffLL || int64_t(S) * p.rows_pad > 0x7fffffffLL)
      return fail(A4G_ERR_RANGE, "panel exceeds TMA coordinate range");
  for (auto& p : hpb)
    if (p.kpad > 0x7fffffffLL || int64_t(S) * p.rows_pad > 0x7fffffffLL)
      return fail(A4G_ERR_RANGE, "panel exceeds TMA coordinate range");
  // split jobs (one per block per panel), grouped by side and source layout
  auto layout_of = [](const DevPlan* dp, bool left) {
    const GemmPlan& h = dp->host;
    const std::vector<int64_t>& orow = left ? h.offLm : h.offRn;
    const std::vector<int64_t>& ok = left ? h.offLk : h.offRk;
    const int64_t rows = int64_t(orow.size()), K = int64_t(ok.size());
    bool rm = true, km = true;
    for (int64_t r = 0; r < rows && (rm || km); ++r) rm &= orow[r] == r, km &= orow[r] == r * K;
    for (int64_t k = 0; k < K && (rm || km); ++k) rm &= ok[k] == k * rows, km &= ok[k] == k;
    return rm ? int(kOzRowsMajor) : km ? int(kOzKMajor) : int(kOzGeneric);
  };
  std::vector<OzSplitJob> host_jobs[2][3];  // [side][layout]
  // The split kernels see B panels through views: a plain panel as it is, a
  // stacked one as one view per member (base and exponents moved down to the
  // member's first row; the slice stride stays the stacked panel's).
  std::vector<OzPanel> hpb_view;
  std::vector<int> view_full;
  for (int side = 0; side < 2; ++side) {
    const bool left = side == 0;
    std::vector<PanelBuild>& src = left ? pa : pb;
    auto add_jobs = [&](const PanelBuild& blocks, int panel_index) {
      for (auto& kv : blocks.koff) {
        const DevPlan* dp = plans[blocks.plan.at(kv.first)];
        OzSplitJob j{};
        j.src = kv.first;
        j.offRow = left ? dp->offLm : dp->offRn;
        j.offK = left ? dp->offLk : dp->offRk;
        j.rows = int(left ? dp->host.M : dp->host.N);
        j.K = int(dp->host.K);
        j.kfast = left ? dp->host.a_kfast : dp->host.b_kfast;
        j.panel = panel_index;
        j.koff = kv.second;
        int lay = layout_of(dp, left);
        if ((reinterpret_cast<uintptr_t>(kv.first) & 15) != 0) lay = kOzGeneric;  // vector loads need 16 B
        host_jobs[side][lay].push_back(j);
      }
    };
    for (size_t pi = 0; pi < src.size(); ++pi) {
      if (!src[pi].used) continue;
      if (left) {
        add_jobs(src[pi], int(pi));
      } else if (src[pi].members.empty()) {
        hpb_view.push_back(hpb[pi]);
        view_full.push_back(int(pi));
        add_jobs(src[pi], int(hpb_view.size()) - 1);
      } else {
        for (const auto& mem : src[pi].members) {
          OzPanel v = hpb[pi];
          v.base += size_t(mem.first) * size_t(v.kpad);
          v.exps += mem.first;
          v.rows = pb[mem.second].rows;
          hpb_view.push_back(v);
          view_full.push_back(int(pi));
          add_jobs(pb[mem.second], int(hpb_view.size()) - 1);
        }
      }
    }
  }
  auto add_jobset = [&](bool left, int lay, int group, const std::vector<OzSplitJob>& jobs) -> int {
    if (jobs.empty()) return A4G_OK;
    a4g_batch::JobSet js;
    js.left = left;
    js.layout = lay;
    js.group = group;
    std::vector<int64_t> pe(1, 0), ps(1, 0);
    for (const OzSplitJob& j : jobs) {
      pe.push_back(pe.back() + oz_exp_tiles(lay, j.rows, j.K));
      ps.push_back(ps.back() + oz_split_tiles(lay, j.rows, j.K));
    }
    js.njobs = int(jobs.size());
    js.tiles_exp = pe.back();
    js.tiles_split = ps.back();
    js.h_jobs = jobs;
    int r;
    if ((r = upload(b, jobs, &js.d_jobs)) || (r = upload(b, pe, &js.d_prefix_exp)) ||
        (r = upload(b, ps, &js.d_prefix_split)))
      return r;
    b->jobsets.push_back(js);
    return A4G_OK;
  };
  void *dmaps_a = nullptr, *dmaps_b64 = nullptr, *dmaps_b128 = nullptr, *dmaps_b256 = nullptr;
  const size_t mbytes_a = maps_a.size() * sizeof(MapBytes), mbytes_b = maps_b128.size() * sizeof(MapBytes);
  if ((rc = device_alloc(b, mbytes_a, &dmaps_a, false))) return rc;
  if ((rc = device_alloc(b, mbytes_b, &dmaps_b64, false))) return rc;
  if ((rc = device_alloc(b, mbytes_b, &dmaps_b128, false))) return rc;
  if ((rc = device_alloc(b, mbytes_b, &dmaps_b256, false))) return rc;
  A4G_CUDA(cudaMemcpy(dmaps_a, maps_a.data(), mbytes_a, cudaMemcpyHostToDevice));
  A4G_CUDA(cudaMemcpy(dmaps_b64, maps_b64.data(), mbytes_b, cudaMemcpyHostToDevice));
  A4G_CUDA(cudaMemcpy(dmaps_b128, maps_b128.data(), mbytes_b, cudaMemcpyHostToDevice));
  A4G_CUDA(cudaMemcpy(dmaps_b256, maps_b256.data(), mbytes_b, cudaMemcpyHostToDevice));
  OzTrip* d_trips = nullptr;
  if ((rc = upload(b, hpa, &b->d_pa)) || (rc = upload(b, hpb, &b->d_pb)) || (rc = upload(b, trips, &d_trips)) ||
      (rc = upload(b, dblocks, &b->d_dblocks)) || (rc = upload(b, hpb_view, &b->d_pb_view)))
    return rc;
  for (int t = 0; t < S; ++t)
    if (oz_chunk_kb(t) < 1) return fail(A4G_ERR_ARG, "slice count too large for exact accumulation");
  int pairs = 0;
  if ((rc = oz_max_pairs(&pairs))) return rc;
  size_t ws_elems = 0;
  // Work units of one form: (level, split, tile), level-major, each split a
  // 1/nsplit share of the tile's concatenated k blocks; direct forms: (tile,
  // level), tile-major, one split.
  auto make_units = [&](const std::vector<OzTile>& tiles, int nsplit, bool tile_major = false) {
    std::vector<OzUnit> units;
    const int nt = int(tiles.size());
    for (int lv = 0; lv < S; ++lv)
      for (int sp = 0; sp < nsplit; ++sp)
        for (int ti = 0; ti < nt; ++ti) {
          const OzTile& t = tiles[ti];
          OzUnit u{};
          u.tile = ti, u.level = lv, u.split = sp;
          u.kb_begin = int(int64_t(t.kb_total) * sp / nsplit);
          u.kb_end = int(int64_t(t.kb_total) * (sp + 1) / nsplit);
          int acc = 0, q = t.trip_begin;
          while (q < t.trip_end && acc + trips[q].nkb <= u.kb_begin) acc += trips[q].nkb, ++q;
          u.trip_first = q;
          u.kb_in_trip = u.kb_begin - acc;
          units.push_back(u);
        }
    if (tile_major) {
      std::vector<OzUnit> tm(units.size());
      for (int lv = 0; lv < S; ++lv)
        for (int ti = 0; ti < nt; ++ti) tm[size_t(ti) * S + lv] = units[size_t(lv) * nt + ti];
      units.swap(tm);
    }
    return units;
  };
  // Direct forms fold the levels of a whole tile into one 64-bit integer,
  //   sum_t S_t 256^(S-1-t),  |S_t| <= (t+1) * K * 2^14  (digits |d| <= 128),
  // so they need |sum| < 2^63 for the longest k range (kept below 2^62 here),
  // and at least one k block per tile.
  bool direct_ok = S <= 6;
  {
    long double weight = 0.0L;
    for (int t = 0; t < S; ++t) weight += (long double)(t + 1) * std::pow(2.0L, 8 * (S - 1 - t));
    for (const OzTile& di : dinfo)
      direct_ok = direct_ok && di.kb_total >= 1 &&
                  (long double)di.kb_total * kOzBK * 16384.0L * weight < std::pow(2.0L, 62);
  }
  // A batch of the same structure tuned before in this process: build only
  // the form it chose, with the split-K count it chose.
  TuneRecord cached;
  const bool have_cached = !b->variant && tune_get(b->signature, &cached) && cached.form >= 0 &&
                           cached.form < a4g_batch::kForms && (cached.form < 4 || direct_ok);
  std::vector<std::vector<OzTile>> form_tiles(a4g_batch::kForms);
  std::vector<std::vector<OzUnit>> form_units(a4g_batch::kForms);
  for (int f = 0; f < a4g_batch::kForms; ++f) {
    a4g_batch::GemmForm& gf = b->forms[f];
    gf.pair = f & 1;
    gf.direct = f >= 4;
    gf.tile_rows = gf.pair ? 2 * kOzBM : kOzBM;
    gf.tile_cols = (f == 2 || f == 3) ? 2 * kOzBN : kOzBN;
    const int P = gf.pair ? pairs : ctx()->num_sms;  // concurrent workers (CTAs or CTA pairs)
    if (P < 1 || (b->variant && b->variant != f + 1)) continue;
    if (have_cached && f != cached.form) continue;
    if (gf.direct && !direct_ok) continue;
    std::vector<OzTile>& tiles = form_tiles[f];
    for (const OzTile& di : dinfo)
      for (int64_t n0 = 0; n0 < di.n0; n0 += gf.tile_cols)
        for (int64_t m0 = 0; m0 < di.m0; m0 += gf.tile_rows)
          tiles.push_back({di.dblock, int(m0), int(n0), di.panel_a, di.panel_b, di.trip_begin, di.trip_end,
                           di.kb_total});
    gf.n_tiles = int(tiles.size());
    // Split-K: units short enough that a level sum of one unit stays below
    // 2^31 (slices * 128^2 * K_unit < 2^31, written as int32), then the
    // smallest split count that gives every worker the same number of equal
    // units per level (the workers then stay in step through the k panels),
    // keeping at least 16 k blocks per unit and the workspace below 6 GB.
    const int max_unit_kb = int(((1LL << 31) - 1) / (int64_t(S) * 128 * 128 * kOzBK));
    int min_kb = 1 << 30, max_kb = 0;
    for (const OzTile& t : tiles) min_kb = std::min(min_kb, t.kb_total), max_kb = std::max(max_kb, t.kb_total);
    const int ns_min = std::max(1, (max_kb + max_unit_kb - 1) / max_unit_kb);
    const double tile_bytes = double(gf.tile_rows) * gf.tile_cols * sizeof(int);
    int nsplit = ns_min;
    double best = -1.0;
    for (int ns = ns_min; !gf.direct && ns <= std::max(64, ns_min); ++ns) {
      if (ns > ns_min && min_kb / ns < 16) break;
      if (ns > ns_min && double(gf.n_tiles) * S * ns * tile_bytes > 6.0 * (1u << 30)) break;
      const int64_t units = int64_t(gf.n_tiles) * ns;
      const double eff = double(units) / double(P * ((units + P - 1) / P));
      if (eff > best + 1e-9) best = eff, nsplit = ns;
      if (eff >= 0.999) break;
    }
    if (gf.direct) nsplit = 1;
    if (have_cached && !gf.direct && cached.nsplit > 0) nsplit = std::max(cached.nsplit, ns_min);
    gf.nsplit = nsplit;
    std::vector<OzUnit>& units = form_units[f];
    units = make_units(tiles, nsplit, gf.direct);
    if (!gf.direct) ws_elems = std::max(ws_elems, size_t(gf.n_tiles) * S * nsplit * gf.tile_rows * gf.tile_cols);
    OzUnit* d_units = nullptr;
    if ((rc = upload(b, tiles, &gf.d_tiles)) || (rc = upload(b, units, &d_units))) return rc;
    OzGemmArgs& ga = gf.args;
    const int bbox = gf.pair ? gf.tile_cols / 2 : gf.tile_cols;  // B rows one CTA loads
    ga.maps_a = dmaps_a, ga.maps_b = bbox == 64 ? dmaps_b64 : bbox == 128 ? dmaps_b128 : dmaps_b256;
    ga.panels_a = b->d_pa, ga.panels_b = b->d_pb;
    ga.tiles = gf.d_tiles, ga.trips = d_trips;
    ga.n_tiles = gf.n_tiles;
    ga.units = d_units;
    ga.n_units = int(units.size());
    ga.slices = S;
    ga.nsplit = nsplit;
    for (int t = 0; t < kOzMaxSlices; ++t) ga.chunk_kb[t] = t < S ? oz_chunk_kb(t) : 1;
    ga.err_flag = ctx()->d_error_flag;
    ga.direct = gf.direct ? 1 : 0;
    ga.mode = b->store_mode();
    ga.dry = 0;
    ga.dblocks = b->d_dblocks;
    const int workers = gf.direct ? gf.n_tiles : ga.n_units;
    gf.grid = gf.pair ? 2 * std::min(workers, pairs) : std::min(workers, ctx()->num_sms);
    gf.built = true;
  }
  void* ws = nullptr;
  if ((rc = device_alloc(b, ws_elems * sizeof(int), &ws, false))) return rc;
  b->d_ws = static_cast<int*>(ws);
  for (auto& gf : b->forms) gf.args.ws = b->d_ws;
  b->form = -1;
  for (int f = 0; f < a4g_batch::kForms; ++f)
    if (b->forms[f].built && (b->form < 0 || b->variant == f + 1)) b->form = f;
  if (b->form < 0) return fail(A4G_ERR_UNSUPPORTED, "no tensor-core GEMM form fits this GPU");
  if (have_cached) {
    for (int f = 0; f < a4g_batch::kForms; ++f) b->forms[f].score_ms = b->forms[f].tuned_ms = cached.score_ms[f];
    for (int i = 0; i < 2; ++i)
      b->split_candidates[i] = cached.split_candidates[i], b->split_cost_ms[i] = cached.split_cost_ms[i];
    b->tuned_from_cache = true;
  }
  const auto tune_t0 = std::chrono::steady_clock::now();
  if (!b->variant && !have_cached) {
    // The panels hold the operands' digits during the autotune: the tensor
    // cores draw far less power on zero panels and would run at clocks the
    // real step does not get.  So the exponent and split passes run once here
    // (on the blocks' contents at creation; every run repeats them).
    for (int side = 0; side < 2 && !rc; ++side)
      for (int lay = 0; lay < 3 && !rc; ++lay) rc = add_jobset(side == 0, lay, 0, host_jobs[side][lay]);
    if (!rc) {
      cudaStream_t s = ctx()->stream;
      A4G_CUDA(cudaMemsetAsync(b->d_exps, 0, b->exps_bytes, s));
      for (const auto& js : b->jobsets)
        if (!rc) rc = oz_launch_exp(js.layout, js.d_jobs, js.d_prefix_exp, js.njobs, js.tiles_exp,
                                    js.left ? b->d_pa : b->d_pb_view, s);
      for (const auto& js : b->jobsets)
        if (!rc) rc = oz_launch_split(js.layout, js.d_jobs, js.d_prefix_split, js.njobs, js.tiles_split,
                                      js.left ? b->d_pa : b->d_pb_view, S, s);
      if (!rc) rc = check_device_flag(s);
    }
    for (const auto& js : b->jobsets) {
      release(b, js.d_jobs, size_t(js.njobs) * sizeof(OzSplitJob));
      release(b, js.d_prefix_exp, size_t(js.njobs + 1) * sizeof(int64_t));
      release(b, js.d_prefix_split, size_t(js.njobs + 1) * sizeof(int64_t));
    }
    b->jobsets.clear();
    if (rc) return rc;
    // Autotune on this batch's own panels: each form's GEMM and, for the
    // workspace forms, the recombine after it, timed once after one untimed
    // run, storing into scratch destination blocks so that the caller's
    // blocks stay untouched; the lowest time wins.  Then the chosen
    // workspace form's split-K count is timed against its double.  If the
    // scratch cannot be had, direct forms run without their stores and the
    // traffic left out is added at the copy rate.
    size_t d_max = 0, d_total = 0;
    double d_bytes = 0.0;
    for (const DGroup& g : groups) {
      const GemmPlan& h = plans[g.plan]->host;
      d_max = std::max(d_max, size_t(h.M) * size_t(h.N));
      d_total += size_t(h.M) * size_t(h.N);
      d_bytes += double(h.M) * double(h.N) * sizeof(double) * (b->beta ? 2 : 1);
    }
    const double ms_per_byte = 1.0 / 6.5e9;  // ~ the measured copy rate, bytes per ms
    // One scratch block per destination block (the real store pattern and
    // footprint) when a quarter of the free memory holds them, else one
    // shared block of the largest size; the column bases point into them.
    size_t free_b = 0, total_b = 0;
    const bool spread = cudaMemGetInfo(&free_b, &total_b) == cudaSuccess && d_total * sizeof(double) <= free_b / 4;
    cudaGetLastError();
    double* scratch = nullptr;
    OzDBlock* sdb = nullptr;
    double** scols = nullptr;
    if (cudaMalloc(&scratch, std::max<size_t>(spread ? d_total : d_max, 1) * sizeof(double)) == cudaSuccess) {
      std::vector<double*> cps;
      cps.reserve(colptr_host.size());
      size_t off = 0;
      for (const std::vector<int>& st : stacks)
        for (int gm : st) {
          const GemmPlan& hm = plans[groups[gm].plan]->host;
          double* base = scratch + (spread ? off : 0);
          for (int64_t n = 0; n < hm.N; ++n) cps.push_back(base + hm.offDn[n]);
          off += size_t(hm.M) * size_t(hm.N);
        }
      std::vector<OzDBlock> hs = dblocks;
      bool ok = cudaMalloc(&scols, std::max<size_t>(cps.size(), 1) * sizeof(double*)) == cudaSuccess &&
                cudaMemcpy(scols, cps.data(), cps.size() * sizeof(double*), cudaMemcpyHostToDevice) == cudaSuccess;
      for (size_t i = 0; i < hs.size(); ++i) hs[i].d = scratch, hs[i].colptr = scols + colptr_at[i];
      ok = ok && cudaMalloc(&sdb, hs.size() * sizeof(OzDBlock)) == cudaSuccess &&
           cudaMemcpy(sdb, hs.data(), hs.size() * sizeof(OzDBlock), cudaMemcpyHostToDevice) == cudaSuccess;
      if (!ok) {
        cudaFree(sdb);
        cudaFree(scols);
        cudaFree(scratch);
        sdb = nullptr, scols = nullptr, scratch = nullptr;
      }
    }
    cudaGetLastError();  // a failed scratch allocation is not an error of the batch
    cudaStream_t s = ctx()->stream;
    cudaEvent_t e0, e1;
    A4G_CUDA(cudaEventCreate(&e0));
    A4G_CUDA(cudaEventCreate(&e1));
    // time one form (GEMM args ga, its tile list) in ms, modelled traffic included
    auto time_form = [&](const a4g_batch::GemmForm& gf, const OzGemmArgs& ga, int grid, float* ms) -> int {
      OzGemmArgs ta = ga;
      if (sdb) ta.dblocks = sdb;
      else ta.dry = 1;
      int r = A4G_OK;
      for (int rep = 0; rep < 2 && !r; ++rep) {
        if (rep == 1 && cudaEventRecord(e0, s) != cudaSuccess) return cuda_fail(cudaGetLastError(), "event");
        r = oz_launch_gemm(ta, grid, gf.pair, gf.tile_cols, s);
        if (!r && !gf.direct && sdb)
          r = oz_launch_recombine(gf.d_tiles, gf.n_tiles, gf.tile_rows, gf.tile_cols, sdb, b->d_pa,
                                  b->d_pb, ta.ws, S, ta.nsplit, b->store_mode(), s);
      }
      if (r) return r;
      A4G_CUDA(cudaEventRecord(e1, s));
      A4G_CUDA(cudaEventSynchronize(e1));
      A4G_CUDA(cudaEventElapsedTime(ms, e0, e1));
      if (!sdb) {
        const double ws_bytes = gf.direct ? 0.0 : double(gf.n_tiles) * S * ta.nsplit * gf.tile_rows *
                                                      gf.tile_cols * sizeof(int);
        *ms += float((ws_bytes + d_bytes) * ms_per_byte);
      }
      return check_device_flag(s);
    };
    float best = 0.f;
    for (int f = 0; f < a4g_batch::kForms && !rc; ++f) {
      a4g_batch::GemmForm& gf = b->forms[f];
      if (!gf.built) continue;
      if ((rc = time_form(gf, gf.args, gf.grid, &gf.score_ms))) break;
      gf.tuned_ms = gf.score_ms;
      if (best == 0.f || gf.score_ms < best) best = gf.score_ms, b->form = f;
    }
    // split-count tuning of the chosen workspace form: the balance-driven
    // count against its double (shorter k windows per unit, twice the
    // workspace for the recombine to read)
    a4g_batch::GemmForm& gf = b->forms[b->form];
    const std::vector<OzTile>& tiles = form_tiles[b->form];
    int min_kb = 1 << 30;
    for (const OzTile& t : tiles) min_kb = std::min(min_kb, t.kb_total);
    const int ns1 = gf.nsplit, ns2 = 2 * ns1;
    const double ws2 = 2.0 * double(gf.n_tiles) * S * ns1 * gf.tile_rows * gf.tile_cols * sizeof(int);
    if (!rc && !gf.direct) {
      b->split_candidates[0] = ns1;
      b->split_cost_ms[0] = gf.score_ms;
    }
    if (!rc && !gf.direct && gf.n_tiles > 0 && ns2 <= 64 && min_kb / ns2 >= 16 && ws2 <= 6.0 * (1u << 30)) {
      std::vector<OzUnit> units2 = make_units(tiles, ns2);
      OzUnit* d_units2 = nullptr;
      void* ws2p = nullptr;
      if (!(rc = upload(b, units2, &d_units2)) && !(rc = device_alloc(b, size_t(ws2), &ws2p, false))) {
        OzGemmArgs a2 = gf.args;
        a2.units = d_units2;
        a2.n_units = int(units2.size());
        a2.nsplit = ns2;
        a2.ws = static_cast<int*>(ws2p);
        const int grid2 = gf.pair ? 2 * std::min(a2.n_units, pairs) : std::min(a2.n_units, ctx()->num_sms);
        float ms2 = 0.f;
        if (!(rc = time_form(gf, a2, grid2, &ms2))) {
          b->split_candidates[1] = ns2;
          b->split_cost_ms[1] = ms2;
          if (ms2 < 0.97f * b->split_cost_ms[0]) {  // a clear win only: one timed run each is noisy
            // the other forms are not run any more: their units and the
            // shared workspace go
            for (int f = 0; f < a4g_batch::kForms; ++f)
              if (b->forms[f].built)
                release(b, const_cast<OzUnit*>(b->forms[f].args.units), form_units[f].size() * sizeof(OzUnit)),
                    b->forms[f].args.units = nullptr;
            release(b, b->d_ws, ws_elems * sizeof(int));
            gf.args = a2;
            gf.nsplit = ns2;
            gf.grid = grid2;
            b->d_ws = a2.ws;
            form_units[b->form].swap(units2);
          } else {
            release(b, d_units2, units2.size() * sizeof(OzUnit));
            release(b, ws2p, size_t(ws2));
          }
        }
      }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (sdb) cudaFree(sdb);
    if (scols) cudaFree(scols);
    if (scratch) cudaFree(scratch);
    if (rc) return rc;
    TuneRecord rec;
    rec.form = b->form;
    rec.nsplit = b->forms[b->form].nsplit;
    for (int f = 0; f < a4g_batch::kForms; ++f) rec.score_ms[f] = b->forms[f].score_ms;
    for (int i = 0; i < 2; ++i)
      rec.split_candidates[i] = b->split_candidates[i], rec.split_cost_ms[i] = b->split_cost_ms[i];
    tune_put(b->signature, rec);
    b->autotune_ms =
        std::chrono::duration<float, std::milli>(std::chrono::steady_clock::now() - tune_t0).count();
  }
  // Pipeline of the chosen form (when the caller asks for one): GEMM parts
  // over consecutive split-K ranges; each k-major right-operand split job
  // joins the group of the first part that reads its columns.  (Those jobs
  // need no shared memory and few registers, so they run beside the
  // persistent GEMM's CTAs; the other split kernels run before the GEMM.)
  const a4g_batch::GemmForm& gf = b->forms[b->form];
  const int ns = gf.nsplit;
  std::vector<OzSplitJob>& kmaj = host_jobs[1][kOzKMajor];
  int P = std::min(std::min(b->pipeline, kOzMaxPipelineParts), ns);
  std::vector<int> job_group(kmaj.size(), 0);
  if (P > 1 && !kmaj.empty()) {
    std::vector<int> part_of_split(ns);
    for (int p = 0; p < P; ++p)
      for (int sp = ns * p / P; sp < ns * (p + 1) / P; ++sp) part_of_split[sp] = p;
    std::vector<std::vector<int>> need(pb.size());
    for (size_t i = 0; i < pb.size(); ++i) need[i].assign(size_t(pb[i].kpad / kOzK16), P);
    const std::vector<OzTile>& tiles = form_tiles[b->form];
    for (const OzUnit& u : form_units[b->form]) {
      if (u.level != 0) continue;  // every level reads the same columns
      const int part = part_of_split[u.split];
      const OzTile& t = tiles[u.tile];
      std::vector<int>& nd = need[t.panel_b];
      int q = u.trip_first, j = u.kb_in_trip;
      for (int kb = u.kb_begin; kb < u.kb_end && q < t.trip_end; ++kb) {
        const int64_t c0 = (trips[q].koff_b + int64_t(j) * kOzBK) / kOzK16;
        for (int64_t c = c0; c < c0 + kOzBK / kOzK16 && c < int64_t(nd.size()); ++c) nd[c] = std::min(nd[c], part);
        if (++j == trips[q].nkb) ++q, j = 0;
      }
    }
    bool any_late = false;
    for (size_t i = 0; i < kmaj.size(); ++i) {
      const std::vector<int>& nd = need[view_full[kmaj[i].panel]];
      int g = P;
      for (int64_t c = kmaj[i].koff / kOzK16; c <= (kmaj[i].koff + kmaj[i].K - 1) / kOzK16; ++c) g = std::min(g, nd[c]);
      job_group[i] = g >= P ? 0 : g;
      any_late |= job_group[i] > 0;
    }
    if (!any_late) P = 1;
  } else {
    P = 1;
  }
  for (int side = 0; side < 2; ++side)
    for (int lay = 0; lay < 3; ++lay) {
      if (side == 1 && lay == kOzKMajor) continue;
      if ((rc = add_jobset(side == 0, lay, 0, host_jobs[side][lay]))) return rc;
    }
  for (int g = 0; g < P; ++g) {
    std::vector<OzSplitJob> grp;
    for (size_t i = 0; i < kmaj.size(); ++i)
      if (job_group[i] == g) grp.push_back(kmaj[i]);
    if ((rc = add_jobset(false, kOzKMajor, g, grp))) return rc;
  }
  b->parts = P;
  if (P > 1) {
    // units of part p: levels from the most expensive down (the launch's
    // tail then holds the cheapest units), its splits, every tile
    const std::vector<OzUnit>& all = form_units[b->form];
    std::vector<OzUnit> units;
    std::vector<size_t> start;
    for (int p = 0; p < P; ++p) {
      start.push_back(units.size());
      for (int lv = S - 1; lv >= 0; --lv)
        for (int sp = ns * p / P; sp < ns * (p + 1) / P; ++sp)
          for (int ti = 0; ti < gf.n_tiles; ++ti) units.push_back(all[(size_t(lv) * ns + sp) * gf.n_tiles + ti]);
    }
    start.push_back(units.size());
    OzUnit* d_units = nullptr;
    if ((rc = upload(b, units, &d_units))) return rc;
    for (int p = 0; p < P; ++p) {
      OzGemmArgs ga = gf.args;
      ga.units = d_units + start[p];
      ga.n_units = int(start[p + 1] - start[p]);
      b->part_args.push_back(ga);
      b->part_grid.push_back(gf.pair ? 2 * std::min(ga.n_units, pairs) : std::min(ga.n_units, ctx()->num_sms));
    }
    A4G_CUDA(cudaStreamCreateWithFlags(&b->side, cudaStreamNonBlocking));
    b->part_ev.resize(P);
    for (auto& e : b->part_ev) A4G_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
  }
  return A4G_OK;
}

// ------------------------------------------------------------ rebind tables
// The tables a rebind rewrites are copied into place by this kernel, reading
// a pinned, mapped host slot over the host link, on the caller's stream.  A
// copy-engine transfer (cudaMemcpyAsync) would queue behind the caller's own
// bulk host-to-device copies on the same engine — the next pardo iteration's
// operands streaming in — and hold the stream for as long as they take.
struct TableCopy {
  const unsigned long long* src;
  unsigned long long* dst;
  int64_t words;  // 8-byte words
};
constexpr int kMaxTableCopies = 16;
struct TableCopies {
  TableCopy c[kMaxTableCopies];
  int n;
};

__global__ void __launch_bounds__(256) copy_tables_kernel(TableCopies t) {
  const int64_t stride = int64_t(gridDim.x) * blockDim.x;
  for (int i = 0; i < t.n; ++i) {
    const TableCopy c = t.c[i];
    for (int64_t w = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; w < c.words; w += stride) c.dst[w] = c.src[w];
  }
}

static_assert(sizeof(OzSplitJob) % 8 == 0 && sizeof(OzDBlock) % 8 == 0 && sizeof(GroupedPair) % 8 == 0 &&
                  sizeof(GroupedF64Tile) % 8 == 0 && sizeof(GroupedF64Reduce) % 8 == 0,
              "tables are copied in 8-byte words");

// One rebind's worth of table copies staged in the next ring slot.
struct Staging {
  a4g_batch* b;
  size_t used = 0;
  int slot = 0;
  std::vector<TableCopy> copies;
  int add(void* dev, const void* host, size_t bytes) {
    if (!bytes) return A4G_OK;
    if (used + bytes > b->stage_bytes) return fail(A4G_ERR_RANGE, "rebind: staging slot overflow");
    const size_t at = size_t(slot) * b->stage_bytes + used;
    std::memcpy(b->h_stage + at, host, bytes);
    copies.push_back({reinterpret_cast<const unsigned long long*>(b->d_stage + at),
                      static_cast<unsigned long long*>(dev), int64_t(bytes / 8)});
    used += bytes;
    return A4G_OK;
  }
};

// Takes the next ring slot (waiting for the copy that last read it), sized
// for every table of the batch.
int stage_begin(a4g_batch* b, size_t bytes, Staging* st) {
  if (!b->h_stage || b->stage_bytes < bytes) {
    for (int i = 0; i < a4g_batch::kStageRing; ++i)
      if (b->stage_busy[i]) {
        A4G_CUDA(cudaEventSynchronize(b->stage_ev[i]));
        b->stage_busy[i] = false;
      }
    if (b->h_stage) cudaFreeHost(b->h_stage), b->h_stage = nullptr;
    b->stage_bytes = std::max<size_t>(bytes, 8);
    void* h = nullptr;
    A4G_CUDA(cudaHostAlloc(&h, b->stage_bytes * a4g_batch::kStageRing, cudaHostAllocMapped));
    b->h_stage = static_cast<char*>(h);
    void* d = nullptr;
    A4G_CUDA(cudaHostGetDevicePointer(&d, h, 0));
    b->d_stage = static_cast<char*>(d);
    for (int i = 0; i < a4g_batch::kStageRing; ++i)
      if (!b->stage_ev[i]) A4G_CUDA(cudaEventCreateWithFlags(&b->stage_ev[i], cudaEventDisableTiming));
  }
  st->b = b;
  st->slot = b->stage_next;
  b->stage_next = (b->stage_next + 1) % a4g_batch::kStageRing;
  if (b->stage_busy[st->slot]) A4G_CUDA(cudaEventSynchronize(b->stage_ev[st->slot]));
  b->stage_busy[st->slot] = false;
  return A4G_OK;
}

int stage_launch(Staging& st, cudaStream_t s) {
  a4g_batch* b = st.b;
  int64_t words = 0;
  for (const TableCopy& c : st.copies) words = std::max(words, c.words);
  const int grid = int(std::max<int64_t>(1, std::min<int64_t>(64, (words + 255) / 256)));
  for (size_t i = 0; i < st.copies.size(); i += kMaxTableCopies) {
    TableCopies t{};
    t.n = int(std::min<size_t>(kMaxTableCopies, st.copies.size() - i));
    for (int k = 0; k < t.n; ++k) t.c[k] = st.copies[i + size_t(k)];
    copy_tables_kernel<<<grid, 256, 0, s>>>(t);
    A4G_CUDA(cudaGetLastError());
  }
  A4G_CUDA(cudaEventRecord(b->stage_ev[st.slot], s));
  b->stage_busy[st.slot] = true;
  return A4G_OK;
}

// Zeroes the exponents of the A panels (side 0) and/or the B panels (side 1).
int clear_exps(a4g_batch* b, bool side_a, bool side_b, cudaStream_t s) {
  const size_t a = b->exps_a_bytes, all = b->exps_bytes;
  if (side_a && side_b) {
    A4G_CUDA(cudaMemsetAsync(b->d_exps, 0, all, s));
  } else if (side_a && a > 0) {
    A4G_CUDA(cudaMemsetAsync(b->d_exps, 0, a, s));
  } else if (side_b && all > a) {
    A4G_CUDA(cudaMemsetAsync(reinterpret_cast<char*>(b->d_exps) + a, 0, all - a, s));
  }
  return A4G_OK;
}

// Exponent and split passes of the split jobs of one side (0: A, 1: B) or of
// both (side < 0), split pipeline groups included.
int slice_side(a4g_batch* b, int side, cudaStream_t s) {
  int rc = clear_exps(b, side != 1, side != 0, s);
  for (const auto& js : b->jobsets)
    if (!rc && (side < 0 || side == (js.left ? 0 : 1)))
      rc = oz_launch_exp(js.layout, js.d_jobs, js.d_prefix_exp, js.njobs, js.tiles_exp,
                         js.left ? b->d_pa : b->d_pb_view, s);
  for (const auto& js : b->jobsets)
    if (!rc && (side < 0 || side == (js.left ? 0 : 1)))
      rc = oz_launch_split(js.layout, js.d_jobs, js.d_prefix_split, js.njobs, js.tiles_split,
                           js.left ? b->d_pa : b->d_pb_view, b->slices, s);
  return rc;
}

// Drops the captured graph (its recorded launches no longer match the
// batch), after the work queued on the device has finished with it.
int drop_graph(a4g_batch* b) {
  if (!b->graph) return A4G_OK;
  A4G_CUDA(cudaDeviceSynchronize());
  A4G_CUDA(cudaGraphExecDestroy(b->graph));
  b->graph = nullptr;
  return A4G_OK;
}

// ev (optional) receives 6 events: before phase 0 and after each of phases 0..4.
int run(a4g_batch* b, cudaStream_t s, const cudaEvent_t* ev = nullptr) {
  int rc = A4G_OK;
  auto mark = [&](int i) -> int {
    if (ev) A4G_CUDA(cudaEventRecord(ev[i], s));
    return A4G_OK;
  };
  if ((rc = mark(0))) return rc;
  if (b->beta == 0)
    for (auto& z : b->zero_blocks)
      if ((rc = launch_fill(z.first, z.second, 0.0, s))) return rc;
  if ((rc = mark(1))) return rc;
  if (b->precision == A4G_PREC_FP64) {
    if ((rc = mark(2)) || (rc = mark(3))) return rc;
    rc = launch_grouped_f64(b->d_f64_tiles, b->n_f64_tiles, b->d_f64_pairs, b->d_plans, b->store_mode(),
                            b->d_f64_ws, b->d_f64_reds, b->n_f64_reds, b->f64_tile_m, b->f64_tile_n, s);
    if (rc) return rc;
    if ((rc = mark(4)) || (rc = mark(5))) return rc;
    return A4G_OK;
  }
  const a4g_batch::GemmForm& gf = b->forms[b->form];
  // a held side keeps the digits a4g_batch_hold sliced: no passes over it
  auto sliced = [&](const a4g_batch::JobSet& js) { return !b->held[js.left ? 0 : 1]; };
  if (gf.n_tiles > 0) {
    if ((rc = clear_exps(b, !b->held[0], !b->held[1], s))) return rc;
    for (const auto& js : b->jobsets)
      if (sliced(js) && (rc = oz_launch_exp(js.layout, js.d_jobs, js.d_prefix_exp, js.njobs, js.tiles_exp,
                                            js.left ? b->d_pa : b->d_pb_view, s)))
        return rc;
  }
  if ((rc = mark(2))) return rc;
  auto split_group = [&](int g, cudaStream_t st) -> int {
    for (const auto& js : b->jobsets)
      if (js.group == g && sliced(js)) {
        const int r = oz_launch_split(js.layout, js.d_jobs, js.d_prefix_split, js.njobs, js.tiles_split,
                                      js.left ? b->d_pa : b->d_pb_view, b->slices, st);
        if (r) return r;
      }
    return A4G_OK;
  };
  if (gf.n_tiles > 0 && (rc = split_group(0, s))) return rc;
  if (gf.n_tiles > 0 && b->parts > 1) {
    // groups 1.. on the side stream, overlapping the GEMM parts before them
    A4G_CUDA(cudaEventRecord(b->part_ev[0], s));
    A4G_CUDA(cudaStreamWaitEvent(b->side, b->part_ev[0], 0));
    for (int g = 1; g < b->parts; ++g) {
      if ((rc = split_group(g, b->side))) return rc;
      A4G_CUDA(cudaEventRecord(b->part_ev[g], b->side));
    }
  }
  if ((rc = mark(3))) return rc;
  if (gf.n_tiles > 0) {
    if (b->parts > 1) {
      for (int p = 0; p < b->parts; ++p) {
        if (p > 0) A4G_CUDA(cudaStreamWaitEvent(s, b->part_ev[p], 0));
        if ((rc = oz_launch_gemm(b->part_args[p], b->part_grid[p], gf.pair, gf.tile_cols, s))) return rc;
      }
    } else if ((rc = oz_launch_gemm(gf.args, gf.grid, gf.pair, gf.tile_cols, s))) {
      return rc;
    }
  }
  if ((rc = mark(4))) return rc;
  if (gf.n_tiles > 0 && !gf.direct &&
      (rc = oz_launch_recombine(gf.d_tiles, gf.n_tiles, gf.tile_rows, gf.tile_cols, b->d_dblocks,
                                b->d_pa, b->d_pb, b->d_ws, b->slices, gf.nsplit, b->store_mode(), s)))
    return rc;
  return mark(5);
}

}  // namespace

extern "C" {

int a4g_batch_create(a4g_batch** out, const int* ptrn, int drank, int lrank, int rrank,
                     const a4g_triple* trip, int64_t n, const a4g_batch_opts* opts) {
  if (!out) return fail(A4G_ERR_ARG, "null output handle");
  *out = nullptr;
  int rc = ensure_init();
  if (rc) return rc;
  if (!ptrn || (n > 0 && !trip)) return fail(A4G_ERR_ARG, "null argument");
  if (drank < 1 || drank > 6 || lrank < 1 || lrank > 6 || rrank < 1 || rrank > 6)
    return fail(A4G_ERR_UNSUPPORTED, "batched contraction needs tensor operands of rank 1..6");
  std::unique_ptr<a4g_batch> b(new a4g_batch());
  if (opts) {
    b->precision = opts->precision;
    b->slices = opts->slices > 0 ? opts->slices : 5;
    b->beta = opts->beta ? 1 : 0;
    b->negate = opts->negate ? 1 : 0;
    b->pipeline = opts->pipeline;
    b->variant = opts->variant;
  }
  if (b->variant < 0 || b->variant > a4g_batch::kForms) return fail(A4G_ERR_ARG, "unknown GEMM variant");
  if (b->precision != A4G_PREC_FP64 && b->precision != A4G_PREC_OZAKI_BF16)
    return fail(A4G_ERR_ARG, "unknown precision mode");
  if (b->slices < 1 || b->slices > kOzMaxUsableSlices) return fail(A4G_ERR_ARG, "slices must be 1..7");
  b->drank = drank, b->lrank = lrank, b->rrank = rrank;
  if (n > 0) b->bound.assign(trip, trip + n);
  if (b->precision == A4G_PREC_OZAKI_BF16) b->signature = batch_signature(b.get(), ptrn, trip, n);

  std::vector<const DevPlan*> plans;
  std::map<const DevPlan*, int> plan_index;
  std::vector<DGroup> groups;
  std::map<double*, int> gindex;
  std::map<double*, int64_t> all_d;
  for (int64_t i = 0; i < n; ++i) {
    const a4g_triple& t = trip[i];
    if (!t.d) return fail(A4G_ERR_ARG, "triple with NULL destination");
    int64_t dsize = 1;
    for (int q = 0; q < drank; ++q) dsize *= t.dext[q];
    all_d[t.d] = dsize;
    if (!t.l || !t.r) continue;  // zero block: skipped
    const DevPlan* p = nullptr;
    if ((rc = get_dev_plan(ptrn, lrank, t.lext, rrank, t.rext, drank, t.dext, &p))) return rc;
    if (p->host.kind != ContractKind::kTensorTensor)
      return fail(A4G_ERR_UNSUPPORTED, "batched contraction of scalar operands");
    if (p->host.M > 0x7fffffff || p->host.N > 0x7fffffff || p->host.K > 0x7fffffff)
      return fail(A4G_ERR_RANGE, "block too large");
    auto pit = plan_index.find(p);
    int pi;
    if (pit == plan_index.end()) {
      pi = int(plans.size());
      plans.push_back(p);
      plan_index[p] = pi;
    } else {
      pi = pit->second;
    }
    auto git = gindex.find(t.d);
    if (git == gindex.end()) {
      gindex[t.d] = int(groups.size());
      groups.push_back(DGroup{t.d, {}, pi});
      git = gindex.find(t.d);
    }
    DGroup& g = groups[git->second];
    const GemmPlan& h0 = plans[g.plan]->host;
    if (h0.M != p->host.M || h0.N != p->host.N)
      return fail(A4G_ERR_ARG, "triples sharing a destination block disagree on its extents");
    g.pairs.push_back({t.l, t.r, pi});
    b->pairs += 1;
    b->flops += 2.0 * double(p->host.M) * double(p->host.N) * double(p->host.K);
  }
  for (auto& kv : all_d)
    if (!gindex.count(kv.first)) b->zero_blocks.push_back({kv.first, kv.second});
  if (b->precision == A4G_PREC_OZAKI_BF16 && !groups.empty()) {
    // The split form's epilogues walk a tile by rows (one TMEM lane per row),
    // so D's unit-stride index belongs along the rows.  When the pattern puts
    // it on the right operand's side, multiply with the roles exchanged: the
    // level sums are exact integer sums over the same digit products, so the
    // result is identical.
    const GemmPlan& h = plans[groups[0].plan]->host;
    if (h.N > 1 && h.offDn[1] - h.offDn[0] == 1 && !(h.M > 1 && h.offDm[1] - h.offDm[0] == 1)) {
      b->swapped = true;
      for (const DevPlan*& p : plans) {
        b->own_plans.emplace_back();
        DevPlan& q = b->own_plans.back();
        q.host = p->host;
        std::swap(q.host.M, q.host.N);
        std::swap(q.host.offLm, q.host.offRn);
        std::swap(q.host.offLk, q.host.offRk);
        std::swap(q.host.offDm, q.host.offDn);
        std::swap(q.host.a_kfast, q.host.b_kfast);
        q.d_tables = nullptr;  // the tables stay owned by the plan cache
        q.offLm = p->offRn, q.offLk = p->offRk, q.offRk = p->offLk, q.offRn = p->offLm;
        q.offDm = p->offDn, q.offDn = p->offDm;
        p = &q;
      }
      for (DGroup& g : groups)
        for (Pair& pr : g.pairs) std::swap(pr.l, pr.r);
    }
  }
  std::vector<PlanRef> refs;
  for (const DevPlan* p : plans) refs.push_back(ref_of(p));
  if ((rc = upload(b.get(), refs, &b->d_plans))) return rc;
  rc = b->precision == A4G_PREC_FP64 ? build_f64(b.get(), groups, plans) : build_ozaki(b.get(), groups, plans);
  if (rc) return rc;
  *out = b.release();
  return A4G_OK;
}

int a4g_batch_run(a4g_batch* b, void* stream) {
  if (!b) return fail(A4G_ERR_ARG, "null batch");
  return run(b, pick(stream));
}

int a4g_batch_run_graph(a4g_batch* b, void* stream) {
  if (!b) return fail(A4G_ERR_ARG, "null batch");
  cudaStream_t s = pick(stream);
  if (!b->graph) {
    // capture on a private stream: the caller's may be the legacy default
    // stream, which cannot be captured; capturing records work, runs none
    if (!b->capture) A4G_CUDA(cudaStreamCreateWithFlags(&b->capture, cudaStreamNonBlocking));
    cudaGraph_t g = nullptr;
    A4G_CUDA(cudaStreamBeginCapture(b->capture, cudaStreamCaptureModeThreadLocal));
    const int rc = run(b, b->capture);
    cudaError_t e = cudaStreamEndCapture(b->capture, &g);
    if (rc) {
      if (g) cudaGraphDestroy(g);
      return rc;
    }
    if (e != cudaSuccess) return cuda_fail(e, "cudaStreamEndCapture");
    e = cudaGraphInstantiate(&b->graph, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) return cuda_fail(e, "cudaGraphInstantiate");
  }
  A4G_CUDA(cudaGraphLaunch(b->graph, s));
  return A4G_OK;
}

int a4g_batch_run_timed(a4g_batch* b, void* stream) {
  if (!b) return fail(A4G_ERR_ARG, "null batch");
  if (int(b->events.size()) <= b->timed_runs) {
    std::vector<cudaEvent_t> ev(6);
    for (auto& e : ev) A4G_CUDA(cudaEventCreate(&e));
    b->events.push_back(ev);
  }
  const int rc = run(b, pick(stream), b->events[b->timed_runs].data());
  if (!rc) ++b->timed_runs;
  return rc;
}

int a4g_batch_timings(a4g_batch* b, float* phase_ms, int nphase, int* runs) {
  if (!b || !phase_ms || nphase < 0) return fail(A4G_ERR_ARG, "bad timing query");
  for (int p = 0; p < nphase; ++p) phase_ms[p] = 0.f;
  if (runs) *runs = b->timed_runs;
  if (b->timed_runs > 0) A4G_CUDA(cudaEventSynchronize(b->events[b->timed_runs - 1][5]));
  for (int r = 0; r < b->timed_runs; ++r)
    for (int p = 0; p < std::min(nphase, 5); ++p) {
      float ms = 0.f;
      A4G_CUDA(cudaEventElapsedTime(&ms, b->events[r][p], b->events[r][p + 1]));
      phase_ms[p] += ms;
    }
  b->timed_runs = 0;
  return A4G_OK;
}

int a4g_batch_info(const a4g_batch* b, int64_t* pairs, double* flops, int64_t* workspace_bytes) {
  if (!b) return fail(A4G_ERR_ARG, "null batch");
  if (pairs) *pairs = b->pairs;
  if (flops) *flops = b->flops;
  if (workspace_bytes) *workspace_bytes = b->device_bytes;
  return A4G_OK;
}

int a4g_batch_launches(const a4g_batch* b, int* kernels_per_run, int* gemm_parts) {
  if (!b) return fail(A4G_ERR_ARG, "null batch");
  int k = b->beta == 0 ? int(b->zero_blocks.size()) : 0;
  int parts = 1;
  if (b->precision == A4G_PREC_FP64) {
    k += b->n_f64_tiles > 0 ? 1 : 0;
    k += b->n_f64_reds > 0 ? 1 : 0;
  } else if (b->forms[b->form].n_tiles > 0) {
    parts = b->parts;
    int sliced = 0;  // job sets of a held side are not run
    for (const auto& js : b->jobsets) sliced += b->held[js.left ? 0 : 1] ? 0 : 1;
    // exponents + splits, GEMM parts, recombine (folded into the GEMM by direct forms)
    k += 2 * sliced + parts + (b->forms[b->form].direct ? 0 : 1);
  }
  if (kernels_per_run) *kernels_per_run = k;
  if (gemm_parts) *gemm_parts = parts;
  return A4G_OK;
}

int a4g_batch_splits(const a4g_batch* b, int* nsplit, int* candidates, float* cost_ms, int n) {
  if (!b) return fail(A4G_ERR_ARG, "null batch");
  if (nsplit) *nsplit = b->precision == A4G_PREC_FP64 ? 0 : b->forms[b->form].nsplit;  // direct forms: 1
  for (int i = 0; i < n; ++i) {
    if (candidates) candidates[i] = i < 2 ? b->split_candidates[i] : 0;
    if (cost_ms) cost_ms[i] = i < 2 ? b->split_cost_ms[i] : -1.f;
  }
  return A4G_OK;
}

int a4g_batch_form(const a4g_batch* b, int* form, float* tuned_ms, int n) {
  if (!b) return fail(A4G_ERR_ARG, "null batch");
  if (form) *form = b->precision == A4G_PREC_FP64 ? 0 : b->form + 1;
  for (int f = 0; f < n && tuned_ms; ++f) tuned_ms[f] = f < a4g_batch::kForms ? b->forms[f].score_ms : -1.f;
  return A4G_OK;
}

int a4g_batch_rebind(a4g_batch* b, const a4g_triple* trip, int64_t n, void* stream) {
  if (!b) return fail(A4G_ERR_ARG, "null batch");
  if (n != int64_t(b->bound.size())) return fail(A4G_ERR_ARG, "rebind: the triple count differs from the batch's");
  if (n > 0 && !trip) return fail(A4G_ERR_ARG, "null argument");
  // old block -> new block, one entry per distinct block whatever its role
  std::unordered_map<const void*, const void*> to;
  auto map_one = [&](const void* o, const void* nw) { return to.emplace(o, nw).first->second == nw; };
  bool moved = false, moved_l = false, moved_r = false;
  for (int64_t i = 0; i < n; ++i) {
    const a4g_triple &o = b->bound[size_t(i)], &t = trip[i];
    if (!t.d) return fail(A4G_ERR_ARG, "rebind: triple with NULL destination");
    if ((o.l == nullptr) != (t.l == nullptr) || (o.r == nullptr) != (t.r == nullptr))
      return fail(A4G_ERR_ARG, "rebind: a zero block (NULL operand) must stay zero and a live block live (triple " +
                                   std::to_string(i) + ")");
    if (std::memcmp(o.dext, t.dext, sizeof(int) * size_t(b->drank)) ||
        std::memcmp(o.lext, t.lext, sizeof(int) * size_t(b->lrank)) ||
        std::memcmp(o.rext, t.rext, sizeof(int) * size_t(b->rrank)))
      return fail(A4G_ERR_ARG, "rebind: block extents differ from the batch's (triple " + std::to_string(i) + ")");
    if (!map_one(o.d, t.d) || (o.l && !map_one(o.l, t.l)) || (o.r && !map_one(o.r, t.r)))
      return fail(A4G_ERR_ARG, "rebind: a block the batch's triples share maps to different new blocks (triple " +
                                   std::to_string(i) + ")");
    moved_l |= o.l != t.l;
    moved_r |= o.r != t.r;
    moved |= o.d != t.d || o.l != t.l || o.r != t.r;
  }
  {  // distinct destination blocks stay distinct (their sums would merge)
    std::unordered_set<const void*> old_d, new_d;
    for (const a4g_triple& o : b->bound)
      if (old_d.insert(o.d).second && !new_d.insert(to[o.d]).second)
        return fail(A4G_ERR_ARG, "rebind: two destination blocks map to one block");
  }
  if (!moved) return A4G_OK;
  if ((b->held[b->swapped ? 1 : 0] && moved_l) || (b->held[b->swapped ? 0 : 1] && moved_r))
    return fail(A4G_ERR_ARG, "rebind: the blocks of a held operand cannot move (release the hold first)");
  auto mp = [&](const void* p) -> const void* {
    if (!p) return p;
    auto it = to.find(p);
    return it == to.end() ? p : it->second;
  };
  cudaStream_t s = pick(stream);
  // every table is rebuilt on the host, checked, then copied in stream order
  // (runs queued before on `stream` still read the old tables)
  size_t total = 0;
  if (b->precision == A4G_PREC_FP64) {
    total = b->h_f64_pairs.size() * sizeof(GroupedPair) + b->h_f64_tiles.size() * sizeof(GroupedF64Tile) +
            b->h_f64_reds.size() * sizeof(GroupedF64Reduce);
  } else {
    for (const auto& js : b->jobsets) total += js.h_jobs.size() * sizeof(OzSplitJob);
    total += b->h_dblocks.size() * sizeof(OzDBlock) + b->h_colptr.size() * sizeof(double*);
  }
  Staging stg;
  int rc = stage_begin(b, total, &stg);
  if (rc) return rc;
  auto put = [&](void* dev, const void* host, size_t bytes) { return stg.add(dev, host, bytes); };
  if (b->precision == A4G_PREC_FP64) {
    std::vector<GroupedPair> pairs = b->h_f64_pairs;
    std::vector<GroupedF64Tile> tiles = b->h_f64_tiles;
    std::vector<GroupedF64Reduce> reds = b->h_f64_reds;
    for (auto& p : pairs)
      p.l = static_cast<const double*>(mp(p.l)), p.r = static_cast<const double*>(mp(p.r));
    for (auto& t : tiles) t.d = const_cast<double*>(static_cast<const double*>(mp(t.d)));
    for (auto& r : reds) r.d = const_cast<double*>(static_cast<const double*>(mp(r.d)));
    if ((rc = put(b->d_f64_pairs, pairs.data(), pairs.size() * sizeof(GroupedPair))) ||
        (rc = put(b->d_f64_tiles, tiles.data(), tiles.size() * sizeof(GroupedF64Tile))) ||
        (rc = put(b->d_f64_reds, reds.data(), reds.size() * sizeof(GroupedF64Reduce))) ||
        (rc = stage_launch(stg, s)))
      return rc;
    b->h_f64_pairs.swap(pairs);
    b->h_f64_tiles.swap(tiles);
    b->h_f64_reds.swap(reds);
  } else {
    std::vector<std::vector<OzSplitJob>> jobs(b->jobsets.size());
    for (size_t i = 0; i < b->jobsets.size(); ++i) {
      jobs[i] = b->jobsets[i].h_jobs;
      for (OzSplitJob& j : jobs[i]) {
        j.src = static_cast<const double*>(mp(j.src));
        if (b->jobsets[i].layout != kOzGeneric && (reinterpret_cast<uintptr_t>(j.src) & 15) != 0)
          return fail(A4G_ERR_ARG, "rebind: an operand block the batch reads with 16-byte loads is not 16-byte aligned");
      }
    }
    std::vector<OzDBlock> dbl = b->h_dblocks;
    for (OzDBlock& d : dbl) d.d = const_cast<double*>(static_cast<const double*>(mp(d.d)));
    std::vector<double*> cols(b->h_colptr.size()), colblk(b->h_colptr.size());
    for (size_t i = 0; i < cols.size(); ++i) {
      double* blk = b->h_colptr_block[i];
      colblk[i] = const_cast<double*>(static_cast<const double*>(mp(blk)));
      cols[i] = colblk[i] + (b->h_colptr[i] - blk);
    }
    for (size_t i = 0; i < b->jobsets.size() && !rc; ++i)
      rc = put(b->jobsets[i].d_jobs, jobs[i].data(), jobs[i].size() * sizeof(OzSplitJob));
    if (rc || (rc = put(b->d_dblocks, dbl.data(), dbl.size() * sizeof(OzDBlock))) ||
        (rc = put(b->d_colptr, cols.data(), cols.size() * sizeof(double*))) || (rc = stage_launch(stg, s)))
      return rc;
    for (size_t i = 0; i < b->jobsets.size(); ++i) b->jobsets[i].h_jobs.swap(jobs[i]);
    for (auto& eg : b->err_groups) eg.d = const_cast<double*>(static_cast<const double*>(mp(eg.d)));
    b->h_dblocks.swap(dbl);
    b->h_colptr.swap(cols);
    b->h_colptr_block.swap(colblk);
  }
  // zero-filled destination blocks are kernel arguments of a captured graph
  bool zero_moved = false;
  for (auto& z : b->zero_blocks) {
    double* nz = const_cast<double*>(static_cast<const double*>(mp(z.first)));
    zero_moved |= nz != z.first;
    z.first = nz;
  }
  if (zero_moved && b->beta == 0 && (rc = drop_graph(b))) return rc;
  b->bound.assign(trip, trip + n);
  return A4G_OK;
}

int a4g_batch_hold(a4g_batch* b, int operand, int hold, void* stream) {
  if (!b) return fail(A4G_ERR_ARG, "null batch");
  if (operand != 0 && operand != 1) return fail(A4G_ERR_ARG, "operand must be 0 (left blocks) or 1 (right blocks)");
  if (b->precision == A4G_PREC_FP64) return A4G_OK;  // nothing is sliced
  const int side = b->swapped ? 1 - operand : operand;
  const bool on = hold != 0;
  int rc = A4G_OK;
  if (on && b->forms[b->form].n_tiles > 0 && (rc = slice_side(b, side, pick(stream)))) return rc;
  if (b->held[side] != on && (rc = drop_graph(b))) return rc;
  b->held[side] = on;
  return A4G_OK;
}

int a4g_batch_error_bound(a4g_batch* b, double target, double* h_bound, void* stream) {
  if (!b || !h_bound) return fail(A4G_ERR_ARG, "null argument");
  *h_bound = 0.0;
  if (b->precision != A4G_PREC_OZAKI_BF16) return fail(A4G_ERR_UNSUPPORTED, "error bound: split-precision batches only");
  if (b->beta) return fail(A4G_ERR_UNSUPPORTED, "error bound: the product alone is in D only with beta = 0");
  cudaStream_t s = pick(stream);
  const int S = b->slices;
  // exponents of the last run, and the squared norm of every destination block
  std::vector<int> ex(b->exps_bytes / sizeof(int));
  const size_t ng = b->err_groups.size();
  double* dev = nullptr;
  const int64_t scratch = dot_scratch_len();
  if (const int rc_ = async_alloc(reinterpret_cast<void**>(&dev), (ng + size_t(scratch)) * sizeof(double), s)) return rc_;
  int rc = A4G_OK;
  for (size_t i = 0; i < ng && !rc; ++i) {
    const a4g_batch::ErrGroup& eg = b->err_groups[i];
    rc = launch_dot(eg.d, eg.d, nullptr, nullptr, eg.size, dev + scratch + i, dev, scratch, s);
  }
  std::vector<double> nrm2(ng);
  if (!rc && ng) {
    A4G_CUDA(cudaMemcpyAsync(nrm2.data(), dev + scratch, ng * sizeof(double), cudaMemcpyDeviceToHost, s));
  }
  if (!rc) A4G_CUDA(cudaMemcpyAsync(ex.data(), b->d_exps, b->exps_bytes, cudaMemcpyDeviceToHost, s));
  cudaFreeAsync(dev, s);
  if (rc) return rc;
  A4G_CUDA(cudaStreamSynchronize(s));
  // |x| < 2^E for the stored biased exponent field f: E = f - 1022.  Per
  // k, the digits carry each operand to within 2^(E - 8S) and the dropped
  // levels t >= S add at most (S - 1) 2^(E + F - 8S) (1 + 2^-8 + ...), so
  //   |D - LR|_mn <= c_S K 2^(E_m + F_n - 8S),  c_S = 1.004 (S - 1) + 2.001,
  // and over a block ||D - LR||_F <= c_S K 2^-8S sqrt(sum_m 4^E_m sum_n 4^F_n)
  // + 2^-53 ||D||_F (the final rounding); relative to ||LR||_F >= ||D||_F -
  // that.  Sums in log2 to keep every exponent in range.
  const double cS = 1.004 * (S - 1) + 2.001;
  auto log2_sum4 = [&](size_t off, int64_t n, bool* nonfinite) {
    int mx = 0;
    for (int64_t i = 0; i < n; ++i) {
      const int f = ex[off + size_t(i)];
      if (f == 2047) *nonfinite = true;
      mx = std::max(mx, f);
    }
    if (mx == 0) return -std::numeric_limits<double>::infinity();
    double acc = 0.0;
    for (int64_t i = 0; i < n; ++i) {
      const int f = ex[off + size_t(i)];
      if (f) acc += std::ldexp(1.0, 2 * (f - mx));
    }
    return 2.0 * (mx - 1022) + std::log2(acc);
  };
  double worst = 0.0;
  for (size_t i = 0; i < ng; ++i) {
    const a4g_batch::ErrGroup& eg = b->err_groups[i];
    bool nonfinite = false;
    const double lr = log2_sum4(eg.exp_rows, eg.rows, &nonfinite), lc = log2_sum4(eg.exp_cols, eg.cols, &nonfinite);
    const double dn = std::sqrt(nrm2[i]);
    double rel;
    if (nonfinite || !std::isfinite(dn)) {
      rel = std::numeric_limits<double>::infinity();
    } else if (std::isinf(lr) || std::isinf(lc)) {
      rel = 0.0;  // an all-zero operand side: the product is exactly zero
    } else {
      const double beta = std::exp2(std::log2(cS * eg.K) - 8.0 * S + 0.5 * (lr + lc)) + 0x1p-53 * dn;
      rel = dn > beta ? beta / (dn - beta) : std::numeric_limits<double>::infinity();
    }
    worst = std::max(worst, rel);
  }
  *h_bound = worst;
  if (target > 0.0 && !(worst <= target))
    return fail(A4G_ERR_PRECISION, "certified relative error bound " + std::to_string(worst) + " exceeds the target " +
                                       std::to_string(target) + " at " + std::to_string(S) + " slices");
  return A4G_OK;
}

int a4g_batch_tuning(const a4g_batch* b, int* from_cache, float* autotune_ms) {
  if (!b) return fail(A4G_ERR_ARG, "null batch");
  if (from_cache) *from_cache = b->tuned_from_cache ? 1 : 0;
  if (autotune_ms) *autotune_ms = b->autotune_ms;
  return A4G_OK;
}

void a4g_tune_cache_clear(void) {
  std::lock_guard<std::mutex> lock(g_tune_mu);
  g_tune.clear();
}

int a4g_tune_cache_save(const char* path) {
  if (!path) return fail(A4G_ERR_ARG, "null path");
  std::FILE* f = std::fopen(path, "w");
  if (!f) return fail(A4G_ERR_ARG, std::string("cannot write ") + path);
  std::lock_guard<std::mutex> lock(g_tune_mu);
  std::fprintf(f, "a4g-tune 1\n");
  for (const auto& kv : g_tune) {
    const TuneRecord& r = kv.second;
    std::fprintf(f, "%016llx %d %d %d %d %.6g %.6g", static_cast<unsigned long long>(kv.first), r.form, r.nsplit,
                 r.split_candidates[0], r.split_candidates[1], r.split_cost_ms[0], r.split_cost_ms[1]);
    for (int i = 0; i < a4g_batch::kForms; ++i) std::fprintf(f, " %.6g", r.score_ms[i]);
    std::fprintf(f, "\n");
  }
  const bool ok = std::fclose(f) == 0;
  return ok ? A4G_OK : fail(A4G_ERR_ARG, std::string("cannot write ") + path);
}

int a4g_tune_cache_load(const char* path) {
  if (!path) return fail(A4G_ERR_ARG, "null path");
  std::FILE* f = std::fopen(path, "r");
  if (!f) return fail(A4G_ERR_ARG, std::string("cannot read ") + path);
  int version = 0;
  if (std::fscanf(f, "a4g-tune %d", &version) != 1 || version != 1) {
    std::fclose(f);
    return fail(A4G_ERR_ARG, std::string(path) + " is not a tuning cache of this library");
  }
  std::vector<std::pair<uint64_t, TuneRecord>> recs;
  for (;;) {
    unsigned long long key = 0;
    TuneRecord r;
    if (std::fscanf(f, "%llx %d %d %d %d %g %g", &key, &r.form, &r.nsplit, &r.split_candidates[0],
                    &r.split_candidates[1], &r.split_cost_ms[0], &r.split_cost_ms[1]) != 7)
      break;
    bool ok = true;
    for (int i = 0; i < a4g_batch::kForms && ok; ++i) ok = std::fscanf(f, "%g", &r.score_ms[i]) == 1;
    if (!ok || r.form < 0 || r.form >= a4g_batch::kForms || r.nsplit < 1) break;
    recs.push_back({uint64_t(key), r});
  }
  const bool eof = std::feof(f) != 0;
  std::fclose(f);
  if (!eof) return fail(A4G_ERR_ARG, std::string("malformed record in ") + path);
  for (const auto& kv : recs) tune_put(kv.first, kv.second);
  return A4G_OK;
}

void a4g_batch_destroy(a4g_batch* b) { delete b; }

}  // extern "C"
