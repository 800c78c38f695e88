// Fused multi-term pardo step (a4g_fused_*): up to two contraction statements
// into the same destination blocks, summed exactly before one rounding, in
// one pass of the split-precision (Ozaki) tensor-core GEMM; optionally the
// orbital-energy reduction of the result instead of storing it.
//
// The reference's (T) pattern (rccsdpt_aaa.sialx:2163-2172) runs, per pardo
// iteration, two contraction statements into W (interpreter.cpp:1210-1262
// for each, the second one through a temporary and handle_block_subtract,
// interpreter.cpp:1935-1997), divides a copy of W by the orbital-energy
// denominators (energy_denominator_rhf.F:399-436) and contracts it with W to
// a scalar (block_contract_to_scalar_op, interpreter.cpp:748).  Here the
// whole sequence is one GEMM pass over the step: W exists only as exact
// integer level sums in TMEM, one tile at a time.
//
// Decomposition.  Every destination index comes from the left or the right
// operand of each term.  Indices that are left in both terms are the GEMM's
// rows, right in both its columns; an index that is left in term 1 and right
// in term 2 (B1), or right in term 1 and left in term 2 (B2), is fixed per
// sub-problem.  For the triples W(a,i,b,j,c,k) = V1(b,c,d,k) T(a,d,i,j) -
// V2(l,c,j,k) T(a,b,i,l): rows (c,k), columns (a,i), B1 = {b}, B2 = {j}; each
// (b, j) is a 576 x 576 product whose k runs over d (term 1) then l (term 2).
//
// Panels.  One A panel per destination block: its rows are the row space,
// its k columns a stretch per B1 value holding the term-1 left blocks at that
// value, then a stretch per B2 value holding the term-2 left blocks.  One B
// panel per distinct set of right blocks (shared by destination blocks that
// read the same ones): a stretch per B2 value (term 1), then per B1 value
// (term 2).  A sub-problem (b, j) multiplies A stretch (1, b) by B stretch
// (1, j), then A (2, j) by B (2, b): two trips of the direct-form GEMM into one
// exact 64-bit level sum.  A panel row's (column's) scale is the maximum over
// the whole panel row, so both terms share the scales and their integer sums
// add exactly; a subtracted term's left digits are sliced from -x.
#include <algorithm>
#include <cstring>
#include <map>
#include <memory>
#include <vector>

#include "a4g_internal.h"
#include "grouped.h"
#include "ozaki.h"

using namespace a4g;

// Kernel parameters of one denominator prefix table: entry (b, j, r, c) at
// at + ((b * nb2 + j) * rkn + r) * ckn + c holds the chain without its last
// term; term q reads dimension coordinate (index of its group / stride) % ext
// of the group (0: r, 1: c, 2: b, 3: j) at orbital off + coordinate.
struct PtabTerm {
  int group, stride, ext, off, sign;
};
struct PtabTable {
  int64_t at, n;
  int rkn, ckn, nb1, nb2;
  int nterms;
  PtabTerm t[5];
};

struct a4g_fused {
  int slices = 5;
  int variant = 0;      // as created: 0 automatic, 5 one level at a time, 7 all levels at once
  bool levels = false;  // the all-levels GEMM form runs
  int drank = 0, lrank = 0, rrank = 0;
  int nterms = 0;
  int beta = 0;
  bool energy = false;
  double efact = 1.0;
  uint64_t signature = 0;  // structure of the creation's inputs (a rebind must match it)
  std::vector<void*> allocs;
  int64_t device_bytes = 0;
  int64_t pairs = 0, elements = 0;
  double flops = 0.0;
  int* d_exps = nullptr;
  size_t exps_bytes = 0;
  OzPanel* d_panels = nullptr;  // A panels, then B panels (split jobs index the whole array)
  OzSplitJob* d_jobs = nullptr;
  int64_t* d_prefix_exp = nullptr;
  int64_t* d_prefix_split = nullptr;
  int njobs = 0;
  int64_t tiles_exp = 0, tiles_split = 0;
  int64_t* d_offs = nullptr;        // split-job address tables
  std::vector<OzSplitJob> h_jobs;   // with offRow/offK as device pointers
  double** d_colptr = nullptr;      // store form: column bases of every sub-block
  size_t n_colptr = 0;
  // energy form
  const double* e_dev = nullptr;
  int rank1 = 1, ld1 = 0;
  double* d_elast = nullptr;
  size_t n_elast = 0;
  double* d_ptab = nullptr;
  PtabTable* d_ptabs = nullptr;
  int n_ptabs = 0;
  int64_t max_ptab_n = 0;
  OzGemmArgs args{};
  int grid = 0;
  double* d_epart = nullptr;
  int epart_len = 0;
  std::vector<std::pair<double*, int64_t>> zero_blocks;  // store mode, beta 0: blocks no pair feeds
  ~a4g_fused() {
    for (void* p : allocs) cudaFree(p);
  }
};

namespace {

int64_t ceil_to(int64_t x, int64_t m) { return (x + m - 1) / m * m; }

struct alignas(64) MapImage {  // host image of one CUtensorMap (128 bytes, 64-byte aligned)
  uint8_t b[128];
};

int falloc(a4g_fused* f, size_t bytes, void** out) {
  void* p = nullptr;
  A4G_CUDA(cudaMalloc(&p, std::max<size_t>(bytes, 256)));
  f->allocs.push_back(p);
  f->device_bytes += int64_t(bytes);
  *out = p;
  return A4G_OK;
}

template <class T>
int fupload(a4g_fused* f, const std::vector<T>& v, T** out) {
  *out = nullptr;
  if (v.empty()) return A4G_OK;
  void* p = nullptr;
  const int rc = falloc(f, v.size() * sizeof(T), &p);
  if (rc) return rc;
  A4G_CUDA(cudaMemcpy(p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice));
  *out = static_cast<T*>(p);
  return A4G_OK;
}

// Offsets sum_d coord_d * stride_d over a mixed-radix enumeration (first
// index fastest) of the extents.
std::vector<int64_t> enum_offsets(const std::vector<int>& ext, const std::vector<int64_t>& stride) {
  int64_t n = 1;
  for (int e : ext) n *= e;
  std::vector<int64_t> out(size_t(std::max<int64_t>(n, 0)));
  std::vector<int> c(ext.size(), 0);
  int64_t off = 0;
  for (int64_t i = 0; i < n; ++i) {
    out[size_t(i)] = off;
    for (size_t q = 0; q < ext.size(); ++q) {  // next coordinate with carries
      off += stride[q];
      if (++c[q] < ext[q]) break;
      off -= stride[q] * ext[q];
      c[q] = 0;
    }
  }
  return out;
}

// Coordinates (first fastest) of index i over the extents.
void coords_of(int64_t i, const std::vector<int>& ext, int* c) {
  for (size_t q = 0; q < ext.size(); ++q) {
    c[q] = int(i % ext[q]);
    i /= ext[q];
  }
}

enum Cat { kRow = 0, kCol = 1, kB1 = 2, kB2 = 3 };

struct Term {
  const int* ptrn = nullptr;
  int sign = 1;
  std::vector<int> dL, dR;                  // per destination dim: the left / right dim it comes from, or -1
  std::vector<std::pair<int, int>> con;     // contracted (left dim, right dim), in left order
};

struct FPair {
  const double* l;
  const double* r;
  const int* lext;
  const int* rext;
};

struct WBlock {
  double* d = nullptr;
  const int* dext = nullptr;
  std::vector<FPair> pairs[2];
};

// Device tables deduplicated by content (offsets, row keys ...), packed into
// one allocation per element type.
template <class T>
struct TablePool {
  std::map<std::vector<T>, size_t> index;
  std::vector<T> data;
  size_t add(const std::vector<T>& v) {
    auto it = index.find(v);
    if (it != index.end()) return it->second;
    const size_t at = data.size();
    data.insert(data.end(), v.begin(), v.end());
    index.emplace(v, at);
    return at;
  }
};

// Host copy of the orbital energies a denominator reads (e or the diagonal
// of the Fock block).
struct Energies {
  int rank1 = 1, ld1 = 0;
  std::vector<double> h;
  double at(int orb) const { return rank1 == 2 ? h[size_t(orb) + size_t(orb) * size_t(ld1)] : h[size_t(orb)]; }
};

// 64-bit FNV-1a over the inputs that decide a fused step's device structure.
struct Fnv64 {
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

// The denominator prefix tables, one thread per entry: the chain's terms in
// the reference's order (the first assigned, then added or subtracted), FP64
// round-to-nearest like the host and the reference.
__global__ void __launch_bounds__(256) ptab_kernel(const PtabTable* __restrict__ tabs, const double* __restrict__ e,
                                                   int rank1, int ld1, double* __restrict__ ptab) {
  const PtabTable T = tabs[blockIdx.y];
  for (int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < T.n; i += int64_t(gridDim.x) * blockDim.x) {
    int64_t q = i;
    const int64_t c = q % T.ckn;
    q /= T.ckn;
    const int64_t r = q % T.rkn;
    q /= T.rkn;
    const int64_t j = q % T.nb2, b = q / T.nb2;
    double v = 0.0;
    for (int k = 0; k < T.nterms; ++k) {
      const PtabTerm t = T.t[k];
      const int64_t g = t.group == 0 ? r : t.group == 1 ? c : t.group == 2 ? b : j;
      const int64_t orb = t.off + (g / t.stride) % t.ext;
      const double ev = rank1 == 2 ? e[orb + orb * ld1] : e[orb];
      v = k == 0 ? ev : (t.sign > 0 ? __dadd_rn(v, ev) : __dsub_rn(v, ev));
    }
    ptab[T.at + i] = v;
  }
}

}  // namespace

namespace {

// Host side of a planned fused step.  Device pointers that do not exist yet
// are held as offsets (cast to pointers) and relocated at creation.
struct Plan {
  uint64_t sig = 0;
  bool levels = false;  // the all-levels GEMM form (128 x 64 tiles), else one level at a time (128 x 128)
  double flops = 0.0;
  int64_t pairs = 0, elements = 0;
  std::vector<OzPanel> panels;  // A panels then B panels; exps as an int offset
  int nA = 0;
  std::vector<int64_t> offs;
  std::vector<OzSplitJob> jobs;  // offRow / offK as offsets into offs
  std::vector<int64_t> rowoffs;
  std::vector<OzDBlock> dblocks;  // rowoff / colptr as offsets
  std::vector<double*> colptr;
  std::vector<OzTile> tiles;
  std::vector<OzTrip> trips;
  std::vector<std::pair<double*, int64_t>> zero_blocks;
  bool energy = false;
  double efact = 1.0;
  const double* e_dev = nullptr;
  int rank1 = 1, ld1 = 0;
  std::vector<int> ikeys;
  std::vector<double> elast;
  std::vector<PtabTable> ptabs;
  int64_t ptab_n = 0;
  std::vector<OzEnergyBlock> eblocks;  // ptab / rk / ck / elast as offsets
};

template <class P>
P* as_offset(size_t off) {
  return reinterpret_cast<P*>(off);
}
size_t offset_of(const void* p) { return reinterpret_cast<size_t>(p); }

int plan_fused(int drank, int lrank, int rrank, const a4g_term* terms, int nterms, const a4g_fused_energy* energy,
               int S, int beta, int variant, Plan* out) {
  Plan& P = *out;
  if (!terms || nterms < 1 || nterms > 2) return fail(A4G_ERR_ARG, "fused step: one or two terms");
  if (drank < 1 || drank > kMaxRank || lrank < 1 || lrank > kMaxRank || rrank < 1 || rrank > kMaxRank)
    return fail(A4G_ERR_ARG, "fused step: ranks out of range (tensor-tensor contractions only)");
  Fnv64 sig;
  sig.put(uint32_t(0x46555344));  // format tag
  if (variant != 0 && variant != 5 && variant != 7) return fail(A4G_ERR_ARG, "fused step: variant 0, 5 or 7");
  sig.put(S), sig.put(beta), sig.put(variant), sig.put(nterms), sig.put(drank), sig.put(lrank), sig.put(rrank);
  sig.put(int(energy != nullptr));

  // ---- the terms' index maps
  std::vector<Term> T(static_cast<size_t>(nterms));
  for (int t = 0; t < nterms; ++t) {
    const a4g_term& tm = terms[t];
    if (!tm.contr_ptrn || (tm.n_triples > 0 && !tm.triples) || tm.n_triples < 0)
      return fail(A4G_ERR_ARG, "fused step: null term");
    if (tm.sign != 1 && tm.sign != -1) return fail(A4G_ERR_ARG, "fused step: term sign must be +1 or -1");
    sig.add(tm.contr_ptrn, sizeof(int) * size_t(lrank + rrank));
    sig.put(tm.sign), sig.put(tm.n_triples);
    Term& x = T[size_t(t)];
    x.ptrn = tm.contr_ptrn, x.sign = tm.sign;
    x.dL.assign(size_t(drank), -1), x.dR.assign(size_t(drank), -1);
    for (int i = 0; i < lrank; ++i) {
      const int p = tm.contr_ptrn[i];
      if (p > 0 && p <= drank) {
        if (x.dL[size_t(p - 1)] >= 0 || x.dR[size_t(p - 1)] >= 0) return fail(A4G_ERR_PATTERN, "fused step: bad pattern");
        x.dL[size_t(p - 1)] = i;
      } else if (p < 0 && -p <= rrank) {
        x.con.push_back({i, -p - 1});
      } else {
        return fail(A4G_ERR_PATTERN, "fused step: bad pattern");
      }
    }
    for (int j = 0; j < rrank; ++j) {
      const int p = tm.contr_ptrn[lrank + j];
      if (p > 0 && p <= drank) {
        if (x.dL[size_t(p - 1)] >= 0 || x.dR[size_t(p - 1)] >= 0) return fail(A4G_ERR_PATTERN, "fused step: bad pattern");
        x.dR[size_t(p - 1)] = j;
      } else if (!(p < 0 && -p <= lrank)) {
        return fail(A4G_ERR_PATTERN, "fused step: bad pattern");
      }
    }
    for (int d = 0; d < drank; ++d)
      if (x.dL[size_t(d)] < 0 && x.dR[size_t(d)] < 0) return fail(A4G_ERR_PATTERN, "fused step: bad pattern");
    if (x.con.empty()) return fail(A4G_ERR_UNSUPPORTED, "fused step: a term without contracted indices");
  }
  std::vector<int> cat(static_cast<size_t>(drank));
  std::vector<int> dims[4];  // destination dims per category, in destination order
  for (int d = 0; d < drank; ++d) {
    const bool l0 = T[0].dL[size_t(d)] >= 0;
    const bool l1 = nterms == 2 ? T[1].dL[size_t(d)] >= 0 : l0;
    cat[size_t(d)] = l0 ? (l1 ? kRow : kB1) : (l1 ? kB2 : kCol);
    dims[cat[size_t(d)]].push_back(d);
  }
  if (dims[kRow].empty() || dims[kCol].empty())
    return fail(A4G_ERR_UNSUPPORTED, "fused step: the terms share no row or no column index");

  // ---- destination blocks and their pairs (zero blocks skipped)
  std::vector<WBlock> wb;
  std::map<double*, size_t> widx;
  for (int t = 0; t < nterms; ++t) {
    const a4g_term& tm = terms[t];
    for (int64_t q = 0; q < tm.n_triples; ++q) {
      const a4g_triple& x = tm.triples[q];
      if (!x.d) return fail(A4G_ERR_ARG, "fused step: null destination block");
      if (!contr_ptrn_ok(tm.contr_ptrn, lrank, rrank, drank, x.lext, x.rext, x.dext))
        return fail(A4G_ERR_PATTERN, "contraction pattern rejected (contr_ptrn_ok)");
      for (int i = 0; i < drank; ++i)
        if (x.dext[i] <= 0) return fail(A4G_ERR_ARG, "non-positive extent");
      auto it = widx.find(x.d);
      if (it == widx.end()) {
        it = widx.emplace(x.d, wb.size()).first;
        WBlock w;
        w.d = x.d, w.dext = x.dext;
        wb.push_back(w);
      }
      WBlock& w = wb[it->second];
      if (!std::equal(x.dext, x.dext + drank, w.dext))
        return fail(A4G_ERR_ARG, "fused step: one destination block with two shapes");
      sig.put(int64_t(it->second)), sig.put(int(x.l != nullptr && x.r != nullptr));
      sig.add(x.lext, sizeof(int) * size_t(lrank)), sig.add(x.rext, sizeof(int) * size_t(rrank));
      if (x.l && x.r) w.pairs[t].push_back({x.l, x.r, x.lext, x.rext});
    }
  }
  for (const WBlock& w : wb) sig.add(w.dext, sizeof(int) * size_t(drank));

  // ---- energy inputs
  Energies en;
  int pos[6] = {0, 1, 2, 3, 4, 5};
  std::vector<std::vector<int>> wb_off(wb.size());  // orbital offset per destination dim
  int dl = -1;                                      // destination dim of the chain's last term
  std::vector<std::pair<int, int>> chain;           // prefix: (destination dim, +1 / -1), the first assigned
  P.energy = energy != nullptr;
  if (energy) {
    if (!(drank == 2 || drank == 4 || drank == 6)) return fail(A4G_ERR_UNSUPPORTED, "fused energy: rank 2, 4 or 6");
    if (!(energy->rank1 == 1 || energy->rank1 == 2) || (drank == 6 && energy->rank1 != 2))
      return fail(A4G_ERR_UNSUPPORTED, "fused energy: unsupported rank combination");
    if (!energy->blocks || !energy->index_values || !energy->ext1 || !energy->e_or_fock ||
        (energy->nsegs > 0 && !energy->seg_sizes))
      return fail(A4G_ERR_ARG, "fused energy: null argument");
    bool seen[6] = {false, false, false, false, false, false};
    for (int q = 0; q < drank; ++q) {
      pos[q] = energy->den_order ? energy->den_order[q] : q;
      if (pos[q] < 0 || pos[q] >= drank || seen[pos[q]])
        return fail(A4G_ERR_ARG, "fused energy: den_order is not a permutation");
      seen[pos[q]] = true;
    }
    sig.add(pos, sizeof(pos));
    // energy_denominator_rhf.F do_rhf_den2/4/6: the occupied positions 1, 3, 5
    // added left to right, then the virtual positions 0, 2, 4 subtracted
    if (drank == 2) chain = {{pos[1], 1}};
    if (drank == 4) chain = {{pos[1], 1}, {pos[3], 1}, {pos[0], -1}};
    if (drank == 6) chain = {{pos[1], 1}, {pos[3], 1}, {pos[5], 1}, {pos[0], -1}, {pos[2], -1}};
    dl = pos[drank - 2];
    if (cat[size_t(dl)] != kRow && cat[size_t(dl)] != kCol)
      return fail(A4G_ERR_UNSUPPORTED, "fused energy: the denominator's last term is a fixed (batch) index");
    en.rank1 = energy->rank1, en.ld1 = energy->ext1[0];
    const int64_t ne = energy->rank1 == 2 ? int64_t(energy->ext1[0]) * energy->ext1[1] : energy->ext1[0];
    if (ne <= 0) return fail(A4G_ERR_ARG, "fused energy: empty energy array");
    sig.put(energy->rank1), sig.put(energy->ext1[0]), sig.put(energy->rank1 == 2 ? energy->ext1[1] : 0);
    en.h.resize(size_t(ne));
    A4G_CUDA(cudaMemcpy(en.h.data(), energy->e_or_fock, size_t(ne) * sizeof(double), cudaMemcpyDeviceToHost));
    const std::vector<int> segs(energy->seg_sizes, energy->seg_sizes + std::max(energy->nsegs, 0));
    for (int64_t i = 0; i < energy->n_blocks; ++i) {
      auto it = widx.find(energy->blocks[i]);
      if (it == widx.end()) continue;  // a block no term writes: zero, adds nothing
      std::vector<int> off(static_cast<size_t>(drank));
      const int rc = denominator_offsets(drank, energy->index_values + i * drank, wb[it->second].dext, energy->rank1,
                                         energy->ext1, segs, off.data());
      if (rc) return rc;
      wb_off[it->second] = off;
    }
    for (size_t w = 0; w < wb.size(); ++w)
      if (wb_off[w].empty()) return fail(A4G_ERR_ARG, "fused energy: a destination block without index values");
    P.efact = energy->efact;
    P.e_dev = energy->e_or_fock;
    P.rank1 = en.rank1, P.ld1 = en.ld1;
  }

  // ---- panels, split jobs, sub-problems, tiles
  std::vector<OzPanel> pa, pb;
  std::map<std::vector<int64_t>, int> pb_index;
  TablePool<int64_t> offs, rowoffs;
  std::vector<OzSplitJob> jobs_a, jobs_b;
  struct SubH {
    size_t w;
    int b, j;
    int trip_begin, trip_end, kb_total;
  };
  std::vector<SubH> subs;
  struct WInfo {
    int M = 0, N = 0, NB1 = 1, NB2 = 1;
    int64_t S1 = 0, S2 = 0;      // stretch lengths (64-aligned)
    std::vector<int64_t> pk[2];  // k offset of each pair inside its stretch
    int pa = -1, pb = -1;
    size_t rowoff_at = 0;
  };
  std::vector<WInfo> wi(wb.size());
  auto new_panel = [](int rows, int64_t kpad) {
    OzPanel o{};
    o.rows = rows;
    o.rows_pad = int(ceil_to(rows, kOzBM));
    o.kpad = kpad;
    return o;
  };
  for (size_t w = 0; w < wb.size(); ++w) {
    const WBlock& W = wb[w];
    WInfo& I = wi[w];
    std::vector<int64_t> ds(static_cast<size_t>(drank));
    int64_t s = 1;
    for (int d = 0; d < drank; ++d) ds[size_t(d)] = s, s *= W.dext[d];
    auto ext_of = [&](int c) {
      std::vector<int> e;
      for (int d : dims[c]) e.push_back(W.dext[d]);
      return e;
    };
    int64_t M = 1, N = 1, NB1 = 1, NB2 = 1;
    for (int d : dims[kRow]) M *= W.dext[d];
    for (int d : dims[kCol]) N *= W.dext[d];
    for (int d : dims[kB1]) NB1 *= W.dext[d];
    for (int d : dims[kB2]) NB2 *= W.dext[d];
    if (M > (1 << 30) || N > (1 << 30) || NB1 * NB2 > (1 << 30))
      return fail(A4G_ERR_RANGE, "fused step: destination block too large");
    I.M = int(M), I.N = int(N), I.NB1 = int(NB1), I.NB2 = int(NB2);
    if (W.pairs[0].empty() && (nterms < 2 || W.pairs[1].empty())) {
      if (!P.energy && beta == 0) P.zero_blocks.push_back({W.d, s});
      continue;
    }
    for (int t = 0; t < nterms; ++t) {
      int64_t k = 0;
      for (const FPair& p : W.pairs[t]) {
        int64_t K = 1;
        for (auto& c : T[size_t(t)].con) K *= p.lext[c.first];
        I.pk[t].push_back(k);
        k += ceil_to(K, 8);  // 8 columns: the split kernels' vector stores stay aligned
        P.flops += 2.0 * double(M) * double(N) * double(NB1 * NB2) * double(K);
        ++P.pairs;
      }
      (t == 0 ? I.S1 : I.S2) = ceil_to(k, kOzBK);
    }
    P.elements += M * N * NB1 * NB2;
    // A panel: per B1 value a term-1 stretch, then per B2 value a term-2 stretch
    I.pa = int(pa.size());
    pa.push_back(new_panel(int(M), NB1 * I.S1 + NB2 * I.S2));
    // B panel: per B2 value a term-1 stretch, then per B1 value a term-2 stretch (shared when identical)
    std::vector<int64_t> key = {N, NB1, NB2, I.S1, I.S2};
    for (int t = 0; t < nterms; ++t) {
      key.push_back(-1);
      for (const FPair& p : W.pairs[t]) {
        key.push_back(int64_t(reinterpret_cast<uintptr_t>(p.r)));
        for (int j = 0; j < rrank; ++j) key.push_back(p.rext[j]);
      }
    }
    auto bit = pb_index.find(key);
    const bool new_b = bit == pb_index.end();
    if (new_b) {
      bit = pb_index.emplace(key, int(pb.size())).first;
      pb.push_back(new_panel(int(N), NB2 * I.S1 + NB1 * I.S2));
    }
    I.pb = bit->second;
    sig.put(I.pb);
    // split jobs
    for (int t = 0; t < nterms; ++t) {
      const Term& tm = T[size_t(t)];
      // left operand: rows = row dims, fixed = B1 (term 1) / B2 (term 2); right: rows = column dims, fixed = B2 / B1
      const int fixL = t == 0 ? kB1 : kB2, fixR = t == 0 ? kB2 : kB1;
      const int64_t nfixL = t == 0 ? NB1 : NB2, nfixR = t == 0 ? NB2 : NB1;
      const int64_t baseA = t == 0 ? 0 : NB1 * I.S1, strideA = t == 0 ? I.S1 : I.S2;
      const int64_t baseB = t == 0 ? 0 : NB2 * I.S1, strideB = t == 0 ? I.S1 : I.S2;
      for (size_t pi = 0; pi < W.pairs[t].size(); ++pi) {
        const FPair& p = W.pairs[t][pi];
        std::vector<int64_t> ls(static_cast<size_t>(lrank)), rs(static_cast<size_t>(rrank));
        int64_t q = 1;
        for (int i = 0; i < lrank; ++i) ls[size_t(i)] = q, q *= p.lext[i];
        q = 1;
        for (int j = 0; j < rrank; ++j) rs[size_t(j)] = q, q *= p.rext[j];
        auto strides = [&](int c, bool left) {
          std::vector<int64_t> st;
          for (int d : dims[c]) st.push_back(left ? ls[size_t(tm.dL[size_t(d)])] : rs[size_t(tm.dR[size_t(d)])]);
          return st;
        };
        std::vector<int> kext;
        std::vector<int64_t> kl, kr;
        for (auto& c : tm.con)
          kext.push_back(p.lext[c.first]), kl.push_back(ls[size_t(c.first)]), kr.push_back(rs[size_t(c.second)]);
        const std::vector<int64_t> okl = enum_offsets(kext, kl), okr = enum_offsets(kext, kr);
        const std::vector<int64_t> orl = enum_offsets(ext_of(kRow), strides(kRow, true));
        const std::vector<int64_t> fl = enum_offsets(ext_of(fixL), strides(fixL, true));
        const size_t rl_at = offs.add(orl), kl_at = offs.add(okl);
        const int K = int(okl.size());
        for (int64_t v = 0; v < nfixL; ++v) {
          OzSplitJob j{};
          j.src = p.l + fl[size_t(v)];
          j.offRow = as_offset<const int64_t>(rl_at), j.offK = as_offset<const int64_t>(kl_at);
          j.rows = int(M), j.K = K;
          j.kfast = K > 1 && okl[1] == 1;
          j.panel = I.pa;
          j.koff = baseA + v * strideA + I.pk[t][pi];
          j.negate = tm.sign < 0;
          jobs_a.push_back(j);
        }
        if (new_b) {
          const std::vector<int64_t> orr = enum_offsets(ext_of(kCol), strides(kCol, false));
          const std::vector<int64_t> fr = enum_offsets(ext_of(fixR), strides(fixR, false));
          const size_t rr_at = offs.add(orr), kr_at = offs.add(okr);
          for (int64_t v = 0; v < nfixR; ++v) {
            OzSplitJob j{};
            j.src = p.r + fr[size_t(v)];
            j.offRow = as_offset<const int64_t>(rr_at), j.offK = as_offset<const int64_t>(kr_at);
            j.rows = int(N), j.K = K;
            j.kfast = K > 1 && okr[1] == 1;
            j.panel = I.pb;  // shifted past the A panels below
            j.koff = baseB + v * strideB + I.pk[t][pi];
            jobs_b.push_back(j);
          }
        }
      }
    }
    // destination offsets of the row space (store mode)
    std::vector<int64_t> dsr;
    for (int d : dims[kRow]) dsr.push_back(ds[size_t(d)]);
    I.rowoff_at = rowoffs.add(enum_offsets(ext_of(kRow), dsr));
    // sub-problems (b, j) and their tiles: trip 1 = A stretch (1, b) x B
    // stretch (1, j), trip 2 = A stretch (2, j) x B stretch (2, b)
    for (int64_t b = 0; b < NB1; ++b)
      for (int64_t j = 0; j < NB2; ++j) {
        const int trip_begin = int(P.trips.size());
        int kb_total = 0;
        if (!W.pairs[0].empty()) {
          OzTrip tr{};
          tr.koff_a = b * I.S1, tr.koff_b = j * I.S1, tr.nkb = int(I.S1 / kOzBK);
          P.trips.push_back(tr);
          kb_total += tr.nkb;
        }
        if (nterms == 2 && !W.pairs[1].empty()) {
          OzTrip tr{};
          tr.koff_a = NB1 * I.S1 + j * I.S2, tr.koff_b = NB2 * I.S1 + b * I.S2, tr.nkb = int(I.S2 / kOzBK);
          P.trips.push_back(tr);
          kb_total += tr.nkb;
        }
        subs.push_back({w, int(b), int(j), trip_begin, int(P.trips.size()), kb_total});
      }
  }
  // ---- the GEMM form, then the tiles of every sub-problem (n fastest)
  bool fit = true;
  for (const SubH& sb : subs) fit = fit && oz_levels_fit(S, sb.kb_total);
  if (variant == 7 && !fit)
    return fail(A4G_ERR_UNSUPPORTED, "fused step: the all-levels form needs at most 5 slices and k <= 320");
  P.levels = variant == 7 || (variant == 0 && fit);
  const int tile_n = P.levels ? kOzLevelsTileCols : kOzBN;
  for (size_t q = 0; q < subs.size(); ++q) {
    const SubH& sb = subs[q];
    const WInfo& I = wi[sb.w];
    for (int64_t m0 = 0; m0 < I.M; m0 += kOzBM)
      for (int64_t n0 = 0; n0 < I.N; n0 += tile_n) {
        OzTile tl{};
        tl.dblock = int(q), tl.m0 = int(m0), tl.n0 = int(n0);
        tl.panel_a = I.pa, tl.panel_b = I.pb;
        tl.trip_begin = sb.trip_begin, tl.trip_end = sb.trip_end;
        tl.kb_total = sb.kb_total;
        P.tiles.push_back(tl);
      }
  }
  if (P.tiles.size() > size_t(0x7fffffff / kOzMaxSlices)) return fail(A4G_ERR_RANGE, "fused step: too many tiles");
  // the 64-bit Horner sum over levels stays below 2^63: |S_t| <= (t+1) K 2^14
  for (const WInfo& I : wi) {
    const double K = double(I.S1 + I.S2);
    double bound = 0.0;
    for (int t = 0; t < S; ++t) bound = bound * 256.0 + double(t + 1) * K * 16384.0;
    if (bound >= 9.2e18) return fail(A4G_ERR_RANGE, "fused step: k too long for the exact 64-bit level sum");
  }
  P.nA = int(pa.size());
  size_t exps_n = 0;
  for (int i = 0; i < int(pa.size() + pb.size()); ++i) {
    OzPanel o = i < P.nA ? pa[size_t(i)] : pb[size_t(i - P.nA)];
    if (o.kpad > 0x7fffffffLL || int64_t(S) * o.rows_pad > 0x7fffffffLL)
      return fail(A4G_ERR_RANGE, "panel exceeds TMA coordinate range");
    o.exps = as_offset<int>(exps_n);
    exps_n += size_t(o.rows_pad);
    P.panels.push_back(o);
  }
  for (OzSplitJob& j : jobs_b) j.panel += P.nA;
  P.jobs = jobs_a;
  P.jobs.insert(P.jobs.end(), jobs_b.begin(), jobs_b.end());
  if (P.jobs.size() > 0x7fffffffu) return fail(A4G_ERR_RANGE, "fused step: too many split jobs");
  P.offs = offs.data;
  P.rowoffs = rowoffs.data;

  // ---- destination sub-blocks (store: column bases; energy: denominator tables)
  struct EW {
    size_t rk_at = 0, ck_at = 0, el_at = 0, ptab_at = 0;
    int ckn = 0, rkn = 0;
  };
  std::vector<EW> ew(wb.size());
  if (P.energy) {
    const bool last_row = cat[size_t(dl)] == kRow;
    TablePool<int> ikeys;
    std::map<std::vector<int>, size_t> ptab_index;  // orbital offsets and extents -> table offset
    for (size_t w = 0; w < wb.size(); ++w) {
      const WBlock& W = wb[w];
      const WInfo& I = wi[w];
      if (I.pa < 0) continue;
      const std::vector<int>& off = wb_off[w];
      std::vector<int> erow, ecol;
      for (int d : dims[kRow]) erow.push_back(W.dext[d]);
      for (int d : dims[kCol]) ecol.push_back(W.dext[d]);
      // rk[m] / ck[n]: the index over the row (column) dims without the last term's dim
      auto keys = [&](const std::vector<int>& cd, const std::vector<int>& ex, int64_t n) {
        std::vector<int> o(static_cast<size_t>(n));
        int c[kMaxRank];
        for (int64_t i = 0; i < n; ++i) {
          coords_of(i, ex, c);
          int64_t k = 0, mul = 1;
          for (size_t q = 0; q < cd.size(); ++q)
            if (cd[q] != dl) k += c[q] * mul, mul *= ex[q];
          o[size_t(i)] = int(k);
        }
        return o;
      };
      EW& E = ew[w];
      E.rk_at = ikeys.add(keys(dims[kRow], erow, I.M));
      E.ck_at = ikeys.add(keys(dims[kCol], ecol, I.N));
      // the last term's energies along its own dim (one array per block: its
      // values change with the block's segments, its place must not)
      {
        const std::vector<int>& cd = last_row ? dims[kRow] : dims[kCol];
        const std::vector<int>& ex = last_row ? erow : ecol;
        const int64_t n = last_row ? I.M : I.N;
        size_t qd = 0;
        while (cd[qd] != dl) ++qd;
        int c[kMaxRank];
        E.el_at = P.elast.size();
        for (int64_t i = 0; i < n; ++i) {
          coords_of(i, ex, c);
          P.elast.push_back(en.at(off[size_t(dl)] + c[qd]));
        }
      }
      // prefix table [b][j][rk][ck] (the chain without its last term), shared by
      // the blocks whose other dims have the same segments
      PtabTable tab{};
      int stride[4] = {1, 1, 1, 1};
      int group_of[kMaxRank], stride_of[kMaxRank];
      const int gcat[4] = {kRow, kCol, kB1, kB2};
      for (int g = 0; g < 4; ++g)
        for (int d : dims[gcat[g]]) {
          if (d == dl) continue;
          group_of[d] = g, stride_of[d] = stride[g];
          stride[g] *= W.dext[d];
        }
      tab.rkn = stride[0], tab.ckn = stride[1], tab.nb1 = stride[2], tab.nb2 = stride[3];
      E.rkn = tab.rkn, E.ckn = tab.ckn;
      tab.n = int64_t(tab.nb1) * tab.nb2 * tab.rkn * tab.ckn;
      tab.nterms = int(chain.size());
      for (size_t q = 0; q < chain.size(); ++q) {
        const int d = chain[q].first;
        tab.t[q] = {group_of[d], stride_of[d], W.dext[d], off[size_t(d)], chain[q].second};
      }
      std::vector<int> key = {tab.rkn, tab.ckn, tab.nb1, tab.nb2};
      for (int d = 0; d < drank; ++d)
        if (d != dl) key.push_back(off[size_t(d)]), key.push_back(W.dext[d]);
      auto it = ptab_index.find(key);
      if (it == ptab_index.end()) {
        if (P.ptab_n + tab.n > (int64_t(1) << 28)) return fail(A4G_ERR_RANGE, "fused energy: denominator tables beyond 2 GB");
        tab.at = P.ptab_n;
        P.ptab_n += tab.n;
        P.ptabs.push_back(tab);
        it = ptab_index.emplace(key, size_t(tab.at)).first;
      }
      E.ptab_at = it->second;
      sig.put(int64_t(E.ptab_at));
    }
    P.ikeys = ikeys.data;
  }
  for (const SubH& sb : subs) {
    const WBlock& W = wb[sb.w];
    const WInfo& I = wi[sb.w];
    OzDBlock db{};
    db.panel_a = I.pa, db.panel_b = I.pb;
    db.M = I.M, db.N = I.N;
    if (!P.energy) {
      std::vector<int64_t> ds(static_cast<size_t>(drank));
      int64_t s = 1;
      for (int d = 0; d < drank; ++d) ds[size_t(d)] = s, s *= W.dext[d];
      auto part = [&](int c, int64_t v) {  // destination offset of value v of category c's dims
        std::vector<int> ex;
        for (int d : dims[c]) ex.push_back(W.dext[d]);
        int cc[kMaxRank];
        coords_of(v, ex, cc);
        int64_t o = 0;
        for (size_t q = 0; q < dims[c].size(); ++q) o += cc[q] * ds[size_t(dims[c][q])];
        return o;
      };
      double* base = W.d + part(kB1, sb.b) + part(kB2, sb.j);
      std::vector<int> ex;
      std::vector<int64_t> st;
      for (int d : dims[kCol]) ex.push_back(W.dext[d]), st.push_back(ds[size_t(d)]);
      db.d = base;
      db.rowoff = as_offset<const int64_t>(I.rowoff_at);
      db.colptr = as_offset<double* const>(P.colptr.size());
      for (int64_t o : enum_offsets(ex, st)) P.colptr.push_back(base + o);
    } else {
      const EW& E = ew[sb.w];
      OzEnergyBlock eb{};
      eb.ptab = as_offset<const double>(E.ptab_at + (size_t(sb.b) * size_t(I.NB2) + size_t(sb.j)) * size_t(E.rkn) *
                                                        size_t(E.ckn));
      eb.rk = as_offset<const int>(E.rk_at);
      eb.ck = as_offset<const int>(E.ck_at);
      eb.elast = as_offset<const double>(E.el_at);
      eb.ckn = E.ckn;
      eb.last_row = cat[size_t(dl)] == kRow;
      P.eblocks.push_back(eb);
    }
    P.dblocks.push_back(db);
  }
  P.sig = sig.h;
  return A4G_OK;
}

// The split jobs with their address tables at d_offs.
std::vector<OzSplitJob> relocated_jobs(const Plan& P, const int64_t* d_offs) {
  std::vector<OzSplitJob> jobs = P.jobs;
  for (OzSplitJob& j : jobs) j.offRow = d_offs + offset_of(j.offRow), j.offK = d_offs + offset_of(j.offK);
  return jobs;
}

int launch_ptab(const a4g_fused* f, cudaStream_t s) {
  if (f->n_ptabs == 0) return A4G_OK;
  const unsigned gx = unsigned(std::min<int64_t>(4096, (f->max_ptab_n + 255) / 256));
  ptab_kernel<<<dim3(std::max(1u, gx), unsigned(f->n_ptabs)), 256, 0, s>>>(f->d_ptabs, f->e_dev, f->rank1, f->ld1,
                                                                           f->d_ptab);
  A4G_CUDA(cudaGetLastError());
  return A4G_OK;
}

}  // namespace

extern "C" {

int a4g_fused_create(a4g_fused** out, int drank, int lrank, int rrank, const a4g_term* terms, int nterms,
                     const a4g_fused_energy* energy, const a4g_batch_opts* opts) {
  if (!out) return fail(A4G_ERR_ARG, "null output handle");
  *out = nullptr;
  int rc = ensure_init();
  if (rc) return rc;
  const int precision = opts ? opts->precision : A4G_PREC_OZAKI_BF16;
  if (precision != A4G_PREC_OZAKI_BF16) return fail(A4G_ERR_UNSUPPORTED, "fused step: split precision only");
  const int S = opts && opts->slices ? opts->slices : 5;
  if (S < 1 || S > kOzMaxUsableSlices) return fail(A4G_ERR_ARG, "slices must be 1..7");
  const int beta = opts ? opts->beta : 0;
  if (beta != 0 && beta != 1) return fail(A4G_ERR_ARG, "beta must be 0 or 1");
  const int variant = opts ? opts->variant : 0;
  Plan P;
  if ((rc = plan_fused(drank, lrank, rrank, terms, nterms, energy, S, beta, variant, &P))) return rc;
  std::unique_ptr<a4g_fused> f(new a4g_fused());
  f->slices = S, f->drank = drank, f->lrank = lrank, f->rrank = rrank, f->nterms = nterms, f->beta = beta;
  f->variant = variant, f->levels = P.levels;
  f->energy = P.energy, f->efact = P.efact, f->signature = P.sig;
  f->flops = P.flops, f->pairs = P.pairs, f->elements = P.elements;
  f->zero_blocks = P.zero_blocks;
  cudaStream_t s = ctx()->stream;

  // ---- panels: exponents, zeroed digit buffers (the split writes live entries only), tensor maps
  std::vector<OzPanel> hp = P.panels;
  if (!hp.empty()) {
    size_t exps_n = 0;
    for (const OzPanel& o : hp) exps_n = std::max(exps_n, offset_of(o.exps) + size_t(o.rows_pad));
    void* p = nullptr;
    if ((rc = falloc(f.get(), exps_n * sizeof(int), &p))) return rc;
    f->d_exps = static_cast<int*>(p);
    f->exps_bytes = exps_n * sizeof(int);
    size_t digit_bytes = 0;
    std::vector<size_t> at(hp.size());
    for (size_t i = 0; i < hp.size(); ++i) {
      at[i] = digit_bytes;
      digit_bytes += ceil_to(int64_t(S) * hp[i].rows_pad * hp[i].kpad * 2, 1024);
    }
    if ((rc = falloc(f.get(), digit_bytes, &p))) return rc;
    A4G_CUDA(cudaMemset(p, 0, digit_bytes));
    std::vector<MapImage> maps(hp.size());
    for (size_t i = 0; i < hp.size(); ++i) {
      hp[i].base = reinterpret_cast<__nv_bfloat16*>(static_cast<char*>(p) + at[i]);
      hp[i].exps = f->d_exps + offset_of(hp[i].exps);
      // all-levels form: 32-wide k boxes of 128 rows (A) or 64 columns (B)
      const int box_rows = P.levels && int(i) >= P.nA ? kOzLevelsTileCols : kOzBM;
      if ((rc = oz_make_tensor_map_k(maps[i].b, hp[i].base, hp[i].kpad, int64_t(S) * hp[i].rows_pad, box_rows,
                                     P.levels ? 32 : kOzBK)))
        return rc;
    }
    MapImage* d_maps = nullptr;
    if ((rc = fupload(f.get(), maps, &d_maps))) return rc;
    if ((rc = fupload(f.get(), hp, &f->d_panels))) return rc;
    f->args.maps_a = d_maps;
    f->args.maps_b = d_maps + P.nA;
  }
  // ---- split jobs (generic layout: any strides, the sign)
  if ((rc = fupload(f.get(), P.offs, &f->d_offs))) return rc;
  f->h_jobs = relocated_jobs(P, f->d_offs);
  std::vector<int64_t> pe(1, 0), ps(1, 0);
  for (const OzSplitJob& j : f->h_jobs) {
    pe.push_back(pe.back() + oz_exp_tiles(kOzGeneric, j.rows, j.K));
    ps.push_back(ps.back() + oz_split_tiles(kOzGeneric, j.rows, j.K));
  }
  f->njobs = int(f->h_jobs.size());
  f->tiles_exp = pe.back(), f->tiles_split = ps.back();
  if ((rc = fupload(f.get(), f->h_jobs, &f->d_jobs)) || (rc = fupload(f.get(), pe, &f->d_prefix_exp)) ||
      (rc = fupload(f.get(), ps, &f->d_prefix_split)))
    return rc;
  // ---- destination sub-blocks
  int64_t* d_rowoffs = nullptr;
  if ((rc = fupload(f.get(), P.rowoffs, &d_rowoffs))) return rc;
  if ((rc = fupload(f.get(), P.colptr, &f->d_colptr))) return rc;
  f->n_colptr = P.colptr.size();
  std::vector<OzDBlock> dblocks = P.dblocks;
  for (OzDBlock& db : dblocks)
    if (!f->energy) db.rowoff = d_rowoffs + offset_of(db.rowoff), db.colptr = f->d_colptr + offset_of(db.colptr);
  std::vector<OzEnergyBlock> eblocks = P.eblocks;
  if (f->energy) {
    int* d_ikeys = nullptr;
    if ((rc = fupload(f.get(), P.ikeys, &d_ikeys)) || (rc = fupload(f.get(), P.elast, &f->d_elast)) ||
        (rc = fupload(f.get(), P.ptabs, &f->d_ptabs)))
      return rc;
    f->n_elast = P.elast.size();
    void* p = nullptr;
    if ((rc = falloc(f.get(), size_t(P.ptab_n) * sizeof(double), &p))) return rc;
    f->d_ptab = static_cast<double*>(p);
    f->n_ptabs = int(P.ptabs.size());
    for (const PtabTable& t : P.ptabs) f->max_ptab_n = std::max(f->max_ptab_n, t.n);
    f->e_dev = P.e_dev, f->rank1 = P.rank1, f->ld1 = P.ld1;
    if ((rc = launch_ptab(f.get(), s))) return rc;
    for (OzEnergyBlock& eb : eblocks) {
      eb.ptab = f->d_ptab + offset_of(eb.ptab);
      eb.rk = d_ikeys + offset_of(eb.rk);
      eb.ck = d_ikeys + offset_of(eb.ck);
      eb.elast = f->d_elast + offset_of(eb.elast);
    }
  }

  // ---- the GEMM: direct form, one SM per tile; one level at a time: work
  // units (tile, level), all levels of a tile in a row; all levels at once:
  // the tiles themselves
  std::vector<OzUnit> units;
  if (!P.levels) units.reserve(P.tiles.size() * size_t(S));
  for (size_t g = 0; g < (P.levels ? 0 : P.tiles.size()); ++g)
    for (int lv = 0; lv < S; ++lv) {
      OzUnit u{};
      u.tile = int(g), u.level = lv, u.split = 0;
      u.kb_begin = 0, u.kb_end = P.tiles[g].kb_total;
      u.trip_first = P.tiles[g].trip_begin, u.kb_in_trip = 0;
      units.push_back(u);
    }
  OzGemmArgs& a = f->args;
  a.panels_a = f->d_panels;
  a.panels_b = f->d_panels ? f->d_panels + P.nA : nullptr;
  OzDBlock* d_dblocks = nullptr;
  OzEnergyBlock* d_eblocks = nullptr;
  OzTile* d_tiles = nullptr;
  OzTrip* d_trips = nullptr;
  OzUnit* d_units = nullptr;
  if ((rc = fupload(f.get(), dblocks, &d_dblocks)) || (rc = fupload(f.get(), eblocks, &d_eblocks)) ||
      (rc = fupload(f.get(), P.tiles, &d_tiles)) || (rc = fupload(f.get(), P.trips, &d_trips)) ||
      (rc = fupload(f.get(), units, &d_units)))
    return rc;
  a.tiles = d_tiles, a.trips = d_trips, a.units = d_units;
  a.n_units = int(units.size()), a.n_tiles = int(P.tiles.size());
  a.slices = S, a.nsplit = 1;
  for (int lv = 0; lv < kOzMaxSlices; ++lv) a.chunk_kb[lv] = lv < S ? oz_chunk_kb(lv) : 1;
  a.ws = nullptr;
  a.err_flag = ctx()->d_error_flag;
  a.direct = 1;
  a.mode = beta;
  a.dry = 0;
  a.dblocks = d_dblocks;
  a.energy = f->energy ? 1 : 0;
  a.eblocks = d_eblocks;
  const int sms = ctx()->num_sms > 0 ? ctx()->num_sms : 152;
  f->grid = int(std::min<int64_t>(sms, std::max<int64_t>(1, int64_t(P.tiles.size()))));
  if (f->energy) {
    f->epart_len = f->grid * 16 * 32;
    void* p = nullptr;
    if ((rc = falloc(f.get(), size_t(f->epart_len) * sizeof(double), &p))) return rc;
    f->d_epart = static_cast<double*>(p);
    a.epart = f->d_epart;
  }
  if ((rc = oz_prepare())) return rc;
  A4G_CUDA(cudaStreamSynchronize(s));
  A4G_CUDA(cudaDeviceSynchronize());
  *out = f.release();
  return A4G_OK;
}

int a4g_fused_rebind(a4g_fused* f, const a4g_term* terms, int nterms, const a4g_fused_energy* energy, void* stream) {
  if (!f) return fail(A4G_ERR_ARG, "null fused step");
  if ((energy != nullptr) != f->energy) return fail(A4G_ERR_ARG, "fused rebind: energy form differs from the creation's");
  Plan P;
  int rc = plan_fused(f->drank, f->lrank, f->rrank, terms, nterms, energy, f->slices, f->beta, f->variant, &P);
  if (rc) return rc;
  if (P.sig != f->signature || P.jobs.size() != f->h_jobs.size() || P.colptr.size() != f->n_colptr ||
      P.elast.size() != f->n_elast || int(P.ptabs.size()) != f->n_ptabs)
    return fail(A4G_ERR_ARG, "fused rebind: the triples' structure differs from the creation's");
  cudaStream_t s = pick(stream);
  // only what depends on the blocks: split-job sources, column bases, energy tables
  f->h_jobs = relocated_jobs(P, f->d_offs);
  A4G_CUDA(cudaMemcpyAsync(f->d_jobs, f->h_jobs.data(), f->h_jobs.size() * sizeof(OzSplitJob), cudaMemcpyHostToDevice, s));
  if (!P.colptr.empty())
    A4G_CUDA(cudaMemcpyAsync(f->d_colptr, P.colptr.data(), P.colptr.size() * sizeof(double*), cudaMemcpyHostToDevice, s));
  f->zero_blocks = P.zero_blocks;
  if (f->energy) {
    A4G_CUDA(cudaMemcpyAsync(f->d_elast, P.elast.data(), P.elast.size() * sizeof(double), cudaMemcpyHostToDevice, s));
    A4G_CUDA(cudaMemcpyAsync(f->d_ptabs, P.ptabs.data(), P.ptabs.size() * sizeof(PtabTable), cudaMemcpyHostToDevice, s));
    f->e_dev = P.e_dev, f->efact = P.efact;
    if ((rc = launch_ptab(f, s))) return rc;
  }
  // the host vectors must outlive the copies: pageable sources are staged before these calls return
  return A4G_OK;
}

int a4g_fused_run(a4g_fused* f, double* esum, void* stream) {
  if (!f) return fail(A4G_ERR_ARG, "null fused step");
  if (f->energy && !esum) return fail(A4G_ERR_ARG, "fused energy: null esum");
  cudaStream_t s = pick(stream);
  int rc;
  for (auto& z : f->zero_blocks)
    if ((rc = launch_fill(z.first, z.second, 0.0, s))) return rc;
  if (f->args.n_tiles <= 0) return A4G_OK;
  A4G_CUDA(cudaMemsetAsync(f->d_exps, 0, f->exps_bytes, s));
  if ((rc = oz_launch_exp(kOzGeneric, f->d_jobs, f->d_prefix_exp, f->njobs, f->tiles_exp, f->d_panels, s)) ||
      (rc = oz_launch_split(kOzGeneric, f->d_jobs, f->d_prefix_split, f->njobs, f->tiles_split, f->d_panels,
                            f->slices, s)) ||
      (rc = f->levels ? oz_launch_levels(f->args, f->grid, s) : oz_launch_gemm(f->args, f->grid, false, kOzBN, s)))
    return rc;
  if (f->energy) return oz_launch_energy_reduce(f->d_epart, f->epart_len, f->efact, esum, s);
  return A4G_OK;
}

int a4g_fused_info(const a4g_fused* f, int64_t* pairs, double* flops, int64_t* elements, int64_t* device_bytes) {
  if (!f) return fail(A4G_ERR_ARG, "null fused step");
  if (pairs) *pairs = f->pairs;
  if (flops) *flops = f->flops;
  if (elements) *elements = f->elements;
  if (device_bytes) *device_bytes = f->device_bytes;
  return A4G_OK;
}

int a4g_fused_form(const a4g_fused* f) { return f ? (f->levels ? 7 : 5) : -1; }

void a4g_fused_destroy(a4g_fused* f) { delete f; }

}  // extern "C"
