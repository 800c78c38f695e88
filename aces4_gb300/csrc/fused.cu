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

struct a4g_fused {
  int slices = 5;
  int drank = 0, lrank = 0, rrank = 0;
  int beta = 0;
  bool energy = false;
  double efact = 1.0;
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

}  // namespace

extern "C" {

int a4g_fused_create(a4g_fused** out, int drank, int lrank, int rrank, const a4g_term* terms, int nterms,
                     const a4g_fused_energy* energy, const a4g_batch_opts* opts) {
  if (!out) return fail(A4G_ERR_ARG, "null output handle");
  *out = nullptr;
  int rc = ensure_init();
  if (rc) return rc;
  if (!terms || nterms < 1 || nterms > 2) return fail(A4G_ERR_ARG, "fused step: one or two terms");
  if (drank < 1 || drank > kMaxRank || lrank < 1 || lrank > kMaxRank || rrank < 1 || rrank > kMaxRank)
    return fail(A4G_ERR_ARG, "fused step: ranks out of range (tensor-tensor contractions only)");
  const int precision = opts ? opts->precision : A4G_PREC_OZAKI_BF16;
  if (precision != A4G_PREC_OZAKI_BF16) return fail(A4G_ERR_UNSUPPORTED, "fused step: split precision only");
  const int S = opts && opts->slices ? opts->slices : 5;
  if (S < 1 || S > kOzMaxUsableSlices) return fail(A4G_ERR_ARG, "slices must be 1..7");
  const int beta = opts ? opts->beta : 0;
  if (beta != 0 && beta != 1) return fail(A4G_ERR_ARG, "beta must be 0 or 1");

  // ---- the terms' index maps
  std::vector<Term> T(static_cast<size_t>(nterms));
  for (int t = 0; t < nterms; ++t) {
    const a4g_term& tm = terms[t];
    if (!tm.contr_ptrn || (tm.n_triples > 0 && !tm.triples) || tm.n_triples < 0)
      return fail(A4G_ERR_ARG, "fused step: null term");
    if (tm.sign != 1 && tm.sign != -1) return fail(A4G_ERR_ARG, "fused step: term sign must be +1 or -1");
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
      if (x.l && x.r) w.pairs[t].push_back({x.l, x.r, x.lext, x.rext});
    }
  }
  std::unique_ptr<a4g_fused> f(new a4g_fused());
  f->slices = S, f->drank = drank, f->lrank = lrank, f->rrank = rrank, f->beta = beta;
  f->energy = energy != nullptr;

  // ---- energy inputs
  Energies en;
  int pos[6] = {0, 1, 2, 3, 4, 5};
  std::map<double*, std::vector<int>> wb_off;  // orbital offset per destination dim
  int dl = -1;                                 // destination dim of the chain's last term
  std::vector<std::pair<int, int>> chain;      // prefix: (destination dim, +1 add / -1 subtract), first assigned
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
      if (pos[q] < 0 || pos[q] >= drank || seen[pos[q]]) return fail(A4G_ERR_ARG, "fused energy: den_order is not a permutation");
      seen[pos[q]] = true;
    }
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
    en.h.resize(size_t(ne));
    A4G_CUDA(cudaMemcpy(en.h.data(), energy->e_or_fock, size_t(ne) * sizeof(double), cudaMemcpyDeviceToHost));
    const std::vector<int> segs(energy->seg_sizes, energy->seg_sizes + std::max(energy->nsegs, 0));
    for (int64_t i = 0; i < energy->n_blocks; ++i) {
      auto it = widx.find(energy->blocks[i]);
      if (it == widx.end()) continue;  // a block no term writes: zero, adds nothing
      std::vector<int> off(static_cast<size_t>(drank));
      rc = denominator_offsets(drank, energy->index_values + i * drank, wb[it->second].dext, energy->rank1,
                               energy->ext1, segs, off.data());
      if (rc) return rc;
      wb_off[energy->blocks[i]] = off;
    }
    for (const WBlock& w : wb)
      if (!wb_off.count(w.d)) return fail(A4G_ERR_ARG, "fused energy: a destination block without index values");
    f->efact = energy->efact;
  }

  // ---- panels, split jobs, sub-problems, tiles
  struct PanelH {
    int rows = 0;
    int64_t kpad = 0;
  };
  std::vector<PanelH> pa, pb;
  std::map<std::vector<int64_t>, int> pb_index;
  TablePool<int64_t> offs;  // split-job address tables
  struct JobH {
    OzSplitJob j;
    size_t row_at, k_at;  // into offs
  };
  std::vector<JobH> jobs_a, jobs_b;
  struct SubH {
    size_t w;
    int b, j;
  };
  std::vector<SubH> subs;
  std::vector<OzDBlock> dblocks;
  std::vector<OzTile> tiles;
  std::vector<OzTrip> trips;
  std::vector<int> sub_pa, sub_pb;
  // per destination block
  struct WInfo {
    int M = 0, N = 0, NB1 = 1, NB2 = 1;
    int64_t S1 = 0, S2 = 0;  // stretch lengths (64-aligned)
    std::vector<int64_t> pk[2];  // k offset of each pair inside its stretch
    int pa = -1, pb = -1;
    size_t rowoff_at = 0;
  };
  std::vector<WInfo> wi(wb.size());
  TablePool<int64_t> rowoffs;
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
      if (!f->energy && beta == 0) f->zero_blocks.push_back({W.d, s});
      continue;
    }
    for (int t = 0; t < nterms; ++t) {
      int64_t k = 0;
      for (const FPair& p : W.pairs[t]) {
        int64_t K = 1;
        for (auto& c : T[size_t(t)].con) K *= p.lext[c.first];
        I.pk[t].push_back(k);
        k += ceil_to(K, 8);  // 8 columns: the split kernels' vector stores stay aligned
        f->flops += 2.0 * double(M) * double(N) * double(NB1 * NB2) * double(K);
        ++f->pairs;
      }
      (t == 0 ? I.S1 : I.S2) = ceil_to(k, kOzBK);
    }
    f->elements += M * N * NB1 * NB2;
    // A panel: per B1 value a term-1 stretch, then per B2 value a term-2 stretch
    PanelH A;
    A.rows = int(M);
    A.kpad = NB1 * I.S1 + NB2 * I.S2;
    I.pa = int(pa.size());
    pa.push_back(A);
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
      PanelH B;
      B.rows = int(N);
      B.kpad = NB2 * I.S1 + NB1 * I.S2;
      bit = pb_index.emplace(key, int(pb.size())).first;
      pb.push_back(B);
    }
    I.pb = bit->second;
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
        for (auto& c : tm.con) kext.push_back(p.lext[c.first]), kl.push_back(ls[size_t(c.first)]), kr.push_back(rs[size_t(c.second)]);
        const std::vector<int64_t> okl = enum_offsets(kext, kl), okr = enum_offsets(kext, kr);
        const std::vector<int64_t> orl = enum_offsets(ext_of(kRow), strides(kRow, true));
        const std::vector<int64_t> fl = enum_offsets(ext_of(fixL), strides(fixL, true));
        const size_t rl_at = offs.add(orl), kl_at = offs.add(okl);
        const int K = int(okl.size());
        for (int64_t v = 0; v < nfixL; ++v) {
          JobH jh{};
          jh.j.src = p.l + fl[size_t(v)];
          jh.j.rows = int(M);
          jh.j.K = K;
          jh.j.kfast = K > 1 && okl[1] == 1;
          jh.j.panel = I.pa;
          jh.j.koff = baseA + v * strideA + I.pk[t][pi];
          jh.j.negate = tm.sign < 0;
          jh.row_at = rl_at, jh.k_at = kl_at;
          jobs_a.push_back(jh);
        }
        if (new_b) {
          const std::vector<int64_t> orr = enum_offsets(ext_of(kCol), strides(kCol, false));
          const std::vector<int64_t> fr = enum_offsets(ext_of(fixR), strides(fixR, false));
          const size_t rr_at = offs.add(orr), kr_at = offs.add(okr);
          for (int64_t v = 0; v < nfixR; ++v) {
            JobH jh{};
            jh.j.src = p.r + fr[size_t(v)];
            jh.j.rows = int(N);
            jh.j.K = K;
            jh.j.kfast = K > 1 && okr[1] == 1;
            jh.j.panel = I.pb;  // shifted past the A panels below
            jh.j.koff = baseB + v * strideB + I.pk[t][pi];
            jh.row_at = rr_at, jh.k_at = kr_at;
            jobs_b.push_back(jh);
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
        const int sub = int(subs.size());
        subs.push_back({w, int(b), int(j)});
        const int trip_begin = int(trips.size());
        int kb_total = 0;
        if (!W.pairs[0].empty()) {
          OzTrip tr{};
          tr.koff_a = b * I.S1, tr.koff_b = j * I.S1, tr.nkb = int(I.S1 / kOzBK);
          trips.push_back(tr);
          kb_total += tr.nkb;
        }
        if (nterms == 2 && !W.pairs[1].empty()) {
          OzTrip tr{};
          tr.koff_a = NB1 * I.S1 + j * I.S2, tr.koff_b = NB2 * I.S1 + b * I.S2, tr.nkb = int(I.S2 / kOzBK);
          trips.push_back(tr);
          kb_total += tr.nkb;
        }
        for (int64_t m0 = 0; m0 < M; m0 += kOzBM)
          for (int64_t n0 = 0; n0 < N; n0 += kOzBN) {
            OzTile tl{};
            tl.dblock = sub, tl.m0 = int(m0), tl.n0 = int(n0);
            tl.panel_a = I.pa, tl.panel_b = I.pb;
            tl.trip_begin = trip_begin, tl.trip_end = int(trips.size());
            tl.kb_total = kb_total;
            tiles.push_back(tl);
          }
      }
  }
  if (tiles.size() > size_t(0x7fffffff / kOzMaxSlices)) return fail(A4G_ERR_RANGE, "fused step: too many tiles");
  // the 64-bit Horner sum over levels stays below 2^63: |S_t| <= (t+1) K 2^14
  for (const WInfo& I : wi) {
    const double K = double(I.S1 + I.S2);
    double bound = 0.0;
    for (int t = 0; t < S; ++t) bound = bound * 256.0 + double(t + 1) * K * 16384.0;
    if (bound >= 9.2e18) return fail(A4G_ERR_RANGE, "fused step: k too long for the exact 64-bit level sum");
  }

  // ---- device memory: exponents, panels, tensor maps
  const int nA = int(pa.size()), nB = int(pb.size());
  size_t exps_n = 0;
  std::vector<OzPanel> hp;
  for (int i = 0; i < nA + nB; ++i) {
    const PanelH& P = i < nA ? pa[size_t(i)] : pb[size_t(i - nA)];
    OzPanel o{};
    o.rows = P.rows;
    o.rows_pad = int(ceil_to(P.rows, kOzBM));
    o.kpad = P.kpad;
    if (o.kpad > 0x7fffffffLL || int64_t(S) * o.rows_pad > 0x7fffffffLL)
      return fail(A4G_ERR_RANGE, "panel exceeds TMA coordinate range");
    o.exps = reinterpret_cast<int*>(exps_n);  // offset for now
    exps_n += size_t(o.rows_pad);
    hp.push_back(o);
  }
  if (!hp.empty()) {
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
    A4G_CUDA(cudaMemset(p, 0, digit_bytes));  // padding stays zero: the split writes live entries only
    std::vector<MapImage> maps(hp.size());
    for (size_t i = 0; i < hp.size(); ++i) {
      hp[i].base = reinterpret_cast<__nv_bfloat16*>(static_cast<char*>(p) + at[i]);
      hp[i].exps = f->d_exps + reinterpret_cast<size_t>(hp[i].exps);
      if ((rc = oz_make_tensor_map(maps[i].b, hp[i].base, hp[i].kpad, int64_t(S) * hp[i].rows_pad, kOzBM)))
        return rc;
    }
    MapImage* d_maps = nullptr;
    if ((rc = fupload(f.get(), maps, &d_maps))) return rc;
    if ((rc = fupload(f.get(), hp, &f->d_panels))) return rc;
    f->args.maps_a = d_maps;
    f->args.maps_b = d_maps + nA;
  }
  // ---- split jobs (generic layout: any strides, the sign)
  int64_t* d_offs = nullptr;
  if ((rc = fupload(f.get(), offs.data, &d_offs))) return rc;
  std::vector<OzSplitJob> jobs;
  std::vector<int64_t> pe(1, 0), ps(1, 0);
  for (int side = 0; side < 2; ++side)
    for (JobH& jh : side == 0 ? jobs_a : jobs_b) {
      jh.j.offRow = d_offs + jh.row_at;
      jh.j.offK = d_offs + jh.k_at;
      if (side == 1) jh.j.panel += nA;
      jobs.push_back(jh.j);
      pe.push_back(pe.back() + oz_exp_tiles(kOzGeneric, jh.j.rows, jh.j.K));
      ps.push_back(ps.back() + oz_split_tiles(kOzGeneric, jh.j.rows, jh.j.K));
    }
  if (jobs.size() > 0x7fffffffu) return fail(A4G_ERR_RANGE, "fused step: too many split jobs");
  f->njobs = int(jobs.size());
  f->tiles_exp = pe.back(), f->tiles_split = ps.back();
  if ((rc = fupload(f.get(), jobs, &f->d_jobs)) || (rc = fupload(f.get(), pe, &f->d_prefix_exp)) ||
      (rc = fupload(f.get(), ps, &f->d_prefix_split)))
    return rc;

  // ---- destination sub-blocks (store: row offsets and column bases; energy: denominator tables)
  int64_t* d_rowoffs = nullptr;
  if ((rc = fupload(f.get(), rowoffs.data, &d_rowoffs))) return rc;
  std::vector<double*> colptr;
  std::vector<OzEnergyBlock> eblocks;
  TablePool<int> ikeys;
  TablePool<double> elast;
  std::map<std::vector<int>, size_t> ptab_index;  // structure key -> offset into ptab
  std::vector<double> ptab;
  struct EW {
    size_t rk_at, ck_at, el_at, ptab_at;
    int ckn, rkn;
  };
  std::vector<EW> ew(wb.size());
  if (f->energy) {
    const bool last_row = cat[size_t(dl)] == kRow;
    for (size_t w = 0; w < wb.size(); ++w) {
      const WBlock& W = wb[w];
      const WInfo& I = wi[w];
      if (I.pa < 0) continue;
      const std::vector<int>& off = wb_off[W.d];
      auto keyed = [&](int c) {  // dims of category c except the last term's, and their extents
        std::vector<int> ds, ex;
        for (int d : dims[c])
          if (d != dl) ds.push_back(d), ex.push_back(W.dext[d]);
        return std::make_pair(ds, ex);
      };
      const auto rkd = keyed(kRow), ckd = keyed(kCol), b1d = keyed(kB1), b2d = keyed(kB2);
      auto count = [](const std::vector<int>& ex) {
        int64_t n = 1;
        for (int e : ex) n *= e;
        return n;
      };
      const int64_t rkn = count(rkd.second), ckn = count(ckd.second);
      // rk[m] / ck[n]: the index over the row (column) dims without the last term's dim
      std::vector<int> erow, ecol;
      for (int d : dims[kRow]) erow.push_back(W.dext[d]);
      for (int d : dims[kCol]) ecol.push_back(W.dext[d]);
      auto keys = [&](const std::vector<int>& cd, const std::vector<int>& ex, int64_t n) {
        std::vector<int> out(static_cast<size_t>(n));
        int c[kMaxRank];
        for (int64_t i = 0; i < n; ++i) {
          coords_of(i, ex, c);
          int64_t k = 0, mul = 1;
          for (size_t q = 0; q < cd.size(); ++q)
            if (cd[q] != dl) k += c[q] * mul, mul *= ex[q];
          out[size_t(i)] = int(k);
        }
        return out;
      };
      EW& E = ew[w];
      E.rkn = int(rkn), E.ckn = int(ckn);
      E.rk_at = ikeys.add(keys(dims[kRow], erow, I.M));
      E.ck_at = ikeys.add(keys(dims[kCol], ecol, I.N));
      // the last term's energies along its own dim
      {
        const std::vector<int>& cd = last_row ? dims[kRow] : dims[kCol];
        const std::vector<int>& ex = last_row ? erow : ecol;
        const int64_t n = last_row ? I.M : I.N;
        size_t qd = 0;
        while (cd[qd] != dl) ++qd;
        std::vector<double> el(static_cast<size_t>(n));
        int c[kMaxRank];
        for (int64_t i = 0; i < n; ++i) {
          coords_of(i, ex, c);
          el[size_t(i)] = en.at(off[size_t(dl)] + c[qd]);
        }
        E.el_at = elast.add(el);
      }
      // prefix table [b][j][rk][ck]: the chain without its last term, in the reference's order
      std::vector<int> key = {int(rkn), int(ckn), I.NB1, I.NB2};
      for (int d = 0; d < drank; ++d)
        if (d != dl) key.push_back(off[size_t(d)]), key.push_back(W.dext[d]);
      auto it = ptab_index.find(key);
      if (it == ptab_index.end()) {
        const int64_t n = int64_t(I.NB1) * I.NB2 * rkn * ckn;
        if (int64_t(ptab.size()) + n > (int64_t(1) << 28))
          return fail(A4G_ERR_RANGE, "fused energy: denominator tables beyond 2 GB");
        const size_t at = ptab.size();
        ptab.resize(at + size_t(n));
        std::vector<int> coord(size_t(drank), 0);
        int c[kMaxRank];
        const std::vector<int>* cdims[4] = {&rkd.first, &ckd.first, &b1d.first, &b2d.first};
        const std::vector<int>* cext[4] = {&rkd.second, &ckd.second, &b1d.second, &b2d.second};
        int64_t i = 0;
        for (int64_t b = 0; b < I.NB1; ++b)
          for (int64_t j = 0; j < I.NB2; ++j)
            for (int64_t r = 0; r < rkn; ++r)
              for (int64_t k = 0; k < ckn; ++k, ++i) {
                const int64_t idx[4] = {r, k, b, j};
                for (int g = 0; g < 4; ++g) {
                  coords_of(idx[g], *cext[g], c);
                  for (size_t q = 0; q < cdims[g]->size(); ++q) coord[size_t((*cdims[g])[q])] = c[q];
                }
                double v = en.at(off[size_t(chain[0].first)] + coord[size_t(chain[0].first)]);
                for (size_t q = 1; q < chain.size(); ++q) {
                  const double e = en.at(off[size_t(chain[q].first)] + coord[size_t(chain[q].first)]);
                  v = chain[q].second > 0 ? v + e : v - e;
                }
                ptab[at + size_t(i)] = v;
              }
        it = ptab_index.emplace(key, at).first;
      }
      E.ptab_at = it->second;
    }
  }
  int* d_ikeys = nullptr;
  double *d_elast = nullptr, *d_ptab = nullptr;
  if (f->energy) {
    if ((rc = fupload(f.get(), ikeys.data, &d_ikeys)) || (rc = fupload(f.get(), elast.data, &d_elast)) ||
        (rc = fupload(f.get(), ptab, &d_ptab)))
      return rc;
  }
  for (const SubH& sb : subs) {
    const WBlock& W = wb[sb.w];
    const WInfo& I = wi[sb.w];
    OzDBlock db{};
    db.panel_a = I.pa, db.panel_b = I.pb;
    db.M = I.M, db.N = I.N;
    if (!f->energy) {
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
      const std::vector<int64_t> co = enum_offsets(ex, st);
      db.d = base;
      db.rowoff = d_rowoffs + I.rowoff_at;
      db.colptr = reinterpret_cast<double* const*>(colptr.size());  // offset for now
      for (int64_t o : co) colptr.push_back(base + o);
    } else {
      const EW& E = ew[sb.w];
      OzEnergyBlock eb{};
      eb.ptab = d_ptab + E.ptab_at + (size_t(sb.b) * size_t(I.NB2) + size_t(sb.j)) * size_t(E.rkn) * size_t(E.ckn);
      eb.rk = d_ikeys + E.rk_at;
      eb.ck = d_ikeys + E.ck_at;
      eb.elast = d_elast + E.el_at;
      eb.ckn = E.ckn;
      eb.last_row = cat[size_t(dl)] == kRow;
      eblocks.push_back(eb);
    }
    dblocks.push_back(db);
  }
  if (!f->energy && !colptr.empty()) {
    double** d_colptr = nullptr;
    if ((rc = fupload(f.get(), colptr, &d_colptr))) return rc;
    for (OzDBlock& db : dblocks) db.colptr = d_colptr + reinterpret_cast<size_t>(db.colptr);
  }

  // ---- the GEMM: direct form, one SM per 128 x 128 tile, all levels of a tile in a row
  std::vector<OzUnit> units;
  units.reserve(tiles.size() * size_t(S));
  for (size_t g = 0; g < tiles.size(); ++g)
    for (int lv = 0; lv < S; ++lv) {
      OzUnit u{};
      u.tile = int(g), u.level = lv, u.split = 0;
      u.kb_begin = 0, u.kb_end = tiles[g].kb_total;
      u.trip_first = tiles[g].trip_begin, u.kb_in_trip = 0;
      units.push_back(u);
    }
  OzGemmArgs& a = f->args;
  a.panels_a = f->d_panels;
  a.panels_b = f->d_panels ? f->d_panels + nA : nullptr;
  OzDBlock* d_dblocks = nullptr;
  OzEnergyBlock* d_eblocks = nullptr;
  OzTile* d_tiles = nullptr;
  OzTrip* d_trips = nullptr;
  OzUnit* d_units = nullptr;
  if ((rc = fupload(f.get(), dblocks, &d_dblocks)) || (rc = fupload(f.get(), eblocks, &d_eblocks)) ||
      (rc = fupload(f.get(), tiles, &d_tiles)) || (rc = fupload(f.get(), trips, &d_trips)) ||
      (rc = fupload(f.get(), units, &d_units)))
    return rc;
  a.tiles = d_tiles, a.trips = d_trips, a.units = d_units;
  a.n_units = int(units.size()), a.n_tiles = int(tiles.size());
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
  f->grid = int(std::min<int64_t>(sms, std::max<int64_t>(1, int64_t(tiles.size()))));
  if (f->energy) {
    f->epart_len = f->grid * 16 * 32;
    void* p = nullptr;
    if ((rc = falloc(f.get(), size_t(f->epart_len) * sizeof(double), &p))) return rc;
    f->d_epart = static_cast<double*>(p);
    a.epart = f->d_epart;
  }
  if ((rc = oz_prepare())) return rc;
  A4G_CUDA(cudaDeviceSynchronize());
  *out = f.release();
  return A4G_OK;
}

int a4g_fused_run(a4g_fused* f, double* esum, void* stream) {
  if (!f) return fail(A4G_ERR_ARG, "null fused step");
  if (f->energy && !esum) return fail(A4G_ERR_ARG, "fused energy: null esum");
  cudaStream_t s = pick(stream);
  int rc;
  for (auto& z : f->zero_blocks)
    if ((rc = launch_fill(z.first, z.second, 0.0, s))) return rc;
  if (f->args.n_units <= 0) return A4G_OK;
  A4G_CUDA(cudaMemsetAsync(f->d_exps, 0, f->exps_bytes, s));
  if ((rc = oz_launch_exp(kOzGeneric, f->d_jobs, f->d_prefix_exp, f->njobs, f->tiles_exp, f->d_panels, s)) ||
      (rc = oz_launch_split(kOzGeneric, f->d_jobs, f->d_prefix_split, f->njobs, f->tiles_split, f->d_panels,
                            f->slices, s)) ||
      (rc = oz_launch_gemm(f->args, f->grid, false, kOzBN, s)))
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

void a4g_fused_destroy(a4g_fused* f) { delete f; }

}  // extern "C"
