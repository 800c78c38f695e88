/*
 * CPU oracle for the ACES4 block-contraction path (TEST INFRASTRUCTURE ONLY).
 *
 * Every function restates the reference algorithm it names, in plain C, with
 * the same argument meaning, the same overwrite/accumulate semantics and the
 * same error codes.  Loops are written for clarity, not speed; OpenMP is used
 * only where the reference itself threads the loop, so the timed CPU baseline
 * is not handicapped.  Reference paths are relative to the ACES4 source tree.
 */
#include "a4_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* ---------------------------------------------------------------------- */
/* tensor_size_by_shape  (src/sip/tensor_algebra/tensor_dil_omp.F90:66-84) */
int64_t a4o_tensor_size_by_shape(int num_dim, const int* dims, int* ierr) {
  int64_t s = 1;
  *ierr = 0;
  if (num_dim > 0) {
    for (int i = 0; i < num_dim; ++i) s *= dims[i];
    if (s <= 0) *ierr = 2;
  } else if (num_dim < 0) {
    *ierr = 1;
    s = 0;
  }
  return s;
}

/* Stable sort of item numbers by key: the reference uses a von Neumann merge
 * sort that never moves a right item ahead of an equal left item
 * (merge_sort_key_int_, tensor_dil_omp.F90:1183-1236), i.e. a stable sort.
 * Any stable sort gives the same permutation; insertion sort is used here.
 * trn holds 1-based item numbers, key is indexed by item number - 1. */
static void stable_sort_by_key(int ni, const int* key, int* trn) {
  for (int i = 1; i < ni; ++i) {
    int t = trn[i];
    int j = i - 1;
    while (j >= 0 && key[trn[j] - 1] > key[t - 1]) {
      trn[j + 1] = trn[j];
      --j;
    }
    trn[j + 1] = t;
  }
}

/* get_contraction_ptrn (tensor_dil_omp.F90:87-142), restated by counting
 * labels instead of sorting them (the library's planner transliterates the
 * reference's stable sort; this restatement takes another route to the same
 * results, so each checks the other).
 * aces_ptrn = [d labels (drank), l labels (lrank), r labels (rrank)].
 * my_ptrn[0 .. lrank+rrank-1]: for an uncontracted operand index the 1-based
 * destination position; for a contracted one minus the 1-based position of
 * its partner in the other operand.
 * The reference sorts the positions by label (stably) and walks the sorted
 * list in pairs: the first pair, in ascending label order, whose labels
 * differ gives ierr 4, and a pair equal to the pair before it ierr 5.  In
 * terms of counts: visiting the distinct labels in ascending order, the
 * first label not used exactly twice decides: used once or three times,
 * ierr 4 (its last use pairs with the next label); four or more times, ierr
 * 5.  Then each label's two positions p < q (in index order) must be a
 * destination position and an operand position (uncontracted), or a left
 * and a right position (contracted); anything else is ierr 6. */
int a4o_get_contraction_ptrn(int drank, int lrank, int rrank, const int* aces_ptrn, int* my_ptrn) {
  if (!(drank >= 0 && lrank >= 0 && rrank >= 0)) return 1;
  const int m = lrank + rrank, n = drank + m;
  if (n % 2 != 0) return 2;
  if (m <= 0) return drank > 0 ? 3 : 0;
  if (n > 3 * A4O_MAX_RANK) return 1;
  /* the distinct labels in ascending order, each with its use count */
  int below = 0, started = 0; /* every label <= below has been visited */
  for (;;) {
    int next = 0, found = 0;
    for (int i = 0; i < n; ++i)
      if ((!started || aces_ptrn[i] > below) && (!found || aces_ptrn[i] < next)) next = aces_ptrn[i], found = 1;
    if (!found) break;
    int count = 0;
    for (int i = 0; i < n; ++i) count += aces_ptrn[i] == next;
    if (count == 1 || count == 3) return 4;
    if (count >= 4) return 5;
    below = next, started = 1;
  }
  /* every label is used exactly twice: classify each pair of positions */
  for (int p = 0; p < n; ++p) {
    int q = -1;
    for (int t = p + 1; t < n; ++t)
      if (aces_ptrn[t] == aces_ptrn[p]) q = t;
    if (q < 0) continue; /* p is the second use of its label */
    const int p_in_d = p < drank, p_in_l = p >= drank && p < drank + lrank;
    const int q_in_d = q < drank, q_in_r = q >= drank + lrank;
    if (p_in_d && !q_in_d) {
      my_ptrn[q - drank] = p + 1;
    } else if (p_in_l && q_in_r) {
      my_ptrn[p - drank] = -(q - drank - lrank + 1);
      my_ptrn[q - drank] = -(p - drank + 1);
    } else {
      return 6;
    }
  }
  return 0;
}

/* contr_ptrn_ok (tensor_dil_omp.F90:861-896).  Returns 1 when valid. */
int a4o_contr_ptrn_ok(const int* ptrn, int lr, int rr, int dr, const int* lext, const int* rext,
                      const int* dext) {
  const int jl = dr + lr + rr;
  if (jl <= 0) return 1;
  int jbus[3 * A4O_MAX_RANK + 2];
  memset(jbus, 0, sizeof(jbus));
  for (int j0 = 1; j0 <= lr; ++j0) {
    const int j1 = ptrn[j0 - 1];
    if (j1 > 0 && j1 <= dr) {
      jbus[j1 - 1]++;
      jbus[dr + j0 - 1]++;
      if (lext[j0 - 1] != dext[j1 - 1]) return 0;
    } else if (j1 < 0 && -j1 <= rr) {
      jbus[dr + lr - j1 - 1]++;
      if (lext[j0 - 1] != rext[-j1 - 1]) return 0;
    } else {
      return 0;
    }
  }
  for (int j0 = lr + 1; j0 <= lr + rr; ++j0) {
    const int j1 = ptrn[j0 - 1];
    if (j1 > 0 && j1 <= dr) {
      jbus[j1 - 1]++;
      jbus[dr + j0 - 1]++;
      if (rext[j0 - lr - 1] != dext[j1 - 1]) return 0;
    } else if (j1 < 0 && -j1 <= lr) {
      jbus[dr - j1 - 1]++;
      if (rext[j0 - lr - 1] != lext[-j1 - 1]) return 0;
    } else {
      return 0;
    }
  }
  for (int j0 = 0; j0 < jl; ++j0)
    if (jbus[j0] != 1) return 0;
  return 1;
}

/* tensor_block_copy_ (tensor_dil_omp.F90:438-660): out = permute(in).
 * dim_transp[0] is the sign slot, dim_transp[1..dim_num] the 1-based O2N
 * permutation: input dimension i becomes output dimension dim_transp[i].
 * The reference's cache blocking only changes the visiting order, not the
 * result, so a plain multi-index walk is used (threaded like the original). */
int a4o_tensor_block_copy(int dim_num, const int* dim_extents, const int* dim_transp,
                          const double* tens_in, double* tens_out) {
  if (dim_num < 0) return dim_num;
  if (dim_num == 0) {
    tens_out[0] = tens_in[0];
    return 0;
  }
  int64_t bases_out[A4O_MAX_RANK];
  int n2o[A4O_MAX_RANK + 1];
  int64_t bs = 1;
  for (int i = 0; i < dim_num; ++i) bs *= dim_extents[i];
  for (int i = 1; i <= dim_num; ++i) n2o[dim_transp[i]] = i;
  int64_t bo = 1;
  for (int i = 1; i <= dim_num; ++i) {
    bases_out[n2o[i] - 1] = bo;
    bo *= dim_extents[n2o[i] - 1];
  }
  const int64_t total = bs;
#pragma omp parallel
  {
    int64_t lo = 0, hi = total;
#ifdef _OPENMP
    const int nt = omp_get_num_threads(), tid = omp_get_thread_num();
    lo = total * tid / nt;
    hi = total * (tid + 1) / nt;
#endif
    if (lo < hi) {
      int im[A4O_MAX_RANK];
      int64_t rem = lo, l_out = 0;
      for (int i = 0; i < dim_num; ++i) {
        im[i] = (int)(rem % dim_extents[i]);
        rem /= dim_extents[i];
        l_out += im[i] * bases_out[i];
      }
      for (int64_t l_in = lo; l_in < hi; ++l_in) {
        tens_out[l_out] = tens_in[l_in];
        for (int i = 0; i < dim_num; ++i) {
          if (im[i] + 1 < dim_extents[i]) {
            im[i]++;
            l_out += bases_out[i];
            break;
          }
          l_out -= (int64_t)im[i] * bases_out[i];
          im[i] = 0;
        }
      }
    }
  }
  return 0;
}

/* determine_index_permutations (tensor_dil_omp.F90:799-859).  Produces the
 * O2N permutations (sign slot at [0]) that bring the operands to matrix form:
 * left = [contracted (in right's order), uncontracted], right = [contracted,
 * uncontracted], destination matrix = [left uncontracted, right uncontracted]. */
typedef struct {
  int lo2n[A4O_MAX_RANK + 1], ro2n[A4O_MAX_RANK + 1], do2n[A4O_MAX_RANK + 1];
  int ltransp, rtransp, dtransp;
  int64_t lld, lrd, lcd, lsize, rsize, dsize;
} plan_t;

static int perm_trivial(int ni, const int* trn) {
  for (int j = 1; j <= ni; ++j)
    if (trn[j] != j) return 0;
  return 1;
}

static void determine_index_permutations(const int* ptrn, int lrank, const int* lext, int rrank,
                                         const int* rext, int drank, const int* dext, plan_t* p) {
  p->lld = p->lrd = p->lcd = 1;
  p->dsize = 1;
  p->ltransp = p->rtransp = p->dtransp = 0;
  if (drank > 0) {
    for (int j = 0; j < drank; ++j) p->dsize *= dext[j];
    p->do2n[0] = 1;
    int j1 = 0;
    for (int j0 = 0; j0 < lrank + rrank; ++j0)
      if (ptrn[j0] > 0) p->do2n[++j1] = ptrn[j0];
    p->dtransp = !perm_trivial(j1, p->do2n);
  }
  p->rsize = 1;
  if (rrank > 0) {
    for (int j = 0; j < rrank; ++j) p->rsize *= rext[j];
    p->ro2n[0] = 1;
    int j1 = 0;
    for (int j0 = 1; j0 <= rrank; ++j0)
      if (ptrn[lrank + j0 - 1] < 0) {
        p->ro2n[j0] = ++j1;
        p->lcd *= rext[j0 - 1];
      }
    for (int j0 = 1; j0 <= rrank; ++j0)
      if (ptrn[lrank + j0 - 1] > 0) {
        p->ro2n[j0] = ++j1;
        p->lrd *= rext[j0 - 1];
      }
    p->rtransp = !perm_trivial(j1, p->ro2n);
  }
  p->lsize = 1;
  if (lrank > 0) {
    for (int j = 0; j < lrank; ++j) p->lsize *= lext[j];
    p->lo2n[0] = 1;
    int jtrn1[A4O_MAX_RANK + 1], jkey[A4O_MAX_RANK + 1], jtrn0[A4O_MAX_RANK + 1];
    int j1 = 0;
    for (int j0 = 1; j0 <= lrank; ++j0)
      if (ptrn[j0 - 1] < 0) {
        ++j1;
        jtrn1[j1] = j0;
        jkey[j1 - 1] = -ptrn[j0 - 1];
      }
    for (int j = 0; j < j1; ++j) jtrn0[j] = j + 1;
    stable_sort_by_key(j1, jkey, jtrn0);
    for (int j0 = 1; j0 <= j1; ++j0) p->lo2n[jtrn1[jtrn0[j0 - 1]]] = j0;
    for (int j0 = 1; j0 <= lrank; ++j0)
      if (ptrn[j0 - 1] > 0) {
        p->lo2n[j0] = ++j1;
        p->lld *= lext[j0 - 1];
      }
    p->ltransp = !perm_trivial(j1, p->lo2n);
  }
}

/* tensor_block_add_ (tensor_dil_omp.F90:394-436): tens0 += tens1*scale_fac,
 * where a factor within 1e-13 of one is treated as exactly one. */
int a4o_tensor_block_add(int dim_num, const int* ext, double* tens0, const double* tens1,
                         double scale_fac) {
  if (dim_num == 0) {
    tens0[0] = tens0[0] + tens1[0] * scale_fac;
    return 0;
  }
  if (dim_num < 0) return -1;
  int64_t n = 1;
  for (int i = 0; i < dim_num; ++i) n *= ext[i];
  if (fabs(scale_fac - 1.0) > 1e-13) {
#pragma omp parallel for schedule(static)
    for (int64_t l = 0; l < n; ++l) tens0[l] = tens0[l] + tens1[l] * scale_fac;
  } else {
#pragma omp parallel for schedule(static)
    for (int64_t l = 0; l < n; ++l) tens0[l] = tens0[l] + tens1[l];
  }
  return 0;
}

/* Naive matrix form of tensor_block_pcontract (tensor_dil_omp.F90:940-1179):
 * d(l1,l2) += sum_l0 l(l0,l1) * r(l0,l2), the dot product taken in l0 order. */
static void gemm_tn_naive(int64_t dl, int64_t dr, int64_t dc, const double* l, const double* r,
                          double* d) {
#pragma omp parallel for collapse(2) schedule(static)
  for (int64_t l2 = 0; l2 < dr; ++l2)
    for (int64_t l1 = 0; l1 < dl; ++l1) {
      double val = d[l2 * dl + l1];
      const double* lp = l + l1 * dc;
      const double* rp = r + l2 * dc;
      for (int64_t l0 = 0; l0 < dc; ++l0) val = val + lp[l0] * rp[l0];
      d[l2 * dl + l1] = val;
    }
}

/* tensor_block_contract_ (tensor_dil_omp.F90:662-797).  The destination is
 * OVERWRITTEN (the reference zeroes it before the product, F90:752,769,777). */
int a4o_tensor_block_contract_ex(const int* contr_ptrn, const double* ltens, int lrank,
                                 const int* lext, const double* rtens, int rrank, const int* rext,
                                 double* dtens, int drank, const int* dext, a4o_gemm_tn_fn gemm,
                                 void* ctx, int nthreads) {
  (void)nthreads;
  if (!(lrank >= 0 && lrank <= A4O_MAX_RANK && rrank >= 0 && rrank <= A4O_MAX_RANK && drank >= 0 &&
        drank <= A4O_MAX_RANK))
    return -1;
  if (!a4o_contr_ptrn_ok(contr_ptrn, lrank, rrank, drank, lext, rext, dext)) return 1;
  plan_t p;
  determine_index_permutations(contr_ptrn, lrank, lext, rrank, rext, drank, dext, &p);
  double *ltp = (double*)ltens, *rtp = (double*)rtens, *dtp = dtens;
  int ierr = 0;
  if (p.ltransp) {
    ltp = (double*)malloc(sizeof(double) * p.lsize);
    if (!ltp) return 1;
    ierr = a4o_tensor_block_copy(lrank, lext, p.lo2n, ltens, ltp);
  }
  if (!ierr && p.rtransp) {
    rtp = (double*)malloc(sizeof(double) * p.rsize);
    if (!rtp) ierr = 1;
    else ierr = a4o_tensor_block_copy(rrank, rext, p.ro2n, rtens, rtp);
  }
  if (!ierr && p.dtransp) {
    dtp = (double*)malloc(sizeof(double) * p.dsize);
    if (!dtp) ierr = 1;
  }
  if (!ierr) {
    for (int64_t k = 0; k < p.dsize; ++k) dtp[k] = 0.0;
    if (drank > 0 && lrank > 0 && rrank > 0) {
      if (gemm)
        gemm(p.lld, p.lrd, p.lcd, ltp, p.lcd, rtp, p.lcd, dtp, p.lld, ctx);
      else
        gemm_tn_naive(p.lld, p.lrd, p.lcd, ltp, rtp, dtp);
    } else if (drank == 0 && lrank > 0 && rrank > 0) {
      /* tensor_block_fcontract (F90:910-938): dtens += sum l*r */
      dtp[0] = 0.0;
      double val = 0.0;
      for (int64_t l0 = 0; l0 < p.lcd; ++l0) val = val + ltp[l0] * rtp[l0];
      dtp[0] = dtp[0] + val;
    } else if (drank > 0 && lrank > 0 && rrank == 0) {
      ierr = a4o_tensor_block_add(drank, dext, dtp, ltp, rtp[0]);
    } else if (drank > 0 && lrank == 0 && rrank > 0) {
      ierr = a4o_tensor_block_add(drank, dext, dtp, rtp, ltp[0]);
    } else if (drank == 0 && lrank == 0 && rrank == 0) {
      dtp[0] = ltp[0] * rtp[0];
    }
  }
  if (!ierr && p.dtransp) {
    int mext[A4O_MAX_RANK];
    for (int k = 1; k <= drank; ++k) mext[k - 1] = dext[p.do2n[k] - 1];
    ierr = a4o_tensor_block_copy(drank, mext, p.do2n, dtp, dtens);
  }
  if (p.ltransp) free(ltp);
  if (p.rtransp && rtp) free(rtp);
  if (p.dtransp && dtp) free(dtp);
  return ierr;
}

int a4o_tensor_block_contract(const int* contr_ptrn, const double* ltens, int lrank, const int* lext,
                              const double* rtens, int rrank, const int* rext, double* dtens,
                              int drank, const int* dext) {
  return a4o_tensor_block_contract_ex(contr_ptrn, ltens, lrank, lext, rtens, rrank, rext, dtens,
                                      drank, dext, NULL, NULL, 1);
}

/* tensor_block_init_ (F90:144-191): tens = sval. */
int a4o_tensor_block_init(double* tens, int rank, const int* ext, double sval) {
  if (rank == 0) {
    tens[0] = sval;
    return 0;
  }
  if (rank < 0) return -1;
  int64_t n = 1;
  for (int i = 0; i < rank; ++i) n *= ext[i];
  for (int64_t l = 0; l < n; ++l) tens[l] = sval;
  return 0;
}

/* tensor_block_scale_ (F90:193-228): tens *= scale_fac. */
int a4o_tensor_block_scale(double* tens, int rank, const int* ext, double scale_fac) {
  if (rank == 0) {
    tens[0] = tens[0] * scale_fac;
    return 0;
  }
  if (rank < 0) return -1;
  int64_t n = 1;
  for (int i = 0; i < rank; ++i) n *= ext[i];
  for (int64_t l = 0; l < n; ++l) tens[l] = tens[l] * scale_fac;
  return 0;
}

/* tensor_block_norm2_ (F90:230-269): sum of squares (taken in element order
 * here; the reference's OpenMP reduction order is unspecified). */
double a4o_tensor_block_norm2(const double* tens, int rank, const int* ext, int* ierr) {
  *ierr = 0;
  if (rank == 0) return tens[0] * tens[0];
  if (rank < 0) {
    *ierr = -1;
    return 0.0;
  }
  int64_t n = 1;
  for (int i = 0; i < rank; ++i) n *= ext[i];
  double val = 0.0;
  for (int64_t l = 0; l < n; ++l) val = val + tens[l] * tens[l];
  return val;
}

/* tensor_block_slice_ (F90:271-330): slice = tens[ext_beg : ext_beg+slice_ext]. */
int a4o_tensor_block_slice(int dim_num, const double* tens, const int* tens_ext, double* slice,
                           const int* slice_ext, const int* ext_beg) {
  if (dim_num == 0) {
    slice[0] = tens[0];
    return 0;
  }
  if (dim_num < 0) return 1;
  int64_t bases_in[A4O_MAX_RANK], n = 1, b = 1;
  for (int i = 0; i < dim_num; ++i) {
    bases_in[i] = b;
    b *= tens_ext[i];
    n *= slice_ext[i];
  }
  int im[A4O_MAX_RANK] = {0};
  for (int64_t l_out = 0; l_out < n; ++l_out) {
    int64_t l_in = 0;
    for (int i = 0; i < dim_num; ++i) l_in += (int64_t)(ext_beg[i] + im[i]) * bases_in[i];
    slice[l_out] = tens[l_in];
    for (int i = 0; i < dim_num; ++i) {
      if (im[i] + 1 < slice_ext[i]) {
        im[i]++;
        break;
      }
      im[i] = 0;
    }
  }
  return 0;
}

/* tensor_block_insert_ (F90:332-392): tens[ext_beg : ext_beg+slice_ext] = slice. */
int a4o_tensor_block_insert(int dim_num, double* tens, const int* tens_ext, const double* slice,
                            const int* slice_ext, const int* ext_beg) {
  if (dim_num == 0) {
    tens[0] = slice[0];
    return 0;
  }
  if (dim_num < 0) return 1;
  int64_t bases_out[A4O_MAX_RANK], n = 1, b = 1;
  for (int i = 0; i < dim_num; ++i) {
    bases_out[i] = b;
    b *= tens_ext[i];
    n *= slice_ext[i];
  }
  int im[A4O_MAX_RANK] = {0};
  for (int64_t l_in = 0; l_in < n; ++l_in) {
    int64_t l_out = 0;
    for (int i = 0; i < dim_num; ++i) l_out += (int64_t)(ext_beg[i] + im[i]) * bases_out[i];
    tens[l_out] = slice[l_in];
    for (int i = 0; i < dim_num; ++i) {
      if (im[i] + 1 < slice_ext[i]) {
        im[i]++;
        break;
      }
      im[i] = 0;
    }
  }
  return 0;
}

/* Block::fill / scale / scale_and_copy / increment_elements / accumulate_data
 * (src/sip/dynamic_data/block.cpp:153-270). */
void a4o_block_fill(double* d, int64_t n, double value) {
  for (int64_t i = 0; i < n; ++i) d[i] = value;
}
void a4o_block_scale(double* d, int64_t n, double factor) {
  for (int64_t i = 0; i < n; ++i) d[i] *= factor;
}
void a4o_block_scale_and_copy(double* d, const double* s, int64_t n, double factor) {
  for (int64_t i = 0; i < n; ++i) d[i] = s[i] * factor;
}
void a4o_block_increment(double* d, int64_t n, double delta) {
  for (int64_t i = 0; i < n; ++i) d[i] += delta;
}
void a4o_block_accumulate(double* d, const double* s, int64_t n) {
  for (int64_t i = 0; i < n; ++i) d[i] += s[i];
}

/* Interpreter::handle_block_add / handle_block_subtract
 * (src/sip/worker/interpreter.cpp:1874-1997) with permute_rhs_to_lhs
 * (:2049-2084).  d = l +/- r.  When d is the same block as l (the "+=" form)
 * r is first permuted into d's index order; otherwise l, r and d must carry the
 * same index labels.  Returns 0, or 2 for incompatible labels (the reference
 * aborts there). */
int a4o_block_add_sub(int subtract, int rank, const int* d_ids, const int* l_ids, const int* r_ids,
                      const int* r_ext, int d_is_l, double* d, const double* l, const double* r) {
  int64_t n = 1;
  for (int i = 0; i < rank; ++i) n *= r_ext[i];
  const double* rd = r;
  double* tmp = NULL;
  if (!d_is_l) {
    for (int i = 0; i < rank; ++i)
      if (l_ids[i] != r_ids[i] || r_ids[i] != d_ids[i]) return 2;
  } else {
    int perm[A4O_MAX_RANK + 1];
    perm[0] = 1;
    for (int i = 0; i < rank; ++i) {
      int j = 0;
      while (j < rank && r_ids[j] != d_ids[i]) ++j;
      if (j >= rank) return 2;
      perm[j + 1] = i + 1;
    }
    tmp = (double*)malloc(sizeof(double) * (n ? n : 1));
    if (!tmp) return 1;
    a4o_tensor_block_copy(rank, r_ext, perm, r, tmp);
    rd = tmp;
  }
  if (subtract)
    for (int64_t i = 0; i < n; ++i) d[i] = l[i] - rd[i];
  else
    for (int64_t i = 0; i < n; ++i) d[i] = l[i] + rd[i];
  free(tmp);
  return 0;
}

/* energy_denominator_rhf (src/sip/super_instructions/qm/qm-generic/
 * energy_denominator_rhf.F:15-447).  In place: data0 /= eps with
 *   rank 2: eps = e_b - e_a                                  (do_rhf_den2 :241)
 *   rank 4: eps = e_b + e_d - e_a - e_c                      (do_rhf_den4 :310)
 *   rank 6: eps = e_b + e_d + e_f - e_a - e_c - e_e          (do_rhf_den6 :399)
 * evaluated left to right.  Orbital energies are the diagonal of the 2-D
 * Fock block (rank1 == 2) or a 1-D vector (rank1 == 1; ranks 2 and 4 only).
 * index_values0 are 1-based segment numbers; the absolute orbital offset of
 * dimension q is the sum of seg_sizes before its segment, except for rank 6
 * where an extent of 1 marks a simple index whose offset is value-1. */
int a4o_energy_denominator_rhf(int rank0, const int* index_values0, const int* extents0,
                               double* data0, int rank1, const int* extents1, const double* data1,
                               int nsegs, const int* seg_sizes) {
  if (!(rank0 == 2 || rank0 == 4 || rank0 == 6)) return 0; /* reference does nothing */
  if (!(rank1 == 1 || rank1 == 2)) return 0;
  if (rank0 == 6 && rank1 != 2) return 0;
  int off[6];
  for (int q = 0; q < rank0; ++q) {
    off[q] = 0;
    if (rank0 == 6 && extents0[q] == 1) {
      off[q] = index_values0[q] - 1;
    } else {
      for (int i = 1; i <= index_values0[q] - 1; ++i) {
        if (i > nsegs) return 3;
        off[q] += seg_sizes[i - 1];
      }
    }
  }
  const int ld = extents1[0];
#define EPS_AT(p) (rank1 == 2 ? data1[(int64_t)(p) + (int64_t)(p)*ld] : data1[(p)])
  int e[6] = {1, 1, 1, 1, 1, 1};
  for (int q = 0; q < rank0; ++q) e[q] = extents0[q];
  int64_t idx = 0;
  for (int f = 0; f < (rank0 == 6 ? e[5] : 1); ++f)
    for (int ee = 0; ee < (rank0 == 6 ? e[4] : 1); ++ee)
      for (int d = 0; d < (rank0 >= 4 ? e[3] : 1); ++d)
        for (int c = 0; c < (rank0 >= 4 ? e[2] : 1); ++c)
          for (int b = 0; b < e[1]; ++b)
            for (int a = 0; a < e[0]; ++a) {
              double eps;
              const double ea = EPS_AT(a + off[0]);
              const double eb = EPS_AT(b + off[1]);
              if (rank0 == 2) {
                eps = eb - ea;
              } else if (rank0 == 4) {
                const double ec = EPS_AT(c + off[2]);
                const double ed = EPS_AT(d + off[3]);
                eps = eb + ed - ea - ec;
              } else {
                const double ec = EPS_AT(c + off[2]);
                const double ed = EPS_AT(d + off[3]);
                const double e5 = EPS_AT(ee + off[4]);
                const double e6 = EPS_AT(f + off[5]);
                eps = eb + ed + e6 - ea - ec - e5;
              }
              data0[idx] = data0[idx] / eps;
              ++idx;
            }
#undef EPS_AT
  return 0;
}

/* fill_block_cyclic (src/sip/super_instructions/qm/tests/fill_block_cyclic.f:23-60):
 * x, x+1, ... ; after writing 20 the running value restarts at 1.  The
 * running value is single precision in the reference; all values are small
 * integers, so double arithmetic gives the same numbers. */
void a4o_fill_block_cyclic(double* d, int64_t n, double start) {
  float val = (float)start;
  for (int64_t i = 0; i < n; ++i) {
    d[i] = val;
    if (val == 20.0f) val = 0.0f;
    val = val + 1.0f;
  }
}

/* fill_block_sequential (fill_block_sequential.f:24-60): x, x+1, x+2, ... */
void a4o_fill_block_sequential(double* d, int64_t n, double start) {
  float val = (float)start;
  for (int64_t i = 0; i < n; ++i) {
    d[i] = val;
    val = val + 1.0f;
  }
}
