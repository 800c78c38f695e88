/*
 * CPU oracle for the ACES4 block-contraction path.
 *
 * TEST INFRASTRUCTURE ONLY.  This is a plain-C restatement of the reference
 * algorithms (tensor_dil_omp.F90, block.cpp, interpreter.cpp handlers,
 * energy_denominator_rhf.F).  Only tests/, __graft_entry__.smoke() and the
 * CPU-baseline leg of bench.py may load it, and only to check results against
 * or as the timed CPU baseline.  The product library never links or calls it.
 *
 * Conventions follow the reference exactly: blocks are column-major (first
 * index fastest), extents are 32-bit ints, permutations are 1-based O2N
 * vectors with a sign slot at position 0, and every routine reports an
 * integer error code (0 = success) with the reference's values.
 */
#ifndef A4_ORACLE_H
#define A4_ORACLE_H
#include <stdint.h>
#ifdef __cplusplus
extern "C" {
#endif

#define A4O_MAX_RANK 32 /* tensor_dil_omp.F90:58 max_tensor_rank */

int64_t a4o_tensor_size_by_shape(int num_dim, const int* dims, int* ierr);
int a4o_get_contraction_ptrn(int drank, int lrank, int rrank, const int* aces_ptrn, int* my_ptrn);
int a4o_contr_ptrn_ok(const int* ptrn, int lr, int rr, int dr, const int* lext, const int* rext,
                      const int* dext);
int a4o_tensor_block_copy(int dim_num, const int* dim_extents, const int* dim_transp,
                          const double* tens_in, double* tens_out);
int a4o_tensor_block_contract(const int* contr_ptrn, const double* ltens, int lrank, const int* lext,
                              const double* rtens, int rrank, const int* rext, double* dtens,
                              int drank, const int* dext);
int a4o_tensor_block_init(double* tens, int rank, const int* ext, double sval);
int a4o_tensor_block_scale(double* tens, int rank, const int* ext, double scale_fac);
double a4o_tensor_block_norm2(const double* tens, int rank, const int* ext, int* ierr);
int a4o_tensor_block_add(int dim_num, const int* ext, double* tens0, const double* tens1,
                         double scale_fac);
int a4o_tensor_block_slice(int dim_num, const double* tens, const int* tens_ext, double* slice,
                           const int* slice_ext, const int* ext_beg);
int a4o_tensor_block_insert(int dim_num, double* tens, const int* tens_ext, const double* slice,
                            const int* slice_ext, const int* ext_beg);

/* Block / interpreter-level element-wise operations. */
void a4o_block_fill(double* d, int64_t n, double value);
void a4o_block_scale(double* d, int64_t n, double factor);
void a4o_block_scale_and_copy(double* d, const double* s, int64_t n, double factor);
void a4o_block_increment(double* d, int64_t n, double delta);
void a4o_block_accumulate(double* d, const double* s, int64_t n);
int a4o_block_add_sub(int subtract, int rank, const int* d_ids, const int* l_ids, const int* r_ids,
                      const int* r_ext, int d_is_l, double* d, const double* l, const double* r);

/* Super instruction energy_denominator_rhf. */
int a4o_energy_denominator_rhf(int rank0, const int* index_values0, const int* extents0,
                               double* data0, int rank1, const int* extents1, const double* data1,
                               int nsegs, const int* seg_sizes);

/* Fill super instructions used by the reference's known-answer tests. */
void a4o_fill_block_cyclic(double* d, int64_t n, double start);
void a4o_fill_block_sequential(double* d, int64_t n, double start);

/* Whole-contraction helper used as the CPU baseline: matrix form of
 * tensor_block_contract__ with the operand permutes and a caller-supplied
 * GEMM (NULL = the naive loop of tensor_block_pcontract). */
typedef void (*a4o_gemm_tn_fn)(int64_t m, int64_t n, int64_t k, const double* a, int64_t lda,
                               const double* b, int64_t ldb, double* c, int64_t ldc, void* ctx);
int a4o_tensor_block_contract_ex(const int* contr_ptrn, const double* ltens, int lrank,
                                 const int* lext, const double* rtens, int rrank, const int* rext,
                                 double* dtens, int drank, const int* dext, a4o_gemm_tn_fn gemm,
                                 void* ctx, int nthreads);

#ifdef __cplusplus
}
#endif
#endif
