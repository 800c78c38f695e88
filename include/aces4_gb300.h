/*
 * aces4_gb300 — GB300 (sm_103a) implementation of the ACES4 SIP block-contraction path.
 *
 * C ABI.  Plain pointers and sizes only.  Three groups of entry points:
 *
 *  1. Drop-in replacements for the reference's Fortran kernels
 *     (src/sip/tensor_algebra/tensor_ops_c_prototypes.h).  Same symbol names,
 *     same argument meaning, HOST buffers, synchronous, same ierr values.  The
 *     reference declares scalars as C++ references (int&); a reference and a
 *     pointer have the same calling convention, so the reference's own header
 *     links against these definitions unchanged.
 *  2. Drop-in replacements for the reference's legacy GPU API
 *     (src/sip/cuda/gpu_super_instructions.h), DEVICE buffers.  The reference
 *     exits the process on a CUDA error; these record the error (a4g_last_error)
 *     and return instead.
 *  3. New a4g_* entry points: device-resident, stream-ordered block operations,
 *     the batched (one pardo step per call) contraction, and the split-precision
 *     (Ozaki, BF16 tensor-core) contraction.  Every a4g_* call returns an int
 *     status (A4G_OK = 0) and never exits or traps.
 *
 * Data layout everywhere: a block is a dense column-major array of doubles
 * (first index fastest) whose extents are the segment sizes of its indices
 * (reference: src/sip/dynamic_data/block_shape.cpp:25-49).  Rank <= 32 for the
 * Fortran-compatible entries (tensor_dil_omp.F90:58), <= 6 for SIAL blocks.
 */
#ifndef ACES4_GB300_H
#define ACES4_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ----------------------------------------------------------------------------
 * Status codes of the a4g_* API
 * ------------------------------------------------------------------------- */
#define A4G_OK 0
#define A4G_ERR_ARG 1        /* invalid argument (rank, extent, pattern, null pointer)        */
#define A4G_ERR_PATTERN 2    /* contraction pattern rejected (reference ierr 1)               */
#define A4G_ERR_CUDA 3       /* a CUDA runtime/driver call failed                             */
#define A4G_ERR_NOMEM 4      /* device or host allocation failed                              */
#define A4G_ERR_TIMEOUT 5    /* a device-side wait hit its iteration limit; kernel bailed out */
#define A4G_ERR_UNSUPPORTED 6
#define A4G_ERR_RANGE 7      /* size beyond a documented maximum                              */
#define A4G_ERR_PRECISION 8  /* a certified error bound exceeds the requested target           */

/* Drop-ins on host blocks (group 1 and energy_denominator_rhf): where the GPU
 * reads and writes pageable host memory through the host's page tables
 * (Grace-Blackwell; cudaDevAttrPageableMemoryAccessUsesHostPageTables), the
 * kernels run on the caller's host blocks in place, with no copies; elsewhere
 * (or after a4g_host_direct(0)) the blocks are staged through device memory.
 * The results and the synchronous return are the same either way.  Returns
 * A4G_ERR_UNSUPPORTED when the GPU cannot access host memory (staging then). */
int a4g_host_direct(int enable);

/* Text of the last error on the calling thread ("" when none). */
const char* a4g_last_error(void);
/* Forget the recorded error (the legacy _gpu_* calls record failures and
 * never clear them, so a host checks a sequence of calls with one read). */
void a4g_clear_error(void);
/* Library version string. */
const char* a4g_version(void);

/* ============================================================================
 * 1. Drop-in replacements: src/sip/tensor_algebra/tensor_ops_c_prototypes.h
 *    (HOST buffers; each call copies to the GPU, computes there, copies back)
 * ========================================================================= */

/* tensor_ops_c_prototypes.h:42 / tensor_dil_omp.F90:66 */
long long tensor_size_by_shape_(int* num_dim, int* dims, int* ierr);
/* tensor_ops_c_prototypes.h:55 / tensor_dil_omp.F90:87.  Host-only integer work. */
void get_contraction_ptrn_(int* drank, int* lrank, int* rrank, int* aces_ptrn, int* my_ptrn,
                           int* ierr);
/* tensor_ops_c_prototypes.h:70 / tensor_dil_omp.F90:144 */
void tensor_block_init__(int* nthreads, double* tens, int* tens_rank, int* tens_dim_extents,
                         double* sval, int* ierr);
/* tensor_ops_c_prototypes.h:84 / tensor_dil_omp.F90:193 */
void tensor_block_scale__(int* nthreads, double* tens, int* tens_rank, int* tens_dim_extents,
                          double* scale_fac, int* ierr);
/* tensor_ops_c_prototypes.h:86 / tensor_dil_omp.F90:230 */
double tensor_block_norm2__(int* nthreads, double* tens, int* tens_rank, int* tens_dim_extents,
                            int* ierr);
/* tensor_ops_c_prototypes.h:101 / tensor_dil_omp.F90:271 */
void tensor_block_slice__(int* nthreads, int* dim_num, double* tens, int* tens_ext, double* slice,
                          int* slice_ext, int* ext_beg, int* ierr);
/* tensor_ops_c_prototypes.h:117 / tensor_dil_omp.F90:332 */
void tensor_block_insert__(int* nthreads, int* dim_num, double* tens, int* tens_ext, double* slice,
                           int* slice_ext, int* ext_beg, int* ierr);
/* tensor_ops_c_prototypes.h:133 / tensor_dil_omp.F90:394  (tens0 += tens1*scale_fac) */
void tensor_block_add__(const int* nthreads, const int* dim_num, int* dim_extents, double* tens0,
                        double* tens1, const double* scale_fac, int* ierr);
/* tensor_ops_c_prototypes.h:152 / tensor_dil_omp.F90:438  (dim_transp: sign slot + 1-based O2N) */
void tensor_block_copy__(int* nthreads, int* dim_num, int* dim_extents, int* dim_transp,
                         double* tens_in, double* tens_out, int* ierr);
/* tensor_ops_c_prototypes.h:178 / tensor_dil_omp.F90:662.  D is OVERWRITTEN. */
void tensor_block_contract__(int* nthreads, int* contr_ptrn, double* ltens, int* ltens_num_dim,
                             int* ltens_dim_extent, double* rtens, int* rtens_num_dim,
                             int* rtens_dim_extent, double* dtens, int* dtens_num_dim,
                             int* dtens_dim_extent, int* ierr);

/* ============================================================================
 * 2. Drop-in replacements: src/sip/cuda/gpu_super_instructions.h:26-126
 *    (DEVICE buffers; synchronous like the reference)
 * ========================================================================= */
void _init_gpu(int* devid, int* myRank);                                         /* .h:26  */
void _gpu_axpy(double* y, double* x, const double alpha, const int numElems);   /* .h:35  */
void _gpu_double_memset(double* g_addr, double value, const int numElems);      /* .h:44  */
void _gpu_selfmultiply(double* x, const double alpha, const int numElems);      /* .h:53  */
/* .h:70: y = x1 * x2, indices given as labels (overwrite, like the reference) */
void _gpu_contract(double* y, const int ny, const int* yDims, const int* yInds, double* x1,
                   const int n1, const int* x1Dims, const int* x1Inds, double* x2, const int n2,
                   const int* x2Dims, const int* x2Inds);
/* .h:86: y = x with the index order given by the labels */
void _gpu_permute(double* y, const int ny, const int* yDims, const int* yInds, double* x,
                  const int nx, const int* xDims, const int* xInds);
void _gpu_host_to_device(double* c_addr, double* g_addr, const int numElems);   /* .h:96  */
double* _gpu_allocate(const int numElems);                                       /* .h:103 */
void _gpu_device_to_host(double* c_addr, double* g_addr, const int numElems);   /* .h:111 */
void _gpu_device_to_device(double* dst, double* src, const int numElems);       /* .h:120 */
void _gpu_free(double* g_addr);                                                  /* .h:126 */

/* ============================================================================
 * Super instruction: energy_denominator_rhf
 * (src/sip/super_instructions/qm/qm-generic/energy_denominator_rhf.F:15, the
 *  "fp2" ABI of src/sip/super_instructions/special_instructions.h:73-74).
 * data_0 (HOST, the amplitude block) is divided in place by orbital-energy
 * denominators read from data_1 (2-D Fock block: its diagonal; or 1-D energies).
 * The segment sizes come from the predefined integer array "moa_seg_ranges",
 * registered with a4g_set_predefined_int_array (sip_interface.h:17-48 role).
 * ========================================================================= */
void energy_denominator_rhf(int* array_slot_0, int* rank_0, int* index_values_0, int* size_0,
                            int* extents_0, double* data_0, int* array_slot_1, int* rank_1,
                            int* index_values_1, int* size_1, int* extents_1, double* data_1,
                            int* ierr);
/* Registers (copies) a predefined integer array by name, e.g. "moa_seg_ranges". */
int a4g_set_predefined_int_array(const char* name, int n, const int* values);

/* ============================================================================
 * 3. Device-resident API (a4g_*).  All pointers are device pointers unless
 *    named h_*; `stream` is a cudaStream_t (NULL = the library's own stream).
 *    Calls are asynchronous on `stream`; a4g_sync(stream) waits and reports
 *    any device-side error flag.
 * ========================================================================= */
int a4g_init(int device);
int a4g_sync(void* stream);
void* a4g_default_stream(void);

/* Contraction of two blocks, reference pattern format (get_contraction_ptrn_).
 * beta = 0: D = L*R (reference overwrite semantics, tensor_dil_omp.F90:752);
 * beta = 1: D += L*R (the contract-accumulate the interpreter lacks,
 * src/sip/worker/interpreter.cpp:743-747).  Plain FP64 on the GPU (DMMA). */
int a4g_contract(const int* contr_ptrn, const double* l, int lrank, const int* lext,
                 const double* r, int rrank, const int* rext, double* d, int drank,
                 const int* dext, int beta, void* stream);
/* Same, indices given as labels like the interpreter's selectors
 * (src/sip/worker/interpreter.cpp:1210-1262). */
int a4g_contract_labels(const int* d_labels, const int* l_labels, const int* r_labels,
                        const double* l, int lrank, const int* lext, const double* r, int rrank,
                        const int* rext, double* d, int drank, const int* dext, int beta,
                        void* stream);
/* tensor_block_copy: out = permute(in), dim_transp = sign slot + 1-based O2N. */
int a4g_permute(int rank, const int* ext, const int* dim_transp, const double* in, double* out,
                void* stream);
/* Element-wise ops on n doubles (block.cpp:153-270, tensor_dil_omp.F90:144-436). */
int a4g_fill(double* d, int64_t n, double value, void* stream);
int a4g_scale(double* d, int64_t n, double factor, void* stream);
int a4g_scale_copy(double* d, const double* s, int64_t n, double factor, void* stream);
int a4g_increment(double* d, int64_t n, double delta, void* stream);
/* tensor_block_add_: t0 += t1*scale (a factor within 1e-13 of one counts as one). */
int a4g_add_scaled(double* t0, const double* t1, int64_t n, double scale, void* stream);
/* d = l +/- r, r given in its own index order (labels); interpreter.cpp:1874-1997.
 * d may alias l (the "+=" form); r is then permuted on the fly, no temp block. */
int a4g_add_sub(int subtract, int rank, const int* d_labels, const int* r_labels, const int* r_ext,
                double* d, const double* l, const double* r, void* stream);
/* Same operation as a4g_add_sub, for callers that cannot allocate device
 * memory while they run (a fixed pre-reserved device budget, or work issued
 * inside CUDA stream capture where cudaMalloc is not allowed).  No
 * counterpart in the reference: it allocates nothing.  When r aliases d in a
 * different index order, the permuted r is staged in a device array built
 * into the library: 2^20 doubles (8 MiB), held by every GPU that loads the
 * library until exit; a larger aliased, permuted operand is rejected with
 * A4G_ERR_RANGE.  The array's device address is looked up on the first call
 * per device, so make that first call outside stream capture.  Calls share
 * the array: calls that overlap on the GPU race.  stream: the caller's
 * stream; NULL = the library's own stream when the library is already
 * initialised on the current device (the stream every other a4g_* call given
 * NULL uses, so such calls stay ordered), else the CUDA legacy default stream
 * (this entry point never creates the library's context or stream). */
int a4g_add_sub_noalloc(int subtract, int rank, const int* d_labels, const int* r_labels,
                        const int* r_ext, double* d, const double* l, const double* r, void* stream);
/* Sum of squares into *h_result (host), tensor_block_norm2_. Synchronous. */
int a4g_norm2(const double* t, int64_t n, double* h_result, void* stream);
/* Slice / insert of a rectangular sub-block (tensor_dil_omp.F90:271-392). */
int a4g_slice(int rank, const double* tens, const int* tens_ext, double* slice,
              const int* slice_ext, const int* ext_beg, void* stream);
int a4g_insert(int rank, double* tens, const int* tens_ext, const double* slice,
               const int* slice_ext, const int* ext_beg, void* stream);
/* energy_denominator_rhf on device data.  e_or_fock: 1-D energies (rank1 = 1)
 * or the 2-D Fock block (rank1 = 2, leading dimension ext1[0]). */
int a4g_energy_denominator(int rank0, const int* index_values0, const int* ext0, double* data0,
                           int rank1, const int* ext1, const double* e_or_fock, int nsegs,
                           const int* seg_sizes, void* stream);
/* Self-test of the device-side bounded waits (no reference counterpart):
 * one thread waits on an mbarrier that nothing arrives at, gives up after
 * limit_ms (1..5000), records the device error flag the pipelines use and
 * returns.  Expected result: A4G_ERR_TIMEOUT, *waited_ms >= limit_ms, and the
 * CUDA context still usable.  Every pipeline wait (TMA stages, MMA
 * accumulators, bulk copies) takes the same path with a 20 s limit. */
int a4g_selftest_wait_timeout(int limit_ms, int* waited_ms, void* stream);
/* Self-tests of the exact-rounding helpers as the kernels run them (no
 * reference counterpart), over n elements of device arrays:
 * a4g_selftest_round: out[i] = (neg[i] ? -1 : 1) * v[i] * 2^e2[i] rounded
 * once to the nearest double (ties to even), the rounding of every
 * split-precision result; a4g_selftest_div: out[i] = a[i] / b[i] rounded to
 * the nearest double, the division of the denominators and the (T) energy.
 * Both are expected to equal IEEE arithmetic bit for bit. */
int a4g_selftest_round(int n, const long long* v, const int* e2, const int* neg, double* out, void* stream);
int a4g_selftest_div(int n, const double* a, const double* b, double* out, void* stream);

/* Amplitude update of one block (a,i,b,j): procedure updatet2 of
 * src/sialx/qm/cc/rlccd_rhf.sialx:557-600, both of its pardo passes fused
 * into one read of the inputs:
 *   t  = T2new[b,j,a,i] + T2new[a,i,b,j];   t1 = T2old[b,j,a,i] + T2old[a,i,b,j]
 *   diis_err   = -0.5 * (t1 - t / eps)      (Eaibj, the DIIS error block; NULL: not stored)
 *   t2old_next = (0.5 * t) / eps            (the next T2old block)
 *   *norm2    += sum diis_err^2             (device double; NULL: not formed)
 * eps as energy_denominator_rhf forms it (index_values / ext: the segments and
 * extents of (a,i,b,j)).  *_pair are the (b,j,a,i) blocks of the same arrays,
 * stored with extents (ext[2], ext[3], ext[0], ext[1]); a diagonal block is
 * its own pair.  The outputs must not overlap any input: the partner block
 * still reads T2old, so the next T2old goes to another buffer (the reference
 * separates the passes with a server barrier).  Elements are bit-identical
 * to the reference's sequence; norm2 is a deterministic sum. */
int a4g_update_t2(const int* index_values, const int* ext, const double* t2new, const double* t2new_pair,
                  const double* t2old, const double* t2old_pair, double* diis_err, double* t2old_next,
                  int rank1, const int* ext1, const double* e_or_fock, int nsegs, const int* seg_sizes,
                  double* norm2, void* stream);
/* Energy contribution of one block, the (T) pattern of
 * src/sialx/qm/cc/rccsdpt_aaa.sialx:2163-2172 (permute to the denominator's
 * index order, energy_denominator_rhf, full contraction of the divided block
 * with the undivided one, times efact, added to esum) fused into one read of
 * data0 that leaves data0 unchanged:
 *     *esum += efact * sum_x data0[x] * fl(data0[x] / eps(x))
 * all in FP64: eps(x) the orbital-energy sum of a4g_energy_denominator (the
 * same terms added in the same order as energy_denominator_rhf), the quotient
 * rounded exactly like the reference's FP64 division (the same bits), the
 * products accumulated in FP64; the result matches the reference's sequence to
 * the rounding of a long FP64 sum.
 * index_values0 / ext0 follow data0's storage order; den_order[q] names the
 * dimension of data0 at position q of the denominator's order (virtual,
 * occupied, virtual, occupied, ...), NULL when data0 is stored in that order.
 * esum is a device double.  The sum is deterministic on a given GPU; calls
 * share the library's reduction scratch, so keep them on one stream. */
int a4g_energy_contract(int rank0, const int* index_values0, const int* ext0, const double* data0,
                        const int* den_order, int rank1, const int* ext1, const double* e_or_fock,
                        int nsegs, const int* seg_sizes, double efact, double* esum, void* stream);

/* ----------------------------------------------------------------------------
 * Batched contraction of one pardo step (one call, many block triples).
 * Every triple uses the same contraction pattern (one SIAL statement); block
 * extents may differ per triple (uneven segments).  Triples that share the
 * same D pointer are summed into that block.  A triple whose L or R pointer
 * is NULL is a zero block and is skipped (the `where`-clause skip).
 * Split precision: a4g_batch_create reads the L and R blocks once (the
 * autotuner times the GEMM forms on their digits; their values need not be
 * final) and writes no D block.  A NaN or an infinity in an operand block
 * makes every result of the row or column it feeds NaN (FP64 gives NaN or
 * +-infinity there); other results keep the split form's accuracy.
 * ------------------------------------------------------------------------- */
typedef struct a4g_triple {
  double* d;
  const double* l;
  const double* r;
  int dext[6];
  int lext[6];
  int rext[6];
} a4g_triple;

#define A4G_PREC_FP64 0       /* plain FP64 (DMMA)                                  */
#define A4G_PREC_OZAKI_BF16 1 /* split-precision: BF16 slices on tcgen05 tensor cores */

typedef struct a4g_batch_opts {
  int precision;   /* A4G_PREC_*                                              */
  int slices;      /* BF16 digit slices per operand (Ozaki), 1..7; 0 = 5.
                      Each slice is a balanced base-256 digit; 5 slices keep
                      the relative error near 1e-11, 6 near 1e-13.          */
  int beta;        /* 0: D = sum of products (overwrite); 1: D += sum        */
  int variant;     /* split precision, tensor-core GEMM form: 0 autotuned at
                      creation (each form timed once and scored with the
                      HBM traffic it leaves to the rest of the step, the
                      lowest score kept), 1: one SM per 128x128 tile, 2: a
                      CTA pair per 256x128 tile (cta_group::2), 3: one SM per
                      128x256 tile, 4: a CTA pair per 256x256 tile (1-4 write
                      integer level sums, a second kernel combines them),
                      5 / 6: forms 1 / 2 storing FP64 directly (the levels of
                      a tile folded exactly in TMEM; available when no split-K
                      is needed and the 64-bit sum cannot overflow, i.e. up
                      to 5 slices for k ranges below ~100000)               */
  int negate;      /* 1: subtract the products: D = -sum (beta 0) or
                      D -= sum (beta 1), e.g. the second term of
                      W = A*B - C*E run as a second batch on the same D      */
  int pipeline;    /* split precision: 0/1 off; p > 1 runs the GEMM as up to
                      p launches over split-K ranges and slices the right
                      operand's later ranges on a second stream beside them.
                      Off by default: on a power-capped GB300 the overlap
                      lowered the clock and the step gained nothing.         */
  int reserved[2];
} a4g_batch_opts;

/* Opaque handle of a planned pardo step: pattern + triple list + workspace. */
typedef struct a4g_batch a4g_batch;

int a4g_batch_create(a4g_batch** out, const int* contr_ptrn, int drank, int lrank, int rrank,
                     const a4g_triple* h_triples, int64_t n_triples, const a4g_batch_opts* opts);
int a4g_batch_run(a4g_batch* b, void* stream);
/* Capture a4g_batch_run into a CUDA graph once; later runs replay it. */
int a4g_batch_run_graph(a4g_batch* b, void* stream);
/* Same as a4g_batch_run, with CUDA events recorded on `stream` between the
 * pipeline phases; a4g_batch_timings returns the summed milliseconds per phase
 * over every timed run since the previous call (it synchronises).  Phases:
 * 0 zero fill, 1 exponents, 2 split, 3 tensor-core GEMM (or the FP64 grouped
 * kernel), 4 recombine. */
int a4g_batch_run_timed(a4g_batch* b, void* stream);
int a4g_batch_timings(a4g_batch* b, float* phase_ms, int nphase, int* runs);
/* Number of block pairs executed (zero blocks skipped) and FP64 flops. */
int a4g_batch_info(const a4g_batch* b, int64_t* pairs, double* flops, int64_t* workspace_bytes);
/* Split-K count of the tensor-core GEMM in use (0 for FP64 batches) and the
 * autotuner's candidates with their scores in ms (GEMM time measured at
 * creation + the recombine's workspace read at the copy rate; 0 / -1 when a
 * candidate was not tried). */
int a4g_batch_splits(const a4g_batch* b, int* nsplit, int* candidates, float* cost_ms, int n);
/* Library kernels one run launches, and the number of tensor-core GEMM
 * launches among them (more than one when the right operand's split runs
 * beside the GEMM on a second stream). */
int a4g_batch_launches(const a4g_batch* b, int* kernels_per_run, int* gemm_parts);
/* The tensor-core GEMM form in use (the `variant` numbering; 0 for FP64
 * batches) and the autotuner's score of each form in ms (-1: not run): the
 * GEMM's measured time + the workspace read and D traffic at the copy rate. */
int a4g_batch_form(const a4g_batch* b, int* form, float* tuned_ms, int n);
void a4g_batch_destroy(a4g_batch* b);

/* ----------------------------------------------------------------------------
 * Device residency of host blocks: the GPU side of the reference's
 * BlockManager (src/sip/dynamic_data/block_manager.cpp:291-446, lazy copies
 * between host and GPU) and of the Block status bits onGPU / dirtyOnHost /
 * dirtyOnGPU (src/sip/dynamic_data/block.h:150-174).  A block is its host
 * data pointer (Block::data_) and element count; its device copy is made on
 * first use and kept until it is evicted (least recently used first, written
 * back first when newer than the host copy) or forgotten.  Blocks must not
 * overlap; a block whose host memory is freed must be forgotten before the
 * address is reused.
 * ------------------------------------------------------------------------- */
typedef struct a4g_blocks a4g_blocks;

#define A4G_BLOCK_READ 0      /* the copy is read                               */
#define A4G_BLOCK_UPDATE 1    /* read and modified                              */
#define A4G_BLOCK_OVERWRITE 2 /* replaced entirely: its old values are not read */

/* capacity_bytes: the most device memory the copies may hold. */
int a4g_blocks_create(a4g_blocks** out, size_t capacity_bytes);
/* Frees every device copy without writing any back (flush first to keep
 * device results); detaches the cache if it is attached. */
void a4g_blocks_destroy(a4g_blocks* c);
/* The device copy of host block h (n doubles) for use on `stream`
 * (lazy_gpu_read/update/write_on_device): READ and UPDATE copy the block in
 * when there is no device copy or the host copy is newer; OVERWRITE copies
 * nothing in; UPDATE and OVERWRITE make the device copy the newer one. */
int a4g_blocks_on_device(a4g_blocks* c, double* h, int64_t n, int mode, double** d, void* stream);
/* The host copy of block h for use on the host (lazy_gpu_read/update/
 * write_on_host): READ and UPDATE copy the block back (synchronously) when
 * the device copy is newer; OVERWRITE copies nothing back; UPDATE and
 * OVERWRITE make the host copy the newer one (the next device use copies it
 * in).  A block with no device copy needs nothing. */
int a4g_blocks_on_host(a4g_blocks* c, double* h, int mode, void* stream);
/* Writes back every device copy that is newer than its host copy. */
int a4g_blocks_flush(a4g_blocks* c, void* stream);
/* Drops block h's device copy without writing it back (the block is being
 * deleted). */
int a4g_blocks_forget(a4g_blocks* c, double* h);
/* Bytes copied host->device and device->host so far, device bytes held, and
 * the number of evictions. */
int a4g_blocks_stats(a4g_blocks* c, int64_t* h2d_bytes, int64_t* d2h_bytes, int64_t* resident_bytes,
                     int64_t* evictions);
/* Makes the drop-in entry points of group 1 (tensor_block_contract__,
 * tensor_block_copy__, tensor_block_add__, tensor_block_scale__,
 * tensor_block_init__, tensor_block_norm2__, tensor_block_slice__,
 * tensor_block_insert__, energy_denominator_rhf) work through cache c
 * (NULL: detach).  Their host operands are then taken from their device
 * copies (copied in only when missing or stale), and their results stay on
 * the device, newer than the host copy, until a4g_blocks_on_host or
 * a4g_blocks_flush brings them back: the interpreter calls on_host before it
 * reads a block on the host, as BlockManager does for GPU blocks.  Detached
 * (the default), the drop-ins copy every operand in and every result back
 * on each call, like the Fortran they replace. */
int a4g_blocks_attach(a4g_blocks* c);

/* ----------------------------------------------------------------------------
 * One batch for a whole pardo loop.  A pardo loop runs the same statement over
 * many segment tuples (src/sip/worker/loop_manager.cpp:289-314): every
 * iteration has the same block shapes and differs only in which blocks it
 * reads and writes (the ladder's 256 (a,b) slabs all read the same T blocks).
 * These calls let one planned, autotuned batch serve every iteration.
 * ------------------------------------------------------------------------- */

/* Points the batch at other blocks of the same shapes.  Triple i replaces
 * triple i of the creation (or of the previous rebind): the same count, the
 * same extents, the same NULL (skipped) operands, and the same sharing —
 * triples that named one block still name one block, distinct destination
 * blocks stay distinct.  Operand blocks read with 16-byte loads must stay
 * 16-byte aligned (blocks of a BlockArray-style allocation always are).  The
 * batch's tables are rewritten by copies queued on `stream`, so runs queued
 * earlier on that stream still use the old blocks and later runs the new
 * ones: rebind on the stream the batch runs on.  A graph captured by
 * a4g_batch_run_graph stays valid (it reads the tables), except that it is
 * recaptured when a zero-filled destination block (beta 0, no live pair)
 * moves.  Blocks of a held operand (a4g_batch_hold) cannot move. */
int a4g_batch_rebind(a4g_batch* b, const a4g_triple* h_triples, int64_t n_triples, void* stream);

/* Split precision: reuse an operand's BF16 digits across runs.  operand 0 =
 * the triples' L blocks, 1 = their R blocks.  hold = 1 slices those blocks now
 * (exponent and split passes queued on `stream`) and makes every later run
 * skip both passes for them, so the caller promises not to change their
 * values while held; hold = 1 again re-slices them (after the caller changed
 * them).  hold = 0 releases: runs slice them again.  A captured graph is
 * recaptured when the hold state changes.  FP64 batches accept and ignore it.
 * The ladder's T blocks, identical for all 256 slabs, are sliced once per
 * contraction this way. */
int a4g_batch_hold(a4g_batch* b, int operand, int hold, void* stream);

/* Certified accuracy of the last run of a split-precision batch (beta 0, so
 * that D holds the product alone).  For every destination block it bounds
 * the relative Frobenius error ||D - L*R||_F / ||L*R||_F for ANY data, from
 * the run's own row and column exponents (E_m, F_n: |x| < 2^E over a row of
 * the step) and the digit count S: per element and per k the digits carry each
 * operand to within 2^(E - 8S) and the levels dropped by the triangular
 * truncation add at most (S - 1) 2^(E + F - 8S) (1 + 2^-8 + ...), so
 *   ||D - LR||_F <= c_S K 2^-8S sqrt(sum_m 4^E_m * sum_n 4^F_n) + 2^-53 ||D||_F
 * with c_S = 1.004 (S - 1) + 2.001 and K the block's k length (the
 * error-free-splitting bounds of Ozaki, Ogita, Oishi, Rump, Numer. Algorithms
 * 59 (2012), for this digit layout), divided by ||LR||_F >= ||D||_F - bound.
 * It is a worst case: every product's error is taken at its maximum with one
 * sign, so on random data it lies orders of magnitude above the error
 * measured against FP64.  *h_bound = the largest over the blocks (infinity
 * for a block with a NaN or infinite operand).  Returns A4G_ERR_PRECISION when
 * target > 0 and the bound exceeds it: more slices are needed to guarantee it.
 * Synchronises `stream` (the stream of the run). */
int a4g_batch_error_bound(a4g_batch* b, double target, double* h_bound, void* stream);

/* Whether the batch's GEMM form and split-K count came from the tuning cache
 * (1) or from timing runs at creation (0), and the host milliseconds the
 * autotuner spent at creation (0 from the cache or with a pinned variant). */
int a4g_batch_tuning(const a4g_batch* b, int* from_cache, float* autotune_ms);
/* The tuning cache: every autotuned split-precision batch records its choice
 * under a key made from its structure (options, pattern, extents, block
 * sharing, operand alignment, SM count); a batch created later with the same
 * key takes the choice without timing.  The cache lives for the process;
 * save/load keep it in a text file across processes. */
void a4g_tune_cache_clear(void);
int a4g_tune_cache_save(const char* path);
int a4g_tune_cache_load(const char* path);

/* ----------------------------------------------------------------------------
 * Fused pardo step: one or two contraction statements into the same
 * destination blocks in one split-precision pass, and optionally the (T)
 * energy of the result without storing it (rccsdpt_aaa.sialx:2163-2172:
 * W = V1*T - V2*T, then energy_denominator_rhf on a copy and the contraction
 * of the two to a scalar, esum += etemp).
 *
 * Store form (energy NULL): every destination block becomes
 *     D = sign1 * L1 R1 + sign2 * L2 R2        (beta 1: D += ...)
 * with both terms' integer level sums added before the one rounding (the two
 * statements of the reference round after each).  Energy form: nothing is
 * written; for every element x of every destination block
 *     *esum += efact * D(x) * fl(D(x) / eps(x))
 * eps(x) the orbital-energy denominator of a4g_energy_contract (the same
 * terms added in the same order: the chain without its last term is
 * tabulated once at creation, the last subtraction and the exactly rounded
 * quotient are formed per element), the products summed in FP64 in a fixed
 * order.  D exists only one tile at a time, as exact integer level sums in
 * tensor memory.
 *
 * GEMM form (opts->variant): 0 automatic (7 where it fits, else 5); 5 one
 * level at a time: 128 x 128 tiles, the exact 64-bit sum over levels folded
 * in tensor memory level by level; 7 all levels at once: 128 x 64 tiles,
 * every level's accumulator in tensor memory together, each k block of the
 * slices loaded once for all slice pairs, the sum over levels formed in
 * registers and tensor memory released before the rounding, the division and
 * the store; it fits at most 5 slices and k <= 320 per sub-problem (the sum
 * of both terms' contracted extents, each stretch rounded up to 64; the
 * triples at segments of 24 and 10 virtual segments: 256 + 64) and is
 * A4G_ERR_UNSUPPORTED beyond.  Both forms give the same D bits; the energy
 * sums differ in the order of the partial sums only.
 *
 * Both terms share the destination ranks and the operand ranks.  Every
 * destination index is a row (left operand in both terms), a column (right
 * in both), or fixed per sub-problem (left in one term, right in the other:
 * the triples' b and j); the energy form needs the denominator's last term
 * on a row or column index.  Split precision only (opts->precision
 * A4G_PREC_OZAKI_BF16); opts->slices, opts->beta and opts->variant apply, the
 * other options are ignored.  A triple with a NULL operand is skipped. */
typedef struct a4g_term {
  const int* contr_ptrn; /* as for a4g_batch_create (lrank + rrank entries)  */
  const a4g_triple* triples;
  int64_t n_triples;
  int sign; /* +1: the term is added, -1: subtracted                       */
} a4g_term;

typedef struct a4g_fused_energy {
  int64_t n_blocks;
  double* const* blocks;   /* the destination blocks (the triples' d pointers) */
  const int* index_values; /* [n_blocks * drank]: as a4g_energy_contract's index_values0 */
  const int* den_order;    /* NULL or [drank], as for a4g_energy_contract */
  int rank1;
  const int* ext1;
  const double* e_or_fock; /* device */
  int nsegs;
  const int* seg_sizes;
  double efact;
} a4g_fused_energy;

typedef struct a4g_fused a4g_fused;

int a4g_fused_create(a4g_fused** out, int drank, int lrank, int rrank, const a4g_term* terms, int nterms,
                     const a4g_fused_energy* energy, const a4g_batch_opts* opts);
/* esum: a device double (energy form), else NULL.  Operands are read at run
 * time (their values may change between runs; their addresses may not). */
int a4g_fused_run(a4g_fused* f, double* esum, void* stream);
/* The next iteration of the same loop (the triples' next (a, b) step): the
 * same terms with other blocks and, in the energy form, other index values,
 * in the same structure (triple counts, extents, zero blocks, which blocks
 * share a destination or a right operand, which destination blocks share a
 * denominator table).  Re-plans on the host, then updates on `stream` only the
 * split jobs' sources, the destination column bases and the denominator
 * tables; the tiles, panels and kernel arguments stay.  A4G_ERR_ARG when the
 * structure differs (create a new step then). */
int a4g_fused_rebind(a4g_fused* f, const a4g_term* terms, int nterms, const a4g_fused_energy* energy, void* stream);
int a4g_fused_info(const a4g_fused* f, int64_t* pairs, double* flops, int64_t* elements, int64_t* device_bytes);
/* The GEMM form the step runs: 5 (one level at a time) or 7 (all levels at once); -1 for NULL. */
int a4g_fused_form(const a4g_fused* f);
void a4g_fused_destroy(a4g_fused* f);

#ifdef __cplusplus
}
#endif
#endif /* ACES4_GB300_H */
