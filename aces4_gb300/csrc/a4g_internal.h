// Internal declarations shared by the library's translation units.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <string>
#include <vector>

#include "../../include/aces4_gb300.h"

namespace a4g {

constexpr int kMaxRank = 32;  // tensor_dil_omp.F90:58 max_tensor_rank

// ---------------------------------------------------------------- errors
void set_error(const std::string& msg);
void clear_error();
const char* last_error_text();
int fail(int code, const std::string& msg);
int cuda_fail(cudaError_t e, const char* what);
#define A4G_CUDA(call)                                    \
  do {                                                    \
    cudaError_t e_ = (call);                              \
    if (e_ != cudaSuccess) return ::a4g::cuda_fail(e_, #call); \
  } while (0)

// ---------------------------------------------------------------- context
// One per process: the current device, the library stream, a grow-only device
// arena for the host-buffer (drop-in) entry points, and a device error flag
// that bounded device-side waits set instead of hanging.
struct Context {
  int device = -1;
  int num_sms = 0;
  cudaStream_t stream = nullptr;
  void* arena = nullptr;
  size_t arena_bytes = 0;
  int* d_error_flag = nullptr;  // device int: nonzero = a kernel gave up a wait
  // Stream-ordered allocations of the library (split-K workspaces, block
  // copies, reduction partials) come from a pool of its own that keeps freed
  // memory for reuse: the default pool hands memory back to the driver at
  // every synchronisation, so a synchronous call would allocate from scratch
  // each time.
  cudaMemPool_t pool = nullptr;
  // Kernels can read and write pageable host memory through the host's page
  // tables (address translation services over the CPU-GPU link): the
  // drop-ins then run on the caller's host blocks in place.
  bool host_access = false;
  int host_direct = 1;  // a4g_host_direct: 1 in place when host_access, 0 always staged
};
Context* ctx();             // initialises on first use (device = current)
int ensure_init();          // returns A4G_OK or an error code
cudaStream_t pick(void* stream);
int arena_reserve(size_t bytes, void** out);  // arena is reused across calls
int check_device_flag(cudaStream_t s);        // syncs s, reads and clears the flag
int async_alloc(void** p, size_t bytes, cudaStream_t s);  // from the library pool, stream-ordered (free: cudaFreeAsync)

// ---------------------------------------------------------------- block cache
// The cache the drop-in entry points use (a4g_blocks_attach), or null; and
// the lazy host -> device step of blocks.cpp (mode: A4G_BLOCK_*).
a4g_blocks* attached_blocks();
int blocks_on_device(a4g_blocks* c, double* h, int64_t n, int mode, double** d, cudaStream_t s);

// ---------------------------------------------------------------- planner
// Pattern handling restated from tensor_dil_omp.F90 (get_contraction_ptrn
// :87-142, contr_ptrn_ok :861-896) plus the GEMM view used by the kernels.
int get_contraction_ptrn(int drank, int lrank, int rrank, const int* aces, int* my);
bool perm_from_labels(int rank, const int* dst_labels, const int* src_labels, int* o2n);
bool contr_ptrn_ok(const int* ptrn, int lr, int rr, int dr, const int* lext, const int* rext,
                   const int* dext);

enum class ContractKind { kTensorTensor, kFull, kRightScalar, kLeftScalar, kScalarScalar };

// Matrix view of a contraction with the permutes folded into address tables:
//   D[offDm[m] + offDn[n]] = sum_k L[offLm[m] + offLk[k]] * R[offRk[k] + offRn[n]]
// m runs over L's uncontracted indices (L order), n over R's uncontracted
// indices (R order), k over the contracted pairs.  No operand is ever
// materialised in transposed form.
struct GemmPlan {
  ContractKind kind;
  int64_t M = 1, N = 1, K = 1;
  std::vector<int64_t> offLm, offLk, offRk, offRn, offDm, offDn;
  bool a_kfast = false;  // L is unit-stride along k (else along m)
  bool b_kfast = true;   // R is unit-stride along k (else along n)
};
int build_gemm_plan(const int* ptrn, int lrank, const int* lext, int rrank, const int* rext,
                    int drank, const int* dext, GemmPlan* p);

// Device copy of a plan's tables (cached by pattern + extents).
struct DevPlan {
  GemmPlan host;
  int64_t* d_tables = nullptr;  // offLm | offLk | offRk | offRn | offDm | offDn
  const int64_t *offLm, *offLk, *offRk, *offRn, *offDm, *offDn;
};
int get_dev_plan(const int* ptrn, int lrank, const int* lext, int rrank, const int* rext,
                 int drank, const int* dext, const DevPlan** out);

// First orbital of each block dimension's segment (energy_denominator_rhf.F:
// 57-88, 140-220), every orbital index checked against the energy array.
int denominator_offsets(int rank0, const int* iv, const int* ext0, int rank1, const int* ext1,
                        const std::vector<int>& segs, int* off);

// ---------------------------------------------------------------- kernels
// Element-wise / permute / reduction launchers (kernels_block.cu).
int launch_fill(double* d, int64_t n, double v, cudaStream_t s);
int launch_scale(double* d, int64_t n, double f, cudaStream_t s);
int launch_scale_copy(double* d, const double* src, int64_t n, double f, cudaStream_t s);
int launch_increment(double* d, int64_t n, double delta, cudaStream_t s);
int launch_add_scaled(double* t0, const double* t1, int64_t n, double scale, cudaStream_t s);
int launch_axpy(double* y, const double* x, int64_t n, double alpha, cudaStream_t s);
int launch_permute(int rank, const int* ext, const int* o2n_1based, const double* in, double* out,
                   cudaStream_t s);
int launch_add_sub_permuted(int subtract, int rank, const int* r_ext, const int* o2n_1based,
                            double* d, const double* l, const double* r, cudaStream_t s);
int launch_dot(const double* a, const double* b, const int64_t* offA, const int64_t* offB,
               int64_t n, double* d_out, double* d_scratch, int64_t scratch_len, cudaStream_t s);
int launch_slice_insert(int insert, int rank, double* tens, const int* tens_ext, double* slice,
                        const int* slice_ext, const int* ext_beg, cudaStream_t s);
int launch_update_t2(const int* off, const int* ext, const double* t2new, const double* t2new_pair,
                     const double* t2old, const double* t2old_pair, double* err, double* next, int rank1, int ld1,
                     const double* e_or_fock, double* norm2, double* d_scratch, int64_t scratch_len,
                     cudaStream_t s);
int launch_energy_contract(int rank0, const int* off, const int* ext0, const int* pos, const double* w,
                           int rank1, int ld1, const double* e_or_fock, double efact, double* esum,
                           double* d_scratch, int scratch_len, cudaStream_t s);
int launch_denominator(int rank0, const int* off, const int* ext0, double* data, int rank1,
                       int ld1, const double* e_or_fock, cudaStream_t s);
int launch_dot_beta(const double* a, const double* b, const int64_t* offA, const int64_t* offB,
                    int64_t n, double* d_out, double* d_scratch, int64_t scratch_len, int beta,
                    cudaStream_t s);
int dot_scratch_len();  // doubles of scratch launch_dot needs

// Permute-fused FP64 contraction (kernels_dmma.cu).
int launch_contract_f64(const DevPlan* p, const double* L, const double* R, double* D, int beta,
                        cudaStream_t s);
// Scalar cases of tensor_block_contract_ (kernels_block.cu).
int launch_scalar_cases(const DevPlan* p, const double* L, const double* R, double* D, int beta,
                        double* d_scratch, cudaStream_t s);

}  // namespace a4g
