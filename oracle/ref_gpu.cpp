// TEST INFRASTRUCTURE ONLY (never part of the product): the reference's
// legacy GPU contraction path, run on this GPU as a baseline and a checker.
//
// The device code is the reference's own: oracle/Makefile compiles
// src/sip/cuda/gpu_super_instructions.cu from the reference tree into
// oracle/_ref/gpu_super_instructions.cubin (sm_103a), and this file loads that
// image and launches its kernels reorderScatter / reorderGather (:307-351)
// with its __constant__ tables dimsDev / stepsDev (:25-26).  The host side of
// __gpu_contract_helper (:369-586) is restated here step for step, because
// the reference's host code cannot be built for the GPU machine's processor
// from this one:
//   three scratch buffers of SCRATCH_BUFFER_SIZE_MB = 40 MB allocated and
//   freed on every call (:400-402, :580-582); the index permutations of x1,
//   x2 and y (:425-466); per operand: its strides written to the constant
//   tables, a device-to-device copy into scratch3, reorderScatter into
//   scratch1 / scratch2 with REORDER_BLOCKS x REORDER_THREADS = 48 x 512
//   (:467-521); cublasDgemm (N, N) issued twice, as the reference does
//   (:534-548); reorderGather of the result and its copy into y (:551-574); a
//   device synchronisation after each step as in the reference.
// gpu_super_instructions.h:18-20 gives the constants.
#include <cublas_v2.h>
#include <cuda.h>
#include <cuda_runtime.h>

#include <cstdio>
#include <cstring>
#include <string>

namespace {

constexpr int kMaxRank = 6;               // aces_defs.h MAX_RANK
constexpr size_t kScratchMB = 40;         // SCRATCH_BUFFER_SIZE_MB
constexpr unsigned kReorderBlocks = 48;   // REORDER_BLOCKS
constexpr unsigned kReorderThreads = 512; // REORDER_THREADS

CUmodule g_mod = nullptr;
CUfunction g_scatter = nullptr, g_gather = nullptr;
CUdeviceptr g_dims = 0, g_steps = 0;
cublasHandle_t g_blas = nullptr;
std::string g_err;

int failed(const std::string& what) {
  g_err = what;
  return 1;
}

#define RCU(x)                                                             \
  do {                                                                     \
    CUresult r_ = (x);                                                     \
    if (r_ != CUDA_SUCCESS) return failed(#x " -> " + std::to_string(int(r_))); \
  } while (0)
#define RRT(x)                                                             \
  do {                                                                     \
    cudaError_t r_ = (x);                                                  \
    if (r_ != cudaSuccess) return failed(#x " -> " + std::string(cudaGetErrorString(r_))); \
  } while (0)
#define RBL(x)                                                             \
  do {                                                                     \
    cublasStatus_t r_ = (x);                                               \
    if (r_ != CUBLAS_STATUS_SUCCESS) return failed(#x " -> " + std::to_string(int(r_))); \
  } while (0)

int set_tables(const int* dims, const int* steps, int n) {
  RCU(cuMemcpyHtoD(g_dims, dims, sizeof(int) * size_t(n)));
  RCU(cuMemcpyHtoD(g_steps, steps, sizeof(int) * size_t(n)));
  return 0;
}

int launch(CUfunction f, double* dst, double* src, int ndims, int size) {
  void* args[] = {&dst, &src, &ndims, &size};
  RCU(cuLaunchKernel(f, kReorderBlocks, 1, 1, kReorderThreads, 1, 1, 0, nullptr, args, nullptr));
  RRT(cudaGetLastError());
  RRT(cudaDeviceSynchronize());
  return 0;
}

}  // namespace

extern "C" {

const char* ref_gpu_error(void) { return g_err.c_str(); }

// Loads the reference's kernels from the cubin (once per process) and makes
// the cuBLAS handle (_init_gpu, :34-66).
int ref_gpu_load(const char* cubin_path) {
  if (g_mod) return 0;
  RRT(cudaFree(nullptr));  // the runtime's primary context is current from here on
  RCU(cuModuleLoad(&g_mod, cubin_path));
  RCU(cuModuleGetFunction(&g_scatter, g_mod, "_Z14reorderScatterPdS_ii"));
  RCU(cuModuleGetFunction(&g_gather, g_mod, "_Z13reorderGatherPdS_ii"));
  size_t bytes = 0;
  RCU(cuModuleGetGlobal(&g_dims, &bytes, g_mod, "dimsDev"));
  if (bytes != sizeof(int) * kMaxRank) return failed("dimsDev size");
  RCU(cuModuleGetGlobal(&g_steps, &bytes, g_mod, "stepsDev"));
  RBL(cublasCreate(&g_blas));
  return 0;
}

// _gpu_contract (:125-165) on device blocks: y = x1 * x2.
int ref_gpu_contract(double* y, int ny, const int* yDims, const int* yInds, double* x1, int n1,
                     const int* x1Dims, const int* x1Inds, double* x2, int n2, const int* x2Dims,
                     const int* x2Inds) {
  if (!g_mod) return failed("ref_gpu_load first");
  if (ny > kMaxRank || n1 > kMaxRank || n2 > kMaxRank) return failed("rank above MAX_RANK");
  double *s1 = nullptr, *s2 = nullptr, *s3 = nullptr;
  RRT(cudaMalloc(&s1, kScratchMB * 1024 * 1024));
  RRT(cudaMalloc(&s2, kScratchMB * 1024 * 1024));
  RRT(cudaMalloc(&s3, kScratchMB * 1024 * 1024));

  int steps[kMaxRank];
  int yIndsP[kMaxRank], yDimsP[kMaxRank], x1IndsP[kMaxRank], x1DimsP[kMaxRank], x2IndsP[kMaxRank],
      x2DimsP[kMaxRank];
  const int nc = (n1 + n2 - ny) / 2;
  // permutations: x1 -> [uncontracted | contracted in x1 order], x2 -> [contracted | uncontracted],
  // y -> [x1's uncontracted | x2's uncontracted in y order]
  int c = 0, k = 0;
  for (int i = 0; i < n1; ++i) {
    bool contracted = false;
    for (int j = 0; j < n2; ++j)
      if (x1Inds[i] == x2Inds[j]) {
        contracted = true;
        x1IndsP[n1 - nc + c] = x1Inds[i], x1DimsP[n1 - nc + c] = x1Dims[i];
        x2IndsP[c] = x2Inds[j], x2DimsP[c] = x2Dims[j];
        ++c;
        break;
      }
    if (!contracted) {
      x1IndsP[k] = x1Inds[i], x1DimsP[k] = x1Dims[i];
      yIndsP[k] = x1Inds[i], yDimsP[k] = x1Dims[i];
      ++k;
    }
  }
  c = 0;
  for (int i = 0; i < n2; ++i)
    for (int j = 0; j < ny; ++j)
      if (x2Inds[i] == yInds[j]) {
        x2IndsP[nc + c] = x2Inds[i], x2DimsP[nc + c] = x2Dims[i];
        yIndsP[k] = yInds[j], yDimsP[k] = yDims[j];
        ++k, ++c;
      }
  // one operand: strides of its permuted order -> constant tables, copy into
  // scratch3, scatter into dst
  auto reorder_in = [&](double* dst, double* src, int n, const int* inds, const int* dims, const int* indsP,
                        const int* dimsP, int* size) -> int {
    int step = 1;
    for (int i = 0; i < n; ++i) {
      for (int j = 0; j < n; ++j)
        if (inds[j] == indsP[i]) {
          steps[j] = step;
          break;
        }
      step *= dimsP[i];
    }
    *size = step;
    if (set_tables(dims, steps, n)) return 1;
    RRT(cudaMemcpy(s3, src, size_t(step) * sizeof(double), cudaMemcpyDeviceToDevice));
    RRT(cudaDeviceSynchronize());
    return launch(g_scatter, dst, s3, n, step);
  };
  int size = 0;
  if (reorder_in(s1, x1, n1, x1Inds, x1Dims, x1IndsP, x1DimsP, &size)) return 1;
  if (reorder_in(s2, x2, n2, x2Inds, x2Dims, x2IndsP, x2DimsP, &size)) return 1;
  const double alpha = 1.0, beta = 0.0;
  int lda = 1, ldb = 1;
  for (int i = 0; i < n1 - nc; ++i) lda *= x1DimsP[i];
  for (int i = 0; i < nc; ++i) ldb *= x2DimsP[i];
  RBL(cublasDgemm(g_blas, CUBLAS_OP_N, CUBLAS_OP_N, lda, size / ldb, ldb, &alpha, s1, lda, s2, ldb, &beta, s3, lda));
  RRT(cudaDeviceSynchronize());
  RRT(cudaDeviceSynchronize());
  RBL(cublasDgemm(g_blas, CUBLAS_OP_N, CUBLAS_OP_N, lda, size / ldb, ldb, &alpha, s1, lda, s2, ldb, &beta, s3, lda));
  RRT(cudaDeviceSynchronize());
  // y: strides of its permuted order, gather from scratch3 into scratch1, copy into y
  int step = 1;
  for (int i = 0; i < ny; ++i) {
    for (int j = 0; j < ny; ++j)
      if (yInds[j] == yIndsP[i]) {
        steps[j] = step;
        break;
      }
    step *= yDimsP[i];
  }
  if (set_tables(yDims, steps, ny)) return 1;
  if (launch(g_gather, s1, s3, ny, step)) return 1;
  RRT(cudaMemcpy(y, s1, size_t(step) * sizeof(double), cudaMemcpyDeviceToDevice));
  RRT(cudaFree(s1));
  RRT(cudaFree(s2));
  RRT(cudaFree(s3));
  RRT(cudaDeviceSynchronize());
  return 0;
}

}  // extern "C"
