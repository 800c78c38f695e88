// Allocation-free variant of the block add/subtract (a4g_add_sub).
//
// Some callers cannot allocate device memory while they run: code that
// executes inside an interpreter or solver with a fixed, pre-reserved device
// budget, code called from within a captured CUDA stream (where cudaMalloc is
// not allowed), or hosts whose memory pool is owned by another allocator.
// For them a4g_add_sub_noalloc does the same work as a4g_add_sub with no
// cudaMalloc/cudaMallocAsync/cudaFree at all: the one case that needs a
// temporary block — "d[i,j,k] += d[k,i,j]", where the right operand is the
// destination itself read in another index order, so it must be permuted
// before d is overwritten (the reference builds a temporary block for this,
// src/sip/worker/interpreter.cpp:1919-1927) — stages the permuted operand in
// a fixed device array compiled into this library.
//
// That array (kNoAllocScratchDoubles doubles, 8 MiB) exists once per GPU that
// loads the library and is held until the process exits.  Every call shares
// it and it keeps the last call's contents; it is fully overwritten before it
// is read, so nothing has to be cleared.  Calls whose work overlaps on the GPU
// (different streams, or a call racing a still-running one) race on the
// array: order them on one stream.
#include <mutex>

#include "a4g_internal.h"

namespace {

constexpr int64_t kNoAllocScratchDoubles = int64_t(1) << 20;  // 8 MiB per GPU
constexpr int kMaxDevices = 64;

static __device__ __align__(256) double g_noalloc_scratch[kNoAllocScratchDoubles];

std::mutex g_scratch_mu;
double* g_scratch_ptr[kMaxDevices] = {nullptr};

// Device address of the array for the current device.  The name
// g_noalloc_scratch in host code is only a host-side stand-in; the address
// the kernels need comes from cudaGetSymbolAddress, looked up once per
// device (on that device's first call) with the device current.
int scratch_for_current_device(double** out) {
  int dev = 0;
  A4G_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= kMaxDevices) return a4g::fail(A4G_ERR_RANGE, "device ordinal beyond 63");
  std::lock_guard<std::mutex> lock(g_scratch_mu);
  if (!g_scratch_ptr[dev]) {
    void* p = nullptr;
    A4G_CUDA(cudaGetSymbolAddress(&p, g_noalloc_scratch));
    g_scratch_ptr[dev] = static_cast<double*>(p);
  }
  *out = g_scratch_ptr[dev];
  return A4G_OK;
}

}  // namespace

extern "C" int a4g_add_sub_noalloc(int subtract, int rank, const int* d_labels, const int* r_labels,
                                   const int* r_ext, double* d, const double* l, const double* r,
                                   void* stream) {
  using namespace a4g;
  if (rank < 0 || rank > kMaxRank) return fail(A4G_ERR_ARG, "rank out of range");
  if (!d || !l || !r || (rank > 0 && (!d_labels || !r_labels || !r_ext)))
    return fail(A4G_ERR_ARG, "null argument");
  int o2n[kMaxRank];
  if (!perm_from_labels(rank, d_labels, r_labels, o2n))
    return fail(A4G_ERR_ARG, "incompatible indices for LHS and RHS");
  int64_t n = 1;
  for (int i = 0; i < rank; ++i) {
    if (r_ext[i] <= 0) return fail(A4G_ERR_ARG, "non-positive extent");
    n *= r_ext[i];
  }
  bool trivial = true;
  for (int i = 0; i < rank; ++i) trivial &= o2n[i] == i + 1;
  // NULL stream: the library's own stream when the library context already
  // exists on this device (so the call stays ordered with the other a4g_*
  // calls given NULL, which run there), else the CUDA legacy default stream.
  // Neither choice allocates: the context is never created here.
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  if (!s) {
    int dev = -1;
    A4G_CUDA(cudaGetDevice(&dev));
    if (ctx()->device >= 0 && ctx()->device == dev) s = ctx()->stream;
  }
  const char *rb = reinterpret_cast<const char*>(r), *db = reinterpret_cast<const char*>(d);
  const bool overlap = rb < db + n * sizeof(double) && db < rb + n * sizeof(double);
  if (!trivial && overlap) {
    if (n > kNoAllocScratchDoubles)
      return fail(A4G_ERR_RANGE, "a4g_add_sub_noalloc: a permuted, aliased right operand of " +
                                     std::to_string(n) + " doubles exceeds the fixed scratch of " +
                                     std::to_string(kNoAllocScratchDoubles) + " doubles");
    double* scratch = nullptr;
    int rc = scratch_for_current_device(&scratch);
    if (rc) return rc;
    rc = launch_permute(rank, r_ext, o2n, r, scratch, s);
    if (rc) return rc;
    int ident[kMaxRank], dext[kMaxRank];
    for (int i = 0; i < rank; ++i) ident[i] = i + 1, dext[o2n[i] - 1] = r_ext[i];
    return launch_add_sub_permuted(subtract, rank, dext, ident, d, l, scratch, s);
  }
  return launch_add_sub_permuted(subtract, rank, r_ext, o2n, d, l, r, s);
}
