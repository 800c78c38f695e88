// extern "C" entry points: the drop-in replacements of the reference's
// Fortran kernels (host buffers), of its legacy GPU API (device buffers), the
// energy-denominator super instruction, and the device-resident a4g_* API.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "a4g_internal.h"
#include "ozaki.h"

using namespace a4g;

namespace {

int64_t count(int rank, const int* ext) {
  int64_t n = 1;
  for (int i = 0; i < rank; ++i) n *= ext[i];
  return n;
}

bool extents_ok(int rank, const int* ext) {
  if (rank > 0 && !ext) return false;
  for (int i = 0; i < rank; ++i)
    if (ext[i] <= 0) return false;
  return true;
}

// Maps an a4g status onto the reference's ierr convention for the drop-ins:
// argument/pattern problems keep the reference's own codes (set by callers);
// runtime failures are reported as negative codes the reference never uses.
int runtime_ierr(int rc) { return rc == A4G_OK ? 0 : -100 - rc; }

// Host-buffer staging through the library arena: copy in, run, copy out, sync.
struct Staged {
  char* base = nullptr;
  size_t used = 0;
  double* take(int64_t n) {
    double* p = reinterpret_cast<double*>(base + used);
    used += (size_t(n) * sizeof(double) + 255) & ~size_t(255);
    return p;
  }
};

int stage(size_t bytes, Staged* st) {
  void* p = nullptr;
  int rc = arena_reserve(bytes, &p);
  if (rc) return rc;
  st->base = static_cast<char*>(p);
  st->used = 0;
  return A4G_OK;
}

size_t rounded(int64_t n) { return (size_t(n) * sizeof(double) + 255) & ~size_t(255); }

int h2d(double* d, const double* h, int64_t n, cudaStream_t s) {
  A4G_CUDA(cudaMemcpyAsync(d, h, size_t(n) * sizeof(double), cudaMemcpyHostToDevice, s));
  return A4G_OK;
}
int d2h(double* h, const double* d, int64_t n, cudaStream_t s) {
  A4G_CUDA(cudaMemcpyAsync(h, d, size_t(n) * sizeof(double), cudaMemcpyDeviceToHost, s));
  return A4G_OK;
}

std::mutex g_host_mu;  // host-buffer entries share one arena

// Device views of one drop-in call's host blocks.  Detached (the default):
// where the GPU reads and writes pageable host memory through the host's page
// tables (Grace-Blackwell), the kernels run on the host blocks in place (no
// copies; a result that aliases an operand of a non-element-wise operation
// goes through a device temporary); elsewhere operands are staged through the
// arena and results copied back; either way the call returns when the results
// are in the host blocks, like the Fortran kernels.  With a block cache attached: the
// cache's device copies (copied in only when missing or stale); results stay
// there, newer than the host copy, until the host asks for them.  Operands
// are declared before results, so a result that is also an operand (the same
// host block) is seen: element-wise operations work on the shared device
// copy, the others compute into a temporary that then replaces it.
struct HostIO {
  cudaStream_t s = nullptr;
  a4g_blocks* cache = nullptr;
  bool direct = false;
  Staged st;
  struct Copy {
    double* dst;
    const double* src;
    int64_t n;
    cudaMemcpyKind kind;
  };
  std::vector<Copy> after;  // results back to the host, or temporaries into device copies
  std::vector<const double*> operands;

  int begin(size_t arena_bytes) {
    s = ctx()->stream;
    cache = attached_blocks();
    direct = !cache && ctx()->host_access && ctx()->host_direct;
    return stage(arena_bytes, &st);
  }
  int in(const double* h, int64_t n, double** d) {
    operands.push_back(h);
    if (cache) return blocks_on_device(cache, const_cast<double*>(h), n, A4G_BLOCK_READ, d, s);
    if (direct) {
      *d = const_cast<double*>(h);
      return A4G_OK;
    }
    *d = st.take(n);
    return h2d(*d, h, n, s);
  }
  // reads: the operation reads the result block's old values;
  // elementwise: it may run in place on an operand's device copy
  int out(double* h, int64_t n, bool reads, bool elementwise, double** d) {
    if (cache) {
      double* dc = nullptr;
      int rc = blocks_on_device(cache, h, n, reads ? A4G_BLOCK_UPDATE : A4G_BLOCK_OVERWRITE, &dc, s);
      if (rc) return rc;
      const bool aliased = std::find(operands.begin(), operands.end(), h) != operands.end();
      if (aliased && !elementwise) {
        *d = st.take(n);
        if (reads) A4G_CUDA(cudaMemcpyAsync(*d, dc, size_t(n) * sizeof(double), cudaMemcpyDeviceToDevice, s));
        after.push_back({dc, *d, n, cudaMemcpyDeviceToDevice});
      } else {
        *d = dc;
      }
      return A4G_OK;
    }
    if (direct) {
      const bool aliased = std::find(operands.begin(), operands.end(), h) != operands.end();
      if (!aliased || elementwise) {
        *d = h;
        return A4G_OK;
      }
      *d = st.take(n);
      if (reads) A4G_CUDA(cudaMemcpyAsync(*d, h, size_t(n) * sizeof(double), cudaMemcpyDefault, s));
      after.push_back({h, *d, n, cudaMemcpyDefault});
      return A4G_OK;
    }
    *d = st.take(n);
    if (reads) {
      const int rc = h2d(*d, h, n, s);
      if (rc) return rc;
    }
    after.push_back({h, *d, n, cudaMemcpyDeviceToHost});
    return A4G_OK;
  }
  double* scratch(int64_t n) { return st.take(n); }
  int finish() {
    for (const Copy& c : after)
      A4G_CUDA(cudaMemcpyAsync(c.dst, c.src, size_t(c.n) * sizeof(double), c.kind, s));
    return check_device_flag(s);
  }
};

std::map<std::string, std::vector<int>> g_predefined;
std::mutex g_predef_mu;

int contract_device(const int* ptrn, const double* l, int lrank, const int* lext, const double* r,
                    int rrank, const int* rext, double* d, int drank, const int* dext, int beta,
                    double* scratch, cudaStream_t s) {
  const DevPlan* p = nullptr;
  int rc = get_dev_plan(ptrn, lrank, lext, rrank, rext, drank, dext, &p);
  if (rc) return rc;
  if (p->host.kind == ContractKind::kTensorTensor) return launch_contract_f64(p, l, r, d, beta, s);
  return launch_scalar_cases(p, l, r, d, beta, scratch, s);
}

// Per-context scratch for the deterministic reductions of the device API.
double* reduction_scratch() {
  static double* p = nullptr;
  if (!p) {
    if (cudaMalloc(&p, sizeof(double) * (dot_scratch_len() + 8)) != cudaSuccess) p = nullptr;
  }
  return p;
}

}  // namespace

extern "C" {

const char* a4g_version(void) { return "aces4_gb300 0.1 (sm_103a)"; }

const char* a4g_last_error(void) { return last_error_text(); }
void a4g_clear_error(void) { clear_error(); }

// ============================================================ drop-in (host)
long long tensor_size_by_shape_(int* num_dim, int* dims, int* ierr) {
  *ierr = 0;
  long long s = 1;
  if (*num_dim > 0) {
    for (int i = 0; i < *num_dim; ++i) s *= dims[i];
    if (s <= 0) *ierr = 2;
  } else if (*num_dim < 0) {
    *ierr = 1;
    s = 0;
  }
  return s;
}

void get_contraction_ptrn_(int* drank, int* lrank, int* rrank, int* aces_ptrn, int* my_ptrn,
                           int* ierr) {
  *ierr = a4g::get_contraction_ptrn(*drank, *lrank, *rrank, aces_ptrn, my_ptrn);
}

void tensor_block_init__(int* nthreads, double* tens, int* tens_rank, int* ext, double* sval,
                         int* ierr) {
  (void)nthreads;
  if (*tens_rank < 0) return void(*ierr = -1);
  if (!extents_ok(*tens_rank, ext) || !tens) return void(*ierr = -1);
  std::lock_guard<std::mutex> lock(g_host_mu);
  int rc = ensure_init();
  const int64_t n = count(*tens_rank, ext);
  HostIO io;
  double* d = nullptr;
  if (!rc) rc = io.begin(rounded(n));
  if (!rc) rc = io.out(tens, n, false, true, &d);
  if (!rc) rc = launch_fill(d, n, *sval, io.s);
  if (!rc) rc = io.finish();
  *ierr = runtime_ierr(rc);
}

void tensor_block_scale__(int* nthreads, double* tens, int* tens_rank, int* ext, double* f,
                          int* ierr) {
  (void)nthreads;
  if (*tens_rank < 0 || !extents_ok(*tens_rank, ext) || !tens) return void(*ierr = -1);
  std::lock_guard<std::mutex> lock(g_host_mu);
  int rc = ensure_init();
  const int64_t n = count(*tens_rank, ext);
  HostIO io;
  double* d = nullptr;
  if (!rc) rc = io.begin(rounded(n));
  if (!rc) rc = io.out(tens, n, true, true, &d);
  if (!rc) rc = launch_scale(d, n, *f, io.s);
  if (!rc) rc = io.finish();
  *ierr = runtime_ierr(rc);
}

double tensor_block_norm2__(int* nthreads, double* tens, int* tens_rank, int* ext, int* ierr) {
  (void)nthreads;
  if (*tens_rank < 0 || !extents_ok(*tens_rank, ext) || !tens) {
    *ierr = -1;
    return 0.0;
  }
  std::lock_guard<std::mutex> lock(g_host_mu);
  int rc = ensure_init();
  const int64_t n = count(*tens_rank, ext);
  double result = 0.0;
  HostIO io;
  double* d = nullptr;
  if (!rc) rc = io.begin(rounded(n) + rounded(dot_scratch_len() + 1));
  if (!rc) rc = io.in(tens, n, &d);
  if (!rc) {
    double* scratch = io.scratch(dot_scratch_len());
    double* out = io.scratch(1);
    rc = launch_dot(d, d, nullptr, nullptr, n, out, scratch, dot_scratch_len(), io.s);
    if (!rc) rc = d2h(&result, out, 1, io.s);
    if (!rc) rc = io.finish();
  }
  *ierr = runtime_ierr(rc);
  return result;
}

static void slice_insert_host(int insert, int* dim_num, double* tens, int* text, double* slice,
                              int* sext, int* beg, int* ierr) {
  if (*dim_num < 0) return void(*ierr = 1);
  if (!tens || !slice) return void(*ierr = 1);
  std::lock_guard<std::mutex> lock(g_host_mu);
  int rc = ensure_init();
  const int64_t nt = count(*dim_num, text), ns = count(*dim_num, sext);
  HostIO io;
  double *dt = nullptr, *ds = nullptr;
  if (!rc) rc = io.begin(2 * (rounded(nt) + rounded(ns)));
  if (!rc && *dim_num == 0) {  // scalars: the slice is the tensor
    rc = insert ? io.in(slice, 1, &ds) : io.in(tens, 1, &dt);
    if (!rc) rc = insert ? io.out(tens, 1, false, false, &dt) : io.out(slice, 1, false, false, &ds);
    if (!rc && cudaMemcpyAsync(insert ? dt : ds, insert ? ds : dt, sizeof(double), cudaMemcpyDeviceToDevice,
                               io.s) != cudaSuccess)
      rc = cuda_fail(cudaGetLastError(), "cudaMemcpyAsync");
  } else if (!rc) {
    rc = insert ? io.in(slice, ns, &ds) : io.in(tens, nt, &dt);
    if (!rc) rc = insert ? io.out(tens, nt, true, false, &dt) : io.out(slice, ns, false, false, &ds);
    if (!rc) rc = launch_slice_insert(insert, *dim_num, dt, text, ds, sext, beg, io.s);
  }
  if (!rc) rc = io.finish();
  *ierr = rc == A4G_ERR_ARG ? 1 : runtime_ierr(rc);
}

void tensor_block_slice__(int* nthreads, int* dim_num, double* tens, int* tens_ext, double* slice,
                          int* slice_ext, int* ext_beg, int* ierr) {
  (void)nthreads;
  slice_insert_host(0, dim_num, tens, tens_ext, slice, slice_ext, ext_beg, ierr);
}

void tensor_block_insert__(int* nthreads, int* dim_num, double* tens, int* tens_ext, double* slice,
                           int* slice_ext, int* ext_beg, int* ierr) {
  (void)nthreads;
  slice_insert_host(1, dim_num, tens, tens_ext, slice, slice_ext, ext_beg, ierr);
}

void tensor_block_add__(const int* nthreads, const int* dim_num, int* ext, double* t0, double* t1,
                        const double* scale_fac, int* ierr) {
  (void)nthreads;
  if (*dim_num < 0 || !extents_ok(*dim_num, ext) || !t0 || !t1) return void(*ierr = -1);
  std::lock_guard<std::mutex> lock(g_host_mu);
  int rc = ensure_init();
  const int64_t n = count(*dim_num, ext);
  HostIO io;
  double *d0 = nullptr, *d1 = nullptr;
  if (!rc) rc = io.begin(2 * rounded(n));
  if (!rc) rc = io.in(t1, n, &d1);
  if (!rc) rc = io.out(t0, n, true, true, &d0);
  if (!rc) rc = launch_add_scaled(d0, d1, n, *scale_fac, io.s);
  if (!rc) rc = io.finish();
  *ierr = runtime_ierr(rc);
}

void tensor_block_copy__(int* nthreads, int* dim_num, int* ext, int* dim_transp, double* tin,
                         double* tout, int* ierr) {
  (void)nthreads;
  if (*dim_num < 0) return void(*ierr = *dim_num);
  if (!tin || !tout || !extents_ok(*dim_num, ext)) return void(*ierr = 1);
  std::lock_guard<std::mutex> lock(g_host_mu);
  int rc = ensure_init();
  const int64_t n = count(*dim_num, ext);
  HostIO io;
  double *din = nullptr, *dout = nullptr;
  if (!rc) rc = io.begin(2 * rounded(n));
  if (!rc) rc = io.in(tin, n, &din);
  if (!rc) rc = io.out(tout, n, false, false, &dout);
  if (!rc) rc = launch_permute(*dim_num, ext, dim_transp + 1, din, dout, io.s);
  if (!rc) rc = io.finish();
  *ierr = rc == A4G_ERR_ARG ? 1 : runtime_ierr(rc);
}

void tensor_block_contract__(int* nthreads, int* ptrn, double* ltens, int* lrank, int* lext,
                             double* rtens, int* rrank, int* rext, double* dtens, int* drank,
                             int* dext, int* ierr) {
  (void)nthreads;
  if (!(*lrank >= 0 && *lrank <= kMaxRank && *rrank >= 0 && *rrank <= kMaxRank && *drank >= 0 &&
        *drank <= kMaxRank))
    return void(*ierr = -1);
  if (!a4g::contr_ptrn_ok(ptrn, *lrank, *rrank, *drank, lext, rext, dext)) return void(*ierr = 1);
  if (!ltens || !rtens || !dtens || !extents_ok(*lrank, lext) || !extents_ok(*rrank, rext))
    return void(*ierr = 1);
  std::lock_guard<std::mutex> lock(g_host_mu);
  int rc = ensure_init();
  const int64_t nl = count(*lrank, lext), nr = count(*rrank, rext), nd = count(*drank, dext);
  HostIO io;
  double *dl = nullptr, *dr = nullptr, *dd = nullptr;
  if (!rc) rc = io.begin(rounded(nl) + rounded(nr) + rounded(nd) + rounded(dot_scratch_len()));
  if (!rc) rc = io.in(ltens, nl, &dl);
  if (!rc) rc = io.in(rtens, nr, &dr);
  if (!rc) rc = io.out(dtens, nd, false, false, &dd);
  if (!rc)
    rc = contract_device(ptrn, dl, *lrank, lext, dr, *rrank, rext, dd, *drank, dext, 0,
                         io.scratch(dot_scratch_len()), io.s);
  if (!rc) rc = io.finish();
  *ierr = rc == A4G_ERR_PATTERN ? 1 : runtime_ierr(rc);
}

// ============================================================ legacy GPU API
void _init_gpu(int* devid, int* myRank) {
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0) {
    *devid = -1;
    set_error("no CUDA device");
    return;
  }
  const int dev = (*myRank) % n;
  if (cudaSetDevice(dev) != cudaSuccess) {
    *devid = -1;
    set_error("cudaSetDevice failed");
    return;
  }
  *devid = dev;
  ensure_init();
}

void _gpu_axpy(double* y, double* x, const double alpha, const int numElems) {
  if (ensure_init()) return;
  if (!launch_axpy(y, x, numElems, alpha, ctx()->stream)) check_device_flag(ctx()->stream);
}

void _gpu_double_memset(double* g, double value, const int numElems) {
  if (ensure_init()) return;
  if (!launch_fill(g, numElems, value, ctx()->stream)) check_device_flag(ctx()->stream);
}

void _gpu_selfmultiply(double* x, const double alpha, const int numElems) {
  if (ensure_init()) return;
  if (!launch_scale(x, numElems, alpha, ctx()->stream)) check_device_flag(ctx()->stream);
}

void _gpu_contract(double* y, const int ny, const int* yDims, const int* yInds, double* x1,
                   const int n1, const int* x1Dims, const int* x1Inds, double* x2, const int n2,
                   const int* x2Dims, const int* x2Inds) {
  if (ensure_init()) return;
  a4g_contract_labels(yInds, x1Inds, x2Inds, x1, n1, x1Dims, x2, n2, x2Dims, y, ny, yDims, 0,
                      nullptr);
  check_device_flag(ctx()->stream);
}

void _gpu_permute(double* y, const int ny, const int* yDims, const int* yInds, double* x,
                  const int nx, const int* xDims, const int* xInds) {
  (void)yDims;
  if (ensure_init()) return;
  if (ny != nx) return set_error("_gpu_permute: rank mismatch");
  int o2n[kMaxRank + 1];
  o2n[0] = 1;
  if (!perm_from_labels(nx, yInds, xInds, o2n + 1)) return set_error("_gpu_permute: labels differ");
  if (!launch_permute(nx, xDims, o2n + 1, x, y, ctx()->stream)) check_device_flag(ctx()->stream);
}

void _gpu_host_to_device(double* c_addr, double* g_addr, const int numElems) {
  cudaError_t e = cudaMemcpy(g_addr, c_addr, size_t(numElems) * sizeof(double), cudaMemcpyHostToDevice);
  if (e != cudaSuccess) cuda_fail(e, "_gpu_host_to_device");
}

double* _gpu_allocate(const int numElems) {
  double* p = nullptr;
  cudaError_t e = cudaMalloc(&p, size_t(numElems > 0 ? numElems : 1) * sizeof(double));
  if (e != cudaSuccess) {
    cuda_fail(e, "_gpu_allocate");
    return nullptr;
  }
  e = cudaMemset(p, 0, size_t(numElems > 0 ? numElems : 1) * sizeof(double));
  if (e != cudaSuccess) cuda_fail(e, "_gpu_allocate memset");
  return p;
}

void _gpu_device_to_host(double* c_addr, double* g_addr, const int numElems) {
  cudaError_t e = cudaMemcpy(c_addr, g_addr, size_t(numElems) * sizeof(double), cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) cuda_fail(e, "_gpu_device_to_host");
}

void _gpu_device_to_device(double* dst, double* src, const int numElems) {
  cudaError_t e = cudaMemcpy(dst, src, size_t(numElems) * sizeof(double), cudaMemcpyDeviceToDevice);
  if (e != cudaSuccess) cuda_fail(e, "_gpu_device_to_device");
}

void _gpu_free(double* g_addr) {
  if (g_addr) cudaFree(g_addr);
}

// ============================================================ super instruction
int a4g_host_direct(int enable) {
  const int rc = ensure_init();
  if (rc) return rc;
  ctx()->host_direct = enable ? 1 : 0;
  return ctx()->host_access ? A4G_OK : A4G_ERR_UNSUPPORTED;
}

int a4g_set_predefined_int_array(const char* name, int n, const int* values) {
  if (!name || n < 0 || (n > 0 && !values)) return fail(A4G_ERR_ARG, "bad predefined array");
  std::lock_guard<std::mutex> lock(g_predef_mu);
  g_predefined[name] = std::vector<int>(values, values + n);
  return A4G_OK;
}

}  // extern "C"

// Orbital offsets of each block dimension (energy_denominator_rhf.F:57-88,
// 140-220): the sum of the segment sizes before the block's segment; for rank
// 6 an extent of 1 marks a simple index whose offset is its value - 1.
// Every orbital index the kernel will read is checked against the energy /
// Fock block here, on the host, so the device never reads out of bounds.
int a4g::denominator_offsets(int rank0, const int* iv, const int* ext0, int rank1, const int* ext1,
                             const std::vector<int>& segs, int* off) {
  const int norb = rank1 == 2 ? std::min(ext1[0], ext1[1]) : ext1[0];
  for (int q = 0; q < rank0; ++q) {
    off[q] = 0;
    if (ext0[q] <= 0) return fail(A4G_ERR_ARG, "non-positive extent");
    if (rank0 == 6 && ext0[q] == 1) {
      off[q] = iv[q] - 1;
    } else {
      for (int i = 1; i <= iv[q] - 1; ++i) {
        if (i > int(segs.size())) return fail(A4G_ERR_ARG, "segment number beyond moa_seg_ranges");
        off[q] += segs[i - 1];
      }
    }
    if (off[q] < 0 || off[q] + ext0[q] > norb)
      return fail(A4G_ERR_ARG, "block orbital range exceeds the orbital-energy array");
  }
  return A4G_OK;
}

extern "C" {

void energy_denominator_rhf(int* array_slot_0, int* rank_0, int* index_values_0, int* size_0,
                            int* extents_0, double* data_0, int* array_slot_1, int* rank_1,
                            int* index_values_1, int* size_1, int* extents_1, double* data_1,
                            int* ierr) {
  (void)array_slot_0, (void)array_slot_1, (void)index_values_1;
  *ierr = 0;
  const int r0 = *rank_0, r1 = *rank_1;
  // the reference acts only on these rank combinations and leaves data untouched otherwise
  if (!((r0 == 2 || r0 == 4) && (r1 == 1 || r1 == 2)) && !(r0 == 6 && r1 == 2)) return;
  std::vector<int> segs;
  {
    std::lock_guard<std::mutex> lock(g_predef_mu);
    auto it = g_predefined.find("moa_seg_ranges");
    if (it == g_predefined.end()) {
      set_error("energy_denominator_rhf: predefined array moa_seg_ranges not registered");
      *ierr = 1;
      return;
    }
    segs = it->second;
  }
  int off[6];
  if (denominator_offsets(r0, index_values_0, extents_0, r1, extents_1, segs, off))
    return void(*ierr = 1);
  std::lock_guard<std::mutex> lock(g_host_mu);
  int rc = ensure_init();
  const int64_t n0 = count(r0, extents_0), n1 = count(r1, extents_1);
  (void)size_0, (void)size_1;
  HostIO io;
  double *d0 = nullptr, *d1 = nullptr;
  if (!rc) rc = io.begin(2 * (rounded(n0) + rounded(n1)));
  if (!rc) rc = io.in(data_1, n1, &d1);
  if (!rc) rc = io.out(data_0, n0, true, false, &d0);
  if (!rc) rc = launch_denominator(r0, off, extents_0, d0, r1, extents_1[0], d1, io.s);
  if (!rc) rc = io.finish();
  *ierr = runtime_ierr(rc);
}

// ============================================================ device API
int a4g_init(int device) {
  if (device >= 0) A4G_CUDA(cudaSetDevice(device));
  return ensure_init();
}

int a4g_sync(void* stream) {
  int rc = ensure_init();
  if (rc) return rc;
  return check_device_flag(pick(stream));
}

void* a4g_default_stream(void) {
  if (ensure_init()) return nullptr;
  return ctx()->stream;
}

int a4g_contract(const int* ptrn, const double* l, int lrank, const int* lext, const double* r,
                 int rrank, const int* rext, double* d, int drank, const int* dext, int beta,
                 void* stream) {
  int rc = ensure_init();
  if (rc) return rc;
  if (!l || !r || !d || !ptrn) return fail(A4G_ERR_ARG, "null pointer");
  double* scratch = reduction_scratch();
  if (!scratch) return fail(A4G_ERR_NOMEM, "reduction scratch");
  return contract_device(ptrn, l, lrank, lext, r, rrank, rext, d, drank, dext, beta ? 1 : 0,
                         scratch, pick(stream));
}

int a4g_contract_labels(const int* d_labels, const int* l_labels, const int* r_labels,
                        const double* l, int lrank, const int* lext, const double* r, int rrank,
                        const int* rext, double* d, int drank, const int* dext, int beta,
                        void* stream) {
  if (drank < 0 || lrank < 0 || rrank < 0 || drank + lrank + rrank > 3 * kMaxRank)
    return fail(A4G_ERR_ARG, "rank out of range");
  int aces[3 * kMaxRank], ptrn[2 * kMaxRank + 1];
  for (int i = 0; i < drank; ++i) aces[i] = d_labels[i];
  for (int i = 0; i < lrank; ++i) aces[drank + i] = l_labels[i];
  for (int i = 0; i < rrank; ++i) aces[drank + lrank + i] = r_labels[i];
  const int ierr = a4g::get_contraction_ptrn(drank, lrank, rrank, aces, ptrn);
  if (ierr) return fail(A4G_ERR_PATTERN, "get_contraction_ptrn ierr " + std::to_string(ierr));
  return a4g_contract(ptrn, l, lrank, lext, r, rrank, rext, d, drank, dext, beta, stream);
}

int a4g_permute(int rank, const int* ext, const int* dim_transp, const double* in, double* out,
                void* stream) {
  int rc = ensure_init();
  if (rc) return rc;
  return launch_permute(rank, ext, dim_transp + 1, in, out, pick(stream));
}

int a4g_fill(double* d, int64_t n, double v, void* stream) {
  int rc = ensure_init();
  return rc ? rc : launch_fill(d, n, v, pick(stream));
}
int a4g_scale(double* d, int64_t n, double f, void* stream) {
  int rc = ensure_init();
  return rc ? rc : launch_scale(d, n, f, pick(stream));
}
int a4g_scale_copy(double* d, const double* s, int64_t n, double f, void* stream) {
  int rc = ensure_init();
  return rc ? rc : launch_scale_copy(d, s, n, f, pick(stream));
}
int a4g_increment(double* d, int64_t n, double delta, void* stream) {
  int rc = ensure_init();
  return rc ? rc : launch_increment(d, n, delta, pick(stream));
}
int a4g_add_scaled(double* t0, const double* t1, int64_t n, double scale, void* stream) {
  int rc = ensure_init();
  return rc ? rc : launch_add_scaled(t0, t1, n, scale, pick(stream));
}

int a4g_add_sub(int subtract, int rank, const int* d_labels, const int* r_labels, const int* r_ext,
                double* d, const double* l, const double* r, void* stream) {
  int rc = ensure_init();
  if (rc) return rc;
  if (rank < 0 || rank > kMaxRank) return fail(A4G_ERR_ARG, "rank out of range");
  int o2n[kMaxRank];
  if (!perm_from_labels(rank, d_labels, r_labels, o2n))
    return fail(A4G_ERR_ARG, "incompatible indices for LHS and RHS");
  bool trivial = true;
  for (int i = 0; i < rank; ++i) trivial &= o2n[i] == i + 1;
  const int64_t n = count(rank, r_ext);
  cudaStream_t s = pick(stream);
  const char *rb = reinterpret_cast<const char*>(r), *db = reinterpret_cast<const char*>(d);
  const bool overlap = rb < db + n * sizeof(double) && db < rb + n * sizeof(double);
  if (!trivial && overlap) {
    // d[i,j] += d[j,i]: the right operand must be read before d is written,
    // as the reference does with its temporary block (interpreter.cpp:1919-1927)
    double* tmp = nullptr;
    if (const int rc_ = async_alloc(reinterpret_cast<void**>(&tmp), size_t(n) * sizeof(double), s)) return rc_;
    rc = launch_permute(rank, r_ext, o2n, r, tmp, s);
    int ident[kMaxRank];
    for (int i = 0; i < rank; ++i) ident[i] = i + 1;
    int dext[kMaxRank];
    for (int i = 0; i < rank; ++i) dext[o2n[i] - 1] = r_ext[i];
    if (!rc) rc = launch_add_sub_permuted(subtract, rank, dext, ident, d, l, tmp, s);
    cudaFreeAsync(tmp, s);
    return rc;
  }
  return launch_add_sub_permuted(subtract, rank, r_ext, o2n, d, l, r, s);
}

int a4g_norm2(const double* t, int64_t n, double* h_result, void* stream) {
  int rc = ensure_init();
  if (rc) return rc;
  double* scratch = reduction_scratch();
  if (!scratch) return fail(A4G_ERR_NOMEM, "reduction scratch");
  cudaStream_t s = pick(stream);
  double* out = scratch + dot_scratch_len();
  rc = launch_dot(t, t, nullptr, nullptr, n, out, scratch, dot_scratch_len(), s);
  if (rc) return rc;
  A4G_CUDA(cudaMemcpyAsync(h_result, out, sizeof(double), cudaMemcpyDeviceToHost, s));
  return check_device_flag(s);
}

int a4g_slice(int rank, const double* tens, const int* text, double* slice, const int* sext,
              const int* beg, void* stream) {
  int rc = ensure_init();
  return rc ? rc
            : launch_slice_insert(0, rank, const_cast<double*>(tens), text, slice, sext, beg,
                                  pick(stream));
}
int a4g_insert(int rank, double* tens, const int* text, const double* slice, const int* sext,
               const int* beg, void* stream) {
  int rc = ensure_init();
  return rc ? rc
            : launch_slice_insert(1, rank, tens, text, const_cast<double*>(slice), sext, beg,
                                  pick(stream));
}

int a4g_energy_denominator(int rank0, const int* iv, const int* ext0, double* data0, int rank1,
                           const int* ext1, const double* e, int nsegs, const int* segs,
                           void* stream) {
  int rc = ensure_init();
  if (rc) return rc;
  if (!((rank0 == 2 || rank0 == 4) && (rank1 == 1 || rank1 == 2)) && !(rank0 == 6 && rank1 == 2))
    return fail(A4G_ERR_UNSUPPORTED, "energy denominator: unsupported rank combination");
  int off[6];
  rc = denominator_offsets(rank0, iv, ext0, rank1, ext1, std::vector<int>(segs, segs + nsegs), off);
  if (rc) return rc;
  return launch_denominator(rank0, off, ext0, data0, rank1, ext1[0], e, pick(stream));
}

int a4g_update_t2(const int* iv, const int* ext, const double* t2new, const double* t2new_pair,
                  const double* t2old, const double* t2old_pair, double* diis_err, double* t2old_next, int rank1,
                  const int* ext1, const double* e_or_fock, int nsegs, const int* segs, double* norm2,
                  void* stream) {
  int rc = ensure_init();
  if (rc) return rc;
  if (!iv || !ext || !t2new || !t2new_pair || !t2old || !t2old_pair || !t2old_next || !ext1 || !e_or_fock ||
      (nsegs > 0 && !segs))
    return fail(A4G_ERR_ARG, "amplitude update: null argument");
  if (rank1 != 1 && rank1 != 2) return fail(A4G_ERR_UNSUPPORTED, "amplitude update: energies must be rank 1 or 2");
  const int64_t n = int64_t(ext[0]) * ext[1] * ext[2] * ext[3];
  auto overlaps = [n](const double* x, const double* y) { return x && y && x < y + n && y < x + n; };
  for (const double* in : {t2new, t2new_pair, t2old, t2old_pair})
    if (overlaps(in, t2old_next) || overlaps(in, diis_err))
      return fail(A4G_ERR_ARG, "amplitude update: outputs must not overlap the inputs");
  if (overlaps(diis_err, t2old_next)) return fail(A4G_ERR_ARG, "amplitude update: outputs overlap");
  int off[6];
  rc = denominator_offsets(4, iv, ext, rank1, ext1, std::vector<int>(segs, segs + std::max(nsegs, 0)), off);
  if (rc) return rc;
  double* scratch = reduction_scratch();
  if (!scratch) return fail(A4G_ERR_NOMEM, "reduction scratch");
  return launch_update_t2(off, ext, t2new, t2new_pair, t2old, t2old_pair, diis_err, t2old_next, rank1, ext1[0],
                          e_or_fock, norm2, scratch, dot_scratch_len(), pick(stream));
}

int a4g_selftest_wait_timeout(int limit_ms, int* waited_ms, void* stream) {
  int rc = ensure_init();
  if (rc) return rc;
  if (limit_ms < 1 || limit_ms > 5000 || !waited_ms) return fail(A4G_ERR_ARG, "wait self-test: limit 1..5000 ms");
  cudaStream_t s = pick(stream);
  if ((rc = oz_wait_timeout_selftest(limit_ms, waited_ms, s))) return rc;
  return check_device_flag(s);  // A4G_ERR_TIMEOUT when the wait gave up, as intended
}

int a4g_selftest_round(int n, const long long* v, const int* e2, const int* neg, double* out, void* stream) {
  int rc = ensure_init();
  if (rc) return rc;
  if (n < 0 || (n > 0 && (!v || !e2 || !neg || !out))) return fail(A4G_ERR_ARG, "rounding self-test: arguments");
  return oz_round_selftest(n, v, e2, neg, out, pick(stream));
}

int a4g_selftest_div(int n, const double* a, const double* b, double* out, void* stream) {
  int rc = ensure_init();
  if (rc) return rc;
  if (n < 0 || (n > 0 && (!a || !b || !out))) return fail(A4G_ERR_ARG, "division self-test: arguments");
  return oz_div_selftest(n, a, b, out, pick(stream));
}

int a4g_energy_contract(int rank0, const int* iv, const int* ext0, const double* data0, const int* den_order,
                        int rank1, const int* ext1, const double* e, int nsegs, const int* segs, double efact,
                        double* esum, void* stream) {
  int rc = ensure_init();
  if (rc) return rc;
  if (!iv || !ext0 || !data0 || !ext1 || !e || !esum || (nsegs > 0 && !segs))
    return fail(A4G_ERR_ARG, "energy contraction: null argument");
  if (!((rank0 == 2 || rank0 == 4) && (rank1 == 1 || rank1 == 2)) && !(rank0 == 6 && rank1 == 2))
    return fail(A4G_ERR_UNSUPPORTED, "energy contraction: unsupported rank combination");
  int pos[6];
  bool seen[6] = {false, false, false, false, false, false};
  for (int q = 0; q < rank0; ++q) {
    pos[q] = den_order ? den_order[q] : q;
    if (pos[q] < 0 || pos[q] >= rank0 || seen[pos[q]])
      return fail(A4G_ERR_ARG, "energy contraction: den_order is not a permutation");
    seen[pos[q]] = true;
  }
  int off[6];
  rc = denominator_offsets(rank0, iv, ext0, rank1, ext1, std::vector<int>(segs, segs + std::max(nsegs, 0)), off);
  if (rc) return rc;
  double* scratch = reduction_scratch();
  if (!scratch) return fail(A4G_ERR_NOMEM, "reduction scratch");
  return launch_energy_contract(rank0, off, ext0, pos, data0, rank1, ext1[0], e, efact, esum, scratch,
                                dot_scratch_len(), pick(stream));
}

}  // extern "C"
