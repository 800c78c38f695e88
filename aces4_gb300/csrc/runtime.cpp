// Runtime support: error reporting, the process context, the contraction
// pattern planner and the device plan cache.
#include <algorithm>
#include <cstring>
#include <mutex>
#include <unordered_map>

#include "a4g_internal.h"

namespace a4g {

// ------------------------------------------------------------------ errors
static thread_local std::string g_last_error;

void set_error(const std::string& msg) { g_last_error = msg; }
void clear_error() { g_last_error.clear(); }
const char* last_error_text() { return g_last_error.c_str(); }
int fail(int code, const std::string& msg) {
  g_last_error = msg;
  return code;
}
int cuda_fail(cudaError_t e, const char* what) {
  g_last_error = std::string(what) + ": " + cudaGetErrorName(e) + " (" + cudaGetErrorString(e) + ")";
  return e == cudaErrorMemoryAllocation ? A4G_ERR_NOMEM : A4G_ERR_CUDA;
}

// ------------------------------------------------------------------ context
static Context g_ctx;
static std::mutex g_mu;

Context* ctx() { return &g_ctx; }

int ensure_init() {
  if (g_ctx.device >= 0) return A4G_OK;
  std::lock_guard<std::mutex> lock(g_mu);
  if (g_ctx.device >= 0) return A4G_OK;
  int dev = 0;
  A4G_CUDA(cudaGetDevice(&dev));
  cudaDeviceProp prop;
  A4G_CUDA(cudaGetDeviceProperties(&prop, dev));
  if (prop.major < 10)
    return fail(A4G_ERR_UNSUPPORTED, "aces4_gb300 needs a Blackwell GPU (sm_103a); found sm_" +
                                         std::to_string(prop.major) + std::to_string(prop.minor));
  A4G_CUDA(cudaStreamCreateWithFlags(&g_ctx.stream, cudaStreamNonBlocking));
  A4G_CUDA(cudaMalloc(&g_ctx.d_error_flag, sizeof(int)));
  A4G_CUDA(cudaMemset(g_ctx.d_error_flag, 0, sizeof(int)));
  cudaMemPoolProps props{};
  props.allocType = cudaMemAllocationTypePinned;
  props.location.type = cudaMemLocationTypeDevice;
  props.location.id = dev;
  A4G_CUDA(cudaMemPoolCreate(&g_ctx.pool, &props));
  uint64_t keep = ~0ull;  // never hand freed memory back on synchronisation
  A4G_CUDA(cudaMemPoolSetAttribute(g_ctx.pool, cudaMemPoolAttrReleaseThreshold, &keep));
  g_ctx.num_sms = prop.multiProcessorCount;
  int pageable = 0, host_tables = 0;
  A4G_CUDA(cudaDeviceGetAttribute(&pageable, cudaDevAttrPageableMemoryAccess, dev));
  A4G_CUDA(cudaDeviceGetAttribute(&host_tables, cudaDevAttrPageableMemoryAccessUsesHostPageTables, dev));
  g_ctx.host_access = pageable == 1 && host_tables == 1;
  g_ctx.device = dev;
  return A4G_OK;
}

int async_alloc(void** p, size_t bytes, cudaStream_t s) {
  A4G_CUDA(cudaMallocFromPoolAsync(p, std::max<size_t>(bytes, 8), g_ctx.pool, s));
  return A4G_OK;
}

cudaStream_t pick(void* stream) {
  return stream ? reinterpret_cast<cudaStream_t>(stream) : g_ctx.stream;
}

int arena_reserve(size_t bytes, void** out) {
  if (bytes > g_ctx.arena_bytes) {
    if (g_ctx.arena) {
      cudaError_t e = cudaStreamSynchronize(g_ctx.stream);
      if (e != cudaSuccess) return cuda_fail(e, "cudaStreamSynchronize");
      cudaFree(g_ctx.arena);
      g_ctx.arena = nullptr;
      g_ctx.arena_bytes = 0;
    }
    size_t want = std::max<size_t>(bytes, size_t(64) << 20);
    A4G_CUDA(cudaMalloc(&g_ctx.arena, want));
    g_ctx.arena_bytes = want;
  }
  *out = g_ctx.arena;
  return A4G_OK;
}

int check_device_flag(cudaStream_t s) {
  A4G_CUDA(cudaStreamSynchronize(s));
  int flag = 0;
  A4G_CUDA(cudaMemcpy(&flag, g_ctx.d_error_flag, sizeof(int), cudaMemcpyDeviceToHost));
  if (flag) {
    A4G_CUDA(cudaMemset(g_ctx.d_error_flag, 0, sizeof(int)));
    return fail(A4G_ERR_TIMEOUT, "a device-side wait reached its iteration limit (code " +
                                     std::to_string(flag) + "); the kernel returned early");
  }
  return A4G_OK;
}

// o2n (1-based) from two label lists: source dim j goes to the destination
// dim i carrying the same label (permute_rhs_to_lhs, interpreter.cpp:2049-2084).
bool perm_from_labels(int rank, const int* dst_labels, const int* src_labels, int* o2n) {
  for (int j = 0; j < rank; ++j) o2n[j] = 0;
  for (int i = 0; i < rank; ++i) {
    int j = 0;
    while (j < rank && src_labels[j] != dst_labels[i]) ++j;
    if (j >= rank || o2n[j] != 0) return false;
    o2n[j] = i + 1;
  }
  return true;
}

// ------------------------------------------------------------------ planner
// Stable sort of 1-based item numbers by key; equal keys keep their order, as
// the reference's merge sort does (merge_sort_key_int_, tensor_dil_omp.F90:1183).
static void stable_sort_by_key(int n, const int* key, int* trn) {
  std::stable_sort(trn, trn + n, [key](int a, int b) { return key[a - 1] < key[b - 1]; });
}

int get_contraction_ptrn(int drank, int lrank, int rrank, const int* aces, int* my) {
  if (!(drank >= 0 && lrank >= 0 && rrank >= 0)) return 1;
  const int m = lrank + rrank, n = drank + m;
  if (n % 2 != 0) return 2;
  if (m <= 0) return drank > 0 ? 3 : 0;
  if (n > 3 * kMaxRank) return 1;
  int trn[3 * kMaxRank];
  for (int i = 0; i < n; ++i) trn[i] = i + 1;
  stable_sort_by_key(n, aces, trn);
  for (int i = 0; i + 1 < n; i += 2) {
    if (aces[trn[i] - 1] == aces[trn[i + 1] - 1]) {
      if (i > 0 && aces[trn[i] - 1] == aces[trn[i - 1] - 1]) return 5;
    } else {
      return 4;
    }
  }
  for (int i = 0; i + 1 < n; i += 2) {
    const int j = trn[i], k = trn[i + 1];
    if (j <= drank && k > drank) {
      my[k - drank - 1] = j;
    } else if (j > drank && j <= drank + lrank && k > drank + lrank) {
      my[j - drank - 1] = -(k - (drank + lrank));
      my[k - drank - 1] = -(j - drank);
    } else {
      return 6;
    }
  }
  return 0;
}

bool contr_ptrn_ok(const int* ptrn, int lr, int rr, int dr, const int* lext, const int* rext,
                   const int* dext) {
  const int jl = dr + lr + rr;
  if (jl <= 0) return true;
  int bus[3 * kMaxRank] = {0};
  for (int j0 = 1; j0 <= lr; ++j0) {
    const int j1 = ptrn[j0 - 1];
    if (j1 > 0 && j1 <= dr) {
      bus[j1 - 1]++;
      bus[dr + j0 - 1]++;
      if (lext[j0 - 1] != dext[j1 - 1]) return false;
    } else if (j1 < 0 && -j1 <= rr) {
      bus[dr + lr - j1 - 1]++;
      if (lext[j0 - 1] != rext[-j1 - 1]) return false;
    } else {
      return false;
    }
  }
  for (int j0 = lr + 1; j0 <= lr + rr; ++j0) {
    const int j1 = ptrn[j0 - 1];
    if (j1 > 0 && j1 <= dr) {
      bus[j1 - 1]++;
      bus[dr + j0 - 1]++;
      if (rext[j0 - lr - 1] != dext[j1 - 1]) return false;
    } else if (j1 < 0 && -j1 <= lr) {
      bus[dr - j1 - 1]++;
      if (rext[j0 - lr - 1] != lext[-j1 - 1]) return false;
    } else {
      return false;
    }
  }
  for (int j = 0; j < jl; ++j)
    if (bus[j] != 1) return false;
  return true;
}

// Enumerates a multi-index (first listed dimension fastest) and writes, for
// each linear position, the sum of index*stride for one or two operands.
static void fill_offsets(const std::vector<int>& exts, const std::vector<int64_t>& s1,
                         const std::vector<int64_t>& s2, std::vector<int64_t>& o1,
                         std::vector<int64_t>& o2) {
  int64_t n = 1;
  for (int e : exts) n *= e;
  o1.assign(n, 0);
  o2.assign(n, 0);
  std::vector<int> im(exts.size(), 0);
  int64_t a = 0, b = 0;
  for (int64_t i = 0; i < n; ++i) {
    o1[i] = a;
    o2[i] = b;
    for (size_t q = 0; q < exts.size(); ++q) {
      if (im[q] + 1 < exts[q]) {
        im[q]++;
        a += s1[q];
        b += s2[q];
        break;
      }
      a -= int64_t(im[q]) * s1[q];
      b -= int64_t(im[q]) * s2[q];
      im[q] = 0;
    }
  }
}

int build_gemm_plan(const int* ptrn, int lrank, const int* lext, int rrank, const int* rext,
                    int drank, const int* dext, GemmPlan* p) {
  if (lrank < 0 || lrank > kMaxRank || rrank < 0 || rrank > kMaxRank || drank < 0 ||
      drank > kMaxRank)
    return fail(A4G_ERR_ARG, "tensor rank out of range [0, 32]");
  if (!contr_ptrn_ok(ptrn, lrank, rrank, drank, lext, rext, dext))
    return fail(A4G_ERR_PATTERN, "contraction pattern rejected (contr_ptrn_ok)");
  for (int i = 0; i < lrank; ++i)
    if (lext[i] <= 0) return fail(A4G_ERR_ARG, "non-positive extent");
  for (int i = 0; i < rrank; ++i)
    if (rext[i] <= 0) return fail(A4G_ERR_ARG, "non-positive extent");
  if (drank > 0 && lrank > 0 && rrank > 0) p->kind = ContractKind::kTensorTensor;
  else if (drank == 0 && lrank > 0 && rrank > 0) p->kind = ContractKind::kFull;
  else if (drank > 0 && lrank > 0 && rrank == 0) p->kind = ContractKind::kRightScalar;
  else if (drank > 0 && lrank == 0 && rrank > 0) p->kind = ContractKind::kLeftScalar;
  else p->kind = ContractKind::kScalarScalar;

  std::vector<int64_t> ls(lrank), rs(rrank), ds(drank);
  int64_t s = 1;
  for (int i = 0; i < lrank; ++i) ls[i] = s, s *= lext[i];
  s = 1;
  for (int i = 0; i < rrank; ++i) rs[i] = s, s *= rext[i];
  s = 1;
  for (int i = 0; i < drank; ++i) ds[i] = s, s *= dext[i];

  // M: L's uncontracted dims in L order (destination strides from the pattern)
  std::vector<int> me, ne, ke;
  std::vector<int64_t> mL, mD, nR, nD, kL, kR;
  for (int j = 0; j < lrank; ++j)
    if (ptrn[j] > 0) me.push_back(lext[j]), mL.push_back(ls[j]), mD.push_back(ds[ptrn[j] - 1]);
  for (int j = 0; j < rrank; ++j)
    if (ptrn[lrank + j] > 0)
      ne.push_back(rext[j]), nR.push_back(rs[j]), nD.push_back(ds[ptrn[lrank + j] - 1]);
  // K: contracted pairs.  Order them so the operand whose unit-stride index is
  // contracted reads contiguously along k (R's order unless only L's first
  // index is contracted); the matrix product is the same for any order.
  const bool l_first_con = lrank > 0 && ptrn[0] < 0;
  const bool r_first_con = rrank > 0 && ptrn[lrank] < 0;
  if (l_first_con && !r_first_con) {
    for (int j = 0; j < lrank; ++j)
      if (ptrn[j] < 0) {
        const int rj = -ptrn[j] - 1;
        ke.push_back(lext[j]), kL.push_back(ls[j]), kR.push_back(rs[rj]);
      }
  } else {
    for (int j = 0; j < rrank; ++j)
      if (ptrn[lrank + j] < 0) {
        const int lj = -ptrn[lrank + j] - 1;
        ke.push_back(rext[j]), kR.push_back(rs[j]), kL.push_back(ls[lj]);
      }
  }
  fill_offsets(me, mL, mD, p->offLm, p->offDm);
  fill_offsets(ne, nR, nD, p->offRn, p->offDn);
  fill_offsets(ke, kL, kR, p->offLk, p->offRk);
  p->M = int64_t(p->offLm.size());
  p->N = int64_t(p->offRn.size());
  p->K = int64_t(p->offLk.size());
  p->a_kfast = p->K > 1 && p->offLk[1] == 1 && !(p->M > 1 && p->offLm[1] == 1);
  p->b_kfast = !(p->N > 1 && p->offRn[1] == 1) || (p->K > 1 && p->offRk[1] == 1);
  return A4G_OK;
}

static std::unordered_map<std::string, DevPlan*> g_plans;
static std::mutex g_plan_mu;

int get_dev_plan(const int* ptrn, int lrank, const int* lext, int rrank, const int* rext,
                 int drank, const int* dext, const DevPlan** out) {
  if (lrank < 0 || lrank > kMaxRank || rrank < 0 || rrank > kMaxRank || drank < 0 ||
      drank > kMaxRank)
    return fail(A4G_ERR_ARG, "tensor rank out of range [0, 32]");
  std::string key;
  key.reserve(4 * (3 + 2 * (lrank + rrank) + drank));
  auto put = [&key](int v) { key.append(reinterpret_cast<const char*>(&v), sizeof(int)); };
  put(lrank), put(rrank), put(drank);
  for (int i = 0; i < lrank + rrank; ++i) put(ptrn[i]);
  for (int i = 0; i < lrank; ++i) put(lext[i]);
  for (int i = 0; i < rrank; ++i) put(rext[i]);
  for (int i = 0; i < drank; ++i) put(dext[i]);
  std::lock_guard<std::mutex> lock(g_plan_mu);
  auto it = g_plans.find(key);
  if (it != g_plans.end()) {
    *out = it->second;
    return A4G_OK;
  }
  DevPlan* dp = new DevPlan();
  int rc = build_gemm_plan(ptrn, lrank, lext, rrank, rext, drank, dext, &dp->host);
  if (rc) {
    delete dp;
    return rc;
  }
  const GemmPlan& h = dp->host;
  const size_t n = h.offLm.size() + h.offLk.size() + h.offRk.size() + h.offRn.size() +
                   h.offDm.size() + h.offDn.size();
  std::vector<int64_t> all;
  all.reserve(n);
  for (auto* v : {&h.offLm, &h.offLk, &h.offRk, &h.offRn, &h.offDm, &h.offDn})
    all.insert(all.end(), v->begin(), v->end());
  cudaError_t e = cudaMalloc(&dp->d_tables, n * sizeof(int64_t));
  if (e == cudaSuccess)
    e = cudaMemcpy(dp->d_tables, all.data(), n * sizeof(int64_t), cudaMemcpyHostToDevice);
  if (e != cudaSuccess) {
    if (dp->d_tables) cudaFree(dp->d_tables);
    delete dp;
    return cuda_fail(e, "plan tables upload");
  }
  int64_t* q = dp->d_tables;
  dp->offLm = q, q += h.offLm.size();
  dp->offLk = q, q += h.offLk.size();
  dp->offRk = q, q += h.offRk.size();
  dp->offRn = q, q += h.offRn.size();
  dp->offDm = q, q += h.offDm.size();
  dp->offDn = q;
  g_plans.emplace(key, dp);
  *out = dp;
  return A4G_OK;
}

}  // namespace a4g
