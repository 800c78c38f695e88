// Device residency of host blocks (a4g_blocks_*): the GPU half of the
// reference's BlockManager (src/sip/dynamic_data/block_manager.cpp:291-446)
// with the Block status bits onGPU / dirtyOnHost / dirtyOnGPU
// (src/sip/dynamic_data/block.h:150-174).  A block is identified by its host
// data pointer (Block::data_, which the interpreter owns); its device copy is
// made on first use and kept, so consecutive operations on the same block do
// not cross the host link.  The lazy copies follow the reference's rules:
//   on device, read / update: copy in when there is no device copy or the
//     host copy is newer; update then marks the device copy newer;
//   on device, overwrite: no copy in (the whole block is about to be
//     replaced), the device copy becomes the newer one;
//   on host, read / update: copy back when the device copy is newer; update
//     then marks the host copy newer; overwrite on host: no copy back.
// A block newer on both sides is an error, as in the reference.  When the
// device copies would exceed the capacity, the least recently used ones are
// dropped (written back first when they are newer than the host).
#include <algorithm>
#include <iterator>
#include <map>
#include <mutex>

#include "a4g_internal.h"

struct a4g_blocks {
  struct Entry {
    double* h = nullptr;
    int64_t n = 0;
    double* d = nullptr;
    bool dirty_host = false;  // the host copy is newer than the device copy
    bool dirty_gpu = false;   // the device copy is newer than the host copy
    uint64_t last_use = 0;
  };
  std::mutex mu;
  size_t capacity = 0, used = 0;
  uint64_t clock = 0;
  std::map<uintptr_t, Entry> by_addr;  // keyed by host address
  int64_t h2d_bytes = 0, d2h_bytes = 0, evictions = 0;
};

namespace a4g {
namespace {

std::mutex g_attach_mu;
a4g_blocks* g_attached = nullptr;

size_t bytes_of(int64_t n) { return size_t(n) * sizeof(double); }

int write_back(a4g_blocks* c, a4g_blocks::Entry& e, cudaStream_t s) {
  if (!e.dirty_gpu) return A4G_OK;
  A4G_CUDA(cudaMemcpyAsync(e.h, e.d, bytes_of(e.n), cudaMemcpyDeviceToHost, s));
  A4G_CUDA(cudaStreamSynchronize(s));
  c->d2h_bytes += int64_t(bytes_of(e.n));
  e.dirty_gpu = false;
  return A4G_OK;
}

int drop(a4g_blocks* c, std::map<uintptr_t, a4g_blocks::Entry>::iterator it, bool keep_data, cudaStream_t s) {
  a4g_blocks::Entry& e = it->second;
  if (keep_data) {
    const int rc = write_back(c, e, s);
    if (rc) return rc;
  }
  if (e.d) {
    A4G_CUDA(cudaFreeAsync(e.d, s));
    c->used -= bytes_of(e.n);
  }
  c->by_addr.erase(it);
  return A4G_OK;
}

// Room for `bytes` more: least recently used device copies go first.
int make_room(a4g_blocks* c, size_t bytes, const a4g_blocks::Entry* keep, cudaStream_t s) {
  while (c->used + bytes > c->capacity) {
    auto victim = c->by_addr.end();
    for (auto it = c->by_addr.begin(); it != c->by_addr.end(); ++it)
      if (it->second.d && &it->second != keep &&
          (victim == c->by_addr.end() || it->second.last_use < victim->second.last_use))
        victim = it;
    if (victim == c->by_addr.end()) return fail(A4G_ERR_NOMEM, "block cache: a block larger than the capacity");
    const int rc = drop(c, victim, true, s);
    if (rc) return rc;
    ++c->evictions;
  }
  return A4G_OK;
}

// The entry of block h (n doubles), created when missing.  A block must not
// overlap another one (each Block owns its data); a block registered with
// another size is a new block at a reused address.
int entry_of(a4g_blocks* c, double* h, int64_t n, a4g_blocks::Entry** out, cudaStream_t s) {
  const uintptr_t a = reinterpret_cast<uintptr_t>(h), end = a + bytes_of(n);
  auto it = c->by_addr.find(a);
  if (it != c->by_addr.end() && it->second.n != n) {
    const int rc = drop(c, it, false, s);
    if (rc) return rc;
    it = c->by_addr.end();
  }
  if (it == c->by_addr.end()) {
    auto nx = c->by_addr.lower_bound(a);
    if (nx != c->by_addr.end() && nx->first < end) return fail(A4G_ERR_ARG, "block cache: overlapping host blocks");
    if (nx != c->by_addr.begin()) {
      auto pv = std::prev(nx);
      if (pv->first + bytes_of(pv->second.n) > a) return fail(A4G_ERR_ARG, "block cache: overlapping host blocks");
    }
    a4g_blocks::Entry e;
    e.h = h, e.n = n;
    it = c->by_addr.emplace(a, e).first;
  }
  *out = &it->second;
  return A4G_OK;
}

}  // namespace

a4g_blocks* attached_blocks() {
  std::lock_guard<std::mutex> lock(g_attach_mu);
  return g_attached;
}

int blocks_on_device(a4g_blocks* c, double* h, int64_t n, int mode, double** d, cudaStream_t s) {
  std::lock_guard<std::mutex> lock(c->mu);
  a4g_blocks::Entry* e = nullptr;
  int rc = entry_of(c, h, n, &e, s);
  if (rc) return rc;
  if (e->dirty_host && e->dirty_gpu) return fail(A4G_ERR_ARG, "block cache: block newer on host and device");
  e->last_use = ++c->clock;
  const bool had = e->d != nullptr;
  if (!had) {
    if ((rc = make_room(c, bytes_of(n), e, s))) return rc;
    if (const int rc_ = async_alloc(reinterpret_cast<void**>(&e->d), std::max<size_t>(bytes_of(n), 8), s)) return rc_;
    c->used += bytes_of(n);
  }
  if (mode != A4G_BLOCK_OVERWRITE && (!had || e->dirty_host)) {
    A4G_CUDA(cudaMemcpyAsync(e->d, h, bytes_of(n), cudaMemcpyHostToDevice, s));
    c->h2d_bytes += int64_t(bytes_of(n));
  }
  e->dirty_host = false;
  if (mode != A4G_BLOCK_READ) e->dirty_gpu = true;
  *d = e->d;
  return A4G_OK;
}

}  // namespace a4g

using namespace a4g;

extern "C" {

int a4g_blocks_create(a4g_blocks** out, size_t capacity_bytes) {
  if (!out) return fail(A4G_ERR_ARG, "null output handle");
  *out = nullptr;
  const int rc = ensure_init();
  if (rc) return rc;
  a4g_blocks* c = new a4g_blocks();
  c->capacity = capacity_bytes;
  *out = c;
  return A4G_OK;
}

void a4g_blocks_destroy(a4g_blocks* c) {
  if (!c) return;
  {
    std::lock_guard<std::mutex> lock(g_attach_mu);
    if (g_attached == c) g_attached = nullptr;
  }
  cudaStream_t s = ctx()->stream;
  for (auto& kv : c->by_addr)
    if (kv.second.d) cudaFreeAsync(kv.second.d, s);
  cudaStreamSynchronize(s);
  delete c;
}

int a4g_blocks_on_device(a4g_blocks* c, double* h, int64_t n, int mode, double** d, void* stream) {
  if (!c || !h || !d || n <= 0) return fail(A4G_ERR_ARG, "block cache: bad argument");
  if (mode < A4G_BLOCK_READ || mode > A4G_BLOCK_OVERWRITE) return fail(A4G_ERR_ARG, "block cache: unknown mode");
  return blocks_on_device(c, h, n, mode, d, pick(stream));
}

int a4g_blocks_on_host(a4g_blocks* c, double* h, int mode, void* stream) {
  if (!c || !h) return fail(A4G_ERR_ARG, "block cache: bad argument");
  if (mode < A4G_BLOCK_READ || mode > A4G_BLOCK_OVERWRITE) return fail(A4G_ERR_ARG, "block cache: unknown mode");
  std::lock_guard<std::mutex> lock(c->mu);
  auto it = c->by_addr.find(reinterpret_cast<uintptr_t>(h));
  if (it == c->by_addr.end()) return A4G_OK;  // never on the device: the host copy is the block
  a4g_blocks::Entry& e = it->second;
  if (e.dirty_host && e.dirty_gpu) return fail(A4G_ERR_ARG, "block cache: block newer on host and device");
  if (mode == A4G_BLOCK_OVERWRITE) {
    e.dirty_gpu = false;
  } else {
    const int rc = write_back(c, e, pick(stream));
    if (rc) return rc;
  }
  if (mode != A4G_BLOCK_READ) e.dirty_host = true;
  return A4G_OK;
}

int a4g_blocks_flush(a4g_blocks* c, void* stream) {
  if (!c) return fail(A4G_ERR_ARG, "null block cache");
  std::lock_guard<std::mutex> lock(c->mu);
  cudaStream_t s = pick(stream);
  for (auto& kv : c->by_addr) {
    const int rc = write_back(c, kv.second, s);
    if (rc) return rc;
  }
  return A4G_OK;
}

int a4g_blocks_forget(a4g_blocks* c, double* h) {
  if (!c || !h) return fail(A4G_ERR_ARG, "block cache: bad argument");
  std::lock_guard<std::mutex> lock(c->mu);
  auto it = c->by_addr.find(reinterpret_cast<uintptr_t>(h));
  if (it == c->by_addr.end()) return A4G_OK;
  return drop(c, it, false, ctx()->stream);
}

int a4g_blocks_stats(a4g_blocks* c, int64_t* h2d_bytes, int64_t* d2h_bytes, int64_t* resident_bytes,
                     int64_t* evictions) {
  if (!c) return fail(A4G_ERR_ARG, "null block cache");
  std::lock_guard<std::mutex> lock(c->mu);
  if (h2d_bytes) *h2d_bytes = c->h2d_bytes;
  if (d2h_bytes) *d2h_bytes = c->d2h_bytes;
  if (resident_bytes) *resident_bytes = int64_t(c->used);
  if (evictions) *evictions = c->evictions;
  return A4G_OK;
}

int a4g_blocks_attach(a4g_blocks* c) {
  std::lock_guard<std::mutex> lock(g_attach_mu);
  g_attached = c;
  return A4G_OK;
}

}  // extern "C"
