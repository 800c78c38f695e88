// Batched (one pardo step) contraction: placeholder until the grouped kernel lands.
#include "a4g_internal.h"

using namespace a4g;

extern "C" {
int a4g_batch_create(a4g_batch** out, const int*, int, int, int, const a4g_triple*, int64_t,
                     const a4g_batch_opts*) {
  if (out) *out = nullptr;
  return fail(A4G_ERR_UNSUPPORTED, "batched contraction not built yet");
}
int a4g_batch_run(a4g_batch*, void*) { return fail(A4G_ERR_UNSUPPORTED, "not built"); }
int a4g_batch_run_graph(a4g_batch*, void*) { return fail(A4G_ERR_UNSUPPORTED, "not built"); }
int a4g_batch_info(const a4g_batch*, int64_t*, double*, int64_t*) {
  return fail(A4G_ERR_UNSUPPORTED, "not built");
}
void a4g_batch_destroy(a4g_batch*) {}
}
