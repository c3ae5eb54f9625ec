// The reference's C++ entry point cluster() (cluster.h:6), implemented on the
// library's clustering path.  One lazily created context per device.
#include <cstdio>
#include <cstdlib>
#include <mutex>

#include <cuda_runtime.h>

#include "fastjet_gb300.h"
#include "fastjet_gb300_compat.h"

static_assert(sizeof(PseudoJet) == sizeof(fjg_pseudojet), "PseudoJet layout");

namespace {

std::mutex g_mu;
fjg_ctx* g_ctx[64] = {};

[[noreturn]] void fail(const char* what, const char* msg) {
  std::fprintf(stderr, "\nfastjet_gb300 cluster(): %s: %s\n", what, msg);
  std::abort();
}

}  // namespace

void cluster(PseudoJet *particles, int size, Algorithm algo, double r) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) fail("cudaGetDevice", "no usable CUDA device");
  fjg_ctx* ctx;
  {
    std::lock_guard<std::mutex> lock(g_mu);
    if (!g_ctx[dev]) {
      fjg_status st = fjg_ctx_create(dev, &g_ctx[dev]);
      if (st != FJG_OK) fail("context", fjg_last_error(nullptr));
    }
    ctx = g_ctx[dev];
  }
  // the reference driver's copies run on the legacy default stream; order after them
  fjg_status st = fjg_cluster_pseudojets(ctx, reinterpret_cast<fjg_pseudojet*>(particles), size,
                                         static_cast<int>(algo), r, (void*)cudaStreamLegacy);
  if (st != FJG_OK) fail(fjg_status_string(st), fjg_last_error(ctx));
}
