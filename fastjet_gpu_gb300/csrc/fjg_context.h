// Library context and the host-side helpers shared by the C ABI translation
// units (fjg_capi.cu, fjg_graph.cu, fjg_tune.cu).  Internal: not installed.
#pragma once

#include <cstdint>
#include <string>

#include <cuda_runtime.h>

#include "fastjet_gb300.h"
#include "fjg_kernels.cuh"

namespace fjg {

// A growable device allocation.  Growing synchronises the device first: the
// old buffer may still be in use by queued work.
struct DeviceBuffer {
  void* ptr = nullptr;
  size_t cap = 0;
  cudaError_t reserve(size_t bytes) {
    if (bytes <= cap) return cudaSuccess;
    if (ptr) {
      cudaDeviceSynchronize();
      cudaFree(ptr);
    }
    ptr = nullptr;
    cap = 0;
    size_t want = bytes + bytes / 4 + 256;
    cudaError_t err = cudaMalloc(&ptr, want);
    if (err == cudaSuccess) cap = want;
    return err;
  }
  void release() {
    if (ptr) cudaFree(ptr);
    ptr = nullptr;
    cap = 0;
  }
};

// Device scratch of one launch sequence: the event lists and counters, the
// FP64 workspace and the tiled kernel's workspace, with their buffers.
struct ScratchSet {
  Scratch sc{};
  DeviceBuffer lists, ws, large;
  cudaError_t reserve_lists(int n_events);         // order/counts/queues/status/hist (+ offsets1)
  cudaError_t reserve_ws(int64_t particles);       // kWsFields doubles per particle
  cudaError_t reserve_large(int64_t particles);    // only when particles > kSmemMaxN
  void release() {
    lists.release();
    ws.release();
    large.release();
    sc = Scratch{};
  }
};

struct DeviceGuard {
  int prev = -1;
  explicit DeviceGuard(int dev) {
    cudaGetDevice(&prev);
    if (prev != dev) cudaSetDevice(dev);
  }
  ~DeviceGuard() {
    int cur = -1;
    cudaGetDevice(&cur);
    if (prev >= 0 && cur != prev) cudaSetDevice(prev);
  }
};

bool valid_algo(int a);

}  // namespace fjg

struct fjg_ctx {
  int device = 0;
  int num_sms = 0;
  cudaStream_t stream = nullptr;
  cudaStream_t side[fjg::kNumQueues] = {};
  cudaEvent_t ev_fork = nullptr;
  cudaEvent_t ev_join[fjg::kNumQueues] = {};
  fjg::ScratchSet scratch;  // the context's own launches
  fjg::DeviceBuffer io;     // device copies for the host-memory entry points
  fjg::DeviceBuffer single; // outputs of fjg_cluster_pseudojets
  fjg::DeviceBuffer select_scratch;  // fjg_select_jets: sort keys of events with many jets
  fjg::Tuning tune = fjg::default_tuning();
  double tuned_rate[fjg::kNumBuckets] = {};
  std::string last_error;
  unsigned long long* phase = nullptr;  // [kPhSlots] phase counters (FJG_PHASE_CLOCKS builds only)
};

namespace fjg {

fjg_status set_error(fjg_ctx* ctx, fjg_status st, const std::string& msg);
fjg_status cuda_error(fjg_ctx* ctx, cudaError_t err, const char* what);
// Status word -> fjg_status (0 -> FJG_OK), with the matching message.
fjg_status status_to_error(fjg_ctx* ctx, int st);

}  // namespace fjg
