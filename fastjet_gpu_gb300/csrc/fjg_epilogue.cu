// Device-side epilogue of a clustered batch and event combination
// (fjg_select_jets, fjg_combine_events in fastjet_gb300.h).
//
// fjg_select_jets does on the device what the reference driver does on the
// host after every event (main.cc:309-327): keep the inclusive jets with
// pt^2 >= ptmin^2 and, optionally, order them by decreasing pt^2.  The
// reference uses std::sort, whose order among equal pt^2 is unspecified; here
// equal pt^2 are ordered by jet label (lowest constituent index), so the
// output is deterministic.  pt^2 = px*px + py*py is rounded as written.
//
// One CTA per event (grid-stride over events): a block-wide scan compacts
// the kept jets, a bitonic sort orders them in shared memory (events of up to
// kSelectSmem jets) or in a global scratch area (larger events).
//
// fjg_combine_events merges every k consecutive events of a CSR batch into
// one (the driver's --combine, main.cc:76-85 and 269): the particles of
// consecutive events are already contiguous, so only the offsets change.
#include <cstdint>

#include "fjg_context.h"

using fjg::cuda_error;
using fjg::DeviceGuard;
using fjg::set_error;

namespace {

constexpr int kSelectT = 256;
constexpr int kSelectSmem = 2048;  // jets sorted in shared memory

__device__ __forceinline__ bool sel_before(double pa, int la, double pb, int lb) {
  return pa > pb || (pa == pb && la < lb);
}

// Bitonic sort of P (a power of two) keys in (pt2, label, idx) arrays.
__device__ void bitonic(double* pt2, int* label, int* idx, int P) {
  for (int k = 2; k <= P; k <<= 1) {
    for (int j = k >> 1; j > 0; j >>= 1) {
      for (int i = threadIdx.x; i < P; i += blockDim.x) {
        const int l = i ^ j;
        if (l > i) {
          const bool up = (i & k) == 0;  // this pair sorts "before" first
          const bool swap = up ? sel_before(pt2[l], label[l], pt2[i], label[i])
                               : sel_before(pt2[i], label[i], pt2[l], label[l]);
          if (swap) {
            const double tp = pt2[i];
            pt2[i] = pt2[l];
            pt2[l] = tp;
            const int tl = label[i];
            label[i] = label[l];
            label[l] = tl;
            const int ti = idx[i];
            idx[i] = idx[l];
            idx[l] = ti;
          }
        }
      }
      __syncthreads();
    }
  }
}

__global__ void __launch_bounds__(kSelectT) k_select_jets(const double* jets, const int32_t* jet_label,
                                                           const int32_t* n_jets, const int64_t* offsets,
                                                           int n_events, double ptmin2, int sort,
                                                           double* out_jets, int32_t* out_label, int32_t* out_n,
                                                           double* g_pt2, int* g_label, int* g_idx) {
  __shared__ double s_pt2[kSelectSmem];
  __shared__ int s_label[kSelectSmem], s_idx[kSelectSmem];
  __shared__ int warp_sum[kSelectT / 32];
  __shared__ int s_total;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  for (int e = blockIdx.x; e < n_events; e += gridDim.x) {
    const int64_t off = offsets[e];
    const int nj = n_jets[e];
    // the selected jets' keys, in promotion order (block-wide scan, 256 at a time)
    if (tid == 0) s_total = 0;
    __syncthreads();
    const bool big = nj > kSelectSmem;
    double* kp = big ? g_pt2 + 2 * off : s_pt2;
    int* kl = big ? g_label + 2 * off : s_label;
    int* ki = big ? g_idx + 2 * off : s_idx;
    for (int base = 0; base < nj; base += kSelectT) {
      const int i = base + tid;
      double pt2 = 0.0;
      bool keep = false;
      if (i < nj) {
        const double px = jets[4 * (off + i)], py = jets[4 * (off + i) + 1];
        pt2 = __dadd_rn(__dmul_rn(px, px), __dmul_rn(py, py));
        keep = !(pt2 < ptmin2);
      }
      const unsigned ball = __ballot_sync(0xffffffffu, keep);
      if (lane == 0) warp_sum[warp] = __popc(ball);
      __syncthreads();
      int before = s_total;
      for (int w = 0; w < warp; ++w) before += warp_sum[w];
      if (keep) {
        const int p = before + __popc(ball & ((1u << lane) - 1));
        kp[p] = pt2;
        kl[p] = jet_label[off + i];
        ki[p] = i;
      }
      __syncthreads();
      if (tid == 0) {
        int t = 0;
        for (int w = 0; w < kSelectT / 32; ++w) t += warp_sum[w];
        s_total += t;
      }
      __syncthreads();
    }
    const int m = s_total;
    if (sort && m > 1) {
      // pad to a power of two P < 2 m with keys that sort last (a big event's
      // global area holds 2 nj >= P entries)
      int P = 1;
      while (P < m) P <<= 1;
      for (int i = m + tid; i < P; i += kSelectT) {
        kp[i] = -1.0;
        kl[i] = 0x7fffffff;
        ki[i] = -1;
      }
      __syncthreads();
      bitonic(kp, kl, ki, P);
    }
    __syncthreads();
    for (int k = tid; k < m; k += kSelectT) {
      const int i = ki[k];
      const double* src = jets + 4 * (off + i);
      double* dst = out_jets + 4 * (off + k);
      dst[0] = src[0];
      dst[1] = src[1];
      dst[2] = src[2];
      dst[3] = src[3];
      out_label[off + k] = kl[k];
    }
    if (tid == 0) out_n[e] = m;
    __syncthreads();
  }
}

__global__ void k_combine_offsets(const int64_t* offsets, int n_events, int k, int n_out, int64_t* out) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i <= n_out; i += gridDim.x * blockDim.x) {
    const int64_t src = (int64_t)i * k;
    out[i] = offsets[src < n_events ? src : n_events];
  }
}

}  // namespace

extern "C" {

fjg_status fjg_select_jets(fjg_ctx* ctx, const double* jets, const int32_t* jet_label, const int32_t* n_jets,
                           const int64_t* offsets, int n_events, int64_t total, double ptmin, int sort,
                           double* out_jets, int32_t* out_label, int32_t* out_n_jets, void* stream) {
  if (!ctx) return set_error(nullptr, FJG_EINVAL, "ctx is null");
  if (n_events < 0 || total < 0 || (n_events > 0 && (!jets || !jet_label || !n_jets || !offsets || !out_jets ||
                                                     !out_label || !out_n_jets)))
    return set_error(ctx, FJG_EINVAL, "bad arguments");
  if (!(ptmin >= 0.0)) return set_error(ctx, FJG_EINVAL, "ptmin must be >= 0");
  if (n_events == 0) return FJG_OK;
  DeviceGuard dg(ctx->device);
  // scratch for events with more jets than the shared-memory sort holds:
  // 2 entries per particle, so that an event's power-of-two padding fits
  const size_t cap = 2 * (size_t)(total > 0 ? total : 1);
  cudaError_t err = ctx->select_scratch.reserve(16 * cap + 256);
  if (err != cudaSuccess) return cuda_error(ctx, err, "scratch allocation");
  char* sp = static_cast<char*>(ctx->select_scratch.ptr);
  double* g_pt2 = reinterpret_cast<double*>(sp);
  int* g_label = reinterpret_cast<int*>(sp + 8 * cap);
  int* g_idx = g_label + cap;
  cudaStream_t s = stream ? (cudaStream_t)stream : ctx->stream;
  const int grid = n_events < 4 * ctx->num_sms ? n_events : 4 * ctx->num_sms;
  k_select_jets<<<grid, kSelectT, 0, s>>>(jets, jet_label, n_jets, offsets, n_events, ptmin * ptmin, sort ? 1 : 0,
                                          out_jets, out_label, out_n_jets, g_pt2, g_label, g_idx);
  err = cudaGetLastError();
  return err == cudaSuccess ? FJG_OK : cuda_error(ctx, err, "fjg_select_jets");
}

fjg_status fjg_combine_events(fjg_ctx* ctx, const int64_t* offsets, int n_events, int k, int64_t* out_offsets,
                              int* n_out, void* stream) {
  if (!ctx) return set_error(nullptr, FJG_EINVAL, "ctx is null");
  if (n_events < 0 || k < 0 || !n_out || (n_events > 0 && (!offsets || !out_offsets)))
    return set_error(ctx, FJG_EINVAL, "bad arguments");
  const int kk = (k == 0 || k > n_events) ? (n_events > 0 ? n_events : 1) : k;
  const int m = n_events == 0 ? 0 : (n_events + kk - 1) / kk;
  *n_out = m;
  if (n_events == 0) return FJG_OK;
  DeviceGuard dg(ctx->device);
  cudaStream_t s = stream ? (cudaStream_t)stream : ctx->stream;
  const int grid = (m + 1 + 255) / 256 > 1024 ? 1024 : (m + 1 + 255) / 256;
  k_combine_offsets<<<grid, 256, 0, s>>>(offsets, n_events, kk, m, out_offsets);
  cudaError_t err = cudaGetLastError();
  return err == cudaSuccess ? FJG_OK : cuda_error(ctx, err, "fjg_combine_events");
}

}  // extern "C"
