// Launch tuning (fjg_get_tuning / fjg_set_tuning / fjg_autotune).
//
// The autotuner times the batch launcher on synthetic events: for each size
// bucket, a batch of events whose sizes are log-uniform over the bucket's
// range, run with every compiled kernel shape of that capacity and a few
// CTA-per-SM counts; for the tiled kernel, a batch of 5000-9000-particle
// events with a few tile sides.  The fastest choice of each is kept in the
// context.  Every choice computes identical results.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <vector>

#include "fjg_context.h"

using fjg::cuda_error;
using fjg::DeviceGuard;
using fjg::set_error;

namespace {

// Deterministic massless particles: pT 0.1 + Exp(0.7) GeV, eta U[-4, 4],
// phi U[0, 2pi) (the soft component of the synthetic events).
struct Rng {
  uint64_t s;
  double uniform() {
    s ^= s >> 12;
    s ^= s << 25;
    s ^= s >> 27;
    return (double)((s * 0x2545F4914F6CDD1Dull) >> 11) * (1.0 / 9007199254740992.0);
  }
};

void make_events(Rng& rng, int n_events, int lo, int hi, std::vector<double>& p4, std::vector<int64_t>& off) {
  p4.clear();
  off.assign(1, 0);
  const double llo = std::log((double)lo), lhi = std::log((double)hi + 1.0);
  for (int e = 0; e < n_events; ++e) {
    int n = (int)std::exp(llo + (lhi - llo) * rng.uniform());
    n = n < lo ? lo : (n > hi ? hi : n);
    for (int i = 0; i < n; ++i) {
      const double pt = 0.1 - 0.7 * std::log(1.0 - rng.uniform());
      const double eta = -4.0 + 8.0 * rng.uniform();
      const double phi = 6.283185307179586 * rng.uniform();
      const double px = pt * std::cos(phi), py = pt * std::sin(phi), pz = pt * std::sinh(eta);
      p4.push_back(px);
      p4.push_back(py);
      p4.push_back(pz);
      p4.push_back(std::sqrt(px * px + py * py + pz * pz));
    }
    off.push_back(off.back() + n);
  }
}

struct TuneBuffers {
  fjg::DeviceBuffer buf;
  double* p4 = nullptr;
  int64_t* off = nullptr;
  double* jets = nullptr;
  int32_t* lab = nullptr;
  int32_t* nj = nullptr;
  cudaError_t load(const std::vector<double>& hp4, const std::vector<int64_t>& hoff, cudaStream_t s) {
    const int64_t total = hoff.back();
    const int ne = (int)hoff.size() - 1;
    auto al = [](size_t x) { return (x + 255) & ~size_t(255); };
    const size_t b_p4 = al(sizeof(double) * 4 * total), b_off = al(sizeof(int64_t) * (ne + 1));
    const size_t b_jets = al(sizeof(double) * 4 * total), b_lab = al(sizeof(int32_t) * total);
    const size_t b_nj = al(sizeof(int32_t) * ne);
    cudaError_t err = buf.reserve(b_p4 + b_off + b_jets + b_lab + b_nj);
    if (err != cudaSuccess) return err;
    char* d = static_cast<char*>(buf.ptr);
    p4 = reinterpret_cast<double*>(d);
    off = reinterpret_cast<int64_t*>(d + b_p4);
    jets = reinterpret_cast<double*>(d + b_p4 + b_off);
    lab = reinterpret_cast<int32_t*>(d + b_p4 + b_off + b_jets);
    nj = reinterpret_cast<int32_t*>(d + b_p4 + b_off + b_jets + b_lab);
    err = cudaMemcpyAsync(p4, hp4.data(), sizeof(double) * hp4.size(), cudaMemcpyHostToDevice, s);
    if (err == cudaSuccess)
      err = cudaMemcpyAsync(off, hoff.data(), sizeof(int64_t) * hoff.size(), cudaMemcpyHostToDevice, s);
    if (err == cudaSuccess) err = cudaStreamSynchronize(s);
    return err;
  }
};

// Seconds per batch with tuning t (one untimed launch, then the best of two).
cudaError_t time_batch(fjg_ctx* ctx, const TuneBuffers& tb, int n_events, int64_t total, int algo, double r,
                       const fjg::Tuning& t, double* seconds) {
  fjg::BatchArgs A{};
  A.particles = total;
  A.p4 = tb.p4;
  A.p4_stride = 4;
  A.offsets = tb.off;
  A.algo_all = algo;
  A.r_all = r;
  A.jets = tb.jets;
  A.jet_label = tb.lab;
  A.n_jets = tb.nj;
  A.status = ctx->scratch.sc.status;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  cudaError_t err = cudaEventCreate(&e0);
  if (err == cudaSuccess) err = cudaEventCreate(&e1);
  double best = 1e30;
  for (int rep = 0; rep < 3 && err == cudaSuccess; ++rep) {
    err = cudaEventRecord(e0, ctx->stream);
    if (err == cudaSuccess)
      err = fjg::launch_batch(A, ctx->scratch.sc, n_events, ctx->num_sms, t, ctx->stream, ctx->side, &ctx->ev_fork,
                              ctx->ev_join);
    if (err == cudaSuccess) err = cudaEventRecord(e1, ctx->stream);
    if (err == cudaSuccess) err = cudaEventSynchronize(e1);
    float ms = 0.f;
    if (err == cudaSuccess) err = cudaEventElapsedTime(&ms, e0, e1);
    if (err == cudaSuccess && rep > 0 && ms * 1e-3 < best) best = ms * 1e-3;
  }
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  *seconds = best;
  (void)total;
  return err;
}

void to_public(const fjg::Tuning& t, const double* rate, fjg_tuning* out) {
  for (int b = 0; b < fjg::kNumBuckets; ++b) {
    const fjg::VariantShape sh = fjg::variant_shape(t.bucket[b].variant);
    out->threads[b] = sh.threads;
    out->slots_per_thread[b] = sh.spt;
    out->ctas_per_sm[b] = t.bucket[b].ctas_per_sm;
    out->events_per_s[b] = rate ? rate[b] : 0.0;
  }
  out->large_ctas_per_sm = t.large_ctas_per_sm;
  out->tile_factor = t.tile_factor;
}

}  // namespace

extern "C" {

fjg_status fjg_get_tuning(fjg_ctx* ctx, fjg_tuning* tuning) {
  if (!ctx || !tuning) return set_error(ctx, FJG_EINVAL, "null argument");
  to_public(ctx->tune, ctx->tuned_rate, tuning);
  return FJG_OK;
}

fjg_status fjg_set_tuning(fjg_ctx* ctx, const fjg_tuning* tuning) {
  if (!ctx || !tuning) return set_error(ctx, FJG_EINVAL, "null argument");
  fjg::Tuning t{};
  for (int b = 0; b < fjg::kNumBuckets; ++b) {
    int found = -1;
    for (int v = 0; v < fjg::kNumVariants; ++v) {
      const fjg::VariantShape sh = fjg::variant_shape(v);
      if (sh.threads == tuning->threads[b] && sh.spt == tuning->slots_per_thread[b]) found = v;
    }
    if (found < 0) return set_error(ctx, FJG_EINVAL, "no compiled kernel of that shape");
    t.bucket[b] = fjg::BucketConfig{found, tuning->ctas_per_sm[b]};
  }
  t.large_ctas_per_sm = tuning->large_ctas_per_sm;
  t.tile_factor = tuning->tile_factor;
  if (!fjg::tuning_valid(t)) return set_error(ctx, FJG_EINVAL, "tuning out of range");
  ctx->tune = t;
  for (int b = 0; b < fjg::kNumBuckets; ++b) ctx->tuned_rate[b] = tuning->events_per_s[b];
  return FJG_OK;
}

fjg_status fjg_autotune(fjg_ctx* ctx, int algo, double r, int flags, fjg_tuning* result) {
  if (!ctx) return set_error(nullptr, FJG_EINVAL, "ctx is null");
  if (!fjg::valid_algo(algo)) return set_error(ctx, FJG_EINVAL, "bad algorithm");
  if (!(r > 0.0)) return set_error(ctx, FJG_EINVAL, "R must be positive");
  DeviceGuard dg(ctx->device);
  Rng rng{0x9E3779B97F4A7C15ull};
  TuneBuffers tb;
  std::vector<double> hp4;
  std::vector<int64_t> hoff;
  fjg::Tuning best = ctx->tune;
  double rate[fjg::kNumBuckets] = {};
  cudaError_t err = cudaSuccess;
  for (int b = 0; b < fjg::kNumBuckets && err == cudaSuccess; ++b) {
    const int cap = 256 << b;
    const int lo = b == 0 ? 16 : cap / 2 + 1;
    int max_occ = 1;
    for (int v = 0; v < fjg::kNumVariants; ++v) {
      const fjg::VariantShape sh = fjg::variant_shape(v);
      if (sh.threads * sh.spt == cap) max_occ = std::max(max_occ, fjg::variant_occupancy(v));
    }
    const int n_events = 3 * ctx->num_sms * max_occ;
    make_events(rng, n_events, lo, cap, hp4, hoff);
    err = tb.load(hp4, hoff, ctx->stream);
    if (err == cudaSuccess) err = ctx->scratch.reserve_lists(n_events);
    if (err == cudaSuccess) err = ctx->scratch.reserve_ws(hoff.back());
    double best_s = 1e30;
    for (int v = 0; v < fjg::kNumVariants && err == cudaSuccess; ++v) {
      const fjg::VariantShape sh = fjg::variant_shape(v);
      if (sh.threads * sh.spt != cap) continue;
      const int occ = fjg::variant_occupancy(v);
      int counts[4] = {occ, occ / 2, 1, 2};
      for (int k = 0; k < 4 && err == cudaSuccess; ++k) {
        const int c = counts[k];
        if (c < 1 || c > occ) continue;
        bool seen = false;
        for (int q = 0; q < k; ++q) seen |= counts[q] == c;
        if (seen) continue;
        fjg::Tuning t = best;
        t.bucket[b] = fjg::BucketConfig{v, c};
        double sec = 0.0;
        err = time_batch(ctx, tb, n_events, hoff.back(), algo, r, t, &sec);
        if (err == cudaSuccess && sec < best_s) {
          best_s = sec;
          best.bucket[b] = t.bucket[b];
        }
      }
    }
    rate[b] = n_events / best_s;
  }
  // the tiled kernel sizes its tiles from each event's density (at least R):
  // no factor above 1 is better for every event size, so none is searched
  // (timed on events of 5000-9000 particles, 1.5-2 R won there and cost
  // large pile-up events half their speed)
  best.tile_factor = 1.0;
  (void)flags;
  if (err != cudaSuccess) return cuda_error(ctx, err, "autotune");
  int st = 0;
  err = cudaMemcpy(&st, ctx->scratch.sc.status, sizeof(int), cudaMemcpyDeviceToHost);
  if (err != cudaSuccess) return cuda_error(ctx, err, "autotune");
  if (st) {
    cudaMemset(ctx->scratch.sc.status, 0, sizeof(int));
    return fjg::status_to_error(ctx, st);
  }
  ctx->tune = best;
  for (int b = 0; b < fjg::kNumBuckets; ++b) ctx->tuned_rate[b] = rate[b];
  if (result) to_public(best, rate, result);
  return FJG_OK;
}

}  // extern "C"
