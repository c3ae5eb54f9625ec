// Clustering of one event per CTA (sm_103a), decision state in shared memory.
//
// Each CTA runs a persistent loop over a list of events.  Per slot (pseudojet):
//   shared memory (what every step reads; 36 bytes a slot, so several CTAs
//   share an SM and hide each other's serial latency):
//     FP32  rap32, phi32                  filter coordinates
//     FP32  wlo (+ int8 wx), nlo/nhi, klo/khi
//                                         intervals bracketing the exact FP64
//                                         weight, dR2 to the nearest neighbour,
//                                         and key
//     int16 nn (slot of the nearest neighbour), label (lowest constituent
//           index), rlist (rescan targets of a step)
//     int8  pair (the key is the pair distance, not the beam distance)
//   global workspace (L2-resident; read at merges and on the rare exact path):
//     FP64  rap, phi, w, px, py, pz, E    exact values
// Active pseudojets occupy slots [0, n); removing a slot moves the last active
// slot into the hole, so scans shrink with n.
//
// Lazy exactness.  GB300 runs FP64 at ~1/64 of the FP32 rate and charges a
// full warp slot per FP64 instruction, so decisions are taken on FP32
// intervals that provably contain the exact FP64 values; FP64 is evaluated
// only when two intervals overlap (near-ties) and for the winner's recorded
// distance.  The selection is the oracle's: argmin over (exact key, label).
//
// One clustering step (the reference launches two kernels per step over the
// full triangular matrix, tri_matrix.cu:316-328):
//   S1  argmin over (klo, label) with a certificate (klo of every other slot
//       above the winner's khi); otherwise an exact argmin among the
//       contenders.  One barrier (three on the rare exact path).
//   S2  the merge warps promote the winner, or merge it with its neighbour
//       (E-scheme, tri_matrix.cu:247-254): with two merge warps one computes
//       the azimuth and the history record, the other the rapidity and weight
//       and the compaction.  Meanwhile the other warps find the slots whose
//       neighbour was the winner or its partner and scan all slots for them
//       (named barrier), leaving per-warp certificates.  Barrier.
//   S3  every thread checks its slots against the new jet; the owners of the
//       rescanned slots finish their searches (adding the new jet as a
//       candidate); barrier; the new jet's owner warp finishes its search.
#pragma once

#include "fjg_device.cuh"

namespace fjg {

// Per-step phase counters, compiled in only with -DFJG_PHASE_CLOCKS (off in
// the product build; python -m fastjet_gpu_gb300.phases builds and reads
// them).  Thread 0 of a CTA accumulates the clock64() time of each phase of a
// step as it passes the phase's closing barrier (S1: argmin up to its
// decision; S2: merge up to B2; S3: new-jet pass and targets up to B3; tail:
// the new jet's neighbour up to the next step's start); lane 0 of each merge
// warp the length of its kinematics chain, and the first rescan thread the
// time of its S2 work.  At the end of an event they are added to A.phase.
enum PhaseSlot {
  kPhS1 = 0, kPhS2, kPhS3, kPhTail, kPhKin0, kPhKin1, kPhKin2, kPhRescan, kPhSteps, kPhEvents,
  // how often the FP32 intervals could not decide and FP64 was evaluated:
  // the argmin (steps), a slot's "is the new jet closer" test, a key's pair-or-
  // beam choice, a neighbour search's certificate (slot searches)
  kPhExactArgmin = 10, kPhExactCloser = 11, kPhExactKey = 22, kPhExactNN = 23,
  // the tiled kernel (events above 4096 particles): rebuild of the tile lists,
  // argmin, merge || target detection, lists + targets + the new jet's window
  // pass, the pass for targets beyond the listed ones, summaries + the new
  // jet's neighbour; the rapidity chain and the first detection thread's
  // merge-phase work
  kPhTRebuild = 12, kPhTS1, kPhTS2, kPhTS3a, kPhTS3b, kPhTS3c, kPhTKin, kPhTDetect, kPhTSteps, kPhTEvents,
  // the tiled kernel's targets: summed over steps, and steps that had any
  kPhTTargets = 24, kPhTTargetSteps,
  // inside the tiled kernel's S3 and S3c: thread 0's list update, warp 1's
  // targets, thread 0's share of the window pass; warp 0's resolution of the
  // new jet's neighbour and its tile's summary, warp 1's other summaries
  kPhTListUpd = 26, kPhTTargetsW1, kPhTWindowT0, kPhTResolveA, kPhTSumA, kPhTSumW1,
  kPhSlots = 32
};
#ifdef FJG_PHASE_CLOCKS
#define FJG_PH(...) __VA_ARGS__
#else
#define FJG_PH(...)
#endif

struct StepRec {
  int32_t a, b;
  double d;
};

// Exact per-slot fields of the global workspace.
enum WsField { kRap = 0, kPhi, kW, kPx, kPy, kPz, kE, kWsFields };

// Description of a batch, passed by value to the kernels.
struct BatchArgs {
  const double* p4;        // particle s of event e: p4 + (offsets[e] + s) * p4_stride
  int p4_stride;           // doubles between consecutive particles (4 for [n][4], 5 for PseudoJet AoS)
  const int64_t* offsets;  // [n_events + 1] (CSR), or [2 n_events] (start, end) pairs when pairs != 0
  const int32_t* algo;     // [n_events] or null
  const double* radius;    // [n_events] or null
  int algo_all;
  double r_all;
  const int32_t* order;    // events for this kernel, in processing order
  const int32_t* n_order;  // device count of entries in order
  int* queue;              // device work counter (zeroed before launch)
  double* ws;              // workspace: field f of slot s of event e at ws[f * ws_stride + offsets[e] + s]
  int64_t ws_stride;       // >= total particles
  double* jets;            // [total][4]
  int32_t* jet_label;      // [total]
  int32_t* n_jets;         // [n_events]
  StepRec* history;        // [total] or null
  int32_t* owner;          // [total] or null
  int* status;             // device error flag (0 = ok)
  unsigned char* large_ws; // tiled-path workspace: event e at large_ws + 96 * offsets[e] (null: none)
  double tile_factor;      // tiled path: tile side >= tile_factor * R (>= 1)
  int serve_order;         // launch priority (host side): 0 largest events first, 1 smallest first
  int pairs;               // offsets hold (start, end) pairs: events need not be contiguous
  int* done;               // null, or completion flags: done[done_slot[e]] = 1 (system scope) per event
  const int32_t* done_slot;
  int32_t* ev_status;      // null, or per-event status bits: an event whose word is set on entry is
                           // skipped (refused, no jets); bits a kernel raises for event e land here too
  unsigned long long* phase;  // [kPhSlots] phase counters (FJG_PHASE_CLOCKS builds only), or null
  int64_t particles;       // batch launcher: particles of the p4 buffer (the caller's `total`); the input
                           // check refuses events that reach past it and reads no momentum beyond it
};

// Status bits raised by kernels (ORed into the device status word).
enum : int { kStatusTooBig = 1, kStatusBadArg = 2, kStatusInternal = 4 };

// Particle range [off, off + N) of event e.
__device__ __forceinline__ void event_range(const BatchArgs& A, int e, int64_t& off, int& N) {
  if (A.pairs) {
    off = A.offsets[2 * (int64_t)e];
    N = (int)(A.offsets[2 * (int64_t)e + 1] - off);
  } else {
    off = A.offsets[e];
    N = (int)(A.offsets[e + 1] - off);
  }
}

// After the last write of event e (call after a block barrier, one thread):
// make the event's outputs visible system-wide, then raise its flag.
__device__ __forceinline__ void signal_done(const BatchArgs& A, int e) {
  if (!A.done) return;
  __threadfence_system();
  int* flag = A.done + A.done_slot[e];
  asm volatile("st.release.sys.global.u32 [%0], %1;" ::"l"(flag), "r"(1) : "memory");
}

// Raise status `bit` for event e: in the batch's word and, when the caller
// keeps per-event words (the request server), in the event's own, so that
// only that event's request fails.
__device__ __forceinline__ void raise_event_status(const BatchArgs& A, int e, int bit) {
  atomicOr(A.status, bit);
  if (A.ev_status) atomicOr(A.ev_status + e, bit);
}

// An event refused before clustering (its per-event word is set): no jets.
// Called by every thread of the CTA after the event was fetched; ends with a
// barrier, as the clustering routines do.
__device__ __forceinline__ bool refused_event(const BatchArgs& A, int e) {
  if (!A.ev_status || *(volatile int32_t*)(A.ev_status + e) == 0) return false;
  if (threadIdx.x == 0) {
    A.n_jets[e] = 0;
    signal_done(A, e);
  }
  __syncthreads();
  return true;
}

constexpr int kRescanChunk = 8;  // targets per register pass
constexpr int kMaxTargets = 16;  // targets per step scanned during the merge

template <int T, int SPT>
struct SmemLayout {
  static constexpr int C = T * SPT;
  static constexpr int W = T / 32;
  // 36 B per slot, so that three CTAs of 2048 slots fit on an SM.  Slots,
  // neighbours and labels are below 4096 (int16).  The weight interval is
  // stored as its lower end and whether it is a single float (wx): the upper
  // end of a directed-rounding pair is the next float up otherwise.
  float rap32[C], phi32[C], wlo[C], nlo[C], nhi[C], klo[C], khi[C];
  int16_t nn[C], label[C], rlist[C];
  int8_t pair[C], wx[C];
  __device__ __forceinline__ float whi(int t) const {
    return wx[t] ? wlo[t] : __int_as_float(__float_as_int(wlo[t]) + 1);
  }
  __device__ __forceinline__ void set_w(int t, double w) {
    const float lo = fjk_to_f32(w, 1);
    wlo[t] = lo;
    wx[t] = fjk_to_f32(w, 2) == lo;
  }
  // reduction and control scratch
  Cert warg[W];
  int wlab[W], wnn[W], wpair[W];  // label, neighbour and kind of each warp's candidate
  Arg wexact[W];
  Cert wcert[W];
  Cert rcert[kMaxTargets][W];
  int n_rescan;
  int event;
  int ctl_njets;
#ifdef FJG_PHASE_CLOCKS
  unsigned ph_exact[4];  // exact-path counts of the event (argmin, closer, key, neighbour)
#endif
  double rap_max_w[W];
};

// Exact FP64 slot data of one event in the global workspace.
struct Ws {
  double* base;
  int64_t stride;
  __device__ __forceinline__ double& at(int f, int s) const { return base[f * stride + s]; }
};

// Interval of the key of a slot with weight interval [wlo, whi], neighbour
// weight interval [vlo, vhi] and neighbour distance interval [dlo, dhi];
// 1/R^2 interval [ilo, ihi].  Returns 1 = pair, 0 = beam, -1 = undecided (the
// FP64 evaluation decides).  The products are rounded outwards and widened by
// 2^-22 relative to cover the two FP64 roundings of the exact key
// (tri_matrix.cu:112 evaluates (min(w_i, w_j) * dR2) * one_over_r2).
__device__ __forceinline__ int key_interval(float wlo, float whi, float vlo, float vhi, float dlo, float dhi,
                                            float ilo, float ihi, float& klo, float& khi) {
  const float mlo = fminf(wlo, vlo), mhi = fminf(whi, vhi);
  const float plo = __fmul_rd(__fmul_rd(__fmul_rd(mlo, dlo), ilo), 0.99999976158142089844f);
  const float phi_ = __fmul_ru(__fmul_ru(__fmul_ru(mhi, dhi), ihi), 1.00000023841857910156f);
  if (phi_ < wlo) {
    klo = plo;
    khi = phi_;
    return 1;
  }
  if (plo >= whi) {
    klo = wlo;
    khi = whi;
    return 0;
  }
  return -1;
}

struct EventCtx {
  int N, algo;
  double inv_r2;
  float ilo, ihi;
  Bound bd;
  Ws g;
};

__device__ __forceinline__ double dr2_slots(const Ws& g, int s, int t) {
  return dr2_64(g.at(kRap, s), g.at(kPhi, s), g.at(kRap, t), g.at(kPhi, t));
}

// Set the key of slot t from its neighbour (or none) and the neighbour
// distance interval already stored; FP64 only when the intervals cannot decide
// between the pair and the beam distance.
template <int T, int SPT>
__device__ __forceinline__ void set_key(SmemLayout<T, SPT>& S, const EventCtx& X, int t) {
  const int nn = S.nn[t];
  if (nn < 0) {
    S.klo[t] = S.wlo[t];
    S.khi[t] = S.whi(t);
    S.pair[t] = 0;
    return;
  }
  float klo, khi;
  const int kind = key_interval(S.wlo[t], S.whi(t), S.wlo[nn], S.whi(nn), S.nlo[t], S.nhi[t], X.ilo, X.ihi, klo, khi);
  if (kind >= 0) {
    S.klo[t] = klo;
    S.khi[t] = khi;
    S.pair[t] = (int8_t)kind;
    return;
  }
  FJG_PH(atomicAdd(&S.ph_exact[2], 1u);)
  const double wt = X.g.at(kW, t);
  const double dp = pair_distance(wt, X.g.at(kW, nn), dr2_slots(X.g, t, nn), X.inv_r2);
  const bool is_pair = dp < wt;
  const double key = is_pair ? dp : wt;
  S.pair[t] = is_pair ? 1 : 0;
  S.klo[t] = fjk_to_f32(key, 1);
  S.khi[t] = fjk_to_f32(key, 2);
}

// The exact key of slot t (FP64), for tie resolution.  A beam key whose
// interval is a single float is that float (e.g. C/A, where every w is 1).
template <int T, int SPT>
__device__ __forceinline__ double exact_key(SmemLayout<T, SPT>& S, const EventCtx& X, int t) {
  if (!S.pair[t]) return S.klo[t] == S.khi[t] ? (double)S.klo[t] : X.g.at(kW, t);
  const int nn = S.nn[t];
  return pair_distance(X.g.at(kW, t), X.g.at(kW, nn), dr2_slots(X.g, t, nn), X.inv_r2);
}

// Resolve the nearest neighbour of slot t among [0, n) \ {t} from a combined
// certificate: returns the slot (or -1) and the dR2 interval.  All 32 lanes of
// the calling warp call.  When the certificate fails (near-tie), every
// candidate whose lower bound does not exceed the best upper bound is
// evaluated in FP64 and the exact minimum (dR2, label) wins.
template <int T, int SPT>
__device__ __forceinline__ int resolve_nn(SmemLayout<T, SPT>& S, const EventCtx& X, int t, int n, const Cert& c,
                                          float& lo_out, float& hi_out) {
  if (c.i1 < 0) {
    lo_out = hi_out = __int_as_float(0x7f800000);
    return -1;
  }
  if (cert_ok(c)) {
    lo_out = c.m1;
    hi_out = c.u1;
    return c.i1;
  }
  const int lane = threadIdx.x & 31;
  FJG_PH(if (lane == 0) atomicAdd(&S.ph_exact[3], 1u);)
  unsigned long long bk = ~0ull;
  int bl = 0x7fffffff, bi = -1;
  const float rt = S.rap32[t], pt = S.phi32[t];
  for (int u = lane; u < n; u += 32) {
    if (u == t) continue;
    float lo, hi;
    dr2_32(rt, pt, S.rap32[u], S.phi32[u], X.bd, lo, hi);
    if (lo <= c.u1) {
      const unsigned long long k = dbits(dr2_slots(X.g, t, u));
      if (arg_less(k, S.label[u], bk, bl)) {
        bk = k;
        bl = S.label[u];
        bi = u;
      }
    }
  }
  const Arg r = arg_warp(bk, bl, bi);
  const double d = __longlong_as_double((long long)r.key);
  lo_out = fjk_to_f32(d, 1);
  hi_out = fjk_to_f32(d, 2);
  return r.idx;
}

// Whole-warp nearest-neighbour search for slot t over [0, n) \ {t}.
template <int T, int SPT>
__device__ __forceinline__ int warp_nn_search(SmemLayout<T, SPT>& S, const EventCtx& X, int t, int n, float& lo,
                                              float& hi) {
  Cert c = cert_empty();
  const float rt = S.rap32[t], pt = S.phi32[t];
  for (int u = threadIdx.x & 31; u < n; u += 32) {
    if (u == t) continue;
    float l, h;
    dr2_32(rt, pt, S.rap32[u], S.phi32[u], X.bd, l, h);
    cert_add(c, l, h, u);
  }
  c = cert_warp(c);
  return resolve_nn<T, SPT>(S, X, t, n, c, lo, hi);
}

// One pass of the rescan warps over the final slots for up to K targets
// (rlist[base .. base+cnt)): per-warp certificates into rcert.  Final slot u's
// data sits in slot u, except u == b whose data is still in slot L; slot a (the
// new jet, being written) is skipped.
template <int K, int T, int SPT>
__device__ __forceinline__ void rescan_chunk(SmemLayout<T, SPT>& S, const EventCtx& X, int base, int cnt, int r0,
                                             int TR, int n_new, int a, int b, int L) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  Cert rc[K];
  int tgt[K];
  float rt[K], pt[K];
#pragma unroll
  for (int r = 0; r < K; ++r) {
    rc[r] = cert_empty();
    tgt[r] = (r < cnt) ? S.rlist[base + r] : -1;
    const int sr = (r < cnt) ? (tgt[r] == b ? L : tgt[r]) : 0;
    rt[r] = S.rap32[sr];
    pt[r] = S.phi32[sr];
  }
  for (int u = r0; u < n_new; u += TR) {
    if (u == a) continue;
    const int su = u == b ? L : u;
    const float ru = S.rap32[su], pu = S.phi32[su];
#pragma unroll
    for (int r = 0; r < K; ++r) {
      if (r < cnt && u != tgt[r]) {
        float lo, hi;
        dr2_32(rt[r], pt[r], ru, pu, X.bd, lo, hi);
        cert_add(rc[r], lo, hi, u);
      }
    }
  }
#pragma unroll
  for (int r = 0; r < K; ++r) {
    if (r < cnt) {
      const Cert wc = cert_warp(rc[r]);
      if (lane == 0) S.rcert[base + r][warp] = wc;
    }
  }
}

// Named barriers: 1 among the rescan warps, 2 among the merge warps.  The
// non-aligned form: the compiler does not see an inline-asm barrier as a
// point where a warp must reconverge, and the threads of a warp may reach it
// apart (after loops whose trip counts differ per thread), which the aligned
// form (bar.sync) does not allow.
__device__ __forceinline__ void named_sync(int id, int threads) {
  asm volatile("barrier.sync %0, %1;" ::"r"(id), "r"(threads) : "memory");
}

// Move slot `from` into slot `to` (shared state by lane 0, workspace fields by
// lanes 1..7 of the calling warp; every lane calls).
template <int T, int SPT>
__device__ __forceinline__ void move_slot_warp(SmemLayout<T, SPT>& S, const Ws& g, int to, int from) {
  const int lane = threadIdx.x & 31;
  if (lane == 0) {
    S.rap32[to] = S.rap32[from];
    S.phi32[to] = S.phi32[from];
    S.wlo[to] = S.wlo[from];
    S.wx[to] = S.wx[from];
    S.nlo[to] = S.nlo[from];
    S.nhi[to] = S.nhi[from];
    S.klo[to] = S.klo[from];
    S.khi[to] = S.khi[from];
    S.nn[to] = S.nn[from];
    S.label[to] = S.label[from];
    S.pair[to] = S.pair[from];
  } else if (lane <= kWsFields) {
    g.at(lane - 1, to) = g.at(lane - 1, from);
  }
}

// The new jet's rapidity chain (one lane): its four-momentum (E-scheme,
// tri_matrix.cu:247-252) and rapidity into slot a, and its label.
template <int T, int SPT>
__device__ __forceinline__ void merge_rapidity(SmemLayout<T, SPT>& S, const Ws& g, int a, double pxc, double pyc,
                                               double pzc, double Ec, double pxj, double pyj, double pzj, double Ej,
                                               int label) {
  const double px = __dadd_rn(pxc, pxj), py = __dadd_rn(pyc, pyj);
  const double pz = __dadd_rn(pzc, pzj), E = __dadd_rn(Ec, Ej);
  const double rap = fjk_rap(px, py, pz, E);
  g.at(kPx, a) = px;
  g.at(kPy, a) = py;
  g.at(kPz, a) = pz;
  g.at(kE, a) = E;
  g.at(kRap, a) = rap;
  S.rap32[a] = fjk_to_f32(rap, 0);
  S.label[a] = label;
}

template <int T, int SPT>
__device__ void cluster_event_smem(SmemLayout<T, SPT>& S, const BatchArgs& A, int e) {
  constexpr int W = T / 32;
  // merge warps: three from 256 threads up; two with 128, so that two warps
  // (not one) scan for the step's targets; one with 64
  constexpr int MW = (T >= 256) ? 3 : (T == 128 ? 2 : 1);
  constexpr int TR = T - 32 * MW;         // rescan threads
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  int64_t off;
  EventCtx X;
  event_range(A, e, off, X.N);
  X.algo = A.algo ? A.algo[e] : A.algo_all;
  const double R = A.radius ? A.radius[e] : A.r_all;
  X.inv_r2 = 1.0 / (R * R);
  X.ilo = fjk_to_f32(X.inv_r2, 1);
  X.ihi = fjk_to_f32(X.inv_r2, 2);
  X.g.base = A.ws + off;
  X.g.stride = A.ws_stride;
  const Ws& g = X.g;
  const int N = X.N;

  // ---- load and kinematics
  double rmax = 0.0;
  for (int k = 0; k < SPT; ++k) {
    const int s = tid + k * T;
    if (s >= N) break;
    const double* p = A.p4 + (off + s) * A.p4_stride;
    const double px = p[0], py = p[1], pz = p[2], E = p[3];
    const Kin kin = kinematics(px, py, pz, E, X.algo);
    g.at(kPx, s) = px;
    g.at(kPy, s) = py;
    g.at(kPz, s) = pz;
    g.at(kE, s) = E;
    g.at(kRap, s) = kin.rap;
    g.at(kPhi, s) = kin.phi;
    g.at(kW, s) = kin.w;
    S.rap32[s] = fjk_to_f32(kin.rap, 0);
    S.phi32[s] = fjk_to_f32(kin.phi, 0);
    S.set_w(s, kin.w);
    S.label[s] = s;
    rmax = fmax(rmax, fabs(kin.rap));
    if (A.owner) A.owner[off + s] = s;  // union-find parent by label
  }
  for (int o = 16; o; o >>= 1) rmax = fmax(rmax, __shfl_xor_sync(kFull, rmax, o));
  if (lane == 0) S.rap_max_w[warp] = rmax;
  if (tid == 0) {
    S.ctl_njets = 0;
    S.n_rescan = 0;
    FJG_PH(for (int k = 0; k < 4; ++k) S.ph_exact[k] = 0;)
  }
  __syncthreads();
  rmax = 0.0;
  for (int k = 0; k < W; ++k) rmax = fmax(rmax, S.rap_max_w[k]);
  X.bd = make_bound(rmax);

  // ---- initial nearest neighbours (each slot scans all others)
  for (int k = 0; k < SPT; ++k) {
    const int t = tid + k * T;
    if (t >= N) break;
    const float rt = S.rap32[t], pt = S.phi32[t];
    Cert c = cert_empty();
    for (int u = 0; u < N; ++u) {
      if (u == t) continue;
      float lo, hi;
      dr2_32(rt, pt, S.rap32[u], S.phi32[u], X.bd, lo, hi);
      cert_add(c, lo, hi, u);
    }
    int nn = c.i1;
    float nlo = c.m1, nhi = c.u1;
    if (nn >= 0 && !cert_ok(c)) {
      unsigned long long bk = ~0ull;
      int bl = 0x7fffffff;
      nn = -1;
      for (int u = 0; u < N; ++u) {
        if (u == t) continue;
        float lo, hi;
        dr2_32(rt, pt, S.rap32[u], S.phi32[u], X.bd, lo, hi);
        if (lo <= c.u1) {
          const unsigned long long du = dbits(dr2_slots(g, t, u));
          if (arg_less(du, S.label[u], bk, bl)) {
            bk = du;
            bl = S.label[u];
            nn = u;
          }
        }
      }
      const double d = __longlong_as_double((long long)bk);
      nlo = fjk_to_f32(d, 1);
      nhi = fjk_to_f32(d, 2);
    }
    S.nn[t] = nn;
    S.nlo[t] = nlo;
    S.nhi[t] = nhi;
  }
  __syncthreads();
  for (int k = 0; k < SPT; ++k) {
    const int t = tid + k * T;
    if (t >= N) break;
    set_key<T, SPT>(S, X, t);
  }
  __syncthreads();

  // ---- clustering steps
  int n = N;
  int step = 0;
  FJG_PH(long long ph_s1 = 0, ph_s2 = 0, ph_s3 = 0, ph_tail = 0, ph_kin = 0, ph_resc = 0, ph_b3 = 0;)
  while (n > 0) {
    FJG_PH(const long long ph0 = clock64(); if (step > 0) ph_tail += ph0 - ph_b3;)
    // S1: argmin over (klo, label) with a certificate.  The winner's neighbour
    // and kind travel with the reduction: once B1 is passed the merge warps
    // may overwrite the winner's slot (compaction) while other warps are still
    // deciding what to do.  The certificate's second-smallest bound m2 leaves
    // out the best candidate's mutual partner: two slots that are each other's
    // neighbour with pair keys hold the same exact key (the same FP64
    // expression of the same pair), and whichever of them is taken, the step
    // merges that pair, so their tie needs no FP64 resolution.
    Cert mine = cert_empty();
    int mlab = 0x7fffffff, mnn = -1, mpair = 0;
    for (int k = 0; k < SPT; ++k) {
      const int t = tid + k * T;
      if (t >= n) break;
      const float lo = S.klo[t];
      const int l = S.label[t];
      if (lo < mine.m1 || (lo == mine.m1 && l < mlab)) {
        const int tnn = S.nn[t], tpair = S.pair[t];
        const bool partners = tpair && mpair && tnn == mine.i1 && mnn == t;
        mine.m2 = partners ? mine.m2 : mine.m1;
        mine.m1 = lo;
        mine.u1 = S.khi[t];
        mine.i1 = t;
        mlab = l;
        mnn = tnn;
        mpair = tpair;
      } else {
        const bool partners = mpair && t == mnn && S.pair[t] && S.nn[t] == mine.i1;
        if (!partners) mine.m2 = fminf(mine.m2, lo);
      }
    }
    {
      // warp combine: smallest klo, then lowest label
      const unsigned mb = __reduce_min_sync(kFull, __float_as_uint(mine.m1));
      const bool at_min = __float_as_uint(mine.m1) == mb && mine.i1 >= 0;
      const unsigned lb = __reduce_min_sync(kFull, at_min ? (unsigned)mlab : 0xffffffffu);
      const unsigned ball = __ballot_sync(kFull, at_min && (unsigned)mlab == lb);
      const int src = ball ? __ffs(ball) - 1 : 0;
      Cert wc;
      wc.m1 = __uint_as_float(mb);
      wc.i1 = __shfl_sync(kFull, mine.i1, src);
      wc.u1 = __shfl_sync(kFull, mine.u1, src);
      if (!ball) wc.i1 = -1;
      const int wnn = __shfl_sync(kFull, mnn, src);
      const int wpair = __shfl_sync(kFull, mpair, src);
      const bool partners = ball && mpair && wpair && mnn == wc.i1 && wnn == mine.i1;
      const unsigned other = (ball && lane == src) ? __float_as_uint(mine.m2)
                                                   : __float_as_uint(partners ? mine.m2 : mine.m1);
      wc.m2 = __uint_as_float(__reduce_min_sync(kFull, other));
      if (lane == 0) {
        S.warg[warp] = wc;
        S.wlab[warp] = ball ? (int)lb : 0x7fffffff;
        S.wnn[warp] = wnn;
        S.wpair[warp] = wpair;
      }
    }
    __syncthreads();  // B1
    int c, cnn, cpair;
    float u1;
    bool certified;
    {
      const Cert x = (lane < W) ? S.warg[lane] : cert_empty();
      const int xl = (lane < W) ? S.wlab[lane] : 0x7fffffff;
      const int xnn = (lane < W) ? S.wnn[lane] : -1;
      const int xpair = (lane < W) ? S.wpair[lane] : 0;
      const unsigned mb = __reduce_min_sync(kFull, __float_as_uint(x.m1));
      const bool at_min = __float_as_uint(x.m1) == mb && x.i1 >= 0;
      const unsigned lb = __reduce_min_sync(kFull, at_min ? (unsigned)xl : 0xffffffffu);
      const unsigned ball = __ballot_sync(kFull, at_min && (unsigned)xl == lb);
      const int src = ball ? __ffs(ball) - 1 : 0;
      c = __shfl_sync(kFull, x.i1, src);
      if (!ball) c = -1;
      u1 = __shfl_sync(kFull, x.u1, src);
      cnn = __shfl_sync(kFull, xnn, src);
      cpair = __shfl_sync(kFull, xpair, src);
      const bool partners = ball && xpair && cpair && xnn == c && cnn == x.i1;
      const unsigned other = (ball && lane == src) ? __float_as_uint(x.m2)
                                                   : __float_as_uint(partners ? x.m2 : x.m1);
      const float m2 = __uint_as_float(__reduce_min_sync(kFull, other));
      certified = (c >= 0) && (u1 < m2);
    }
    if (!certified && c >= 0) {
      FJG_PH(if (tid == 0) ++S.ph_exact[0];)
      // near-tie (every thread takes this branch: same shared inputs): exact
      // keys of all slots whose klo does not exceed the winner's khi
      __syncthreads();  // everyone has read warg
      unsigned long long bk = ~0ull;
      int bl = 0x7fffffff, bi = -1, bnn = -1, bpair = 0;
      for (int k = 0; k < SPT; ++k) {
        const int t = tid + k * T;
        if (t >= n) break;
        if (S.klo[t] <= u1) {
          const unsigned long long kk = dbits(exact_key<T, SPT>(S, X, t));
          if (arg_less(kk, S.label[t], bk, bl)) {
            bk = kk;
            bl = S.label[t];
            bi = t;
            bnn = S.nn[t];
            bpair = S.pair[t];
          }
        }
      }
      const Arg wa = arg_warp(bk, bl, bi);
      const unsigned wball = __ballot_sync(kFull, bi == wa.idx && bi >= 0);
      const int wsrc = wball ? __ffs(wball) - 1 : 0;
      const int wnn = __shfl_sync(kFull, bnn, wsrc);
      const int wpair = __shfl_sync(kFull, bpair, wsrc);
      if (lane == 0) {
        S.wexact[warp] = wa;
        S.wnn[warp] = wnn;
        S.wpair[warp] = wpair;
      }
      __syncthreads();
      const Arg y = (lane < W) ? S.wexact[lane] : Arg{~0ull, 0x7fffffff, -1};
      const int ynn = (lane < W) ? S.wnn[lane] : -1;
      const int ypair = (lane < W) ? S.wpair[lane] : 0;
      const Arg win = arg_warp(y.key, y.label, y.idx);
      const unsigned yball = __ballot_sync(kFull, y.idx == win.idx && y.idx >= 0);
      const int ysrc = yball ? __ffs(yball) - 1 : 0;
      c = win.idx;
      cnn = __shfl_sync(kFull, ynn, ysrc);
      cpair = __shfl_sync(kFull, ypair, ysrc);
      __syncthreads();  // wexact, wnn, wpair may be reused in the next step
    }
    if (c < 0) {  // no candidate although n > 0: cannot happen for finite inputs
      if (tid == 0) raise_event_status(A, e, kStatusInternal);
      break;
    }

    // S2: decisions every thread takes from the same values
    FJG_PH(const long long ph1 = clock64(); ph_s1 += ph1 - ph0;)
    const bool pair = cpair != 0 && cnn >= 0;
    const int j = pair ? cnn : -1;
    const int a = pair ? min(c, j) : -1;
    const int b = pair ? max(c, j) : c;
    const int L = n - 1;
    const int n_new = n - 1;

    if (warp < MW) {
      // Merge warps.  With three: warp 0 computes the azimuth, warp 1 the
      // rapidity and four-momentum, warp 2 the weight and the history record
      // and then compacts (its chain is the shortest); with two, warp 0 takes
      // the azimuth and then warp 2's part; with one, warp 0 does all of it.
      // Everything read of slots c and j is read before barrier 2 (or before
      // the compaction): the compaction may overwrite one of those slots.
      const int role = (MW == 1) ? -1 : warp;
      double pxc = 0, pyc = 0, pzc = 0, Ec = 0, pxj = 0, pyj = 0, pzj = 0, Ej = 0;
      double rc = 0, fc = 0, wc = 0, rj = 0, fj = 0, wj = 0;
      int lc = 0, lj = 0;
      if (lane == 0) {
        pxc = g.at(kPx, c);
        pyc = g.at(kPy, c);
        pzc = g.at(kPz, c);
        Ec = g.at(kE, c);
        wc = g.at(kW, c);
        lc = S.label[c];
        if (pair) {
          pxj = g.at(kPx, j);
          pyj = g.at(kPy, j);
          pzj = g.at(kPz, j);
          Ej = g.at(kE, j);
          wj = g.at(kW, j);
          lj = S.label[j];
          rc = g.at(kRap, c);
          fc = g.at(kPhi, c);
          rj = g.at(kRap, j);
          fj = g.at(kPhi, j);
        }
      }
      __syncwarp();
      if (MW > 1) named_sync(2, 32 * MW);  // every merge warp holds its inputs
      FJG_PH(const long long pk0 = clock64();)
      const int lo_l = pair ? min(lc, lj) : lc, hi_l = max(lc, lj);
      const bool phi_role = role <= 0, rap_role = role == -1 || role == 1,
                 w_role = role == -1 || role == 2 || (MW == 2 && role == 0);
      if (pair) {
        const double px = __dadd_rn(pxc, pxj), py = __dadd_rn(pyc, pyj);
        if (lane == 0 && phi_role) {
          const double phi = fjk_phi(px, py);
          g.at(kPhi, a) = phi;
          S.phi32[a] = fjk_to_f32(phi, 0);
        }
        if (lane == 0 && rap_role) merge_rapidity<T, SPT>(S, g, a, pxc, pyc, pzc, Ec, pxj, pyj, pzj, Ej, lo_l);
        if (lane == 0 && w_role) {
          const double w = fjk_weight(px, py, X.algo);
          g.at(kW, a) = w;
          S.set_w(a, w);
          const double d = pair_distance(wc, wj, dr2_64(rc, fc, rj, fj), X.inv_r2);
          if (A.history) A.history[off + step] = StepRec{lo_l, hi_l, d};
          if (A.owner) A.owner[off + hi_l] = lo_l;
        }
      } else if (lane == 0 && w_role) {
        const int nj = S.ctl_njets;
        double* jo = A.jets + (off + nj) * 4;
        jo[0] = pxc;
        jo[1] = pyc;
        jo[2] = pzc;
        jo[3] = Ec;
        A.jet_label[off + nj] = lc;
        if (A.history) A.history[off + step] = StepRec{lc, -1, wc};
        if (A.owner) A.owner[off + lc] = -(nj + 1);
        S.ctl_njets = nj + 1;
      }
      FJG_PH(if (lane == 0) ph_kin += clock64() - pk0;)
      if (w_role) {
        __syncwarp();
        if (b != L) move_slot_warp<T, SPT>(S, g, b, L);  // compaction (never touches slot a)
      }
      __syncwarp();
    } else {
      // Rescan targets: final slots (slot L moves to b) whose neighbour was c or
      // j.  While the merge warps write slots a and b, these warps read
      // neither: data of final slot u is read from src(u) (= L for u == b), and
      // a is skipped.
      const int r0 = tid - 32 * MW;
      for (int u = r0; u < n_new; u += TR) {
        if (u == a) continue;
        const int nu = S.nn[u == b ? L : u];
        if (nu == c || (pair && nu == j)) {
          const int pos = atomicAdd(&S.n_rescan, 1);
          S.rlist[pos] = u;
        }
      }
      named_sync(1, TR);
      const int nr = min(S.n_rescan, kMaxTargets);
      for (int base = 0; base < nr; base += kRescanChunk) {
        const int cnt = min(kRescanChunk, nr - base);
        if (cnt == 1)
          rescan_chunk<1, T, SPT>(S, X, base, cnt, r0, TR, n_new, a, b, L);
        else if (cnt == 2)
          rescan_chunk<2, T, SPT>(S, X, base, cnt, r0, TR, n_new, a, b, L);
        else if (cnt <= 4)
          rescan_chunk<4, T, SPT>(S, X, base, cnt, r0, TR, n_new, a, b, L);
        else
          rescan_chunk<8, T, SPT>(S, X, base, cnt, r0, TR, n_new, a, b, L);
      }
      FJG_PH(if (r0 == 0) ph_resc += clock64() - ph1;)
    }
    __syncthreads();  // B2: new jet and compaction written, rescan partials ready
    FJG_PH(const long long ph2 = clock64(); ph_s2 += ph2 - ph1;)
    n = n_new;
    ++step;
    if (n == 0) break;
    const int nr_all = S.n_rescan;
    const int nr = min(nr_all, kMaxTargets);

    // S3: every slot against the new jet; finish the rescans
    Cert ca = cert_empty();
    float ra = 0.f, pa = 0.f;
    if (pair) {
      ra = S.rap32[a];
      pa = S.phi32[a];
    }
    for (int k = 0; k < SPT; ++k) {
      const int t = tid + k * T;
      if (t >= n) break;
      if (t == a) continue;
      int cn = S.nn[t];  // still in the numbering before this step
      const bool target = (cn == c || (pair && cn == j));
      float lo = 0.f, hi = 0.f;
      if (pair) {
        dr2_32(S.rap32[t], S.phi32[t], ra, pa, X.bd, lo, hi);
        cert_add(ca, lo, hi, t);
      }
      if (target) continue;
      if (cn == L) {
        cn = b;
        S.nn[t] = b;
      }
      if (!pair) continue;
      const float nlo = S.nlo[t], nhi = S.nhi[t];
      bool closer;
      float ulo = lo, uhi = hi;
      if (hi < nlo) {
        closer = true;
      } else if (lo > nhi) {
        closer = false;
      } else {
        FJG_PH(atomicAdd(&S.ph_exact[1], 1u);)
        const double da = dr2_slots(g, t, a);
        const double dc = dr2_slots(g, t, cn);
        closer = da < dc || (da == dc && S.label[a] < S.label[cn]);
        ulo = fjk_to_f32(da, 1);
        uhi = fjk_to_f32(da, 2);
      }
      if (closer) {
        S.nn[t] = a;
        S.nlo[t] = ulo;
        S.nhi[t] = uhi;
        set_key<T, SPT>(S, X, t);
      }
    }
    if (pair) {
      const Cert wc = cert_warp(ca);
      if (lane == 0) S.wcert[warp] = wc;
    }
    // finish the scanned targets: the owner warp combines the rescan warps'
    // partials with the new jet
    for (int r = 0; r < nr; ++r) {
      const int t = S.rlist[r];
      if (warp != (t % T) / 32) continue;
      Cert x = (lane >= MW && lane < W) ? S.rcert[r][lane] : cert_empty();
      if (pair && lane == 0) {
        float lo, hi;
        dr2_32(S.rap32[t], S.phi32[t], ra, pa, X.bd, lo, hi);
        cert_add(x, lo, hi, a);
      }
      x = cert_warp(x);
      float lo, hi;
      const int nn = resolve_nn<T, SPT>(S, X, t, n, x, lo, hi);
      if (tid == t % T) {
        S.nn[t] = nn;
        S.nlo[t] = lo;
        S.nhi[t] = hi;
        set_key<T, SPT>(S, X, t);
      }
    }
    // targets beyond one S2 pass (a slot is the neighbour of many others only
    // in degenerate inputs such as repeated particles): one warp each
    for (int r = kMaxTargets + warp; r < nr_all; r += W) {
      const int t = S.rlist[r];
      float lo, hi;
      const int nn = warp_nn_search<T, SPT>(S, X, t, n, lo, hi);
      if (lane == 0) {
        S.nn[t] = nn;
        S.nlo[t] = lo;
        S.nhi[t] = hi;
        set_key<T, SPT>(S, X, t);
      }
      __syncwarp();
    }
    __syncthreads();  // B3: the new jet's partials are ready
    FJG_PH(ph_b3 = clock64(); ph_s3 += ph_b3 - ph2;)
    if (pair && warp == (a % T) / 32) {
      Cert x = (lane < W) ? S.wcert[lane] : cert_empty();
      x = cert_warp(x);
      float lo, hi;
      const int nn = resolve_nn<T, SPT>(S, X, a, n, x, lo, hi);
      if (tid == a % T) {
        S.nn[a] = nn;
        S.nlo[a] = lo;
        S.nhi[a] = hi;
        set_key<T, SPT>(S, X, a);
      }
    }
    if (tid == 0) S.n_rescan = 0;
    // the next S1 reads keys written by their owner thread, or before B3
  }

  // ---- epilogue: jet count, and constituent ownership from the union-find
  // parents (owner[label] = parent label, or -(jet+1) once promoted)
  __syncthreads();
  if (tid == 0) A.n_jets[e] = S.ctl_njets;
  FJG_PH(if (A.phase) {
    if (tid == 0) {
      atomicAdd(A.phase + kPhS1, (unsigned long long)ph_s1);
      atomicAdd(A.phase + kPhS2, (unsigned long long)ph_s2);
      atomicAdd(A.phase + kPhS3, (unsigned long long)ph_s3);
      atomicAdd(A.phase + kPhTail, (unsigned long long)ph_tail);
      atomicAdd(A.phase + kPhSteps, (unsigned long long)step);
      atomicAdd(A.phase + kPhEvents, 1ull);
      atomicAdd(A.phase + kPhExactArgmin, (unsigned long long)S.ph_exact[0]);
      atomicAdd(A.phase + kPhExactCloser, (unsigned long long)S.ph_exact[1]);
      atomicAdd(A.phase + kPhExactKey, (unsigned long long)S.ph_exact[2]);
      atomicAdd(A.phase + kPhExactNN, (unsigned long long)S.ph_exact[3]);
    }
    if (warp < MW && lane == 0) atomicAdd(A.phase + kPhKin0 + warp, (unsigned long long)ph_kin);
    if (tid == 32 * MW) atomicAdd(A.phase + kPhRescan, (unsigned long long)ph_resc);
  })
  if (A.owner) {
    for (int s = tid; s < N; s += T) {
      int x = s, guard = 0;
      int v = A.owner[off + x];
      while (v >= 0 && v != x && guard < N) {
        x = v;
        v = A.owner[off + x];
        ++guard;
      }
      S.nn[s] = (v < 0) ? (-v - 1) : -1;
    }
    __syncthreads();
    for (int s = tid; s < N; s += T) A.owner[off + s] = S.nn[s];
  }
  __syncthreads();
}

}  // namespace fjg
