// Shared-memory-resident clustering of one event per CTA (sm_103a).
//
// Each CTA runs a persistent loop over a list of events; one event's whole
// state lives in shared memory as a structure of arrays over "slots":
//   FP64  rap, phi, w, nnd (dR2 to the nearest neighbour), key, px, py, pz, E
//   FP32  rap32, phi32 (filter copies), thr (nnd rounded up)
//   int32 nn (slot of the nearest neighbour), label (lowest constituent index)
// Active pseudojets occupy slots [0, n); removing a slot moves the last active
// slot into the hole, so scans shrink with n.  Thread t owns slots t, t+T, ...
//
// One clustering step (reference: tri_matrix.cu:316-328 runs it as two kernel
// launches over the full triangular matrix; n_array.cu:135-199 rescans all
// pairs):
//   1. argmin over (key, label): per-thread, warp redux, one barrier;
//   2. thread 0 promotes the winner or merges it with its neighbour (E-scheme,
//      tri_matrix.cu:247-254), recomputes kinematics, records history and
//      compacts; one barrier;
//   3. every thread checks its slots against the new jet (FP32 filter, exact
//      FP64 only for candidates), collects slots whose neighbour was merged and
//      accumulates the new jet's own neighbour search; one barrier;
//   4. the owner warp of the new jet certifies its neighbour; slots whose
//      neighbour disappeared are rescanned block-wide (one barrier per chunk of
//      targets).
#pragma once

#include "fjg_device.cuh"

namespace fjg {

struct StepRec {
  int32_t a, b;
  double d;
};

// Description of a batch, passed by value to the kernels.
struct BatchArgs {
  const double* p4;        // particle s of event e: p4 + (offsets[e] + s) * p4_stride
  int p4_stride;           // doubles between consecutive particles (4 for [n][4], 5 for PseudoJet AoS)
  const int64_t* offsets;  // [n_events + 1]
  const int32_t* algo;     // [n_events] or null
  const double* radius;    // [n_events] or null
  int algo_all;
  double r_all;
  const int32_t* order;    // events for this kernel, in processing order
  const int32_t* n_order;  // device count of entries in order
  int* queue;              // device work counter (zeroed before launch)
  double* jets;            // [total][4]
  int32_t* jet_label;      // [total]
  int32_t* n_jets;         // [n_events]
  StepRec* history;        // [total] or null
  int32_t* owner;          // [total] or null
  int* status;             // device error flag (0 = ok)
};

constexpr int kRescanChunk = 8;
constexpr int kMaxWarps = 32;

template <int T, int SPT>
struct SmemLayout {
  static constexpr int C = T * SPT;
  static constexpr int W = T / 32;
  double rap[C], phi[C], w[C], nnd[C], key[C], px[C], py[C], pz[C], E[C];
  float rap32[C], phi32[C], thr[C];
  int32_t nn[C], label[C];
  // control and reduction scratch
  Arg warg[W];
  Cert wcert[W];
  Cert rcert[kRescanChunk][W];
  int rlist[C];
  int n_rescan;
  int event;
  int ctl_a, ctl_b, ctl_L, ctl_pair, ctl_njets;
  double rap_max_w[W];
};

// Exact nearest neighbour of slot t among [0, n) \ {t}, from a warp-combined
// certificate; all 32 lanes of the calling warp must call.  Returns the slot
// (or -1) and its FP64 dR2.
template <int T, int SPT>
__device__ __forceinline__ int resolve_nn_warp(SmemLayout<T, SPT>& S, int t, int n, const Cert& c, const Bound& bd,
                                               double& d_out) {
  if (c.i1 < 0) {
    d_out = __longlong_as_double(0x7ff0000000000000LL);
    return -1;
  }
  if (cert_ok(c)) {
    d_out = dr2_64(S.rap[t], S.phi[t], S.rap[c.i1], S.phi[c.i1]);
    return c.i1;
  }
  // near-tie: every slot whose lower bound does not exceed the best upper bound
  const int lane = threadIdx.x & 31;
  unsigned long long bk = ~0ull;
  int bl = 0x7fffffff, bi = -1;
  const float rt = S.rap32[t], pt = S.phi32[t];
  for (int u = lane; u < n; u += 32) {
    if (u == t) continue;
    float lo, hi;
    dr2_32(rt, pt, S.rap32[u], S.phi32[u], bd, lo, hi);
    if (lo <= c.u1) {
      const double d = dr2_64(S.rap[t], S.phi[t], S.rap[u], S.phi[u]);
      const unsigned long long k = dbits(d);
      if (arg_less(k, S.label[u], bk, bl)) {
        bk = k;
        bl = S.label[u];
        bi = u;
      }
    }
  }
  const Arg r = arg_warp(bk, bl, bi);
  d_out = __longlong_as_double((long long)r.key);
  return r.idx;
}

template <int T, int SPT>
__device__ void cluster_event_smem(SmemLayout<T, SPT>& S, const BatchArgs& A, int e) {
  constexpr int W = T / 32;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int64_t off = A.offsets[e];
  const int N = (int)(A.offsets[e + 1] - off);
  const int algo = A.algo ? A.algo[e] : A.algo_all;
  const double R = A.radius ? A.radius[e] : A.r_all;
  const double inv_r2 = 1.0 / (R * R);

  // ---- load and kinematics
  double rmax = 0.0;
  for (int k = 0; k < SPT; ++k) {
    const int s = tid + k * T;
    if (s >= N) break;
    const double* p = A.p4 + (off + s) * A.p4_stride;
    const double px = p[0], py = p[1], pz = p[2], E = p[3];
    const Kin kin = kinematics(px, py, pz, E, algo);
    S.px[s] = px;
    S.py[s] = py;
    S.pz[s] = pz;
    S.E[s] = E;
    S.rap[s] = kin.rap;
    S.phi[s] = kin.phi;
    S.w[s] = kin.w;
    S.rap32[s] = __double2float_rn(kin.rap);
    S.phi32[s] = __double2float_rn(kin.phi);
    S.label[s] = s;
    rmax = fmax(rmax, fabs(kin.rap));
    if (A.owner) A.owner[off + s] = s;  // union-find parent by label
  }
  for (int o = 16; o; o >>= 1) rmax = fmax(rmax, __shfl_xor_sync(kFull, rmax, o));
  if (lane == 0) S.rap_max_w[warp] = rmax;
  __syncthreads();
  rmax = 0.0;
  for (int k = 0; k < W; ++k) rmax = fmax(rmax, S.rap_max_w[k]);
  const Bound bd = make_bound(rmax);

  // ---- initial nearest neighbours (each slot scans all others)
  for (int k = 0; k < SPT; ++k) {
    const int t = tid + k * T;
    if (t >= N) break;
    const float rt = S.rap32[t], pt = S.phi32[t];
    Cert c = cert_empty();
    for (int u = 0; u < N; ++u) {
      if (u == t) continue;
      float lo, hi;
      dr2_32(rt, pt, S.rap32[u], S.phi32[u], bd, lo, hi);
      cert_add(c, lo, hi, u);
    }
    int nn = c.i1;
    double d = __longlong_as_double(0x7ff0000000000000LL);
    if (nn >= 0) {
      if (cert_ok(c)) {
        d = dr2_64(S.rap[t], S.phi[t], S.rap[nn], S.phi[nn]);
      } else {
        unsigned long long bk = ~0ull;
        int bl = 0x7fffffff;
        nn = -1;
        for (int u = 0; u < N; ++u) {
          if (u == t) continue;
          float lo, hi;
          dr2_32(rt, pt, S.rap32[u], S.phi32[u], bd, lo, hi);
          if (lo <= c.u1) {
            const double du = dr2_64(S.rap[t], S.phi[t], S.rap[u], S.phi[u]);
            if (arg_less(dbits(du), S.label[u], bk, bl)) {
              bk = dbits(du);
              bl = S.label[u];
              nn = u;
            }
          }
        }
        d = __longlong_as_double((long long)bk);
      }
    }
    S.nn[t] = nn;
    S.nnd[t] = d;
    S.thr[t] = __double2float_ru(d);
  }
  __syncthreads();
  for (int k = 0; k < SPT; ++k) {
    const int t = tid + k * T;
    if (t >= N) break;
    const int nn = S.nn[t];
    S.key[t] = make_key(S.w[t], nn >= 0 ? S.w[nn] : 0.0, S.nnd[t], inv_r2, nn >= 0);
  }
  if (tid == 0) S.ctl_njets = 0;
  __syncthreads();

  // ---- clustering steps
  int n = N;
  int step = 0;
  while (n > 0) {
    // 1. argmin over (key, label)
    unsigned long long bk = ~0ull;
    int bl = 0x7fffffff, bi = -1;
    for (int k = 0; k < SPT; ++k) {
      const int t = tid + k * T;
      if (t >= n) break;
      const unsigned long long kk = dbits(S.key[t]);
      const int l = S.label[t];
      if (arg_less(kk, l, bk, bl)) {
        bk = kk;
        bl = l;
        bi = t;
      }
    }
    Arg wa = arg_warp(bk, bl, bi);
    if (lane == 0) S.warg[warp] = wa;
    __syncthreads();  // B1
    if (tid < 32) {
      Arg x = (lane < W) ? S.warg[lane] : Arg{~0ull, 0x7fffffff, -1};
      x = arg_warp(x.key, x.label, x.idx);
      // 2. promote or merge (thread 0)
      if (tid == 0 && x.idx < 0) {
        // no candidate although n > 0: cannot happen for finite inputs; stop this event
        atomicOr(A.status, 4);
        S.ctl_pair = -1;
      } else if (tid == 0) {
        const int s = x.idx;
        const double key = S.key[s];
        const int L = n - 1;
        int a = -1, b;
        int pair = 0;
        if (key < S.w[s] && S.nn[s] >= 0) {
          pair = 1;
          const int j = S.nn[s];
          a = min(s, j);
          b = max(s, j);
          const int la = S.label[s], lb = S.label[j];
          const int lo_l = min(la, lb), hi_l = max(la, lb);
          const double px = __dadd_rn(S.px[s], S.px[j]);
          const double py = __dadd_rn(S.py[s], S.py[j]);
          const double pz = __dadd_rn(S.pz[s], S.pz[j]);
          const double E = __dadd_rn(S.E[s], S.E[j]);
          const Kin kin = kinematics(px, py, pz, E, algo);
          S.px[a] = px;
          S.py[a] = py;
          S.pz[a] = pz;
          S.E[a] = E;
          S.rap[a] = kin.rap;
          S.phi[a] = kin.phi;
          S.w[a] = kin.w;
          S.rap32[a] = __double2float_rn(kin.rap);
          S.phi32[a] = __double2float_rn(kin.phi);
          S.label[a] = lo_l;
          if (A.history) A.history[off + step] = StepRec{lo_l, hi_l, key};
          if (A.owner) A.owner[off + hi_l] = lo_l;
        } else {
          b = s;
          const int nj = S.ctl_njets;
          double* jo = A.jets + (off + nj) * 4;
          jo[0] = S.px[s];
          jo[1] = S.py[s];
          jo[2] = S.pz[s];
          jo[3] = S.E[s];
          A.jet_label[off + nj] = S.label[s];
          if (A.history) A.history[off + step] = StepRec{S.label[s], -1, key};
          if (A.owner) A.owner[off + S.label[s]] = -(nj + 1);
          S.ctl_njets = nj + 1;
        }
        if (b != L) {
          S.rap[b] = S.rap[L];
          S.phi[b] = S.phi[L];
          S.w[b] = S.w[L];
          S.nnd[b] = S.nnd[L];
          S.key[b] = S.key[L];
          S.px[b] = S.px[L];
          S.py[b] = S.py[L];
          S.pz[b] = S.pz[L];
          S.E[b] = S.E[L];
          S.rap32[b] = S.rap32[L];
          S.phi32[b] = S.phi32[L];
          S.thr[b] = S.thr[L];
          S.nn[b] = S.nn[L];
          S.label[b] = S.label[L];
        }
        S.ctl_a = a;
        S.ctl_b = b;
        S.ctl_L = L;
        S.ctl_pair = pair;
        S.n_rescan = 0;
      }
    }
    __syncthreads();  // B2
    if (S.ctl_pair < 0) break;
    --n;
    ++step;
    const int a = S.ctl_a, b = S.ctl_b, L = S.ctl_L;
    const bool pair = S.ctl_pair != 0;

    // 3. update against the new jet; collect rescans
    Cert ca = cert_empty();
    float ra = 0.f, pa = 0.f;
    if (pair) {
      ra = S.rap32[a];
      pa = S.phi32[a];
    }
    for (int k = 0; k < SPT; ++k) {
      const int t = tid + k * T;
      if (t >= n) break;
      if (pair && t == a) continue;
      int c = S.nn[t];
      const bool resc = pair ? (c == a || c == b) : (c == b);
      if (!resc && c == L) {
        c = b;
        S.nn[t] = b;
      }
      if (resc) {
        const int pos = atomicAdd(&S.n_rescan, 1);
        S.rlist[pos] = t;
      }
      if (pair) {
        float lo, hi;
        dr2_32(S.rap32[t], S.phi32[t], ra, pa, bd, lo, hi);
        cert_add(ca, lo, hi, t);
        if (!resc && lo <= S.thr[t]) {
          const double d = dr2_64(S.rap[t], S.phi[t], S.rap[a], S.phi[a]);
          const double D = S.nnd[t];
          if (d < D || (d == D && S.label[a] < S.label[c])) {
            S.nn[t] = a;
            S.nnd[t] = d;
            S.thr[t] = __double2float_ru(d);
            S.key[t] = make_key(S.w[t], S.w[a], d, inv_r2, true);
          }
        }
      }
    }
    if (pair) {
      const Cert wc = cert_warp(ca);
      if (lane == 0) S.wcert[warp] = wc;
    }
    __syncthreads();  // B3

    // 4a. the new jet's neighbour: owner warp combines and certifies
    if (pair && warp == (a % T) / 32) {
      Cert c = (lane < W) ? S.wcert[lane] : cert_empty();
      c = cert_warp(c);
      double d;
      const int nn = resolve_nn_warp<T, SPT>(S, a, n, c, bd, d);
      if (tid == a % T) {
        S.nn[a] = nn;
        S.nnd[a] = d;
        S.thr[a] = __double2float_ru(d);
        S.key[a] = make_key(S.w[a], nn >= 0 ? S.w[nn] : 0.0, d, inv_r2, nn >= 0);
      }
    }

    // 4b. rescans of slots whose neighbour was merged or promoted
    const int nr = S.n_rescan;
    for (int base = 0; base < nr; base += kRescanChunk) {
      const int cnt = min(kRescanChunk, nr - base);
      Cert rc[kRescanChunk];
      int tgt[kRescanChunk];
      float rt[kRescanChunk], pt[kRescanChunk];
#pragma unroll
      for (int r = 0; r < kRescanChunk; ++r) {
        rc[r] = cert_empty();
        tgt[r] = (r < cnt) ? S.rlist[base + r] : -1;
        rt[r] = (r < cnt) ? S.rap32[tgt[r]] : 0.f;
        pt[r] = (r < cnt) ? S.phi32[tgt[r]] : 0.f;
      }
      for (int k = 0; k < SPT; ++k) {
        const int u = tid + k * T;
        if (u >= n) break;
        const float ru = S.rap32[u], pu = S.phi32[u];
#pragma unroll
        for (int r = 0; r < kRescanChunk; ++r) {
          if (r < cnt && u != tgt[r]) {
            float lo, hi;
            dr2_32(rt[r], pt[r], ru, pu, bd, lo, hi);
            cert_add(rc[r], lo, hi, u);
          }
        }
      }
#pragma unroll
      for (int r = 0; r < kRescanChunk; ++r) {
        if (r < cnt) {
          const Cert wc = cert_warp(rc[r]);
          if (lane == 0) S.rcert[r][warp] = wc;
        }
      }
      __syncthreads();  // B4
      for (int r = 0; r < cnt; ++r) {
        const int t = tgt[r];
        if (warp != (t % T) / 32) continue;
        Cert c = (lane < W) ? S.rcert[r][lane] : cert_empty();
        c = cert_warp(c);
        double d;
        const int nn = resolve_nn_warp<T, SPT>(S, t, n, c, bd, d);
        if (tid == t % T) {
          S.nn[t] = nn;
          S.nnd[t] = d;
          S.thr[t] = __double2float_ru(d);
          S.key[t] = make_key(S.w[t], nn >= 0 ? S.w[nn] : 0.0, d, inv_r2, nn >= 0);
        }
      }
      if (base + kRescanChunk < nr) __syncthreads();  // rcert reuse
    }
    // the next argmin reads only keys its own thread wrote, or keys written
    // before B2/B3/B4 by other threads
  }

  // ---- epilogue: jet count, and constituent ownership from the union-find
  // parents (owner[label] = parent label, or -(jet+1) once promoted)
  __syncthreads();
  if (tid == 0) A.n_jets[e] = S.ctl_njets;
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
