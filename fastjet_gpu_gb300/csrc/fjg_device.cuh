// Device primitives shared by the clustering kernels (sm_103a).
//
// Exactness contract.  Every value that takes part in a clustering decision
// (rapidity, azimuth, weight, dR2, d_ij, d_iB) is an FP64 value of the
// reference's expressions (tri_matrix.cu:61-113, grid.cu:110-201), rounded
// exactly as written: products and sums use __dmul_rn/__dadd_rn so that nvcc
// cannot contract them into FMAs, divisions are correctly rounded, and log /
// atan2 come from fjg_kin.h (correctly rounded except within ~2^-12 ulp of a
// rounding boundary).  The CPU oracle (compiled with -ffp-contract=off) agrees
// bit for bit in its portable-kinematics form; its libm form differs only
// where the host libm and fjg_kin.h round a log/atan2 differently.
//
// GB300 executes FP64 at a small fraction of its FP32 rate, so the O(n) scans
// that look for nearest neighbours run in FP32 with a rigorous per-pair error
// bound: each FP32 distance e32 comes with [lo, hi] such that the exact FP64
// distance lies inside.  A scan keeps the smallest lo (and its index), that
// candidate's hi, and the second-smallest lo; when hi < second-smallest lo
// the candidate is certified to be the unique FP64 minimum and only that one
// pair is evaluated in FP64.  Otherwise (near-ties, rare) every candidate whose
// lo does not exceed hi is evaluated in FP64.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "fjg_kin.h"

namespace fjg {

constexpr double kPi = 3.141592653589793238462643383279502884197;
constexpr double kTwoPi = 6.283185307179586476925286766559005768394;
constexpr double kMaxRap = 1e5;
constexpr float kTwoPiF = 6.28318548202514648f;  // float(2*pi), rounded up
constexpr unsigned kFull = 0xffffffffu;

struct Kin {
  double rap, phi, w;
};

// Rapidity, azimuth and weight of a four-momentum (tri_matrix.cu:61-100;
// weight per algorithm grid.cu:153-166, safe_inverse grid.cu:110), with the
// logarithm, arctangent and divisions done in integer arithmetic (fjg_kin.h).
__device__ __forceinline__ Kin kinematics(double px, double py, double pz, double E, int algo) {
  Kin k;
  fjk_kinematics(px, py, pz, E, algo, &k.rap, &k.phi, &k.w);
  return k;
}

// dR2 = dphi^2 + drap^2 with dphi folded at pi (tri_matrix.cu:102-109).
__device__ __forceinline__ double dr2_64(double rap1, double phi1, double rap2, double phi2) {
  double dphi = fabs(__dsub_rn(phi1, phi2));
  if (dphi > kPi) dphi = __dsub_rn(kTwoPi, dphi);
  const double drap = __dsub_rn(rap1, rap2);
  return __dadd_rn(__dmul_rn(dphi, dphi), __dmul_rn(drap, drap));
}

// d_ij = (min(w_i, w_j) * dR2) * (1/R^2), left to right (tri_matrix.cu:111-113).
__device__ __forceinline__ double pair_distance(double wi, double wj, double dr2, double inv_r2) {
  return __dmul_rn(__dmul_rn(fmin(wi, wj), dr2), inv_r2);
}

// Candidate key of a pseudojet with weight w whose nearest neighbour has
// weight wn at distance dr2: the pair distance if it beats the beam distance
// w, otherwise w (promotion).  No neighbour: w.
__device__ __forceinline__ double make_key(double w, double wn, double dr2, double inv_r2, bool has_nn) {
  if (!has_nn) return w;
  const double d = pair_distance(w, wn, dr2, inv_r2);
  return d < w ? d : w;
}

// Error-bound constants of the FP32 filter for one event.  rap_max bounds
// |rapidity| of every pseudojet of the event (a merged jet's rapidity lies
// between its constituents'), phi is in [0, 2pi).  With u = 2^-24:
//   |e32 - e64| <= 12u*e32 + 6u*rap_max*|drap32| + 28*pi*u*dphi32 + c0
// (derivation: rounding of the FP32 coordinates, of the FP32 differences and
// of the fused square-sum, plus the FP64 rounding of e64 itself, each term
// inflated by 25%).
struct Bound {
  float ce, cr, cp, c0;
};

__device__ __forceinline__ Bound make_bound(double rap_max) {
  const double u = 5.9604644775390625e-08;  // 2^-24
  const double rm = rap_max * 1.01 + 1e-6;
  Bound b;
  b.ce = (float)(12.0 * u);
  b.cr = (float)(6.0 * u * rm);
  b.cp = (float)(28.0 * kPi * u);
  const double s = u * (2.0 * rm + 10.0 * kPi);
  b.c0 = (float)(5.0 * s * s) + 1e-37f;
  return b;
}

// FP32 distance with its bound: returns lo (clamped at 0) and hi.
__device__ __forceinline__ void dr2_32(float r1, float p1, float r2, float p2, const Bound& b, float& lo,
                                       float& hi) {
  const float dr = __fsub_rn(r1, r2);
  float dp = fabsf(__fsub_rn(p1, p2));
  dp = fminf(dp, __fsub_rn(kTwoPiF, dp));
  const float e = __fmaf_rn(dp, dp, __fmul_rn(dr, dr));
  const float delta = __fmaf_rn(b.cr, fabsf(dr), __fmaf_rn(b.cp, dp, __fmaf_rn(b.ce, e, b.c0)));
  lo = fmaxf(__fsub_rn(e, delta), 0.0f);
  hi = __fadd_rn(e, delta);
}

// Partial result of a certified FP32 minimum search.
struct Cert {
  float m1;  // smallest lower bound
  int i1;    // its index (slot), -1 if none
  float u1;  // upper bound of that candidate
  float m2;  // second-smallest lower bound
};

__device__ __forceinline__ Cert cert_empty() { return Cert{__int_as_float(0x7f800000), -1, __int_as_float(0x7f800000), __int_as_float(0x7f800000)}; }

__device__ __forceinline__ void cert_add(Cert& c, float lo, float hi, int idx) {
  if (lo < c.m1) {
    c.m2 = c.m1;
    c.m1 = lo;
    c.u1 = hi;
    c.i1 = idx;
  } else {
    c.m2 = fminf(c.m2, lo);
  }
}

// Certified when the best candidate's upper bound is below every other lower bound.
__device__ __forceinline__ bool cert_ok(const Cert& c) { return c.i1 >= 0 && c.u1 < c.m2; }

// Combine the partials of all lanes (all 32 lanes must call).  Lower bounds are
// non-negative floats, so their bit patterns order like unsigned integers.
__device__ __forceinline__ Cert cert_warp(const Cert& c) {
  const unsigned lane = threadIdx.x & 31u;
  const unsigned mb = __reduce_min_sync(kFull, __float_as_uint(c.m1));
  const unsigned ball = __ballot_sync(kFull, __float_as_uint(c.m1) == mb && c.i1 >= 0);
  Cert r;
  r.m1 = __uint_as_float(mb);
  if (ball == 0) {
    r.i1 = -1;
    r.u1 = __int_as_float(0x7f800000);
    r.m2 = __int_as_float(0x7f800000);
    return r;
  }
  const int src = __ffs(ball) - 1;
  r.i1 = __shfl_sync(kFull, c.i1, src);
  r.u1 = __shfl_sync(kFull, c.u1, src);
  const unsigned other = (lane == (unsigned)src) ? __float_as_uint(c.m2) : __float_as_uint(c.m1);
  r.m2 = __uint_as_float(__reduce_min_sync(kFull, other));
  return r;
}

// Lexicographic warp argmin of (key as unsigned 64-bit, label), returning the
// winning (key, label, idx).  All 32 lanes must call; lanes without a
// candidate pass key = ~0, label = INT32_MAX, idx = -1.
struct Arg {
  unsigned long long key;
  int label;
  int idx;
};

__device__ __forceinline__ Arg arg_warp(unsigned long long key, int label, int idx) {
  const unsigned hi = (unsigned)(key >> 32), lo = (unsigned)key;
  const unsigned mh = __reduce_min_sync(kFull, hi);
  const unsigned ml = __reduce_min_sync(kFull, hi == mh ? lo : 0xffffffffu);
  const bool same = (hi == mh && lo == ml);
  const unsigned mlab = __reduce_min_sync(kFull, same ? (unsigned)label : 0xffffffffu);
  const unsigned ball = __ballot_sync(kFull, same && (unsigned)label == mlab);
  const int src = __ffs(ball) - 1;
  Arg r;
  r.key = ((unsigned long long)mh << 32) | ml;
  r.label = (int)mlab;
  r.idx = __shfl_sync(kFull, idx, src < 0 ? 0 : src);
  return r;
}

__device__ __forceinline__ bool arg_less(unsigned long long k1, int l1, unsigned long long k2, int l2) {
  return k1 < k2 || (k1 == k2 && l1 < l2);
}

__device__ __forceinline__ unsigned long long dbits(double x) { return (unsigned long long)__double_as_longlong(x); }

}  // namespace fjg
