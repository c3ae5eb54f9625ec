// FP64 kinematics of a pseudojet from integer arithmetic (GB300: keeps the
// serial merge step off the FP64 pipe, which runs at ~1/64 of the FP32 rate
// and charges a full warp slot per instruction even for one active lane).
//
// Portable C99 + __int128: compiled into the CUDA kernels (device functions)
// and into a host build used by the tests, so both run the same bits.
//
//   fjk_div_rn(a, b)  correctly rounded a / b (IEEE round-to-nearest-even) for
//                     positive normal operands and a normal result; anything
//                     else goes to the hardware division (FJK_HW_DIV);
//   fjk_log(x)        natural logarithm, Tang's table method: two table
//                     reductions (7 bits, then 8 bits) leave |z| <= 2^-13 and
//                     log1p(z) = z + z^2 (-1/2 + z/3 - z^2/4 + z^3/5 - z^4/6)
//                     in 64-bit fixed point; sums in 128-bit fixed point at
//                     scale 2^-112; one final rounding.  Positive normal x only
//                     (else FJK_LIBM_LOG).  Absolute error ~2^-75, relative
//                     precision kept near x = 1;
//   fjk_atan2(y, x)   octant reduction to t = min/max in [0, 1]; for t >= 2^-6
//                     the table atan(c), c = k/256 nearest to t, plus atan(d),
//                     d = (t - c)/(1 + t c) = (num - c den)/(den + c num) as
//                     one exact integer division, |d| <= 2^-9, odd series to
//                     d^7, at scale 2^-120; for t < 2^-5 the series
//                     t (1 - t^2/3 + ... - t^12/13) on a 128-bit quotient,
//                     with relative precision; one final rounding.  Finite nonzero normal operands only
//                     (else FJK_LIBM_ATAN2).
// The results are the correctly rounded values except when the exact value
// lies within ~2^-12 ulp of a rounding boundary; the tests measure the
// agreement with CUDA's and the host's libm.
#pragma once

#include <stdint.h>

#if defined(__CUDACC__)
#define FJK_FN static __device__ __forceinline__
// the three long routines stay out of line: one copy each instead of one per
// call site keeps the kernels' instruction footprint small (measured: 4 %
// fewer cycles per merge step with three CTAs sharing an SM)
#define FJK_BIG static __device__ __noinline__
#define FJK_TABLE static __device__ __constant__ const
#define FJK_HW_DIV(a, b) __ddiv_rn((a), (b))
#define FJK_LIBM_LOG(x) log(x)
#define FJK_LIBM_ATAN2(y, x) atan2((y), (x))
#define FJK_DMUL(a, b) __dmul_rn((a), (b))
#define FJK_DADD(a, b) __dadd_rn((a), (b))
#define FJK_DSUB(a, b) __dsub_rn((a), (b))
#else
#include <math.h>
#define FJK_FN static inline
#define FJK_BIG static inline
#define FJK_TABLE static const
#define FJK_HW_DIV(a, b) ((a) / (b))
#define FJK_LIBM_LOG(x) log(x)
#define FJK_LIBM_ATAN2(y, x) atan2((y), (x))
#define FJK_DMUL(a, b) ((a) * (b))
#define FJK_DADD(a, b) ((a) + (b))
#define FJK_DSUB(a, b) ((a) - (b))
#endif

#include "fjg_kin_tables.h"

typedef unsigned __int128 fjk_u128;
typedef __int128 fjk_i128;

#define FJK_MASK52 0x000FFFFFFFFFFFFFull
#define FJK_HID52 0x0010000000000000ull

FJK_FN uint64_t fjk_bits(double x) {
#if defined(__CUDACC__)
  return (uint64_t)__double_as_longlong(x);
#else
  union {
    double d;
    uint64_t u;
  } c;
  c.d = x;
  return c.u;
#endif
}

FJK_FN double fjk_double(uint64_t b) {
#if defined(__CUDACC__)
  return __longlong_as_double((long long)b);
#else
  union {
    double d;
    uint64_t u;
  } c;
  c.u = b;
  return c.d;
#endif
}

FJK_FN int fjk_clz64(uint64_t x) {
#if defined(__CUDACC__)
  return __clzll((long long)x);
#else
  return x ? __builtin_clzll(x) : 64;
#endif
}

FJK_FN fjk_i128 fjk_i128_of(int64_t hi, uint64_t lo) {
  return (fjk_i128)(((fjk_u128)(uint64_t)hi << 64) | (fjk_u128)lo);
}

FJK_FN uint64_t fjk_mulhi_u(uint64_t a, uint64_t b) { return (uint64_t)(((fjk_u128)a * b) >> 64); }

FJK_FN int64_t fjk_mulhi_s(int64_t a, int64_t b) { return (int64_t)(((fjk_i128)a * b) >> 64); }

FJK_FN float fjk_float_of(uint32_t b) {
#if defined(__CUDACC__)
  return __uint_as_float(b);
#else
  union {
    float f;
    uint32_t u;
  } c;
  c.u = b;
  return c.f;
#endif
}

FJK_FN uint32_t fjk_bits_of(float f) {
#if defined(__CUDACC__)
  return __float_as_uint(f);
#else
  union {
    float f;
    uint32_t u;
  } c;
  c.f = f;
  return c.u;
#endif
}

// double -> float with round-to-nearest-even (mode 0), toward -inf (mode 1)
// or toward +inf (mode 2), from the bit pattern (the hardware conversion is a
// ~90-cycle operation on GB300).  Results outside the float normal range and
// non-finite inputs use the hardware conversion.
FJK_FN float fjk_to_f32(double x, int mode) {
  const uint64_t b = fjk_bits(x);
  const uint32_t sign = (uint32_t)(b >> 63);
  const int e = (int)((b >> 52) & 0x7ff) - 1023 + 127;
  if (e < 1 || e > 254) {
#if defined(__CUDACC__)
    return mode == 0 ? __double2float_rn(x) : mode == 1 ? __double2float_rd(x) : __double2float_ru(x);
#else
    // host: round to nearest, then step outward if that went the wrong way
    float f = (float)x;
    if (mode == 1 && (double)f > x) f = nextafterf(f, -INFINITY);
    if (mode == 2 && (double)f < x) f = nextafterf(f, INFINITY);
    return f;
#endif
  }
  const uint64_t m = b & FJK_MASK52;
  const uint32_t rem = (uint32_t)(m & 0x1fffffffu);  // the 29 bits below the float mantissa
  const uint32_t out = (sign << 31) | ((uint32_t)e << 23) | (uint32_t)(m >> 29);
  int up;
  if (mode == 0)
    up = rem > 0x10000000u || (rem == 0x10000000u && (out & 1));
  else if (mode == 1)
    up = sign && rem;  // the magnitude grows toward -inf for negatives
  else
    up = !sign && rem;
  return fjk_float_of(out + (uint32_t)up);  // a carry moves into the exponent (or to inf)
}

// V ~ floor(2^127 / D) for D in [2^63, 2^64); never above the true value, at
// most a few units below.  The FP32 reciprocal of the top 24 bits of D seeds
// two Newton steps in 64-bit fixed point.  The seed is built from and read
// back into bit patterns: integer<->float conversions cost ~90 cycles on
// GB300, the bit moves a few.
FJK_FN uint64_t fjk_recip64(uint64_t D) {
  const float f = fjk_float_of(0x3f800000u | ((uint32_t)(D >> 40) & 0x7fffffu));  // top bits, in [1, 2)
#if defined(__CUDACC__)
  const float r = __frcp_rn(f);
#else
  const float r = 1.0f / f;
#endif
  const uint32_t rb = fjk_bits_of(r);  // r in (1/2, 1]
  uint64_t V = ((rb >> 23) < 127u) ? ((uint64_t)((rb & 0x7fffffu) | 0x800000u) << 40) : ~0ull;  // r 2^64
  V -= V >> 21;  // make it an underestimate
  for (int it = 0; it < 2; ++it) {
    const fjk_u128 e = ((fjk_u128)1 << 127) - (fjk_u128)D * V;  // > 0
    V += (uint64_t)(((fjk_u128)V * (uint64_t)(e >> 64)) >> 63);
  }
  return V;
}

// floor(N / D) for D in [2^63, 2^64) and N < D * 2^64, with the remainder.
// The estimate from the high word of N never exceeds the quotient and is at
// most ~10 below it; the loop adds the difference.
FJK_FN uint64_t fjk_divq(fjk_u128 N, uint64_t D, uint64_t V, uint64_t* rem) {
  uint64_t q = (uint64_t)(((fjk_u128)(uint64_t)(N >> 64) * V) >> 63);
  fjk_u128 r = N - (fjk_u128)q * D;
  for (int guard = 0; guard < 24 && r >= D; ++guard) {
    ++q;
    r -= D;
  }
  *rem = (uint64_t)r;
  return q;
}

// Round the positive value A * 2^-F to the nearest double (ties to even);
// the value must lie in the normal range.
FJK_FN double fjk_round_fixed(fjk_u128 A, int F, int negative) {
  if (A == 0) return negative ? -0.0 : 0.0;
  const uint64_t hi = (uint64_t)(A >> 64), lo = (uint64_t)A;
  const int p = hi ? 127 - fjk_clz64(hi) : 63 - fjk_clz64(lo);
  int E = p - F;
  uint64_t mant;
  if (p > 52) {
    const int sh = p - 52;
    mant = (uint64_t)(A >> sh);
    const fjk_u128 rem = A & (((fjk_u128)1 << sh) - 1);
    const fjk_u128 half = (fjk_u128)1 << (sh - 1);
    if (rem > half || (rem == half && (mant & 1))) {
      ++mant;
      if (mant >> 53) {
        mant >>= 1;
        ++E;
      }
    }
  } else {
    mant = (uint64_t)A << (52 - p);
  }
  uint64_t b = ((uint64_t)(E + 1023) << 52) | (mant & FJK_MASK52);
  if (negative) b |= 1ull << 63;
  return fjk_double(b);
}

// Correctly rounded a / b.
FJK_BIG double fjk_div_rn(double a, double b) {
  const uint64_t ab = fjk_bits(a), bb = fjk_bits(b);
  const int ea = (int)((ab >> 52) & 0x7ff), eb = (int)((bb >> 52) & 0x7ff);
  if (ea == 0 || ea == 0x7ff || eb == 0 || eb == 0x7ff || (ab >> 63) || (bb >> 63)) return FJK_HW_DIV(a, b);
  const uint64_t Ma = (ab & FJK_MASK52) | FJK_HID52, Mb = (bb & FJK_MASK52) | FJK_HID52;
  const uint64_t D = Mb << 11;
  const uint64_t V = fjk_recip64(D);
  uint64_t r;
  // Q = floor(Ma * 2^54 / Mb) in [2^53, 2^55)
  const uint64_t Q = fjk_divq((fjk_u128)Ma << 65, D, V, &r);
  int E = ea - eb;
  uint64_t mant;
  int guard, sticky = (r != 0);
  if (Q >> 54) {  // quotient in [1, 2)
    mant = Q >> 2;
    guard = (int)((Q >> 1) & 1);
    sticky |= (int)(Q & 1);
  } else {  // quotient in (1/2, 1)
    mant = Q >> 1;
    guard = (int)(Q & 1);
    E -= 1;
  }
  if (guard && (sticky || (mant & 1))) {
    ++mant;
    if (mant >> 53) {
      mant >>= 1;
      ++E;
    }
  }
  const int biased = E + 1023;
  if (biased < 1 || biased > 2046) return FJK_HW_DIV(a, b);
  return fjk_double(((uint64_t)biased << 52) | (mant & FJK_MASK52));
}

// Natural logarithm, positive normal x (see the header comment).
FJK_BIG double fjk_log_scaled(double x, int halve) {
  const uint64_t bits = fjk_bits(x);
  const int ex = (int)((bits >> 52) & 0x7ff);
  if (ex == 0 || ex == 0x7ff || (bits >> 63)) {
    const double l = FJK_LIBM_LOG(x);
    return halve ? FJK_DMUL(0.5, l) : l;
  }
  const int i1 = (int)((bits >> 45) & 0x7f);
  const int s = i1 >= 53;  // reduce m >= 1.4140625 as m / 2
  const int e = ex - 1023 + s;
  const uint64_t M = (bits & FJK_MASK52) | FJK_HID52;
  const uint64_t P = M * (uint64_t)FJK_LOG_C1[i1];  // y1 = P 2^-(61+s), exact
  const int64_t D1 = (int64_t)(P - (1ull << (61 + s)));
  int i2 = (int)((D1 + (1ll << (54 + s))) >> (48 + s));  // floor((z1 + 2^-7) 2^13)
  i2 = i2 < 0 ? 0 : (i2 > 255 ? 255 : i2);
  const fjk_u128 P2 = (fjk_u128)P * FJK_LOG_C2[i2];  // y2 = P2 2^-(75+s), exact
  const fjk_i128 D2 = (fjk_i128)P2 - ((fjk_i128)1 << (75 + s));
  const int64_t Z = (int64_t)(D2 * (2 - s));  // z2 at scale 2^-76, |z2| <= 2^-13
  // q = -1/2 + z/3 - z^2/4 + z^3/5 - z^4/6 at scale 2^-63
  int64_t q = FJK_LQ4;
  q = FJK_LQ3 + (fjk_mulhi_s(Z, q) >> 12);
  q = FJK_LQ2 + (fjk_mulhi_s(Z, q) >> 12);
  q = FJK_LQ1 + (fjk_mulhi_s(Z, q) >> 12);
  q = FJK_LQ0 + (fjk_mulhi_s(Z, q) >> 12);
  const int64_t T = fjk_mulhi_s(Z, q) >> 12;  // z q at scale 2^-63
  fjk_i128 S = fjk_i128_of(FJK_LN2_112_HI, FJK_LN2_112_LO) * e;
  S += fjk_i128_of(FJK_LOG1_HI[i1], FJK_LOG1_LO[i1]);
  S += fjk_i128_of(FJK_LOG2_HI[i2], FJK_LOG2_LO[i2]);
  S += (fjk_i128)Z * ((fjk_i128)1 << 36);  // z at scale 2^-112
  S += ((fjk_i128)Z * T) >> 27;         // z (z q): 2^-139 -> 2^-112
  const int neg = S < 0;
  const fjk_u128 A = neg ? (fjk_u128)(-S) : (fjk_u128)S;
  return fjk_round_fixed(A, 112 + halve, neg);
}

FJK_FN double fjk_log(double x) { return fjk_log_scaled(x, 0); }

// atan2 for finite nonzero normal operands (see the header comment).
FJK_BIG double fjk_atan2(double y, double x) {
  const uint64_t xb = fjk_bits(x), yb = fjk_bits(y);
  const uint64_t ax = xb & ~(1ull << 63), ay = yb & ~(1ull << 63);
  const int exn = (int)(ax >> 52), eyn = (int)(ay >> 52);
  if (exn == 0 || eyn == 0 || exn == 0x7ff || eyn == 0x7ff) return FJK_LIBM_ATAN2(y, x);
  const int swap = ay > ax;  // |y| > |x|
  const uint64_t nb = swap ? ax : ay, db = swap ? ay : ax;
  const int k = (int)(db >> 52) - (int)(nb >> 52);  // >= 0; t = (Mn / Md) 2^-k <= 1
  if (k > 1000) return FJK_LIBM_ATAN2(y, x);          // result near the subnormal range
  const uint64_t Mn = (nb & FJK_MASK52) | FJK_HID52, Md = (db & FJK_MASK52) | FJK_HID52;
  const int x_neg = (int)(xb >> 63), y_neg = (int)(yb >> 63);
  fjk_i128 res;  // atan(t) at scale 2^-120
  if (k >= 6) {
    // t < 2^-5: t to 128 bits, atan(t) = t (1 - corr), corr = t^2/3 - ... - t^12/13
    const uint64_t D = Md << 11;
    const uint64_t V = fjk_recip64(D);
    uint64_t r1, r2;
    const uint64_t Q1 = fjk_divq((fjk_u128)Mn << 74, D, V, &r1);  // (Mn/Md) 2^63
    const uint64_t Q2 = fjk_divq((fjk_u128)r1 << 64, D, V, &r2);  // next 64 bits
    const fjk_u128 Tq = ((fjk_u128)Q1 << 64) | Q2;                // t = Tq 2^-(127+k)
    const int sh = 2 * k - 2;  // t^2 at scale 2^-64 = (Q1^2 >> 64) >> (2k - 2)
    const uint64_t t2 = sh >= 64 ? 0 : (fjk_mulhi_u(Q1, Q1) >> sh);
    uint64_t p = FJK_AQ13;
    p = FJK_AQ11 - fjk_mulhi_u(t2, p);
    p = FJK_AQ9 - fjk_mulhi_u(t2, p);
    p = FJK_AQ7 - fjk_mulhi_u(t2, p);
    p = FJK_AQ5 - fjk_mulhi_u(t2, p);
    p = FJK_AQ3 - fjk_mulhi_u(t2, p);
    const uint64_t corr = fjk_mulhi_u(t2, p);  // scale 2^-64
    const fjk_u128 dec = (fjk_u128)fjk_mulhi_u(Q2, corr) + (fjk_u128)Q1 * corr;  // (Tq corr) >> 64
    const fjk_u128 At = Tq - dec;
    if (!swap && !x_neg) return fjk_round_fixed(At, 127 + k, y_neg);
    res = (fjk_i128)(At >> (7 + k));
  } else {
    // nearest table point c = kk/256 from an FP32 estimate of t (bit patterns)
    const float fn = fjk_float_of(0x3f800000u | (uint32_t)((Mn >> 29) & 0x7fffffu));
    const float fd = fjk_float_of(0x3f800000u | (uint32_t)((Md >> 29) & 0x7fffffu));
    const uint32_t tb = fjk_bits_of(fn / fd);         // Mn/Md in (1/2, 2)
    const int et = (int)(tb >> 23) - 127;             // -1 or 0
    const uint32_t mt = (tb & 0x7fffffu) | 0x800000u;  // 24-bit mantissa
    const int s = 15 - et + k;                         // 256 t = mt 2^-s
    int kk = (int)((mt + (1u << (s - 1))) >> s);
    kk = kk > 256 ? 256 : kk;
    // d = (t - c) / (1 + t c) = N / Dd exactly, with both scaled by 256 Md 2^k
    const fjk_i128 N = ((fjk_i128)Mn << 8) - ((fjk_i128)((fjk_u128)Md * (uint64_t)kk) << k);
    const fjk_u128 Dd = ((fjk_u128)Md << (8 + k)) + (fjk_u128)Mn * (uint64_t)kk;  // in [2^60, 2^67)
    res = fjk_i128_of(FJK_ATAN_HI[kk], FJK_ATAN_LO[kk]);
    if (N != 0) {
      const uint64_t dh = (uint64_t)(Dd >> 64);
      const int bl = dh ? 128 - fjk_clz64(dh) : 64 - fjk_clz64((uint64_t)Dd);  // bit length, 61..67
      const int sh = bl - 64;                                                 // -4..3
      const uint64_t Dn = (uint64_t)(sh >= 0 ? (Dd >> sh) : (Dd << -sh));    // [2^63, 2^64)
      const fjk_u128 aN = (fjk_u128)(N < 0 ? -N : N);
      uint64_t rr;
      const uint64_t d72 = fjk_divq(aN << (72 - sh), Dn, fjk_recip64(Dn), &rr);  // |d| 2^72, < 2^63
      const uint64_t d2 = fjk_mulhi_u(d72, d72);                                  // d^2 at scale 2^-80
      uint64_t p = FJK_AQ7;
      p = FJK_AQ5 - (fjk_mulhi_u(d2, p) >> 16);
      p = FJK_AQ3 - (fjk_mulhi_u(d2, p) >> 16);
      const uint64_t corr = fjk_mulhi_u(d2, p) >> 16;      // d^2 P at scale 2^-64
      const uint64_t ad72 = d72 - fjk_mulhi_u(d72, corr);  // atan(|d|) at scale 2^-72
      const fjk_i128 add = (fjk_i128)((fjk_u128)ad72 << 48);
      res = (N < 0) ? res - add : res + add;
    }
  }
  if (swap) res = fjk_i128_of(FJK_PI_2_120_HI, FJK_PI_2_120_LO) - res;
  if (x_neg) res = fjk_i128_of(FJK_PI_120_HI, FJK_PI_120_LO) - res;
  return fjk_round_fixed((fjk_u128)res, 120, y_neg);
}

// The reference's pseudojet kinematics (tri_matrix.cu:61-100, weights
// grid.cu:153-166) with fjk_atan2 / fjk_log / fjk_div_rn in place of the libm
// calls and divisions; every other operation rounds as written.  Split in two
// so that the azimuth and the rapidity/weight chains can run on different
// warps.

// Azimuth in [0, 2pi).
FJK_FN double fjk_phi(double px, double py) {
  const double kTwoPi = 6.283185307179586476925286766559005768394;
  const double pt2 = FJK_DADD(FJK_DMUL(px, px), FJK_DMUL(py, py));
  double phi = (pt2 == 0.0) ? 0.0 : fjk_atan2(py, px);
  if (phi < 0.0) phi = FJK_DADD(phi, kTwoPi);
  if (phi >= kTwoPi) phi = FJK_DSUB(phi, kTwoPi);
  return phi;
}

// Rapidity (MaxRap = 1e5 branch for E == |pz|, pt == 0).
FJK_FN double fjk_rap(double px, double py, double pz, double E) {
  const double pt2 = FJK_DADD(FJK_DMUL(px, px), FJK_DMUL(py, py));
  const double apz = fabs(pz);
  if (E == apz && pt2 == 0.0) {
    const double mr = FJK_DADD(1e5, apz);
    return (pz >= 0.0) ? mr : -mr;
  }
  const double m2 = fmax(0.0, FJK_DSUB(FJK_DMUL(FJK_DADD(E, pz), FJK_DSUB(E, pz)), pt2));
  const double epz = FJK_DADD(E, apz);
  const double rap = fjk_log_scaled(fjk_div_rn(FJK_DADD(pt2, m2), FJK_DMUL(epz, epz)), 1);
  return (pz > 0.0) ? -rap : rap;
}

// Clustering weight: kt pt^2, C/A 1, anti-kt 1/pt^2 (1e300 below pt^2 = 1e-300).
FJK_FN double fjk_weight(double px, double py, int algo) {
  const double pt2 = FJK_DADD(FJK_DMUL(px, px), FJK_DMUL(py, py));
  return (algo == 1) ? pt2 : (algo == 0) ? 1.0 : ((pt2 > 1e-300) ? fjk_div_rn(1.0, pt2) : 1e300);
}

FJK_FN void fjk_rap_w(double px, double py, double pz, double E, int algo, double* rap_out, double* w_out) {
  *rap_out = fjk_rap(px, py, pz, E);
  *w_out = fjk_weight(px, py, algo);
}

FJK_FN void fjk_kinematics(double px, double py, double pz, double E, int algo, double* rap_out, double* phi_out,
                           double* w_out) {
  *phi_out = fjk_phi(px, py);
  fjk_rap_w(px, py, pz, E, algo, rap_out, w_out);
}
