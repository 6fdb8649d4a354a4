/*
 * sampo_math.h - deterministic single-precision transcendentals for the SAMPO
 * agent model, identical on the host (C/C++) and on the GPU (CUDA).
 *
 * The reference calls OpenCL built-ins exp, pow, log, sin, sqrt and ceil on
 * float arguments (kernel/killAgents.cl:90-92,106,120-124,137;
 * include/gpuRand.h:60-62; include/properties.h:262,301). OpenCL leaves the
 * accuracy of exp/pow/log/sin implementation-defined (3-16 ulp), so the
 * reference itself gives different bits on different devices. This project
 * fixes one definition: every function is evaluated in IEEE binary64 with the
 * published methods named below and rounded once to binary32. The result is
 * correctly rounded except when the exact value lies within ~2^-50 relative
 * of a binary32 rounding boundary, and - what parity relies on - it is
 * bit-identical wherever the operation sequence below is executed with IEEE
 * binary64 add/mul/div/fma (x86-64 SSE2, aarch64, sm_103a). Callers compile
 * with FP contraction off (-ffp-contract=off / --fmad=false); every fused
 * multiply-add used here is spelled out with fma().
 *
 * Methods (textbook; J.-M. Muller, "Elementary Functions", ch. 11):
 *   exp: Cody-Waite reduction x = k*ln2 + r, |r| <= ln2/2, Taylor series of
 *        e^r to degree 14, scaling by 2^k through the exponent field.
 *   log: x = 2^e * m, m in [sqrt(1/2), sqrt(2)), log m = 2 atanh(s) with
 *        s = (m-1)/(m+1) and the odd series of atanh to s^25.
 *   sin: Cody-Waite reduction by pi/2 with a three-part constant, Taylor
 *        series of sin/cos to degree 17/18 on |r| <= pi/4, quadrant select.
 *   pow: exp(y * log(x)) evaluated in binary64, C99 special cases.
 * Constants are the binary64 roundings of ln 2, 1/ln 2, 2/pi, sqrt 2, pi/2
 * split into 30-bit pieces, 1/n! and 1/(2k+1), computed with mpmath at 300
 * bits and written as hexadecimal literals.
 */
#ifndef SAMPO_MATH_H
#define SAMPO_MATH_H

#include <stdint.h>

#if defined(__CUDACC__)
#define SAMPO_HD __host__ __device__ __forceinline__
#else
#define SAMPO_HD static inline
#endif

#if !defined(__CUDA_ARCH__)
#include <math.h>
#include <string.h>
#endif

SAMPO_HD uint64_t sampo_d2bits(double d) {
#if defined(__CUDA_ARCH__)
  return (uint64_t)__double_as_longlong(d);
#else
  uint64_t u; memcpy(&u, &d, 8); return u;
#endif
}
SAMPO_HD double sampo_bits2d(uint64_t u) {
#if defined(__CUDA_ARCH__)
  return __longlong_as_double((long long)u);
#else
  double d; memcpy(&d, &u, 8); return d;
#endif
}
SAMPO_HD uint32_t sampo_f2bits(float f) {
#if defined(__CUDA_ARCH__)
  return (uint32_t)__float_as_uint(f);
#else
  uint32_t u; memcpy(&u, &f, 4); return u;
#endif
}
SAMPO_HD float sampo_bits2f(uint32_t u) {
#if defined(__CUDA_ARCH__)
  return __uint_as_float(u);
#else
  float f; memcpy(&f, &u, 4); return f;
#endif
}
SAMPO_HD double sampo_fma(double a, double b, double c) { return fma(a, b, c); }
SAMPO_HD double sampo_floor(double a) { return floor(a); }

#define SAMPO_INF_F   (sampo_bits2f(0x7F800000u))
#define SAMPO_NAN_F   (sampo_bits2f(0x7FC00000u))

/* exp(x) in binary64 for |x| <= 700 (callers clamp the argument). */
SAMPO_HD double sampo_exp_d(double x) {
  const double INV_LN2 = 0x1.71547652b82fep+0;
  const double LN2_HI = 0x1.62e42fee00000p-1; /* 32 significant bits */
  const double LN2_LO = 0x1.a39ef35793c76p-33;
  double k = sampo_floor(sampo_fma(x, INV_LN2, 0.5));
  /* k*LN2_HI is exact (|k| < 2^11, 32-bit constant) */
  double r = sampo_fma(-k, LN2_HI, x);
  r = sampo_fma(-k, LN2_LO, r);
  double p = 0x1.93974a8c07c9dp-37;             /* 1/14! */
  p = sampo_fma(p, r, 0x1.6124613a86d09p-33);   /* 1/13! */
  p = sampo_fma(p, r, 0x1.1eed8eff8d898p-29);   /* 1/12! */
  p = sampo_fma(p, r, 0x1.ae64567f544e4p-26);   /* 1/11! */
  p = sampo_fma(p, r, 0x1.27e4fb7789f5cp-22);   /* 1/10! */
  p = sampo_fma(p, r, 0x1.71de3a556c734p-19);   /* 1/9!  */
  p = sampo_fma(p, r, 0x1.a01a01a01a01ap-16);   /* 1/8!  */
  p = sampo_fma(p, r, 0x1.a01a01a01a01ap-13);   /* 1/7!  */
  p = sampo_fma(p, r, 0x1.6c16c16c16c17p-10);   /* 1/6!  */
  p = sampo_fma(p, r, 0x1.1111111111111p-7);    /* 1/5!  */
  p = sampo_fma(p, r, 0x1.5555555555555p-5);    /* 1/4!  */
  p = sampo_fma(p, r, 0x1.5555555555555p-3);    /* 1/3!  */
  p = sampo_fma(p, r, 0.5);
  p = sampo_fma(p, r, 1.0);
  p = sampo_fma(p, r, 1.0);
  int64_t ki = (int64_t)k;
  double scale = sampo_bits2d((uint64_t)(ki + 1023) << 52);
  return p * scale;
}

/* log(x) in binary64 for finite x > 0 (normal or subnormal). */
SAMPO_HD double sampo_log_d(double x) {
  const double LN2_HI = 0x1.62e42fee00000p-1;
  const double LN2_LO = 0x1.a39ef35793c76p-33;
  const double SQRT2 = 0x1.6a09e667f3bcdp+0;
  uint64_t u = sampo_d2bits(x);
  int64_t e = (int64_t)((u >> 52) & 0x7FF);
  if (e == 0) { /* subnormal: scale by 2^54 */
    u = sampo_d2bits(x * 0x1p54);
    e = (int64_t)((u >> 52) & 0x7FF) - 54;
  }
  e -= 1023;
  double m = sampo_bits2d((u & 0x000FFFFFFFFFFFFFULL) | 0x3FF0000000000000ULL); /* [1,2) */
  if (m > SQRT2) { m *= 0.5; e += 1; }
  double f = m - 1.0;          /* exact */
  double s = f / (m + 1.0);
  double z = s * s;
  double p = 0x1.47ae147ae147bp-5;              /* 1/25 */
  p = sampo_fma(p, z, 0x1.642c8590b2164p-5);    /* 1/23 */
  p = sampo_fma(p, z, 0x1.8618618618618p-5);    /* 1/21 */
  p = sampo_fma(p, z, 0x1.af286bca1af28p-5);    /* 1/19 */
  p = sampo_fma(p, z, 0x1.e1e1e1e1e1e1ep-5);    /* 1/17 */
  p = sampo_fma(p, z, 0x1.1111111111111p-4);    /* 1/15 */
  p = sampo_fma(p, z, 0x1.3b13b13b13b14p-4);    /* 1/13 */
  p = sampo_fma(p, z, 0x1.745d1745d1746p-4);    /* 1/11 */
  p = sampo_fma(p, z, 0x1.c71c71c71c71cp-4);    /* 1/9  */
  p = sampo_fma(p, z, 0x1.2492492492492p-3);    /* 1/7  */
  p = sampo_fma(p, z, 0x1.999999999999ap-3);    /* 1/5  */
  p = sampo_fma(p, z, 0x1.5555555555555p-2);    /* 1/3  */
  double s2 = s + s;                            /* log m = 2s + 2s*z*p */
  double logm = sampo_fma(s2 * z, p, s2);
  double ed = (double)e;
  return sampo_fma(ed, LN2_HI, sampo_fma(ed, LN2_LO, logm));
}

/* ---------------- binary32 entry points ---------------- */

SAMPO_HD float sampo_expf(float x) {
  if (x != x) return x;
  if (x > 100.0f) return SAMPO_INF_F;
  if (x < -120.0f) return 0.0f;
  return (float)sampo_exp_d((double)x);
}

SAMPO_HD float sampo_logf(float x) {
  if (x != x) return x;
  if (x < 0.0f) return SAMPO_NAN_F;
  if (x == 0.0f) return -SAMPO_INF_F;
  if (x == SAMPO_INF_F) return x;
  return (float)sampo_log_d((double)x);
}

/* sin(x); accurate for |x| < 2^20 (the model evaluates [0, 2*pi]). Larger
 * arguments are reduced with the same constants: still deterministic, less
 * accurate. */
SAMPO_HD float sampo_sinf(float xf) {
  if (xf != xf) return xf;
  if (xf == SAMPO_INF_F || xf == -SAMPO_INF_F) return SAMPO_NAN_F;
  const double TWO_OVER_PI = 0x1.45f306dc9c883p-1;
  const double PIO2_1 = 0x1.921fb54000000p+0;
  const double PIO2_2 = 0x1.10b4611800000p-30;
  const double PIO2_3 = 0x1.313198a2e0370p-61;
  double x = (double)xf;
  double k = sampo_floor(sampo_fma(x, TWO_OVER_PI, 0.5));
  double r = sampo_fma(-k, PIO2_1, x);
  r = sampo_fma(-k, PIO2_2, r);
  r = sampo_fma(-k, PIO2_3, r);
  int64_t q = ((int64_t)k) & 3;
  double z = r * r;
  /* sin r = r + r*z*(-1/3! + z/5! - ...), cos r = 1 + z*(-1/2! + z/4! - ...) */
  double ps = 0x1.952c77030ad4ap-49;             /* +1/17! */
  ps = sampo_fma(ps, z, -0x1.ae7f3e733b81fp-41); /* -1/15! */
  ps = sampo_fma(ps, z, 0x1.6124613a86d09p-33);  /* +1/13! */
  ps = sampo_fma(ps, z, -0x1.ae64567f544e4p-26); /* -1/11! */
  ps = sampo_fma(ps, z, 0x1.71de3a556c734p-19);  /* +1/9!  */
  ps = sampo_fma(ps, z, -0x1.a01a01a01a01ap-13); /* -1/7!  */
  ps = sampo_fma(ps, z, 0x1.1111111111111p-7);   /* +1/5!  */
  ps = sampo_fma(ps, z, -0x1.5555555555555p-3);  /* -1/3!  */
  double sn = sampo_fma(r * z, ps, r);
  double pc = -0x1.6827863b97d97p-53;            /* -1/18! */
  pc = sampo_fma(pc, z, 0x1.ae7f3e733b81fp-45);  /* +1/16! */
  pc = sampo_fma(pc, z, -0x1.93974a8c07c9dp-37); /* -1/14! */
  pc = sampo_fma(pc, z, 0x1.1eed8eff8d898p-29);  /* +1/12! */
  pc = sampo_fma(pc, z, -0x1.27e4fb7789f5cp-22); /* -1/10! */
  pc = sampo_fma(pc, z, 0x1.a01a01a01a01ap-16);  /* +1/8!  */
  pc = sampo_fma(pc, z, -0x1.6c16c16c16c17p-10); /* -1/6!  */
  pc = sampo_fma(pc, z, 0x1.5555555555555p-5);   /* +1/4!  */
  pc = sampo_fma(pc, z, -0.5);                   /* -1/2!  */
  double cs = sampo_fma(z, pc, 1.0);
  double res = (q == 0) ? sn : (q == 1) ? cs : (q == 2) ? -sn : -cs;
  return (float)res;
}

/* pow(x, y) with the C99 special cases the model can reach. */
SAMPO_HD float sampo_powf(float x, float y) {
  if (y == 0.0f) return 1.0f;
  if (x == 1.0f) return 1.0f;
  if (x != x || y != y) return SAMPO_NAN_F;
  double sign = 1.0;
  if (x < 0.0f) {
    float yi = (float)sampo_floor((double)y);
    if (yi != y) return SAMPO_NAN_F;              /* negative base, non-integer y */
    double half = (double)y * 0.5;
    if (sampo_floor(half) != half) sign = -1.0;   /* odd integer y */
    x = -x;
  }
  if (x == 0.0f) return (float)(sign * (y > 0.0f ? 0.0 : (double)SAMPO_INF_F));
  if (x == SAMPO_INF_F) return (float)(sign * (y > 0.0f ? (double)SAMPO_INF_F : 0.0));
  double t = (double)y * sampo_log_d((double)x);
  if (t > 100.0) return (float)(sign * (double)SAMPO_INF_F);
  if (t < -120.0) return (float)(sign * 0.0);
  return (float)(sign * sampo_exp_d(t));
}

/* Float -> uint32 conversion that is defined for every input: truncation
 * toward zero, NaN and negatives give 0, values >= 2^32 give UINT32_MAX.
 * Used where the reference casts a possibly out-of-range float to UINT
 * (include/properties.h:260), which C leaves undefined. */
SAMPO_HD uint32_t sampo_f2u_sat(float x) {
  if (!(x > 0.0f)) return 0u;                       /* NaN, negative, zero */
  if (x >= 4294967296.0f) return 0xFFFFFFFFu;
  return (uint32_t)x;
}

/* OpenCL min/max on floats as IEEE minNum/maxNum: a NaN operand is ignored. */
SAMPO_HD float sampo_fminf(float a, float b) {
  if (a != a) return b;
  if (b != b) return a;
  return (b < a) ? b : a;
}
SAMPO_HD float sampo_fmaxf(float a, float b) {
  if (a != a) return b;
  if (b != b) return a;
  return (b > a) ? b : a;
}

#endif /* SAMPO_MATH_H */
