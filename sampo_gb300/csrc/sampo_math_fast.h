/*
 * sampo_math_fast.h - binary32-only evaluations of three binary64 results
 * of the SAMPO model, for the GPU, where binary64 instructions issue at a
 * small fraction of the binary32 rate.
 *
 *   sampo_logf_bm(x)  = sampo_logf(x)   for the normal draw's log
 *   sampo_sinf_bm(x)  = sampo_sinf(x)   for the normal draw's sin
 *                                       (include/gpuRand.h:56-63)
 *   sampo_sporo_add() = (float)((double)s + d), the sporogonic development
 *                       update done in double (kernel/updateAgents.cl:69-70)
 *
 * Each function computes its result as an unevaluated pair of binary32
 * numbers H + L with the error-free transformations TwoSum (Knuth, TAOCP
 * vol. 2, 4.2.2) and TwoProd through fmaf, from a table of breakpoints
 * (Tang's table-driven method, ACM TOMS 15(2), 1989, with the tables of
 * sampo_fast_tables.h), and then applies Ziv's rounding test: when every
 * value within the error bound of H + L rounds to the same binary32 number,
 * that number is the rounding of the exact result and, because the binary64
 * definitions in sampo_math.h are accurate to better than 2^-48 relative,
 * also the definition's result. Otherwise the binary64 definition itself is
 * evaluated. The error bounds were measured over every input of the domains
 * the model produces (log: x in {0} and [2^-32, 1]; sin: x = fl(2*pi_f * u)
 * for those u), and tests/fastmath_check.c checks that the results equal the
 * binary64 definitions bit for bit on those domains.
 *
 * Compile with FP contraction off (-ffp-contract=off / --fmad=false): the
 * transformations rely on every + and * rounding separately.
 */
#ifndef SAMPO_MATH_FAST_H
#define SAMPO_MATH_FAST_H

#include "sampo_math.h"
#include "sampo_fast_tables.h"

#if defined(__CUDACC__)
static __device__ __align__(16) const float sampo_log_tab_d[128][4] = SAMPO_LOG_TABLE_INIT;
static __device__ __align__(16) const float sampo_sin_tab_d[513][2][4] = SAMPO_SIN_TABLE_INIT;
#endif
#if !defined(__CUDA_ARCH__)
static const float sampo_log_tab_h[128][4] __attribute__((aligned(16))) = SAMPO_LOG_TABLE_INIT;
static const float sampo_sin_tab_h[513][2][4] __attribute__((aligned(16))) = SAMPO_SIN_TABLE_INIT;
#endif

/* Relative error bounds of H + L, each at least 4 times the largest error
 * measured over the whole domain (log 2^-40.12, sin 2^-38.75) plus 2^-48 for
 * the binary64 definition; the add's bound follows from its two roundings
 * (below 2^-45) and the double rounding of the definition (2^-52). */
#define SAMPO_FAST_LOG_EPS 0x1p-38f
#define SAMPO_FAST_SIN_EPS 0x1p-36f
#define SAMPO_FAST_ADD_EPS 0x1p-40f

SAMPO_HD float sampo_fmaf(float a, float b, float c) {
#if defined(__CUDA_ARCH__)
  return __fmaf_rn(a, b, c);
#else
  return fmaf(a, b, c);
#endif
}

SAMPO_HD float sampo_fabsf(float a) { return sampo_bits2f(sampo_f2bits(a) & 0x7FFFFFFFu); }

/* s + e = a + b exactly */
SAMPO_HD void sampo_two_sum(float a, float b, float* s, float* e) {
  const float t = a + b;
  const float bb = t - a;
  *e = (a - (t - bb)) + (b - bb);
  *s = t;
}

/* Load a table row of 4 floats. */
SAMPO_HD void sampo_log_row(uint32_t i, float* r) {
#if defined(__CUDA_ARCH__)
  const float4 v = __ldg(reinterpret_cast<const float4*>(sampo_log_tab_d[i]));
  r[0] = v.x; r[1] = v.y; r[2] = v.z;
#else
  r[0] = sampo_log_tab_h[i][0]; r[1] = sampo_log_tab_h[i][1]; r[2] = sampo_log_tab_h[i][2];
#endif
}
SAMPO_HD void sampo_sin_row(uint32_t k, float* p, float* sc) {
#if defined(__CUDA_ARCH__)
  const float4 a = __ldg(reinterpret_cast<const float4*>(sampo_sin_tab_d[k][0]));
  const float4 b = __ldg(reinterpret_cast<const float4*>(sampo_sin_tab_d[k][1]));
  p[0] = a.x; p[1] = a.y; p[2] = a.z;
  sc[0] = b.x; sc[1] = b.y; sc[2] = b.z; sc[3] = b.w;
#else
  for (int j = 0; j < 3; j++) p[j] = sampo_sin_tab_h[k][0][j];
  for (int j = 0; j < 4; j++) sc[j] = sampo_sin_tab_h[k][1][j];
#endif
}

/* Ziv's test: 1 and *out = the rounding of every value in H + L +- eps*|H|. */
SAMPO_HD int sampo_round_test(float H, float L, float eps, float* out) {
  const float err = sampo_fabsf(H) * eps;
  const float f1 = H + (L - err);
  const float f2 = H + (L + err);
  *out = f1;
  return f1 == f2;
}

/* log(x) as H + L for positive normal x; 0 for other x. */
SAMPO_HD int sampo_log_pair(float x, float* H, float* L) {
  const uint32_t ix = sampo_f2bits(x);
  if (ix - 0x00800000u >= 0x7F000000u) return 0;       /* zero, subnormal, negative, inf, NaN */
  /* x = 2^k * m, m in [0.703125, 1.40625); i = the 7 mantissa bits after the offset */
  const uint32_t t = ix - 0x3F340000u;
  const int32_t k = (int32_t)t >> 23;
  const uint32_t i = (t >> 16) & 127u;
  const float m = sampo_bits2f(ix - (t & 0xFF800000u));
  float row[3];
  sampo_log_row(i, row);
  const float c = row[0], th = row[1], tl = row[2];
  /* r = m*c - 1 exactly as r1 + r2 (p - 1 is exact for p in [0.5, 2]) */
  const float p = m * c;
  const float pe = sampo_fmaf(m, c, -p);
  float r1, r2;
  sampo_two_sum(p - 1.0f, pe, &r1, &r2);
  /* log(1 + r) = r - r^2/2 + r^3 (1/3 - r/4 + r^2/5 - r^3/6 + r^4/7), |r| < 2^-7 */
  const float zh = r1 * r1;
  const float ze = sampo_fmaf(r1, r1, -zh);
  const float tail = (r1 * zh) * (0x1.555556p-2f + r1 * (-0.25f + r1 * (0x1.99999ap-3f +
                     r1 * (-0x1.555556p-3f + r1 * 0x1.24924ap-3f))));
  const float hz = 0.5f * zh;
  const float u = r1 - hz;                               /* |r1| >= |hz| */
  const float ue = (r1 - u) - hz;
  const float pl = ((ue + r2) - (0.5f * ze + r1 * r2)) + tail;
  /* k log 2 - log c + log(1 + r) */
  const float kf = sampo_bits2f(0x4B400000u + (uint32_t)k) - 12582912.0f;  /* exact for |k| < 2^22 */
  float s1, e1, s2, e2;
  sampo_two_sum(kf * SAMPO_FAST_LN2_A, th, &s1, &e1);
  sampo_two_sum(s1, u, &s2, &e2);
  const float lo = (e1 + e2) + ((kf * SAMPO_FAST_LN2_B + tl) + (pl + kf * SAMPO_FAST_LN2_C));
  sampo_two_sum(s2, lo, H, L);
  return 1;
}

/* sin(x) as H + L for 0 <= x <= 6.2831855 (= 2*pi rounded up); 0 otherwise. */
SAMPO_HD int sampo_sin_pair(float x, float* H, float* L) {
  if (!(x >= 0.0f && x <= 0x1.921fb6p+2f)) return 0;    /* also NaN */
  /* k = nearest integer to x*256/pi, 0..512 */
  const uint32_t k = sampo_f2bits(x * SAMPO_FAST_256_OVER_PI + 12582912.0f) - 0x4B400000u;
  float P[3], S[4];
  sampo_sin_row(k, P, S);
  const float sh = S[0], sl = S[1], ch = S[2], cl = S[3];
  /* r = x - k*pi/256 as rh + rl (x - Ph is exact: Sterbenz, or Ph = 0) */
  float rh, rl;
  sampo_two_sum(x - P[0], -P[1], &rh, &rl);
  rl = rl - P[2];
  /* sin(x_k + r) = S + C r - S r^2/2 - C r^3/6 + S r^4/24 + C r^5/120, |r| <= pi/512 */
  const float zh = rh * rh;
  const float ze = sampo_fmaf(rh, rh, -zh);
  const float p1 = ch * rh;
  const float p1e = sampo_fmaf(ch, rh, -p1);
  const float p2 = sh * zh;
  const float p2e = sampo_fmaf(sh, zh, -p2);
  float s1, e1, s2, e2;
  sampo_two_sum(sh, p1, &s1, &e1);
  sampo_two_sum(s1, -0.5f * p2, &s2, &e2);
  const float r3 = rh * zh;
  const float t4 = ch * (r3 * 0x1.555556p-3f);
  const float t5 = sh * ((zh * zh) * 0x1.555556p-5f);
  const float t6 = ch * ((r3 * zh) * 0x1.111112p-7f);
  const float small = (sl + (ch * rl + cl * rh)) - (0.5f * ((p2e + sh * ze) + sl * zh) + (sh * rh) * rl);
  const float lo = ((e1 + e2) + p1e) + ((small - t4) + (t5 + t6));
  sampo_two_sum(s2, lo, H, L);
  return 1;
}

SAMPO_HD float sampo_logf_bm(float x) {
  float H, L, f;
  if (sampo_log_pair(x, &H, &L) && sampo_round_test(H, L, SAMPO_FAST_LOG_EPS, &f)) return f;
  return sampo_logf(x);
}

SAMPO_HD float sampo_sinf_bm(float x) {
  float H, L, f;
  if (sampo_sin_pair(x, &H, &L) && sampo_round_test(H, L, SAMPO_FAST_SIN_EPS, &f)) return f;
  return sampo_sinf(x);
}

/* d = dh + dm + dl exactly, dh = (float)d: the binary32 split of a binary64. */
SAMPO_HD void sampo_split_double(double d, float* dh, float* dm, float* dl) {
  const float h = (float)d;
  const double r = d - (double)h;          /* exact */
  const float m = (float)r;
  *dh = h; *dm = m; *dl = (float)(r - (double)m);
}

/* (float)((double)s + d) for s >= 0 and d = dh + dm + dl > 0. */
SAMPO_HD float sampo_sporo_add(float s, float dh, float dm, float dl, double d) {
  float a, b, f;
  sampo_two_sum(s, dh, &a, &b);           /* s + d = a + b + dm + dl exactly */
  if (sampo_round_test(a, (b + dm) + dl, SAMPO_FAST_ADD_EPS, &f)) return f;
  return (float)((double)s + d);
}

#endif
