/*
 * fastmath_check.c - checks the binary32 fast paths of sampo_math_fast.h
 * against the binary64 definitions of sampo_math.h.
 *
 *   fastmath_check STRIDE SPORO_CASES
 *
 * log: every STRIDE-th float x in [2^-32, 1], plus 0 (the uniform draws of
 *      the generator are k * 2^-32 rounded to binary32);
 * sin: x = fl(6.2831855f * u) for the same u (the draw's angle);
 * sporo: SPORO_CASES pseudo-random (s, T) pairs and accumulation runs.
 * For each function it prints the largest relative error of the unrounded
 * pair H + L (against libm in binary64), how many inputs took the binary64
 * fallback, and how many results differ from the definition (must be 0).
 * Exit status 1 when any result differs.
 *
 * Build: gcc -O2 -ffp-contract=off -fopenmp -I sampo_gb300/csrc fastmath_check.c -lm
 */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <stdint.h>

#include "sampo_math_fast.h"

typedef struct { double maxrel; long long fallbacks, mismatches, n; } stats;

static void merge(stats* a, const stats* b) {
  if (b->maxrel > a->maxrel) a->maxrel = b->maxrel;
  a->fallbacks += b->fallbacks; a->mismatches += b->mismatches; a->n += b->n;
}

static void check_log(float x, stats* st) {
  float H, L, f;
  st->n++;
  if (sampo_log_pair(x, &H, &L)) {
    double ref = log((double)x);
    if (ref != 0.0) {
      double rel = fabs(((double)H + (double)L) - ref) / fabs(ref);
      if (rel > st->maxrel) st->maxrel = rel;
    }
    if (!sampo_round_test(H, L, SAMPO_FAST_LOG_EPS, &f)) st->fallbacks++;
  } else {
    st->fallbacks++;
  }
  if (sampo_f2bits(sampo_logf_bm(x)) != sampo_f2bits(sampo_logf(x))) {
    if (st->mismatches < 5) printf("log mismatch x=%a\n", (double)x);
    st->mismatches++;
  }
}

static void check_sin(float x, stats* st) {
  float H, L, f;
  st->n++;
  if (sampo_sin_pair(x, &H, &L)) {
    double ref = sin((double)x);
    if (ref != 0.0) {
      double rel = fabs(((double)H + (double)L) - ref) / fabs(ref);
      if (rel > st->maxrel) st->maxrel = rel;
    }
    if (!sampo_round_test(H, L, SAMPO_FAST_SIN_EPS, &f)) st->fallbacks++;
  } else {
    st->fallbacks++;
  }
  if (sampo_f2bits(sampo_sinf_bm(x)) != sampo_f2bits(sampo_sinf(x))) {
    if (st->mismatches < 5) printf("sin mismatch x=%a\n", (double)x);
    st->mismatches++;
  }
}

static uint64_t next64(uint64_t* s) {  /* splitmix64 */
  uint64_t z = (*s += 0x9E3779B97F4A7C15ull);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

static void check_sporo(float s, float T, stats* st) {
  /* the increment as the step context computes it */
  double d = 1.0 / ((double)(111.0f / (T - 16.0f)) * 14.0);
  float dh, dm, dl, a, b, f;
  sampo_split_double(d, &dh, &dm, &dl);
  st->n++;
  sampo_two_sum(s, dh, &a, &b);
  if (!sampo_round_test(a, (b + dm) + dl, SAMPO_FAST_ADD_EPS, &f)) st->fallbacks++;
  float want = (float)((double)s + d);
  if (sampo_f2bits(sampo_sporo_add(s, dh, dm, dl, d)) != sampo_f2bits(want)) {
    if (st->mismatches < 5) printf("sporo mismatch s=%a T=%a\n", (double)s, (double)T);
    st->mismatches++;
  }
}

int main(int argc, char** argv) {
  const uint32_t stride = argc > 1 ? (uint32_t)strtoul(argv[1], NULL, 10) : 1u;
  const long long sporo_cases = argc > 2 ? atoll(argv[2]) : 1000000;
  const uint32_t lo = sampo_f2bits(0x1p-32f), hi = sampo_f2bits(1.0f);
  stats sl = {0, 0, 0, 0}, ss = {0, 0, 0, 0}, sp = {0, 0, 0, 0};
  check_log(0.0f, &sl);
  check_sin(0.0f, &ss);
  const long long span = (long long)(hi - lo) / stride + 1;
#pragma omp parallel
  {
    stats a = {0, 0, 0, 0}, b = {0, 0, 0, 0};
#pragma omp for schedule(static)
    for (long long j = 0; j < span; j++) {
      const float u = sampo_bits2f(lo + (uint32_t)(j * stride));
      check_log(u, &a);
      check_sin(0x1.921fb6p+2f * u, &b);
    }
#pragma omp critical
    { merge(&sl, &a); merge(&ss, &b); }
  }
  /* sporogonic development: random values and accumulation runs */
#pragma omp parallel
  {
    stats a = {0, 0, 0, 0};
#pragma omp for schedule(static)
    for (long long j = 0; j < sporo_cases; j++) {
      uint64_t st = 0x5A17ull + (uint64_t)j;
      const uint64_t r = next64(&st);
      const float T = 16.0f + (float)((r >> 40) % 28000u) * 0.001f + 0.0005f;
      if (j & 1) {
        check_sporo((float)((r & 0xFFFFFFu) * 0x1p-18), T, &a);   /* s in [0, 64) */
      } else {
        float s = 0.0f;
        double d = 1.0 / ((double)(111.0f / (T - 16.0f)) * 14.0);
        for (int h = 0; h < 64; h++) {
          check_sporo(s, T, &a);
          s = (float)((double)s + d);
        }
      }
    }
#pragma omp critical
    merge(&sp, &a);
  }
  printf("log   n=%lld maxrel=2^%.2f fallbacks=%lld mismatches=%lld\n", sl.n, log2(sl.maxrel), sl.fallbacks, sl.mismatches);
  printf("sin   n=%lld maxrel=2^%.2f fallbacks=%lld mismatches=%lld\n", ss.n, log2(ss.maxrel), ss.fallbacks, ss.mismatches);
  printf("sporo n=%lld fallbacks=%lld mismatches=%lld\n", sp.n, sp.fallbacks, sp.mismatches);
  return (sl.mismatches || ss.mismatches || sp.mismatches) ? 1 : 0;
}
