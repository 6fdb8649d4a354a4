// sampo_host.cpp - host helpers of the C ABI: the glibc-compatible seed
// stream and the readers of the reference's input files.
#include <stdio.h>
#include <string.h>
#include "../../include/sampo.h"

// glibc's srand/rand (TYPE_3 state, the default) as a published algorithm:
// r[0] = seed (1 when 0); r[i] = 16807 * r[i-1] mod (2^31 - 1) for
// i = 1..30, evaluated on a signed 32-bit value with Schrage's method;
// r[31..33] = r[0..2]; r[i] = r[i-3] + r[i-31] mod 2^32 afterwards; the first
// 310 values past r[33] are discarded and each output is the value >> 1.
// The state lives in the caller's struct, so independent streams (one per
// replicate or request) can run side by side.
extern "C" void sampo_rand_seed(sampo_rand_state* st, uint32_t seed) {
  int32_t w = (int32_t)(seed == 0 ? 1u : seed);
  st->r[0] = (uint32_t)w;
  for (int i = 1; i < 31; i++) {
    int64_t hi = w / 127773, lo = w % 127773;
    int64_t t = 16807 * lo - 2836 * hi;
    if (t < 0) t += 2147483647;
    w = (int32_t)t;
    st->r[i] = (uint32_t)w;
  }
  st->i = 34;
  for (int k = 0; k < 310; k++) (void)sampo_rand_next(st);
}

extern "C" uint32_t sampo_rand_next(sampo_rand_state* st) {
  uint32_t i = st->i++;
  uint32_t v = st->r[i % 31] + st->r[(i - 3) % 31];
  st->r[i % 31] = v;
  return v >> 1;
}

// generateSeeds (src/abms.c:145-150): z1, z2, z3, z4 for seed slot 0, then 1..3.
extern "C" void sampo_rand_seeds(sampo_rand_state* st, sampo_seeds* out, uint32_t nsteps) {
  for (uint32_t s = 0; s < nsteps; s++)
    for (int k = 0; k < 4; k++) {
      sampo_seeds& z = out[(size_t)s * 4 + k];
      z.z1 = sampo_rand_next(st);
      z.z2 = sampo_rand_next(st);
      z.z3 = sampo_rand_next(st);
      z.z4 = sampo_rand_next(st);
    }
}

// readSingleValFile (src/abms.c:94-108).
extern "C" int sampo_read_temperature_file(const char* path, float* out, uint32_t nsteps) {
  FILE* f = fopen(path, "r");
  if (!f) return SAMPO_ERR_IO;
  for (uint32_t i = 0; i < nsteps; i++)
    if (fscanf(f, "%f", &out[i]) != 1) { fclose(f); return SAMPO_ERR_IO; }
  fclose(f);
  return SAMPO_OK;
}

// readEnvironment (src/abms.c:110-137): four coverage*effectiveness products
// (IRS, ITN, larvicide, ovitrap) and bloodmealSuccess per row.
extern "C" int sampo_read_environment_file(const char* path, sampo_environment* out, uint32_t nsteps, float cc) {
  FILE* f = fopen(path, "r");
  if (!f) return SAMPO_ERR_IO;
  for (uint32_t i = 0; i < nsteps; i++) {
    float c, e;
    sampo_environment& v = out[i];
    if (fscanf(f, "%f, %f, ", &c, &e) != 2) goto short_file;
    v.IRSValue = c * e;
    if (fscanf(f, "%f, %f, ", &c, &e) != 2) goto short_file;
    v.ITNValue = c * e;
    if (fscanf(f, "%f, %f, ", &c, &e) != 2) goto short_file;
    v.larvacideValue = c * e;
    if (fscanf(f, "%f, %f, ", &c, &e) != 2) goto short_file;
    v.oviTrapValue = c * e;
    if (fscanf(f, "%f", &v.bloodmealSuccess) != 1) goto short_file;
    v.carryingCapacity = cc;
  }
  fclose(f);
  return SAMPO_OK;
short_file:
  fclose(f);
  return SAMPO_ERR_IO;
}
