/*
 * sampo_oracle.h - TEST INFRASTRUCTURE ONLY.
 *
 * CPU restatement of the SAMPO per-step agent update (the reference's
 * .cl files under kernel/ plus the host loop in src/abms.c), used as the parity oracle
 * for the CUDA path and as the timed CPU baseline. Only tests/, the smoke
 * check and bench.py's CPU-baseline leg may load this code; the product
 * (sampo_gb300/) never does.
 *
 * Pinning: the restatement is checked against "ref-as-C" (oracle/ref_build:
 * the reference's own kernels and src/abms.c compiled from the reference
 * tree as C/C++ over an emulated lib_icl) through golden traces committed
 * under tests/golden/. See tests/test_oracle_golden.py.
 */
#ifndef SAMPO_ORACLE_H
#define SAMPO_ORACLE_H
#include <stdint.h>
#ifdef __cplusplus
extern "C" {
#endif

typedef struct { uint32_t start, end; } orc_range;
/* struct Population (include/agent.h:109-123), state order EGG..GRAVID */
typedef struct { orc_range r[8]; uint32_t L1de, numFemale, numPotInf; } orc_pop;
/* struct Environment (include/agent.h:22-35) */
typedef struct { float bloodmealSuccess, ITNValue, IRSValue, carryingCapacity, larvacideValue, oviTrapValue; } orc_env;
/* struct Seeds (include/agent.h:145-150) */
typedef struct { uint32_t z1, z2, z3, z4; } orc_seeds;
/* Population + BitesNcycles at the start of a step: what printStats uses. */
typedef struct { orc_pop pop; uint32_t numCycles, sumCycles, numBites, numInfectBites; } orc_row;

/* Host SoA view of a pool (slots [0, n)). state is 0..7 (EGG..GRAVID). */
typedef struct {
  float *age, *his, *delay, *sporo;
  uint32_t *uni, *avail, *cycle, *hbc, *batches;
  uint8_t *female, *state;
} orc_pool_view;

typedef struct orc_sim orc_sim;

orc_sim* orc_create(uint64_t capacity, int nthreads);
void orc_destroy(orc_sim* s);
/* initAgents over [0,n) (kernel/initAgents.cl:26-65) and the initial ranges of
 * src/abms.c:201-219. age_days_max >= 0 draws ageInHours = hoursInState =
 * 24*U{0..age_days_max} per slot from splitmix64(age_seed, slot). */
int orc_init_eggs(orc_sim* s, uint32_t n, float T0, const orc_seeds seeds[4], int age_days_max, uint64_t age_seed);
int orc_load_pool(orc_sim* s, const orc_pop* pop, const orc_pool_view* v);
int orc_read_pool(orc_sim* s, orc_pop* pop, orc_pool_view* v);  /* v arrays sized >= pop end */
/* One hourly step: calcStats, kill, update, egg creation, compaction. */
int orc_step(orc_sim* s, const orc_env* env, float T, uint32_t worldTime, const orc_seeds seeds[4], orc_row* out);
/* Stats of the current pool (what the next step would report). */
void orc_current_row(orc_sim* s, orc_row* out);
void orc_histogram(orc_sim* s, uint32_t out[100]);
uint64_t orc_pool_hash(orc_sim* s);
uint32_t orc_pool_end(orc_sim* s);

/* glibc srand/rand restatement (additive feedback generator, TYPE_3). */
typedef struct { uint32_t r[31]; uint32_t i; } orc_glibc_rand;
void orc_rand_seed(orc_glibc_rand* g, uint32_t seed);
uint32_t orc_rand_next(orc_glibc_rand* g);
/* Test hook: fn 0 exp, 1 log, 2 sin, 3 pow (x, y) with the shared definitions. */
void orc_eval_math(int fn, const float* x, const float* y, float* out, uint32_t n);

#ifdef __cplusplus
}
#endif
#endif
