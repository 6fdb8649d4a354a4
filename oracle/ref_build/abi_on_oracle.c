/*
 * abi_on_oracle.c - TEST INFRASTRUCTURE ONLY. The part of the C ABI
 * (include/sampo.h) that sampo_gb300/host/icl_sampo.cpp calls, implemented on
 * the CPU oracle (oracle/sampo_oracle.c) in place of libsampo_cuda.so, so
 * that the reference's unmodified src/abms.c over icl_sampo.cpp runs on a
 * machine without a GPU and its output can be compared with the golden
 * traces. The GPU library behind the same calls is checked against the same
 * oracle by the GPU tests.
 */
#include <stdlib.h>
#include <string.h>
#include "sampo.h"
#include "../sampo_oracle.h"

struct sampo_sim {
  orc_sim* o;
  float T0;
};

int sampo_abi_version(void) { return SAMPO_ABI_VERSION; }
const char* sampo_last_error(const sampo_sim* s) { (void)s; return "oracle stand-in"; }

int sampo_create(const sampo_config* cfg, sampo_sim** out) {
  if (!cfg || !out) return SAMPO_ERR_ARG;
  sampo_sim* s = (sampo_sim*)calloc(1, sizeof(sampo_sim));
  s->o = orc_create(cfg->capacity, 0);
  if (!s->o) { free(s); return SAMPO_ERR_CAPACITY; }
  *out = s;
  return SAMPO_OK;
}
int sampo_destroy(sampo_sim* s) {
  if (s) { orc_destroy(s->o); free(s); }
  return SAMPO_OK;
}
int sampo_set_inputs(sampo_sim* s, uint32_t first, const float* T, const sampo_environment* env, uint32_t n) {
  (void)env;
  if (first == 0 && n) s->T0 = T[0];
  return SAMPO_OK;
}
int sampo_init_population(sampo_sim* s, uint32_t n, const sampo_seeds init_seeds[4], int age_days_max, uint64_t age_seed) {
  return orc_init_eggs(s->o, n, s->T0, (const orc_seeds*)init_seeds, age_days_max, age_seed) == 0 ? SAMPO_OK : SAMPO_ERR_CAPACITY;
}
int sampo_step(sampo_sim* s, const sampo_environment* env, float T, uint32_t wt, const sampo_seeds seeds[4], sampo_stats_row* row) {
  orc_row r;
  if (orc_step(s->o, (const orc_env*)env, T, wt, (const orc_seeds*)seeds, &r) != 0) return SAMPO_ERR_CAPACITY;
  if (row) memcpy(row, &r, sizeof(*row));
  return SAMPO_OK;
}
int sampo_current_row(sampo_sim* s, sampo_stats_row* row) {
  orc_row r;
  orc_current_row(s->o, &r);
  memcpy(row, &r, sizeof(*row));
  return SAMPO_OK;
}
int sampo_histogram(sampo_sim* s, uint32_t out[100]) {
  orc_histogram(s->o, out);
  return SAMPO_OK;
}
int sampo_species_compile(const char* path, int device, char* log, size_t log_size, sampo_species** out) {
  (void)path; (void)device; (void)out;
  if (log && log_size) strncpy(log, "the oracle stand-in has the built-in species only", log_size - 1);
  return SAMPO_ERR_UNSUPPORTED;
}
int sampo_set_species(sampo_sim* s, const sampo_species* sp) { (void)s; (void)sp; return SAMPO_ERR_UNSUPPORTED; }
void sampo_species_free(sampo_species* sp) { (void)sp; }
