/*
 * sampo_oracle.c - TEST INFRASTRUCTURE ONLY (see sampo_oracle.h).
 *
 * Plain-C restatement of one SAMPO hourly step, written from the reference
 * and citing it line by line. Structure follows the reference's own kernel
 * sequence (src/abms.c:502-529): calcStats -> generateSeeds (caller) ->
 * killAgents -> updateAgents -> initAgents (new eggs) -> per-state scans ->
 * oldToNewAgents. The scan uses the semantics of the reference's serial scan
 * (kernel/serialScan.cl:83-106): the 0-based rank of a live agent among live
 * agents of the same new state, in slot order. Per-slot work is parallel
 * with OpenMP; every reduction is an integer sum, so results do not depend on
 * the thread count.
 *
 * Build: gcc -O2 -ffp-contract=off -fopenmp (contraction must stay off so
 * that float expressions round exactly as written, as in the reference).
 */
#include "sampo_oracle.h"
#include "../sampo_gb300/csrc/sampo_math.h"
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

enum { EGG = 0, LARVA, PUPA, IMMATURE, MATESEEKING, BMS, BMD, GRAVID, NSTATE };
#define LAYOUT_ALIGN 64u /* LOCAL_SIZE, include/agent.h:9-17: a layout constant */

typedef struct {
  float *age, *his, *delay, *sporo;
  uint32_t *uni, *avail, *cycle, *hbc, *batches;
  uint8_t *female, *state, *dead;
} pool_t;

struct orc_sim {
  uint64_t cap;
  pool_t p[2];
  int cur;
  orc_pop pop;           /* ranges of the current pool (reference pop[1]) */
  uint32_t bnc[4];       /* numCycles, sumCycles, numBites, numInfectBites */
  int nthreads;
  uint64_t* chunk_cnt;   /* per-chunk state counts for the parallel compaction */
  int nchunks;
};

/* ---------------- RNG: include/gpuRand.h:14-50 ---------------- */
static inline uint32_t taus_step(uint32_t z, int S1, int S2, int S3, uint32_t M) {
  uint32_t b = (((z << S1) ^ z) >> S2);
  return (((z & M) << S3) ^ b);
}
static inline float hybrid_taus(const orc_seeds* s, uint32_t gid) {
  uint32_t z1 = s->z1 + 128u;
  uint32_t z2 = s->z2 + 128u + gid;
  uint32_t z3 = s->z3 + 128u;
  uint32_t z4 = s->z4 * gid;
  uint32_t v = taus_step(z1, 13, 19, 12, 4294967294u) ^ taus_step(z2, 2, 25, 4, 4294967288u) ^
               taus_step(z3, 3, 11, 17, 4294967280u) ^ (1664525u * z4 + 1013904223u);
  return 2.3283064365387e-10f * (float)v;
}
/* include/gpuRand.h:56-63; called with seeds+1, so u0 uses slot 1, u1 slot 2 */
static inline float box_muller(const orc_seeds* s, uint32_t gid, float mean, float sd) {
  float u0 = hybrid_taus(&s[0], gid), u1 = hybrid_taus(&s[1], gid);
  float r = sqrtf(-2.0f * sampo_logf(u0));
  float theta = (2.0f * 3.14159274101257f) * u1; /* 2*M_PI_F*u1 */
  return (r * sampo_sinf(theta)) * sd + mean;
}

/* ---------------- species plugin: include/properties.h ---------------- */
static inline float eggs_incubation(float T) { return -0.923f * T + 60.923f; }         /* :29-31 */
static inline float eggs_hatching(float p) {                                              /* :39-60 */
  float m, b;
  if (p < 0.5f) { m = 48.0f; b = 0.0f; }
  else if (p < 0.85f) { m = 68.5714f; b = -10.2857f; }
  else if (p < 0.90f) { m = 480.0f; b = -360.0f; }
  else if (p < 0.94f) { m = 600.00f; b = -468.0f; }
  else { m = 2400.0f; b = -2160.0f; }
  return (float)sampo_f2u_sat(m * p + b + 0.5f);
}
static const float dev_rates[32] = {                                                     /* :94-98 */
  0.000175044f, 0.000549094f, 0.00109031f, 0.001494158f, 0.001752487f, 0.001962866f, 0.002171238f,
  0.002392989f, 0.002633689f, 0.00289619f, 0.003182685f, 0.003495287f, 0.003836204f, 0.004207789f,
  0.004612566f, 0.005053243f, 0.005532729f, 0.006054144f, 0.006620836f, 0.007236393f, 0.007904657f,
  0.008629745f, 0.009416051f, 0.010267388f, 0.011113704f, 0.011960019f, 0.012806335f, 0.010401163f,
  0.007995991f, 0.00033845f, 0.00000533086f, 0.0000000840986f};
/* :105-109. Returns 0 and sets *oob when the reference would read past the
 * 32-entry table (T >= 44 C, a known reference bug). */
static inline float larva_development(float T, int* oob) {
  float c = sampo_fminf(sampo_fmaxf(T, 12.0f), 48.0f);
  int i = (int)c - 12;
  if (i > 31) { *oob = 1; return 0.0f; }
  return dev_rates[i];
}
static inline float pupa_delay(float T) { return (float)(-0.923 * (double)T + 60.923); }  /* :133-135 (double) */
static inline float immature_delay(float T) { return -2.667f * T + 120.0f; }             /* :159-161 */
static inline float bm_digesting_delay(float T) { return -1.231f * T + 77.231f; }        /* :239-241 */
static inline int window_night(uint32_t wt) { return wt <= 6u || wt >= 18u; }            /* :117-119 etc. */

/* ---------------- splitmix64 for the optional initial ages ---------------- */
static inline uint64_t mix64(uint64_t z) {
  z += 0x9E3779B97F4A7C15ULL;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
  return z ^ (z >> 31);
}

/* ---------------- pool management ---------------- */
static int pool_alloc(pool_t* p, uint64_t n) {
  memset(p, 0, sizeof(*p));
  p->age = (float*)calloc(n, 4); p->his = (float*)calloc(n, 4);
  p->delay = (float*)calloc(n, 4); p->sporo = (float*)calloc(n, 4);
  p->uni = (uint32_t*)calloc(n, 4); p->avail = (uint32_t*)calloc(n, 4);
  p->cycle = (uint32_t*)calloc(n, 4); p->hbc = (uint32_t*)calloc(n, 4);
  p->batches = (uint32_t*)calloc(n, 4);
  p->female = (uint8_t*)calloc(n, 1); p->state = (uint8_t*)calloc(n, 1); p->dead = (uint8_t*)calloc(n, 1);
  return p->age && p->his && p->delay && p->sporo && p->uni && p->avail && p->cycle && p->hbc &&
         p->batches && p->female && p->state && p->dead;
}
static void pool_free(pool_t* p) {
  free(p->age); free(p->his); free(p->delay); free(p->sporo); free(p->uni); free(p->avail);
  free(p->cycle); free(p->hbc); free(p->batches); free(p->female); free(p->state); free(p->dead);
}

orc_sim* orc_create(uint64_t capacity, int nthreads) {
  orc_sim* s = (orc_sim*)calloc(1, sizeof(orc_sim));
  if (!s) return NULL;
  s->cap = capacity;
  if (!pool_alloc(&s->p[0], capacity) || !pool_alloc(&s->p[1], capacity)) { orc_destroy(s); return NULL; }
#ifdef _OPENMP
  s->nthreads = nthreads > 0 ? nthreads : omp_get_max_threads();
#else
  s->nthreads = 1; (void)nthreads;
#endif
  s->nchunks = s->nthreads * 4;
  s->chunk_cnt = (uint64_t*)calloc((size_t)s->nchunks * NSTATE, sizeof(uint64_t));
  return s;
}
void orc_destroy(orc_sim* s) {
  if (!s) return;
  pool_free(&s->p[0]); pool_free(&s->p[1]); free(s->chunk_cnt); free(s);
}
uint32_t orc_pool_end(orc_sim* s) { return s->pop.r[GRAVID].end; }

/* Slot validity by range, as every reference kernel tests it
 * (e.g. kernel/killAgents.cl:28-35). Returns the range index or -1. */
static inline int slot_range(const orc_pop* pop, uint32_t gid) {
  if (gid < pop->r[EGG].end) return EGG;
  for (int k = 1; k < NSTATE; k++) {
    if (gid < pop->r[k].start) return -1;
    if (gid < pop->r[k].end) return k;
  }
  return -1;
}

/* ---------------- egg creation: kernel/initAgents.cl:26-65 ---------------- */
static void create_eggs(pool_t* p, uint32_t n, float T, const orc_seeds* seeds) {
  float inc = eggs_incubation(T);
  #pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < (int64_t)n; i++) {
    uint32_t id = (uint32_t)i;
    p->state[id] = EGG; p->dead[id] = 0;
    p->age[id] = 0.0f; p->his[id] = 0.0f;
    p->female[id] = hybrid_taus(&seeds[3], id) <= 0.5f;
    p->sporo[id] = 0.0f;
    p->hbc[id] = 0u; p->avail[id] = 0u; p->cycle[id] = 0u;
    p->uni[id] = 0u; /* cumulativeLarvalDelay = 0.0f */
    float prob = hybrid_taus(&seeds[2], id);
    p->delay[id] = inc + eggs_hatching(prob);
    p->batches[id] = 0u;
  }
}

int orc_init_eggs(orc_sim* s, uint32_t n, float T0, const orc_seeds seeds[4], int age_days_max, uint64_t age_seed) {
  if ((uint64_t)n + 1 > s->cap) return -1;
  s->cur = 0;
  pool_t* p = &s->p[0];
  create_eggs(p, n, T0, seeds);
  if (age_days_max >= 0) {
    uint64_t m = (uint64_t)age_days_max + 1;
    for (uint32_t i = 0; i < n; i++) {
      uint64_t z = mix64(age_seed ^ mix64((uint64_t)i));
      float h = 24.0f * (float)(uint32_t)((z >> 32) % m);
      p->age[i] = h; p->his[i] = h;
    }
  }
  memset(&s->pop, 0, sizeof(s->pop));
  s->pop.r[EGG].start = 0; s->pop.r[EGG].end = n;
  if (age_days_max < 0) {
    /* src/abms.c:201-219: every empty range at [n+1, n+1). */
    for (int k = 1; k < NSTATE; k++) { s->pop.r[k].start = n + 1; s->pop.r[k].end = n + 1; }
  } else {
    /* Aged initial eggs are an extension. They can hatch in the first step,
     * and with the reference's shared [n+1, n+1) ranges the first
     * compaction would read one prefix-sum entry for several range ends
     * (kernel/oldToNewAgents.cl:270,279,288) and create agents from
     * uninitialised memory. Use the padded layout a compaction produces. */
    for (int k = 1; k < NSTATE; k++) {
      s->pop.r[k].start = ((s->pop.r[k - 1].end + LAYOUT_ALIGN) / LAYOUT_ALIGN) * LAYOUT_ALIGN;
      s->pop.r[k].end = s->pop.r[k].start;
    }
  }
  if ((uint64_t)s->pop.r[GRAVID].end > s->cap) return -1;
  memset(s->bnc, 0, sizeof(s->bnc));
  return 0;
}

int orc_load_pool(orc_sim* s, const orc_pop* pop, const orc_pool_view* v) {
  if ((uint64_t)pop->r[GRAVID].end + LAYOUT_ALIGN > s->cap) return -1;
  s->cur = 0;
  pool_t* p = &s->p[0];
  uint32_t n = pop->r[GRAVID].end;
  memcpy(p->age, v->age, (size_t)n * 4); memcpy(p->his, v->his, (size_t)n * 4);
  memcpy(p->delay, v->delay, (size_t)n * 4); memcpy(p->sporo, v->sporo, (size_t)n * 4);
  memcpy(p->uni, v->uni, (size_t)n * 4); memcpy(p->avail, v->avail, (size_t)n * 4);
  memcpy(p->cycle, v->cycle, (size_t)n * 4); memcpy(p->hbc, v->hbc, (size_t)n * 4);
  memcpy(p->batches, v->batches, (size_t)n * 4); memcpy(p->female, v->female, n);
  memcpy(p->state, v->state, n); memset(p->dead, 0, n);
  s->pop = *pop;
  memset(s->bnc, 0, sizeof(s->bnc));
  return 0;
}

int orc_read_pool(orc_sim* s, orc_pop* pop, orc_pool_view* v) {
  pool_t* p = &s->p[s->cur];
  uint32_t n = s->pop.r[GRAVID].end;
  *pop = s->pop;
  if (!v) return 0;
  memcpy(v->age, p->age, (size_t)n * 4); memcpy(v->his, p->his, (size_t)n * 4);
  memcpy(v->delay, p->delay, (size_t)n * 4); memcpy(v->sporo, p->sporo, (size_t)n * 4);
  memcpy(v->uni, p->uni, (size_t)n * 4); memcpy(v->avail, p->avail, (size_t)n * 4);
  memcpy(v->cycle, p->cycle, (size_t)n * 4); memcpy(v->hbc, p->hbc, (size_t)n * 4);
  memcpy(v->batches, p->batches, (size_t)n * 4); memcpy(v->female, p->female, n);
  memcpy(v->state, p->state, n);
  return 0;
}

/* ---------------- calcStats: kernel/calcL1de.cl, kernel/calcGender.cl ---------------- */
void orc_current_row(orc_sim* s, orc_row* out) {
  pool_t* p = &s->p[s->cur];
  orc_pop* pop = &s->pop;
  uint32_t l1 = 0, fem = 0, inf = 0;
  /* calcL1dePerGroup/Total (kernel/calcL1de.cl:28-92): sum of floor(age/24)
   * over the larva range; 0 when the range is empty. u32 wrap-around. */
  if (pop->r[LARVA].end > pop->r[LARVA].start) {
    #pragma omp parallel for reduction(+:l1) schedule(static)
    for (int64_t i = pop->r[LARVA].start; i < (int64_t)pop->r[LARVA].end; i++)
      l1 += sampo_f2u_sat(p->age[i] / 24.0f);
  }
  /* calcFemalesPerGroup (kernel/calcGender.cl:17-54): adult ranges only. */
  for (int k = IMMATURE; k <= GRAVID; k++) {
    uint32_t a = pop->r[k].start, b = pop->r[k].end;
    #pragma omp parallel for reduction(+:fem,inf) schedule(static)
    for (int64_t i = a; i < (int64_t)b; i++) {
      if (p->female[i]) { fem++; inf += p->sporo[i] >= 1.0f; }
    }
  }
  out->pop = *pop;
  out->pop.L1de = l1; out->pop.numFemale = fem; out->pop.numPotInf = inf;
  out->numCycles = s->bnc[0]; out->sumCycles = s->bnc[1];
  out->numBites = s->bnc[2]; out->numInfectBites = s->bnc[3];
}

/* ---------------- one step ---------------- */
int orc_step(orc_sim* s, const orc_env* env, float T, uint32_t worldTime, const orc_seeds seeds[4], orc_row* out) {
  orc_row row;
  orc_current_row(s, &row);          /* calcStats, src/abms.c:230-310 */
  if (out) *out = row;
  orc_pop pop = row.pop;             /* reference pop[0] for this step */
  pool_t* p = &s->p[s->cur];
  pool_t* q = &s->p[s->cur ^ 1];
  const uint32_t end = pop.r[GRAVID].end;
  const float cc = env->carryingCapacity;

  /* killAgents gid 0 (kernel/killAgents.cl:37-50) */
  uint32_t totalBiomass = pop.L1de + pop.r[EGG].end + (pop.r[PUPA].end - pop.r[PUPA].start);
  s->bnc[0] = s->bnc[1] = s->bnc[2] = s->bnc[3] = 0;

  /* Hourly mortality of eggs and pupae does not depend on the agent
   * (kernel/killAgents.cl:103-115, 135-147). */
  const float hmr_aquatic = 1.0f - sampo_powf(1.0f - 0.1f, 1.0f / 24.0f);

  uint32_t newEggs = 0, nb = 0, nib = 0, ncy = 0, scy = 0;
  int oob = 0;
  #pragma omp parallel for schedule(static) reduction(+:newEggs,nb,nib,ncy,scy) reduction(|:oob)
  for (int64_t gi = 0; gi < (int64_t)end; gi++) {
    uint32_t gid = (uint32_t)gi;
    int rg = slot_range(&pop, gid);
    if (rg < 0) continue;
    /* ---- killAgents (kernel/killAgents.cl:52-147) ---- */
    float age0 = p->age[gid];
    uint32_t ageInDays = sampo_f2u_sat(sampo_fminf(age0 / 24.0f, 99.0f));
    float prob = hybrid_taus(&seeds[0], gid);
    float hmr;
    if (rg >= IMMATURE) {
      const float a = 0.1f, B = 25.0f, sg = 0.1f;
      float e = sampo_expf((float)ageInDays / B);
      float dmr = (a * e) / (1.0f + (a * B * sg * (e - 1.0f)));
      float dsr = 1.0f - dmr;
      float hsr = sampo_powf(dsr, 1.0f / 24.0f);
      hmr = 1.0f - hsr;
    } else if (rg == LARVA) {
      float dmr = 0.1f * sampo_expf((float)pop.L1de / ((float)ageInDays * cc * 1.0f));
      dmr = sampo_fminf(dmr, 0.8f);
      float dsr = 1.0f - dmr;
      float hsr = sampo_powf(dsr, 1.0f / 24.0f);
      hmr = 1.0f - hsr;
    } else {
      hmr = hmr_aquatic;
    }
    uint8_t dead = prob <= hmr;
    p->state[gid] = (uint8_t)rg;
    p->dead[gid] = dead;
    if (dead) continue;

    /* ---- updateAgents (kernel/updateAgents.cl:57-270) ---- */
    float age = age0 + 1.0f, his = p->his[gid] + 1.0f;
    float delay = p->delay[gid];
    uint32_t hbc = p->hbc[gid];
    {
      double inc = (double)(T > 16.0f && hbc > 0u) * (1.0 / ((double)(111.0f / (T - 16.0f)) * 14.0));
      p->sporo[gid] = (float)((double)p->sporo[gid] + inc);
    }
    float sporo = p->sporo[gid];
    uint8_t st = (uint8_t)rg, isdead = 0;
    switch (rg) {
      case EGG:
        if (his >= delay) {
          age = 24.0f; his = 0.0f;
          delay = box_muller(&seeds[1], gid, 1.0f, 0.1f);  /* larvaDelay */
          st = LARVA;
        }
        break;
      case LARVA: {
        if (env->larvacideValue > 0.0f && his == 1.0f) {
          float l = hybrid_taus(&seeds[2], gid);
          if (l <= env->larvacideValue) { isdead = 1; break; }
        }
        float cld = sampo_bits2f(p->uni[gid]) + larva_development(T, &oob);
        p->uni[gid] = sampo_f2bits(cld);
        if (cld >= delay && window_night(worldTime)) {
          his = 0.0f; delay = pupa_delay(T); st = PUPA;
        }
        break;
      }
      case PUPA:
        if (his >= delay && window_night(worldTime)) {
          age = 0.0f; his = 0.0f; delay = immature_delay(T); st = IMMATURE;
        }
        break;
      case IMMATURE:
        if (his >= delay) { delay = 1.0f; his = 0.0f; st = MATESEEKING; }
        break;
      case MATESEEKING:
        if (his >= delay && p->female[gid] && worldTime == 18u) { his = 0.0f; delay = 0.0f; st = BMS; }
        break;
      case BMS:
        p->cycle[gid] += 1u;
        if (his >= delay && window_night(worldTime)) {
          float bm = hybrid_taus(&seeds[1], gid);
          if (bm <= env->bloodmealSuccess) {
            if (env->ITNValue * 1.0f * 1.0f > 0.0f) {
              float itn = hybrid_taus(&seeds[2], gid);
              if (itn <= env->ITNValue * 1.0f * 1.0f) { isdead = 1; break; }
            }
            hbc += 1u;
            p->hbc[gid] = hbc;
            nb++;
            his = 0.0f; delay = bm_digesting_delay(T); st = BMD;
            if (sporo >= 1.0f) nib++;
          }
        }
        break;
      case BMD:
        if (env->IRSValue * 1.0f > 0.0f) {
          float irs = hybrid_taus(&seeds[2], gid);
          if (irs <= env->IRSValue * 1.0f) { isdead = 1; break; }
        }
        p->cycle[gid] += 1u;
        if (his >= delay) {
          if (p->avail[gid] <= 0u && p->female[gid]) {
            /* generateEggs (include/properties.h:257-266) */
            uint32_t eggs = sampo_f2u_sat(box_muller(&seeds[1], gid, 170.0f, 30.0f) + 0.5f);
            uint32_t nbat = p->batches[gid];
            eggs = sampo_f2u_sat((float)eggs * sampo_powf(0.8f, (float)nbat) + 0.5f);
            p->batches[gid] = nbat + 1u;
            p->avail[gid] = eggs;
          }
          his = 0.0f; p->uni[gid] = 0u; st = GRAVID;
        }
        break;
      case GRAVID:
        p->cycle[gid] += 1u;
        if (window_night(worldTime)) {
          int lay = hybrid_taus(&seeds[1], gid) < 0.25f;
          if (lay) {
            uint32_t avail = p->avail[gid];
            uint8_t d2 = 0;
            if (env->oviTrapValue > 0.0f) {
              float ov = hybrid_taus(&seeds[2], gid);
              if (ov <= env->oviTrapValue) { d2 = 1; avail = 0u; }
            }
            if (!d2) {
              /* layEggs (include/properties.h:296-307) */
              uint32_t ovi = p->uni[gid];
              float nbm = (float)totalBiomass / (((float)ovi + 1.0f) * env->carryingCapacity);
              float pbm = sampo_fmaxf(0.0f, 1.0f - nbm);
              uint32_t pe = sampo_f2u_sat(ceilf((float)avail * pbm));
              newEggs += pe;
              avail = avail - pe;
            }
            p->uni[gid] += 1u;
            p->avail[gid] = avail;
            if (avail == 0u) {
              ncy++; scy += p->cycle[gid];
              p->cycle[gid] = 0u;
              his = 0.0f; delay = 0.0f; st = BMS;
            }
            if (d2) isdead = 1;
          }
        }
        break;
    }
    if (isdead) { p->dead[gid] = 1; continue; }
    p->age[gid] = age; p->his[gid] = his; p->delay[gid] = delay; p->state[gid] = st;
  }
  if (oob) return -2;
  s->bnc[0] = ncy; s->bnc[1] = scy; s->bnc[2] = nb; s->bnc[3] = nib;

  /* ---- new layout: kernel/oldToNewAgents.cl:57-95 ---- */
  const int nch = s->nchunks;
  uint64_t* cc8 = s->chunk_cnt;
  memset(cc8, 0, sizeof(uint64_t) * (size_t)nch * NSTATE);
  #pragma omp parallel for schedule(static)
  for (int c = 0; c < nch; c++) {
    uint64_t lo = (uint64_t)end * c / nch, hi = (uint64_t)end * (c + 1) / nch;
    uint64_t* cnt = cc8 + (size_t)c * NSTATE;
    for (uint64_t i = lo; i < hi; i++)
      if (slot_range(&pop, (uint32_t)i) >= 0 && !p->dead[i]) cnt[p->state[i]]++;
  }
  uint64_t tot[NSTATE] = {0};
  for (int c = 0; c < nch; c++)
    for (int k = 0; k < NSTATE; k++) { uint64_t t = cc8[(size_t)c * NSTATE + k]; cc8[(size_t)c * NSTATE + k] = tot[k]; tot[k] += t; }
  orc_pop np;
  memset(&np, 0, sizeof(np));
  np.r[EGG].start = 0;
  np.r[EGG].end = (uint32_t)tot[EGG] + newEggs;
  for (int k = 1; k < NSTATE; k++) {
    np.r[k].start = ((np.r[k - 1].end + LAYOUT_ALIGN) / LAYOUT_ALIGN) * LAYOUT_ALIGN;
    np.r[k].end = np.r[k].start + (uint32_t)tot[k];
  }
  if ((uint64_t)np.r[GRAVID].end > s->cap) return -1; /* out of capacity */
  uint32_t base[NSTATE];
  base[EGG] = newEggs;
  for (int k = 1; k < NSTATE; k++) base[k] = np.r[k].start;

  /* New eggs at [0, newEggs) of the new buffer (initAgents as createEggs,
   * src/abms.c:391-397), then survivors in old slot order per state. */
  create_eggs(q, newEggs, T, seeds);
  #pragma omp parallel for schedule(static)
  for (int c = 0; c < nch; c++) {
    uint64_t lo = (uint64_t)end * c / nch, hi = (uint64_t)end * (c + 1) / nch;
    uint64_t off[NSTATE];
    for (int k = 0; k < NSTATE; k++) off[k] = base[k] + cc8[(size_t)c * NSTATE + k];
    for (uint64_t i = lo; i < hi; i++) {
      if (slot_range(&pop, (uint32_t)i) < 0 || p->dead[i]) continue;
      uint64_t d = off[p->state[i]]++;
      q->age[d] = p->age[i]; q->his[d] = p->his[i]; q->delay[d] = p->delay[i]; q->sporo[d] = p->sporo[i];
      q->uni[d] = p->uni[i]; q->avail[d] = p->avail[i]; q->cycle[d] = p->cycle[i]; q->hbc[d] = p->hbc[i];
      q->batches[d] = p->batches[i]; q->female[d] = p->female[i]; q->state[d] = p->state[i]; q->dead[d] = 0;
    }
  }
  s->pop = np;
  s->cur ^= 1;
  return 0;
}

/* ---------------- ageHistogram: kernel/ageHistogram.cl:13-35 ---------------- */
void orc_histogram(orc_sim* s, uint32_t out[100]) {
  pool_t* p = &s->p[s->cur];
  memset(out, 0, 100 * sizeof(uint32_t));
  for (int k = IMMATURE; k <= GRAVID; k++)
    for (uint32_t i = s->pop.r[k].start; i < s->pop.r[k].end; i++) {
      uint32_t bin = sampo_f2u_sat(p->age[i] / 24.0f);
      if (bin > 99u) bin = 99u;
      out[bin]++;
    }
}

/* ---------------- position-dependent pool hash ---------------- */
uint64_t orc_pool_hash(orc_sim* s) {
  pool_t* p = &s->p[s->cur];
  uint64_t h = 0;
  for (int k = 0; k < NSTATE; k++) {
    h += mix64(((uint64_t)k << 40) ^ ((uint64_t)s->pop.r[k].start << 20) ^ (uint64_t)s->pop.r[k].end);
    #pragma omp parallel for reduction(+:h) schedule(static)
    for (int64_t i = s->pop.r[k].start; i < (int64_t)s->pop.r[k].end; i++) {
      uint64_t x = mix64((uint64_t)i);
      x = mix64(x ^ ((uint64_t)p->state[i] | ((uint64_t)p->female[i] << 8)));
      x = mix64(x ^ sampo_f2bits(p->age[i])); x = mix64(x ^ sampo_f2bits(p->his[i]));
      x = mix64(x ^ sampo_f2bits(p->delay[i])); x = mix64(x ^ sampo_f2bits(p->sporo[i]));
      x = mix64(x ^ p->uni[i]); x = mix64(x ^ p->avail[i]); x = mix64(x ^ p->cycle[i]);
      x = mix64(x ^ p->hbc[i]); x = mix64(x ^ p->batches[i]);
      h += x;
    }
  }
  return h;
}

/* ---------------- glibc rand() restatement ----------------
 * srand/rand in glibc use an additive lagged-Fibonacci generator
 * r[i] = r[i-3] + r[i-31] (mod 2^32), seeded by r[0] = seed (1 if 0),
 * r[i] = 16807 * r[i-1] mod (2^31-1) for i < 31 (Schrage's method on a
 * signed 32-bit value), r[31..33] = r[0..2], the first 310 outputs
 * discarded, and each output shifted right by one bit. */
void orc_rand_seed(orc_glibc_rand* g, uint32_t seed) {
  int32_t w = (int32_t)(seed == 0 ? 1u : seed);
  g->r[0] = (uint32_t)w;
  for (int i = 1; i < 31; i++) {
    int64_t hi = w / 127773, lo = w % 127773;
    int64_t t = 16807 * lo - 2836 * hi;
    if (t < 0) t += 2147483647;
    w = (int32_t)t;
    g->r[i] = (uint32_t)w;
  }
  g->i = 34;
  for (int k = 0; k < 310; k++) (void)orc_rand_next(g);
}
uint32_t orc_rand_next(orc_glibc_rand* g) {
  uint32_t i = g->i++;
  uint32_t v = g->r[i % 31] + g->r[(i - 3) % 31];
  g->r[i % 31] = v;
  return v >> 1;
}

/* ---------------- test hooks: the shared transcendental definitions ---------------- */
void orc_eval_math(int fn, const float* x, const float* y, float* out, uint32_t n) {
  for (uint32_t i = 0; i < n; i++) {
    switch (fn) {
      case 0: out[i] = sampo_expf(x[i]); break;
      case 1: out[i] = sampo_logf(x[i]); break;
      case 2: out[i] = sampo_sinf(x[i]); break;
      case 3: out[i] = sampo_powf(x[i], y[i]); break;
      default: out[i] = 0.0f;
    }
  }
}
