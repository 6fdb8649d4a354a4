/*
 * sampo_main.c - the sampo command: SAMPO's driver (src/abms.c: main,
 * readArguments, run) with the OpenCL device code replaced by the GB300
 * library libsampo_cuda.so through its C ABI (include/sampo.h).
 *
 *   sampo [options] [temperatureFile [environmentFile [speciesHeader]]]
 *
 * Same positional arguments, defaults, input parsing and output as the
 * reference: the three header lines, one stats line per hourly step
 * (printStats, src/abms.c:67-81), the final ranges (printPopulation, :83-92),
 * histogram.txt (storeHistogram, :160-183) and the execution time. The seeds
 * come from the C library's rand() after srand(seed) in the reference's call
 * order (src/abms.c:145-150, 611, 671, 511): 16 draws before the initial
 * population, then 16 per step.
 *
 * Options (extensions; the reference hard-codes these):
 *   --seed S        srand seed (default: time(NULL), as the reference)
 *   --initial N     initial eggs (default 32000 = initialAgentCount)
 *   --cc X          carrying capacity (default 160000 = carryingCapacity)
 *   --steps K       hourly steps (default 8760 = maxSteps)
 *   --capacity C    slots per pool buffer (default 6000000 = maxAgents)
 *   --age-days D    initial egg ages 24*U{0..D} hours (seeded by --age-seed)
 *   --age-seed A
 *   --per-step      one library call per step (the reference's host loop);
 *                   default: day graphs in 30-day chunks; a printer thread
 *                   formats chunk k from one pinned row buffer while the GPU
 *                   runs chunk k + 1 into the other
 *   --device D      CUDA device
 *   --checkpoint K F  write a checkpoint of the state after K steps to F
 *   --resume F      continue from checkpoint F (same --seed, --cc and
 *                   inputs): prints the stats lines from its step on, which
 *                   equal those of the uninterrupted run
 * The species header (third argument, default properties.h): properties.h
 * is the built-in species; any other header file is compiled into the step
 * kernels at start-up (sampo_species_compile), as the reference compiles its
 * kernels with -DSPECIES=argv[3] (src/abms.c:565-568). The path is opened as
 * given (the reference looks it up on its kernel include path).
 */
#include <pthread.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

#include "sampo.h"

static double now_ms(void) {
  struct timespec ts;
  clock_gettime(CLOCK_MONOTONIC, &ts);
  return ts.tv_sec * 1e3 + ts.tv_nsec * 1e-6;
}

static void print_range(const sampo_range* r) {
  printf("[%d\t%d]\t%d\r\n", (int)r->start, (int)r->end, (int)(r->end - r->start));
}

static void print_population(const sampo_population* p) {
  static const char* names[8] = {"Eggs \t\t", "Larvae \t\t", "Pupae \t\t", "Immatures \t",
                                 "MateSeeking \t", "BMS \t\t", "BMD \t\t", "Gravids \t"};
  for (int k = 0; k < 8; k++) {
    printf("%s", names[k]);
    print_range(&p->r[k]);
  }
}

static uint32_t num(const sampo_population* p, int k) { return p->r[k].end - p->r[k].start; }

/* calcStats (src/abms.c:230-310) from the row of a step's start and printStats
 * (:67-81). The adult-range test uses the population of the previous step
 * (*prev), as the reference's host copy does. Returns the live agent count. */
static uint32_t print_stats(const sampo_stats_row* row, const sampo_population* prev, uint32_t step, float T) {
  const sampo_population* p = &row->pop;
  uint32_t ub = prev->r[SAMPO_IMMATURE].end;
  if (prev->r[SAMPO_BMS].end > ub) ub = prev->r[SAMPO_BMS].end;
  if (prev->r[SAMPO_BMD].end > ub) ub = prev->r[SAMPO_BMD].end;
  if (prev->r[SAMPO_GRAVID].end > ub) ub = prev->r[SAMPO_GRAVID].end;
  const uint32_t adults_range = ub - prev->r[SAMPO_IMMATURE].start;
  const uint32_t eggs = num(p, 0), larvae = num(p, 1), pupae = num(p, 2), imm = num(p, 3), mat = num(p, 4);
  const uint32_t bms = num(p, 5), bmd = num(p, 6), ovi = num(p, 7);
  const uint32_t l1 = larvae > 0 ? p->numLarvae1DayEquiv : 0;
  const uint32_t fem = adults_range > 0 ? p->numFemale : 0;
  const uint32_t inf = adults_range > 0 ? p->numPotentiallyInfective : 0;
  const uint32_t mature = imm + mat + bms + bmd + ovi;
  const float hours = 1.0f * (float)step;
  printf("%0.1f, %0.1f", hours, T);
  printf(", %d, %d, %d, %d, %d, %d, %d, %d, %d", (int)mature, (int)imm, (int)mat, (int)bms, (int)bmd, (int)ovi, (int)fem,
         (int)inf, (int)(mature - fem));
  printf(", %d, %d, %d, %d, %d, ", (int)eggs, (int)larvae, (int)pupae, (int)l1, (int)(l1 + eggs + pupae));
  const sampo_bites_cycles* b = &row->bnc;
  printf("%d, %d, %d\r\n", b->numCyclesReported > 0 ? (int)(b->sumCyclesReported / b->numCyclesReported) : 0,
         (int)b->numBitesReported, (int)b->numInfectBitesReported);
  return eggs + larvae + pupae + imm + mat + bms + bmd + ovi;
}

/* The reference's two asserts of calcStats (src/abms.c:306-307). */
static void check_agents(uint32_t n, uint64_t capacity) {
  if (!(n <= capacity * 0.95)) {
    fflush(stdout);
    fprintf(stderr, "sampo: Assertion `nAgents <= maxAgents * 0.95 && \"not enough capacity\"' failed.\n");
    abort();
  }
  if (!(n > 0)) {
    fflush(stdout);
    fprintf(stderr, "sampo: Assertion `nAgents > 0 && \"No more agents left\"' failed.\n");
    abort();
  }
}

static void draw_seeds(sampo_seeds* s) { /* generateSeeds (src/abms.c:145-150) */
  for (int i = 0; i < 4; i++) {
    s[i].z1 = (uint32_t)rand();
    s[i].z2 = (uint32_t)rand();
    s[i].z3 = (uint32_t)rand();
    s[i].z4 = (uint32_t)rand();
  }
}

/* The stats printer of the chunked mode: prints and checks the rows of one
 * chunk at a time, in step order, on its own thread. */
typedef struct {
  pthread_mutex_t mu;
  pthread_cond_t cv;
  const sampo_stats_row* rows;  /* chunk handed over, or NULL when idle */
  uint32_t first, n;
  int quit;
  const float* T;
  uint64_t capacity;
  sampo_population prev;        /* population of the last printed row */
} printer_t;

static void print_rows(printer_t* p, const sampo_stats_row* rows, uint32_t first, uint32_t n) {
  for (uint32_t j = 0; j < n; j++) {
    check_agents(print_stats(&rows[j], &p->prev, first + j, p->T[first + j]), p->capacity);
    p->prev = rows[j].pop;
  }
}

static void* printer_main(void* arg) {
  printer_t* p = (printer_t*)arg;
  pthread_mutex_lock(&p->mu);
  for (;;) {
    while (!p->rows && !p->quit) pthread_cond_wait(&p->cv, &p->mu);
    if (!p->rows) break;
    const sampo_stats_row* rows = p->rows;
    const uint32_t first = p->first, n = p->n;
    pthread_mutex_unlock(&p->mu);
    print_rows(p, rows, first, n);
    pthread_mutex_lock(&p->mu);
    p->rows = NULL;
    pthread_cond_broadcast(&p->cv);
  }
  pthread_mutex_unlock(&p->mu);
  return NULL;
}

/* Waits until the printer has finished the chunk it holds. */
static void printer_idle(printer_t* p) {
  pthread_mutex_lock(&p->mu);
  while (p->rows) pthread_cond_wait(&p->cv, &p->mu);
  pthread_mutex_unlock(&p->mu);
}

static void printer_submit(printer_t* p, const sampo_stats_row* rows, uint32_t first, uint32_t n) {
  pthread_mutex_lock(&p->mu);
  p->rows = rows;
  p->first = first;
  p->n = n;
  pthread_cond_broadcast(&p->cv);
  pthread_mutex_unlock(&p->mu);
}

static void fail(sampo_sim* s, const char* what, int rc) {
  fflush(stdout);
  fprintf(stderr, "sampo: %s failed (%d): %s\n", what, rc, s ? sampo_last_error(s) : "");
  exit(1);
}

int main(int argc, char** argv) {
  unsigned seed = (unsigned)time(NULL);
  uint32_t initial = 32000, steps = 8760;
  uint64_t capacity = 6000000ull, age_seed = 0;
  float cc = 160000.0f;
  int age_days = -1, per_step = 0, device = 0;
  uint32_t ck_step = 0xffffffffu;
  const char* ck_path = NULL;
  const char* resume_path = NULL;
  const char* pos[3] = {"temp.txt", "environment.txt", "properties.h"};
  int np = 0;
  for (int i = 1; i < argc; i++) {
    if (!strcmp(argv[i], "-h")) {
      printf("Usage: bin\\abms temperatueFileName environmentFileName speciesHeaderFileName\n");
      return 0;
    } else if (!strcmp(argv[i], "--seed") && i + 1 < argc) seed = (unsigned)strtoul(argv[++i], 0, 10);
    else if (!strcmp(argv[i], "--initial") && i + 1 < argc) initial = (uint32_t)strtoul(argv[++i], 0, 10);
    else if (!strcmp(argv[i], "--cc") && i + 1 < argc) cc = strtof(argv[++i], 0);
    else if (!strcmp(argv[i], "--steps") && i + 1 < argc) steps = (uint32_t)strtoul(argv[++i], 0, 10);
    else if (!strcmp(argv[i], "--capacity") && i + 1 < argc) capacity = strtoull(argv[++i], 0, 10);
    else if (!strcmp(argv[i], "--age-days") && i + 1 < argc) age_days = atoi(argv[++i]);
    else if (!strcmp(argv[i], "--age-seed") && i + 1 < argc) age_seed = strtoull(argv[++i], 0, 10);
    else if (!strcmp(argv[i], "--per-step")) per_step = 1;
    else if (!strcmp(argv[i], "--device") && i + 1 < argc) device = atoi(argv[++i]);
    else if (!strcmp(argv[i], "--checkpoint") && i + 2 < argc) {
      ck_step = (uint32_t)strtoul(argv[++i], 0, 10);
      ck_path = argv[++i];
    } else if (!strcmp(argv[i], "--resume") && i + 1 < argc) resume_path = argv[++i];
    else if (np < 3 && argv[i][0] != '-') pos[np++] = argv[i];
    else {
      fprintf(stderr, "sampo: unexpected argument %s\n", argv[i]);
      return 2;
    }
  }
  printf("Temperature:\t%s\nEnvironment:\t%s\nSpecies:\t%s\n", pos[0], pos[1], pos[2]);
  const char* base = strrchr(pos[2], '/');
  base = base ? base + 1 : pos[2];
  const int builtin_species = strcmp(base, "properties.h") == 0;
  if (steps == 0) return 0;
  srand(seed);

  float* T = (float*)malloc(sizeof(float) * steps);
  sampo_environment* env = (sampo_environment*)malloc(sizeof(sampo_environment) * steps);
  if (!T || !env) return 1;
  /* readSingleValFile / readEnvironment (src/abms.c:94-137) */
  if (sampo_read_temperature_file(pos[0], T, steps) != SAMPO_OK) {
    printf("Cannot open %s. Check temperature file path\n", pos[0]);
    return -1;
  }
  if (sampo_read_environment_file(pos[1], env, steps, cc) != SAMPO_OK) {
    printf("Cannot open %s. Check environment file path\n", pos[1]);
    return -1;
  }

  const double t0 = now_ms();
  sampo_species* species = NULL;
  if (!builtin_species) {  /* the kernels' build with the user's header */
    char log[16384];
    const int crc = sampo_species_compile(pos[2], device, log, sizeof(log), &species);
    if (crc != SAMPO_OK) {
      fflush(stdout);
      fprintf(stderr, "sampo: species header %s did not build (%d)\n%s\n", pos[2], crc, log);
      return 2;
    }
  }
  sampo_config cfg = {capacity, cc, device, steps + 1};
  sampo_sim* s = NULL;
  if (sampo_create(&cfg, &s) != SAMPO_OK) {
    printf("Cannot find any CUDA device\n");
    return 0;
  }
  int rc;
  if (species && (rc = sampo_set_species(s, species)) != SAMPO_OK) fail(s, "species", rc);
  if ((rc = sampo_set_inputs(s, 0, T, env, steps)) != SAMPO_OK) fail(s, "inputs", rc);
  sampo_seeds init[4];
  draw_seeds(init);
  sampo_seeds* seeds = (sampo_seeds*)malloc(sizeof(sampo_seeds) * 4 * (size_t)steps);
  if (!seeds) return 1;
  for (uint32_t i = 0; i < steps; i++) draw_seeds(seeds + 4 * (size_t)i);
  if ((rc = sampo_set_seeds(s, 0, seeds, steps)) != SAMPO_OK) fail(s, "seeds", rc);
  uint32_t first = 0;
  sampo_population prev;
  if (resume_path) {
    int has_prev = 0;
    if (sampo_checkpoint_info(resume_path, &first, NULL, &prev, &has_prev) != SAMPO_OK) {
      fprintf(stderr, "sampo: cannot read checkpoint %s\n", resume_path);
      return 2;
    }
    if (first > steps) first = steps;
    if ((rc = sampo_checkpoint_load(s, resume_path)) != SAMPO_OK) fail(s, "checkpoint", rc);
    if (!has_prev && (rc = sampo_read_pool(s, &prev, NULL)) != SAMPO_OK) fail(s, "population", rc);
  } else {
    if ((rc = sampo_init_population(s, initial, init, age_days, age_seed)) != SAMPO_OK) fail(s, "initial population", rc);
    if ((rc = sampo_read_pool(s, &prev, NULL)) != SAMPO_OK) fail(s, "population", rc);
  }

  if (per_step) {
    for (uint32_t i = first; i < steps; i++) {
      if (i == ck_step && (rc = sampo_checkpoint_save(s, ck_path)) != SAMPO_OK) fail(s, "checkpoint", rc);
      sampo_stats_row row;
      /* the row of step i is the state the step starts from: print and
       * check it first, as the reference does before its update */
      if ((rc = sampo_current_row(s, &row)) != SAMPO_OK) fail(s, "row", rc);
      check_agents(print_stats(&row, &prev, i, T[i]), capacity);
      prev = row.pop;
      if ((rc = sampo_step(s, &env[i], T[i], i % 24u, seeds + 4 * (size_t)i, NULL)) != SAMPO_OK) fail(s, "step", rc);
    }
  } else {
    const uint32_t chunk = 24 * 30;
    sampo_stats_row* rows[2];
    rows[0] = (sampo_stats_row*)sampo_host_alloc(sizeof(sampo_stats_row) * chunk);
    rows[1] = (sampo_stats_row*)sampo_host_alloc(sizeof(sampo_stats_row) * chunk);
    if (!rows[0] || !rows[1]) return 1;
    printer_t pr;
    memset(&pr, 0, sizeof(pr));
    pthread_mutex_init(&pr.mu, NULL);
    pthread_cond_init(&pr.cv, NULL);
    pr.T = T;
    pr.capacity = capacity;
    pr.prev = prev;
    pthread_t th;
    if (pthread_create(&th, NULL, printer_main, &pr) != 0) return 1;
    uint32_t k = 0, n = 0;
    for (uint32_t at = first; at < steps; at += n, k ^= 1u) {
      if (at == ck_step && (rc = sampo_checkpoint_save(s, ck_path)) != SAMPO_OK) fail(s, "checkpoint", rc);
      n = steps - at < chunk ? steps - at : chunk;
      if (at < ck_step && ck_step - at < n) n = ck_step - at;  /* a chunk ends at the checkpoint */
      rc = sampo_run(s, n, rows[k]);  /* meanwhile the printer formats the other buffer */
      printer_idle(&pr);
      if (rc != SAMPO_OK) {
        print_rows(&pr, rows[k], at, n - 1);  /* the rows before the failed step */
        fail(s, "run", rc);
      }
      printer_submit(&pr, rows[k], at, n);
    }
    printer_idle(&pr);
    pthread_mutex_lock(&pr.mu);
    pr.quit = 1;
    pthread_cond_broadcast(&pr.cv);
    pthread_mutex_unlock(&pr.mu);
    pthread_join(th, NULL);
    sampo_host_free(rows[0]);
    sampo_host_free(rows[1]);
  }

  if (ck_path && ck_step == steps && (rc = sampo_checkpoint_save(s, ck_path)) != SAMPO_OK) fail(s, "checkpoint", rc);
  sampo_population final;
  if ((rc = sampo_read_pool(s, &final, NULL)) != SAMPO_OK) fail(s, "population", rc);
  print_population(&final);
  uint32_t hist[100];
  if ((rc = sampo_histogram(s, hist)) != SAMPO_OK) fail(s, "histogram", rc);
  FILE* h = fopen("histogram.txt", "w");
  if (h) {
    for (int i = 0; i < 100; i++) fprintf(h, "%d, ", (int)hist[i]);
    fclose(h);
  }
  sampo_destroy(s);
  sampo_species_free(species);
  printf("Execution time: %f ms\n", now_ms() - t0);
  free(seeds);
  free(T);
  free(env);
  return 0;
}
