/*
 * sampo_oracle_main.c - command-line driver of the CPU oracle port (TEST
 * INFRASTRUCTURE ONLY). Reads the same inputs and prints the same per-step
 * lines, final ranges and histogram.txt as the reference's src/abms.c
 * (readSingleValFile :94-108, readEnvironment :110-137, printStats :67-81,
 * printPopulation :83-92, storeHistogram :176-180), so its output can be
 * diffed against the ref-as-C build and against the CUDA drop-in.
 *
 *   sampo_oracle [--seed S] [--initial N] [--cc CC] [--steps K] [--capacity C]
 *                [--age-days D --age-seed A] [--hash-file F] [--threads T]
 *                [--quiet] [TEMP [ENV [SPECIES]]]
 */
#include "sampo_oracle.h"
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

static double now_ms(void) {
  struct timespec ts;
  clock_gettime(CLOCK_MONOTONIC, &ts);
  return ts.tv_sec * 1e3 + ts.tv_nsec * 1e-6;
}

static void print_range(const orc_range* r) {
  printf("[%d\t%d]\t%d\r\n", (int)r->start, (int)r->end, (int)(r->end - r->start));
}

int main(int argc, char** argv) {
  unsigned seed = 1, initial = 32000, age_days = 0;
  int use_age = 0, threads = 0, quiet = 0;
  unsigned long long age_seed = 0, capacity = 6000000ULL;
  float cc = 160000.0f;
  long long steps = 8760;
  const char* hash_file = NULL;
  const char* pos[3] = {"temp.txt", "environment.txt", "properties.h"};
  int np = 0;
  for (int i = 1; i < argc; i++) {
    if (!strcmp(argv[i], "--seed") && i + 1 < argc) seed = (unsigned)strtoul(argv[++i], 0, 10);
    else if (!strcmp(argv[i], "--initial") && i + 1 < argc) initial = (unsigned)strtoul(argv[++i], 0, 10);
    else if (!strcmp(argv[i], "--cc") && i + 1 < argc) cc = strtof(argv[++i], 0);
    else if (!strcmp(argv[i], "--steps") && i + 1 < argc) steps = strtoll(argv[++i], 0, 10);
    else if (!strcmp(argv[i], "--capacity") && i + 1 < argc) capacity = strtoull(argv[++i], 0, 10);
    else if (!strcmp(argv[i], "--age-days") && i + 1 < argc) { age_days = (unsigned)atoi(argv[++i]); use_age = 1; }
    else if (!strcmp(argv[i], "--age-seed") && i + 1 < argc) age_seed = strtoull(argv[++i], 0, 10);
    else if (!strcmp(argv[i], "--hash-file") && i + 1 < argc) hash_file = argv[++i];
    else if (!strcmp(argv[i], "--threads") && i + 1 < argc) threads = atoi(argv[++i]);
    else if (!strcmp(argv[i], "--quiet")) quiet = 1;
    else if (np < 3) pos[np++] = argv[i];
    else { fprintf(stderr, "unexpected argument %s\n", argv[i]); return 2; }
  }
  printf("Temperature:\t%s\nEnvironment:\t%s\nSpecies:\t%s\n", pos[0], pos[1], pos[2]);

  float* T = (float*)malloc(sizeof(float) * (size_t)steps);
  orc_env* env = (orc_env*)malloc(sizeof(orc_env) * (size_t)steps);
  FILE* f = fopen(pos[0], "r");
  if (!f) { printf("Cannot open %s. Check temperature file path\n", pos[0]); return 1; }
  for (long long i = 0; i < steps; i++) if (fscanf(f, "%f", &T[i]) != 1) { fprintf(stderr, "short temperature file\n"); return 1; }
  fclose(f);
  f = fopen(pos[1], "r");
  if (!f) { printf("Cannot open %s. Check environment file path\n", pos[1]); return 1; }
  for (long long i = 0; i < steps; i++) {
    float c, e;
    if (fscanf(f, "%f, %f, ", &c, &e) != 2) { fprintf(stderr, "short environment file\n"); return 1; }
    env[i].IRSValue = c * e;
    if (fscanf(f, "%f, %f, ", &c, &e) != 2) return 1;
    env[i].ITNValue = c * e;
    if (fscanf(f, "%f, %f, ", &c, &e) != 2) return 1;
    env[i].larvacideValue = c * e;
    if (fscanf(f, "%f, %f, ", &c, &e) != 2) return 1;
    env[i].oviTrapValue = c * e;
    if (fscanf(f, "%f", &env[i].bloodmealSuccess) != 1) return 1;
    env[i].carryingCapacity = cc;
  }
  fclose(f);

  orc_sim* s = orc_create(capacity, threads);
  if (!s) { fprintf(stderr, "cannot allocate the pool\n"); return 1; }
  printf("CPU: sampo oracle port\n");
  double t0 = now_ms();
  orc_glibc_rand g;
  orc_rand_seed(&g, seed);
  orc_seeds sd[4];
  for (int k = 0; k < 4; k++) { sd[k].z1 = orc_rand_next(&g); sd[k].z2 = orc_rand_next(&g); sd[k].z3 = orc_rand_next(&g); sd[k].z4 = orc_rand_next(&g); }
  if (orc_init_eggs(s, initial, T[0], sd, use_age ? (int)age_days : -1, age_seed)) { fprintf(stderr, "capacity\n"); return 1; }
  FILE* hf = hash_file ? fopen(hash_file, "w") : NULL;
  orc_pop prev;
  orc_read_pool(s, &prev, NULL);
  for (long long i = 0; i < steps; i++) {
    orc_row row;
    orc_current_row(s, &row);
    uint32_t num[8];
    for (int k = 0; k < 8; k++) num[k] = row.pop.r[k].end - row.pop.r[k].start;
    uint32_t adults = num[3] + num[4] + num[5] + num[6] + num[7];
    /* src/abms.c:235-236 computes the adult range from the host copy of the
     * population BEFORE it is refreshed at :280, i.e. from the previous
     * step's ranges (the initial ranges at step 0). */
    uint32_t adultsRange = 0;
    {
      uint32_t ub = prev.r[3].end;
      if (prev.r[5].end > ub) ub = prev.r[5].end;
      if (prev.r[6].end > ub) ub = prev.r[6].end;
      if (prev.r[7].end > ub) ub = prev.r[7].end;
      adultsRange = ub - prev.r[3].start;
    }
    prev = row.pop;
    uint32_t l1 = num[1] > 0 ? row.pop.L1de : 0;
    uint32_t fem = adultsRange > 0 ? row.pop.numFemale : 0;
    uint32_t inf = adultsRange > 0 ? row.pop.numPotInf : 0;
    uint32_t nAgents = num[0] + num[1] + num[2] + adults;
    if (!(nAgents <= capacity * 0.95)) { fprintf(stderr, "not enough capacity\n"); return 3; }
    if (nAgents == 0) { fprintf(stderr, "No more agents left\n"); return 3; }
    if (!quiet) {
      printf("%0.1f, %0.1f", (double)(1.0f * (float)(uint32_t)i), (double)T[i]);
      printf(", %d, %d, %d, %d, %d, %d, %d, %d, %d", (int)adults, (int)num[3], (int)num[4], (int)num[5], (int)num[6], (int)num[7],
             (int)fem, (int)inf, (int)(adults - fem));
      printf(", %d, %d, %d, %d, %d, ", (int)num[0], (int)num[1], (int)num[2], (int)l1, (int)(l1 + num[0] + num[2]));
      printf("%d, %d, %d\r\n", (int)(row.numCycles > 0 ? row.sumCycles / row.numCycles : 0), (int)row.numBites, (int)row.numInfectBites);
    }
    for (int k = 0; k < 4; k++) { sd[k].z1 = orc_rand_next(&g); sd[k].z2 = orc_rand_next(&g); sd[k].z3 = orc_rand_next(&g); sd[k].z4 = orc_rand_next(&g); }
    int rc = orc_step(s, &env[i], T[i], (uint32_t)(1.0f * (float)(uint32_t)i) % 24u, sd, NULL);
    if (rc) { fprintf(stderr, "step %lld failed (%d)\n", i, rc); return 3; }
    if (hf) fprintf(hf, "%016llx\n", (unsigned long long)orc_pool_hash(s));
  }
  if (hf) fclose(hf);
  orc_pop pop;
  orc_read_pool(s, &pop, NULL);
  static const char* names[8] = {"Eggs \t\t", "Larvae \t\t", "Pupae \t\t", "Immatures \t", "MateSeeking \t", "BMS \t\t", "BMD \t\t", "Gravids \t"};
  for (int k = 0; k < 8; k++) { printf("%s", names[k]); print_range(&pop.r[k]); }
  uint32_t hist[100];
  orc_histogram(s, hist);
  FILE* hfile = fopen("histogram.txt", "w");
  for (int i = 0; i < 100; i++) fprintf(hfile, "%d, ", (int)hist[i]);
  fclose(hfile);
  printf("Execution time: %f ms\n", now_ms() - t0);
  orc_destroy(s);
  free(T); free(env);
  return 0;
}
