/*
 * icl_sampo_main.c - TEST INFRASTRUCTURE ONLY. Entry point of the reference's
 * unmodified src/abms.c (main renamed to abms_main) built over
 * sampo_gb300/host/icl_sampo.cpp: sets the run parameters abms.c keeps in
 * file-scope globals (src/abms.c:15-19), the srand() seed (abms.c seeds
 * with time(NULL); link with -Wl,--wrap=srand) and the aged-egg extension.
 *
 *   abms_icl_sampo [--seed S] [--initial N] [--cc CC] [--steps K]
 *                  [--age-days D --age-seed A] TEMP ENV [SPECIES]
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

extern long long maxSteps;
extern unsigned int initialAgentCount;
extern float carryingCapacity;
int abms_main(int argc, char** argv);
void icl_sampo_initial_ages(int age_days_max, unsigned long long age_seed);
void __real_srand(unsigned);

static unsigned g_seed = 1;
void __wrap_srand(unsigned s) { (void)s; __real_srand(g_seed); }

int main(int argc, char** argv) {
  char* pos[4] = {argv[0], NULL, NULL, NULL};
  int np = 1, age_days = -1;
  unsigned long long age_seed = 0;
  for (int i = 1; i < argc; i++) {
    if (!strcmp(argv[i], "--seed") && i + 1 < argc) g_seed = (unsigned)strtoul(argv[++i], 0, 10);
    else if (!strcmp(argv[i], "--initial") && i + 1 < argc) initialAgentCount = (unsigned)strtoul(argv[++i], 0, 10);
    else if (!strcmp(argv[i], "--cc") && i + 1 < argc) carryingCapacity = strtof(argv[++i], 0);
    else if (!strcmp(argv[i], "--steps") && i + 1 < argc) maxSteps = strtoll(argv[++i], 0, 10);
    else if (!strcmp(argv[i], "--age-days") && i + 1 < argc) age_days = atoi(argv[++i]);
    else if (!strcmp(argv[i], "--age-seed") && i + 1 < argc) age_seed = strtoull(argv[++i], 0, 10);
    else if (np < 4) pos[np++] = argv[i];
    else { fprintf(stderr, "abms_icl_sampo: unexpected argument %s\n", argv[i]); return 2; }
  }
  if (np < 3) { fprintf(stderr, "usage: abms_icl_sampo [options] TEMP ENV [SPECIES]\n"); return 2; }
  if (age_days >= 0) icl_sampo_initial_ages(age_days, age_seed);
  return abms_main(np, pos);
}
