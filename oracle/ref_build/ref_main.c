/*
 * ref_main.c - entry point of the ref-as-C oracle (TEST INFRASTRUCTURE ONLY).
 *
 * Runs the reference's own src/abms.c (compiled unmodified with its main()
 * renamed to abms_main) after setting the run parameters that abms.c keeps
 * in file-scope globals (src/abms.c:15-19): maxSteps, initialAgentCount and
 * carryingCapacity. The srand() seed and the pinning hooks are set through
 * the emulator (icl_emul.cpp).
 *
 *   sampo_ref [--seed S] [--initial N] [--cc CC] [--steps K]
 *             [--age-days D --age-seed A | --pool FILE] [--hash-file F]
 *             TEMP ENV [SPECIES]
 *
 * --pool FILE starts from a mixed-stage pool (format in icl_emul.cpp) in
 * place of the initial eggs.
 *
 * SPECIES is passed on as abms.c's argv[3]; the kernels were compiled with
 * the species header at build time (ref_build/Makefile, target species).
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

extern long long maxSteps;
extern unsigned int initialAgentCount;
extern float carryingCapacity;
extern unsigned sampo_ref_seed;
extern int sampo_ref_age_days;
extern unsigned long long sampo_ref_age_seed;
extern const char* sampo_ref_hash_file;
extern const char* sampo_ref_pool_file;
int abms_main(int argc, char** argv);

int main(int argc, char** argv) {
  char* pos[4] = {argv[0], NULL, NULL, NULL};
  int np = 1;
  for (int i = 1; i < argc; i++) {
    if (!strcmp(argv[i], "--seed") && i + 1 < argc) sampo_ref_seed = (unsigned)strtoul(argv[++i], 0, 10);
    else if (!strcmp(argv[i], "--initial") && i + 1 < argc) initialAgentCount = (unsigned)strtoul(argv[++i], 0, 10);
    else if (!strcmp(argv[i], "--cc") && i + 1 < argc) carryingCapacity = strtof(argv[++i], 0);
    else if (!strcmp(argv[i], "--steps") && i + 1 < argc) maxSteps = strtoll(argv[++i], 0, 10);
    else if (!strcmp(argv[i], "--age-days") && i + 1 < argc) sampo_ref_age_days = atoi(argv[++i]);
    else if (!strcmp(argv[i], "--age-seed") && i + 1 < argc) sampo_ref_age_seed = strtoull(argv[++i], 0, 10);
    else if (!strcmp(argv[i], "--hash-file") && i + 1 < argc) sampo_ref_hash_file = argv[++i];
    else if (!strcmp(argv[i], "--pool") && i + 1 < argc) sampo_ref_pool_file = argv[++i];
    else if (np < 4) pos[np++] = argv[i];
    else { fprintf(stderr, "sampo_ref: unexpected argument %s\n", argv[i]); return 2; }
  }
  if (np < 3) { fprintf(stderr, "usage: sampo_ref [options] TEMP ENV [SPECIES]\n"); return 2; }
  return abms_main(np, pos);
}
