/*
 * sampo.h - C ABI of the GB300 implementation of SAMPO's per-step agent
 * update (libsampo_cuda.so). Plain C types only; every call returns an int
 * status (SAMPO_OK = 0, negative on error) and never exits the process.
 * Handles are not thread-safe; one handle drives one simulation on one GPU.
 *
 * The reference crosses its host/device boundary through the OpenCL wrapper
 * lib_icl (include/lib_icl.h:100-159) and the scan driver
 * (include/scan.h:5-11), called from src/abms.c. Its per-step sequence
 * calcStats -> generateSeeds -> update -> createNewAgents -> swap
 * (src/abms.c:502-529) becomes one sampo_step / sampo_run call here. Each
 * declaration below names the reference code it replaces.
 */
#ifndef SAMPO_H
#define SAMPO_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define SAMPO_ABI_VERSION 1

/* ---- status codes ---- */
#define SAMPO_OK 0
#define SAMPO_ERR_ARG -1          /* invalid argument */
#define SAMPO_ERR_CUDA -2         /* CUDA runtime error (see sampo_last_error) */
#define SAMPO_ERR_CAPACITY -3     /* the next layout does not fit the pool */
#define SAMPO_ERR_TEMPERATURE -4  /* T >= 44 C: the reference reads past devRates (include/properties.h:105-109) */
#define SAMPO_ERR_STATE -5        /* call out of order (no population yet, inputs missing) */
#define SAMPO_ERR_INTERNAL -6     /* a device-side consistency check failed */
#define SAMPO_ERR_IO -7           /* input file missing or short */
#define SAMPO_ERR_SPECIES -8      /* the species header did not compile (see the log) */
#define SAMPO_ERR_UNSUPPORTED -9  /* NVRTC or the CUDA driver entry points are unavailable */

/* ---- device error bits (sampo_device_status) ---- */
#define SAMPO_DEV_ERR_CAPACITY   0x1u
#define SAMPO_DEV_ERR_DEVRATES   0x2u
#define SAMPO_DEV_ERR_TILECOUNT  0x4u
#define SAMPO_DEV_ERR_LARVATABLE 0x8u
#define SAMPO_DEV_ERR_TMA        0x10u  /* a tile's bulk copy did not land within the wait limit */
#define SAMPO_DEV_ERR_BARRIER    0x20u  /* the one-launch step's grid barrier was not met within the wait limit */
/* warning bit: the step ran on the reference's initial layout with shared
 * empty ranges and produced agents in the ranges whose ends coincide; the
 * reference's compaction would have read one prefix-sum entry for several
 * ends (kernel/oldToNewAgents.cl:270,279,288) and created agents from
 * uninitialised memory. This implementation counts them correctly. */
#define SAMPO_DEV_WARN_REF_LAYOUT 0x100u

/* State order of the ranges (enum State, include/agent.h:54-63). */
enum { SAMPO_EGG = 0, SAMPO_LARVA, SAMPO_PUPA, SAMPO_IMMATURE, SAMPO_MATESEEKING,
       SAMPO_BMS, SAMPO_BMD, SAMPO_GRAVID, SAMPO_NSTATES };

/* struct AgentRange / struct Population (include/agent.h:104-123). */
typedef struct { uint32_t start, end; } sampo_range;
typedef struct {
  sampo_range r[SAMPO_NSTATES];
  uint32_t numLarvae1DayEquiv, numFemale, numPotentiallyInfective;
} sampo_population;

/* struct Environment (include/agent.h:22-35), same field order. */
typedef struct {
  float bloodmealSuccess, ITNValue, IRSValue, carryingCapacity, larvacideValue, oviTrapValue;
} sampo_environment;

/* struct Seeds (include/agent.h:145-150). Four per step (src/abms.c:145-150). */
typedef struct { uint32_t z1, z2, z3, z4; } sampo_seeds;

/* struct BitesNcycles (include/agent.h:44-50). */
typedef struct { uint32_t numCyclesReported, sumCyclesReported, numBitesReported, numInfectBitesReported; } sampo_bites_cycles;

/* What src/abms.c reads back each step (pop[0] at :280 and bnc at :506):
 * the population at the START of a step and the counters of the previous
 * step's update. */
typedef struct { sampo_population pop; sampo_bites_cycles bnc; } sampo_stats_row;

/* Host SoA view of a pool; slots [0, pop.r[GRAVID].end). state is 0..7.
 * The union field of struct Agent (cumulativeLarvalDelay as float bits for
 * larvae, ovipositionAttemps for gravids) is carried as raw 32 bits. */
typedef struct {
  float* ageInHours; float* hoursInState; float* delay; float* cumulativeSporogonicDevelopment;
  uint32_t* larvalDelayOrOviAttempts; uint32_t* availableEggs; uint32_t* cycleLength;
  uint32_t* humanBloodmealCount; uint32_t* numEggBatches;
  uint8_t* isFemale; uint8_t* state;
} sampo_pool_view;

typedef struct {
  uint64_t capacity;          /* slots per pool buffer (reference: maxAgents, include/abms.h:16) */
  float carrying_capacity;    /* reference: carryingCapacity (src/abms.c:19) */
  int device;                 /* CUDA device ordinal */
  uint32_t max_steps;         /* length of the per-step input arrays (reference: maxSteps) */
} sampo_config;

typedef struct sampo_sim sampo_sim;

/* Replaces icl_init_devices/icl_get_device and the buffer creation of
 * src/abms.c:614-654, 466-474. Allocates both pool buffers and the step
 * state on the device. */
int sampo_create(const sampo_config* cfg, sampo_sim** out);
/* Replaces icl_release_buffers/icl_release_kernel/icl_release_devices
 * (src/abms.c:543-554, 694). */
int sampo_destroy(sampo_sim* s);
/* Text of the last error on this handle (replaces ICL_ASSERT's message,
 * include/lib_icl.h:19-25). */
const char* sampo_last_error(const sampo_sim* s);

/* Per-step inputs: temperature and Environment rows for steps
 * [first, first+nsteps) (replaces readSingleValFile/readEnvironment,
 * src/abms.c:94-137, and the by-value kernel arguments at :319-340).
 * World time of step i is i % 24 (src/abms.c:514). */
int sampo_set_inputs(sampo_sim* s, uint32_t first, const float* temperature, const sampo_environment* env, uint32_t nsteps);
/* Seeds for steps [first, first+nsteps): 4 per step, in the order
 * generateSeeds draws them (src/abms.c:145-150). */
int sampo_set_seeds(sampo_sim* s, uint32_t first, const sampo_seeds* seeds, uint32_t nsteps);

/* createInitialPopulation (src/abms.c:185-228, kernel/initAgents.cl:26-65):
 * n eggs at [0, n) from init_seeds and temperature[0]. age_days_max < 0
 * keeps the reference's ages (0) and its initial ranges ([n+1, n+1) for
 * every empty state); age_days_max >= 0 (an extension) sets ageInHours =
 * hoursInState = 24*U{0..age_days_max} per slot from splitmix64(age_seed)
 * and uses the padded layout a compaction produces. */
int sampo_init_population(sampo_sim* s, uint32_t n, const sampo_seeds init_seeds[4], int age_days_max, uint64_t age_seed);
/* Uploads a prepared pool (an extension: mixed-stage initial populations). */
int sampo_load_pool(sampo_sim* s, const sampo_population* pop, const sampo_pool_view* pool);

/* One hourly step with explicit inputs - the body of the reference's loop
 * (src/abms.c:503-521: calcStats, update = killAgents + updateAgents,
 * createNewAgents = initAgents + preScan/scan x3 + oldToNewAgents, swap).
 * *row receives the stats at the START of the step (what printStats shows).
 * Synchronous. */
int sampo_step(sampo_sim* s, const sampo_environment* env, float temperature, uint32_t world_time,
               const sampo_seeds seeds[4], sampo_stats_row* row);
/* nsteps steps from the arrays given to sampo_set_inputs/sampo_set_seeds,
 * starting at the simulation's current step; world time = step % 24.
 * Days are replayed as CUDA graphs of 24 steps. rows (may be NULL)
 * receives nsteps stats rows. */
int sampo_run(sampo_sim* s, uint32_t nsteps, sampo_stats_row* rows);
/* sampo_run without waiting (the stats rows of src/abms.c:502-529 streamed
 * to the host while the caller formats earlier ones): the steps and the
 * copies of their rows are queued on the simulation's stream and the call
 * returns. rows must stay valid until sampo_sync; page-locked rows
 * (sampo_host_alloc) keep the copies asynchronous. Further sampo_run_async
 * calls queue behind; any other call on the handle first waits for the queue
 * and returns its error, if any. Device errors of queued steps (capacity,
 * temperature) are reported by sampo_sync. With timing on it waits like
 * sampo_run. */
int sampo_run_async(sampo_sim* s, uint32_t nsteps, sampo_stats_row* rows);
/* Waits for the steps sampo_run_async queued; their status, and the device
 * time from the first queued step to the last for sampo_last_run_ms. */
int sampo_sync(sampo_sim* s);
/* Stats at the start of the current (next) step. */
int sampo_current_row(sampo_sim* s, sampo_stats_row* row);
/* Index of the next step (after the steps sampo_run_async queued). */
int sampo_get_step(sampo_sim* s, uint32_t* step);

/* storeHistogram (src/abms.c:160-183, kernel/ageHistogram.cl:13-35):
 * 100 bins of min(floor(age/24), 99) over adults of the current pool. */
int sampo_histogram(sampo_sim* s, uint32_t out[100]);

/* Copies the current pool to the host (replaces icl_read_buffer of the
 * agent buffers; used for parity tests). The view's arrays must hold
 * pop.r[GRAVID].end entries; pass NULL to read the ranges only. */
int sampo_read_pool(sampo_sim* s, sampo_population* pop, sampo_pool_view* pool);

/* Checkpoint / resume at a step boundary (no counterpart in the reference,
 * which runs a simulation to the end in one process). The file holds the
 * step index, the population with its statistics, the counters the next stats
 * row reports and every live slot; a simulation resumed from it continues bit
 * for bit as if it had not stopped, given the same inputs and seeds for the
 * later steps (seeds are the caller's: with srand/rand they are the stream
 * after 16 x (step + 1) draws). Loading needs a handle with the file's
 * carrying capacity and room for its pool. */
int sampo_checkpoint_save(sampo_sim* s, const char* path);
/* Autotuner (no counterpart in the reference): times the step kernels on the
 * coming step of this simulation for each tile size (1024- and 512-slot
 * tiles: 4 or 2 slots per thread) at every persistent grid size the
 * occupancy allows (CTAs per SM of the count and update/scatter passes),
 * keeps the fastest for the following steps and returns the grids (the tile
 * size: sampo_items_per_thread). The trials leave the simulation's course
 * unchanged. Needs the coming step's inputs. */
int sampo_autotune(sampo_sim* s, uint32_t* count_ctas_per_sm, uint32_t* scatter_ctas_per_sm);
/* Sets the grid sizes sampo_autotune would pick, e.g. a choice tuned earlier
 * on the same workload: 1 .. the occupancy limit of each pass. */
int sampo_set_grids(sampo_sim* s, uint32_t count_ctas_per_sm, uint32_t scatter_ctas_per_sm);
/* Slots per thread of the count and update/scatter passes: 4 (1024-slot
 * tiles, the default) or 2 (512-slot tiles); results do not depend on it. A
 * run-time species runs 4. Setting it resets the grids to the largest the
 * occupancy allows. */
int sampo_set_items_per_thread(sampo_sim* s, uint32_t items);
int sampo_items_per_thread(sampo_sim* s, uint32_t* items);
/* One-launch step for small pools (for such pools it replaces the per-step
 * launch sequence of src/abms.c:502-529 that the three-kernel step already
 * shortens). sampo_run picks each day's graph from the pool size it last
 * saw (it learns the size after each day, one day behind the queued work):
 * a pool of at most max_tiles 1024-slot tiles takes one launch of a
 * cooperative kernel that runs the day's 24 hourly steps (update, scan and
 * compaction with two bounded grid barriers per hour) on a grid sized to the
 * pool, a larger one the count, update/scatter and publish kernels every
 * hour. Both give the same results at any size. SAMPO_SMALL_STEP_DEFAULT:
 * the largest co-resident grid of the one-launch kernel, one tile per CTA
 * (the default); 0: never. sampo_run_async picks by the size seen at its
 * call; sampo_step, runs with timing on and a run-time species
 * (sampo_set_species) always take the three-kernel step. */
#define SAMPO_SMALL_STEP_DEFAULT 0xffffffffu
int sampo_set_small_step(sampo_sim* s, uint32_t max_tiles);
/* Slots per thread of the one-launch step: 0 (the default) takes the
 * smallest tiles, 256 (1), 512 (2) or 1024 slots (4), that the pool leaves
 * the largest grid room for; 1, 2 or 4 fix it. The results do not depend on
 * it. */
int sampo_set_small_step_items(sampo_sim* s, uint32_t items);
/* The one-launch step's largest grid (CTAs; 0 when it cannot run here), the
 * current max_tiles, the kind of the last day launched (0 none yet, 1
 * three-kernel steps, 2 one-launch steps launched cooperatively, 3 the same
 * as plain launches of the same co-resident grid) and the days of each path
 * since creation or sampo_set_timing. */
int sampo_small_step_info(sampo_sim* s, uint32_t* grid, uint32_t* max_tiles, int* last_day_kind, uint64_t* days_one_launch,
                          uint64_t* days_three_kernel);
int sampo_checkpoint_load(sampo_sim* s, const char* path);
/* Header of a checkpoint file (no device needed): the step it resumes at,
 * the population then, and the population at the previous step's start
 * (*has_prev = 0 for step 0 or a version-1 file). Any pointer may be NULL. */
int sampo_checkpoint_info(const char* path, uint32_t* step, sampo_population* pop, sampo_population* prev, int* has_prev);
/* ---- species headers compiled at run time ----
 * The reference compiles its kernels at start-up with the species header
 * named by argv[3] (src/abms.c:565-568; default properties.h, which is built
 * into this library). sampo_species_compile compiles the step kernels with
 * NVRTC against a properties.h-style header (OpenCL C: the functions
 * eggsIncubation ... layEggs and the *_PROBABILITY macros of
 * include/properties.h, with include/gpuRand.h's HybridTaus and BoxMuller
 * and OpenCL math) for the given device; log (may be NULL) receives the
 * compiler's messages. A simulation or batch uses it after
 * sampo_set_species / sampo_batch_set_species (set it before
 * sampo_init_population: the initial eggs use the species too); NULL
 * returns to the built-in species. Free it after the handles that use it.
 * sampo_step_noalloc always uses the built-in species. */
typedef struct sampo_species sampo_species;
int sampo_species_compile(const char* header_path, int device, char* log, size_t log_size, sampo_species** out);
int sampo_species_compile_text(const char* name, const char* text, int device, char* log, size_t log_size,
                               sampo_species** out);
void sampo_species_free(sampo_species* sp);
/* The device a species was compiled and loaded for (-1 for NULL). */
int sampo_species_device(const sampo_species* sp);
/* Compiles without loading, for sm_<sm>a (e.g. 103): a syntax check that
 * needs no GPU. */
int sampo_species_check_text(const char* name, const char* text, int sm, char* log, size_t log_size);
int sampo_set_species(sampo_sim* s, const sampo_species* sp);

/* Sticky device status bits (SAMPO_DEV_*) since creation or the last clear. */
int sampo_device_status(sampo_sim* s, uint32_t* bits, int clear);

/* Per-kernel timing (the reference's TIMING build: CUDA events replace
 * icl_profile_event, src/abms.c:522-528). With timing on, sampo_run launches
 * every kernel on its own between events instead of replaying day graphs.
 * Turning it on or off clears the sums. */
int sampo_set_timing(sampo_sim* s, int on);
/* Sums since sampo_set_timing, in milliseconds: out[0] count pass,
 * out[1] update+scatter pass, out[2] the whole step (both + the per-step
 * publish kernel); *launches = kernels launched. */
int sampo_kernel_times(sampo_sim* s, double out[3], uint64_t* launches);
/* Device time of the last sampo_run, in milliseconds, from CUDA events
 * recorded on the simulation's stream around its launches. */
int sampo_last_run_ms(sampo_sim* s, double* ms);

/* Page-locked host memory for the per-step inputs and rows (cudaMallocHost
 * on the handle's device), and a write of a scratch buffer larger than the
 * L2 cache on the handle's stream (benchmarks flush L2 between iterations). */
void* sampo_host_alloc(size_t bytes);
void sampo_host_free(void* p);
int sampo_flush_l2(sampo_sim* s);

/* ---- host helpers ---- */
/* glibc-compatible rand() stream (srand/rand as used by src/abms.c:611,
 * 145-150) with private state, so replicates can run side by side. */
typedef struct { uint32_t r[31]; uint32_t i; } sampo_rand_state;
void sampo_rand_seed(sampo_rand_state* st, uint32_t seed);
uint32_t sampo_rand_next(sampo_rand_state* st);
/* Fills 4*nsteps seeds: the draws of nsteps generateSeeds calls. */
void sampo_rand_seeds(sampo_rand_state* st, sampo_seeds* out, uint32_t nsteps);

/* readSingleValFile / readEnvironment (src/abms.c:94-137), same fscanf
 * formats; env[i].carryingCapacity = carrying_capacity. */
int sampo_read_temperature_file(const char* path, float* out, uint32_t nsteps);
int sampo_read_environment_file(const char* path, sampo_environment* out, uint32_t nsteps, float carrying_capacity);

/* ---- one step without any device allocation ----
 * No counterpart in the reference. For callers that cannot call cudaMalloc:
 * code running where allocation is forbidden or unsafe (inside another
 * framework's memory pool or arena, a host that must not grow device memory
 * after start-up, a memory-capped sandbox). They bring their own pool
 * buffers; the step's scratch (step state, per-tile prefix tables and
 * look-back counts, one step of inputs and stats) lives in a fixed array
 * inside the library, sized for pools of up to SAMPO_NOALLOC_MAX_SLOTS slots
 * (about 15 MB, held by every GPU that loads the library until the process
 * exits).
 *
 * in/out: device columns of two pool buffers; each column 16-byte aligned
 * with 16 bytes of slack after capacity elements; flags = state |
 * isFemale << 3. pop_in: ranges of `in` (stats are recomputed). Writes the
 * next pool into `out`; *row = stats at the start of the step (bnc zero),
 * *pop_out = ranges and stats of `out`, *bnc_out = this step's counters.
 * Capacities above SAMPO_NOALLOC_MAX_SLOTS, and `in` and `out` columns that
 * overlap, return SAMPO_ERR_ARG.
 * The first call on a device resolves the scratch array's device address
 * (cudaGetSymbolAddress) with that device current.
 * All calls share the one array and it keeps the last call's contents:
 * calls that overlap on the GPU (other threads, other streams) race. The
 * call is synchronous: it copies the step's inputs from host memory and
 * waits on `stream` (NULL = the default stream) for the results, so it
 * must not be made on a stream that is capturing a graph (SAMPO_ERR_STATE). */
#define SAMPO_NOALLOC_MAX_SLOTS (1u << 24)
typedef struct {
  float* ageInHours; float* hoursInState; float* delay; float* cumulativeSporogonicDevelopment;
  uint32_t* larvalDelayOrOviAttempts; uint32_t* availableEggs; uint32_t* cycleLength;
  uint32_t* humanBloodmealCount; uint32_t* numEggBatches;
  uint8_t* flags;
} sampo_device_pool;
int sampo_step_noalloc(const sampo_device_pool* in, uint32_t in_capacity, const sampo_device_pool* out,
                       uint32_t out_capacity, const sampo_population* pop_in, const sampo_environment* env,
                       float temperature, uint32_t world_time, const sampo_seeds seeds[4], float carrying_capacity,
                       sampo_stats_row* row, sampo_population* pop_out, sampo_bites_cycles* bnc_out, int device,
                       void* stream);

/* Diagnostic: evaluates the model's deterministic transcendentals on the
 * device (fn 0 exp(x), 1 log(x), 2 sin(x), 3 pow(x, y), and the binary32
 * evaluations the normal draw uses: 4 log(x), 5 sin(x)); they must equal the
 * host definitions of 0-3 bit for bit. No counterpart in the reference, whose
 * OpenCL built-ins are implementation-defined. */
int sampo_eval_math(int fn, const float* x, const float* y, float* out, uint32_t n, int device);

/* ---- batches: many independent simulations stepped together ----
 * No counterpart in the reference, which runs one simulation per process.
 * A batch owns up to max_replicates slots on one GPU; every slot holds one
 * simulation (a "replicate": its own pool, carrying capacity, seeds, inputs
 * and step counter). sampo_batch_run advances every active replicate by the
 * same number of steps in one pass of the step kernels per hour (tiles of all
 * replicates share the persistent CTAs), replayed as a CUDA graph per day.
 * Each replicate's results are bit-identical to the same simulation run
 * alone through sampo_step / sampo_run. Slots can be filled and emptied
 * between runs (continuous batching); pools are allocated stream-ordered
 * from the batch's memory pool. */
#define SAMPO_BATCH_MAX_REPLICATES 1024u
typedef struct sampo_batch sampo_batch;
typedef struct {
  uint32_t max_replicates;   /* slots (<= SAMPO_BATCH_MAX_REPLICATES) */
  uint32_t ring_steps;       /* per-replicate ring of inputs and stats rows, in steps (>= 2) */
  int device;
} sampo_batch_config;
typedef struct {
  uint64_t capacity;         /* slots per pool buffer */
  float carrying_capacity;   /* constant per run (src/abms.c:19,132) */
  uint32_t stop_step;        /* the replicate stops once it has run this many steps; 0xffffffff: never */
} sampo_replicate_config;

int sampo_batch_create(const sampo_batch_config* cfg, sampo_batch** out);
int sampo_batch_destroy(sampo_batch* b);
const char* sampo_batch_last_error(const sampo_batch* b);
/* Device bytes one replicate of this capacity holds in a batch of this ring. */
uint64_t sampo_batch_replicate_bytes(uint64_t capacity, uint32_t ring_steps);
/* Takes a free slot and allocates its buffers; the replicate is inactive
 * until sampo_batch_init_population. */
int sampo_batch_add(sampo_batch* b, const sampo_replicate_config* rc, uint32_t* slot);
/* Frees the slot and its buffers (stream-ordered after the work queued so far). */
int sampo_batch_remove(sampo_batch* b, uint32_t slot);
/* As sampo_set_inputs / sampo_set_seeds, for one replicate. */
int sampo_batch_set_inputs(sampo_batch* b, uint32_t slot, uint32_t first, const float* temperature,
                           const sampo_environment* env, uint32_t nsteps);
int sampo_batch_set_seeds(sampo_batch* b, uint32_t slot, uint32_t first, const sampo_seeds* seeds, uint32_t nsteps);
/* As sampo_init_population; activates the replicate at step 0. */
int sampo_batch_init_population(sampo_batch* b, uint32_t slot, uint32_t n, const sampo_seeds init_seeds[4],
                                int age_days_max, uint64_t age_seed);
/* Device-side seed stream (the host loop's srand/rand, src/abms.c:611 and
 * 145-150, moved onto the GPU): from the replicate's coming step on, the
 * seeds of every step are the next 16 draws of `st`, made on the device once
 * per step, so no seeds travel per step. `st` is the stream right before the
 * coming step's draws (after the 16 initial ones for a replicate at step 0).
 * Call after sampo_batch_init_population; sampo_batch_set_seeds then fails
 * for the slot. */
int sampo_batch_seed_stream(sampo_batch* b, uint32_t slot, const sampo_rand_state* st);
/* The slot's device stream after the draws of every step before *next_step
 * (a state sampo_rand_next continues). */
int sampo_batch_seed_state(sampo_batch* b, uint32_t slot, sampo_rand_state* st, uint32_t* next_step);
/* Advances every active replicate by nsteps (a replicate stops at its
 * stop_step). Asynchronous unless wait != 0; status of the replicates is
 * read with sampo_batch_state after sampo_batch_sync. */
int sampo_batch_run(sampo_batch* b, uint32_t nsteps, int wait);
int sampo_batch_sync(sampo_batch* b);
/* Rows of steps [first, first + n) of one replicate (row k = stats at the
 * start of step k, as sampo_run returns them); the ring must still hold them. */
int sampo_batch_rows(sampo_batch* b, uint32_t slot, uint32_t first, uint32_t n, sampo_stats_row* out);
/* Step reached, whether still active, and device error/warning bits. */
int sampo_batch_state(sampo_batch* b, uint32_t slot, uint32_t* step, uint32_t* active, uint32_t* status_bits);
/* Growing pools (no counterpart in the reference, whose maxAgents is a
 * compile-time constant with an assert at 95 %, include/abms.h:16,
 * src/abms.c:305-307). A replicate whose next layout does not fit its
 * capacity does not stop: it pauses at that step, inactive, with
 * SAMPO_DEV_ERR_CAPACITY set and its pool, constants and seed stream as they
 * were. sampo_batch_grow moves its pool into a new allocation of `capacity`
 * slots (at least the pool's current end) - the slots keep their indices, so
 * the generator keys do not change - clears the capacity bit and reactivates
 * it; the paused step then runs again with the same result. A running slot
 * may be grown too (ahead of need). Stream-ordered after the work queued so
 * far; the old buffers are freed stream-ordered. */
int sampo_batch_grow(sampo_batch* b, uint32_t slot, uint64_t capacity);
/* State of every slot in one read (after the queued work): step, active,
 * device status bits, the pool's end (live slots plus gaps) and capacity;
 * unused slots report capacity 0. */
typedef struct {
  uint32_t step, active, status, end;
  uint64_t capacity;
} sampo_slot_state;
int sampo_batch_states(sampo_batch* b, sampo_slot_state* out, uint32_t nslots);
int sampo_batch_histogram(sampo_batch* b, uint32_t slot, uint32_t out[100]);
int sampo_batch_read_pool(sampo_batch* b, uint32_t slot, sampo_population* pop, sampo_pool_view* v);
/* The autotuner of sampo_autotune over the batch's coming step. */
int sampo_batch_autotune(sampo_batch* b, uint32_t* count_ctas_per_sm, uint32_t* scatter_ctas_per_sm);
int sampo_batch_set_grids(sampo_batch* b, uint32_t count_ctas_per_sm, uint32_t scatter_ctas_per_sm);
/* As sampo_set_items_per_thread / sampo_items_per_thread, for the batch. */
int sampo_batch_set_items_per_thread(sampo_batch* b, uint32_t items);
int sampo_batch_items_per_thread(sampo_batch* b, uint32_t* items);
/* The species of every replicate of the batch (NULL: built in); as
 * sampo_set_species. */
int sampo_batch_set_species(sampo_batch* b, const sampo_species* sp);
/* Checkpoints of one slot in the format of sampo_checkpoint_save: a file
 * written by either loads into either (same carrying capacity, enough
 * capacity). A slot's device seed stream travels with it. Load into a slot
 * taken with sampo_batch_add (it replaces init_population); the slot resumes
 * at the file's step and needs inputs from there. */
int sampo_batch_checkpoint_save(sampo_batch* b, uint32_t slot, const char* path);
int sampo_batch_checkpoint_load(sampo_batch* b, uint32_t slot, const char* path);
/* Device time of the last sampo_batch_run, in milliseconds (after sync). */
int sampo_batch_last_run_ms(sampo_batch* b, double* ms);
/* Kernels sampo_batch_run has launched since creation (a day graph's
 * replay counts its kernel nodes). */
int sampo_batch_launches(sampo_batch* b, uint64_t* launches);

/* Library version and build information. */
int sampo_abi_version(void);

#ifdef __cplusplus
}
#endif
#endif
