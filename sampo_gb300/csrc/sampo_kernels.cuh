// sampo_kernels.cuh - device state shared by the kernels and the host API.
//
// The kernels step a batch of independent simulations ("replicates") at
// once: every replicate has its own pool buffers, state, look-back arrays and
// input rings (RepParams), and the persistent kernels hand out tiles of all
// active replicates from one ticket counter. A single simulation is a batch
// of one.
#pragma once
#include <stdint.h>
#ifndef __CUDACC_RTC__
#include <string.h>
#endif
#include "../../include/sampo.h"
#include "sampo_math.h"
#include "sampo_model.cuh"

namespace sampo {

constexpr int kBlock = 256;                 // threads per CTA
constexpr int kItems = 4;                   // slots per thread per tile (striped by kBlock); 2 or 4 in the count and update/scatter passes
constexpr int kTile = kBlock * kItems;      // slots per tile
constexpr int kTileMin = kBlock * 2;        // the smallest tile the passes run with (the tile arrays have room for its count)
constexpr int kWarps = kBlock / 32;
constexpr uint32_t kMaxRep = 1024;          // replicates per batch

// One pool buffer: structure of arrays, one column per agent field.
struct DevPool {
  float* age; float* his; float* delay; float* sporo;
  uint32_t* uni; uint32_t* avail; uint32_t* cycle; uint32_t* hbc; uint32_t* batches;
  uint8_t* flags;   // bits 0-2 state (0..7), bit 3 isFemale
};

// Device-resident state of one simulation.
// A glibc rand() stream held on the device (generateSeeds, src/abms.c:145-150,
// drawn by k_publish for each coming step). The 31 words are kept rotated so
// that st.r[0] is the oldest (the next draw is r[0] + r[28]); st.i is a
// multiple of 31, so the state also continues on the host's sampo_rand_next.
struct DevSeedStream {
  uint32_t next;              // step whose seeds are drawn next; kNoStream: seeds come from the host
  sampo_rand_state st;
};
constexpr uint32_t kNoStream = 0xffffffffu;

struct SimDev {
  sampo_population pop;       // ranges + stats of the current pool (reference pop[0] at step start)
  sampo_bites_cycles bnc;     // counters of the last update (printed with the next row)
  uint32_t step;              // index of the next step
  uint32_t cur;               // current pool buffer (0/1)
  uint32_t epoch;             // look-back flag value of the running step (never reused)
  uint32_t cnt[8];            // count pass: survivors by next state
  uint32_t newEggs;           // count pass: eggs laid (EggsNbiomass.newEggs)
  uint32_t acc_bnc[4];        // scatter pass: numCycles, sumCycles, numBites, numInfectBites
  uint32_t acc_L1de, acc_fem, acc_inf, acc_dmin, acc_dmax;  // stats of the next pool
  uint32_t error;             // sticky SAMPO_DEV_ERR_* bits
  uint32_t warn;              // sticky SAMPO_DEV_WARN_* bits
  uint32_t capacity;
  float cc;                   // carrying capacity (constant per run, src/abms.c:19,132)
  uint32_t active;            // 1: the replicate takes part in the batch's steps
  uint32_t stop_step;         // becomes inactive once step reaches this
  DevSeedStream rnd;          // the replicate's own rand() stream, when its seeds are drawn on the device
  StepCtx ctx;                // constants of step `step` (valid while active)
  float larvaHMR[100];        // larval hourly mortality of step `step` by age in days
};

// Batch-wide counters of the persistent kernels (tickets reset by k_publish).
struct BatchDev {
  uint32_t ticket1;           // count pass tile ticket
  uint32_t ticket2;           // scatter pass tile ticket
  uint32_t bar;               // one-launch step: CTAs past the decision phase (reset by its last CTA)
  uint32_t done;              // one-launch step: CTAs finished (reset by its last CTA)
};

// The count pass's in-tile prefix table of one tile: for each (round, warp)
// chunk of 32 slots (slot k * kBlock + tid is round k of warp tid / 32) and a
// final entry for the whole tile, the survivors of the chunks before it by next
// state (16-bit pairs: states 0-1, 2-3, 4-5, 6-7) and over all states.
constexpr uint32_t kChunks = kItems * kWarps;
constexpr uint32_t kPreEntryWords = 5;
constexpr uint32_t kPreWords = ((kChunks + 1) * kPreEntryWords + 3) / 4 * 4;  // whole 16-byte units
constexpr uint32_t kPreWordsMax = kPreWords;  // prefix-table words of one tile at I = 4, the largest
constexpr uint32_t kPreWordsMin = ((2 * kWarps + 1) * kPreEntryWords + 3) / 4 * 4;  // at I = 2
// Words of a pool's tile arrays for max_tiles tiles of kTileMin slots: the
// prefix tables (max_tiles of the smaller tile's tables, plus one larger
// table: ceil(C / kTile) tables of kPreWordsMax words fit in that too),
// aggregates (8 per tile) and inclusive prefixes with their epochs (8 x 64 bits
// per tile).
constexpr uint32_t kPreRegionPad = kPreWordsMax;
__host__ __device__ constexpr size_t tile_pre_words(uint32_t max_tiles) {
  return (size_t)max_tiles * kPreWordsMin + kPreRegionPad;
}
__host__ __device__ constexpr size_t tile_array_words(uint32_t max_tiles) {
  return tile_pre_words(max_tiles) + (size_t)max_tiles * (8 + 16);
}
static_assert(kPreWordsMin % 4 == 0 && kPreRegionPad % 4 == 0, "the inclusive prefixes start on a 16-byte boundary");
static_assert(2 * kPreWordsMin >= kPreWordsMax, "two small tables hold one large table");

// Everything the kernels need of one replicate.
struct RepParams {
  SimDev* sim;
  DevPool pool[2];
  uint32_t* tilePre;          // [tiles][pre_words(I)] in-tile prefix tables (count pass), tile_pre_words(maxTiles) words
  uint32_t* tileAgg;          // [maxTiles][8] per-tile survivor counts (count pass)
  unsigned long long* tileIncl;  // [maxTiles][8] inclusive prefixes | epoch << 32 (scatter pass)
  const float* T;             // [ring] temperature per step
  const sampo_environment* env;  // [ring]
  sampo_seeds* seeds;         // [ring][4] (written by the device for a device seed stream)
  const uint32_t* wt;         // [ring] world time per step
  sampo_stats_row* rows;      // [ring] stats at the start of each step
  uint32_t ring;
  uint32_t maxTiles;
};

struct KParams {
  const RepParams* reps;      // device array [nrep]
  uint32_t nrep;
  BatchDev* bat;
  const ModelConst* mc;
  const void* ks;             // host: the kernels compiled for a user species (sampo_species.cu), or null
};

// Modes of k_publish: PUB_AFTER_STEP turns the step's counts into the next
// pool's start; PUB_INITIAL publishes the current pool (after init/load);
// PUB_REFRESH recomputes the coming step's input-dependent constants (run it
// after writing that step's inputs).
enum : int { PUB_INITIAL = 0, PUB_AFTER_STEP = 1, PUB_REFRESH = 2 };

#ifndef __CUDACC_RTC__  // host side (the run-time compiler sees the device part only)

// Hourly mortality tables that do not change during a run
// (kernel/killAgents.cl:84-115,135-147), computed on the host with the same
// deterministic functions the device uses.
inline void fill_constant_tables(ModelConst& h) {
  for (int d = 0; d < 100; d++) {
    const float a = 0.1f, B = 25.0f, sg = 0.1f;
    float e = sampo_expf((float)(uint32_t)d / B);
    float dmr = (a * e) / (1.0f + (a * B * sg * (e - 1.0f)));
    float dsr = 1.0f - dmr;
    float hsr = sampo_powf(dsr, 1.0f / 24.0f);
    h.kill.adultHMR[d] = 1.0f - hsr;
  }
  float dmr = 0.1f;
  float dsr = 1.0f - dmr;
  h.kill.aquaticHMR = 1.0f - sampo_powf(dsr, 1.0f / 24.0f);
  for (uint32_t k = 0; k < kEggBatchTable; k++) h.eggBatchScale[k] = egg_batch_scale(k);
}

// The tile arrays of a pool of max_tiles tiles of kTileMin slots at base
// (16-byte aligned, for the bulk copies of the prefix tables): the prefix
// tables (tile_pre_words words, indexed by the running tile size's table
// length), then aggregates and inclusive prefixes.
inline void set_tile_arrays(RepParams& r, uint32_t* base, uint32_t max_tiles) {
  r.tilePre = base;
  r.tileAgg = base + tile_pre_words(max_tiles);
  r.tileIncl = reinterpret_cast<unsigned long long*>(r.tileAgg + (size_t)max_tiles * 8);
  r.maxTiles = max_tiles;
}

// Why a pool's ranges cannot be stepped, or null when they can: the egg
// range starts at slot 0, no range ends before it starts, the ranges are
// ordered with a gap between them (every layout kernel/oldToNewAgents.cl:57-95
// and createInitialPopulation, src/abms.c:185-228, produce), and the pool's
// end fits `capacity`. Shared by every entry point that takes ranges from
// its caller or from a file.
inline const char* ranges_error(const sampo_population& pop, uint64_t capacity) {
  if (pop.r[0].start != 0) return "the egg range must start at slot 0";
  for (int k = 0; k < 8; k++) {
    if (pop.r[k].end < pop.r[k].start) return "range end before start";
    if (k > 0 && pop.r[k].start <= pop.r[k - 1].end) return "ranges must be ordered with a gap";
  }
  if ((uint64_t)pop.r[7].end > capacity) return "pool exceeds the capacity";
  return nullptr;
}

// Initial device state of a simulation (before its pool is published).
inline SimDev initial_sim_state(uint32_t capacity, float cc) {
  SimDev h;
  memset(&h, 0, sizeof(h));
  h.capacity = capacity;
  h.cc = cc;
  h.acc_dmin = 0xffffffffu;
  h.epoch = 1;
  h.stop_step = 0xffffffffu;
  h.rnd.next = kNoStream;
  return h;
}

// Launch helpers (sampo_kernels.cu). The step kernels take every replicate of
// p; init, pool statistics and the histogram take p.reps[0] only. They launch
// the built-in kernels, or p.ks's when a species was compiled at run time.
// persistent grid sizes (CTAs resident on all SMs) for batches of nrep replicates
int grid_blocks_count(uint32_t nrep, const void* ks = nullptr, int items = kItems);
int grid_blocks_scatter(uint32_t nrep, const void* ks = nullptr, int items = kItems);
// The kernels of a run-time species (sampo_species.cu): launch one, and its
// resident CTAs per SM.
enum : int { KID_COUNT, KID_SCATTER, KID_PUBLISH, KID_INIT_EGGS, KID_POOL_STATS, KID_HISTOGRAM, KID_TRIAL_RESET, KID_N };
cudaError_t species_launch(const void* ks, int kid, dim3 grid, dim3 block, size_t smem, cudaStream_t st, void** args);
int species_occupancy(const void* ks, int kid, int threads, size_t smem);
// dynamic shared memory the persistent kernels may request
size_t count_smem_max();
size_t scatter_smem_max();
// (the built-in passes for `items` = 2 or 4 slots per thread; a run-time
// species is built for 4)
cudaError_t launch_count(const KParams& p, int grid, cudaStream_t st, int items = kItems);
cudaError_t launch_scatter(const KParams& p, int grid, cudaStream_t st, int items = kItems);
// k_publish over every replicate of p (modes PUB_*, above).
cudaError_t launch_publish(const KParams& p, int mode, cudaStream_t st);
cudaError_t launch_init_eggs(const KParams& p, uint32_t n, float T0, const sampo_seeds* seeds_dev,
                             int age_days_max, uint64_t age_seed, cudaStream_t st);
// statistics of p.reps[0]'s current pool, then its publish (PUB_INITIAL)
cudaError_t launch_publish_start(const KParams& p, cudaStream_t st);
cudaError_t launch_histogram(const KParams& p, uint32_t* hist_dev, cudaStream_t st);
cudaError_t launch_eval_math(int fn, const float* x, const float* y, float* out, uint32_t n, cudaStream_t st);
// Kernel nodes in a captured graph (the launches one replay makes).
cudaError_t graph_kernel_nodes(cudaGraph_t g, uint32_t* kernels);
// The one-launch steps of a single simulation (sampo_small_step.cuh) with
// tiles of kBlock * items slots (items 1, 2 or 4): the largest grid (CTAs
// resident on all SMs, 0 if it cannot run) and a launch of `nsteps` hourly
// steps (a cooperative launch when `cooperative`) on `grid` CTAs.
int grid_blocks_small(int items = kItems);
cudaError_t launch_small(const KParams& p, int grid, bool cooperative, uint32_t nsteps, cudaStream_t st,
                         int items = kItems);
// Times count + scatter of the coming step for each tile size (4 and, for
// the built-in species, 2 slots per thread) at every (count, scatter) number
// of CTAs per SM the occupancy allows, and returns the fastest tile size and
// grids. The trials leave the simulations' course unchanged (k_trial_reset);
// the coming step's constants must be current (PUB_REFRESH) before the call.
cudaError_t tune_grids(const KParams& p, cudaStream_t st, int* grid_count, int* grid_scatter, int* items, double* best_ms);

#endif  // __CUDACC_RTC__

}  // namespace sampo
