// sampo_noalloc.cu - one hourly step for callers that cannot allocate device
// memory (see sampo_step_noalloc in include/sampo.h).
//
// The caller owns both pool buffers. Everything else the step needs - the
// device step state, the per-tile survivor counts and look-back prefixes,
// one step of inputs and two stats rows - lives in g_noalloc_scratch, a
// fixed file-scope device array sized for pools of up to
// SAMPO_NOALLOC_MAX_SLOTS slots. The kernels are the ones sampo_step runs;
// only where their scratch lives differs. Nothing here calls cudaMalloc,
// cudaFree or any routine that allocates device memory.
#include <cuda_runtime.h>
#include <stddef.h>
#include <string.h>
#include <mutex>
#include "sampo_model.cuh"
#include "sampo_kernels.cuh"

using namespace sampo;

namespace {

constexpr uint32_t kMaxTiles = SAMPO_NOALLOC_MAX_SLOTS / kTileMin;  // tile arrays in kTileMin-slot tiles

// One step of inputs (ring of two, as the kernels index step % ring).
struct InputBlock {
  float T[2];
  uint32_t wt[2];
  sampo_environment env[2];
  sampo_seeds seeds[8];
};

struct Scratch {
  __align__(16) uint32_t tiles[tile_array_words(kMaxTiles)];  // prefix tables | counts | inclusive prefixes
  SimDev sim;
  RepParams rep;
  BatchDev bat;
  ModelConst mc;
  sampo_stats_row rows[2];
  InputBlock in;
};

}  // namespace

// Held by every GPU that loads the library, until the process exits.
static __device__ __align__(256) unsigned char g_noalloc_scratch[sizeof(Scratch)];

// The array's device address, resolved once per device with that device
// current. In host code g_noalloc_scratch names a host-side stand-in, never
// a device address, so kernels only ever receive the resolved pointer.
static std::mutex g_scratch_mutex;
static unsigned char* g_scratch_addr[64];

static cudaError_t scratch_address(int device, unsigned char** out) {
  std::lock_guard<std::mutex> lock(g_scratch_mutex);
  if (device < 0 || device >= 64) return cudaErrorInvalidDevice;
  if (!g_scratch_addr[device]) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) return e;
    g_scratch_addr[device] = (unsigned char*)p;
  }
  *out = g_scratch_addr[device];
  return cudaSuccess;
}

static bool aligned16(const void* p) { return ((uintptr_t)p & 15u) == 0; }

static bool pool_ok(const sampo_device_pool* d) {
  return aligned16(d->ageInHours) && aligned16(d->hoursInState) && aligned16(d->delay) &&
         aligned16(d->cumulativeSporogonicDevelopment) && aligned16(d->larvalDelayOrOviAttempts) &&
         aligned16(d->availableEggs) && aligned16(d->cycleLength) && aligned16(d->humanBloodmealCount) &&
         aligned16(d->numEggBatches) && aligned16(d->flags) && d->ageInHours && d->flags;
}

// Whether any column of buffer a (a_cap slots) overlaps any column of buffer
// b (b_cap slots): the step reads `in` while it writes `out`, so the two
// must be disjoint.
static bool pools_overlap(const sampo_device_pool* a, uint32_t a_cap, const sampo_device_pool* b, uint32_t b_cap) {
  const void* ca[10] = {a->ageInHours, a->hoursInState, a->delay, a->cumulativeSporogonicDevelopment,
                        a->larvalDelayOrOviAttempts, a->availableEggs, a->cycleLength, a->humanBloodmealCount,
                        a->numEggBatches, a->flags};
  const void* cb[10] = {b->ageInHours, b->hoursInState, b->delay, b->cumulativeSporogonicDevelopment,
                        b->larvalDelayOrOviAttempts, b->availableEggs, b->cycleLength, b->humanBloodmealCount,
                        b->numEggBatches, b->flags};
  for (int i = 0; i < 10; i++) {
    const uintptr_t a0 = (uintptr_t)ca[i], a1 = a0 + (uintptr_t)a_cap * (i == 9 ? 1u : 4u) + 16u;
    for (int j = 0; j < 10; j++) {
      const uintptr_t b0 = (uintptr_t)cb[j], b1 = b0 + (uintptr_t)b_cap * (j == 9 ? 1u : 4u) + 16u;
      if (a0 < b1 && b0 < a1) return true;
    }
  }
  return false;
}

static DevPool to_dev(const sampo_device_pool* d) {
  DevPool p;
  p.age = d->ageInHours; p.his = d->hoursInState; p.delay = d->delay; p.sporo = d->cumulativeSporogonicDevelopment;
  p.uni = d->larvalDelayOrOviAttempts; p.avail = d->availableEggs; p.cycle = d->cycleLength;
  p.hbc = d->humanBloodmealCount; p.batches = d->numEggBatches; p.flags = d->flags;
  return p;
}

static int run_step(const sampo_device_pool* in, uint32_t in_capacity, const sampo_device_pool* out, uint32_t out_capacity,
                    const sampo_population* pop_in, const sampo_environment* env, float temperature, uint32_t world_time,
                    const sampo_seeds seeds[4], float cc, sampo_stats_row* row, sampo_population* pop_out,
                    sampo_bites_cycles* bnc_out, int device, cudaStream_t st) {
  unsigned char* base = nullptr;
  if (scratch_address(device, &base) != cudaSuccess) return SAMPO_ERR_CUDA;
  Scratch* sc = (Scratch*)base;

  SimDev h = initial_sim_state(out_capacity, cc);
  h.pop = *pop_in;
  h.pop.numLarvae1DayEquiv = h.pop.numFemale = h.pop.numPotentiallyInfective = 0;
  h.active = 1;
  ModelConst mc;
  fill_constant_tables(mc);
  BatchDev bat;
  memset(&bat, 0, sizeof(bat));
  InputBlock ib;
  memset(&ib, 0, sizeof(ib));
  ib.T[0] = temperature;
  ib.wt[0] = world_time;
  ib.env[0] = *env;
  for (int k = 0; k < 4; k++) ib.seeds[k] = seeds[k];

  // The array keeps the previous call's contents: reset the state, and clear
  // the inclusive prefixes of the tiles this step uses (a stale word carrying
  // this step's epoch would be taken for a published prefix).
  const uint32_t ntiles = (pop_in->r[7].end + kTile - 1) / kTile;
  RepParams rp;
  rp.sim = &sc->sim;
  rp.pool[0] = to_dev(in);
  rp.pool[1] = to_dev(out);
  set_tile_arrays(rp, sc->tiles, kMaxTiles);
  rp.T = sc->in.T;
  rp.env = sc->in.env;
  rp.seeds = sc->in.seeds;
  rp.wt = sc->in.wt;
  rp.rows = sc->rows;
  rp.ring = 2;
  if (cudaMemcpyAsync(&sc->sim, &h, sizeof(h), cudaMemcpyHostToDevice, st) != cudaSuccess ||
      cudaMemcpyAsync(&sc->rep, &rp, sizeof(rp), cudaMemcpyHostToDevice, st) != cudaSuccess ||
      cudaMemcpyAsync(&sc->bat, &bat, sizeof(bat), cudaMemcpyHostToDevice, st) != cudaSuccess ||
      cudaMemcpyAsync(&sc->mc, &mc, sizeof(mc), cudaMemcpyHostToDevice, st) != cudaSuccess ||
      cudaMemcpyAsync(&sc->in, &ib, sizeof(ib), cudaMemcpyHostToDevice, st) != cudaSuccess)
    return SAMPO_ERR_CUDA;
  if (ntiles && cudaMemsetAsync(rp.tileIncl, 0, (size_t)ntiles * 8 * sizeof(unsigned long long), st) != cudaSuccess)
    return SAMPO_ERR_CUDA;

  KParams p;
  p.reps = &sc->rep;
  p.nrep = 1;
  p.bat = &sc->bat;
  p.mc = &sc->mc;
  p.ks = nullptr;  // the built-in species
  if (launch_publish_start(p, st) != cudaSuccess) return SAMPO_ERR_CUDA;
  if (launch_count(p, grid_blocks_count(1), st) != cudaSuccess) return SAMPO_ERR_CUDA;
  if (launch_scatter(p, grid_blocks_scatter(1), st) != cudaSuccess) return SAMPO_ERR_CUDA;
  if (launch_publish(p, PUB_AFTER_STEP, st) != cudaSuccess) return SAMPO_ERR_CUDA;

  uint32_t err = 0;
  if (cudaMemcpyAsync(row, &sc->rows[0], sizeof(*row), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
      cudaMemcpyAsync(pop_out, &sc->sim.pop, sizeof(*pop_out), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
      cudaMemcpyAsync(bnc_out, &sc->sim.bnc, sizeof(*bnc_out), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
      cudaMemcpyAsync(&err, &sc->sim.error, sizeof(err), cudaMemcpyDeviceToHost, st) != cudaSuccess)
    return SAMPO_ERR_CUDA;
  if (cudaStreamSynchronize(st) != cudaSuccess) return SAMPO_ERR_CUDA;
  if (err & SAMPO_DEV_ERR_CAPACITY) return SAMPO_ERR_CAPACITY;
  if (err & SAMPO_DEV_ERR_DEVRATES) return SAMPO_ERR_TEMPERATURE;
  if (err) return SAMPO_ERR_INTERNAL;
  return SAMPO_OK;
}

extern "C" int sampo_step_noalloc(const sampo_device_pool* in, uint32_t in_capacity, const sampo_device_pool* out,
                                  uint32_t out_capacity, const sampo_population* pop_in, const sampo_environment* env,
                                  float temperature, uint32_t world_time, const sampo_seeds seeds[4], float carrying_capacity,
                                  sampo_stats_row* row, sampo_population* pop_out, sampo_bites_cycles* bnc_out, int device,
                                  void* stream) {
  if (!in || !out || !pop_in || !env || !seeds || !row || !pop_out || !bnc_out) return SAMPO_ERR_ARG;
  if (in_capacity > SAMPO_NOALLOC_MAX_SLOTS || out_capacity > SAMPO_NOALLOC_MAX_SLOTS || out_capacity < 128)
    return SAMPO_ERR_ARG;  // the fixed scratch covers pools of up to SAMPO_NOALLOC_MAX_SLOTS slots
  if (!(carrying_capacity > 0.0f) || env->carryingCapacity != carrying_capacity) return SAMPO_ERR_ARG;
  if (ranges_error(*pop_in, in_capacity)) return SAMPO_ERR_ARG;
  if (!pool_ok(in) || !pool_ok(out)) return SAMPO_ERR_ARG;
  if (pools_overlap(in, in_capacity, out, out_capacity)) return SAMPO_ERR_ARG;
  int prev = -1;
  if (cudaGetDevice(&prev) != cudaSuccess) return SAMPO_ERR_CUDA;
  if (cudaSetDevice(device) != cudaSuccess) return SAMPO_ERR_CUDA;
  // the call copies from host memory and waits for the step: it cannot be
  // recorded into a graph
  cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
  if (cudaStreamIsCapturing((cudaStream_t)stream, &cap) != cudaSuccess || cap != cudaStreamCaptureStatusNone) {
    cudaSetDevice(prev);
    return SAMPO_ERR_STATE;
  }
  const int rc = run_step(in, in_capacity, out, out_capacity, pop_in, env, temperature, world_time, seeds,
                          carrying_capacity, row, pop_out, bnc_out, device, (cudaStream_t)stream);
  cudaSetDevice(prev);
  return rc;
}
