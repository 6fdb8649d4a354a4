// sampo_api.cu - host side of the C ABI declared in include/sampo.h.
//
// One handle owns one simulation on one GPU: two pool buffers, the device
// step state, the per-tile look-back arrays and rings of per-step inputs and
// stats rows; the kernels see it as a batch of one replicate. No call exits
// the process; errors come back as status codes with a message in
// sampo_last_error.
#include <cuda_runtime.h>
#include <string.h>
#include <stdio.h>
#include <stdlib.h>
#include <string>
#include <vector>
#include "sampo_model.cuh"
#include "sampo_kernels.cuh"
#include "sampo_checkpoint.cuh"

using namespace sampo;

struct sampo_sim {
  int device = 0;
  const void* species = nullptr;     // kernels compiled for a user species, or null (built in)
  cudaStream_t stream = nullptr;
  uint64_t capacity = 0;
  uint32_t ring = 0;
  float cc = 0.0f;
  void* pool_mem[2] = {nullptr, nullptr};
  DevPool pool[2];
  SimDev* sim_dev = nullptr;
  RepParams* rep_dev = nullptr;        // this simulation as a batch of one
  BatchDev* bat_dev = nullptr;
  ModelConst* mc_dev = nullptr;
  uint32_t* tile_mem = nullptr;
  uint32_t max_tiles = 0;
  float* T_dev = nullptr;
  sampo_environment* env_dev = nullptr;
  sampo_seeds* seeds_dev = nullptr;
  uint32_t* wt_dev = nullptr;
  sampo_stats_row* rows_dev = nullptr;
  sampo_stats_row* rows_pinned = nullptr;
  sampo_seeds* init_seeds_dev = nullptr;
  uint32_t* hist_dev = nullptr;
  std::vector<float> T_host;           // inputs as set (for temperature[0] and checks)
  std::vector<uint8_t> have_inputs;    // per ring slot: inputs present for absolute step
  std::vector<uint32_t> input_step;    // absolute step whose inputs occupy the slot
  std::vector<uint32_t> seed_step;     // absolute step whose seeds occupy the slot
  std::vector<uint32_t> wt_staging;    // world times being uploaded
  void* flush_buf = nullptr;           // L2 flush scratch (allocated on first use)
  size_t flush_bytes = 0;
  double last_run_ms = 0;
  SimDev host_state;                   // template for (re)initialisation
  uint32_t step = 0;                   // host mirror of the device step index
  uint32_t epoch = 1;                  // host mirror of the device epoch
  bool have_pop = false;
  bool pending = false;                // steps queued by sampo_run_async, not yet synced
  int grid_count = 0, grid_scatter = 0;
  int items = kItems;                  // slots per thread of the count and update/scatter passes (2 or 4)
  cudaGraphExec_t day_graph = nullptr;  // 24 three-kernel steps
  uint32_t day_graph_kernels = 0;      // kernel nodes of day_graph (counted at capture)
  // One-launch step for small pools: day graphs of 24 one-launch steps on
  // grids sized to the pool (kSmallBuckets sizes up to small_grid), picked
  // per day from the pool end the host last saw (known_end).
  int small_grid = 0;                  // largest grid of the one-launch step (0: it cannot run on this device)
  uint32_t small_tiles = 0;            // largest pool in 1024-slot tiles that takes the one-launch step (0: never)
  int small_items = 0;                 // its slots per thread: 1, 2, 4, or 0 (by pool size)
  cudaGraphExec_t small_graph[3][8] = {};  // [256-, 512-, 1024-slot tiles][grid bucket]
  int small_graph_kind[3][8] = {};     // DG_* of each
  uint32_t known_end = 0;              // pool end at the start of the coming day, as last seen by the host
  uint32_t* end_pinned = nullptr;      // pool end after a day, copied back one day behind the queue
  cudaEvent_t ev_day[2] = {nullptr, nullptr};
  int last_day_kind = 0;               // DG_* of the last day launched
  uint64_t days_small = 0, days_three = 0;
  bool timing = false;
  cudaEvent_t ev[5] = {nullptr, nullptr, nullptr, nullptr, nullptr};
  double t_count = 0, t_scatter = 0, t_total = 0;
  uint64_t launches = 0;
  std::string err;
};

// How a day graph steps the simulation: the three-kernel step every hour, or
// the one-launch step launched cooperatively or (where a graph cannot hold a
// cooperative launch) as a plain launch of the same co-resident grid.
enum : int { DG_PLAIN = 1, DG_SMALL_COOP = 2, DG_SMALL = 3 };
// Grid sizes of the one-launch day graphs (the last one is the largest
// co-resident grid), and the growth a pool is allowed between the day whose
// end the host saw and the end of the day it picks for (one day behind, one
// day of growth): a grid of at least kSmallGrowth CTAs per tile seen.
constexpr int kSmallBuckets = 8;
constexpr uint32_t kSmallGrowth = 2;
static uint32_t small_bucket_grid(const sampo_sim* s, int b) {
  const uint32_t g = 8u << b;
  return (b == kSmallBuckets - 1 || g >= (uint32_t)s->small_grid) ? (uint32_t)s->small_grid : g;
}

static int fail(sampo_sim* s, int code, const std::string& msg) {
  if (s) s->err = msg;
  return code;
}
static int cuda_fail(sampo_sim* s, cudaError_t e, const char* what) {
  return fail(s, SAMPO_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}
#define CK(call, what)                                   \
  do {                                                   \
    cudaError_t e_ = (call);                             \
    if (e_ != cudaSuccess) return cuda_fail(s, e_, what); \
  } while (0)

extern "C" int sampo_sync(sampo_sim* s);
// Every call that reads or changes the simulation first waits for the steps
// sampo_run_async queued, and returns their error if they failed.
#define SETTLE(s)                          \
  do {                                     \
    if ((s)->pending) {                    \
      int rc_ = sampo_sync(s);             \
      if (rc_ != SAMPO_OK) return rc_;     \
    }                                      \
  } while (0)

static size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

static RepParams make_rep(sampo_sim* s) {
  RepParams r;
  r.sim = s->sim_dev;
  r.pool[0] = s->pool[0];
  r.pool[1] = s->pool[1];
  set_tile_arrays(r, s->tile_mem, s->max_tiles);
  r.T = s->T_dev;
  r.env = s->env_dev;
  r.seeds = s->seeds_dev;
  r.wt = s->wt_dev;
  r.rows = s->rows_dev;
  r.ring = s->ring;
  return r;
}

static KParams make_params(sampo_sim* s) {
  KParams p;
  p.reps = s->rep_dev;
  p.nrep = 1;
  p.bat = s->bat_dev;
  p.mc = s->mc_dev;
  p.ks = s->species;
  return p;
}

extern "C" int sampo_abi_version(void) { return SAMPO_ABI_VERSION; }

extern "C" const char* sampo_last_error(const sampo_sim* s) { return s ? s->err.c_str() : "null handle"; }

extern "C" int sampo_destroy(sampo_sim* s) {
  if (!s) return SAMPO_OK;
  cudaSetDevice(s->device);
  if (s->stream) cudaStreamSynchronize(s->stream);
  if (s->day_graph) cudaGraphExecDestroy(s->day_graph);
  for (auto& row : s->small_graph)
    for (auto& g : row) if (g) cudaGraphExecDestroy(g);
  for (auto& e : s->ev_day) if (e) cudaEventDestroy(e);
  if (s->end_pinned) cudaFreeHost(s->end_pinned);
  for (auto& e : s->ev) if (e) cudaEventDestroy(e);
  cudaFree(s->pool_mem[0]); cudaFree(s->pool_mem[1]);
  cudaFree(s->sim_dev); cudaFree(s->tile_mem);
  cudaFree(s->rep_dev); cudaFree(s->bat_dev); cudaFree(s->mc_dev);
  cudaFree(s->T_dev); cudaFree(s->env_dev); cudaFree(s->seeds_dev); cudaFree(s->wt_dev);
  cudaFree(s->rows_dev); cudaFree(s->init_seeds_dev); cudaFree(s->hist_dev); cudaFree(s->flush_buf);
  if (s->rows_pinned) cudaFreeHost(s->rows_pinned);
  if (s->stream) cudaStreamDestroy(s->stream);
  delete s;
  return SAMPO_OK;
}

extern "C" int sampo_create(const sampo_config* cfg, sampo_sim** out) {
  if (!cfg || !out) return SAMPO_ERR_ARG;
  *out = nullptr;
  if (cfg->capacity < 128 || cfg->capacity > 0xFFFFFF00ull) return SAMPO_ERR_ARG;
  if (!(cfg->carrying_capacity > 0.0f)) return SAMPO_ERR_ARG;
  sampo_sim* s = new sampo_sim();
  s->device = cfg->device;
  s->capacity = cfg->capacity;
  s->ring = cfg->max_steps >= 2 ? cfg->max_steps : 8760;
  s->cc = cfg->carrying_capacity;
  int rc = SAMPO_OK;
  do {
    cudaError_t e = cudaSetDevice(s->device);
    if (e != cudaSuccess) { rc = cuda_fail(s, e, "cudaSetDevice"); break; }
    if ((e = cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking)) != cudaSuccess) { rc = cuda_fail(s, e, "stream"); break; }
    const size_t C = s->capacity;
    // 16 bytes of slack per column: tile copies are rounded up to 16 bytes
    // and may read up to 15 bytes past the last slot.
    const size_t col4 = align256(C * 4 + 16), col1 = align256(C + 16);
    const size_t bytes = 9 * col4 + col1;
    for (int b = 0; b < 2; b++) {
      if ((e = cudaMalloc(&s->pool_mem[b], bytes)) != cudaSuccess) { rc = cuda_fail(s, e, "pool allocation"); break; }
      char* m = (char*)s->pool_mem[b];
      DevPool& P = s->pool[b];
      P.age = (float*)(m + 0 * col4); P.his = (float*)(m + 1 * col4); P.delay = (float*)(m + 2 * col4);
      P.sporo = (float*)(m + 3 * col4); P.uni = (uint32_t*)(m + 4 * col4); P.avail = (uint32_t*)(m + 5 * col4);
      P.cycle = (uint32_t*)(m + 6 * col4); P.hbc = (uint32_t*)(m + 7 * col4); P.batches = (uint32_t*)(m + 8 * col4);
      P.flags = (uint8_t*)(m + 9 * col4);
    }
    if (rc) break;
    s->max_tiles = (uint32_t)((C + kTileMin - 1) / kTileMin);  // room for the smaller tile's count
    if ((e = cudaMalloc(&s->tile_mem, tile_array_words(s->max_tiles) * 4)) != cudaSuccess) { rc = cuda_fail(s, e, "tile arrays"); break; }
    cudaMemsetAsync(s->tile_mem, 0, tile_array_words(s->max_tiles) * 4, s->stream);
    if ((e = cudaMalloc(&s->sim_dev, sizeof(SimDev))) != cudaSuccess ||
        (e = cudaMalloc(&s->rep_dev, sizeof(RepParams))) != cudaSuccess ||
        (e = cudaMalloc(&s->bat_dev, sizeof(BatchDev))) != cudaSuccess ||
        (e = cudaMalloc(&s->mc_dev, sizeof(ModelConst))) != cudaSuccess) {
      rc = cuda_fail(s, e, "state");
      break;
    }
    const size_t R = s->ring;
    if ((e = cudaMalloc(&s->T_dev, R * sizeof(float))) != cudaSuccess ||
        (e = cudaMalloc(&s->env_dev, R * sizeof(sampo_environment))) != cudaSuccess ||
        (e = cudaMalloc(&s->seeds_dev, R * 4 * sizeof(sampo_seeds))) != cudaSuccess ||
        (e = cudaMalloc(&s->wt_dev, R * sizeof(uint32_t))) != cudaSuccess ||
        (e = cudaMalloc(&s->rows_dev, R * sizeof(sampo_stats_row))) != cudaSuccess ||
        (e = cudaMalloc(&s->init_seeds_dev, 4 * sizeof(sampo_seeds))) != cudaSuccess ||
        (e = cudaMalloc(&s->hist_dev, 100 * sizeof(uint32_t))) != cudaSuccess ||
        (e = cudaMallocHost(&s->rows_pinned, R * sizeof(sampo_stats_row))) != cudaSuccess) {
      rc = cuda_fail(s, e, "input rings");
      break;
    }
    s->T_host.assign(R, 0.0f);
    s->have_inputs.assign(R, 0);
    s->input_step.assign(R, 0xffffffffu);
    s->seed_step.assign(R, 0xffffffffu);
    s->host_state = initial_sim_state((uint32_t)C, s->cc);
    s->host_state.active = 1;
    ModelConst mc;
    fill_constant_tables(mc);
    const RepParams rep = make_rep(s);
    if ((e = cudaMemcpyAsync(s->sim_dev, &s->host_state, sizeof(SimDev), cudaMemcpyHostToDevice, s->stream)) != cudaSuccess ||
        (e = cudaMemcpyAsync(s->rep_dev, &rep, sizeof(RepParams), cudaMemcpyHostToDevice, s->stream)) != cudaSuccess ||
        (e = cudaMemcpyAsync(s->mc_dev, &mc, sizeof(ModelConst), cudaMemcpyHostToDevice, s->stream)) != cudaSuccess ||
        (e = cudaMemsetAsync(s->bat_dev, 0, sizeof(BatchDev), s->stream)) != cudaSuccess) {
      rc = cuda_fail(s, e, "state upload");
      break;
    }
    s->grid_count = grid_blocks_count(1);
    s->grid_scatter = grid_blocks_scatter(1);
    s->small_grid = std::min(grid_blocks_small(1), std::min(grid_blocks_small(2), grid_blocks_small(4)));
    s->small_tiles = s->small_grid > 0 ? (uint32_t)s->small_grid : 0u;  // one tile per CTA
    if ((e = cudaMallocHost(&s->end_pinned, 2 * sizeof(uint32_t))) != cudaSuccess) { rc = cuda_fail(s, e, "pinned"); break; }
    for (auto& ev : s->ev_day) cudaEventCreateWithFlags(&ev, cudaEventDisableTiming);
    for (auto& ev : s->ev) cudaEventCreate(&ev);
    if ((e = cudaStreamSynchronize(s->stream)) != cudaSuccess) { rc = cuda_fail(s, e, "create"); break; }
  } while (0);
  if (rc) {
    fprintf(stderr, "sampo_create: %s\n", s->err.c_str());
    sampo_destroy(s);
    return rc;
  }
  *out = s;
  return SAMPO_OK;
}

extern "C" int sampo_set_inputs(sampo_sim* s, uint32_t first, const float* temperature, const sampo_environment* env,
                                uint32_t nsteps) {
  if (!s || !temperature || !env) return SAMPO_ERR_ARG;
  SETTLE(s);
  if (nsteps == 0 || nsteps > s->ring) return fail(s, SAMPO_ERR_ARG, "nsteps exceeds the input ring (config.max_steps)");
  for (uint32_t i = 0; i < nsteps; i++)
    if (env[i].carryingCapacity != s->cc)
      return fail(s, SAMPO_ERR_ARG, "environment carryingCapacity differs from the configured carrying capacity");
  cudaSetDevice(s->device);
  if (s->wt_staging.size() < nsteps) s->wt_staging.resize(nsteps);
  uint32_t done = 0;
  while (done < nsteps) {
    const uint32_t step = first + done, slot = step % s->ring;
    const uint32_t n = std::min(nsteps - done, s->ring - slot);
    for (uint32_t i = 0; i < n; i++) {
      s->wt_staging[done + i] = (step + i) % 24u;  // (UINT)(currentStep * hoursInTimeStep) % 24u, src/abms.c:514
      s->T_host[slot + i] = temperature[done + i];
      s->have_inputs[slot + i] = 1;
      s->input_step[slot + i] = step + i;
    }
    CK(cudaMemcpyAsync(s->T_dev + slot, temperature + done, n * sizeof(float), cudaMemcpyHostToDevice, s->stream), "inputs");
    CK(cudaMemcpyAsync(s->env_dev + slot, env + done, n * sizeof(sampo_environment), cudaMemcpyHostToDevice, s->stream), "inputs");
    CK(cudaMemcpyAsync(s->wt_dev + slot, s->wt_staging.data() + done, n * sizeof(uint32_t), cudaMemcpyHostToDevice, s->stream), "inputs");
    done += n;
  }
  CK(cudaStreamSynchronize(s->stream), "inputs");
  return SAMPO_OK;
}

extern "C" int sampo_set_seeds(sampo_sim* s, uint32_t first, const sampo_seeds* seeds, uint32_t nsteps) {
  if (!s || !seeds) return SAMPO_ERR_ARG;
  SETTLE(s);
  if (nsteps == 0 || nsteps > s->ring) return fail(s, SAMPO_ERR_ARG, "nsteps exceeds the seed ring (config.max_steps)");
  cudaSetDevice(s->device);
  uint32_t done = 0;
  while (done < nsteps) {
    uint32_t step = first + done;
    uint32_t slot = step % s->ring;
    uint32_t n = std::min(nsteps - done, s->ring - slot);
    CK(cudaMemcpyAsync(s->seeds_dev + (size_t)slot * 4, seeds + (size_t)done * 4, (size_t)n * 4 * sizeof(sampo_seeds),
                       cudaMemcpyHostToDevice, s->stream), "seeds");
    for (uint32_t i = 0; i < n; i++) s->seed_step[slot + i] = step + i;
    done += n;
  }
  CK(cudaStreamSynchronize(s->stream), "seeds");
  return SAMPO_OK;
}

static int reset_state(sampo_sim* s, const sampo_population& pop) {
  SimDev h = s->host_state;
  h.pop = pop;
  h.active = 1;
  h.step = 0;
  h.cur = 0;
  // The look-back trusts a tile's inclusive prefix when its flag equals the
  // running step's epoch. Epochs restart here, so flags left by an earlier
  // run must go: clear the tile arrays before the first step.
  h.epoch = 1;
  CK(cudaMemsetAsync(s->tile_mem, 0, tile_array_words(s->max_tiles) * 4, s->stream), "tile reset");
  // the one-launch step's grid barrier and exit counters start from zero
  CK(cudaMemsetAsync(&s->bat_dev->bar, 0, 2 * sizeof(uint32_t), s->stream), "barrier reset");
  CK(cudaMemcpyAsync(s->sim_dev, &h, sizeof(SimDev), cudaMemcpyHostToDevice, s->stream), "state reset");
  s->step = 0;
  return SAMPO_OK;
}

static int publish_initial(sampo_sim* s) {
  KParams p = make_params(s);
  CK(launch_publish_start(p, s->stream), "initial statistics");
  CK(cudaMemcpyAsync(s->end_pinned, &s->sim_dev->pop.r[GRAVID].end, sizeof(uint32_t), cudaMemcpyDeviceToHost, s->stream),
     "initial statistics");
  CK(cudaStreamSynchronize(s->stream), "initial statistics");
  s->known_end = s->end_pinned[0];
  s->have_pop = true;
  return SAMPO_OK;
}

extern "C" int sampo_init_population(sampo_sim* s, uint32_t n, const sampo_seeds init_seeds[4], int age_days_max, uint64_t age_seed) {
  if (!s || !init_seeds) return SAMPO_ERR_ARG;
  SETTLE(s);
  if (!s->have_inputs[0] || s->input_step[0] != 0)
    return fail(s, SAMPO_ERR_STATE, "set the inputs first: the initial eggs use temperature[0] (src/abms.c:198)");
  cudaSetDevice(s->device);
  sampo_population pop;
  memset(&pop, 0, sizeof(pop));
  pop.r[0].start = 0;
  pop.r[0].end = n;
  if (age_days_max < 0) {
    for (int k = 1; k < 8; k++) { pop.r[k].start = n + 1; pop.r[k].end = n + 1; }  // src/abms.c:204-219
  } else {
    for (int k = 1; k < 8; k++) {
      pop.r[k].start = ((pop.r[k - 1].end + kLayoutAlign) / kLayoutAlign) * kLayoutAlign;
      pop.r[k].end = pop.r[k].start;
    }
  }
  if ((uint64_t)pop.r[7].end > s->capacity) return fail(s, SAMPO_ERR_CAPACITY, "initial population exceeds the capacity");
  int rc = reset_state(s, pop);
  if (rc) return rc;
  CK(cudaMemcpyAsync(s->init_seeds_dev, init_seeds, 4 * sizeof(sampo_seeds), cudaMemcpyHostToDevice, s->stream), "seeds");
  KParams p = make_params(s);
  CK(launch_init_eggs(p, n, s->T_host[0], s->init_seeds_dev, age_days_max, age_seed, s->stream), "initAgents");
  return publish_initial(s);
}

extern "C" int sampo_load_pool(sampo_sim* s, const sampo_population* pop, const sampo_pool_view* v) {
  if (!s || !pop || !v) return SAMPO_ERR_ARG;
  SETTLE(s);
  if (const char* why = ranges_error(*pop, UINT64_MAX)) return fail(s, SAMPO_ERR_ARG, why);
  const uint32_t n = pop->r[7].end;
  if ((uint64_t)n > s->capacity) return fail(s, SAMPO_ERR_CAPACITY, "pool exceeds the capacity");
  cudaSetDevice(s->device);
  sampo_population p0 = *pop;
  int rc = reset_state(s, p0);
  if (rc) return rc;
  const DevPool& P = s->pool[0];
  const size_t b4 = (size_t)n * 4;
  CK(cudaMemcpyAsync(P.age, v->ageInHours, b4, cudaMemcpyHostToDevice, s->stream), "pool upload");
  CK(cudaMemcpyAsync(P.his, v->hoursInState, b4, cudaMemcpyHostToDevice, s->stream), "pool upload");
  CK(cudaMemcpyAsync(P.delay, v->delay, b4, cudaMemcpyHostToDevice, s->stream), "pool upload");
  CK(cudaMemcpyAsync(P.sporo, v->cumulativeSporogonicDevelopment, b4, cudaMemcpyHostToDevice, s->stream), "pool upload");
  CK(cudaMemcpyAsync(P.uni, v->larvalDelayOrOviAttempts, b4, cudaMemcpyHostToDevice, s->stream), "pool upload");
  CK(cudaMemcpyAsync(P.avail, v->availableEggs, b4, cudaMemcpyHostToDevice, s->stream), "pool upload");
  CK(cudaMemcpyAsync(P.cycle, v->cycleLength, b4, cudaMemcpyHostToDevice, s->stream), "pool upload");
  CK(cudaMemcpyAsync(P.hbc, v->humanBloodmealCount, b4, cudaMemcpyHostToDevice, s->stream), "pool upload");
  CK(cudaMemcpyAsync(P.batches, v->numEggBatches, b4, cudaMemcpyHostToDevice, s->stream), "pool upload");
  std::vector<uint8_t> flags(n);
  for (uint32_t i = 0; i < n; i++) flags[i] = (uint8_t)((v->state[i] & 7u) | ((v->isFemale[i] ? 1u : 0u) << 3));
  CK(cudaMemcpyAsync(P.flags, flags.data(), n, cudaMemcpyHostToDevice, s->stream), "pool upload");
  CK(cudaStreamSynchronize(s->stream), "pool upload");
  return publish_initial(s);
}

static int check_device(sampo_sim* s) {
  uint32_t st[2];
  CK(cudaMemcpyAsync(st, &s->sim_dev->error, 2 * sizeof(uint32_t), cudaMemcpyDeviceToHost, s->stream), "status");
  CK(cudaMemcpyAsync(s->end_pinned, &s->sim_dev->pop.r[GRAVID].end, sizeof(uint32_t), cudaMemcpyDeviceToHost, s->stream), "status");
  CK(cudaStreamSynchronize(s->stream), "status");
  s->known_end = s->end_pinned[0];  // the pool end the coming day's graph is picked by
  if (st[0] & SAMPO_DEV_ERR_CAPACITY) return fail(s, SAMPO_ERR_CAPACITY, "not enough capacity for the next layout");
  if (st[0] & SAMPO_DEV_ERR_DEVRATES) return fail(s, SAMPO_ERR_TEMPERATURE, "temperature >= 44 C: the reference reads past devRates");
  if (st[0]) return fail(s, SAMPO_ERR_INTERNAL, "device consistency check failed (bits " + std::to_string(st[0]) + ")");
  return SAMPO_OK;
}

static cudaError_t launch_step(sampo_sim* s, const KParams& p) {
  cudaError_t e = launch_count(p, s->grid_count, s->stream, s->items);
  if (e != cudaSuccess) return e;
  if ((e = launch_scatter(p, s->grid_scatter, s->stream, s->items)) != cudaSuccess) return e;
  return launch_publish(p, PUB_AFTER_STEP, s->stream);
}

extern "C" int sampo_step(sampo_sim* s, const sampo_environment* env, float temperature, uint32_t world_time,
                          const sampo_seeds seeds[4], sampo_stats_row* row) {
  if (!s || !env || !seeds) return SAMPO_ERR_ARG;
  SETTLE(s);
  if (!s->have_pop) return fail(s, SAMPO_ERR_STATE, "no population: call sampo_init_population or sampo_load_pool");
  if (env->carryingCapacity != s->cc) return fail(s, SAMPO_ERR_ARG, "environment carryingCapacity differs from the configured carrying capacity");
  cudaSetDevice(s->device);
  const uint32_t slot = s->step % s->ring;
  CK(cudaMemcpyAsync(s->T_dev + slot, &temperature, sizeof(float), cudaMemcpyHostToDevice, s->stream), "step inputs");
  CK(cudaMemcpyAsync(s->env_dev + slot, env, sizeof(sampo_environment), cudaMemcpyHostToDevice, s->stream), "step inputs");
  CK(cudaMemcpyAsync(s->wt_dev + slot, &world_time, sizeof(uint32_t), cudaMemcpyHostToDevice, s->stream), "step inputs");
  CK(cudaMemcpyAsync(s->seeds_dev + (size_t)slot * 4, seeds, 4 * sizeof(sampo_seeds), cudaMemcpyHostToDevice, s->stream), "step inputs");
  s->T_host[slot] = temperature;
  s->have_inputs[slot] = 1;
  s->input_step[slot] = s->step;
  s->seed_step[slot] = s->step;
  if (row) CK(cudaMemcpyAsync(row, s->rows_dev + slot, sizeof(sampo_stats_row), cudaMemcpyDeviceToHost, s->stream), "row");
  KParams p = make_params(s);
  CK(launch_publish(p, PUB_REFRESH, s->stream), "step constants");  // this step's inputs were just written
  CK(launch_step(s, p), "step kernels");
  s->launches += 4;
  s->step++;
  return check_device(s);
}

static int build_day_graph(sampo_sim* s) {
  if (s->day_graph) return SAMPO_OK;
  KParams p = make_params(s);
  cudaGraph_t g = nullptr;
  CK(cudaStreamBeginCapture(s->stream, cudaStreamCaptureModeThreadLocal), "capture");
  cudaError_t e = cudaSuccess;
  for (int h = 0; h < 24 && e == cudaSuccess; h++) e = launch_step(s, p);
  cudaError_t e2 = cudaStreamEndCapture(s->stream, &g);
  if (e != cudaSuccess) { if (g) cudaGraphDestroy(g); return cuda_fail(s, e, "capture launch"); }
  if (e2 != cudaSuccess) return cuda_fail(s, e2, "end capture");
  // the launches a replay makes: the kernel nodes the capture recorded
  uint32_t kernels = 0;
  e = graph_kernel_nodes(g, &kernels);
  if (e != cudaSuccess) { cudaGraphDestroy(g); return cuda_fail(s, e, "graph nodes"); }
  s->day_graph_kernels = kernels;
  e = cudaGraphInstantiate(&s->day_graph, g, 0);
  cudaGraphDestroy(g);
  if (e != cudaSuccess) { s->day_graph = nullptr; return cuda_fail(s, e, "graph instantiate"); }
  return SAMPO_OK;
}

static void drop_day_graph(sampo_sim* s) {
  if (s->day_graph) {
    cudaGraphExecDestroy(s->day_graph);
    s->day_graph = nullptr;
  }
}

// A day on grid bucket b: one launch of 24 one-launch steps, cooperative
// where a graph takes a cooperative launch, else a plain launch of the same
// co-resident grid (its grid barriers are bounded either way).
static cudaError_t build_small_graph(sampo_sim* s, int items, int b) {
  const KParams p = make_params(s);
  const int grid = (int)small_bucket_grid(s, b);
  const int ti = items == 1 ? 0 : items == 2 ? 1 : 2;
  cudaError_t e = cudaErrorUnknown;
  for (int kind : {DG_SMALL_COOP, DG_SMALL}) {
    cudaGraph_t g = nullptr;
    e = cudaStreamBeginCapture(s->stream, cudaStreamCaptureModeThreadLocal);
    if (e != cudaSuccess) break;
    e = launch_small(p, grid, kind == DG_SMALL_COOP, 24u, s->stream, items);
    const cudaError_t e2 = cudaStreamEndCapture(s->stream, &g);
    if (e == cudaSuccess) e = e2;
    if (e == cudaSuccess) e = cudaGraphInstantiate(&s->small_graph[ti][b], g, 0);
    if (g) cudaGraphDestroy(g);
    if (e == cudaSuccess) {
      s->small_graph_kind[ti][b] = kind;
      return cudaSuccess;
    }
    s->small_graph[ti][b] = nullptr;
    (void)cudaGetLastError();
  }
  return e;
}

// The graph of the coming day and its kernel launches: the one-launch step
// (grid of at least kSmallGrowth CTAs per tile of the pool end last seen)
// when that pool has at most small_tiles 1024-slot tiles, else the
// three-kernel step. The one-launch step takes the smallest tiles (the
// shortest chain of updates per thread: 256, then 512, then 1024 slots) the
// largest grid has room for. Any pick gives the same results at any size: a
// pool that outgrew its pick is stepped by the one-launch kernel's
// extra-tile route.
static int day_graph_for(sampo_sim* s, cudaGraphExec_t* gx, uint32_t* kernels, int* kind) {
  const uint32_t end = s->known_end;
  const uint32_t t4 = (end + kTile - 1) / kTile;
  if (!s->species && s->small_grid > 0 && s->small_tiles > 0 && t4 <= s->small_tiles) {
    auto tiles_of = [&](int items) { const uint32_t t = (end + kBlock * items - 1) / (kBlock * items); return t ? t : 1u; };
    int items = s->small_items;
    if (items == 0) {
      items = 4;
      for (int i : {2, 1})
        if ((uint64_t)tiles_of(i) * kSmallGrowth <= (uint64_t)s->small_grid) items = i;
    }
    const uint64_t want = (uint64_t)tiles_of(items) * kSmallGrowth;
    const int ti = items == 1 ? 0 : items == 2 ? 1 : 2;
    int b = 0;
    while (b + 1 < kSmallBuckets && small_bucket_grid(s, b) < want) b++;
    if (s->small_graph[ti][b] || build_small_graph(s, items, b) == cudaSuccess) {
      *gx = s->small_graph[ti][b];
      *kernels = 1;
      *kind = s->small_graph_kind[ti][b];
      return SAMPO_OK;
    }
  }
  int rc = build_day_graph(s);
  if (rc) return rc;
  *gx = s->day_graph;
  *kernels = s->day_graph_kernels;
  *kind = DG_PLAIN;
  return SAMPO_OK;
}

extern "C" int sampo_set_small_step(sampo_sim* s, uint32_t max_tiles) {
  if (!s) return SAMPO_ERR_ARG;
  SETTLE(s);
  if (max_tiles == SAMPO_SMALL_STEP_DEFAULT) max_tiles = s->small_grid > 0 ? (uint32_t)s->small_grid : 0u;
  s->small_tiles = max_tiles;
  return SAMPO_OK;
}

extern "C" int sampo_set_small_step_items(sampo_sim* s, uint32_t items) {
  if (!s) return SAMPO_ERR_ARG;
  if (items != 0 && items != 1 && items != 2 && items != 4)
    return fail(s, SAMPO_ERR_ARG, "slots per thread of the one-launch step: 0, 1, 2 or 4");
  SETTLE(s);
  s->small_items = (int)items;
  return SAMPO_OK;
}

extern "C" int sampo_small_step_info(sampo_sim* s, uint32_t* grid, uint32_t* max_tiles, int* last_day_kind,
                                     uint64_t* days_one_launch, uint64_t* days_three_kernel) {
  if (!s) return SAMPO_ERR_ARG;
  if (grid) *grid = (uint32_t)s->small_grid;
  if (max_tiles) *max_tiles = s->small_tiles;
  if (last_day_kind) *last_day_kind = s->last_day_kind;
  if (days_one_launch) *days_one_launch = s->days_small;
  if (days_three_kernel) *days_three_kernel = s->days_three;
  return SAMPO_OK;
}

extern "C" int sampo_set_timing(sampo_sim* s, int on) {
  if (!s) return SAMPO_ERR_ARG;
  SETTLE(s);
  s->timing = on != 0;
  s->t_count = s->t_scatter = s->t_total = 0;
  s->launches = 0;
  s->days_small = s->days_three = 0;
  return SAMPO_OK;
}

// Queues nsteps steps and the copies of their rows on the simulation's
// stream. With wait, the device status is checked after every chunk of
// ring - 1 steps (a synchronisation) and the device time is summed per chunk;
// without, the run is left pending for sampo_sync, which checks the status
// once and times the whole queue.
static int queue_run(sampo_sim* s, uint32_t nsteps, sampo_stats_row* rows, bool wait) {
  if (!s->have_pop) return fail(s, SAMPO_ERR_STATE, "no population: call sampo_init_population or sampo_load_pool");
  if (nsteps == 0) return SAMPO_OK;
  cudaSetDevice(s->device);
  for (uint32_t i = 0; i < nsteps; i++) {
    uint32_t st = s->step + i, slot = st % s->ring;
    if (!s->have_inputs[slot] || s->input_step[slot] != st) return fail(s, SAMPO_ERR_STATE, "no inputs for step " + std::to_string(st));
    if (s->seed_step[slot] != st) return fail(s, SAMPO_ERR_STATE, "no seeds for step " + std::to_string(st));
  }
  KParams p = make_params(s);
  CK(launch_publish(p, PUB_REFRESH, s->stream), "step constants");  // inputs may postdate the last publish
  s->launches += 1;
  uint32_t done = 0;
  // rows of steps [s->step, s->step + n) are read back in chunks no longer than the ring allows
  const uint32_t chunk_max = s->ring - 1;
  if (wait || !s->pending) {
    s->last_run_ms = 0;
    CK(cudaEventRecord(s->ev[3], s->stream), "event");
  }
  s->pending = !wait;
  while (done < nsteps) {
    if (wait && done) CK(cudaEventRecord(s->ev[3], s->stream), "event");
    const uint32_t n = std::min(nsteps - done, chunk_max);
    const uint32_t first = s->step;
    if (s->timing) {
      for (uint32_t i = 0; i < n; i++) {
        CK(cudaEventRecord(s->ev[0], s->stream), "event");
        CK(launch_count(p, s->grid_count, s->stream, s->items), "count kernel");
        CK(cudaEventRecord(s->ev[1], s->stream), "event");
        CK(launch_scatter(p, s->grid_scatter, s->stream, s->items), "scatter kernel");
        CK(cudaEventRecord(s->ev[2], s->stream), "event");
        CK(launch_publish(p, PUB_AFTER_STEP, s->stream), "publish kernel");
        CK(cudaEventRecord(s->ev[4], s->stream), "event");
        CK(cudaEventSynchronize(s->ev[4]), "event");
        float a = 0, b = 0, c = 0;
        cudaEventElapsedTime(&a, s->ev[0], s->ev[1]);
        cudaEventElapsedTime(&b, s->ev[1], s->ev[2]);
        cudaEventElapsedTime(&c, s->ev[2], s->ev[4]);
        s->t_count += a; s->t_scatter += b; s->t_total += a + b + c;
        s->launches += 3;
      }
    } else {
      uint32_t i = 0;
      // with the one-launch step available, a waiting run learns the pool end
      // after each day one day behind the queue (the GPU keeps the next day
      // queued meanwhile) and picks each day's graph from it
      const bool track = wait && !s->species && s->small_grid > 0 && s->small_tiles > 0;
      for (uint32_t day = 0; i + 24 <= n; i += 24, day++) {
        cudaGraphExec_t gx = nullptr;
        uint32_t kernels = 0;
        int kind = 0;
        int rc = day_graph_for(s, &gx, &kernels, &kind);
        if (rc) return rc;
        CK(cudaGraphLaunch(gx, s->stream), "day graph");
        s->launches += kernels;
        s->last_day_kind = kind;
        (kind == DG_PLAIN ? s->days_three : s->days_small) += 1;
        if (track) {
          const uint32_t k = day & 1u;
          CK(cudaMemcpyAsync(&s->end_pinned[k], &s->sim_dev->pop.r[GRAVID].end, sizeof(uint32_t), cudaMemcpyDeviceToHost,
                             s->stream), "pool end");
          CK(cudaEventRecord(s->ev_day[k], s->stream), "event");
          if (day >= 1) {
            CK(cudaEventSynchronize(s->ev_day[k ^ 1u]), "event");
            s->known_end = s->end_pinned[k ^ 1u];
          }
        }
      }
      for (; i < n; i++) {
        CK(launch_step(s, p), "step kernels");
        s->launches += 3;
      }
    }
    CK(cudaEventRecord(s->ev[2], s->stream), "event");
    if (rows) {
      // rows[first .. first+n) live in ring slots first % ring ...
      uint32_t c = 0;
      while (c < n) {
        uint32_t slot = (first + c) % s->ring;
        uint32_t m = std::min(n - c, s->ring - slot);
        CK(cudaMemcpyAsync(rows + done + c, s->rows_dev + slot, (size_t)m * sizeof(sampo_stats_row), cudaMemcpyDeviceToHost, s->stream), "rows");
        c += m;
      }
    }
    s->step += n;
    done += n;
    if (!wait) continue;
    int rc = check_device(s);
    float ms = 0;
    cudaEventElapsedTime(&ms, s->ev[3], s->ev[2]);
    s->last_run_ms += ms;
    if (rc) return rc;
  }
  return SAMPO_OK;
}

extern "C" int sampo_sync(sampo_sim* s) {
  if (!s) return SAMPO_ERR_ARG;
  if (!s->pending) return SAMPO_OK;
  s->pending = false;
  cudaSetDevice(s->device);
  int rc = check_device(s);  // waits for the queued steps and row copies
  float ms = 0;
  if (cudaEventElapsedTime(&ms, s->ev[3], s->ev[2]) == cudaSuccess) s->last_run_ms = ms;
  return rc;
}

extern "C" int sampo_run(sampo_sim* s, uint32_t nsteps, sampo_stats_row* rows) {
  if (!s) return SAMPO_ERR_ARG;
  SETTLE(s);
  return queue_run(s, nsteps, rows, true);
}

extern "C" int sampo_run_async(sampo_sim* s, uint32_t nsteps, sampo_stats_row* rows) {
  if (!s) return SAMPO_ERR_ARG;
  if (s->timing) {  // per-kernel timing waits for every step
    SETTLE(s);
    return queue_run(s, nsteps, rows, true);
  }
  return queue_run(s, nsteps, rows, false);
}

extern "C" int sampo_last_run_ms(sampo_sim* s, double* ms) {
  if (!s || !ms) return SAMPO_ERR_ARG;
  SETTLE(s);
  *ms = s->last_run_ms;
  return SAMPO_OK;
}

extern "C" void* sampo_host_alloc(size_t bytes) {
  void* p = nullptr;
  if (cudaMallocHost(&p, bytes ? bytes : 1) != cudaSuccess) return nullptr;
  return p;
}

extern "C" void sampo_host_free(void* p) {
  if (p) cudaFreeHost(p);
}

extern "C" int sampo_flush_l2(sampo_sim* s) {
  if (!s) return SAMPO_ERR_ARG;
  SETTLE(s);
  cudaSetDevice(s->device);
  if (!s->flush_buf) {
    int l2 = 0;
    cudaDeviceGetAttribute(&l2, cudaDevAttrL2CacheSize, s->device);
    s->flush_bytes = std::max<size_t>((size_t)l2 * 2, (size_t)256 << 20);
    CK(cudaMalloc(&s->flush_buf, s->flush_bytes), "L2 flush buffer");
  }
  CK(cudaMemsetAsync(s->flush_buf, (int)(s->launches & 0xff), s->flush_bytes, s->stream), "L2 flush");
  return SAMPO_OK;
}

extern "C" int sampo_current_row(sampo_sim* s, sampo_stats_row* row) {
  if (!s || !row) return SAMPO_ERR_ARG;
  SETTLE(s);
  if (!s->have_pop) return fail(s, SAMPO_ERR_STATE, "no population");
  cudaSetDevice(s->device);
  CK(cudaMemcpyAsync(row, s->rows_dev + s->step % s->ring, sizeof(sampo_stats_row), cudaMemcpyDeviceToHost, s->stream), "row");
  CK(cudaStreamSynchronize(s->stream), "row");
  return SAMPO_OK;
}

extern "C" int sampo_get_step(sampo_sim* s, uint32_t* step) {
  if (!s || !step) return SAMPO_ERR_ARG;
  *step = s->step;
  return SAMPO_OK;
}

extern "C" int sampo_histogram(sampo_sim* s, uint32_t out[100]) {
  if (!s || !out) return SAMPO_ERR_ARG;
  SETTLE(s);
  if (!s->have_pop) return fail(s, SAMPO_ERR_STATE, "no population");
  cudaSetDevice(s->device);
  CK(cudaMemsetAsync(s->hist_dev, 0, 100 * sizeof(uint32_t), s->stream), "histogram");
  KParams p = make_params(s);
  CK(launch_histogram(p, s->hist_dev, s->stream), "histogram");
  CK(cudaMemcpyAsync(out, s->hist_dev, 100 * sizeof(uint32_t), cudaMemcpyDeviceToHost, s->stream), "histogram");
  CK(cudaStreamSynchronize(s->stream), "histogram");
  return SAMPO_OK;
}

extern "C" int sampo_read_pool(sampo_sim* s, sampo_population* pop, sampo_pool_view* v) {
  if (!s || !pop) return SAMPO_ERR_ARG;
  SETTLE(s);
  if (!s->have_pop) return fail(s, SAMPO_ERR_STATE, "no population");
  cudaSetDevice(s->device);
  SimDev h;
  CK(cudaMemcpyAsync(&h, s->sim_dev, sizeof(SimDev), cudaMemcpyDeviceToHost, s->stream), "state");
  CK(cudaStreamSynchronize(s->stream), "state");
  *pop = h.pop;
  if (!v) return SAMPO_OK;
  const uint32_t n = h.pop.r[7].end;
  const DevPool& P = s->pool[h.cur & 1u];
  const size_t b4 = (size_t)n * 4;
  CK(cudaMemcpyAsync(v->ageInHours, P.age, b4, cudaMemcpyDeviceToHost, s->stream), "pool read");
  CK(cudaMemcpyAsync(v->hoursInState, P.his, b4, cudaMemcpyDeviceToHost, s->stream), "pool read");
  CK(cudaMemcpyAsync(v->delay, P.delay, b4, cudaMemcpyDeviceToHost, s->stream), "pool read");
  CK(cudaMemcpyAsync(v->cumulativeSporogonicDevelopment, P.sporo, b4, cudaMemcpyDeviceToHost, s->stream), "pool read");
  CK(cudaMemcpyAsync(v->larvalDelayOrOviAttempts, P.uni, b4, cudaMemcpyDeviceToHost, s->stream), "pool read");
  CK(cudaMemcpyAsync(v->availableEggs, P.avail, b4, cudaMemcpyDeviceToHost, s->stream), "pool read");
  CK(cudaMemcpyAsync(v->cycleLength, P.cycle, b4, cudaMemcpyDeviceToHost, s->stream), "pool read");
  CK(cudaMemcpyAsync(v->humanBloodmealCount, P.hbc, b4, cudaMemcpyDeviceToHost, s->stream), "pool read");
  CK(cudaMemcpyAsync(v->numEggBatches, P.batches, b4, cudaMemcpyDeviceToHost, s->stream), "pool read");
  std::vector<uint8_t> flags(n);
  CK(cudaMemcpyAsync(flags.data(), P.flags, n, cudaMemcpyDeviceToHost, s->stream), "pool read");
  CK(cudaStreamSynchronize(s->stream), "pool read");
  for (uint32_t i = 0; i < n; i++) {
    v->state[i] = flags[i] & 7u;
    v->isFemale[i] = (flags[i] >> 3) & 1u;
  }
  return SAMPO_OK;
}

// ---- checkpoints: "SAMPOCK1", u32 version, u32 step, f32 cc, population,
//      bites/cycles, u32 n, u32 0, then nine columns of n 4-byte values and
//      the n flag bytes (state | isFemale << 3) ----
extern "C" int sampo_checkpoint_save(sampo_sim* s, const char* path) {
  if (!s || !path) return SAMPO_ERR_ARG;
  SETTLE(s);
  if (!s->have_pop) return fail(s, SAMPO_ERR_STATE, "no population");
  cudaSetDevice(s->device);
  SimDev h;
  CK(cudaMemcpyAsync(&h, s->sim_dev, sizeof(SimDev), cudaMemcpyDeviceToHost, s->stream), "state");
  CkHeader hd;
  memset(&hd, 0, sizeof(hd));
  memcpy(hd.magic, kCkMagic, 8);
  hd.version = 2;
  hd.step = h.step;
  hd.cc = s->cc;
  hd.pop = h.pop;
  hd.bnc = h.bnc;
  hd.n = h.pop.r[7].end;
  if (h.step > 0) {  // the previous step's row is still in the ring
    sampo_stats_row prev;
    CK(cudaMemcpyAsync(&prev, s->rows_dev + (h.step - 1) % s->ring, sizeof(prev), cudaMemcpyDeviceToHost, s->stream), "rows");
    CK(cudaStreamSynchronize(s->stream), "rows");
    hd.prev = prev.pop;
    hd.flags |= CK_PREV;
  }
  CK(cudaStreamSynchronize(s->stream), "state");
  const std::string err = ck_write(path, hd, s->pool[h.cur & 1u]);
  if (!err.empty()) return fail(s, SAMPO_ERR_IO, err);
  return SAMPO_OK;
}

extern "C" int sampo_checkpoint_info(const char* path, uint32_t* step, sampo_population* pop, sampo_population* prev,
                                     int* has_prev) {
  if (!path) return SAMPO_ERR_ARG;
  CkHeader hd;
  FILE* f = nullptr;
  if (!ck_open(path, hd, &f).empty()) return SAMPO_ERR_IO;
  fclose(f);
  if (step) *step = hd.step;
  if (pop) *pop = hd.pop;
  if (prev) *prev = hd.prev;
  if (has_prev) *has_prev = (hd.flags & CK_PREV) ? 1 : 0;
  return SAMPO_OK;
}

extern "C" int sampo_checkpoint_load(sampo_sim* s, const char* path) {
  if (!s || !path) return SAMPO_ERR_ARG;
  SETTLE(s);
  CkHeader hd;
  FILE* f = nullptr;
  const std::string err = ck_open(path, hd, &f);
  if (!err.empty()) return fail(s, SAMPO_ERR_IO, err);
  if (hd.cc != s->cc) { fclose(f); return fail(s, SAMPO_ERR_ARG, "checkpoint carrying capacity differs from the handle's"); }
  if ((uint64_t)hd.n > s->capacity) { fclose(f); return fail(s, SAMPO_ERR_CAPACITY, "checkpoint pool exceeds the capacity"); }
  if (const char* why = ranges_error(hd.pop, s->capacity)) {
    fclose(f);
    return fail(s, SAMPO_ERR_IO, std::string("inconsistent checkpoint (") + why + "): " + path);
  }
  cudaSetDevice(s->device);
  // the columns are copied on the legacy stream: nothing of this handle may
  // still run on its own stream
  const cudaError_t se = cudaStreamSynchronize(s->stream);
  if (se != cudaSuccess) {
    fclose(f);
    return cuda_fail(s, se, "checkpoint");
  }
  const std::string rerr = ck_read_pool(f, hd, s->pool[0]);
  if (!rerr.empty()) return fail(s, SAMPO_ERR_IO, rerr + ": " + path);
  // the state as a step boundary left it: step, ranges, the counters the next
  // row reports; the statistics and step constants are recomputed
  SimDev h = s->host_state;
  h.pop = hd.pop;
  h.pop.numLarvae1DayEquiv = h.pop.numFemale = h.pop.numPotentiallyInfective = 0;
  h.bnc = hd.bnc;
  h.step = hd.step;
  h.active = 1;
  CK(cudaMemsetAsync(s->tile_mem, 0, tile_array_words(s->max_tiles) * 4, s->stream), "tile reset");
  CK(cudaMemcpyAsync(s->sim_dev, &h, sizeof(SimDev), cudaMemcpyHostToDevice, s->stream), "state");
  s->step = hd.step;
  const int rc = publish_initial(s);
  if (rc) return rc;
  sampo_population p;
  SimDev back;
  CK(cudaMemcpyAsync(&back, s->sim_dev, sizeof(SimDev), cudaMemcpyDeviceToHost, s->stream), "state");
  CK(cudaStreamSynchronize(s->stream), "state");
  p = back.pop;
  if (p.numLarvae1DayEquiv != hd.pop.numLarvae1DayEquiv || p.numFemale != hd.pop.numFemale ||
      p.numPotentiallyInfective != hd.pop.numPotentiallyInfective)
    return fail(s, SAMPO_ERR_INTERNAL, "checkpoint statistics do not match its pool");
  return SAMPO_OK;
}

extern "C" int sampo_autotune(sampo_sim* s, uint32_t* count_ctas_per_sm, uint32_t* scatter_ctas_per_sm) {
  if (!s) return SAMPO_ERR_ARG;
  SETTLE(s);
  if (!s->have_pop) return fail(s, SAMPO_ERR_STATE, "no population");
  const uint32_t slot = s->step % s->ring;
  if (!s->have_inputs[slot] || s->input_step[slot] != s->step || s->seed_step[slot] != s->step)
    return fail(s, SAMPO_ERR_STATE, "no inputs or seeds for the coming step");
  cudaSetDevice(s->device);
  const KParams p = make_params(s);
  CK(launch_publish(p, PUB_REFRESH, s->stream), "step constants");
  int gc = 0, gs = 0, items = kItems;
  CK(tune_grids(p, s->stream, &gc, &gs, &items, nullptr), "autotune");
  int sms = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, s->device);
  if (sms <= 0) sms = 1;
  if (gc != s->grid_count || gs != s->grid_scatter || items != s->items) {
    s->grid_count = gc;
    s->grid_scatter = gs;
    s->items = items;
    drop_day_graph(s);  // captured with the old grids
  }
  if (count_ctas_per_sm) *count_ctas_per_sm = (uint32_t)(gc / sms);
  if (scatter_ctas_per_sm) *scatter_ctas_per_sm = (uint32_t)(gs / sms);
  return check_device(s);
}

extern "C" int sampo_set_species(sampo_sim* s, const sampo_species* sp) {
  if (!s) return SAMPO_ERR_ARG;
  SETTLE(s);
  if (sp && sampo_species_device(sp) != s->device) return fail(s, SAMPO_ERR_ARG, "species compiled for another device");
  cudaSetDevice(s->device);
  if (s->species == sp) return SAMPO_OK;
  s->species = sp;
  if (sp) s->items = kItems;  // a run-time species is built for 4 slots per thread
  s->grid_count = grid_blocks_count(1, sp, s->items);
  s->grid_scatter = grid_blocks_scatter(1, sp, s->items);
  drop_day_graph(s);  // captured with the other kernels
  return SAMPO_OK;
}

extern "C" int sampo_set_grids(sampo_sim* s, uint32_t count_ctas_per_sm, uint32_t scatter_ctas_per_sm) {
  if (!s) return SAMPO_ERR_ARG;
  SETTLE(s);
  cudaSetDevice(s->device);
  int sms = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, s->device);
  if (sms <= 0) sms = 1;
  const uint32_t max_c = (uint32_t)(grid_blocks_count(1, s->species, s->items) / sms);
  const uint32_t max_s = (uint32_t)(grid_blocks_scatter(1, s->species, s->items) / sms);
  if (count_ctas_per_sm < 1 || count_ctas_per_sm > max_c || scatter_ctas_per_sm < 1 || scatter_ctas_per_sm > max_s)
    return fail(s, SAMPO_ERR_ARG, "CTAs per SM outside 1.." + std::to_string(max_c) + " (count) / 1.." + std::to_string(max_s) +
                                      " (update/scatter)");
  const int gc = (int)count_ctas_per_sm * sms, gs = (int)scatter_ctas_per_sm * sms;
  if (gc != s->grid_count || gs != s->grid_scatter) {
    s->grid_count = gc;
    s->grid_scatter = gs;
    drop_day_graph(s);  // captured with the old grids
  }
  return SAMPO_OK;
}

extern "C" int sampo_set_items_per_thread(sampo_sim* s, uint32_t items) {
  if (!s) return SAMPO_ERR_ARG;
  SETTLE(s);
  if (items != 2 && items != 4) return fail(s, SAMPO_ERR_ARG, "items per thread must be 2 or 4");
  if (s->species && items != (uint32_t)kItems) return fail(s, SAMPO_ERR_ARG, "a run-time species runs 4 items per thread");
  cudaSetDevice(s->device);
  if ((int)items != s->items) {
    s->items = (int)items;
    s->grid_count = grid_blocks_count(1, s->species, s->items);
    s->grid_scatter = grid_blocks_scatter(1, s->species, s->items);
    drop_day_graph(s);
  }
  return SAMPO_OK;
}

extern "C" int sampo_items_per_thread(sampo_sim* s, uint32_t* items) {
  if (!s || !items) return SAMPO_ERR_ARG;
  *items = (uint32_t)s->items;
  return SAMPO_OK;
}

extern "C" int sampo_device_status(sampo_sim* s, uint32_t* bits, int clear) {
  if (!s || !bits) return SAMPO_ERR_ARG;
  if (s->pending) (void)sampo_sync(s);  // the bits below include the queued steps
  cudaSetDevice(s->device);
  uint32_t st[2];
  CK(cudaMemcpyAsync(st, &s->sim_dev->error, 2 * sizeof(uint32_t), cudaMemcpyDeviceToHost, s->stream), "status");
  CK(cudaStreamSynchronize(s->stream), "status");
  *bits = st[0] | st[1];
  if (clear) {
    uint32_t z[2] = {0, 0};
    CK(cudaMemcpyAsync(&s->sim_dev->error, z, sizeof(z), cudaMemcpyHostToDevice, s->stream), "status");
    CK(cudaStreamSynchronize(s->stream), "status");
  }
  return SAMPO_OK;
}

extern "C" int sampo_kernel_times(sampo_sim* s, double out[3], uint64_t* launches) {
  if (!s || !out) return SAMPO_ERR_ARG;
  SETTLE(s);
  out[0] = s->t_count; out[1] = s->t_scatter; out[2] = s->t_total;
  if (launches) *launches = s->launches;
  return SAMPO_OK;
}

extern "C" int sampo_eval_math(int fn, const float* x, const float* y, float* out, uint32_t n, int device) {
  if (!x || !out || fn < 0 || fn > 5 || (fn == 3 && !y)) return SAMPO_ERR_ARG;
  if (n == 0) return SAMPO_OK;
  sampo_sim* s = nullptr;  // CK() reports through a null handle
  CK(cudaSetDevice(device), "device");
  float *dx = nullptr, *dy = nullptr, *dout = nullptr;
  CK(cudaMalloc(&dx, (size_t)n * 4 * 3), "eval buffers");
  dy = dx + n;
  dout = dx + 2 * (size_t)n;
  cudaError_t e = cudaMemcpy(dx, x, (size_t)n * 4, cudaMemcpyHostToDevice);
  if (e == cudaSuccess && y) e = cudaMemcpy(dy, y, (size_t)n * 4, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = launch_eval_math(fn, dx, dy, dout, n, 0);
  if (e == cudaSuccess) e = cudaMemcpy(out, dout, (size_t)n * 4, cudaMemcpyDeviceToHost);
  cudaFree(dx);
  return e == cudaSuccess ? SAMPO_OK : SAMPO_ERR_CUDA;
}
