// sampo_batch.cu - host side of the batch C ABI (sampo_batch_* in
// include/sampo.h): many independent simulations stepped by the same kernels.
//
// The batch owns, on one GPU and one stream:
//   * a SimDev per slot and the RepParams array the kernels walk (fixed
//     addresses, so a captured day graph stays valid while slots change);
//   * per used slot, one stream-ordered allocation from the batch's memory
//     pool holding the two pool buffers, the look-back tile arrays and the
//     rings of inputs and stats rows.
// A slot's replicate is bit-identical to the same simulation run alone: the
// kernels index its RNG by its own slots and its own step.
#include <cuda_runtime.h>
#include <string.h>
#include <algorithm>
#include <string>
#include <vector>
#include "sampo_model.cuh"
#include "sampo_kernels.cuh"
#include "sampo_checkpoint.cuh"

using namespace sampo;

namespace {

size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

// Byte layout of one replicate's allocation.
struct RepLayout {
  size_t col4, col1, pool, tiles, T, env, seeds, wt, rows, total;
  uint32_t max_tiles;
  RepLayout(uint64_t capacity, uint32_t ring) {
    // 16 bytes of slack per column: tile copies round up to 16 bytes
    col4 = align256(capacity * 4 + 16);
    col1 = align256(capacity + 16);
    pool = 9 * col4 + col1;
    max_tiles = (uint32_t)((capacity + kTileMin - 1) / kTileMin);  // room for the smaller tile's count
    tiles = align256(tile_array_words(max_tiles) * 4);
    T = align256((size_t)ring * sizeof(float));
    env = align256((size_t)ring * sizeof(sampo_environment));
    seeds = align256((size_t)ring * 4 * sizeof(sampo_seeds));
    wt = align256((size_t)ring * sizeof(uint32_t));
    rows = align256((size_t)ring * sizeof(sampo_stats_row));
    total = 2 * pool + tiles + T + env + seeds + wt + rows;
  }
};

struct Replicate {
  bool used = false;
  bool have_pop = false;
  bool active = false;         // host mirror of SimDev::active
  uint32_t step = 0;           // host mirror of SimDev::step
  uint32_t stop_step = 0xffffffffu;
  uint64_t capacity = 0;
  float cc = 0.0f;
  void* mem = nullptr;
  RepParams rp;                // host copy of the kernels' view
  std::vector<uint32_t> input_step, seed_step;  // per ring slot: absolute step held
  bool dev_seeds = false;      // seeds drawn on the device (sampo_batch_seed_stream)
  std::vector<float> T_host;
};

}  // namespace

struct sampo_batch {
  int device = 0;
  const void* species = nullptr;     // kernels compiled for a user species, or null (built in)
  cudaStream_t stream = nullptr;
  cudaMemPool_t mempool = nullptr;
  uint32_t nslots = 0, ring = 0;
  SimDev* sims_dev = nullptr;
  RepParams* reps_dev = nullptr;
  BatchDev* bat_dev = nullptr;
  ModelConst* mc_dev = nullptr;
  sampo_seeds* init_seeds_dev = nullptr;  // [nslots][4]
  uint32_t* hist_dev = nullptr;
  std::vector<Replicate> reps;
  std::vector<uint32_t> wt_staging;
  int grid_count = 0, grid_scatter = 0;
  int items = kItems;                // slots per thread of the count and update/scatter passes (2 or 4)
  cudaGraphExec_t day_graph = nullptr;
  uint32_t day_graph_kernels = 0;    // kernel nodes of day_graph
  uint64_t launches = 0;             // kernels sampo_batch_run launched
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  bool timed = false;
  std::string err;
};

static int bfail(sampo_batch* b, int code, const std::string& msg) {
  if (b) b->err = msg;
  return code;
}
#define BCK(call, what)                                                                             \
  do {                                                                                              \
    cudaError_t e_ = (call);                                                                        \
    if (e_ != cudaSuccess) return bfail(b, SAMPO_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e_)); \
  } while (0)

static KParams all_params(sampo_batch* b) {
  KParams p;
  p.reps = b->reps_dev;
  p.nrep = b->nslots;
  p.bat = b->bat_dev;
  p.mc = b->mc_dev;
  p.ks = b->species;
  return p;
}
static KParams slot_params(sampo_batch* b, uint32_t slot) {
  KParams p = all_params(b);
  p.reps = b->reps_dev + slot;
  p.nrep = 1;
  return p;
}

static Replicate* get_slot(sampo_batch* b, uint32_t slot) {
  if (!b || slot >= b->nslots || !b->reps[slot].used) return nullptr;
  return &b->reps[slot];
}

extern "C" uint64_t sampo_batch_replicate_bytes(uint64_t capacity, uint32_t ring_steps) {
  return RepLayout(capacity, ring_steps).total;
}

extern "C" const char* sampo_batch_last_error(const sampo_batch* b) { return b ? b->err.c_str() : "null handle"; }

extern "C" int sampo_batch_destroy(sampo_batch* b) {
  if (!b) return SAMPO_OK;
  cudaSetDevice(b->device);
  if (b->stream) cudaStreamSynchronize(b->stream);
  if (b->day_graph) cudaGraphExecDestroy(b->day_graph);
  for (auto& r : b->reps)
    if (r.mem) cudaFreeAsync(r.mem, b->stream);
  if (b->stream) cudaStreamSynchronize(b->stream);
  cudaFree(b->sims_dev); cudaFree(b->reps_dev); cudaFree(b->bat_dev); cudaFree(b->mc_dev);
  cudaFree(b->init_seeds_dev); cudaFree(b->hist_dev);
  if (b->ev0) cudaEventDestroy(b->ev0);
  if (b->ev1) cudaEventDestroy(b->ev1);
  if (b->mempool) cudaMemPoolDestroy(b->mempool);
  if (b->stream) cudaStreamDestroy(b->stream);
  delete b;
  return SAMPO_OK;
}

extern "C" int sampo_batch_create(const sampo_batch_config* cfg, sampo_batch** out) {
  if (!cfg || !out) return SAMPO_ERR_ARG;
  *out = nullptr;
  if (cfg->max_replicates == 0 || cfg->max_replicates > SAMPO_BATCH_MAX_REPLICATES || cfg->ring_steps < 2) return SAMPO_ERR_ARG;
  static_assert(SAMPO_BATCH_MAX_REPLICATES <= kMaxRep, "the kernels plan at most kMaxRep replicates");
  sampo_batch* b = new sampo_batch();
  b->device = cfg->device;
  b->nslots = cfg->max_replicates;
  b->ring = cfg->ring_steps;
  b->reps.resize(b->nslots);
  int rc = SAMPO_OK;
  do {
    cudaError_t e;
    if ((e = cudaSetDevice(b->device)) != cudaSuccess ||
        (e = cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking)) != cudaSuccess) {
      rc = bfail(b, SAMPO_ERR_CUDA, std::string("device: ") + cudaGetErrorString(e));
      break;
    }
    cudaMemPoolProps props;
    memset(&props, 0, sizeof(props));
    props.allocType = cudaMemAllocationTypePinned;
    props.location.type = cudaMemLocationTypeDevice;
    props.location.id = b->device;
    if ((e = cudaMemPoolCreate(&b->mempool, &props)) != cudaSuccess) {
      rc = bfail(b, SAMPO_ERR_CUDA, std::string("memory pool: ") + cudaGetErrorString(e));
      break;
    }
    uint64_t keep = ~0ull;  // freed pools stay reserved for the next replicates
    cudaMemPoolSetAttribute(b->mempool, cudaMemPoolAttrReleaseThreshold, &keep);
    const size_t n = b->nslots;
    if ((e = cudaMalloc(&b->sims_dev, n * sizeof(SimDev))) != cudaSuccess ||
        (e = cudaMalloc(&b->reps_dev, n * sizeof(RepParams))) != cudaSuccess ||
        (e = cudaMalloc(&b->bat_dev, sizeof(BatchDev))) != cudaSuccess ||
        (e = cudaMalloc(&b->mc_dev, sizeof(ModelConst))) != cudaSuccess ||
        (e = cudaMalloc(&b->init_seeds_dev, n * 4 * sizeof(sampo_seeds))) != cudaSuccess ||
        (e = cudaMalloc(&b->hist_dev, 100 * sizeof(uint32_t))) != cudaSuccess) {
      rc = bfail(b, SAMPO_ERR_CUDA, std::string("batch state: ") + cudaGetErrorString(e));
      break;
    }
    std::vector<SimDev> sims(n, initial_sim_state(0, 1.0f));
    std::vector<RepParams> rps(n);
    memset(rps.data(), 0, n * sizeof(RepParams));
    for (size_t i = 0; i < n; i++) {
      rps[i].sim = b->sims_dev + i;  // empty slots: inactive state, no buffers
      rps[i].ring = b->ring;
      b->reps[i].rp = rps[i];
    }
    ModelConst mc;
    fill_constant_tables(mc);
    if ((e = cudaMemcpyAsync(b->sims_dev, sims.data(), n * sizeof(SimDev), cudaMemcpyHostToDevice, b->stream)) != cudaSuccess ||
        (e = cudaMemcpyAsync(b->reps_dev, rps.data(), n * sizeof(RepParams), cudaMemcpyHostToDevice, b->stream)) != cudaSuccess ||
        (e = cudaMemcpyAsync(b->mc_dev, &mc, sizeof(mc), cudaMemcpyHostToDevice, b->stream)) != cudaSuccess ||
        (e = cudaMemsetAsync(b->bat_dev, 0, sizeof(BatchDev), b->stream)) != cudaSuccess ||
        (e = cudaStreamSynchronize(b->stream)) != cudaSuccess) {
      rc = bfail(b, SAMPO_ERR_CUDA, std::string("batch upload: ") + cudaGetErrorString(e));
      break;
    }
    b->grid_count = grid_blocks_count(b->nslots);
    b->grid_scatter = grid_blocks_scatter(b->nslots);
    cudaEventCreate(&b->ev0);
    cudaEventCreate(&b->ev1);
  } while (0);
  if (rc) {
    sampo_batch_destroy(b);
    return rc;
  }
  *out = b;
  return SAMPO_OK;
}

// The kernels' view of one replicate's allocation `mem` (layout L).
static RepParams carve(const RepLayout& L, void* mem, SimDev* sim, uint32_t ring) {
  RepParams rp;
  memset(&rp, 0, sizeof(rp));
  char* m = (char*)mem;
  rp.sim = sim;
  for (int k = 0; k < 2; k++) {
    char* q = m + k * L.pool;
    DevPool& P = rp.pool[k];
    P.age = (float*)(q + 0 * L.col4); P.his = (float*)(q + 1 * L.col4); P.delay = (float*)(q + 2 * L.col4);
    P.sporo = (float*)(q + 3 * L.col4); P.uni = (uint32_t*)(q + 4 * L.col4); P.avail = (uint32_t*)(q + 5 * L.col4);
    P.cycle = (uint32_t*)(q + 6 * L.col4); P.hbc = (uint32_t*)(q + 7 * L.col4); P.batches = (uint32_t*)(q + 8 * L.col4);
    P.flags = (uint8_t*)(q + 9 * L.col4);
  }
  char* q = m + 2 * L.pool;
  set_tile_arrays(rp, (uint32_t*)q, L.max_tiles);
  q += L.tiles;
  rp.T = (const float*)q; q += L.T;
  rp.env = (const sampo_environment*)q; q += L.env;
  rp.seeds = (sampo_seeds*)q; q += L.seeds;
  rp.wt = (const uint32_t*)q; q += L.wt;
  rp.rows = (sampo_stats_row*)q;
  rp.ring = ring;
  return rp;
}

// The device state of every slot up to its step constants (one strided copy).
static int read_headers(sampo_batch* b, std::vector<SimDev>& h) {
  h.resize(b->nslots);
  BCK(cudaMemcpy2DAsync(h.data(), sizeof(SimDev), b->sims_dev, sizeof(SimDev), offsetof(SimDev, ctx), b->nslots,
                        cudaMemcpyDeviceToHost, b->stream), "slot states");
  BCK(cudaStreamSynchronize(b->stream), "slot states");
  return SAMPO_OK;
}

// The host mirrors of the replicates' steps and activity from the device (a
// replicate that paused for capacity did not advance).
static int refresh_mirrors(sampo_batch* b) {
  std::vector<SimDev> h;
  const int rc = read_headers(b, h);
  if (rc) return rc;
  for (uint32_t i = 0; i < b->nslots; i++) {
    Replicate& r = b->reps[i];
    if (!r.used || !r.have_pop) continue;
    r.step = h[i].step;
    r.active = h[i].active != 0;
  }
  return SAMPO_OK;
}

static int upload_slot(sampo_batch* b, uint32_t slot, const SimDev& h) {
  BCK(cudaMemcpyAsync(b->sims_dev + slot, &h, sizeof(SimDev), cudaMemcpyHostToDevice, b->stream), "slot state");
  BCK(cudaMemcpyAsync(b->reps_dev + slot, &b->reps[slot].rp, sizeof(RepParams), cudaMemcpyHostToDevice, b->stream), "slot params");
  return SAMPO_OK;
}

extern "C" int sampo_batch_add(sampo_batch* b, const sampo_replicate_config* rc, uint32_t* slot) {
  if (!b || !rc || !slot) return SAMPO_ERR_ARG;
  if (rc->capacity < 128 || rc->capacity > 0xFFFFFF00ull || !(rc->carrying_capacity > 0.0f)) return SAMPO_ERR_ARG;
  uint32_t i = 0;
  while (i < b->nslots && b->reps[i].used) i++;
  if (i == b->nslots) return bfail(b, SAMPO_ERR_CAPACITY, "no free slot in the batch");
  cudaSetDevice(b->device);
  const RepLayout L(rc->capacity, b->ring);
  void* mem = nullptr;
  cudaError_t e = cudaMallocFromPoolAsync(&mem, L.total, b->mempool, b->stream);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return bfail(b, SAMPO_ERR_CAPACITY, std::string("replicate buffers: ") + cudaGetErrorString(e));
  }
  Replicate& r = b->reps[i];
  r = Replicate();
  r.used = true;
  r.capacity = rc->capacity;
  r.cc = rc->carrying_capacity;
  r.stop_step = rc->stop_step;
  r.mem = mem;
  r.input_step.assign(b->ring, 0xffffffffu);
  r.seed_step.assign(b->ring, 0xffffffffu);
  r.T_host.assign(b->ring, 0.0f);
  RepParams& rp = r.rp;
  rp = carve(L, mem, b->sims_dev + i, b->ring);
  BCK(cudaMemsetAsync(rp.tilePre, 0, tile_array_words(L.max_tiles) * 4, b->stream), "tile arrays");
  SimDev h = initial_sim_state((uint32_t)rc->capacity, rc->carrying_capacity);
  h.stop_step = rc->stop_step;
  const int st = upload_slot(b, i, h);
  if (st) return st;
  *slot = i;
  return SAMPO_OK;
}

extern "C" int sampo_batch_remove(sampo_batch* b, uint32_t slot) {
  Replicate* r = get_slot(b, slot);
  if (!r) return SAMPO_ERR_ARG;
  cudaSetDevice(b->device);
  SimDev h = initial_sim_state(0, 1.0f);
  RepParams empty;
  memset(&empty, 0, sizeof(empty));
  empty.sim = b->sims_dev + slot;
  empty.ring = b->ring;
  void* mem = r->mem;
  *r = Replicate();
  r->rp = empty;
  const int st = upload_slot(b, slot, h);
  if (st) return st;
  BCK(cudaFreeAsync(mem, b->stream), "free replicate");
  return SAMPO_OK;
}

extern "C" int sampo_batch_set_inputs(sampo_batch* b, uint32_t slot, uint32_t first, const float* temperature,
                                      const sampo_environment* env, uint32_t nsteps) {
  Replicate* r = get_slot(b, slot);
  if (!r || !temperature || !env) return SAMPO_ERR_ARG;
  if (nsteps == 0 || nsteps > b->ring) return bfail(b, SAMPO_ERR_ARG, "nsteps exceeds the input ring");
  for (uint32_t i = 0; i < nsteps; i++)
    if (env[i].carryingCapacity != r->cc)
      return bfail(b, SAMPO_ERR_ARG, "environment carryingCapacity differs from the replicate's carrying capacity");
  cudaSetDevice(b->device);
  if (b->wt_staging.size() < nsteps) b->wt_staging.resize(nsteps);
  uint32_t done = 0;
  while (done < nsteps) {
    const uint32_t step = first + done, rs = step % b->ring;
    const uint32_t n = std::min(nsteps - done, b->ring - rs);
    for (uint32_t i = 0; i < n; i++) {
      b->wt_staging[done + i] = (step + i) % 24u;  // (UINT)(currentStep * hoursInTimeStep) % 24u, src/abms.c:514
      r->T_host[rs + i] = temperature[done + i];
      r->input_step[rs + i] = step + i;
    }
    BCK(cudaMemcpyAsync((float*)r->rp.T + rs, temperature + done, n * sizeof(float), cudaMemcpyHostToDevice, b->stream), "inputs");
    BCK(cudaMemcpyAsync((sampo_environment*)r->rp.env + rs, env + done, n * sizeof(sampo_environment), cudaMemcpyHostToDevice,
                        b->stream), "inputs");
    BCK(cudaMemcpyAsync((uint32_t*)r->rp.wt + rs, b->wt_staging.data() + done, n * sizeof(uint32_t), cudaMemcpyHostToDevice,
                        b->stream), "inputs");
    done += n;
  }
  BCK(cudaStreamSynchronize(b->stream), "inputs");  // wt_staging is reused
  return SAMPO_OK;
}

extern "C" int sampo_batch_set_seeds(sampo_batch* b, uint32_t slot, uint32_t first, const sampo_seeds* seeds, uint32_t nsteps) {
  Replicate* r = get_slot(b, slot);
  if (!r || !seeds) return SAMPO_ERR_ARG;
  if (nsteps == 0 || nsteps > b->ring) return bfail(b, SAMPO_ERR_ARG, "nsteps exceeds the seed ring");
  if (r->dev_seeds) return bfail(b, SAMPO_ERR_STATE, "the slot draws its seeds on the device");
  cudaSetDevice(b->device);
  uint32_t done = 0;
  while (done < nsteps) {
    const uint32_t step = first + done, rs = step % b->ring;
    const uint32_t n = std::min(nsteps - done, b->ring - rs);
    BCK(cudaMemcpyAsync((sampo_seeds*)r->rp.seeds + (size_t)rs * 4, seeds + (size_t)done * 4, (size_t)n * 4 * sizeof(sampo_seeds),
                        cudaMemcpyHostToDevice, b->stream), "seeds");
    for (uint32_t i = 0; i < n; i++) r->seed_step[rs + i] = step + i;
    done += n;
  }
  BCK(cudaStreamSynchronize(b->stream), "seeds");  // the caller may reuse its buffer on return
  return SAMPO_OK;
}

extern "C" int sampo_batch_init_population(sampo_batch* b, uint32_t slot, uint32_t n, const sampo_seeds init_seeds[4],
                                           int age_days_max, uint64_t age_seed) {
  Replicate* r = get_slot(b, slot);
  if (!r || !init_seeds) return SAMPO_ERR_ARG;
  if (r->input_step[0] != 0)
    return bfail(b, SAMPO_ERR_STATE, "set the inputs first: the initial eggs use temperature[0] (src/abms.c:198)");
  sampo_population pop;
  memset(&pop, 0, sizeof(pop));
  pop.r[0].end = n;
  for (int k = 1; k < 8; k++) {
    if (age_days_max < 0) {
      pop.r[k].start = n + 1; pop.r[k].end = n + 1;  // src/abms.c:204-219
    } else {
      pop.r[k].start = ((pop.r[k - 1].end + kLayoutAlign) / kLayoutAlign) * kLayoutAlign;
      pop.r[k].end = pop.r[k].start;
    }
  }
  if ((uint64_t)pop.r[7].end > r->capacity) return bfail(b, SAMPO_ERR_CAPACITY, "initial population exceeds the capacity");
  cudaSetDevice(b->device);
  SimDev h = initial_sim_state((uint32_t)r->capacity, r->cc);
  h.pop = pop;
  h.active = 1;
  h.stop_step = r->stop_step;
  const int st = upload_slot(b, slot, h);
  if (st) return st;
  BCK(cudaMemsetAsync(r->rp.tilePre, 0, tile_array_words(r->rp.maxTiles) * 4, b->stream), "tile arrays");
  BCK(cudaMemcpyAsync(b->init_seeds_dev + (size_t)slot * 4, init_seeds, 4 * sizeof(sampo_seeds), cudaMemcpyHostToDevice, b->stream),
      "seeds");
  const KParams p = slot_params(b, slot);
  BCK(launch_init_eggs(p, n, r->T_host[0], b->init_seeds_dev + (size_t)slot * 4, age_days_max, age_seed, b->stream), "initAgents");
  BCK(launch_publish_start(p, b->stream), "initial statistics");
  r->have_pop = true;
  r->step = 0;
  r->active = r->stop_step > 0;
  r->dev_seeds = false;
  return SAMPO_OK;
}

extern "C" int sampo_batch_seed_stream(sampo_batch* b, uint32_t slot, const sampo_rand_state* st) {
  Replicate* r = get_slot(b, slot);
  if (!r || !st) return SAMPO_ERR_ARG;
  if (!r->have_pop) return bfail(b, SAMPO_ERR_STATE, "initialise the population first");
  // rotate so that the oldest word comes first (the draw at position i reads
  // r[i % 31] and r[(i - 3) % 31])
  DevSeedStream h;
  h.next = r->step;
  for (uint32_t j = 0; j < 31; j++) h.st.r[j] = st->r[(st->i + j) % 31];
  h.st.i = 31u * (st->i / 31u + 1u);
  cudaSetDevice(b->device);
  BCK(cudaMemcpyAsync(&b->sims_dev[slot].rnd, &h, sizeof(h), cudaMemcpyHostToDevice, b->stream), "seed stream");
  BCK(cudaStreamSynchronize(b->stream), "seed stream");
  r->dev_seeds = true;
  return SAMPO_OK;
}

extern "C" int sampo_batch_checkpoint_save(sampo_batch* b, uint32_t slot, const char* path) {
  Replicate* r = get_slot(b, slot);
  if (!r || !path) return SAMPO_ERR_ARG;
  if (!r->have_pop) return bfail(b, SAMPO_ERR_STATE, "no population");
  cudaSetDevice(b->device);
  BCK(cudaStreamSynchronize(b->stream), "checkpoint");  // the slot is at a step boundary
  SimDev h;
  BCK(cudaMemcpy(&h, b->sims_dev + slot, sizeof(SimDev), cudaMemcpyDeviceToHost), "state");
  if ((h.error & SAMPO_DEV_ERR_CAPACITY) && !h.active && h.step < h.stop_step)
    return bfail(b, SAMPO_ERR_STATE, "the slot is paused for capacity: grow it (sampo_batch_grow) first");
  CkHeader hd;
  memset(&hd, 0, sizeof(hd));
  memcpy(hd.magic, kCkMagic, 8);
  hd.version = 2;
  hd.step = h.step;
  hd.cc = r->cc;
  hd.pop = h.pop;
  hd.bnc = h.bnc;
  hd.n = h.pop.r[7].end;
  if (h.step > 0) {
    sampo_stats_row prev;
    BCK(cudaMemcpy(&prev, r->rp.rows + (h.step - 1) % b->ring, sizeof(prev), cudaMemcpyDeviceToHost), "rows");
    hd.prev = prev.pop;
    hd.flags |= CK_PREV;
  }
  if (r->dev_seeds) {
    hd.rnd = h.rnd;
    hd.flags |= CK_SEED_STREAM;
    if (h.rnd.next == h.step + 1) {  // the coming step's seeds are already drawn
      BCK(cudaMemcpy(hd.coming, r->rp.seeds + (size_t)(h.step % b->ring) * 4, sizeof(hd.coming), cudaMemcpyDeviceToHost),
          "seeds");
      hd.flags |= CK_COMING_SEEDS;
    }
  }
  const std::string err = ck_write(path, hd, r->rp.pool[h.cur & 1u]);
  if (!err.empty()) return bfail(b, SAMPO_ERR_IO, err);
  return SAMPO_OK;
}

extern "C" int sampo_batch_checkpoint_load(sampo_batch* b, uint32_t slot, const char* path) {
  Replicate* r = get_slot(b, slot);
  if (!r || !path) return SAMPO_ERR_ARG;
  CkHeader hd;
  FILE* f = nullptr;
  const std::string err = ck_open(path, hd, &f);
  if (!err.empty()) return bfail(b, SAMPO_ERR_IO, err);
  if (hd.cc != r->cc) { fclose(f); return bfail(b, SAMPO_ERR_ARG, "checkpoint carrying capacity differs from the slot's"); }
  if ((uint64_t)hd.n > r->capacity) { fclose(f); return bfail(b, SAMPO_ERR_CAPACITY, "checkpoint pool exceeds the slot's capacity"); }
  if (const char* why = ranges_error(hd.pop, r->capacity)) {
    fclose(f);
    return bfail(b, SAMPO_ERR_IO, std::string("inconsistent checkpoint (") + why + "): " + path);
  }
  cudaSetDevice(b->device);
  BCK(cudaStreamSynchronize(b->stream), "checkpoint");
  const std::string rerr = ck_read_pool(f, hd, r->rp.pool[0]);
  if (!rerr.empty()) return bfail(b, SAMPO_ERR_IO, rerr + ": " + path);
  SimDev h = initial_sim_state((uint32_t)r->capacity, r->cc);
  h.pop = hd.pop;
  h.pop.numLarvae1DayEquiv = h.pop.numFemale = h.pop.numPotentiallyInfective = 0;
  h.bnc = hd.bnc;
  h.step = hd.step;
  h.stop_step = r->stop_step;
  h.active = hd.step < r->stop_step;
  r->dev_seeds = (hd.flags & CK_SEED_STREAM) != 0;
  if (r->dev_seeds) {
    h.rnd = hd.rnd;
    if (hd.flags & CK_COMING_SEEDS)
      BCK(cudaMemcpyAsync((sampo_seeds*)r->rp.seeds + (size_t)(hd.step % b->ring) * 4, hd.coming, sizeof(hd.coming),
                          cudaMemcpyHostToDevice, b->stream), "seeds");
  }
  const int st = upload_slot(b, slot, h);
  if (st) return st;
  BCK(cudaMemsetAsync(r->rp.tilePre, 0, tile_array_words(r->rp.maxTiles) * 4, b->stream), "tile arrays");
  BCK(launch_publish_start(slot_params(b, slot), b->stream), "checkpoint statistics");
  SimDev back;
  BCK(cudaMemcpyAsync(&back, b->sims_dev + slot, sizeof(SimDev), cudaMemcpyDeviceToHost, b->stream), "state");
  BCK(cudaStreamSynchronize(b->stream), "state");
  if (back.pop.numLarvae1DayEquiv != hd.pop.numLarvae1DayEquiv || back.pop.numFemale != hd.pop.numFemale ||
      back.pop.numPotentiallyInfective != hd.pop.numPotentiallyInfective)
    return bfail(b, SAMPO_ERR_INTERNAL, "checkpoint statistics do not match its pool");
  r->have_pop = true;
  r->step = hd.step;
  r->active = h.active != 0;
  return SAMPO_OK;
}

extern "C" int sampo_batch_seed_state(sampo_batch* b, uint32_t slot, sampo_rand_state* st, uint32_t* next_step) {
  Replicate* r = get_slot(b, slot);
  if (!r || !st || !next_step) return SAMPO_ERR_ARG;
  if (!r->dev_seeds) return bfail(b, SAMPO_ERR_STATE, "the slot has no device seed stream");
  cudaSetDevice(b->device);
  DevSeedStream h;
  BCK(cudaMemcpyAsync(&h, &b->sims_dev[slot].rnd, sizeof(h), cudaMemcpyDeviceToHost, b->stream), "seed stream");
  BCK(cudaStreamSynchronize(b->stream), "seed stream");
  *st = h.st;
  *next_step = h.next;
  return SAMPO_OK;
}

static cudaError_t launch_batch_step(sampo_batch* b, const KParams& p) {
  cudaError_t e = launch_count(p, b->grid_count, b->stream, b->items);
  if (e == cudaSuccess) e = launch_scatter(p, b->grid_scatter, b->stream, b->items);
  if (e == cudaSuccess) e = launch_publish(p, PUB_AFTER_STEP, b->stream);
  return e;
}

static int build_batch_graph(sampo_batch* b) {
  if (b->day_graph) return SAMPO_OK;
  const KParams p = all_params(b);
  cudaGraph_t g = nullptr;
  BCK(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal), "capture");
  cudaError_t e = cudaSuccess;
  for (int h = 0; h < 24 && e == cudaSuccess; h++) e = launch_batch_step(b, p);
  cudaError_t e2 = cudaStreamEndCapture(b->stream, &g);
  if (e != cudaSuccess) {
    if (g) cudaGraphDestroy(g);
    return bfail(b, SAMPO_ERR_CUDA, std::string("capture launch: ") + cudaGetErrorString(e));
  }
  if (e2 != cudaSuccess) return bfail(b, SAMPO_ERR_CUDA, std::string("end capture: ") + cudaGetErrorString(e2));
  uint32_t kernels = 0;
  e = graph_kernel_nodes(g, &kernels);
  if (e != cudaSuccess) {
    cudaGraphDestroy(g);
    return bfail(b, SAMPO_ERR_CUDA, std::string("graph nodes: ") + cudaGetErrorString(e));
  }
  b->day_graph_kernels = kernels;
  e = cudaGraphInstantiate(&b->day_graph, g, 0);
  cudaGraphDestroy(g);
  if (e != cudaSuccess) {
    b->day_graph = nullptr;
    return bfail(b, SAMPO_ERR_CUDA, std::string("graph instantiate: ") + cudaGetErrorString(e));
  }
  return SAMPO_OK;
}

extern "C" int sampo_batch_run(sampo_batch* b, uint32_t nsteps, int wait) {
  if (!b) return SAMPO_ERR_ARG;
  if (nsteps == 0) return SAMPO_OK;
  // every active replicate needs inputs and seeds for the steps it will run
  for (uint32_t i = 0; i < b->nslots; i++) {
    const Replicate& r = b->reps[i];
    if (!r.used || !r.have_pop || !r.active) continue;
    const uint32_t last = (uint32_t)std::min<uint64_t>((uint64_t)r.step + nsteps, r.stop_step);
    for (uint32_t st = r.step; st < last; st++) {
      const uint32_t rs = st % b->ring;
      if (r.input_step[rs] != st || (!r.dev_seeds && r.seed_step[rs] != st))
        return bfail(b, SAMPO_ERR_STATE, "slot " + std::to_string(i) + ": no inputs or seeds for step " + std::to_string(st));
    }
  }
  cudaSetDevice(b->device);
  const KParams p = all_params(b);
  BCK(cudaEventRecord(b->ev0, b->stream), "event");
  BCK(launch_publish(p, PUB_REFRESH, b->stream), "step constants");  // inputs may postdate the last publish
  b->launches += 1;
  uint32_t i = 0;
  if (nsteps >= 24) {
    const int rc = build_batch_graph(b);
    if (rc) return rc;
    for (; i + 24 <= nsteps; i += 24) {
      BCK(cudaGraphLaunch(b->day_graph, b->stream), "day graph");
      b->launches += b->day_graph_kernels;
    }
  }
  for (; i < nsteps; i++) {
    BCK(launch_batch_step(b, p), "step kernels");
    b->launches += 3;
  }
  BCK(cudaEventRecord(b->ev1, b->stream), "event");
  b->timed = true;
  for (auto& r : b->reps) {
    if (!r.used || !r.have_pop || !r.active) continue;
    r.step = (uint32_t)std::min<uint64_t>((uint64_t)r.step + nsteps, r.stop_step);
    r.active = r.step < r.stop_step;
  }
  if (wait) {
    BCK(cudaStreamSynchronize(b->stream), "batch run");
    return refresh_mirrors(b);
  }
  return SAMPO_OK;
}

extern "C" int sampo_batch_launches(sampo_batch* b, uint64_t* launches) {
  if (!b || !launches) return SAMPO_ERR_ARG;
  *launches = b->launches;
  return SAMPO_OK;
}

extern "C" int sampo_batch_autotune(sampo_batch* b, uint32_t* count_ctas_per_sm, uint32_t* scatter_ctas_per_sm) {
  if (!b) return SAMPO_ERR_ARG;
  for (uint32_t i = 0; i < b->nslots; i++) {
    const Replicate& r = b->reps[i];
    if (!r.used || !r.have_pop || !r.active) continue;
    const uint32_t rs = r.step % b->ring;
    if (r.input_step[rs] != r.step || (!r.dev_seeds && r.seed_step[rs] != r.step))
      return bfail(b, SAMPO_ERR_STATE, "slot " + std::to_string(i) + ": no inputs or seeds for the coming step");
  }
  cudaSetDevice(b->device);
  const KParams p = all_params(b);
  BCK(launch_publish(p, PUB_REFRESH, b->stream), "step constants");
  int gc = 0, gs = 0, items = kItems;
  BCK(tune_grids(p, b->stream, &gc, &gs, &items, nullptr), "autotune");
  int sms = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, b->device);
  if (sms <= 0) sms = 1;
  if (gc != b->grid_count || gs != b->grid_scatter || items != b->items) {
    b->grid_count = gc;
    b->grid_scatter = gs;
    b->items = items;
    if (b->day_graph) {
      cudaGraphExecDestroy(b->day_graph);
      b->day_graph = nullptr;
    }
  }
  if (count_ctas_per_sm) *count_ctas_per_sm = (uint32_t)(gc / sms);
  if (scatter_ctas_per_sm) *scatter_ctas_per_sm = (uint32_t)(gs / sms);
  return SAMPO_OK;
}

extern "C" int sampo_batch_set_species(sampo_batch* b, const sampo_species* sp) {
  if (!b) return SAMPO_ERR_ARG;
  if (sp && sampo_species_device(sp) != b->device) return bfail(b, SAMPO_ERR_ARG, "species compiled for another device");
  cudaSetDevice(b->device);
  if (b->species == sp) return SAMPO_OK;
  b->species = sp;
  if (sp) b->items = kItems;  // a run-time species is built for 4 slots per thread
  b->grid_count = grid_blocks_count(b->nslots, sp, b->items);
  b->grid_scatter = grid_blocks_scatter(b->nslots, sp, b->items);
  if (b->day_graph) {
    cudaGraphExecDestroy(b->day_graph);
    b->day_graph = nullptr;
  }
  return SAMPO_OK;
}

extern "C" int sampo_batch_set_grids(sampo_batch* b, uint32_t count_ctas_per_sm, uint32_t scatter_ctas_per_sm) {
  if (!b) return SAMPO_ERR_ARG;
  cudaSetDevice(b->device);
  int sms = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, b->device);
  if (sms <= 0) sms = 1;
  const uint32_t max_c = (uint32_t)(grid_blocks_count(b->nslots, b->species, b->items) / sms);
  const uint32_t max_s = (uint32_t)(grid_blocks_scatter(b->nslots, b->species, b->items) / sms);
  if (count_ctas_per_sm < 1 || count_ctas_per_sm > max_c || scatter_ctas_per_sm < 1 || scatter_ctas_per_sm > max_s)
    return bfail(b, SAMPO_ERR_ARG, "CTAs per SM outside 1.." + std::to_string(max_c) + " (count) / 1.." +
                                       std::to_string(max_s) + " (update/scatter)");
  const int gc = (int)count_ctas_per_sm * sms, gs = (int)scatter_ctas_per_sm * sms;
  if (gc != b->grid_count || gs != b->grid_scatter) {
    b->grid_count = gc;
    b->grid_scatter = gs;
    if (b->day_graph) {
      cudaGraphExecDestroy(b->day_graph);
      b->day_graph = nullptr;
    }
  }
  return SAMPO_OK;
}

extern "C" int sampo_batch_set_items_per_thread(sampo_batch* b, uint32_t items) {
  if (!b) return SAMPO_ERR_ARG;
  if (items != 2 && items != 4) return bfail(b, SAMPO_ERR_ARG, "items per thread must be 2 or 4");
  if (b->species && items != (uint32_t)kItems) return bfail(b, SAMPO_ERR_ARG, "a run-time species runs 4 items per thread");
  cudaSetDevice(b->device);
  if ((int)items != b->items) {
    b->items = (int)items;
    b->grid_count = grid_blocks_count(b->nslots, b->species, b->items);
    b->grid_scatter = grid_blocks_scatter(b->nslots, b->species, b->items);
    if (b->day_graph) {
      cudaGraphExecDestroy(b->day_graph);
      b->day_graph = nullptr;
    }
  }
  return SAMPO_OK;
}

extern "C" int sampo_batch_items_per_thread(sampo_batch* b, uint32_t* items) {
  if (!b || !items) return SAMPO_ERR_ARG;
  *items = (uint32_t)b->items;
  return SAMPO_OK;
}

extern "C" int sampo_batch_sync(sampo_batch* b) {
  if (!b) return SAMPO_ERR_ARG;
  cudaSetDevice(b->device);
  BCK(cudaStreamSynchronize(b->stream), "batch sync");
  return refresh_mirrors(b);
}

extern "C" int sampo_batch_states(sampo_batch* b, sampo_slot_state* out, uint32_t nslots) {
  if (!b || !out || nslots > b->nslots) return SAMPO_ERR_ARG;
  cudaSetDevice(b->device);
  std::vector<SimDev> h;
  const int rc = read_headers(b, h);
  if (rc) return rc;
  for (uint32_t i = 0; i < nslots; i++) {
    const Replicate& r = b->reps[i];
    sampo_slot_state& o = out[i];
    o.step = h[i].step;
    o.active = h[i].active;
    o.status = h[i].error | h[i].warn;
    o.end = r.have_pop ? h[i].pop.r[7].end : 0u;
    o.capacity = r.used ? r.capacity : 0u;
  }
  return SAMPO_OK;
}

extern "C" int sampo_batch_grow(sampo_batch* b, uint32_t slot, uint64_t capacity) {
  Replicate* r = get_slot(b, slot);
  if (!r) return SAMPO_ERR_ARG;
  if (!r->have_pop) return bfail(b, SAMPO_ERR_STATE, "no population");
  if (capacity > 0xFFFFFF00ull) return bfail(b, SAMPO_ERR_ARG, "capacity above 0xFFFFFF00 slots");
  cudaSetDevice(b->device);
  std::vector<SimDev> hs;
  int rc = read_headers(b, hs);  // waits for the queued work
  if (rc) return rc;
  SimDev h = hs[slot];
  const uint32_t end = h.pop.r[7].end;
  if (capacity < end || capacity < 128) return bfail(b, SAMPO_ERR_ARG, "capacity below the pool's end");
  const RepLayout L(capacity, b->ring), L0(r->capacity, b->ring);
  void* mem = nullptr;
  cudaError_t e = cudaMallocFromPoolAsync(&mem, L.total, b->mempool, b->stream);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return bfail(b, SAMPO_ERR_CAPACITY, std::string("grown replicate buffers: ") + cudaGetErrorString(e));
  }
  const RepParams rp = carve(L, mem, b->sims_dev + slot, b->ring);
  const RepParams& old = r->rp;
  // the current pool into buffer 0, column by column: slot indices unchanged
  const DevPool& S = old.pool[h.cur & 1u];
  const DevPool& D = rp.pool[0];
  const size_t b4 = (size_t)end * 4;
  if (end) {
    BCK(cudaMemcpyAsync(D.age, S.age, b4, cudaMemcpyDeviceToDevice, b->stream), "grow");
    BCK(cudaMemcpyAsync(D.his, S.his, b4, cudaMemcpyDeviceToDevice, b->stream), "grow");
    BCK(cudaMemcpyAsync(D.delay, S.delay, b4, cudaMemcpyDeviceToDevice, b->stream), "grow");
    BCK(cudaMemcpyAsync(D.sporo, S.sporo, b4, cudaMemcpyDeviceToDevice, b->stream), "grow");
    BCK(cudaMemcpyAsync(D.uni, S.uni, b4, cudaMemcpyDeviceToDevice, b->stream), "grow");
    BCK(cudaMemcpyAsync(D.avail, S.avail, b4, cudaMemcpyDeviceToDevice, b->stream), "grow");
    BCK(cudaMemcpyAsync(D.cycle, S.cycle, b4, cudaMemcpyDeviceToDevice, b->stream), "grow");
    BCK(cudaMemcpyAsync(D.hbc, S.hbc, b4, cudaMemcpyDeviceToDevice, b->stream), "grow");
    BCK(cudaMemcpyAsync(D.batches, S.batches, b4, cudaMemcpyDeviceToDevice, b->stream), "grow");
    BCK(cudaMemcpyAsync(D.flags, S.flags, end, cudaMemcpyDeviceToDevice, b->stream), "grow");
  }
  // the rings of inputs, seeds and rows (same ring length, same layout)
  BCK(cudaMemcpyAsync((void*)rp.T, old.T, L.T + L.env + L.seeds + L.wt + L.rows, cudaMemcpyDeviceToDevice, b->stream),
      "grow rings");
  // fresh look-back arrays: zero epochs never match the running step's
  BCK(cudaMemsetAsync(rp.tilePre, 0, tile_array_words(L.max_tiles) * 4, b->stream), "tile arrays");
  h.capacity = (uint32_t)capacity;
  h.cur = 0;
  h.error &= ~SAMPO_DEV_ERR_CAPACITY;
  h.active = h.step < h.stop_step ? 1u : 0u;
  BCK(cudaMemcpyAsync(b->sims_dev + slot, &h, offsetof(SimDev, ctx), cudaMemcpyHostToDevice, b->stream), "slot state");
  BCK(cudaMemcpyAsync(b->reps_dev + slot, &rp, sizeof(RepParams), cudaMemcpyHostToDevice, b->stream), "slot params");
  BCK(cudaFreeAsync(r->mem, b->stream), "free replicate");
  (void)L0;
  r->mem = mem;
  r->rp = rp;
  r->capacity = capacity;
  r->step = h.step;
  r->active = h.active != 0;
  BCK(cudaStreamSynchronize(b->stream), "grow");  // h lives on this stack
  return SAMPO_OK;
}

extern "C" int sampo_batch_last_run_ms(sampo_batch* b, double* ms) {
  if (!b || !ms) return SAMPO_ERR_ARG;
  *ms = 0;
  if (!b->timed) return SAMPO_OK;
  cudaSetDevice(b->device);
  BCK(cudaEventSynchronize(b->ev1), "event");
  float f = 0;
  BCK(cudaEventElapsedTime(&f, b->ev0, b->ev1), "event");
  *ms = f;
  return SAMPO_OK;
}

extern "C" int sampo_batch_rows(sampo_batch* b, uint32_t slot, uint32_t first, uint32_t n, sampo_stats_row* out) {
  Replicate* r = get_slot(b, slot);
  if (!r || (!out && n)) return SAMPO_ERR_ARG;
  if (!r->have_pop) return bfail(b, SAMPO_ERR_STATE, "no population");
  if ((uint64_t)first + n > (uint64_t)r->step + 1) return bfail(b, SAMPO_ERR_ARG, "rows past the replicate's current step");
  if (n && r->step - first >= b->ring) return bfail(b, SAMPO_ERR_ARG, "rows already overwritten in the ring");
  cudaSetDevice(b->device);
  uint32_t c = 0;
  while (c < n) {
    const uint32_t rs = (first + c) % b->ring;
    const uint32_t m = std::min(n - c, b->ring - rs);
    BCK(cudaMemcpyAsync(out + c, r->rp.rows + rs, (size_t)m * sizeof(sampo_stats_row), cudaMemcpyDeviceToHost, b->stream), "rows");
    c += m;
  }
  BCK(cudaStreamSynchronize(b->stream), "rows");
  return SAMPO_OK;
}

extern "C" int sampo_batch_state(sampo_batch* b, uint32_t slot, uint32_t* step, uint32_t* active, uint32_t* status_bits) {
  Replicate* r = get_slot(b, slot);
  if (!r) return SAMPO_ERR_ARG;
  cudaSetDevice(b->device);
  SimDev h;
  BCK(cudaMemcpyAsync(&h, b->sims_dev + slot, offsetof(SimDev, ctx), cudaMemcpyDeviceToHost, b->stream), "state");
  BCK(cudaStreamSynchronize(b->stream), "state");
  if (step) *step = h.step;
  if (active) *active = h.active;
  if (status_bits) *status_bits = h.error | h.warn;
  return SAMPO_OK;
}

extern "C" int sampo_batch_histogram(sampo_batch* b, uint32_t slot, uint32_t out[100]) {
  Replicate* r = get_slot(b, slot);
  if (!r || !out) return SAMPO_ERR_ARG;
  if (!r->have_pop) return bfail(b, SAMPO_ERR_STATE, "no population");
  cudaSetDevice(b->device);
  BCK(cudaMemsetAsync(b->hist_dev, 0, 100 * sizeof(uint32_t), b->stream), "histogram");
  BCK(launch_histogram(slot_params(b, slot), b->hist_dev, b->stream), "histogram");
  BCK(cudaMemcpyAsync(out, b->hist_dev, 100 * sizeof(uint32_t), cudaMemcpyDeviceToHost, b->stream), "histogram");
  BCK(cudaStreamSynchronize(b->stream), "histogram");
  return SAMPO_OK;
}

extern "C" int sampo_batch_read_pool(sampo_batch* b, uint32_t slot, sampo_population* pop, sampo_pool_view* v) {
  Replicate* r = get_slot(b, slot);
  if (!r || !pop) return SAMPO_ERR_ARG;
  if (!r->have_pop) return bfail(b, SAMPO_ERR_STATE, "no population");
  cudaSetDevice(b->device);
  SimDev h;
  BCK(cudaMemcpyAsync(&h, b->sims_dev + slot, offsetof(SimDev, ctx), cudaMemcpyDeviceToHost, b->stream), "state");
  BCK(cudaStreamSynchronize(b->stream), "state");
  *pop = h.pop;
  if (!v) return SAMPO_OK;
  const uint32_t n = h.pop.r[7].end;
  const DevPool& P = r->rp.pool[h.cur & 1u];
  const size_t b4 = (size_t)n * 4;
  BCK(cudaMemcpyAsync(v->ageInHours, P.age, b4, cudaMemcpyDeviceToHost, b->stream), "pool read");
  BCK(cudaMemcpyAsync(v->hoursInState, P.his, b4, cudaMemcpyDeviceToHost, b->stream), "pool read");
  BCK(cudaMemcpyAsync(v->delay, P.delay, b4, cudaMemcpyDeviceToHost, b->stream), "pool read");
  BCK(cudaMemcpyAsync(v->cumulativeSporogonicDevelopment, P.sporo, b4, cudaMemcpyDeviceToHost, b->stream), "pool read");
  BCK(cudaMemcpyAsync(v->larvalDelayOrOviAttempts, P.uni, b4, cudaMemcpyDeviceToHost, b->stream), "pool read");
  BCK(cudaMemcpyAsync(v->availableEggs, P.avail, b4, cudaMemcpyDeviceToHost, b->stream), "pool read");
  BCK(cudaMemcpyAsync(v->cycleLength, P.cycle, b4, cudaMemcpyDeviceToHost, b->stream), "pool read");
  BCK(cudaMemcpyAsync(v->humanBloodmealCount, P.hbc, b4, cudaMemcpyDeviceToHost, b->stream), "pool read");
  BCK(cudaMemcpyAsync(v->numEggBatches, P.batches, b4, cudaMemcpyDeviceToHost, b->stream), "pool read");
  std::vector<uint8_t> flags(n);
  BCK(cudaMemcpyAsync(flags.data(), P.flags, n, cudaMemcpyDeviceToHost, b->stream), "pool read");
  BCK(cudaStreamSynchronize(b->stream), "pool read");
  for (uint32_t i = 0; i < n; i++) {
    v->state[i] = flags[i] & 7u;
    v->isFemale[i] = (flags[i] >> 3) & 1u;
  }
  return SAMPO_OK;
}
