// sampo_kernels.cu - host side of the step kernels: grid sizes, launchers
// and the grid autotuner. The device code is in sampo_step_kernels.cuh.
#include <cuda_runtime.h>
#include <mutex>
#include <vector>
#include "sampo_step_kernels.cuh"
#include "sampo_small_step.cuh"

namespace sampo {

// ------------------------------------------------------------------------
// Per-device set-up, once per device under a once_flag: the SM count and the
// dynamic shared memory limit of the two persistent kernels (a function
// attribute applies to the device that is current when it is set, so every
// device the library runs on gets its own). Devices beyond kMaxDevices are
// set up on every call under a mutex.
// The built-in count and update/scatter passes for `items` slots per thread.
static const void* count_fn(int items) { return items == 2 ? (const void*)k_count<2> : (const void*)k_count<4>; }
static const void* scatter_fn(int items) { return items == 2 ? (const void*)k_scatter<2> : (const void*)k_scatter<4>; }

namespace {
constexpr int kMaxDevices = 64;
struct DeviceSetup {
  std::once_flag once;
  int sms = 1;
};
DeviceSetup g_setup[kMaxDevices];
std::mutex g_setup_mu;

int setup_current_device(int dev) {
  int sms = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  for (int items : {2, 4}) {
    cudaFuncSetAttribute(count_fn(items), cudaFuncAttributeMaxDynamicSharedMemorySize, (int)(count_smem(items) + plan_bytes(kMaxRep)));
    cudaFuncSetAttribute(scatter_fn(items), cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)(scatter_smem(items) + plan_bytes(kMaxRep)));
  }
  return sms > 0 ? sms : 1;
}
}  // namespace

// The SM count of the current device, after its one-time set-up.
static int sm_count() {
  int dev = 0;
  cudaGetDevice(&dev);
  if (dev < 0 || dev >= kMaxDevices) {
    std::lock_guard<std::mutex> lk(g_setup_mu);
    return setup_current_device(dev);
  }
  DeviceSetup& d = g_setup[dev];
  std::call_once(d.once, [&] { d.sms = setup_current_device(dev); });
  return d.sms;
}
static void set_smem_attrs() { (void)sm_count(); }
size_t count_smem_max() { return kCountSmem + plan_bytes(kMaxRep); }
size_t scatter_smem_max() { return kScatterSmem + plan_bytes(kMaxRep); }

// Resident CTAs per SM of a persistent kernel, built in (for `items` slots
// per thread) or of p.ks (4 slots per thread).
static int occupancy(const void* ks, int kid, int items, int threads, size_t smem) {
  if (ks) return species_occupancy(ks, kid, threads, smem);
  set_smem_attrs();
  int per = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, kid == KID_COUNT ? count_fn(items) : scatter_fn(items), threads, smem);
  return per;
}
int grid_blocks_count(uint32_t nrep, const void* ks, int items) {
  const int per = occupancy(ks, KID_COUNT, items, kBlock, count_smem(items) + plan_bytes(nrep));
  return sm_count() * (per > 0 ? per : 1);
}
int grid_blocks_scatter(uint32_t nrep, const void* ks, int items) {
  const int per = occupancy(ks, KID_SCATTER, items, kScatterThreads, scatter_smem(items) + plan_bytes(nrep));
  return sm_count() * (per > 0 ? per : 1);
}

// One launch of kernel kid: the built-in one (fn) or p.ks's.
static cudaError_t launch(const KParams& p, int kid, const void* fn, dim3 grid, dim3 block, size_t smem, cudaStream_t st,
                          void** args) {
  if (p.ks) return species_launch(p.ks, kid, grid, block, smem, st, args);
  set_smem_attrs();
  return cudaLaunchKernel(fn, grid, block, args, smem, st);
}

cudaError_t launch_count(const KParams& p, int grid, cudaStream_t st, int items) {
  KParams q = p;
  void* args[] = {&q};
  if (p.ks) items = kItems;  // a run-time species is built for 4 slots per thread
  return launch(p, KID_COUNT, count_fn(items), grid, kBlock, count_smem(items) + plan_bytes(p.nrep), st, args);
}
cudaError_t launch_scatter(const KParams& p, int grid, cudaStream_t st, int items) {
  KParams q = p;
  void* args[] = {&q};
  if (p.ks) items = kItems;
  return launch(p, KID_SCATTER, scatter_fn(items), grid, kScatterThreads, scatter_smem(items) + plan_bytes(p.nrep), st, args);
}
cudaError_t launch_publish(const KParams& p, int mode, cudaStream_t st) {
  KParams q = p;
  void* args[] = {&q, &mode};
  return launch(p, KID_PUBLISH, (const void*)k_publish, p.nrep, mode == PUB_REFRESH ? 32 : kPublishThreads, 0, st, args);
}
cudaError_t launch_init_eggs(const KParams& p, uint32_t n, float T0, const sampo_seeds* seeds_dev, int age_days_max,
                             uint64_t age_seed, cudaStream_t st) {
  KParams q = p;
  void* args[] = {&q, &n, &T0, &seeds_dev, &age_days_max, &age_seed};
  return launch(p, KID_INIT_EGGS, (const void*)k_init_eggs, sm_count() * 4, 256, 0, st, args);
}
cudaError_t launch_publish_start(const KParams& p, cudaStream_t st) {
  KParams q = p;
  void* args[] = {&q};
  cudaError_t e = launch(p, KID_POOL_STATS, (const void*)k_pool_stats, sm_count() * 4, 256, 0, st, args);
  if (e != cudaSuccess) return e;
  int mode = PUB_INITIAL;
  void* args2[] = {&q, &mode};
  return launch(p, KID_PUBLISH, (const void*)k_publish, 1, kPublishThreads, 0, st, args2);
}
cudaError_t launch_histogram(const KParams& p, uint32_t* hist_dev, cudaStream_t st) {
  KParams q = p;
  void* args[] = {&q, &hist_dev};
  return launch(p, KID_HISTOGRAM, (const void*)k_histogram, sm_count() * 4, 256, 0, st, args);
}
static cudaError_t launch_trial_reset(const KParams& p, cudaStream_t st) {
  KParams q = p;
  void* args[] = {&q};
  return launch(p, KID_TRIAL_RESET, (const void*)k_trial_reset, (int)((p.nrep + 255) / 256), 256, 0, st, args);
}
// The built-in kernels only: a run-time species is tuned at one tile size.
static cudaError_t launch_clear_lookback(const KParams& p, cudaStream_t st) {
  KParams q = p;
  void* args[] = {&q};
  return cudaLaunchKernel((const void*)k_clear_lookback, sm_count() * 4, 256, args, 0, st);
}
// The grid tuner of one tile size: see tune_grids.
static cudaError_t tune_grids_items(const KParams& p, cudaStream_t st, int items, cudaEvent_t* ev, int* grid_count,
                                    int* grid_scatter, double* best_ms) {
  int max_c = occupancy(p.ks, KID_COUNT, items, kBlock, count_smem(items) + plan_bytes(p.nrep));
  int max_s = occupancy(p.ks, KID_SCATTER, items, kScatterThreads, scatter_smem(items) + plan_bytes(p.nrep));
  if (max_c < 1) max_c = 1;
  if (max_s < 1) max_s = 1;
  const int sms = sm_count();
  cudaError_t e = cudaSuccess;
  // each kernel's time is taken on its own (the best count grid does not
  // depend on the scatter grid), minimum over every trial that ran it (eight
  // per pair: small pools run the kernels in tens of microseconds, where
  // single timings differ by more than the grids do); one untimed trial first
  double tc[9], ts[9];
  for (int i = 0; i < 9; i++) tc[i] = ts[i] = 1e30;
  max_c = max_c > 8 ? 8 : max_c;
  max_s = max_s > 8 ? 8 : max_s;
  for (int c = 1; c <= max_c && e == cudaSuccess; c++) {
    for (int s = 1; s <= max_s && e == cudaSuccess; s++) {
      for (int rep = (c == 1 && s == 1) ? -1 : 0; rep < 8 && e == cudaSuccess; rep++) {
        if ((e = launch_trial_reset(p, st)) != cudaSuccess) break;
        if ((e = cudaEventRecord(ev[0], st)) != cudaSuccess) break;
        if ((e = launch_count(p, c * sms, st, items)) != cudaSuccess) break;
        if ((e = cudaEventRecord(ev[1], st)) != cudaSuccess) break;
        if ((e = launch_scatter(p, s * sms, st, items)) != cudaSuccess) break;
        if ((e = cudaEventRecord(ev[2], st)) != cudaSuccess) break;
        if ((e = cudaEventSynchronize(ev[2])) != cudaSuccess) break;
        if (rep < 0) continue;
        float m0 = 0, m1 = 0;
        cudaEventElapsedTime(&m0, ev[0], ev[1]);
        cudaEventElapsedTime(&m1, ev[1], ev[2]);
        if (m0 < tc[c]) tc[c] = m0;
        if (m1 < ts[s]) ts[s] = m1;
      }
    }
  }
  int bc = max_c, bs = max_s;
  for (int c = 1; c <= max_c; c++)
    if (tc[c] < tc[bc]) bc = c;
  for (int s = 1; s <= max_s; s++)
    if (ts[s] < ts[bs]) bs = s;
  // the kernels run back to back in a step, where a small pool's times are
  // mostly start-up and tail: the pick and the largest grids, run that way
  double tj[2] = {1e30, 1e30};
  const int gc[2] = {bc, max_c}, gs[2] = {bs, max_s};
  for (int rep = 0; rep < 8 && e == cudaSuccess; rep++) {
    for (int v = 0; v < 2 && e == cudaSuccess; v++) {
      if (v == 1 && bc == max_c && bs == max_s) break;
      if ((e = launch_trial_reset(p, st)) != cudaSuccess) break;
      if ((e = cudaEventRecord(ev[0], st)) != cudaSuccess) break;
      if ((e = launch_count(p, gc[v] * sms, st, items)) != cudaSuccess) break;
      if ((e = launch_scatter(p, gs[v] * sms, st, items)) != cudaSuccess) break;
      if ((e = cudaEventRecord(ev[2], st)) != cudaSuccess) break;
      if ((e = cudaEventSynchronize(ev[2])) != cudaSuccess) break;
      float m = 0;
      cudaEventElapsedTime(&m, ev[0], ev[2]);
      if (m < tj[v]) tj[v] = m;
    }
  }
  if (bc != max_c || bs != max_s) {
    if (tj[1] <= tj[0]) {
      bc = max_c;
      bs = max_s;
      tj[0] = tj[1];
    }
  }
  *grid_count = bc * sms;
  *grid_scatter = bs * sms;
  *best_ms = tj[0];
  return e;
}

cudaError_t tune_grids(const KParams& p, cudaStream_t st, int* grid_count, int* grid_scatter, int* items, double* best_ms) {
  cudaEvent_t ev[3] = {nullptr, nullptr, nullptr};
  cudaError_t e = cudaSuccess;
  for (int i = 0; i < 3 && e == cudaSuccess; i++) e = cudaEventCreate(&ev[i]);
  // tile sizes: 1024-slot tiles (4 slots per thread) and, for the built-in
  // species, 512-slot tiles; the step as a whole decides
  double best = 1e30;
  int bi = kItems, bgc = 0, bgs = 0;
  for (int it : {4, 2}) {
    if (e != cudaSuccess || (it != kItems && p.ks)) break;
    int gc = 0, gs = 0;
    double ms = 1e30;
    if (!p.ks) e = launch_clear_lookback(p, st);  // the other tile size's trial prefixes
    if (e == cudaSuccess) e = tune_grids_items(p, st, it, ev, &gc, &gs, &ms);
    if (e == cudaSuccess && ms < best) {
      best = ms;
      bi = it;
      bgc = gc;
      bgs = gs;
    }
  }
  if (e == cudaSuccess) e = launch_trial_reset(p, st);
  if (e == cudaSuccess && !p.ks) e = launch_clear_lookback(p, st);  // the step may run at either tile size
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  for (int i = 0; i < 3; i++)
    if (ev[i]) cudaEventDestroy(ev[i]);
  *grid_count = bgc;
  *grid_scatter = bgs;
  *items = bi;
  if (best_ms) *best_ms = best;
  return e;
}
static const void* small_fn(int items) {
  return items == 1 ? (const void*)k_step_small<1> : items == 2 ? (const void*)k_step_small<2> : (const void*)k_step_small<4>;
}
int grid_blocks_small(int items) {
  int per = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, small_fn(items), kSmallThreads, small_stage(items)) != cudaSuccess) {
    (void)cudaGetLastError();
    return 0;
  }
  return sm_count() * per;
}

cudaError_t graph_kernel_nodes(cudaGraph_t g, uint32_t* kernels) {
  size_t nn = 0;
  cudaError_t e = cudaGraphGetNodes(g, nullptr, &nn);
  std::vector<cudaGraphNode_t> nodes(nn);
  if (e == cudaSuccess && nn) e = cudaGraphGetNodes(g, nodes.data(), &nn);
  uint32_t k = 0;
  for (size_t i = 0; i < nn && e == cudaSuccess; i++) {
    cudaGraphNodeType t;
    e = cudaGraphNodeGetType(nodes[i], &t);
    k += t == cudaGraphNodeTypeKernel ? 1u : 0u;
  }
  *kernels = k;
  return e;
}

cudaError_t launch_small(const KParams& p, int grid, bool cooperative, uint32_t nsteps, cudaStream_t st, int items) {
  KParams q = p;
  void* args[] = {&q, &nsteps};
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(grid);
  cfg.blockDim = dim3(kSmallThreads);
  cfg.dynamicSmemBytes = small_stage(items);
  cfg.stream = st;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeCooperative;
  attr[0].val.cooperative = 1;
  cfg.attrs = attr;
  cfg.numAttrs = cooperative ? 1 : 0;
  return cudaLaunchKernelExC(&cfg, small_fn(items), args);
}
cudaError_t launch_eval_math(int fn, const float* x, const float* y, float* out, uint32_t n, cudaStream_t st) {
  k_eval_math<<<sm_count() * 2, 256, 0, st>>>(fn, x, y, out, n);
  return cudaGetLastError();
}

}  // namespace sampo
