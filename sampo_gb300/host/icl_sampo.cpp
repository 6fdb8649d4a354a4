/*
 * icl_sampo.cpp - the reference's device layer, lib_icl (include/lib_icl.h:
 * 100-159) and the scan driver (include/scan.h:5-11), as src/abms.c uses
 * them, implemented on this library's C ABI (include/sampo.h). The
 * reference's src/abms.c links against this file and libsampo_cuda.so
 * unmodified and runs its hourly loop on the GPU: no OpenCL platform, no
 * kernel sources, no scan buffers.
 *
 * How abms.c's calls map (src/abms.c line numbers):
 *   icl_create_buffer      no device storage: the pool lives in the library.
 *                          The parts the host writes or reads (the Population
 *                          pair, BitesNcycles, EggsNbiomass, the seeds, and
 *                          the histogram storeHistogram keeps at the start of
 *                          the scratch buffer, :541) get a host mirror on
 *                          first use.
 *   initAgents, 1st launch createInitialPopulation (:185-228): remembers the
 *                          egg count (EggsNbiomass written at :650), the
 *                          temperature and the seeds (generateSeeds at :671).
 *   calcL1de*, calcFemales* calcStats (:230-310): the mirror's pop[0] becomes
 *                          the population at the step's start.
 *   killAgents             update (:319-327): the carrying capacity and the
 *                          pool size (the AgentAge buffer's length).
 *   updateAgents           update (:329-340): one sampo_step with the step's
 *                          Environment, temperature, world time and the
 *                          seeds the host wrote; the simulation is created
 *                          and initialised at the first one.
 *   initAgents (later), preScan, scan, oldToNewAgents   createNewAgents
 *                          (:381-462): done by that sampo_step.
 *   ageHistogram           storeHistogram (:160-183): sampo_histogram.
 * The buffer swaps of :517-519 change nothing here.
 *
 * A species header other than properties.h (abms.c's argv[3], passed as
 * -DSPECIES= in every kernel's build options) is compiled into the step
 * kernels with sampo_species_compile, looked up as given and then in the
 * -I directory of the build options.
 *
 * Build: see icl_sampo.mk beside this file.
 */
#include <CL/cl.h>
#include <stdarg.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>
#include <string>
#include <vector>
extern "C" {
#include "lib_icl.h"
}
#include "sampo.h"

namespace {

// Host accesses reach at most this far into a buffer (the largest is the
// 400-byte histogram; the pool buffers themselves are never read back).
constexpr size_t kMirrorMax = 1 << 16;
// struct AgentAge (include/agent.h:90-95): four 4-byte fields per slot.
constexpr size_t kAgentAgeBytes = 16;

struct Buffer {
  icl_buffer b;                     // what abms.c holds (its first member, so the pointers convert)
  std::vector<unsigned char> host;  // the mirror of the part the host has touched (zero-filled at first use)
};
struct Kernel {
  icl_kernel k;
  std::string name;
};
// struct EggsNbiomass (include/agent.h:38-41)
struct Enb {
  int32_t totalBiomass;
  uint32_t newEggs;
};

struct State {
  icl_device dev;
  sampo_sim* sim = nullptr;
  sampo_species* species = nullptr;
  std::string species_name = "properties.h", include_dir;
  bool have_init = false;           // the first initAgents launch was seen
  uint32_t n0 = 0;
  float T0 = 0.0f;
  sampo_seeds seeds0[4];
  uint64_t capacity = 0;
  float cc = 0.0f;
  int age_days = -1;                // icl_sampo_initial_ages (an extension)
  unsigned long long age_seed = 0;
  int pop_writes = 0;
} g;

[[noreturn]] void die(const char* what, const char* detail) {
  fprintf(stderr, "icl_sampo: %s%s%s\n", what, detail ? ": " : "", detail ? detail : "");
  exit(-1);
}

unsigned char* mirror(icl_buffer* b, size_t off, size_t size) {
  Buffer* x = reinterpret_cast<Buffer*>(b);
  if (off + size > x->b.size) die("access past the end of a buffer", nullptr);
  if (off + size > kMirrorMax) die("host access to the pool", nullptr);
  if (x->host.size() < off + size) x->host.resize(off + size, 0);
  return x->host.data() + off;
}

// The simulation, at the first step: abms.c has by then created the pool
// buffers, written the initial Population and run createInitialPopulation.
void start(const sampo_environment& env0) {
  if (!g.have_init) die("a step before createInitialPopulation", nullptr);
  sampo_config cfg;
  memset(&cfg, 0, sizeof(cfg));
  cfg.capacity = g.capacity;
  cfg.carrying_capacity = g.cc;
  cfg.device = 0;
  cfg.max_steps = 2;  // steps run one at a time with explicit inputs
  if (sampo_create(&cfg, &g.sim) != SAMPO_OK) die("sampo_create failed", nullptr);
  if (g.species_name != "properties.h") {
    static char log[1 << 16];
    std::string path = g.species_name;
    if (FILE* f = fopen(path.c_str(), "r")) fclose(f);
    else if (!g.include_dir.empty()) path = g.include_dir + "/" + g.species_name;
    if (sampo_species_compile(path.c_str(), 0, log, sizeof(log), &g.species) != SAMPO_OK) die("species header", log);
    if (sampo_set_species(g.sim, g.species) != SAMPO_OK) die("sampo_set_species", sampo_last_error(g.sim));
  }
  // initAgents reads temperature[0] (src/abms.c:198); its world time and
  // Environment are those of step 0
  if (sampo_set_inputs(g.sim, 0, &g.T0, &env0, 1) != SAMPO_OK) die("sampo_set_inputs", sampo_last_error(g.sim));
  if (sampo_init_population(g.sim, g.n0, g.seeds0, g.age_days, g.age_seed) != SAMPO_OK)
    die("sampo_init_population", sampo_last_error(g.sim));
}

// The mirrors the host reads after a step: the population at the coming
// step's start (both halves of the pair) and the counters it prints.
void publish(icl_buffer* pop, icl_buffer* bnc) {
  sampo_stats_row row;
  if (sampo_current_row(g.sim, &row) != SAMPO_OK) die("sampo_current_row", sampo_last_error(g.sim));
  memcpy(mirror(pop, 0, sizeof(sampo_population)), &row.pop, sizeof(sampo_population));
  memcpy(mirror(pop, sizeof(sampo_population), sizeof(sampo_population)), &row.pop, sizeof(sampo_population));
  memcpy(mirror(bnc, 0, sizeof(sampo_bites_cycles)), &row.bnc, sizeof(sampo_bites_cycles));
}

long long now_ns() {
  struct timespec ts;
  clock_gettime(CLOCK_MONOTONIC, &ts);
  return (long long)ts.tv_sec * 1000000000LL + ts.tv_nsec;
}

}  // namespace

extern "C" {

/* Aged initial eggs (an extension of this library, sampo_init_population's
 * age_days_max >= 0): call before abms.c's main. The initial layout is then
 * the padded one a compaction produces, and the host's own copy of the
 * initial Population is switched to it when abms.c writes it (:477). */
void icl_sampo_initial_ages(int age_days_max, unsigned long long age_seed) {
  g.age_days = age_days_max;
  g.age_seed = age_seed;
}

cl_int clFinish(cl_command_queue) { return CL_SUCCESS; }
cl_int clWaitForEvents(cl_uint, const cl_event*) { return CL_SUCCESS; }

void icl_init_devices(cl_device_type) {
  memset(&g.dev, 0, sizeof(g.dev));
  g.dev.name = (char*)"libsampo_cuda";
  g.dev.vendor = (char*)"NVIDIA";
  g.dev.version = (char*)"sampo C ABI";
  g.dev.type = CL_DEVICE_TYPE_GPU;
}
cl_uint icl_get_num_devices() { return 1; }
icl_device* icl_get_device(cl_uint) { return &g.dev; }
void icl_release_devices() {
  if (g.sim) sampo_destroy(g.sim);
  g.sim = nullptr;
  if (g.species) sampo_species_free(g.species);
  g.species = nullptr;
}
void icl_print_device_short_info(icl_device* dev) {
  printf("GPU: %s | %s | %s (ABI %d)\n", dev->name, dev->vendor, dev->version, sampo_abi_version());
}
void icl_print_device_infos(icl_device* dev) { icl_print_device_short_info(dev); }

icl_buffer* icl_create_buffer(icl_device* dev, cl_mem_flags, size_t size) {
  Buffer* x = new Buffer();
  x->b.mem = nullptr;
  x->b.size = size;
  x->b.dev = dev;
  return &x->b;
}
void icl_read_buffer(const icl_buffer* buf, cl_bool, size_t size, void* ptr, icl_event*, icl_event*) {
  memcpy(ptr, mirror(const_cast<icl_buffer*>(buf), 0, size), size);
}
void icl_read_buffer_offset(const icl_buffer* buf, cl_bool, size_t off, size_t size, void* ptr, icl_event*, icl_event*) {
  memcpy(ptr, mirror(const_cast<icl_buffer*>(buf), off, size), size);
}
void icl_write_buffer(icl_buffer* buf, cl_bool, size_t size, const void* ptr, icl_event*, icl_event*) {
  memcpy(mirror(buf, 0, size), ptr, size);
}
void icl_write_buffer_offset(icl_buffer* buf, cl_bool, size_t off, size_t size, const void* ptr, icl_event*, icl_event*) {
  // the initial Population (src/abms.c:477); with aged eggs the host's copy
  // takes the padded layout the library uses (the pointer is abms.c's own
  // non-const struct)
  if (g.age_days >= 0 && size == sizeof(sampo_population) && off == sizeof(sampo_population) && g.pop_writes++ == 0) {
    sampo_population* p = (sampo_population*)const_cast<void*>(ptr);
    for (int k = 1; k < 8; k++) {
      p->r[k].start = ((p->r[k - 1].end + 64u) / 64u) * 64u;
      p->r[k].end = p->r[k].start;
    }
  }
  memcpy(mirror(buf, off, size), ptr, size);
}
void icl_copy_buffer(icl_buffer* src, icl_buffer* dst, size_t size, icl_event*, icl_event*) {
  memcpy(mirror(dst, 0, size), mirror(src, 0, size), size);
}
void icl_release_buffer(icl_buffer* buf) { delete reinterpret_cast<Buffer*>(buf); }
void icl_release_buffers(cl_uint num, ...) {
  va_list ap;
  va_start(ap, num);
  for (cl_uint i = 0; i < num; i++) icl_release_buffer(va_arg(ap, icl_buffer*));
  va_end(ap);
}

icl_kernel* icl_create_kernel(icl_device* dev, const char*, const char* name, const char* opts, icl_create_kernel_flag) {
  if (opts) {  // "-I<kernel include path> -DSPECIES=<header>" (src/abms.c:566-569)
    const std::string o = opts;
    const size_t s = o.find("-DSPECIES=");
    if (s != std::string::npos) g.species_name = o.substr(s + 10, o.find(' ', s) == std::string::npos ? std::string::npos : o.find(' ', s) - s - 10);
    const size_t i = o.find("-I");
    if (i != std::string::npos) g.include_dir = o.substr(i + 2, o.find(' ', i) == std::string::npos ? std::string::npos : o.find(' ', i) - i - 2);
  }
  Kernel* k = new Kernel();
  k->k.kernel = nullptr;
  k->k.dev = dev;
  k->name = name;
  return &k->k;
}
void icl_release_kernel(icl_kernel* k) { delete reinterpret_cast<Kernel*>(k); }

void icl_run_kernel(const icl_kernel* kernel, cl_uint, const size_t*, const size_t*, icl_event*, icl_event*, cl_uint nargs, ...) {
  size_t size[16];
  void* val[16];
  va_list ap;
  va_start(ap, nargs);
  for (cl_uint i = 0; i < nargs && i < 16; i++) {
    size[i] = va_arg(ap, size_t);
    val[i] = va_arg(ap, void*);
  }
  va_end(ap);
  auto buf = [&](int i) { return (icl_buffer*)val[i]; };
  const std::string& nm = reinterpret_cast<const Kernel*>(kernel)->name;
  if (nm == "initAgents") {
    // (agents, ages, states, EggsNbiomass, temperature, seeds)
    if (!g.have_init) {
      Enb e;
      memcpy(&e, mirror(buf(3), 0, sizeof(e)), sizeof(e));
      g.n0 = e.newEggs;
      g.T0 = *(const float*)val[4];
      memcpy(g.seeds0, mirror(buf(5), 0, sizeof(g.seeds0)), sizeof(g.seeds0));
      g.have_init = true;
    }
  } else if (nm == "calcL1deTotal" || nm == "calcFemalesTotal") {
    // (popD, ...): pop[0] = the population at the step's start. Before the
    // first step: the initial Population the host wrote to pop[1] (eggs
    // only: no larvae, no adults, so its L1de and female counts are 0).
    if (!g.sim) {
      sampo_population p;
      memcpy(&p, mirror(buf(0), sizeof(p), sizeof(p)), sizeof(p));
      p.numLarvae1DayEquiv = p.numFemale = p.numPotentiallyInfective = 0;
      memcpy(mirror(buf(0), 0, sizeof(p)), &p, sizeof(p));
    }
  } else if (nm == "killAgents") {
    // (ages, states, popD, EggsNbiomass, bnc, seeds, carryingCapacity)
    g.capacity = buf(0)->size / kAgentAgeBytes;
    g.cc = *(const float*)val[6];
  } else if (nm == "updateAgents") {
    // (agents, ages, states, popD, Environment, temperature, bnc, EggsNbiomass, seeds, hours, worldTime)
    if (size[4] != sizeof(sampo_environment)) die("struct Environment differs from sampo_environment", nullptr);
    const sampo_environment env = *(const sampo_environment*)val[4];
    const float T = *(const float*)val[5];
    const uint32_t wt = *(const uint32_t*)val[10];
    if (!g.sim) start(env);
    sampo_seeds sd[4];
    memcpy(sd, mirror(buf(8), 0, sizeof(sd)), sizeof(sd));
    sampo_stats_row row;
    if (sampo_step(g.sim, &env, T, wt, sd, &row) != SAMPO_OK) die("sampo_step", sampo_last_error(g.sim));
    publish(buf(3), buf(6));
  } else if (nm == "ageHistogram") {
    // (ages, popD, histogram): the kernel adds to the zeroed histogram
    uint32_t h[100];
    if (!g.sim || sampo_histogram(g.sim, h) != SAMPO_OK) die("sampo_histogram", g.sim ? sampo_last_error(g.sim) : nullptr);
    uint32_t* out = (uint32_t*)mirror(buf(2), 0, sizeof(h));
    for (int i = 0; i < 100; i++) out[i] += h[i];
  }
  // calcL1dePerGroup, calcFemalesPerGroup, preScan, serialScan,
  // oldToNewAgents and the later initAgents launches: done by sampo_step
}

icl_event* icl_create_event() {
  icl_event* e = (icl_event*)malloc(sizeof(icl_event));
  e->event = (cl_event*)calloc(1, sizeof(cl_event));
  e->num_event = 1;
  return e;
}
void icl_release_event(icl_event* e) {
  if (!e) return;
  free(e->event);
  free(e);
}
void icl_release_events(cl_uint num, ...) {
  va_list ap;
  va_start(ap, num);
  for (cl_uint i = 0; i < num; i++) icl_release_event(va_arg(ap, icl_event*));
  va_end(ap);
}
double icl_profile_event(icl_event*, icl_event_flag, icl_event_flag, icl_time_flag) { return 0.0; }

icl_timer* icl_init_timer(icl_time_flag f) {
  icl_timer* t = (icl_timer*)calloc(1, sizeof(icl_timer));
  t->time_flag = f;
  return t;
}
void icl_start_timer(icl_timer* t) { t->start = now_ns(); }
void icl_restart_timer(icl_timer* t) {
  t->current_time = 0;
  t->start = now_ns();
}
double icl_stop_timer(icl_timer* t) {
  const double ns = (double)(now_ns() - t->start);
  const double v = t->time_flag == ICL_SEC ? ns * 1e-9 : t->time_flag == ICL_MILLI ? ns * 1e-6 : ns;
  t->current_time += v;
  return t->current_time;
}
void icl_release_timer(icl_timer* t) { free(t); }

/* include/scan.h: the Bolt scan-by-key of createNewAgents is part of sampo_step. */
void segmented_scan_init(size_t, unsigned int, icl_device*, const char*, icl_create_kernel_flag) {}
void segmented_scan_release() {}
void scan(icl_buffer*, icl_buffer*, unsigned int) {}

}  /* extern "C" */
