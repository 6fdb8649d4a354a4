/*
 * icl_emul.cpp - a host-only implementation of the reference's lib_icl API
 * (include/lib_icl.h:100-159) so that the reference's unmodified
 * src/abms.c and src/boltScan.c run on the CPU. TEST INFRASTRUCTURE ONLY.
 *
 * Buffers are host allocations; icl_run_kernel dispatches on the kernel name
 * to the reference's barrier-free kernels compiled verbatim as C++
 * (k_*.cpp) and loops the work-item index over the global size. The kernels
 * that use work-group barriers are restated here by their effect:
 *   calcL1dePerGroup/Total (kernel/calcL1de.cl:17-93): sum of floor(age/24)
 *     over the larva range of pop[1], copied with the ranges into pop[0];
 *   calcFemalesPerGroup/Total (kernel/calcGender.cl:17-89): adult female and
 *     potentially-infective counts over pop[0];
 *   perBlockScanByKey + intraBlockInclusiveScanByKey + perBlockAdditionByKey
 *     (kernel/boltScan.cl:22-220 driven by src/boltScan.c:36-126): together an
 *     inclusive scan by key plus init; computed whole in the first call.
 * All of these are integer sums, so the restatement is exact.
 *
 * Hooks for pinning (not part of the reference): the seed given to srand is
 * replaced (link with -Wl,--wrap=srand), optional initial ages are applied
 * right after the first initAgents launch, an optional mixed-stage pool file
 * replaces the initial population (below), and a position-dependent hash of
 * the pool written by each oldToNewAgents launch is appended to a file.
 *
 * Pool file (little-endian): the 8 bytes "SAMPOPL1", the eight ranges as
 * uint32 start/end pairs, uint32 n (= the last range's end), then the n
 * slots as the reference's device records: n struct Agent, n struct
 * AgentAge, n struct AgentState (include/agent.h:66-102). Its layout must be
 * one a compaction produces (kernel/oldToNewAgents.cl:57-95): eggs from slot
 * 0, each next range at ((previous end + 64) / 64) * 64. The slots replace
 * what the first initAgents launch wrote, and the ranges replace the host
 * Population that src/abms.c:477 writes to the device (abms.c keeps using
 * the same struct, so its host view agrees).
 */
#include <cstdarg>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <ctime>
#include <string>
extern "C" {
#include "lib_icl.h"
}

thread_local size_t clc_tls_gid = 0;
thread_local size_t clc_tls_gsize = 0;

extern "C" {
void refk_killAgents(size_t, void*, void*, void*, void*, void*, void*, float);
void refk_updateAgents(size_t, void*, void*, void*, void*, const void*, float, void*, void*, void*, float, unsigned);
void refk_initAgents(size_t, void*, void*, void*, void*, float, void*);
void refk_preScan(size_t, void*, void*, void*, void*, unsigned, unsigned, unsigned, unsigned, int);
void refk_oldToNewAgents(size_t, void*, void*, void*, void*, void*, void*, void*, void*, void*, void*, void*);
void refk_ageHistogram(size_t, void*, void*, void*);
size_t refk_environment_size(void);
void __real_srand(unsigned);
}

/* Same layouts as the reference's device structs (include/agent.h:66-123). */
struct EAgent { uint32_t availableEggs, cycleLength, hbc; float delay; uint32_t numEggBatches, uni; };
struct EAgentAge { float age, his; int32_t isFemale; float sporo; };
struct EAgentState { int32_t dead, state; };
struct ERange { uint32_t start, end; };
struct EPop { ERange r[8]; uint32_t L1de, numFemale, numPotInf; };
struct EEnb { int32_t totalBiomass; uint32_t newEggs; };

/* ---- options set by ref_main.c ---- */
extern "C" {
unsigned sampo_ref_seed = 1;
int sampo_ref_age_days = -1;
unsigned long long sampo_ref_age_seed = 0;
const char* sampo_ref_hash_file = nullptr;
const char* sampo_ref_pool_file = nullptr;
}

static EPop g_pool_pop;
static bool g_pool_ready = false;

extern "C" void __wrap_srand(unsigned) { __real_srand(sampo_ref_seed); }

static icl_device g_dev;
static int g_init_launches = 0;
static FILE* g_hash_fp = nullptr;

static inline uint64_t mix64(uint64_t z) {
  z += 0x9E3779B97F4A7C15ULL;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
  return z ^ (z >> 31);
}
static inline uint32_t fbits(float f) { uint32_t u; memcpy(&u, &f, 4); return u; }
static inline uint32_t state_index(int32_t s) { return (uint32_t)__builtin_ctz((unsigned)s); }

static uint64_t pool_hash(const EAgent* a, const EAgentAge* g, const EAgentState* st, const EPop* pop) {
  uint64_t h = 0;
  for (int k = 0; k < 8; k++) {
    h += mix64(((uint64_t)k << 40) ^ ((uint64_t)pop->r[k].start << 20) ^ (uint64_t)pop->r[k].end);
    for (uint64_t i = pop->r[k].start; i < pop->r[k].end; i++) {
      uint64_t x = mix64(i);
      x = mix64(x ^ ((uint64_t)state_index(st[i].state) | ((uint64_t)(g[i].isFemale != 0) << 8)));
      x = mix64(x ^ fbits(g[i].age)); x = mix64(x ^ fbits(g[i].his));
      x = mix64(x ^ fbits(a[i].delay)); x = mix64(x ^ fbits(g[i].sporo));
      x = mix64(x ^ a[i].uni); x = mix64(x ^ a[i].availableEggs); x = mix64(x ^ a[i].cycleLength);
      x = mix64(x ^ a[i].hbc); x = mix64(x ^ a[i].numEggBatches);
      h += x;
    }
  }
  return h;
}

extern "C" {

cl_int clFinish(cl_command_queue) { return CL_SUCCESS; }
cl_int clWaitForEvents(cl_uint, const cl_event*) { return CL_SUCCESS; }

void icl_init_devices(cl_device_type) {
  memset(&g_dev, 0, sizeof(g_dev));
  g_dev.name = (char*)"ref-as-C (reference kernels compiled for the host CPU)";
  g_dev.vendor = (char*)"sampo-gb300 oracle";
  g_dev.version = (char*)"OpenCL 1.2 emulation";
  g_dev.type = CL_DEVICE_TYPE_CPU;
}
cl_uint icl_get_num_devices() { return 1; }
icl_device* icl_get_device(cl_uint) { return &g_dev; }
void icl_release_devices() {
  if (g_hash_fp) { fclose(g_hash_fp); g_hash_fp = nullptr; }
}

icl_buffer* icl_create_buffer(icl_device* dev, cl_mem_flags, size_t size) {
  icl_buffer* b = (icl_buffer*)malloc(sizeof(icl_buffer));
  b->mem = (cl_mem)calloc(size ? size : 1, 1);
  if (!b->mem) { fprintf(stderr, "icl_emul: out of host memory (%zu bytes)\n", size); exit(-1); }
  b->size = size;
  b->dev = dev;
  return b;
}
void icl_read_buffer(const icl_buffer* buf, cl_bool, size_t size, void* ptr, icl_event*, icl_event*) {
  memcpy(ptr, buf->mem, size);
}
void icl_read_buffer_offset(const icl_buffer* buf, cl_bool, size_t off, size_t size, void* ptr, icl_event*, icl_event*) {
  memcpy(ptr, (char*)buf->mem + off, size);
}
void icl_write_buffer(icl_buffer* buf, cl_bool, size_t size, const void* ptr, icl_event*, icl_event*) {
  memcpy(buf->mem, ptr, size);
}
static int g_pop_writes = 0;
void icl_write_buffer_offset(icl_buffer* buf, cl_bool, size_t off, size_t size, const void* ptr, icl_event*, icl_event*) {
  /* src/abms.c:477 writes the host copy of the initial Population into
   * pop[1]. With aged initial eggs (an extension) the host copy is switched
   * to the padded layout first (the same one the CPU port and the CUDA path
   * use); the pointer is abms.c's own non-const struct. */
  if (g_pool_ready && size == sizeof(EPop) && off == sizeof(EPop) && g_pop_writes == 0) {
    g_pop_writes++;
    EPop* p = (EPop*)const_cast<void*>(ptr);
    for (int k = 0; k < 8; k++) p->r[k] = g_pool_pop.r[k];
  } else if (sampo_ref_age_days >= 0 && size == sizeof(EPop) && off == sizeof(EPop) && g_pop_writes++ == 0) {
    EPop* p = (EPop*)const_cast<void*>(ptr);
    for (int k = 1; k < 8; k++) {
      p->r[k].start = ((p->r[k - 1].end + 64u) / 64u) * 64u;
      p->r[k].end = p->r[k].start;
    }
  }
  memcpy((char*)buf->mem + off, ptr, size);
}
void icl_copy_buffer(icl_buffer* src, icl_buffer* dst, size_t size, icl_event*, icl_event*) {
  memcpy(dst->mem, src->mem, size);
}
void icl_release_buffer(icl_buffer* buf) {
  if (!buf) return;
  free(buf->mem);
  free(buf);
}
void icl_release_buffers(cl_uint num, ...) {
  va_list ap;
  va_start(ap, num);
  for (cl_uint i = 0; i < num; i++) icl_release_buffer(va_arg(ap, icl_buffer*));
  va_end(ap);
}

// the species header the kernel objects were compiled with (-DSPECIES)
#ifndef REF_SPECIES_NAME
#define REF_SPECIES_NAME "properties.h"
#endif

struct EKernel { std::string name; };

icl_kernel* icl_create_kernel(icl_device* dev, const char* file, const char* name, const char* opts, icl_create_kernel_flag) {
  if (opts && !strstr(opts, "SPECIES=" REF_SPECIES_NAME)) {
    fprintf(stderr, "icl_emul: only the shipped species header is compiled in (%s)\n", opts);
    exit(-1);
  }
  (void)file;
  icl_kernel* k = (icl_kernel*)malloc(sizeof(icl_kernel));
  k->kernel = (cl_kernel)(void*)new EKernel{name};
  k->dev = dev;
  return k;
}
void icl_release_kernel(icl_kernel* k) {
  if (!k) return;
  delete (EKernel*)(void*)k->kernel;
  free(k);
}

/* Arguments arrive as (size, pointer) pairs; size 0 means an icl_buffer*. */
struct Args {
  size_t size[16];
  void* val[16];
  void* buf(int i) const { return ((icl_buffer*)val[i])->mem; }
  float f(int i) const { return *(const float*)val[i]; }
  uint32_t u(int i) const { return *(const uint32_t*)val[i]; }
  int32_t s(int i) const { return *(const int32_t*)val[i]; }
};

static void apply_initial_ages(EAgentAge* g, uint32_t n) {
  if (sampo_ref_age_days < 0) return;
  uint64_t m = (uint64_t)sampo_ref_age_days + 1;
  for (uint32_t i = 0; i < n; i++) {
    uint64_t z = mix64(sampo_ref_age_seed ^ mix64((uint64_t)i));
    float h = 24.0f * (float)(uint32_t)((z >> 32) % m);
    g[i].age = h; g[i].his = h;
  }
}

static void load_pool_file(icl_buffer* agents, icl_buffer* ages, icl_buffer* states) {
  FILE* f = fopen(sampo_ref_pool_file, "rb");
  char magic[8];
  uint32_t rg[16], n = 0;
  bool ok = f && fread(magic, 8, 1, f) == 1 && memcmp(magic, "SAMPOPL1", 8) == 0 && fread(rg, sizeof(rg), 1, f) == 1 &&
            fread(&n, 4, 1, f) == 1 && n == rg[15] && rg[0] == 0;
  for (int k = 1; k < 8 && ok; k++) ok = rg[2 * k] == ((rg[2 * k - 1] + 64u) / 64u) * 64u && rg[2 * k + 1] >= rg[2 * k];
  ok = ok && (size_t)n * sizeof(EAgent) <= agents->size && (size_t)n * sizeof(EAgentAge) <= ages->size &&
       (size_t)n * sizeof(EAgentState) <= states->size;
  ok = ok && fread(agents->mem, sizeof(EAgent), n, f) == n && fread(ages->mem, sizeof(EAgentAge), n, f) == n &&
       fread(states->mem, sizeof(EAgentState), n, f) == n;
  if (f) fclose(f);
  if (!ok) {
    fprintf(stderr, "icl_emul: bad pool file %s\n", sampo_ref_pool_file);
    exit(-1);
  }
  for (int k = 0; k < 8; k++) g_pool_pop.r[k] = ERange{rg[2 * k], rg[2 * k + 1]};
  g_pool_ready = true;
}

void icl_run_kernel(const icl_kernel* kernel, cl_uint, const size_t* gws, const size_t*, icl_event*, icl_event*, cl_uint nargs, ...) {
  Args a;
  va_list ap;
  va_start(ap, nargs);
  for (cl_uint i = 0; i < nargs && i < 16; i++) {
    a.size[i] = va_arg(ap, size_t);
    a.val[i] = va_arg(ap, void*);
  }
  va_end(ap);
  const std::string& nm = ((EKernel*)(void*)kernel->kernel)->name;
  size_t G = gws[0];

  if (nm == "initAgents") {
    refk_initAgents(G, a.buf(0), a.buf(1), a.buf(2), a.buf(3), a.f(4), a.buf(5));
    if (g_init_launches++ == 0) {
      if (sampo_ref_pool_file) load_pool_file((icl_buffer*)a.val[0], (icl_buffer*)a.val[1], (icl_buffer*)a.val[2]);
      else apply_initial_ages((EAgentAge*)a.buf(1), ((EEnb*)a.buf(3))->newEggs);
    }
  } else if (nm == "killAgents") {
    refk_killAgents(G, a.buf(0), a.buf(1), a.buf(2), a.buf(3), a.buf(4), a.buf(5), a.f(6));
  } else if (nm == "updateAgents") {
    if (a.size[4] != refk_environment_size()) { fprintf(stderr, "icl_emul: Environment size mismatch\n"); exit(-1); }
    refk_updateAgents(G, a.buf(0), a.buf(1), a.buf(2), a.buf(3), a.val[4], a.f(5), a.buf(6), a.buf(7), a.buf(8), a.f(9), a.u(10));
  } else if (nm == "preScan") {
    refk_preScan(G, a.buf(0), a.buf(1), a.buf(2), a.buf(3), a.u(4), a.u(5), a.u(6), a.u(7), a.s(8));
  } else if (nm == "oldToNewAgents") {
    refk_oldToNewAgents(G, a.buf(0), a.buf(1), a.buf(2), a.buf(3), a.buf(4), a.buf(5), a.buf(6), a.buf(7), a.buf(8), a.buf(9), a.buf(10));
    if (sampo_ref_hash_file) {
      if (!g_hash_fp) g_hash_fp = fopen(sampo_ref_hash_file, "w");
      EPop* pop = (EPop*)a.buf(9);
      uint64_t h = pool_hash((EAgent*)a.buf(3), (EAgentAge*)a.buf(4), (EAgentState*)a.buf(5), &pop[1]);
      fprintf(g_hash_fp, "%016llx\n", (unsigned long long)h);
    }
  } else if (nm == "ageHistogram") {
    refk_ageHistogram(G, a.buf(0), a.buf(1), a.buf(2));
  } else if (nm == "calcL1dePerGroup") {
    const EAgentAge* g = (const EAgentAge*)a.buf(0);
    const EPop* pop = (const EPop*)a.buf(1);
    uint32_t* part = (uint32_t*)a.buf(2);
    if (pop[1].r[1].end > pop[1].r[1].start) {
      uint32_t s = 0;
      for (uint32_t i = pop[1].r[1].start; i < pop[1].r[1].end; i++) s += (uint32_t)(g[i].age / 24.0f);
      part[0] = s;
      for (int i = 1; i < 64; i++) part[i] = 0;
    }
  } else if (nm == "calcL1deTotal") {
    EPop* pop = (EPop*)a.buf(0);
    const uint32_t* part = (const uint32_t*)a.buf(1);
    uint32_t slots = a.u(2), tot = 0;
    if (pop[1].r[1].end - pop[1].r[1].start != 0)
      for (uint32_t i = 0; i < 64 && i < slots; i++) tot += part[i];
    EPop p = pop[1];
    p.L1de = tot;
    pop[0] = p;
  } else if (nm == "calcFemalesPerGroup") {
    const EAgentAge* g = (const EAgentAge*)a.buf(0);
    const EPop* pop = (const EPop*)a.buf(1);
    uint32_t* part = (uint32_t*)a.buf(2);
    uint32_t fem = 0, inf = 0;
    for (int k = 3; k < 8; k++)
      for (uint32_t i = pop[0].r[k].start; i < pop[0].r[k].end; i++)
        if (g[i].isFemale) { fem++; inf += g[i].sporo >= 1.0f; }
    for (int i = 0; i < 128; i++) part[i] = 0;
    part[0] = fem; part[64] = inf;
  } else if (nm == "calcFemalesTotal") {
    EPop* pop = (EPop*)a.buf(0);
    const uint32_t* part = (const uint32_t*)a.buf(1);
    uint32_t fem = 0, inf = 0;
    for (int i = 0; i < 64; i++) { fem += part[i]; inf += part[64 + i]; }
    pop[0].numFemale = fem; pop[0].numPotInf = inf;
  } else if (nm == "perBlockScanByKey") {
    const uint32_t* keys = (const uint32_t*)a.buf(0);
    int32_t* vals = (int32_t*)a.buf(1);
    int32_t init = a.s(2);
    uint32_t n = a.u(3);
    int32_t run = 0;
    for (uint32_t i = 0; i < n; i++) {
      if (i == 0 || keys[i] != keys[i - 1]) run = 0;
      run += vals[i];
      vals[i] = run + init;
    }
  } else if (nm == "intraBlockInclusiveScanByKey" || nm == "perBlockAdditionByKey") {
    /* folded into perBlockScanByKey above */
  } else {
    fprintf(stderr, "icl_emul: unknown kernel %s\n", nm.c_str());
    exit(-1);
  }
}

void icl_print_device_short_info(icl_device* dev) {
  printf("CPU: %s | %s | %s\n", dev->name, dev->vendor, dev->version);
}
void icl_print_device_infos(icl_device* dev) { icl_print_device_short_info(dev); }

icl_event* icl_create_event() {
  icl_event* e = (icl_event*)malloc(sizeof(icl_event));
  e->event = (cl_event*)malloc(sizeof(cl_event));
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

static long long now_ns() {
  struct timespec ts;
  clock_gettime(CLOCK_MONOTONIC, &ts);
  return (long long)ts.tv_sec * 1000000000LL + ts.tv_nsec;
}
icl_timer* icl_init_timer(icl_time_flag f) {
  icl_timer* t = (icl_timer*)calloc(1, sizeof(icl_timer));
  t->time_flag = f;
  return t;
}
void icl_start_timer(icl_timer* t) { t->start = now_ns(); }
void icl_restart_timer(icl_timer* t) { t->current_time = 0; t->start = now_ns(); }
double icl_stop_timer(icl_timer* t) {
  double ns = (double)(now_ns() - t->start);
  double v = t->time_flag == ICL_SEC ? ns * 1e-9 : t->time_flag == ICL_MILLI ? ns * 1e-6 : ns;
  t->current_time += v;
  return t->current_time;
}
void icl_release_timer(icl_timer* t) { free(t); }

} /* extern "C" */
