// sampo_species_prelude.h - the OpenCL C a properties.h-style species header
// is written against, for compiling it into the step kernels with NVRTC.
// Included inside namespace sampo_user, right before the user's header (the
// loader registers empty device_types.h, agent.h and gpuRand.h, so the
// header's own includes resolve to this file's definitions).
//
//  - types and qualifiers of include/device_types.h (REAL = float, the
//    address-space qualifiers empty: the kernels are compiled with
//    -default-device, so the header's functions and tables are device code);
//  - the structs a species function receives (include/agent.h: Agent,
//    AgentState, EggsNbiomass, State with its bit values);
//  - Seeds: one generator slot of the step as the header sees it (the two
//    seed words that do not depend on the slot index already folded, as the
//    kernels keep them) plus the slot index; HybridTaus and BoxMuller give
//    exactly the kernels' draws (include/gpuRand.h:33-63);
//  - exp/log/sin/pow through this library's deterministic functions (the
//    values the CPU oracle and the built-in species use), float min/max as
//    IEEE minNum/maxNum, sqrt and ceil exact;
//  - atomic_add/atomic_inc on the EggsNbiomass the adapter passes (a
//    per-agent copy, so plain adds).

typedef unsigned int uint;
#define REAL float
#define INT int
#define UINT uint
#define BOOL bool
#define __kernel
#define __global
#define __constant
#define __local
#define __private
#define M_PI_F 3.14159274101257f
#ifndef LOCAL_SIZE
#define LOCAL_SIZE 64
#endif
typedef REAL Temperature;

struct EggsNbiomass {
  INT totalBiomass;
  UINT newEggs;
};
struct BitesNcycles {
  UINT numCyclesReported;
  UINT sumCyclesReported;
  UINT numBitesReported;
  UINT numInfectBitesReported;
};
enum State { EGG = 1, LARVA = 2, PUPA = 4, IMMATURE = 8, MATESEEKING = 16, BMS = 32, BMD = 64, GRAVID = 128 };
#ifndef MAX_OVIPOSITION_ATTEMPTS
#define MAX_OVIPOSITION_ATTEMPTS 3
#endif
struct Agent {
  UINT availableEggs;
  UINT cycleLength;
  UINT humanBloodmealCount;
  REAL delay;
  UINT numEggBatches;
  union {
    UINT ovipositionAttemps;
    REAL cumulativeLarvalDelay;
  };
};
struct AgentState {
  BOOL dead;
  enum State state;
};

struct Seeds {
  uint c13, z2, z4, gid;
};

static inline REAL HybridTaus(const struct Seeds* s) { return ::sampo::rng_folded(s->c13, s->z2, s->z4, s->gid); }
static inline REAL BoxMuller(const struct Seeds* s, REAL mean, REAL stdDev) {
  return ::sampo::box_muller_u(HybridTaus(&s[0]), HybridTaus(&s[1]), mean, stdDev);
}

static inline float exp(float x) { return sampo_expf(x); }
static inline float log(float x) { return sampo_logf(x); }
static inline float sin(float x) { return sampo_sinf(x); }
static inline float pow(float x, float y) { return sampo_powf(x, y); }
static inline float sqrt(float x) { return __fsqrt_rn(x); }
static inline float ceil(float x) { return ceilf(x); }
static inline float floor(float x) { return floorf(x); }
static inline float fabs(float x) { return fabsf(x); }
static inline float min(float a, float b) { return sampo_fminf(a, b); }
static inline float max(float a, float b) { return sampo_fmaxf(a, b); }
static inline uint min(uint a, uint b) { return a < b ? a : b; }
static inline uint max(uint a, uint b) { return a > b ? a : b; }
static inline int min(int a, int b) { return a < b ? a : b; }
static inline int max(int a, int b) { return a > b ? a : b; }
static inline float clamp(float x, float lo, float hi) { return min(max(x, lo), hi); }

static inline uint atomic_add(uint* p, uint v) { const uint o = *p; *p = o + v; return o; }
static inline int atomic_add(int* p, int v) { const int o = *p; *p = o + v; return o; }
static inline uint atomic_inc(uint* p) { const uint o = *p; *p = o + 1u; return o; }
