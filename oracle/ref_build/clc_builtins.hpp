/*
 * OpenCL C built-ins needed to compile the reference's kernel/*.cl files as
 * C++ (TEST INFRASTRUCTURE ONLY). Included INSIDE the namespace that wraps
 * each kernel file, so unqualified calls such as exp(x) or min(a,b) in the
 * kernel resolve to these overloads and not to <math.h>.
 *
 *  - get_global_id/get_global_size read the work-item index the emulator's
 *    dispatch loop sets before each call.
 *  - atomic_add/atomic_inc are relaxed atomic read-modify-writes (the
 *    dispatch loop runs work-items on several threads).
 *  - exp/log/sin/pow use the project's deterministic definitions
 *    (sampo_gb300/csrc/sampo_math.h), the same ones the CPU port and the
 *    CUDA kernels use. sqrt and ceil are exact IEEE operations.
 *  - float min/max are IEEE minNum/maxNum (a NaN operand is ignored).
 */
typedef unsigned int uint;

static inline size_t get_global_id(uint) { return clc_tls_gid; }
static inline size_t get_global_size(uint) { return clc_tls_gsize; }
/* work-group id for a local size of 64 (the only size the reference's
 * barrier-free kernels are launched with); only read, never used. */
static inline size_t get_group_id(uint) { return clc_tls_gid / 64; }

static inline uint atomic_add(uint* p, uint v) { return __atomic_fetch_add(p, v, __ATOMIC_RELAXED); }
static inline int atomic_add(int* p, int v) { return __atomic_fetch_add(p, v, __ATOMIC_RELAXED); }
static inline uint atomic_inc(uint* p) { return __atomic_fetch_add(p, 1u, __ATOMIC_RELAXED); }

static inline float exp(float x) { return sampo_expf(x); }
static inline float log(float x) { return sampo_logf(x); }
static inline float sin(float x) { return sampo_sinf(x); }
static inline float pow(float x, float y) { return sampo_powf(x, y); }
static inline float sqrt(float x) { return sqrtf(x); }
static inline float ceil(float x) { return ceilf(x); }

static inline float min(float a, float b) { return sampo_fminf(a, b); }
static inline float max(float a, float b) { return sampo_fmaxf(a, b); }
static inline uint min(uint a, uint b) { return a < b ? a : b; }
static inline uint max(uint a, uint b) { return a > b ? a : b; }
static inline int min(int a, int b) { return a < b ? a : b; }
static inline int max(int a, int b) { return a > b ? a : b; }

#define M_PI_F 3.14159274101257f
