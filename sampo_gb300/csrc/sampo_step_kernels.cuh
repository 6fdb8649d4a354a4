// sampo_step_kernels.cuh - the device code of the SAMPO hourly step (sm_103a):
// helpers, k_count, k_publish, k_scatter and the pool kernels. Compiled into
// the library by nvcc (sampo_kernels.cu) and, for a user species header, at
// run time by NVRTC (sampo_species.cu).
//
// A step of a batch of simulations is two persistent-CTA kernels over every
// active replicate's current pool buffer, whose 1024-slot tiles they take
// from one ticket counter, and a small one with a CTA per replicate:
//
//  k_count   reads the ~12 bytes per agent that decide survival, the next
//            state and the eggs laid (killAgents + the decision part of
//            updateAgents), and publishes per tile the number of survivors
//            per next state, the tile's prefix table over its (round, warp)
//            chunks, and the replicate's newEggs total.
//  k_scatter recomputes the same decisions with the complete record,
//            obtains each survivor's stable rank within its next state
//            (warp match/popc, the tile's prefix table, and a decoupled
//            look-back over the tile counts that k_count already published,
//            within the replicate, so no CTA ever waits on another and the
//            consumer warps share no barrier), writes the updated
//            record to its slot in the other buffer (the reference's
//            oldToNewAgents layout, kernel/oldToNewAgents.cl:57-95,126-226),
//            writes the new eggs at [0, newEggs) (initAgents,
//            kernel/initAgents.cl:26-65), and accumulates the next step's
//            statistics (calcL1de.cl, calcGender.cl).
//  k_publish turns each replicate's counts into its next population, stats
//            row, step constants and larval mortality table.
//
// Both kernels stream tiles through shared memory with TMA bulk copies
// (cp.async.bulk + mbarrier, double-buffered: tile j+1 is in flight while
// tile j is processed). k_count loads only the columns the tile's ranges
// need. In k_scatter a producer warp claims and describes tiles ahead and
// issues their loads; the eight consumer warps release a stage as soon as
// they have read it and write every survivor from registers straight to its
// slot in the next buffer (a next state's survivors are contiguous within a
// warp, so these stores coalesce).
//
// This replaces the reference's 19 kernels per step (killAgents,
// updateAgents, initAgents, 3 x preScan + 3 x Bolt scan-by-key,
// oldToNewAgents, calcL1de x2, calcFemales x2) and its blocking transfers.
#pragma once
#include "sampo_kernels.cuh"

namespace sampo {


constexpr uint32_t kColBytes = kTile * 4;                    // one 4-byte column of a tile
constexpr uint32_t kCountStage = 5 * kColBytes + kTile;      // age, his, delay, uni, avail, flags
constexpr uint32_t kPreOff = 9 * kColBytes + kTile;          // the nine 4-byte columns and the flags,
constexpr uint32_t kScatterStage = kPreOff + kPreWords * 4;   // then the tile's prefix table
static_assert(kPreOff % 16 == 0 && kScatterStage % 16 == 0, "bulk copies land on 16-byte boundaries");

// The count and update/scatter passes are built for I slots per thread
// (tiles of 256 * I slots: I = 2 or 4, picked per workload by the
// autotuner). Inside them these local constants stand for the tile sizes
// above, which are those of I = 4.
#define SAMPO_TILE_CONSTANTS(I)                                                         \
  constexpr int kItems = (I);                                                         \
  constexpr int kTile = kBlock * (I);                                                 \
  constexpr uint32_t kChunks = (uint32_t)(I) * kWarps;                                \
  constexpr uint32_t kPreWords = ((kChunks + 1) * kPreEntryWords + 3) / 4 * 4;        \
  constexpr uint32_t kColBytes = (uint32_t)kTile * 4;                                 \
  constexpr uint32_t kCountStage = 5 * kColBytes + kTile;                             \
  constexpr uint32_t kPreOff = 9 * kColBytes + kTile;                                 \
  constexpr uint32_t kScatterStage = kPreOff + kPreWords * 4;                         \
  constexpr size_t kCountSmem = 2 * (size_t)kCountStage;                              \
  constexpr size_t kScatterSmem = 2 * (size_t)kScatterStage;                          \
  static_assert(kPreOff % 16 == 0 && kScatterStage % 16 == 0 && kChunks <= 32 && kPreWords <= kPreWordsMax, \
                "bulk copies land on 16-byte boundaries; one chunk per lane; tables fit the tile arrays"); \
  (void)kItems; (void)kChunks; (void)kCountSmem; (void)kScatterSmem
constexpr uint32_t kWaitLimit = 1u << 22;                    // bounded mbarrier waits

// ---------------- memory-model and TMA helpers ----------------
__device__ __forceinline__ uint4 ld_cg_v4(const uint32_t* p) {
  uint4 v;
  asm volatile("ld.global.cg.v4.u32 {%0,%1,%2,%3}, [%4];" : "=r"(v.x), "=r"(v.y), "=r"(v.z), "=r"(v.w) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ uint32_t lanemask_lt() {
  uint32_t m;
  asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
  return m;
}
__device__ __forceinline__ uint32_t smem_addr(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }
__device__ __forceinline__ void mbar_init(uint64_t* bar) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_addr(bar)) : "memory");
}
__device__ __forceinline__ void fence_mbar_init() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }
__device__ __forceinline__ void fence_proxy_async() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
__device__ __forceinline__ void mbar_arrive_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes) : "memory");
}
__device__ __forceinline__ void mbar_init_count(uint64_t* bar, uint32_t n) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(n) : "memory");
}
__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_addr(bar)) : "memory");
}
// 1-D bulk copy global -> shared, completion counted on bar (both addresses
// 16-byte aligned, bytes a multiple of 16).
__device__ __forceinline__ void bulk_load(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
               ::"r"(smem_addr(dst)), "l"(src), "r"(bytes), "r"(smem_addr(bar)) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile("{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n}"
               : "=r"(ok) : "r"(smem_addr(bar)), "r"(parity) : "memory");
  return ok != 0;
}
// Waits for the phase with the given parity; gives up after kWaitLimit polls.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity) {
  for (uint32_t i = 0; i < kWaitLimit; i++)
    if (mbar_try_wait(bar, parity)) return true;
  return false;
}

// Range of slot g in the current layout, -1 for gaps and the tail
// (the validity test of every reference kernel, e.g. kernel/killAgents.cl:28-35).
__device__ __forceinline__ int range_of(const sampo_population& pop, uint32_t g) {
  if (g < pop.r[0].end) return 0;
#pragma unroll
  for (int k = 1; k < 8; k++) {
    if (g < pop.r[k].start) return -1;
    if (g < pop.r[k].end) return k;
  }
  return -1;
}

// Layout of the next pool from the survivor counts (kernel/oldToNewAgents.cl:57-95).
__device__ __forceinline__ void next_layout(const uint32_t cnt[8], uint32_t newEggs, sampo_population& np, uint32_t base[8]) {
  np.r[0].start = 0;
  np.r[0].end = newEggs + cnt[0];
  base[0] = newEggs;
#pragma unroll
  for (int k = 1; k < 8; k++) {
    np.r[k].start = ((np.r[k - 1].end + kLayoutAlign) / kLayoutAlign) * kLayoutAlign;
    np.r[k].end = np.r[k].start + cnt[k];
    base[k] = np.r[k].start;
  }
  np.numLarvae1DayEquiv = 0; np.numFemale = 0; np.numPotentiallyInfective = 0;
}

// Whether the next layout (kernel/oldToNewAgents.cl:57-95) fits in one buffer.
__device__ __forceinline__ bool layout_fits(const uint32_t cnt[8], uint32_t newEggs, uint32_t capacity) {
  const uint64_t tot = (uint64_t)newEggs + cnt[0];
  uint64_t e = tot;
#pragma unroll
  for (int k = 1; k < 8; k++) e = ((e + kLayoutAlign) / kLayoutAlign) * kLayoutAlign + cnt[k];
  return tot <= 0xffffffffull && e <= (uint64_t)capacity;
}

// The inputs of step `step` of one replicate (its ring slot).
struct CtxInputs {
  sampo_seeds sd[4];
  sampo_environment env;
  float T;
  uint32_t wt;
};
__device__ __forceinline__ void load_ctx_inputs(const RepParams& rp, uint32_t step, CtxInputs& in) {
  const uint32_t i = step % rp.ring;
#pragma unroll
  for (int k = 0; k < 4; k++) in.sd[k] = rp.seeds[(size_t)i * 4 + k];
  in.env = rp.env[i];
  in.T = rp.T[i];
  in.wt = rp.wt[i];
}

// The constants of a step of one simulation starting from `pop`, from the
// step's inputs: HybridTaus with z1 and z3 folded per seed slot
// (include/gpuRand.h:33-50), the species functions of the step's temperature
// (include/properties.h) and the biomass of the pool
// (kernel/killAgents.cl:42-43). The larval mortality table is filled
// separately (k_publish).
__device__ void make_ctx(const CtxInputs& in, const float* larvaHMR, const sampo_population& pop, StepCtx& c) {
  c.larvaHMR = larvaHMR;
#pragma unroll
  for (int k = 0; k < 4; k++) {
    c.rng_c13[k] = taus_step(in.sd[k].z1 + 128u, 13, 19, 12, 4294967294u) ^ taus_step(in.sd[k].z3 + 128u, 3, 11, 17, 4294967280u);
    c.rng_z2[k] = in.sd[k].z2 + 128u;
    c.rng_z4[k] = in.sd[k].z4;
  }
  c.env = in.env;
  const float T = in.T;
  c.T = T;
  c.wt = in.wt;
  c.totalBiomass = pop.numLarvae1DayEquiv + pop.r[EGG].end + (pop.r[PUPA].end - pop.r[PUPA].start);
  species_step(T, c.wt, c);
  c.sporoOn = T > 16.0f;                                             // kernel/updateAgents.cl:69-70
  c.sporoInc = __ddiv_rn(1.0, __dmul_rn((double)(111.0f / (T - 16.0f)), 14.0));
  sampo_split_double(c.sporoInc, &c.sporoH, &c.sporoM, &c.sporoL);
}

// generateSeeds (src/abms.c:145-150) on the device: the 16 rand() draws of a
// step (z1..z4 of seed slots 0..3) from the replicate's rotated glibc TYPE_3
// state, by one warp. Lane j holds r[j]; draw k is r[k] + r[k+28] for k < 3
// and r[k] + draw(k-3) after that, resolved in five shuffle rounds. The draws
// go to the step's ring slot (output = value >> 1) and the state keeps the 31
// newest values, oldest first.
__device__ void draw_step_seeds(const RepParams& rp, uint32_t step) {
  DevSeedStream& s = rp.sim->rnd;
  const uint32_t lane = threadIdx.x & 31u;
  const uint32_t x = lane < 31u ? s.st.r[lane] : 0u;
  uint32_t v = x + __shfl_sync(0xffffffffu, x, (lane + 28u) & 31u);  // final on lanes 0..2
#pragma unroll
  for (int it = 0; it < 5; it++) {  // after round it, lanes below 3 * (it + 2) are final
    const uint32_t prev = __shfl_up_sync(0xffffffffu, v, 3);
    if (lane >= 3u) v = x + prev;
  }
  uint32_t* out = reinterpret_cast<uint32_t*>(rp.seeds + (size_t)(step % rp.ring) * 4);
  if (lane < 16u) out[lane] = v >> 1;
  const uint32_t kept = __shfl_sync(0xffffffffu, x, (lane + 16u) & 31u);
  const uint32_t drawn = __shfl_sync(0xffffffffu, v, (lane + 17u) & 31u);  // lane j >= 15: draw j - 15
  if (lane < 31u) s.st.r[lane] = lane < 15u ? kept : drawn;
  if (lane == 0u) s.next = step + 1u;
}

template <class T>
__device__ void load_model_const(const T* g, T& s) {
  const float* src = reinterpret_cast<const float*>(g);
  float* dst = reinterpret_cast<float*>(&s);
  for (int k = threadIdx.x; k < (int)(sizeof(T) / 4); k += blockDim.x) dst[k] = src[k];
}

// Exclusive scan of one value per thread over the CTA (blockDim.x a multiple
// of 32); s_w holds 33 words. Ends with all threads synchronised.
__device__ uint32_t block_exclusive_scan(uint32_t v, uint32_t* s_w, uint32_t* total) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  uint32_t incl = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t y = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o) incl += y;
  }
  if (lane == 31) s_w[warp] = incl;
  __syncthreads();
  if (warp == 0) {
    const uint32_t w = lane < nw ? s_w[lane] : 0u;
    uint32_t wi = w;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t y = __shfl_up_sync(0xffffffffu, wi, o);
      if (lane >= o) wi += y;
    }
    s_w[lane] = wi - w;
    if (lane == 31) s_w[32] = wi;
  }
  __syncthreads();
  const uint32_t r = s_w[warp] + incl - v;
  *total = s_w[32];
  __syncthreads();
  return r;
}

// Ticket ranges of a pass over the batch: replicate r owns tickets
// [s_pre[r], s_pre[r+1]); s_pre[nrep] is the number of tickets. tiles(r) is
// r's tile count in this pass. All threads; ends synchronised.
template <class F>
__device__ void plan_tickets(uint32_t nrep, uint32_t* s_pre, uint32_t* s_w, F tiles) {
  if (nrep == 1) {  // a single simulation
    if (threadIdx.x == 0) {
      s_pre[0] = 0;
      s_pre[1] = tiles(0u);
    }
    __syncthreads();
    return;
  }
  const uint32_t per = (nrep + blockDim.x - 1) / blockDim.x;  // <= 4: nrep <= kMaxRep, blockDim.x >= 256
  const uint32_t r0 = min(threadIdx.x * per, nrep), r1 = min(r0 + per, nrep);
  uint32_t loc[4], sum = 0;
#pragma unroll
  for (int k = 0; k < 4; k++) {
    loc[k] = r0 + k < r1 ? tiles(r0 + k) : 0u;
    sum += loc[k];
  }
  uint32_t total;
  uint32_t run = block_exclusive_scan(sum, s_w, &total);
#pragma unroll
  for (int k = 0; k < 4; k++) {
    if (r0 + k < r1) s_pre[r0 + k] = run;
    run += loc[k];
  }
  if (threadIdx.x == 0) s_pre[nrep] = total;
  __syncthreads();
}

// The replicate owning ticket t < s_pre[nrep].
__device__ __forceinline__ uint32_t find_rep(const uint32_t* s_pre, uint32_t nrep, uint32_t t) {
  uint32_t lo = 0, hi = nrep;  // s_pre[lo] <= t < s_pre[hi]
  while (hi - lo > 1) {
    const uint32_t mid = (lo + hi) >> 1;
    if (s_pre[mid] <= t) lo = mid;
    else hi = mid;
  }
  return lo;
}

__device__ __forceinline__ void copy16(void* dst, const void* src, int bytes, int i, int n) {
  const uint4* s = reinterpret_cast<const uint4*>(src);
  uint4* d = reinterpret_cast<uint4*>(dst);
  for (int k = i; k < bytes / 16; k += n) d[k] = s[k];
}
static_assert(sizeof(StepCtx) % 16 == 0, "StepCtx is copied in 16-byte words");

// ------------------------------------------------------------------------
// Count pass
// ------------------------------------------------------------------------
enum : uint32_t { CA_AGE = 1, CA_HIS = 2, CA_DELAY = 4, CA_UNI = 8, CA_AVAIL = 16, CA_FLAGS = 32 };

// Columns the decision part of the update reads, by range (see update_agent<false>).
__device__ __forceinline__ uint32_t count_cols(int rg, bool larvicide) {
  switch (rg) {
    case EGG: case PUPA: return CA_HIS | CA_DELAY;
    case LARVA: return CA_AGE | CA_UNI | CA_DELAY | (larvicide ? CA_HIS : 0u);
    case MATESEEKING: return CA_AGE | CA_HIS | CA_DELAY | CA_FLAGS;
    case GRAVID: return CA_AGE | CA_AVAIL | CA_UNI;
    default: return CA_AGE | CA_HIS | CA_DELAY;  // IMMATURE, BMS, BMD
  }
}

template <int I>
__device__ void issue_count_tile(const DevPool& src, uint8_t* st, uint64_t* bar, const sampo_population& pop,
                                 uint32_t lo, uint32_t n, bool larvicide) {
  SAMPO_TILE_CONSTANTS(I);
  uint32_t m = 0;
  for (int k = 0; k < 8; k++)
    if (pop.r[k].end > pop.r[k].start && pop.r[k].start < lo + n && pop.r[k].end > lo) m |= count_cols(k, larvicide);
  const uint32_t b4 = (n * 4 + 15) & ~15u, b1 = (n + 15) & ~15u;
  uint32_t tx = __popc(m & 31u) * b4 + ((m & CA_FLAGS) ? b1 : 0u);
  mbar_arrive_tx(bar, tx);
  if (m & CA_AGE) bulk_load(st + 0 * kColBytes, src.age + lo, b4, bar);
  if (m & CA_HIS) bulk_load(st + 1 * kColBytes, src.his + lo, b4, bar);
  if (m & CA_DELAY) bulk_load(st + 2 * kColBytes, src.delay + lo, b4, bar);
  if (m & CA_UNI) bulk_load(st + 3 * kColBytes, src.uni + lo, b4, bar);
  if (m & CA_AVAIL) bulk_load(st + 4 * kColBytes, src.avail + lo, b4, bar);
  if (m & CA_FLAGS) bulk_load(st + 5 * kColBytes, src.flags + lo, b1, bar);
}

// One tile in flight or in work in a count stage. The replicate's part
// (c .. larv) is reloaded only when the stage moves on to another replicate.
struct alignas(16) CountStage {
  StepCtx c;
  sampo_population pop;
  DevPool src;
  uint32_t* tileAgg;
  uint32_t* tilePre;
  uint32_t rep, lt, end, larv;    // replicate, its tile index, its pool end, larvicide on
  uint32_t tick;                  // the tile's ticket; >= the ticket total: no more tiles
  int urg;                        // the range that holds every slot of the tile, or -1
  uint32_t left;                  // warps that have not finished the tile
  uint32_t crep;                  // replicate whose survivor counts `cnt` holds
  uint32_t cnt[8];                // survivors by next state of the stage's tiles of crep, not yet added to its totals
};

// Dynamic shared memory of the persistent kernels: the two stages, then the
// batch's ticket prefix (nrep + 1 words), sized at launch so that a single
// simulation pays 8 bytes for it.
constexpr size_t kCountSmem = 2 * kCountStage;
constexpr size_t kScatterSmem = 2 * kScatterStage;
// the same for I slots per thread (the stages scale with the tile; the
// prefix table has 8 I + 1 entries)
__host__ __device__ constexpr uint32_t pre_words(int items) { return ((items * kWarps + 1) * kPreEntryWords + 3) / 4 * 4; }
__host__ __device__ constexpr size_t count_smem(int items) { return 2 * (size_t)(5 * kBlock * items * 4 + kBlock * items); }
__host__ __device__ constexpr size_t scatter_smem(int items) {
  return 2 * (size_t)(9 * kBlock * items * 4 + kBlock * items + pre_words(items) * 4);
}
static_assert(count_smem(kItems) == kCountSmem && scatter_smem(kItems) == kScatterSmem, "one definition");
__host__ __device__ constexpr size_t plan_bytes(uint32_t nrep) { return ((size_t)(nrep + 1) * 4 + 15) & ~(size_t)15; }
constexpr uint32_t kNoRep = 0xffffffffu;

// One warp's items of a count-pass tile in stage memory st: the decision
// part of the update for each of its slots, and per (round, warp) chunk the
// survivors by next state into ent (8-bit fields, states 0-3 | 4-7).
// RG >= 0: every slot of the tile lies in range RG, so only that state's
// code is compiled in; RG = -1: a tile that spans ranges.
template <int I, int RG>
__device__ __forceinline__ void count_items(const CountStage& cs, const uint8_t* st, const KillConst& mc, uint32_t lo,
                                            uint32_t end, int tid, uint2* ent, Acc& acc, uint32_t& devoob) {
  SAMPO_TILE_CONSTANTS(I);
  const int lane = tid & 31, warp = tid >> 5;
  const StepCtx& c = cs.c;
  const bool larvicide = c.env.larvacideValue > 0.0f;
  const float* s_age = (const float*)(st + 0 * kColBytes);
  const float* s_his = (const float*)(st + 1 * kColBytes);
  const float* s_delay = (const float*)(st + 2 * kColBytes);
  const uint32_t* s_uni = (const uint32_t*)(st + 3 * kColBytes);
  const uint32_t* s_avail = (const uint32_t*)(st + 4 * kColBytes);
  const uint8_t* s_flags = st + 5 * kColBytes;
#pragma unroll
  for (int k = 0; k < kItems; k++) {
    const uint32_t i = k * kBlock + tid;
    const uint32_t g = lo + i;
    int rg;
    bool valid;
    if (RG >= 0) {
      rg = RG;
      valid = g < end;
    } else {
      rg = g < end ? range_of(cs.pop, g) : -1;
      valid = rg >= 0;
    }
    uint32_t pk0 = 0, pk1 = 0;  // this slot's next state as an 8-bit counter: states 0-3, 4-7
    if (valid) {
      Rec a;
      a.age = (rg == LARVA || rg >= IMMATURE) ? s_age[i] : 0.0f;
      a.his = (rg != GRAVID && (rg != LARVA || larvicide)) ? s_his[i] : 0.0f;
      a.delay = rg != GRAVID ? s_delay[i] : 0.0f;
      a.uni = (rg == LARVA || rg == GRAVID) ? s_uni[i] : 0u;
      a.avail = rg == GRAVID ? s_avail[i] : 0u;
      a.female = rg == MATESEEKING ? (s_flags[i] >> 3) & 1u : 0u;
      a.sporo = 0.0f; a.cycle = 0u; a.hbc = 0u; a.batches = 0u;
      devoob |= (rg == LARVA) & c.devOOB;
      const int ns = update_agent<false>(c, mc, rg, g, a, acc);
      if (ns >= 0) {
        if (ns < 4) pk0 = 1u << (8 * ns);
        else pk1 = 1u << (8 * (ns - 4));
      }
    }
    pk0 = __reduce_add_sync(0xffffffffu, pk0);
    pk1 = __reduce_add_sync(0xffffffffu, pk1);
    if (lane == 0) ent[k * kWarps + warp] = make_uint2(pk0, pk1);
  }
}

// The count pass. Its warps share no barrier once the tiles flow: each warp
// takes the stages' tiles in turn (stage it & 1 for its it-th tile, behind
// the stage's mbarrier), and the LAST warp to finish a tile does the tile's
// bookkeeping while the others go on with the tile in the other stage: it
// builds the tile's prefix table from the warps' chunk counts, adds the
// tile's totals to the stage's counts, claims the next ticket and starts
// that tile's copies into the stage it has just emptied. A warp's stall is
// then the wait for a tile's data, never the wait for the slowest warp.
template <int I>
__global__ void __launch_bounds__(kBlock, 5) k_count(KParams p) {
  SAMPO_TILE_CONSTANTS(I);
  extern __shared__ __align__(128) uint8_t dsm[];
  __shared__ CountStage s_cs[2];
  __shared__ KillConst s_mc;
  __shared__ uint32_t s_w[33];
  uint32_t* s_pre = reinterpret_cast<uint32_t*>(dsm + kCountSmem);
  __shared__ __align__(8) uint64_t bars[2];
  __shared__ uint32_t s_tnext;                // the next ticket, drawn one claim ahead
  __shared__ uint2 s_ent[2][kChunks];         // per stage, per (round, warp): survivors by state, 8-bit fields (states 0-3 | 4-7)
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  load_model_const(&p.mc->kill, s_mc);
  plan_tickets(p.nrep, s_pre, s_w, [&](uint32_t r) -> uint32_t {
    const SimDev* sim = p.reps[r].sim;
    return sim->active ? (sim->pop.r[GRAVID].end + kTile - 1) / kTile : 0u;
  });
  const uint32_t total = s_pre[p.nrep];
  // a step with no more tiles than CTAs gives CTA b tile b (no CTA queues a
  // second tile while others have none)
  const bool one_each = total <= gridDim.x;

  // the whole warp: add the stage's counts to their replicate's totals
  auto flush_stage = [&](CountStage& cs) {
    if (cs.crep != kNoRep && lane < 8 && cs.cnt[lane]) atomicAdd(&p.reps[cs.crep].sim->cnt[lane], cs.cnt[lane]);
    __syncwarp();
    if (lane < 8) cs.cnt[lane] = 0;
    if (lane == 0) cs.crep = kNoRep;
    __syncwarp();
  };
  // the whole warp: take the next ticket into stage sidx (emptied by every
  // warp), describe its tile and start its copies. The description is
  // written before the arrival on bars[sidx] that the waiting warps acquire.
  // Tickets run from the last tile down: the scatter pass then starts on the
  // tiles whose decision columns and prefix tables this pass touched last,
  // while they are still in L2.
  auto claim = [&](uint32_t sidx) {
    CountStage& cs = s_cs[sidx];
    uint32_t t = 0;
    if (lane == 0) t = s_tnext;
    t = __shfl_sync(0xffffffffu, t, 0);
    const uint32_t tile = total - 1u - t;
    const uint32_t r = t < total ? find_rep(s_pre, p.nrep, tile) : kNoRep;
    const uint32_t cur = cs.rep;
    __syncwarp();
    if (cur != r) {  // uniform: the stage moves on to another replicate
      flush_stage(cs);
      if (r != kNoRep) {
        const RepParams& rp = p.reps[r];
        const SimDev* sim = rp.sim;
        copy16(&cs.c, &sim->ctx, (int)sizeof(StepCtx), lane, 32);
        if (lane == 0) {
          cs.pop = sim->pop;
          cs.end = cs.pop.r[GRAVID].end;
          cs.src = rp.pool[sim->cur];
          cs.tileAgg = rp.tileAgg;
          cs.tilePre = rp.tilePre;
          cs.larv = sim->ctx.env.larvacideValue > 0.0f;
          cs.crep = r;
        }
      }
      if (lane == 0) cs.rep = r;
      __syncwarp();
    }
    if (lane == 0) {
      cs.tick = t;
      cs.left = kWarps;
      if (t >= total) {
        mbar_arrive(&bars[sidx]);  // no copy: the waiting warps see the end
      } else {
        cs.lt = tile - s_pre[r];
        const uint32_t lo = cs.lt * kTile, n = min((uint32_t)kTile, cs.end - lo);
        const int u = range_of(cs.pop, lo);
        cs.urg = (u >= 0 && lo + n <= cs.pop.r[u].end) ? u : -1;
        fence_proxy_async();  // the stage was last read through the generic proxy
        issue_count_tile<I>(cs.src, dsm + sidx * kCountStage, &bars[sidx], cs.pop, lo, n, cs.larv != 0);
        // the ticket of the claim after this one, drawn once the copies are
        // on their way (its round trip stays off the stage's refill)
        s_tnext = one_each ? 0xffffffffu : atomicAdd(&p.bat->ticket1, 1u);
      }
    }
  };

  if (tid == 0) {
    mbar_init(&bars[0]);
    mbar_init(&bars[1]);
    fence_mbar_init();
    s_tnext = one_each ? blockIdx.x : atomicAdd(&p.bat->ticket1, 1u);
  }
  if (tid < 2) {
    s_cs[tid].rep = kNoRep;
    s_cs[tid].crep = kNoRep;
  }
  if (tid < 16) s_cs[tid >> 3].cnt[tid & 7] = 0;
  __syncthreads();
  if (warp == 0) {
    claim(0);
    claim(1);
  }
  __syncthreads();

  Acc acc = {0, 0, 0, 0, 0, 0};
  uint32_t devoob = 0, w_rep = kNoRep;
  // the warp's own accumulators into replicate r's totals
  auto flush_warp = [&](uint32_t r) {
    const uint32_t ne = __reduce_add_sync(0xffffffffu, acc.newEggs);
    if (lane == 0 && ne) atomicAdd(&p.reps[r].sim->newEggs, ne);
    const uint32_t bad = __reduce_or_sync(0xffffffffu, (acc.bad ? SAMPO_DEV_ERR_LARVATABLE : 0u) | (devoob ? SAMPO_DEV_ERR_DEVRATES : 0u));
    if (lane == 0 && bad) atomicOr(&p.reps[r].sim->error, bad);
    acc.newEggs = 0; acc.bad = 0; devoob = 0;
  };

  uint32_t it = 0;
  bool failed = false;
  for (;; it++) {
    const uint32_t sidx = it & 1u;
    CountStage& cs = s_cs[sidx];
    if (!__all_sync(0xffffffffu, mbar_wait(&bars[sidx], (it >> 1) & 1u))) {  // bounded; acquires the description
      failed = true;
      break;
    }
    const uint32_t t = cs.tick;
    if (t >= total) break;
    const uint32_t rep = cs.rep;
    if (rep != w_rep) {
      if (w_rep != kNoRep) flush_warp(w_rep);
      w_rep = rep;
    }
    const uint8_t* st = dsm + sidx * kCountStage;
    const uint32_t end = cs.end, lo = cs.lt * kTile;
    uint2* ent = s_ent[sidx];
    switch (cs.urg) {  // CTA-uniform: a tile inside one range runs that state's code only
      case EGG: count_items<I, EGG>(cs, st, s_mc, lo, end, tid, ent, acc, devoob); break;
      case LARVA: count_items<I, LARVA>(cs, st, s_mc, lo, end, tid, ent, acc, devoob); break;
      case PUPA: count_items<I, PUPA>(cs, st, s_mc, lo, end, tid, ent, acc, devoob); break;
      case IMMATURE: count_items<I, IMMATURE>(cs, st, s_mc, lo, end, tid, ent, acc, devoob); break;
      case MATESEEKING: count_items<I, MATESEEKING>(cs, st, s_mc, lo, end, tid, ent, acc, devoob); break;
      case BMS: count_items<I, BMS>(cs, st, s_mc, lo, end, tid, ent, acc, devoob); break;
      case BMD: count_items<I, BMD>(cs, st, s_mc, lo, end, tid, ent, acc, devoob); break;
      case GRAVID: count_items<I, GRAVID>(cs, st, s_mc, lo, end, tid, ent, acc, devoob); break;
      default: count_items<I, -1>(cs, st, s_mc, lo, end, tid, ent, acc, devoob); break;
    }
    // this warp is done with the stage: the last warp out does the tile's bookkeeping
    uint32_t last = 0;
    __syncwarp();
    if (lane == 0) {
      __threadfence_block();  // this warp's entries and its reads of the stage come first
      last = atomicSub(&cs.left, 1u) == 1u;
      __threadfence_block();  // and the other warps' before the last warp's work
    }
    if (!__shfl_sync(0xffffffffu, last, 0)) continue;
    {
      // the tile's prefix table: exclusive prefix of the 32 (round, warp)
      // chunks, 16-bit packed, and the tile's totals (the update/scatter pass
      // reads both; the totals also feed the look-back)
      const uint2 e = lane < kChunks ? s_ent[sidx][lane] : make_uint2(0u, 0u);
      uint32_t w[5], x[5];
      w[0] = (e.x & 0xffu) | ((e.x & 0xff00u) << 8);
      w[1] = ((e.x >> 16) & 0xffu) | ((e.x >> 8) & 0xff0000u);
      w[2] = (e.y & 0xffu) | ((e.y & 0xff00u) << 8);
      w[3] = ((e.y >> 16) & 0xffu) | ((e.y >> 8) & 0xff0000u);
      w[4] = ((e.x * 0x01010101u) >> 24) + ((e.y * 0x01010101u) >> 24);  // byte sums <= 32 cannot carry
#pragma unroll
      for (int q = 0; q < 5; q++) x[q] = w[q];
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
#pragma unroll
        for (int q = 0; q < 5; q++) {
          const uint32_t y = __shfl_up_sync(0xffffffffu, x[q], o);
          if (lane >= o) x[q] += y;
        }
      }
      uint32_t* pre = cs.tilePre + (size_t)cs.lt * kPreWords;
      if (lane < kChunks) {
#pragma unroll
        for (int q = 0; q < 5; q++) pre[lane * kPreEntryWords + q] = x[q] - w[q];
      }
      if (lane == kChunks - 1) {
#pragma unroll
        for (int q = 0; q < 5; q++) pre[kChunks * kPreEntryWords + q] = x[q];
      }
      uint32_t tw = 0;  // lanes 0..7: the tile's survivors of next state `lane`
#pragma unroll
      for (int q = 0; q < 4; q++) {
        const uint32_t tq = __shfl_sync(0xffffffffu, x[q], kChunks - 1);
        if ((lane >> 1) == q) tw = (tq >> (16 * (lane & 1))) & 0xffffu;
      }
      if (lane < 8) {
        cs.tileAgg[(size_t)cs.lt * 8 + lane] = tw;
        cs.cnt[lane] += tw;
      }
      __syncwarp();
    }
    claim(sidx);  // the next tile into the stage this tile emptied
  }
  // (each stage's counts were added to their totals by the claim that found
  // no more tickets for it: the claims alternate stages in iteration order)
  if (w_rep != kNoRep) flush_warp(w_rep);
  if (failed && lane == 0) {
    const uint32_t r = s_cs[it & 1u].rep;
    atomicOr(&p.reps[r != kNoRep ? r : 0u].sim->error, SAMPO_DEV_ERR_TMA);
    // let copies still in flight land before the warp exits (bounded waits)
    (void)mbar_wait(&bars[it & 1u], (it >> 1) & 1u);
    (void)mbar_wait(&bars[(it + 1) & 1u], ((it + 1) >> 1) & 1u);
  }
}

// ------------------------------------------------------------------------
// Publishing the start of a step
// ------------------------------------------------------------------------
// warp 0 publishes; warps 1-4 fill the 100 entries of the larval table at once
constexpr int kPublishThreads = 160;

// A replicate's state read through L2 (ld.global.cg): in the one-launch step
// other CTAs of the same kernel wrote it, and this SM's L1 may hold older
// copies of the same lines.
template <class T>
__device__ __forceinline__ T ld_l2(const T* p) {
  static_assert(sizeof(T) % 4 == 0, "whole words");
  T v;
  uint32_t* d = reinterpret_cast<uint32_t*>(&v);
  const uint32_t* q = reinterpret_cast<const uint32_t*>(p);
#pragma unroll
  for (int k = 0; k < (int)(sizeof(T) / 4); k++) d[k] = __ldcg(q + k);
  return v;
}

// The larval hourly mortality of larvae d days old in a pool of L1de l1
// (kernel/killAgents.cl:117-125); NaN outside the ages [dmin, dmax] present.
__device__ __forceinline__ float larva_hmr_entry(uint32_t d, uint32_t dmin, uint32_t dmax, uint32_t l1, float cc) {
  if (d < dmin || d > dmax) return SAMPO_NAN_F;
  float dmr = 0.1f * sampo_expf((float)l1 / ((float)d * cc * 1.0f));
  dmr = sampo_fminf(dmr, 0.8f);
  const float dsr = 1.0f - dmr;
  const float hsr = sampo_powf(dsr, 1.0f / 24.0f);
  return 1.0f - hsr;
}

// The publish of replicate r by the calling CTA (at least kPublishThreads
// threads; all of them call it): after a step, the next layout from the
// survivor counts (kernel/oldToNewAgents.cl:57-95); then the pool's L1de,
// female and infective counts (calcStats, src/abms.c:230-310), the stats
// row, the next step's constants and the larval hourly mortality for every
// larva age present (kernel/killAgents.cl:117-133 depends on the age and
// L1de only). Reads and clears the acc_* accumulators. Mode PUB_REFRESH only
// recomputes the input-dependent step constants (the inputs of the coming
// step may have been written after its publish). When the next layout does
// not fit the replicate's capacity (the scatter pass then flagged
// SAMPO_DEV_ERR_CAPACITY and wrote nothing), the replicate pauses instead:
// it becomes inactive at the same step with the same pool, constants and
// larval table, and only the step's counters are cleared, so that the step
// runs again, with the same result, once its pool has been moved into a
// larger one (sampo_batch_grow). Returns the end of the replicate's pool
// after the publish (0 when it is inactive) to every thread.
__device__ uint32_t publish_rep(const KParams& p, uint32_t r, int mode) {
  __shared__ uint32_t s_go, s_l1, s_dmin, s_dmax, s_end, s_pause;
  __shared__ float s_cc;
  const RepParams& rp = p.reps[r];
  SimDev* sim = rp.sim;
  if (threadIdx.x < 32) {
    // a device seed stream draws the coming step's seeds once, before thread 0 reads them
    const uint32_t coming = __ldcg(&sim->step) + (mode == PUB_AFTER_STEP ? 1u : 0u);
    if (__ldcg(&sim->active) && __ldcg(&sim->rnd.next) == coming && coming < __ldcg(&sim->stop_step))
      draw_step_seeds(rp, coming);
    __syncwarp();
  }
  if (mode == PUB_REFRESH) {
    if (threadIdx.x == 0 && sim->active) {
      CtxInputs in;
      load_ctx_inputs(rp, sim->step, in);
      StepCtx c;
      make_ctx(in, sim->larvaHMR, sim->pop, c);
      sim->ctx = c;
    }
    return 0u;
  }
  const bool after_step = mode == PUB_AFTER_STEP;
  // Thread 0 reads all it needs before its first store (a store that may
  // alias a later load would hold that load back until the store is issued,
  // turning the reads into a chain), hands the larval table's inputs to the
  // other warps and does its writes while they fill the table.
  sampo_population np;
  sampo_bites_cycles bnc;
  CtxInputs in;
  uint32_t step = 0, stop = 0, epoch = 0, cur = 0, warn = 0;
  bool relayout = false, shared_end_warn = false, pause = false;
  if (threadIdx.x == 0) {
    const uint32_t active = __ldcg(&sim->active);
    np = ld_l2(&sim->pop);
    bnc = ld_l2(&sim->bnc);
    uint32_t cnt[8], abnc[4];
#pragma unroll
    for (int k = 0; k < 8; k++) cnt[k] = __ldcg(&sim->cnt[k]);
#pragma unroll
    for (int q = 0; q < 4; q++) abnc[q] = __ldcg(&sim->acc_bnc[q]);
    const uint32_t ne = __ldcg(&sim->newEggs), capacity = __ldcg(&sim->capacity);
    const uint32_t aL1 = __ldcg(&sim->acc_L1de), afem = __ldcg(&sim->acc_fem), ainf = __ldcg(&sim->acc_inf);
    const uint32_t dmin = __ldcg(&sim->acc_dmin), dmax = __ldcg(&sim->acc_dmax);
    const float cc = __ldcg(&sim->cc);
    step = __ldcg(&sim->step);
    stop = __ldcg(&sim->stop_step);
    epoch = __ldcg(&sim->epoch);
    cur = __ldcg(&sim->cur);
    warn = __ldcg(&sim->warn);
    if (after_step) {
      // the reference's shared empty initial ranges (src/abms.c:204-219) make
      // oldToNewAgents read one prefix-sum entry for several range ends
      bool shared_end = false;
      uint32_t moved = 0;
      for (int k = 1; k < 8; k++) {
        shared_end |= np.r[k].end == np.r[k - 1].end;
        moved += cnt[k];
      }
      shared_end_warn = shared_end && moved;
      if (layout_fits(cnt, ne, capacity)) {
        uint32_t base[8];
        next_layout(cnt, ne, np, base);
        relayout = true;
      } else {
        pause = true;  // the scatter pass flagged the capacity error and wrote nothing
      }
      step += 1u;
      bnc.numCyclesReported = abnc[0];
      bnc.sumCyclesReported = abnc[1];
      bnc.numBitesReported = abnc[2];
      bnc.numInfectBitesReported = abnc[3];
    }
    np.numLarvae1DayEquiv = (np.r[LARVA].end > np.r[LARVA].start) ? aL1 : 0u;  // kernel/calcL1de.cl:259-280
    np.numFemale = afem;
    np.numPotentiallyInfective = ainf;
    if (active) load_ctx_inputs(rp, step, in);
    s_go = active;
    s_pause = pause;
    s_end = active ? np.r[GRAVID].end : 0u;
    s_l1 = np.numLarvae1DayEquiv;
    s_dmin = dmin;
    s_dmax = dmax;
    s_cc = cc;
  }
  __syncthreads();
  const uint32_t pool_end = s_end;
  if (!s_go) return pool_end;
  if (s_pause) {
    if (threadIdx.x == 0) {
#pragma unroll
      for (int k = 0; k < 8; k++) sim->cnt[k] = 0;
      sim->newEggs = 0;
      sim->acc_L1de = 0; sim->acc_fem = 0; sim->acc_inf = 0;
      sim->acc_dmin = 0xffffffffu; sim->acc_dmax = 0;
      sim->acc_bnc[0] = sim->acc_bnc[1] = sim->acc_bnc[2] = sim->acc_bnc[3] = 0;
      sim->active = 0;
    }
    return 0u;
  }
  if (threadIdx.x == 0) {
    if (shared_end_warn) sim->warn = warn | SAMPO_DEV_WARN_REF_LAYOUT;
    if (after_step) {
      if (relayout) sim->cur = cur ^ 1u;
      sim->step = step;
      sim->epoch = epoch + 1u;
#pragma unroll
      for (int k = 0; k < 8; k++) sim->cnt[k] = 0;
      sim->newEggs = 0;
      sim->bnc = bnc;
    }
    sim->pop = np;
    sampo_stats_row row;
    row.pop = np;
    row.bnc = bnc;
    rp.rows[step % rp.ring] = row;
    sim->acc_L1de = 0; sim->acc_fem = 0; sim->acc_inf = 0;
    sim->acc_dmin = 0xffffffffu; sim->acc_dmax = 0;
    sim->acc_bnc[0] = sim->acc_bnc[1] = sim->acc_bnc[2] = sim->acc_bnc[3] = 0;
    StepCtx c;
    make_ctx(in, sim->larvaHMR, np, c);
    sim->ctx = c;
    if (step >= stop) sim->active = 0;
  } else if (threadIdx.x >= 32) {
    for (int d = threadIdx.x - 32; d < 100; d += blockDim.x - 32) {
      sim->larvaHMR[d] = larva_hmr_entry((uint32_t)d, s_dmin, s_dmax, s_l1, s_cc);
    }
  }
  return pool_end;
}

// Publishing the start of a step for every replicate of p (one CTA each);
// block 0 rearms the tickets.
__global__ void __launch_bounds__(kPublishThreads) k_publish(KParams p, int mode) {
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    p.bat->ticket1 = 0u;
    p.bat->ticket2 = 0u;
  }
  (void)publish_rep(p, blockIdx.x, mode);
}

// ------------------------------------------------------------------------
// Update + scatter pass
// ------------------------------------------------------------------------
template <int I>
__device__ void issue_scatter_tile(const DevPool& src, const uint32_t* pre, uint8_t* st, uint64_t* bar, uint32_t lo, uint32_t n) {
  SAMPO_TILE_CONSTANTS(I);
  const uint32_t b4 = (n * 4 + 15) & ~15u, b1 = (n + 15) & ~15u;
  mbar_arrive_tx(bar, 9 * b4 + b1 + kPreWords * 4);
  bulk_load(st + kPreOff, pre, kPreWords * 4, bar);
  bulk_load(st + 0 * kColBytes, src.age + lo, b4, bar);
  bulk_load(st + 1 * kColBytes, src.his + lo, b4, bar);
  bulk_load(st + 2 * kColBytes, src.delay + lo, b4, bar);
  bulk_load(st + 3 * kColBytes, src.sporo + lo, b4, bar);
  bulk_load(st + 4 * kColBytes, src.uni + lo, b4, bar);
  bulk_load(st + 5 * kColBytes, src.avail + lo, b4, bar);
  bulk_load(st + 6 * kColBytes, src.cycle + lo, b4, bar);
  bulk_load(st + 7 * kColBytes, src.hbc + lo, b4, bar);
  bulk_load(st + 8 * kColBytes, src.batches + lo, b4, bar);
  bulk_load(st + 9 * kColBytes, src.flags + lo, b1, bar);
}

// Decoupled look-back for tile t of one replicate by one warp over the count
// pass's tile aggregates: sums earlier tiles' aggregates back to the nearest
// published inclusive prefix (no waiting). A published prefix is eight 64-bit
// words, each holding a state's inclusive prefix and the step's epoch: every
// word is written and read whole (single-copy atomic), so a reader validates
// each by its epoch and no fence or flag is needed on either side. Lane 0
// publishes t's words. Every lane returns the exclusive prefix ex[] and t's
// counts cnt[].
struct LookbackArrays {
  uint32_t* agg;             // count pass tile aggregates
  unsigned long long* incl;  // inclusive prefixes: value | epoch << 32
};

__device__ __forceinline__ void ld_relaxed_v2u64(const unsigned long long* p, unsigned long long& a, unsigned long long& b) {
  asm volatile("ld.relaxed.gpu.global.v2.u64 {%0,%1}, [%2];" : "=l"(a), "=l"(b) : "l"(p) : "memory");
}
__device__ __forceinline__ void st_relaxed_v2u64(unsigned long long* p, unsigned long long a, unsigned long long b) {
  asm volatile("st.relaxed.gpu.global.v2.u64 [%0], {%1,%2};" ::"l"(p), "l"(a), "l"(b) : "memory");
}

__device__ void tile_lookback(const LookbackArrays& rp, uint32_t t, uint32_t epoch, int lane, uint32_t ex[8], uint32_t cnt[8]) {
#pragma unroll
  for (int b = 0; b < 8; b++) ex[b] = 0;
  int64_t pos = (int64_t)t - 1;
  while (pos >= 0) {
    const int64_t idx = pos - lane;
    const bool valid = idx >= 0;
    uint32_t v[8];
    bool pub = false;
#pragma unroll
    for (int b = 0; b < 8; b++) v[b] = 0;
    if (valid) {
      const uint4 a0 = ld_cg_v4(rp.agg + (size_t)idx * 8), a1 = ld_cg_v4(rp.agg + (size_t)idx * 8 + 4);
      unsigned long long w[8];
#pragma unroll
      for (int q = 0; q < 4; q++) ld_relaxed_v2u64(rp.incl + (size_t)idx * 8 + 2 * q, w[2 * q], w[2 * q + 1]);
      pub = true;
#pragma unroll
      for (int b = 0; b < 8; b++) pub = pub && (uint32_t)(w[b] >> 32) == epoch;
      const uint32_t ag[8] = {a0.x, a0.y, a0.z, a0.w, a1.x, a1.y, a1.z, a1.w};
#pragma unroll
      for (int b = 0; b < 8; b++) v[b] = pub ? (uint32_t)w[b] : ag[b];
    }
    const uint32_t m = __ballot_sync(0xffffffffu, !valid || pub);
    const int stop = m ? __ffs(m) - 1 : 32;
    if (lane > stop) {  // beyond the nearest published tile (or the first tile)
#pragma unroll
      for (int b = 0; b < 8; b++) v[b] = 0;
    }
#pragma unroll
    for (int b = 0; b < 8; b++) ex[b] += __reduce_add_sync(0xffffffffu, v[b]);
    if (m) break;
    pos -= 32;
  }
  const uint32_t* ag = rp.agg + (size_t)t * 8;
  const uint4 a0 = ld_cg_v4(ag), a1 = ld_cg_v4(ag + 4);
  cnt[0] = a0.x; cnt[1] = a0.y; cnt[2] = a0.z; cnt[3] = a0.w; cnt[4] = a1.x; cnt[5] = a1.y; cnt[6] = a1.z; cnt[7] = a1.w;
  if (lane == 0) {
    const unsigned long long e = (unsigned long long)epoch << 32;
    unsigned long long* q = rp.incl + (size_t)t * 8;
#pragma unroll
    for (int b = 0; b < 8; b += 2) st_relaxed_v2u64(q + b, e | (ex[b] + cnt[b]), e | (ex[b + 1] + cnt[b + 1]));
  }
}


constexpr int kScatterThreads = kBlock + 32;  // eight consumer warps and one producer warp
static_assert(kChunks <= 32, "one (round, warp) chunk per lane");
// resident CTAs per SM the registers of the update/scatter pass are sized for
__host__ __device__ constexpr int scatter_min_blocks(int items) { return items >= 4 ? 2 : 3; }
enum : uint32_t { TK_OLD = 0, TK_EGG = 1, TK_END = 2 };

// What the producer warp hands the consumers with a tile. The replicate's
// part (c .. base) is reloaded only when the slot changes replicate.
struct alignas(16) ScatterStage {
  StepCtx c;                 // the replicate's step constants
  sampo_population pop;      // its current ranges
  DevPool dst, src;          // its next and current buffers
  LookbackArrays lb;         // its look-back arrays
  const uint32_t* pre;       // its prefix tables
  uint32_t rep, end, newEggs, nold, epoch;  // replicate, pool end, eggs laid, old tiles, look-back epoch
  uint32_t base[8];          // first slot of each next-state range
  uint32_t kind, lo;         // TK_*, first slot (old tile) or first egg id (egg tile)
  int urg;                   // old tile: the range that holds every slot of the tile, or -1
  uint32_t d0[8], cnt[8];    // per next state: the tile's first slot in it, survivors
};
constexpr int kAhead = 3;                 // the producer describes tiles this far ahead of the consumers
constexpr int kDescSlots = kAhead + 1;    // tile descriptions in flight
// Each pass of the loop issues tile seq + 2; with kAhead >= 3 it was described
// by an earlier pass, with kAhead == 2 the pass describes it first.
static_assert(kAhead >= 2 && kDescSlots <= 16, "issue() needs tile seq + 2 described; 2 kind bits per slot");

// A survivor's owed normal draw (include/gpuRand.h:56-63): its slot in the
// next buffer, its slot in the current one (the generator's gid), its
// numEggBatches after the step, BM_*.
struct BmEntry { uint32_t d, gid, batches, kind; };

// Phase A of the update/scatter pass for one warp's items of an old tile in
// stage memory st: the full update of each slot, and each survivor's slot in
// the next buffer (dk; 0xffffffff for none): the tile's first slot of its
// next state + the survivors of that state in earlier (round, warp) chunks
// (the count pass's prefix table) + its rank within its chunk. nb gets the
// next state (8: none) | female << 4 | owed draw << 5. RG >= 0: every slot
// of the tile lies in range RG, so only that state's code is compiled in;
// RG = -1: a tile that spans ranges.
template <int I, int RG>
__device__ __forceinline__ void scatter_phase_a(const ScatterStage& si, const uint8_t* st, const KillConst& kc, int tid,
                                                Rec (&a)[I], uint32_t (&nb)[I], uint32_t (&dk)[I], Acc& acc,
                                                uint32_t& tilebad) {
  SAMPO_TILE_CONSTANTS(I);
  const int warp = tid >> 5;
  const float* c_age = (const float*)(st + 0 * kColBytes);
  const float* c_his = (const float*)(st + 1 * kColBytes);
  const float* c_delay = (const float*)(st + 2 * kColBytes);
  const float* c_sporo = (const float*)(st + 3 * kColBytes);
  const uint32_t* c_uni = (const uint32_t*)(st + 4 * kColBytes);
  const uint32_t* c_avail = (const uint32_t*)(st + 5 * kColBytes);
  const uint32_t* c_cycle = (const uint32_t*)(st + 6 * kColBytes);
  const uint32_t* c_hbc = (const uint32_t*)(st + 7 * kColBytes);
  const uint32_t* c_batches = (const uint32_t*)(st + 8 * kColBytes);
  const uint8_t* c_flags = st + 9 * kColBytes;
  const uint32_t* c_pre = (const uint32_t*)(st + kPreOff);
  const StepCtx& c = si.c;
  const uint32_t lo = si.lo, end = si.end;
#pragma unroll
  for (int k = 0; k < kItems; k++) {
    const uint32_t i = k * kBlock + tid;
    const uint32_t g = lo + i;
    int rg;
    bool valid;
    if (RG >= 0) {
      rg = RG;
      valid = g < end;
    } else {
      rg = g < end ? range_of(si.pop, g) : -1;
      valid = rg >= 0;
    }
    nb[k] = 8;
    a[k].bm = BM_NONE;
    a[k].female = 0u;
    if (valid) {
      a[k].age = c_age[i]; a[k].his = c_his[i]; a[k].delay = c_delay[i]; a[k].sporo = c_sporo[i];
      a[k].uni = c_uni[i]; a[k].avail = c_avail[i]; a[k].cycle = c_cycle[i]; a[k].hbc = c_hbc[i];
      a[k].batches = c_batches[i];
      a[k].female = (c_flags[i] >> 3) & 1u;
      const int ns = update_agent<true>(c, kc, rg, g, a[k], acc);
      if (ns >= 0) nb[k] = ns;
    }
    const uint32_t peers = __match_any_sync(0xffffffffu, nb[k]);
    const uint32_t rk = __popc(peers & lanemask_lt());
    const uint32_t* e0 = c_pre + (k * kWarps + warp) * kPreEntryWords;  // this chunk's entry
    const uint32_t* e1 = e0 + kPreEntryWords;                         // the next one
    const int b = nb[k];
    dk[k] = 0xffffffffu;
    if (b < 8) {
      const uint32_t sh = 16 * (b & 1);
      const uint32_t j = ((e0[b >> 1] >> sh) & 0xffffu) + rk;
      // the two passes disagree when a survivor falls outside its chunk's run
      if (j < ((e1[b >> 1] >> sh) & 0xffffu)) dk[k] = si.d0[b] + j;
      else tilebad = 1;
    }
    // ... or when the chunk's survivors are not the count pass's
    const uint32_t ns = __popc(__ballot_sync(0xffffffffu, b < 8));
    if (ns != e1[4] - e0[4]) tilebad = 1;
    nb[k] = (uint32_t)b | (a[k].female << 4) | (a[k].bm << 5);
  }
}

// The producer warp describes tiles three ahead (ticket, replicate data,
// look-back, layout) and hands each to the consumers in a free stage with
// its TMA loads (full[s]: the expect-tx arrival + the arrival that publishes
// the description). A stage carries the tile's columns and the count pass's
// prefix table of its (round, warp) chunks, so every consumer warp knows
// where its survivors go without the other warps: the consumer warps share
// no barrier. Each releases a stage (empty[s], 256 arrivals) as soon as it
// has read its inputs, then writes every survivor straight to its slot in the
// next buffer: the survivors of one next state are contiguous within a warp,
// so the stores coalesce.
template <int I>
__global__ void __launch_bounds__(kScatterThreads, scatter_min_blocks(I)) k_scatter(KParams p) {
  SAMPO_TILE_CONSTANTS(I);
  extern __shared__ __align__(128) uint8_t dsm[];
  __shared__ ScatterStage s_si[kDescSlots];
  __shared__ ModelConst s_mc;
  __shared__ uint32_t s_w[33];
  uint32_t* s_pre = reinterpret_cast<uint32_t*>(dsm + kScatterSmem);
  __shared__ __align__(8) uint64_t full[2], empty[2];
  __shared__ BmEntry s_bmq[kWarps][kItems * 32];    // per warp: owed draws of the tile
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  load_model_const(p.mc, s_mc);
  plan_tickets(p.nrep, s_pre, s_w, [&](uint32_t r) -> uint32_t {
    SimDev* sim = p.reps[r].sim;
    if (!sim->active) return 0u;
    uint32_t cnt[8];
    for (int k = 0; k < 8; k++) cnt[k] = sim->cnt[k];
    const uint32_t ne = sim->newEggs;
    if (!layout_fits(cnt, ne, sim->capacity)) {
      if (blockIdx.x == 0) atomicOr(&sim->error, SAMPO_DEV_ERR_CAPACITY);
      return 0u;
    }
    return (sim->pop.r[GRAVID].end + kTile - 1) / kTile + (ne + kTile - 1) / kTile;
  });
  const uint32_t total = s_pre[p.nrep];
  if (tid == 0) {
    mbar_init_count(&full[0], 2);
    mbar_init_count(&full[1], 2);
    mbar_init_count(&empty[0], kBlock);
    mbar_init_count(&empty[1], kBlock);
    fence_mbar_init();
    for (int k = 0; k < kDescSlots; k++) s_si[k].rep = 0xffffffffu;
  }
  __syncthreads();

  uint32_t fail = 0, fail_rep = 0;
  if (warp == kWarps) {
    // ================= producer warp =================
    // describe tile `seq` (slot seq % kDescSlots): take a ticket, load the
    // replicate's data when the slot changes replicate, run the look-back,
    // lay out the tile's runs. Touches no stage.
    // lane 0 draws each ticket one description ahead, so the atomic's round
    // trip overlaps a tile; a step with no more tiles than CTAs gives CTA b
    // tile b (no CTA queues several tiles while others have none)
    const bool one_each = total <= gridDim.x;
    uint32_t t_next = 0;
    if (lane == 0) t_next = one_each ? blockIdx.x : atomicAdd(&p.bat->ticket2, 1u);
    auto describe = [&](uint32_t seq) -> uint32_t {
      uint32_t t = 0;
      if (lane == 0) {
        t = t_next;
        t_next = one_each ? 0xffffffffu : atomicAdd(&p.bat->ticket2, 1u);
      }
      t = __shfl_sync(0xffffffffu, t, 0);
      ScatterStage& si = s_si[seq % kDescSlots];
      if (t >= total) {
        if (lane == 0) si.kind = TK_END;
        __syncwarp();
        return TK_END;
      }
      const uint32_t r = find_rep(s_pre, p.nrep, t);
      const uint32_t j = t - s_pre[r];
      if (si.rep != r) {  // uniform: the slot's replicate data, once per replicate
        const RepParams& rp = p.reps[r];
        SimDev* sim = rp.sim;
        copy16(&si.c, &sim->ctx, (int)sizeof(StepCtx), lane, 32);
        if (lane == 0) {
          const uint32_t cur = sim->cur, ne = sim->newEggs;
          si.pop = sim->pop;
          si.end = si.pop.r[GRAVID].end;
          si.nold = (si.end + kTile - 1) / kTile;
          si.newEggs = ne;
          si.epoch = sim->epoch;
          si.src = rp.pool[cur];
          si.dst = rp.pool[cur ^ 1u];
          si.lb.agg = rp.tileAgg;
          si.lb.incl = rp.tileIncl;
          si.pre = rp.tilePre;
          uint32_t tc[8], base[8];
          for (int k = 0; k < 8; k++) tc[k] = sim->cnt[k];
          sampo_population np;
          next_layout(tc, ne, np, base);
          for (int k = 0; k < 8; k++) si.base[k] = base[k];
        }
        __syncwarp();
        if (lane == 0) si.rep = r;
        __syncwarp();
      }
      if (j < si.nold) {
        uint32_t ex[8], cnt[8];
        tile_lookback(si.lb, j, si.epoch, lane, ex, cnt);
        if (lane == 0) {
#pragma unroll
          for (int b = 0; b < 8; b++) {
            si.d0[b] = si.base[b] + ex[b];
            si.cnt[b] = cnt[b];
          }
          si.kind = TK_OLD;
          si.lo = j * kTile;
          const uint32_t n = min((uint32_t)kTile, si.end - si.lo);
          const int u = range_of(si.pop, si.lo);
          si.urg = (u >= 0 && si.lo + n <= si.pop.r[u].end) ? u : -1;
        }
        __syncwarp();
        return TK_OLD;
      }
      if (lane == 0) {
        si.kind = TK_EGG;
        si.lo = (j - si.nold) * kTile;
      }
      __syncwarp();
      return TK_EGG;
    };
    // hand tile `seq` to the consumers in stage seq & 1 (free): its loads
    // (expect-tx arrival) and the arrival that publishes its description
    auto issue = [&](uint32_t seq) {
      const uint32_t s = seq & 1u;
      const ScatterStage& si = s_si[seq % kDescSlots];
      if (lane == 0) {
        if (si.kind == TK_OLD) {
          fence_proxy_async();  // the stage was last read through the generic proxy
          issue_scatter_tile<I>(si.src, si.pre + (size_t)(si.lo / kTile) * kPreWords, dsm + s * kScatterStage, &full[s], si.lo,
                             min((uint32_t)kTile, si.end - si.lo));
        } else {
          mbar_arrive(&full[s]);
        }
        mbar_arrive(&full[s]);  // description written (release)
      }
    };
    uint32_t kinds = 0, ph = 0;  // 2 bits per described tile, slot seq % kDescSlots
    auto kind_of = [&](uint32_t seq) { return (kinds >> (2 * (seq % kDescSlots))) & 3u; };
    auto set_kind = [&](uint32_t seq, uint32_t k) {
      const uint32_t sh = 2 * (seq % kDescSlots);
      kinds = (kinds & ~(3u << sh)) | (k << sh);
    };
    set_kind(0, describe(0));
    issue(0);
    set_kind(1, describe(1));
    issue(1);
    for (uint32_t seq = 2; seq < (uint32_t)kAhead; seq++) set_kind(seq, describe(seq));
    for (uint32_t seq = 0;; seq++) {
      const uint32_t s = seq & 1u;
      if (kind_of(seq) == TK_END) break;
      uint32_t ok = 1;
      if (lane == 0) ok = mbar_wait(&empty[s], (ph >> s) & 1u) ? 1u : 0u;  // tile seq's inputs are read
      ok = __shfl_sync(0xffffffffu, ok, 0);
      if (!ok) { fail = 1; fail_rep = s_si[seq % kDescSlots].rep; break; }
      ph ^= 1u << s;
      // slot (seq + kAhead) % kDescSlots held tile seq - 1, whose consumers
      // are done: they released tile seq's inputs after finishing it
      if (kAhead == 2) {
        set_kind(seq + 2, describe(seq + 2));
        issue(seq + 2);
      } else {
        issue(seq + 2);
        set_kind(seq + kAhead, describe(seq + kAhead));
      }
    }
  } else {
    // ================= consumer warps =================
    const ModelConst& mc = s_mc;
    Acc acc = {0, 0, 0, 0, 0, 0};
    uint32_t l1 = 0, fem = 0, inf = 0, dmin = 0xffffffffu, dmax = 0, tilebad = 0;
    uint32_t cur_rep = 0xffffffffu;
    // this warp's statistics of replicate r into its totals
    auto flush = [&](uint32_t r) {
      SimDev* sim = p.reps[r].sim;
      uint32_t v[8] = {l1, fem, inf, acc.cycles, acc.sumCycles, acc.bites, acc.infectBites,
                       (acc.bad ? SAMPO_DEV_ERR_LARVATABLE : 0u) | (tilebad ? SAMPO_DEV_ERR_TILECOUNT : 0u)};
#pragma unroll
      for (int j = 0; j < 8; j++) v[j] = j == 7 ? __reduce_or_sync(0xffffffffu, v[j]) : __reduce_add_sync(0xffffffffu, v[j]);
      const uint32_t mn = __reduce_min_sync(0xffffffffu, dmin), mx = __reduce_max_sync(0xffffffffu, dmax);
      if (lane == 0) {
        if (v[0]) atomicAdd(&sim->acc_L1de, v[0]);
        if (v[1]) atomicAdd(&sim->acc_fem, v[1]);
        if (v[2]) atomicAdd(&sim->acc_inf, v[2]);
        if (v[3]) atomicAdd(&sim->acc_bnc[0], v[3]);
        if (v[4]) atomicAdd(&sim->acc_bnc[1], v[4]);
        if (v[5]) atomicAdd(&sim->acc_bnc[2], v[5]);
        if (v[6]) atomicAdd(&sim->acc_bnc[3], v[6]);
        if (v[7]) atomicOr(&sim->error, v[7]);
        if (mn != 0xffffffffu) { atomicMin(&sim->acc_dmin, mn); atomicMax(&sim->acc_dmax, mx); }
      }
      acc = Acc{0, 0, 0, 0, 0, 0};
      l1 = fem = inf = dmax = tilebad = 0;
      dmin = 0xffffffffu;
    };
    uint32_t ph = 0;
    for (uint32_t it = 0;; it++) {
      const uint32_t s = it & 1u;
      const uint8_t* st = dsm + s * kScatterStage;
      const bool ok = __all_sync(0xffffffffu, mbar_wait(&full[s], (ph >> s) & 1u));  // bounded; acquires the stage
      if (ok) ph ^= 1u << s;  // else the phase is still owed: the exit path waits for it again
      const ScatterStage& si = s_si[it % kDescSlots];
      const uint32_t kind = ok ? si.kind : TK_END;
      if (kind != TK_END && si.rep != cur_rep) {
        if (cur_rep != 0xffffffffu) flush(cur_rep);
        cur_rep = si.rep;
      }
      // ---- phase A (old tiles): recompute the step for the tile's agents and
      //      find each survivor's slot: the tile's first slot of its next
      //      state + the survivors of that state in earlier (round, warp)
      //      chunks (prefix table) + its rank within its chunk ----
      Rec a[kItems];
      uint32_t nb[kItems];  // after phase A: next state (8: none) | female << 4 | owed draw << 5
      uint32_t dk[kItems];
      if (kind == TK_OLD) {
        switch (si.urg) {  // CTA-uniform: a tile inside one range runs that state's code only
          case EGG: scatter_phase_a<I, EGG>(si, st, mc.kill, tid, a, nb, dk, acc, tilebad); break;
          case LARVA: scatter_phase_a<I, LARVA>(si, st, mc.kill, tid, a, nb, dk, acc, tilebad); break;
          case PUPA: scatter_phase_a<I, PUPA>(si, st, mc.kill, tid, a, nb, dk, acc, tilebad); break;
          case IMMATURE: scatter_phase_a<I, IMMATURE>(si, st, mc.kill, tid, a, nb, dk, acc, tilebad); break;
          case MATESEEKING: scatter_phase_a<I, MATESEEKING>(si, st, mc.kill, tid, a, nb, dk, acc, tilebad); break;
          case BMS: scatter_phase_a<I, BMS>(si, st, mc.kill, tid, a, nb, dk, acc, tilebad); break;
          case BMD: scatter_phase_a<I, BMD>(si, st, mc.kill, tid, a, nb, dk, acc, tilebad); break;
          case GRAVID: scatter_phase_a<I, GRAVID>(si, st, mc.kill, tid, a, nb, dk, acc, tilebad); break;
          default: scatter_phase_a<I, -1>(si, st, mc.kill, tid, a, nb, dk, acc, tilebad); break;
        }
      }
      if (kind != TK_END) mbar_arrive(&empty[s]);  // this thread is done with the stage's inputs
      if (!ok) { fail = 1; fail_rep = cur_rep == 0xffffffffu ? 0u : cur_rep; break; }
      if (kind == TK_END) break;
      const StepCtx& c = si.c;
      const DevPool& dst = si.dst;
      if (kind == TK_OLD) {
        BmEntry* bmq = s_bmq[warp];
        uint32_t nq = 0;
        // ---- phase B: every survivor to its slot in the next buffer ----
#pragma unroll
        for (int k = 0; k < kItems; k++) {
          const int b = (int)(nb[k] & 15u);
          const uint32_t female = (nb[k] >> 4) & 1u;
          const uint32_t d = dk[k];
          // queue this warp's owed draws; their column is written after the draw
          const uint32_t owed = d != 0xffffffffu ? nb[k] >> 5 : BM_NONE;
          const uint32_t om = __ballot_sync(0xffffffffu, owed != BM_NONE);
          if (owed != BM_NONE) {
            BmEntry q;
            q.d = d; q.gid = si.lo + k * kBlock + tid; q.batches = a[k].batches; q.kind = owed;
            bmq[nq + __popc(om & lanemask_lt())] = q;
          }
          nq += __popc(om);
          if (d != 0xffffffffu) {
            dst.age[d] = a[k].age; dst.his[d] = a[k].his; dst.sporo[d] = a[k].sporo; dst.uni[d] = a[k].uni;
            dst.cycle[d] = a[k].cycle; dst.hbc[d] = a[k].hbc; dst.batches[d] = a[k].batches;
            dst.flags[d] = (uint8_t)(b | (female << 3));
            if (owed != BM_LARVA_DELAY) dst.delay[d] = a[k].delay;
            if (owed != BM_EGG_BATCH) dst.avail[d] = a[k].avail;
            // statistics of the next pool (kernel/calcL1de.cl:28-30, kernel/calcGender.cl:24-37)
            if (b == LARVA) {
              l1 += age_days_uncapped(a[k].age);
              const uint32_t dd = age_days(a[k].age);
              dmin = min(dmin, dd); dmax = max(dmax, dd);
            } else if (b >= IMMATURE && female) {
              fem += 1u;
              inf += a[k].sporo >= 1.0f ? 1u : 0u;
            }
          }
        }
        // ---- the warp's owed draws, dense over its lanes ----
        if (nq) {
          __syncwarp();
          for (uint32_t jq = lane; jq < nq; jq += 32) {
            const BmEntry q = bmq[jq];
            const uint32_t v = finish_box_muller(c, mc, q.gid, q.kind, q.batches);
            if (q.kind == BM_LARVA_DELAY) dst.delay[q.d] = __uint_as_float(v);
            else dst.avail[q.d] = v;
          }
          __syncwarp();  // the queue is rewritten by the next tile
        }
      } else {
        // ---- new eggs at [0, newEggs) of the next buffer ----
        const uint32_t e0 = si.lo, ne = si.newEggs;
#pragma unroll
        for (int k = 0; k < kItems; k++) {
          const uint32_t id = e0 + k * kBlock + tid;
          if (id < ne) {
            Rec a;
            new_egg(c, id, a);
            dst.age[id] = a.age; dst.his[id] = a.his; dst.delay[id] = a.delay; dst.sporo[id] = a.sporo;
            dst.uni[id] = a.uni; dst.avail[id] = a.avail; dst.cycle[id] = a.cycle; dst.hbc[id] = a.hbc;
            dst.batches[id] = a.batches;
            dst.flags[id] = (uint8_t)(EGG | (a.female << 3));
          }
        }
      }
    }
    if (cur_rep != 0xffffffffu) flush(cur_rep);
    if (fail && lane == 0) {
      // let loads still in flight land before the CTA exits (bounded waits)
      for (int s = 0; s < 2; s++) (void)mbar_wait(&full[s], (ph >> s) & 1u);
    }
  }
  if (fail && (lane == 0)) atomicOr(&p.reps[fail_rep].sim->error, SAMPO_DEV_ERR_TMA);
}

// ------------------------------------------------------------------------
// Initial population of p.reps[0]: initAgents over [0, n)
// (kernel/initAgents.cl:26-65), optionally with ages 24*U{0..age_days_max}
// from splitmix64 (an extension).
// ------------------------------------------------------------------------
__device__ __forceinline__ uint64_t mix64(uint64_t z) {
  z += 0x9E3779B97F4A7C15ULL;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
  return z ^ (z >> 31);
}

__global__ void k_init_eggs(KParams p, uint32_t n, float T0, const sampo_seeds* seeds, int age_days_max, uint64_t age_seed) {
  __shared__ StepCtx c;
  if (threadIdx.x == 0) {
    for (int k = 0; k < 4; k++) {
      c.rng_c13[k] = taus_step(seeds[k].z1 + 128u, 13, 19, 12, 4294967294u) ^ taus_step(seeds[k].z3 + 128u, 3, 11, 17, 4294967280u);
      c.rng_z2[k] = seeds[k].z2 + 128u;
      c.rng_z4[k] = seeds[k].z4;
    }
    species_step(T0, 0u, c);  // eggsIncubation(temperature[0]) (kernel/initAgents.cl:57)
  }
  __syncthreads();
  const DevPool dst = p.reps[0].pool[0];
  // 64-bit counters: a bound within one grid stride of 2^32 must not wrap
  for (uint64_t i64 = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i64 < n; i64 += (uint64_t)gridDim.x * blockDim.x) {
    const uint32_t id = (uint32_t)i64;
    Rec a;
    new_egg(c, id, a);
    if (age_days_max >= 0) {
      uint64_t z = mix64(age_seed ^ mix64((uint64_t)id));
      float h = 24.0f * (float)(uint32_t)((z >> 32) % ((uint64_t)age_days_max + 1));
      a.age = h; a.his = h;
    }
    dst.age[id] = a.age; dst.his[id] = a.his; dst.delay[id] = a.delay; dst.sporo[id] = a.sporo;
    dst.uni[id] = a.uni; dst.avail[id] = a.avail; dst.cycle[id] = a.cycle; dst.hbc[id] = a.hbc;
    dst.batches[id] = a.batches;
    dst.flags[id] = (uint8_t)(EGG | (a.female << 3));
  }
}

// Before and after a timing trial of the step kernels: zero what they add to
// (survivor counts, eggs laid, next-pool statistics, tickets). Their other
// writes - the next buffer, and tile counts and prefixes equal to the ones
// the real step computes at the same tile size (k_clear_lookback clears the
// prefixes between tile sizes) - leave the simulation's course unchanged.
__global__ void k_trial_reset(KParams p) {
  for (uint32_t r = blockIdx.x * blockDim.x + threadIdx.x; r < p.nrep; r += gridDim.x * blockDim.x) {
    SimDev* sim = p.reps[r].sim;
    for (int k = 0; k < 8; k++) sim->cnt[k] = 0;
    sim->newEggs = 0;
    sim->acc_L1de = sim->acc_fem = sim->acc_inf = 0;
    sim->acc_dmin = 0xffffffffu;
    sim->acc_dmax = 0;
    for (int k = 0; k < 4; k++) sim->acc_bnc[k] = 0;
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    p.bat->ticket1 = 0;
    p.bat->ticket2 = 0;
  }
}

// Between timing trials of different tile sizes, and after them: every
// replicate's inclusive prefixes to zero. A trial leaves prefixes tagged with
// the coming step's epoch; at another tile size they sum other slots, and the
// look-back would take them as published. Zero epochs match no step (epochs
// start at 1).
__global__ void k_clear_lookback(KParams p) {
  const size_t i0 = (size_t)blockIdx.x * blockDim.x + threadIdx.x, stride = (size_t)gridDim.x * blockDim.x;
  for (uint32_t r = 0; r < p.nrep; r++) {
    unsigned long long* incl = p.reps[r].tileIncl;
    const size_t n = (size_t)p.reps[r].maxTiles * 8;
    for (size_t i = i0; i < n; i += stride) incl[i] = 0ull;
  }
}

// Statistics of p.reps[0]'s current pool (grid-stride), accumulated into acc_*.
__global__ void k_pool_stats(KParams p) {
  SimDev* sim = p.reps[0].sim;
  const sampo_population pop = sim->pop;
  const DevPool src = p.reps[0].pool[sim->cur];
  uint32_t l1 = 0, fem = 0, inf = 0, dmin = 0xffffffffu, dmax = 0;
  const uint32_t end = pop.r[GRAVID].end;
  for (uint64_t g64 = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; g64 < end; g64 += (uint64_t)gridDim.x * blockDim.x) {
    const uint32_t g = (uint32_t)g64;
    int rg = range_of(pop, g);
    if (rg == LARVA) {
      float age = src.age[g];
      l1 += age_days_uncapped(age);
      uint32_t dd = age_days(age);
      dmin = min(dmin, dd); dmax = max(dmax, dd);
    } else if (rg >= IMMATURE) {
      if ((src.flags[g] >> 3) & 1u) { fem++; inf += src.sporo[g] >= 1.0f ? 1u : 0u; }
    }
  }
  l1 = __reduce_add_sync(0xffffffffu, l1);
  fem = __reduce_add_sync(0xffffffffu, fem);
  inf = __reduce_add_sync(0xffffffffu, inf);
  dmin = __reduce_min_sync(0xffffffffu, dmin);
  dmax = __reduce_max_sync(0xffffffffu, dmax);
  if ((threadIdx.x & 31) == 0) {
    if (l1) atomicAdd(&sim->acc_L1de, l1);
    if (fem) atomicAdd(&sim->acc_fem, fem);
    if (inf) atomicAdd(&sim->acc_inf, inf);
    if (dmin != 0xffffffffu) { atomicMin(&sim->acc_dmin, dmin); atomicMax(&sim->acc_dmax, dmax); }
  }
}

// ageHistogram (kernel/ageHistogram.cl:13-35) of p.reps[0] with
// warp-aggregated shared atomics: lanes that fall in the same bin add once.
__global__ void k_histogram(KParams p, uint32_t* hist) {
  __shared__ uint32_t h[100];
  for (int k = threadIdx.x; k < 100; k += blockDim.x) h[k] = 0;
  __syncthreads();
  SimDev* sim = p.reps[0].sim;
  const sampo_population pop = sim->pop;
  const DevPool src = p.reps[0].pool[sim->cur];
  const uint32_t lo = pop.r[IMMATURE].start, hi = pop.r[GRAVID].end;
  const uint32_t span = hi > lo ? hi - lo : 0u;
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t base = (uint64_t)blockIdx.x * blockDim.x; base < span; base += stride) {  // warp-uniform
    const uint32_t g = lo + (uint32_t)base + threadIdx.x;
    int rg = (base + threadIdx.x < span) ? range_of(pop, g) : -1;
    uint32_t bin = 0xffffffffu;
    if (rg >= IMMATURE) {
      bin = age_days_uncapped(src.age[g]);
      bin = bin < 99u ? bin : 99u;
    }
    const uint32_t peers = __match_any_sync(0xffffffffu, bin);
    if (bin != 0xffffffffu && (threadIdx.x & 31) == (uint32_t)(__ffs(peers) - 1)) atomicAdd(&h[bin], (uint32_t)__popc(peers));
  }
  __syncthreads();
  for (int k = threadIdx.x; k < 100; k += blockDim.x)
    if (h[k]) atomicAdd(&hist[k], h[k]);
}

// Diagnostic: the model's transcendental definitions evaluated on the device.
__global__ void k_eval_math(int fn, const float* x, const float* y, float* out, uint32_t n) {
  for (uint64_t i64 = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i64 < n; i64 += (uint64_t)gridDim.x * blockDim.x) {
    const size_t i = (size_t)i64;
    float v = 0.0f;
    switch (fn) {
      case 0: v = sampo_expf(x[i]); break;
      case 1: v = sampo_logf(x[i]); break;
      case 2: v = sampo_sinf(x[i]); break;
      case 3: v = sampo_powf(x[i], y[i]); break;
      case 4: v = sampo_logf_bm(x[i]); break;
      case 5: v = sampo_sinf_bm(x[i]); break;
      default: break;
    }
    out[i] = v;
  }
}

}  // namespace sampo
