// sampo_kernels.cu - the SAMPO hourly step on GB300 (sm_103a).
//
// A step is two persistent-CTA kernels over the current pool buffer:
//
//  k_count   reads the ~12 bytes per agent that decide survival, the next
//            state and the eggs laid (killAgents + the decision part of
//            updateAgents), and publishes per 1024-slot tile the number of
//            survivors per next state plus the step's newEggs total.
//  k_scatter recomputes the same decisions with the complete record,
//            obtains each survivor's stable rank within its next state
//            (warp match/popc + a block scan + a decoupled look-back over
//            the tile counts that k_count already published, so no CTA ever
//            waits on another), writes the updated record to its slot in the
//            other buffer (the reference's oldToNewAgents layout,
//            kernel/oldToNewAgents.cl:57-95,126-226), writes the new eggs at
//            [0, newEggs) (initAgents, kernel/initAgents.cl:26-65), and
//            accumulates the next step's statistics (calcL1de.cl,
//            calcGender.cl). The last CTA to finish publishes the next
//            population, the stats row and the larval mortality table.
//
// Both kernels stream tiles through shared memory with TMA bulk copies
// (cp.async.bulk + mbarrier, double-buffered: tile j+1 is in flight while
// tile j is processed). k_count loads only the columns the tile's ranges
// need; k_scatter reuses the input stage as the output staging area, sorted
// by next state, and writes each state's run with coalesced stores.
//
// This replaces the reference's 19 kernels per step (killAgents,
// updateAgents, initAgents, 3 x preScan + 3 x Bolt scan-by-key,
// oldToNewAgents, calcL1de x2, calcFemales x2) and its blocking transfers.
#include <cuda_runtime.h>
#include "sampo_model.cuh"
#include "sampo_kernels.cuh"

namespace sampo {

// include/properties.h:94-98 (double literals stored as float, as there)
__device__ const float kDevRates[32] = {
    0.000175044, 0.000549094, 0.00109031, 0.001494158, 0.001752487, 0.001962866, 0.002171238, 0.002392989,
    0.002633689, 0.00289619, 0.003182685, 0.003495287, 0.003836204, 0.004207789, 0.004612566, 0.005053243,
    0.005532729, 0.006054144, 0.006620836, 0.007236393, 0.007904657, 0.008629745, 0.009416051, 0.010267388,
    0.011113704, 0.011960019, 0.012806335, 0.010401163, 0.007995991, 0.00033845, 0.00000533086, 0.0000000840986};

constexpr uint32_t kColBytes = kTile * 4;                    // one 4-byte column of a tile
constexpr uint32_t kCountStage = 5 * kColBytes + kTile;      // age, his, delay, uni, avail, flags
// Output staging: each next-state run starts at a staging element with the
// same residue modulo 16 as its destination slot, so that shared and global
// addresses of a run agree modulo 16 bytes for every column (the condition
// for bulk stores); 8 runs add at most 8 x 30 elements of padding.
constexpr uint32_t kStg = kTile + 256;                       // staging elements per column
constexpr uint32_t kScatterStage = 9 * kStg * 4 + kStg;      // >= the input layout (9 x kColBytes + kTile)
constexpr uint32_t kWaitLimit = 1u << 22;                    // bounded mbarrier waits

// ---------------- memory-model and TMA helpers ----------------
__device__ __forceinline__ uint32_t ld_acquire_u32(const uint32_t* p) {
  uint32_t v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void st_release_u32(uint32_t* p, uint32_t v) {
  asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
__device__ __forceinline__ uint4 ld_cg_v4(const uint32_t* p) {
  uint4 v;
  asm volatile("ld.global.cg.v4.u32 {%0,%1,%2,%3}, [%4];" : "=r"(v.x), "=r"(v.y), "=r"(v.z), "=r"(v.w) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void st_cg_v4(uint32_t* p, uint4 v) {
  asm volatile("st.global.cg.v4.u32 [%0], {%1,%2,%3,%4};" ::"l"(p), "r"(v.x), "r"(v.y), "r"(v.z), "r"(v.w) : "memory");
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
// 1-D bulk copy shared -> global in the issuing thread's bulk group (both
// addresses 16-byte aligned, bytes a multiple of 16).
__device__ __forceinline__ void bulk_store(void* dst, const void* src, uint32_t bytes) {
  asm volatile("cp.async.bulk.global.shared::cta.bulk_group [%0], [%1], %2;" ::"l"(dst), "r"(smem_addr(src)), "r"(bytes)
               : "memory");
}
__device__ __forceinline__ void bulk_commit() { asm volatile("cp.async.bulk.commit_group;" ::: "memory"); }
// the shared-memory sources of this thread's bulk stores may be overwritten
__device__ __forceinline__ void bulk_wait_read() { asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory"); }
// this thread's bulk stores are complete
__device__ __forceinline__ void bulk_wait_all() { asm volatile("cp.async.bulk.wait_group 0;" ::: "memory"); }

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

struct alignas(16) SharedCtx {
  StepCtx c;
  sampo_population pop;
  uint32_t cur, epoch, step;
};

__device__ void load_ctx(const KParams& p, SharedCtx& s) {
  SimDev* sim = p.sim;
  if (threadIdx.x == 0) {
    StepCtx& c = s.c;
    uint32_t step = sim->step;
    uint32_t i = step % p.ring;
    const sampo_seeds* sd = p.seeds + (size_t)i * 4;
#pragma unroll
    for (int k = 0; k < 4; k++) {
      c.rng_c13[k] = taus_step(sd[k].z1 + 128u, 13, 19, 12, 4294967294u) ^ taus_step(sd[k].z3 + 128u, 3, 11, 17, 4294967280u);
      c.rng_z2[k] = sd[k].z2 + 128u;
      c.rng_z4[k] = sd[k].z4;
    }
    c.env = p.env[i];
    float T = p.T[i];
    c.T = T;
    c.wt = p.wt[i];
    s.pop = sim->pop;
    c.totalBiomass = s.pop.numLarvae1DayEquiv + s.pop.r[EGG].end + (s.pop.r[PUPA].end - s.pop.r[PUPA].start);
    c.aquaticHMR = sim->aquaticHMR;
    c.eggIncubation = -0.923f * T + 60.923f;                           // include/properties.h:29-31
    float cl = sampo_fminf(sampo_fmaxf(T, 12.0f), 48.0f);               // :105-109
    int di = (int)cl - 12;
    c.devOOB = di > 31;
    c.larvaDev = di > 31 ? 0.0f : kDevRates[di];
    c.pupaDelay = __double2float_rn(__dadd_rn(__dmul_rn(-0.923, (double)T), 60.923));  // :133-135
    c.immatureDelay = -2.667f * T + 120.0f;                            // :159-161
    c.bmdDelay = -1.231f * T + 77.231f;                                // :239-241
    c.sporoOn = T > 16.0f;                                             // kernel/updateAgents.cl:69-70
    c.sporoInc = __ddiv_rn(1.0, __dmul_rn((double)(111.0f / (T - 16.0f)), 14.0));
    sampo_split_double(c.sporoInc, &c.sporoH, &c.sporoM, &c.sporoL);
    s.cur = sim->cur;
    s.epoch = sim->epoch;
    s.step = step;
  }
  for (int k = threadIdx.x; k < 100; k += blockDim.x) {
    s.c.adultHMR[k] = sim->adultHMR[k];
    s.c.larvaHMR[k] = sim->larvaHMR[k];
    if (k < kEggBatchTable) s.c.eggBatchScale[k] = sim->eggBatchScale[k];
  }
  __syncthreads();
}

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

__device__ void issue_count_tile(const DevPool& src, uint8_t* st, uint64_t* bar, const sampo_population& pop,
                                 uint32_t lo, uint32_t n, bool larvicide) {
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

__global__ void __launch_bounds__(kBlock) k_count(KParams p) {
  extern __shared__ __align__(128) uint8_t dsm[];
  __shared__ SharedCtx S;
  __shared__ __align__(8) uint64_t bars[2];
  __shared__ uint32_t s_tick[2];
  __shared__ uint32_t s_wcnt[kWarps][8];
  load_ctx(p, S);
  const StepCtx& c = S.c;
  SimDev* sim = p.sim;
  const DevPool src = p.pool[S.cur];
  const uint32_t end = S.pop.r[GRAVID].end;
  const uint32_t ntiles = (end + kTile - 1) / kTile;
  const bool larvicide = c.env.larvacideValue > 0.0f;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  Acc acc = {0, 0, 0, 0, 0, 0};
  uint32_t cta_cnt = 0;  // thread b < 8: this CTA's survivors of next state b
  uint32_t devoob = 0, phase = 0, pend = 0;  // pend (thread 0): stages with a copy in flight
  bool failed = false;

  if (tid == 0) {
    mbar_init(&bars[0]);
    mbar_init(&bars[1]);
    fence_mbar_init();
    fence_proxy_async();
    const uint32_t t = atomicAdd(&sim->ticket1, 1u);
    s_tick[0] = t;
    if (t < ntiles) {
      issue_count_tile(src, dsm, &bars[0], S.pop, t * kTile, min((uint32_t)kTile, end - t * kTile), larvicide);
      pend |= 1u;
    }
  }
  __syncthreads();

  for (uint32_t it = 0;; it++) {
    const uint32_t sidx = it & 1u;
    const uint32_t t = s_tick[sidx];
    if (t >= ntiles) break;
    uint8_t* st = dsm + sidx * kCountStage;
    if (tid == 0) {  // prefetch the next tile into the other stage
      const uint32_t t2 = atomicAdd(&sim->ticket1, 1u);
      s_tick[sidx ^ 1u] = t2;
      if (t2 < ntiles) {
        fence_proxy_async();
        issue_count_tile(src, dsm + (sidx ^ 1u) * kCountStage, &bars[sidx ^ 1u], S.pop, t2 * kTile,
                         min((uint32_t)kTile, end - t2 * kTile), larvicide);
        pend |= 2u >> sidx;
      }
    }
    const bool ok = mbar_wait(&bars[sidx], (phase >> sidx) & 1u);
    if (ok) {
      phase ^= 1u << sidx;
      pend &= ~(1u << sidx);
    }
    const uint32_t lo = t * kTile;
    const float* s_age = (const float*)(st + 0 * kColBytes);
    const float* s_his = (const float*)(st + 1 * kColBytes);
    const float* s_delay = (const float*)(st + 2 * kColBytes);
    const uint32_t* s_uni = (const uint32_t*)(st + 3 * kColBytes);
    const uint32_t* s_avail = (const uint32_t*)(st + 4 * kColBytes);
    const uint8_t* s_flags = st + 5 * kColBytes;
    uint32_t pk0 = 0, pk1 = 0;  // 8-bit survivor counters: buckets 0-3, 4-7
#pragma unroll
    for (int k = 0; k < kItems; k++) {
      const uint32_t i = k * kBlock + tid;
      const uint32_t g = lo + i;
      const int rg = (ok && g < end) ? range_of(S.pop, g) : -1;
      if (rg >= 0) {
        Rec a;
        a.age = (rg == LARVA || rg >= IMMATURE) ? s_age[i] : 0.0f;
        a.his = (rg != GRAVID && (rg != LARVA || larvicide)) ? s_his[i] : 0.0f;
        a.delay = rg != GRAVID ? s_delay[i] : 0.0f;
        a.uni = (rg == LARVA || rg == GRAVID) ? s_uni[i] : 0u;
        a.avail = rg == GRAVID ? s_avail[i] : 0u;
        a.female = rg == MATESEEKING ? (s_flags[i] >> 3) & 1u : 0u;
        a.sporo = 0.0f; a.cycle = 0u; a.hbc = 0u; a.batches = 0u;
        devoob |= (rg == LARVA) & c.devOOB;
        const int ns = update_agent<false>(c, rg, g, a, acc);
        if (ns >= 0) {
          if (ns < 4) pk0 += 1u << (8 * ns);
          else pk1 += 1u << (8 * (ns - 4));
        }
      }
    }
    pk0 = __reduce_add_sync(0xffffffffu, pk0);
    pk1 = __reduce_add_sync(0xffffffffu, pk1);
    if (lane < 8) s_wcnt[warp][lane] = ((lane < 4 ? pk0 : pk1) >> (8 * (lane & 3))) & 0xffu;
    __syncthreads();
    if (tid < 8) {
      uint32_t sum = 0;
#pragma unroll
      for (int w = 0; w < kWarps; w++) sum += s_wcnt[w][tid];
      p.tileAgg[(size_t)t * 8 + tid] = sum;
      cta_cnt += sum;
    }
    if (__syncthreads_or(!ok)) { failed = true; break; }
  }
  if (failed && tid == 0) {
    atomicOr(&sim->error, SAMPO_DEV_ERR_TMA);
    for (int s = 0; s < 2; s++)  // let copies still in flight land before the CTA exits
      if ((pend >> s) & 1u) (void)mbar_wait(&bars[s], (phase >> s) & 1u);
  }
  if (tid < 8 && cta_cnt) atomicAdd(&sim->cnt[tid], cta_cnt);
  const uint32_t ne = __reduce_add_sync(0xffffffffu, acc.newEggs);
  if (lane == 0 && ne) atomicAdd(&sim->newEggs, ne);
  const uint32_t bad = __reduce_or_sync(0xffffffffu, (acc.bad ? SAMPO_DEV_ERR_LARVATABLE : 0u) | (devoob ? SAMPO_DEV_ERR_DEVRATES : 0u));
  if (lane == 0 && bad) atomicOr(&sim->error, bad);
}

// ------------------------------------------------------------------------
// Publishing the statistics of the pool a step starts from: L1de, female and
// infective counts (calcStats, src/abms.c:230-310), the stats row, and the
// larval hourly mortality for every larva age present this step
// (kernel/killAgents.cl:117-133 depends on the age and L1de only). Run by one
// CTA, all threads. Reads and clears the acc_* accumulators.
// ------------------------------------------------------------------------
__device__ void publish_start(const KParams& p, const sampo_population& ranges, bool count_bnc) {
  SimDev* sim = p.sim;
  __shared__ uint32_t s_l1, s_dmin, s_dmax;
  __shared__ float s_cc;
  if (threadIdx.x == 0) {
    volatile SimDev* vs = sim;
    sampo_population np = ranges;
    uint32_t l1 = vs->acc_L1de;
    np.numLarvae1DayEquiv = (np.r[LARVA].end > np.r[LARVA].start) ? l1 : 0u;  // kernel/calcL1de.cl:259-280
    np.numFemale = vs->acc_fem;
    np.numPotentiallyInfective = vs->acc_inf;
    sim->pop = np;
    if (count_bnc) {
      sim->bnc.numCyclesReported = vs->acc_bnc[0];
      sim->bnc.sumCyclesReported = vs->acc_bnc[1];
      sim->bnc.numBitesReported = vs->acc_bnc[2];
      sim->bnc.numInfectBitesReported = vs->acc_bnc[3];
    }
    sampo_stats_row row;
    row.pop = np;
    row.bnc = sim->bnc;
    p.rows[sim->step % p.ring] = row;
    s_l1 = np.numLarvae1DayEquiv;
    s_dmin = vs->acc_dmin;
    s_dmax = vs->acc_dmax;
    s_cc = sim->cc;
    sim->acc_L1de = 0; sim->acc_fem = 0; sim->acc_inf = 0;
    sim->acc_dmin = 0xffffffffu; sim->acc_dmax = 0;
    sim->acc_bnc[0] = sim->acc_bnc[1] = sim->acc_bnc[2] = sim->acc_bnc[3] = 0;
  }
  __syncthreads();
  for (int d = threadIdx.x; d < 100; d += blockDim.x) {
    float hmr = SAMPO_NAN_F;
    if ((uint32_t)d >= s_dmin && (uint32_t)d <= s_dmax) {
      // kernel/killAgents.cl:117-125
      float dmr = 0.1f * sampo_expf((float)s_l1 / ((float)(uint32_t)d * s_cc * 1.0f));
      dmr = sampo_fminf(dmr, 0.8f);
      float dsr = 1.0f - dmr;
      float hsr = sampo_powf(dsr, 1.0f / 24.0f);
      hmr = 1.0f - hsr;
    }
    sim->larvaHMR[d] = hmr;
  }
}

// ------------------------------------------------------------------------
// Update + scatter pass
// ------------------------------------------------------------------------
__device__ void issue_scatter_tile(const DevPool& src, uint8_t* st, uint64_t* bar, uint32_t lo, uint32_t n) {
  const uint32_t b4 = (n * 4 + 15) & ~15u, b1 = (n + 15) & ~15u;
  mbar_arrive_tx(bar, 9 * b4 + b1);
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

// Decoupled look-back for tile t by one warp over the count pass's tile
// aggregates: sums earlier tiles' aggregates back to the nearest published
// inclusive prefix (no waiting). Lane 0 publishes t's inclusive prefix.
// Every lane returns the exclusive prefix ex[] and t's counts cnt[].
__device__ void tile_lookback(const KParams& p, uint32_t t, uint32_t epoch, int lane, uint32_t ex[8], uint32_t cnt[8]) {
#pragma unroll
  for (int b = 0; b < 8; b++) ex[b] = 0;
  int64_t pos = (int64_t)t - 1;
  while (pos >= 0) {
    const int64_t idx = pos - lane;
    const bool valid = idx >= 0;
    const uint32_t f = valid ? ld_acquire_u32(&p.tileFlag[idx]) : 0u;
    const uint32_t m = __ballot_sync(0xffffffffu, !valid || f == epoch);
    const int stop = m ? __ffs(m) - 1 : 32;
    uint4 v0 = make_uint4(0, 0, 0, 0), v1 = v0;
    if (valid && lane <= stop) {
      const uint32_t* q = (lane == stop ? p.tileIncl : p.tileAgg) + (size_t)idx * 8;
      v0 = ld_cg_v4(q);
      v1 = ld_cg_v4(q + 4);
    }
    ex[0] += __reduce_add_sync(0xffffffffu, v0.x); ex[1] += __reduce_add_sync(0xffffffffu, v0.y);
    ex[2] += __reduce_add_sync(0xffffffffu, v0.z); ex[3] += __reduce_add_sync(0xffffffffu, v0.w);
    ex[4] += __reduce_add_sync(0xffffffffu, v1.x); ex[5] += __reduce_add_sync(0xffffffffu, v1.y);
    ex[6] += __reduce_add_sync(0xffffffffu, v1.z); ex[7] += __reduce_add_sync(0xffffffffu, v1.w);
    if (m) break;
    pos -= 32;
  }
  const uint32_t* ag = p.tileAgg + (size_t)t * 8;
  const uint4 a0 = ld_cg_v4(ag), a1 = ld_cg_v4(ag + 4);
  cnt[0] = a0.x; cnt[1] = a0.y; cnt[2] = a0.z; cnt[3] = a0.w; cnt[4] = a1.x; cnt[5] = a1.y; cnt[6] = a1.z; cnt[7] = a1.w;
  if (lane == 0) {
    st_cg_v4(p.tileIncl + (size_t)t * 8, make_uint4(ex[0] + a0.x, ex[1] + a0.y, ex[2] + a0.z, ex[3] + a0.w));
    st_cg_v4(p.tileIncl + (size_t)t * 8 + 4, make_uint4(ex[4] + a1.x, ex[5] + a1.y, ex[6] + a1.z, ex[7] + a1.w));
    st_release_u32(&p.tileFlag[t], epoch);
  }
}

// Named barrier of the eight consumer warps (the producer warp is not in it).
__device__ __forceinline__ void consumer_sync() { asm volatile("bar.sync 1, 256;" ::: "memory"); }
__device__ __forceinline__ void mbar_init_count(uint64_t* bar, uint32_t n) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(n) : "memory");
}
__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_addr(bar)) : "memory");
}

constexpr int kScatterThreads = kBlock + 32;  // eight consumer warps and one producer warp
static_assert(kBlock == 256, "consumer_sync() names 256 threads");
enum : uint32_t { TK_OLD = 0, TK_EGG = 1, TK_END = 2 };

// The producer warp keeps two tiles in flight ahead of the consumers: it
// takes tickets, issues the TMA loads, runs the look-back and lays out the
// staging runs (full[s]: its expect-tx arrival + one arrival once the layout
// is written); after the consumers have staged a tile (empty[s]: 256
// arrivals) it sends the runs with bulk stores and refills the stage.
__global__ void __launch_bounds__(kScatterThreads, 2) k_scatter(KParams p) {
  extern __shared__ __align__(128) uint8_t dsm[];
  __shared__ SharedCtx S;
  __shared__ __align__(8) uint64_t full[2], empty[2];
  __shared__ sampo_population s_np;
  __shared__ uint32_t s_base[8], s_newEggs, s_ok, s_last, s_tick[2], s_fullok[2];
  __shared__ uint32_t s_d0[2][8], s_sb[2][8], s_cnt[2][8];  // per stage and next state: first slot, staging start, survivors
  __shared__ uint32_t s_off[kItems][kWarps][8];
  __shared__ uint32_t s_red[kWarps][8];
  __shared__ uint32_t s_mn[kWarps], s_mx[kWarps];
  __shared__ uint32_t s_bmq[kTile], s_bmn;  // owed Box-Muller draws: staging slot | item << 11 | kind << 21
  load_ctx(p, S);
  const StepCtx& c = S.c;
  SimDev* sim = p.sim;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  if (tid == 0) {
    uint32_t cnt[8];
    for (int k = 0; k < 8; k++) cnt[k] = sim->cnt[k];
    s_newEggs = sim->newEggs;
    next_layout(cnt, s_newEggs, s_np, s_base);
    uint64_t tot = (uint64_t)s_newEggs + cnt[0];
    bool ok = tot <= 0xffffffffull;
    uint64_t e = tot;
    for (int k = 1; k < 8; k++) e = ((e + kLayoutAlign) / kLayoutAlign) * kLayoutAlign + cnt[k];
    ok = ok && e <= (uint64_t)sim->capacity;
    s_ok = ok;
    if (!ok && blockIdx.x == 0) atomicOr(&sim->error, SAMPO_DEV_ERR_CAPACITY);
    mbar_init_count(&full[0], 2);
    mbar_init_count(&full[1], 2);
    mbar_init_count(&empty[0], kBlock);
    mbar_init_count(&empty[1], kBlock);
    fence_mbar_init();
  }
  __syncthreads();
  const DevPool src = p.pool[S.cur];
  const DevPool dst = p.pool[S.cur ^ 1];
  const uint32_t end = S.pop.r[GRAVID].end;
  const uint32_t nold = s_ok ? (end + kTile - 1) / kTile : 0u;
  const uint32_t negg = s_ok ? (s_newEggs + kTile - 1) / kTile : 0u;
  const uint32_t ntot = nold + negg;
  const uint32_t epoch = S.epoch;

  Acc acc = {0, 0, 0, 0, 0, 0};
  uint32_t l1 = 0, fem = 0, inf = 0, dmin = 0xffffffffu, dmax = 0, tilebad = 0, fail = 0;

  if (warp == kWarps) {
    // ================= producer warp =================
    // fill stage s with the next ticket's tile; returns its kind
    auto fill = [&](uint32_t s) -> uint32_t {
      uint32_t t = 0;
      if (lane == 0) {
        t = atomicAdd(&sim->ticket2, 1u);
        s_tick[s] = t;
      }
      t = __shfl_sync(0xffffffffu, t, 0);
      if (t < nold) {
        if (lane == 0) {
          fence_proxy_async();  // the stage was last written through the generic proxy
          issue_scatter_tile(src, dsm + s * kScatterStage, &full[s], t * kTile, min((uint32_t)kTile, end - t * kTile));
        }
        uint32_t ex[8], cnt[8];
        tile_lookback(p, t, epoch, lane, ex, cnt);
        if (lane == 0) {
          uint32_t pos = 0;
#pragma unroll
          for (int b = 0; b < 8; b++) {
            const uint32_t d0 = s_base[b] + ex[b];
            const uint32_t sb = ((pos + 15u) & ~15u) + (d0 & 15u);
            s_d0[s][b] = d0;
            s_sb[s][b] = sb;
            s_cnt[s][b] = cnt[b];
            pos = sb + cnt[b];
          }
          mbar_arrive(&full[s]);  // layout written (release)
        }
        return TK_OLD;
      }
      if (lane == 0) {
        mbar_arrive(&full[s]);
        mbar_arrive(&full[s]);
      }
      return t < ntot ? TK_EGG : TK_END;
    };
    uint32_t kind0 = fill(0), kind1 = fill(1), ph = 0;
    for (uint32_t it = 0;; it++) {
      const uint32_t s = it & 1u;
      const uint32_t k = s ? kind1 : kind0;
      if (k == TK_END) break;
      uint32_t ok = 1;
      if (lane == 0) ok = mbar_wait(&empty[s], (ph >> s) & 1u) ? 1u : 0u;
      ok = __shfl_sync(0xffffffffu, ok, 0);
      if (!ok) { fail = 1; break; }
      ph ^= 1u << s;
      if (k == TK_OLD && lane == 0) {
        // ---- each state's run to its slots in the next buffer ----
        // staging and destination agree modulo 16 bytes: the aligned body of
        // every run and column leaves with one bulk store; the consumers
        // wrote the unaligned heads and tails. Runs lie inside the next
        // layout by construction (d0 + count <= range end).
        uint8_t* st = dsm + s * kScatterStage;
        fence_proxy_async();  // staging written through the generic proxy
#pragma unroll 1
        for (int b = 0; b < 8; b++) {
          const uint32_t n = s_cnt[s][b], d0 = s_d0[s][b], sb = s_sb[s][b];
          if (!n) continue;
          const uint32_t h4 = min((4u - (d0 & 3u)) & 3u, n), n4 = (n - h4) & ~3u;
          if (n4) {
            const uint32_t o = h4, by = n4 * 4, so = (sb + o) * 4;
            bulk_store(dst.age + d0 + o, st + 0 * kStg * 4 + so, by);
            bulk_store(dst.his + d0 + o, st + 1 * kStg * 4 + so, by);
            bulk_store(dst.delay + d0 + o, st + 2 * kStg * 4 + so, by);
            bulk_store(dst.sporo + d0 + o, st + 3 * kStg * 4 + so, by);
            bulk_store(dst.uni + d0 + o, st + 4 * kStg * 4 + so, by);
            bulk_store(dst.avail + d0 + o, st + 5 * kStg * 4 + so, by);
            bulk_store(dst.cycle + d0 + o, st + 6 * kStg * 4 + so, by);
            bulk_store(dst.hbc + d0 + o, st + 7 * kStg * 4 + so, by);
            bulk_store(dst.batches + d0 + o, st + 8 * kStg * 4 + so, by);
          }
          const uint32_t h1 = min((16u - (d0 & 15u)) & 15u, n), n1 = (n - h1) & ~15u;
          if (n1) bulk_store(dst.flags + d0 + h1, st + 9 * kStg * 4 + sb + h1, n1);
        }
        bulk_commit();
      }
      if (lane == 0) bulk_wait_read();  // the stage's sources are read: it may be refilled
      __syncwarp();
      const uint32_t nk = fill(s);
      if (s) kind1 = nk;
      else kind0 = nk;
    }
    if (lane == 0) bulk_wait_all();  // this CTA's bulk stores are complete
  } else {
    // ================= consumer warps =================
    uint32_t ph = 0;
    for (uint32_t it = 0;; it++) {
      const uint32_t s = it & 1u;
      uint8_t* st = dsm + s * kScatterStage;
      for (int q = tid; q < kItems * kWarps * 8; q += kBlock) (&s_off[0][0][0])[q] = 0u;
      if (tid == 0) {
        s_bmn = 0;
        s_fullok[s] = mbar_wait(&full[s], (ph >> s) & 1u) ? 1u : 0u;
      }
      consumer_sync();
      if (!s_fullok[s]) { fail = 1; break; }
      (void)mbar_try_wait(&full[s], (ph >> s) & 1u);  // the completed phase, observed by this thread
      ph ^= 1u << s;
      const uint32_t t = s_tick[s];
      if (t >= ntot) break;
      if (t < nold) {
        // ---- recompute the step for the tile's agents (inputs from shared memory) ----
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
        const uint32_t lo = t * kTile;
        Rec a[kItems];
        int nb[kItems];
        uint32_t rk[kItems];
#pragma unroll
        for (int k = 0; k < kItems; k++) {
          const uint32_t i = k * kBlock + tid;
          const uint32_t g = lo + i;
          const int rg = g < end ? range_of(S.pop, g) : -1;
          nb[k] = 8;
          a[k].bm = BM_NONE;
          if (rg >= 0) {
            a[k].age = c_age[i]; a[k].his = c_his[i]; a[k].delay = c_delay[i]; a[k].sporo = c_sporo[i];
            a[k].uni = c_uni[i]; a[k].avail = c_avail[i]; a[k].cycle = c_cycle[i]; a[k].hbc = c_hbc[i];
            a[k].batches = c_batches[i];
            a[k].female = (c_flags[i] >> 3) & 1u;
            const int ns = update_agent<true>(c, rg, g, a[k], acc);
            if (ns >= 0) nb[k] = ns;
          }
          const uint32_t peers = __match_any_sync(0xffffffffu, nb[k]);
          rk[k] = __popc(peers & lanemask_lt());
          if (nb[k] < 8 && lane == __ffs(peers) - 1) s_off[k][warp][nb[k]] = __popc(peers);
        }
        consumer_sync();  // inputs consumed (the stage becomes the output staging area), counts written
        // ---- exclusive scan of the (round, warp) counts, one warp per state ----
        {
          const int b = warp;
          const uint32_t v = (&s_off[0][0][0])[lane * 8 + b];  // entry (round, warp) = lane, kItems*kWarps == 32
          uint32_t incl = v;
#pragma unroll
          for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o) incl += y;
          }
          (&s_off[0][0][0])[lane * 8 + b] = incl - v;
          if (lane == 31 && incl != s_cnt[s][b]) tilebad = 1;
        }
        consumer_sync();
        float* g_age = (float*)(st + 0 * kStg * 4);
        float* g_his = (float*)(st + 1 * kStg * 4);
        float* g_delay = (float*)(st + 2 * kStg * 4);
        float* g_sporo = (float*)(st + 3 * kStg * 4);
        uint32_t* g_uni = (uint32_t*)(st + 4 * kStg * 4);
        uint32_t* g_avail = (uint32_t*)(st + 5 * kStg * 4);
        uint32_t* g_cycle = (uint32_t*)(st + 6 * kStg * 4);
        uint32_t* g_hbc = (uint32_t*)(st + 7 * kStg * 4);
        uint32_t* g_batches = (uint32_t*)(st + 8 * kStg * 4);
        uint8_t* g_flags = st + 9 * kStg * 4;
        // ---- survivors into the staging area, sorted by next state ----
#pragma unroll
        for (int k = 0; k < kItems; k++) {
          const int b = nb[k];
          uint32_t q = 0xffffffffu;
          if (b < 8) {
            const uint32_t j = s_off[k][warp][b] + rk[k];
            if (j < s_cnt[s][b]) q = s_sb[s][b] + j;
            else tilebad = 1;  // the two passes disagree: stay inside this state's run
          }
          // queue the owed Box-Muller draws (warp-aggregated slot reservation)
          const bool owe = q != 0xffffffffu && a[k].bm != BM_NONE;
          const uint32_t om = __ballot_sync(0xffffffffu, owe);
          if (om) {
            uint32_t qb = 0;
            if (lane == __ffs(om) - 1) qb = atomicAdd(&s_bmn, (uint32_t)__popc(om));
            qb = __shfl_sync(0xffffffffu, qb, __ffs(om) - 1);
            if (owe) s_bmq[qb + __popc(om & lanemask_lt())] = q | ((uint32_t)(k * kBlock + tid) << 11) | (a[k].bm << 21);
          }
          if (q != 0xffffffffu) {
            g_age[q] = a[k].age; g_his[q] = a[k].his; g_delay[q] = a[k].delay; g_sporo[q] = a[k].sporo;
            g_uni[q] = a[k].uni; g_avail[q] = a[k].avail; g_cycle[q] = a[k].cycle; g_hbc[q] = a[k].hbc;
            g_batches[q] = a[k].batches;
            g_flags[q] = (uint8_t)(b | (a[k].female << 3));
            // statistics of the next pool (kernel/calcL1de.cl:28-30, kernel/calcGender.cl:24-37)
            if (b == LARVA) {
              l1 += age_days_uncapped(a[k].age);
              const uint32_t dd = age_days(a[k].age);
              dmin = min(dmin, dd); dmax = max(dmax, dd);
            } else if (b >= IMMATURE && a[k].female) {
              fem += 1u;
              inf += a[k].sporo >= 1.0f ? 1u : 0u;
            }
          }
        }
        consumer_sync();
        // ---- the owed Box-Muller draws, in dense warps, patched into the staging area ----
        const uint32_t nbm = s_bmn;
        if (nbm) {
          for (uint32_t j = tid; j < nbm; j += kBlock) {
            const uint32_t e = s_bmq[j];
            const uint32_t q = e & 2047u, kind = e >> 21;
            const uint32_t v = finish_box_muller(c, lo + ((e >> 11) & 1023u), kind, g_batches[q]);
            if (kind == BM_LARVA_DELAY) g_delay[q] = __uint_as_float(v);
            else g_avail[q] = v;
          }
          consumer_sync();
        }
        // ---- heads and tails of the runs: per state at most 15 + 15 flag
        //      elements, of which the four-byte columns need at most 3 + 3 ----
        {
          const int b = warp, e = lane;
          const uint32_t n = s_cnt[s][b], d0 = s_d0[s][b], sb = s_sb[s][b];
          const uint32_t h4 = min((4u - (d0 & 3u)) & 3u, n), n4 = (n - h4) & ~3u;
          const uint32_t h1 = min((16u - (d0 & 15u)) & 15u, n), n1 = (n - h1) & ~15u;
          const uint32_t j = (uint32_t)e < h1 ? (uint32_t)e : h1 + n1 + ((uint32_t)e - h1);
          if (e < 30 && j < n) {
            const uint32_t q = sb + j, d = d0 + j;
            dst.flags[d] = g_flags[q];
            if (j < h4 || j >= h4 + n4) {
              dst.age[d] = g_age[q]; dst.his[d] = g_his[q]; dst.delay[d] = g_delay[q]; dst.sporo[d] = g_sporo[q];
              dst.uni[d] = g_uni[q]; dst.avail[d] = g_avail[q]; dst.cycle[d] = g_cycle[q]; dst.hbc[d] = g_hbc[q];
              dst.batches[d] = g_batches[q];
            }
          }
        }
      } else {
        // ---- new eggs at [0, newEggs) of the next buffer ----
        const uint32_t e0 = (t - nold) * kTile;
#pragma unroll
        for (int k = 0; k < kItems; k++) {
          const uint32_t id = e0 + k * kBlock + tid;
          if (id < s_newEggs) {
            Rec a;
            new_egg(c, id, a);
            dst.age[id] = a.age; dst.his[id] = a.his; dst.delay[id] = a.delay; dst.sporo[id] = a.sporo;
            dst.uni[id] = a.uni; dst.avail[id] = a.avail; dst.cycle[id] = a.cycle; dst.hbc[id] = a.hbc;
            dst.batches[id] = a.batches;
            dst.flags[id] = (uint8_t)(EGG | (a.female << 3));
          }
        }
      }
      mbar_arrive(&empty[s]);  // staged (release): the producer may send and refill the stage
    }
  }
  if (fail) atomicOr(&sim->error, SAMPO_DEV_ERR_TMA);
  __syncthreads();

  // ---- per-CTA reduction of the accumulators, one atomic each ----
  {
    uint32_t v[8] = {l1, fem, inf, acc.cycles, acc.sumCycles, acc.bites, acc.infectBites,
                     (acc.bad ? SAMPO_DEV_ERR_LARVATABLE : 0u) | (tilebad ? SAMPO_DEV_ERR_TILECOUNT : 0u)};
#pragma unroll
    for (int j = 0; j < 8; j++) v[j] = j == 7 ? __reduce_or_sync(0xffffffffu, v[j]) : __reduce_add_sync(0xffffffffu, v[j]);
    const uint32_t mn = __reduce_min_sync(0xffffffffu, dmin), mx = __reduce_max_sync(0xffffffffu, dmax);
    if (lane == 0 && warp < kWarps) {
#pragma unroll
      for (int j = 0; j < 8; j++) s_red[warp][j] = v[j];
      s_mn[warp] = mn;
      s_mx[warp] = mx;
    }
    __syncthreads();
    if (tid == 0) {
      uint32_t r[8] = {0, 0, 0, 0, 0, 0, 0, 0}, rmn = 0xffffffffu, rmx = 0;
      for (int w = 0; w < kWarps; w++) {
        for (int j = 0; j < 7; j++) r[j] += s_red[w][j];
        r[7] |= s_red[w][7];
        rmn = min(rmn, s_mn[w]); rmx = max(rmx, s_mx[w]);
      }
      if (r[0]) atomicAdd(&sim->acc_L1de, r[0]);
      if (r[1]) atomicAdd(&sim->acc_fem, r[1]);
      if (r[2]) atomicAdd(&sim->acc_inf, r[2]);
      if (r[3]) atomicAdd(&sim->acc_bnc[0], r[3]);
      if (r[4]) atomicAdd(&sim->acc_bnc[1], r[4]);
      if (r[5]) atomicAdd(&sim->acc_bnc[2], r[5]);
      if (r[6]) atomicAdd(&sim->acc_bnc[3], r[6]);
      if (r[7]) atomicOr(&sim->error, r[7]);
      if (rmn != 0xffffffffu) { atomicMin(&sim->acc_dmin, rmn); atomicMax(&sim->acc_dmax, rmx); }
      __threadfence();
      s_last = atomicAdd(&sim->done2, 1u) == gridDim.x - 1;
    }
    __syncthreads();
  }
  if (!s_last) return;

  // ---- epilogue: the last CTA publishes the next step's start ----
  __threadfence();
  if (tid == 0) {
    // the reference's shared empty initial ranges (src/abms.c:204-219) make
    // oldToNewAgents read one prefix-sum entry for several range ends
    const sampo_population& op = S.pop;
    bool shared_end = false;
    for (int k = 1; k < 8; k++) shared_end |= op.r[k].end == op.r[k - 1].end;
    uint32_t moved = 0;
    for (int k = 1; k < 8; k++) moved += sim->cnt[k];
    if (shared_end && moved) atomicOr(&sim->warn, SAMPO_DEV_WARN_REF_LAYOUT);
    if (s_ok) sim->cur = S.cur ^ 1u;
    sim->step = S.step + 1u;
    sim->epoch = S.epoch + 1u;
    for (int k = 0; k < 8; k++) sim->cnt[k] = 0;
    sim->newEggs = 0;
    sim->ticket1 = 0;
    sim->ticket2 = 0;
    sim->done2 = 0;
  }
  __syncthreads();
  if (s_ok) publish_start(p, s_np, true);
  else publish_start(p, S.pop, true);
}

// ------------------------------------------------------------------------
// Initial population: initAgents over [0, n) (kernel/initAgents.cl:26-65),
// optionally with ages 24*U{0..age_days_max} from splitmix64 (an extension).
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
    c.eggIncubation = -0.923f * T0 + 60.923f;
  }
  __syncthreads();
  const DevPool dst = p.pool[0];
  for (uint32_t id = blockIdx.x * blockDim.x + threadIdx.x; id < n; id += gridDim.x * blockDim.x) {
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

// Statistics of the current pool (grid-stride), accumulated into acc_*.
__global__ void k_pool_stats(KParams p) {
  SimDev* sim = p.sim;
  const sampo_population pop = sim->pop;
  const DevPool src = p.pool[sim->cur];
  uint32_t l1 = 0, fem = 0, inf = 0, dmin = 0xffffffffu, dmax = 0;
  const uint32_t end = pop.r[GRAVID].end;
  for (uint32_t g = blockIdx.x * blockDim.x + threadIdx.x; g < end; g += gridDim.x * blockDim.x) {
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

__global__ void k_publish_start(KParams p) {
  __shared__ sampo_population ranges;
  if (threadIdx.x == 0) ranges = p.sim->pop;
  __syncthreads();
  publish_start(p, ranges, false);
}

// ageHistogram (kernel/ageHistogram.cl:13-35) with warp-aggregated shared
// atomics: lanes that fall in the same bin add once.
__global__ void k_histogram(KParams p, uint32_t* hist) {
  __shared__ uint32_t h[100];
  for (int k = threadIdx.x; k < 100; k += blockDim.x) h[k] = 0;
  __syncthreads();
  SimDev* sim = p.sim;
  const sampo_population pop = sim->pop;
  const DevPool src = p.pool[sim->cur];
  const uint32_t lo = pop.r[IMMATURE].start, hi = pop.r[GRAVID].end;
  const uint32_t span = hi > lo ? hi - lo : 0u;
  const uint32_t stride = gridDim.x * blockDim.x;
  for (uint32_t base = blockIdx.x * blockDim.x; base < span; base += stride) {
    const uint32_t g = lo + base + threadIdx.x;
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
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
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

// ------------------------------------------------------------------------
static int sm_count() {
  static int sms = 0;
  if (!sms) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (sms <= 0) sms = 1;
  }
  return sms;
}
constexpr size_t kCountSmem = 2 * kCountStage;
constexpr size_t kScatterSmem = 2 * kScatterStage;

static void set_smem_attrs() {
  static bool done = false;
  if (done) return;
  cudaFuncSetAttribute(k_count, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kCountSmem);
  cudaFuncSetAttribute(k_scatter, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kScatterSmem);
  done = true;
}
int grid_blocks_count() {
  set_smem_attrs();
  int per = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_count, kBlock, kCountSmem);
  return sm_count() * (per > 0 ? per : 1);
}
int grid_blocks_scatter() {
  set_smem_attrs();
  int per = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_scatter, kScatterThreads, kScatterSmem);
  return sm_count() * (per > 0 ? per : 1);
}
cudaError_t launch_count(const KParams& p, int grid, cudaStream_t st) {
  set_smem_attrs();
  k_count<<<grid, kBlock, kCountSmem, st>>>(p);
  return cudaGetLastError();
}
cudaError_t launch_scatter(const KParams& p, int grid, cudaStream_t st) {
  set_smem_attrs();
  k_scatter<<<grid, kScatterThreads, kScatterSmem, st>>>(p);
  return cudaGetLastError();
}
cudaError_t launch_init_eggs(const KParams& p, uint32_t n, float T0, const sampo_seeds* seeds_dev, int age_days_max,
                             uint64_t age_seed, cudaStream_t st) {
  k_init_eggs<<<sm_count() * 4, 256, 0, st>>>(p, n, T0, seeds_dev, age_days_max, age_seed);
  return cudaGetLastError();
}
cudaError_t launch_publish_start(const KParams& p, cudaStream_t st) {
  k_pool_stats<<<sm_count() * 4, 256, 0, st>>>(p);
  k_publish_start<<<1, 128, 0, st>>>(p);
  return cudaGetLastError();
}
cudaError_t launch_histogram(const KParams& p, uint32_t* hist_dev, cudaStream_t st) {
  k_histogram<<<sm_count() * 4, 256, 0, st>>>(p, hist_dev);
  return cudaGetLastError();
}
cudaError_t launch_eval_math(int fn, const float* x, const float* y, float* out, uint32_t n, cudaStream_t st) {
  k_eval_math<<<sm_count() * 2, 256, 0, st>>>(fn, x, y, out, n);
  return cudaGetLastError();
}

}  // namespace sampo
