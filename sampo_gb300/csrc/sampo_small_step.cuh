// sampo_small_step.cuh - the hourly step of one simulation in one launch, for
// pools of up to a few hundred 1024-slot tiles (sm_103a).
//
// At that size the three-kernel step (k_count, k_scatter, k_publish) is bound
// by each kernel's start-up and latency chain, not by bandwidth. k_step_small
// does the same step in one cooperative launch with one CTA per tile:
//
//  phase 1  CTA b loads tile b (TMA bulk copies) and runs the full update of
//           its agents once (killAgents + updateAgents with the species
//           functions and the normal draws). The updated records stay in the
//           CTA's shared memory with their next state in the flag byte; the
//           CTA builds the tile's prefix table over its (round, warp) chunks
//           in shared memory and publishes the tile's survivors per next
//           state, its eggs laid and its share of the next pool's statistics
//           (calcL1de.cl, calcGender.cl) to global memory.
//  barrier  a grid barrier with a bounded wait.
//  phase 2  every CTA sums the per-tile counts: the totals give the next
//           layout (kernel/oldToNewAgents.cl:57-95), the tiles before its own
//           the tile's first slot in each next-state range. It writes its
//           survivors from shared memory to their slots in the next buffer
//           and the new eggs of its egg tiles at [0, newEggs)
//           (kernel/initAgents.cl:26-65), then computes the next step's
//           state from the totals (the k_publish code); the last CTA also
//           stores it for the host.
//  barrier  a second grid barrier; the next hour's tile copies go out.
//
// Pools with more tiles than CTAs are still stepped correctly: CTA b also
// takes tiles b + G, b + 2G, ... (G CTAs); their decisions are counted in
// phase 1 and the tile is loaded and updated again in phase 2.
//
// Built into the library for the built-in species only (a user species keeps
// the three-kernel step).
#pragma once
#include "sampo_step_kernels.cuh"

namespace sampo {

constexpr int kSmallThreads = kBlock;      // eight warps, I slots per thread (tiles of kBlock * I slots: I = 1, 2 or 4)
constexpr int kSmallMinBlocks = 3;         // resident CTAs per SM the registers are sized for
__host__ __device__ constexpr uint32_t small_stage(int items) { return 9 * kBlock * items * 4 + kBlock * items; }  // ten columns
constexpr uint32_t kSmallRows = 9;         // per-tile counts: survivors by next state, eggs laid
constexpr uint8_t kGone = 0xffu;           // flag byte of a slot without a survivor
constexpr uint32_t kSmallHours = 24;       // hours whose inputs a CTA holds in shared memory
// Per-CTA statistics of the next pool (CTA b's column, b < the tiles):
// L1de, females, infective, cycles, sum of cycles, bites, infective bites
// (sums) and the min and max larva age in days.
enum : uint32_t { SA_L1 = 0, SA_FEM, SA_INF, SA_CYC, SA_SUMCYC, SA_BITES, SA_IBITES, SA_DMIN, SA_DMAX, kSmallStats };
// The rows' stride is twice the pool's count of 512-slot tiles (room for
// 256-slot tiles): they fit the prefix-table array.
static_assert(2 * (kSmallRows + kSmallStats) <= kPreWordsMin, "the per-tile rows fit the prefix-table array");

__device__ __forceinline__ uint32_t ld_acquire_u32(const uint32_t* p) {
  uint32_t v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

// A grid barrier in two halves. small_grid_arrive (every thread): the CTA's
// writes so far are ordered before its arrival by the CTA barrier and the
// release of the arrival. small_grid_wait (every thread): all CTAs of the
// grid (co-resident: a cooperative launch) wait until the arrival counter
// reaches `target` (the grid size times the barriers passed so far in the
// launch); the acquire of the counter orders the reads that follow. Bounded:
// false when the others did not arrive within the limit; every thread gets
// the same answer. Work that needs no other CTA can go between the halves.
__device__ __forceinline__ void small_grid_arrive(uint32_t* bar) {
  __syncthreads();
  if (threadIdx.x == 0) asm volatile("red.release.gpu.global.add.u32 [%0], 1;" ::"l"(bar) : "memory");
}
__device__ bool small_grid_wait(uint32_t* bar, uint32_t target, uint32_t* s_flag) {
  if (threadIdx.x == 0) {
    uint32_t ok = 0;
    for (uint32_t i = 0; i < kWaitLimit; i++) {
      if (ld_acquire_u32(bar) >= target) { ok = 1; break; }
      if (i >= 32) __nanosleep(32);
    }
    *s_flag = ok;
  }
  __syncthreads();
  return *s_flag != 0;
}
__device__ bool small_grid_barrier(uint32_t* bar, uint32_t target, uint32_t* s_flag) {
  small_grid_arrive(bar);
  return small_grid_wait(bar, target, s_flag);
}

struct SmallAcc {
  Acc acc;                            // counters of the update (bites, cycles, eggs laid, table misses)
  uint32_t l1, fem, inf, dmin, dmax;  // statistics of the next pool
  uint32_t devoob, tilebad;
};

// Phase 1 (and phase 2 for a tile updated again): the full update of the
// tile in stage memory st (slots lo .. lo + kTile of the current pool). With
// KEEP the updated records and their next state (flag byte; kGone for none)
// are written back to the stage. Every (round, warp) chunk's survivors by
// next state go to s_ent. EGGS / STATS: the eggs laid / the update's
// counters and the next pool's statistics go to sa (a tile updated twice
// counts its eggs the first time and the rest the second).
template <int I, bool KEEP, bool EGGS, bool STATS>
__device__ __forceinline__ void small_update_tile(const StepCtx& c, const ModelConst& mc, const sampo_population& pop,
                                                  uint8_t* st, uint32_t lo, uint32_t end, uint2* s_ent, SmallAcc& sa) {
  SAMPO_TILE_CONSTANTS(I);
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  float* c_age = (float*)(st + 0 * kColBytes);
  float* c_his = (float*)(st + 1 * kColBytes);
  float* c_delay = (float*)(st + 2 * kColBytes);
  float* c_sporo = (float*)(st + 3 * kColBytes);
  uint32_t* c_uni = (uint32_t*)(st + 4 * kColBytes);
  uint32_t* c_avail = (uint32_t*)(st + 5 * kColBytes);
  uint32_t* c_cycle = (uint32_t*)(st + 6 * kColBytes);
  uint32_t* c_hbc = (uint32_t*)(st + 7 * kColBytes);
  uint32_t* c_batches = (uint32_t*)(st + 8 * kColBytes);
  uint8_t* c_flags = st + 9 * kColBytes;
  Acc t = {0, 0, 0, 0, 0, 0};
#pragma unroll 1
  for (int k = 0; k < kItems; k++) {
    const uint32_t i = k * kBlock + tid;
    const uint32_t g = lo + i;
    const int rg = g < end ? range_of(pop, g) : -1;
    uint32_t pk0 = 0, pk1 = 0;  // this slot's next state as an 8-bit counter: states 0-3, 4-7
    uint8_t fb = kGone;
    if (rg >= 0) {
      Rec a;
      a.age = c_age[i]; a.his = c_his[i]; a.delay = c_delay[i]; a.sporo = c_sporo[i];
      a.uni = c_uni[i]; a.avail = c_avail[i]; a.cycle = c_cycle[i]; a.hbc = c_hbc[i];
      a.batches = c_batches[i];
      a.female = (c_flags[i] >> 3) & 1u;
      a.bm = BM_NONE;
      sa.devoob |= (rg == LARVA) & c.devOOB;
      const int ns = update_agent<true, true, false>(c, mc.kill, rg, g, a, t);
      if (ns >= 0) {
        if (a.bm != BM_NONE) {  // the owed normal draw (include/gpuRand.h:56-63)
          const uint32_t v = finish_box_muller(c, mc, g, a.bm, a.batches);
          if (a.bm == BM_LARVA_DELAY) a.delay = __uint_as_float(v);
          else a.avail = v;
        }
        if (ns < 4) pk0 = 1u << (8 * ns);
        else pk1 = 1u << (8 * (ns - 4));
        fb = (uint8_t)(ns | (a.female << 3));
        if (STATS) {  // kernel/calcL1de.cl:28-30, kernel/calcGender.cl:24-37
          if (ns == LARVA) {
            sa.l1 += age_days_uncapped(a.age);
            const uint32_t dd = age_days(a.age);
            sa.dmin = min(sa.dmin, dd); sa.dmax = max(sa.dmax, dd);
          } else if (ns >= IMMATURE && a.female) {
            sa.fem += 1u;
            sa.inf += a.sporo >= 1.0f ? 1u : 0u;
          }
        }
        if (KEEP) {
          c_age[i] = a.age; c_his[i] = a.his; c_delay[i] = a.delay; c_sporo[i] = a.sporo;
          c_uni[i] = a.uni; c_avail[i] = a.avail; c_cycle[i] = a.cycle; c_hbc[i] = a.hbc;
          c_batches[i] = a.batches;
        }
      }
    }
    if (KEEP) c_flags[i] = fb;
    pk0 = __reduce_add_sync(0xffffffffu, pk0);
    pk1 = __reduce_add_sync(0xffffffffu, pk1);
    if (lane == 0) s_ent[k * kWarps + warp] = make_uint2(pk0, pk1);
  }
  if (EGGS) sa.acc.newEggs += t.newEggs;
  if (STATS) {
    sa.acc.bites += t.bites; sa.acc.infectBites += t.infectBites;
    sa.acc.cycles += t.cycles; sa.acc.sumCycles += t.sumCycles;
  }
  sa.acc.bad |= t.bad;
}

// Warp 0, after the tile's chunk counts are in s_ent: the tile's prefix table
// (the same 16-bit packed entries as the count pass's) into s_tab, and the
// tile's survivors of next state `lane` to lanes 0..7.
template <int I>
__device__ __forceinline__ uint32_t small_build_table(const uint2* s_ent, uint32_t* s_tab) {
  SAMPO_TILE_CONSTANTS(I);
  const int lane = threadIdx.x & 31;
  const uint2 e = lane < (int)kChunks ? s_ent[lane] : make_uint2(0u, 0u);
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
  if (lane < (int)kChunks) {
#pragma unroll
    for (int q = 0; q < 5; q++) s_tab[lane * kPreEntryWords + q] = x[q] - w[q];
  }
  if (lane == (int)kChunks - 1) {
#pragma unroll
    for (int q = 0; q < 5; q++) s_tab[kChunks * kPreEntryWords + q] = x[q];
  }
  uint32_t tw = 0;
#pragma unroll
  for (int q = 0; q < 4; q++) {
    const uint32_t tq = __shfl_sync(0xffffffffu, x[q], kChunks - 1);
    if ((lane >> 1) == q) tw = (tq >> (16 * (lane & 1))) & 0xffffu;
  }
  return tw;
}

// Phase 2: the survivors of the tile in stage memory st (after
// small_update_tile<true, ...> and its table) to their slots in the next
// buffer: the tile's first slot of the state (s_d0) + the survivors of that
// state in earlier chunks (s_tab) + the rank within the chunk. A survivor
// whose slot falls outside its chunk's run sets tilebad and is not stored.
template <int I>
__device__ __forceinline__ void small_scatter_tile(const uint8_t* st, const uint32_t* s_tab, const uint32_t* s_d0,
                                                   const DevPool& dst, uint32_t& tilebad) {
  SAMPO_TILE_CONSTANTS(I);
  const int tid = threadIdx.x, warp = tid >> 5;
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
#pragma unroll
  for (int k = 0; k < kItems; k++) {
    const uint32_t i = k * kBlock + tid;
    const uint8_t fb = c_flags[i];
    const int b = fb == kGone ? 8 : (fb & 7);
    const uint32_t peers = __match_any_sync(0xffffffffu, (uint32_t)b);
    const uint32_t rk = __popc(peers & lanemask_lt());
    if (b < 8) {
      const uint32_t* e0 = s_tab + (k * kWarps + warp) * kPreEntryWords;
      const uint32_t* e1 = e0 + kPreEntryWords;
      const uint32_t sh = 16 * (b & 1);
      const uint32_t j = ((e0[b >> 1] >> sh) & 0xffffu) + rk;
      if (j < ((e1[b >> 1] >> sh) & 0xffffu)) {
        const uint32_t d = s_d0[b] + j;
        dst.age[d] = c_age[i]; dst.his[d] = c_his[i]; dst.delay[d] = c_delay[i]; dst.sporo[d] = c_sporo[i];
        dst.uni[d] = c_uni[i]; dst.avail[d] = c_avail[i]; dst.cycle[d] = c_cycle[i]; dst.hbc[d] = c_hbc[i];
        dst.batches[d] = c_batches[i];
        dst.flags[d] = fb;
      } else {
        tilebad = 1;
      }
    }
  }
}

// Phase 2, all threads: over the per-tile counts (rows 0..8), the sums of
// tiles [0, t) into s_ex and, with `totals`, of all nold tiles into s_tot,
// followed by the statistics rows over the columns of the CTAs that held
// tiles (min(nold, G); sums, min and max) into s_tot[kSmallRows ..]. Thread
// i takes columns i, i + blockDim.x, ...: every row of a column is loaded at
// once, so one round trip to L2 serves them all. Rows are state-major:
// rows[row * stride + column], read through L2. Ends synchronised.
constexpr uint32_t kSumWords = 2 * kSmallRows + kSmallStats;  // ex, tot, statistics
__device__ __forceinline__ void small_sum_rows(const uint32_t* rows, uint32_t stride, uint32_t nold, uint32_t t,
                                               bool totals, uint32_t* s_ex, uint32_t* s_tot,
                                               uint32_t (*s_part)[kSumWords]) {
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  uint32_t ex[kSmallRows], tot[kSmallRows], st[kSmallStats];
#pragma unroll
  for (int r = 0; r < (int)kSmallRows; r++) ex[r] = tot[r] = 0;
#pragma unroll
  for (int k = 0; k < (int)kSmallStats; k++) st[k] = k == (int)SA_DMIN ? 0xffffffffu : 0u;
  const uint32_t lim = totals ? nold : t;
  for (uint32_t j = tid; j < lim; j += blockDim.x) {
    uint32_t v[kSmallRows];
#pragma unroll
    for (int r = 0; r < (int)kSmallRows; r++) v[r] = __ldcg(rows + (size_t)r * stride + j);
#pragma unroll
    for (int r = 0; r < (int)kSmallRows; r++) {
      tot[r] += v[r];
      ex[r] += j < t ? v[r] : 0u;
    }
  }
  if (totals) {
    const uint32_t cols = min(nold, gridDim.x);  // one column per CTA with tiles
    for (uint32_t j = tid; j < cols; j += blockDim.x) {
      uint32_t v[kSmallStats];
#pragma unroll
      for (int k = 0; k < (int)kSmallStats; k++) v[k] = __ldcg(rows + (size_t)(kSmallRows + k) * stride + j);
#pragma unroll
      for (int k = 0; k < (int)kSmallStats; k++)
        st[k] = k == (int)SA_DMIN ? min(st[k], v[k]) : k == (int)SA_DMAX ? max(st[k], v[k]) : st[k] + v[k];
    }
  }
#pragma unroll
  for (int r = 0; r < (int)kSmallRows; r++) {
    ex[r] = __reduce_add_sync(0xffffffffu, ex[r]);
    tot[r] = __reduce_add_sync(0xffffffffu, tot[r]);
  }
#pragma unroll
  for (int k = 0; k < (int)kSmallStats; k++)
    st[k] = k == (int)SA_DMIN ? __reduce_min_sync(0xffffffffu, st[k])
          : k == (int)SA_DMAX ? __reduce_max_sync(0xffffffffu, st[k]) : __reduce_add_sync(0xffffffffu, st[k]);
  if (lane == 0) {
#pragma unroll
    for (int r = 0; r < (int)kSmallRows; r++) {
      s_part[warp][r] = ex[r];
      s_part[warp][kSmallRows + r] = tot[r];
    }
#pragma unroll
    for (int k = 0; k < (int)kSmallStats; k++) s_part[warp][2 * kSmallRows + k] = st[k];
  }
  __syncthreads();
  if (tid < (int)kSumWords) {
    const int k = tid - 2 * (int)kSmallRows;  // statistic, for the last kSmallStats words
    uint32_t x = s_part[0][tid];
    for (int w = 1; w < kWarps; w++) {
      const uint32_t y = s_part[w][tid];
      x = k == (int)SA_DMIN ? min(x, y) : k == (int)SA_DMAX ? max(x, y) : x + y;
    }
    if (tid < (int)kSmallRows) s_ex[tid] = x;
    else if (totals) s_tot[tid - kSmallRows] = x;
  }
  __syncthreads();
}

// Phase 1's end: the CTA's statistics of the next pool (its tiles) to its
// column of the statistics rows, in two halves around a CTA barrier: each
// warp's totals into s_red (every thread), then the CTA's totals out by the
// threads of warp `w` (the other warps may do other work meanwhile).
__device__ __forceinline__ void small_stats_warps(const SmallAcc& sa, uint32_t (*s_red)[kSmallStats]) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  uint32_t v[kSmallStats] = {sa.l1, sa.fem, sa.inf, sa.acc.cycles, sa.acc.sumCycles, sa.acc.bites, sa.acc.infectBites,
                             sa.dmin, sa.dmax};
#pragma unroll
  for (int j = 0; j < (int)SA_DMIN; j++) v[j] = __reduce_add_sync(0xffffffffu, v[j]);
  v[SA_DMIN] = __reduce_min_sync(0xffffffffu, v[SA_DMIN]);
  v[SA_DMAX] = __reduce_max_sync(0xffffffffu, v[SA_DMAX]);
  if (lane == 0) {
#pragma unroll
    for (int j = 0; j < (int)kSmallStats; j++) s_red[warp][j] = v[j];
  }
}
__device__ __forceinline__ void small_stats_store(uint32_t* rows, uint32_t stride, uint32_t b,
                                                  const uint32_t (*s_red)[kSmallStats], int w) {
  const int k = (int)threadIdx.x - 32 * w;
  if (k >= 0 && k < (int)kSmallStats) {
    uint32_t x = s_red[0][k];
    for (int i = 1; i < kWarps; i++) {
      const uint32_t y = s_red[i][k];
      x = k == (int)SA_DMIN ? min(x, y) : k == (int)SA_DMAX ? max(x, y) : x + y;
    }
    __stcg(rows + (size_t)(kSmallRows + k) * stride + b, x);
  }
}

// Every thread waits (bounded) for the bulk copies of the stage's tile;
// false for all when any wait ran out.
__device__ __forceinline__ bool small_wait_stage(uint64_t* bar, uint32_t& phase) {
  const bool ok = mbar_wait(bar, phase);
  phase ^= 1u;
  return __syncthreads_and(ok) != 0;
}

template <int I>
__device__ __forceinline__ void small_issue_tile(const DevPool& src, uint8_t* st, uint64_t* bar, uint32_t lo, uint32_t n) {
  SAMPO_TILE_CONSTANTS(I);
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

__device__ __forceinline__ void fence_proxy_async_global() { asm volatile("fence.proxy.async.global;" ::: "memory"); }

// The one-launch steps of p.reps[0] (a single simulation without a device
// seed stream): `nsteps` hourly steps in one cooperative launch (a day graph
// launches it once with 24). Per hour: the update (phase 1), whose per-tile
// counts and per-CTA statistics of the next pool go to rows in global
// memory; a grid barrier; the scatter (phase 2) and the arrival at a second
// grid barrier, after which every CTA computes the next hour's layout,
// statistics row, step constants and larval table itself from the same
// totals (the k_publish arithmetic; the last CTA, the one least likely to
// hold a tile, also writes them to the replicate's state for the host) before
// it waits there; then the next hour's tile copies go out. The step inputs of
// the launch's hours are read into shared memory at its start (the host
// writes them before the launch). The rows use the replicate's prefix-table
// array (tilePre: kSmallRows + kSmallStats words per column, at a stride of
// twice its count of 512-slot tiles), which the three-kernel step rewrites
// before it reads it. The pool the scatter wrote with ordinary stores is
// read by the next hour's bulk copies after proxy fences.
template <int I>
__global__ void __launch_bounds__(kSmallThreads, kSmallMinBlocks) k_step_small(KParams p, uint32_t nsteps) {
  SAMPO_TILE_CONSTANTS(I);
  extern __shared__ __align__(128) uint8_t stage[];
  __shared__ StepCtx s_c;
  __shared__ ModelConst s_mc;
  __shared__ float s_hmr[100];
  __shared__ sampo_population s_pop;
  __shared__ CtxInputs s_in[kSmallHours];
  __shared__ __align__(8) uint64_t s_mbar;
  __shared__ uint2 s_ent[kChunks];
  __shared__ __align__(16) uint32_t s_tab[(kChunks + 1) * kPreEntryWords];
  __shared__ uint32_t s_ex[kSmallRows], s_tot[kSmallRows + kSmallStats], s_d0[8], s_ne[kWarps];
  __shared__ uint32_t s_red[kWarps][kSmallStats], s_part[kWarps][kSumWords];
  __shared__ uint32_t s_flag, s_ok, s_last;
  __shared__ uint32_t s_active, s_end, s_nold, s_cur, s_cap, s_step, s_epoch, s_stop;
  __shared__ float s_cc;
  const RepParams& rp = p.reps[0];
  SimDev* sim = rp.sim;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const uint32_t G = gridDim.x, b = blockIdx.x;
  uint32_t phase = 0, barriers = 0;
  bool met = true, ok = true;
  const uint32_t stride = 2u * rp.maxTiles;  // >= the tiles of any pool that fits, at 256-slot tiles
  uint32_t* rows = rp.tilePre;  // [kSmallRows + kSmallStats][stride]

  // ---- the replicate's state at the launch (the previous kernel wrote it) ----
  if (tid == 0) {
    mbar_init(&s_mbar);
    fence_mbar_init();
    const uint32_t active = sim->active;
    s_pop = sim->pop;
    s_active = active;
    s_end = active ? s_pop.r[GRAVID].end : 0u;
    s_nold = (s_end + kTile - 1) / kTile;
    s_cur = sim->cur;
    s_cap = sim->capacity;
    s_step = sim->step;
    s_epoch = sim->epoch;
    s_stop = sim->stop_step;
    s_cc = sim->cc;
    if (b < s_nold) {
      const uint32_t lo = b * kTile;
      small_issue_tile<I>(rp.pool[s_cur], stage, &s_mbar, lo, min((uint32_t)kTile, s_end - lo));
    }
  }
  copy16(&s_c, &sim->ctx, (int)sizeof(StepCtx), tid, blockDim.x);
  for (int k = tid; k < 100; k += blockDim.x) s_hmr[k] = sim->larvaHMR[k];
  load_model_const(p.mc, s_mc);
  __syncthreads();
  if (tid == 0) s_c.larvaHMR = s_hmr;
  // the inputs of the steps that follow the launch's hours
  for (uint32_t j = tid; j < min(nsteps, kSmallHours); j += blockDim.x) load_ctx_inputs(rp, s_step + 1u + j, s_in[j]);
  __syncthreads();

  for (uint32_t hour = 0; hour < nsteps; hour++) {
    if (!s_active) break;  // stopped or paused (uniform)
    const uint32_t nold = s_nold, end = s_end;
    SmallAcc sa;
    sa.acc = Acc{0, 0, 0, 0, 0, 0};
    sa.l1 = sa.fem = sa.inf = sa.dmax = sa.devoob = sa.tilebad = 0;
    sa.dmin = 0xffffffffu;

    // ---- phase 1: decide (and, for tile b, finish) every tile of this CTA ----
    if (nold > G && b < nold) {
      // more tiles than CTAs: count tile b (its copies are on their way)
      // without keeping it, then the other tiles of this CTA one after the
      // other in the stage, then load tile b again and keep it
      ok = small_wait_stage(&s_mbar, phase);
      for (uint32_t t = b; t < nold && ok; t += G) {
        if (t != b) {
          if (tid == 0) {
            fence_proxy_async();
            small_issue_tile<I>(rp.pool[s_cur], stage, &s_mbar, t * kTile, min((uint32_t)kTile, end - t * kTile));
          }
          ok = small_wait_stage(&s_mbar, phase);
          if (!ok) break;
        }
        const uint32_t eggs_before = sa.acc.newEggs;
        small_update_tile<I, false, true, true>(s_c, s_mc, s_pop, stage, t * kTile, end, s_ent, sa);
        const uint32_t ne = __reduce_add_sync(0xffffffffu, sa.acc.newEggs - eggs_before);
        if (lane == 0) s_ne[warp] = ne;
        __syncthreads();
        if (warp == 0) {
          const uint32_t tw = small_build_table<I>(s_ent, s_tab);
          if (lane < 8) __stcg(rows + (size_t)lane * stride + t, tw);
          uint32_t e = lane < kWarps ? s_ne[lane] : 0u;
          e = __reduce_add_sync(0xffffffffu, e);
          if (lane == 0) __stcg(rows + (size_t)8 * stride + t, e);
        }
        __syncthreads();  // the stage is read before the next copy overwrites it
      }
      if (ok) {
        if (tid == 0) {
          fence_proxy_async();
          small_issue_tile<I>(rp.pool[s_cur], stage, &s_mbar, b * kTile, min((uint32_t)kTile, end - b * kTile));
        }
        ok = small_wait_stage(&s_mbar, phase);
        if (ok) {
          small_update_tile<I, true, false, false>(s_c, s_mc, s_pop, stage, b * kTile, end, s_ent, sa);  // counted above
          small_stats_warps(sa, s_red);
          __syncthreads();
          if (warp == 0) (void)small_build_table<I>(s_ent, s_tab);
          else if (warp == 1) small_stats_store(rows, stride, b, s_red, 1);
        }
      }
    } else if (b < nold) {
      ok = small_wait_stage(&s_mbar, phase);
      if (ok) {
        const uint32_t eggs_before = sa.acc.newEggs;
        small_update_tile<I, true, true, true>(s_c, s_mc, s_pop, stage, b * kTile, end, s_ent, sa);
        const uint32_t ne = __reduce_add_sync(0xffffffffu, sa.acc.newEggs - eggs_before);
        if (lane == 0) s_ne[warp] = ne;
        small_stats_warps(sa, s_red);
        __syncthreads();
        if (warp == 0) {  // the tile's table and counts
          const uint32_t tw = small_build_table<I>(s_ent, s_tab);
          if (lane < 8) __stcg(rows + (size_t)lane * stride + b, tw);
          uint32_t e = lane < kWarps ? s_ne[lane] : 0u;
          e = __reduce_add_sync(0xffffffffu, e);
          if (lane == 0) __stcg(rows + (size_t)8 * stride + b, e);
        } else if (warp == 1) {  // meanwhile the CTA's statistics
          small_stats_store(rows, stride, b, s_red, 1);
        }
      }
    }
    if (tid == 0) s_ok = ok ? 1u : 0u;

    // ---- grid barrier A: every tile's counts and every CTA's statistics are published ----
    met = small_grid_barrier(&p.bat->bar, G * ++barriers, &s_flag);
    ok = s_ok != 0;  // this CTA's copies all landed

    // ---- phase 2: totals, next layout, this tile's first slots; scatter ----
    small_sum_rows(rows, stride, nold, b < nold ? b : nold, true, s_ex, s_tot, s_part);
    uint32_t tot[8], base[8];
#pragma unroll
    for (int k = 0; k < 8; k++) tot[k] = s_tot[k];
    const uint32_t ne = s_tot[8];
    const bool fits = layout_fits(tot, ne, s_cap);
    sampo_population np;
    next_layout(tot, ne, np, base);
    const bool write = ok && met && fits;
    const DevPool dst = rp.pool[s_cur ^ 1u];
    if (write && b < nold) {
      if (tid < 8) s_d0[tid] = base[tid] + s_ex[tid];
      __syncthreads();
      small_scatter_tile<I>(stage, s_tab, s_d0, dst, sa.tilebad);
      // more tiles than CTAs: the other tiles of this CTA, loaded and updated again
      for (uint32_t t = b + G; t < nold; t += G) {
        __syncthreads();  // the stage is read
        if (tid == 0) {
          fence_proxy_async();
          small_issue_tile<I>(rp.pool[s_cur], stage, &s_mbar, t * kTile, min((uint32_t)kTile, end - t * kTile));
        }
        if (!small_wait_stage(&s_mbar, phase)) { ok = false; break; }
        small_update_tile<I, true, false, false>(s_c, s_mc, s_pop, stage, t * kTile, end, s_ent, sa);
        small_sum_rows(rows, stride, nold, t, false, s_ex, s_tot, s_part);
        if (warp == 0) {
          const uint32_t tw = small_build_table<I>(s_ent, s_tab);
          // the update again must give the counts of phase 1
          if (lane < 8 && tw != __ldcg(rows + (size_t)lane * stride + t)) sa.tilebad = 1;
          if (lane < 8) s_d0[lane] = base[lane] + s_ex[lane];
        }
        if (__syncthreads_or(sa.tilebad)) break;
        small_scatter_tile<I>(stage, s_tab, s_d0, dst, sa.tilebad);
      }
    }
    if (write) {
      // new eggs at [0, newEggs) of the next buffer, egg tile e on CTA G-1-(e mod G)
      const uint32_t negg = (ne + kTile - 1) / kTile;
      for (uint32_t e = G - 1 - b; e < negg; e += G) {
#pragma unroll
        for (int k = 0; k < kItems; k++) {
          const uint32_t id = e * kTile + k * kBlock + tid;
          if (id < ne) {
            Rec a;
            new_egg(s_c, id, a);
            dst.age[id] = a.age; dst.his[id] = a.his; dst.delay[id] = a.delay; dst.sporo[id] = a.sporo;
            dst.uni[id] = a.uni; dst.avail[id] = a.avail; dst.cycle[id] = a.cycle; dst.hbc[id] = a.hbc;
            dst.batches[id] = a.batches;
            dst.flags[id] = (uint8_t)(EGG | (a.female << 3));
          }
        }
      }
    }
    fence_proxy_async_global();  // the next hour reads these stores with bulk copies

    // ---- this CTA's error bits (the capacity bit from CTA 0 only) ----
    {
      uint32_t x = (sa.acc.bad ? SAMPO_DEV_ERR_LARVATABLE : 0u) | (sa.tilebad ? SAMPO_DEV_ERR_TILECOUNT : 0u) |
                   (sa.devoob ? SAMPO_DEV_ERR_DEVRATES : 0u) | (ok ? 0u : SAMPO_DEV_ERR_TMA) |
                   (met ? 0u : SAMPO_DEV_ERR_BARRIER) | (fits ? 0u : SAMPO_DEV_ERR_CAPACITY);
      x = __reduce_or_sync(0xffffffffu, x);
      if (b != 0) x &= ~SAMPO_DEV_ERR_CAPACITY;
      if (lane == 0 && x) atomicOr(&sim->error, x);
    }
    if (!met || !ok) break;  // the error bits are set; nothing after this hour is valid
    if (!fits) {
      // the next layout does not fit: the replicate pauses at this step with
      // its pool and constants (k_publish does the same for the three-kernel step)
      if (b == G - 1u && tid == 0) sim->active = 0;
      break;
    }

    // ---- the next hour's state (the k_publish arithmetic, publish_rep), by
    //      every CTA from the same totals, between its arrival at the grid
    //      barrier (its stores are in) and its wait there ----
    const uint32_t step = s_step + 1u;
    const bool active = step < s_stop;
    const bool more = hour + 1u < nsteps && active;  // another hour in this launch
    if (more) small_grid_arrive(&p.bat->bar);
    const uint32_t next_end = np.r[GRAVID].end, next_nold = (next_end + kTile - 1) / kTile;
    const uint32_t* st = s_tot + kSmallRows;
    // the next pool's statistics (kernel/calcL1de.cl:259-280, calcGender.cl)
    np.numLarvae1DayEquiv = (np.r[LARVA].end > np.r[LARVA].start) ? st[SA_L1] : 0u;
    np.numFemale = st[SA_FEM];
    np.numPotentiallyInfective = st[SA_INF];
    __syncthreads();  // every thread is past its last read of s_c, s_hmr and s_pop
    if (tid == 0) {
      CtxInputs& in = s_in[hour % kSmallHours];
      if (hour >= kSmallHours) load_ctx_inputs(rp, step, in);  // (its slot's hour is done)
      StepCtx c;
      make_ctx(in, sim->larvaHMR, np, c);  // the global table: the last CTA stores this one
      if (b == G - 1u) {
        // the replicate's state and the coming step's row for the host
        sampo_bites_cycles nbnc;
        nbnc.numCyclesReported = st[SA_CYC];
        nbnc.sumCyclesReported = st[SA_SUMCYC];
        nbnc.numBitesReported = st[SA_BITES];
        nbnc.numInfectBitesReported = st[SA_IBITES];
        // the reference's shared empty initial ranges (src/abms.c:204-219)
        bool shared_end = false;
        uint32_t moved = 0;
        for (int k = 1; k < 8; k++) {
          shared_end |= s_pop.r[k].end == s_pop.r[k - 1].end;
          moved += s_tot[k];
        }
        if (shared_end && moved) sim->warn = __ldcg(&sim->warn) | SAMPO_DEV_WARN_REF_LAYOUT;
        sim->ctx = c;
        sim->pop = np;
        sim->bnc = nbnc;
        sim->step = step;
        sim->cur = s_cur ^ 1u;
        sim->epoch = s_epoch + 1u;
        sampo_stats_row row;
        row.pop = np;
        row.bnc = nbnc;
        rp.rows[step % rp.ring] = row;
        if (!active) sim->active = 0;
      }
      c.larvaHMR = s_hmr;
      s_c = c;
      s_pop = np;
      s_step = step;
      s_epoch += 1u;
      s_cur ^= 1u;
      s_end = next_end;
      s_nold = next_nold;
      s_active = active;
    }
    {  // the next hour's larval table (every CTA; the last one also stores it)
      const uint32_t dmin = st[SA_DMIN], dmax = st[SA_DMAX], l1 = np.numLarvae1DayEquiv;
      for (int d = tid - 32; d >= 0 && d < 100; d += blockDim.x - 32) {
        const float h = larva_hmr_entry((uint32_t)d, dmin, dmax, l1, s_cc);
        s_hmr[d] = h;
        if (b == G - 1u) sim->larvaHMR[d] = h;
      }
    }
    if (!more) break;  // (no copy is in flight)

    // ---- the grid barrier's wait: every CTA's stores are in; the next hour's tile ----
    met = small_grid_wait(&p.bat->bar, G * ++barriers, &s_flag);
    if (!met) break;
    if (tid == 0 && b < next_nold) {
      fence_proxy_async_global();
      fence_proxy_async();
      small_issue_tile<I>(dst, stage, &s_mbar, b * kTile, min((uint32_t)kTile, next_end - b * kTile));
    }
  }
  if (!met && tid == 0) atomicOr(&sim->error, SAMPO_DEV_ERR_BARRIER);
  // a copy that did not land in time may still be in flight: let it land
  // (bounded) before the CTA can exit
  if (tid == 0 && !ok) (void)mbar_wait(&s_mbar, phase ^ 1u);  // the phase whose wait ran out

  // ---- the last CTA out rearms the barrier for the next launch ----
  __syncthreads();
  if (tid == 0) {
    __threadfence();
    s_last = atomicAdd(&p.bat->done, 1u) == G - 1u ? 1u : 0u;
    if (s_last) {
      p.bat->bar = 0u;
      p.bat->done = 0u;
    }
  }
}

}  // namespace sampo
