// sampo_model.cuh - the per-agent SAMPO model on the GPU (sm_103a).
//
// One hourly step of one agent: killAgents (kernel/killAgents.cl:24-148)
// followed by updateAgents (kernel/updateAgents.cl:39-270) with the species
// functions of sampo_species.cuh (include/properties.h, or a user's header
// compiled in at run time) and the generator of include/gpuRand.h.
// Float expressions are written in the reference's operation order and the
// file is compiled with --fmad=false, so every product and sum rounds exactly
// as the reference's C semantics say; the two places where the reference
// promotes to double (include/properties.h:134, kernel/updateAgents.cl:69-70)
// stay double.
//
// update_agent<FULL> is used twice per step: FULL=false by the counting pass
// (only the fields that decide survival, the next state and the number of
// eggs laid) and FULL=true by the scatter pass (the complete record). Both
// instantiations run the same decision code on the same inputs, so they
// agree bit for bit. EGGS adds the eggs laid to Acc::newEggs (the counting
// pass, and the one-launch step, whose single update decides and writes).
// LDG reads the larval mortality table through the read-only cache; the
// one-launch step, which rewrites the table between the hours of one launch,
// keeps a copy in shared memory instead.
#pragma once
#include <stdint.h>
#include "sampo_math.h"
#include "sampo_math_fast.h"
#include "../../include/sampo.h"

namespace sampo {

enum : int { EGG = 0, LARVA, PUPA, IMMATURE, MATESEEKING, BMS, BMD, GRAVID, NSTATE };
constexpr uint32_t kLayoutAlign = 64;  // LOCAL_SIZE (include/agent.h:9-17): a layout constant
constexpr uint32_t kEggBatchTable = 64;  // batches with a tabulated 0.8^(n-1)

// The egg-batch factor pow(0.8f, n) (include/properties.h:262), tabulated on
// the host for n < kEggBatchTable with the same definition.
__host__ __device__ __forceinline__ float egg_batch_scale(uint32_t n) { return sampo_powf(0.8f, (float)n); }

// One agent record in registers (the SoA columns of the pool).
struct Rec {
  float age, his, delay, sporo;
  uint32_t uni;      // cumulativeLarvalDelay (float bits) for larvae, ovipositionAttemps for gravids
  uint32_t avail, cycle, hbc, batches;
  uint32_t female;   // 0/1
  uint32_t bm;       // Box-Muller draw still owed: 0 none, BM_LARVA_DELAY, BM_EGG_BATCH
};

// The two normal draws of the model (include/gpuRand.h:56-63) cost a binary64
// log and sin each. They happen on rare transitions, one lane in a warp at a
// time, so the full update leaves them owed in Rec::bm and the scatter kernel
// evaluates them afterwards in dense warps (finish_box_muller).
enum : uint32_t { BM_NONE = 0, BM_LARVA_DELAY = 1, BM_EGG_BATCH = 2 };

// Tables that do not change during a run and are the same for every
// simulation (kernel/killAgents.cl:84-115,135-147; include/properties.h:262).
// The count pass needs only the mortality part (KillConst, a prefix).
struct KillConst {
  float aquaticHMR;            // eggs and pupae (kernel/killAgents.cl:103-115,135-147)
  float adultHMR[100];
};
struct ModelConst {
  KillConst kill;
  float eggBatchScale[kEggBatchTable];  // egg_batch_scale(n)
};

// Per-step constants of one simulation, shared by every agent of the step.
// Computed once per step (k_publish) and copied to shared memory by the
// kernels that step the simulation.
struct alignas(16) StepCtx {
  // HybridTaus (include/gpuRand.h:33-50): z1 and z3 do not depend on the
  // work-item, so their Tausworthe steps are folded per seed slot.
  uint32_t rng_c13[4], rng_z2[4], rng_z4[4];
  sampo_environment env;
  float T;
  uint32_t wt;                 // world time = step % 24
  uint32_t totalBiomass;       // kernel/killAgents.cl:42-43
  float eggIncubation;         // eggsIncubation(T)
  float larvaDev;              // larvaDevelopment(T)
  float pupaDelay, immatureDelay, bmdDelay;
  float mateDelay, bmsDelay;   // mateSeekingDelay(T), bloodMealSeekingDelay(T)
  uint32_t tt;                 // transition-time bits of the hour (TT_*, sampo_species.cuh)
  double sporoInc;             // 1/((111/(T-16))*14) in double, used when T > 16 and bitten
  float sporoH, sporoM, sporoL;  // sporoInc = sporoH + sporoM + sporoL exactly
  uint32_t sporoOn;            // T > 16
  uint32_t devOOB;             // T >= 44: the reference reads past devRates
  const float* larvaHMR;       // [100] in global memory; NaN outside the larvae's age range of the step
};

// Counters an agent update contributes to (BitesNcycles, EggsNbiomass).
struct Acc {
  uint32_t newEggs, bites, infectBites, cycles, sumCycles;
  uint32_t bad;                // larva table miss (must stay 0)
};

__host__ __device__ __forceinline__ uint32_t taus_step(uint32_t z, int S1, int S2, int S3, uint32_t M) {
  uint32_t b = (((z << S1) ^ z) >> S2);
  return (((z & M) << S3) ^ b);
}

// Exact int <-> float conversions from FP32 adds and integer ops only: the
// hardware conversion instructions issue at a fraction of the FP32 rate.
// (float)v rounded to nearest: both 16-bit halves are exact as 2^23-biased
// floats, hi * 2^16 is exact, so the one rounding of the final add is the
// correct rounding of v.
__device__ __forceinline__ float u32_to_f32_rn(uint32_t v) {
  const float hi = __uint_as_float(0x4B000000u | (v >> 16)) - 8388608.0f;
  const float lo = __uint_as_float(0x4B000000u | (v & 0xFFFFu)) - 8388608.0f;
  return __fadd_rn(__fmul_rn(hi, 65536.0f), lo);
}
// (uint32_t)x truncated toward zero for 0 <= x < 2^22 (x + 2^23 rounds to
// the nearest integer; step back when that rounded up); NaN and x <= 0 give 0.
__device__ __forceinline__ uint32_t f32_to_u32_small(float x) {
  if (!(x > 0.0f)) return 0u;
  const float r = __fadd_rn(x, 8388608.0f);
  const uint32_t n = __float_as_uint(r) - 0x4B000000u;
  return __fadd_rn(r, -8388608.0f) > x ? n - 1u : n;
}
// sampo_f2u_sat(x) for every x, through FP32 adds below 2^22.
__device__ __forceinline__ uint32_t f2u_sat_fast(float x) {
  return x < 4194304.0f ? f32_to_u32_small(x) : sampo_f2u_sat(x);
}
// (float)sampo_f2u_sat(x) for every x, through FP32 adds below 2^22.
__device__ __forceinline__ float trunc_sat_fast(float x) {
  if (!(x > 0.0f)) return 0.0f;
  if (!(x < 4194304.0f)) return (float)sampo_f2u_sat(x);
  const float r = __fadd_rn(__fadd_rn(x, 8388608.0f), -8388608.0f);  // x rounded to an integer
  return r > x ? __fadd_rn(r, -1.0f) : r;
}

// HybridTaus of one seed slot whose z1 and z3 parts are folded into c13.
__device__ __forceinline__ float rng_folded(uint32_t c13, uint32_t z2, uint32_t z4, uint32_t gid) {
  uint32_t v = c13 ^ taus_step(z2 + gid, 2, 25, 4, 4294967288u) ^ (1664525u * (z4 * gid) + 1013904223u);
  return 2.3283064365387e-10f * u32_to_f32_rn(v);  // (float)v * 2^-32
}
__device__ __forceinline__ float rng(const StepCtx& c, int slot, uint32_t gid) {
  return rng_folded(c.rng_c13[slot], c.rng_z2[slot], c.rng_z4[slot], gid);
}

// BoxMuller (include/gpuRand.h:56-63) of two uniform draws.
__device__ __forceinline__ float box_muller_u(float u0, float u1, float mean, float sd) {
  float r = __fsqrt_rn(-2.0f * sampo_logf_bm(u0));
  float theta = (2.0f * 3.14159274101257f) * u1;
  return (r * sampo_sinf_bm(theta)) * sd + mean;
}
// BoxMuller(seeds+1, ...): u0 from slot 1, u1 from slot 2.
__device__ __forceinline__ float box_muller(const StepCtx& c, uint32_t gid, float mean, float sd) {
  return box_muller_u(rng(c, 1, gid), rng(c, 2, gid), mean, sd);
}

}  // namespace sampo

#include "sampo_species.cuh"

namespace sampo {

__device__ __forceinline__ uint32_t age_days(float age) {
  return f32_to_u32_small(sampo_fminf(age / 24.0f, 99.0f));  // kernel/killAgents.cl:55
}
// (UINT)(age / 24.0f) without the 99-day cap (kernel/calcL1de.cl:30)
__device__ __forceinline__ uint32_t age_days_uncapped(float age) {
  return f2u_sat_fast(age / 24.0f);
}

// Kill then update one valid agent of range rg at slot gid.
// Returns the next state (0..7), or -1 when the agent dies this step.
template <bool FULL, bool EGGS = !FULL, bool LDG = true>
__device__ __forceinline__ int update_agent(const StepCtx& c, const KillConst& mc, int rg, uint32_t gid, Rec& a, Acc& acc) {
  // ---- killAgents (kernel/killAgents.cl:52-147) ----
  {
    float prob = rng(c, 0, gid);
    float hmr;
    if (rg >= IMMATURE) {
      hmr = mc.adultHMR[age_days(a.age)];
    } else if (rg == LARVA) {
      hmr = LDG ? __ldg(c.larvaHMR + age_days(a.age)) : c.larvaHMR[age_days(a.age)];
      if (hmr != hmr) acc.bad = 1;  // table entry not prepared
    } else {
      hmr = mc.aquaticHMR;
    }
    if (prob <= hmr) return -1;
  }
  // ---- updateAgents (kernel/updateAgents.cl:57-270), elapsedTimeInHours = 1.0f ----
  a.age = a.age + 1.0f;
  a.his = a.his + 1.0f;
  if (FULL && c.sporoOn && a.hbc > 0u)  // kernel/updateAgents.cl:69-70, in double
    a.sporo = sampo_sporo_add(a.sporo, c.sporoH, c.sporoM, c.sporoL, c.sporoInc);
  switch (rg) {
    case EGG:
      if (a.his >= a.delay && (c.tt & TT_EGG)) {
        if (FULL) {
          a.age = 24.0f; a.his = 0.0f;
#ifdef SAMPO_USER_SPECIES
          a.delay = species_larva_delay(c, gid);
#else
          a.bm = BM_LARVA_DELAY;  // delay = larvaDelay (include/properties.h:87-91), owed
#endif
        }
        return LARVA;
      }
      return EGG;
    case LARVA: {
      if (c.env.larvacideValue > 0.0f && a.his == 1.0f) {
        if (rng(c, 2, gid) <= c.env.larvacideValue) return -1;
      }
      float cld = __uint_as_float(a.uni) + c.larvaDev;
      if (FULL) a.uni = __float_as_uint(cld);
      if (cld >= a.delay && (c.tt & TT_LARVA)) {
        if (FULL) { a.his = 0.0f; a.delay = c.pupaDelay; }
        return PUPA;
      }
      return LARVA;
    }
    case PUPA:
      if (a.his >= a.delay && (c.tt & TT_PUPA)) {
        if (FULL) { a.age = 0.0f; a.his = 0.0f; a.delay = c.immatureDelay; }
        return IMMATURE;
      }
      return PUPA;
    case IMMATURE:
      if (a.his >= a.delay && (c.tt & TT_IMMATURE)) {
        if (FULL) { a.delay = c.mateDelay; a.his = 0.0f; }
        return MATESEEKING;
      }
      return IMMATURE;
    case MATESEEKING:
      if (a.his >= a.delay && a.female && (c.tt & TT_MATESEEKING)) {
        if (FULL) { a.his = 0.0f; a.delay = c.bmsDelay; }
        return BMS;
      }
      return MATESEEKING;
    case BMS:
      if (FULL) a.cycle += 1u;
      if (a.his >= a.delay && (c.tt & TT_BMS)) {
        if (rng(c, 1, gid) <= c.env.bloodmealSuccess) {
          if (c.env.ITNValue * SAMPO_BITE_HUMAN * SAMPO_BITE_INDOOR > 0.0f) {
            if (rng(c, 2, gid) <= c.env.ITNValue * SAMPO_BITE_HUMAN * SAMPO_BITE_INDOOR) return -1;
          }
          if (FULL) {
            // bitesAhuman (kernel/updateAgents.cl:175)
            const uint32_t bites = SAMPO_BITE_HUMAN < 1.0f ? (rng(c, 3, gid) <= SAMPO_BITE_HUMAN ? 1u : 0u) : 1u;
            a.hbc += bites;
            acc.bites += 1u;
            a.his = 0.0f; a.delay = c.bmdDelay;
            if (a.sporo >= 1.0f && bites) acc.infectBites += 1u;
          }
          return BMD;
        }
      }
      return BMS;
    case BMD:
      if (c.env.IRSValue * SAMPO_REST_INDOOR > 0.0f) {
        if (rng(c, 2, gid) <= c.env.IRSValue * SAMPO_REST_INDOOR) return -1;
      }
      if (FULL) a.cycle += 1u;
      if (a.his >= a.delay && (c.tt & TT_BMD)) {
        if (FULL) {
          if (a.avail <= 0u && a.female) {
#ifdef SAMPO_USER_SPECIES
            a.avail = species_generate_eggs(c, gid, a.batches);
#else
            // generateEggs (include/properties.h:257-266): the batch size is
            // owed; numEggBatches is incremented now, the draw uses the old value
            a.batches += 1u;
            a.bm = BM_EGG_BATCH;
#endif
          }
          a.his = 0.0f; a.uni = 0u;
        }
        return GRAVID;
      }
      return BMD;
    default: {  // GRAVID
      if (FULL) a.cycle += 1u;
      if (c.tt & TT_LAY) {
        if (rng(c, 1, gid) < 0.25f) {
          uint32_t avail = a.avail;
          bool trapped = false;
          if (c.env.oviTrapValue > 0.0f) {
            if (rng(c, 2, gid) <= c.env.oviTrapValue) { trapped = true; avail = 0u; }
          }
          if (!trapped) {
#ifdef SAMPO_USER_SPECIES
            uint32_t pe = 0;
            avail = species_lay_eggs(c, gid, a, avail, pe);
            if (EGGS) acc.newEggs += pe;
#else
            // layEggs (include/properties.h:296-307)
            float nbm = u32_to_f32_rn(c.totalBiomass) / ((u32_to_f32_rn(a.uni) + 1.0f) * c.env.carryingCapacity);
            float pbm = sampo_fmaxf(0.0f, 1.0f - nbm);
            uint32_t pe = f2u_sat_fast(ceilf(u32_to_f32_rn(avail) * pbm));
            if (EGGS) acc.newEggs += pe;
            avail = avail - pe;
#endif
          }
          if (FULL) { a.uni += 1u; a.avail = avail; }
          if (avail == 0u) {
            if (FULL) {
              acc.cycles += 1u; acc.sumCycles += a.cycle;
              a.cycle = 0u; a.his = 0.0f; a.delay = c.bmsDelay;
            }
            if (trapped) return -1;
            return BMS;
          }
        }
      }
      return GRAVID;
    }
  }
}

// The owed draw of an agent at slot gid: larvaDelay (include/properties.h:87-91)
// returns the new delay bits; generateEggs (:257-266) returns availableEggs,
// given numEggBatches after its increment.
__device__ __forceinline__ uint32_t finish_box_muller(const StepCtx& c, const ModelConst& mc, uint32_t gid, uint32_t kind,
                                                      uint32_t batches_after) {
  if (kind == BM_LARVA_DELAY) return __float_as_uint(box_muller(c, gid, 1.0f, 0.1f));
  uint32_t eggs = f2u_sat_fast(box_muller(c, gid, 170.0f, 30.0f) + 0.5f);
  const uint32_t n = batches_after - 1u;
  const float scale = n < kEggBatchTable ? mc.eggBatchScale[n] : egg_batch_scale(n);
  return f2u_sat_fast(u32_to_f32_rn(eggs) * scale + 0.5f);
}

// initAgents (kernel/initAgents.cl:34-64) for new slot id.
__device__ __forceinline__ void new_egg(const StepCtx& c, uint32_t id, Rec& a) {
  a.age = 0.0f; a.his = 0.0f;
  a.female = rng(c, 3, id) <= 0.5f ? 1u : 0u;
  a.sporo = 0.0f;
  a.hbc = 0u; a.avail = 0u; a.cycle = 0u; a.uni = 0u;
  a.delay = c.eggIncubation + species_eggs_hatching(rng(c, 2, id));
  a.batches = 0u;
}

}  // namespace sampo
