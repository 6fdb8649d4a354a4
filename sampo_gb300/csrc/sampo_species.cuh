// sampo_species.cuh - the species functions of the step (include/properties.h
// in the reference: delays, development rate, transition times, hatching,
// the two normal draws and egg laying), behind one interface the model uses.
//
// Built in: the reference's shipped properties.h, restated in this file's
// own code; the per-step functions are evaluated once per step (make_ctx)
// and the normal draws are deferred to dense warps (finish_box_muller).
//
// SAMPO_USER_SPECIES: the step kernels are compiled at run time by NVRTC
// against a user's properties.h-style header (the reference compiles its
// kernels with the header named by argv[3], src/abms.c:565-568). The header
// is included inside namespace sampo_user after sampo_species_prelude.h, which
// gives it the OpenCL C types, qualifiers and built-ins it expects (math
// through this library's deterministic functions, HybridTaus and BoxMuller
// through the step's generator), and the adapters below call its functions
// where updateAgents.cl and initAgents.cl call them.
#pragma once

namespace sampo {

// Transition-time bits of a step (StepCtx::tt): which states may leave this
// hour (eggsTransitionTime ... gravidsEggLayTime).
enum : uint32_t {
  TT_EGG = 1u, TT_LARVA = 2u, TT_PUPA = 4u, TT_IMMATURE = 8u,
  TT_MATESEEKING = 16u, TT_BMS = 32u, TT_BMD = 64u, TT_LAY = 128u
};

}  // namespace sampo

#ifndef SAMPO_USER_SPECIES

namespace sampo {

// BITE_HUMAN_PROBABILITY, BITE_INDOOR_PROBABILITY, REST_INDOOR_PROBABILITY
// (include/properties.h:12-14; kernel/updateAgents.cl:15-23 defaults)
#define SAMPO_BITE_HUMAN 1.0f
#define SAMPO_BITE_INDOOR 1.0f
#define SAMPO_REST_INDOOR 1.0f

// include/properties.h:94-98 (double literals stored as float, as there)
__device__ const float kDevRates[32] = {
    0.000175044, 0.000549094, 0.00109031, 0.001494158, 0.001752487, 0.001962866, 0.002171238, 0.002392989,
    0.002633689, 0.00289619, 0.003182685, 0.003495287, 0.003836204, 0.004207789, 0.004612566, 0.005053243,
    0.005532729, 0.006054144, 0.006620836, 0.007236393, 0.007904657, 0.008629745, 0.009416051, 0.010267388,
    0.011113704, 0.011960019, 0.012806335, 0.010401163, 0.007995991, 0.00033845, 0.00000533086, 0.0000000840986};

__host__ __device__ __forceinline__ bool night(uint32_t wt) { return wt <= 6u || wt >= 18u; }

// The species constants of one step at temperature T and world time wt.
__device__ __forceinline__ void species_step(float T, uint32_t wt, StepCtx& c) {
  c.eggIncubation = -0.923f * T + 60.923f;                           // include/properties.h:29-31
  const float cl = sampo_fminf(sampo_fmaxf(T, 12.0f), 48.0f);         // :105-109
  const int di = (int)cl - 12;
  c.devOOB = di > 31;
  c.larvaDev = di > 31 ? 0.0f : kDevRates[di];
  c.pupaDelay = __double2float_rn(__dadd_rn(__dmul_rn(-0.923, (double)T), 60.923));  // :133-135
  c.immatureDelay = -2.667f * T + 120.0f;                            // :159-161
  c.mateDelay = 1.0f;                                                // :182-184
  c.bmsDelay = 0.0f;                                                 // :208-210
  c.bmdDelay = -1.231f * T + 77.231f;                                // :239-241
  // :68-70, 117-119, 143-145, 169-171, 195-197, 222-224, 249-251, 280-282
  c.tt = TT_EGG | TT_IMMATURE | TT_BMD | (wt == 18u ? TT_MATESEEKING : 0u) |
         (night(wt) ? (TT_LARVA | TT_PUPA | TT_BMS | TT_LAY) : 0u);
}

// eggsHatching (include/properties.h:39-60)
__device__ __forceinline__ float species_eggs_hatching(float p) {
  float m, b;
  if (p < 0.5f) { m = 48.0f; b = 0.0f; }
  else if (p < 0.85f) { m = 68.5714f; b = -10.2857f; }
  else if (p < 0.90f) { m = 480.0f; b = -360.0f; }
  else if (p < 0.94f) { m = 600.00f; b = -468.0f; }
  else { m = 2400.0f; b = -2160.0f; }
  return trunc_sat_fast(m * p + b + 0.5f);
}

}  // namespace sampo

#else  // SAMPO_USER_SPECIES

namespace sampo_user {
#include "sampo_species_prelude.h"
#include "sampo_user_species.h"
}  // namespace sampo_user

namespace sampo {

#ifdef BITE_HUMAN_PROBABILITY
#define SAMPO_BITE_HUMAN ((float)(BITE_HUMAN_PROBABILITY))
#else
#define SAMPO_BITE_HUMAN 1.0f
#endif
#ifdef BITE_INDOOR_PROBABILITY
#define SAMPO_BITE_INDOOR ((float)(BITE_INDOOR_PROBABILITY))
#else
#define SAMPO_BITE_INDOOR 1.0f
#endif
#ifdef REST_INDOOR_PROBABILITY
#define SAMPO_REST_INDOOR ((float)(REST_INDOOR_PROBABILITY))
#else
#define SAMPO_REST_INDOOR 1.0f
#endif

// The step's four generator slots for slot index gid, as the header sees them.
__device__ __forceinline__ void user_seeds(const StepCtx& c, uint32_t gid, sampo_user::Seeds s[4]) {
#pragma unroll
  for (int k = 0; k < 4; k++) {
    s[k].c13 = c.rng_c13[k];
    s[k].z2 = c.rng_z2[k];
    s[k].z4 = c.rng_z4[k];
    s[k].gid = gid;
  }
}

// The per-step functions depend on the temperature and the world time only,
// so they are evaluated once per step.
__device__ __forceinline__ void species_step(float T, uint32_t wt, StepCtx& c) {
  using namespace sampo_user;
  c.eggIncubation = eggsIncubation(T);
  c.larvaDev = larvaDevelopment(T);
  c.devOOB = 0;
  c.pupaDelay = pupaDelay(T);
  c.immatureDelay = immatureDelay(T);
  c.mateDelay = mateSeekingDelay(T);
  c.bmsDelay = bloodMealSeekingDelay(T);
  c.bmdDelay = bloodMealDigestingDelay(T);
  c.tt = (eggsTransitionTime(wt) ? TT_EGG : 0u) | (larvaeTransitionTime(wt) ? TT_LARVA : 0u) |
         (pupaeTransitionTime(wt) ? TT_PUPA : 0u) | (immaturesTransitionTime(wt) ? TT_IMMATURE : 0u) |
         (mateSeekingsTransitionTime(wt) ? TT_MATESEEKING : 0u) | (bloodMealSeekingsTransitionTime(wt) ? TT_BMS : 0u) |
         (bloodMealDigestingsTransitionTime(wt) ? TT_BMD : 0u) | (gravidsEggLayTime(wt) ? TT_LAY : 0u);
}

__device__ __forceinline__ float species_eggs_hatching(float p) { return sampo_user::eggsHatching(p); }

// larvaDelay(seeds + 1) (kernel/updateAgents.cl:79)
__device__ __forceinline__ float species_larva_delay(const StepCtx& c, uint32_t gid) {
  sampo_user::Seeds s[4];
  user_seeds(c, gid, s);
  return sampo_user::larvaDelay(s + 1);
}

// generateEggs(seeds + 1, &numEggBatches) (kernel/updateAgents.cl:213)
__device__ __forceinline__ uint32_t species_generate_eggs(const StepCtx& c, uint32_t gid, uint32_t& batches) {
  sampo_user::Seeds s[4];
  user_seeds(c, gid, s);
  uint32_t nb = batches;
  const uint32_t eggs = (uint32_t)sampo_user::generateEggs(s + 1, &nb);
  batches = nb;
  return eggs;
}

// layEggs(&agent, &agentState, enb, seeds, carryingCapacity)
// (kernel/updateAgents.cl:246): the gravid's eggs left; *laid = what it
// added to enb->newEggs. The record carries the fields both passes load.
__device__ __forceinline__ uint32_t species_lay_eggs(const StepCtx& c, uint32_t gid, const Rec& a, uint32_t avail,
                                                     uint32_t& laid) {
  sampo_user::Seeds s[4];
  user_seeds(c, gid, s);
  sampo_user::Agent ag;
  ag.availableEggs = avail;
  ag.cycleLength = a.cycle;
  ag.humanBloodmealCount = a.hbc;
  ag.delay = a.delay;
  ag.numEggBatches = a.batches;
  ag.ovipositionAttemps = a.uni;
  sampo_user::AgentState st;
  st.dead = false;
  st.state = sampo_user::GRAVID;
  sampo_user::EggsNbiomass enb;
  enb.totalBiomass = (int)c.totalBiomass;
  enb.newEggs = 0u;
  const uint32_t left = (uint32_t)sampo_user::layEggs(&ag, &st, &enb, s, c.env.carryingCapacity);
  laid = enb.newEggs;
  return left;
}

}  // namespace sampo

#endif  // SAMPO_USER_SPECIES
