/*
 * hot_species.h - a species header in the form the reference's
 * include/properties.h takes (OpenCL C, the same function names and
 * signatures), used by the tests of run-time species compilation. Every
 * function the step kernels take from a species header differs from the
 * shipped species, and the three *_PROBABILITY macros are below 1, so that a
 * simulation with this header departs from the built-in one at every hook:
 * delays, development table, transition windows, hatching, both normal
 * draws, egg laying, the ITN/IRS factors and the bitesAhuman draw.
 */
#pragma once

#include "device_types.h"
#include "agent.h"
#include "gpuRand.h"

#define BITE_HUMAN_PROBABILITY 0.9f
#define BITE_INDOOR_PROBABILITY 0.8f
#define REST_INDOOR_PROBABILITY 0.7f

/* eggs */
REAL eggsIncubation(Temperature temperature) {
	return 52.5f - 0.75f * temperature;
}

REAL eggsHatching(REAL probability) {
	if (probability < 0.6f) return (UINT)(40.0f * probability + 0.5f);
	if (probability < 0.9f) return (UINT)(90.0f * probability - 30.0f + 0.5f);
	return (UINT)(600.0f * probability - 489.0f + 0.5f);
}

bool eggsTransitionTime(UINT worldTime) {
	return worldTime >= 4u && worldTime <= 21u;
}

/* larvae: development per hour by whole degree from 14 to 37 C */
REAL larvaDelay(__constant struct Seeds* seeds) {
	return BoxMuller(seeds, 0.9f, 0.12f);
}

__constant REAL hotDevRates[] = {
	0.00031f, 0.00062f, 0.00098f, 0.00141f, 0.00190f, 0.00246f, 0.00309f, 0.00378f,
	0.00454f, 0.00537f, 0.00626f, 0.00722f, 0.00825f, 0.00934f, 0.01050f, 0.01172f,
	0.01230f, 0.01188f, 0.01047f, 0.00851f, 0.00602f, 0.00344f, 0.00128f, 0.00020f };

REAL larvaDevelopment(Temperature temperature) {
	Temperature t = min(max(temperature, 14.0f), 37.0f);
	return hotDevRates[((int)t) - 14];
}

bool larvaeTransitionTime(UINT worldTime) {
	return worldTime <= 8u || worldTime >= 17u;
}

/* pupae (a double expression, as in the shipped header) */
REAL pupaDelay(Temperature temperature) {
	return 55.0 - 0.85 * temperature;
}

bool pupaeTransitionTime(UINT worldTime) {
	return worldTime <= 9u || worldTime >= 16u;
}

/* adults */
REAL immatureDelay(Temperature temperature) {
	return 100.0f - 2.2f * temperature;
}

bool immaturesTransitionTime(UINT worldTime) {
	return worldTime != 12u;
}

REAL mateSeekingDelay(Temperature temperature) {
	return 2.0f;
}

bool mateSeekingsTransitionTime(UINT worldTime) {
	return worldTime == 18u || worldTime == 19u;
}

REAL bloodMealSeekingDelay(Temperature temperature) {
	return 1.0f;
}

bool bloodMealSeekingsTransitionTime(UINT worldTime) {
	return worldTime <= 5u || worldTime >= 19u;
}

REAL bloodMealDigestingDelay(Temperature temperature) {
	return 70.0f - 1.1f * temperature;
}

bool bloodMealDigestingsTransitionTime(UINT worldTime) {
	return worldTime != 0u;
}

UINT generateEggs(__constant struct Seeds* seeds, UINT* numEggBatches) {
	UINT eggs = (UINT)(BoxMuller(seeds, 140.0f, 25.0f) + 0.5f);
	eggs = (UINT)(eggs * pow(0.85f, (REAL)*numEggBatches) + 0.5f);
	++(*numEggBatches);
	return eggs;
}

bool gravidsEggLayTime(UINT worldTime) {
	return worldTime <= 7u || worldTime >= 17u;
}

INT layEggs(__private struct Agent* agent, __private struct AgentState* agentState, __global struct EggsNbiomass* enb,
		__constant struct Seeds* seeds, REAL carryingCapacity) {
	REAL crowding = ((REAL)enb->totalBiomass) / (carryingCapacity * (1.0f + 0.5f * (REAL)agent->ovipositionAttemps));
	REAL room = max(0.0f, 1.0f - crowding);
	UINT laid = (UINT)ceil((REAL)agent->availableEggs * room);
	atomic_add(&(enb->newEggs), laid);
	return agent->availableEggs - laid;
}
