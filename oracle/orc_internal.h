/*
 * orc_internal.h — shared internals of the oracle (test infrastructure).
 */
#ifndef ORC_INTERNAL_H
#define ORC_INTERNAL_H

#include "orc.h"

/* Counter-based random numbers.  Each draw is a pure function of
 * (seed, pixel, sample, counter), so the oracle and the device core consume
 * identical streams no matter how paths are scheduled.  The mixing function
 * is the 64-bit finaliser of SplitMix64 (Steele, Lea, Flood 2014).  This
 * replaces rt.cpp's per-row std::mt19937 seeded from std::random_device
 * (rt.cpp:348-351), whose stream is not reproducible. */
static inline uint64_t orc_mix64(uint64_t z) {
	z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
	z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
	return z ^ (z >> 31);
}
static inline uint64_t orc_key(uint64_t seed, uint32_t pixel, uint32_t sample) {
	return orc_mix64(((uint64_t)pixel << 32 | (uint64_t)sample) + seed * 0xD1B54A32D192ED03ULL);
}
static inline uint32_t orc_u32(uint64_t key, uint32_t ctr) {
	return (uint32_t)(orc_mix64(key + (uint64_t)(ctr + 1u) * 0x9E3779B97F4A7C15ULL) >> 32);
}
/* 24-bit uniform in [0,1): exact in both float and double. */
static inline float orc_uniform(uint64_t key, uint32_t ctr) {
	return (float)(orc_u32(key, ctr) >> 8) * 5.9604644775390625e-8f;
}

/* Counter layout per path: 0,1 pixel jitter; 2,3 lens; bounce b uses
 * 8+8b .. 8+8b+7: +0,+1 direction, +2 third direction draw / dielectric
 * choice, +3 Russian roulette. */
#define ORC_CTR_BOUNCE(b) (8u + 8u * (uint32_t)(b))

typedef struct orc_node {
	double bmin[3], bmax[3];
	int32_t left, right; /* children, -1 for a leaf */
	int32_t first, count;
} orc_node;

struct orc_ctx {
	orc_scene s;
	int32_t n_prims;
	int32_t use_bvh;
	orc_node *nodes;
	int32_t n_nodes;
	int32_t *prim_ids; /* leaf order */
};

/* Global id -> (type, local index). */
static inline int orc_prim_type(const orc_scene *s, int32_t id, int32_t *local) {
	if (id < s->n_spheres) {
		*local = id;
		return 0;
	}
	id -= s->n_spheres;
	if (id < s->n_quads) {
		*local = id;
		return 1;
	}
	*local = id - s->n_quads;
	return 2;
}

#endif
