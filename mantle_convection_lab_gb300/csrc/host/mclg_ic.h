/*
 * Seeded synthetic initial temperatures.
 *
 * The reference seeds its random perturbations with the unseeded C rand()
 * (Initial_condition.c:41-52, 98-120), so runs are not reproducible across
 * machines.  This header replaces that with a counter-based generator
 * (Philox4x32-10, Salmon et al., "Parallel random numbers: as easy as 1, 2,
 * 3", SC'11) keyed by a 64-bit seed and counted by the global node id, so the
 * same field comes out on every host and in every language that restates it.
 *
 * Temperature kinds (selected with T_ini=-2 and ic_kind=<k> in the .input file):
 *   1  conductive profile + one cosine mode + uniform noise
 *      T = (H - z) + a_p sin(pi (H - z)/H) cos(k pi x / L) + U(-a_n, a_n)
 *      (the reference's conductive_T, Initial_condition.c:55-75, plus noise)
 *   2  tanh boundary layers of thickness delta + m seeded cosine modes
 *      T = 1/2 + 1/2 (1 - tanh(z/delta)) - 1/2 (1 - tanh((H - z)/delta))
 *          + sum_j a_m cos(p_j pi x / L + phi_j) sin(q_j pi z / H)
 * Dirichlet rows are reset afterwards by the caller (apply_T_bc_values,
 * Initial_condition.c:122-136).
 *
 * Header-only so that the host library, the test oracle and the reference
 * dump harness draw exactly the same numbers.
 */
#ifndef MCLG_IC_H
#define MCLG_IC_H

#include <math.h>
#include <stdint.h>

typedef struct mclg_ic_params {
	int kind;              /* 1 or 2, see above */
	uint64_t seed;         /* Philox key */
	double noise;          /* a_n: half-width of the uniform noise */
	double perturb;        /* a_p: cosine-mode amplitude for kind 1 */
	int wave;              /* k: cosine wave number for kind 1 */
	double bl_thickness;   /* delta for kind 2 */
	int nmodes;            /* m for kind 2 */
	double mode_amp;       /* a_m for kind 2 */
	double length, height; /* L, H: model box */
} mclg_ic_params;

#define MCLG_PHILOX_M0 0xD2511F53u
#define MCLG_PHILOX_M1 0xCD9E8D57u
#define MCLG_PHILOX_W0 0x9E3779B9u
#define MCLG_PHILOX_W1 0xBB67AE85u

static inline void mclg_philox4x32_10(const uint32_t ctr_in[4], uint64_t key64, uint32_t out[4])
{
	uint32_t c0 = ctr_in[0], c1 = ctr_in[1], c2 = ctr_in[2], c3 = ctr_in[3];
	uint32_t k0 = (uint32_t)key64, k1 = (uint32_t)(key64 >> 32);
	int r;
	for (r = 0; r < 10; r++) {
		uint64_t p0 = (uint64_t)MCLG_PHILOX_M0 * c0;
		uint64_t p1 = (uint64_t)MCLG_PHILOX_M1 * c2;
		uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
		uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
		c0 = hi1 ^ c1 ^ k0;
		c1 = lo1;
		c2 = hi0 ^ c3 ^ k1;
		c3 = lo0;
		k0 += MCLG_PHILOX_W0;
		k1 += MCLG_PHILOX_W1;
	}
	out[0] = c0; out[1] = c1; out[2] = c2; out[3] = c3;
}

/* Uniform double in [0,1) from stream `stream`, counter `n` (53 random bits). */
static inline double mclg_uniform01(uint64_t seed, uint32_t stream, uint32_t n)
{
	uint32_t ctr[4] = {n, stream, 0u, 0u}, o[4];
	uint64_t m;
	mclg_philox4x32_10(ctr, seed, o);
	m = ((uint64_t)o[0] << 21) ^ (uint64_t)(o[1] >> 11);
	return (double)m * (1.0 / 9007199254740992.0);
}

/* Temperature at node (x, z) whose global node id (iz + ix*gnoz) is gid. */
static inline double mclg_ic_temperature(const mclg_ic_params *p, double x, double z, uint32_t gid)
{
	const double pi = 3.14159265358979323846;
	double T = 0.0;
	if (p->kind == 1) {
		T = (p->height - z)
		  + p->perturb * sin(pi * (p->height - z) / p->height) * cos(p->wave * pi * x / p->length);
		T += p->noise * (2.0 * mclg_uniform01(p->seed, 0u, gid) - 1.0);
	} else if (p->kind == 2) {
		int j;
		double d = p->bl_thickness;
		T = 0.5 + 0.5 * (1.0 - tanh(z / d)) - 0.5 * (1.0 - tanh((p->height - z) / d));
		for (j = 0; j < p->nmodes; j++) {
			/* mode parameters come from stream 1, counters 3j..3j+2 */
			int pj = 1 + (int)(4.0 * mclg_uniform01(p->seed, 1u, 3u * (uint32_t)j));
			int qj = 1 + (int)(4.0 * mclg_uniform01(p->seed, 1u, 3u * (uint32_t)j + 1u));
			double ph = 2.0 * pi * mclg_uniform01(p->seed, 1u, 3u * (uint32_t)j + 2u);
			T += p->mode_amp * cos(pj * pi * x / p->length + ph) * sin(qj * pi * z / p->height);
		}
		T += p->noise * (2.0 * mclg_uniform01(p->seed, 0u, gid) - 1.0);
	}
	return T;
}

#endif
