/*
 * Grain-size rheology (grain_damage=1), Grain_size_evolution.c:3-152: host
 * work of the engine.
 *
 * The reference integrates, per node, the grain size r with explicit steps of
 * 100 years while a clock shared by every call (a static) is behind the model
 * time in seconds; each step updates r (growth minus damage) and sets the
 * composite creep viscosity at the node's stress and new r, clipped to
 * [lowest_vis, highest_vis].  A node's steps depend on one another and each is
 * a chain of FP64 pow/exp: on GB300 one thread per node would need of the
 * order of 10^4 cycles a step (FP64 at 1/64 of the FP32 rate), no faster than
 * a host core, so this runs on host threads, nodes in chunks.
 *
 * Restructured from the reference's loop order (all nodes per step) into all
 * steps per node, which is the same arithmetic: nodes do not interact inside
 * the loop, and the number of steps depends on the clock alone.  One exact
 * shortcut: once a step leaves a node's r unchanged, every later step repeats
 * it bit for bit (same r, stress and temperature), so the node stops there.
 *
 * Every expression keeps the reference's operand order; the file is compiled
 * without floating-point contraction.
 */
#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>

#include "mclg_host.h"

/* the routine's constants (Grain_size_evolution.c:27-60) */
static const double kMu = 0.72, kGamma = 1.0, kQ = 4.0, kP = 2.0, kTM = 1500.0, kTW = 285.0, kTref = 2500.0;
static const double kF1 = 1e-12, kF2 = 1e-2, kK = 2, kN = 3.0, kM = 3.0;
static const double kEdisp = 530.0 * 1e3, kEdiff = 300 * 1e3, kEG = 300 * 1e3;
static const double kAlpha = 1e-5, kKappa = 1e-6, kD = 2890e3, kRho = 3300.0, kG = 9.8, kY2s = 3.1536e7;

typedef struct {
	const double *X, *T;
	double *stress, *vis, *gs;
	int nno, K;
	double vis_ref, lo, hi, A0, B0, G0, dt;
} grain_job;

static void grain_nodes(const grain_job *j, long i0, long i1)
{
	for (long i = i0; i < i1; i++) {
		const double z = j->X[j->nno + i];
		if (2890 * (1.0 - z) > 200.0) {   /* deeper than 200 km: stress 0, viscosity kept */
			j->stress[i] = 0.0;
			continue;
		}
		const double T = j->T[i] * kTref + 273.5 + 2890.0 * (1.0 - z) * 0.3;
		const double A = j->A0 * exp(0.0 - kEdisp / (8.3145 * T));
		const double B = pow(M_PI * 0.5, 0.0 - kM) * j->B0 * exp(0.0 - kEdiff / (8.3145 * T));
		const double tau = j->stress[i];
		const double GG = j->G0 * exp(0.0 - kEG / (8.3145 * T));
		const double GI = kQ / kP * pow(1e-6, kQ - kP) * GG / 250.0;
		const double x = (pow(kTM, kK) - pow(T, kK)) / (pow(kTM, kK) - pow(kTW, kK));
		const double fI = kF1 * pow(kF2 / kF1, x);
		const double rF = pow(B / (A * pow(tau, kN - 1)), 1.0 / kM);
		double r = j->gs[i], v = j->vis[i];
		for (int s = 0; s < j->K; s++) {
			const double psi = 2 * A * pow(tau, kN + 1) * (1.0 + pow(rF / r, kM));
			const double dr = kMu * GI / (kQ * pow(r, kQ - 1)) - fI * r * r * psi / (kGamma * kMu);
			const double rn = r + dr * j->dt;
			v = 0.5 * tau / (A * pow(tau, kN) + B * tau / pow(rn, kM));
			v /= j->vis_ref;
			if (v < j->lo)
				v = j->lo;
			if (v > j->hi)
				v = j->hi;
			if (rn == r)   /* a fixed point: the remaining steps repeat this one */
				break;
			r = rn;
		}
		j->gs[i] = r;
		j->vis[i] = v;
	}
}

typedef struct {
	const grain_job *j;
	long i0, i1;
} grain_chunk;

static void *grain_run(void *p)
{
	const grain_chunk *c = (const grain_chunk *)p;
	grain_nodes(c->j, c->i0, c->i1);
	return NULL;
}

/* the routine's statics (first-call flag, clock) and the nodal grain size */
struct mclg_grain_state {
	int init, nno;
	double t;
	double *gs;
};

int mclg_grain_new(mclg_grain_state **g)
{
	if (g == NULL)
		return MCLG_BAD_INPUT;
	*g = (mclg_grain_state *)calloc(1, sizeof **g);
	return *g ? MCLG_OK : MCLG_BAD_INPUT;
}

void mclg_grain_delete(mclg_grain_state *g)
{
	if (g == NULL)
		return;
	free(g->gs);
	free(g);
}

int mclg_grain_get(const mclg_grain_state *g, double *gs, size_t n)
{
	if (g == NULL || gs == NULL || g->gs == NULL || n != (size_t)g->nno) {
		mclg_set_error("grain size: no state of %zu nodes", n);
		return MCLG_BAD_INPUT;
	}
	memcpy(gs, g->gs, n * sizeof(double));
	return MCLG_OK;
}

int mclg_grain_update(mclg_grain_state *g, int nno, const double *X, const double *T, double *stress,
                      double *vis, double model_time, double Ra, double lowest_vis, double highest_vis,
                      int threads)
{
	const double vis_ref = (kRho * kG * kAlpha * kTref * kD * kD * kD) / (Ra * kKappa);
	const double stress_scale = (vis_ref * kKappa) / (kD * kD), time_scale = kD * kD / kKappa;
	const double dt = 1e2 * kY2s;
	grain_job j;
	if (g == NULL || X == NULL || T == NULL || stress == NULL || vis == NULL || nno < 1)
		return MCLG_BAD_INPUT;
	if (g->gs == NULL || g->nno != nno) {
		double *p = (double *)realloc(g->gs, (size_t)(nno > 0 ? nno : 1) * sizeof(double));
		if (p == NULL) {
			mclg_set_error("grain size: out of host memory");
			return MCLG_BAD_INPUT;
		}
		g->gs = p;
		g->nno = nno;
	}
	if (!g->init) {   /* the first call sets r = 1e-3 and changes nothing else */
		for (int i = 0; i < nno; i++)
			g->gs[i] = 1e-3;
		g->init = 1;
		return MCLG_OK;
	}
	for (int i = 0; i < nno; i++)
		stress[i] *= stress_scale;
	/* the reference's clock: steps of dt while it is behind the model time */
	j.K = 0;
	while (g->t < model_time * time_scale) {
		g->t += dt;
		j.K++;
	}
	if (j.K == 0)
		return MCLG_OK;
	j.X = X;
	j.T = T;
	j.stress = stress;
	j.vis = vis;
	j.gs = g->gs;
	j.nno = nno;
	j.vis_ref = vis_ref;
	j.lo = lowest_vis;
	j.hi = highest_vis;
	j.A0 = 1.1e5 / pow(1e6, kN);
	j.B0 = 13.6 * pow(1e-6, kM) / 1e6;
	j.G0 = 2e4 * pow(1e-6, kP);
	j.dt = dt;
	{
		enum { kMaxT = 16 };
		grain_chunk ch[kMaxT];
		pthread_t th[kMaxT];
		int started[kMaxT], nt = threads < 1 ? 1 : threads > kMaxT ? kMaxT : threads;
		if (nt > nno)
			nt = nno > 0 ? nno : 1;
		for (int k = 0; k < nt; k++) {
			ch[k].j = &j;
			ch[k].i0 = (long)nno * k / nt;
			ch[k].i1 = (long)nno * (k + 1) / nt;
			started[k] = k < nt - 1 && pthread_create(&th[k], NULL, grain_run, &ch[k]) == 0;
			if (!started[k])
				grain_run(&ch[k]);
		}
		for (int k = 0; k < nt; k++)
			if (started[k])
				pthread_join(th[k], NULL);
	}
	return MCLG_OK;
}
