/*
 * CPU oracle: a plain-C restatement of the reference's per-step hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  Only tests/, __graft_entry__.smoke() and the
 * cpu_baseline / --impl reference legs of bench.py load this code, as the
 * checker; the product (libmclg.so, mclg_run) never links or calls it.
 *
 * It follows the reference step for step, with its data structures: K, G and
 * the heat K/C are assembled per step into ragged sorted rows (at most 36 / 18
 * columns, global_variables.h:28-29) by element loops in element order, and
 * every solver is the reference's iteration verbatim:
 *   buoyancy_force          Buoyancy.c:3-22, Parallel.c:354-454
 *   viscosity               Viscosity.c:3-24
 *   visc_from_grain_size    Grain_size_evolution.c:3-152 (grain_damage=1, single-level meshes)
 *   K / F / G assembly      Build_matrix.c:42-381, 720-744
 *   citcom_solver (Uzawa)   Solver.c:14-249, initial_d_p :251-278
 *   Conj_Grad / jacobi      Solver.c:1589-1864, K_prod_d :360-386
 *   gauss_seidel            Solver.c:1866-1929
 *   multigrid / MG          Solver.c:668-768, get_residual :1291-1317, project_res
 *                           :770-832 and interp_error :1009-1143 (the local parts)
 *   G_prod_p / GT_prod_d    Solver.c:569-591, 645-666
 *   enforce_constrain_veq   Solver.c:1368-1482
 *   v_to_nodes, stress      Solver.c:1319-1366, Grain_size_evolution.c:154-213
 *   update_temperature      Update_temperature.c:3-133, 135-177, 241-594, 788-962, 1140-1354
 * The mesh (ien, node list, BC codes, hanging nodes) is an input: it comes
 * from the host mesh builder, which tests/test_mesh_golden.py pins bit-exact
 * against the reference's own arrays.  The dT/dt bookkeeping of
 * update_temperature is skipped: a stray ';' (Update_temperature.c:64) keeps
 * it out of every result.  With OpenMP and threads > 1 the dot products and
 * row loops run in parallel; with one thread every sum has the reference's order.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define VCOL 36
#define TCOL 18

typedef struct orc {
	int nel, nno, nh, gnox, gnoz, fl, neq, hneq, threads;
	const int *ienl, *elev, *gnode, *hni, *hci0, *hci1;
	const double *X, *vbcval, *tbcval;
	const char *vbc, *tbc;
	double dx[16], dz[16];
	double *dxh, *dzh, *jac, *area;
	int *id, *hid, *p2n_cnt, *p2n_el;
	double Ra, A, refT, lmj, Q, theta, accuracy, citcom_accu, vmin, vmax;
	int max_citcom, max_cg, precond, check_v_only, solver, zero_P, AMR, auto_acc;
	double N[4][4], dNdxi[4][4], dNdeta[4][4], dNdxi_c[4], dNdeta_c[4];
	double *T, *vis, *buoy, *V0, *V1, *stress, *d, *p, *F, *Kdiag;
	int *Kncol, *Kcol, *Gncol, *Gcol;
	double *Kval, *Gval;
	int *HKncol, *HKcol, *HCncol, *HCcol;
	double *HKval, *HCval, *HAval, *HF, *tau0, *tau1, *hd;
	double dt, model_time, res_m, res_c;
	int p_init, uzawa_cycles, cg_cycles, heat_cycles;
	/* grain-size rheology (grain_damage=1): the reference's static first-call flag
	 * and clock, the nodal grain size, and the clip of the viscosity it sets */
	int grain, gs_init;
	double gs_t, gs_lo, gs_hi, *gs;
	struct orc_mg *mg;   /* solver="mg": the coarser levels and the transfer maps */
} orc;

/* solver codes (G.solver, Input.c:10) */
enum { SOLVER_CG = 0, SOLVER_JC = 1, SOLVER_GS = 2, SOLVER_MG = 3 };

/* The multigrid hierarchy of solver="mg": lv[0] is mg_min_level, lv[nlev-1]
 * the owning (finest) level.  Maps are the reference's, equation-indexed:
 * itp_n[k] / itp_src[k] (k >= 1) from level k-1 to level k
 * (G.interp[lev].local_eq_n / local_eq), prj[k] (k < nlev-1) the equation of
 * level k+1 whose residual equation l of level k takes (G.project). */
typedef struct orc_mg {
	int nlev, cycles, fine_it, coarse_it;
	struct orc *lv[16];
	int *itp_n[16], *itp_src[16], *prj[16];
	double *err[16];     /* G.err[lev] */
} orc_mg;

static void shape_tables(orc *o)
{
	const double BETA = 1.0 / sqrt(3.0);
	const double pts[4][2] = {{-1.0, -1.0}, {-1.0, 1.0}, {1.0, 1.0}, {1.0, -1.0}};
	int d;
	for (d = 0; d < 4; d++) {
		double xi = pts[d][0] * BETA, eta = pts[d][1] * BETA;
		o->N[0][d] = 0.25 * (1 - xi) * (1 - eta);
		o->N[1][d] = 0.25 * (1 - xi) * (1 + eta);
		o->N[2][d] = 0.25 * (1 + xi) * (1 + eta);
		o->N[3][d] = 0.25 * (1 + xi) * (1 - eta);
		o->dNdxi[0][d] = 0.25 * (-1.0) * (1 - eta);
		o->dNdxi[1][d] = 0.25 * (-1.0) * (1 + eta);
		o->dNdxi[2][d] = 0.25 * (1.0) * (1 + eta);
		o->dNdxi[3][d] = 0.25 * (1.0) * (1 - eta);
		o->dNdeta[0][d] = 0.25 * (1.0 - xi) * (-1.0);
		o->dNdeta[1][d] = 0.25 * (1.0 - xi) * (1.0);
		o->dNdeta[2][d] = 0.25 * (1.0 + xi) * (1.0);
		o->dNdeta[3][d] = 0.25 * (1.0 + xi) * (-1.0);
	}
	o->dNdxi_c[0] = -0.25; o->dNdxi_c[1] = -0.25; o->dNdxi_c[2] = 0.25; o->dNdxi_c[3] = 0.25;
	o->dNdeta_c[0] = -0.25; o->dNdeta_c[1] = 0.25; o->dNdeta_c[2] = 0.25; o->dNdeta_c[3] = -0.25;
}

/* ---- vector helpers (global_v_prod / global_p_prod with nsh = 1) ---------- */
static double dot(const orc *o, const double *x, const double *y, int n)
{
	double s = 0.0;
	int i;
#pragma omp parallel for reduction(+ : s) num_threads(o->threads) if (o->threads > 1 && n > 4096)
	for (i = 0; i < n; i++)
		s += x[i] * y[i];
	return s;
}

static int row_find(const int *col, int n, int c)
{
	int k;
	for (k = 0; k < n; k++)
		if (col[k] == c)
			return k;
	return -1;
}

static void sort_row(int *col, double *val, int n)
{
	int swapped = 1, j;
	while (swapped) {
		swapped = 0;
		for (j = 0; j < n - 1; j++)
			if (col[j] > col[j + 1]) {
				int t = col[j]; double v = val[j];
				col[j] = col[j + 1]; val[j] = val[j + 1];
				col[j + 1] = t; val[j + 1] = v;
				swapped = 1;
			}
	}
}

/* ---- buoyancy (Buoyancy.c:3-22 with get_node_horiz_avg, Parallel.c:354-454) */
static double na(int a, double xi, double eta)
{
	switch (a) {
	case 0: return 0.25 * (1.0 - xi) * (1.0 - eta);
	case 1: return 0.25 * (1.0 - xi) * (1.0 + eta);
	case 2: return 0.25 * (1.0 + xi) * (1.0 + eta);
	default: return 0.25 * (1.0 + xi) * (1.0 - eta);
	}
}

static void buoyancy_force(orc *o)
{
	int i, e, a, k, gnoz = o->gnoz, gnox = o->gnox;
	double *avg = calloc((size_t)gnoz, sizeof(double));
	for (i = 0; i < o->nno; i++)
		o->buoy[i] = o->Ra * o->T[i];
	for (e = 0; e < o->nel; e++) {
		int idx[4], ix0, iz0, ix1, iz1, n0, n2;
		double xi, eta;
		for (a = 0; a < 4; a++)
			idx[a] = o->ienl[a * o->nel + e];
		n0 = o->gnode[idx[0]];
		n2 = o->gnode[idx[2]];
		ix0 = n0 / gnoz; iz0 = n0 - ix0 * gnoz;
		ix1 = n2 / gnoz; iz1 = n2 - ix1 * gnoz;
		for (i = ix0; i < ix1; i++) {
			xi = (2 * i - ix0 - ix1) / (ix1 - ix0);
			for (k = iz0; k < iz1; k++) {
				eta = (2 * k - iz0 - iz1) / (iz1 - iz0);
				for (a = 0; a < 4; a++)
					avg[k] += na(a, xi, eta) * o->buoy[idx[a]];
			}
		}
		if (iz1 == gnoz - 1) {
			k = iz1;
			for (i = ix0; i < ix1; i++) {
				xi = (2 * i - ix0 - ix1) / (ix1 - ix0);
				eta = 1.0;
				for (a = 0; a < 4; a++)
					avg[k] += na(a, xi, eta) * o->buoy[idx[a]];
			}
		}
		if (ix1 == gnox - 1) {
			xi = 1.0;
			for (k = iz0; k < iz1; k++) {
				eta = (2 * k - iz0 - iz1) / (iz1 - iz0);
				for (a = 0; a < 4; a++)
					avg[k] += na(a, xi, eta) * o->buoy[idx[a]];
			}
		}
		if (n2 == gnox * gnoz - 1)
			avg[gnoz - 1] += o->buoy[o->nno - 1];
	}
	for (i = 0; i < gnoz; i++)
		avg[i] = avg[i] / gnox;
	for (i = 0; i < o->nno; i++) {
		int n = o->gnode[i], ix = n / gnoz, iz = n - ix * gnoz;
		o->buoy[i] -= avg[iz];
	}
	free(avg);
}

static void viscosity(orc *o)
{
	int i;
	for (i = 0; i < o->nno; i++) {
		double v = exp(o->A * (o->refT - o->T[i]));
		if (o->X[o->nno + i] < 0.77)
			v *= o->lmj;
		if (o->vmax > 0.0)
			v = fmin(fmax(v, o->vmin), o->vmax);
		o->vis[i] = v;
	}
}

/* ---- grain-size rheology (Grain_size_evolution.c:3-152), one level ---------
 * Called after viscosity() when grain_damage=1.  The reference keeps a static
 * first-call flag and a static clock t (seconds) shared by every call:
 *   - the first call sets the grain size r = 1e-3 everywhere and returns;
 *   - every later call scales the nodal stress to Pa, then, while t is behind
 *     the model time in seconds, takes one explicit 100-year step over the
 *     nodes: those deeper than 200 km get stress 0 and keep their viscosity;
 *     the others update r by growth minus damage at the absolute temperature
 *     T*2500 + 273.5 + 0.3 K/km * depth and get the composite viscosity of
 *     dislocation and diffusion creep at their stress and new r, scaled by the
 *     reference viscosity and clipped to [lowest_vis, highest_vis].
 * On a single-level mesh the level visited is the finest one, so this is
 * exactly the reference's result.  Every expression keeps the reference's
 * operand order (the library is built without contraction). */
static double gs_creep_A(double A0, double Edisp, double T) { return A0 * exp(0.0 - Edisp / (8.3145 * T)); }
static double gs_creep_B(double B0, double Ediff, double T, double m)
{
	return pow(M_PI * 0.5, 0.0 - m) * B0 * exp(0.0 - Ediff / (8.3145 * T));
}
static double gs_growth(double G0, double EG, double T) { return G0 * exp(0.0 - EG / (8.3145 * T)); }
static double gs_damage_fraction(double f1, double f2, double T_M, double T_W, double T, double k)
{
	const double x = (pow(T_M, k) - pow(T, k)) / (pow(T_M, k) - pow(T_W, k));
	return f1 * pow(f2 / f1, x);
}

static void grain_size(orc *o)
{
	const double mu = 0.72, gamma = 1.0, q = 4.0, p = 2.0, T_M = 1500.0, T_W = 285.0, Tref = 2500.0;
	const double f1 = 1e-12, f2 = 1e-2, k = 2, n = 3.0, m = 3.0;
	const double A0 = 1.1e5 / pow(1e6, n), Edisp = 530.0 * 1e3;
	const double B0 = 13.6 * pow(1e-6, m) / 1e6, Ediff = 300 * 1e3;
	const double G0 = 2e4 * pow(1e-6, p), EG = 300 * 1e3;
	const double alpha = 1e-5, kappa = 1e-6, D = 2890e3, rho = 3300.0, g = 9.8, y2s = 3.1536e7;
	const double vis_ref = (rho * g * alpha * Tref * D * D * D) / (o->Ra * kappa);
	const double stress_scale = (vis_ref * kappa) / (D * D), time_scale = D * D / kappa;
	const double dt = 1e2 * y2s;
	int i;
	if (!o->gs_init) {
		for (i = 0; i < o->nno; i++)
			o->gs[i] = 1e-3;
		o->gs_init = 1;
		return;
	}
	for (i = 0; i < o->nno; i++)
		o->stress[i] *= stress_scale;
	while (o->gs_t < o->model_time * time_scale) {
		for (i = 0; i < o->nno; i++) {
			const double z = o->X[o->nno + i];
			double T, r, A, B, tau, GG, GI, fI, ratio, rF, psi, dr, v;
			if (2890 * (1.0 - z) > 200.0) {
				o->stress[i] = 0.0;
				continue;
			}
			T = o->T[i] * Tref + 273.5 + 2890.0 * (1.0 - z) * 0.3;
			r = o->gs[i];
			A = gs_creep_A(A0, Edisp, T);
			B = gs_creep_B(B0, Ediff, T, m);
			tau = o->stress[i];
			GG = gs_growth(G0, EG, T);
			GI = q / p * pow(1e-6, q - p) * GG / 250.0;
			fI = gs_damage_fraction(f1, f2, T_M, T_W, T, k);
			ratio = B / (A * pow(tau, n - 1));
			rF = pow(ratio, 1.0 / m);
			psi = 2 * A * pow(tau, n + 1) * (1.0 + pow(rF / r, m));
			dr = mu * GI / (q * pow(r, q - 1)) - fI * r * r * psi / (gamma * mu);
			o->gs[i] += dr * dt;
			v = 0.5 * tau / (A * pow(tau, n) + B * tau / pow(o->gs[i], m));
			v /= vis_ref;
			if (v < o->gs_lo)
				v = o->gs_lo;
			if (v > o->gs_hi)
				v = o->gs_hi;
			o->vis[i] = v;
		}
		o->gs_t += dt;
	}
}

static void viscosity_step(orc *o)
{
	viscosity(o);
	if (o->grain)
		grain_size(o);
}

/* ---- Stokes assembly (Build_matrix.c) -------------------------------------- */
static void element_K(const orc *o, int e, double K[8][8])
{
	int a, i, b, j, p, q, g, dd, node[4];
	double dzh = o->dzh[e], dxh = o->dxh[e];
	for (dd = 0; dd < 4; dd++)
		node[dd] = o->ienl[dd * o->nel + e];
	for (a = 0; a < 4; a++)
		for (i = 0; i < 2; i++) {
			p = 2 * a + i;
			for (b = a; b < 4; b++)
				for (j = 0; j < 2; j++) {
					q = 2 * b + j;
					K[p][q] = 0.0;
					for (g = 0; g < 4; g++) {
						double eta = 0.0, D00, D22;
						double dNa_dx, dNa_dz, dNb_dx, dNb_dz;
						for (dd = 0; dd < 4; dd++)
							eta += o->N[dd][g] * o->vis[node[dd]];
						D00 = 2.0 * eta;
						D22 = eta;
						dNa_dx = o->dNdxi[a][g] * dzh - o->dNdeta[a][g] * 0.0;
						dNa_dz = o->dNdeta[a][g] * dxh - o->dNdxi[a][g] * 0.0;
						dNb_dx = o->dNdxi[b][g] * dzh - o->dNdeta[b][g] * 0.0;
						dNb_dz = o->dNdeta[b][g] * dxh - o->dNdxi[b][g] * 0.0;
						if (i == 0 && j == 0)
							K[p][q] += ((dNa_dx * D00 + dNa_dz * 0.0) * dNb_dx + (dNa_dx * 0.0 + dNa_dz * D22) * dNb_dz);
						else if (i == 1 && j == 0)
							K[p][q] += ((dNa_dz * 0.0 + dNa_dx * 0.0) * dNb_dx + (dNa_dz * 0.0 + dNa_dx * D22) * dNb_dz);
						else if (i == 0 && j == 1)
							K[p][q] += ((dNa_dx * 0.0 + dNa_dz * 0.0) * dNb_dz + (dNa_dx * 0.0 + dNa_dz * D22) * dNb_dx);
						else
							K[p][q] += ((dNa_dz * D00 + dNa_dx * 0.0) * dNb_dz + (dNa_dz * 0.0 + dNa_dx * D22) * dNb_dx);
					}
					K[p][q] /= o->jac[e];
				}
		}
	for (p = 0; p < 8; p++)
		for (q = 0; q < 8; q++)
			K[q][p] = K[p][q];
}

static void element_F(const orc *o, int e, double F[8])
{
	int a, d, i, idx[4], nat[2];
	double force[4];
	for (a = 0; a < 4; a++)
		idx[a] = o->ienl[a * o->nel + e];
	for (d = 0; d < 4; d++) {
		force[d] = 0.0;
		for (a = 0; a < 4; a++)
			force[d] += o->N[a][d] * o->buoy[idx[a]];
	}
	for (i = 0; i < 2; i++) {
		nat[i] = 0;
		for (a = 0; a < 4; a++)
			if (o->vbc[i * o->nno + idx[a]] == 'S')
				nat[i] += a;
		if (nat[i] == 3)
			nat[i] = 1;
		else if (nat[i] == 1 || nat[i] == 5)
			nat[i] = 2;
		else if (nat[i] == 0 || nat[i] == 2)
			nat[i] = 0;
	}
	for (i = 0; i < 2; i++)
		for (a = 0; a < 4; a++) {
			int p = 2 * a + i;
			F[p] = 0.0;
			if (i == 1) {
				for (d = 0; d < 4; d++)
					F[p] += o->N[a][d] * force[d];
				F[p] *= o->jac[e];
			}
			if (nat[i] != 0) {
				double L = o->X[i * o->nno + idx[2]] - o->X[i * o->nno + idx[0]];
				F[p] += 0.5 * L * o->vbcval[i * o->nno + idx[a]];
			}
		}
}

static void element_G(const orc *o, int e, double g[8])
{
	int a, gs;
	for (a = 0; a < 4; a++) {
		g[2 * a] = 0.0;
		for (gs = 0; gs < 4; gs++)
			g[2 * a] -= o->dNdxi[a][gs] * o->dzh[e] - o->dNdeta[a][gs] * 0.0;
	}
	for (a = 0; a < 4; a++) {
		g[2 * a + 1] = 0.0;
		for (gs = 0; gs < 4; gs++)
			g[2 * a + 1] -= o->dNdeta[a][gs] * o->dxh[e] - o->dNdxi[a][gs] * 0.0;
	}
}

static void assemble_stokes(orc *o)
{
	int e, i, a, j, b, P, Q, k;
	double K[8][8], F[8], g[8];
	memset(o->F, 0, sizeof(double) * (size_t)o->neq);
	for (i = 0; i < o->neq; i++) {
		o->Kncol[i] = 0;
		o->Gncol[i] = 0;
		memset(&o->Kval[(size_t)i * VCOL], 0, VCOL * sizeof(double));
		memset(&o->Gval[(size_t)i * VCOL], 0, VCOL * sizeof(double));
	}
	for (e = 0; e < o->nel; e++) { /* K_matrix, Build_matrix.c:42-115 */
		element_K(o, e, K);
		for (i = 0; i < 2; i++)
			for (a = 0; a < 4; a++) {
				int An = o->ienl[a * o->nel + e];
				P = o->id[i * o->nno + An];
				for (j = 0; j < 2; j++)
					for (b = 0; b < 4; b++) {
						int Bn = o->ienl[b * o->nel + e];
						Q = o->id[j * o->nno + Bn];
						if (P >= 0 && Q >= 0) {
							int *col = &o->Kcol[(size_t)P * VCOL];
							double *val = &o->Kval[(size_t)P * VCOL];
							k = row_find(col, o->Kncol[P], Q);
							if (k >= 0)
								val[k] += K[2 * a + i][2 * b + j];
							else {
								col[o->Kncol[P]] = Q;
								val[o->Kncol[P]] += K[2 * a + i][2 * b + j];
								o->Kncol[P]++;
							}
						}
						if (P >= 0 && o->vbc[j * o->nno + Bn] == 'V')
							o->F[P] -= K[2 * a + i][2 * b + j] * o->vbcval[j * o->nno + Bn];
					}
			}
	}
	for (e = 0; e < o->nel; e++) { /* F_matrix, :117-140 */
		element_F(o, e, F);
		for (i = 0; i < 2; i++)
			for (a = 0; a < 4; a++) {
				P = o->id[i * o->nno + o->ienl[a * o->nel + e]];
				if (P >= 0)
					o->F[P] += F[2 * a + i];
			}
	}
	for (e = 0; e < o->nel; e++) { /* G_matrix, :142-190 */
		element_G(o, e, g);
		for (i = 0; i < 2; i++)
			for (a = 0; a < 4; a++) {
				P = o->id[i * o->nno + o->ienl[a * o->nel + e]];
				if (P < 0)
					continue;
				{
					int *col = &o->Gcol[(size_t)P * VCOL];
					double *val = &o->Gval[(size_t)P * VCOL];
					k = row_find(col, o->Gncol[P], e);
					if (k >= 0)
						val[k] += g[2 * a + i];
					else {
						col[o->Gncol[P]] = e;
						val[o->Gncol[P]] += g[2 * a + i];
						o->Gncol[P]++;
					}
				}
			}
	}
	for (i = 0; i < o->neq; i++) { /* row sort and Kdiag, :720-744 */
		sort_row(&o->Kcol[(size_t)i * VCOL], &o->Kval[(size_t)i * VCOL], o->Kncol[i]);
		k = row_find(&o->Kcol[(size_t)i * VCOL], o->Kncol[i], i);
		o->Kdiag[i] = o->Kval[(size_t)i * VCOL + k];
	}
}

/* ---- Stokes operators ------------------------------------------------------ */
static void K_prod(const orc *o, const double *x, double *y)
{
	int i;
#pragma omp parallel for num_threads(o->threads) if (o->threads > 1)
	for (i = 0; i < o->neq; i++) {
		const int *col = &o->Kcol[(size_t)i * VCOL];
		const double *val = &o->Kval[(size_t)i * VCOL];
		double s = 0.0;
		int j;
		for (j = 0; j < o->Kncol[i]; j++)
			s += val[j] * x[col[j]];
		y[i] = s;
	}
}

static void G_prod(const orc *o, const double *p, double *y)
{
	int i;
#pragma omp parallel for num_threads(o->threads) if (o->threads > 1)
	for (i = 0; i < o->neq; i++) {
		double s = 0.0;
		int j;
		for (j = 0; j < o->Gncol[i]; j++)
			s += o->Gval[(size_t)i * VCOL + j] * p[o->Gcol[(size_t)i * VCOL + j]];
		y[i] = s;
	}
}

static void GT_prod(const orc *o, const double *x, double *p)
{
	int i, j;
	memset(p, 0, sizeof(double) * (size_t)o->nel);
	for (i = 0; i < o->neq; i++)
		for (j = 0; j < o->Gncol[i]; j++)
			p[o->Gcol[(size_t)i * VCOL + j]] += o->Gval[(size_t)i * VCOL + j] * x[i];
}

static void constrain_v(const orc *o, double *x)
{
	int h, d, c;
	for (h = 0; h < o->nh; h++) {
		double t[2];
		int ci[2] = {o->hci0[h], o->hci1[h]};
		for (d = 0; d < 2; d++) {
			t[d] = 0.0;
			for (c = 0; c < 2; c++) {
				int eq = o->id[d * o->nno + ci[c]];
				t[d] += eq != -1 ? x[eq] : o->vbcval[d * o->nno + ci[c]];
			}
			t[d] *= 0.5;
		}
		for (d = 0; d < 2; d++) {
			int eq = o->id[d * o->nno + o->hni[h]];
			if (eq >= 0)
				x[eq] = t[d];
		}
	}
}

static int conj_grad(orc *o, const double *b, double *x, double accu, int max_cycle)
{
	int n = o->neq, i, cycle = 0;
	double *r = malloc(sizeof(double) * (size_t)n), *s = malloc(sizeof(double) * (size_t)n);
	double *dd = malloc(sizeof(double) * (size_t)n), *q = malloc(sizeof(double) * (size_t)n);
	double delta_new, delta0, delta_old, alpha, beta, res;
	const int pc = o->precond;
	K_prod(o, x, r);
	for (i = 0; i < n; i++) {
		r[i] = b[i] - r[i];
		dd[i] = pc ? r[i] / o->Kdiag[i] : r[i];
	}
	delta_new = dot(o, r, dd, n);
	delta0 = delta_new;
	/* element-wise loops give the same result on any thread count; only the
	 * dot products (dot) change their summation order with threads > 1 */
	while (cycle < max_cycle && delta_new > accu * delta0) {
		const int par = o->threads > 1 && n > 4096;
		K_prod(o, dd, q);
		alpha = delta_new / dot(o, dd, q, n);
#pragma omp parallel for num_threads(o->threads) if (par)
		for (i = 0; i < n; i++)
			x[i] += alpha * dd[i];
		constrain_v(o, x);
		if (cycle % 50 == 0) {
			K_prod(o, x, r);
#pragma omp parallel for num_threads(o->threads) if (par)
			for (i = 0; i < n; i++)
				r[i] = b[i] - r[i];
		} else {
#pragma omp parallel for num_threads(o->threads) if (par)
			for (i = 0; i < n; i++)
				r[i] -= alpha * q[i];
		}
#pragma omp parallel for num_threads(o->threads) if (par)
		for (i = 0; i < n; i++)
			s[i] = pc ? r[i] / o->Kdiag[i] : r[i];
		delta_old = delta_new;
		delta_new = dot(o, r, s, n);
		beta = delta_new / delta_old;
#pragma omp parallel for num_threads(o->threads) if (par)
		for (i = 0; i < n; i++)
			dd[i] = s[i] + beta * dd[i];
		cycle++;
		res = 0.0;
#pragma omp parallel for reduction(max : res) num_threads(o->threads) if (par)
		for (i = 0; i < n; i++)
			if (fabs(alpha * r[i]) > res)
				res = fabs(alpha * r[i]);
		if (res < accu)
			break;
	}
	free(r); free(s); free(dd); free(q);
	return cycle;
}

static int jacobi(orc *o, const double *b, double *x, double accu, int max_cycle)
{
	int n = o->neq, i, cycle = 0;
	double *xt = malloc(sizeof(double) * (size_t)n);
	while (cycle < max_cycle) {
		double diff = 0.0;
		memcpy(xt, x, sizeof(double) * (size_t)n);
		for (i = 0; i < n; i++) {
			double prod = 0.0, diag = 1.0;
			int j;
			for (j = 0; j < o->Kncol[i]; j++) {
				int c = o->Kcol[(size_t)i * VCOL + j];
				if (c != i)
					prod += o->Kval[(size_t)i * VCOL + j] * xt[c];
				else
					diag = o->Kval[(size_t)i * VCOL + j];
			}
			x[i] = (b[i] - prod) / diag;
		}
		cycle++;
		for (i = 0; i < n; i++)
			if (fabs(x[i] - xt[i]) > diff)
				diff = fabs(x[i] - xt[i]);
		if (diff < accu)
			break;
	}
	free(xt);
	return cycle;
}

/* gauss_seidel, Solver.c:1866-1929: rows in equation order, each from the
 * newest x, until the largest change is below accu */
static int gauss_seidel(const orc *o, const double *b, double *x, double accu, int max_cycle)
{
	int n = o->neq, i, cycle = 0;
	double *xt = malloc(sizeof(double) * (size_t)(n + 1)), *prod = malloc(sizeof(double) * (size_t)(n + 1));
	while (cycle < max_cycle) {
		double diff = 0.0;
		for (i = 0; i < n; i++) {
			xt[i] = x[i];
			prod[i] = 0.0;
		}
		for (i = 0; i < n; i++) {
			double diag = 1.0;
			int j;
			for (j = 0; j < o->Kncol[i]; j++) {
				int c = o->Kcol[(size_t)i * VCOL + j];
				if (c != i)
					prod[i] += o->Kval[(size_t)i * VCOL + j] * x[c];
				else
					diag = o->Kval[(size_t)i * VCOL + j];
			}
			x[i] = (b[i] - prod[i]) / diag;
		}
		cycle++;
		for (i = 0; i < n; i++)
			if (fabs(x[i] - xt[i]) > diff)
				diff = fabs(x[i] - xt[i]);
		if (diff < accu)
			break;
	}
	free(xt);
	free(prod);
	return cycle;
}

/* get_residual, Solver.c:1291-1317: res = b - K x, column by column */
static void get_residual(const orc *o, const double *b, const double *x, double *res)
{
	int i, j;
	for (i = 0; i < o->neq; i++)
		res[i] = b[i];
	for (i = 0; i < o->neq; i++)
		for (j = 0; j < o->Kncol[i]; j++)
			res[i] -= o->Kval[(size_t)i * VCOL + j] * x[o->Kcol[(size_t)i * VCOL + j]];
}

/* MG, Solver.c:715-768, at hierarchy index k (> 0).  Below the top, x is
 * err[k] itself, so interp_error overwrites it before x += err[k] doubles it,
 * as in the reference. */
static void mg_level(orc_mg *g, int k, const double *b, double *x, double accu)
{
	orc *u = g->lv[k], *l = g->lv[k - 1];
	double *res_u = malloc(sizeof(double) * (size_t)(u->neq + 1));
	double *res_l = calloc((size_t)l->neq + 1, sizeof(double));
	double *eu = g->err[k], *el = g->err[k - 1];
	int i, j;
	gauss_seidel(u, b, x, accu, g->fine_it);
	get_residual(u, b, x, res_u);
	for (i = 0; i < l->neq; i++) /* project_res, :770-783 */
		if (g->prj[k - 1][i] >= 0)
			res_l[i] = res_u[g->prj[k - 1][i]];
	if (k - 1 == 0)
		gauss_seidel(l, res_l, el, accu, 1000);
	else
		mg_level(g, k - 1, res_l, el, accu);
	for (i = 0; i < u->neq; i++) { /* interp_error, :1029-1046 */
		const int n = g->itp_n[k][i];
		if (n <= 0)
			continue;
		eu[i] = 0.0;
		for (j = 0; j < n; j++) {
			const int s = g->itp_src[k][(size_t)j * u->neq + i];
			if (s != -1)
				eu[i] += el[s];
		}
		eu[i] /= n;
	}
	for (i = 0; i < u->neq; i++)
		x[i] += eu[i];
	gauss_seidel(u, b, x, accu, g->coarse_it);
	free(res_u);
	free(res_l);
}

/* multigrid, Solver.c:668-713 */
static int multigrid(orc *o, const double *b, double *x, double accu)
{
	orc_mg *g = o->mg;
	const int top = g->nlev - 1;
	int k, i, cycle = 0, conv = 0;
	double *xt = malloc(sizeof(double) * (size_t)(o->neq + 1));
	for (k = 0; k < g->nlev; k++)
		memset(g->err[k], 0, sizeof(double) * (size_t)g->lv[k]->neq);
	while (!conv && cycle < g->cycles) {
		double diff = 0.0;
		memcpy(xt, x, sizeof(double) * (size_t)o->neq);
		mg_level(g, top, b, x, accu);
		for (i = 0; i < o->neq; i++) /* check_convergency, :1267-1289 */
			if (fabs(x[i] - xt[i]) > diff)
				diff = fabs(x[i] - xt[i]);
		conv = diff < accu;
		cycle++;
	}
	free(xt);
	return cycle;
}

static int inner(orc *o, const double *b, double *x, double accu)
{
	switch (o->solver) {
	case SOLVER_JC: return jacobi(o, b, x, accu, 1000);
	case SOLVER_GS: return gauss_seidel(o, b, x, accu, 1000);
	case SOLVER_MG: return multigrid(o, b, x, accu);
	default: return conj_grad(o, b, x, accu, o->max_cg);
	}
}

/* citcom_solver, Solver.c:14-249 */
static void citcom_solver(orc *o)
{
	int nel = o->nel, neq = o->neq, i, cycle = 0;
	double *r0 = calloc(nel, sizeof(double)), *r1 = calloc(nel, sizeof(double)), *r2 = calloc(nel, sizeof(double));
	double *z0 = calloc(nel, sizeof(double)), *z1 = calloc(nel, sizeof(double)), *s1 = calloc(nel, sizeof(double));
	double *s2 = calloc(nel, sizeof(double)), *Ah = calloc(neq > nel ? neq : nel, sizeof(double));
	double *u1 = calloc(neq, sizeof(double)), *bab = calloc(nel, sizeof(double)), *sh;
	double dv = 1.0, dp = 1.0, accu = o->accuracy;
	int cg_total;
	if (o->auto_acc)
		accu = o->citcom_accu * sqrt(dot(o, o->F, o->F, neq) / neq);
	for (i = 0; i < neq; i++) {
		int j;
		for (j = 0; j < o->Gncol[i]; j++) {
			double g = o->Gval[(size_t)i * VCOL + j];
			bab[o->Gcol[(size_t)i * VCOL + j]] += g * g / o->Kdiag[i];
		}
	}
	K_prod(o, o->d, u1);
	G_prod(o, o->p, Ah);
	for (i = 0; i < neq; i++)
		Ah[i] = o->F[i] - Ah[i] - u1[i];
	cg_total = inner(o, Ah, u1, accu);
	for (i = 0; i < neq; i++)
		o->d[i] += u1[i];
	GT_prod(o, o->d, r1);
	while ((dv > o->citcom_accu || (dp > o->citcom_accu && o->check_v_only == 0)) && cycle < o->max_citcom) {
		double r1z1, r0z0, delta, alpha, t1, t2, t3, t4;
		for (i = 0; i < nel; i++)
			z1[i] = bab[i] * r1[i];
		r1z1 = dot(o, r1, z1, nel);
		if (cycle == 0)
			memcpy(s2, z1, sizeof(double) * (size_t)nel);
		else {
			r0z0 = dot(o, r0, z0, nel);
			if (!(r0z0 > 0.0))
				break;
			delta = r1z1 / r0z0;
			for (i = 0; i < nel; i++)
				s2[i] = z1[i] + delta * s1[i];
		}
		G_prod(o, s2, Ah);
		memset(u1, 0, sizeof(double) * (size_t)neq);
		cg_total += inner(o, Ah, u1, accu);
		GT_prod(o, u1, Ah);
		alpha = r1z1 / dot(o, s2, Ah, nel);
		for (i = 0; i < nel; i++) {
			r2[i] = r1[i] - alpha * Ah[i];
			o->p[i] += alpha * s2[i];
		}
		for (i = 0; i < neq; i++)
			o->d[i] -= alpha * u1[i];
		t1 = dot(o, s2, s2, nel);
		t2 = dot(o, o->p, o->p, nel);
		t3 = dot(o, u1, u1, neq);
		t4 = dot(o, o->d, o->d, neq);
		dp = alpha * sqrt(t1 / (1.0e-32 + t2));
		dv = alpha * sqrt(t3 / (1.0e-32 + t4));
		cycle++;
		sh = s1; s1 = s2; s2 = sh;
		sh = r0; r0 = r1; r1 = r2; r2 = sh;
		sh = z0; z0 = z1; z1 = sh;
		if (!isfinite(dv) || !isfinite(dp))
			break;
	}
	o->uzawa_cycles = cycle;
	o->cg_cycles = cg_total;
	{ /* true residual |[F - K d - G p; G^T d]| / |F| */
		double *kd = calloc(neq, sizeof(double)), *gp = calloc(neq, sizeof(double)), *dg = calloc(nel, sizeof(double));
		double rm = 0.0, rc = 0.0, f = 0.0;
		K_prod(o, o->d, kd);
		G_prod(o, o->p, gp);
		GT_prod(o, o->d, dg);
		for (i = 0; i < neq; i++) {
			double r = o->F[i] - kd[i] - gp[i];
			rm += r * r;
			f += o->F[i] * o->F[i];
		}
		for (i = 0; i < nel; i++)
			rc += dg[i] * dg[i];
		o->res_m = sqrt(rm) / sqrt(f);
		o->res_c = sqrt(rc) / sqrt(f);
		free(kd); free(gp); free(dg);
	}
	free(r0); free(r1); free(r2); free(z0); free(z1); free(s1); free(s2); free(Ah); free(u1); free(bab);
}

static void solve_velocity_pressure(orc *o)
{
	int i, d, e, a;
	double *se = malloc(sizeof(double) * (size_t)o->nel);
	memset(o->d, 0, sizeof(double) * (size_t)o->neq);  /* initial_d_p */
	if (!(o->p_init && o->AMR == 0 && o->zero_P == 0))
		memset(o->p, 0, sizeof(double) * (size_t)o->nel);
	o->p_init = 1;
	citcom_solver(o);
	for (i = 0; i < o->nno; i++) /* v_to_nodes */
		for (d = 0; d < 2; d++) {
			int eq = o->id[d * o->nno + i];
			double v = eq >= 0 ? o->d[eq] : o->vbcval[d * o->nno + i];
			if (d == 0) o->V0[i] = v; else o->V1[i] = v;
		}
	for (e = 0; e < o->nel; e++) { /* compute_stress */
		double eta = 0.0, u11 = 0.0, u22 = 0.0, u12 = 0.0, sr;
		for (a = 0; a < 4; a++)
			eta += 0.25 * o->vis[o->ienl[a * o->nel + e]];
		for (a = 0; a < 4; a++) {
			int n = o->ienl[a * o->nel + e];
			double dNa_dx = o->dNdxi_c[a] * o->dzh[e] - o->dNdeta_c[a] * 0.0;
			double dNa_dz = o->dNdeta_c[a] * o->dxh[e] - o->dNdxi_c[a] * 0.0;
			u11 += dNa_dx * o->V0[n];
			u22 += dNa_dz * o->V1[n];
			u12 += dNa_dz * o->V0[n];
		}
		u11 /= o->jac[e]; u22 /= o->jac[e]; u12 /= o->jac[e];
		sr = u11 * u11 + u22 * u22 + u12 * u12 * 2.0;
		sr = sqrt(0.5 * sr);
		se[e] = 2.0 * eta * sr;
	}
	for (i = 0; i < o->nno; i++) { /* p_to_nodes */
		double s = 0.0, ta = 0.0;
		int k;
		for (k = 0; k < o->p2n_cnt[i]; k++) {
			int el = o->p2n_el[k * o->nno + i];
			s += o->area[el] * se[el];
			ta += o->area[el];
		}
		o->stress[i] = s / ta;
	}
	free(se);
}

/* ---- temperature (Update_temperature.c) ------------------------------------ */
static void tau_all(orc *o)
{
	int e, a, d;
	for (e = 0; e < o->nel; e++) {
		int lv = o->elev[e];
		double L[2] = {o->dx[lv], o->dz[lv]}, u[2], xi[2], us, kh;
		for (d = 0; d < 2; d++) {
			double alpha;
			u[d] = 0.0;
			for (a = 0; a < 4; a++) {
				int n = o->ienl[a * o->nel + e];
				u[d] += 0.25 * (d == 0 ? o->V0[n] : o->V1[n]);
			}
			alpha = 0.5 * u[d] * L[d] / 1.0;
			xi[d] = fabs(alpha) < o->accuracy ? 0.0 : cosh(alpha) / sinh(alpha) - 1.0 / alpha;
		}
		us = u[0] * u[0] + u[1] * u[1];
		kh = (xi[0] * u[0] * L[0] + xi[1] * u[1] * L[1]) * 0.5;
		o->tau0[e] = kh * u[0] / us;
		o->tau1[e] = kh * u[1] / us;
	}
}

static void heat_element(const orc *o, int e, double k[4][4], double c[4][4], double f[4])
{
	int a, b, g, idx[4], nat = 0;
	double u1 = 0.0, u2 = 0.0, dzh = o->dzh[e], dxh = o->dxh[e], t0 = o->tau0[e], t1 = o->tau1[e];
	for (a = 0; a < 4; a++) {
		idx[a] = o->ienl[a * o->nel + e];
		u1 += o->V0[idx[a]] * 0.25;
		u2 += o->V1[idx[a]] * 0.25;
	}
	for (a = 0; a < 4; a++)
		for (b = 0; b < 4; b++) {
			k[a][b] = 0.0;
			c[a][b] = 0.0;
			for (g = 0; g < 4; g++) {
				double dNa_dx = o->dNdxi[a][g] * dzh - o->dNdeta[a][g] * 0.0;
				double dNa_dz = o->dNdeta[a][g] * dxh - o->dNdxi[a][g] * 0.0;
				double dNb_dx = o->dNdxi[b][g] * dzh - o->dNdeta[b][g] * 0.0;
				double dNb_dz = o->dNdeta[b][g] * dxh - o->dNdxi[b][g] * 0.0;
				double na_hat = t0 * dNa_dx + t1 * dNa_dz;
				double tmp1 = u1 * o->N[a][g] * dNb_dx + u2 * o->N[a][g] * dNb_dz;
				double tmp2 = u1 * na_hat * dNb_dx + u2 * na_hat * dNb_dz;
				double tmp3 = dNa_dx * 1.0 * dNb_dx + dNa_dx * 0.0 * dNb_dz + dNa_dz * 0.0 * dNb_dx + dNa_dz * 1.0 * dNb_dz;
				k[a][b] += tmp1 + (tmp2 + tmp3) / o->jac[e];
				c[a][b] += (o->N[a][g] + na_hat) * o->N[b][g];
			}
			c[a][b] *= o->jac[e];
		}
	for (a = 0; a < 4; a++)
		if (o->tbc[idx[a]] == 'F')
			nat += a;
	if (nat == 3) nat = 1;
	else if (nat == 1 || nat == 5) nat = 2;
	else if (nat == 0 || nat == 2) nat = 0;
	for (a = 0; a < 4; a++) {
		f[a] = 0.0;
		for (g = 0; g < 4; g++) {
			double dNa_dx = o->dNdxi[a][g] * dzh - o->dNdeta[a][g] * 0.0;
			double dNa_dz = o->dNdeta[a][g] * dxh - o->dNdxi[a][g] * 0.0;
			double na_hat = t0 * dNa_dx + t1 * dNa_dz;
			f[a] += (o->N[a][g] + na_hat) * o->Q;
		}
		f[a] *= o->jac[e];
		if (nat != 0)
			f[a] -= 0.5 * o->dz[o->elev[e]] * o->tbcval[idx[a]];
	}
}

static void assemble_heat(orc *o)
{
	int e, a, b, i, k;
	double kk[4][4], cc[4][4], ff[4];
	for (i = 0; i < o->hneq; i++) {
		o->HKncol[i] = o->HCncol[i] = 0;
		memset(&o->HKval[(size_t)i * TCOL], 0, TCOL * sizeof(double));
		memset(&o->HCval[(size_t)i * TCOL], 0, TCOL * sizeof(double));
		o->HF[i] = 0.0;
	}
	for (e = 0; e < o->nel; e++) { /* K_matrix_heat + lifting; C rows */
		heat_element(o, e, kk, cc, ff);
		for (a = 0; a < 4; a++) {
			int P = o->hid[o->ienl[a * o->nel + e]];
			for (b = 0; b < 4; b++) {
				int Bn = o->ienl[b * o->nel + e], Q = o->hid[Bn];
				if (P >= 0 && Q >= 0) {
					int *col = &o->HKcol[(size_t)P * TCOL];
					double *val = &o->HKval[(size_t)P * TCOL];
					k = row_find(col, o->HKncol[P], Q);
					if (k >= 0)
						val[k] += kk[a][b];
					else {
						col[o->HKncol[P]] = Q;
						val[o->HKncol[P]] += kk[a][b];
						o->HKncol[P]++;
					}
					col = &o->HCcol[(size_t)P * TCOL];
					val = &o->HCval[(size_t)P * TCOL];
					k = row_find(col, o->HCncol[P], Q);
					if (k >= 0)
						val[k] += cc[a][b];
					else {
						col[o->HCncol[P]] = Q;
						val[o->HCncol[P]] += cc[a][b];
						o->HCncol[P]++;
					}
				}
				if (P >= 0 && o->tbc[Bn] == 'T')
					o->HF[P] -= kk[a][b] * o->tbcval[Bn];
			}
		}
	}
	for (e = 0; e < o->nel; e++) { /* F_matrix_heat */
		heat_element(o, e, kk, cc, ff);
		for (a = 0; a < 4; a++) {
			int P = o->hid[o->ienl[a * o->nel + e]];
			if (P >= 0)
				o->HF[P] += ff[a];
		}
	}
	for (i = 0; i < o->hneq; i++) {
		sort_row(&o->HKcol[(size_t)i * TCOL], &o->HKval[(size_t)i * TCOL], o->HKncol[i]);
		sort_row(&o->HCcol[(size_t)i * TCOL], &o->HCval[(size_t)i * TCOL], o->HCncol[i]);
	}
}

static double advection_dt(const orc *o)
{
	int e, a, lv = 0;
	double diff = 1e10, dt = 1e10;
	for (e = 0; e < o->nel; e++) {
		double L0, L1;
		lv = o->elev[e];
		L0 = o->dx[lv] * o->dx[lv];
		L1 = o->dz[lv] * o->dz[lv];
		if (diff > L0) diff = L0;
		if (diff > L1) diff = L1;
	}
	for (e = 0; e < o->nel; e++) {
		double u1 = 0.0, u2 = 0.0, u, step;
		for (a = 0; a < 4; a++) {
			int n = o->ienl[a * o->nel + e];
			u1 += 0.25 * o->V0[n];
			u2 += 0.25 * o->V1[n];
		}
		u = fabs(u1) / o->dx[lv] + fabs(u2) / o->dz[lv];
		step = 0.5 / u;
		dt = (step < dt) ? step : dt;
	}
	return (dt < diff) ? dt : diff;
}


static void heat_prod(const orc *o, const double *val, const int *col, const int *ncol, int width,
                      const double *x, double *y)
{
	int i;
#pragma omp parallel for num_threads(o->threads) if (o->threads > 1)
	for (i = 0; i < o->hneq; i++) {
		double s = 0.0;
		int j;
		for (j = 0; j < ncol[i]; j++)
			s += val[(size_t)i * width + j] * x[col[(size_t)i * width + j]];
		y[i] = s;
	}
}

static void constrain_T(const orc *o, double *x)
{
	int h, c;
	for (h = 0; h < o->nh; h++) {
		int ci[2] = {o->hci0[h], o->hci1[h]}, eq;
		double t = 0.0;
		for (c = 0; c < 2; c++) {
			eq = o->hid[ci[c]];
			t += eq != -1 ? x[eq] : o->tbcval[ci[c]];
		}
		t *= 0.5;
		eq = o->hid[o->hni[h]];
		if (eq >= 0)
			x[eq] = t;
	}
}

static int conj_grad_heat(orc *o, const double *A, const double *b, double *x, double accu, int max_cycle)
{
	int n = o->hneq, i, cycle = 0;
	double *r = malloc(sizeof(double) * (size_t)n), *s = malloc(sizeof(double) * (size_t)n);
	double *dd = malloc(sizeof(double) * (size_t)n), *q = malloc(sizeof(double) * (size_t)n);
	double *dg = malloc(sizeof(double) * (size_t)n);
	double delta_new, delta0, delta_old, alpha, beta, res;
	const int pc = o->precond;
	for (i = 0; i < n; i++) {
		int k = row_find(&o->HKcol[(size_t)i * TCOL], o->HKncol[i], i);
		dg[i] = A[(size_t)i * TCOL + k];
	}
	heat_prod(o, A, o->HKcol, o->HKncol, TCOL, x, r);
	for (i = 0; i < n; i++) {
		r[i] = b[i] - r[i];
		dd[i] = pc ? r[i] / dg[i] : r[i];
	}
	delta_new = dot(o, r, dd, n);
	delta0 = delta_new;
	while (cycle < max_cycle && delta_new > accu * delta0) {
		heat_prod(o, A, o->HKcol, o->HKncol, TCOL, dd, q);
		alpha = delta_new / dot(o, dd, q, n);
		for (i = 0; i < n; i++)
			x[i] += alpha * dd[i];
		constrain_T(o, x);
		if (cycle % 50 == 0) {
			heat_prod(o, A, o->HKcol, o->HKncol, TCOL, x, r);
			for (i = 0; i < n; i++)
				r[i] = b[i] - r[i];
		} else
			for (i = 0; i < n; i++)
				r[i] -= alpha * q[i];
		for (i = 0; i < n; i++)
			s[i] = pc ? r[i] / dg[i] : r[i];
		delta_old = delta_new;
		delta_new = dot(o, r, s, n);
		beta = delta_new / delta_old;
		for (i = 0; i < n; i++)
			dd[i] = s[i] + beta * dd[i];
		cycle++;
		res = 0.0;
		for (i = 0; i < n; i++)
			if (fabs(alpha * r[i]) > res)
				res = fabs(alpha * r[i]);
		if (res < accu && (pc || cycle > 10))
			break;
	}
	free(r); free(s); free(dd); free(q); free(dg);
	return cycle;
}

static void update_temperature(orc *o)
{
	int i, n = o->hneq;
	double *B = malloc(sizeof(double) * (size_t)(n + 1)), *CT = malloc(sizeof(double) * (size_t)(n + 1));
	double tdt;
	tau_all(o);
	assemble_heat(o);
	for (i = 0; i < o->nno; i++) /* heat.d: T on the free nodes */
		if (o->hid[i] >= 0)
			o->hd[o->hid[i]] = o->T[i];
	o->dt = advection_dt(o) * 0.75;
	o->model_time += o->dt;
	tdt = o->theta * o->dt;
	heat_prod(o, o->HCval, o->HCcol, o->HCncol, TCOL, o->hd, CT);
	for (i = 0; i < n; i++)
		B[i] = o->HF[i] + CT[i] / tdt;
	for (i = 0; i < n; i++) {
		int j;
		for (j = 0; j < o->HKncol[i]; j++)
			o->HAval[(size_t)i * TCOL + j] = o->HCval[(size_t)i * TCOL + j] / tdt + o->HKval[(size_t)i * TCOL + j];
	}
	o->heat_cycles = conj_grad_heat(o, o->HAval, B, o->hd, 1e-3, 1000);
	for (i = 0; i < o->nno; i++)
		o->T[i] = o->hid[i] >= 0 ? o->hd[o->hid[i]] : o->tbcval[i];
	free(B);
	free(CT);
}

/* ---- exported API (ctypes) -------------------------------------------------- */
orc *orc_new(int nel, int nno, int gnox, int gnoz, int fine_level, const int *ienl, const int *elev,
             const int *gnode, const double *X, const char *vbc, const double *vbcval, const char *tbc,
             const double *tbcval, int nh, const int *hni, const int *hci0, const int *hci1,
             const double *dx, const double *dz, const double *dparam, const int *iparam)
{
	orc *o = calloc(1, sizeof(orc));
	int e, a, A, d, P;
	o->nel = nel; o->nno = nno; o->gnox = gnox; o->gnoz = gnoz; o->fl = fine_level;
	o->ienl = ienl; o->elev = elev; o->gnode = gnode; o->X = X; o->vbc = vbc; o->vbcval = vbcval;
	o->tbc = tbc; o->tbcval = tbcval; o->nh = nh; o->hni = hni; o->hci0 = hci0; o->hci1 = hci1;
	memcpy(o->dx, dx, sizeof o->dx);
	memcpy(o->dz, dz, sizeof o->dz);
	o->Ra = dparam[0]; o->A = dparam[1]; o->refT = dparam[2]; o->lmj = dparam[3]; o->Q = dparam[4];
	o->theta = dparam[5]; o->accuracy = dparam[6]; o->citcom_accu = dparam[7]; o->vmin = dparam[8];
	o->vmax = dparam[9];
	o->gs_lo = dparam[10]; o->gs_hi = dparam[11];
	o->max_citcom = iparam[0]; o->max_cg = iparam[1]; o->precond = iparam[2]; o->check_v_only = iparam[3];
	o->solver = iparam[4]; o->zero_P = iparam[5]; o->AMR = iparam[6]; o->auto_acc = iparam[7];
	o->threads = iparam[8] > 0 ? iparam[8] : 1;
	o->grain = iparam[9];
	shape_tables(o);
	o->dxh = malloc(sizeof(double) * nel); o->dzh = malloc(sizeof(double) * nel);
	o->jac = malloc(sizeof(double) * nel); o->area = malloc(sizeof(double) * nel);
	for (e = 0; e < nel; e++) {
		int n0 = ienl[e], n2 = ienl[2 * nel + e];
		o->dxh[e] = 0.5 * o->dx[elev[e]];
		o->dzh[e] = 0.5 * o->dz[elev[e]];
		o->jac[e] = o->dxh[e] * o->dzh[e] - 0.0 * 0.0;
		o->area[e] = (X[n2] - X[n0]) * (X[nno + n2] - X[nno + n0]);
	}
	o->id = malloc(sizeof(int) * 2 * nno);
	o->hid = malloc(sizeof(int) * nno);
	for (P = 0, A = 0; A < nno; A++)
		for (d = 0; d < 2; d++)
			o->id[d * nno + A] = vbc[d * nno + A] == 'V' ? -1 : P++;
	o->neq = P;
	for (P = 0, A = 0; A < nno; A++)
		o->hid[A] = tbc[A] == 'T' ? -1 : P++;
	o->hneq = P;
	o->p2n_cnt = calloc(nno, sizeof(int));
	o->p2n_el = malloc(sizeof(int) * 4 * nno);
	for (e = 0; e < nel; e++)
		for (a = 0; a < 4; a++) {
			int n = ienl[a * nel + e];
			o->p2n_el[o->p2n_cnt[n]++ * nno + n] = e;
		}
	o->T = calloc(nno, sizeof(double)); o->vis = calloc(nno, sizeof(double)); o->buoy = calloc(nno, sizeof(double));
	o->V0 = calloc(nno, sizeof(double)); o->V1 = calloc(nno, sizeof(double)); o->stress = calloc(nno, sizeof(double));
	o->gs = calloc(nno, sizeof(double));
	o->d = calloc(o->neq + 1, sizeof(double)); o->p = calloc(nel, sizeof(double));
	o->F = calloc(o->neq + 1, sizeof(double)); o->Kdiag = calloc(o->neq + 1, sizeof(double));
	o->Kncol = calloc(o->neq + 1, sizeof(int)); o->Gncol = calloc(o->neq + 1, sizeof(int));
	o->Kcol = calloc((size_t)(o->neq + 1) * VCOL, sizeof(int)); o->Gcol = calloc((size_t)(o->neq + 1) * VCOL, sizeof(int));
	o->Kval = calloc((size_t)(o->neq + 1) * VCOL, sizeof(double)); o->Gval = calloc((size_t)(o->neq + 1) * VCOL, sizeof(double));
	o->HKncol = calloc(o->hneq + 1, sizeof(int)); o->HCncol = calloc(o->hneq + 1, sizeof(int));
	o->HKcol = calloc((size_t)(o->hneq + 1) * TCOL, sizeof(int)); o->HCcol = calloc((size_t)(o->hneq + 1) * TCOL, sizeof(int));
	o->HKval = calloc((size_t)(o->hneq + 1) * TCOL, sizeof(double)); o->HCval = calloc((size_t)(o->hneq + 1) * TCOL, sizeof(double));
	o->HF = calloc(o->hneq + 1, sizeof(double)); o->hd = calloc(o->hneq + 1, sizeof(double));
	o->tau0 = calloc(nel, sizeof(double)); o->tau1 = calloc(nel, sizeof(double));
	o->HAval = calloc((size_t)(o->hneq + 1) * TCOL, sizeof(double));
	return o;
}

void orc_free(orc *o)
{
	if (!o)
		return;
	if (o->mg) {
		int k;
		for (k = 0; k < o->mg->nlev; k++) {
			free(o->mg->err[k]); free(o->mg->itp_n[k]); free(o->mg->itp_src[k]); free(o->mg->prj[k]);
		}
		free(o->mg);
	}
	free(o->dxh); free(o->dzh); free(o->jac); free(o->area); free(o->id); free(o->hid); free(o->p2n_cnt);
	free(o->p2n_el); free(o->T); free(o->vis); free(o->buoy); free(o->V0); free(o->V1); free(o->stress);
	free(o->gs);
	free(o->d); free(o->p); free(o->F); free(o->Kdiag); free(o->Kncol); free(o->Gncol); free(o->Kcol);
	free(o->Gcol); free(o->Kval); free(o->Gval); free(o->HKncol); free(o->HCncol); free(o->HKcol);
	free(o->HCcol); free(o->HKval); free(o->HCval); free(o->HAval); free(o->HF); free(o->hd); free(o->tau0); free(o->tau1);
	free(o);
}

/* solver="mg": attach the coarser levels (lv[nlev-1] == top) and the maps;
 * the maps are copied. */
int orc_mg_attach(orc *top, int nlev, orc **lv, int **itp_n, int **itp_src, int **prj, int cycles, int fine_it,
                  int coarse_it)
{
	orc_mg *g;
	int k;
	if (nlev < 2 || nlev > 16 || lv[nlev - 1] != top)
		return -1;
	g = calloc(1, sizeof(orc_mg));
	g->nlev = nlev; g->cycles = cycles; g->fine_it = fine_it; g->coarse_it = coarse_it;
	for (k = 0; k < nlev; k++) {
		const size_t n = (size_t)lv[k]->neq + 1;
		g->lv[k] = lv[k];
		g->err[k] = calloc(n, sizeof(double));
		if (k > 0) {
			g->itp_n[k] = malloc(n * sizeof(int));
			g->itp_src[k] = malloc(4 * n * sizeof(int));
			memcpy(g->itp_n[k], itp_n[k], (n - 1) * sizeof(int));
			memcpy(g->itp_src[k], itp_src[k], 4 * (n - 1) * sizeof(int));
		}
		if (k < nlev - 1) {
			g->prj[k] = malloc(n * sizeof(int));
			memcpy(g->prj[k], prj[k], (n - 1) * sizeof(int));
		}
	}
	top->mg = g;
	return 0;
}

void orc_set_T(orc *o, const double *T) { memcpy(o->T, T, sizeof(double) * (size_t)o->nno); }

/* viscosity and K of the coarser levels (Viscosity.c:8, Build_matrix.c:8 run
 * over every level); their T stays the initial temperature */
static void assemble_coarse(orc *o)
{
	int k;
	if (o->mg == NULL)
		return;
	for (k = 0; k < o->mg->nlev - 1; k++) {
		viscosity(o->mg->lv[k]);
		assemble_stokes(o->mg->lv[k]);
	}
}

static double wall_s(void)
{
	struct timespec ts;
	clock_gettime(CLOCK_MONOTONIC, &ts);
	return (double)ts.tv_sec + 1e-9 * (double)ts.tv_nsec;
}

/* One time step of Main.c:58-64 (no output).  stats: uzawa, cg, heat cycles,
 * dt, model_time, residual momentum, residual continuity, then the wall
 * seconds of the assembly (buoyancy .. K/F/G), of the Stokes solve and of the
 * temperature update. */
void orc_step(orc *o, double *stats)
{
	double t0 = wall_s(), t1, t2;
	buoyancy_force(o);
	viscosity_step(o);
	assemble_stokes(o);
	assemble_coarse(o);
	t1 = wall_s();
	solve_velocity_pressure(o);
	t2 = wall_s();
	update_temperature(o);
	stats[0] = o->uzawa_cycles; stats[1] = o->cg_cycles; stats[2] = o->heat_cycles;
	stats[3] = o->dt; stats[4] = o->model_time; stats[5] = o->res_m; stats[6] = o->res_c;
	stats[7] = t1 - t0; stats[8] = t2 - t1; stats[9] = wall_s() - t2;
}

/* The caps of the Uzawa loop and of its inner CG (max_citcom_cycle,
 * max_cg_cycle); for bounded timing samples of the CPU baseline. */
void orc_set_caps(orc *o, int max_citcom, int max_cg)
{
	o->max_citcom = max_citcom;
	o->max_cg = max_cg;
}

/* The Stokes half only (buoyancy .. solve), for operator-level checks. */
void orc_stokes(orc *o, double *stats)
{
	buoyancy_force(o);
	viscosity_step(o);
	assemble_stokes(o);
	assemble_coarse(o);
	solve_velocity_pressure(o);
	stats[0] = o->uzawa_cycles; stats[1] = o->cg_cycles; stats[5] = o->res_m; stats[6] = o->res_c;
}

void orc_assemble(orc *o)
{
	buoyancy_force(o);
	viscosity_step(o);
	assemble_stokes(o);
	assemble_coarse(o);
}

/* which: 0 T, 1 V0, 2 V1, 3 P, 4 d, 5 stress, 6 vis, 7 buoyancy, 8 F, 9 Kdiag, 10 tau0, 11 tau1, 12 heat F,
 * 13 grain size */
int orc_get(const orc *o, int which, double *out)
{
	switch (which) {
	case 0: memcpy(out, o->T, sizeof(double) * o->nno); return o->nno;
	case 1: memcpy(out, o->V0, sizeof(double) * o->nno); return o->nno;
	case 2: memcpy(out, o->V1, sizeof(double) * o->nno); return o->nno;
	case 3: memcpy(out, o->p, sizeof(double) * o->nel); return o->nel;
	case 4: memcpy(out, o->d, sizeof(double) * o->neq); return o->neq;
	case 5: memcpy(out, o->stress, sizeof(double) * o->nno); return o->nno;
	case 6: memcpy(out, o->vis, sizeof(double) * o->nno); return o->nno;
	case 7: memcpy(out, o->buoy, sizeof(double) * o->nno); return o->nno;
	case 8: memcpy(out, o->F, sizeof(double) * o->neq); return o->neq;
	case 9: memcpy(out, o->Kdiag, sizeof(double) * o->neq); return o->neq;
	case 10: memcpy(out, o->tau0, sizeof(double) * o->nel); return o->nel;
	case 11: memcpy(out, o->tau1, sizeof(double) * o->nel); return o->nel;
	case 12: memcpy(out, o->HF, sizeof(double) * o->hneq); return o->hneq;
	case 13: memcpy(out, o->gs, sizeof(double) * o->nno); return o->nno;
	default: return -1;
	}
}

void orc_kmul(const orc *o, const double *x, double *y) { K_prod(o, x, y); }
void orc_gmul(const orc *o, const double *p, double *y) { G_prod(o, p, y); }
void orc_gtmul(const orc *o, const double *x, double *p) { GT_prod(o, x, p); }
int orc_sizes(const orc *o, int *out)
{
	out[0] = o->nel; out[1] = o->nno; out[2] = o->neq; out[3] = o->hneq;
	return 4;
}

/* Timing sample for the CPU baseline: n inner CG iterations on the current
 * K (one Uzawa inner solve's worth of work per iteration). */
int orc_cg_sample(orc *o, int n)
{
	double *b = malloc(sizeof(double) * (size_t)o->neq), *x = calloc(o->neq, sizeof(double));
	int i, c;
	for (i = 0; i < o->neq; i++)
		b[i] = o->F[i];
	c = conj_grad(o, b, x, 0.0, n);
	free(b);
	free(x);
	return c;
}

/* Seeded initial temperature for T_ini 0, 1 and -2 (Initial_condition.c:3-75
 * for 0 and 1; the counter-based field of mclg_ic.h for -2) at n nodes, with
 * the same libm calls as the engine's host code; Dirichlet values are applied
 * by the caller (apply_T_bc_values, Initial_condition.c:122-136). */
#include <stdint.h>
#include "mclg_ic.h"
void orc_initial_temperature(int T_ini, const double *dpar, const int *ipar, uint64_t seed, int n, const double *X,
                             const int *gid, double *T)
{
	/* dpar: length, height, T_mantle, T_mantle_perturb, ic_noise, ic_bl_thickness, ic_mode_amp
	 * ipar: T_wave_number, ic_kind, ic_modes */
	const double pi = M_PI, L = dpar[0], H = dpar[1];
	int i;
	mclg_ic_params p;
	memset(&p, 0, sizeof p);
	p.kind = ipar[1];
	p.seed = seed;
	p.noise = dpar[4];
	p.perturb = dpar[3];
	p.wave = ipar[0];
	p.bl_thickness = dpar[5];
	p.nmodes = ipar[2];
	p.mode_amp = dpar[6];
	p.length = L;
	p.height = H;
	for (i = 0; i < n; i++) {
		double x = X[i], z = X[n + i];
		if (T_ini == 0)
			T[i] = H - z + dpar[3] * sin(pi * (H - z) / H) * cos(ipar[0] * pi * x / L);
		else if (T_ini == 1)
			T[i] = dpar[2] + dpar[3] * sin(pi * (H - z) / H) * cos(ipar[0] * pi * x / L);
		else
			T[i] = mclg_ic_temperature(&p, x, z, (uint32_t)gid[i]);
	}
}
