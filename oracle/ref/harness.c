/*
 * Dump harness for the reference built from source (test infrastructure).
 *
 * oracle/ref/Makefile compiles the reference's own .c files unchanged, except
 * that three entry points are renamed on the compiler command line so that
 * this file can wrap them:
 *   output()               Output.c:4            -> mcc_ref_output()
 *   update_temperature()   Update_temperature.c:3 -> mcc_ref_update_temperature()
 *   initial_temperature()  Initial_condition.c:3  -> mcc_ref_initial_temperature()
 * Main.c:55-64 then calls the wrappers below.  They call the reference
 * function and, when MCLG_DUMP_DIR is set, write the reference's in-memory
 * state (mesh, numbering, assembled operators, fields per step) as binary
 * records that tests/golden/make_golden.py turns into fixtures.
 *
 * T_ini=-2 selects the seeded synthetic initial temperature of mclg_ic.h on
 * every MG level (the reference's own T_ini values are passed through).
 *
 * Record format: char name[32]; char dtype[4] ("f8", "i4", "u1"); int64 n;
 * then n little-endian values.
 */
#include "global_variables.h"
#include "mclg_ic.h"

void mcc_ref_output();
void mcc_ref_update_temperature();
void mcc_ref_initial_temperature();
void K_prod_d();
void G_prod_p();
void GT_prod_d();
void K_prod_d_heat();
double global_v_prod();

static const char *dump_dir(void)
{
	return getenv("MCLG_DUMP_DIR");
}

static FILE *dump_open(const char *fmt, int step)
{
	char path[2048], name[256];
	FILE *fp;
	snprintf(name, sizeof name, fmt, step);
	snprintf(path, sizeof path, "%s/%s", dump_dir(), name);
	fp = fopen(path, "wb");
	if (fp == NULL) {
		fprintf(stderr, "harness: cannot open %s\n", path);
		exit(3);
	}
	return fp;
}

static void rec(FILE *fp, const char *name, const char *dtype, const void *data, long long n, size_t esz)
{
	char nm[32] = {0}, dt[4] = {0};
	strncpy(nm, name, 31);
	strncpy(dt, dtype, 3);
	fwrite(nm, 1, 32, fp);
	fwrite(dt, 1, 4, fp);
	fwrite(&n, sizeof n, 1, fp);
	if (n > 0)
		fwrite(data, esz, (size_t)n, fp);
}

static void rec_f8(FILE *fp, const char *name, const double *a, long long n) { rec(fp, name, "f8", a, n, 8); }
static void rec_i4(FILE *fp, const char *name, const int *a, long long n) { rec(fp, name, "i4", a, n, 4); }
static void rec_u1(FILE *fp, const char *name, const char *a, long long n) { rec(fp, name, "u1", a, n, 1); }
static void rec_scalar(FILE *fp, const char *name, double v) { rec_f8(fp, name, &v, 1); }

static void lname(char *buf, const char *base, int lev)
{
	sprintf(buf, "%s@%d", base, lev);
}

/* Ragged row storage (Krow_col/Krow_val with ncol per row) -> CSR records. */
static void rec_ragged(FILE *fp, const char *base, int lev, int nrow, int *ncol, int **col, double **val)
{
	char nm[64];
	long long nnz = 0, k = 0;
	int i, j, *ptr, *c;
	double *v;
	for (i = 0; i < nrow; i++)
		nnz += ncol[i];
	ptr = malloc((nrow + 1) * sizeof(int));
	c = malloc((nnz + 1) * sizeof(int));
	v = malloc((nnz + 1) * sizeof(double));
	ptr[0] = 0;
	for (i = 0; i < nrow; i++) {
		for (j = 0; j < ncol[i]; j++, k++) {
			c[k] = col[i][j];
			v[k] = val[i][j];
		}
		ptr[i + 1] = (int)k;
	}
	sprintf(nm, "%s_ptr@%d", base, lev); rec_i4(fp, nm, ptr, nrow + 1);
	sprintf(nm, "%s_col@%d", base, lev); rec_i4(fp, nm, c, nnz);
	sprintf(nm, "%s_val@%d", base, lev); rec_f8(fp, nm, v, nnz);
	free(ptr); free(c); free(v);
}

static double *seeded(uint32_t stream, int n)
{
	int i;
	double *a = malloc((n + 1) * sizeof(double));
	for (i = 0; i < n; i++)
		a[i] = 2.0 * mclg_uniform01(20240601u, stream, (uint32_t)i) - 1.0;
	return a;
}

static void dump_mesh(void)
{
	int lev, a, d;
	char nm[64];
	FILE *fp = dump_open("mesh.dump", 0);
	int iv[8] = {G.min_level, G.max_level, G.gnox, G.gnoz, 0, 0, 0, 0};
	rec_i4(fp, "levels", iv, 4);
	rec_f8(fp, "dx", G.dx, G.max_level);
	rec_f8(fp, "dz", G.dz, G.max_level);
	for (lev = G.min_level; lev < G.max_level; lev++) {
		int ne = G.nel[lev], nn = G.nno[lev];
		int *buf = malloc((size_t)(8 * ne + 2 * nn + 8) * sizeof(int));
		lname(nm, "Mcode", lev); rec_i4(fp, nm, G.Mcode[lev], ne);
		lname(nm, "node", lev); rec_i4(fp, nm, G.node[lev], nn);
		for (a = 0; a < NEN; a++)
			memcpy(buf + (size_t)a * ne, G.ien[lev][a], ne * sizeof(int));
		lname(nm, "ien", lev); rec_i4(fp, nm, buf, 4LL * ne);
		for (d = 0; d < NSD; d++)
			memcpy(buf + (size_t)d * nn, G.id[lev][d], nn * sizeof(int));
		lname(nm, "id", lev); rec_i4(fp, nm, buf, 2LL * nn);
		lname(nm, "heat_id", lev); rec_i4(fp, nm, G.heat[lev].id, nn);
		for (d = 0; d < NSD; d++)
			for (a = 0; a < NEN; a++)
				memcpy(buf + (size_t)(d * NEN + a) * ne, G.lm[lev][d][a], ne * sizeof(int));
		lname(nm, "lm", lev); rec_i4(fp, nm, buf, 8LL * ne);
		for (a = 0; a < NEN; a++)
			memcpy(buf + (size_t)a * ne, G.heat[lev].lm[a], ne * sizeof(int));
		lname(nm, "heat_lm", lev); rec_i4(fp, nm, buf, 4LL * ne);
		free(buf);
		lname(nm, "T_bc", lev); rec_u1(fp, nm, G.bc.T_bc[lev], nn);
		lname(nm, "T_bc_val", lev); rec_f8(fp, nm, G.bc.T_bc_val[lev], nn);
		lname(nm, "v_bc0", lev); rec_u1(fp, nm, G.bc.v_bc[lev][0], nn);
		lname(nm, "v_bc1", lev); rec_u1(fp, nm, G.bc.v_bc[lev][1], nn);
		lname(nm, "v_bc_val0", lev); rec_f8(fp, nm, G.bc.v_bc_val[lev][0], nn);
		lname(nm, "v_bc_val1", lev); rec_f8(fp, nm, G.bc.v_bc_val[lev][1], nn);
		lname(nm, "X0", lev); rec_f8(fp, nm, G.X[lev][0], nn);
		lname(nm, "X1", lev); rec_f8(fp, nm, G.X[lev][1], nn);
		lname(nm, "jacobi", lev); rec_f8(fp, nm, G.jacobi[lev], ne);
		lname(nm, "area", lev); rec_f8(fp, nm, G.eco[lev].area, ne);
		lname(nm, "hang_node", lev); rec_i4(fp, nm, G.hangle[lev].node, G.hangle[lev].nh);
		lname(nm, "hang_c0", lev); rec_i4(fp, nm, G.hangle[lev].cnode[0], G.hangle[lev].nh);
		lname(nm, "hang_c1", lev); rec_i4(fp, nm, G.hangle[lev].cnode[1], G.hangle[lev].nh);
		iv[0] = G.neq[lev]; iv[1] = G.heat[lev].neq; iv[2] = ne; iv[3] = nn; iv[4] = G.hangle[lev].nh;
		lname(nm, "sizes", lev); rec_i4(fp, nm, iv, 5);
	}
	fclose(fp);
}

/* Assembled Stokes operators and their products with seeded vectors. */
static void dump_stokes_ops(void)
{
	int lev, i, j;
	char nm[64];
	FILE *fp = dump_open("stokes_ops.dump", 0);
	for (lev = G.min_level; lev < G.max_level; lev++) {
		int neq = G.neq[lev], ne = G.nel[lev];
		double *x = seeded(7u, neq), *pp = seeded(8u, ne);
		double *y = malloc((neq + 1) * sizeof(double));
		double *g = malloc((neq + 1) * sizeof(double));
		double *gt = malloc((ne + 1) * sizeof(double));
		double *bab = calloc(ne + 1, sizeof(double));
		lname(nm, "F", lev); rec_f8(fp, nm, G.F[lev], neq);
		lname(nm, "Kdiag", lev); rec_f8(fp, nm, G.Kdiag[lev], neq);
		lname(nm, "buoyancy", lev); rec_f8(fp, nm, G.buoyancy[lev], G.nno[lev]);
		lname(nm, "vis", lev); rec_f8(fp, nm, G.vis[lev], G.nno[lev]);
		lname(nm, "T", lev); rec_f8(fp, nm, G.T[lev], G.nno[lev]);
		rec_ragged(fp, "K", lev, neq, G.Kncol[lev], G.Krow_col[lev], G.Krow_val[lev]);
		rec_ragged(fp, "G", lev, neq, G.Gncol[lev], G.Grow_col[lev], G.Grow_val[lev]);
		K_prod_d(G.Krow_val[lev], G.Krow_col[lev], G.Kncol[lev], x, y, neq, neq, lev, 'v');
		G_prod_p(G.Grow_val[lev], G.Grow_col[lev], G.Gncol[lev], pp, g, G.neq_m[lev], ne, lev);
		GT_prod_d(G.Grow_val[lev], G.Grow_col[lev], G.Gncol[lev], x, gt, G.neq_m[lev], ne, lev);
		for (i = 0; i < G.neq_m[lev]; i++)
			for (j = 0; j < G.Gncol[lev][i]; j++)
				bab[G.Grow_col[lev][i][j]] += G.Grow_val[lev][i][j] * G.Grow_val[lev][i][j] / G.Kdiag[lev][i];
		lname(nm, "probe_x", lev); rec_f8(fp, nm, x, neq);
		lname(nm, "probe_p", lev); rec_f8(fp, nm, pp, ne);
		lname(nm, "Kx", lev); rec_f8(fp, nm, y, neq);
		lname(nm, "Gp", lev); rec_f8(fp, nm, g, neq);
		lname(nm, "GTx", lev); rec_f8(fp, nm, gt, ne);
		lname(nm, "BAB", lev); rec_f8(fp, nm, bab, ne);
		free(x); free(pp); free(y); free(g); free(gt); free(bab);
	}
	fclose(fp);
}

/* Momentum and continuity residual of the Stokes solution on the finest level. */
static void stokes_residual(double out[3])
{
	int lev = G.max_level - 1, neq = G.neq[lev], ne = G.nel[lev], i;
	double *kd = malloc((neq + 1) * sizeof(double)), *gp = malloc((neq + 1) * sizeof(double));
	double *div = malloc((ne + 1) * sizeof(double));
	double rm = 0.0, rc = 0.0, f = 0.0;
	K_prod_d(G.Krow_val[lev], G.Krow_col[lev], G.Kncol[lev], G.d[lev], kd, neq, neq, lev, 'v');
	G_prod_p(G.Grow_val[lev], G.Grow_col[lev], G.Gncol[lev], G.p[lev], gp, G.neq_m[lev], ne, lev);
	GT_prod_d(G.Grow_val[lev], G.Grow_col[lev], G.Gncol[lev], G.d[lev], div, G.neq_m[lev], ne, lev);
	for (i = 0; i < neq; i++) {
		double r = G.F[lev][i] - kd[i] - gp[i];
		rm += r * r;
		f += G.F[lev][i] * G.F[lev][i];
	}
	for (i = 0; i < ne; i++)
		rc += div[i] * div[i];
	out[0] = sqrt(rm); out[1] = sqrt(rc); out[2] = sqrt(f);
	free(kd); free(gp); free(div);
}

void output()
{
	static int first = 1;
	int lev = G.max_level - 1;
	double res[3];
	FILE *fp;
	if (getenv("MCLG_REF_TEXT") != NULL)
		mcc_ref_output();
	if (dump_dir() == NULL)
		return;
	if (first) {
		dump_mesh();
		dump_stokes_ops();
		first = 0;
	}
	fp = dump_open("step_%07d.dump", G.timestep);
	rec_scalar(fp, "timestep", (double)G.timestep);
	rec_scalar(fp, "model_time", G.model_time);
	rec_f8(fp, "T", G.T[lev], G.nno[lev]);
	rec_f8(fp, "V0", G.V[lev][0], G.nno[lev]);
	rec_f8(fp, "V1", G.V[lev][1], G.nno[lev]);
	rec_f8(fp, "p", G.p[lev], G.nel[lev]);
	rec_f8(fp, "d", G.d[lev], G.neq[lev]);
	rec_f8(fp, "stress", G.stress[lev], G.nno[lev]);
	rec_f8(fp, "vis", G.vis[lev], G.nno[lev]);
	rec_f8(fp, "buoyancy", G.buoyancy[lev], G.nno[lev]);
	rec_f8(fp, "F", G.F[lev], G.neq[lev]);
	if (G.control.grain_damage == 1 && G.gs != NULL && G.gs[lev] != NULL)
		rec_f8(fp, "gs", G.gs[lev], G.nno[lev]);   /* grain size (Grain_size_evolution.c:64-110) */
	stokes_residual(res);
	rec_f8(fp, "residual", res, 3);
	fclose(fp);
}

void update_temperature()
{
	static int first = 1;
	int lev = G.max_level - 1;
	FILE *fp;
	mcc_ref_update_temperature();
	if (dump_dir() == NULL)
		return;
	fp = dump_open("heat_%07d.dump", G.timestep);
	rec_scalar(fp, "dt", G.heat[lev].dt);
	rec_scalar(fp, "model_time", G.model_time);
	rec_f8(fp, "T", G.T[lev], G.nno[lev]);
	rec_f8(fp, "heat_d", G.heat[lev].d, G.heat[lev].neq);
	rec_f8(fp, "ddot", G.heat[lev].ddot, G.heat[lev].neq);
	rec_f8(fp, "tau0", G.heat[lev].tau[0], G.nel[lev]);
	rec_f8(fp, "tau1", G.heat[lev].tau[1], G.nel[lev]);
	rec_f8(fp, "heat_F", G.heat[lev].F, G.heat[lev].neq);
	if (first) {
		int n = G.heat[lev].neq;
		double *x = seeded(9u, n), *y = malloc((n + 1) * sizeof(double)), *z = malloc((n + 1) * sizeof(double));
		rec_ragged(fp, "HK", lev, n, G.heat[lev].Kncol, G.heat[lev].Krow_col, G.heat[lev].Krow_val);
		rec_ragged(fp, "HC", lev, n, G.heat[lev].Cncol, G.heat[lev].Crow_col, G.heat[lev].Crow_val);
		K_prod_d_heat(G.heat[lev].Krow_val, G.heat[lev].Krow_col, G.heat[lev].Kncol, x, y, n, n, lev, 'T');
		K_prod_d_heat(G.heat[lev].Crow_val, G.heat[lev].Crow_col, G.heat[lev].Cncol, x, z, n, n, lev, 'T');
		rec_f8(fp, "heat_probe_x", x, n);
		rec_f8(fp, "HKx", y, n);
		rec_f8(fp, "HCx", z, n);
		free(x); free(y); free(z);
		first = 0;
	}
	fclose(fp);
}

void initial_temperature()
{
	int lev, i, ival;
	char sbuf[256];
	mclg_ic_params p;
	if (G.control.T_ini != -2) {
		mcc_ref_initial_temperature();
		return;
	}
	memset(&p, 0, sizeof p);
	input_int("ic_kind", &p.kind, "1");
	input_string("ic_seed", sbuf, "0");
	p.seed = strtoull(sbuf, NULL, 10);
	input_double("ic_noise", &p.noise, "0.0");
	input_double("ic_bl_thickness", &p.bl_thickness, "0.02");
	input_int("ic_modes", &ival, "8");
	p.nmodes = ival;
	input_double("ic_mode_amp", &p.mode_amp, "0.005");
	p.perturb = G.control.T_mantle_perturb;
	p.wave = G.control.T_wave_number;
	p.length = G.global.length;
	p.height = G.global.height;
	G.model_time = 0.0;
	for (lev = G.min_level; lev < G.max_level; lev++) {
		G.T[lev] = realloc(G.T[lev], G.nno[lev] * sizeof(double));
		for (i = 0; i < G.nno[lev]; i++)
			G.T[lev][i] = mclg_ic_temperature(&p, G.X[lev][0][i], G.X[lev][1][i], (uint32_t)G.node[lev][i]);
	}
	apply_T_bc_values();
}
