// C ABI of the engine (include/mclg.h): context life cycle, the Main.c:55-64
// operator sequence, field access and single-operator entry points.
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <algorithm>
#include <chrono>
#include <mutex>
#include <thread>
#include <vector>
#include "k_mg.cuh"
#include "cnn.cuh"
#include "mclg_writer.cuh"
#include "k_qt.cuh"
#include "../host/mclg_host.h"

namespace mclg {
void upload_shape_tables_elem(const ShapeTables &s, cudaStream_t st);
void upload_shape_tables_uzawa(const ShapeTables &s, cudaStream_t st);
void upload_shape_tables_heat(const ShapeTables &s, cudaStream_t st);
void *uzawa_kernel_ptr(int ref);
void *heat_cg_kernel_ptr();
__global__ void k_buoy_rowavg(DevLevel L, const double *T, double Ra, double *avg);
__global__ void k_buoy_vis(DevLevel L, const double *T, double Ra, const double *avg, double Aexp, double refT,
                           double lm_jump, double vmin, double vmax, double *buoy, double *vis);
__global__ void k_assemble_stokes(DevLevel L, const double *vis, const double *buoy, double4 *K, double2 *F,
                                  double2 *Kdiag, int withK);
void upload_shape_tables_mg(const ShapeTables &s, cudaStream_t st);
void upload_shape_tables_qt(const ShapeTables &s, cudaStream_t st);
__global__ void k_qt_extrapolate(int n2, int ne, const double *d1, const double *d2, const double *p1, const double *p2,
                                 double *d, double *p);
__global__ void k_qt_shift(int n2, int ne, const double *d, const double *p, double *d1, double *p1, const double *d2,
                           const double *p2);
__global__ void k_qt_inject(int n, const int *map, const double *src, double *dst, int avg, int nno_f,
                            const int *nb_f, const unsigned char *cnt_f, const double *X_f);
void upload_op_tables(const ShapeTables &S, double r, cudaStream_t st);
// refined meshes: levels of at most this many nodes run in one block of the
// solver kernel (block barriers instead of grid barriers); from a sweep on
// configuration 2 (2048: 25.8, 512: 27.5, 128: 27.8, 0: 27.4 steps/s)
constexpr int kQtBlockNodes = 256;
void *stokes_mg_kernel(int fp64);
void *stokes_mg_batch_kernel(int fp64);
__global__ void k_bab(DevLevel L, const double2 *Kdiag, double *bab);
__global__ void k_stress_elem(DevLevel L, const double *vis, const double2 *V, double *se);
__global__ void k_elem_to_node(DevLevel L, const double *pe, double *pn);
__global__ void k_kmul(DevLevel L, const double4 *K, const double2 *x, double2 *y);
__global__ void k_gmul(DevLevel L, const double *p, double2 *y);
__global__ void k_gtmul(DevLevel L, const double2 *u, double *p);
__global__ void k_tau(DevLevel L, const double2 *V, double accuracy, double *tau0, double *tau1,
                      unsigned long long *mins, int safe);
__global__ void k_assemble_heat(DevLevel L, const double2 *V, const double *tau0, const double *tau1, double Q,
                                double *HK, double *HC, double *HF);
__global__ void k_assemble_heat_fast(DevLevel L, const double2 *V, const double *tau0, const double *tau1,
                                     double Q, double *HK, double *HC, double *HF);
__global__ void k_heat_dt(DevLevel L, const double2 *V, unsigned long long *mins);
__global__ void k_heat_system(DevLevel L, const unsigned long long *mins, double theta, const double *T,
                              const double *HK, const double *HC, const double *HF, double *HA, double *B,
                              double *x0, double *idiag, StepScalars *sc);
__global__ void k_heat_writeback(DevLevel L, const double *x, double *T);
__global__ void k_heat_mul(DevLevel L, const double *M, const double *x, double *y);
__global__ void k_inv_diag2(int n, const double2 *d, double2 *inv);
}  // namespace mclg

using namespace mclg;

struct DevLevelBuf {
	int *node, *ienl, *elev, *p2n_cnt, *p2n_el, *p2n_a, *nb, *hang_ni, *hang_ci0, *hang_ci1, *cell_elem;
	unsigned char *kslot, *self_slot;
	double *dxh, *dzh, *jac, *area, *vbcval, *tbcval, *X, *dx, *dz;
	char *vbc, *tbc;
};

struct mclg_ctx {
	mclg_config cfg;
	mclg_mesh mesh;
	int fl;                       // finest level index
	cudaStream_t st;
	cudaEvent_t ev[7];
	int num_sms;
	int coop_uzawa, coop_heat;    // cooperative grid sizes
	DevLevelBuf lb;
	DevLevel L;
	// fields (finest level)
	double *T, *vis, *buoy, *avg, *stress, *stress_e;
	double2 *V;
	// Stokes
	double4 *K;
	double2 *F, *Kdiag, *idiag, *d, *u1, *Ah, *r, *s, *dd, *q, *xt;
	double *bab, *p, *pe[8];
	// heat
	double *tau0, *tau1, *HK, *HC, *HF, *HA, *HB, *hx, *hidiag, *hr, *hs, *hd, *hq;
	unsigned long long *mins;
	double *red_part;
	StepScalars *sc;              // device
	StepScalars *sc_host;         // pinned
	int timestep;
	int p_initialized;
	long long launches;
	// scratch for the parity API
	double *tmpA, *tmpB;
	// converged solvers on uniform meshes (precision 1 and 2)
	int coop_mg;
	double remesh_ms[5];   // the last remesh: numbering, lists, state, wait, carry (host ms)
	MGArgs<float> mgf;
	MGArgs<double> mgd;
	void *mg_ptr[192];
	int mg_nptr;
	// learned initial guess (converged solvers, warm_start=1)
	mclg_cnn *gnet;
	int gmode, gs, gnc;           // mode, coarsening factor, coarse elements per side
	int ghist;                    // solutions seen since the guess was switched on
	int hist_shift;               // steps until the history is shifted after a remesh (see launch_stokes_qt)
	int gsample, gtimed;          // a sample from the last solve exists; ev[6] was recorded
	double2 *d_h1, *d_h2, *d_cand;   // last two solutions, second candidate guess
	double *p_h1, *p_h2, *p_cand, *gscale;
	double2 *d_h3;                // warm_start=4: the solution before d_h2
	double *p_h3;
	float *gX, *gYt, *gYs;        // features, target and filter scratch on the coarse node grid
	CnnWork gw;
	int goff, gbad;               // steps left with the network off; consecutive steps it did not pay
	bool g_extrap, g_feat;        // this step's solve started from extrapolation / computed features
	bool st_borrowed;             // the stream belongs to an ensemble
	int git_prev;                 // inner iterations of the last step solved from the last solution (-1: none)
	// the reference's own inner solvers (solver="gs" / "mg"): levels ref_lo..fl
	int ref_kind, ref_lo;
	RefMG *ref_dev;
	// levels below the finest resident on the device (solver="mg", and the
	// converged solver on refined meshes), indexed from the coarsest used
	DevLevelBuf lvl_lb[MCLG_MAX_LEVEL];   // (the finest is lb)
	DevLevel lvl_L[MCLG_MAX_LEVEL];
	double *lvl_T[MCLG_MAX_LEVEL], *lvl_vis[MCLG_MAX_LEVEL], *lvl_buoy[MCLG_MAX_LEVEL];
	double4 *lvl_K[MCLG_MAX_LEVEL];
	double2 *lvl_F[MCLG_MAX_LEVEL], *lvl_Kd[MCLG_MAX_LEVEL];
	int *lvl_map[MCLG_MAX_LEVEL];         // node -> the same node one level up
	void **ref_ptr;                       // device allocations of the above, freed together
	int ref_nptr, ref_cap;
	// converged solver on refined meshes (precision 1/2 with hanging nodes)
	int qt_on, coop_qt;
	QtArgs<float> qtf;
	QtArgs<double> qtd;
	OutWriter *writer;            // asynchronous output, created on first use
	struct RemeshJob *rj;         // a remesh begun and not yet finished
	mclg_grain_state *grain;      // grain_damage=1: the grain-size routine's state (host)
};

static int cuda_fail(cudaError_t e, const char *what)
{
	mclg_set_error("%s: %s", what, cudaGetErrorString(e));
	return MCLG_CUDA_ERROR;
}

#define CK(call)                                  \
	do {                                          \
		cudaError_t e_ = (call);                  \
		if (e_ != cudaSuccess)                    \
			return cuda_fail(e_, #call);          \
	} while (0)

template <class T>
static cudaError_t dalloc(T **p, size_t n)
{
	return cudaMalloc((void **)p, (n + 1) * sizeof(T));
}

template <class T>
static cudaError_t upload(T **p, const T *h, size_t n, cudaStream_t st)
{
	cudaError_t e = dalloc(p, n);
	if (e != cudaSuccess)
		return e;
	if (n == 0)
		return cudaSuccess;
	return cudaMemcpyAsync(*p, h, n * sizeof(T), cudaMemcpyHostToDevice, st);
}

static void shape_tables(ShapeTables &S)
{
	// Shape_function.c:17-121
	const double BETA = 1.0 / sqrt(3.0);
	const double pts[4][2] = {{-1.0, -1.0}, {-1.0, 1.0}, {1.0, 1.0}, {1.0, -1.0}};
	for (int d = 0; d < 4; d++) {
		const double xi = pts[d][0] * BETA, eta = pts[d][1] * BETA;
		S.N[0][d] = 0.25 * (1 - xi) * (1 - eta);
		S.N[1][d] = 0.25 * (1 - xi) * (1 + eta);
		S.N[2][d] = 0.25 * (1 + xi) * (1 + eta);
		S.N[3][d] = 0.25 * (1 + xi) * (1 - eta);
		S.dNdxi[0][d] = 0.25 * (-1.0) * (1 - eta);
		S.dNdxi[1][d] = 0.25 * (-1.0) * (1 + eta);
		S.dNdxi[2][d] = 0.25 * (1.0) * (1 + eta);
		S.dNdxi[3][d] = 0.25 * (1.0) * (1 - eta);
		S.dNdeta[0][d] = 0.25 * (1.0 - xi) * (-1.0);
		S.dNdeta[1][d] = 0.25 * (1.0 - xi) * (1.0);
		S.dNdeta[2][d] = 0.25 * (1.0 + xi) * (1.0);
		S.dNdeta[3][d] = 0.25 * (1.0 + xi) * (-1.0);
	}
	const double xi = 0.0, eta = 0.0;
	S.dNdxi_c[0] = 0.25 * (-1.0) * (1 - eta);
	S.dNdxi_c[1] = 0.25 * (-1.0) * (1 + eta);
	S.dNdxi_c[2] = 0.25 * (1.0) * (1 + eta);
	S.dNdxi_c[3] = 0.25 * (1.0) * (1 - eta);
	S.dNdeta_c[0] = 0.25 * (1.0 - xi) * (-1.0);
	S.dNdeta_c[1] = 0.25 * (1.0 - xi) * (1.0);
	S.dNdeta_c[2] = 0.25 * (1.0 + xi) * (1.0);
	S.dNdeta_c[3] = 0.25 * (1.0 + xi) * (-1.0);
}

static int upload_level_into(mclg_ctx *c, int lev, DevLevelBuf &b, DevLevel &L)
{
	const mclg_mesh &m = c->mesh;
	const mclg_level &H = m.lev[lev];
	const size_t ne = H.nel, nn = H.nno, nh = H.nh;
	cudaStream_t st = c->st;
	std::vector<int> ienl(H.ienl, H.ienl + 4 * ne);
	std::vector<unsigned char> self(nn);
	for (size_t A = 0; A < nn; A++) {
		self[A] = 0;
		for (int k = 0; k < H.nb_cnt[A]; k++)
			if (H.nb[(size_t)k * nn + A] == (int)A)
				self[A] = (unsigned char)k;
	}
	CK(upload(&b.node, H.node, nn, st));
	CK(upload(&b.ienl, H.ienl, 4 * ne, st));
	CK(upload(&b.elev, H.elev, ne, st));
	CK(upload(&b.p2n_cnt, H.p2n_cnt, nn, st));
	CK(upload(&b.p2n_el, H.p2n_el, 4 * nn, st));
	CK(upload(&b.p2n_a, H.p2n_a, 4 * nn, st));
	CK(upload(&b.nb, H.nb, (size_t)H.nbw * nn, st));
	CK(upload(&b.kslot, H.kslot, 16 * ne, st));
	CK(upload(&b.self_slot, self.data(), nn, st));
	CK(upload(&b.hang_ni, H.hang_ni, nh, st));
	CK(upload(&b.hang_ci0, H.hang_ci0, nh, st));
	CK(upload(&b.hang_ci1, H.hang_ci1, nh, st));
	if (H.cell_elem != NULL)
		CK(upload(&b.cell_elem, H.cell_elem, (size_t)(m.gnox - 1) * (m.gnoz - 1), st));
	else
		CK(dalloc(&b.cell_elem, 1));
	CK(upload(&b.dxh, H.dx_dxi, ne, st));
	CK(upload(&b.dzh, H.dz_deta, ne, st));
	CK(upload(&b.jac, H.jacobi, ne, st));
	CK(upload(&b.area, H.area, ne, st));
	CK(upload(&b.vbc, H.v_bc, 2 * nn, st));
	CK(upload(&b.vbcval, H.v_bc_val, 2 * nn, st));
	CK(upload(&b.tbc, H.T_bc, nn, st));
	CK(upload(&b.tbcval, H.T_bc_val, nn, st));
	CK(upload(&b.X, H.X, 2 * nn, st));
	CK(upload(&b.dx, m.dx, MCLG_MAX_LEVEL, st));
	CK(upload(&b.dz, m.dz, MCLG_MAX_LEVEL, st));
	CK(cudaStreamSynchronize(st));
	L.nel = (int)ne;
	L.nno = (int)nn;
	L.nbw = H.nbw;
	L.nh = H.nh;
	L.hang_chained = H.hang_chained;
	L.gnox = m.gnox;
	L.gnoz = m.gnoz;
	L.fine_level = m.max_level - 1;
	L.node = b.node;
	L.ienl = b.ienl;
	L.elev = b.elev;
	L.dxh = b.dxh;
	L.dzh = b.dzh;
	L.jac = b.jac;
	L.area = b.area;
	L.vbc = b.vbc;
	L.vbcval = b.vbcval;
	L.tbc = b.tbc;
	L.tbcval = b.tbcval;
	L.X = b.X;
	L.p2n_cnt = b.p2n_cnt;
	L.p2n_el = b.p2n_el;
	L.p2n_a = b.p2n_a;
	L.nb = b.nb;
	L.self_slot = b.self_slot;
	L.kslot = b.kslot;
	L.hang_ni = b.hang_ni;
	L.hang_ci0 = b.hang_ci0;
	L.hang_ci1 = b.hang_ci1;
	L.cell_elem = b.cell_elem;
	L.dx = b.dx;
	L.dz = b.dz;
	return MCLG_OK;
}

static int upload_level(mclg_ctx *c, int lev)
{
	return upload_level_into(c, lev, c->lb, c->L);
}

static void free_level_buf(DevLevelBuf &b)
{
	void *ptrs[] = {b.node, b.ienl, b.elev, b.p2n_cnt, b.p2n_el, b.p2n_a, b.nb, b.hang_ni, b.hang_ci0, b.hang_ci1,
	                b.cell_elem, b.kslot, b.self_slot, b.dxh, b.dzh, b.jac, b.area, b.vbcval, b.tbcval, b.X, b.dx,
	                b.dz, b.vbc, b.tbc};
	for (void *q : ptrs)
		if (q)
			cudaFree(q);
	memset(&b, 0, sizeof b);
}

static int coop_blocks(void *kernel, int num_sms, int work)
{
	int per_sm = 0;
	if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, kBlock, 0) != cudaSuccess || per_sm < 1)
		return 0;
	int maxb = per_sm * num_sms;
	int need = (work + kBlock - 1) / kBlock;
	int nb = need < maxb ? need : maxb;
	if (nb > kMaxCoopBlocks)
		nb = kMaxCoopBlocks;
	return nb < 1 ? 1 : nb;
}

// ---- converged solvers: hierarchy of the uniform mesh -------------------------
template <class T>
static cudaError_t mg_alloc(mclg_ctx *c, T **p, size_t n)
{
	if (c->mg_nptr >= (int)(sizeof c->mg_ptr / sizeof c->mg_ptr[0]))
		return cudaErrorMemoryAllocation;
	cudaError_t e = cudaMalloc((void **)p, (n + 1) * sizeof(T));
	if (e == cudaSuccess) {
		c->mg_ptr[c->mg_nptr++] = *p;
		cudaMemsetAsync(*p, 0, (n + 1) * sizeof(T), c->st);
	}
	return e;
}

// Level l has N0 >> l elements per side; its node (cx, cz) is the fine node
// (cx << l, cz << l), whose BC codes give the Dirichlet mask.
template <class TI>
static int mg_setup(mclg_ctx *c, MGArgs<TI> &a)
{
	typedef typename V2T<TI>::t VI;
	const mclg_mesh &m = c->mesh;
	const mclg_level &H = m.lev[c->fl];
	const int N0 = m.max_elx[c->fl], n0 = N0 + 1;
	int Nc = c->cfg.mg_coarse;
	if (c->cfg.stokes_method != 0 && c->cfg.stokes_method != 1) {
		mclg_set_error("stokes_method=%d: 0 (Uzawa) or 1 (MINRES)", c->cfg.stokes_method);
		return MCLG_BAD_INPUT;
	}
	if (Nc < 2 || Nc > 8 || (Nc & (Nc - 1)) || Nc > N0) {
		mclg_set_error("mg_coarse=%d: need a power of two in [2, min(8, %d)]", Nc, N0);
		return MCLG_BAD_INPUT;
	}
	memset(&a, 0, sizeof a);
	int nlev = 1;
	while ((N0 >> (nlev - 1)) > Nc)
		nlev++;
	if (nlev > kMaxLev || nlev < 2) {
		mclg_set_error("%d multigrid levels from %d to %d elements per side: need 2..%d", nlev, N0, Nc, kMaxLev);
		return MCLG_BAD_INPUT;
	}
	a.H.nlev = nlev;
	a.H.nblk = nlev;
	for (int l = 0; l < nlev; l++)
		if ((N0 >> l) <= c->cfg.mg_block_n) {   // small grids: one block beats grid barriers
			a.H.nblk = l;
			break;
		}
	std::vector<unsigned char> mk;
	for (int l = 0; l < nlev; l++) {
		MGLevel<TI> &L = a.H.lv[l];
		L.N = N0 >> l;
		L.n = L.N + 1;
		const size_t nn = (size_t)L.n * L.n;
		mk.assign(nn, 0);
		for (int cx = 0; cx < L.n; cx++)
			for (int cz = 0; cz < L.n; cz++) {
				const size_t Af = (size_t)(cz << l) + (size_t)(cx << l) * n0;
				mk[cz + (size_t)cx * L.n] = (unsigned char)((H.v_bc[Af] == 'V' ? 1 : 0) |
				                                            (H.v_bc[(size_t)H.nno + Af] == 'V' ? 2 : 0));
			}
		unsigned char *dm;
		CK(mg_alloc(c, &dm, nn));
		CK(cudaMemcpyAsync(dm, mk.data(), nn, cudaMemcpyHostToDevice, c->st));
		CK(cudaStreamSynchronize(c->st));
		L.mask = dm;
		CK(mg_alloc(c, &L.eta, nn));
		CK(mg_alloc(c, &L.invD, nn));
		CK(mg_alloc(c, &L.xa, nn));
		CK(mg_alloc(c, &L.xb, nn));
		CK(mg_alloc(c, &L.b, nn));
		CK(mg_alloc(c, &L.r, nn));
		if (l == 0)
			a.mask0 = dm;
	}
	const int ncn = a.H.lv[nlev - 1].n;
	a.H.cnd = 2 * ncn * ncn;
	CK(mg_alloc(c, &a.H.cinv, (size_t)a.H.cnd * a.H.cnd));
	CK(mg_alloc(c, &a.H.cwork, (size_t)a.H.cnd * 2 * a.H.cnd));
	a.H.omega = (TI)c->cfg.mg_omega;
	a.H.nu = c->cfg.mg_smooth < 1 ? 1 : c->cfg.mg_smooth;
	a.H.nu_c = c->cfg.mg_smooth_coarse < 1 ? a.H.nu : c->cfg.mg_smooth_coarse;
	a.H.lfine = c->cfg.mg_fine_levels < 0 ? 0 : c->cfg.mg_fine_levels;
	a.H.eta_avg = c->cfg.mg_eta_avg;
	// degree-2 Chebyshev on [lmax/ratio, lmax]: theta, delta the centre and half-width,
	// rho_k the recurrence of the scaled polynomials (Saad, Iterative Methods for
	// Sparse Linear Systems, Alg. 12.1)
	a.H.cheb = 0;
	a.H.w1 = a.H.w2 = a.H.c1 = a.H.c0 = (TI)0;
	if (c->cfg.mg_smoother == 1) {
		const double lmax = c->cfg.mg_cheb_lmax, ratio = c->cfg.mg_cheb_ratio;
		if (!(lmax > 0.0) || !(ratio > 1.0)) {
			mclg_set_error("mg_smoother=1 needs mg_cheb_lmax > 0 and mg_cheb_ratio > 1");
			return MCLG_BAD_INPUT;
		}
		const double lo = lmax / ratio, th = 0.5 * (lmax + lo), de = 0.5 * (lmax - lo), sg = th / de;
		const double r0 = 1.0 / sg, r1 = 1.0 / (2.0 * sg - r0);
		a.H.cheb = 1;
		a.H.w1 = (TI)(1.0 / th);
		a.H.c0 = (TI)(r1 * r0);
		a.H.c1 = (TI)(1.0 + r1 * r0);
		a.H.w2 = (TI)(2.0 * r1 / de);
	}
	const size_t nn0 = (size_t)n0 * n0, ne = (size_t)N0 * N0;
	CK(mg_alloc(c, &a.H.px, nn0));
	CK(mg_alloc(c, &a.H.pr, nn0));
	CK(mg_alloc(c, &a.H.pz, nn0));
	CK(mg_alloc(c, &a.H.pp, nn0));
	CK(mg_alloc(c, &a.H.pq, nn0));
	a.N0 = N0;
	a.hx = 0.5 * m.dx[c->fl];
	a.hz = 0.5 * m.dz[c->fl];
	{
		// element_g (mclg_dev.cuh) for the uniform mesh: g0 = -sum dN/dxi * hz, g1 = -sum dN/deta * hx
		ShapeTables S;
		shape_tables(S);
		for (int k = 0; k < 4; k++) {
			double g0 = 0.0, g1 = 0.0;
			for (int gs = 0; gs < 4; gs++) {
				g0 -= S.dNdxi[k][gs] * a.hz;
				g1 -= S.dNdeta[k][gs] * a.hx;
			}
			a.gt.g0[k] = g0;
			a.gt.g1[k] = g1;
			a.gt.g0h[k] = (float)g0;
			a.gt.g0l[k] = (float)(g0 - (double)a.gt.g0h[k]);
			a.gt.g1h[k] = (float)g1;
			a.gt.g1l[k] = (float)(g1 - (double)a.gt.g1h[k]);
		}
	}
	a.vis = c->vis;
	a.vbcval = c->lb.vbcval;
	a.F = c->F;
	a.d = c->d;
	a.p = c->p;
	a.V = c->V;
	CK(mg_alloc(c, &a.R, nn0));
	CK(mg_alloc(c, &a.dd, nn0));
	CK(mg_alloc(c, &a.u1, nn0));
	CK(mg_alloc(c, &a.Kd, nn0));
	CK(mg_alloc(c, &a.invD64, nn0));
	CK(mg_alloc(c, &a.kdiag64, nn0));
	double **ev[] = {&a.Rc, &a.r0, &a.r1, &a.r2, &a.z0, &a.z1, &a.s1, &a.s2, &a.Ahp, &a.dpv, &a.bab};
	for (double **pp : ev)
		CK(mg_alloc(c, pp, ne));
	a.method = c->cfg.stokes_method;
	if (a.method == 1) {
		for (int k = 0; k < 2; k++) {
			CK(mg_alloc(c, &a.mv[k], nn0));
			CK(mg_alloc(c, &a.mw[k], nn0));
			CK(mg_alloc(c, &a.mvp[k], ne));
			CK(mg_alloc(c, &a.mzp[k], ne));
			CK(mg_alloc(c, &a.mwp[k], ne));
		}
	}
	a.red.part = c->red_part;
	a.sc = c->sc;
	a.rtol = c->cfg.stokes_rtol;
	a.outer_rtol = c->cfg.outer_rtol;
	a.inner_rtol = c->cfg.inner_rtol;
	a.max_refine = c->cfg.max_refine;
	a.max_outer = c->cfg.max_outer;
	a.max_inner = c->cfg.max_inner;
	(void)sizeof(VI);
	CK(cudaStreamSynchronize(c->st));
	return MCLG_OK;
}

// History buffers of the converged solvers: the last two solutions (for
// warm_start=3 and the learned guess) and a second candidate guess.
// ---- the reference's own inner solvers: solver="gs" and solver="mg" ---------
static int blocks_for(size_t n)
{
	return (int)((n + kBlock - 1) / kBlock);
}

static int check_launch(mclg_ctx *c, const char *what)
{
	cudaError_t e = cudaGetLastError();
	c->launches++;
	if (e != cudaSuccess)
		return cuda_fail(e, what);
	return MCLG_OK;
}

static cudaError_t dev_track(mclg_ctx *c, void *p)
{
	if (c->ref_nptr == c->ref_cap) {
		const int cap = c->ref_cap ? 2 * c->ref_cap : 64;
		void **q = (void **)realloc(c->ref_ptr, cap * sizeof(void *));
		if (q == NULL) {
			cudaFree(p);
			return cudaErrorMemoryAllocation;
		}
		c->ref_ptr = q;
		c->ref_cap = cap;
	}
	c->ref_ptr[c->ref_nptr++] = p;
	return cudaSuccess;
}

template <class T>
static cudaError_t dev_zeros(mclg_ctx *c, T **p, size_t n)
{
	cudaError_t e = dalloc(p, n);
	if (e != cudaSuccess)
		return e;
	if ((e = dev_track(c, *p)) != cudaSuccess)
		return e;
	return cudaMemsetAsync(*p, 0, (n + 1) * sizeof(T), c->st);
}

template <class T>
static cudaError_t dev_upload(mclg_ctx *c, T **p, const std::vector<T> &h)
{
	cudaError_t e = upload(p, h.data(), h.size(), c->st);
	if (e != cudaSuccess)
		return e;
	return dev_track(c, *p);
}

// Node-layout dof (2*node + direction) of every equation of a level.
static std::vector<int> eq_dofs(const mclg_level &H)
{
	std::vector<int> dof(H.neq > 0 ? H.neq : 1, -1);
	for (int A = 0; A < H.nno; A++)
		for (int d = 0; d < 2; d++) {
			const int eq = H.id[(size_t)d * H.nno + A];
			if (eq >= 0)
				dof[eq] = 2 * A + d;
		}
	return dof;
}

// The hierarchy of solver="mg" (mg_min_level .. finest; Connection.c:20-29
// builds its maps) or the finest level alone for solver="gs": per level the
// Gauss-Seidel wavefronts, work vectors and transfer maps, and below the
// finest level the operator K of the level's own initial temperature.  The
// reference assembles every level every step (Viscosity.c:8,
// Build_matrix.c:8) but only the finest level's T changes, so the coarse K
// are built once here.
static int ref_setup(mclg_ctx *c)
{
	const mclg_mesh &m = c->mesh;
	const mclg_config &f = c->cfg;
	c->ref_kind = strcmp(f.solver, "mg") == 0 ? kRefMG : kRefGS;
	const int top = c->fl, lo = c->ref_kind == kRefMG ? m.min_level : top;
	if (c->ref_kind == kRefMG && lo >= top) {   // Solver.c:677-682
		mclg_set_error("solver=\"mg\" needs mg_min_level (%d) below level-1 (%d)", lo, top);
		return MCLG_BAD_INPUT;
	}
	if (c->ref_kind == kRefMG && (f.mg_cycle < 0 || f.mg_finest_iteration < 0 || f.mg_coarse_iteration < 0)) {
		mclg_set_error("mg_cycle, mg_finest_iteration and mg_coarse_iteration must be >= 0");
		return MCLG_BAD_INPUT;
	}
	c->ref_lo = lo;
	RefMG h;
	memset(&h, 0, sizeof h);
	h.nlev = top - lo + 1;
	h.cycles = f.mg_cycle;
	h.fine_it = f.mg_finest_iteration;
	h.coarse_it = f.mg_coarse_iteration;
	double *zeros_gnoz = NULL;
	CK(dev_zeros(c, &zeros_gnoz, (size_t)m.gnoz));
	for (int lev = lo; lev <= top; lev++) {
		const int k = lev - lo;
		const mclg_level &H = m.lev[lev];
		const size_t nn = H.nno;
		RefLevel &R = h.lev[k];
		if (lev == top) {
			c->lvl_L[k] = c->L;
			R.K = c->K;
		} else {
			DevLevel &L = c->lvl_L[k];
			memset(&L, 0, sizeof L);
			int rc = upload_level_into(c, lev, c->lvl_lb[k], L);
			if (rc != MCLG_OK)
				return rc;
			std::vector<double> T(nn);
			if ((rc = mclg_host_initial_temperature(&m, &f, lev, T.data())) != MCLG_OK)
				return rc;
			double *buoy = NULL;
			double2 *F = NULL, *Kd = NULL;
			CK(dev_upload(c, &c->lvl_T[k], T));
			CK(dev_zeros(c, &c->lvl_vis[k], nn));
			CK(dev_zeros(c, &buoy, nn));
			CK(dev_zeros(c, &c->lvl_K[k], (size_t)H.nbw * nn));
			CK(dev_zeros(c, &F, nn));
			CK(dev_zeros(c, &Kd, nn));
			// viscosity of the level's T; the buoyancy (Ra = 0 here) only feeds F, which no level below the finest uses
			k_buoy_vis<<<blocks_for(nn), kBlock, 0, c->st>>>(L, c->lvl_T[k], 0.0, zeros_gnoz, f.A, f.refT,
			                                                 f.lower_mantle_jump, f.vis_min, f.vis_max, buoy,
			                                                 c->lvl_vis[k]);
			if ((rc = check_launch(c, "k_buoy_vis")))
				return rc;
			k_assemble_stokes<<<blocks_for(nn), kBlock, 0, c->st>>>(L, c->lvl_vis[k], buoy, c->lvl_K[k], F, Kd, 1);
			if ((rc = check_launch(c, "k_assemble_stokes")))
				return rc;
			R.K = c->lvl_K[k];
		}
		const DevLevel &L = c->lvl_L[k];
		R.nno = (int)nn;
		R.nbw = H.nbw;
		R.nb = L.nb;
		R.self_slot = L.self_slot;
		R.vbc = L.vbc;
		// Gauss-Seidel wavefronts, nodes grouped by wavefront
		std::vector<int> wave(nn), order(nn), off;
		mclg_refmg_waves(&H, wave.data());
		int nw = 0;
		for (size_t A = 0; A < nn; A++)
			nw = wave[A] + 1 > nw ? wave[A] + 1 : nw;
		off.assign((size_t)nw + 1, 0);
		for (size_t A = 0; A < nn; A++)
			off[wave[A] + 1]++;
		for (int w = 0; w < nw; w++)
			off[w + 1] += off[w];
		std::vector<int> fill(off.begin(), off.end() - 1);
		for (size_t A = 0; A < nn; A++)
			order[fill[wave[A]]++] = (int)A;
		R.nwave = nw;
		CK(dev_upload(c, (int **)&R.wave, order));
		CK(dev_upload(c, (int **)&R.wave_off, off));
		CK(dev_zeros(c, &R.err, nn));
		CK(dev_zeros(c, &R.rhs, nn));
		CK(dev_zeros(c, &R.res, nn));
		CK(dev_zeros(c, &R.xt, nn));
		// interp_error's map from the level below (Connection.c:708-930)
		std::vector<int> itp_n(2 * nn, 0), itp_src(8 * nn, -1);
		if (k > 0) {
			const int neq = H.neq;
			std::vector<int> n(neq > 0 ? neq : 1), src(4 * (size_t)(neq > 0 ? neq : 1));
			if (mclg_refmg_interp(&m, lev, n.data(), src.data()) != MCLG_OK) {
				mclg_set_error("level %d: interpolation map has more than 4 terms", lev);
				return MCLG_BAD_INPUT;
			}
			const std::vector<int> lo_dof = eq_dofs(m.lev[lev - 1]);
			for (size_t A = 0; A < nn; A++)
				for (int d = 0; d < 2; d++) {
					const int eu = H.id[(size_t)d * nn + A];
					if (eu < 0)
						continue;
					itp_n[(size_t)d * nn + A] = n[eu];
					for (int i = 0; i < 4; i++) {
						const int el = src[(size_t)i * neq + eu];
						itp_src[(size_t)(i * 2 + d) * nn + A] = el >= 0 ? lo_dof[el] : -1;
					}
				}
		}
		CK(dev_upload(c, (int **)&R.itp_n, itp_n));
		CK(dev_upload(c, (int **)&R.itp_src, itp_src));
		// project_res's map to the level above (Connection.c:1051-1251)
		std::vector<int> prj(2 * nn, -1);
		if (lev < top) {
			std::vector<int> up_eq(H.neq > 0 ? H.neq : 1);
			mclg_refmg_project(&m, lev, up_eq.data());
			const std::vector<int> up_dof = eq_dofs(m.lev[lev + 1]);
			for (size_t A = 0; A < nn; A++)
				for (int d = 0; d < 2; d++) {
					const int el = H.id[(size_t)d * nn + A];
					if (el < 0)
						continue;
					if (up_eq[el] < 0) {   // the reference would read res_u[-1] or leave res_l unset
						mclg_set_error("level %d: equation %d has no equation on level %d to take its residual from",
						               lev, el, lev + 1);
						return MCLG_BAD_INPUT;
					}
					prj[(size_t)d * nn + A] = up_dof[up_eq[el]];
				}
		}
		CK(dev_upload(c, (int **)&R.prj, prj));
	}
	void *p = NULL;
	CK(cudaMalloc(&p, sizeof(RefMG)));
	CK(dev_track(c, p));
	c->ref_dev = (RefMG *)p;
	CK(cudaMemcpyAsync(c->ref_dev, &h, sizeof h, cudaMemcpyHostToDevice, c->st));
	CK(cudaStreamSynchronize(c->st));
	return MCLG_OK;
}

// A level below the finest that is resident on the device (solver="mg"); k is its index in the hierarchy.
static bool coarse_level(const mclg_ctx *c, int lev, int *k)
{
	if (c->ref_kind != kRefMG || lev < c->ref_lo || lev >= c->fl)
		return false;
	*k = lev - c->ref_lo;
	return true;
}

// ---- converged solver on refined meshes ------------------------------------------
// Host structures of a model built ahead of it (a remesh prepares them on a
// worker thread while the GPU keeps stepping the old mesh).
// The constant-memory tables of the kernels are the same for every context on a
// device (the Q1 element tables are fixed; the operator tables depend on the
// box's aspect ratio r): each kind is uploaded once per device (again when r
// changes) and waited for, so that no context's kernel reads a table before
// its upload and no upload rewrites a table while another context's kernels
// run (a remesh builds the new context on a worker thread while the old one
// steps).
enum { kTabElem = 1, kTabUzawa = 2, kTabHeat = 4, kTabMg = 8, kTabOp = 16, kTabQt = 32 };
static std::mutex g_tab_mu;
static unsigned g_tab_done[64];
static double g_tab_r[64];

static int tables_once(mclg_ctx *c, unsigned kinds, double r)
{
	int dev = 0;
	if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64)
		return cuda_fail(cudaErrorInvalidDevice, "tables_once");
	std::lock_guard<std::mutex> lock(g_tab_mu);
	unsigned need = kinds & ~g_tab_done[dev];
	if ((kinds & kTabOp) && (g_tab_done[dev] & kTabOp) && g_tab_r[dev] != r)
		need |= kTabOp;
	if (need == 0)
		return MCLG_OK;
	ShapeTables S;
	shape_tables(S);
	if (need & kTabElem) upload_shape_tables_elem(S, c->st);
	if (need & kTabUzawa) upload_shape_tables_uzawa(S, c->st);
	if (need & kTabHeat) upload_shape_tables_heat(S, c->st);
	if (need & kTabMg) upload_shape_tables_mg(S, c->st);
	if (need & kTabOp) upload_op_tables(S, r, c->st);
	if (need & kTabQt) upload_shape_tables_qt(S, c->st);
	cudaError_t e = cudaGetLastError();
	if (e == cudaSuccess)
		e = cudaStreamSynchronize(c->st);
	if (e != cudaSuccess)
		return cuda_fail(e, "constant tables");
	g_tab_done[dev] |= need;
	if (need & kTabOp)
		g_tab_r[dev] = r;
	return MCLG_OK;
}

struct Prebuilt {
	mclg_mesh mesh;
	mclg_qt_level q[MCLG_MAX_LEVEL];
	int nq;                        // levels of q built (refined meshes with a converged solver)
};

static void prebuilt_free(Prebuilt *pb)
{
	for (int i = 0; i < pb->nq; i++)
		mclg_qt_free(&pb->q[i]);
	pb->nq = 0;
	mclg_mesh_free(&pb->mesh);
}

template <class TW, class TS>
static cudaError_t dev_upload_cast(mclg_ctx *c, TW **p, const TS *h, size_t n)
{
	std::vector<TW> v(n ? n : 1);
	for (size_t i = 0; i < n; i++)
		v[i] = (TW)h[i];
	return dev_upload(c, p, v);
}

template <class T>
static cudaError_t dev_upload_n(mclg_ctx *c, T **p, const T *h, size_t n)
{
	std::vector<T> v(h, h + n);
	if (v.empty())
		v.push_back(T());
	return dev_upload(c, p, v);
}

// Levels mg_min_level .. finest of the mesh, their constrained-space lists
// (mclg_qtmg.c), the TI operators and work vectors, the coarsest level's
// dense inverse and the FP64 MINRES vectors.
template <class TI>
static int qt_setup(mclg_ctx *c, QtArgs<TI> &a, Prebuilt *pre)
{
	typedef typename Q2T<TI>::t V;
	typedef typename V4T<TI>::t K4;
	const mclg_mesh &m = c->mesh;
	const mclg_config &f = c->cfg;
	const int top = c->fl, lo = m.min_level, nlev = top - lo + 1;
	if (nlev < 2 || nlev > 16) {
		mclg_set_error("the refined-mesh solver needs 2..16 levels (mg_min_level %d, finest %d)", lo, top);
		return MCLG_BAD_INPUT;
	}
	for (int l = lo; l <= top; l++)
		for (int i = 0; i < 2 * m.lev[l].nno; i++)
			if (m.lev[l].v_bc[i] == 'V' && m.lev[l].v_bc_val[i] != 0.0) {
				mclg_set_error("the refined-mesh solver takes homogeneous velocity boundary values only");
				return MCLG_BAD_INPUT;
			}
	std::vector<mclg_qt_level> q((size_t)nlev);
	int rc = MCLG_OK;
	if (pre != NULL && pre->nq == nlev) {   // built ahead: take them over
		for (int i = 0; i < nlev; i++)
			q[i] = pre->q[i];
		memset(pre->q, 0, sizeof pre->q);
		pre->nq = 0;
	} else {
		rc = mclg_qt_build(&m, lo, q.data());
	}
	struct Free {
		std::vector<mclg_qt_level> &q;
		~Free()
		{
			for (auto &x : q)
				mclg_qt_free(&x);
		}
	} guard{q};
	if (rc != MCLG_OK)
		return rc;
	memset(&a, 0, sizeof a);
	a.L = c->L;
	a.F = c->F;
	a.bab = c->bab;
	a.d = c->d;
	a.V = c->V;
	a.p = c->p;
	QtHier<TI> &H = a.H;
	H.nlev = nlev;
	H.smooth = f.mg_smooth > 0 ? f.mg_smooth : 1;
	H.omega = (TI)f.mg_omega;
	// the smallest levels (at most kQtBlockNodes nodes) run in one block
	H.nblk = 0;
	while (H.nblk < nlev - 1 && m.lev[lo + H.nblk].nno <= kQtBlockNodes)
		H.nblk++;
	for (int l = lo; l <= top; l++) {
		const int k = l - lo;
		const mclg_level &ML = m.lev[l];
		const mclg_qt_level &S = q[k];
		QtLevel<TI> &Q = H.lv[k];
		const size_t nn = ML.nno, nk = (size_t)ML.nbw * nn;
		if (l == top) {
			Q.K64 = c->K;
		} else {
			DevLevel &L = c->lvl_L[k];
			memset(&L, 0, sizeof L);
			if ((rc = upload_level_into(c, l, c->lvl_lb[k], L)) != MCLG_OK)
				return rc;
			CK(dev_zeros(c, &c->lvl_K[k], nk));
			CK(dev_zeros(c, &c->lvl_vis[k], nn));
			CK(dev_zeros(c, &c->lvl_buoy[k], nn));
			CK(dev_zeros(c, &c->lvl_F[k], nn));
			CK(dev_zeros(c, &c->lvl_Kd[k], nn));
			CK(dev_upload_n(c, &c->lvl_map[k], S.node_map, nn));
			Q.K64 = c->lvl_K[k];
		}
		Q.nno = (int)nn;
		Q.nbw = ML.nbw;
		{   // neighbour columns flagged where a component is constrained, and counts
			std::vector<int> nbf(nk);
			std::vector<unsigned char> cnt(nn);
			for (size_t A = 0; A < nn; A++) {
				cnt[A] = (unsigned char)ML.nb_cnt[A];
				for (int kk = 0; kk < ML.nbw; kk++) {
					const int B = ML.nb[(size_t)kk * nn + A];
					const bool con = S.kind[2 * B] == 2 || S.kind[2 * B + 1] == 2;
					nbf[(size_t)kk * nn + A] = con ? (B | kQtCon) : B;
				}
			}
			CK(dev_upload(c, (int **)&Q.nb, nbf));
			CK(dev_upload(c, (unsigned char **)&Q.cnt, cnt));
		}
		K4 *Kr = NULL;
		TI *invD = NULL;
		CK(dev_zeros(c, &Kr, (size_t)S.rnbw * nn));
		CK(dev_zeros(c, &invD, 2 * nn));
		Q.Kr = Kr;
		Q.invD = invD;
		Q.rnbw = S.rnbw;
		CK(dev_upload_n(c, (int **)&Q.rnb, S.rnb, (size_t)S.rnbw * nn));
		CK(dev_upload_n(c, (unsigned char **)&Q.rcnt, S.rcnt, nn));
		CK(dev_upload_n(c, (int **)&Q.rc_off, S.rc_off, nn + 1));
		CK(dev_upload_n(c, (int **)&Q.rc_tgt, S.rc_tgt, (size_t)S.n_rc));
		CK(dev_upload_n(c, (int **)&Q.rc_src, S.rc_src, (size_t)S.n_rc));
		CK(dev_upload_cast(c, (float **)&Q.rc_w, S.rc_w, (size_t)S.n_rc));
		const size_t nd = 2 * nn;
		CK(dev_upload_n(c, (unsigned char **)&Q.kind, S.kind, nd));
		CK(dev_upload_n(c, (int **)&Q.ex_off, S.ex_off, nd + 1));
		CK(dev_upload_n(c, (int **)&Q.ex_src, S.ex_src, (size_t)S.n_ex));
		CK(dev_upload_cast(c, (TI **)&Q.ex_w, S.ex_w, (size_t)S.n_ex));
		CK(dev_upload_n(c, (int **)&Q.fo_off, S.fo_off, nd + 1));
		CK(dev_upload_n(c, (int **)&Q.fo_dof, S.fo_dof, (size_t)S.n_fo));
		CK(dev_upload_cast(c, (TI **)&Q.fo_w, S.fo_w, (size_t)S.n_fo));
		if (k > 0) {
			CK(dev_upload_n(c, (int **)&Q.p_off, S.p_off, nd + 1));
			CK(dev_upload_n(c, (int **)&Q.p_src, S.p_src, (size_t)S.n_p));
			CK(dev_upload_cast(c, (TI **)&Q.p_w, S.p_w, (size_t)S.n_p));
		}
		if (l < top) {
			CK(dev_upload_n(c, (int **)&Q.r_off, S.r_off, nd + 1));
			CK(dev_upload_n(c, (int **)&Q.r_src, S.r_src, (size_t)S.n_r));
			CK(dev_upload_cast(c, (TI **)&Q.r_w, S.r_w, (size_t)S.n_r));
		}
		for (int i = 0; i < 2; i++)
			CK(dev_zeros(c, &Q.x[i], nn));
		CK(dev_zeros(c, &Q.b, nn));
		CK(dev_zeros(c, &Q.r, nn));
	}
	// the coarsest level's reduced dofs and its dense inverse's storage
	{
		const mclg_qt_level &S = q[0];
		std::vector<int> cd;
		for (int d = 0; d < 2 * S.nno; d++)
			if (S.kind[d] == 1)
				cd.push_back(d);
		if (cd.empty() || cd.size() > 1024) {
			mclg_set_error("the coarsest level (%d) has %zu unknowns; it needs 1..1024 (lower mg_min_level)", lo,
			               cd.size());
			return MCLG_BAD_INPUT;
		}
		H.nc = (int)cd.size();
		CK(dev_upload(c, (int **)&H.cdof, cd));
		CK(dev_zeros(c, &H.cwork, (size_t)H.nc * 2 * H.nc));
		CK(dev_zeros(c, &H.cinv, (size_t)H.nc * H.nc));
		CK(dev_zeros(c, &H.cvec, 2 * (size_t)S.nno));
	}
	const size_t nn = c->L.nno, ne = c->L.nel;
	CK(dev_zeros(c, &a.R, nn));
	CK(dev_zeros(c, &a.Kd, nn));
	CK(dev_zeros(c, &a.dd, nn));
	CK(dev_zeros(c, &a.u1, nn));
	CK(dev_zeros(c, &a.Rc, ne));
	CK(dev_zeros(c, &a.dpv, ne));
	CK(dev_zeros(c, &a.Ahp, ne));
	for (int i = 0; i < 2; i++) {
		CK(dev_zeros(c, &a.mv[i], nn));
		CK(dev_zeros(c, &a.mw[i], nn));
		CK(dev_zeros(c, &a.mvp[i], ne));
		CK(dev_zeros(c, &a.mzp[i], ne));
		CK(dev_zeros(c, &a.mwp[i], ne));
		CK(dev_zeros(c, &a.mz[i], nn));
	}
	a.red.part = c->red_part;
	a.red.flip = 0;
	a.sc = c->sc;
	a.rtol = f.stokes_rtol;
	a.outer_rtol = f.outer_rtol;
	a.max_refine = f.max_refine;
	a.max_outer = f.max_outer;
	(void)sizeof(V);
	if ((rc = tables_once(c, kTabQt, 0.0)) != MCLG_OK)
		return rc;
	CK(cudaStreamSynchronize(c->st));
	c->qt_on = 1;
	return MCLG_OK;
}

// One converged solve on a refined mesh: warm start, the coarse levels'
// viscosity (the finer level's value at the same node) and K, then the
// solver (one cooperative launch here; a batched launch for ensemble members,
// see stokes_qt_finish), the warm-start history.
static int stokes_qt_prepare(mclg_ctx *c)
{
	const mclg_config &f = c->cfg;
	const size_t nn = c->L.nno, ne = c->L.nel;
	int rc;
	if (f.warm_start != 1 && f.warm_start != 3 && f.warm_start != 4)
		CK(cudaMemsetAsync(c->d, 0, nn * sizeof(double2), c->st));
	if (f.warm_start == 0)
		CK(cudaMemsetAsync(c->p, 0, ne * sizeof(double), c->st));
	CK(cudaMemsetAsync(&c->sc->status, 0, sizeof(int), c->st));
	CK(cudaMemsetAsync(&c->sc->guess_used, 0xff, sizeof(int), c->st));
	const bool track = c->d_h1 != NULL;
	if (track) {   // history: d_h2 <- d_h1, d_h1 <- d (the last two solutions)
		const size_t n = 2 * nn > ne ? 2 * nn : ne;
		if (c->hist_shift == 1 && (f.warm_start == 3 || f.warm_start == 4) && c->ghist >= 2) {
			// the second step after a remesh: d_h1, d_h2 are the last two solutions of
			// the old mesh interpolated, d the first solution on the new one.  Their
			// extrapolation 2 d - d_h1 would add the interpolation error of d_h1 once
			// more; d_h1 <- d - (d_h1 - d_h2) makes it d + (d_h1 - d_h2), the last
			// interpolated increment on top of the new mesh's solution.
			k_qt_shift<<<blocks_for(n), kBlock, 0, c->st>>>((int)(2 * nn), (int)ne, (const double *)c->d, c->p,
			                                               (double *)c->d_h1, c->p_h1, (const double *)c->d_h2,
			                                               c->p_h2);
			if ((rc = check_launch(c, "k_qt_shift")))
				return rc;
		}
		if (c->hist_shift > 0)
			c->hist_shift--;
		CK(cudaMemcpyAsync(c->d_h2, c->d_h1, nn * sizeof(double2), cudaMemcpyDeviceToDevice, c->st));
		CK(cudaMemcpyAsync(c->p_h2, c->p_h1, ne * sizeof(double), cudaMemcpyDeviceToDevice, c->st));
		CK(cudaMemcpyAsync(c->d_h1, c->d, nn * sizeof(double2), cudaMemcpyDeviceToDevice, c->st));
		CK(cudaMemcpyAsync(c->p_h1, c->p, ne * sizeof(double), cudaMemcpyDeviceToDevice, c->st));
		if ((f.warm_start == 3 || f.warm_start == 4) && c->ghist >= 2) {
			k_qt_extrapolate<<<blocks_for(n), kBlock, 0, c->st>>>((int)(2 * nn), (int)ne, (const double *)c->d_h1,
			                                                       (const double *)c->d_h2, c->p_h1, c->p_h2,
			                                                       (double *)c->d, c->p);
			if ((rc = check_launch(c, "k_qt_extrapolate")))
				return rc;
		}
	}
	const int nlev = c->cfg.precision == 2 ? c->qtd.H.nlev : c->qtf.H.nlev;
	for (int k = nlev - 2; k >= 0; k--) {
		const DevLevel &L = c->lvl_L[k];
		const DevLevel &U = k == nlev - 2 ? c->L : c->lvl_L[k + 1];
		const double *src = k == nlev - 2 ? c->vis : c->lvl_vis[k + 1];
		const int *nbu = c->cfg.precision == 2 ? c->qtd.H.lv[k + 1].nb : c->qtf.H.lv[k + 1].nb;
		const unsigned char *cntu = c->cfg.precision == 2 ? c->qtd.H.lv[k + 1].cnt : c->qtf.H.lv[k + 1].cnt;
		k_qt_inject<<<blocks_for(L.nno), kBlock, 0, c->st>>>(L.nno, c->lvl_map[k], src, c->lvl_vis[k],
		                                                      c->cfg.mg_eta_avg, U.nno, nbu, cntu, U.X);
		if ((rc = check_launch(c, "k_qt_inject")))
			return rc;
		k_assemble_stokes<<<blocks_for(L.nno), kBlock, 0, c->st>>>(L, c->lvl_vis[k], c->lvl_buoy[k], c->lvl_K[k],
		                                                           c->lvl_F[k], c->lvl_Kd[k], 1);
		if ((rc = check_launch(c, "k_assemble_stokes")))
			return rc;
	}
	(void)track;
	return MCLG_OK;
}

// after the solve: the warm-start history counts one more solution
static void stokes_qt_finish(mclg_ctx *c)
{
	if (c->d_h1 != NULL)
		c->ghist++;
}

// The persistent solver kernels hold every SM for the whole solve.  While a
// remesh is pending they leave a few blocks' room free, so that the kernels
// with which the remesh worker sets up the new mesh's device state run beside
// the solve instead of queueing behind it (measured on configuration 2: the
// setup took 51 ms on the worker against 18 ms on an idle device).
static int solver_grid(const mclg_ctx *c, int coop)
{
	constexpr int kSpare = 8;
	return (c->rj != NULL && coop > 4 * kSpare) ? coop - kSpare : coop;
}

static int launch_stokes_qt(mclg_ctx *c)
{
	int rc = stokes_qt_prepare(c);
	if (rc)
		return rc;
	const dim3 grid(solver_grid(c, c->coop_qt));
	if (c->cfg.precision == 2) {
		void *args[] = {&c->qtd};
		CK(cudaLaunchCooperativeKernel(qt_kernel(1), grid, dim3(kBlock), args, 0, c->st));
	} else {
		void *args[] = {&c->qtf};
		CK(cudaLaunchCooperativeKernel(qt_kernel(0), grid, dim3(kBlock), args, 0, c->st));
	}
	c->launches++;
	stokes_qt_finish(c);
	return MCLG_OK;
}

static int alloc_history(mclg_ctx *c)
{
	if (c->d_h1 != NULL)
		return MCLG_OK;
	const size_t nn = (size_t)c->L.nno, ne = (size_t)c->L.nel;
	CK(dalloc(&c->d_h1, nn));
	CK(dalloc(&c->d_h2, nn));
	CK(dalloc(&c->d_cand, nn));
	CK(dalloc(&c->p_h1, ne));
	CK(dalloc(&c->p_h2, ne));
	CK(dalloc(&c->p_cand, ne));
	CK(dalloc(&c->gscale, 4));
	if (c->cfg.warm_start == 4) {
		CK(dalloc(&c->d_h3, nn));
		CK(dalloc(&c->p_h3, ne));
		const MGArgs<float> &mf = c->mgf;
		(void)mf;
		c->mgf.h1d = c->mgd.h1d = c->d_h1;
		c->mgf.h2d = c->mgd.h2d = c->d_h2;
		c->mgf.h3d = c->mgd.h3d = c->d_h3;
		c->mgf.h1p = c->mgd.h1p = c->p_h1;
		c->mgf.h2p = c->mgd.h2p = c->p_h2;
		c->mgf.h3p = c->mgd.h3p = c->p_h3;
	}
	c->ghist = 0;
	return MCLG_OK;
}

// The converged solve of one step in three parts, so that a batch can run the
// parts of many models around one launch of the batched kernel:
// stokes_mg_prepare (warm start, learned guess), the solver kernel,
// stokes_mg_finish (guess targets, history).
static int stokes_mg_prepare(mclg_ctx *c)
{
	const mclg_config &f = c->cfg;
	// warm_start: 0 = zero guess; 1 = previous (d, p); 2 = the reference's
	// policy for zero_P=0 (initial_d_p, Solver.c:251-278): d zeroed, p kept;
	// 3 = linear extrapolation in time of the last two solutions (previous
	// solution until two exist)
	if (f.warm_start != 1 && f.warm_start != 3 && f.warm_start != 4)
		CK(cudaMemsetAsync(c->d, 0, c->L.nno * sizeof(double2), c->st));
	if (f.warm_start == 0)
		CK(cudaMemsetAsync(c->p, 0, c->L.nel * sizeof(double), c->st));
	CK(cudaMemsetAsync(&c->sc->status, 0, sizeof(int), c->st));
	CK(cudaMemsetAsync(&c->sc->guess_used, 0xff, sizeof(int), c->st));   // -1: not judged
	const int N0 = c->mgf.N0 ? c->mgf.N0 : c->mgd.N0;
	const unsigned char *mask0 = c->mgf.N0 ? c->mgf.mask0 : c->mgd.mask0;
	const size_t nn = (size_t)c->L.nno, ne = (size_t)c->L.nel;
	const bool track = c->d_h1 != NULL;
	const bool hist2 = track && c->ghist >= 2;
	const bool extrap = hist2 && f.warm_start == 3;
	const bool net_on = hist2 && (c->gmode == MCLG_GUESS_LEARNED || c->gmode == MCLG_GUESS_FORCED) &&
	                    c->gnet != NULL && c->goff == 0;
	const bool feat = hist2 && (c->gmode == MCLG_GUESS_RECORD || net_on);
	const double2 *d_alt = nullptr;
	const double *p_alt = nullptr;
	c->gtimed = 0;
	c->gsample = 0;
	if (track) {
		// features from (T, eta, last two solutions) before d is overwritten
		if (feat)
			guess_features(c->st, N0, c->gs, c->T, c->vis, c->d, c->p, c->d_h1, c->p_h1, c->gX, c->gscale);
		// history: d_h2 <- d_h1, d_h1 <- d (the last two solutions; device copies,
		// so that a captured step replays unchanged), and d_h3 <- d_h2 before them
		// for warm_start=4, whose start the solver kernel forms from the three
		if (c->d_h3 != NULL) {
			CK(cudaMemcpyAsync(c->d_h3, c->d_h2, nn * sizeof(double2), cudaMemcpyDeviceToDevice, c->st));
			CK(cudaMemcpyAsync(c->p_h3, c->p_h2, ne * sizeof(double), cudaMemcpyDeviceToDevice, c->st));
		}
		CK(cudaMemcpyAsync(c->d_h2, c->d_h1, nn * sizeof(double2), cudaMemcpyDeviceToDevice, c->st));
		CK(cudaMemcpyAsync(c->p_h2, c->p_h1, ne * sizeof(double), cudaMemcpyDeviceToDevice, c->st));
		CK(cudaMemcpyAsync(c->d_h1, c->d, nn * sizeof(double2), cudaMemcpyDeviceToDevice, c->st));
		CK(cudaMemcpyAsync(c->p_h1, c->p, ne * sizeof(double), cudaMemcpyDeviceToDevice, c->st));
		if (extrap) {
			guess_extrapolate(c->st, (int)nn, (int)ne, mask0, c->d_h1, c->p_h1, c->d_h2, c->p_h2, c->d, c->p);
			c->launches++;
		}
		if (net_on) {
			// the network's change on top of that base guess; the kernel
			// keeps whichever of the two has the smaller FP64 residual
			CK(cudaMemcpyAsync(c->d_cand, c->d, nn * sizeof(double2), cudaMemcpyDeviceToDevice, c->st));
			CK(cudaMemcpyAsync(c->p_cand, c->p, ne * sizeof(double), cudaMemcpyDeviceToDevice, c->st));
			int rc = cnn_forward_dev(c->gnet, c->gw, c->gX, c->st);
			if (rc)
				return rc;
			float *Y = const_cast<float *>(cnn_output(c->gnet, c->gw));
			guess_smooth(c->st, c->gnc + 1, f.guess_smooth, Y, c->gYs);
			guess_apply(c->st, N0, c->gs, Y, c->gscale, mask0, c->d_cand, c->p_cand, c->d, c->p);
			c->launches += 2 * (f.guess_smooth > 0 ? f.guess_smooth : 0);
			d_alt = c->d_cand;
			p_alt = c->p_cand;
			c->launches += 1 + cnn_layers(c->gnet);
		}
		if (feat)
			c->launches += 2;
		CK(cudaGetLastError());
		CK(cudaEventRecord(c->ev[6], c->st));
		c->gtimed = 1;
	}
	c->mgf.d_alt = d_alt;
	c->mgf.p_alt = p_alt;
	c->mgd.d_alt = d_alt;
	c->mgd.p_alt = p_alt;
	c->mgf.guess_force = c->mgd.guess_force = c->gmode == MCLG_GUESS_FORCED;
	c->g_extrap = extrap;
	c->g_feat = feat;
	return MCLG_OK;
}

static int stokes_mg_finish(mclg_ctx *c)
{
	const int N0 = c->mgf.N0 ? c->mgf.N0 : c->mgd.N0;
	const bool track = c->d_h1 != NULL, extrap = c->g_extrap, feat = c->g_feat;
	if (track) {
		if (feat) {
			// target: the converged solution minus the base guess (extrapolation or the last solution)
			guess_target(c->st, N0, c->gs, c->d, c->p, c->d_h1, c->p_h1, extrap ? c->d_h2 : nullptr,
			             extrap ? c->p_h2 : nullptr, c->gscale, c->gYt);
			c->gsample = 1;
			c->launches++;
		}
		CK(cudaGetLastError());
		c->ghist++;
	}
	return MCLG_OK;
}

static int launch_stokes_mg(mclg_ctx *c)
{
	int rc = stokes_mg_prepare(c);
	if (rc)
		return rc;
	const dim3 grid(solver_grid(c, c->coop_mg));
	if (c->cfg.precision == 2) {
		void *args[] = {&c->mgd};
		CK(cudaLaunchCooperativeKernel(stokes_mg_kernel(1), grid, dim3(kBlock), args, 0, c->st));
	} else {
		void *args[] = {&c->mgf};
		CK(cudaLaunchCooperativeKernel(stokes_mg_kernel(0), grid, dim3(kBlock), args, 0, c->st));
	}
	c->launches++;
	return stokes_mg_finish(c);
}

// Switch the network off for 16 steps after 3 consecutive judged steps on which
// it did not pay: its guess lost the residual test, or won it but took more
// inner iterations than the last step solved from the previous solution.
static void guess_bookkeeping(mclg_ctx *c)
{
	if (c->gmode != MCLG_GUESS_LEARNED || c->cfg.precision == 0)
		return;   // MCLG_GUESS_FORCED never switches the network off
	const StepScalars &s = *c->sc_host;
	if (s.guess_used == 1) {
		if (c->git_prev >= 0 && s.cg_cycles > c->git_prev)
			c->gbad++;
		else
			c->gbad = 0;
	} else {
		if (s.guess_used == 0)   // judged, and the previous solution was the better start
			c->gbad++;
		c->git_prev = s.cg_cycles;
		if (c->goff > 0)
			c->goff--;
	}
	if (c->gbad >= 3) {
		c->goff = 16;
		c->gbad = 0;
	}
}

extern "C" {
static int launch_uzawa(mclg_ctx *c);
}

static int launch_stokes(mclg_ctx *c)
{
	if (c->cfg.precision == 0)
		return launch_uzawa(c);
	return c->qt_on ? launch_stokes_qt(c) : launch_stokes_mg(c);
}

extern "C" {

const char *mclg_status_string(int s)
{
	switch (s) {
	case MCLG_OK: return "ok";
	case MCLG_CAP_REACHED: return "iteration cap reached";
	case MCLG_NAN: return "non-finite value in a solver";
	case MCLG_BREAKDOWN: return "CG breakdown";
	case MCLG_BAD_INPUT: return "bad input";
	case MCLG_CUDA_ERROR: return "CUDA error";
	case MCLG_IO_ERROR: return "I/O error";
	case MCLG_NO_DEVICE: return "no CUDA device";
	default: return "unknown status";
	}
}

void mclg_destroy(mclg_ctx *c);

// leaves != NULL: the mesh is built from that leaf set instead of develop_mode
// The configuration the mesh is built with: the converged solvers' hierarchy on
// a refined mesh goes down to a grid of mg_coarse elements per side, so the
// mesh keeps levels that far down.
static mclg_config mesh_config(const mclg_config *cfg)
{
	mclg_config mcfg = *cfg;
	if (cfg->precision != 0) {
		int cl = 1;
		while ((1 << (cl + 1)) <= cfg->mg_coarse)
			cl++;
		if (cl < mcfg.mg_min_level)
			mcfg.mg_min_level = cl;
	}
	return mcfg;
}

// The host structures of a model on a leaf set: the mesh and, for a converged
// solver on a refined mesh, its constrained-space lists.  No device work.
// have_mesh: pb->mesh was numbered already (on the device), only the lists
// remain.
static int prebuild(Prebuilt *pb, const mclg_config *cfg, const int *leaves, long n, bool have_mesh = false)
{
	int rc = MCLG_OK;
	if (!have_mesh) {
		memset(pb, 0, sizeof *pb);
		const mclg_config mcfg = mesh_config(cfg);
		rc = mclg_mesh_build_leaves(&pb->mesh, &mcfg, leaves, n);
		if (rc != MCLG_OK)
			return rc;
	}
	const int top = pb->mesh.max_level - 1, lo = pb->mesh.min_level, nlev = top - lo + 1;
	if (cfg->precision != 0 && !pb->mesh.uniform && nlev >= 2 && nlev <= 16) {
		rc = mclg_qt_build(&pb->mesh, lo, pb->q);
		pb->nq = nlev;
	}
	return rc;
}

// pre: host structures built ahead (taken over; NULL: built here)
static int create_impl(mclg_ctx **out, const mclg_config *cfg, const int *leaves, long nleaves, Prebuilt *pre = NULL)
{
	if (out == NULL || cfg == NULL)
		return MCLG_BAD_INPUT;
	*out = NULL;
	if (cfg->lg_mul != 0) {
		mclg_set_error("the lg_mul path is not part of this engine (set lg_mul=0)");
		return MCLG_BAD_INPUT;
	}
	// grain-size rheology: the reference evolves the grain size on the first level its
	// viscosity() visits (mg_min_level); only on a single-level mesh is that the level
	// solved, and only the FP64 replica runs the reference's iteration on it
	if (cfg->grain_damage != 0 &&
	    (cfg->grain_damage != 1 || cfg->mg_min_level != cfg->level - 1 || cfg->precision != 0 ||
	     (strcmp(cfg->solver, "cg") != 0 && strcmp(cfg->solver, "jc") != 0))) {
		mclg_set_error("grain_damage=1 needs a single-level mesh (mg_min_level = level-1), precision=fp64 and "
		               "solver \"cg\" or \"jc\"");
		return MCLG_BAD_INPUT;
	}
	const bool ref_solver = strcmp(cfg->solver, "gs") == 0 || strcmp(cfg->solver, "mg") == 0;
	if (strcmp(cfg->solver, "cg") != 0 && strcmp(cfg->solver, "jc") != 0 && !ref_solver) {
		mclg_set_error("solver=\"%s\": the reference's solvers are \"cg\", \"jc\", \"gs\" and \"mg\"", cfg->solver);
		return MCLG_BAD_INPUT;
	}
	int ndev = 0;
	if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev < 1) {
		cudaGetLastError();
		mclg_set_error("no CUDA device visible");
		return MCLG_NO_DEVICE;
	}
	mclg_ctx *c = (mclg_ctx *)calloc(1, sizeof(mclg_ctx));
	if (c == NULL)
		return MCLG_BAD_INPUT;
	c->cfg = *cfg;
	const mclg_config mcfg = mesh_config(cfg);
	int rc = MCLG_OK;
	if (pre != NULL) {   // take the mesh over
		c->mesh = pre->mesh;
		memset(&pre->mesh, 0, sizeof pre->mesh);
	} else {
		rc = leaves ? mclg_mesh_build_leaves_device(&c->mesh, &mcfg, leaves, nleaves, NULL)
		            : mclg_mesh_build(&c->mesh, &mcfg);
	}
	if (rc != MCLG_OK) {
		mclg_mesh_free(&c->mesh);
		free(c);
		return rc;
	}
	c->fl = c->mesh.max_level - 1;
	*out = c;
#define CKD(call)                                  \
	do {                                           \
		cudaError_t e_ = (call);                   \
		if (e_ != cudaSuccess) {                   \
			int r_ = cuda_fail(e_, #call);         \
			mclg_destroy(c);                       \
			*out = NULL;                           \
			return r_;                             \
		}                                          \
	} while (0)
	CKD(cudaStreamCreateWithFlags(&c->st, cudaStreamNonBlocking));
	for (int i = 0; i < 7; i++)
		CKD(cudaEventCreate(&c->ev[i]));
	c->git_prev = -1;
	int dev = 0;
	CKD(cudaGetDevice(&dev));
	CKD(cudaDeviceGetAttribute(&c->num_sms, cudaDevAttrMultiProcessorCount, dev));
	int coop = 0;
	CKD(cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev));
	if (!coop) {
		mclg_set_error("device does not support cooperative launch");
		mclg_destroy(c);
		*out = NULL;
		return MCLG_NO_DEVICE;
	}
	rc = upload_level(c, c->fl);
	if (rc != MCLG_OK) {
		mclg_destroy(c);
		*out = NULL;
		return rc;
	}
	if ((rc = tables_once(c, kTabElem | kTabUzawa | kTabHeat, 0.0)) != MCLG_OK) {
		mclg_destroy(c);
		*out = NULL;
		return rc;
	}
	const size_t nn = c->L.nno, ne = c->L.nel, nbw = c->L.nbw;
	CKD(dalloc(&c->T, nn));
	CKD(dalloc(&c->vis, nn));
	CKD(dalloc(&c->buoy, nn));
	CKD(dalloc(&c->avg, (size_t)c->mesh.gnoz));
	CKD(dalloc(&c->stress, nn));
	CKD(dalloc(&c->stress_e, ne));
	CKD(dalloc(&c->V, nn));
	CKD(dalloc(&c->K, nbw * nn));
	CKD(dalloc(&c->F, nn));
	CKD(dalloc(&c->Kdiag, nn));
	CKD(dalloc(&c->idiag, nn));
	CKD(dalloc(&c->d, nn));
	CKD(dalloc(&c->u1, nn));
	CKD(dalloc(&c->Ah, nn));
	CKD(dalloc(&c->r, nn));
	CKD(dalloc(&c->s, nn));
	CKD(dalloc(&c->dd, nn));
	CKD(dalloc(&c->q, nn));
	CKD(dalloc(&c->xt, nn));
	CKD(dalloc(&c->bab, ne));
	CKD(dalloc(&c->p, ne));
	for (int i = 0; i < 8; i++)
		CKD(dalloc(&c->pe[i], ne));
	CKD(dalloc(&c->tau0, ne));
	CKD(dalloc(&c->tau1, ne));
	CKD(dalloc(&c->HK, nbw * nn));
	CKD(dalloc(&c->HC, nbw * nn));
	CKD(dalloc(&c->HA, nbw * nn));
	CKD(dalloc(&c->HF, nn));
	CKD(dalloc(&c->HB, nn));
	CKD(dalloc(&c->hx, nn));
	CKD(dalloc(&c->hidiag, nn));
	CKD(dalloc(&c->hr, nn));
	CKD(dalloc(&c->hs, nn));
	CKD(dalloc(&c->hd, nn));
	CKD(dalloc(&c->hq, nn));
	CKD(dalloc(&c->mins, 2));
	CKD(dalloc(&c->red_part, (size_t)2 * kMaxCoopBlocks * kRedWidth));
	CKD(dalloc(&c->sc, 1));
	CKD(dalloc(&c->tmpA, 2 * nn + ne));
	CKD(dalloc(&c->tmpB, 2 * nn + ne));
	CKD(cudaMallocHost((void **)&c->sc_host, sizeof(StepScalars)));
	if (cfg->grain_damage == 1 && mclg_grain_new(&c->grain) != MCLG_OK) {
		mclg_set_error("grain size: out of host memory");
		mclg_destroy(c);
		*out = NULL;
		return MCLG_BAD_INPUT;
	}
	CKD(cudaMemsetAsync(c->sc, 0, sizeof(StepScalars), c->st));
	CKD(cudaMemsetAsync(c->d, 0, nn * sizeof(double2), c->st));
	CKD(cudaMemsetAsync(c->p, 0, ne * sizeof(double), c->st));
	CKD(cudaMemsetAsync(c->V, 0, nn * sizeof(double2), c->st));
	CKD(cudaMemsetAsync(c->T, 0, nn * sizeof(double), c->st));
	if (ref_solver && cfg->precision == 0 && (rc = ref_setup(c)) != MCLG_OK) {
		mclg_destroy(c);
		*out = NULL;
		return rc;
	}
	const int work = (int)(nn > ne ? nn : ne);
	c->coop_uzawa = coop_blocks(uzawa_kernel_ptr(c->ref_kind != kRefNone), c->num_sms, work);
	c->coop_heat = coop_blocks(heat_cg_kernel_ptr(), c->num_sms, (int)nn);
	if (cfg->precision != 0 && !c->mesh.uniform) {
		rc = cfg->precision == 2 ? qt_setup<double>(c, c->qtd, pre) : qt_setup<float>(c, c->qtf, pre);
		if (rc == MCLG_OK)
			c->coop_qt = coop_blocks(qt_kernel(cfg->precision == 2), c->num_sms, (int)nn);
		if (rc == MCLG_OK && c->coop_qt < 1) {
			mclg_set_error("cooperative occupancy query failed");
			rc = MCLG_CUDA_ERROR;
		}
		if (rc == MCLG_OK && (cfg->warm_start == 3 || cfg->warm_start == 4))   // 4 acts as 3 here
			rc = alloc_history(c);
		if (rc != MCLG_OK) {
			mclg_destroy(c);
			*out = NULL;
			return rc;
		}
	} else if (cfg->precision != 0) {
		rc = cfg->precision == 2 ? mg_setup<double>(c, c->mgd) : mg_setup<float>(c, c->mgf);
		if (rc != MCLG_OK) {
			mclg_destroy(c);
			*out = NULL;
			return rc;
		}
		if ((rc = tables_once(c, kTabMg | kTabOp, c->mesh.dz[c->fl] / c->mesh.dx[c->fl])) != MCLG_OK) {
			mclg_destroy(c);
			*out = NULL;
			return rc;
		}
		c->coop_mg = coop_blocks(stokes_mg_kernel(cfg->precision == 2), c->num_sms, 1 << 30);
		if ((cfg->warm_start == 3 || cfg->warm_start == 4) && (rc = alloc_history(c)) != MCLG_OK) {
			mclg_destroy(c);
			*out = NULL;
			return rc;
		}
	}
	if (c->coop_uzawa < 1 || c->coop_heat < 1) {
		mclg_set_error("cooperative occupancy query failed");
		mclg_destroy(c);
		*out = NULL;
		return MCLG_CUDA_ERROR;
	}
	CKD(cudaStreamSynchronize(c->st));
	return MCLG_OK;
#undef CKD
}

int mclg_create(mclg_ctx **out, const mclg_config *cfg)
{
	return create_impl(out, cfg, NULL, 0);
}

int mclg_create_leaves(mclg_ctx **out, const mclg_config *cfg, const int *leaves, size_t n)
{
	if (out == NULL || cfg == NULL || leaves == NULL)
		return MCLG_BAD_INPUT;
	return create_impl(out, cfg, leaves, (long)n);
}

static void remesh_job_free(mclg_ctx *c);

void mclg_destroy(mclg_ctx *c)
{
	if (c == NULL)
		return;
	writer_free(c->writer);   // pending outputs are written first
	mclg_grain_delete(c->grain);
	remesh_job_free(c);
	if (c->st)
		cudaStreamSynchronize(c->st);
	free_level_buf(c->lb);
	for (int k = 0; k < MCLG_MAX_LEVEL; k++)
		free_level_buf(c->lvl_lb[k]);
	for (int i = 0; i < c->ref_nptr; i++)
		cudaFree(c->ref_ptr[i]);
	free(c->ref_ptr);
	void *ptrs[] = {c->T, c->vis, c->buoy, c->avg, c->stress, c->stress_e, c->V,
	                c->K, c->F, c->Kdiag, c->idiag, c->d, c->u1, c->Ah, c->r, c->s, c->dd, c->q, c->xt, c->bab,
	                c->p, c->tau0, c->tau1, c->HK, c->HC, c->HF, c->HA, c->HB, c->hx, c->hidiag, c->hr, c->hs,
	                c->hd, c->hq, c->mins, c->red_part, c->sc, c->tmpA, c->tmpB};
	for (size_t i = 0; i < sizeof ptrs / sizeof ptrs[0]; i++)
		if (ptrs[i])
			cudaFree(ptrs[i]);
	for (int i = 0; i < 8; i++)
		if (c->pe[i])
			cudaFree(c->pe[i]);
	for (int i = 0; i < c->mg_nptr; i++)
		cudaFree(c->mg_ptr[i]);
	if (c->sc_host)
		cudaFreeHost(c->sc_host);
	for (int i = 0; i < 7; i++)
		if (c->ev[i])
			cudaEventDestroy(c->ev[i]);
	void *gptrs[] = {c->d_h1, c->d_h2, c->d_h3, c->d_cand, c->p_h1, c->p_h2, c->p_h3, c->p_cand, c->gscale, c->gX,
	                 c->gYt, c->gYs};
	for (void *q : gptrs)
		if (q)
			cudaFree(q);
	cnn_work_free(c->gw);
	if (c->st && !c->st_borrowed)
		cudaStreamDestroy(c->st);
	mclg_mesh_free(&c->mesh);
	free(c);
}


int mclg_initial_temperature(mclg_ctx *c)
{
	if (c == NULL)
		return MCLG_BAD_INPUT;
	const mclg_level &H = c->mesh.lev[c->fl];
	std::vector<double> T(H.nno);
	int rc = mclg_host_initial_temperature(&c->mesh, &c->cfg, c->fl, T.data());
	if (rc != MCLG_OK)
		return rc;
	CK(cudaMemcpyAsync(c->T, T.data(), T.size() * sizeof(double), cudaMemcpyHostToDevice, c->st));
	CK(cudaStreamSynchronize(c->st));
	c->timestep = 0;
	double zero = 0.0;
	CK(cudaMemcpy(&c->sc->model_time, &zero, sizeof zero, cudaMemcpyHostToDevice));
	return MCLG_OK;
}

static int launch_buoy_vis(mclg_ctx *c)
{
	const mclg_config &f = c->cfg;
	k_buoy_rowavg<<<c->mesh.gnoz, kBlock, 0, c->st>>>(c->L, c->T, f.Rayleigh, c->avg);
	int rc = check_launch(c, "k_buoy_rowavg");
	if (rc)
		return rc;
	k_buoy_vis<<<blocks_for(c->L.nno), kBlock, 0, c->st>>>(c->L, c->T, f.Rayleigh, c->avg, f.A, f.refT,
	                                                       f.lower_mantle_jump, f.vis_min, f.vis_max, c->buoy,
	                                                       c->vis);
	return check_launch(c, "k_buoy_vis");
}

int mclg_buoyancy_force(mclg_ctx *c)
{
	if (c == NULL)
		return MCLG_BAD_INPUT;
	return launch_buoy_vis(c);
}

// grain_damage=1, after the exponential viscosity (Viscosity.c:19-20): the
// grain-size routine on the host (mclg_grain.c) with this step's temperature,
// the last step's nodal stress and the model time; it leaves the viscosity of
// the nodes it integrates and the stress it scaled.
static int grain_step(mclg_ctx *c)
{
	if (c->grain == NULL)
		return MCLG_OK;
	const size_t nn = (size_t)c->L.nno;
	std::vector<double> T(nn), stress(nn), vis(nn);
	double mt = 0.0;
	CK(cudaMemcpyAsync(T.data(), c->T, nn * sizeof(double), cudaMemcpyDeviceToHost, c->st));
	CK(cudaMemcpyAsync(stress.data(), c->stress, nn * sizeof(double), cudaMemcpyDeviceToHost, c->st));
	CK(cudaMemcpyAsync(vis.data(), c->vis, nn * sizeof(double), cudaMemcpyDeviceToHost, c->st));
	CK(cudaMemcpyAsync(&mt, &c->sc->model_time, sizeof(double), cudaMemcpyDeviceToHost, c->st));
	CK(cudaStreamSynchronize(c->st));
	const mclg_config &f = c->cfg;
	const int rc = mclg_grain_update(c->grain, (int)nn, c->mesh.lev[c->fl].X, T.data(), stress.data(), vis.data(),
	                                 mt, f.Rayleigh, f.lowest_vis, f.highest_vis, 8);
	if (rc)
		return rc;
	CK(cudaMemcpyAsync(c->vis, vis.data(), nn * sizeof(double), cudaMemcpyHostToDevice, c->st));
	CK(cudaMemcpyAsync(c->stress, stress.data(), nn * sizeof(double), cudaMemcpyHostToDevice, c->st));
	CK(cudaStreamSynchronize(c->st));
	return MCLG_OK;
}

int mclg_viscosity(mclg_ctx *c)
{
	if (c == NULL)
		return MCLG_BAD_INPUT;
	const int rc = launch_buoy_vis(c);
	return rc ? rc : grain_step(c);
}

int mclg_velocity_pressure_KGF_matrix(mclg_ctx *c)
{
	if (c == NULL)
		return MCLG_BAD_INPUT;
	const int withK = c->cfg.precision == 0 || c->qt_on;
	k_assemble_stokes<<<blocks_for(c->L.nno), kBlock, 0, c->st>>>(c->L, c->vis, c->buoy, c->K, c->F, c->Kdiag,
	                                                               withK);
	int rc = check_launch(c, "k_assemble_stokes");
	if (rc || !withK)
		return rc;
	k_inv_diag2<<<blocks_for(c->L.nno), kBlock, 0, c->st>>>(c->L.nno, c->Kdiag, c->idiag);
	if ((rc = check_launch(c, "k_inv_diag2")))
		return rc;
	k_bab<<<blocks_for(c->L.nel), kBlock, 0, c->st>>>(c->L, c->Kdiag, c->bab);
	return check_launch(c, "k_bab");
}

static int status_from_bits(int bits)
{
	if (bits & 2)
		return MCLG_NAN;
	if (bits & 4)
		return MCLG_BREAKDOWN;
	if (bits & 1)
		return MCLG_CAP_REACHED;
	return MCLG_OK;
}

static int read_scalars(mclg_ctx *c)
{
	CK(cudaMemcpyAsync(c->sc_host, c->sc, sizeof(StepScalars), cudaMemcpyDeviceToHost, c->st));
	CK(cudaStreamSynchronize(c->st));
	return MCLG_OK;
}

static int launch_uzawa(mclg_ctx *c)
{
	const mclg_config &f = c->cfg;
	const size_t nn = c->L.nno;
	// initial_d_p (Solver.c:251-278): d = 0 every step; p = 0 unless kept
	CK(cudaMemsetAsync(c->d, 0, nn * sizeof(double2), c->st));
	if (!(c->p_initialized && f.AMR == 0 && f.zero_P == 0))
		CK(cudaMemsetAsync(c->p, 0, c->L.nel * sizeof(double), c->st));
	c->p_initialized = 1;
	CK(cudaMemsetAsync(&c->sc->status, 0, sizeof(int), c->st));
	UzawaArgs a;
	memset(&a, 0, sizeof a);
	a.L = c->L;
	a.K = c->K;
	a.idiag = c->idiag;
	a.F = c->F;
	a.bab = c->bab;
	a.d = c->d;
	a.u1 = c->u1;
	a.Ah = c->Ah;
	a.r = c->r;
	a.s = c->s;
	a.dd = c->dd;
	a.q = c->q;
	a.xt = c->xt;
	a.V = c->V;
	a.p = c->p;
	a.r0 = c->pe[0];
	a.r1 = c->pe[1];
	a.r2 = c->pe[2];
	a.z0 = c->pe[3];
	a.z1 = c->pe[4];
	a.s1 = c->pe[5];
	a.s2 = c->pe[6];
	a.Ahp = c->pe[7];
	a.red.part = c->red_part;
	a.red.flip = 0;
	a.sc = c->sc;
	a.max_citcom = f.max_citcom_cycle;
	a.max_cg = f.max_cg_cycle;
	a.precond = f.cg_precondition;
	a.check_v_only = f.check_v_only;
	a.solver_jc = strcmp(f.solver, "jc") == 0;
	a.auto_accuracy = f.auto_accuracy;
	a.neq = c->mesh.lev[c->fl].neq;
	a.citcom_accu = f.citcom_solver_accu;
	a.accuracy = f.accuracy;
	a.ref_kind = c->ref_kind;
	a.ref = c->ref_dev;
	void *args[] = {&a};
	CK(cudaLaunchCooperativeKernel(uzawa_kernel_ptr(c->ref_kind != kRefNone), dim3(c->coop_uzawa), dim3(kBlock), args, 0,
	                               c->st));
	c->launches++;
	return MCLG_OK;
}

static int launch_stress(mclg_ctx *c)
{
	k_stress_elem<<<blocks_for(c->L.nel), kBlock, 0, c->st>>>(c->L, c->vis, c->V, c->stress_e);
	int rc = check_launch(c, "k_stress_elem");
	if (rc)
		return rc;
	k_elem_to_node<<<blocks_for(c->L.nno), kBlock, 0, c->st>>>(c->L, c->stress_e, c->stress);
	return check_launch(c, "k_elem_to_node");
}

static void fill_stats_stokes(mclg_ctx *c, mclg_step_stats *st)
{
	if (st == NULL)
		return;
	const StepScalars &s = *c->sc_host;
	st->timestep = c->timestep;
	st->uzawa_cycles = s.uzawa_cycles;
	st->cg_cycles = s.cg_cycles;
	st->dv = s.dv;
	st->dp = s.dp;
	st->res_momentum = s.res_m;
	st->res_continuity = s.res_c;
	st->status = status_from_bits(s.status);
	st->refine_passes = s.refine_passes;
	st->guess_used = c->cfg.precision != 0 ? s.guess_used : -1;
	st->res_guess_learned = st->guess_used >= 0 ? s.res_learned : 0.0;
	st->res_guess_prev = st->guess_used >= 0 ? s.res_prev : 0.0;
	st->warm_alpha = c->cfg.warm_start == 4 ? s.warm_a : 0.0;
	st->warm_beta = c->cfg.warm_start == 4 ? s.warm_b : 0.0;
	for (int k = 0; k < 5; k++)
		(&st->remesh_ms_numbering)[k] = c->remesh_ms[k];
}

int mclg_solve_velocity_pressure(mclg_ctx *c, mclg_step_stats *st)
{
	if (c == NULL)
		return MCLG_BAD_INPUT;
	int rc = launch_stokes(c);
	if (rc)
		return rc;
	if ((rc = launch_stress(c)))
		return rc;
	if ((rc = read_scalars(c)))
		return rc;
	guess_bookkeeping(c);
	fill_stats_stokes(c, st);
	return MCLG_OK;
}

static int launch_heat(mclg_ctx *c)
{
	const mclg_config &f = c->cfg;
	const DevLevel &L = c->L;
	int rc;
	k_tau<<<blocks_for(L.nel), kBlock, 0, c->st>>>(L, c->V, f.accuracy, c->tau0, c->tau1, c->mins,
	                                                f.precision != 0);
	if ((rc = check_launch(c, "k_tau")))
		return rc;
	// the converged solvers take the heat rows with fewer FP64 operations (equal to
	// the reference's to the last bits); the FP64 replica keeps its operation order
	if (c->cfg.precision != 0)
		k_assemble_heat_fast<<<blocks_for(L.nno), kBlock, 0, c->st>>>(L, c->V, c->tau0, c->tau1, f.Q, c->HK, c->HC,
		                                                              c->HF);
	else
		k_assemble_heat<<<blocks_for(L.nno), kBlock, 0, c->st>>>(L, c->V, c->tau0, c->tau1, f.Q, c->HK, c->HC, c->HF);
	if ((rc = check_launch(c, "k_assemble_heat")))
		return rc;
	k_heat_dt<<<blocks_for(L.nel), kBlock, 0, c->st>>>(L, c->V, c->mins);
	if ((rc = check_launch(c, "k_heat_dt")))
		return rc;
	k_heat_system<<<blocks_for(L.nno), kBlock, 0, c->st>>>(L, c->mins, f.theta, c->T, c->HK, c->HC, c->HF, c->HA,
	                                                        c->HB, c->hx, c->hidiag, c->sc);
	if ((rc = check_launch(c, "k_heat_system")))
		return rc;
	HeatArgs a;
	memset(&a, 0, sizeof a);
	a.op.L = L;
	a.op.HA = c->HA;
	a.op.idiag = c->hidiag;
	a.B = c->HB;
	a.x = c->hx;
	a.r = c->hr;
	a.s = c->hs;
	a.d = c->hd;
	a.q = c->hq;
	a.red.part = c->red_part;
	a.red.flip = 0;
	a.sc = c->sc;
	a.max_cycle = 1000;
	a.precond = f.cg_precondition;
	a.accu = 1e-3;
	void *args[] = {&a};
	CK(cudaLaunchCooperativeKernel(heat_cg_kernel_ptr(), dim3(c->coop_heat), dim3(kBlock), args, 0, c->st));
	c->launches++;
	k_heat_writeback<<<blocks_for(L.nno), kBlock, 0, c->st>>>(L, c->hx, c->T);
	return check_launch(c, "k_heat_writeback");
}

int mclg_update_temperature(mclg_ctx *c, mclg_step_stats *st)
{
	if (c == NULL)
		return MCLG_BAD_INPUT;
	int rc = launch_heat(c);
	if (rc)
		return rc;
	if ((rc = read_scalars(c)))
		return rc;
	if (st) {
		st->heat_cg_cycles = c->sc_host->heat_cycles;
		st->dt = c->sc_host->dt;
		st->model_time = c->sc_host->model_time;
		int s2 = status_from_bits(c->sc_host->status);
		if (s2 != MCLG_OK && st->status == MCLG_OK)
			st->status = s2;
	}
	c->timestep++;
	return MCLG_OK;
}

int mclg_output_async(mclg_ctx *c, const char *dir, int timestep, int flags)
{
	if (c == NULL || (flags & ~(MCLG_OUT_TEXT | MCLG_OUT_BINARY)) != 0)
		return MCLG_BAD_INPUT;
	if (flags == 0)
		return MCLG_OK;
	if (c->writer == NULL)
		c->writer = writer_new();
	return writer_submit(c->writer, c->st, &c->mesh.lev[c->fl], dir ? dir : c->cfg.data_dir, timestep, flags, c->T,
	                     c->V, c->stress, c->vis, c->p, (size_t)c->L.nel, &c->sc->model_time);
}

int mclg_output_wait(mclg_ctx *c)
{
	if (c == NULL)
		return MCLG_BAD_INPUT;
	return c->writer ? writer_wait(c->writer) : MCLG_OK;
}

int mclg_output(mclg_ctx *c, const char *dir, int timestep)
{
	int rc = mclg_output_async(c, dir, timestep, MCLG_OUT_TEXT);
	return rc ? rc : mclg_output_wait(c);
}

int mclg_step(mclg_ctx *c, int write_output, mclg_step_stats *st)
{
	if (c == NULL)
		return MCLG_BAD_INPUT;
	mclg_step_stats local;
	if (st == NULL)
		st = &local;
	memset(st, 0, sizeof *st);
	const long long l0 = c->launches;
	int rc;
	CK(cudaEventRecord(c->ev[0], c->st));
	if ((rc = launch_buoy_vis(c)) || (rc = grain_step(c)))
		return rc;
	if ((rc = mclg_velocity_pressure_KGF_matrix(c)))
		return rc;
	CK(cudaEventRecord(c->ev[4], c->st));
	if ((rc = launch_stokes(c)))
		return rc;
	CK(cudaEventRecord(c->ev[5], c->st));
	if ((rc = launch_stress(c)))
		return rc;
	CK(cudaEventRecord(c->ev[1], c->st));
	if (write_output && c->cfg.save_spacing > 0 && c->timestep % c->cfg.save_spacing == 0) {
		if ((rc = mclg_output_async(c, NULL, c->timestep, MCLG_OUT_TEXT)))
			return rc;
	}
	CK(cudaEventRecord(c->ev[2], c->st));
	if ((rc = launch_heat(c)))
		return rc;
	CK(cudaEventRecord(c->ev[3], c->st));
	if ((rc = read_scalars(c)))
		return rc;
	guess_bookkeeping(c);
	fill_stats_stokes(c, st);
	const StepScalars &s = *c->sc_host;
	st->heat_cg_cycles = s.heat_cycles;
	st->dt = s.dt;
	st->model_time = s.model_time;
	float ms = 0.f;
	cudaEventElapsedTime(&ms, c->ev[0], c->ev[1]);
	st->ms_stokes = ms;
	cudaEventElapsedTime(&ms, c->ev[2], c->ev[3]);
	st->ms_heat = ms;
	cudaEventElapsedTime(&ms, c->ev[0], c->ev[3]);
	st->ms_total = ms;
	cudaEventElapsedTime(&ms, c->gtimed ? c->ev[6] : c->ev[4], c->ev[5]);
	st->solver_kernel_ms = ms;
	st->ms_guess = 0.0;
	if (c->gtimed) {
		cudaEventElapsedTime(&ms, c->ev[4], c->ev[6]);
		st->ms_guess = ms;
	}
	st->solver_kernel_launches = 1;
	st->kernel_launches = c->launches - l0;
	c->timestep++;
	return MCLG_OK;
}

int mclg_step_host(mclg_ctx *c, const double *T_in, double *T_out, double *V_out, double *P_out,
                   mclg_step_stats *st)
{
	if (c == NULL)
		return MCLG_BAD_INPUT;
	const size_t nn = c->L.nno, ne = c->L.nel;
	if (T_in)
		CK(cudaMemcpyAsync(c->T, T_in, nn * sizeof(double), cudaMemcpyHostToDevice, c->st));
	int rc = mclg_step(c, 0, st);
	if (rc)
		return rc;
	if (T_out)
		CK(cudaMemcpyAsync(T_out, c->T, nn * sizeof(double), cudaMemcpyDeviceToHost, c->st));
	if (V_out)
		CK(cudaMemcpyAsync(V_out, c->V, 2 * nn * sizeof(double), cudaMemcpyDeviceToHost, c->st));
	if (P_out)
		CK(cudaMemcpyAsync(P_out, c->p, ne * sizeof(double), cudaMemcpyDeviceToHost, c->st));
	CK(cudaStreamSynchronize(c->st));
	return MCLG_OK;
}

// ---- field access --------------------------------------------------------
static int field_info(mclg_ctx *c, int which, size_t *n, void **dptr, int *kind)
{
	const mclg_level &H = c->mesh.lev[c->fl];
	// kind: 0 node scalar, 1 element scalar, 2 velocity eq vector (node double2 on device),
	//       3 node double2 component 0, 4 component 1, 5 heat eq vector (node scalar)
	switch (which) {
	case MCLG_F_T: *n = H.nno; *dptr = c->T; *kind = 0; break;
	case MCLG_F_V0: *n = H.nno; *dptr = c->V; *kind = 3; break;
	case MCLG_F_V1: *n = H.nno; *dptr = c->V; *kind = 4; break;
	case MCLG_F_P: *n = H.nel; *dptr = c->p; *kind = 1; break;
	case MCLG_F_D: *n = H.neq; *dptr = c->d; *kind = 2; break;
	case MCLG_F_STRESS: *n = H.nno; *dptr = c->stress; *kind = 0; break;
	case MCLG_F_VIS: *n = H.nno; *dptr = c->vis; *kind = 0; break;
	case MCLG_F_BUOY: *n = H.nno; *dptr = c->buoy; *kind = 0; break;
	case MCLG_F_F: *n = H.neq; *dptr = c->F; *kind = 2; break;
	case MCLG_F_KDIAG: *n = H.neq; *dptr = c->Kdiag; *kind = 2; break;
	case MCLG_F_BAB: *n = H.nel; *dptr = c->bab; *kind = 1; break;
	case MCLG_F_TAU0: *n = H.nel; *dptr = c->tau0; *kind = 1; break;
	case MCLG_F_TAU1: *n = H.nel; *dptr = c->tau1; *kind = 1; break;
	case MCLG_F_HEAT_F: *n = H.heat_neq; *dptr = c->HF; *kind = 5; break;
	case MCLG_F_X0: *n = H.nno; *dptr = c->lb.X; *kind = 0; break;
	case MCLG_F_X1: *n = H.nno; *dptr = c->lb.X + H.nno; *kind = 0; break;
	default:
		mclg_set_error("unknown field %d", which);
		return MCLG_BAD_INPUT;
	}
	return MCLG_OK;
}

static int download_raw(mclg_ctx *c, void *dptr, size_t bytes, std::vector<double> &buf)
{
	buf.resize(bytes / sizeof(double) + 1);
	CK(cudaMemcpyAsync(buf.data(), dptr, bytes, cudaMemcpyDeviceToHost, c->st));
	CK(cudaStreamSynchronize(c->st));
	return MCLG_OK;
}

int mclg_get_field(mclg_ctx *c, int which, int lev, double *out, size_t n)
{
	if (c == NULL || out == NULL)
		return MCLG_BAD_INPUT;
	if (which == MCLG_F_GRAIN) {   // host state of the grain-size routine
		if (c->grain == NULL || (lev >= 0 && lev != c->fl)) {
			mclg_set_error("no grain size: grain_damage=1 keeps it for the finest level only");
			return MCLG_BAD_INPUT;
		}
		return mclg_grain_get(c->grain, out, n);
	}
	int k;
	if (coarse_level(c, lev, &k) && (which == MCLG_F_T || which == MCLG_F_VIS)) {   // a coarser level's T, vis
		const size_t need = (size_t)c->mesh.lev[lev].nno;
		if (n != need) {
			mclg_set_error("field %d of level %d has %zu entries, buffer has %zu", which, lev, need, n);
			return MCLG_BAD_INPUT;
		}
		CK(cudaMemcpyAsync(out, which == MCLG_F_T ? c->lvl_T[k] : c->lvl_vis[k], n * sizeof(double),
		                   cudaMemcpyDeviceToHost, c->st));
		CK(cudaStreamSynchronize(c->st));
		return MCLG_OK;
	}
	if (lev >= 0 && lev != c->fl) {
		mclg_set_error("only the finest level (%d) is resident on the device", c->fl);
		return MCLG_BAD_INPUT;
	}
	size_t need;
	void *dptr;
	int kind, rc;
	if ((rc = field_info(c, which, &need, &dptr, &kind)))
		return rc;
	if (n != need) {
		mclg_set_error("field %d has %zu entries, buffer has %zu", which, need, n);
		return MCLG_BAD_INPUT;
	}
	const mclg_level &H = c->mesh.lev[c->fl];
	const size_t nn = H.nno;
	std::vector<double> buf;
	if (kind == 0 || kind == 1) {
		CK(cudaMemcpyAsync(out, dptr, n * sizeof(double), cudaMemcpyDeviceToHost, c->st));
		CK(cudaStreamSynchronize(c->st));
		return MCLG_OK;
	}
	if (kind == 5) {
		if ((rc = download_raw(c, dptr, nn * sizeof(double), buf)))
			return rc;
		for (size_t A = 0; A < nn; A++)
			if (H.heat_id[A] >= 0)
				out[H.heat_id[A]] = buf[A];
		return MCLG_OK;
	}
	if ((rc = download_raw(c, dptr, 2 * nn * sizeof(double), buf)))
		return rc;
	if (kind == 3 || kind == 4) {
		for (size_t A = 0; A < nn; A++)
			out[A] = buf[2 * A + (kind - 3)];
		return MCLG_OK;
	}
	for (size_t A = 0; A < nn; A++)
		for (int d = 0; d < 2; d++) {
			const int eq = H.id[d * nn + A];
			if (eq >= 0)
				out[eq] = buf[2 * A + d];
		}
	return MCLG_OK;
}

int mclg_set_field(mclg_ctx *c, int which, int lev, const double *in, size_t n)
{
	if (c == NULL || in == NULL)
		return MCLG_BAD_INPUT;
	if (lev >= 0 && lev != c->fl) {
		mclg_set_error("only the finest level (%d) is resident on the device", c->fl);
		return MCLG_BAD_INPUT;
	}
	size_t need;
	void *dptr;
	int kind, rc;
	if ((rc = field_info(c, which, &need, &dptr, &kind)))
		return rc;
	if (n != need) {
		mclg_set_error("field %d has %zu entries, buffer has %zu", which, need, n);
		return MCLG_BAD_INPUT;
	}
	if (which != MCLG_F_T && which != MCLG_F_P && which != MCLG_F_D && which != MCLG_F_VIS &&
	    which != MCLG_F_V0 && which != MCLG_F_V1) {
		mclg_set_error("field %d is derived and cannot be set", which);
		return MCLG_BAD_INPUT;
	}
	const mclg_level &H = c->mesh.lev[c->fl];
	const size_t nn = H.nno;
	if (kind == 0 || kind == 1) {
		CK(cudaMemcpyAsync(dptr, in, n * sizeof(double), cudaMemcpyHostToDevice, c->st));
		CK(cudaStreamSynchronize(c->st));
		if (which == MCLG_F_P)
			c->p_initialized = 1;
		return MCLG_OK;
	}
	std::vector<double> buf;
	if ((rc = download_raw(c, dptr, 2 * nn * sizeof(double), buf)))
		return rc;
	if (kind == 3 || kind == 4) {
		for (size_t A = 0; A < nn; A++)
			buf[2 * A + (kind - 3)] = in[A];
	} else {
		for (size_t A = 0; A < nn; A++)
			for (int d = 0; d < 2; d++) {
				const int eq = H.id[d * nn + A];
				buf[2 * A + d] = eq >= 0 ? in[eq] : 0.0;
			}
	}
	CK(cudaMemcpyAsync(dptr, buf.data(), 2 * nn * sizeof(double), cudaMemcpyHostToDevice, c->st));
	CK(cudaStreamSynchronize(c->st));
	return MCLG_OK;
}

int mclg_host_mesh_get(const mclg_mesh *m, int which, int lev, int *out, size_t n);

int mclg_get_mesh(mclg_ctx *c, int which, int lev, int *out, size_t n)
{
	if (c == NULL)
		return MCLG_BAD_INPUT;
	return mclg_host_mesh_get(&c->mesh, which, lev, out, n);
}

// ---- single operators ----------------------------------------------------
static int eq_to_node(mclg_ctx *c, const double *x, double *dev, int lev = -1)
{
	const mclg_level &H = c->mesh.lev[lev < 0 ? c->fl : lev];
	const size_t nn = H.nno;
	std::vector<double> buf(2 * nn, 0.0);
	for (size_t A = 0; A < nn; A++)
		for (int d = 0; d < 2; d++) {
			const int eq = H.id[d * nn + A];
			if (eq >= 0)
				buf[2 * A + d] = x[eq];
		}
	CK(cudaMemcpyAsync(dev, buf.data(), 2 * nn * sizeof(double), cudaMemcpyHostToDevice, c->st));
	CK(cudaStreamSynchronize(c->st));
	return MCLG_OK;
}

static int node_to_eq(mclg_ctx *c, const double *dev, double *y, int lev = -1)
{
	const mclg_level &H = c->mesh.lev[lev < 0 ? c->fl : lev];
	const size_t nn = H.nno;
	std::vector<double> buf(2 * nn);
	CK(cudaMemcpyAsync(buf.data(), dev, 2 * nn * sizeof(double), cudaMemcpyDeviceToHost, c->st));
	CK(cudaStreamSynchronize(c->st));
	for (size_t A = 0; A < nn; A++)
		for (int d = 0; d < 2; d++) {
			const int eq = H.id[d * nn + A];
			if (eq >= 0)
				y[eq] = buf[2 * A + d];
		}
	return MCLG_OK;
}

static int check_lev(mclg_ctx *c, int lev)
{
	if (lev >= 0 && lev != c->fl) {
		mclg_set_error("only the finest level (%d) is resident on the device", c->fl);
		return MCLG_BAD_INPUT;
	}
	return MCLG_OK;
}

int mclg_stokes_matvec(mclg_ctx *c, int lev, const double *x, double *y)
{
	int k;
	if (c != NULL && x != NULL && y != NULL && coarse_level(c, lev, &k)) {   // K of a coarser level
		int rc = eq_to_node(c, x, c->tmpA, lev);
		if (rc)
			return rc;
		k_kmul<<<blocks_for(c->lvl_L[k].nno), kBlock, 0, c->st>>>(c->lvl_L[k], c->lvl_K[k], (const double2 *)c->tmpA,
		                                                            (double2 *)c->tmpB);
		if ((rc = check_launch(c, "k_kmul")))
			return rc;
		return node_to_eq(c, c->tmpB, y, lev);
	}
	if (c == NULL || x == NULL || y == NULL || check_lev(c, lev))
		return MCLG_BAD_INPUT;
	int rc = eq_to_node(c, x, c->tmpA);
	if (rc)
		return rc;
	k_kmul<<<blocks_for(c->L.nno), kBlock, 0, c->st>>>(c->L, c->K, (const double2 *)c->tmpA, (double2 *)c->tmpB);
	if ((rc = check_launch(c, "k_kmul")))
		return rc;
	return node_to_eq(c, c->tmpB, y);
}

int mclg_stokes_G(mclg_ctx *c, int lev, const double *p, double *y)
{
	if (c == NULL || p == NULL || y == NULL || check_lev(c, lev))
		return MCLG_BAD_INPUT;
	CK(cudaMemcpyAsync(c->tmpA, p, c->L.nel * sizeof(double), cudaMemcpyHostToDevice, c->st));
	k_gmul<<<blocks_for(c->L.nno), kBlock, 0, c->st>>>(c->L, c->tmpA, (double2 *)c->tmpB);
	int rc = check_launch(c, "k_gmul");
	if (rc)
		return rc;
	return node_to_eq(c, c->tmpB, y);
}

int mclg_stokes_GT(mclg_ctx *c, int lev, const double *x, double *p)
{
	if (c == NULL || x == NULL || p == NULL || check_lev(c, lev))
		return MCLG_BAD_INPUT;
	int rc = eq_to_node(c, x, c->tmpA);
	if (rc)
		return rc;
	k_gtmul<<<blocks_for(c->L.nel), kBlock, 0, c->st>>>(c->L, (const double2 *)c->tmpA, c->tmpB);
	if ((rc = check_launch(c, "k_gtmul")))
		return rc;
	CK(cudaMemcpyAsync(p, c->tmpB, c->L.nel * sizeof(double), cudaMemcpyDeviceToHost, c->st));
	CK(cudaStreamSynchronize(c->st));
	return MCLG_OK;
}

int mclg_heat_matvec(mclg_ctx *c, int which, const double *x, double *y)
{
	if (c == NULL || x == NULL || y == NULL || (which != MCLG_HEAT_K && which != MCLG_HEAT_C))
		return MCLG_BAD_INPUT;
	const mclg_level &H = c->mesh.lev[c->fl];
	const size_t nn = H.nno;
	std::vector<double> buf(nn, 0.0);
	for (size_t A = 0; A < nn; A++)
		if (H.heat_id[A] >= 0)
			buf[A] = x[H.heat_id[A]];
	CK(cudaMemcpyAsync(c->tmpA, buf.data(), nn * sizeof(double), cudaMemcpyHostToDevice, c->st));
	k_heat_mul<<<blocks_for(nn), kBlock, 0, c->st>>>(c->L, which == MCLG_HEAT_K ? c->HK : c->HC, c->tmpA, c->tmpB);
	int rc = check_launch(c, "k_heat_mul");
	if (rc)
		return rc;
	CK(cudaMemcpyAsync(buf.data(), c->tmpB, nn * sizeof(double), cudaMemcpyDeviceToHost, c->st));
	CK(cudaStreamSynchronize(c->st));
	for (size_t A = 0; A < nn; A++)
		if (H.heat_id[A] >= 0)
			y[H.heat_id[A]] = buf[A];
	return MCLG_OK;
}

}  // extern "C"

namespace mclg {
__global__ void k_inv_diag2(int n, const double2 *__restrict__ d, double2 *__restrict__ inv)
{
	const int i = blockIdx.x * blockDim.x + threadIdx.x;
	if (i >= n)
		return;
	const double2 v = d[i];
	inv[i] = make_double2(1.0 / v.x, 1.0 / v.y);
}
}  // namespace mclg

// ---- Stokes solve without allocation -----------------------------------------
// mclg_solve_velocity_pressure_noalloc: the FP64 Uzawa solve of
// mclg_solve_velocity_pressure, with every scratch vector taken from one
// file-scope device array instead of the context's own buffers.  It is for
// callers whose device memory is handed out up front by their host program
// (a memory planner that reserves the whole device at start-up, or a time
// loop where the latency and device synchronisation of cudaMalloc are not
// acceptable): the call itself allocates nothing.
//
// The array is sized for meshes of at most MCLG_NOALLOC_MAX_NODES nodes and
// MCLG_NOALLOC_MAX_ELEMS elements; every GPU that loads this library holds it
// until the process exits.  All calls share it and it keeps the last call's
// contents, so two calls whose work overlaps on the GPU (different streams or
// contexts at the same time) race on it; each call clears the scalars it
// needs zeroed before it starts.  In host code the array's name is only a
// host-side handle: its device address is looked up once per device with
// cudaGetSymbolAddress on the first call made while that device is current,
// so that first call should come before any stream capture.
namespace {
constexpr size_t kNoallocNodeVecs = 7;      // u1, Ah, r, s, dd, q, xt (double2 per node)
constexpr size_t kNoallocElemVecs = 9;      // r0, r1, r2, z0, z1, s1, s2, Ahp, stress_e
constexpr size_t kNoallocPartBytes = 2ull * kMaxCoopBlocks * kRedWidth * sizeof(double);
constexpr size_t kNoallocBytes = kNoallocNodeVecs * MCLG_NOALLOC_MAX_NODES * sizeof(double2) +
                                 kNoallocElemVecs * MCLG_NOALLOC_MAX_ELEMS * sizeof(double) + kNoallocPartBytes +
                                 256 + sizeof(StepScalars);
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoallocBytes];
constexpr int kNoallocMaxDevices = 64;
static unsigned char *g_noalloc_addr[kNoallocMaxDevices];
}  // namespace

extern "C" int mclg_solve_velocity_pressure_noalloc(mclg_ctx *c, mclg_step_stats *st)
{
	if (c == NULL)
		return MCLG_BAD_INPUT;
	if (c->cfg.precision != 0) {
		mclg_set_error("the allocation-free solve runs the FP64 replica (precision=fp64) only");
		return MCLG_BAD_INPUT;
	}
	const size_t nn = c->L.nno, ne = c->L.nel;
	if (nn > MCLG_NOALLOC_MAX_NODES || ne > MCLG_NOALLOC_MAX_ELEMS) {
		mclg_set_error("mesh of %zu nodes / %zu elements exceeds the allocation-free limit of %d nodes / %d elements",
		               nn, ne, MCLG_NOALLOC_MAX_NODES, MCLG_NOALLOC_MAX_ELEMS);
		return MCLG_BAD_INPUT;
	}
	int dev = 0;
	CK(cudaGetDevice(&dev));
	if (dev < 0 || dev >= kNoallocMaxDevices) {
		mclg_set_error("device %d is beyond the allocation-free table", dev);
		return MCLG_BAD_INPUT;
	}
	if (g_noalloc_addr[dev] == NULL) {
		void *p = NULL;
		CK(cudaGetSymbolAddress(&p, g_noalloc_scratch));
		g_noalloc_addr[dev] = (unsigned char *)p;
	}
	unsigned char *base = g_noalloc_addr[dev];
	double2 *nv[kNoallocNodeVecs];
	double *ev[kNoallocElemVecs];
	for (size_t i = 0; i < kNoallocNodeVecs; i++)
		nv[i] = (double2 *)(base + i * MCLG_NOALLOC_MAX_NODES * sizeof(double2));
	unsigned char *ebase = base + kNoallocNodeVecs * MCLG_NOALLOC_MAX_NODES * sizeof(double2);
	for (size_t i = 0; i < kNoallocElemVecs; i++)
		ev[i] = (double *)(ebase + i * MCLG_NOALLOC_MAX_ELEMS * sizeof(double));
	double *part = (double *)(ebase + kNoallocElemVecs * MCLG_NOALLOC_MAX_ELEMS * sizeof(double));
	StepScalars *sc = (StepScalars *)((unsigned char *)part + kNoallocPartBytes + 256 -
	                                  ((uintptr_t)((unsigned char *)part + kNoallocPartBytes) & 255u));

	const mclg_config &f = c->cfg;
	// initial_d_p (Solver.c:251-278), as in mclg_solve_velocity_pressure
	CK(cudaMemsetAsync(c->d, 0, nn * sizeof(double2), c->st));
	if (!(c->p_initialized && f.AMR == 0 && f.zero_P == 0))
		CK(cudaMemsetAsync(c->p, 0, ne * sizeof(double), c->st));
	c->p_initialized = 1;
	CK(cudaMemsetAsync(sc, 0, sizeof(StepScalars), c->st));
	// this solve reports its status through the array's scalars; a status that
	// an earlier regular solve left in the context's own scalars must not reach
	// the mclg_update_temperature that follows
	CK(cudaMemsetAsync(&c->sc->status, 0, sizeof(int), c->st));
	UzawaArgs a;
	memset(&a, 0, sizeof a);
	a.L = c->L;
	a.K = c->K;
	a.idiag = c->idiag;
	a.F = c->F;
	a.bab = c->bab;
	a.d = c->d;
	a.u1 = nv[0];
	a.Ah = nv[1];
	a.r = nv[2];
	a.s = nv[3];
	a.dd = nv[4];
	a.q = nv[5];
	a.xt = nv[6];
	a.V = c->V;
	a.p = c->p;
	a.r0 = ev[0];
	a.r1 = ev[1];
	a.r2 = ev[2];
	a.z0 = ev[3];
	a.z1 = ev[4];
	a.s1 = ev[5];
	a.s2 = ev[6];
	a.Ahp = ev[7];
	a.red.part = part;
	a.red.flip = 0;
	a.sc = sc;
	a.max_citcom = f.max_citcom_cycle;
	a.max_cg = f.max_cg_cycle;
	a.precond = f.cg_precondition;
	a.check_v_only = f.check_v_only;
	a.solver_jc = strcmp(f.solver, "jc") == 0;
	a.auto_accuracy = f.auto_accuracy;
	a.neq = c->mesh.lev[c->fl].neq;
	a.citcom_accu = f.citcom_solver_accu;
	a.accuracy = f.accuracy;
	a.ref_kind = c->ref_kind;
	a.ref = c->ref_dev;
	void *args[] = {&a};
	CK(cudaLaunchCooperativeKernel(uzawa_kernel_ptr(c->ref_kind != kRefNone), dim3(c->coop_uzawa), dim3(kBlock), args, 0,
	                               c->st));
	c->launches++;
	// compute_stress with the element stresses in the same array
	k_stress_elem<<<blocks_for(ne), kBlock, 0, c->st>>>(c->L, c->vis, c->V, ev[8]);
	int rc = check_launch(c, "k_stress_elem");
	if (rc)
		return rc;
	k_elem_to_node<<<blocks_for(nn), kBlock, 0, c->st>>>(c->L, ev[8], c->stress);
	if ((rc = check_launch(c, "k_elem_to_node")))
		return rc;
	StepScalars hs;
	CK(cudaMemcpyAsync(&hs, sc, sizeof hs, cudaMemcpyDeviceToHost, c->st));
	CK(cudaStreamSynchronize(c->st));
	if (st) {
		st->timestep = c->timestep;
		st->uzawa_cycles = hs.uzawa_cycles;
		st->cg_cycles = hs.cg_cycles;
		st->dv = hs.dv;
		st->dp = hs.dp;
		st->res_momentum = hs.res_m;
		st->res_continuity = hs.res_c;
		st->status = status_from_bits(hs.status);
		st->refine_passes = 0;
		st->guess_used = -1;
	}
	return MCLG_OK;
}

// ---- learned initial guess --------------------------------------------------------
extern "C" int mclg_guess_set(mclg_ctx *c, int mode, int grid, mclg_cnn *net)
{
	if (c == NULL || mode < MCLG_GUESS_OFF || mode > MCLG_GUESS_FORCED)
		return MCLG_BAD_INPUT;
	if (mode == MCLG_GUESS_OFF) {
		c->gmode = MCLG_GUESS_OFF;
		c->gnet = NULL;
		c->gsample = 0;
		return MCLG_OK;
	}
	if (c->cfg.precision == 0 || (c->cfg.warm_start != 1 && c->cfg.warm_start != 3)) {
		mclg_set_error("the learned guess needs a converged solver (precision=mixed/fp64mg) with warm_start=1 or 3");
		return MCLG_BAD_INPUT;
	}
	const int N0 = c->mgf.N0 ? c->mgf.N0 : c->mgd.N0;
	if (grid < 2 || grid > N0 || N0 % grid != 0) {
		mclg_set_error("guess grid %d: need 2 <= grid <= %d dividing %d", grid, N0, N0);
		return MCLG_BAD_INPUT;
	}
	if (mode == MCLG_GUESS_LEARNED || mode == MCLG_GUESS_FORCED) {
		int cin = 0, cout = 0;
		if (net == NULL || cnn_channels(net, &cin, &cout) != MCLG_OK || cin != kGuessCin || cout != kGuessCout) {
			mclg_set_error("the learned guess needs a network with %d input and %d output channels", kGuessCin,
			               kGuessCout);
			return MCLG_BAD_INPUT;
		}
	}
	const size_t plane = (size_t)(grid + 1) * (grid + 1);
	int rc = alloc_history(c);
	if (rc)
		return rc;
	if (c->gX == NULL || c->gnc != grid) {
		if (c->gX)
			cudaFree(c->gX);
		if (c->gYt)
			cudaFree(c->gYt);
		if (c->gYs)
			cudaFree(c->gYs);
		c->gX = c->gYt = c->gYs = NULL;
		CK(dalloc(&c->gX, (size_t)kGuessCin * plane));
		CK(dalloc(&c->gYt, (size_t)kGuessCout * plane));
		CK(dalloc(&c->gYs, (size_t)kGuessCout * plane));
	}
	if (mode == MCLG_GUESS_LEARNED || mode == MCLG_GUESS_FORCED) {
		rc = cnn_work_ensure(net, c->gw, 1, grid + 1, grid + 1);
		if (rc)
			return rc;
	}
	c->gmode = mode;
	c->gnet = (mode == MCLG_GUESS_LEARNED || mode == MCLG_GUESS_FORCED) ? net : NULL;
	c->gs = N0 / grid;
	c->gnc = grid;
	c->goff = c->gbad = 0;
	c->git_prev = -1;
	return MCLG_OK;
}

extern "C" int mclg_guess_sample(mclg_ctx *c, float *x, size_t nx, float *y, size_t ny)
{
	if (c == NULL || x == NULL || y == NULL)
		return MCLG_BAD_INPUT;
	const size_t plane = (size_t)(c->gnc + 1) * (c->gnc + 1);
	if (c->gmode == MCLG_GUESS_OFF || !c->gsample) {
		mclg_set_error("no guess sample: the last solve did not follow two earlier solves with the guess on");
		return MCLG_BAD_INPUT;
	}
	if (nx != kGuessCin * plane || ny != kGuessCout * plane) {
		mclg_set_error("sample buffers have %zu and %zu entries, need %zu and %zu", nx, ny, kGuessCin * plane,
		               kGuessCout * plane);
		return MCLG_BAD_INPUT;
	}
	CK(cudaMemcpyAsync(x, c->gX, nx * sizeof(float), cudaMemcpyDeviceToHost, c->st));
	CK(cudaMemcpyAsync(y, c->gYt, ny * sizeof(float), cudaMemcpyDeviceToHost, c->st));
	CK(cudaStreamSynchronize(c->st));
	return MCLG_OK;
}

// ---- batched ensembles ------------------------------------------------------------
// Many independent models stepped together.  Every member is an ordinary
// context (own mesh, fields, hierarchy) on the ensemble's one stream; each
// step runs the members' element kernels, then ONE launch of the batched
// converged solver for all members (a block per model, taken from a queue
// ordered by decreasing mesh size), then the members' stress and heat kernels.
struct mclg_ensemble {
	int n;
	mclg_ctx **m;          // members, caller's order
	int *order;            // queue order: decreasing elements per side
	cudaStream_t st;
	cudaEvent_t ev[4];
	void *dargs;           // device MGArgs<TI>[n], queue order
	int *queue;            // device work counter
	int fp64;
	// autotuner: cluster sizes of the batched launch (blocks that solve one
	// model together), each timed on one step; the fastest per inner
	// iteration is kept
	static const int kCand = 5;
	int cs_cand[kCand], grid_cand[kCand];
	float cand_cost[kCand];
	int cs, grid;          // chosen cluster size and grid
	int qcs, qgrid;        // ... and those of the refined members' batched launch
	long long steps;
	int nbatch;            // members in the batched launch (uniform meshes)
	// refined members of at most kQtBatchNodes nodes: a second batched launch
	// of the refined-mesh solver (a model per cluster, largest first); larger
	// ones keep a cooperative launch of their own
	static const int kQtBatchNodes = 1 << 20;
	int *qorder, nqt;
	void *dargs_qt;        // device QtArgs<TI>[nqt], queue order
	int *queue_qt;
	cudaStream_t st_qt;    // the refined batch runs beside the uniform one
	cudaEvent_t ev_qt[2];
	int qcs_cand[kCand], qgrid_cand[kCand];
	int *amr, namr;        // larger refined members, solved one cooperative launch each
	// the whole step as a CUDA graph, captured once the autotuner has chosen and
	// every member's warm start is in its steady form, replayed afterwards
	cudaGraphExec_t graph;
	int graph_failed;
	long long graph_launches;   // kernels one replay launches
};

static cudaError_t launch_qt_batch(mclg_ensemble *e, int cs, int grid)
{
	cudaLaunchConfig_t lc;
	memset(&lc, 0, sizeof lc);
	lc.gridDim = dim3(grid);
	lc.blockDim = dim3(kBlock);
	lc.stream = e->st_qt;
	cudaLaunchAttribute at[1];
	at[0].id = cudaLaunchAttributeClusterDimension;
	at[0].val.clusterDim.x = cs;
	at[0].val.clusterDim.y = 1;
	at[0].val.clusterDim.z = 1;
	lc.attrs = at;
	lc.numAttrs = 1;
	void *kargs[] = {&e->dargs_qt, &e->nqt, &e->queue_qt};
	return cudaLaunchKernelExC(&lc, qt_batch_kernel(e->fp64), kargs);
}

static cudaError_t launch_batch(mclg_ensemble *e, int cs, int grid)
{
	cudaLaunchConfig_t lc;
	memset(&lc, 0, sizeof lc);
	lc.gridDim = dim3(grid);
	lc.blockDim = dim3(kBlock);
	lc.stream = e->st;
	cudaLaunchAttribute at[1];
	at[0].id = cudaLaunchAttributeClusterDimension;
	at[0].val.clusterDim.x = cs;
	at[0].val.clusterDim.y = 1;
	at[0].val.clusterDim.z = 1;
	lc.attrs = at;
	lc.numAttrs = 1;
	void *kargs[] = {&e->dargs, &e->nbatch, &e->queue};
	return cudaLaunchKernelExC(&lc, stokes_mg_batch_kernel(e->fp64), kargs);
}

// Blocks of a batched launch of `kern` with clusters of cs: as many clusters
// as can be resident at once, but no more than there are models (nmodels).
static int batch_grid(mclg_ensemble *e, int cs, void *kern, int nmodels)
{
	cudaLaunchConfig_t lc;
	memset(&lc, 0, sizeof lc);
	lc.gridDim = dim3(cs);
	lc.blockDim = dim3(kBlock);
	cudaLaunchAttribute at[1];
	at[0].id = cudaLaunchAttributeClusterDimension;
	at[0].val.clusterDim.x = cs;
	at[0].val.clusterDim.y = 1;
	at[0].val.clusterDim.z = 1;
	lc.attrs = at;
	lc.numAttrs = 1;
	int nc = 0;
	if (cudaOccupancyMaxActiveClusters(&nc, kern, &lc) != cudaSuccess) {
		cudaGetLastError();
		nc = cs <= 8 ? 2 * e->m[0]->num_sms / cs : 0;
	}
	if (nc < 1)
		return 0;
	if (nc > nmodels)
		nc = nmodels;
	return (nc < 1 ? 1 : nc) * cs;
}

extern "C" {

void mclg_ensemble_destroy(mclg_ensemble *e)
{
	if (e == NULL)
		return;
	if (e->st)
		cudaStreamSynchronize(e->st);
	if (e->graph)   // before the members: the graph records their events
		cudaGraphExecDestroy(e->graph);
	for (int i = 0; i < e->n; i++)
		if (e->m && e->m[i])
			mclg_destroy(e->m[i]);
	free(e->m);
	free(e->order);
	free(e->amr);
	free(e->qorder);
	if (e->dargs)
		cudaFree(e->dargs);
	if (e->queue)
		cudaFree(e->queue);
	if (e->dargs_qt)
		cudaFree(e->dargs_qt);
	if (e->queue_qt)
		cudaFree(e->queue_qt);
	for (int i = 0; i < 4; i++)
		if (e->ev[i])
			cudaEventDestroy(e->ev[i]);
	for (int i = 0; i < 2; i++)
		if (e->ev_qt[i])
			cudaEventDestroy(e->ev_qt[i]);
	if (e->st_qt) {
		cudaStreamSynchronize(e->st_qt);
		cudaStreamDestroy(e->st_qt);
	}
	if (e->st)
		cudaStreamDestroy(e->st);
	free(e);
}

static int ensemble_create(mclg_ensemble **out, const mclg_config *cfgs, const int *amr_levels, int n)
{
	if (out == NULL || cfgs == NULL || n < 1)
		return MCLG_BAD_INPUT;
	*out = NULL;
	for (int i = 0; i < n; i++)
		if (cfgs[i].precision == 0 || cfgs[i].precision != cfgs[0].precision) {
			mclg_set_error("ensemble member %d: every member needs the same converged solver (precision=mixed or "
			               "fp64mg)", i);
			return MCLG_BAD_INPUT;
		}
	mclg_ensemble *e = (mclg_ensemble *)calloc(1, sizeof(mclg_ensemble));
	if (e == NULL)
		return MCLG_BAD_INPUT;
	e->n = n;
	e->fp64 = cfgs[0].precision == 2;
	e->m = (mclg_ctx **)calloc((size_t)n, sizeof(mclg_ctx *));
	e->order = (int *)calloc((size_t)n, sizeof(int));
#define CKE(call)                                  \
	do {                                           \
		cudaError_t e_ = (call);                   \
		if (e_ != cudaSuccess) {                   \
			int r_ = cuda_fail(e_, #call);         \
			mclg_ensemble_destroy(e);              \
			return r_;                             \
		}                                          \
	} while (0)
	if (e->m == NULL || e->order == NULL) {
		mclg_ensemble_destroy(e);
		return MCLG_BAD_INPUT;
	}
	e->amr = (int *)calloc((size_t)n, sizeof(int));
	e->qorder = (int *)calloc((size_t)n, sizeof(int));
	if (e->amr == NULL || e->qorder == NULL) {
		mclg_ensemble_destroy(e);
		return MCLG_BAD_INPUT;
	}
	for (int i = 0; i < n; i++) {
		const int lv = amr_levels ? amr_levels[i] : 0;
		int rc;
		if (lv <= 0) {
			rc = mclg_create(&e->m[i], &cfgs[i]);
		} else {
			// a member with refinement: its configuration's grid is the base; the
			// mesh is refined up to lv levels by |grad T| > 0.2 max of its initial
			// temperature, as configuration 2's remeshing does
			mclg_config cf = cfgs[i];
			const int base = cf.level - 1;
			cf.level = base + lv + 1;
			const int F = cf.level - 1;
			if (lv > 4 || F >= MCLG_MAX_LEVEL - 1 || base < 1) {
				mclg_set_error("ensemble member %d: %d refinement levels on a %d-level grid", i, lv, base);
				mclg_ensemble_destroy(e);
				return MCLG_BAD_INPUT;
			}
			std::vector<int> leaves((size_t)1 << (2 * base));
			for (size_t k = 0; k < leaves.size(); k++)
				leaves[k] = (int)(k << (2 * (F - base)));
			rc = create_impl(&e->m[i], &cf, leaves.data(), (long)leaves.size());
			if (rc == MCLG_OK)
				rc = mclg_initial_temperature(e->m[i]);
			if (rc == MCLG_OK)
				rc = mclg_amr_remesh(e->m[i], 0.2, base, F, NULL);
		}
		if (rc != MCLG_OK) {
			mclg_ensemble_destroy(e);
			return rc;
		}
		if (e->m[i]->qt_on) {
			if (e->m[i]->L.nno <= mclg_ensemble::kQtBatchNodes)
				e->qorder[e->nqt++] = i;
			else
				e->amr[e->namr++] = i;
		}
	}
	CKE(cudaStreamCreateWithFlags(&e->st, cudaStreamNonBlocking));
	CKE(cudaStreamCreateWithFlags(&e->st_qt, cudaStreamNonBlocking));
	for (int i = 0; i < 4; i++)
		CKE(cudaEventCreate(&e->ev[i]));
	for (int i = 0; i < 2; i++)
		CKE(cudaEventCreateWithFlags(&e->ev_qt[i], cudaEventDisableTiming));
	// one stream for all members; the solver's element tables are shared
	// constants, so every member must have the same element aspect ratio
	int first = 0;
	while (first < n && e->m[first]->qt_on)
		first++;
	const mclg_ctx *c0 = e->m[first < n ? first : 0];
	const double r0 = c0->mesh.dz[c0->fl] / c0->mesh.dx[c0->fl];
	for (int i = 0; i < n; i++) {
		mclg_ctx *c = e->m[i];
		const double r = c->mesh.dz[c->fl] / c->mesh.dx[c->fl];
		if (!c->qt_on && fabs(r - r0) > 1e-12 * r0) {
			mclg_set_error("ensemble member %d: element aspect ratio %g differs from member 0's %g", i, r, r0);
			mclg_ensemble_destroy(e);
			return MCLG_BAD_INPUT;
		}
		if (c->qt_on && c->L.nno > mclg_ensemble::kQtBatchNodes)
			continue;   // large refined members keep their own stream: their steps run concurrently
		CKE(cudaStreamSynchronize(c->st));
		CKE(cudaStreamDestroy(c->st));
		c->st = e->st;
		c->st_borrowed = true;
	}
	e->nbatch = 0;
	for (int i = 0; i < n; i++)
		if (!e->m[i]->qt_on)
			e->order[e->nbatch++] = i;
	auto N0 = [&](int i) { return e->fp64 ? e->m[i]->mgd.N0 : e->m[i]->mgf.N0; };
	std::stable_sort(e->order, e->order + e->nbatch, [&](int a, int b) { return N0(a) > N0(b); });
	const size_t asz = e->fp64 ? sizeof(MGArgs<double>) : sizeof(MGArgs<float>);
	std::vector<unsigned char> h(asz * (size_t)(e->nbatch > 0 ? e->nbatch : 1));
	for (int k = 0; k < e->nbatch; k++) {
		mclg_ctx *c = e->m[e->order[k]];
		if (e->fp64)
			memcpy(&h[asz * k], &c->mgd, asz);
		else
			memcpy(&h[asz * k], &c->mgf, asz);
	}
	CKE(cudaMalloc(&e->dargs, asz * (size_t)(e->nbatch > 0 ? e->nbatch : 1)));
	CKE(cudaMemcpyAsync(e->dargs, h.data(), asz * (size_t)(e->nbatch > 0 ? e->nbatch : 1), cudaMemcpyHostToDevice,
	                    e->st));
	CKE(cudaMalloc((void **)&e->queue, sizeof(int)));
	// the batched refined members, largest first
	std::stable_sort(e->qorder, e->qorder + e->nqt,
	                 [&](int a, int b) { return e->m[a]->L.nno > e->m[b]->L.nno; });
	if (e->nqt > 0) {
		const size_t qsz = e->fp64 ? sizeof(QtArgs<double>) : sizeof(QtArgs<float>);
		std::vector<unsigned char> hq(qsz * (size_t)e->nqt);
		for (int k = 0; k < e->nqt; k++) {
			mclg_ctx *c = e->m[e->qorder[k]];
			if (e->fp64)
				memcpy(&hq[qsz * k], &c->qtd, qsz);
			else
				memcpy(&hq[qsz * k], &c->qtf, qsz);
		}
		CKE(cudaMalloc(&e->dargs_qt, hq.size()));
		CKE(cudaMemcpyAsync(e->dargs_qt, hq.data(), hq.size(), cudaMemcpyHostToDevice, e->st));
		CKE(cudaMalloc((void **)&e->queue_qt, sizeof(int)));
	}
	// 16 blocks per cluster is beyond the portable 8: allowed by an opt-in
	// attribute, dropped from the candidates where the device refuses it
	const bool allow16 = cudaFuncSetAttribute(stokes_mg_batch_kernel(e->fp64),
	                                          cudaFuncAttributeNonPortableClusterSizeAllowed, 1) == cudaSuccess;
	cudaGetLastError();
	const bool allow16q = cudaFuncSetAttribute(qt_batch_kernel(e->fp64),
	                                           cudaFuncAttributeNonPortableClusterSizeAllowed, 1) == cudaSuccess;
	cudaGetLastError();
	for (int k = 0; k < mclg_ensemble::kCand; k++) {
		e->cs_cand[k] = 1 << k;
		e->grid_cand[k] = (k < 4 || allow16) ? batch_grid(e, e->cs_cand[k], stokes_mg_batch_kernel(e->fp64),
		                                                  e->nbatch) : 0;
		if (e->grid_cand[k] < e->cs_cand[k]) {   // not launchable: fall back to the previous size
			e->cs_cand[k] = e->cs_cand[k - 1];
			e->grid_cand[k] = e->grid_cand[k - 1];
		}
		e->qcs_cand[k] = 1 << k;
		e->qgrid_cand[k] = (k < 4 || allow16q) ? batch_grid(e, e->qcs_cand[k], qt_batch_kernel(e->fp64), e->nqt)
		                                       : 0;
		if (e->qgrid_cand[k] < e->qcs_cand[k] && k > 0) {
			e->qcs_cand[k] = e->qcs_cand[k - 1];
			e->qgrid_cand[k] = e->qgrid_cand[k - 1];
		}
	}
	e->cs = 1;
	e->grid = e->grid_cand[0];
	e->qcs = e->qcs_cand[0];
	e->qgrid = e->qgrid_cand[0];
	CKE(cudaStreamSynchronize(e->st));
#undef CKE
	*out = e;
	return MCLG_OK;
}

int mclg_ensemble_create(mclg_ensemble **out, const mclg_config *cfgs, int n)
{
	return ensemble_create(out, cfgs, NULL, n);
}

int mclg_ensemble_create_amr(mclg_ensemble **out, const mclg_config *cfgs, const int *amr_levels, int n)
{
	if (amr_levels == NULL)
		return MCLG_BAD_INPUT;
	return ensemble_create(out, cfgs, amr_levels, n);
}

int mclg_ensemble_graph(const mclg_ensemble *e)
{
	return e != NULL && e->graph != NULL;
}

int mclg_ensemble_size(const mclg_ensemble *e)
{
	return e ? e->n : 0;
}

int mclg_ensemble_member(mclg_ensemble *e, int i, mclg_ctx **ctx)
{
	if (e == NULL || ctx == NULL || i < 0 || i >= e->n)
		return MCLG_BAD_INPUT;
	*ctx = e->m[i];
	return MCLG_OK;
}

int mclg_ensemble_initial_temperature(mclg_ensemble *e)
{
	if (e == NULL)
		return MCLG_BAD_INPUT;
	for (int i = 0; i < e->n; i++) {
		int rc = mclg_initial_temperature(e->m[i]);
		if (rc)
			return rc;
	}
	return MCLG_OK;
}

// The work of one ensemble step, issued on the ensemble's stream (refined
// members fork onto their own streams and join back).
static int ensemble_issue(mclg_ensemble *e, int cs, int grid, int qcs, int qgrid)
{
	int rc;
	// large refined members: the whole step on the member's own stream, concurrent
	// with one another and with the batched members
	for (int k = 0; k < e->namr; k++) {
		mclg_ctx *c = e->m[e->amr[k]];
		CK(cudaStreamWaitEvent(c->st, e->ev[0], 0));
		if ((rc = launch_buoy_vis(c)) || (rc = mclg_velocity_pressure_KGF_matrix(c)) || (rc = launch_stokes_qt(c)) ||
		    (rc = launch_stress(c)) || (rc = launch_heat(c)))
			return rc;
		CK(cudaMemcpyAsync(c->sc_host, c->sc, sizeof(StepScalars), cudaMemcpyDeviceToHost, c->st));
		CK(cudaEventRecord(c->ev[5], c->st));
	}
	for (int i = 0; i < e->n; i++) {
		mclg_ctx *c = e->m[i];
		if (c->qt_on)
			continue;
		if ((rc = launch_buoy_vis(c)) || (rc = mclg_velocity_pressure_KGF_matrix(c)) || (rc = stokes_mg_prepare(c)))
			return rc;
	}
	for (int k = 0; k < e->nqt; k++) {
		mclg_ctx *c = e->m[e->qorder[k]];
		if ((rc = launch_buoy_vis(c)) || (rc = mclg_velocity_pressure_KGF_matrix(c)) || (rc = stokes_qt_prepare(c)))
			return rc;
	}
	CK(cudaEventRecord(e->ev[1], e->st));
	// the refined batch on its own stream, beside the uniform batch
	if (e->nqt > 0) {
		CK(cudaEventRecord(e->ev_qt[0], e->st));
		CK(cudaStreamWaitEvent(e->st_qt, e->ev_qt[0], 0));
		CK(cudaMemsetAsync(e->queue_qt, 0, sizeof(int), e->st_qt));
		CK(launch_qt_batch(e, qcs, qgrid));
		CK(cudaEventRecord(e->ev_qt[1], e->st_qt));
	}
	if (e->nbatch > 0) {
		CK(cudaMemsetAsync(e->queue, 0, sizeof(int), e->st));
		CK(launch_batch(e, cs, grid));
	}
	if (e->nqt > 0)
		CK(cudaStreamWaitEvent(e->st, e->ev_qt[1], 0));
	CK(cudaEventRecord(e->ev[2], e->st));
	for (int i = 0; i < e->n; i++) {
		mclg_ctx *c = e->m[i];
		if (c->qt_on && c->L.nno > mclg_ensemble::kQtBatchNodes)
			continue;
		if (c->qt_on)
			stokes_qt_finish(c);
		else if ((rc = stokes_mg_finish(c)))
			return rc;
		if ((rc = launch_stress(c)) || (rc = launch_heat(c)))
			return rc;
		CK(cudaMemcpyAsync(c->sc_host, c->sc, sizeof(StepScalars), cudaMemcpyDeviceToHost, e->st));
	}
	for (int k = 0; k < e->namr; k++)
		CK(cudaStreamWaitEvent(e->st, e->m[e->amr[k]]->ev[5], 0));
	return MCLG_OK;
}

// Every member's warm start is in the form it keeps from now on (a graph
// replays exactly what it captured).
static bool ensemble_steady(const mclg_ensemble *e)
{
	for (int i = 0; i < e->n; i++) {
		const mclg_ctx *c = e->m[i];
		if (c->gmode != MCLG_GUESS_OFF || c->gnet != NULL)
			return false;
		if (c->d_h1 != NULL && c->ghist < 2)
			return false;
	}
	return true;
}

int mclg_ensemble_step(mclg_ensemble *e, mclg_step_stats *st, int *grid_used)
{
	if (e == NULL)
		return MCLG_BAD_INPUT;
	int rc;
	long long l0 = 0;
	for (int i = 0; i < e->n; i++)
		l0 += e->m[i]->launches;
	// autotuner: steps 2, 3, ... (the warm start settles after two steps) time one
	// candidate cluster size each; later steps use the cheapest per inner iteration
	int tune = -1;
	if (e->steps >= 2 && e->steps < 2 + mclg_ensemble::kCand)
		tune = (int)(e->steps - 2);
	const int cs = tune >= 0 ? e->cs_cand[tune] : e->cs;
	const int grid = tune >= 0 ? e->grid_cand[tune] : e->grid;
	const int qcs = tune >= 0 ? e->qcs_cand[tune] : e->qcs;
	const int qgrid = tune >= 0 ? e->qgrid_cand[tune] : e->qgrid;
	// capture the step once the tuning is over and the warm starts are steady
	if (tune < 0 && e->steps >= 2 + mclg_ensemble::kCand && e->graph == NULL && !e->graph_failed &&
	    ensemble_steady(e)) {
		cudaGraph_t g = NULL;
		std::vector<int> ghist0(e->n);
		std::vector<long long> launches0(e->n);
		for (int i = 0; i < e->n; i++) {
			ghist0[i] = e->m[i]->ghist;
			launches0[i] = e->m[i]->launches;
		}
		cudaError_t ce = cudaStreamBeginCapture(e->st, cudaStreamCaptureModeThreadLocal);
		if (ce == cudaSuccess) {
			ce = cudaEventRecord(e->ev[0], e->st);
			rc = ce == cudaSuccess ? ensemble_issue(e, cs, grid, qcs, qgrid) : MCLG_CUDA_ERROR;
			const cudaError_t ee = cudaStreamEndCapture(e->st, &g);   // always ends the capture
			if (ce == cudaSuccess)
				ce = ee;
			if (rc == MCLG_OK && ce == cudaSuccess && g != NULL)
				ce = cudaGraphInstantiate(&e->graph, g, 0);
			else if (ce == cudaSuccess)
				ce = cudaErrorUnknown;
		}
		if (g)
			cudaGraphDestroy(g);
		long long per_step = 0;
		for (int i = 0; i < e->n; i++) {   // the capture ran nothing: undo its bookkeeping
			per_step += e->m[i]->launches - launches0[i];
			e->m[i]->launches = launches0[i];
			e->m[i]->ghist = ghist0[i];
		}
		if (ce != cudaSuccess) {
			cudaGetLastError();
			e->graph = NULL;
			e->graph_failed = 1;
		} else {
			e->graph_launches = per_step;
		}
	}
	CK(cudaEventRecord(e->ev[0], e->st));
	if (e->graph != NULL) {
		CK(cudaGraphLaunch(e->graph, e->st));
		for (int i = 0; i < e->n; i++) {   // what the issue path counts on the host
			mclg_ctx *c = e->m[i];
			if (c->d_h1 != NULL)
				c->ghist++;
		}
		e->m[0]->launches += e->graph_launches;
	} else if ((rc = ensemble_issue(e, cs, grid, qcs, qgrid))) {
		return rc;
	}
	CK(cudaEventRecord(e->ev[3], e->st));
	CK(cudaStreamSynchronize(e->st));
	float ms_total = 0.f, ms_solver = 0.f;
	CK(cudaEventElapsedTime(&ms_total, e->ev[0], e->ev[3]));
	// the solver's own window (ev[1]..ev[2]) lies inside the graph when one is
	// replayed and is not timed then
	if (e->graph == NULL)
		CK(cudaEventElapsedTime(&ms_solver, e->ev[1], e->ev[2]));
	if (tune >= 0) {
		long long inner = 0;
		for (int i = 0; i < e->n; i++)
			inner += e->m[i]->sc_host->cg_cycles;
		e->cand_cost[tune] = ms_solver / (float)(inner > 0 ? inner : 1);
		if (tune == mclg_ensemble::kCand - 1) {
			int best = 0;
			for (int k = 1; k < mclg_ensemble::kCand; k++)
				if (e->cand_cost[k] < e->cand_cost[best])
					best = k;
			e->cs = e->cs_cand[best];
			e->grid = e->grid_cand[best];
			e->qcs = e->qcs_cand[best];
			e->qgrid = e->qgrid_cand[best];
		}
	}
	long long l1 = 0;
	for (int i = 0; i < e->n; i++)
		l1 += e->m[i]->launches;
	for (int i = 0; i < e->n; i++) {
		mclg_ctx *c = e->m[i];
		if (st) {
			mclg_step_stats *s = &st[i];
			memset(s, 0, sizeof *s);
			fill_stats_stokes(c, s);
			const StepScalars &h = *c->sc_host;
			s->heat_cg_cycles = h.heat_cycles;
			s->dt = h.dt;
			s->model_time = h.model_time;
			const int s2 = status_from_bits(h.status);
			if (s2 != MCLG_OK && s->status == MCLG_OK)
				s->status = s2;
			s->ms_total = ms_total;
			s->solver_kernel_ms = ms_solver;
			s->solver_kernel_launches = (e->nbatch > 0) + (e->nqt > 0) + e->namr;
			s->kernel_launches = (l1 - l0) + 1;
		}
		c->timestep++;
	}
	if (grid_used)
		*grid_used = cs;
	e->steps++;
	return MCLG_OK;
}

}  // extern "C"

// ---- |grad T| adaptive refinement ----------------------------------------------------
namespace mclg {
cudaError_t amr_tree_leaves(cudaStream_t st, int nel, const int *Mcode, const unsigned char *flags, int F, int base,
                            int target, std::vector<int> &leaves, long long *launches);
void amr_flags(cudaStream_t st, const DevLevel &L, const double *T, double frac, double *g, unsigned char *flags,
               double *gmax);
}

extern "C" {

int mclg_amr_flags(mclg_ctx *c, double frac, unsigned char *flags, size_t n, double *gmax)
{
	if (c == NULL || flags == NULL || !(frac >= 0.0))
		return MCLG_BAD_INPUT;
	if (n != (size_t)c->L.nel) {
		mclg_set_error("flag buffer has %zu entries, the mesh %d elements", n, c->L.nel);
		return MCLG_BAD_INPUT;
	}
	double *g = NULL, *dmax = NULL;
	unsigned char *df = NULL;
	cudaError_t e = cudaMalloc((void **)&g, (n + 1) * sizeof(double));
	if (e == cudaSuccess) e = cudaMalloc((void **)&df, n + 1);
	if (e == cudaSuccess) e = cudaMalloc((void **)&dmax, sizeof(double));
	if (e == cudaSuccess) {
		amr_flags(c->st, c->L, c->T, frac, g, df, dmax);
		c->launches += 2;
		e = cudaGetLastError();
	}
	double hm = 0.0;
	if (e == cudaSuccess) e = cudaMemcpyAsync(flags, df, n, cudaMemcpyDeviceToHost, c->st);
	if (e == cudaSuccess) e = cudaMemcpyAsync(&hm, dmax, sizeof(double), cudaMemcpyDeviceToHost, c->st);
	if (e == cudaSuccess) e = cudaStreamSynchronize(c->st);
	cudaFree(g);
	cudaFree(df);
	cudaFree(dmax);
	if (e != cudaSuccess)
		return cuda_fail(e, "mclg_amr_flags");
	if (gmax)
		*gmax = hm;
	return MCLG_OK;
}

// The refined tree's leaves from per-element flags on the device (df: device
// flags of the finest level's elements, NULL to compute them from T with frac).
static int device_leaves(mclg_ctx *c, const unsigned char *df_in, double frac, int base_level, int target_level,
                         std::vector<int> &leaves)
{
	const int F = c->mesh.max_level - 1;
	if (base_level < 0 || base_level > target_level || target_level > F) {
		mclg_set_error("refinement levels base=%d target=%d: need 0 <= base <= target <= %d", base_level,
		               target_level, F);
		return MCLG_BAD_INPUT;
	}
	const mclg_level &H = c->mesh.lev[c->fl];
	const size_t n = (size_t)H.nel;
	int *dM = NULL;
	double *g = NULL, *dmax = NULL;
	unsigned char *df = NULL;
	cudaError_t e = cudaMalloc((void **)&dM, (n + 1) * sizeof(int));
	if (e == cudaSuccess)
		e = cudaMemcpyAsync(dM, H.Mcode, n * sizeof(int), cudaMemcpyHostToDevice, c->st);
	if (e == cudaSuccess && df_in == NULL) {
		e = cudaMalloc((void **)&g, (n + 1) * sizeof(double));
		if (e == cudaSuccess) e = cudaMalloc((void **)&df, n + 1);
		if (e == cudaSuccess) e = cudaMalloc((void **)&dmax, sizeof(double));
		if (e == cudaSuccess) {
			amr_flags(c->st, c->L, c->T, frac, g, df, dmax);
			c->launches += 2;
			e = cudaGetLastError();
		}
	}
	if (e == cudaSuccess)
		e = amr_tree_leaves(c->st, (int)n, dM, df_in ? df_in : df, F, base_level, target_level, leaves, &c->launches);
	cudaFree(dM);
	cudaFree(g);
	cudaFree(df);
	cudaFree(dmax);
	if (e != cudaSuccess)
		return cuda_fail(e, "refined tree on the device");
	return MCLG_OK;
}

int mclg_amr_leaves(mclg_ctx *c, const unsigned char *flags, size_t n, int base_level, int target_level, int *leaves,
                    size_t cap, size_t *nleaves)
{
	if (c == NULL || flags == NULL || leaves == NULL || nleaves == NULL)
		return MCLG_BAD_INPUT;
	if (n != (size_t)c->L.nel) {
		mclg_set_error("flag buffer has %zu entries, the mesh %d elements", n, c->L.nel);
		return MCLG_BAD_INPUT;
	}
	unsigned char *df = NULL;
	cudaError_t e = cudaMalloc((void **)&df, n + 1);
	if (e == cudaSuccess)
		e = cudaMemcpyAsync(df, flags, n, cudaMemcpyHostToDevice, c->st);
	if (e != cudaSuccess) {
		cudaFree(df);
		return cuda_fail(e, "mclg_amr_leaves");
	}
	std::vector<int> out;
	const int rc = device_leaves(c, df, 0.0, base_level, target_level, out);
	cudaFree(df);
	if (rc)
		return rc;
	*nleaves = out.size();
	if (out.size() > cap) {
		mclg_set_error("the refined tree has %zu leaves, the buffer holds %zu", out.size(), cap);
		return MCLG_BAD_INPUT;
	}
	memcpy(leaves, out.data(), out.size() * sizeof(int));
	return MCLG_OK;
}

// Flags on the device, the new tree and the temperature transfer on the host,
// then the context is rebuilt on the new mesh in place: the handle stays
// valid, time step and model time carry over, velocity and pressure restart
// from zero.
// A remesh in two halves: begin() computes the flags, the new tree and the new
// mesh's numbering on the device and starts a worker thread that builds the
// solver's lists and the new context's device state (on a stream of its own); end()
// waits for it, carries the fields over and swaps the new state in.  Between
// them the caller may go on stepping the old mesh.
struct RemeshJob {
	std::thread th;
	mclg_config cfg;
	std::vector<int> leaves;
	Prebuilt pb;       // its mesh numbered on the device by begin()
	int device;        // the caller's device (the current device is per thread)
	mclg_ctx *n;       // the new context, created by the worker
	int rc;
	char err[512];
	double ms[3];      // numbering (begin), lists and state (worker)
};

static double ms_since(std::chrono::steady_clock::time_point t0)
{
	return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
}

// The worker: the host structures, then the new context's device state on a
// stream of its own (the old context keeps stepping on its stream meanwhile).
static void remesh_work(RemeshJob *j)
{
	j->rc = cudaSetDevice(j->device) == cudaSuccess ? MCLG_OK : MCLG_CUDA_ERROR;
	if (j->rc != MCLG_OK)
		mclg_set_error("remesh worker: cannot select device %d", j->device);
	auto t0 = std::chrono::steady_clock::now();
	if (j->rc == MCLG_OK)
		j->rc = prebuild(&j->pb, &j->cfg, j->leaves.data(), (long)j->leaves.size(), true);
	j->ms[1] = ms_since(t0);
	t0 = std::chrono::steady_clock::now();
	if (j->rc == MCLG_OK)
		j->rc = create_impl(&j->n, &j->cfg, j->leaves.data(), (long)j->leaves.size(), &j->pb);
	j->ms[2] = ms_since(t0);
	if (j->rc != MCLG_OK)
		snprintf(j->err, sizeof j->err, "%s", mclg_last_error());
}

static void remesh_job_free(mclg_ctx *c)
{
	if (c->rj == NULL)
		return;
	if (c->rj->th.joinable())
		c->rj->th.join();
	prebuilt_free(&c->rj->pb);
	if (c->rj->n != NULL)
		mclg_destroy(c->rj->n);
	delete c->rj;
	c->rj = NULL;
}

int mclg_amr_remesh_begin(mclg_ctx *c, double frac, int base_level, int target_level)
{
	if (c == NULL)
		return MCLG_BAD_INPUT;
	if (c->rj != NULL) {
		mclg_set_error("a remesh is already pending: finish it with mclg_amr_remesh_end");
		return MCLG_BAD_INPUT;
	}
	if (c->grain != NULL) {
		mclg_set_error("grain_damage=1 runs on a fixed single-level mesh: no remeshing");
		return MCLG_BAD_INPUT;
	}
	if (!(frac >= 0.0))
		return MCLG_BAD_INPUT;
	// flags and the new tree on the device
	std::vector<int> leaves;
	int rc = device_leaves(c, NULL, frac, base_level, target_level, leaves);
	if (rc)
		return rc;
	RemeshJob *j = new RemeshJob();
	j->cfg = c->cfg;
	j->leaves.swap(leaves);
	j->rc = MCLG_OK;
	j->err[0] = 0;
	j->n = NULL;
	memset(&j->pb, 0, sizeof j->pb);
	if (cudaGetDevice(&j->device) != cudaSuccess) {
		delete j;
		return cuda_fail(cudaErrorInvalidDevice, "mclg_amr_remesh_begin");
	}
	// the new mesh's numbering and hanging nodes on the device, on the model's
	// stream (after the step in flight); the worker builds the solver's lists
	const mclg_config mcfg = mesh_config(&c->cfg);
	const auto t0 = std::chrono::steady_clock::now();
	rc = mclg_mesh_build_leaves_device(&j->pb.mesh, &mcfg, j->leaves.data(), (long)j->leaves.size(), c->st);
	j->ms[0] = ms_since(t0);
	if (rc != MCLG_OK) {
		delete j;
		return rc;
	}
	c->rj = j;
	try {
		j->th = std::thread(remesh_work, j);
	} catch (...) {   // no thread: build here
		remesh_work(j);
	}
	return MCLG_OK;
}

int mclg_amr_remesh_end(mclg_ctx *c, size_t *nel_out)
{
	if (c == NULL || c->rj == NULL) {
		mclg_set_error("no remesh is pending");
		return MCLG_BAD_INPUT;
	}
	RemeshJob *j = c->rj;
	const auto t_wait = std::chrono::steady_clock::now();
	if (j->th.joinable())
		j->th.join();
	const double ms_wait = ms_since(t_wait);
	const auto t_carry = std::chrono::steady_clock::now();
	const double ms_job[3] = {j->ms[0], j->ms[1], j->ms[2]};
	if (j->rc != MCLG_OK) {
		const int rc = j->rc;
		mclg_set_error("%s", j->err);
		remesh_job_free(c);
		return rc;
	}
	const size_t ne = (size_t)c->L.nel, nn = (size_t)c->L.nno;
	const mclg_config cfg = c->cfg;
	mclg_ctx *n = j->n;   // created by the worker
	j->n = NULL;
	remesh_job_free(c);
	std::vector<double> T_old(nn), T_new((size_t)n->L.nno);
	int rc = mclg_get_field(c, MCLG_F_T, -1, T_old.data(), nn);
	if (rc == MCLG_OK)
		rc = mclg_amr_transfer(&c->mesh, T_old.data(), &n->mesh, T_new.data());
	if (rc == MCLG_OK)
		rc = mclg_set_field(n, MCLG_F_T, -1, T_new.data(), T_new.size());
	// converged solvers: the velocity (bilinear, as T) and the pressure (area mean of the
	// old pressure over the new element) start the first solve on the new mesh; the FP64
	// replica starts as the reference does (d = 0, p = 0 on a new mesh)
	const bool carry = cfg.precision != 0;
	const mclg_level &HN = n->mesh.lev[n->fl], &HO = c->mesh.lev[c->fl];
	const size_t nn2 = (size_t)HN.nno, ne2 = (size_t)HN.nel;
	std::vector<double> V_old(nn), V_new(nn2), d_new((size_t)(HN.neq > 0 ? HN.neq : 1), 0.0);
	for (int comp = 0; comp < 2 && rc == MCLG_OK && carry; comp++) {
		rc = mclg_get_field(c, comp ? MCLG_F_V1 : MCLG_F_V0, -1, V_old.data(), nn);
		if (rc == MCLG_OK)
			rc = mclg_amr_transfer(&c->mesh, V_old.data(), &n->mesh, V_new.data());
		if (rc == MCLG_OK)
			rc = mclg_set_field(n, comp ? MCLG_F_V1 : MCLG_F_V0, -1, V_new.data(), nn2);
		for (size_t A = 0; A < nn2 && rc == MCLG_OK; A++) {
			const int eq = HN.id[(size_t)comp * nn2 + A];
			if (eq >= 0)
				d_new[eq] = V_new[A];
		}
	}
	if (rc == MCLG_OK && carry && HN.neq > 0)
		rc = mclg_set_field(n, MCLG_F_D, -1, d_new.data(), (size_t)HN.neq);
	if (rc == MCLG_OK && carry) {
		std::vector<double> P_old(ne), P_new(ne2);
		rc = mclg_get_field(c, MCLG_F_P, -1, P_old.data(), ne);
		if (rc == MCLG_OK)
			rc = mclg_amr_transfer_elem(&c->mesh, P_old.data(), &n->mesh, P_new.data());
		if (rc == MCLG_OK)
			rc = mclg_set_field(n, MCLG_F_P, -1, P_new.data(), ne2);
		// the previous step's solution too, so that the extrapolated warm start
		// goes on across the remesh
		if (rc == MCLG_OK && c->d_h1 != NULL && n->d_h1 != NULL && c->ghist >= 2) {
			std::vector<double> D_old(2 * nn), D_new(2 * nn2, 0.0), comp_old(nn), comp_new(nn2), Ph(ne), Phn(ne2);
			cudaError_t e = cudaMemcpy(D_old.data(), c->d_h1, 2 * nn * sizeof(double), cudaMemcpyDeviceToHost);
			if (e == cudaSuccess)
				e = cudaMemcpy(Ph.data(), c->p_h1, ne * sizeof(double), cudaMemcpyDeviceToHost);
			if (e != cudaSuccess)
				rc = cuda_fail(e, "mclg_amr_remesh");
			for (int comp = 0; comp < 2 && rc == MCLG_OK; comp++) {
				for (size_t A = 0; A < nn; A++)
					comp_old[A] = D_old[2 * A + comp];
				rc = mclg_amr_transfer(&c->mesh, comp_old.data(), &n->mesh, comp_new.data());
				for (size_t A = 0; A < nn2 && rc == MCLG_OK; A++)
					if (HN.id[(size_t)comp * nn2 + A] >= 0)
						D_new[2 * A + comp] = comp_new[A];
			}
			if (rc == MCLG_OK)
				rc = mclg_amr_transfer_elem(&c->mesh, Ph.data(), &n->mesh, Phn.data());
			if (rc == MCLG_OK) {
				e = cudaMemcpy(n->d_h1, D_new.data(), 2 * nn2 * sizeof(double), cudaMemcpyHostToDevice);
				if (e == cudaSuccess)
					e = cudaMemcpy(n->p_h1, Phn.data(), ne2 * sizeof(double), cudaMemcpyHostToDevice);
				if (e != cudaSuccess)
					rc = cuda_fail(e, "mclg_amr_remesh");
				n->ghist = c->ghist;
				n->hist_shift = 2;
			}
		}
	}
	if (rc == MCLG_OK) {
		cudaError_t e = cudaMemcpyAsync(n->sc, c->sc, sizeof(StepScalars), cudaMemcpyDeviceToDevice, n->st);
		if (e == cudaSuccess)
			e = cudaStreamSynchronize(n->st);
		if (e != cudaSuccess)
			rc = cuda_fail(e, "mclg_amr_remesh");
	}
	if (rc) {
		mclg_destroy(n);
		return rc;
	}
	n->timestep = c->timestep;
	n->launches = c->launches;
	for (int k = 0; k < 3; k++)
		n->remesh_ms[k] = ms_job[k];
	n->remesh_ms[3] = ms_wait;
	n->remesh_ms[4] = ms_since(t_carry);   // without the release of the old state below
	// the caller's handle takes the new state; the old state is released
	mclg_ctx tmp;
	memcpy(&tmp, c, sizeof tmp);
	memcpy(c, n, sizeof tmp);
	memcpy(n, &tmp, sizeof tmp);
	mclg_destroy(n);
	if (nel_out)
		*nel_out = (size_t)c->L.nel;
	return MCLG_OK;
}

int mclg_amr_remesh(mclg_ctx *c, double frac, int base_level, int target_level, size_t *nel_out)
{
	const int rc = mclg_amr_remesh_begin(c, frac, base_level, target_level);
	return rc ? rc : mclg_amr_remesh_end(c, nel_out);
}

// ---- checkpoint / restart ------------------------------------------------------
// One binary file: a fixed header, the finest level's leaf start codes (the mesh
// of any develop_mode or remeshed tree), then the fields in node layout and the
// solver state a continued run reads: T, V, stress, d, p, the warm-start history
// of the converged solvers, and the learned guess's switch-off counters.  A
// 64-bit FNV-1a sum over everything before it closes the file.
static const char kCkpMagic[8] = {'M', 'C', 'L', 'G', 'C', 'K', 'P', '1'};

struct CkpHeader {
	char magic[8];
	int32_t version, level, min_level, nel, nno, neq, nleaves, timestep;
	int32_t p_initialized, has_history, ghist, goff, gbad, git_prev, precision;
	double model_time, length, height;
};

static uint64_t fnv1a(uint64_t h, const void *p, size_t n)
{
	const unsigned char *b = (const unsigned char *)p;
	for (size_t i = 0; i < n; i++) {
		h ^= b[i];
		h *= 1099511628211ull;
	}
	return h;
}

struct CkpFile {
	FILE *f;
	uint64_t h;
	bool ok;
	bool put(const void *p, size_t n)
	{
		h = fnv1a(h, p, n);
		ok = ok && fwrite(p, 1, n, f) == n;
		return ok;
	}
	bool get(void *p, size_t n)
	{
		ok = ok && fread(p, 1, n, f) == n;
		if (ok)
			h = fnv1a(h, p, n);
		return ok;
	}
};

// (device pointer, bytes) of each array the file holds, in file order
static int ckp_arrays(mclg_ctx *c, bool history, void **ptr, size_t *bytes)
{
	const size_t nn = c->L.nno, ne = c->L.nel;
	int n = 0;
	ptr[n] = c->T; bytes[n++] = nn * sizeof(double);
	ptr[n] = c->V; bytes[n++] = nn * sizeof(double2);
	ptr[n] = c->stress; bytes[n++] = nn * sizeof(double);
	ptr[n] = c->d; bytes[n++] = nn * sizeof(double2);
	ptr[n] = c->p; bytes[n++] = ne * sizeof(double);
	if (history) {
		ptr[n] = c->d_h1; bytes[n++] = nn * sizeof(double2);   // the previous step's solution
		ptr[n] = c->p_h1; bytes[n++] = ne * sizeof(double);
	}
	return n;
}

extern "C" int mclg_checkpoint_save(mclg_ctx *c, const char *path)
{
	if (c == NULL || path == NULL)
		return MCLG_BAD_INPUT;
	if (c->grain != NULL) {
		mclg_set_error("the grain-size state (grain_damage=1) is not part of a checkpoint");
		return MCLG_BAD_INPUT;
	}
	const mclg_level &H = c->mesh.lev[c->fl];
	CkpHeader hd;
	memset(&hd, 0, sizeof hd);
	memcpy(hd.magic, kCkpMagic, sizeof hd.magic);
	hd.version = 1;
	hd.level = c->mesh.max_level;
	hd.min_level = c->mesh.min_level;
	hd.nel = H.nel;
	hd.nno = H.nno;
	hd.neq = H.neq;
	hd.nleaves = H.nel;
	hd.timestep = c->timestep;
	hd.p_initialized = c->p_initialized;
	hd.has_history = c->d_h1 != NULL;
	hd.ghist = c->ghist;
	hd.goff = c->goff;
	hd.gbad = c->gbad;
	hd.git_prev = c->git_prev;
	hd.precision = c->cfg.precision;
	hd.length = c->mesh.length;
	hd.height = c->mesh.height;
	CK(cudaMemcpyAsync(&hd.model_time, &c->sc->model_time, sizeof(double), cudaMemcpyDeviceToHost, c->st));
	CK(cudaStreamSynchronize(c->st));
	std::vector<int> leaves(H.nel);
	for (int e = 0; e < H.nel; e++)
		leaves[e] = H.Mcode[e] >> MCLG_LEVEL_BITS;
	void *ptr[8];
	size_t bytes[8];
	const int na = ckp_arrays(c, hd.has_history, ptr, bytes);
	FILE *f = fopen(path, "wb");
	if (f == NULL) {
		mclg_set_error("cannot write %s", path);
		return MCLG_IO_ERROR;
	}
	CkpFile w = {f, 14695981039346656037ull, true};
	w.put(&hd, sizeof hd);
	w.put(leaves.data(), leaves.size() * sizeof(int));
	std::vector<unsigned char> buf;
	for (int i = 0; i < na && w.ok; i++) {
		buf.resize(bytes[i]);
		if (cudaMemcpyAsync(buf.data(), ptr[i], bytes[i], cudaMemcpyDeviceToHost, c->st) != cudaSuccess ||
		    cudaStreamSynchronize(c->st) != cudaSuccess) {
			fclose(f);
			return cuda_fail(cudaGetLastError(), "mclg_checkpoint_save");
		}
		w.put(buf.data(), bytes[i]);
	}
	const uint64_t sum = w.h;
	w.ok = w.ok && fwrite(&sum, 1, sizeof sum, f) == sizeof sum;
	if (fclose(f) != 0 || !w.ok) {
		mclg_set_error("writing %s failed", path);
		return MCLG_IO_ERROR;
	}
	return MCLG_OK;
}

// Reads the header and leaves; leaves may be NULL.
static int ckp_open(const char *path, FILE **fp, CkpFile &r, CkpHeader &hd, std::vector<int> *leaves)
{
	FILE *f = fopen(path, "rb");
	if (f == NULL) {
		mclg_set_error("cannot read %s", path);
		return MCLG_IO_ERROR;
	}
	r = {f, 14695981039346656037ull, true};
	if (!r.get(&hd, sizeof hd) || memcmp(hd.magic, kCkpMagic, sizeof hd.magic) != 0 || hd.version != 1 ||
	    hd.nleaves < 2 || hd.nno < 1 || hd.nel < 1) {
		fclose(f);
		mclg_set_error("%s is not a checkpoint of this engine", path);
		return MCLG_BAD_INPUT;
	}
	std::vector<int> lv((size_t)hd.nleaves);
	if (!r.get(lv.data(), lv.size() * sizeof(int))) {
		fclose(f);
		mclg_set_error("%s is truncated", path);
		return MCLG_IO_ERROR;
	}
	if (leaves)
		leaves->swap(lv);
	*fp = f;
	return MCLG_OK;
}

extern "C" int mclg_checkpoint_load(mclg_ctx *c, const char *path)
{
	if (c == NULL || path == NULL)
		return MCLG_BAD_INPUT;
	FILE *f = NULL;
	CkpFile r;
	CkpHeader hd;
	std::vector<int> leaves;
	int rc = ckp_open(path, &f, r, hd, &leaves);
	if (rc)
		return rc;
	const mclg_level &H = c->mesh.lev[c->fl];
	bool same = hd.level == c->mesh.max_level && hd.nel == H.nel && hd.nno == H.nno && hd.neq == H.neq &&
	            hd.length == c->mesh.length && hd.height == c->mesh.height;
	for (int e = 0; same && e < H.nel; e++)
		same = leaves[e] == (H.Mcode[e] >> MCLG_LEVEL_BITS);
	if (!same) {
		fclose(f);
		mclg_set_error("%s holds another mesh (%d elements at level %d; this model: %d at level %d)", path, hd.nel,
		               hd.level - 1, H.nel, c->fl);
		return MCLG_BAD_INPUT;
	}
	const bool hist = hd.has_history && c->d_h1 != NULL;
	void *ptr[8];
	size_t bytes[8];
	const int na = ckp_arrays(c, hd.has_history != 0, ptr, bytes);
	std::vector<std::vector<unsigned char>> data(na);
	for (int i = 0; i < na; i++) {
		data[i].resize(bytes[i]);
		if (!r.get(data[i].data(), bytes[i]))
			break;
	}
	uint64_t sum = 0;
	const uint64_t want = r.h;
	const bool tail = r.ok && fread(&sum, 1, sizeof sum, f) == sizeof sum;
	fclose(f);
	if (!tail || sum != want) {
		mclg_set_error("%s is truncated or corrupt (checksum)", path);
		return MCLG_IO_ERROR;
	}
	for (int i = 0; i < na; i++) {
		if (i >= 5 && !hist)   // a history the model does not keep (warm_start != 3)
			break;
		CK(cudaMemcpyAsync(ptr[i], data[i].data(), bytes[i], cudaMemcpyHostToDevice, c->st));
	}
	CK(cudaMemcpyAsync(&c->sc->model_time, &hd.model_time, sizeof(double), cudaMemcpyHostToDevice, c->st));
	CK(cudaStreamSynchronize(c->st));
	c->timestep = hd.timestep;
	c->p_initialized = hd.p_initialized;
	if (c->d_h1 != NULL)
		c->ghist = hist ? hd.ghist : 0;
	if (c->d_h3 != NULL) {
		// warm_start=4: the checkpoint holds the last two solutions, not a third;
		// the next solve starts from one difference, the one after from two
		const int ns = c->ghist < 2 ? c->ghist : 2;
		CK(cudaMemcpyAsync(&c->sc->nsolved, &ns, sizeof(int), cudaMemcpyHostToDevice, c->st));
		CK(cudaStreamSynchronize(c->st));
	}
	c->goff = hd.goff;
	c->gbad = hd.gbad;
	c->git_prev = hd.git_prev;
	return MCLG_OK;
}

extern "C" int mclg_get_time(mclg_ctx *c, int *timestep, double *model_time)
{
	if (c == NULL)
		return MCLG_BAD_INPUT;
	if (timestep)
		*timestep = c->timestep;
	if (model_time) {
		CK(cudaMemcpyAsync(model_time, &c->sc->model_time, sizeof(double), cudaMemcpyDeviceToHost, c->st));
		CK(cudaStreamSynchronize(c->st));
	}
	return MCLG_OK;
}

extern "C" int mclg_restart(mclg_ctx **out, const mclg_config *cfg, const char *path)
{
	if (out == NULL || cfg == NULL || path == NULL)
		return MCLG_BAD_INPUT;
	*out = NULL;
	FILE *f = NULL;
	CkpFile r;
	CkpHeader hd;
	std::vector<int> leaves;
	int rc = ckp_open(path, &f, r, hd, &leaves);
	if (rc)
		return rc;
	fclose(f);
	if (hd.level != cfg->level) {
		mclg_set_error("%s was written with level=%d, the configuration has level=%d", path, hd.level, cfg->level);
		return MCLG_BAD_INPUT;
	}
	mclg_ctx *c = NULL;
	if ((rc = create_impl(&c, cfg, leaves.data(), (long)leaves.size())) != MCLG_OK)
		return rc;
	if ((rc = mclg_checkpoint_load(c, path)) != MCLG_OK) {
		mclg_destroy(c);
		return rc;
	}
	*out = c;
	return MCLG_OK;
}

}  // extern "C"
