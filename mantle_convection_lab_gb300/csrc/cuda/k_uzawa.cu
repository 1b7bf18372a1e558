// FP64 Stokes solve: the reference's Uzawa iteration (citcom_solver,
// Solver.c:14-249) with its inner Jacobi-preconditioned CG (Conj_Grad,
// Solver.c:1589-1797) or Jacobi sweeps (jacobi, Solver.c:1800-1864), run as
// ONE persistent cooperative kernel per time step.  All loop control stays
// on the device; grid barriers replace the reference's MPI_Allreduce calls.
#include <math.h>
#include "cg_solve.cuh"

namespace mclg {

MCLG_SHAPE_UPLOAD(upload_shape_tables_uzawa)

// ---- the assembled operator in node-block-ELL form ----------------------
// y_A = sum_k K[k][A] x[nb[k][A]]: the reference's K_prod_d (Solver.c:360-386)
// over a row's sorted columns.
__device__ __forceinline__ void kmul_node(const DevLevel &L, const double4 *__restrict__ K,
                                          const double2 *__restrict__ x, int A, double &y0, double &y1)
{
	double s0 = 0.0, s1 = 0.0;
	for (int k = 0; k < L.nbw; k++) {
		const int B = L.nb[(size_t)k * L.nno + A];
		const double4 kb = K[(size_t)k * L.nno + A];
		const double2 xb = x[B];
		s0 += kb.x * xb.x;
		s0 += kb.y * xb.y;
		s1 += kb.z * xb.x;
		s1 += kb.w * xb.y;
	}
	y0 = vfree(L, A, 0) ? s0 : 0.0;
	y1 = vfree(L, A, 1) ? s1 : 0.0;
}

// Hanging-node overwrite (enforce_constrain_veq, Solver.c:1368-1482):
// x_h = (x_c0 + x_c1)/2 per component, a Dirichlet parent contributing its
// BC value.  A Dirichlet component of the hanging node itself is left alone
// (the reference writes it through index -1).
__device__ __forceinline__ void hang_one(const DevLevel &L, double2 *x, int h)
{
	const int ni = L.hang_ni[h], c0 = L.hang_ci0[h], c1 = L.hang_ci1[h];
	const double2 x0 = x[c0], x1 = x[c1];
	double t0 = (vfree(L, c0, 0) ? x0.x : L.vbcval[c0]) + (vfree(L, c1, 0) ? x1.x : L.vbcval[c1]);
	double t1 = (vfree(L, c0, 1) ? x0.y : L.vbcval[L.nno + c0]) + (vfree(L, c1, 1) ? x1.y : L.vbcval[L.nno + c1]);
	t0 *= 0.5;
	t1 *= 0.5;
	double2 xh = x[ni];
	if (vfree(L, ni, 0))
		xh.x = t0;
	if (vfree(L, ni, 1))
		xh.y = t1;
	x[ni] = xh;
}

struct StokesOp {
	static constexpr int NC = 2;
	DevLevel L;
	const double4 *K;
	const double2 *idiag;
	__device__ int nunits() const { return L.nno; }
	__device__ bool is_free(int A, int c) const { return vfree(L, A, c); }
	__device__ double inv_diag(int A, int c) const { return c == 0 ? idiag[A].x : idiag[A].y; }
	__device__ void apply(const double *x, int A, double (&y)[2]) const
	{
		kmul_node(L, K, reinterpret_cast<const double2 *>(x), A, y[0], y[1]);
	}
	__device__ int nhang() const { return L.nh; }
	__device__ void constrain(double *xv, int tid, int nth) const
	{
		double2 *x = reinterpret_cast<double2 *>(xv);
		if (L.hang_chained) {
			if (tid == 0)
				for (int h = 0; h < L.nh; h++)
					hang_one(L, x, h);
		} else {
			for (int h = tid; h < L.nh; h += nth)
				hang_one(L, x, h);
		}
	}
};


// jacobi (Solver.c:1800-1864): x = (b - offdiag x_old) / diag until the
// largest change is below accu; at most max_cycle sweeps.
__device__ int jacobi_solve(cg::grid_group &g, GridRed &red, const UzawaArgs &a, const double2 *b, double2 *x,
                            double2 *xt, double accu, int max_cycle, int *status)
{
	const DevLevel &L = a.L;
	const int tid = blockIdx.x * blockDim.x + threadIdx.x, nth = gridDim.x * blockDim.x;
	int cycle = 0;
	while (cycle < max_cycle) {
		for (int A = tid; A < L.nno; A += nth)
			xt[A] = x[A];
		g.sync();
		double mx[1] = {0.0};
		for (int A = tid; A < L.nno; A += nth) {
			double s0 = 0.0, s1 = 0.0, d0 = 1.0, d1 = 1.0;
			const int ks = L.self_slot[A];
			for (int k = 0; k < L.nbw; k++) {
				const int B = L.nb[(size_t)k * L.nno + A];
				const double4 kb = a.K[(size_t)k * L.nno + A];
				const double2 xb = xt[B];
				if (k == ks) {   // skip the row's own column (Solver.c:1823-1834)
					s0 += kb.y * xb.y;
					s1 += kb.z * xb.x;
					d0 = kb.x;
					d1 = kb.w;
				} else {
					s0 += kb.x * xb.x;
					s0 += kb.y * xb.y;
					s1 += kb.z * xb.x;
					s1 += kb.w * xb.y;
				}
			}
			double2 xn = x[A];
			const double2 bb = b[A];
			if (vfree(L, A, 0)) {
				xn.x = (bb.x - s0) / d0;
				mx[0] = fmax(mx[0], fabs(xn.x - xt[A].x));
			}
			if (vfree(L, A, 1)) {
				xn.y = (bb.y - s1) / d1;
				mx[0] = fmax(mx[0], fabs(xn.y - xt[A].y));
			}
			x[A] = xn;
		}
		cycle++;
		grid_reduce<1>(g, red, mx, 1u);
		if (mx[0] < accu)
			break;
	}
	if (cycle >= max_cycle && tid == 0)
		atomicOr(status, kStatCap);
	g.sync();
	return cycle;
}

// ---- the reference's own inner solvers: gauss_seidel and multigrid --------
// Both run in one thread block (block 0 of the cooperative Uzawa kernel; the
// other blocks wait at the next grid barrier).  The sequential sweep becomes
// a sweep over wavefronts: nodes of one wavefront share no matrix entry, and
// every node's lower neighbours sit in earlier wavefronts and its upper ones
// in later wavefronts, so each row reads exactly the values the sequential
// sweep reads.  Rows sum their columns in the reference's order with every
// product and sum rounded on its own (__dmul_rn / __dadd_rn: no fused
// multiply-add), so the arithmetic is the reference's.

// Both rows of node A (gauss_seidel, Solver.c:1883-1902): the row's own
// column skipped and taken as the diagonal; row 1 reads row 0's new value.
__device__ __forceinline__ void ref_gs_node(const RefLevel &R, const double2 *__restrict__ b, double2 *x, int A)
{
	const int nno = R.nno, ks = R.self_slot[A];
	double2 xa = x[A];
	if (R.vbc[A] != 'V') {
		double s = 0.0, dg = 1.0;
		for (int k = 0; k < R.nbw; k++) {
			const double4 kb = R.K[(size_t)k * nno + A];
			if (k == ks) {
				dg = kb.x;
				s = __dadd_rn(s, __dmul_rn(kb.y, xa.y));
				continue;
			}
			const int B = R.nb[(size_t)k * nno + A];
			if (B == A)   // padding slot
				continue;
			const double2 xb = x[B];
			s = __dadd_rn(s, __dmul_rn(kb.x, xb.x));
			s = __dadd_rn(s, __dmul_rn(kb.y, xb.y));
		}
		xa.x = (b[A].x - s) / dg;
	}
	if (R.vbc[nno + A] != 'V') {
		double s = 0.0, dg = 1.0;
		for (int k = 0; k < R.nbw; k++) {
			const double4 kb = R.K[(size_t)k * nno + A];
			if (k == ks) {
				s = __dadd_rn(s, __dmul_rn(kb.z, xa.x));
				dg = kb.w;
				continue;
			}
			const int B = R.nb[(size_t)k * nno + A];
			if (B == A)
				continue;
			const double2 xb = x[B];
			s = __dadd_rn(s, __dmul_rn(kb.z, xb.x));
			s = __dadd_rn(s, __dmul_rn(kb.w, xb.y));
		}
		xa.y = (b[A].y - s) / dg;
	}
	x[A] = xa;
}

// gauss_seidel (Solver.c:1866-1929): sweeps until the largest change is
// below accu, at most max_cycle.  Block-wide; returns the sweeps done.
__device__ int ref_gs(const RefLevel &R, const double2 *b, double2 *x, double accu, int max_cycle)
{
	const int tid = threadIdx.x, nth = blockDim.x;
	int cycle = 0;
	while (cycle < max_cycle) {
		for (int A = tid; A < R.nno; A += nth)
			R.xt[A] = x[A];
		__syncthreads();
		for (int w = 0; w < R.nwave; w++) {
			const int i1 = R.wave_off[w + 1];
			for (int i = R.wave_off[w] + tid; i < i1; i += nth)
				ref_gs_node(R, b, x, R.wave[i]);
			__syncthreads();
		}
		cycle++;
		double mx[1] = {0.0};
		for (int A = tid; A < R.nno; A += nth) {
			const double2 xn = x[A], xo = R.xt[A];
			if (R.vbc[A] != 'V')
				mx[0] = fmax(mx[0], fabs(xn.x - xo.x));
			if (R.vbc[R.nno + A] != 'V')
				mx[0] = fmax(mx[0], fabs(xn.y - xo.y));
		}
		block_reduce<1>(mx, 1u);
		if (mx[0] < accu)
			break;
	}
	return cycle;
}

// get_residual (Solver.c:1291-1317): res = b, minus each column's product in turn.
__device__ void ref_residual(const RefLevel &R, const double2 *__restrict__ b, const double2 *__restrict__ x,
                             double2 *__restrict__ res)
{
	const int nno = R.nno;
	for (int A = threadIdx.x; A < nno; A += blockDim.x) {
		const int ks = R.self_slot[A];
		double r0 = b[A].x, r1 = b[A].y;
		for (int k = 0; k < R.nbw; k++) {
			const int B = R.nb[(size_t)k * nno + A];
			if (B == A && k != ks)
				continue;
			const double4 kb = R.K[(size_t)k * nno + A];
			const double2 xb = x[B];
			r0 = __dsub_rn(r0, __dmul_rn(kb.x, xb.x));
			r0 = __dsub_rn(r0, __dmul_rn(kb.y, xb.y));
			r1 = __dsub_rn(r1, __dmul_rn(kb.z, xb.x));
			r1 = __dsub_rn(r1, __dmul_rn(kb.w, xb.y));
		}
		res[A] = make_double2(R.vbc[A] != 'V' ? r0 : 0.0, R.vbc[nno + A] != 'V' ? r1 : 0.0);
	}
}

// multigrid (Solver.c:668-713) with MG (Solver.c:715-768) unrolled into a
// descent and an ascent.  Below the finest level MG's x is G.err[lev]
// itself: interp_error overwrites the entries it sets and x += err then
// doubles every entry, as in the reference.  G.err is zeroed once per call,
// not per V-cycle.  Returns the V-cycles done.
__device__ int ref_mg(const RefMG &M, const double2 *b_top, double2 *x_top, double accu)
{
	const int tid = threadIdx.x, nth = blockDim.x, top = M.nlev - 1;
	for (int k = 0; k < M.nlev; k++)
		for (int A = tid; A < M.lev[k].nno; A += nth)
			M.lev[k].err[A] = make_double2(0.0, 0.0);
	__syncthreads();
	int cycle = 0;
	while (cycle < M.cycles) {
		const RefLevel &T = M.lev[top];
		for (int A = tid; A < T.nno; A += nth)   // multigrid's x_tmp
			T.rhs[A] = x_top[A];
		__syncthreads();
		for (int k = top; k > 0; k--) {
			const RefLevel &R = M.lev[k], &Lo = M.lev[k - 1];
			const double2 *b = k == top ? b_top : R.rhs;
			double2 *x = k == top ? x_top : R.err;
			ref_gs(R, b, x, accu, M.fine_it);
			ref_residual(R, b, x, R.res);
			__syncthreads();
			const double *ru = reinterpret_cast<const double *>(R.res);
			for (int A = tid; A < Lo.nno; A += nth) {   // project_res (Solver.c:770-783)
				const int u0 = Lo.prj[A], u1 = Lo.prj[Lo.nno + A];
				Lo.rhs[A] = make_double2(u0 >= 0 ? ru[u0] : 0.0, u1 >= 0 ? ru[u1] : 0.0);
			}
			__syncthreads();
		}
		ref_gs(M.lev[0], M.lev[0].rhs, M.lev[0].err, accu, 1000);
		for (int k = 1; k <= top; k++) {
			const RefLevel &R = M.lev[k], &Lo = M.lev[k - 1];
			const double2 *b = k == top ? b_top : R.rhs;
			double2 *x = k == top ? x_top : R.err;
			const double *el = reinterpret_cast<const double *>(Lo.err);
			double *eu = reinterpret_cast<double *>(R.err);
			for (int A = tid; A < R.nno; A += nth)   // interp_error (Solver.c:1029-1046)
				for (int c = 0; c < 2; c++) {
					const int n = R.itp_n[c * R.nno + A];
					if (n <= 0)
						continue;
					double s = 0.0;
					for (int i = 0; i < n; i++) {
						const int l = R.itp_src[(size_t)(i * 2 + c) * R.nno + A];
						if (l != -1)
							s = __dadd_rn(s, el[l]);
					}
					eu[2 * A + c] = s / n;
				}
			__syncthreads();
			for (int A = tid; A < R.nno; A += nth) {
				const double2 e = R.err[A];
				double2 xv = x[A];
				xv.x = __dadd_rn(xv.x, e.x);
				xv.y = __dadd_rn(xv.y, e.y);
				x[A] = xv;
			}
			__syncthreads();
			ref_gs(R, b, x, accu, M.coarse_it);
		}
		cycle++;
		double mx[1] = {0.0};   // check_convergency (Solver.c:1267-1289)
		for (int A = tid; A < T.nno; A += nth) {
			const double2 xn = x_top[A], xo = T.rhs[A];
			if (T.vbc[A] != 'V')
				mx[0] = fmax(mx[0], fabs(xn.x - xo.x));
			if (T.vbc[T.nno + A] != 'V')
				mx[0] = fmax(mx[0], fabs(xn.y - xo.y));
		}
		block_reduce<1>(mx, 1u);
		if (mx[0] < accu)
			break;
	}
	return cycle;
}

// REF: the kernel instance that runs the reference's gauss_seidel / multigrid
// (a separate instance keeps the CG instance's registers as they were).
template <bool REF>
__device__ int inner_solve(cg::grid_group &g, const UzawaArgs &a, GridRed &red, const StokesOp &op, double2 *b,
                           double2 *x, double accu, int *status)
{
	if (REF) {
		__shared__ int done;
		if (blockIdx.x == 0) {
			const int n = a.ref_kind == kRefMG ? ref_mg(*a.ref, b, x, accu)
			                                   : ref_gs(a.ref->lev[a.ref->nlev - 1], b, x, accu, 1000);
			if (threadIdx.x == 0)
				done = n;
		}
		g.sync();
		return blockIdx.x == 0 ? done : 0;
	}
	if (a.solver_jc)
		return jacobi_solve(g, red, a, b, x, a.xt, accu, 1000, status);
	return cg_solve(g, red, op, reinterpret_cast<const double *>(b), reinterpret_cast<double *>(x),
	                reinterpret_cast<double *>(a.r), reinterpret_cast<double *>(a.s),
	                reinterpret_cast<double *>(a.dd), reinterpret_cast<double *>(a.q), accu, a.max_cg,
	                a.precond != 0, false, status);
}

template <bool REF>
__global__ void __launch_bounds__(kBlock) k_uzawa(UzawaArgs a)
{
	cg::grid_group g = cg::this_grid();
	const DevLevel &L = a.L;
	const int tid = blockIdx.x * blockDim.x + threadIdx.x, nth = gridDim.x * blockDim.x;
	GridRed red = a.red;
	StokesOp op;
	op.L = a.L;
	op.K = a.K;
	op.idiag = a.idiag;
	int *status = &a.sc->status;
	double accu = a.accuracy;

	if (a.auto_accuracy) {  // Solver.c:40-51
		double f[1] = {0.0};
		for (int A = tid; A < L.nno; A += nth) {
			const double2 fa = a.F[A];
			f[0] += fa.x * fa.x + fa.y * fa.y;
		}
		grid_reduce<1>(g, red, f, 0u);
		accu = a.citcom_accu * sqrt(f[0] / a.neq);
	}

	// u1 = K d;  Ah = F - G p - u1  (Solver.c:67-77)
	for (int A = tid; A < L.nno; A += nth) {
		double k0, k1, g0, g1;
		kmul_node(L, a.K, a.d, A, k0, k1);
		gmul_node(L, a.p, A, g0, g1);
		const double2 f = a.F[A];
		a.u1[A] = make_double2(k0, k1);
		a.Ah[A] = make_double2(vfree(L, A, 0) ? f.x - g0 - k0 : 0.0, vfree(L, A, 1) ? f.y - g1 - k1 : 0.0);
	}
	g.sync();
	int cg_total = inner_solve<REF>(g, a, red, op, a.Ah, a.u1, accu, status);
	for (int A = tid; A < L.nno; A += nth) {
		double2 dv = a.d[A];
		const double2 u = a.u1[A];
		dv.x += u.x;
		dv.y += u.y;
		a.d[A] = dv;
	}
	g.sync();
	double *r0 = a.r0, *r1 = a.r1, *r2 = a.r2, *z0 = a.z0, *z1 = a.z1, *s1 = a.s1, *s2 = a.s2;
	for (int e = tid; e < L.nel; e += nth)
		r1[e] = gtmul_elem(L, a.d, e);

	double dvel = 1.0, dpre = 1.0;
	int cycle = 0;
	while ((dvel > a.citcom_accu || (dpre > a.citcom_accu && a.check_v_only == 0)) && cycle < a.max_citcom) {
		double rz[2] = {0.0, 0.0};
		for (int e = tid; e < L.nel; e += nth) {
			const double z = a.bab[e] * r1[e];
			z1[e] = z;
			rz[0] += r1[e] * z;
			if (cycle > 0)
				rz[1] += r0[e] * z0[e];
		}
		grid_reduce<2>(g, red, rz, 0u);
		const double r1dotz1 = rz[0];
		if (cycle > 0 && !(rz[1] > 0.0)) {   // assert(r0dotr0 > 0.0), Solver.c:150
			if (tid == 0)
				atomicOr(status, kStatBreakdown);
			break;
		}
		const double delta = cycle == 0 ? 0.0 : r1dotz1 / rz[1];
		for (int e = tid; e < L.nel; e += nth)
			s2[e] = cycle == 0 ? z1[e] : z1[e] + delta * s1[e];
		g.sync();
		for (int A = tid; A < L.nno; A += nth) {
			double g0, g1;
			gmul_node(L, s2, A, g0, g1);
			a.Ah[A] = make_double2(g0, g1);
			a.u1[A] = make_double2(0.0, 0.0);
		}
		g.sync();
		cg_total += inner_solve<REF>(g, a, red, op, a.Ah, a.u1, accu, status);
		double sa[1] = {0.0};
		for (int e = tid; e < L.nel; e += nth) {
			const double t = gtmul_elem(L, a.u1, e);
			a.Ahp[e] = t;
			sa[0] += s2[e] * t;
		}
		grid_reduce<1>(g, red, sa, 0u);
		const double alpha = r1dotz1 / sa[0];
		double t[4] = {0.0, 0.0, 0.0, 0.0};
		for (int e = tid; e < L.nel; e += nth) {
			r2[e] = r1[e] - alpha * a.Ahp[e];
			const double pe = a.p[e] + alpha * s2[e];
			a.p[e] = pe;
			t[0] += s2[e] * s2[e];
			t[1] += pe * pe;
		}
		for (int A = tid; A < L.nno; A += nth) {
			const double2 u = a.u1[A];
			double2 dv = a.d[A];
			dv.x -= alpha * u.x;
			dv.y -= alpha * u.y;
			a.d[A] = dv;
			t[2] += u.x * u.x + u.y * u.y;
			t[3] += dv.x * dv.x + dv.y * dv.y;
		}
		grid_reduce<4>(g, red, t, 0u);
		dpre = alpha * sqrt(t[0] / (1.0e-32 + t[1]));
		dvel = alpha * sqrt(t[2] / (1.0e-32 + t[3]));
		cycle++;
		double *sh = s1; s1 = s2; s2 = sh;
		sh = r0; r0 = r1; r1 = r2; r2 = sh;
		sh = z0; z0 = z1; z1 = sh;
		if (!isfinite(dvel) || !isfinite(dpre)) {
			if (tid == 0)
				atomicOr(status, kStatNan);
			break;
		}
	}
	if (cycle >= a.max_citcom && tid == 0)
		atomicOr(status, kStatCap);
	g.sync();

	// true residual |[F - K d - G p ; G^T d]| / |F|, and v_to_nodes (Solver.c:1319-1343)
	double rs[3] = {0.0, 0.0, 0.0};
	for (int A = tid; A < L.nno; A += nth) {
		double k0, k1, g0, g1;
		kmul_node(L, a.K, a.d, A, k0, k1);
		gmul_node(L, a.p, A, g0, g1);
		const double2 f = a.F[A];
		const double m0 = vfree(L, A, 0) ? f.x - k0 - g0 : 0.0;
		const double m1 = vfree(L, A, 1) ? f.y - k1 - g1 : 0.0;
		rs[0] += m0 * m0 + m1 * m1;
		rs[2] += f.x * f.x + f.y * f.y;
		const double2 dv = a.d[A];
		a.V[A] = make_double2(vfree(L, A, 0) ? dv.x : L.vbcval[A], vfree(L, A, 1) ? dv.y : L.vbcval[L.nno + A]);
	}
	for (int e = tid; e < L.nel; e += nth) {
		const double dvg = gtmul_elem(L, a.d, e);
		rs[1] += dvg * dvg;
	}
	grid_reduce<3>(g, red, rs, 0u);
	if (tid == 0) {
		StepScalars *sc = a.sc;
		sc->uzawa_cycles = cycle;
		sc->cg_cycles = cg_total;
		sc->dv = dvel;
		sc->dp = dpre;
		sc->res_m = sqrt(rs[0]) / sqrt(rs[2]);
		sc->res_c = sqrt(rs[1]) / sqrt(rs[2]);
		sc->accuracy = accu;
	}
}

// ---- single operators for the parity API --------------------------------
__global__ void __launch_bounds__(kBlock) k_kmul(DevLevel L, const double4 *__restrict__ K,
                                                 const double2 *__restrict__ x, double2 *__restrict__ y)
{
	const int A = blockIdx.x * blockDim.x + threadIdx.x;
	if (A >= L.nno)
		return;
	double y0, y1;
	kmul_node(L, K, x, A, y0, y1);
	y[A] = make_double2(y0, y1);
}

__global__ void __launch_bounds__(kBlock) k_gmul(DevLevel L, const double *__restrict__ p, double2 *__restrict__ y)
{
	const int A = blockIdx.x * blockDim.x + threadIdx.x;
	if (A >= L.nno)
		return;
	double y0, y1;
	gmul_node(L, p, A, y0, y1);
	y[A] = make_double2(y0, y1);
}

__global__ void __launch_bounds__(kBlock) k_gtmul(DevLevel L, const double2 *__restrict__ u, double *__restrict__ p)
{
	const int e = blockIdx.x * blockDim.x + threadIdx.x;
	if (e >= L.nel)
		return;
	p[e] = gtmul_elem(L, u, e);
}

// v_to_nodes alone (used when the Stokes solve is skipped by the caller).
__global__ void __launch_bounds__(kBlock) k_v_to_nodes(DevLevel L, const double2 *__restrict__ d, double2 *__restrict__ V)
{
	const int A = blockIdx.x * blockDim.x + threadIdx.x;
	if (A >= L.nno)
		return;
	const double2 dv = d[A];
	V[A] = make_double2(vfree(L, A, 0) ? dv.x : L.vbcval[A], vfree(L, A, 1) ? dv.y : L.vbcval[L.nno + A]);
}

void *uzawa_kernel_ptr(int ref) { return ref ? (void *)k_uzawa<true> : (void *)k_uzawa<false>; }
void *kmul_kernel_ptr() { return (void *)k_kmul; }

}  // namespace mclg
