// Converged Stokes solve on quadtree meshes with hanging nodes; see k_qt.cuh.
// One persistent cooperative kernel per time step.  Vectors are node layout
// (both components of a node together); a primal vector stores its reduced
// dofs and is read through the constraints (qt_val), a dual vector (operator
// output, residual) is zero outside the reduced dofs.
#include <math.h>
#include "k_qt.cuh"

namespace mclg {

MCLG_SHAPE_UPLOAD(upload_shape_tables_qt)

// ---- values through the constraints ----------------------------------------------
// dof (2*node + component) of a primal vector: stored if reduced, the weighted
// sum of its reduced dofs if constrained, 0 if fixed.
template <class T, class X>
__device__ __forceinline__ X qt_val(const QtLevel<T> &L, const X *__restrict__ xf, int dof)
{
	const unsigned char k = L.kind[dof];
	if (k == 1)
		return xf[dof];
	X s = X(0);
	if (k == 2)
		for (int i = L.ex_off[dof]; i < L.ex_off[dof + 1]; i++)
			s += (X)L.ex_w[i] * xf[L.ex_src[i]];
	return s;
}

// Both components of node B of a primal vector through the constraints (the
// rare path of a row: a column with a constrained component).
template <class T, class X>
__device__ __noinline__ typename Q2T<X>::t qt_val2(const QtLevel<T> &L, const X *__restrict__ xf, int B)
{
	typename Q2T<X>::t v;
	v.x = qt_val(L, xf, 2 * B);
	v.y = qt_val(L, xf, 2 * B + 1);
	return v;
}

// Both rows of node j of K x~ (x~ the expanded x), with K in the level's TI
// blocks or its FP64 blocks.  Columns go in chunks of four: the chunk's index
// and block loads, then its gathers, are issued before any is used (a short
// chunk is padded with the node itself and a zero block).
template <class T, class K4, class X>
__device__ __forceinline__ void qt_rows(const QtLevel<T> &L, const K4 *__restrict__ K, const X *__restrict__ xf, int j,
                                        X &y0, X &y1)
{
	typedef typename Q2T<X>::t X2;
	const X2 *x2 = reinterpret_cast<const X2 *>(xf);
	X s0 = X(0), s1 = X(0);
	const int n = L.cnt[j];
	for (int k0 = 0; k0 < n; k0 += 4) {
		int Bf[4];
		K4 kb[4];
		X2 xv[4];
#pragma unroll
		for (int u = 0; u < 4; u++) {
			const bool in = k0 + u < n;
			Bf[u] = in ? L.nb[(size_t)(k0 + u) * L.nno + j] : j;
			kb[u] = in ? K[(size_t)(k0 + u) * L.nno + j] : K4{};
		}
#pragma unroll
		for (int u = 0; u < 4; u++)
			xv[u] = x2[Bf[u] & ~kQtCon];
#pragma unroll
		for (int u = 0; u < 4; u++) {
			if (Bf[u] & kQtCon)
				xv[u] = qt_val2(L, xf, Bf[u] & ~kQtCon);
			s0 += (X)kb[u].x * xv[u].x + (X)kb[u].y * xv[u].y;
			s1 += (X)kb[u].z * xv[u].x + (X)kb[u].w * xv[u].y;
		}
	}
	y0 = s0;
	y1 = s1;
}

// (C^T K C x) at both dofs of node A: the node's own rows plus the rows of
// the constrained dofs whose expansion holds them; 0 outside reduced dofs.
template <class T, class K4, class X>
__device__ __forceinline__ void qt_op_node(const QtLevel<T> &L, const K4 *__restrict__ K, const X *__restrict__ xf,
                                           int A, X &y0, X &y1)
{
	X y[2];
	qt_rows(L, K, xf, A, y[0], y[1]);
#pragma unroll
	for (int c = 0; c < 2; c++) {
		const int dof = 2 * A + c;
		if (L.kind[dof] != 1) {
			y[c] = X(0);
			continue;
		}
		for (int i = L.fo_off[dof]; i < L.fo_off[dof + 1]; i++) {
			const int h = L.fo_dof[i];
			X h0, h1;
			qt_rows(L, K, xf, h >> 1, h0, h1);
			y[c] += (X)L.fo_w[i] * ((h & 1) ? h1 : h0);
		}
	}
	y0 = y[0];
	y1 = y[1];
}

// Sources of the x a V-cycle pass reads at a node: the stored vector, or the
// first Jacobi sweep from zero, omega D^-1 b, formed where it is read (so the
// pass after it needs no barrier for it) with the operations, in the order, of
// the pass it replaces.  (Forming the prolongation x + P xc the same way inside
// the first sweep up was measured 2x slower on configuration 2: every
// neighbour's prolongation is recomputed through a deeper chain of gathers.)
template <class TI>
struct QtXStored {
	typedef typename Q2T<TI>::t X2;
	const X2 *x;
	__device__ __forceinline__ X2 operator()(int B) const { return x[B]; }
};

template <class TI>
struct QtXFirst {
	typedef typename Q2T<TI>::t X2;
	const X2 *b;
	const TI *invD;
	TI omega;
	__device__ __forceinline__ X2 operator()(int B) const
	{
		const X2 bv = b[B];
		X2 o;
		o.x = omega * invD[2 * B] * bv.x;
		o.y = omega * invD[2 * B + 1] * bv.y;
		return o;
	}
};

// (C^T K C x) at both dofs of node A from the assembled reduced operator: a
// plain node-block ELL row (x's constrained and fixed entries are stored as 0
// and the reduced columns hold every coupling); x read through src.
template <class TI, class XS>
__device__ __forceinline__ void qt_kr_node_src(const QtLevel<TI> &L, const XS &src, int A, TI &y0, TI &y1)
{
	typedef typename Q2T<TI>::t X2;
	typedef typename V4T<TI>::t K4;
	TI s0 = TI(0), s1 = TI(0);
	const int n = L.rcnt[A];
	for (int k0 = 0; k0 < n; k0 += 4) {
		int B[4];
		K4 kb[4];
#pragma unroll
		for (int u = 0; u < 4; u++) {
			const bool in = k0 + u < n;
			B[u] = in ? L.rnb[(size_t)(k0 + u) * L.nno + A] : A;
			kb[u] = in ? L.Kr[(size_t)(k0 + u) * L.nno + A] : K4{};
		}
		X2 xv[4];
#pragma unroll
		for (int u = 0; u < 4; u++)
			xv[u] = src(B[u]);
#pragma unroll
		for (int u = 0; u < 4; u++) {
			s0 += kb[u].x * xv[u].x + kb[u].y * xv[u].y;
			s1 += kb[u].z * xv[u].x + kb[u].w * xv[u].y;
		}
	}
	y0 = s0;
	y1 = s1;
}

template <class TI>
__device__ __forceinline__ void qt_kr_node(const QtLevel<TI> &L, const TI *__restrict__ xf, int A, TI &y0, TI &y1)
{
	const QtXStored<TI> src{reinterpret_cast<const typename Q2T<TI>::t *>(xf)};
	qt_kr_node_src(L, src, A, y0, y1);
}

// (C^T G p) at both dofs of node A (FP64, the finest level)
template <class T>
__device__ __forceinline__ void qt_g_node(const QtLevel<T> &Q, const DevLevel &L, const double *__restrict__ p, int A,
                                          double &y0, double &y1)
{
	double y[2];
	gmul_node(L, p, A, y[0], y[1]);
#pragma unroll
	for (int c = 0; c < 2; c++) {
		const int dof = 2 * A + c;
		if (Q.kind[dof] != 1) {
			y[c] = 0.0;
			continue;
		}
		for (int i = Q.fo_off[dof]; i < Q.fo_off[dof + 1]; i++) {
			const int h = Q.fo_dof[i];
			double h0, h1;
			gmul_node(L, p, h >> 1, h0, h1);
			y[c] += (double)Q.fo_w[i] * ((h & 1) ? h1 : h0);
		}
	}
	y0 = y[0];
	y1 = y[1];
}

// (G^T C u)_e of a primal vector u (flat, X) on the finest level
template <class T, class X>
__device__ __forceinline__ double qt_gt_elem(const QtLevel<T> &Q, const DevLevel &L, const X *__restrict__ uf, int e)
{
	double s = 0.0;
#pragma unroll
	for (int c = 0; c < 4; c++) {
		const int a = kSortedCorner[c];
		const int A = L.ienl[a * L.nel + e];
		double g0, g1;
		element_g(cS, L.dzh[e], L.dxh[e], a, g0, g1);
		s += g0 * (double)qt_val(Q, uf, 2 * A);
		s += g1 * (double)qt_val(Q, uf, 2 * A + 1);
	}
	return s;
}

// ---- the V-cycle (TI) -------------------------------------------------------------
// One damped Jacobi sweep on the constrained operator: xo = xi + w D^-1 (b - A xi),
// xi read through src.
template <class TI, class XS>
__device__ __forceinline__ void qt_sweep_src(const QtLevel<TI> &L, TI omega, const XS &src,
                                             typename Q2T<TI>::t *xo, int tid, int nth)
{
	typedef typename Q2T<TI>::t V;
	for (int A = tid; A < L.nno; A += nth) {
		TI y0, y1;
		qt_kr_node_src(L, src, A, y0, y1);
		const V x = src(A), b = L.b[A];
		V o;
		o.x = L.kind[2 * A] == 1 ? x.x + omega * L.invD[2 * A] * (b.x - y0) : TI(0);
		o.y = L.kind[2 * A + 1] == 1 ? x.y + omega * L.invD[2 * A + 1] * (b.y - y1) : TI(0);
		xo[A] = o;
	}
}

template <class TI>
__device__ __forceinline__ void qt_sweep(const QtLevel<TI> &L, TI omega, const typename Q2T<TI>::t *xi,
                                         typename Q2T<TI>::t *xo, int tid, int nth)
{
	const QtXStored<TI> src{xi};
	qt_sweep_src(L, omega, src, xo, tid, nth);
}

// The part of the solve's team running a part of the V-cycle: the whole team,
// or its leading block alone for the smallest levels (block barriers instead
// of team barriers).
struct QtTeam {
	Sync *sy;
	bool wide;
	int tid, nth;
	__device__ void sync()
	{
		if (wide)
			sy->sync();
		else
			__syncthreads();
	}
};

// Buffer index holding a level's result: the coarsest solve writes x[0]; a
// finer level runs smooth-1 sweeps from the first one, then smooth after the
// correction, so it ends in x[(2 smooth - 1) & 1].
template <class TI>
__device__ __forceinline__ int qt_final(const QtHier<TI> &H, int l)
{
	return l == 0 ? 0 : (2 * H.smooth - 1) & 1;
}

// Level l on the way down: smoothing from zero, residual, restriction into l-1.
// The first sweep from zero, x0 = w D^-1 b, is formed where the next pass reads
// it (the residual, or the second sweep), so it costs no barrier of its own.
template <class TI>
__device__ void qt_down(const QtHier<TI> &H, int l, QtTeam &t)
{
	typedef typename Q2T<TI>::t V;
	const QtLevel<TI> &L = H.lv[l];
	const QtXFirst<TI> first{L.b, L.invD, H.omega};
	int cur;
	if (H.smooth == 1) {
		// x0 stored for the way up, and the residual b - A x0 in the same pass
		V *x0 = L.x[0];
		for (int A = t.tid; A < L.nno; A += t.nth) {
			TI y0, y1;
			qt_kr_node_src(L, first, A, y0, y1);
			x0[A] = first(A);
			const V b = L.b[A];
			V r;
			r.x = L.kind[2 * A] == 1 ? b.x - y0 : TI(0);
			r.y = L.kind[2 * A + 1] == 1 ? b.y - y1 : TI(0);
			L.r[A] = r;
		}
		cur = 0;
		t.sync();
	} else {
		qt_sweep_src(L, H.omega, first, L.x[1], t.tid, t.nth);   // sweeps 1 and 2
		cur = 1;
		t.sync();
		for (int s = 2; s < H.smooth; s++) {
			qt_sweep(L, H.omega, L.x[cur], L.x[1 - cur], t.tid, t.nth);
			cur = 1 - cur;
			t.sync();
		}
		const TI *xf = reinterpret_cast<const TI *>(L.x[cur]);
		for (int A = t.tid; A < L.nno; A += t.nth) {
			TI y0, y1;
			qt_kr_node(L, xf, A, y0, y1);
			const V b = L.b[A];
			V r;
			r.x = L.kind[2 * A] == 1 ? b.x - y0 : TI(0);
			r.y = L.kind[2 * A + 1] == 1 ? b.y - y1 : TI(0);
			L.r[A] = r;
		}
		t.sync();
	}
	const QtLevel<TI> &C = H.lv[l - 1];
	const TI *rf = reinterpret_cast<const TI *>(L.r);
	TI *cb = reinterpret_cast<TI *>(C.b);
	for (int d = t.tid; d < 2 * C.nno; d += t.nth) {   // restriction: P^T by rows
		TI s = TI(0);
		for (int i = C.r_off[d]; i < C.r_off[d + 1]; i++)
			s += C.r_w[i] * rf[C.r_src[i]];
		cb[d] = s;
	}
	t.sync();
}

// Level l on the way up: prolongation of level l-1's result added, smoothing.
template <class TI>
__device__ void qt_up(const QtHier<TI> &H, int l, QtTeam &t)
{
	const QtLevel<TI> &L = H.lv[l];
	int cur = (H.smooth - 1) & 1;
	const TI *xc = reinterpret_cast<const TI *>(H.lv[l - 1].x[qt_final(H, l - 1)]);
	TI *xf = reinterpret_cast<TI *>(L.x[cur]);
	for (int d = t.tid; d < 2 * L.nno; d += t.nth) {
		if (L.p_off[d] == L.p_off[d + 1])
			continue;
		TI s = TI(0);
		for (int i = L.p_off[d]; i < L.p_off[d + 1]; i++)
			s += L.p_w[i] * xc[L.p_src[i]];
		xf[d] += s;
	}
	t.sync();
	for (int s = 0; s < H.smooth; s++) {
		qt_sweep(L, H.omega, L.x[cur], L.x[1 - cur], t.tid, t.nth);
		cur = 1 - cur;
		t.sync();
	}
}

// coarsest level: the dense inverse on its reduced dofs
template <class TI>
__device__ void qt_coarse_solve(const QtHier<TI> &H, QtTeam &t)
{
	const QtLevel<TI> &C = H.lv[0];
	const TI *bf = reinterpret_cast<const TI *>(C.b);
	TI *xf = reinterpret_cast<TI *>(C.x[0]);
	for (int i = t.tid; i < H.nc; i += t.nth) {
		TI s = TI(0);
		for (int j = 0; j < H.nc; j++)
			s += H.cinv[(size_t)i * H.nc + j] * bf[H.cdof[j]];
		xf[H.cdof[i]] = s;
	}
	t.sync();
}

// z = V-cycle(b) with b in the finest level's b; returns the buffer holding z.
template <class TI>
__device__ const typename Q2T<TI>::t *qt_vcycle(Sync &sy, const QtHier<TI> &H)
{
	const int top = H.nlev - 1, nb = H.nblk < top ? H.nblk : top;   // the finest level always runs on the team
	QtTeam team{&sy, true, sy.tid, sy.nth};
	for (int l = top; l >= (nb > 1 ? nb : 1); l--)
		qt_down(H, l, team);
	if (nb > 0) {
		if (sy.leader()) {
			QtTeam blk{&sy, false, (int)threadIdx.x, (int)blockDim.x};
			for (int l = nb - 1; l >= 1; l--)
				qt_down(H, l, blk);
			qt_coarse_solve(H, blk);
			for (int l = 1; l < nb; l++)
				qt_up(H, l, blk);
		}
		sy.sync();
	} else {
		qt_coarse_solve(H, team);
	}
	for (int l = nb > 1 ? nb : 1; l <= top; l++)
		qt_up(H, l, team);
	return H.lv[top].x[qt_final(H, top)];
}

// Dense inverse of the coarsest level's constrained operator on its reduced
// dofs, columns from the operator applied to unit vectors (FP64), inverted
// by Gauss-Jordan (the operator is SPD: no pivoting).  Block 0 only.
template <class TI>
__device__ void qt_coarse_build(const QtHier<TI> &H)
{
	const QtLevel<TI> &C = H.lv[0];
	const int nc = H.nc, w2 = 2 * nc;
	double *M = H.cwork, *e = H.cvec;
	for (int k = threadIdx.x; k < nc * w2; k += blockDim.x)
		M[k] = ((k % w2) == nc + k / w2) ? 1.0 : 0.0;
	for (int k = threadIdx.x; k < 2 * C.nno; k += blockDim.x)
		e[k] = 0.0;
	__syncthreads();
	for (int j = 0; j < nc; j++) {
		if (threadIdx.x == 0)
			e[H.cdof[j]] = 1.0;
		__syncthreads();
		for (int i = threadIdx.x; i < nc; i += blockDim.x) {
			const int d = H.cdof[i];
			double y0, y1;
			qt_op_node(C, C.K64, (const double *)e, d >> 1, y0, y1);
			M[(size_t)i * w2 + j] = (d & 1) ? y1 : y0;
		}
		__syncthreads();
		if (threadIdx.x == 0)
			e[H.cdof[j]] = 0.0;
		__syncthreads();
	}
	__shared__ double piv;
	for (int k = 0; k < nc; k++) {
		if (threadIdx.x == 0)
			piv = M[(size_t)k * w2 + k];
		__syncthreads();
		for (int c = threadIdx.x; c < w2; c += blockDim.x)
			M[(size_t)k * w2 + c] /= piv;
		__syncthreads();
		for (int r = threadIdx.x; r < nc; r += blockDim.x) {
			if (r == k)
				continue;
			const double f = M[(size_t)r * w2 + k];
			if (f != 0.0)
				for (int c = 0; c < w2; c++)
					M[(size_t)r * w2 + c] -= f * M[(size_t)k * w2 + c];
		}
		__syncthreads();
	}
	for (int k = threadIdx.x; k < nc * nc; k += blockDim.x) {
		const int r = k / nc, c = k - r * nc;
		H.cinv[k] = (TI)M[(size_t)r * w2 + nc + c];
	}
	__syncthreads();
}

// ---- FP64 residual and the preconditioner ------------------------------------------
// R = [C^T (F - K d - G p) ; G^T C d] (FP64); rs = |R_m|^2, |R_c|^2, |C^T F|^2.
template <class TI>
__device__ void qt_residual(Sync &sy, const QtArgs<TI> &a, const double2 *d, const double *p, double (&rs)[3])
{
	const int tid = sy.tid, nth = sy.nth;
	const DevLevel &L = a.L;
	const QtLevel<TI> &Q = a.H.lv[a.H.nlev - 1];
	const double *df = reinterpret_cast<const double *>(d);
	const double *Ff = reinterpret_cast<const double *>(a.F);
	rs[0] = rs[1] = rs[2] = 0.0;
	for (int A = tid; A < L.nno; A += nth) {
		double k0, k1, g0, g1;
		qt_op_node(Q, Q.K64, df, A, k0, k1);
		qt_g_node(Q, L, p, A, g0, g1);
		double f[2] = {0.0, 0.0};
		for (int c = 0; c < 2; c++) {   // C^T F
			const int dof = 2 * A + c;
			if (Q.kind[dof] != 1)
				continue;
			f[c] = Ff[dof];
			for (int i = Q.fo_off[dof]; i < Q.fo_off[dof + 1]; i++)
				f[c] += (double)Q.fo_w[i] * Ff[Q.fo_dof[i]];
		}
		const double2 r = make_double2(Q.kind[2 * A] == 1 ? f[0] - k0 - g0 : 0.0,
		                               Q.kind[2 * A + 1] == 1 ? f[1] - k1 - g1 : 0.0);
		a.R[A] = r;
		rs[0] += r.x * r.x + r.y * r.y;
		rs[2] += f[0] * f[0] + f[1] * f[1];
	}
	for (int e = tid; e < L.nel; e += nth) {
		const double c = qt_gt_elem(Q, L, df, e);
		a.Rc[e] = c;
		rs[1] += c * c;
	}
	sy.reduce<3>(rs);
}

// z = M^-1 v, M = diag(V-cycle, BAB); returns <z, v>.
template <class TI>
__device__ double qt_precond(Sync &sy, const QtArgs<TI> &a, const double2 *vu, const double *vp,
                             typename Q2T<TI>::t *zu, double *zp)
{
	const int tid = sy.tid, nth = sy.nth;
	typedef typename Q2T<TI>::t V;
	const QtHier<TI> &H = a.H;
	const QtLevel<TI> &Q = H.lv[H.nlev - 1];
	for (int A = tid; A < Q.nno; A += nth) {
		const double2 v = vu[A];
		V w;
		w.x = (TI)v.x;
		w.y = (TI)v.y;
		Q.b[A] = w;
	}
	sy.sync();
	const V *x = qt_vcycle(sy, H);
	double dot[1] = {0.0};
	for (int A = tid; A < Q.nno; A += nth) {
		const V z = x[A];
		zu[A] = z;
		const double2 v = vu[A];
		dot[0] += (double)z.x * v.x + (double)z.y * v.y;
	}
	for (int e = tid; e < a.L.nel; e += nth) {
		const double z = vp[e] / a.bab[e];
		zp[e] = z;
		dot[0] += z * vp[e];
	}
	sy.reduce<1>(dot);
	return dot[0];
}

// Correction solve by preconditioned MINRES (Elman, Silvester and Wathen,
// "Finite Elements and Fast Iterative Solvers", Alg. 4.1) on the constrained
// system [C^T K C, C^T G; G^T C, 0][x_u; x_p] = [R_m; -R_c] from zero; K in TI,
// G in FP64, Lanczos and direction vectors FP64; x into a.dd, a.dpv.
template <class TI>
__device__ int qt_minres(Sync &sy, const QtArgs<TI> &a, double rtol, int maxit, int *status)
{
	const int tid = sy.tid, nth = sy.nth;
	typedef typename Q2T<TI>::t V;
	const DevLevel &L = a.L;
	const QtLevel<TI> &Q = a.H.lv[a.H.nlev - 1];
	const int nn = L.nno, ne = L.nel;
	double2 *vu[2] = {a.mv[0], a.mv[1]}, *wu[2] = {a.mw[0], a.mw[1]};
	double *vp[2] = {a.mvp[0], a.mvp[1]}, *zp[2] = {a.mzp[0], a.mzp[1]}, *wp[2] = {a.mwp[0], a.mwp[1]};
	V *zu[2] = {a.mz[0], a.mz[1]};
	const double2 zero2 = make_double2(0.0, 0.0);
	for (int A = tid; A < nn; A += nth) {
		vu[0][A] = a.R[A];
		vu[1][A] = zero2;
		wu[0][A] = zero2;
		wu[1][A] = zero2;
		a.dd[A] = zero2;
	}
	for (int e = tid; e < ne; e += nth) {
		vp[0][e] = -a.Rc[e];
		vp[1][e] = 0.0;
		wp[0][e] = 0.0;
		wp[1][e] = 0.0;
		a.dpv[e] = 0.0;
	}
	sy.sync();
	double gam2 = qt_precond(sy, a, vu[0], vp[0], zu[0], zp[0]);
	if (!(gam2 > 0.0))
		return 0;
	double gam = sqrt(gam2), gam_prev = 1.0;
	const double eta0 = gam;
	double eta = gam, c_prev = 1.0, c_cur = 1.0, s_prev = 0.0, s_cur = 0.0;
	int cv = 0, cw = 0, it = 0;
	while (it < maxit) {
		const TI *zf = reinterpret_cast<const TI *>(zu[cv]);
		double dl[1] = {0.0};
		for (int A = tid; A < nn; A += nth) {
			TI k0, k1;
			double g0, g1;
			qt_kr_node(Q, zf, A, k0, k1);
			qt_g_node(Q, L, zp[cv], A, g0, g1);
			const double2 az = make_double2((double)k0 + g0, (double)k1 + g1);
			a.Kd[A] = az;
			const V z = zu[cv][A];
			dl[0] += az.x * (double)z.x + az.y * (double)z.y;
		}
		for (int e = tid; e < ne; e += nth) {
			const double t = qt_gt_elem(Q, L, zf, e);
			a.Ahp[e] = t;
			dl[0] += t * zp[cv][e];
		}
		sy.reduce<1>(dl);
		const double delta = dl[0] / (gam * gam);
		const double ig = 1.0 / gam, dg = delta / gam, gg = gam / gam_prev;
		for (int A = tid; A < nn; A += nth) {
			const double2 az = a.Kd[A], v = vu[cv][A], vo = vu[1 - cv][A];
			vu[1 - cv][A] = make_double2(az.x * ig - dg * v.x - gg * vo.x, az.y * ig - dg * v.y - gg * vo.y);
		}
		for (int e = tid; e < ne; e += nth)
			vp[1 - cv][e] = a.Ahp[e] * ig - dg * vp[cv][e] - gg * vp[1 - cv][e];
		sy.sync();
		const double gn2 = qt_precond(sy, a, vu[1 - cv], vp[1 - cv], zu[1 - cv], zp[1 - cv]);
		const double gam_next = sqrt(fmax(gn2, 0.0));
		const double a0 = c_cur * delta - c_prev * s_cur * gam;
		const double a1 = sqrt(a0 * a0 + gam_next * gam_next);
		const double a2 = s_cur * delta + c_prev * c_cur * gam;
		const double a3 = s_prev * gam;
		if (!(a1 > 0.0) || !isfinite(a1)) {
			if (!isfinite(a1) && tid == 0)
				atomicOr(status, kStatNan);
			break;
		}
		const double c_next = a0 / a1, s_next = gam_next / a1;
		const double ia1 = 1.0 / a1, step = c_next * eta;
		for (int A = tid; A < nn; A += nth) {
			const V z = zu[cv][A];
			const double2 wo = wu[1 - cw][A], w = wu[cw][A];
			const double2 wn = make_double2(((double)z.x * ig - a3 * wo.x - a2 * w.x) * ia1,
			                                ((double)z.y * ig - a3 * wo.y - a2 * w.y) * ia1);
			wu[1 - cw][A] = wn;
			double2 x = a.dd[A];
			x.x += step * wn.x;
			x.y += step * wn.y;
			a.dd[A] = x;
		}
		for (int e = tid; e < ne; e += nth) {
			const double wn = (zp[cv][e] * ig - a3 * wp[1 - cw][e] - a2 * wp[cw][e]) * ia1;
			wp[1 - cw][e] = wn;
			a.dpv[e] += step * wn;
		}
		eta = -s_next * eta;
		it++;
		cv = 1 - cv;
		cw = 1 - cw;
		gam_prev = gam;
		gam = gam_next;
		c_prev = c_cur;
		c_cur = c_next;
		s_prev = s_cur;
		s_cur = s_next;
		if (!isfinite(eta)) {
			if (tid == 0)
				atomicOr(status, kStatNan);
			break;
		}
		if (!(fabs(eta) > rtol * eta0) || !(gam > 0.0))
			break;
		sy.sync();
	}
	sy.sync();
	return it;
}

// The whole converged solve of one refined model on the team `sy`.
template <class TI>
__device__ void qt_solve(const QtArgs<TI> &a, Sync &sy)
{
	const int tid = sy.tid, nth = sy.nth;
	const QtHier<TI> &H = a.H;
	const DevLevel &L = a.L;
	int *status = &a.sc->status;

	// -- per step: every level's reduced operator C^T K C in TI, and its diagonal
	for (int l = 0; l < H.nlev; l++) {
		const QtLevel<TI> &Q = H.lv[l];
		const double *K64f = reinterpret_cast<const double *>(Q.K64);
		TI *Krf = reinterpret_cast<TI *>(Q.Kr);
		for (int A = tid; A < Q.nno; A += nth) {
			for (int u = 0; u < Q.rnbw; u++) {
				const size_t b = ((size_t)u * Q.nno + A) * 4;
				Krf[b] = Krf[b + 1] = Krf[b + 2] = Krf[b + 3] = TI(0);
			}
			int self = -1;
			for (int u = 0; u < Q.rcnt[A]; u++)
				if (Q.rnb[(size_t)u * Q.nno + A] == A)
					self = u;
			double dgl[2] = {0.0, 0.0};
			const int i1 = Q.rc_off[A + 1];
			for (int i = Q.rc_off[A]; i < i1;) {
				const int t = Q.rc_tgt[i];
				double v = 0.0;
				for (; i < i1 && Q.rc_tgt[i] == t; i++)
					v += (double)Q.rc_w[i] * K64f[Q.rc_src[i]];
				const int slot = t >> 2, cc = t & 3;
				Krf[((size_t)slot * Q.nno + A) * 4 + cc] = (TI)v;
				if (slot == self && (cc == 0 || cc == 3))
					dgl[cc == 3] = v;
			}
			for (int c = 0; c < 2; c++)
				Q.invD[2 * A + c] = Q.kind[2 * A + c] == 1 && dgl[c] > 0.0 ? (TI)(1.0 / dgl[c]) : TI(0);
		}
	}
	sy.sync();
	if (sy.leader())
		qt_coarse_build(H);
	sy.sync();

	int refine = 0, minres_total = 0, vcycles = 0, capped = 0;
	double res_m = 0.0, res_c = 0.0;
	while (true) {
		double rs[3];
		qt_residual(sy, a, a.d, a.p, rs);
		// a zero load (|C^T F| = 0): the residual is measured absolutely
		const double fnorm = rs[2] > 0.0 ? sqrt(rs[2]) : 1.0;
		res_m = sqrt(rs[0]) / fnorm;
		res_c = sqrt(rs[1]) / fnorm;
		const double res = sqrt(rs[0] + rs[1]) / fnorm;
		if (!isfinite(res)) {
			if (tid == 0)
				atomicOr(status, kStatNan);
			break;
		}
		if (!(res >= a.rtol))
			break;
		if (refine >= a.max_refine) {
			capped = 1;
			break;
		}
		refine++;
		// far from the target a pass reduces by 1e-2, close to it by what is
		// left (factor 2 margin), not below outer_rtol
		const double prt = res > 1e4 * a.rtol ? 1e-2 : fmax(a.outer_rtol, 0.5 * a.rtol / res);
		const int it = qt_minres(sy, a, prt, a.max_outer, status);
		minres_total += it;
		vcycles += it + 1;
		for (int A = tid; A < L.nno; A += nth) {
			const double2 c = a.dd[A];
			double2 v = a.d[A];
			v.x += c.x;
			v.y += c.y;
			a.d[A] = v;
		}
		for (int e = tid; e < L.nel; e += nth)
			a.p[e] += a.dpv[e];
		sy.sync();
	}
	if (capped && tid == 0)
		atomicOr(status, kStatCap);
	// the hanging nodes' values, and the velocity with its boundary values (v_to_nodes)
	const QtLevel<TI> &Q = H.lv[H.nlev - 1];
	double *df = reinterpret_cast<double *>(a.d);
	for (int A = tid; A < L.nno; A += nth) {
		double v[2];
		for (int c = 0; c < 2; c++)
			v[c] = qt_val(Q, (const double *)df, 2 * A + c);
		a.V[A] = make_double2(vfree(L, A, 0) ? v[0] : L.vbcval[A], vfree(L, A, 1) ? v[1] : L.vbcval[L.nno + A]);
	}
	sy.sync();
	for (int A = tid; A < L.nno; A += nth)
		for (int c = 0; c < 2; c++)
			if (Q.kind[2 * A + c] == 2)
				df[2 * A + c] = vfree(L, A, c) ? (c ? a.V[A].y : a.V[A].x) : 0.0;
	if (tid == 0) {
		StepScalars *sc = a.sc;
		sc->uzawa_cycles = minres_total;
		sc->cg_cycles = vcycles;
		sc->refine_passes = refine;
		sc->res_m = res_m;
		sc->res_c = res_c;
		sc->dv = 0.0;
		sc->dp = 0.0;
	}
}

// One refined model on the whole cooperative grid.
template <class TI>
__global__ void __launch_bounds__(kBlock) k_stokes_qt(QtArgs<TI> a)
{
	cg::grid_group g = cg::this_grid();
	Sync sy;
	sy.mode = SYNC_GRID;
	sy.g = &g;
	sy.red = a.red;
	sy.cpart = nullptr;
	sy.cflip = 0;
	sy.rank = blockIdx.x;
	sy.size = gridDim.x;
	sy.tid = blockIdx.x * blockDim.x + threadIdx.x;
	sy.nth = gridDim.x * blockDim.x;
	qt_solve<TI>(a, sy);
}

// A batch of independent refined models, launched with clusters of `cs`
// blocks (cs = 1: plain blocks).  Each cluster takes the next model from the
// queue (ordered largest first by the host) and solves it alone with cluster
// barriers, so clusters never wait on one another.  The rank-0 block draws and
// every block reads the draw from its shared memory.
template <class TI>
__global__ void __launch_bounds__(kBlock) k_stokes_qt_batch(const QtArgs<TI> *models, int nmodels, int *queue)
{
	__shared__ int next;
	__shared__ double cpart[2 * kRedWidth];
	cg::cluster_group cl = cg::this_cluster();
	const int cs = (int)cl.num_blocks(), rank = (int)cl.block_rank();
	for (;;) {
		if (rank == 0 && threadIdx.x == 0)
			next = atomicAdd(queue, 1);
		Sync sy;
		sy.g = nullptr;
		sy.cflip = 0;
		if (cs > 1) {
			cl.sync();
			const int m = *cl.map_shared_rank(&next, 0);
			cl.sync();   // every block has read the draw before the next one
			if (m >= nmodels)
				break;
			sy.mode = SYNC_CLUSTER;
			sy.red = models[m].red;
			sy.cpart = cpart;
			sy.rank = rank;
			sy.size = cs;
			sy.tid = rank * blockDim.x + threadIdx.x;
			sy.nth = cs * blockDim.x;
			qt_solve<TI>(models[m], sy);
			cl.sync();   // no block starts the next model (or leaves) while another reads its partials
		} else {
			__syncthreads();
			const int m = next;
			__syncthreads();
			if (m >= nmodels)
				break;
			sy.mode = SYNC_BLOCK;
			sy.red = models[m].red;
			sy.cpart = nullptr;
			sy.rank = 0;
			sy.size = 1;
			sy.tid = threadIdx.x;
			sy.nth = blockDim.x;
			qt_solve<TI>(models[m], sy);
			__syncthreads();
		}
	}
}

// linear extrapolation of the last two solutions: x = 2 x1 - x2
__global__ void __launch_bounds__(kBlock) k_qt_extrapolate(int n2, int ne, const double *d1, const double *d2,
                                                           const double *p1, const double *p2, double *d, double *p)
{
	const int i = blockIdx.x * blockDim.x + threadIdx.x;
	if (i < n2)
		d[i] = 2.0 * d1[i] - d2[i];
	if (i < ne)
		p[i] = 2.0 * p1[i] - p2[i];
}

// d1 <- d - (d1 - d2): the history shift of the second step after a remesh
__global__ void __launch_bounds__(kBlock) k_qt_shift(int n2, int ne, const double *d, const double *p, double *d1,
                                                     double *p1, const double *d2, const double *p2)
{
	const int i = blockIdx.x * blockDim.x + threadIdx.x;
	if (i < n2)
		d1[i] = d[i] - d1[i] + d2[i];
	if (i < ne)
		p1[i] = p[i] - p1[i] + p2[i];
}

// Coarse-level viscosity from the finer level around the same node: the value
// there (avg 0), or the mean (1) or log-mean (2) over the node and its matrix
// neighbours on the finer level, weighted 1 (the node), 1/2 (a neighbour
// along an axis), 1/4 (a diagonal neighbour) -- full weighting where the
// finer level is uniform.
__global__ void __launch_bounds__(kBlock) k_qt_inject(int n, const int *map, const double *src, double *dst, int avg,
                                                      int nno_f, const int *nb_f, const unsigned char *cnt_f,
                                                      const double *X_f)
{
	const int i = blockIdx.x * blockDim.x + threadIdx.x;
	if (i >= n)
		return;
	const int a = map[i];
	if (avg == 0) {
		dst[i] = src[a];
		return;
	}
	const double xa = X_f[a], za = X_f[nno_f + a];
	double s = 0.0, ws = 0.0;
	for (int k = 0; k < cnt_f[a]; k++) {
		const int B = nb_f[(size_t)k * nno_f + a] & ~kQtCon;
		const bool ax = X_f[B] == xa, az = X_f[nno_f + B] == za;
		const double w = (ax && az) ? 1.0 : (ax || az) ? 0.5 : 0.25;
		s += w * (avg == 2 ? log(src[B]) : src[B]);
		ws += w;
	}
	s /= ws;
	dst[i] = avg == 2 ? exp(s) : s;
}

void *qt_kernel(int fp64) { return fp64 ? (void *)k_stokes_qt<double> : (void *)k_stokes_qt<float>; }
void *qt_batch_kernel(int fp64)
{
	return fp64 ? (void *)k_stokes_qt_batch<double> : (void *)k_stokes_qt_batch<float>;
}

}  // namespace mclg
