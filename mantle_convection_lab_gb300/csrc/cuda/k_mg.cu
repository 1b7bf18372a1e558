// Converged Stokes solve for uniform meshes: FP64 iterative refinement around
// the reference's Uzawa iteration, whose inner velocity solves run as
// multigrid-preconditioned CG in TI (float for the mixed-precision solver,
// double for the plain FP64 one).  One persistent cooperative kernel per
// time step; every loop has a cap.
//
//   refinement (FP64):  R = [F - K d - G p ; G^T d],  stop when |R|/|F| < rtol
//   correction:        the Uzawa loop of citcom_solver (Solver.c:14-249) on
//                      [K G; G^T 0][dd; dp] = [R_m; -R_c], preconditioned by
//                      dividing by BAB (the reference multiplies by BAB,
//                      Solver.c:133-134, which squares the viscosity contrast
//                      instead of cancelling it), run to outer_rtol
//   inner K^-1:         CG preconditioned by one V(nu,nu) cycle: damped Jacobi
//                      smoothing, full-weighting restriction R = P^T, bilinear
//                      prolongation P (coincident / edge / centre weights 1,
//                      1/2, 1/4 as in interp_error, Solver.c:1009-1143),
//                      re-discretised coarse operators with injected
//                      viscosity, dense inverse on the coarsest grid.
//
// The operator is matrix-free.  A tile of 8 x 32 nodes stages its patch of
// nodal velocity and viscosity (10 x 34 nodes) in shared memory, computes the
// three stress components at the 4 Gauss points of each of its 9 x 33
// elements into shared memory, then every thread gathers the two rows of its
// own node from its 4 elements in a fixed order (deterministic, no atomics).
// With D = diag(2 eta, 2 eta, eta) and unit-Jacobian derivatives
// Dx = dN/dxi * sqrt(r), Dz = dN/deta / sqrt(r), r = dz/dx, this is exactly
// the element matrix of get_element_K (Build_matrix.c:192-271).
#include <math.h>
#include "k_mg.cuh"

namespace mclg {

MCLG_SHAPE_UPLOAD(upload_shape_tables_mg)


template <class T>
struct OpTab {
	T N[4][4], Dx[4][4], Dz[4][4];
};
__constant__ OpTab<float> cTf;
__constant__ OpTab<double> cTd;
template <class T> __device__ __forceinline__ const OpTab<T> &tab();
template <> __device__ __forceinline__ const OpTab<float> &tab<float>() { return cTf; }
template <> __device__ __forceinline__ const OpTab<double> &tab<double>() { return cTd; }

// Fill the unit-Jacobian tables: r = dz/dx of the (square-per-level) elements.
void upload_op_tables(const ShapeTables &S, double r, cudaStream_t st)
{
	OpTab<double> d;
	OpTab<float> f;
	const double sr = sqrt(r);
	for (int a = 0; a < 4; a++)
		for (int g = 0; g < 4; g++) {
			d.N[a][g] = S.N[a][g];
			d.Dx[a][g] = S.dNdxi[a][g] * sr;
			d.Dz[a][g] = S.dNdeta[a][g] / sr;
			f.N[a][g] = (float)d.N[a][g];
			f.Dx[a][g] = (float)d.Dx[a][g];
			f.Dz[a][g] = (float)d.Dz[a][g];
		}
	cudaMemcpyToSymbolAsync(cTd, &d, sizeof d, 0, cudaMemcpyHostToDevice, st);
	cudaMemcpyToSymbolAsync(cTf, &f, sizeof f, 0, cudaMemcpyHostToDevice, st);
}

// ---- small helpers ----------------------------------------------------------
// Elements per thread and trip of the FP64 vector loops: their loads are all
// issued before the arithmetic, so each thread keeps several in flight.
constexpr int kVecU = 4;
__device__ __forceinline__ void span(Part pt, int &start, int &stride)
{
	start = pt.rank * blockDim.x + threadIdx.x;
	stride = pt.size * blockDim.x;
}

__device__ __forceinline__ unsigned spread_bits(unsigned v)
{
	v &= 0xffffu;
	v = (v | (v << 8)) & 0x00ff00ffu;
	v = (v | (v << 4)) & 0x0f0f0f0fu;
	v = (v | (v << 2)) & 0x33333333u;
	v = (v | (v << 1)) & 0x55555555u;
	return v;
}

// Morton index of element (ex, ez) on a uniform mesh: x in the odd bits
// (morton, Tree.c:447-456).
__device__ __forceinline__ int morton(int ex, int ez)
{
	return (int)((spread_bits((unsigned)ex) << 1) | spread_bits((unsigned)ez));
}

// ---- the tiled matrix-free operator ----------------------------------------
#include "k_tile.cuh"

// Inverse diagonal of the level operator (the element diagonals summed).
template <class T, class V>
__device__ void level_invdiag(Part pt, int N, const unsigned char *mask, const T *eta, V *invD, double2 *kdiag64)
{
	const OpTab<T> &O = tab<T>();
	const int n = N + 1;
	int i0, st;
	span(pt, i0, st);
	for (int A = i0; A < n * n; A += st) {
		const int ix = A / n, iz = A - ix * n;
		T du = 0, dw = 0;
		const int eox[4] = {ix - 1, ix - 1, ix, ix}, eoz[4] = {iz - 1, iz, iz, iz - 1}, ea[4] = {2, 3, 0, 1};
#pragma unroll
		for (int q = 0; q < 4; q++) {
			const int ex = eox[q], ez = eoz[q];
			if (ex < 0 || ex >= N || ez < 0 || ez >= N)
				continue;
			const T e[4] = {eta[ez + ex * n], eta[ez + 1 + ex * n], eta[ez + 1 + (ex + 1) * n], eta[ez + (ex + 1) * n]};
			const int a = ea[q];
#pragma unroll
			for (int g = 0; g < 4; g++) {
				T eg = 0;
#pragma unroll
				for (int c = 0; c < 4; c++)
					eg += O.N[c][g] * e[c];
				du += 2 * eg * O.Dx[a][g] * O.Dx[a][g] + eg * O.Dz[a][g] * O.Dz[a][g];
				dw += 2 * eg * O.Dz[a][g] * O.Dz[a][g] + eg * O.Dx[a][g] * O.Dx[a][g];
			}
		}
		const unsigned m = mask[A];
		V v;
		v.x = (m & 1u) ? T(0) : T(1) / du;
		v.y = (m & 2u) ? T(0) : T(1) / dw;
		invD[A] = v;
		if (kdiag64)
			kdiag64[A] = make_double2((m & 1u) ? 1.0 : (double)du, (m & 2u) ? 1.0 : (double)dw);
	}
}

// b_c = P^T r_f over the coarse nodes (full weighting 1, 1/2, 1/4).
template <class T, class V>
__device__ void restrict_res(Part pt, const MGLevel<T> &F, const MGLevel<T> &C)
{
	int i0, st;
	span(pt, i0, st);
	for (int A = i0; A < C.n * C.n; A += st) {
		const int cx = A / C.n, cz = A - cx * C.n;
		T su = 0, sw = 0;
#pragma unroll
		for (int dx = -1; dx <= 1; dx++)
#pragma unroll
			for (int dz = -1; dz <= 1; dz++) {
				const int fx = 2 * cx + dx, fz = 2 * cz + dz;
				if (fx < 0 || fx >= F.n || fz < 0 || fz >= F.n)
					continue;
				const T wgt = (dx == 0 ? T(1) : T(0.5)) * (dz == 0 ? T(1) : T(0.5));
				const V r = F.r[fz + fx * F.n];
				su += wgt * r.x;
				sw += wgt * r.y;
			}
		const unsigned m = C.mask[A];
		V o;
		o.x = (m & 1u) ? T(0) : su;
		o.y = (m & 2u) ? T(0) : sw;
		C.b[A] = o;
	}
}

// out = x_f + P x_c (bilinear).
template <class T, class V>
__device__ void prolong_add(Part pt, const MGLevel<T> &F, const V *xf, V *out, const MGLevel<T> &C, const V *xc)
{
	int i0, st;
	span(pt, i0, st);
	for (int A = i0; A < F.n * F.n; A += st) {
		const int fx = A / F.n, fz = A - fx * F.n;
		const int x0 = fx >> 1, z0 = fz >> 1, x1 = (fx + 1) >> 1, z1 = (fz + 1) >> 1;
		const V a = xc[z0 + x0 * C.n], b = xc[z1 + x0 * C.n], c = xc[z0 + x1 * C.n], d = xc[z1 + x1 * C.n];
		const T cu = T(0.25) * ((a.x + b.x) + (c.x + d.x)), cw = T(0.25) * ((a.y + b.y) + (c.y + d.y));
		const unsigned m = F.mask[A];
		V o = xf[A];
		o.x = (m & 1u) ? T(0) : o.x + cu;
		o.y = (m & 2u) ? T(0) : o.y + cw;
		out[A] = o;
	}
}

// ---- coarsest grid: dense inverse -------------------------------------------
// Assemble the coarsest operator densely (FP64), put identity rows on the
// Dirichlet dofs and invert it by Gauss-Jordan; block 0 only.
template <class T>
__device__ void coarse_build(const MGHier<T> &H)
{
	const MGLevel<T> &L = H.lv[H.nlev - 1];
	const OpTab<double> &O = tab<double>();
	const int nd = H.cnd, n = L.n, N = L.N, w2 = 2 * nd;
	double *M = H.cwork;
	for (int k = threadIdx.x; k < nd * w2; k += blockDim.x)
		M[k] = ((k % w2) == nd + k / w2) ? 1.0 : 0.0;
	__syncthreads();
	for (int e = 0; e < N * N; e++) {
		const int ex = e / N, ez = e - ex * N;
		const int cn[4] = {ez + ex * n, ez + 1 + ex * n, ez + 1 + (ex + 1) * n, ez + (ex + 1) * n};
		if (threadIdx.x < 64) {
			const int p = threadIdx.x >> 3, q = threadIdx.x & 7;
			const int a = p >> 1, i = p & 1, b = q >> 1, j = q & 1;
			double kv = 0.0;
			for (int g = 0; g < 4; g++) {
				double eg = 0.0;
				for (int c = 0; c < 4; c++)
					eg += O.N[c][g] * (double)L.eta[cn[c]];
				double t;
				if (i == 0 && j == 0)
					t = 2 * O.Dx[a][g] * O.Dx[b][g] + O.Dz[a][g] * O.Dz[b][g];
				else if (i == 1 && j == 1)
					t = 2 * O.Dz[a][g] * O.Dz[b][g] + O.Dx[a][g] * O.Dx[b][g];
				else if (i == 0)
					t = O.Dz[a][g] * O.Dx[b][g];
				else
					t = O.Dx[a][g] * O.Dz[b][g];
				kv += eg * t;
			}
			M[(2 * cn[a] + i) * w2 + 2 * cn[b] + j] += kv;
		}
		__syncthreads();
	}
	// Dirichlet rows and columns -> identity
	for (int k = threadIdx.x; k < nd * nd; k += blockDim.x) {
		const int r = k / nd, c = k - r * nd;
		const bool dr = (L.mask[r >> 1] >> (r & 1)) & 1u, dc = (L.mask[c >> 1] >> (c & 1)) & 1u;
		if (dr || dc)
			M[r * w2 + c] = (r == c) ? 1.0 : 0.0;
	}
	__syncthreads();
	// Gauss-Jordan on [M | I]; the operator is SPD, no pivoting needed
	for (int k = 0; k < nd; k++) {
		__shared__ double piv;
		if (threadIdx.x == 0)
			piv = M[k * w2 + k];
		__syncthreads();
		for (int c = threadIdx.x; c < w2; c += blockDim.x)
			M[k * w2 + c] /= piv;
		__syncthreads();
		for (int idx = threadIdx.x; idx < nd * w2; idx += blockDim.x) {
			const int r = idx / w2, c = idx - r * w2;
			if (r != k) {
				const double f = M[r * w2 + k];
				if (c != k)
					M[r * w2 + c] -= f * M[k * w2 + c];
			}
		}
		__syncthreads();
		for (int r = threadIdx.x; r < nd; r += blockDim.x)
			if (r != k)
				M[r * w2 + k] = 0.0;
		__syncthreads();
	}
	for (int k = threadIdx.x; k < nd * nd; k += blockDim.x)
		H.cinv[k] = (T)M[(k / nd) * w2 + nd + (k % nd)];
	__syncthreads();
}

template <class T, class V>
__device__ void coarse_solve(const MGHier<T> &H, V *x)
{
	const MGLevel<T> &L = H.lv[H.nlev - 1];
	const int nd = H.cnd;
	const T *b = reinterpret_cast<const T *>(L.b);
	T *xo = reinterpret_cast<T *>(x);
	for (int i = threadIdx.x; i < nd; i += blockDim.x) {
		T s = 0;
		for (int j = 0; j < nd; j++)
			s += H.cinv[i * nd + j] * b[j];
		xo[i] = s;
	}
	__syncthreads();
}

// ---- one V(nu,nu) cycle: out0 = B rhs0 -----------------------------------------
// Levels below nblk run on the whole grid (grid barriers); the small levels
// from nblk down run inside block 0 alone (block barriers).  Every block walks
// the same buffer bookkeeping so that all of them know where each level's
// result lies; only the active blocks do the work.
template <class T>
__device__ void level_down(Sync &sy, unsigned char *sm, const MGHier<T> &H, int l,
                           const typename V2T<T>::t *rhs0, bool grid, bool active, typename V2T<T>::t **xcur)
{
	typedef typename V2T<T>::t V;
	const MGLevel<T> &L = H.lv[l];
	const V *b = (l == 0) ? rhs0 : L.b;
	const int nu = l < H.lfine ? H.nu : H.nu_c;
	// below the finest level the right-hand side P^T r of the finer level is
	// formed in this level's first pass (and stored for its later passes)
	const int xs0 = l >= 1 ? XS_ZERO_R : XS_ZERO;
	const V *rf = l >= 1 ? H.lv[l - 1].r : nullptr;
	const int nf = l >= 1 ? H.lv[l - 1].n : 0;
	V *bo = l >= 1 ? L.b : nullptr;
	V *x = L.xa, *xt = L.xb;
	if (nu == 1) {
		// one sweep from zero, x = omega D^-1 b, formed inside the residual pass
		if (active) {
			tile_pass<T, V>(sm, sy.part(grid), L.N, L.mask, L.eta, xt, b, L.invD, L.r, PASS_RESID, H.omega, nullptr,
			                xs0, rf, nf, nullptr, nullptr, nullptr, nullptr, bo, x);
			barrier(sy, grid);
		}
	} else {
		// sweep 1 (from zero) fused into sweep 2; the Chebyshev pair from zero is
		// x1 = w1 D^-1 b, x2 = c1 x1 + w2 D^-1 (b - A x1)
		const bool ch = H.cheb && nu == 2;
		if (active) {
			tile_pass<T, V>(sm, sy.part(grid), L.N, L.mask, L.eta, xt, b, L.invD, x, PASS_SMOOTH,
			                ch ? H.w2 : H.omega, nullptr, xs0, rf, nf, nullptr, nullptr, nullptr, nullptr, bo, nullptr,
			                ch ? H.w1 : T(-1), ch ? H.c1 : T(1));
			barrier(sy, grid);
		}
		for (int s = 2; s < nu; s++) {
			if (active) {
				tile_pass<T, V>(sm, sy.part(grid), L.N, L.mask, L.eta, x, b, L.invD, xt, PASS_SMOOTH, H.omega, nullptr);
				barrier(sy, grid);
			}
			V *tmp = x;
			x = xt;
			xt = tmp;
		}
		if (active) {
			tile_pass<T, V>(sm, sy.part(grid), L.N, L.mask, L.eta, x, b, L.invD, L.r, PASS_RESID, H.omega, nullptr);
			barrier(sy, grid);
		}
	}
	// the next level forms its right-hand side from L.r in its first pass,
	// except the coarsest (a dense solve)
	if (active && l + 1 == H.nlev - 1) {
		restrict_res<T, V>(sy.part(grid), L, H.lv[l + 1]);
		barrier(sy, grid);
	}
	xcur[l] = x;
}

// With dotv (level 0 only), the last sweep also accumulates this thread's
// share of out0.dotv into *dot and is not followed by a barrier: the caller's
// reduction provides it.
template <class T>
__device__ void level_up(Sync &sy, unsigned char *sm, const MGHier<T> &H, int l,
                         const typename V2T<T>::t *rhs0, typename V2T<T>::t *out0, bool grid, bool active,
                         typename V2T<T>::t **xcur, const double2 *dotv = nullptr, double *dot = nullptr)
{
	typedef typename V2T<T>::t V;
	const MGLevel<T> &L = H.lv[l];
	const V *b = (l == 0) ? rhs0 : L.b;
	V *x = xcur[l];
	V *xt = (x == L.xa) ? L.xb : L.xa;
	const MGLevel<T> &C = H.lv[l + 1];
	const int nu = l < H.lfine ? H.nu : H.nu_c;
	// the coarse-grid correction x + P xc is formed inside the first post-smoothing
	// sweep; the Chebyshev pair keeps that iterate (x0) in L.r, free on the way up,
	// for x2 = c1 x1 - c0 x0 + w2 D^-1 (b - A x1)
	const bool ch = H.cheb && nu == 2;
	for (int s = 0; s < nu; s++) {
		const bool last = l == 0 && s == nu - 1;
		V *dst = last ? out0 : xt;
		double *dp = (last && dotv) ? dot : nullptr;
		if (active) {
			if (s == 0)
				tile_pass<T, V>(sm, sy.part(grid), L.N, L.mask, L.eta, x, b, L.invD, dst, PASS_SMOOTH,
				                ch ? H.w1 : H.omega, dp, XS_PROLONG, xcur[l + 1], C.n, dotv, nullptr, nullptr, nullptr,
				                nullptr, ch ? L.r : nullptr);
			else if (ch)
				tile_pass<T, V>(sm, sy.part(grid), L.N, L.mask, L.eta, x, b, L.invD, dst, PASS_SMOOTH, H.w2, dp,
				                XS_PLAIN, nullptr, 0, dotv, nullptr, nullptr, nullptr, nullptr, nullptr, T(-1), H.c1,
				                L.r, H.c0);
			else
				tile_pass<T, V>(sm, sy.part(grid), L.N, L.mask, L.eta, x, b, L.invD, dst, PASS_SMOOTH, H.omega, dp,
				                XS_PLAIN, nullptr, 0, dotv);
			if (!dp)
				barrier(sy, grid);
		}
		xt = x;
		x = dst;
	}
	xcur[l] = x;
}

// out0 = B rhs0.  With dotv, *dot receives this thread's share of out0.dotv
// and the cycle ends without a barrier (the caller reduces *dot, which
// synchronises the team); without it the cycle ends with a barrier.
template <class T>
__device__ void vcycle(Sync &sy, unsigned char *sm, const MGHier<T> &H, const typename V2T<T>::t *rhs0,
                       typename V2T<T>::t *out0, const double2 *dotv = nullptr, double *dot = nullptr)
{
	typedef typename V2T<T>::t V;
	V *xcur[kMaxLev];
	const int lc = H.nlev - 1;
	// first block-local level (the coarsest always is; in a batch all are)
	const int nb = sy.size > 1 ? (H.nblk < lc ? H.nblk : lc) : 0;
	const bool b0 = sy.leader();
	if (dot)
		*dot = 0.0;
	for (int l = 0; l < lc; l++)
		level_down<T>(sy, sm, H, l, rhs0, l < nb, l < nb || b0, xcur);
	if (b0)
		coarse_solve<T, V>(H, H.lv[lc].xa);
	xcur[lc] = H.lv[lc].xa;
	for (int l = lc - 1; l >= 0; l--) {
		if (l == nb - 1)
			sy.sync();   // block 0's coarse-level results become visible to every block
		level_up<T>(sy, sm, H, l, rhs0, out0, l < nb, l < nb || b0, xcur, dotv, dot);
	}
	if (nb == 0 && !dotv)
		sy.sync();
}

// ---- inner solve: CG preconditioned by one V-cycle, all in T -----------------
template <class T>
__device__ int pcg_inner(Sync &sy, unsigned char *sm, const MGHier<T> &H, const typename V2T<T>::t *b,
                         typename V2T<T>::t *x, double rtol, int maxit)
{
	typedef typename V2T<T>::t V;
	const MGLevel<T> &L = H.lv[0];
	const int nn = L.n * L.n;
	const int tid = sy.tid, nth = sy.nth;
	V *r = H.pr, *z = H.pz, *p = H.pp, *q = H.pq;
	double bb[1] = {0.0};
	for (int A = tid; A < nn; A += nth) {
		const V bv = b[A];
		r[A] = bv;
		V zero;
		zero.x = T(0);
		zero.y = T(0);
		x[A] = zero;
		bb[0] += (double)bv.x * bv.x + (double)bv.y * bv.y;
	}
	sy.reduce<1>(bb);
	if (!(bb[0] > 0.0))
		return 0;
	vcycle<T>(sy, sm, H, r, z);
	double rz[1] = {0.0};
	for (int A = tid; A < nn; A += nth) {
		const V rv = r[A], zv = z[A];
		rz[0] += (double)rv.x * zv.x + (double)rv.y * zv.y;
		p[A] = zv;
	}
	sy.reduce<1>(rz);
	double rho = rz[0];
	int it = 0;
	while (it < maxit) {
		double pq[1];
		tile_pass<T, V>(sm, sy.part(true), L.N, L.mask, L.eta, p, nullptr, nullptr, q, PASS_MATVEC, T(0), pq);
		sy.reduce<1>(pq);
		const double alpha = rho / pq[0];
		double rr[1] = {0.0};
		for (int A = tid; A < nn; A += nth) {
			V xv = x[A], rv = r[A];
			const V pv = p[A], qv = q[A];
			xv.x += (T)alpha * pv.x;
			xv.y += (T)alpha * pv.y;
			rv.x -= (T)alpha * qv.x;
			rv.y -= (T)alpha * qv.y;
			x[A] = xv;
			r[A] = rv;
			rr[0] += (double)rv.x * rv.x + (double)rv.y * rv.y;
		}
		sy.reduce<1>(rr);
		it++;
		if (!(rr[0] > rtol * rtol * bb[0]) || !isfinite(alpha))
			break;
		vcycle<T>(sy, sm, H, r, z);
		double rz2[1] = {0.0};
		for (int A = tid; A < nn; A += nth) {
			const V rv = r[A], zv = z[A];
			rz2[0] += (double)rv.x * zv.x + (double)rv.y * zv.y;
		}
		sy.reduce<1>(rz2);
		const double beta = rz2[0] / rho;
		rho = rz2[0];
		for (int A = tid; A < nn; A += nth) {
			const V zv = z[A];
			V pv = p[A];
			pv.x = zv.x + (T)beta * pv.x;
			pv.y = zv.y + (T)beta * pv.y;
			p[A] = pv;
		}
		sy.sync();
	}
	sy.sync();
	return it;
}

// ---- FP64 operators on the fine uniform mesh -----------------------------------
__device__ __forceinline__ void g_entries(double hx, double hz, int a, double &g0, double &g1)
{
	element_g(cS, hz, hx, a, g0, g1);
}

// y = G s at every node (masked); s in Morton order.
__device__ void gmul64(int N0, const unsigned char *mask, const GTab &gt, const double *s, double2 *y, int tid,
                       int nth)
{
	const int n = N0 + 1;
	for (int A = tid; A < n * n; A += nth) {
		const int ix = A / n, iz = A - ix * n;
		double s0 = 0.0, s1 = 0.0;
		const int eox[4] = {ix - 1, ix - 1, ix, ix}, eoz[4] = {iz - 1, iz, iz, iz - 1}, ea[4] = {2, 3, 0, 1};
#pragma unroll
		for (int q = 0; q < 4; q++) {
			const int ex = eox[q], ez = eoz[q];
			if (ex < 0 || ex >= N0 || ez < 0 || ez >= N0)
				continue;
			const double g0 = gt.g0[ea[q]], g1 = gt.g1[ea[q]];
			const double se = s[morton(ex, ez)];
			s0 += g0 * se;
			s1 += g1 * se;
		}
		const unsigned m = mask[A];
		y[A] = make_double2((m & 1u) ? 0.0 : s0, (m & 2u) ? 0.0 : s1);
	}
}

// (G^T u)_e at element (ex, ez), free dofs in ascending equation order.
__device__ __forceinline__ double gtmul64_elem(int N0, const unsigned char *mask, const GTab &gt,
                                               const double2 *u, int ex, int ez)
{
	const int n = N0 + 1;
	const int cn[4] = {ez + ex * n, ez + 1 + ex * n, ez + 1 + (ex + 1) * n, ez + (ex + 1) * n};
	double s = 0.0;
#pragma unroll
	for (int c = 0; c < 4; c++) {
		const int a = kSortedCorner[c];
		const double g0 = gt.g0[a], g1 = gt.g1[a];
		const double2 ua = u[cn[a]];
		const unsigned m = mask[cn[a]];
		if (!(m & 1u))
			s += g0 * ua.x;
		if (!(m & 2u))
			s += g1 * ua.y;
	}
	return s;
}

// FP64 residual R = [F - K d - G p ; G^T d] into a.R, a.Rc; rs = {|R_m|^2, |R_c|^2, |F|^2}
// summed over the grid (every block holds the same values on return).
template <class TI>
__device__ void stokes_residual(const MGArgs<TI> &a, unsigned char *sm, Sync &sy, const double2 *d, const double *p,
                                double (&rs)[3])
{
	const int tid = sy.tid, nth = sy.nth;
	const int N0 = a.N0, n0 = N0 + 1, nn = n0 * n0, ne = N0 * N0;
	const GTab &gt = a.gt;
	tile_pass<double, double2>(sm, sy.part(true), N0, a.mask0, a.vis, d, nullptr, nullptr, a.Kd, PASS_MATVEC, 0.0, nullptr);
	gmul64(N0, a.mask0, gt, p, a.R, tid, nth);
	sy.sync();
	rs[0] = rs[1] = rs[2] = 0.0;
	for (int A = tid; A < nn; A += nth) {
		const double2 f = a.F[A], kd = a.Kd[A], gp = a.R[A];
		const double2 r = make_double2(f.x - kd.x - gp.x, f.y - kd.y - gp.y);
		a.R[A] = r;
		rs[0] += r.x * r.x + r.y * r.y;
		rs[2] += f.x * f.x + f.y * f.y;
	}
	for (int e = tid; e < ne; e += nth) {
		const int ex = e / N0, ez = e - ex * N0;
		const double c = gtmul64_elem(N0, a.mask0, gt, d, ex, ez);
		a.Rc[morton(ex, ez)] = c;
		rs[1] += c * c;
	}
	sy.reduce<3>(rs);
}

// (G^T u)_e for a TI velocity field (free dofs only).
template <class V>
__device__ __forceinline__ double gtmul_elem_t(int N0, const unsigned char *mask, const GTab &gt, const V *u, int ex,
                                               int ez)
{
	const int n = N0 + 1;
	const int cn[4] = {ez + ex * n, ez + 1 + ex * n, ez + 1 + (ex + 1) * n, ez + (ex + 1) * n};
	double s = 0.0;
#pragma unroll
	for (int c = 0; c < 4; c++) {
		const int a = kSortedCorner[c];
		const double g0 = gt.g0[a], g1 = gt.g1[a];
		const V ua = u[cn[a]];
		const unsigned m = mask[cn[a]];
		if (!(m & 1u))
			s += g0 * (double)ua.x;
		if (!(m & 2u))
			s += g1 * (double)ua.y;
	}
	return s;
}

// a + b = s + e exactly (Knuth's TwoSum, six FP32 additions)
__device__ __forceinline__ void two_sum_f(float a, float b, float &s, float &e)
{
	s = __fadd_rn(a, b);
	const float bb = __fsub_rn(s, a);
	e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}

// (sh, sl) += (gh + gl) x in double-float arithmetic: the product gh x and its
// rounding error (by FMA), gl x, and a TwoSum into the running pair.
__device__ __forceinline__ void df_axpy(float &sh, float &sl, float gh, float gl, float x)
{
	const float p = __fmul_rn(gh, x);
	float pe = __fmaf_rn(gh, x, -p);
	pe = __fmaf_rn(gl, x, pe);
	float t;
	two_sum_f(sh, p, sh, t);
	sl = __fadd_rn(sl, __fadd_rn(t, pe));
}

// (G^T u)_e for an FP32 velocity field: the eight products and their sum in
// double-float arithmetic on the FP32 pipe (about 48 bits, in the same corner
// order as the FP64 form), so that the FP64 pipe -- 1/64 of FP32 on GB300 --
// only converts and adds the final pair.
__device__ __forceinline__ double gtmul_elem_t(int N0, const unsigned char *mask, const GTab &gt, const float2 *u,
                                               int ex, int ez)
{
	const int n = N0 + 1;
	const int cn[4] = {ez + ex * n, ez + 1 + ex * n, ez + 1 + (ex + 1) * n, ez + (ex + 1) * n};
	float sh = 0.0f, sl = 0.0f;
#pragma unroll
	for (int c = 0; c < 4; c++) {
		const int a = kSortedCorner[c];
		const float2 ua = u[cn[a]];
		const unsigned m = mask[cn[a]];
		if (!(m & 1u))
			df_axpy(sh, sl, gt.g0h[a], gt.g0l[a], ua.x);
		if (!(m & 2u))
			df_axpy(sh, sl, gt.g1h[a], gt.g1l[a], ua.y);
	}
	return (double)sh + (double)sl;
}

// ---- MINRES vector kernels (FP64), kVecU elements per thread and trip ---------
// Separate functions so that their registers do not compete with the solver's
// state; every load of a trip is issued before its arithmetic.

// Ahp = G^T z_u per element (Morton order), in FP64; returns this thread's
// share of Ahp.z_p.
template <class VI>
__device__ __noinline__ double minres_gt_dot(int N0, const unsigned char *__restrict__ mask, const GTab &gt,
                                             const VI *__restrict__ zu, const double *__restrict__ zp,
                                             double *__restrict__ Ahp, int tid, int nth)
{
	const int ne = N0 * N0;
	double acc = 0.0;
	for (int e0 = tid; e0 < ne; e0 += kVecU * nth) {
		double t[kVecU], zpe[kVecU];
		int me[kVecU];
#pragma unroll
		for (int u = 0; u < kVecU; u++) {
			const int e = e0 + u * nth;
			if (e < ne) {
				const int ex = e / N0, ez = e - ex * N0;
				me[u] = morton(ex, ez);
				t[u] = gtmul_elem_t(N0, mask, gt, zu, ex, ez);
				zpe[u] = zp[me[u]];
			}
		}
#pragma unroll
		for (int u = 0; u < kVecU; u++)
			if (e0 + u * nth < ne) {
				Ahp[me[u]] = t[u];
				acc += t[u] * zpe[u];
			}
	}
	return acc;
}

// v_old <- az ig - dg v - gg v_old (velocity, with its TI copy into bI) and the
// same for the pressure part with Ahp.
template <class VI>
__device__ __noinline__ void minres_v_update(int nn, int ne, int tid, int nth, const double2 *__restrict__ az_,
                                             const double2 *__restrict__ v_, double2 *__restrict__ vo_,
                                             VI *__restrict__ bI, const double *__restrict__ ah_,
                                             const double *__restrict__ p0_, double *__restrict__ p1_, double ig,
                                             double dg, double gg)
{
	typedef decltype(VI().x) TI;
	for (int A0 = tid; A0 < nn; A0 += kVecU * nth) {
		double2 az[kVecU], v[kVecU], vo[kVecU];
#pragma unroll
		for (int u = 0; u < kVecU; u++) {
			const int A = A0 + u * nth;
			if (A < nn) {
				az[u] = az_[A];
				v[u] = v_[A];
				vo[u] = vo_[A];
			}
		}
#pragma unroll
		for (int u = 0; u < kVecU; u++) {
			const int A = A0 + u * nth;
			if (A < nn) {
				const double2 vn = make_double2(az[u].x * ig - dg * v[u].x - gg * vo[u].x,
				                                az[u].y * ig - dg * v[u].y - gg * vo[u].y);
				vo_[A] = vn;
				VI w;
				w.x = (TI)vn.x;
				w.y = (TI)vn.y;
				bI[A] = w;
			}
		}
	}
	for (int e0 = tid; e0 < ne; e0 += kVecU * nth) {
		double ah[kVecU], p0[kVecU], p1[kVecU];
#pragma unroll
		for (int u = 0; u < kVecU; u++) {
			const int e = e0 + u * nth;
			if (e < ne) {
				ah[u] = ah_[e];
				p0[u] = p0_[e];
				p1[u] = p1_[e];
			}
		}
#pragma unroll
		for (int u = 0; u < kVecU; u++) {
			const int e = e0 + u * nth;
			if (e < ne)
				p1_[e] = ah[u] * ig - dg * p0[u] - gg * p1[u];
		}
	}
}

// w_old <- (z ig - a3 w_old - a2 w) ia1 and x += step w_old, for the velocity
// (z in TI) and the pressure parts.
template <class VI>
__device__ __noinline__ void minres_w_update(int nn, int ne, int tid, int nth, const VI *__restrict__ z_,
                                             double2 *__restrict__ wo_, const double2 *__restrict__ w_,
                                             double2 *__restrict__ x_, const double *__restrict__ zp_,
                                             double *__restrict__ wpo_, const double *__restrict__ wp_,
                                             double *__restrict__ xp_, double ig, double a3, double a2, double ia1,
                                             double step)
{
	for (int A0 = tid; A0 < nn; A0 += kVecU * nth) {
		VI z[kVecU];
		double2 wo[kVecU], w[kVecU], x[kVecU];
#pragma unroll
		for (int u = 0; u < kVecU; u++) {
			const int A = A0 + u * nth;
			if (A < nn) {
				z[u] = z_[A];
				wo[u] = wo_[A];
				w[u] = w_[A];
				x[u] = x_[A];
			}
		}
#pragma unroll
		for (int u = 0; u < kVecU; u++) {
			const int A = A0 + u * nth;
			if (A < nn) {
				const double2 wn = make_double2(((double)z[u].x * ig - a3 * wo[u].x - a2 * w[u].x) * ia1,
				                                ((double)z[u].y * ig - a3 * wo[u].y - a2 * w[u].y) * ia1);
				wo_[A] = wn;
				x_[A] = make_double2(x[u].x + step * wn.x, x[u].y + step * wn.y);
			}
		}
	}
	for (int e0 = tid; e0 < ne; e0 += kVecU * nth) {
		double zz[kVecU], wo[kVecU], w[kVecU], x[kVecU];
#pragma unroll
		for (int u = 0; u < kVecU; u++) {
			const int e = e0 + u * nth;
			if (e < ne) {
				zz[u] = zp_[e];
				wo[u] = wpo_[e];
				w[u] = wp_[e];
				x[u] = xp_[e];
			}
		}
#pragma unroll
		for (int u = 0; u < kVecU; u++) {
			const int e = e0 + u * nth;
			if (e < ne) {
				const double wn = (zz[u] * ig - a3 * wo[u] - a2 * w[u]) * ia1;
				wpo_[e] = wn;
				xp_[e] = x[u] + step * wn;
			}
		}
	}
}

// z_p = v_p / BAB (ibab = 1/BAB); returns this thread's share of z_p.v_p.
__device__ __noinline__ double precond_pressure(int ne, int tid, int nth, const double *__restrict__ vp,
                                                const double *__restrict__ ibab, double *__restrict__ zp)
{
	double acc = 0.0;
	for (int e0 = tid; e0 < ne; e0 += kVecU * nth) {
		double v[kVecU], ib[kVecU];
#pragma unroll
		for (int u = 0; u < kVecU; u++) {
			const int e = e0 + u * nth;
			if (e < ne) {
				v[u] = vp[e];
				ib[u] = ibab[e];
			}
		}
#pragma unroll
		for (int u = 0; u < kVecU; u++) {
			const int e = e0 + u * nth;
			if (e < ne) {
				const double z = v[u] * ib[u];
				zp[e] = z;
				acc += z * v[u];
			}
		}
	}
	return acc;
}

// z = M^-1 v for M = diag(one V-cycle of K, BAB): the velocity part goes
// through the TI hierarchy (z_u stays in TI), the pressure part is multiplied
// by 1/BAB (a.bab holds the reciprocal).  Returns <z, v> over the team.  With
// converted, the caller has already written v_u in TI to the finest level's
// right-hand side (H.lv[0].b) and synchronised.
template <class TI>
__device__ double block_precond(const MGArgs<TI> &a, unsigned char *sm, Sync &sy, const double2 *vu, const double *vp,
                                typename V2T<TI>::t *zu, double *zp, bool converted = false)
{
	typedef typename V2T<TI>::t VI;
	const MGHier<TI> &H = a.H;
	const int tid = sy.tid, nth = sy.nth;
	const int N0 = a.N0, n0 = N0 + 1, nn = n0 * n0, ne = N0 * N0;
	VI *bI = H.lv[0].b;
	if (!converted) {
		for (int A = tid; A < nn; A += nth) {
			const double2 v = vu[A];
			VI w;
			w.x = (TI)v.x;
			w.y = (TI)v.y;
			bI[A] = w;
		}
		sy.sync();
	}
	double dot[1] = {0.0};
	vcycle<TI>(sy, sm, H, bI, zu, vu, &dot[0]);   // the last sweep forms <z_u, v_u>
	dot[0] += precond_pressure(ne, tid, nth, vp, a.bab, zp);
	sy.reduce<1>(dot);
	return dot[0];
}

// Y = K u + G p and Yc = G^T u in FP64 (the Stokes operator applied to (u, p));
// a.Kd is scratch.  Ends with a team barrier: Yc is written at Morton indices,
// which other threads read.
template <class TI>
__device__ void stokes_apply(const MGArgs<TI> &a, unsigned char *sm, Sync &sy, const double2 *u, const double *p,
                             double2 *Y, double *Yc)
{
	const int tid = sy.tid, nth = sy.nth;
	const int N0 = a.N0, n0 = N0 + 1, nn = n0 * n0, ne = N0 * N0;
	tile_pass<double, double2>(sm, sy.part(true), N0, a.mask0, a.vis, u, nullptr, nullptr, Y, PASS_MATVEC, 0.0, nullptr);
	gmul64(N0, a.mask0, a.gt, p, a.Kd, tid, nth);
	sy.sync();
	for (int A = tid; A < nn; A += nth) {
		const double2 y = Y[A], g = a.Kd[A];
		Y[A] = make_double2(y.x + g.x, y.y + g.y);
	}
	for (int e = tid; e < ne; e += nth) {
		const int ex = e / N0, ez = e - ex * N0;
		Yc[morton(ex, ez)] = gtmul64_elem(N0, a.mask0, a.gt, u, ex, ez);
	}
	sy.sync();
}

// warm_start=4: the start of the solve is the member of
//     x(alpha, beta) = h1 + alpha (h1 - h2) + beta (h1 - 2 h2 + h3)
// (h1, h2, h3 the last three solutions) whose residual under this step's
// operator is smallest in the norm the MINRES correction works in,
// |r|_M^2 = <r, M^-1 r> with M = diag(V-cycle, BAB): a least-squares problem in
// (alpha, beta) from the residual r0 at h1 and the operator applied to the two
// differences, a_k = A D_k; with M symmetric only M^-1 a_1 and M^-1 a_2 are
// needed.  The family holds the previous solution (0, 0), the linear (1, 0)
// and the quadratic (1, 1) extrapolation in time.  (In the plain L2 norm the
// minimiser chose coefficients of 10^5 along the second difference, whose
// operator image is tiny, and the solves diverged.)  ndir = 1 uses h1, h2 only
// (beta = 0).  Coefficients outside [-4, 8] fall back to the linear
// extrapolation.  Scratch: the MINRES and inner-CG vectors, free until the
// correction solve starts.
// Measured on the 1024^2 viscosity-contrast workload: the minimiser picks the
// quadratic member, MINRES needs about half the iterations of the linear start
// for some ten steps, then more and more (the error the solves leave behind is
// carried on and amplified from step to step), 111 against 100 per step over
// 30 steps; warm_start=3 stays the default there.
template <class TI>
__device__ void warm_guess(const MGArgs<TI> &a, unsigned char *sm, Sync &sy, int ndir)
{
	typedef typename V2T<TI>::t VI;
	const int tid = sy.tid, nth = sy.nth;
	const int N0 = a.N0, n0 = N0 + 1, nn = n0 * n0, ne = N0 * N0;
	double2 *U1 = a.mw[0], *U2 = a.mw[1], *Y1 = a.mv[0], *Y2 = a.mv[1];
	double *P1 = a.mwp[0], *P2 = a.mwp[1], *Yc1 = a.mvp[0], *Yc2 = a.mvp[1];
	VI *Z1 = a.H.px, *Z2 = a.H.pr;
	double *Zp1 = a.mzp[0], *Zp2 = a.mzp[1];
	double rs[3];
	stokes_residual(a, sm, sy, a.h1d, a.h1p, rs);   // a.R = F - K h1 - G p1, a.Rc = G^T h1
	for (int A = tid; A < nn; A += nth) {
		const double2 x1 = a.h1d[A], x2 = a.h2d[A];
		U1[A] = make_double2(x1.x - x2.x, x1.y - x2.y);
		if (ndir == 2) {
			const double2 x3 = a.h3d[A];
			U2[A] = make_double2(x1.x - 2.0 * x2.x + x3.x, x1.y - 2.0 * x2.y + x3.y);
		}
	}
	for (int e = tid; e < ne; e += nth) {
		P1[e] = a.h1p[e] - a.h2p[e];
		if (ndir == 2)
			P2[e] = a.h1p[e] - 2.0 * a.h2p[e] + a.h3p[e];
	}
	sy.sync();
	stokes_apply(a, sm, sy, U1, P1, Y1, Yc1);
	if (ndir == 2)
		stokes_apply(a, sm, sy, U2, P2, Y2, Yc2);
	// M^-1 a_k (the preconditioner's pressure part divides by BAB); the signs of
	// the continuity parts follow r = [F - K d - G p ; -G^T d]
	double q[5];   // <a1, M^-1 a1>, <a2, M^-1 a1>, <a2, M^-1 a2>, <r0, M^-1 a1>, <r0, M^-1 a2>
	q[0] = block_precond(a, sm, sy, Y1, Yc1, Z1, Zp1);
	q[2] = ndir == 2 ? block_precond(a, sm, sy, Y2, Yc2, Z2, Zp2) : 0.0;
	double c[3] = {0.0, 0.0, 0.0};
	for (int A = tid; A < nn; A += nth) {
		const double2 r = a.R[A];
		const VI z1 = Z1[A];
		c[1] += (double)z1.x * r.x + (double)z1.y * r.y;
		if (ndir == 2) {
			const double2 y2 = Y2[A];
			const VI z2 = Z2[A];
			c[0] += (double)z1.x * y2.x + (double)z1.y * y2.y;
			c[2] += (double)z2.x * r.x + (double)z2.y * r.y;
		}
	}
	for (int e = tid; e < ne; e += nth) {
		const double rc = -a.Rc[e];
		c[1] += Zp1[e] * rc;
		if (ndir == 2) {
			c[0] += Zp1[e] * Yc2[e];
			c[2] += Zp2[e] * rc;
		}
	}
	sy.reduce<3>(c);
	q[1] = c[0];
	q[3] = c[1];
	q[4] = c[2];
	// every thread holds the same q: the same coefficients and branches
	double al = q[0] > 0.0 ? q[3] / q[0] : 1.0, be = 0.0;
	if (ndir == 2) {
		const double det = q[0] * q[2] - q[1] * q[1];
		if (det > 1e-12 * q[0] * q[2]) {
			al = (q[3] * q[2] - q[4] * q[1]) / det;
			be = (q[4] * q[0] - q[3] * q[1]) / det;
		}
	}
	if (!isfinite(al) || !isfinite(be) || al < -4.0 || al > 8.0 || be < -4.0 || be > 8.0) {
		al = 1.0;
		be = 0.0;
	}
	for (int A = tid; A < nn; A += nth) {
		const double2 x1 = a.h1d[A], u1 = U1[A];
		double2 d = make_double2(x1.x + al * u1.x, x1.y + al * u1.y);
		if (ndir == 2) {
			const double2 u2 = U2[A];
			d.x += be * u2.x;
			d.y += be * u2.y;
		}
		a.d[A] = d;
	}
	for (int e = tid; e < ne; e += nth)
		a.p[e] = a.h1p[e] + al * P1[e] + (ndir == 2 ? be * P2[e] : 0.0);
	if (tid == 0) {
		a.sc->warm_a = al;
		a.sc->warm_b = be;
	}
	sy.sync();
}

// Correction solve by preconditioned MINRES (the Lanczos-based algorithm of
// Elman, Silvester and Wathen, "Finite Elements and Fast Iterative Solvers",
// Alg. 4.1) on [K G; G^T 0][x_u; x_p] = [R_m; -R_c] from a zero start, with
// the block-diagonal SPD preconditioner diag(V-cycle, BAB).  K is applied in
// TI by the tiled operator, G and G^T in FP64; Lanczos and direction vectors
// are FP64 and x_u, x_p accumulate in a.dd, a.dpv.  The FP64 refinement
// around this solve restores full accuracy.  Stops when the M^-1-norm of the
// residual has dropped by rtol.  Returns the iterations.
template <class TI>
__device__ int minres_correction(const MGArgs<TI> &a, unsigned char *sm, Sync &sy, double rtol, int maxit,
                                 int *status)
{
	typedef typename V2T<TI>::t VI;
	const MGHier<TI> &H = a.H;
	const MGLevel<TI> &L0 = H.lv[0];
	const int tid = sy.tid, nth = sy.nth;
	const int N0 = a.N0, n0 = N0 + 1, nn = n0 * n0, ne = N0 * N0;
	double2 *vu[2] = {a.mv[0], a.mv[1]}, *wu[2] = {a.mw[0], a.mw[1]};
	double *vp[2] = {a.mvp[0], a.mvp[1]}, *zp[2] = {a.mzp[0], a.mzp[1]}, *wp[2] = {a.mwp[0], a.mwp[1]};
	VI *zu[2] = {H.pz, H.pp}, *kz = H.pq;   // inner-CG vectors, free while MINRES runs
	const GTab &gt = a.gt;
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
	double gam2 = block_precond(a, sm, sy, vu[0], vp[0], zu[0], zp[0]);
	if (!(gam2 > 0.0))
		return 0;
	double gam = sqrt(gam2), gam_prev = 1.0;
	const double eta0 = gam;
	double eta = gam, c_prev = 1.0, c_cur = 1.0, s_prev = 0.0, s_cur = 0.0;
	int cv = 0, cw = 0, it = 0;   // index cv: z(j), v(j); 1-cv: v(j-1).  cw: w(j); 1-cw: w(j-1)
	while (it < maxit) {
		// A z(j), unscaled (z~ = z / gam): K z_u + G z_p into a.Kd with its
		// product with z_u formed in the same pass, and G^T z_u per element
		double dl[1] = {0.0};
		tile_pass<TI, VI>(sm, sy.part(true), L0.N, L0.mask, L0.eta, zu[cv], nullptr, nullptr, kz, PASS_STOKES, TI(0),
		                  &dl[0], XS_PLAIN, nullptr, 0, nullptr, zp[cv], &gt, a.Kd);
		dl[0] += minres_gt_dot<VI>(N0, a.mask0, gt, zu[cv], zp[cv], a.Ahp, tid, nth);
		sy.reduce<1>(dl);
		const double delta = dl[0] / (gam * gam);
		// v(j+1) = A z~ - (delta/gam) v(j) - (gam/gam_prev) v(j-1), into v(j-1)'s
		// buffer, and its TI copy as the V-cycle's right-hand side
		const double ig = 1.0 / gam, dg = delta / gam, gg = gam / gam_prev;
		minres_v_update<VI>(nn, ne, tid, nth, a.Kd, vu[cv], vu[1 - cv], H.lv[0].b, a.Ahp, vp[cv], vp[1 - cv], ig, dg, gg);
		sy.sync();
		const double gn2 = block_precond(a, sm, sy, vu[1 - cv], vp[1 - cv], zu[1 - cv], zp[1 - cv], true);
		const double gam_next = sqrt(fmax(gn2, 0.0));
		// Givens rotations
		const double a0 = c_cur * delta - c_prev * s_cur * gam;
		const double a1 = sqrt(a0 * a0 + gam_next * gam_next);
		const double a2 = s_cur * delta + c_prev * c_cur * gam;
		const double a3 = s_prev * gam;
		if (!(a1 > 0.0) || !isfinite(a1)) {
			if (!isfinite(a1) && tid == 0)
				atomicOr(status, 2);
			break;
		}
		const double c_next = a0 / a1, s_next = gam_next / a1;
		// w(j+1) = (z~(j) - a3 w(j-1) - a2 w(j)) / a1 into w(j-1)'s buffer; x += c_next eta w(j+1)
		const double ia1 = 1.0 / a1, step = c_next * eta;
		minres_w_update<VI>(nn, ne, tid, nth, zu[cv], wu[1 - cw], wu[cw], a.dd, zp[cv], wp[1 - cw], wp[cw], a.dpv, ig,
		                    a3, a2, ia1, step);
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
				atomicOr(status, 2);
			break;
		}
		if (!(fabs(eta) > rtol * eta0) || !(gam > 0.0))
			break;
		// no barrier here: the next operator pass reads z(j+1) and z_p(j+1),
		// complete since the reduction in block_precond, and touches none of
		// the vectors the updates above wrote
	}
	sy.sync();
	return it;
}

// ---- one converged Stokes solve ----------------------------------------------------
// The whole solve of one time step: per-step setup of the hierarchy, FP64
// refinement, correction solves.  Runs on the cooperative grid (one model) or
// inside one block (one model of a batch), as `sy` says.
template <class TI>
__device__ void stokes_solve(const MGArgs<TI> &a, unsigned char *sm, Sync &sy)
{
	typedef typename V2T<TI>::t VI;
	const MGHier<TI> &H = a.H;
	const int tid = sy.tid, nth = sy.nth;
	const int N0 = a.N0, n0 = N0 + 1, nn = n0 * n0, ne = N0 * N0;
	int *status = &a.sc->status;
	const GTab &gt = a.gt;

	// -- per-step setup: viscosity on every level, inverse diagonals, BAB, coarse inverse
	for (int A = tid; A < nn; A += nth)
		H.lv[0].eta[A] = (TI)a.vis[A];
	sy.sync();
	for (int l = 1; l < H.nlev; l++) {
		const MGLevel<TI> &C = H.lv[l], &F = H.lv[l - 1];
		for (int A = tid; A < C.n * C.n; A += nth) {
			const int cx = A / C.n, cz = A - cx * C.n;
			if (H.eta_avg == 0) {
				C.eta[A] = F.eta[2 * cz + 2 * cx * F.n];
			} else {
				double s = 0.0, wsum = 0.0;
				for (int dx = -1; dx <= 1; dx++)
					for (int dz = -1; dz <= 1; dz++) {
						const int fx = 2 * cx + dx, fz = 2 * cz + dz;
						if (fx < 0 || fx >= F.n || fz < 0 || fz >= F.n)
							continue;
						const double w = (dx == 0 ? 1.0 : 0.5) * (dz == 0 ? 1.0 : 0.5);
						const double ev = (double)F.eta[fz + fx * F.n];
						s += w * (H.eta_avg == 2 ? log(ev) : ev);
						wsum += w;
					}
				s /= wsum;
				C.eta[A] = (TI)(H.eta_avg == 2 ? exp(s) : s);
			}
		}
		sy.sync();
	}
	for (int l = 0; l < H.nlev; l++)
		level_invdiag<TI, VI>(sy.part(true), H.lv[l].N, H.lv[l].mask, H.lv[l].eta, H.lv[l].invD, nullptr);
	level_invdiag<double, double2>(sy.part(true), N0, a.mask0, a.vis, a.invD64, a.kdiag64);
	sy.sync();
	for (int e = tid; e < ne; e += nth) {
		const int ex = e / N0, ez = e - ex * N0;
		const int cn[4] = {ez + ex * n0, ez + 1 + ex * n0, ez + 1 + (ex + 1) * n0, ez + (ex + 1) * n0};
		double s = 0.0;
#pragma unroll
		for (int c = 0; c < 4; c++) {
			const int ac = kSortedCorner[c];
			double g0, g1;
			g_entries(a.hx, a.hz, ac, g0, g1);
			const double2 kd = a.kdiag64[cn[ac]];
			const unsigned m = a.mask0[cn[ac]];
			if (!(m & 1u))
				s += g0 * g0 / kd.x;
			if (!(m & 2u))
				s += g1 * g1 / kd.y;
		}
		a.bab[morton(ex, ez)] = 1.0 / s;   // the solvers multiply by 1/BAB
	}
	if (sy.leader())
		coarse_build<TI>(H);
	sy.sync();

	int refine = 0, outer_total = 0, inner_total = 0, capped = 0;
	double res_m = 0.0, res_c = 0.0, fnorm = 1.0;
	if (a.method == 1 && a.h1d != nullptr) {
		const int nh = a.sc->nsolved < 3 ? a.sc->nsolved : 3;   // solutions in the history
		if (nh >= 2)
			warm_guess<TI>(a, sm, sy, nh - 1);
	}
	if (a.d_alt != nullptr) {
		// Two candidate guesses: (d, p) from the network and (d_alt, p_alt),
		// the previous step's solution.  Keep the one with the smaller FP64
		// residual; a non-finite network guess always loses.
		double rl[3], rp[3];
		stokes_residual(a, sm, sy, a.d, a.p, rl);
		stokes_residual(a, sm, sy, a.d_alt, a.p_alt, rp);
		const double el = rl[0] + rl[1], ep = rp[0] + rp[1];
		const bool learned = isfinite(el) && (a.guess_force || el < ep);
		if (!learned) {
			for (int A = tid; A < nn; A += nth)
				a.d[A] = a.d_alt[A];
			for (int e = tid; e < ne; e += nth)
				a.p[e] = a.p_alt[e];
		}
		if (tid == 0) {
			a.sc->guess_used = learned ? 1 : 0;
			a.sc->res_learned = sqrt(el / rl[2]);
			a.sc->res_prev = sqrt(ep / rp[2]);
		}
		sy.sync();
	}
	while (true) {
		// -- FP64 residual R = [F - K d - G p ; G^T d]
		double rs[3];
		stokes_residual(a, sm, sy, a.d, a.p, rs);
		// a zero load (|F| = 0): the residual is measured absolutely
		fnorm = rs[2] > 0.0 ? sqrt(rs[2]) : 1.0;
		res_m = sqrt(rs[0]) / fnorm;
		res_c = sqrt(rs[1]) / fnorm;
		const double res = sqrt(rs[0] + rs[1]) / fnorm;
		if (!isfinite(res)) {
			if (tid == 0)
				atomicOr(status, 2);
			break;
		}
		if (!(res >= a.rtol))
			break;
		if (refine >= a.max_refine) {
			capped = 1;
			break;
		}
		refine++;

		if (a.method == 1) {
			// -- correction solve: MINRES on [K G; G^T 0][dd; dp] = [R_m; -R_c].
			// Far from the target (res > 1e4 rtol) a pass reduces by 1e-2,
			// where MINRES converges fastest; close to it, by what is left to
			// reach rtol (with a factor 2 margin), but not below outer_rtol.
			const double prt = res > 1e4 * a.rtol ? 1e-2 : fmax(a.outer_rtol, 0.5 * a.rtol / res);
			const int it = minres_correction<TI>(a, sm, sy, prt, a.max_outer, status);
			outer_total += it;
			inner_total += it + 1;
			for (int A = tid; A < nn; A += nth) {
				const double2 c = a.dd[A];
				double2 v = a.d[A];
				v.x += c.x;
				v.y += c.y;
				a.d[A] = v;
			}
			for (int e = tid; e < ne; e += nth)
				a.p[e] += a.dpv[e];
			sy.sync();
			continue;
		}

		// -- correction solve: Uzawa on [K G; G^T 0][dd; dp] = [R_m; -R_c]
		VI *bI = H.lv[0].b, *xI = H.px;   // level-0 buffers double as CG input/output here
		for (int A = tid; A < nn; A += nth) {
			const double2 r = a.R[A];
			VI v;
			v.x = (TI)r.x;
			v.y = (TI)r.y;
			bI[A] = v;
		}
		sy.sync();
		inner_total += pcg_inner<TI>(sy, sm, H, bI, xI, a.inner_rtol, a.max_inner);
		for (int A = tid; A < nn; A += nth) {
			const VI v = xI[A];
			a.dd[A] = make_double2((double)v.x, (double)v.y);
		}
		sy.sync();
		double *r0 = a.r0, *r1 = a.r1, *r2 = a.r2, *z0 = a.z0, *z1 = a.z1, *s1 = a.s1, *s2 = a.s2;
		double c0[1] = {0.0};
		for (int e = tid; e < ne; e += nth) {
			const int ex = e / N0, ez = e - ex * N0;
			const int me = morton(ex, ez);
			const double v = a.Rc[me] + gtmul64_elem(N0, a.mask0, gt, a.dd, ex, ez);
			r1[me] = v;
			a.dpv[me] = 0.0;
			c0[0] += v * v;
		}
		sy.reduce<1>(c0);
		const double rnorm0 = sqrt(c0[0]);
		double rnorm = rnorm0;
		int cycle = 0;
		while (cycle < a.max_outer && rnorm > a.outer_rtol * rnorm0 && rnorm > 0.0) {
			double rz[2] = {0.0, 0.0};
			for (int e = tid; e < ne; e += nth) {
				const double z = r1[e] * a.bab[e];
				z1[e] = z;
				rz[0] += r1[e] * z;
				if (cycle > 0)
					rz[1] += r0[e] * z0[e];
			}
			sy.reduce<2>(rz);
			const double delta = cycle == 0 ? 0.0 : rz[0] / rz[1];
			for (int e = tid; e < ne; e += nth)
				s2[e] = cycle == 0 ? z1[e] : z1[e] + delta * s1[e];
			sy.sync();
			gmul64(N0, a.mask0, gt, s2, a.u1, tid, nth);
			for (int A = tid; A < nn; A += nth) {
				const double2 v = a.u1[A];
				VI w;
				w.x = (TI)v.x;
				w.y = (TI)v.y;
				bI[A] = w;
			}
			sy.sync();
			inner_total += pcg_inner<TI>(sy, sm, H, bI, xI, a.inner_rtol, a.max_inner);
			for (int A = tid; A < nn; A += nth) {
				const VI v = xI[A];
				a.u1[A] = make_double2((double)v.x, (double)v.y);
			}
			sy.sync();
			double sa[1] = {0.0};
			for (int e = tid; e < ne; e += nth) {
				const int ex = e / N0, ez = e - ex * N0;
				const int me = morton(ex, ez);
				const double t = gtmul64_elem(N0, a.mask0, gt, a.u1, ex, ez);
				a.Ahp[me] = t;
				sa[0] += s2[me] * t;
			}
			sy.reduce<1>(sa);
			const double alpha = rz[0] / sa[0];
			double rr[1] = {0.0};
			for (int e = tid; e < ne; e += nth) {
				const double v = r1[e] - alpha * a.Ahp[e];
				r2[e] = v;
				a.dpv[e] += alpha * s2[e];
				rr[0] += v * v;
			}
			for (int A = tid; A < nn; A += nth) {
				const double2 u = a.u1[A];
				double2 v = a.dd[A];
				v.x -= alpha * u.x;
				v.y -= alpha * u.y;
				a.dd[A] = v;
			}
			sy.reduce<1>(rr);
			rnorm = sqrt(rr[0]);
			cycle++;
			double *sh = s1; s1 = s2; s2 = sh;
			sh = r0; r0 = r1; r1 = r2; r2 = sh;
			sh = z0; z0 = z1; z1 = sh;
			if (!isfinite(alpha) || !isfinite(rnorm)) {
				if (tid == 0)
					atomicOr(status, 2);
				break;
			}
		}
		outer_total += cycle;
		// apply the correction in FP64
		for (int A = tid; A < nn; A += nth) {
			const double2 c = a.dd[A];
			double2 v = a.d[A];
			v.x += c.x;
			v.y += c.y;
			a.d[A] = v;
		}
		for (int e = tid; e < ne; e += nth)
			a.p[e] += a.dpv[e];
		sy.sync();
	}
	if (capped && tid == 0)
		atomicOr(status, 1);
	// nodal velocity (v_to_nodes, Solver.c:1319-1343)
	for (int A = tid; A < nn; A += nth) {
		const double2 dv = a.d[A];
		const unsigned m = a.mask0[A];
		a.V[A] = make_double2((m & 1u) ? a.vbcval[A] : dv.x, (m & 2u) ? a.vbcval[nn + A] : dv.y);
	}
	if (tid == 0) {
		a.sc->uzawa_cycles = outer_total;
		a.sc->cg_cycles = inner_total;
		a.sc->refine_passes = refine;
		if (a.sc->nsolved < 1000000)
			a.sc->nsolved++;
		a.sc->res_m = res_m;
		a.sc->res_c = res_c;
		a.sc->dv = 0.0;
		a.sc->dp = 0.0;
	}
}

// One model on the whole cooperative grid.
template <class TI>
__global__ void __launch_bounds__(kBlock, 2) k_stokes_mg(MGArgs<TI> a)
{
	__shared__ __align__(16) unsigned char sm[kSmemBytes];
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
	stokes_solve<TI>(a, sm, sy);
}

// A batch of independent models.  Launched with clusters of `cs` blocks
// (cs = 1: plain blocks); each cluster takes the next model from the queue
// (ordered largest first by the host) and solves it alone with cluster
// barriers, so the launch is an ordinary one and clusters never wait on each
// other.  The cluster's rank-0 block draws from the queue and every block
// reads the draw from its shared memory; all blocks of a cluster leave the
// loop on the same draw.
template <class TI>
__global__ void __launch_bounds__(kBlock, 2) k_stokes_mg_batch(const MGArgs<TI> *models, int nmodels, int *queue)
{
	__shared__ __align__(16) unsigned char sm[kSmemBytes];
	__shared__ int next;
	__shared__ double cpart[2 * kRedWidth];
	cg::cluster_group cl = cg::this_cluster();
	const int cs = (int)cl.num_blocks(), rank = (int)cl.block_rank();
	for (;;) {
		if (rank == 0 && threadIdx.x == 0)
			next = atomicAdd(queue, 1);
		if (cs > 1) {
			cl.sync();
			const int m = *cl.map_shared_rank(&next, 0);
			cl.sync();   // every block has read the draw before the next one
			if (m >= nmodels)
				break;
			Sync sy;
			sy.mode = SYNC_CLUSTER;
			sy.g = nullptr;
			sy.red = models[m].red;
			sy.cpart = cpart;
			sy.cflip = 0;
			sy.rank = rank;
			sy.size = cs;
			sy.tid = rank * blockDim.x + threadIdx.x;
			sy.nth = cs * blockDim.x;
			stokes_solve<TI>(models[m], sm, sy);
			cl.sync();   // no block starts the next model (or leaves) while another reads its partials
		} else {
			__syncthreads();
			const int m = next;
			__syncthreads();
			if (m >= nmodels)
				break;
			Sync sy;
			sy.mode = SYNC_BLOCK;
			sy.g = nullptr;
			sy.red = models[m].red;
			sy.cpart = nullptr;
			sy.cflip = 0;
			sy.rank = 0;
			sy.size = 1;
			sy.tid = threadIdx.x;
			sy.nth = blockDim.x;
			stokes_solve<TI>(models[m], sm, sy);
			__syncthreads();
		}
	}
}

void *stokes_mg_kernel(int fp64) { return fp64 ? (void *)k_stokes_mg<double> : (void *)k_stokes_mg<float>; }
void *stokes_mg_batch_kernel(int fp64)
{
	return fp64 ? (void *)k_stokes_mg_batch<double> : (void *)k_stokes_mg_batch<float>;
}

}  // namespace mclg
