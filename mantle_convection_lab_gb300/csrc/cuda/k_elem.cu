// Element loops that feed the Stokes solve: buoyancy (with the horizontal
// average), viscosity, assembly of K / F / Kdiag, BAB, and the element stress.
//
// Assembly is node-centric: the thread that owns node A visits the elements
// touching A in ascending element order (the order Build_matrix.c:42-140
// accumulates them in) and adds the element rows of A into A's own block row,
// so no two threads write the same memory and no atomics are needed.
#include "mclg_dev.cuh"

namespace mclg {

MCLG_SHAPE_UPLOAD(upload_shape_tables_elem)

// ---- buoyancy: Ra*T minus its horizontal average (Buoyancy.c:3-22) -------
// get_node_horiz_avg (Parallel.c:354-437) interpolates Ra*T at every fine-grid
// position (i,k) from the element covering it and sums over i.  Its local
// coordinates use integer division, (2i - ix0 - ix1)/(ix1 - ix0), which is
// exact only for elements one or two fine cells wide; that is reproduced.
__device__ __forceinline__ double na_val(int a, double xi, double eta)
{
	switch (a) {
	case 0: return 0.25 * (1.0 - xi) * (1.0 - eta);
	case 1: return 0.25 * (1.0 - xi) * (1.0 + eta);
	case 2: return 0.25 * (1.0 + xi) * (1.0 + eta);
	default: return 0.25 * (1.0 + xi) * (1.0 - eta);
	}
}

// One block per fine row k; avg[k] = sum_i interp(i,k) / gnox.
__global__ void __launch_bounds__(kBlock) k_buoy_rowavg(DevLevel L, const double *__restrict__ T, double Ra,
                                                        double *__restrict__ avg)
{
	const int k = blockIdx.x, gnox = L.gnox, gnoz = L.gnoz, ncz = gnoz - 1;
	double acc[1] = {0.0};
	for (int i = threadIdx.x; i < gnox; i += blockDim.x) {
		double v = 0.0;
		if (i == gnox - 1 && k == gnoz - 1) {
			v = Ra * T[L.nno - 1];
		} else {
			const int ci = (i == gnox - 1) ? i - 1 : i, ck = (k == gnoz - 1) ? k - 1 : k;
			const int e = L.cell_elem[ci * ncz + ck];
			const int s = 1 << (L.fine_level - L.elev[e]);
			const int n0 = L.node[L.ienl[e]];
			const int ix0 = n0 / gnoz, iz0 = n0 - ix0 * gnoz;
			const int ix1 = ix0 + s, iz1 = iz0 + s;
			const double xi = (i == gnox - 1) ? 1.0 : (double)((2 * i - ix0 - ix1) / (ix1 - ix0));
			const double eta = (k == gnoz - 1) ? 1.0 : (double)((2 * k - iz0 - iz1) / (iz1 - iz0));
#pragma unroll
			for (int a = 0; a < 4; a++)
				v += na_val(a, xi, eta) * (Ra * T[L.ienl[a * L.nel + e]]);
		}
		acc[0] += v;
	}
	block_reduce<1>(acc, 0u);
	if (threadIdx.x == 0)
		avg[k] = acc[0] / gnox;
}

// buoyancy = Ra*T - avg[row]  and  viscosity (Viscosity.c:3-24), one pass.
__global__ void __launch_bounds__(kBlock) k_buoy_vis(DevLevel L, const double *__restrict__ T, double Ra,
                                                     const double *__restrict__ avg, double Aexp, double refT,
                                                     double lm_jump, double vmin, double vmax,
                                                     double *__restrict__ buoy, double *__restrict__ vis)
{
	const int A = blockIdx.x * blockDim.x + threadIdx.x;
	if (A >= L.nno)
		return;
	const double z = L.X[L.nno + A];
	const int n = L.node[A], iz = n - (n / L.gnoz) * L.gnoz;
	buoy[A] = Ra * T[A] - avg[iz];
	double v = exp(Aexp * (refT - T[A]));
	if (z < 0.77)
		v *= lm_jump;
	if (vmax > 0.0)
		v = fmin(fmax(v, vmin), vmax);
	vis[A] = v;
}

// ---- Stokes assembly (Build_matrix.c:42-344, 720-744) ---------------------
// Entry (a,i),(b,j) of the element stiffness of get_element_K (Build_matrix.c:192-271).
// The reference computes entries with node b >= a and mirrors the rest,
// so entry (p,q) with p's node after q's takes the value computed for (q,p).
__device__ __forceinline__ double ke_entry(const double (&etag)[4], double dxh, double dzh, double jac,
                                           int a, int i, int b, int j)
{
	if (b < a || (b == a && i > j)) {
		int t = a; a = b; b = t;
		t = i; i = j; j = t;
	}
	double k = 0.0;
#pragma unroll
	for (int g = 0; g < 4; g++) {
		const double eta = etag[g];
		const double two_eta = 2.0 * eta;
		const double dNa_dx = cS.dNdxi[a][g] * dzh, dNa_dz = cS.dNdeta[a][g] * dxh;
		const double dNb_dx = cS.dNdxi[b][g] * dzh, dNb_dz = cS.dNdeta[b][g] * dxh;
		double t;
		if (i == 0 && j == 0)
			t = (dNa_dx * two_eta) * dNb_dx + (dNa_dz * eta) * dNb_dz;
		else if (i == 1 && j == 0)
			t = (dNa_dx * eta) * dNb_dz;
		else if (i == 0 && j == 1)
			t = (dNa_dz * eta) * dNb_dx;
		else
			t = (dNa_dz * two_eta) * dNb_dz + (dNa_dx * eta) * dNb_dx;
		k += t;
	}
	return k / jac;
}

__device__ __forceinline__ void gauss_eta(const DevLevel &L, const double *__restrict__ vis, int e, double (&etag)[4])
{
	double v[4];
#pragma unroll
	for (int d = 0; d < 4; d++)
		v[d] = vis[L.ienl[d * L.nel + e]];
#pragma unroll
	for (int g = 0; g < 4; g++) {
		double s = 0.0;
#pragma unroll
		for (int d = 0; d < 4; d++)
			s += cS.N[d][g] * v[d];
		etag[g] = s;
	}
}

// One thread per node: block row of K, F and Kdiag.  With withK == 0 only F
// is formed (the matrix-free solvers never need the assembled K).
__global__ void __launch_bounds__(kBlock) k_assemble_stokes(DevLevel L, const double *__restrict__ vis,
                                                            const double *__restrict__ buoy,
                                                            double4 *__restrict__ K, double2 *__restrict__ F,
                                                            double2 *__restrict__ Kdiag, int withK)
{
	const int A = blockIdx.x * blockDim.x + threadIdx.x;
	if (A >= L.nno)
		return;
	const int nno = L.nno, nel = L.nel, cnt = L.p2n_cnt[A];
	const bool fr[2] = {vfree(L, A, 0), vfree(L, A, 1)};
	if (withK)
		for (int k = 0; k < L.nbw; k++)
			K[(size_t)k * nno + A] = make_double4(0.0, 0.0, 0.0, 0.0);
	double f[2] = {0.0, 0.0};
	// pass 1: K entries and Dirichlet lifting (K_matrix, Build_matrix.c:42-115)
	for (int s = 0; s < cnt; s++) {
		const int e = L.p2n_el[s * nno + A], a = L.p2n_a[s * nno + A];
		double etag[4];
		gauss_eta(L, vis, e, etag);
		const double dxh = L.dxh[e], dzh = L.dzh[e], jac = L.jac[e];
		for (int i = 0; i < 2; i++) {
			if (!fr[i])
				continue;
			for (int j = 0; j < 2; j++)
				for (int b = 0; b < 4; b++) {
					const int B = L.ienl[b * nel + e];
					if (!withK && vfree(L, B, j))
						continue;
					const double kv = ke_entry(etag, dxh, dzh, jac, a, i, b, j);
					if (vfree(L, B, j)) {
						const int slot = L.kslot[(a * 4 + b) * nel + e];
						double *blk = reinterpret_cast<double *>(&K[(size_t)slot * nno + A]);
						blk[i * 2 + j] += kv;
					} else {
						f[i] -= kv * L.vbcval[j * nno + B];
					}
				}
		}
	}
	// pass 2: element loads (F_matrix / get_element_F, Build_matrix.c:117-140, 273-344)
	for (int s = 0; s < cnt; s++) {
		const int e = L.p2n_el[s * nno + A], a = L.p2n_a[s * nno + A];
		int idx[4];
#pragma unroll
		for (int d = 0; d < 4; d++)
			idx[d] = L.ienl[d * nel + e];
		double fe[2] = {0.0, 0.0};
		{
			double force[4];
#pragma unroll
			for (int g = 0; g < 4; g++) {
				double t = 0.0;
#pragma unroll
				for (int d = 0; d < 4; d++)
					t += cS.N[d][g] * buoy[idx[d]];
				force[g] = t;
			}
			double t = 0.0;
#pragma unroll
			for (int g = 0; g < 4; g++)
				t += cS.N[a][g] * force[g];
			fe[1] = t * L.jac[e];
		}
		for (int i = 0; i < 2; i++) {
			int nat = 0;
#pragma unroll
			for (int d = 0; d < 4; d++)
				if (L.vbc[i * nno + idx[d]] == 'S')
					nat += d;
			if (nat == 3)
				nat = 1;
			else if (nat == 1 || nat == 5)
				nat = 2;
			else if (nat == 0 || nat == 2)
				nat = 0;
			if (nat != 0) {
				const double Ln = L.X[i * nno + idx[2]] - L.X[i * nno + idx[0]];
				fe[i] += 0.5 * Ln * L.vbcval[i * nno + idx[a]];
			}
			if (fr[i])
				f[i] += fe[i];
		}
	}
	F[A] = make_double2(fr[0] ? f[0] : 0.0, fr[1] ? f[1] : 0.0);
	if (!withK)
		return;
	// Kdiag (Build_matrix.c:740-744): the self slot of the block row
	double2 dg = make_double2(1.0, 1.0);
	{
		const double4 blk = K[(size_t)L.self_slot[A] * nno + A];
		if (fr[0])
			dg.x = blk.x;
		if (fr[1])
			dg.y = blk.w;
	}
	Kdiag[A] = dg;
}

// BAB[e] = sum over the element's free dofs of G^2/Kdiag (Solver.c:54-64),
// in ascending equation order.
__global__ void __launch_bounds__(kBlock) k_bab(DevLevel L, const double2 *__restrict__ Kdiag,
                                                double *__restrict__ bab)
{
	const int e = blockIdx.x * blockDim.x + threadIdx.x;
	if (e >= L.nel)
		return;
	double s = 0.0;
#pragma unroll
	for (int c = 0; c < 4; c++) {
		const int a = kSortedCorner[c];
		const int A = L.ienl[a * L.nel + e];
		double g0, g1;
		element_g(cS, L.dzh[e], L.dxh[e], a, g0, g1);
		const double2 kd = Kdiag[A];
		if (vfree(L, A, 0))
			s += g0 * g0 / kd.x;
		if (vfree(L, A, 1))
			s += g1 * g1 / kd.y;
	}
	bab[e] = s;
}

// ---- stress (compute_stress, Grain_size_evolution.c:154-213) -------------
__global__ void __launch_bounds__(kBlock) k_stress_elem(DevLevel L, const double *__restrict__ vis,
                                                        const double2 *__restrict__ V, double *__restrict__ se)
{
	const int e = blockIdx.x * blockDim.x + threadIdx.x;
	if (e >= L.nel)
		return;
	double eta = 0.0, u11 = 0.0, u22 = 0.0, u12 = 0.0;
#pragma unroll
	for (int a = 0; a < 4; a++)
		eta += 0.25 * vis[L.ienl[a * L.nel + e]];
#pragma unroll
	for (int a = 0; a < 4; a++) {
		const int i = L.ienl[a * L.nel + e];
		const double dNa_dx = cS.dNdxi_c[a] * L.dzh[e];
		const double dNa_dz = cS.dNdeta_c[a] * L.dxh[e];
		const double2 v = V[i];
		u11 += dNa_dx * v.x;
		u22 += dNa_dz * v.y;
		u12 += dNa_dz * v.x;
	}
	u11 /= L.jac[e];
	u22 /= L.jac[e];
	u12 /= L.jac[e];
	const double u21 = u12;   // the reference reuses du/dz for dw/dx
	double sr = u11 * u11 + u22 * u22 + u12 * u21 * 2.0;
	sr = sqrt(0.5 * sr);
	se[e] = 2.0 * eta * sr;
}

// p_to_nodes (Solver.c:1345-1366): area-weighted average over the node's elements.
__global__ void __launch_bounds__(kBlock) k_elem_to_node(DevLevel L, const double *__restrict__ pe,
                                                         double *__restrict__ pn)
{
	const int A = blockIdx.x * blockDim.x + threadIdx.x;
	if (A >= L.nno)
		return;
	double s = 0.0, ta = 0.0;
	for (int k = 0; k < L.p2n_cnt[A]; k++) {
		const int e = L.p2n_el[k * L.nno + A];
		const double ar = L.area[e];
		s += ar * pe[e];
		ta += ar;
	}
	pn[A] = s / ta;
}

}  // namespace mclg
