// SUPG temperature update (update_temperature, Update_temperature.c:3-133):
// artificial diffusivity tau, node-centric assembly of the heat K, C and F,
// the time step, the generalized-trapezoid system A = C/(theta dt) + K with
// B = F + C T/(theta dt), its CG solve in one persistent kernel, and the
// write-back of T.  The reference also tracks dT/dt (initial_T_dot and the
// ddot update, :30-34, :113-117) but a stray ';' at :64 drops it from B, so it
// never reaches any output; that dead computation is not performed here.
#include <math.h>
#include "cg_solve.cuh"

namespace mclg {

MCLG_SHAPE_UPLOAD(upload_shape_tables_heat)

// calculate_artificial_diffusivity (Update_temperature.c:241-291)
// Thread 0 also seeds the two minima of advection_dt with its 1e10 start value.
// xi = coth(alpha) - 1/alpha.  The reference evaluates cosh(alpha)/sinh(alpha),
// which overflows to inf/inf = NaN for |alpha| > 710; the heat solve then
// stops at iteration 0 and T silently stays unchanged.  With safe != 0,
// |alpha| > 20 uses coth = sign(alpha): for 20 < |alpha| <= 710 the reference's
// ratio already rounds to exactly +-1, so results only differ where the
// reference produces NaN.
__global__ void __launch_bounds__(kBlock) k_tau(DevLevel L, const double2 *__restrict__ V, double accuracy,
                                                double *__restrict__ tau0, double *__restrict__ tau1,
                                                unsigned long long *__restrict__ mins, int safe)
{
	const int e = blockIdx.x * blockDim.x + threadIdx.x;
	if (e == 0) {
		mins[0] = (unsigned long long)__double_as_longlong(1e10);
		mins[1] = (unsigned long long)__double_as_longlong(1e10);
	}
	if (e >= L.nel)
		return;
	const int lv = L.elev[e];
	const double Ld[2] = {L.dx[lv], L.dz[lv]};
	double u[2] = {0.0, 0.0}, xi[2];
#pragma unroll
	for (int d = 0; d < 2; d++) {
#pragma unroll
		for (int a = 0; a < 4; a++) {
			const double2 v = V[L.ienl[a * L.nel + e]];
			u[d] += 0.25 * (d == 0 ? v.x : v.y);
		}
		const double alpha = 0.5 * u[d] * Ld[d] / 1.0;
		if (fabs(alpha) < accuracy)
			xi[d] = 0.0;
		else if (safe && fabs(alpha) > 20.0)
			xi[d] = copysign(1.0, alpha) - 1.0 / alpha;
		else
			xi[d] = cosh(alpha) / sinh(alpha) - 1.0 / alpha;
	}
	const double us = u[0] * u[0] + u[1] * u[1];
	const double kh = (xi[0] * u[0] * Ld[0] + xi[1] * u[1] * Ld[1]) * 0.5;
	tau0[e] = kh * u[0] / us;
	tau1[e] = kh * u[1] / us;
}

// get_element_K_heat (:365-423) row a, and get_element_C_heat (:566-594) row a.
__device__ __forceinline__ void heat_rows(const DevLevel &L, const double2 *__restrict__ V, double t0, double t1,
                                          int e, int a, double (&kr)[4], double (&cr)[4])
{
	double u1 = 0.0, u2 = 0.0;
#pragma unroll
	for (int b = 0; b < 4; b++) {
		const double2 v = V[L.ienl[b * L.nel + e]];
		u1 += v.x * 0.25;
		u2 += v.y * 0.25;
	}
	const double dzh = L.dzh[e], dxh = L.dxh[e], jac = L.jac[e];
#pragma unroll
	for (int b = 0; b < 4; b++) {
		double k = 0.0, c = 0.0;
#pragma unroll
		for (int g = 0; g < 4; g++) {
			const double dNa_dx = cS.dNdxi[a][g] * dzh, dNa_dz = cS.dNdeta[a][g] * dxh;
			const double dNb_dx = cS.dNdxi[b][g] * dzh, dNb_dz = cS.dNdeta[b][g] * dxh;
			const double na_hat = t0 * dNa_dx + t1 * dNa_dz;
			const double tmp1 = u1 * cS.N[a][g] * dNb_dx + u2 * cS.N[a][g] * dNb_dz;
			const double tmp2 = u1 * na_hat * dNb_dx + u2 * na_hat * dNb_dz;
			const double tmp3 = dNa_dx * 1.0 * dNb_dx + dNa_dx * 0.0 * dNb_dz + dNa_dz * 0.0 * dNb_dx
			                  + dNa_dz * 1.0 * dNb_dz;
			k += tmp1 + (tmp2 + tmp3) / jac;
			c += (cS.N[a][g] + na_hat) * cS.N[b][g];
		}
		kr[b] = k;
		cr[b] = c * jac;
	}
}

// The same rows with the common factors taken out of the Gauss-point loop:
// u.grad N_b per (b, g) once, one reciprocal of the Jacobian instead of a
// division per term, and the terms multiplied by the reference's zero
// off-diagonal conductivity dropped.  About a third of the FP64 operations of
// heat_rows (FP64 runs at 1/64 of FP32 on GB300); the rows differ from the
// reference's in the last bits, so the converged solvers use it and the FP64
// replica keeps heat_rows.
__device__ __forceinline__ void heat_rows_fast(const DevLevel &L, const double2 *__restrict__ V, double t0,
                                               double t1, int e, int a, double (&kr)[4], double (&cr)[4])
{
	double u1 = 0.0, u2 = 0.0;
#pragma unroll
	for (int b = 0; b < 4; b++) {
		const double2 v = V[L.ienl[b * L.nel + e]];
		u1 += v.x * 0.25;
		u2 += v.y * 0.25;
	}
	const double dzh = L.dzh[e], dxh = L.dxh[e], jac = L.jac[e], ijac = 1.0 / jac;
	double ax[4], az[4], ah[4], an[4];
#pragma unroll
	for (int g = 0; g < 4; g++) {
		ax[g] = cS.dNdxi[a][g] * dzh;
		az[g] = cS.dNdeta[a][g] * dxh;
		ah[g] = t0 * ax[g] + t1 * az[g];
		an[g] = cS.N[a][g];
	}
#pragma unroll
	for (int b = 0; b < 4; b++) {
		double k = 0.0, c = 0.0;
#pragma unroll
		for (int g = 0; g < 4; g++) {
			const double bx = cS.dNdxi[b][g] * dzh, bz = cS.dNdeta[b][g] * dxh;
			const double ub = u1 * bx + u2 * bz;
			k += an[g] * ub + (ah[g] * ub + ax[g] * bx + az[g] * bz) * ijac;
			c += (an[g] + ah[g]) * cS.N[b][g];
		}
		kr[b] = k;
		cr[b] = c * jac;
	}
}

// One thread per node: rows of heat K, C (same slots as the Stokes blocks) and F.
template <bool FAST>
__device__ __forceinline__ void assemble_heat_node(DevLevel L, const double2 *__restrict__ V,
                                                   const double *__restrict__ tau0, const double *__restrict__ tau1,
                                                   double Q, double *__restrict__ HK, double *__restrict__ HC,
                                                   double *__restrict__ HF)
{
	const int A = blockIdx.x * blockDim.x + threadIdx.x;
	if (A >= L.nno)
		return;
	const int nno = L.nno, nel = L.nel, cnt = L.p2n_cnt[A];
	for (int k = 0; k < L.nbw; k++) {
		HK[(size_t)k * nno + A] = 0.0;
		HC[(size_t)k * nno + A] = 0.0;
	}
	if (!tfree(L, A)) {
		HF[A] = 0.0;
		return;
	}
	double f = 0.0;
	// K rows and Dirichlet lifting (K_matrix_heat, :293-363); C rows (C_matrix_heat, :510-563)
	for (int s = 0; s < cnt; s++) {
		const int e = L.p2n_el[s * nno + A], a = L.p2n_a[s * nno + A];
		double kr[4], cr[4];
		if (FAST)
			heat_rows_fast(L, V, tau0[e], tau1[e], e, a, kr, cr);
		else
			heat_rows(L, V, tau0[e], tau1[e], e, a, kr, cr);
#pragma unroll
		for (int b = 0; b < 4; b++) {
			const int B = L.ienl[b * nel + e];
			if (tfree(L, B)) {
				const int slot = L.kslot[(a * 4 + b) * nel + e];
				HK[(size_t)slot * nno + A] += kr[b];
				HC[(size_t)slot * nno + A] += cr[b];
			} else {
				f -= kr[b] * L.tbcval[B];
			}
		}
	}
	// element loads (F_matrix_heat / get_element_F_heat, :425-508)
	for (int s = 0; s < cnt; s++) {
		const int e = L.p2n_el[s * nno + A], a = L.p2n_a[s * nno + A];
		const double t0 = tau0[e], t1 = tau1[e];
		double fa = 0.0;
#pragma unroll
		for (int g = 0; g < 4; g++) {
			const double dNa_dx = cS.dNdxi[a][g] * L.dzh[e], dNa_dz = cS.dNdeta[a][g] * L.dxh[e];
			const double na_hat = t0 * dNa_dx + t1 * dNa_dz;
			fa += (cS.N[a][g] + na_hat) * Q;
		}
		fa *= L.jac[e];
		int nat = 0;
#pragma unroll
		for (int d = 0; d < 4; d++)
			if (L.tbc[L.ienl[d * nel + e]] == 'F')
				nat += d;
		if (nat == 3)
			nat = 1;
		else if (nat == 1 || nat == 5)
			nat = 2;
		else if (nat == 0 || nat == 2)
			nat = 0;
		if (nat != 0)
			fa -= 0.5 * L.dz[L.elev[e]] * L.tbcval[A];
		f += fa;
	}
	HF[A] = f;
}

__global__ void __launch_bounds__(kBlock) k_assemble_heat(DevLevel L, const double2 *__restrict__ V,
                                                          const double *__restrict__ tau0,
                                                          const double *__restrict__ tau1, double Q,
                                                          double *__restrict__ HK, double *__restrict__ HC,
                                                          double *__restrict__ HF)
{
	assemble_heat_node<false>(L, V, tau0, tau1, Q, HK, HC, HF);
}

__global__ void __launch_bounds__(kBlock) k_assemble_heat_fast(DevLevel L, const double2 *__restrict__ V,
                                                               const double *__restrict__ tau0,
                                                               const double *__restrict__ tau1, double Q,
                                                               double *__restrict__ HK, double *__restrict__ HC,
                                                               double *__restrict__ HF)
{
	assemble_heat_node<true>(L, V, tau0, tau1, Q, HK, HC, HF);
}

// advection_dt (:135-177): min over elements of L^2 and of 0.5/(|u|/L0 + |w|/L1),
// where L0, L1 in the CFL term are those of the LAST element (the reference
// reuses the variable left by its first loop).  Positive doubles order like
// their bit patterns, so an integer minimum is the exact minimum: each block
// reduces its elements' bit patterns (a NaN step contributes nothing, as
// ULLONG_MAX) and one atomicMin per block and value merges the blocks.
__global__ void __launch_bounds__(kBlock) k_heat_dt(DevLevel L, const double2 *__restrict__ V,
                                                    unsigned long long *__restrict__ mins)
{
	__shared__ unsigned long long sh[2][kBlock / 32];
	const int e = blockIdx.x * blockDim.x + threadIdx.x;
	unsigned long long bd = ~0ULL, bs = ~0ULL;
	if (e < L.nel) {
		const int lv = L.elev[e], lvl = L.elev[L.nel - 1];
		const double dx = L.dx[lv], dz = L.dz[lv];
		const double diff = fmin(dx * dx, dz * dz);
		double u1 = 0.0, u2 = 0.0;
#pragma unroll
		for (int a = 0; a < 4; a++) {
			const double2 v = V[L.ienl[a * L.nel + e]];
			u1 += 0.25 * v.x;
			u2 += 0.25 * v.y;
		}
		const double u = fabs(u1) / L.dx[lvl] + fabs(u2) / L.dz[lvl];
		const double step = 0.5 / u;
		bd = (unsigned long long)__double_as_longlong(diff);
		if (!isnan(step))
			bs = (unsigned long long)__double_as_longlong(step);
	}
#pragma unroll
	for (int o = 16; o > 0; o >>= 1) {
		const unsigned long long od = __shfl_xor_sync(0xffffffffu, bd, o), os = __shfl_xor_sync(0xffffffffu, bs, o);
		bd = od < bd ? od : bd;
		bs = os < bs ? os : bs;
	}
	const int w = threadIdx.x >> 5;
	if ((threadIdx.x & 31) == 0) {
		sh[0][w] = bd;
		sh[1][w] = bs;
	}
	__syncthreads();
	if (threadIdx.x == 0) {
		for (int k = 1; k < kBlock / 32; k++) {
			bd = sh[0][k] < bd ? sh[0][k] : bd;
			bs = sh[1][k] < bs ? sh[1][k] : bs;
		}
		atomicMin(&mins[0], bd);
		if (bs != ~0ULL)
			atomicMin(&mins[1], bs);
	}
}

// dt = 0.75 * advection_dt (:37); model_time += dt; A = C/(theta dt) + K;
// B = F + (C T)/(theta dt) (:53-84); x0 = current T on free nodes; 1/diag(A).
__global__ void __launch_bounds__(kBlock) k_heat_system(DevLevel L, const unsigned long long *__restrict__ mins,
                                                        double theta, const double *__restrict__ T,
                                                        const double *__restrict__ HK, const double *__restrict__ HC,
                                                        const double *__restrict__ HF, double *__restrict__ HA,
                                                        double *__restrict__ B, double *__restrict__ x0,
                                                        double *__restrict__ idiag, StepScalars *sc)
{
	const int A = blockIdx.x * blockDim.x + threadIdx.x;
	const double dmin = __longlong_as_double((long long)mins[0]);
	const double cmin = __longlong_as_double((long long)mins[1]);
	const double dt = 0.75 * (cmin < dmin ? cmin : dmin);
	if (A == 0) {
		sc->dt = dt;
		sc->model_time += dt;
	}
	if (A >= L.nno)
		return;
	const int nno = L.nno;
	if (!tfree(L, A)) {
		for (int k = 0; k < L.nbw; k++)
			HA[(size_t)k * nno + A] = 0.0;
		B[A] = 0.0;
		x0[A] = 0.0;
		idiag[A] = 1.0;
		return;
	}
	const double tdt = theta * dt;
	double ct = 0.0;
	for (int k = 0; k < L.nbw; k++) {
		const int Bn = L.nb[(size_t)k * nno + A];
		const double c = HC[(size_t)k * nno + A];
		ct += c * (tfree(L, Bn) ? T[Bn] : 0.0);
		HA[(size_t)k * nno + A] = c / tdt + HK[(size_t)k * nno + A];
	}
	B[A] = HF[A] + ct / tdt;
	x0[A] = T[A];
	idiag[A] = 1.0 / HA[(size_t)L.self_slot[A] * nno + A];
}

__global__ void __launch_bounds__(kBlock) k_heat_cg(HeatArgs a)
{
	cg::grid_group g = cg::this_grid();
	GridRed red = a.red;
	const int cyc = cg_solve(g, red, a.op, a.B, a.x, a.r, a.s, a.d, a.q, a.accu, a.max_cycle, a.precond != 0,
	                         a.precond == 0, &a.sc->status);
	if (blockIdx.x == 0 && threadIdx.x == 0)
		a.sc->heat_cycles = cyc;
}

// T[node] = solution or BC value (:101-111)
__global__ void __launch_bounds__(kBlock) k_heat_writeback(DevLevel L, const double *__restrict__ x,
                                                           double *__restrict__ T)
{
	const int A = blockIdx.x * blockDim.x + threadIdx.x;
	if (A >= L.nno)
		return;
	T[A] = tfree(L, A) ? x[A] : L.tbcval[A];
}

// K x or C x for the parity API (K_prod_d_heat, :935-962)
__global__ void __launch_bounds__(kBlock) k_heat_mul(DevLevel L, const double *__restrict__ M,
                                                     const double *__restrict__ x, double *__restrict__ y)
{
	const int A = blockIdx.x * blockDim.x + threadIdx.x;
	if (A >= L.nno)
		return;
	double s = 0.0;
	for (int k = 0; k < L.nbw; k++)
		s += M[(size_t)k * L.nno + A] * x[L.nb[(size_t)k * L.nno + A]];
	y[A] = tfree(L, A) ? s : 0.0;
}

void *heat_cg_kernel_ptr() { return (void *)k_heat_cg; }

}  // namespace mclg
