// Refinement flags of the |grad T| criterion on the device.
//
// g_e = |grad T| at the centre of finest-level element e from its four corner
// temperatures: with corners 0 (x,z), 1 (x,z+s), 2 (x+s,z+s), 3 (x+s,z) and
// half-widths hx, hz,
//     dT/dx = ((T3 + T2) - (T0 + T1)) / (4 hx),  dT/dz = ((T1 + T2) - (T0 + T3)) / (4 hz).
// An element is flagged when g_e > frac * max_e g_e.  Every operation is an
// explicitly rounded IEEE double operation (no contraction into FMA), so the
// flags are bit-identical to the same formula evaluated on the CPU.
#include "mclg_dev.cuh"

namespace mclg {

__global__ void k_amr_grad(DevLevel L, const double *__restrict__ T, double *__restrict__ g)
{
	for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < L.nel; e += gridDim.x * blockDim.x) {
		const double t0 = T[L.ienl[e]], t1 = T[L.ienl[L.nel + e]], t2 = T[L.ienl[2 * L.nel + e]],
		             t3 = T[L.ienl[3 * L.nel + e]];
		const double gx = __ddiv_rn(__dsub_rn(__dadd_rn(t3, t2), __dadd_rn(t0, t1)), __dmul_rn(4.0, L.dxh[e]));
		const double gz = __ddiv_rn(__dsub_rn(__dadd_rn(t1, t2), __dadd_rn(t0, t3)), __dmul_rn(4.0, L.dzh[e]));
		g[e] = __dsqrt_rn(__dadd_rn(__dmul_rn(gx, gx), __dmul_rn(gz, gz)));
	}
}

// One block: gmax = max_e g_e (order-independent), then the flags.
__global__ void __launch_bounds__(1024) k_amr_flags(int nel, const double *__restrict__ g, double frac,
                                                    unsigned char *__restrict__ flags, double *__restrict__ gmax)
{
	__shared__ double sh[1024];
	double m = 0.0;
	for (int e = threadIdx.x; e < nel; e += blockDim.x)
		m = fmax(m, g[e]);
	sh[threadIdx.x] = m;
	__syncthreads();
	for (int k = blockDim.x / 2; k > 0; k >>= 1) {
		if (threadIdx.x < k)
			sh[threadIdx.x] = fmax(sh[threadIdx.x], sh[threadIdx.x + k]);
		__syncthreads();
	}
	const double thr = __dmul_rn(frac, sh[0]);
	if (threadIdx.x == 0)
		*gmax = sh[0];
	for (int e = threadIdx.x; e < nel; e += blockDim.x)
		flags[e] = g[e] > thr ? 1 : 0;
}

void amr_flags(cudaStream_t st, const DevLevel &L, const double *T, double frac, double *g, unsigned char *flags,
               double *gmax)
{
	int nb = (L.nel + 255) / 256;
	nb = nb < 4096 ? nb : 4096;
	k_amr_grad<<<nb, 256, 0, st>>>(L, T, g);
	k_amr_flags<<<1, 1024, 0, st>>>(L.nel, g, frac, flags, gmax);
}

}  // namespace mclg
