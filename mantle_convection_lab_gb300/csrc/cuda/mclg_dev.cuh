// Device-side layout and helpers of the GB300 time-step engine.
//
// Vectors live in node-major layout: a velocity vector is double2 per node
// (u, w) over the sorted node list, a temperature vector one double per node.
// Dirichlet entries are held at exactly zero, so dot products equal the
// reference's sums over its compressed equation numbering (G.id / G.heat.id,
// Construct_ien_id_lm.c:79-144), which only drops those zeros.
//
// The assembled Stokes operator is stored node-block-ELL: for node A and
// neighbour slot k (neighbours sorted by node index, as the reference sorts
// each row, Build_matrix.c:720-738) one 2x2 block
//     K[(k*nno + A)] = {K_uu, K_uw, K_wu, K_ww}
// so a row's sum visits columns in the reference's order.  Heat K, C and A
// use the same neighbour slots with one double per slot.
#pragma once
#include <cooperative_groups.h>
#include <cuda_runtime.h>
#include <stdint.h>

namespace mclg {

namespace cg = cooperative_groups;

constexpr int kBlock = 256;            // threads per block of every kernel
constexpr int kMaxCoopBlocks = 4096;   // partial-sum slots per reduction buffer
constexpr int kRedWidth = 4;           // values reduced together

// Q1 shape-function tables at the 4 Gauss points and the centre,
// computed on the host exactly as Shape_function.c:17-121 does.
struct ShapeTables {
	double N[4][4];        // N[a][g]
	double dNdxi[4][4];    // dN_dxi[a][g]
	double dNdeta[4][4];   // dN_deta[a][g]
	double dNdxi_c[4];     // at the centre
	double dNdeta_c[4];
};

// The tables live in constant memory.  Without relocatable device code a
// __constant__ symbol is private to its translation unit, so every .cu file
// that reads cS holds its own copy and exports an upload function defined
// with MCLG_SHAPE_UPLOAD; the context fills all of them at creation.
static __constant__ ShapeTables cS;
#define MCLG_SHAPE_UPLOAD(fn)                                                     \
	void fn(const ShapeTables &s, cudaStream_t st)                                \
	{                                                                             \
		cudaMemcpyToSymbolAsync(cS, &s, sizeof s, 0, cudaMemcpyHostToDevice, st); \
	}

// Device copy of one mesh level (pointers into device memory).
struct DevLevel {
	int nel, nno, nbw, nh, hang_chained, gnox, gnoz, fine_level;
	const int *node;            // [nno]   sorted global node ids (iz + ix*gnoz)
	const int *ienl;            // [4*nel] local corner nodes, ienl[a*nel + e]
	const int *elev;            // [nel]   element level
	const double *dxh, *dzh, *jac, *area;  // [nel] dx_dxi, dz_deta, jacobi, area
	const char *vbc;            // [2*nno] velocity BC code, vbc[d*nno + A]
	const double *vbcval;       // [2*nno]
	const char *tbc;            // [nno]
	const double *tbcval;       // [nno]
	const double *X;            // [2*nno]
	const int *p2n_cnt, *p2n_el, *p2n_a;  // [nno], [4*nno], [4*nno]
	const int *nb;              // [nbw*nno] neighbour nodes
	const unsigned char *self_slot;  // [nno] slot k with nb[k][A] == A
	const unsigned char *kslot; // [16*nel]
	const int *hang_ni, *hang_ci0, *hang_ci1;  // [nh]
	const int *cell_elem;       // [(gnox-1)*(gnoz-1)]
	const double *dx, *dz;      // [levels] element size per level
};

// Scalars shared by the kernels of one step, resident on the device so that
// no kernel needs a host round trip.
// Status bits written to StepScalars::status.
constexpr int kStatCap = 1, kStatNan = 2, kStatBreakdown = 4;

struct StepScalars {
	double dt, model_time;
	double accuracy;            // inner tolerance in use (auto_accuracy may rescale it)
	double dv, dp;
	double res_m, res_c, fnorm;
	int uzawa_cycles, cg_cycles, heat_cycles, status;
	int refine_passes;
	int nsolved;                // converged solves since the warm-start history began (warm_start=4)
	double warm_a, warm_b;      // warm_start=4: the coefficients of the chosen start
	int guess_used;             // learned guess: 1 network, 0 previous solution, -1 not judged
	double res_learned, res_prev;   // relative FP64 residuals of the two candidates
};

// ---- deterministic grid-wide reductions -----------------------------------
// Every block writes one partial per value, the grid synchronises, and every
// block then sums all partials in the same fixed order, so all blocks hold
// bitwise-identical scalars and take identical branches.  Two partial buffers
// alternate: a block can only overwrite a buffer after the next grid barrier,
// by which time every block has finished reading it.
struct GridRed {
	double *part;   // [2][kMaxCoopBlocks][kRedWidth]
	int flip;
};

__device__ __forceinline__ double warp_sum(double v)
{
#pragma unroll
	for (int o = 16; o > 0; o >>= 1)
		v += __shfl_xor_sync(0xffffffffu, v, o);
	return v;
}

__device__ __forceinline__ double warp_max(double v)
{
#pragma unroll
	for (int o = 16; o > 0; o >>= 1)
		v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
	return v;
}

// Reduce NV values over the block; op bit k set => value k is a max, else a sum.
// Result is valid in every thread.
template <int NV>
__device__ __forceinline__ void block_reduce(double (&v)[NV], unsigned op)
{
	__shared__ double sh[kBlock / 32][kRedWidth];
	__shared__ double out[kRedWidth];
	const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
	for (int k = 0; k < NV; k++)
		v[k] = ((op >> k) & 1u) ? warp_max(v[k]) : warp_sum(v[k]);
	__syncthreads();   // protect sh/out from a previous call
	if (lane == 0) {
#pragma unroll
		for (int k = 0; k < NV; k++)
			sh[wid][k] = v[k];
	}
	__syncthreads();
	if (wid == 0) {
#pragma unroll
		for (int k = 0; k < NV; k++) {
			const bool mx = (op >> k) & 1u;
			double t = lane < kBlock / 32 ? sh[lane][k] : (mx ? -1.0 : 0.0);
			t = mx ? warp_max(t) : warp_sum(t);
			if (lane == 0)
				out[k] = t;
		}
	}
	__syncthreads();
#pragma unroll
	for (int k = 0; k < NV; k++)
		v[k] = out[k];
}

// Grid-wide reduction (contains one grid barrier).  Max values must be >= 0.
template <int NV>
__device__ __forceinline__ void grid_reduce(cg::grid_group &g, GridRed &red, double (&v)[NV], unsigned op)
{
	block_reduce<NV>(v, op);
	double *buf = red.part + (size_t)red.flip * kMaxCoopBlocks * kRedWidth;
	if (threadIdx.x == 0) {
#pragma unroll
		for (int k = 0; k < NV; k++)
			buf[blockIdx.x * kRedWidth + k] = v[k];
	}
	g.sync();
	double acc[NV];
#pragma unroll
	for (int k = 0; k < NV; k++)
		acc[k] = ((op >> k) & 1u) ? 0.0 : 0.0;
	for (unsigned b = threadIdx.x; b < gridDim.x; b += blockDim.x) {
#pragma unroll
		for (int k = 0; k < NV; k++) {
			const double t = buf[b * kRedWidth + k];
			acc[k] = ((op >> k) & 1u) ? fmax(acc[k], t) : acc[k] + t;
		}
	}
	block_reduce<NV>(acc, op);
#pragma unroll
	for (int k = 0; k < NV; k++)
		v[k] = acc[k];
	red.flip ^= 1;
}

__device__ __forceinline__ bool vfree(const DevLevel &L, int A, int c)
{
	return L.vbc[c * L.nno + A] != 'V';
}

__device__ __forceinline__ bool tfree(const DevLevel &L, int A)
{
	return L.tbc[A] != 'T';
}

// G_e entries (get_element_G, Build_matrix.c:346-381): g[2a+0], g[2a+1].
__device__ __forceinline__ void element_g(const ShapeTables &S, double dzh, double dxh, int a, double &g0, double &g1)
{
	g0 = 0.0;
	g1 = 0.0;
#pragma unroll
	for (int gs = 0; gs < 4; gs++) {
		g0 -= S.dNdxi[a][gs] * dzh;
		g1 -= S.dNdeta[a][gs] * dxh;
	}
}

// Corner order of an element sorted by node index: ien corners 0=(x,z),
// 1=(x,z+s), 2=(x+s,z+s), 3=(x+s,z) have node ids n0 < n1 < n3 < n2.
__constant__ static const int kSortedCorner[4] = {0, 1, 3, 2};

// G p at node A (G_prod_p, Solver.c:569-591): row entries in element order.
__device__ __forceinline__ void gmul_node(const DevLevel &L, const double *__restrict__ p, int A,
                                          double &y0, double &y1)
{
	double s0 = 0.0, s1 = 0.0;
	for (int k = 0; k < L.p2n_cnt[A]; k++) {
		const int e = L.p2n_el[k * L.nno + A], a = L.p2n_a[k * L.nno + A];
		double g0, g1;
		element_g(cS, L.dzh[e], L.dxh[e], a, g0, g1);
		s0 += g0 * p[e];
		s1 += g1 * p[e];
	}
	y0 = vfree(L, A, 0) ? s0 : 0.0;
	y1 = vfree(L, A, 1) ? s1 : 0.0;
}

// (G^T u)_e (GT_prod_d, Solver.c:645-666): the element's free dofs in
// ascending equation order.
__device__ __forceinline__ double gtmul_elem(const DevLevel &L, const double2 *__restrict__ u, int e)
{
	double s = 0.0;
#pragma unroll
	for (int c = 0; c < 4; c++) {
		const int a = kSortedCorner[c];
		const int A = L.ienl[a * L.nel + e];
		double g0, g1;
		element_g(cS, L.dzh[e], L.dxh[e], a, g0, g1);
		const double2 ua = u[A];
		if (vfree(L, A, 0))
			s += g0 * ua.x;
		if (vfree(L, A, 1))
			s += g1 * ua.y;
	}
	return s;
}

// ---- kernel argument blocks (shared by the host launch code) ---------------
// One level of the hierarchy of the reference's own inner solvers
// (solver="gs": the finest level alone; solver="mg": mg_min_level up to the
// finest).  Node layout, both directions of node A in one double2.  Transfer
// entries name a dof of the neighbouring level as 2*node + direction.
struct RefLevel {
	int nno, nbw, nwave;
	const int *nb;                  // [nbw*nno] matrix neighbours (the level's sorted node list)
	const unsigned char *self_slot; // [nno] slot of the node itself in nb
	const char *vbc;                // [2*nno] BC codes: 'V' fixed
	const double4 *K;               // [nbw*nno] 2x2 blocks
	const int *wave;                // [nno] nodes ordered by Gauss-Seidel wavefront
	const int *wave_off;            // [nwave+1]
	const int *itp_n;               // [2*nno] terms of the interpolated error (0: not set), from the level below
	const int *itp_src;             // [8*nno] itp_src[(i*2+c)*nno + A]: dof of the level below, -1 fixed
	const int *prj;                 // [2*nno] dof of the level above whose residual this dof takes, -1 fixed
	double2 *err, *rhs, *res, *xt;  // G.err[lev], projected right-hand side, residual, sweep copy
};
struct RefMG {
	int nlev, cycles, fine_it, coarse_it;   // levels lev[0] (coarsest) .. lev[nlev-1] (finest)
	RefLevel lev[16];
};
enum { kRefNone = 0, kRefGS = 1, kRefMG = 2 };

struct UzawaArgs {
	DevLevel L;
	const double4 *K;
	const double2 *idiag, *F;
	const double *bab;
	double2 *d, *u1, *Ah, *r, *s, *dd, *q, *xt, *V;
	double *p, *r0, *r1, *r2, *z0, *z1, *s1, *s2, *Ahp;
	GridRed red;
	StepScalars *sc;
	int max_citcom, max_cg, precond, check_v_only, solver_jc, auto_accuracy, neq;
	double citcom_accu, accuracy;
	int ref_kind;          // kRefGS / kRefMG: the inner solve is the reference's gauss_seidel / multigrid
	const RefMG *ref;      // device copy of the hierarchy
};

// Scalar heat operator A = C/(theta dt) + K on the neighbour slots.
struct HeatOp {
	static constexpr int NC = 1;
	DevLevel L;
	const double *HA, *idiag;
	__device__ int nunits() const { return L.nno; }
	__device__ bool is_free(int A, int) const { return tfree(L, A); }
	__device__ double inv_diag(int A, int) const { return idiag[A]; }
	__device__ void apply(const double *x, int A, double (&y)[1]) const
	{
		double s = 0.0;
		for (int k = 0; k < L.nbw; k++)
			s += HA[(size_t)k * L.nno + A] * x[L.nb[(size_t)k * L.nno + A]];
		y[0] = tfree(L, A) ? s : 0.0;
	}
	__device__ int nhang() const { return L.nh; }
	// enforce_constrain_Teq (Update_temperature.c:829-933)
	__device__ void hang_one(double *x, int h) const
	{
		const int ni = L.hang_ni[h], c0 = L.hang_ci0[h], c1 = L.hang_ci1[h];
		double t = (tfree(L, c0) ? x[c0] : L.tbcval[c0]) + (tfree(L, c1) ? x[c1] : L.tbcval[c1]);
		t *= 0.5;
		if (tfree(L, ni))
			x[ni] = t;
	}
	__device__ void constrain(double *x, int tid, int nth) const
	{
		if (L.hang_chained) {
			if (tid == 0)
				for (int h = 0; h < L.nh; h++)
					hang_one(x, h);
		} else {
			for (int h = tid; h < L.nh; h += nth)
				hang_one(x, h);
		}
	}
};

struct HeatArgs {
	HeatOp op;
	const double *B;
	double *x, *r, *s, *d, *q;
	GridRed red;
	StepScalars *sc;
	int max_cycle, precond;
	double accu;
};

}  // namespace mclg
