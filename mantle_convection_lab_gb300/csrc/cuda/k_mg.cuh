// Types shared by the converged-solve kernel (k_mg.cu) and its host launcher.
#pragma once
#include "team.cuh"

namespace mclg {

constexpr int kMaxLev = 14;

template <class T> struct V2T;
template <> struct V2T<float> { typedef float2 t; };
template <> struct V2T<double> { typedef double2 t; };

// One level of the structured hierarchy (level 0 = finest).  Nodes are
// x-major, A = iz + ix*n, as the reference numbers them on a uniform mesh.
template <class T>
struct MGLevel {
	int N, n;                    // elements / nodes per side
	const unsigned char *mask;   // [n*n] bit0: u Dirichlet, bit1: w Dirichlet
	T *eta;                      // [n*n] viscosity (level 0: converted, coarser: injected)
	typename V2T<T>::t *invD, *xa, *xb, *b, *r;
};

template <class T>
struct MGHier {
	int nlev;                    // number of levels
	int nblk;                    // levels >= nblk run inside block 0 only
	MGLevel<T> lv[kMaxLev];
	T *cinv;                     // dense inverse of the coarsest operator [cnd*cnd]
	double *cwork;               // [cnd * 2*cnd] scratch for the inversion
	int cnd;                     // 2 * n_coarsest^2
	T omega;
	int nu;                      // smoothing sweeps per side on the lfine finest levels
	int nu_c, lfine;             // ... and on the coarser ones
	int eta_avg;                 // coarse viscosity: 0 injection, 1 full-weighted mean, 2 full-weighted log-mean
	// degree-2 Chebyshev smoothing (cheb != 0, nu == nu_c == 2): x1 = x0 + w1 D^-1 r0,
	// x2 = c1 x1 - c0 x0 + w2 D^-1 r1
	int cheb;
	T w1, w2, c1, c0;
	// inner CG vectors on level 0
	typename V2T<T>::t *px, *pr, *pz, *pp, *pq;
};

// G coefficients (Build_matrix.c get_element_G) of the 4 corners of an
// element of the uniform mesh, filled on the host.
struct GTab {
	double g0[4], g1[4];
	float g0h[4], g0l[4], g1h[4], g1l[4];   // the same as float pairs: g = h + l
};

// The converged Stokes solve of one time step (FP64 state, TI inner solves).
template <class TI>
struct MGArgs {
	MGHier<TI> H;
	int N0;                      // fine elements per side
	double hx, hz;               // fine element half-widths (dx_dxi, dz_deta)
	GTab gt;                     // G coefficients for those half-widths
	const double *vis;           // [nno] viscosity (FP64, G.node order == x-major)
	const unsigned char *mask0;  // fine-level Dirichlet mask
	const double *vbcval;        // [2*nno] BC values (for the nodal velocity)
	const double2 *F;            // [nno] right-hand side (Dirichlet rows zero)
	double2 *d;                  // [nno] velocity (FP64 state, warm start on entry)
	double *p;                   // [nel] pressure, Morton order
	double2 *V;                  // [nno] nodal velocity out (v_to_nodes)
	double2 *R, *dd, *u1, *Kd, *invD64, *kdiag64;   // FP64 node vectors
	double *Rc, *r0, *r1, *r2, *z0, *z1, *s1, *s2, *Ahp, *dpv, *bab;  // FP64 element vectors
	int method;                  // correction solve: 0 Uzawa with inner MG-PCG, 1 MINRES (block-diagonal preconditioner)
	double2 *mv[2], *mw[2];      // MINRES Lanczos and direction vectors, velocity part (z_u lives in TI)
	double *mvp[2], *mzp[2], *mwp[2]; // Lanczos, preconditioned and direction vectors, pressure part (Morton)
	// warm_start=4: the last three solutions (h1 the most recent), or null
	const double2 *h1d, *h2d, *h3d;
	const double *h1p, *h2p, *h3p;
	const double2 *d_alt;        // second candidate guess (previous solution) or null
	const double *p_alt;
	int guess_force;             // keep (d, p) without judging it against (d_alt, p_alt)
	GridRed red;
	StepScalars *sc;
	double rtol, outer_rtol, inner_rtol;
	int max_refine, max_outer, max_inner;
};

}  // namespace mclg
