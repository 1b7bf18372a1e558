// Converged Stokes solve on quadtree meshes with hanging nodes (k_qt.cu):
// the conforming system C^T K C d + C^T G p = C^T F, G^T C d = 0 (C expands
// the reduced dofs to hanging nodes), solved by FP64 iterative refinement
// around MINRES with the block-diagonal preconditioner diag(V-cycle, BAB).
// The V-cycle runs in TI on the mesh's own level hierarchy (the reference's
// MG levels, Tree.c) with the reference's averaging prolongation
// (Connection.c:708-930), its transpose as restriction, damped Jacobi on the
// constrained operator and a dense solve on the coarsest level.
#pragma once
#include "team.cuh"

namespace mclg {

template <class T> struct V4T;
template <> struct V4T<float> { typedef float4 t; };
template <> struct V4T<double> { typedef double4 t; };
template <class T> struct Q2T;
template <> struct Q2T<float> { typedef float2 t; };
template <> struct Q2T<double> { typedef double2 t; };

// One level; dofs are 2*node + component, vectors node layout (T2 per node).
// A column entry of nbf: the neighbour node, with kQtCon set when one of its
// components is constrained (read through the expansion; the others are read
// as stored, fixed entries being kept at 0).
constexpr int kQtCon = 1 << 30;

template <class T>
struct QtLevel {
	int nno, nbw;
	const int *nb;                          // [nbw*nno] matrix neighbours (flagged, see kQtCon)
	const unsigned char *cnt;               // [nno] neighbours of each node
	const double4 *K64;                     // [nbw*nno] FP64 blocks assembled this step
	const unsigned char *kind;              // [2*nno] 0 fixed, 1 reduced, 2 constrained
	const int *ex_off, *ex_src;             // [2*nno+1] constrained dof = sum ex_w * x[ex_src]
	const T *ex_w;
	const int *fo_off, *fo_dof;             // [2*nno+1] reduced dof <- constrained dofs holding it
	const T *fo_w;
	int rnbw;                               // C^T K C as node-block ELL over reduced columns:
	const int *rnb;                         // [rnbw*nno] columns (padded with the row node)
	const unsigned char *rcnt;              // [nno] columns per row
	const int *rc_off, *rc_tgt, *rc_src;    // its assembly from K64 (see mclg_qt_level)
	const float *rc_w;
	typename V4T<T>::t *Kr;                 // [rnbw*nno] the assembled blocks in T
	const int *p_off, *p_src;               // prolongation from the level below (rows: this level)
	const T *p_w;
	const int *r_off, *r_src;               // restriction from the level above (rows: this level)
	const T *r_w;
	T *invD;                                // [2*nno]
	typename Q2T<T>::t *x[2], *b, *r;       // work vectors
};

template <class T>
struct QtHier {
	int nlev;                               // lv[0] coarsest .. lv[nlev-1] finest
	QtLevel<T> lv[16];
	int smooth;                             // Jacobi sweeps before and after the coarse correction
	T omega;
	int nblk;                               // levels lv[0..nblk-1] are small: block 0 alone runs them
	int nc;                                 // reduced dofs of the coarsest level
	const int *cdof;                        // [nc] their dof numbers
	double *cwork;                          // [nc * 2nc] Gauss-Jordan workspace
	T *cinv;                                // [nc * nc] inverse of the coarsest constrained operator
	double *cvec;                           // [2 * nno_coarsest] unit-vector scratch (FP64)
};

template <class TI>
struct QtArgs {
	DevLevel L;                             // the finest level
	QtHier<TI> H;
	const double2 *F;
	const double *bab;
	double2 *d, *V;
	double *p;
	// FP64 refinement and MINRES vectors
	double2 *R, *Kd, *dd, *u1, *mv[2], *mw[2];
	double *Rc, *dpv, *Ahp, *mvp[2], *mzp[2], *mwp[2];
	typename Q2T<TI>::t *mz[2], *kz;
	GridRed red;
	StepScalars *sc;
	double rtol, outer_rtol;
	int max_refine, max_outer;
};

void *qt_kernel(int fp64);
// Refined members of an ensemble solved in one launch: each thread-block
// cluster (or block) takes the next model from a queue (QtArgs<TI>[n] on the
// device, largest first) and solves it with team barriers only.
void *qt_batch_kernel(int fp64);

}  // namespace mclg
