// The team of blocks that runs one converged solve, shared by the uniform
// (k_mg.cu) and the refined-mesh (k_qt.cu) solvers: the whole cooperative
// grid (one model per launch), one thread-block cluster of a batched launch,
// or one block of a batched launch.
#pragma once
#include "mclg_dev.cuh"

namespace mclg {

// The blocks that share a pass over a level: block `rank` of `size` (the
// whole grid, a thread-block cluster, or one block alone).
struct Part {
	int rank, size;
};

// ---- where a solve runs ---------------------------------------------------------
// The team of blocks that solves one model:
//   SYNC_GRID     the whole cooperative grid (grid barriers, deterministic
//                 grid reductions through global memory);
//   SYNC_CLUSTER  one thread-block cluster of a batch (cluster barriers,
//                 reductions over the blocks' shared memory, read through
//                 distributed shared memory in rank order);
//   SYNC_BLOCK    one block of a batch (block barriers and reductions).
enum { SYNC_GRID = 0, SYNC_CLUSTER = 1, SYNC_BLOCK = 2 };

struct Sync {
	int mode;
	cg::grid_group *g;
	GridRed red;
	double *cpart;               // SYNC_CLUSTER: this block's [2][kRedWidth] partials (shared memory)
	int cflip;
	int rank, size;              // this block in the team
	int tid, nth;
	__device__ void sync()
	{
		if (mode == SYNC_GRID)
			g->sync();
		else if (mode == SYNC_CLUSTER)
			cg::this_cluster().sync();
		else
			__syncthreads();
	}
	template <int NV>
	__device__ void reduce(double (&v)[NV])
	{
		if (mode == SYNC_GRID) {
			grid_reduce<NV>(*g, red, v, 0u);
		} else if (mode == SYNC_CLUSTER) {
			block_reduce<NV>(v, 0u);
			double *mine = cpart + cflip * kRedWidth;
			if (threadIdx.x == 0)
				for (int k = 0; k < NV; k++)
					mine[k] = v[k];
			cg::cluster_group cl = cg::this_cluster();
			cl.sync();
			double acc[NV];
			for (int k = 0; k < NV; k++)
				acc[k] = 0.0;
			for (int r = 0; r < size; r++) {
				const double *other = cl.map_shared_rank(mine, r);
				for (int k = 0; k < NV; k++)
					acc[k] += other[k];
			}
			for (int k = 0; k < NV; k++)
				v[k] = acc[k];
			cflip ^= 1;   // the next reduction writes the other buffer (see GridRed)
		} else {
			block_reduce<NV>(v, 0u);
		}
	}
	__device__ bool leader() const { return rank == 0; }
	// the blocks of a pass: the team for team-wide levels, this block alone otherwise
	__device__ Part part(bool wide) const { return wide ? Part{rank, size} : Part{0, 1}; }
};

__device__ __forceinline__ void barrier(Sync &sy, bool grid)
{
	if (grid)
		sy.sync();
	else
		__syncthreads();
}

}  // namespace mclg
