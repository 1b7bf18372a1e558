// Refinement flags of the |grad T| criterion on the device.
//
// g_e = |grad T| at the centre of finest-level element e from its four corner
// temperatures: with corners 0 (x,z), 1 (x,z+s), 2 (x+s,z+s), 3 (x+s,z) and
// half-widths hx, hz,
//     dT/dx = ((T3 + T2) - (T0 + T1)) / (4 hx),  dT/dz = ((T1 + T2) - (T0 + T3)) / (4 hz).
// An element is flagged when g_e > frac * max_e g_e.  Every operation is an
// explicitly rounded IEEE double operation (no contraction into FMA), so the
// flags are bit-identical to the same formula evaluated on the CPU.
#include <cstring>
#include <vector>
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

// ---- the refined tree on the device --------------------------------------------
// The same three stages as the host builder (mclg_amr.c), on byte grids of
// NF x NF finest cells (x-major), each stage a pass over cells that reads the
// previous stage's grid only, so that the result equals the host's sequential
// loops exactly:
//   1. the level each fine cell asks for: target under a flagged element,
//      base elsewhere; its max over 2^k x 2^k blocks (a pyramid);
//   2. top-down split: the leaf level of a cell is the first l >= base at which
//      l == target or no fine cell of its level-l ancestor asks for more;
//   3. 2:1 balance across edges and corners: a leaf with a neighbouring cell more
//      than one level finer splits once per pass, until a pass changes nothing;
// then the leaves' start codes, compacted in Morton order.

__device__ __forceinline__ unsigned tree_compact16(unsigned v)
{
	v &= 0x55555555u;
	v = (v | (v >> 1)) & 0x33333333u;
	v = (v | (v >> 2)) & 0x0f0f0f0fu;
	v = (v | (v >> 4)) & 0x00ff00ffu;
	v = (v | (v >> 8)) & 0x0000ffffu;
	return v;
}

constexpr int kTreeLevelBits = 4;   // Mcode: level in the low 4 bits (Tree.c:302-358)

__global__ void k_tree_request(int nel, const int *__restrict__ Mcode, const unsigned char *__restrict__ flags, int F,
                               int NF, unsigned char target, unsigned char *__restrict__ tgt)
{
	for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < nel; e += gridDim.x * blockDim.x) {
		if (!flags[e])
			continue;
		const int lvl = Mcode[e] & ((1 << kTreeLevelBits) - 1);
		const unsigned code = (unsigned)(Mcode[e] >> kTreeLevelBits);
		const int x0 = (int)tree_compact16(code >> 1), z0 = (int)tree_compact16(code), s = 1 << (F - lvl);
		for (int i = 0; i < s; i++)
			for (int j = 0; j < s; j++)
				tgt[(size_t)(x0 + i) * NF + z0 + j] = target;
	}
}

// pyramid level k (n x n) from level k-1 (2n x 2n)
__global__ void k_tree_pyramid(int n, const unsigned char *__restrict__ prev, unsigned char *__restrict__ cur)
{
	const size_t tot = (size_t)n * n, np = 2 * (size_t)n;
	for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < tot; i += (size_t)gridDim.x * blockDim.x) {
		const size_t x = i / n, z = i - x * n;
		const unsigned char a = prev[2 * x * np + 2 * z], b = prev[2 * x * np + 2 * z + 1];
		const unsigned char c = prev[(2 * x + 1) * np + 2 * z], d = prev[(2 * x + 1) * np + 2 * z + 1];
		unsigned char m = a > b ? a : b;
		m = m > c ? m : c;
		cur[i] = m > d ? m : d;
	}
}

struct TreePyr {
	const unsigned char *lv[16];   // lv[k]: the pyramid's level k, (NF >> k)^2 entries
};

__global__ void k_tree_split(int F, int NF, int base, int target, TreePyr P, unsigned char *__restrict__ lv)
{
	const size_t tot = (size_t)NF * NF;
	for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < tot; i += (size_t)gridDim.x * blockDim.x) {
		const int x = (int)(i / NF), z = (int)(i - (size_t)x * NF);
		int l = base;
		for (; l < target; l++) {
			const int k = F - l, n = NF >> k;
			if (P.lv[k][(size_t)(x >> k) * n + (z >> k)] <= l)
				break;
		}
		lv[i] = (unsigned char)l;
	}
}

__global__ void k_tree_mark(int F, int NF, const unsigned char *__restrict__ lv, unsigned char *__restrict__ mark)
{
	const size_t tot = (size_t)NF * NF;
	for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < tot; i += (size_t)gridDim.x * blockDim.x) {
		const int x = (int)(i / NF), z = (int)(i - (size_t)x * NF);
		const int l = lv[i];
		bool need = false;
		for (int dx = -1; dx <= 1 && !need; dx++)
			for (int dz = -1; dz <= 1; dz++) {
				const int nx = x + dx, nz = z + dz;
				if (nx < 0 || nx >= NF || nz < 0 || nz >= NF)
					continue;
				if (lv[(size_t)nx * NF + nz] > l + 1) {
					need = true;
					break;
				}
			}
		if (need) {   // every cell of the leaf writes the same value at its start cell
			const int s = 1 << (F - l);
			mark[(size_t)(x & ~(s - 1)) * NF + (z & ~(s - 1))] = (unsigned char)(l + 1);
		}
	}
}

__global__ void k_tree_apply(int F, int NF, const unsigned char *__restrict__ mark, unsigned char *__restrict__ lv,
                             int *__restrict__ changed)
{
	const size_t tot = (size_t)NF * NF;
	int any = 0;
	for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < tot; i += (size_t)gridDim.x * blockDim.x) {
		const int x = (int)(i / NF), z = (int)(i - (size_t)x * NF);
		const int s = 1 << (F - lv[i]);
		const unsigned char m = mark[(size_t)(x & ~(s - 1)) * NF + (z & ~(s - 1))];
		if (m) {
			lv[i] = m;
			any = 1;
		}
	}
	if (__syncthreads_or(any) && threadIdx.x == 0)
		atomicOr(changed, 1);
}

// whether the fine cell at Morton code `code` starts its leaf
__device__ __forceinline__ int tree_is_start(int F, int NF, const unsigned char *lv, unsigned code)
{
	const int x = (int)tree_compact16(code >> 1), z = (int)tree_compact16(code);
	const int s = 1 << (F - lv[(size_t)x * NF + z]);
	return ((x | z) & (s - 1)) == 0;
}

constexpr int kTreeChunk = 1024;   // codes per block of the compaction

__global__ void __launch_bounds__(kTreeChunk) k_tree_count(int F, int NF, const unsigned char *__restrict__ lv,
                                                           int *__restrict__ cnt)
{
	const size_t code = (size_t)blockIdx.x * kTreeChunk + threadIdx.x;
	const int f = code < (size_t)NF * NF ? tree_is_start(F, NF, lv, (unsigned)code) : 0;
	const int c = __syncthreads_count(f);
	if (threadIdx.x == 0)
		cnt[blockIdx.x] = c;
}

// one block: off[b] = sum of cnt[0..b-1]; off[nb] = the total
__global__ void __launch_bounds__(1024) k_tree_scan(int nb, const int *__restrict__ cnt, int *__restrict__ off)
{
	__shared__ int sh[1024];
	const int per = (nb + 1023) / 1024, b0 = threadIdx.x * per;
	int s = 0;
	for (int b = b0; b < b0 + per && b < nb; b++)
		s += cnt[b];
	sh[threadIdx.x] = s;
	__syncthreads();
	for (int k = 1; k < 1024; k <<= 1) {   // inclusive scan of the thread sums
		const int v = threadIdx.x >= k ? sh[threadIdx.x - k] : 0;
		__syncthreads();
		sh[threadIdx.x] += v;
		__syncthreads();
	}
	int run = sh[threadIdx.x] - s;
	for (int b = b0; b < b0 + per && b < nb; b++) {
		off[b] = run;
		run += cnt[b];
	}
	if (threadIdx.x == 1023)
		off[nb] = sh[1023];
}

__global__ void __launch_bounds__(kTreeChunk) k_tree_write(int F, int NF, const unsigned char *__restrict__ lv,
                                                           const int *__restrict__ off, int *__restrict__ leaves)
{
	__shared__ int wsum[kTreeChunk / 32];
	const size_t code = (size_t)blockIdx.x * kTreeChunk + threadIdx.x;
	const int f = code < (size_t)NF * NF ? tree_is_start(F, NF, lv, (unsigned)code) : 0;
	const unsigned bal = __ballot_sync(0xffffffffu, f);
	const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
	if (lane == 0)
		wsum[w] = __popc(bal);
	__syncthreads();
	int before = 0;
	for (int k = 0; k < w; k++)
		before += wsum[k];
	if (f)
		leaves[off[blockIdx.x] + before + __popc(bal & ((1u << lane) - 1u))] = (int)code;
}

static int tree_grid(size_t n)
{
	const size_t b = (n + 255) / 256;
	return (int)(b < 8192 ? (b < 1 ? 1 : b) : 8192);
}

// Leaves (finest-level Morton start codes, sorted) of the refined tree from
// per-element flags, all on the device.  Mcode and flags: the finest level's
// elements (device).  Levels are checked by the caller.  Work memory is
// allocated here and released before returning.
cudaError_t amr_tree_leaves(cudaStream_t st, int nel, const int *Mcode, const unsigned char *flags, int F, int base,
                            int target, std::vector<int> &leaves, long long *launches)
{
	const int NF = 1 << F;
	const size_t cells = (size_t)NF * NF;
	const int nk = F - base;                       // pyramid levels above the fine grid
	if (F < 0 || F > 14 || nk < 0 || nk >= 16)
		return cudaErrorInvalidValue;
	const int nb = (int)((cells + kTreeChunk - 1) / kTreeChunk);
	size_t pyr_bytes = 0;
	for (int k = 1; k <= nk; k++)
		pyr_bytes += (size_t)(NF >> k) * (NF >> k);
	unsigned char *buf = NULL;
	int *ibuf = NULL, *dleaves = NULL;
	cudaError_t e = cudaMalloc((void **)&buf, 3 * cells + pyr_bytes + 16);
	if (e == cudaSuccess)
		e = cudaMalloc((void **)&ibuf, (2 * (size_t)nb + 2) * sizeof(int));
	unsigned char *tgt = buf, *lv = buf + cells, *mark = buf + 2 * cells, *pyr = buf + 3 * cells;
	int *cnt = ibuf, *off = ibuf + nb, *changed = ibuf + 2 * nb + 1;
	int total = 0, flag = 0;
	TreePyr P;
	memset(&P, 0, sizeof P);
	if (e == cudaSuccess)
		e = cudaMemsetAsync(tgt, base, cells, st);
	if (e == cudaSuccess) {
		k_tree_request<<<tree_grid(nel), 256, 0, st>>>(nel, Mcode, flags, F, NF, (unsigned char)target, tgt);
		P.lv[0] = tgt;
		unsigned char *p = pyr;
		for (int k = 1; k <= nk; k++) {
			const int n = NF >> k;
			k_tree_pyramid<<<tree_grid((size_t)n * n), 256, 0, st>>>(n, P.lv[k - 1], p);
			P.lv[k] = p;
			p += (size_t)n * n;
		}
		k_tree_split<<<tree_grid(cells), 256, 0, st>>>(F, NF, base, target, P, lv);
		*launches += 2 + nk;
		e = cudaGetLastError();
	}
	// each pass raises some leaf by one level; levels are bounded by F, so a
	// correct pass count is at most (F + 1) per leaf chain: cap it generously
	for (int pass = 0; e == cudaSuccess && pass < 4 * (F + 2); pass++) {
		e = cudaMemsetAsync(mark, 0, cells, st);
		if (e == cudaSuccess)
			e = cudaMemsetAsync(changed, 0, sizeof(int), st);
		if (e != cudaSuccess)
			break;
		k_tree_mark<<<tree_grid(cells), 256, 0, st>>>(F, NF, lv, mark);
		k_tree_apply<<<tree_grid(cells), 256, 0, st>>>(F, NF, mark, lv, changed);
		*launches += 2;
		e = cudaGetLastError();
		if (e == cudaSuccess)
			e = cudaMemcpyAsync(&flag, changed, sizeof(int), cudaMemcpyDeviceToHost, st);
		if (e == cudaSuccess)
			e = cudaStreamSynchronize(st);
		if (e != cudaSuccess || !flag)
			break;
	}
	if (e == cudaSuccess && flag)
		e = cudaErrorUnknown;   // no fixed point within the cap (cannot happen for a valid level grid)
	if (e == cudaSuccess) {
		k_tree_count<<<nb, kTreeChunk, 0, st>>>(F, NF, lv, cnt);
		k_tree_scan<<<1, 1024, 0, st>>>(nb, cnt, off);
		*launches += 2;
		e = cudaGetLastError();
	}
	if (e == cudaSuccess)
		e = cudaMemcpyAsync(&total, off + nb, sizeof(int), cudaMemcpyDeviceToHost, st);
	if (e == cudaSuccess)
		e = cudaStreamSynchronize(st);
	if (e == cudaSuccess)
		e = cudaMalloc((void **)&dleaves, ((size_t)total + 1) * sizeof(int));
	if (e == cudaSuccess) {
		k_tree_write<<<nb, kTreeChunk, 0, st>>>(F, NF, lv, off, dleaves);
		*launches += 1;
		e = cudaGetLastError();
	}
	if (e == cudaSuccess) {
		leaves.resize((size_t)total);
		e = cudaMemcpyAsync(leaves.data(), dleaves, (size_t)total * sizeof(int), cudaMemcpyDeviceToHost, st);
	}
	if (e == cudaSuccess)
		e = cudaStreamSynchronize(st);
	cudaFree(dleaves);
	cudaFree(ibuf);
	cudaFree(buf);
	return e;
}

}  // namespace mclg
