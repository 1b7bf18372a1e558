// Numbering, boundary codes, geometry and hanging nodes of a quadtree mesh on
// the device.  Every array equals the host builder's (mclg_mesh.c) byte for
// byte: the orders that the host gets from sequential loops -- the sorted node
// list, the equation numbers, the hanging-node list in element-then-edge
// order, the node->element map in ascending element order -- come from
// exclusive scans here, and each floating-point value is the same single
// IEEE operation (explicitly rounded, no contraction).
//   leaf levels, MG projection   Tree.c:340-389
//   ien / node list              Construct_ien_id_lm.c:3-66
//   id / heat id                 Construct_ien_id_lm.c:79-144
//   boundary codes               Boundary_condition.c:10-110
//   coordinates, geometry        Mesh.c:430-452, Shape_function.c:123-167, Construct_ien_id_lm.c:198-244
//   hanging nodes                Connection.c:59-276 (the single-rank part)
// The leaf list must describe a quadtree (each gap to the next start code a
// power of 4 that the code is aligned to); the host builder does not check
// that, this one rejects other lists.
#include <cuda_runtime.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <mutex>
#include <vector>
#include "../host/mclg_host.h"

#define CUDA_TRY(x)                             \
	do {                                        \
		const cudaError_t e_ = (x);             \
		if (e_ != cudaSuccess)                  \
			return e_;                          \
	} while (0)

namespace {

constexpr int kT = 256;
constexpr int kScanT = 512, kScanPer = 8, kScanTile = kScanT * kScanPer;
constexpr long kLutMax = 1L << 22;   // the host keeps a node-id table up to this many ids

int grid_for(long n)
{
	const long g = (n + kT - 1) / kT;
	return (int)(g < 1 ? 1 : g > 8192 ? 8192 : g);
}

#define GRID_STRIDE(i, n) for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < (n); i += (long)gridDim.x * blockDim.x)

__device__ __forceinline__ int d_log4i(int a)
{
	int b = 0;
	while (a >>= 2)
		b++;
	return b;
}

// x from the odd bits, z from the even bits (demorton_no_lev, Tree.c:433-444)
__device__ __forceinline__ void d_demorton(int code, int &x, int &z)
{
	const unsigned c = (unsigned)code;
	x = z = 0;
	for (int i = 0; i < 16; i++) {
		x |= (int)(((c >> (2 * i + 1)) & 1u) << i);
		z |= (int)(((c >> (2 * i)) & 1u) << i);
	}
}

__device__ __forceinline__ int d_morton(int x, int z)
{
	unsigned c = 0;
	for (int i = 0; i < 16; i++)
		c |= ((((unsigned)x >> i) & 1u) << (2 * i + 1)) | ((((unsigned)z >> i) & 1u) << (2 * i));
	return (int)c;
}

__device__ __forceinline__ int pack_mcode(int loc, int level)
{
	return (int)(((unsigned)loc << MCLG_LEVEL_BITS) | (unsigned)level);
}

// ---- exclusive scan of int arrays (in place) -------------------------------

__global__ void __launch_bounds__(kScanT) k_scan_tile(int *a, long n, int *tile_sum)
{
	__shared__ int sh[kScanT];
	const long base = (long)blockIdx.x * kScanTile + (long)threadIdx.x * kScanPer;
	int v[kScanPer], s = 0;
	for (int i = 0; i < kScanPer; i++) {
		v[i] = base + i < n ? a[base + i] : 0;
		s += v[i];
	}
	sh[threadIdx.x] = s;
	__syncthreads();
	for (int off = 1; off < kScanT; off <<= 1) {
		const int t = threadIdx.x >= off ? sh[threadIdx.x - off] : 0;
		__syncthreads();
		sh[threadIdx.x] += t;
		__syncthreads();
	}
	int run = sh[threadIdx.x] - s;
	if (threadIdx.x == kScanT - 1 && tile_sum != nullptr)
		tile_sum[blockIdx.x] = sh[threadIdx.x];
	for (int i = 0; i < kScanPer; i++) {
		if (base + i < n)
			a[base + i] = run;
		run += v[i];
	}
}

__global__ void __launch_bounds__(kScanT) k_scan_add(int *a, long n, const int *tile_off)
{
	const int o = tile_off[blockIdx.x];
	long k = (long)blockIdx.x * kScanTile + threadIdx.x;
	for (int i = 0; i < kScanPer; i++, k += kScanT)
		if (k < n)
			a[k] += o;
}

// ---- device temporaries and the copy to the host -----------------------------
// The arrays of a build are carved from a few large blocks of a memory pool of
// the library's own, which keeps its memory between builds (a remesh every
// few steps would otherwise map fresh memory for each of some 200 arrays).
// The results reach the host through one pinned staging buffer, also kept
// between builds: a level's arrays are copied into it asynchronously, then
// into the host mesh's own arrays.

constexpr size_t kArenaChunk = (size_t)64 << 20;

struct Shared {
	std::mutex mu;
	cudaMemPool_t pool[64] = {};
	void *stage = nullptr;
	size_t stage_bytes = 0;
};

Shared &shared()
{
	static Shared s;
	return s;
}

cudaError_t mesh_pool(cudaMemPool_t *out)
{
	int dev = 0;
	CUDA_TRY(cudaGetDevice(&dev));
	if (dev < 0 || dev >= 64)
		return cudaErrorInvalidDevice;
	Shared &S = shared();
	std::lock_guard<std::mutex> lk(S.mu);
	if (S.pool[dev] == nullptr) {
		cudaMemPoolProps props;
		memset(&props, 0, sizeof props);
		props.allocType = cudaMemAllocationTypePinned;
		props.location.type = cudaMemLocationTypeDevice;
		props.location.id = dev;
		cudaMemPool_t p;
		CUDA_TRY(cudaMemPoolCreate(&p, &props));
		unsigned long long keep = ~0ULL;
		CUDA_TRY(cudaMemPoolSetAttribute(p, cudaMemPoolAttrReleaseThreshold, &keep));
		S.pool[dev] = p;
	}
	*out = S.pool[dev];
	return cudaSuccess;
}

struct Pool {
	cudaStream_t st;
	cudaMemPool_t mp = nullptr;
	std::vector<void *> blocks;
	char *cur = nullptr;
	size_t left = 0;
	cudaError_t err = cudaSuccess;
	explicit Pool(cudaStream_t s) : st(s) { err = mesh_pool(&mp); }
	template <class T> T *get(long n)
	{
		const size_t bytes = ((size_t)(n + 1) * sizeof(T) + 255) & ~(size_t)255;
		if (err != cudaSuccess)
			return nullptr;
		if (bytes > left) {
			const size_t sz = bytes > kArenaChunk ? bytes : kArenaChunk;
			void *q = nullptr;
			err = cudaMallocFromPoolAsync(&q, sz, mp, st);
			if (err != cudaSuccess)
				return nullptr;
			blocks.push_back(q);
			cur = (char *)q;
			left = sz;
		}
		T *r = (T *)cur;
		cur += bytes;
		left -= bytes;
		return r;
	}
	~Pool()
	{
		for (void *q : blocks)
			cudaFreeAsync(q, st);
	}
};

// device -> host copies of one level, through the staging buffer
struct Fetch {
	struct Item {
		void **dst;
		const void *src;
		size_t bytes, elem;
	};
	std::vector<Item> items;
	template <class T> void add(T **dst, const T *src, long n)
	{
		items.push_back(Item{(void **)dst, src, (size_t)(n > 0 ? n : 0) * sizeof(T), sizeof(T)});
	}
	cudaError_t run(cudaStream_t st)
	{
		size_t total = 0;
		for (const Item &it : items)
			total += (it.bytes + 255) & ~(size_t)255;
		Shared &S = shared();
		std::lock_guard<std::mutex> lk(S.mu);
		if (S.stage_bytes < total) {
			if (S.stage != nullptr)
				cudaFreeHost(S.stage);
			S.stage = nullptr;
			S.stage_bytes = 0;
			size_t want = total + total / 4;
			CUDA_TRY(cudaMallocHost(&S.stage, want));
			S.stage_bytes = want;
		}
		char *p = (char *)S.stage;
		for (const Item &it : items) {
			if (it.bytes > 0)
				CUDA_TRY(cudaMemcpyAsync(p, it.src, it.bytes, cudaMemcpyDeviceToHost, st));
			p += (it.bytes + 255) & ~(size_t)255;
		}
		CUDA_TRY(cudaStreamSynchronize(st));
		p = (char *)S.stage;
		for (const Item &it : items) {
			// calloc'ed n+1 entries, as the host builder allocates
			void *h = calloc(it.bytes / it.elem + 1, it.elem);
			if (h == nullptr)
				return cudaErrorMemoryAllocation;
			memcpy(h, p, it.bytes);
			*it.dst = h;
			p += (it.bytes + 255) & ~(size_t)255;
		}
		return cudaSuccess;
	}
};

#define CK(x)                                   \
	do {                                        \
		const cudaError_t e_ = (x);             \
		if (e_ != cudaSuccess)                  \
			return e_;                          \
	} while (0)
#define GET(ptr, T, n)                          \
	T *ptr = pool.get<T>(n);                    \
	if (ptr == nullptr)                         \
		return pool.err

cudaError_t scan(int *a, long n, Pool &pool)
{
	const long nt = (n + kScanTile - 1) / kScanTile;
	if (nt <= 1) {
		k_scan_tile<<<1, kScanT, 0, pool.st>>>(a, n, nullptr);
		return cudaGetLastError();
	}
	GET(ts, int, nt);
	k_scan_tile<<<(unsigned)nt, kScanT, 0, pool.st>>>(a, n, ts);
	CK(cudaGetLastError());
	CK(scan(ts, nt, pool));
	k_scan_add<<<(unsigned)nt, kScanT, 0, pool.st>>>(a, n, ts);
	return cudaGetLastError();
}

// a[n] of an array whose first n entries were just scanned (a[n] held 0)
cudaError_t total_of(const int *a, long n, cudaStream_t st, int *out)
{
	CK(cudaMemcpyAsync(out, a + n, sizeof(int), cudaMemcpyDeviceToHost, st));
	return cudaStreamSynchronize(st);
}

// ---- leaf levels and the MG projection (Tree.c:340-389) ---------------------

// level of each leaf from the gap to the next start code (the last leaf: to
// the end of the domain); bad[0] counts gaps that are not a power of 4 the
// code is aligned to
__global__ void k_leaf_levels(const int *leaves, int n, int max_nel, int *Mc, int *bad)
{
	GRID_STRIDE(e, n) {
		const int code = leaves[e], next = e + 1 < n ? leaves[e + 1] : max_nel, gap = next - code;
		const bool pow4 = gap > 0 && (gap & (gap - 1)) == 0 && (__ffs(gap) - 1) % 2 == 0;
		if (!pow4 || (code & (gap - 1)) != 0)
			atomicAdd(bad, 1);
		Mc[e] = pack_mcode(code, d_log4i(max_nel / gap));
	}
}

// Tree.c:361-389 walks the finer level keeping an element of a coarser level
// and merging the 4 children of a parent at level `lev`; the children of a
// merged parent are consecutive, the first one starts at the parent's code
__global__ void k_proj_keep(const int *U, int n, int lev, int fl, int *keep)
{
	const int span = 1 << (2 * (fl - lev + 1));
	GRID_STRIDE(e, n) {
		const int level = U[e] & ((1 << MCLG_LEVEL_BITS) - 1), loc = U[e] >> MCLG_LEVEL_BITS;
		keep[e] = (level < lev || (loc & (span - 1)) == 0) ? 1 : 0;
	}
}

__global__ void k_proj_write(const int *U, int n, int lev, const int *pos, int *D)
{
	GRID_STRIDE(e, n) {
		if (pos[e + 1] > pos[e]) {
			const int level = U[e] & ((1 << MCLG_LEVEL_BITS) - 1), loc = U[e] >> MCLG_LEVEL_BITS;
			D[pos[e]] = pack_mcode(loc, level < lev ? level : level - 1);
		}
	}
}

// ---- one level ---------------------------------------------------------------

struct BcCodes {
	char top_T, bot_T, lef_T, rig_T;
	double top_Tv, bot_Tv, lef_Tv, rig_Tv;
	char top_v[2], bot_v[2], lef_v[2], rig_v[2];
	double top_vv[2], bot_vv[2], lef_vv[2], rig_vv[2];
};

struct LevelDims {
	int ne, fl, lev, gnox, gnoz;
	double dxf, dzf;        // spacing of the finest level
	double dx[MCLG_MAX_LEVEL], dz[MCLG_MAX_LEVEL];
};

// ien (Construct_ien_id_lm.c:3-41) and the used node ids
__global__ void k_ien(const int *Mc, LevelDims P, int *ien, int *elev, int *mark)
{
	GRID_STRIDE(e, P.ne) {
		const int level = Mc[e] & ((1 << MCLG_LEVEL_BITS) - 1), loc = Mc[e] >> MCLG_LEVEL_BITS;
		int x, z;
		d_demorton(loc, x, z);
		const int node = z + x * P.gnoz, step = 1 << (P.fl - level);
		const int c[4] = {node, node + step, node + step + step * P.gnoz, node + step * P.gnoz};
		elev[e] = level;
		for (int a = 0; a < 4; a++) {
			ien[(long)a * P.ne + e] = c[a];
			mark[c[a]] = 1;
		}
	}
}

// the sorted node list (Construct_ien_id_lm.c:43-66) and the id -> index table
__global__ void k_node_list(const int *pos, long ng, int *node, int *lut)
{
	GRID_STRIDE(g, ng) {
		const bool used = pos[g + 1] > pos[g];
		if (used)
			node[pos[g]] = (int)g;
		lut[g] = used ? pos[g] : -1;
	}
}

__global__ void k_ienl(const int *ien, long n, const int *lut, int *ienl)
{
	GRID_STRIDE(k, n)
		ienl[k] = lut[ien[k]];
}

// coordinates (Mesh.c:430-452), BC codes (Boundary_condition.c:10-110) and the
// flags the equation numbers count (Construct_ien_id_lm.c:79-144)
__global__ void k_node_attr(const int *node, int nn, LevelDims P, BcCodes B, double *X, char *T_bc, double *T_bc_val,
                            char *v_bc, double *v_bc_val, int *vflag, int *hflag)
{
	const int gnoz = P.gnoz, gnox = P.gnox;
	GRID_STRIDE(A, nn) {
		const int n = node[A], ix = n / gnoz, iz = n - ix * gnoz;
		X[A] = __dmul_rn((double)ix, P.dxf);
		X[nn + A] = __dmul_rn((double)iz, P.dzf);
		char tb = 'N';
		double tv = 0.0;
		if ((n + 1) % gnoz == 0) {
			tb = B.top_T;
			tv = B.top_Tv;
		} else if (n % gnoz == 0) {
			tb = B.bot_T;
			tv = B.bot_Tv;
		} else if (n < gnoz) {
			tb = B.lef_T;
			tv = B.lef_Tv;
		} else if (n > (gnox - 1) * gnoz - 1) {
			tb = B.rig_T;
			tv = B.rig_Tv;
		}
		T_bc[A] = tb;
		T_bc_val[A] = tv;
		hflag[A] = tb != 'T';
		for (int d = 0; d < 2; d++) {
			char bc = 'N';
			double bv = 0.0;
			if ((n + 1) % gnoz == 0) {
				bc = B.top_v[d];
				bv = B.top_vv[d];
			} else if (n % gnoz == 0) {
				bc = B.bot_v[d];
				bv = B.bot_vv[d];
			}
			if (n < gnoz) {
				if (bc != 'V')
					bc = B.lef_v[d];
				bv = B.lef_vv[d];
			} else if (n > (gnox - 1) * gnoz - 1) {
				if (bc != 'V')
					bc = B.rig_v[d];
				bv = B.rig_vv[d];
			}
			v_bc[(long)d * nn + A] = bc;
			v_bc_val[(long)d * nn + A] = bv;
			vflag[2L * A + d] = bc != 'V';
		}
	}
}

__global__ void k_ids(const int *vpos, const int *hpos, int nn, int *id, int *heat_id)
{
	GRID_STRIDE(A, nn) {
		for (int d = 0; d < 2; d++) {
			const long k = 2L * A + d;
			id[(long)d * nn + A] = vpos[k + 1] > vpos[k] ? vpos[k] : -1;
		}
		heat_id[A] = hpos[A + 1] > hpos[A] ? hpos[A] : -1;
	}
}

// element geometry (Shape_function.c:123-167, Construct_ien_id_lm.c:198-218)
__global__ void k_geom(const int *ienl, const int *elev, const double *X, int nn, LevelDims P, double *dx_dxi,
                       double *dz_deta, double *jacobi, double *area)
{
	GRID_STRIDE(e, P.ne) {
		const int n0 = ienl[e], n2 = ienl[2L * P.ne + e], l = elev[e];
		const double hx = __dmul_rn(0.5, P.dx[l]), hz = __dmul_rn(0.5, P.dz[l]);
		dx_dxi[e] = hx;
		dz_deta[e] = hz;
		jacobi[e] = __dsub_rn(__dmul_rn(hx, hz), __dmul_rn(0.0, 0.0));
		area[e] = __dmul_rn(__dsub_rn(X[n2], X[n0]), __dsub_rn(X[nn + n2], X[nn + n0]));
	}
}

// node -> elements (Construct_ien_id_lm.c:220-244): gathered in any order, then
// each node's (at most 4) entries sorted by element
__global__ void k_p2n_gather(const int *ienl, int ne, int nn, int *cnt, int *tel, int *ta, int *over)
{
	GRID_STRIDE(k, 4L * ne) {
		const int a = (int)(k / ne), e = (int)(k - (long)a * ne), i = ienl[k];
		const int s = atomicAdd(&cnt[i], 1);
		if (s < 4) {
			tel[(long)s * nn + i] = e;
			ta[(long)s * nn + i] = a;
		} else {
			atomicMax(over, i + 1);
		}
	}
}

__global__ void k_p2n_sort(const int *cnt, const int *tel, const int *ta, int nn, int *p2n_el, int *p2n_a)
{
	GRID_STRIDE(A, nn) {
		const int n = cnt[A] < 4 ? cnt[A] : 4;
		int el[4], ac[4];
		for (int s = 0; s < n; s++) {
			el[s] = tel[(long)s * nn + A];
			ac[s] = ta[(long)s * nn + A];
		}
		for (int s = 1; s < n; s++)
			for (int k = s; k > 0 && el[k - 1] > el[k]; k--) {
				const int te = el[k], tc = ac[k];
				el[k] = el[k - 1];
				ac[k] = ac[k - 1];
				el[k - 1] = te;
				ac[k - 1] = tc;
			}
		for (int s = 0; s < 4; s++) {
			p2n_el[(long)s * nn + A] = s < n ? el[s] : -1;
			p2n_a[(long)s * nn + A] = s < n ? ac[s] : 0;
		}
	}
}

// hanging nodes (Connection.c:59-276): the mid-edge node of an element coarser
// than the level, where the mesh has one; counted, scanned, then written in
// element-then-edge order
template <bool WRITE>
__global__ void k_hang(const int *ien, const int *elev, LevelDims P, const int *lut, int *hc, int *hn, int *h0,
                       int *h1, int *hni, int *hci0, int *hci1)
{
	GRID_STRIDE(e, P.ne) {
		int c = 0;
		long k = WRITE ? hc[e] : 0;
		if (elev[e] != P.lev) {
			for (int i = 0; i < 4; i++) {
				const int c0 = ien[(long)i * P.ne + e], c1 = ien[(long)((i + 1) % 4) * P.ne + e];
				const int mid = (c0 + c1) / 2, mi = lut[mid];
				if (mi < 0)
					continue;
				if (WRITE) {
					hn[k] = mid;
					h0[k] = c0;
					h1[k] = c1;
					hni[k] = mi;
					hci0[k] = lut[c0];
					hci1[k] = lut[c1];
					k++;
				}
				c++;
			}
		}
		if (!WRITE)
			hc[e] = c;
	}
}

__global__ void k_hang_mark(const int *hni, int nh, unsigned char *is_h)
{
	GRID_STRIDE(h, nh)
		is_h[hni[h]] = 1;
}

__global__ void k_hang_chain(const int *hci0, const int *hci1, int nh, const unsigned char *is_h, int *chained)
{
	GRID_STRIDE(h, nh)
		if (is_h[hci0[h]] || is_h[hci1[h]])
			*chained = 1;
}

// sorted distinct neighbours of each node (the corners of its elements)
__global__ void k_nb_lists(const int *p2n_cnt, const int *p2n_el, const int *ienl, int ne, int nn, int *lists,
                           int *nb_cnt, int *wmax)
{
	GRID_STRIDE(A, nn) {
		int v[16], n = 0;
		for (int s = 0; s < p2n_cnt[A] && s < 4; s++) {
			const int el = p2n_el[(long)s * nn + A];
			for (int j = 0; j < 4; j++)
				v[n++] = ienl[(long)j * ne + el];
		}
		for (int i = 1; i < n; i++) {
			const int x = v[i];
			int k = i;
			for (; k > 0 && v[k - 1] > x; k--)
				v[k] = v[k - 1];
			v[k] = x;
		}
		int m = n > 0 ? 1 : 0;
		for (int i = 1; i < n; i++)
			if (v[i] != v[m - 1])
				v[m++] = v[i];
		for (int i = 0; i < m; i++)
			lists[16L * A + i] = v[i];
		nb_cnt[A] = m;
		atomicMax(wmax, m);
	}
}

__global__ void k_nb_fill(const int *lists, const int *nb_cnt, int nn, int w, int *nb)
{
	GRID_STRIDE(k, (long)w * nn) {
		const int j = (int)(k / nn), A = (int)(k - (long)j * nn);
		nb[k] = j < nb_cnt[A] ? lists[16L * A + j] : A;
	}
}

__global__ void k_kslot(const int *ienl, int ne, int nn, const int *nb, const int *nb_cnt, unsigned char *kslot,
                        int *bad)
{
	GRID_STRIDE(e, ne) {
		for (int a = 0; a < 4; a++) {
			const int An = ienl[(long)a * ne + e];
			for (int b = 0; b < 4; b++) {
				const int Bn = ienl[(long)b * ne + e];
				int slot = -1;
				for (int j = 0; j < nb_cnt[An]; j++)
					if (nb[(long)j * nn + An] == Bn) {
						slot = j;
						break;
					}
				if (slot < 0) {
					*bad = 1;
					slot = 0;
				}
				kslot[(long)(a * 4 + b) * ne + e] = (unsigned char)slot;
			}
		}
	}
}

// fine cell -> covering element: the last leaf whose start code is at most the
// cell's Morton code (the leaves tile the domain)
__global__ void k_cell_elem(const int *Mc, int ne, int gnoz, int *cell_elem)
{
	const int ncz = gnoz - 1;
	GRID_STRIDE(k, (long)ncz * ncz) {
		const int ix = (int)(k / ncz), iz = (int)(k - (long)ix * ncz), m = d_morton(ix, iz);
		int lo = 0, hi = ne - 1;
		while (lo < hi) {
			const int mid = (lo + hi + 1) >> 1;
			if ((Mc[mid] >> MCLG_LEVEL_BITS) <= m)
				lo = mid;
			else
				hi = mid - 1;
		}
		cell_elem[k] = lo;
	}
}

// ---- host side ---------------------------------------------------------------

struct Fail {
	int rc;
	char msg[256];
};

cudaError_t build_level(mclg_mesh *m, const mclg_config *c, int lev, const int *dMc, int ne, Pool &pool, Fail &f)
{
	cudaStream_t st = pool.st;
	mclg_level *L = &m->lev[lev];
	const int fl = m->max_level - 1, gnox = m->gnox, gnoz = m->gnoz;
	const long ng = (long)gnox * gnoz;
	LevelDims P;
	P.ne = ne;
	P.fl = fl;
	P.lev = lev;
	P.gnox = gnox;
	P.gnoz = gnoz;
	P.dxf = m->dx[fl];
	P.dzf = m->dz[fl];
	for (int l = 0; l < MCLG_MAX_LEVEL; l++) {
		P.dx[l] = m->dx[l];
		P.dz[l] = m->dz[l];
	}
	L->nel = ne;
	// ien and the node list
	GET(ien, int, 4L * ne);
	GET(elev, int, ne);
	GET(pos, int, ng + 1);
	GET(lut, int, ng);
	CK(cudaMemsetAsync(pos, 0, (size_t)(ng + 1) * sizeof(int), st));
	k_ien<<<grid_for(ne), kT, 0, st>>>(dMc, P, ien, elev, pos);
	CK(cudaGetLastError());
	CK(scan(pos, ng + 1, pool));
	int nn = 0;
	CK(total_of(pos, ng, st, &nn));
	L->nno = nn;
	GET(node, int, nn);
	k_node_list<<<grid_for(ng), kT, 0, st>>>(pos, ng, node, lut);
	GET(ienl, int, 4L * ne);
	k_ienl<<<grid_for(4L * ne), kT, 0, st>>>(ien, 4L * ne, lut, ienl);
	CK(cudaGetLastError());
	// coordinates, BC codes, equation numbers
	BcCodes B;
	B.top_T = c->top_T_bc; B.bot_T = c->bot_T_bc; B.lef_T = c->lef_T_bc; B.rig_T = c->rig_T_bc;
	B.top_Tv = c->top_T_bc_val; B.bot_Tv = c->bot_T_bc_val; B.lef_Tv = c->lef_T_bc_val; B.rig_Tv = c->rig_T_bc_val;
	for (int d = 0; d < 2; d++) {
		B.top_v[d] = c->top_v_bc[d]; B.bot_v[d] = c->bot_v_bc[d];
		B.lef_v[d] = c->lef_v_bc[d]; B.rig_v[d] = c->rig_v_bc[d];
		B.top_vv[d] = c->top_v_bc_val[d]; B.bot_vv[d] = c->bot_v_bc_val[d];
		B.lef_vv[d] = c->lef_v_bc_val[d]; B.rig_vv[d] = c->rig_v_bc_val[d];
	}
	GET(X, double, 2L * nn);
	GET(T_bc, char, nn);
	GET(T_bc_val, double, nn);
	GET(v_bc, char, 2L * nn);
	GET(v_bc_val, double, 2L * nn);
	GET(vflag, int, 2L * nn + 1);
	GET(hflag, int, (long)nn + 1);
	CK(cudaMemsetAsync(vflag + 2L * nn, 0, sizeof(int), st));
	CK(cudaMemsetAsync(hflag + nn, 0, sizeof(int), st));
	k_node_attr<<<grid_for(nn), kT, 0, st>>>(node, nn, P, B, X, T_bc, T_bc_val, v_bc, v_bc_val, vflag, hflag);
	CK(cudaGetLastError());
	CK(scan(vflag, 2L * nn + 1, pool));
	CK(scan(hflag, (long)nn + 1, pool));
	GET(id, int, 2L * nn);
	GET(heat_id, int, nn);
	k_ids<<<grid_for(nn), kT, 0, st>>>(vflag, hflag, nn, id, heat_id);
	CK(cudaGetLastError());
	CK(total_of(vflag, 2L * nn, st, &L->neq));
	CK(total_of(hflag, nn, st, &L->heat_neq));
	// geometry
	GET(dx_dxi, double, ne);
	GET(dz_deta, double, ne);
	GET(jacobi, double, ne);
	GET(area, double, ne);
	k_geom<<<grid_for(ne), kT, 0, st>>>(ienl, elev, X, nn, P, dx_dxi, dz_deta, jacobi, area);
	CK(cudaGetLastError());
	// node -> elements
	GET(p2n_cnt, int, nn);
	GET(tel, int, 4L * nn);
	GET(ta, int, 4L * nn);
	GET(p2n_el, int, 4L * nn);
	GET(p2n_a, int, 4L * nn);
	GET(flags, int, 4);   // [0] node touching > 4 elements (+1), [1] chained, [2] width, [3] bad slot
	CK(cudaMemsetAsync(p2n_cnt, 0, (size_t)nn * sizeof(int), st));
	CK(cudaMemsetAsync(flags, 0, 4 * sizeof(int), st));
	k_p2n_gather<<<grid_for(4L * ne), kT, 0, st>>>(ienl, ne, nn, p2n_cnt, tel, ta, flags);
	k_p2n_sort<<<grid_for(nn), kT, 0, st>>>(p2n_cnt, tel, ta, nn, p2n_el, p2n_a);
	CK(cudaGetLastError());
	// hanging nodes
	GET(hc, int, (long)ne + 1);
	CK(cudaMemsetAsync(hc + ne, 0, sizeof(int), st));
	k_hang<false><<<grid_for(ne), kT, 0, st>>>(ien, elev, P, lut, hc, nullptr, nullptr, nullptr, nullptr, nullptr,
	                                           nullptr);
	CK(cudaGetLastError());
	CK(scan(hc, (long)ne + 1, pool));
	int nh = 0;
	CK(total_of(hc, ne, st, &nh));
	L->nh = nh;
	GET(hn, int, nh);
	GET(h0, int, nh);
	GET(h1, int, nh);
	GET(hni, int, nh);
	GET(hci0, int, nh);
	GET(hci1, int, nh);
	GET(is_h, unsigned char, nn);
	CK(cudaMemsetAsync(is_h, 0, (size_t)nn + 1, st));
	k_hang<true><<<grid_for(ne), kT, 0, st>>>(ien, elev, P, lut, hc, hn, h0, h1, hni, hci0, hci1);
	if (nh > 0) {
		k_hang_mark<<<grid_for(nh), kT, 0, st>>>(hni, nh, is_h);
		k_hang_chain<<<grid_for(nh), kT, 0, st>>>(hci0, hci1, nh, is_h, flags + 1);
	}
	CK(cudaGetLastError());
	// neighbour lists and the element slot map
	GET(lists, int, 16L * nn);
	GET(nb_cnt, int, nn);
	k_nb_lists<<<grid_for(nn), kT, 0, st>>>(p2n_cnt, p2n_el, ienl, ne, nn, lists, nb_cnt, flags + 2);
	CK(cudaGetLastError());
	int hf[4];
	CK(cudaMemcpyAsync(hf, flags, sizeof hf, cudaMemcpyDeviceToHost, st));
	CK(cudaStreamSynchronize(st));
	if (hf[0] != 0) {
		int gid = -1;
		CK(cudaMemcpy(&gid, node + (hf[0] - 1), sizeof(int), cudaMemcpyDeviceToHost));
		f.rc = MCLG_BAD_INPUT;
		snprintf(f.msg, sizeof f.msg, "node %d touches more than 4 elements", gid);
		return cudaSuccess;
	}
	const int w = hf[2];
	if (w > MCLG_NB_MAX) {
		f.rc = MCLG_BAD_INPUT;
		snprintf(f.msg, sizeof f.msg, "a node has %d neighbours (max %d)", w, MCLG_NB_MAX);
		return cudaSuccess;
	}
	L->hang_chained = hf[1];
	L->nbw = w;
	int *hflags_dst = nullptr;
	GET(nb, int, (long)w * nn);
	GET(kslot, unsigned char, 16L * ne);
	k_nb_fill<<<grid_for((long)w * nn), kT, 0, st>>>(lists, nb_cnt, nn, w, nb);
	k_kslot<<<grid_for(ne), kT, 0, st>>>(ienl, ne, nn, nb, nb_cnt, kslot, flags + 3);
	CK(cudaGetLastError());
	int *cell = nullptr;
	if (lev == fl) {
		cell = pool.get<int>((long)(gnox - 1) * (gnoz - 1));
		if (cell == nullptr)
			return pool.err;
		k_cell_elem<<<grid_for((long)(gnox - 1) * (gnoz - 1)), kT, 0, st>>>(dMc, ne, gnoz, cell);
		CK(cudaGetLastError());
	}
	// into host arrays (calloc'ed n+1 like the host builder's)
	Fetch F;
	F.add(&L->Mcode, dMc, ne);
	F.add(&L->ien, ien, 4L * ne);
	F.add(&L->elev, elev, ne);
	F.add(&L->node, node, nn);
	if (ng <= kLutMax) {
		L->lut_n = ng;
		F.add(&L->node_lut, lut, ng);
	}
	F.add(&L->ienl, ienl, 4L * ne);
	F.add(&L->X, X, 2L * nn);
	F.add(&L->T_bc, T_bc, nn);
	F.add(&L->T_bc_val, T_bc_val, nn);
	F.add(&L->v_bc, v_bc, 2L * nn);
	F.add(&L->v_bc_val, v_bc_val, 2L * nn);
	F.add(&L->id, id, 2L * nn);
	F.add(&L->heat_id, heat_id, nn);
	F.add(&L->dx_dxi, dx_dxi, ne);
	F.add(&L->dz_deta, dz_deta, ne);
	F.add(&L->jacobi, jacobi, ne);
	F.add(&L->area, area, ne);
	F.add(&L->p2n_cnt, p2n_cnt, nn);
	F.add(&L->p2n_el, p2n_el, 4L * nn);
	F.add(&L->p2n_a, p2n_a, 4L * nn);
	F.add(&L->hang_node, hn, nh);
	F.add(&L->hang_c0, h0, nh);
	F.add(&L->hang_c1, h1, nh);
	F.add(&L->hang_ni, hni, nh);
	F.add(&L->hang_ci0, hci0, nh);
	F.add(&L->hang_ci1, hci1, nh);
	F.add(&L->nb, nb, (long)w * nn);
	F.add(&L->nb_cnt, nb_cnt, nn);
	F.add(&L->kslot, kslot, 16L * ne);
	if (cell != nullptr)
		F.add(&L->cell_elem, cell, (long)(gnox - 1) * (gnoz - 1));
	F.add(&hflags_dst, flags, 4);
	CK(F.run(st));
	if (hflags_dst[3] != 0) {
		f.rc = MCLG_BAD_INPUT;
		snprintf(f.msg, sizeof f.msg, "internal: neighbour slot not found");
	}
	free(hflags_dst);
	return cudaSuccess;
}

cudaError_t build_all(mclg_mesh *m, const mclg_config *c, const int *leaves, long n, Pool &pool, Fail &f)
{
	cudaStream_t st = pool.st;
	const int fl = m->max_level - 1;
	GET(dleaves, int, n);
	GET(bad, int, 1);
	CK(cudaMemcpyAsync(dleaves, leaves, (size_t)n * sizeof(int), cudaMemcpyHostToDevice, st));
	CK(cudaMemsetAsync(bad, 0, sizeof(int), st));
	std::vector<const int *> Mc(MCLG_MAX_LEVEL, nullptr);
	std::vector<int> nel(MCLG_MAX_LEVEL, 0);
	GET(fine, int, n);
	k_leaf_levels<<<grid_for(n), kT, 0, st>>>(dleaves, (int)n, m->max_nel[fl], fine, bad);
	CK(cudaGetLastError());
	int hb = 0;
	CK(cudaMemcpyAsync(&hb, bad, sizeof(int), cudaMemcpyDeviceToHost, st));
	CK(cudaStreamSynchronize(st));
	if (hb != 0) {
		f.rc = MCLG_BAD_INPUT;
		snprintf(f.msg, sizeof f.msg, "%d leaves are not quadtree cells (gap to the next code)", hb);
		return cudaSuccess;
	}
	Mc[fl] = fine;
	nel[fl] = (int)n;
	// project_Mcode (Tree.c:361-389) down to the lowest MG level
	for (int lev = fl; lev > m->min_level; lev--) {
		const int nu = nel[lev];
		GET(keep, int, (long)nu + 1);
		CK(cudaMemsetAsync(keep + nu, 0, sizeof(int), st));
		k_proj_keep<<<grid_for(nu), kT, 0, st>>>(Mc[lev], nu, lev, fl, keep);
		CK(cudaGetLastError());
		CK(scan(keep, (long)nu + 1, pool));
		int nd = 0;
		CK(total_of(keep, nu, st, &nd));
		GET(D, int, nd);
		k_proj_write<<<grid_for(nu), kT, 0, st>>>(Mc[lev], nu, lev, keep, D);
		CK(cudaGetLastError());
		Mc[lev - 1] = D;
		nel[lev - 1] = nd;
	}
	for (int lev = m->min_level; lev <= fl && f.rc == MCLG_OK; lev++)
		CK(build_level(m, c, lev, Mc[lev], nel[lev], pool, f));
	return cudaSuccess;
}

}  // namespace

extern "C" int mclg_mesh_build_leaves_device(mclg_mesh *m, const mclg_config *c, const int *leaves, long n, void *stream)
{
	if (m == NULL || c == NULL || leaves == NULL) {
		if (m != NULL)
			memset(m, 0, sizeof *m);
		mclg_set_error("mclg_mesh_build_leaves_device: null argument");
		return MCLG_BAD_INPUT;
	}
	int rc = mclg_mesh_frame(m, c);
	if (rc == MCLG_OK)
		rc = mclg_mesh_check_leaves(m, leaves, n);
	if (rc != MCLG_OK) {
		memset(m, 0, sizeof *m);
		return rc;
	}
	cudaStream_t st = (cudaStream_t)stream, own = nullptr;
	if (st == nullptr) {
		if (cudaStreamCreateWithFlags(&own, cudaStreamNonBlocking) != cudaSuccess) {
			cudaGetLastError();
			mclg_set_error("mclg_mesh_build_leaves_device: no stream");
			memset(m, 0, sizeof *m);
			return MCLG_CUDA_ERROR;
		}
		st = own;
	}
	Fail f;
	f.rc = MCLG_OK;
	f.msg[0] = 0;
	cudaError_t e;
	{
		Pool pool(st);
		e = build_all(m, c, leaves, n, pool, f);
		if (e == cudaSuccess)
			e = pool.err;
	}
	const cudaError_t e2 = cudaStreamSynchronize(st);
	if (e == cudaSuccess)
		e = e2;
	if (own != nullptr)
		cudaStreamDestroy(own);
	if (e != cudaSuccess) {
		cudaGetLastError();
		mclg_set_error("mesh numbering on the device: %s", cudaGetErrorString(e));
		rc = MCLG_CUDA_ERROR;
	} else if (f.rc != MCLG_OK) {
		mclg_set_error("%s", f.msg);
		rc = f.rc;
	}
	if (rc != MCLG_OK) {
		mclg_mesh_free(m);
		return rc;
	}
	const mclg_level *L = &m->lev[m->max_level - 1];
	m->uniform = (L->nel == m->max_nel[m->max_level - 1] && L->nh == 0);
	return MCLG_OK;
}
