/*
 * Quadtree mesh, numbering, boundary codes and hanging-node constraints for
 * one rank, built on the host once per mesh.
 *
 * The results are bit-identical to the reference's single-rank arrays:
 *   leaf Morton codes  Tree.c:67-93 (build_quad_tree), 101-298 (initial_refine),
 *                      302-338 (split_mul_lev/split_Mcode), 340-389 (levels, MG projection)
 *   ien / node list    Construct_ien_id_lm.c:3-66
 *   id / heat.id / lm  Construct_ien_id_lm.c:79-196
 *   boundary codes     Boundary_condition.c:10-110
 *   geometry           Mesh.c:396-452, Shape_function.c:123-167, Construct_ien_id_lm.c:198-244
 *   hanging nodes      Connection.c:59-276 (the single-rank part)
 * The reference builds its leaf list with an O(n) linked-list append and an
 * O(n^2) quicksort on almost-sorted input (Tree.c:43-64, Array_work.c:48-73);
 * here the same set of codes is collected in a growable array and sorted with
 * qsort, which yields the same sorted, de-duplicated list.
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <stdarg.h>
#include <math.h>
#include <pthread.h>
#include "mclg_host.h"
#include "mclg_ic.h"

static _Thread_local char g_err[512];

void mclg_set_error(const char *fmt, ...)
{
	va_list ap;
	va_start(ap, fmt);
	vsnprintf(g_err, sizeof g_err, fmt, ap);
	va_end(ap);
}

const char *mclg_last_error(void)
{
	return g_err;
}

typedef struct ivec {
	int *a;
	long n, cap;
} ivec;

static int ivec_push(ivec *v, int x)
{
	if (v->n == v->cap) {
		long cap = v->cap ? 2 * v->cap : 1024;
		int *a = (int *)realloc(v->a, (size_t)cap * sizeof(int));
		if (a == NULL)
			return -1;
		v->a = a;
		v->cap = cap;
	}
	v->a[v->n++] = x;
	return 0;
}

static int cmp_int(const void *x, const void *y)
{
	int a = *(const int *)x, b = *(const int *)y;
	return (a > b) - (a < b);
}

static long sort_unique(int *a, long n)
{
	long i, j = 0;
	if (n <= 1)
		return n;
	for (i = 1; i < n && a[i - 1] < a[i]; i++)
		;
	if (i == n)   /* already strictly increasing (a leaf list) */
		return n;
	if (n <= 32) {   /* a node's neighbours: insertion sort */
		for (i = 1; i < n; i++) {
			const int v = a[i];
			long k = i;
			for (; k > 0 && a[k - 1] > v; k--)
				a[k] = a[k - 1];
			a[k] = v;
		}
	} else {
		qsort(a, (size_t)n, sizeof(int), cmp_int);
	}
	for (i = 1; i < n; i++)
		if (a[i] != a[j])
			a[++j] = a[i];
	return j + 1;
}

static int log4i(int a)
{
	int b = 0;
	while (a >>= 2)
		b++;
	return b;
}

/* Bit de-interleave of a Morton code: x from the odd bits, z from the even
 * bits (demorton_no_lev, Tree.c:433-444). */
static void demorton(int code, int *x, int *z)
{
	int i;
	unsigned int c = (unsigned int)code;
	*x = *z = 0;
	for (i = 0; i < 16; i++) {
		*x |= (int)(((c >> (2 * i + 1)) & 1u) << i);
		*z |= (int)(((c >> (2 * i)) & 1u) << i);
	}
}

typedef struct tree_ctx {
	ivec *out;
	int fine_nel;   /* max_nel of the finest level */
} tree_ctx;

/* Append the 4 children of `code` at depth level+1 and recurse num-1 more
 * times (split_mul_lev + split_Mcode, Tree.c:302-338). */
static int split_mul(tree_ctx *t, ivec *out, int code, int num, int level)
{
	int i, child[4];
	if (num == 0)
		return 0;
	for (i = 0; i < 4; i++)
		child[i] = code + i * (t->fine_nel >> (2 * (level + 1)));
	for (i = 0; i < 4; i++)
		if (ivec_push(out, child[i]) != 0)
			return -1;
	for (i = 0; i < 4; i++)
		if (split_mul(t, out, child[i], num - 1, level + 1) != 0)
			return -1;
	return 0;
}

/* refine_bottom (Tree.c:459-529) for one rank (rank 0, start code 0): every
 * code of the current list is split again according to its z band, and the
 * new list replaces the old one. */
static int refine_bottom(tree_ctx *t, ivec *head, int dev_mode)
{
	ivec add = {0};
	long k;
	for (k = 0; k < head->n; k++) {
		int a, b, c = head->a[k], rc = 0;
		demorton(c, &a, &b);
		if (dev_mode == 2) {
			if (b <= 112) rc = split_mul(t, &add, c, 4, 5);
			else if (b <= 240) rc = split_mul(t, &add, c, 3, 5);
			else if (b <= 368) rc = split_mul(t, &add, c, 2, 5);
			else rc = split_mul(t, &add, c, 1, 5);
		} else if (dev_mode == 3 || dev_mode == 10) {
			if (b <= 48) rc = split_mul(t, &add, c, 4, 4);
			else if (b <= 112) rc = split_mul(t, &add, c, 3, 4);
			else if (b <= 240) rc = split_mul(t, &add, c, 2, 4);
			else rc = split_mul(t, &add, c, 1, 4);
		} else if (dev_mode == 9) {
			if (b <= 48) rc = split_mul(t, &add, c, 4, 5);
			else if (b <= 240) rc = split_mul(t, &add, c, 3, 5);
			else if (b <= 368) rc = split_mul(t, &add, c, 2, 5);
			else rc = split_mul(t, &add, c, 1, 5);
		}
		if (rc != 0) {
			free(add.a);
			return -1;
		}
	}
	free(head->a);
	*head = add;
	return 0;
}

/* initial_refine (Tree.c:101-298) on rank 0 of a 1x1 rank grid. */
static int initial_refine(tree_ctx *t, ivec *head, int dev_mode, int max_level)
{
	int rc = 0, i, a, b, mul, width;
	switch (dev_mode) {
	case 0:
	case 7:
		rc = split_mul(t, head, 0, max_level - 1, 0);
		break;
	case 1:
		rc = split_mul(t, head, 0, 1, 0);
		break;
	case 2:
	case 9:
		rc = split_mul(t, head, 0, 5, 0);
		if (rc == 0)
			rc = refine_bottom(t, head, dev_mode);
		break;
	case 3:
	case 10:
		rc = split_mul(t, head, 0, 4, 0);
		if (rc == 0)
			rc = refine_bottom(t, head, dev_mode);
		break;
	case 4:
		rc = split_mul(t, head, 0, 2, 0);
		break;
	case 5:
		rc = split_mul(t, head, 0, 6, 0);
		break;
	case 6:
		i = max_level - 1;
		rc = split_mul(t, head, 0, i > 4 ? i : 4, 0);
		break;
	case 8: {
		static const int c1[8] = {64, 80, 96, 112, 192, 208, 224, 240};
		static const int c2[4] = {212, 220, 244, 252};
		rc = split_mul(t, head, 0, 2, 0);
		for (i = 0; i < 8 && rc == 0; i++)
			rc = split_mul(t, head, c1[i], 1, 2);
		for (i = 0; i < 4 && rc == 0; i++)
			rc = split_mul(t, head, c2[i], 1, 3);
		break;
	}
	case 11:
	case 12:
	case 14:
		rc = split_mul(t, head, 0, max_level - 2, 0);
		mul = 1 << (max_level - 1);
		width = (dev_mode == 14) ? mul / 2 + 1 : mul / 8;
		for (i = 0; i < mul * mul && rc == 0; i += 4) {
			int hit;
			demorton(i, &a, &b);
			if (dev_mode == 11)
				hit = (b < width || b >= mul - width) || (a < width || a >= mul - width);
			else if (dev_mode == 12)
				hit = b >= mul - width;
			else
				hit = b <= width;
			if (hit)
				rc = split_mul(t, head, i, 1, max_level - 2);
		}
		break;
	case 13:
		rc = split_mul(t, head, 0, max_level - 6, 0);
		mul = 1 << (max_level - 1);
		width = mul / 64;
		for (i = 0; i < mul * mul && rc == 0; i += 1024) {
			demorton(i, &a, &b);
			if (b <= width) rc = split_mul(t, head, i, 5, max_level - 6);
			else if (b <= 4 * width) rc = split_mul(t, head, i, 4, max_level - 6);
			else if (b <= 8 * width) rc = split_mul(t, head, i, 3, max_level - 6);
			else if (b <= 12 * width) rc = split_mul(t, head, i, 2, max_level - 6);
			else rc = split_mul(t, head, i, 1, max_level - 6);
		}
		break;
	default:
		mclg_set_error("develop_mode=%d is not a refinement pattern of the reference", dev_mode);
		return MCLG_BAD_INPUT;
	}
	return rc == 0 ? MCLG_OK : MCLG_BAD_INPUT;
}

int mclg_node_index(const mclg_level *L, int gid)
{
	if (L->node_lut != NULL)
		return gid >= 0 && gid < L->lut_n ? L->node_lut[gid] : -1;
	int lo = 0, hi = L->nno - 1;
	while (lo <= hi) {
		int mid = lo + ((hi - lo) >> 1);
		if (L->node[mid] == gid)
			return mid;
		if (L->node[mid] < gid)
			lo = mid + 1;
		else
			hi = mid - 1;
	}
	return -1;
}

#define ALLOC(p, n) do { (p) = calloc((size_t)(n) + 1, sizeof(*(p))); if ((p) == NULL) goto oom; } while (0)

/* fn(ctx, i0, i1) over [0, n) in chunks of at least `grain` items, one thread
 * per chunk (at most 8); each chunk writes only its own items, so the result
 * does not depend on the split. */
typedef struct {
	void (*fn)(void *, long, long);
	void *ctx;
	long i0, i1;
} pf_job;

static void *pf_run(void *p)
{
	pf_job *j = (pf_job *)p;
	j->fn(j->ctx, j->i0, j->i1);
	return NULL;
}

void mclg_parallel_for(long n, long grain, void (*fn)(void *, long, long), void *ctx)
{
	enum { kMaxT = 8 };
	pf_job jobs[kMaxT];
	pthread_t th[kMaxT];
	int started[kMaxT], nt = (int)(n / (grain > 0 ? grain : 1)), i;
	nt = nt < 1 ? 1 : nt > kMaxT ? kMaxT : nt;
	for (i = 0; i < nt; i++) {
		jobs[i].fn = fn;
		jobs[i].ctx = ctx;
		jobs[i].i0 = n * i / nt;
		jobs[i].i1 = n * (i + 1) / nt;
		started[i] = i < nt - 1 && pthread_create(&th[i], NULL, pf_run, &jobs[i]) == 0;
		if (!started[i])
			pf_run(&jobs[i]);
	}
	for (i = 0; i < nt; i++)
		if (started[i])
			pthread_join(th[i], NULL);
}

/* a node's neighbours: the distinct nodes of the elements touching it, sorted */
typedef struct {
	const mclg_level *L;
	int *lists;   /* [16*nno] */
} nb_ctx;

static void nb_lists(void *p, long a0, long a1)
{
	nb_ctx *x = (nb_ctx *)p;
	const mclg_level *L = x->L;
	const long nn = L->nno, ne = L->nel;
	for (long A = a0; A < a1; A++) {
		int *nb = x->lists + 16 * A, cnt = 0;
		for (int s = 0; s < L->p2n_cnt[A]; s++) {
			const int el = L->p2n_el[(long)s * nn + A];
			for (int j = 0; j < 4; j++)
				nb[cnt++] = L->ienl[(long)j * ne + el];
		}
		L->nb_cnt[A] = (int)sort_unique(nb, cnt);
	}
}

typedef struct {
	const mclg_level *L;
	const int *lists;
	int w;
	int *nb;
} nb_fill_ctx;

static void nb_fill(void *p, long a0, long a1)
{
	nb_fill_ctx *x = (nb_fill_ctx *)p;
	const long nn = x->L->nno;
	for (long A = a0; A < a1; A++)
		for (int j = 0; j < x->w; j++)
			x->nb[(long)j * nn + A] = j < x->L->nb_cnt[A] ? x->lists[16 * A + j] : (int)A;
}

/* the slot of corner b in the neighbour list of corner a, per element */
typedef struct {
	mclg_level *L;
	int bad;
} kslot_ctx;

static void kslot_fill(void *p, long e0, long e1)
{
	kslot_ctx *x = (kslot_ctx *)p;
	mclg_level *L = x->L;
	const long nn = L->nno, ne = L->nel;
	for (long e = e0; e < e1; e++)
		for (int a = 0; a < 4; a++) {
			const int An = L->ienl[(long)a * ne + e];
			for (int b = 0; b < 4; b++) {
				const int Bn = L->ienl[(long)b * ne + e];
				int slot = -1;
				for (int j = 0; j < L->nb_cnt[An]; j++)
					if (L->nb[(long)j * nn + An] == Bn) {
						slot = j;
						break;
					}
				if (slot < 0) {
					x->bad = 1;
					slot = 0;
				}
				L->kslot[(long)(a * 4 + b) * ne + e] = (unsigned char)slot;
			}
		}
}

/* the per-element and per-node loops of a level that write only their own item */
typedef struct {
	const mclg_mesh *m;
	const mclg_config *c;
	mclg_level *L;
	int lev, fl, gnox, gnoz;
} lvl_ctx;

static void ien_range(void *p, long e0, long e1)   /* Construct_ien_id_lm.c:3-41 */
{
	const lvl_ctx *x = (const lvl_ctx *)p;
	mclg_level *L = x->L;
	const long ne = L->nel;
	for (long e = e0; e < e1; e++) {
		int level = L->Mcode[e] & ((1 << MCLG_LEVEL_BITS) - 1);
		int loc = L->Mcode[e] >> MCLG_LEVEL_BITS, xx, z, step, node;
		demorton(loc, &xx, &z);
		node = z + xx * x->gnoz;
		step = 1 << (x->fl - level);
		L->elev[e] = level;
		L->ien[0L * ne + e] = node;
		L->ien[1L * ne + e] = node + step;
		L->ien[2L * ne + e] = node + step + step * x->gnoz;
		L->ien[3L * ne + e] = node + step * x->gnoz;
	}
}

static void ienl_range(void *p, long k0, long k1)
{
	mclg_level *L = ((const lvl_ctx *)p)->L;
	for (long k = k0; k < k1; k++)
		L->ienl[k] = mclg_node_index(L, L->ien[k]);
}

/* coordinates (Mesh.c:430-452) and BC codes (Boundary_condition.c:10-110) */
static void node_range(void *p, long a0, long a1)
{
	const lvl_ctx *x = (const lvl_ctx *)p;
	const mclg_config *c = x->c;
	mclg_level *L = x->L;
	const long nn = L->nno;
	const int gnoz = x->gnoz, gnox = x->gnox;
	for (long A = a0; A < a1; A++) {
		const int n = L->node[A], ix = n / gnoz, iz = n - ix * gnoz;
		L->X[A] = ix * x->m->dx[x->fl];
		L->X[nn + A] = iz * x->m->dz[x->fl];
		L->T_bc[A] = 'N';
		L->T_bc_val[A] = 0.0;
		if ((n + 1) % gnoz == 0) {
			L->T_bc[A] = c->top_T_bc;
			L->T_bc_val[A] = c->top_T_bc_val;
		} else if (n % gnoz == 0) {
			L->T_bc[A] = c->bot_T_bc;
			L->T_bc_val[A] = c->bot_T_bc_val;
		} else if (n < gnoz) {
			if (L->T_bc[A] != 'T')
				L->T_bc[A] = c->lef_T_bc;
			L->T_bc_val[A] = c->lef_T_bc_val;
		} else if (n > (gnox - 1) * gnoz - 1) {
			if (L->T_bc[A] != 'T')
				L->T_bc[A] = c->rig_T_bc;
			L->T_bc_val[A] = c->rig_T_bc_val;
		}
		for (int d = 0; d < 2; d++) {
			char *bc = &L->v_bc[d * nn + A];
			double *bv = &L->v_bc_val[d * nn + A];
			*bc = 'N';
			*bv = 0.0;
			if ((n + 1) % gnoz == 0) {
				*bc = c->top_v_bc[d];
				*bv = c->top_v_bc_val[d];
			} else if (n % gnoz == 0) {
				*bc = c->bot_v_bc[d];
				*bv = c->bot_v_bc_val[d];
			}
			if (n < gnoz) {
				if (*bc != 'V')
					*bc = c->lef_v_bc[d];
				*bv = c->lef_v_bc_val[d];
			} else if (n > (gnox - 1) * gnoz - 1) {
				if (*bc != 'V')
					*bc = c->rig_v_bc[d];
				*bv = c->rig_v_bc_val[d];
			}
		}
	}
}

/* element geometry (Shape_function.c:123-167, Construct_ien_id_lm.c:198-218) */
static void geom_range(void *p, long e0, long e1)
{
	const lvl_ctx *x = (const lvl_ctx *)p;
	mclg_level *L = x->L;
	const long ne = L->nel, nn = L->nno;
	for (long e = e0; e < e1; e++) {
		int n0 = L->ienl[e], n2 = L->ienl[2L * ne + e];
		L->dx_dxi[e] = 0.5 * x->m->dx[L->elev[e]];
		L->dz_deta[e] = 0.5 * x->m->dz[L->elev[e]];
		L->jacobi[e] = L->dx_dxi[e] * L->dz_deta[e] - 0.0 * 0.0;
		L->area[e] = (L->X[n2] - L->X[n0]) * (L->X[nn + n2] - L->X[nn + n0]);
	}
}

/* fine cell -> covering element (elements cover disjoint cells) */
static void cell_range(void *p, long e0, long e1)
{
	const lvl_ctx *x = (const lvl_ctx *)p;
	mclg_level *L = x->L;
	const long ncz = x->gnoz - 1;
	for (long e = e0; e < e1; e++) {
		int n0 = L->ien[e], ix0 = n0 / x->gnoz, iz0 = n0 - ix0 * x->gnoz, s = 1 << (x->fl - L->elev[e]), i, j;
		for (i = 0; i < s; i++)
			for (j = 0; j < s; j++)
				L->cell_elem[(long)(ix0 + i) * ncz + iz0 + j] = (int)e;
	}
}

static int build_level_arrays(mclg_mesh *m, const mclg_config *c, int lev)
{
	mclg_level *L = &m->lev[lev];
	int ne = L->nel, e, a, A, d, gnoz = m->gnoz, gnox = m->gnox, fl = m->max_level - 1;
	long k, nn;
	ivec nodes = {0};
	lvl_ctx lc = {m, c, L, lev, fl, gnox, gnoz};

	/* ien (Construct_ien_id_lm.c:3-41) */
	ALLOC(L->ien, 4L * ne);
	ALLOC(L->elev, ne);
	mclg_parallel_for(ne, 16384, ien_range, &lc);
	/* node list (Construct_ien_id_lm.c:43-66): the sorted distinct ids of ien.
	 * Grids of up to 4M node ids keep a direct id -> index table, which also
	 * serves node_index; larger ones sort and binary-search. */
	if ((long)gnox * gnoz <= (1L << 22)) {
		const long ng = (long)gnox * gnoz;
		L->lut_n = ng;
		L->node_lut = (int *)malloc((size_t)ng * sizeof(int));
		if (L->node_lut == NULL)
			goto oom;
		memset(L->node_lut, 0xff, (size_t)ng * sizeof(int));
		for (k = 0; k < 4L * ne; k++)
			L->node_lut[L->ien[k]] = 0;
		nn = 0;
		for (long g = 0; g < ng; g++)
			if (L->node_lut[g] == 0)
				nn++;
		ALLOC(nodes.a, nn);
		nn = 0;
		for (long g = 0; g < ng; g++)
			if (L->node_lut[g] == 0) {
				nodes.a[nn] = (int)g;
				L->node_lut[g] = (int)nn++;
			}
	} else {
		for (k = 0; k < 4L * ne; k++)
			if (ivec_push(&nodes, L->ien[k]) != 0)
				goto oom;
		nn = sort_unique(nodes.a, nodes.n);
	}
	L->nno = (int)nn;
	L->node = nodes.a;
	ALLOC(L->ienl, 4L * ne);
	mclg_parallel_for(4L * ne, 65536, ienl_range, &lc);

	/* coordinates (Mesh.c:430-452), temperature and velocity BC codes
	 * (Boundary_condition.c:10-110) */
	ALLOC(L->X, 2 * nn);
	ALLOC(L->T_bc, nn);
	ALLOC(L->T_bc_val, nn);
	ALLOC(L->v_bc, 2 * nn);
	ALLOC(L->v_bc_val, 2 * nn);
	mclg_parallel_for(nn, 16384, node_range, &lc);
	/* equation numbers (Construct_ien_id_lm.c:79-144) */
	ALLOC(L->id, 2 * nn);
	ALLOC(L->heat_id, nn);
	{
		int P = 0;
		for (A = 0; A < nn; A++)
			for (d = 0; d < 2; d++)
				L->id[d * nn + A] = (L->v_bc[d * nn + A] == 'V') ? -1 : P++;
		L->neq = P;
		P = 0;
		for (A = 0; A < nn; A++)
			L->heat_id[A] = (L->T_bc[A] == 'T') ? -1 : P++;
		L->heat_neq = P;
	}
	/* element geometry (Shape_function.c:123-167, Construct_ien_id_lm.c:198-218) */
	ALLOC(L->dx_dxi, ne);
	ALLOC(L->dz_deta, ne);
	ALLOC(L->jacobi, ne);
	ALLOC(L->area, ne);
	mclg_parallel_for(ne, 16384, geom_range, &lc);
	/* node -> element map in ascending element order (Construct_ien_id_lm.c:220-244) */
	ALLOC(L->p2n_cnt, nn);
	ALLOC(L->p2n_el, 4 * nn);
	ALLOC(L->p2n_a, 4 * nn);
	for (A = 0; A < 4 * nn; A++) {
		L->p2n_el[A] = -1;
		L->p2n_a[A] = 0;
	}
	for (e = 0; e < ne; e++)
		for (a = 0; a < 4; a++) {
			int i = L->ienl[(long)a * ne + e], s = L->p2n_cnt[i]++;
			if (s >= 4) {
				mclg_set_error("node %d touches more than 4 elements", L->node[i]);
				return MCLG_BAD_INPUT;
			}
			L->p2n_el[(long)s * nn + i] = e;
			L->p2n_a[(long)s * nn + i] = a;
		}
	/* hanging nodes (Connection.c:59-276, single rank: the local part only) */
	{
		ivec hn = {0}, h0 = {0}, h1 = {0};
		int h;
		for (e = 0; e < ne; e++) {
			int i;
			if (L->elev[e] == lev)
				continue;
			for (i = 0; i < 4; i++) {
				int c0 = L->ien[(long)i * ne + e], c1 = L->ien[(long)((i + 1) % 4) * ne + e];
				int mid = (c0 + c1) / 2;
				if (mclg_node_index(L, mid) >= 0) {
					if (ivec_push(&hn, mid) || ivec_push(&h0, c0) || ivec_push(&h1, c1))
						goto oom;
				}
			}
		}
		L->nh = (int)hn.n;
		L->hang_node = hn.a ? hn.a : calloc(1, sizeof(int));
		L->hang_c0 = h0.a ? h0.a : calloc(1, sizeof(int));
		L->hang_c1 = h1.a ? h1.a : calloc(1, sizeof(int));
		ALLOC(L->hang_ni, L->nh);
		ALLOC(L->hang_ci0, L->nh);
		ALLOC(L->hang_ci1, L->nh);
		for (h = 0; h < L->nh; h++) {
			L->hang_ni[h] = mclg_node_index(L, L->hang_node[h]);
			L->hang_ci0[h] = mclg_node_index(L, L->hang_c0[h]);
			L->hang_ci1[h] = mclg_node_index(L, L->hang_c1[h]);
		}
		/* a parent that is itself hanging makes the overwrite order matter */
		L->hang_chained = 0;
		if (L->nh > 0) {
			char *is_h = calloc((size_t)nn + 1, 1);
			if (is_h == NULL)
				goto oom;
			for (h = 0; h < L->nh; h++)
				is_h[L->hang_ni[h]] = 1;
			for (h = 0; h < L->nh; h++)
				if (is_h[L->hang_ci0[h]] || is_h[L->hang_ci1[h]])
					L->hang_chained = 1;
			free(is_h);
		}
	}
	/* sorted neighbour lists and element slot map (for the node-block operator),
	 * node and element loops in chunks on threads */
	{
		int w = 0;
		nb_ctx nc;
		nb_fill_ctx fc;
		kslot_ctx kc;
		ALLOC(L->nb_cnt, nn);
		nc.L = L;
		nc.lists = (int *)malloc((size_t)16 * nn * sizeof(int));
		if (nc.lists == NULL)
			goto oom;
		mclg_parallel_for(nn, 16384, nb_lists, &nc);
		for (A = 0; A < nn; A++)
			if (L->nb_cnt[A] > w)
				w = L->nb_cnt[A];
		if (w > MCLG_NB_MAX) {
			free(nc.lists);
			mclg_set_error("a node has %d neighbours (max %d)", w, MCLG_NB_MAX);
			return MCLG_BAD_INPUT;
		}
		L->nbw = w;
		L->nb = (int *)calloc((size_t)w * nn + 1, sizeof(int));
		if (L->nb == NULL) {
			free(nc.lists);
			goto oom;
		}
		fc.L = L;
		fc.lists = nc.lists;
		fc.w = w;
		fc.nb = L->nb;
		mclg_parallel_for(nn, 16384, nb_fill, &fc);
		free(nc.lists);
		ALLOC(L->kslot, 16L * ne);
		kc.L = L;
		kc.bad = 0;
		mclg_parallel_for(ne, 16384, kslot_fill, &kc);
		if (kc.bad) {
			mclg_set_error("internal: neighbour slot not found");
			return MCLG_BAD_INPUT;
		}
	}
	/* fine cell -> covering element (the horizontal average and the field
	 * transfers of the finest level; coarser levels do not need it) */
	if (lev == fl) {
		long ncx = gnox - 1, ncz = gnoz - 1;
		ALLOC(L->cell_elem, ncx * ncz);
		mclg_parallel_for(ne, 16384, cell_range, &lc);
	}
	return MCLG_OK;
oom:
	mclg_set_error("out of host memory while building level %d", lev);
	return MCLG_BAD_INPUT;
}

/* leaves != NULL: the finest-level Morton start codes of a given leaf set
 * (sorted, covering the domain) replace initial_refine; the last leaf's level
 * then comes from the codes left to the end of the domain. */
typedef struct {
	mclg_mesh *m;
	const mclg_config *c;
	int lev, rc;
	char err[512];
} lvl_job;

static void *level_worker(void *p)
{
	lvl_job *j = (lvl_job *)p;
	j->rc = build_level_arrays(j->m, j->c, j->lev);
	if (j->rc != MCLG_OK)
		snprintf(j->err, sizeof j->err, "%s", mclg_last_error());
	return NULL;
}

int mclg_mesh_frame(mclg_mesh *m, const mclg_config *c)
{
	int lev, fl;
	memset(m, 0, sizeof *m);
	if (c->nprox != 1 || c->nproz != 1) {
		mclg_set_error("nprox=%d nproz=%d: one device holds the whole mesh, set nprox=nproz=1",
		               c->nprox, c->nproz);
		return MCLG_BAD_INPUT;
	}
	if (c->level < 2 || c->level > 15 || c->mg_min_level >= c->level || c->mg_min_level < 0) {
		mclg_set_error("level=%d mg_min_level=%d: need 0 <= mg_min_level < level <= 15",
		               c->level, c->mg_min_level);
		return MCLG_BAD_INPUT;
	}
	m->min_level = c->mg_min_level;
	m->max_level = c->level;
	fl = m->max_level - 1;
	/* get_time_independent_variables (Mesh.c:396-428), one rank */
	m->length = c->model_length;
	m->height = c->model_height;
	for (lev = 0; lev < m->max_level; lev++) {
		int mul = 1 << lev;
		m->max_elx[lev] = mul;
		m->max_nel[lev] = mul * mul;
		m->dx[lev] = m->length / mul;
		m->dz[lev] = m->height / mul;
	}
	m->gnox = m->max_elx[fl] + 1;
	m->gnoz = m->max_elx[fl] + 1;
	return MCLG_OK;
}

int mclg_mesh_check_leaves(const mclg_mesh *m, const int *leaves, long n)
{
	const int cap = m->max_nel[m->max_level - 1];
	for (long i = 0; i < n; i++)
		if (leaves[i] < 0 || leaves[i] >= cap || (i > 0 && leaves[i] <= leaves[i - 1])) {
			mclg_set_error("leaf %ld: codes must increase within [0, %d)", i, cap);
			return MCLG_BAD_INPUT;
		}
	if (n < 2) {
		mclg_set_error("refinement produced %ld elements", n);
		return MCLG_BAD_INPUT;
	}
	return MCLG_OK;
}

static int mesh_build_impl(mclg_mesh *m, const mclg_config *c, const int *leaves, long nleaves)
{
	int lev, fl, rc;
	ivec head = {0};
	tree_ctx t;

	rc = mclg_mesh_frame(m, c);
	if (rc != MCLG_OK)
		return rc;
	fl = m->max_level - 1;

	/* build_quad_tree (Tree.c:67-93) */
	t.out = &head;
	t.fine_nel = m->max_nel[fl];
	if (leaves != NULL) {
		long i;
		for (i = 0; i < nleaves; i++) {
			if (leaves[i] < 0 || leaves[i] >= m->max_nel[fl] || (i > 0 && leaves[i] <= leaves[i - 1])) {
				free(head.a);
				mclg_set_error("leaf %ld: codes must increase within [0, %d)", i, m->max_nel[fl]);
				return MCLG_BAD_INPUT;
			}
			if (ivec_push(&head, leaves[i]) != 0) {
				free(head.a);
				return MCLG_BAD_INPUT;
			}
		}
		rc = MCLG_OK;
	} else {
		rc = initial_refine(&t, &head, c->develop_mode, m->max_level);
	}
	if (rc != MCLG_OK) {
		free(head.a);
		return rc;
	}
	{
		mclg_level *L = &m->lev[fl];
		long n = sort_unique(head.a, head.n), e;
		if (n < 2) {
			free(head.a);
			mclg_set_error("refinement produced %ld elements", n);
			return MCLG_BAD_INPUT;
		}
		L->nel = (int)n;
		L->Mcode = head.a;
		/* append_level_to_Mcode (Tree.c:340-358): level from the gap to the next code */
		for (e = 0; e < n - 1; e++)
			L->Mcode[e] = (L->Mcode[e] << MCLG_LEVEL_BITS) | log4i(m->max_nel[fl] / (L->Mcode[e + 1] - L->Mcode[e]));
		e = n - 1;
		if (leaves != NULL)
			L->Mcode[e] = (L->Mcode[e] << MCLG_LEVEL_BITS) | log4i(m->max_nel[fl] / (m->max_nel[fl] - L->Mcode[e]));
		else
			L->Mcode[e] = (L->Mcode[e] << MCLG_LEVEL_BITS)
			            | log4i(m->max_nel[fl] / (L->Mcode[e] - (L->Mcode[e - 1] >> MCLG_LEVEL_BITS)));
	}
	/* project_Mcode (Tree.c:361-389) down to mg_min_level */
	for (lev = fl; lev > m->min_level; lev--) {
		mclg_level *U = &m->lev[lev], *D = &m->lev[lev - 1];
		int e = 0;
		D->Mcode = malloc((size_t)U->nel * sizeof(int) + sizeof(int));
		if (D->Mcode == NULL)
			return MCLG_BAD_INPUT;
		D->nel = 0;
		while (e < U->nel) {
			int level = U->Mcode[e] & ((1 << MCLG_LEVEL_BITS) - 1), loc = U->Mcode[e] >> MCLG_LEVEL_BITS;
			if (level < lev)
				e++;
			else {
				e += 4;
				level -= 1;
			}
			D->Mcode[D->nel++] = (loc << MCLG_LEVEL_BITS) | level;
		}
	}
	{   /* the levels' arrays are independent of one another: one thread per level */
		lvl_job jobs[MCLG_MAX_LEVEL];
		pthread_t th[MCLG_MAX_LEVEL];
		int started[MCLG_MAX_LEVEL], i, nl = m->max_level - m->min_level;
		for (i = 0; i < nl; i++) {
			jobs[i].m = m;
			jobs[i].c = c;
			jobs[i].lev = m->min_level + i;
			jobs[i].rc = MCLG_OK;
			jobs[i].err[0] = 0;
			started[i] = pthread_create(&th[i], NULL, level_worker, &jobs[i]) == 0;
			if (!started[i])
				level_worker(&jobs[i]);
		}
		for (i = 0; i < nl; i++)
			if (started[i])
				pthread_join(th[i], NULL);
		for (i = 0; i < nl; i++)
			if (jobs[i].rc != MCLG_OK) {
				mclg_set_error("%s", jobs[i].err);
				return jobs[i].rc;
			}
	}
	{
		mclg_level *L = &m->lev[fl];
		m->uniform = (L->nel == m->max_nel[fl] && L->nh == 0);
	}
	return MCLG_OK;
}

int mclg_mesh_build(mclg_mesh *m, const mclg_config *c)
{
	return mesh_build_impl(m, c, NULL, 0);
}

int mclg_mesh_build_leaves(mclg_mesh *m, const mclg_config *c, const int *leaves, long n)
{
	if (leaves == NULL || n < 2) {
		memset(m, 0, sizeof *m);
		mclg_set_error("a leaf list needs at least 2 leaves");
		return MCLG_BAD_INPUT;
	}
	return mesh_build_impl(m, c, leaves, n);
}

void mclg_mesh_free(mclg_mesh *m)
{
	int lev;
	for (lev = 0; lev < MCLG_MAX_LEVEL; lev++) {
		mclg_level *L = &m->lev[lev];
		free(L->Mcode); free(L->node); free(L->ien); free(L->ienl); free(L->elev);
		free(L->id); free(L->heat_id); free(L->v_bc); free(L->v_bc_val); free(L->T_bc);
		free(L->T_bc_val); free(L->X); free(L->dx_dxi); free(L->dz_deta); free(L->jacobi);
		free(L->area); free(L->hang_node); free(L->hang_c0); free(L->hang_c1); free(L->hang_ni);
		free(L->hang_ci0); free(L->hang_ci1); free(L->p2n_cnt); free(L->p2n_el); free(L->p2n_a);
		free(L->nb); free(L->nb_cnt); free(L->kslot); free(L->cell_elem); free(L->node_lut);
	}
	memset(m, 0, sizeof *m);
}

/* Initial_condition.c:3-136 on one level; T_ini=-2 is the seeded field of
 * mclg_ic.h.  T_ini=-1 reads the restart file on the finest level
 * (Initial_condition.c:171-195); coarser levels take the finest level's value
 * at the same node (the reference leaves them unset). */
int mclg_host_initial_temperature(const mclg_mesh *m, const mclg_config *c, int lev, double *T)
{
	const mclg_level *L = &m->lev[lev];
	const double pi = M_PI;
	int i, nn = L->nno;
	switch (c->T_ini) {
	case 0:
		for (i = 0; i < nn; i++) {
			double x = L->X[i], z = L->X[nn + i];
			T[i] = m->height - z + c->T_mantle_perturb * sin(pi * (m->height - z) / m->height)
			     * cos(c->T_wave_number * pi * x / m->length);
		}
		break;
	case 1:
		for (i = 0; i < nn; i++) {
			double x = L->X[i], z = L->X[nn + i];
			T[i] = c->T_mantle + c->T_mantle_perturb * sin(pi * (m->height - z) / m->height)
			     * cos(c->T_wave_number * pi * x / m->length);
		}
		break;
	case -2: {
		mclg_ic_params p;
		memset(&p, 0, sizeof p);
		p.kind = c->ic_kind;
		p.seed = c->ic_seed;
		p.noise = c->ic_noise;
		p.perturb = c->T_mantle_perturb;
		p.wave = c->T_wave_number;
		p.bl_thickness = c->ic_bl_thickness;
		p.nmodes = c->ic_modes;
		p.mode_amp = c->ic_mode_amp;
		p.length = m->length;
		p.height = m->height;
		for (i = 0; i < nn; i++)
			T[i] = mclg_ic_temperature(&p, L->X[i], L->X[nn + i], (uint32_t)L->node[i]);
		break;
	}
	case -1: {
		const mclg_level *F = &m->lev[m->max_level - 1];
		char path[2048], line[1000];
		double *Tf = malloc(((size_t)F->nno + 1) * sizeof(double));
		FILE *fp;
		if (Tf == NULL)
			return MCLG_BAD_INPUT;
		snprintf(path, sizeof path, "%s/%07d/temperature.%d.%07d", c->old_T_file,
		         c->old_T_timestep, 0, c->old_T_timestep);
		fp = fopen(path, "r");
		if (fp == NULL) {
			free(Tf);
			mclg_set_error("cannot find file: %s", path);
			return MCLG_IO_ERROR;
		}
		for (i = 0; i < F->nno; i++) {
			if (fgets(line, sizeof line, fp) == NULL || sscanf(line, "%lf", &Tf[i]) != 1) {
				fclose(fp);
				free(Tf);
				mclg_set_error("%s: expected %d lines", path, F->nno);
				return MCLG_IO_ERROR;
			}
		}
		fclose(fp);
		for (i = 0; i < nn; i++) {
			int j = mclg_node_index(F, L->node[i]);
			T[i] = j >= 0 ? Tf[j] : 0.0;
		}
		free(Tf);
		break;
	}
	default:
		mclg_set_error("T_ini=%d is not supported (0, 1, -1 or -2)", c->T_ini);
		return MCLG_BAD_INPUT;
	}
	/* apply_T_bc_values (Initial_condition.c:122-136) */
	for (i = 0; i < nn; i++)
		if (L->T_bc[i] == 'T')
			T[i] = L->T_bc_val[i];
	return MCLG_OK;
}
