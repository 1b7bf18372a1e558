/*
 * |grad T| adaptive refinement: a new quadtree from per-element refinement
 * flags, and the transfer of a nodal field between two meshes.
 *
 * The reference has no runtime refinement (adaptive_mesh_refine is empty,
 * Tree.c:95-99); its trees come from the fixed patterns of initial_refine
 * (Tree.c:184-300).  This builds trees of the same kind -- Morton-ordered
 * leaves whose start codes mclg_mesh_build_leaves turns into the whole mesh
 * stack (numbering, hanging nodes, MG levels) -- from a refinement
 * criterion:
 *   1. every fine cell covered by a flagged leaf of the current mesh asks for
 *      target_level, every other cell for base_level;
 *   2. top-down from the uniform base_level grid, a cell splits while some
 *      fine cell under it asks for a finer level;
 *   3. 2:1 balance across edges and corners: a leaf with a neighbouring leaf
 *      more than one level finer splits, until none does.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>
#include "mclg_host.h"

/* Morton codes hold x in the odd bits and z in the even bits (morton,
 * Tree.c:447-456); compact16 extracts one of them. */
static unsigned compact16(unsigned v)
{
	v &= 0x55555555u;
	v = (v | (v >> 1)) & 0x33333333u;
	v = (v | (v >> 2)) & 0x0f0f0f0fu;
	v = (v | (v >> 4)) & 0x00ff00ffu;
	v = (v | (v >> 8)) & 0x0000ffffu;
	return v;
}

typedef struct amr_tree {
	int F, NF;                 /* finest level, fine cells per side */
	unsigned char **pyr;       /* pyr[k]: max requested level over 2^k x 2^k blocks of fine cells */
	unsigned char *lv;         /* [NF*NF] level of the leaf covering each fine cell, x-major */
	int target;
} amr_tree;

static void fill(unsigned char *a, int NF, int x0, int z0, int s, unsigned char v)
{
	int i, j;
	for (i = 0; i < s; i++)
		for (j = 0; j < s; j++)
			a[(long)(x0 + i) * NF + z0 + j] = v;
}

static void split_down(amr_tree *t, int l, int x, int z)
{
	const int k = t->F - l;
	const int nk = t->NF >> k;
	if (l < t->target && t->pyr[k][(long)x * nk + z] > l) {
		split_down(t, l + 1, 2 * x, 2 * z);
		split_down(t, l + 1, 2 * x, 2 * z + 1);
		split_down(t, l + 1, 2 * x + 1, 2 * z);
		split_down(t, l + 1, 2 * x + 1, 2 * z + 1);
	} else {
		fill(t->lv, t->NF, x << k, z << k, 1 << k, (unsigned char)l);
	}
}

int mclg_amr_build_leaves(const mclg_mesh *m, const unsigned char *flags, int base_level, int target_level,
                          int **leaves, long *n)
{
	const int F = m->max_level - 1, NF = 1 << F;
	const mclg_level *L = &m->lev[F];
	unsigned char *tgt = NULL, *mark = NULL;
	amr_tree t;
	int k, e, rc = MCLG_OK;
	long code, cnt, cap;
	*leaves = NULL;
	*n = 0;
	if (base_level < 0 || base_level > target_level || target_level > F) {
		mclg_set_error("refinement levels base=%d target=%d: need 0 <= base <= target <= %d", base_level,
		               target_level, F);
		return MCLG_BAD_INPUT;
	}
	memset(&t, 0, sizeof t);
	t.F = F;
	t.NF = NF;
	t.target = target_level;
	t.pyr = (unsigned char **)calloc((size_t)(F - base_level + 1), sizeof(unsigned char *));
	tgt = (unsigned char *)malloc((size_t)NF * NF);
	t.lv = (unsigned char *)malloc((size_t)NF * NF);
	mark = (unsigned char *)malloc((size_t)NF * NF);
	if (t.pyr == NULL || tgt == NULL || t.lv == NULL || mark == NULL) {
		free(tgt);
		goto oom;
	}
	/* 1. requested level per fine cell */
	memset(tgt, base_level, (size_t)NF * NF);
	for (e = 0; e < L->nel; e++) {
		int lvl, x0, z0;
		if (!flags[e])
			continue;
		lvl = L->Mcode[e] & ((1 << MCLG_LEVEL_BITS) - 1);
		x0 = (int)compact16((unsigned)(L->Mcode[e] >> MCLG_LEVEL_BITS) >> 1);
		z0 = (int)compact16((unsigned)(L->Mcode[e] >> MCLG_LEVEL_BITS));
		fill(tgt, NF, x0, z0, 1 << (F - lvl), (unsigned char)target_level);
	}
	/* max pyramid */
	t.pyr[0] = tgt;
	for (k = 1; k <= F - base_level; k++) {
		const int nk = NF >> k, np = NF >> (k - 1);
		int x, z;
		t.pyr[k] = (unsigned char *)malloc((size_t)nk * nk);
		if (t.pyr[k] == NULL)
			goto oom;
		for (x = 0; x < nk; x++)
			for (z = 0; z < nk; z++) {
				const unsigned char *p = t.pyr[k - 1];
				unsigned char a = p[(long)(2 * x) * np + 2 * z], b = p[(long)(2 * x) * np + 2 * z + 1];
				unsigned char c = p[(long)(2 * x + 1) * np + 2 * z], d = p[(long)(2 * x + 1) * np + 2 * z + 1];
				unsigned char mx = a > b ? a : b;
				mx = mx > c ? mx : c;
				t.pyr[k][(long)x * nk + z] = mx > d ? mx : d;
			}
	}
	/* 2. top-down from the base grid */
	{
		const int nb = 1 << base_level;
		int x, z;
		for (x = 0; x < nb; x++)
			for (z = 0; z < nb; z++)
				split_down(&t, base_level, x, z);
	}
	/* 3. 2:1 balance over the 8 neighbours of every fine cell */
	for (;;) {
		int x, z, changed = 0;
		memset(mark, 0, (size_t)NF * NF);
		for (x = 0; x < NF; x++)
			for (z = 0; z < NF; z++) {
				const int l = t.lv[(long)x * NF + z];
				int dx, dz, need = 0;
				for (dx = -1; dx <= 1 && !need; dx++)
					for (dz = -1; dz <= 1; dz++) {
						const int nx = x + dx, nz = z + dz;
						if (nx < 0 || nx >= NF || nz < 0 || nz >= NF)
							continue;
						if (t.lv[(long)nx * NF + nz] > l + 1) {
							need = 1;
							break;
						}
					}
				if (need) {
					const int s = 1 << (F - l);
					mark[(long)(x & ~(s - 1)) * NF + (z & ~(s - 1))] = (unsigned char)(l + 1);
				}
			}
		for (x = 0; x < NF; x++)
			for (z = 0; z < NF; z++) {
				const unsigned char nl = mark[(long)x * NF + z];
				if (nl) {
					fill(t.lv, NF, x, z, 1 << (F - nl + 1), nl);
					changed = 1;
				}
			}
		if (!changed)
			break;
	}
	/* leaves in Morton order */
	cap = 1024;
	*leaves = (int *)malloc((size_t)cap * sizeof(int));
	if (*leaves == NULL)
		goto oom;
	cnt = 0;
	for (code = 0; code < (long)NF * NF;) {
		const int x = (int)compact16((unsigned)code >> 1), z = (int)compact16((unsigned)code);
		const int l = t.lv[(long)x * NF + z];
		if (cnt == cap) {
			int *a;
			cap *= 2;
			a = (int *)realloc(*leaves, (size_t)cap * sizeof(int));
			if (a == NULL)
				goto oom;
			*leaves = a;
		}
		(*leaves)[cnt++] = (int)code;
		code += 1L << (2 * (F - l));
	}
	*n = cnt;
	goto done;
oom:
	mclg_set_error("out of host memory building the refined tree");
	free(*leaves);
	*leaves = NULL;
	rc = MCLG_BAD_INPUT;
done:
	if (t.pyr)
		for (k = 0; k <= F - base_level; k++)
			free(t.pyr[k]);   /* pyr[0] is tgt */
	free(t.pyr);
	free(t.lv);
	free(mark);
	return rc;
}

/* Mean of an element field of `from` over the square of fine cells (x0, z0, s):
 * the covering leaf's value where that leaf is at least as large, else the mean
 * of the four quadrants' means. */
static double region_mean(const mclg_level *A, int F, int ncell, const double *P, int x0, int z0, int s)
{
	const int e = A->cell_elem[(long)x0 * ncell + z0];
	const int so = 1 << (F - (A->Mcode[e] & ((1 << MCLG_LEVEL_BITS) - 1)));
	const int h = s >> 1;
	if (so >= s)
		return P[e];
	return 0.25 * ((region_mean(A, F, ncell, P, x0, z0, h) + region_mean(A, F, ncell, P, x0, z0 + h, h)) +
	               (region_mean(A, F, ncell, P, x0 + h, z0, h) + region_mean(A, F, ncell, P, x0 + h, z0 + h, h)));
}

/* P_to per finest-level element of `to`: the area mean of the element field
 * P_from of `from` over it.  Where the leaf of `from` covering the new element
 * is as large or larger, that is its value; where `from` was finer, the mean of
 * its leaves there, so that the integral of P is kept and a pattern alternating
 * over the children (the Q1-P0 pressure's checkerboard modes) averages out
 * instead of being sampled into the new element.  Both meshes must share the
 * finest level and the box.  Elements in chunks on threads. */
typedef struct {
	const mclg_level *A, *B;
	const double *P_from;
	double *P_to;
	int F, ncell;
} elem_tr;

static void elem_tr_run(void *p, long e0, long e1)
{
	const elem_tr *t = (const elem_tr *)p;
	for (long e = e0; e < e1; e++) {
		const int lvl = t->B->Mcode[e] & ((1 << MCLG_LEVEL_BITS) - 1);
		const unsigned code = (unsigned)(t->B->Mcode[e] >> MCLG_LEVEL_BITS);
		t->P_to[e] = region_mean(t->A, t->F, t->ncell, t->P_from, (int)compact16(code >> 1), (int)compact16(code),
		                         1 << (t->F - lvl));
	}
}

int mclg_amr_transfer_elem(const mclg_mesh *from, const double *P_from, const mclg_mesh *to, double *P_to)
{
	const int F = from->max_level - 1;
	const mclg_level *A = &from->lev[F], *B = &to->lev[to->max_level - 1];
	elem_tr t;
	if (to->max_level != from->max_level || to->gnox != from->gnox ||
	    fabs(from->length - to->length) > 1e-12 * from->length ||
	    fabs(from->height - to->height) > 1e-12 * from->height) {
		mclg_set_error("element field transfer between meshes of different finest level or box");
		return MCLG_BAD_INPUT;
	}
	if (A->cell_elem == NULL) {
		mclg_set_error("element field transfer: the source mesh has no cell map");
		return MCLG_BAD_INPUT;
	}
	t.A = A;
	t.B = B;
	t.P_from = P_from;
	t.P_to = P_to;
	t.F = F;
	t.ncell = from->gnox - 1;
	mclg_parallel_for(B->nel, 16384, elem_tr_run, &t);
	return MCLG_OK;
}

/* T_to at the finest-level nodes of `to`: the bilinear interpolant of T_from
 * on the finest-level leaf of `from` that contains each node (hanging nodes
 * of `from` hold their parents' mean, so the interpolant is continuous).
 * Nodes in chunks on threads. */
typedef struct {
	const mclg_level *A, *B;
	const double *T_from;
	double *T_to;
	int ncell;
	double dxc, dzc;
} node_tr;

static void node_tr_run(void *p, long i0, long i1)
{
	const node_tr *t = (const node_tr *)p;
	const mclg_level *A = t->A, *B = t->B;
	const int ncell = t->ncell;
	for (long i = i0; i < i1; i++) {
		const double x = B->X[i], z = B->X[B->nno + i];
		int cx = (int)(x / t->dxc), cz = (int)(z / t->dzc), e;
		double x0, z0, w, h, xi, ze;
		int n0, n1, n2, n3;
		cx = cx < 0 ? 0 : cx >= ncell ? ncell - 1 : cx;
		cz = cz < 0 ? 0 : cz >= ncell ? ncell - 1 : cz;
		e = A->cell_elem[(long)cx * ncell + cz];
		n0 = A->ienl[e];
		n1 = A->ienl[A->nel + e];
		n2 = A->ienl[2 * A->nel + e];
		n3 = A->ienl[3 * A->nel + e];
		x0 = A->X[n0];
		z0 = A->X[A->nno + n0];
		w = A->X[n3] - x0;
		h = A->X[A->nno + n1] - z0;
		xi = (x - x0) / w;
		ze = (z - z0) / h;
		t->T_to[i] = (1 - xi) * ((1 - ze) * t->T_from[n0] + ze * t->T_from[n1]) +
		             xi * (ze * t->T_from[n2] + (1 - ze) * t->T_from[n3]);
	}
}

int mclg_amr_transfer(const mclg_mesh *from, const double *T_from, const mclg_mesh *to, double *T_to)
{
	const int F = from->max_level - 1, G = to->max_level - 1;
	node_tr t;
	if (fabs(from->length - to->length) > 1e-12 * from->length ||
	    fabs(from->height - to->height) > 1e-12 * from->height) {
		mclg_set_error("field transfer between boxes of different size");
		return MCLG_BAD_INPUT;
	}
	t.A = &from->lev[F];
	t.B = &to->lev[G];
	t.T_from = T_from;
	t.T_to = T_to;
	t.ncell = from->gnox - 1;
	t.dxc = from->length / t.ncell;
	t.dzc = from->height / t.ncell;
	mclg_parallel_for(t.B->nno, 16384, node_tr_run, &t);
	return MCLG_OK;
}
