/* Transfer maps and sweep order of the reference's own inner solvers
 * solver="mg" (multigrid, Solver.c:668-768) and solver="gs" (Gauss-Seidel,
 * Solver.c:1866-1929), for one rank.
 *
 * Both maps are equation-indexed, as the reference keeps them:
 *
 *   interp (build_interp_conn, Connection.c:708-930): equation u of level
 *     lev+1 receives the mean of n(u) errors of level lev.  Three passes, in
 *     the reference's order, each claiming a node of lev+1 the first time it
 *     is met: the midpoint of every edge of every leaf element of lev (n = 2,
 *     corners p and (p+1)%4), the element centre (n = 4, corners in ien
 *     order), then the nodes lev and lev+1 share (n = 1).  A term whose
 *     lower equation is fixed (id = -1) stays in the mean's count.
 *   project (build_project_conn + setup_project_comm_frame,
 *     Connection.c:1051-1250): equation l of lev takes the residual of the
 *     equation of the same node and direction on lev+1 (injection).
 *
 * The Gauss-Seidel wavefronts are this engine's: wave(A) is one more than
 * the wave of every matrix neighbour B < A (whose new value row A reads) and
 * one less than that of every neighbour C > A (whose old value it reads), so
 * sweeping the wavefronts in order, nodes of one wavefront in parallel, does
 * the arithmetic of the sequential sweep in equation order exactly. */
#include <stdlib.h>
#include <string.h>

#include "mclg_host.h"

int mclg_refmg_interp(const mclg_mesh *m, int lev, int *n, int *src)
{
	if (lev <= m->min_level || lev >= m->max_level)
		return MCLG_BAD_INPUT;
	const mclg_level *lo = &m->lev[lev - 1], *up = &m->lev[lev];
	const int neq = up->neq, nlo = lo->nno, nup = up->nno, nel = lo->nel;
	char *check = (char *)calloc((size_t)nup + 1, 1);
	if (check == NULL)
		return MCLG_BAD_INPUT;
	for (int u = 0; u < neq; u++) {
		n[u] = 0;
		for (int i = 0; i < 4; i++)
			src[(size_t)i * neq + u] = -1;
	}
	for (int e = 0; e < nel; e++) {
		if (lo->elev[e] > lev - 1)   /* leaf test of Connection.c:753-754 */
			continue;
		/* edge midpoints: 2 -> 1 */
		for (int p = 0; p < 4; p++) {
			const int n1 = lo->ien[(size_t)p * nel + e], n2 = lo->ien[(size_t)((p + 1) % 4) * nel + e];
			const int j = mclg_node_index(up, (n1 + n2) / 2);
			if (j < 0 || check[j])
				continue;
			check[j] = 1;
			const int i1 = mclg_node_index(lo, n1), i2 = mclg_node_index(lo, n2);
			for (int d = 0; d < 2; d++) {
				const int eu = up->id[(size_t)d * nup + j];
				if (eu < 0)
					continue;
				src[eu] = lo->id[(size_t)d * nlo + i1];
				src[(size_t)neq + eu] = lo->id[(size_t)d * nlo + i2];
				n[eu] = 2;
			}
		}
		/* element centre: 4 -> 1 */
		int c = 0;
		for (int p = 0; p < 4; p++)
			c += lo->ien[(size_t)p * nel + e];
		const int j = mclg_node_index(up, c / 4);
		if (j < 0 || check[j])
			continue;
		check[j] = 1;
		for (int d = 0; d < 2; d++) {
			const int eu = up->id[(size_t)d * nup + j];
			if (eu < 0)
				continue;
			for (int p = 0; p < 4; p++) {
				const int i = mclg_node_index(lo, lo->ien[(size_t)p * nel + e]);
				src[(size_t)p * neq + eu] = lo->id[(size_t)d * nlo + i];
			}
			n[eu] = 4;
		}
	}
	/* nodes on both levels: 1 -> 1 */
	int rc = MCLG_OK;
	for (int i = 0; i < nlo; i++) {
		const int j = mclg_node_index(up, lo->node[i]);
		if (j < 0 || check[j])
			continue;
		check[j] = 1;
		for (int d = 0; d < 2; d++) {
			const int eu = up->id[(size_t)d * nup + j];
			if (eu < 0)
				continue;
			if (n[eu] >= 4) {
				rc = MCLG_BAD_INPUT;
				continue;
			}
			src[(size_t)n[eu] * neq + eu] = lo->id[(size_t)d * nlo + i];
			n[eu]++;
		}
	}
	free(check);
	return rc;
}

int mclg_refmg_project(const mclg_mesh *m, int lev, int *up_eq)
{
	if (lev < m->min_level || lev >= m->max_level - 1)
		return MCLG_BAD_INPUT;
	const mclg_level *lo = &m->lev[lev], *up = &m->lev[lev + 1];
	for (int l = 0; l < lo->neq; l++)
		up_eq[l] = -1;
	for (int i = 0; i < up->nno; i++) {
		const int j = mclg_node_index(lo, up->node[i]);
		if (j < 0)
			continue;
		for (int d = 0; d < 2; d++) {
			const int el = lo->id[(size_t)d * lo->nno + j];
			if (el >= 0)
				up_eq[el] = up->id[(size_t)d * up->nno + i];
		}
	}
	return MCLG_OK;
}

int mclg_refmg_waves(const mclg_level *L, int *wave)
{
	const int nno = L->nno;
	for (int A = 0; A < nno; A++)
		wave[A] = 0;
	for (int A = 0; A < nno; A++) {
		for (int k = 0; k < L->nb_cnt[A]; k++) {
			const int B = L->nb[(size_t)k * nno + A];
			if (B < A && wave[B] + 1 > wave[A])
				wave[A] = wave[B] + 1;
		}
		/* wave[A] is final: every neighbour below A has pulled or pushed */
		for (int k = 0; k < L->nb_cnt[A]; k++) {
			const int C = L->nb[(size_t)k * nno + A];
			if (C > A && wave[A] + 1 > wave[C])
				wave[C] = wave[A] + 1;
		}
	}
	return MCLG_OK;
}
