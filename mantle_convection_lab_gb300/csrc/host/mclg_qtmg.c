/* Constrained-space structure of the converged solver on quadtree meshes.
 *
 * On a mesh with hanging nodes the velocity space is conforming: the value of
 * a hanging node's free component is the mean of its two parents'
 * (Connection.c:59-276 finds them; enforce_constrain_veq, Solver.c:1368-1482,
 * imposes the same relation inside the reference's CG), so the unknowns are
 * the free components of the other nodes ("reduced" dofs) and the discrete
 * system is C^T K C d + C^T G p = C^T F, G^T C d = 0 with C the expansion of
 * reduced dofs to all dofs.  The reference's iteration applies the relation
 * by overwriting inside CG without folding the hanging rows into their
 * parents, so its system has no exact solution on such meshes; this one has.
 *
 * Per level, dofs are 2*node + component:
 *   kind      0 fixed (Dirichlet 'V'), 1 reduced, 2 constrained (hanging, free)
 *   expand    constrained dof = sum w * reduced dof (parents' chains resolved;
 *             a fixed parent contributes its value, 0 for the homogeneous
 *             corrections this structure is used for)
 *   fold      the transpose: for a reduced dof, the constrained dofs whose
 *             expansion holds it, with the same weights
 *   C^T K C   the reduced operator as node-block ELL rows, assembled on the
 *             device each step from per-row contribution lists
 *   P         prolongation from the level below to this level's reduced dofs:
 *             the reference's averaging map (build_interp_conn,
 *             Connection.c:708-930) applied to the coarse expanded field
 *   R         restriction to this level from the level above, P^T by rows.
 * All lists are CSR by dof, built in ascending order so device gathers sum in
 * a fixed order. */
#include <pthread.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "mclg_host.h"

typedef struct {
	int *idx;
	double *w;
	long n, cap;
} csr_b;

static int csr_push(csr_b *c, int idx, double w)
{
	if (c->n == c->cap) {
		long cap = c->cap ? 2 * c->cap : 256;
		int *i2 = (int *)realloc(c->idx, (size_t)cap * sizeof(int));
		if (i2 == NULL)
			return -1;
		c->idx = i2;
		double *w2 = (double *)realloc(c->w, (size_t)cap * sizeof(double));
		if (w2 == NULL)
			return -1;
		c->w = w2;
		c->cap = cap;
	}
	c->idx[c->n] = idx;
	c->w[c->n] = w;
	c->n++;
	return 0;
}

/* a term list: (dof, weight) pairs, merged by dof */
typedef struct {
	int dof[64];
	double w[64];
	int n;
} terms;

static int terms_add(terms *t, int dof, double w)
{
	int i;
	for (i = 0; i < t->n; i++)
		if (t->dof[i] == dof) {
			t->w[i] += w;
			return 0;
		}
	if (t->n == 64)
		return -1;
	t->dof[t->n] = dof;
	t->w[t->n] = w;
	t->n++;
	return 0;
}

static void terms_sort(terms *t)
{
	int i, j;
	for (i = 1; i < t->n; i++)
		for (j = i; j > 0 && t->dof[j - 1] > t->dof[j]; j--) {
			int d = t->dof[j];
			double w = t->w[j];
			t->dof[j] = t->dof[j - 1];
			t->w[j] = t->w[j - 1];
			t->dof[j - 1] = d;
			t->w[j - 1] = w;
		}
}

/* expansion of dof (2*A + c) of level L into reduced dofs, through chains of
 * hanging parents; hang_of[A] = index in the hanging list or -1 */
static int expand_dof(const mclg_level *L, const int *hang_of, int dof, double w, int depth, terms *out)
{
	const int A = dof >> 1, c = dof & 1;
	if (L->v_bc[(size_t)c * L->nno + A] == 'V')
		return 0;   /* fixed: value 0 in the homogeneous space */
	const int h = hang_of[A];
	if (h < 0)
		return terms_add(out, dof, w);
	if (depth > 16)
		return -1;   /* a cycle of hanging parents: not a quadtree */
	if (expand_dof(L, hang_of, 2 * L->hang_ci0[h] + c, 0.5 * w, depth + 1, out))
		return -1;
	return expand_dof(L, hang_of, 2 * L->hang_ci1[h] + c, 0.5 * w, depth + 1, out);
}

static void free_csr(int **off, int **idx, double **w)
{
	free(*off);
	free(*idx);
	free(*w);
	*off = NULL;
	*idx = NULL;
	*w = NULL;
}

void mclg_qt_free(mclg_qt_level *q)
{
	free(q->kind);
	free_csr(&q->ex_off, &q->ex_src, &q->ex_w);
	free_csr(&q->fo_off, &q->fo_dof, &q->fo_w);
	free_csr(&q->p_off, &q->p_src, &q->p_w);
	free_csr(&q->r_off, &q->r_src, &q->r_w);
	free(q->node_map);
	free(q->rnb);
	free(q->rcnt);
	free(q->rc_off);
	free(q->rc_tgt);
	free(q->rc_src);
	free(q->rc_w);
	memset(q, 0, sizeof *q);
}

/* hand a built list's arrays over (never NULL) */
static int take(csr_b *b, int **idx, double **w)
{
	*idx = b->idx ? b->idx : (int *)malloc(sizeof(int));
	*w = b->w ? b->w : (double *)malloc(sizeof(double));
	return (*idx && *w) ? 0 : -1;
}

/* kind, expand and fold lists of one level */
static int build_constraints(const mclg_level *L, mclg_qt_level *q)
{
	const int nno = L->nno, nd = 2 * nno;
	int *hang_of = (int *)malloc((size_t)nno * sizeof(int));
	csr_b ex = {0}, fo = {0};
	int rc = MCLG_BAD_INPUT, h, d, i;
	q->nno = nno;
	q->kind = (unsigned char *)calloc((size_t)nd + 1, 1);
	q->ex_off = (int *)calloc((size_t)nd + 1, sizeof(int));
	q->fo_off = (int *)calloc((size_t)nd + 1, sizeof(int));
	if (!hang_of || !q->kind || !q->ex_off || !q->fo_off)
		goto out;
	for (i = 0; i < nno; i++)
		hang_of[i] = -1;
	for (h = 0; h < L->nh; h++)
		hang_of[L->hang_ni[h]] = h;
	for (d = 0; d < nd; d++) {
		const int A = d >> 1, c = d & 1;
		q->kind[d] = L->v_bc[(size_t)c * nno + A] == 'V' ? 0 : hang_of[A] >= 0 ? 2 : 1;
	}
	/* expand lists of constrained dofs */
	for (d = 0; d < nd; d++) {
		q->ex_off[d] = (int)ex.n;
		if (q->kind[d] != 2)
			continue;
		const int A = d >> 1, c = d & 1, hh = hang_of[A];
		terms t;
		t.n = 0;
		if (expand_dof(L, hang_of, 2 * L->hang_ci0[hh] + c, 0.5, 1, &t) ||
		    expand_dof(L, hang_of, 2 * L->hang_ci1[hh] + c, 0.5, 1, &t)) {
			mclg_set_error("hanging node %d: its parents' chain does not end", A);
			goto out;
		}
		terms_sort(&t);
		for (i = 0; i < t.n; i++)
			if (csr_push(&ex, t.dof[i], t.w[i]))
				goto out;
	}
	q->ex_off[nd] = (int)ex.n;
	/* fold: transpose of expand, by reduced dof, constrained dofs ascending */
	{
		int *cnt = (int *)calloc((size_t)nd + 1, sizeof(int));
		if (cnt == NULL)
			goto out;
		for (long k = 0; k < ex.n; k++)
			cnt[ex.idx[k]]++;
		q->fo_off[0] = 0;
		for (d = 0; d < nd; d++)
			q->fo_off[d + 1] = q->fo_off[d] + cnt[d];
		fo.n = fo.cap = ex.n;
		fo.idx = (int *)malloc((size_t)(ex.n + 1) * sizeof(int));
		fo.w = (double *)malloc((size_t)(ex.n + 1) * sizeof(double));
		if (!fo.idx || !fo.w) {
			free(cnt);
			goto out;
		}
		memcpy(cnt, q->fo_off, (size_t)nd * sizeof(int));
		for (d = 0; d < nd; d++)   /* constrained dofs in ascending order */
			for (int k = q->ex_off[d]; k < q->ex_off[d + 1]; k++) {
				const int a = ex.idx[k];
				fo.idx[cnt[a]] = d;
				fo.w[cnt[a]] = ex.w[k];
				cnt[a]++;
			}
		free(cnt);
	}
	if (take(&ex, &q->ex_src, &q->ex_w) || take(&fo, &q->fo_dof, &q->fo_w))
		goto out;
	ex.idx = NULL;
	ex.w = NULL;
	fo.idx = NULL;
	fo.w = NULL;
	q->n_ex = q->ex_off[nd];
	q->n_fo = q->fo_off[nd];
	rc = MCLG_OK;
out:
	free(hang_of);
	free(ex.idx);
	free(ex.w);
	free(fo.idx);
	free(fo.w);
	return rc;
}

/* P of level `lev` (rows: its reduced dofs; columns: reduced dofs of lev-1) */
static int build_prolongation(const mclg_mesh *m, int lev, const mclg_qt_level *lo, mclg_qt_level *up)
{
	const mclg_level *U = &m->lev[lev], *D = &m->lev[lev - 1];
	const int neq = U->neq, nd = 2 * U->nno;
	int *n = (int *)malloc((size_t)(neq > 0 ? neq : 1) * sizeof(int));
	int *src = (int *)malloc(4 * (size_t)(neq > 0 ? neq : 1) * sizeof(int));
	int *dof_lo = (int *)malloc((size_t)(D->neq > 0 ? D->neq : 1) * sizeof(int));
	csr_b p = {0};
	int rc = MCLG_BAD_INPUT, d, A, c;
	up->p_off = (int *)calloc((size_t)nd + 1, sizeof(int));
	if (!n || !src || !dof_lo || !up->p_off)
		goto out;
	if (mclg_refmg_interp(m, lev, n, src) != MCLG_OK)
		goto out;
	for (A = 0; A < D->nno; A++)
		for (c = 0; c < 2; c++) {
			const int eq = D->id[(size_t)c * D->nno + A];
			if (eq >= 0)
				dof_lo[eq] = 2 * A + c;
		}
	for (d = 0; d < nd; d++) {
		up->p_off[d] = (int)p.n;
		if (up->kind[d] != 1)
			continue;
		A = d >> 1;
		c = d & 1;
		const int eu = U->id[(size_t)c * U->nno + A];
		if (eu < 0 || n[eu] <= 0) {
			mclg_set_error("level %d: reduced dof %d has no interpolation from level %d", lev, d, lev - 1);
			goto out;
		}
		terms t;
		t.n = 0;
		for (int i = 0; i < n[eu]; i++) {
			const int el = src[(size_t)i * neq + eu];
			if (el < 0)
				continue;   /* a fixed coarse dof: 0, still counted in the mean (Solver.c:1036-1043) */
			const int dl = dof_lo[el];
			if (lo->kind[dl] == 1) {
				if (terms_add(&t, dl, 1.0 / n[eu]))
					goto out;
			} else if (lo->kind[dl] == 2) {
				for (int k = lo->ex_off[dl]; k < lo->ex_off[dl + 1]; k++)
					if (terms_add(&t, lo->ex_src[k], lo->ex_w[k] / n[eu]))
						goto out;
			}
		}
		terms_sort(&t);
		for (int i = 0; i < t.n; i++)
			if (csr_push(&p, t.dof[i], t.w[i]))
				goto out;
	}
	up->p_off[nd] = (int)p.n;
	up->n_p = (int)p.n;
	if (take(&p, &up->p_src, &up->p_w))
		goto out;
	p.idx = NULL;
	p.w = NULL;
	rc = MCLG_OK;
out:
	free(n);
	free(src);
	free(dof_lo);
	free(p.idx);
	free(p.w);
	return rc;
}

/* R of level lev-1 = P(lev)^T, rows by coarse dof, fine dofs ascending */
static int build_restriction(const mclg_qt_level *up, mclg_qt_level *lo)
{
	const int ndl = 2 * lo->nno, ndu = 2 * up->nno;
	int *cnt = (int *)calloc((size_t)ndl + 1, sizeof(int));
	lo->r_off = (int *)calloc((size_t)ndl + 1, sizeof(int));
	lo->r_src = (int *)malloc((size_t)(up->n_p + 1) * sizeof(int));
	lo->r_w = (double *)malloc((size_t)(up->n_p + 1) * sizeof(double));
	if (!cnt || !lo->r_off || !lo->r_src || !lo->r_w) {
		free(cnt);
		return MCLG_BAD_INPUT;
	}
	for (int k = 0; k < up->n_p; k++)
		cnt[up->p_src[k]]++;
	for (int d = 0; d < ndl; d++)
		lo->r_off[d + 1] = lo->r_off[d] + cnt[d];
	memcpy(cnt, lo->r_off, (size_t)ndl * sizeof(int));
	for (int u = 0; u < ndu; u++)
		for (int k = up->p_off[u]; k < up->p_off[u + 1]; k++) {
			const int a = up->p_src[k];
			lo->r_src[cnt[a]] = u;
			lo->r_w[cnt[a]] = up->p_w[k];
			cnt[a]++;
		}
	lo->n_r = up->n_p;
	free(cnt);
	return MCLG_OK;
}

/* The reduced operator C^T K C of a level as node-block ELL rows over reduced
 * columns, assembled on the device each step from K by a per-row list of
 * contributions: entry (slot s, component pair cc) of row A accumulates
 * w * K[k][j].cc for every row j holding A (A itself, weight 1, and the
 * constrained dofs folded into A) and every column of row j expanded into
 * reduced dofs. */
typedef struct {
	int B, tgt, src;
	double w;
} contrib;

static int cmp_contrib(const void *a, const void *b)
{
	const contrib *x = (const contrib *)a, *y = (const contrib *)b;
	if (x->tgt != y->tgt)
		return x->tgt < y->tgt ? -1 : 1;
	return x->src < y->src ? -1 : x->src > y->src;
}

/* One row of C^T K C: its contributions (tgt = 4*slot + cc, sorted by tgt, then
 * src) and its reduced columns (sorted).  row/rcap: a growable scratch list;
 * cols: room for 512 columns.  Returns 0, or -1 when out of memory or a row
 * has more than 512 columns. */
static int reduced_row(const mclg_level *L, const mclg_qt_level *q, int A, contrib **rowp, long *rcap, int *cols,
                       long *rn_out, int *ncols_out)
{
	const int nno = L->nno;
	contrib *row = *rowp;
	long rn = 0;
	int ncols = 0;
#define PUSH_CONTRIB(B_, tgt_, src_, w_)                                            \
	do {                                                                           \
		if (rn == *rcap) {                                                         \
			long cap_ = *rcap ? 2 * *rcap : 256;                                   \
			contrib *r2_ = (contrib *)realloc(row, (size_t)cap_ * sizeof(contrib)); \
			if (r2_ == NULL)                                                       \
				goto fail;                                                         \
			row = r2_;                                                             \
			*rowp = row;                                                           \
			*rcap = cap_;                                                          \
		}                                                                          \
		row[rn].B = (B_);                                                          \
		row[rn].tgt = (tgt_);                                                      \
		row[rn].src = (src_);                                                      \
		row[rn].w = (w_);                                                          \
		rn++;                                                                      \
	} while (0)
	/* the common row: nothing folded into it and no constrained column, so its
	 * reduced row is K's row, in K's (sorted) column order */
	int plain = q->fo_off[2 * A + 2] == q->fo_off[2 * A];
	for (int k = 0; plain && k < L->nb_cnt[A]; k++) {
		const int B = L->nb[(size_t)k * nno + A];
		plain = q->kind[2 * B] != 2 && q->kind[2 * B + 1] != 2;
	}
	if (plain) {
		for (int k = 0; k < L->nb_cnt[A]; k++) {
			const int B = L->nb[(size_t)k * nno + A];
			if (q->kind[2 * B] == 0 && q->kind[2 * B + 1] == 0)
				continue;
			for (int cc = 0; cc < 4; cc++) {
				const int c = cc >> 1, c2 = cc & 1;
				if (q->kind[2 * A + c] != 1 || q->kind[2 * B + c2] != 1)
					continue;
				PUSH_CONTRIB(B, 4 * ncols + cc, (int)(((size_t)k * nno + A) * 4 + (size_t)cc), 1.0);
			}
			if (ncols == 512)
				goto fail;
			cols[ncols++] = B;
		}
		*rn_out = rn;
		*ncols_out = ncols;
		return 0;
	}
	for (int c = 0; c < 2; c++) {
		const int da = 2 * A + c;
		if (q->kind[da] != 1)
			continue;
		/* rows holding dof (A,c): itself and the constrained dofs folded into it */
		for (int t = -1; t < q->fo_off[da + 1] - q->fo_off[da]; t++) {
			const int jd = t < 0 ? da : q->fo_dof[q->fo_off[da] + t];
			const double wj = t < 0 ? 1.0 : q->fo_w[q->fo_off[da] + t];
			const int j = jd >> 1;
			for (int k = 0; k < L->nb_cnt[j]; k++) {
				const int B = L->nb[(size_t)k * nno + j];
				for (int c2 = 0; c2 < 2; c2++) {
					const int db = 2 * B + c2;
					const int src = (int)(((size_t)k * nno + j) * 4 + (size_t)(c * 2 + c2));
					int ni = 1, first = 0;
					if (q->kind[db] == 0)
						continue;
					if (q->kind[db] == 2) {
						first = q->ex_off[db];
						ni = q->ex_off[db + 1] - first;
					}
					for (int i = 0; i < ni; i++) {
						const int Bp = q->kind[db] == 2 ? q->ex_src[first + i] >> 1 : B;
						const double wb = q->kind[db] == 2 ? q->ex_w[first + i] : 1.0;
						PUSH_CONTRIB(Bp, c * 2 + c2, src, wj * wb);   /* slot added below */
					}
				}
			}
		}
	}
#undef PUSH_CONTRIB
	/* the row's reduced columns, sorted */
	for (long i = 0; i < rn; i++) {
		int f = 0;
		for (int u = 0; u < ncols; u++)
			if (cols[u] == row[i].B) {
				f = 1;
				break;
			}
		if (!f) {
			if (ncols == 512)
				goto fail;
			cols[ncols++] = row[i].B;
		}
	}
	for (int u = 1; u < ncols; u++)
		for (int v = u; v > 0 && cols[v - 1] > cols[v]; v--) {
			int t = cols[v];
			cols[v] = cols[v - 1];
			cols[v - 1] = t;
		}
	for (long i = 0; i < rn; i++) {
		int slot = 0;
		while (cols[slot] != row[i].B)
			slot++;
		row[i].tgt += 4 * slot;
	}
	qsort(row, (size_t)rn, sizeof(contrib), cmp_contrib);
	*rn_out = rn;
	*ncols_out = ncols;
	return 0;
fail:
	return -1;
}

/* Rows [A0, A1) of a level, on a thread of their own.  Pass 0 builds each
 * row, counts its contributions and columns and keeps both in the chunk's
 * own lists; pass 1 copies them to the offsets the counts gave, into the
 * level's arrays (rows are independent, so the result does not depend on how
 * the rows are split). */
typedef struct {
	const mclg_level *L;
	mclg_qt_level *q;
	int A0, A1, pass, maxw, rc;
	int *cnt;           /* pass 0: [nno] contributions per row; rcnt holds the columns */
	int *ktgt, *ksrc;   /* the chunk's rows as pass 0 built them */
	double *kw;
	int *kcol;
	long kn, kcap, kc, kccap;
} ro_chunk;

static int keep_row(ro_chunk *o, const contrib *row, long rn, const int *cols, int ncols)
{
	if (o->kn + rn > o->kcap) {
		long cap = o->kcap ? 2 * o->kcap : 4096;
		while (cap < o->kn + rn)
			cap *= 2;
		int *t = (int *)realloc(o->ktgt, (size_t)cap * sizeof(int));
		if (t == NULL)
			return -1;
		o->ktgt = t;
		t = (int *)realloc(o->ksrc, (size_t)cap * sizeof(int));
		if (t == NULL)
			return -1;
		o->ksrc = t;
		double *w = (double *)realloc(o->kw, (size_t)cap * sizeof(double));
		if (w == NULL)
			return -1;
		o->kw = w;
		o->kcap = cap;
	}
	if (o->kc + ncols > o->kccap) {
		long cap = o->kccap ? 2 * o->kccap : 4096;
		while (cap < o->kc + ncols)
			cap *= 2;
		int *t = (int *)realloc(o->kcol, (size_t)cap * sizeof(int));
		if (t == NULL)
			return -1;
		o->kcol = t;
		o->kccap = cap;
	}
	for (long i = 0; i < rn; i++) {
		o->ktgt[o->kn + i] = row[i].tgt;
		o->ksrc[o->kn + i] = row[i].src;
		o->kw[o->kn + i] = row[i].w;
	}
	o->kn += rn;
	memcpy(o->kcol + o->kc, cols, (size_t)ncols * sizeof(int));
	o->kc += ncols;
	return 0;
}

static void *reduced_rows(void *arg)
{
	ro_chunk *o = (ro_chunk *)arg;
	const mclg_level *L = o->L;
	mclg_qt_level *q = o->q;
	const int nno = L->nno;
	o->rc = MCLG_BAD_INPUT;
	if (o->pass == 1) {
		long pk = 0, pc = 0;
		for (int A = o->A0; A < o->A1; A++) {
			const size_t at = (size_t)q->rc_off[A];
			const int rn = o->cnt[A], ncols = q->rcnt[A];
			memcpy(q->rc_tgt + at, o->ktgt + pk, (size_t)rn * sizeof(int));
			memcpy(q->rc_src + at, o->ksrc + pk, (size_t)rn * sizeof(int));
			memcpy(q->rc_w + at, o->kw + pk, (size_t)rn * sizeof(double));
			pk += rn;
			for (int u = 0; u < q->rnbw; u++)
				q->rnb[(size_t)u * nno + A] = u < ncols ? o->kcol[pc + u] : A;
			pc += ncols;
		}
		o->rc = MCLG_OK;
		return NULL;
	}
	contrib *row = NULL;
	long rn, rcap = 0;
	int *cols = (int *)malloc(512 * sizeof(int)), ncols;
	o->maxw = 1;
	o->ktgt = o->ksrc = o->kcol = NULL;
	o->kw = NULL;
	o->kn = o->kcap = o->kc = o->kccap = 0;
	if (cols == NULL)
		goto out;
	for (int A = o->A0; A < o->A1; A++) {
		if (reduced_row(L, q, A, &row, &rcap, cols, &rn, &ncols))
			goto out;
		o->cnt[A] = (int)rn;
		if (ncols > 255)
			goto out;
		q->rcnt[A] = (unsigned char)ncols;
		if (ncols > o->maxw)
			o->maxw = ncols;
		if (keep_row(o, row, rn, cols, ncols))
			goto out;
	}
	o->rc = MCLG_OK;
out:
	free(cols);
	free(row);
	return NULL;
}

static void chunk_free(ro_chunk *o)
{
	free(o->ktgt);
	free(o->ksrc);
	free(o->kw);
	free(o->kcol);
	o->ktgt = o->ksrc = o->kcol = NULL;
	o->kw = NULL;
}

static int build_reduced_operator(const mclg_level *L, mclg_qt_level *q)
{
	enum { kMaxChunks = 16 };
	const int nno = L->nno;
	/* rows in chunks of at least 8192 nodes, one thread each */
	int nch = nno / 8192;
	nch = nch < 1 ? 1 : nch > kMaxChunks ? kMaxChunks : nch;
	ro_chunk ch[kMaxChunks];
	pthread_t th[kMaxChunks];
	int started[kMaxChunks];
	int rc = MCLG_BAD_INPUT, maxw = 1;
	long tot = 0;
	int *cnt = (int *)malloc(((size_t)nno + 1) * sizeof(int));
	memset(ch, 0, sizeof ch);
	q->rc_off = (int *)malloc(((size_t)nno + 1) * sizeof(int));
	q->rcnt = (unsigned char *)malloc((size_t)nno + 1);
	if (!cnt || !q->rc_off || !q->rcnt)
		goto out;
	for (int pass = 0; pass < 2; pass++) {
		for (int i = 0; i < nch; i++) {
			ch[i].L = L;
			ch[i].q = q;
			ch[i].A0 = (int)((long)nno * i / nch);
			ch[i].A1 = (int)((long)nno * (i + 1) / nch);
			ch[i].pass = pass;
			ch[i].cnt = cnt;
			started[i] = nch > 1 && pthread_create(&th[i], NULL, reduced_rows, &ch[i]) == 0;
			if (!started[i])
				reduced_rows(&ch[i]);
		}
		for (int i = 0; i < nch; i++)
			if (started[i])
				pthread_join(th[i], NULL);
		for (int i = 0; i < nch; i++)
			if (ch[i].rc != MCLG_OK)
				goto out;
		if (pass == 1)
			break;
		for (int i = 0; i < nch; i++)
			if (ch[i].maxw > maxw)
				maxw = ch[i].maxw;
		for (int A = 0; A < nno; A++) {
			q->rc_off[A] = (int)tot;
			tot += cnt[A];
		}
		q->rc_off[nno] = (int)tot;
		q->rnbw = maxw;
		q->rc_tgt = (int *)malloc((size_t)(tot > 0 ? tot : 1) * sizeof(int));
		q->rc_src = (int *)malloc((size_t)(tot > 0 ? tot : 1) * sizeof(int));
		q->rc_w = (double *)malloc((size_t)(tot > 0 ? tot : 1) * sizeof(double));
		q->rnb = (int *)malloc((size_t)maxw * nno * sizeof(int));
		if (!q->rc_tgt || !q->rc_src || !q->rc_w || !q->rnb)
			goto out;
	}
	q->n_rc = (int)tot;
	rc = MCLG_OK;
out:
	if (rc != MCLG_OK)
		mclg_set_error("refined-mesh operator of a %d-node level: a row with more than 255 reduced "
		               "columns, or out of host memory", nno);
	for (int i = 0; i < nch; i++)
		chunk_free(&ch[i]);
	free(cnt);
	return rc;
}

/* one level's lists, run on a thread of its own: phase 0 the constraint lists,
 * C^T K C and the node map; phase 1 the transfers to the level below */
typedef struct {
	const mclg_mesh *m;
	mclg_qt_level *q;   /* q[0] is level lo */
	int lo, lev, phase, rc;
	char err[512];
} qt_job;

static void *qt_worker(void *p)
{
	qt_job *j = (qt_job *)p;
	const mclg_mesh *m = j->m;
	const int lev = j->lev, top = m->max_level - 1;
	mclg_qt_level *Q = &j->q[lev - j->lo];
	j->rc = MCLG_OK;
	if (j->phase == 0) {
		memset(Q, 0, sizeof *Q);
		if ((j->rc = build_constraints(&m->lev[lev], Q)) == MCLG_OK)
			j->rc = build_reduced_operator(&m->lev[lev], Q);
		/* node_map: this level's node -> the same node one level up (every node of a
		 * level exists on the finer levels) */
		if (j->rc == MCLG_OK && lev < top) {
			const mclg_level *L = &m->lev[lev], *U = &m->lev[lev + 1];
			Q->node_map = (int *)malloc((size_t)L->nno * sizeof(int));
			if (Q->node_map == NULL)
				j->rc = MCLG_BAD_INPUT;
			for (int A = 0; Q->node_map && A < L->nno; A++) {
				Q->node_map[A] = mclg_node_index(U, L->node[A]);
				if (Q->node_map[A] < 0) {
					mclg_set_error("level %d: node %d is missing on level %d", lev, L->node[A], lev + 1);
					j->rc = MCLG_BAD_INPUT;
					break;
				}
			}
		}
	} else if (lev > j->lo) {
		if ((j->rc = build_prolongation(m, lev, &j->q[lev - j->lo - 1], Q)) == MCLG_OK)
			j->rc = build_restriction(Q, &j->q[lev - j->lo - 1]);
	}
	if (j->rc != MCLG_OK)
		snprintf(j->err, sizeof j->err, "%s", mclg_last_error());
	return NULL;
}

int mclg_qt_build(const mclg_mesh *m, int lo, mclg_qt_level *q)
{
	const int top = m->max_level - 1;
	qt_job jobs[MCLG_MAX_LEVEL];
	pthread_t th[MCLG_MAX_LEVEL];
	int started[MCLG_MAX_LEVEL];
	if (lo < m->min_level || lo >= top)
		return MCLG_BAD_INPUT;
	const int nl = top - lo + 1;
	for (int phase = 0; phase < 2; phase++) {
		for (int i = 0; i < nl; i++) {
			jobs[i].m = m;
			jobs[i].q = q;
			jobs[i].lo = lo;
			jobs[i].lev = lo + i;
			jobs[i].phase = phase;
			jobs[i].err[0] = 0;
			started[i] = pthread_create(&th[i], NULL, qt_worker, &jobs[i]) == 0;
			if (!started[i])
				qt_worker(&jobs[i]);
		}
		for (int i = 0; i < nl; i++)
			if (started[i])
				pthread_join(th[i], NULL);
		for (int i = 0; i < nl; i++)
			if (jobs[i].rc != MCLG_OK) {
				mclg_set_error("%s", jobs[i].err);
				return jobs[i].rc;
			}
	}
	return MCLG_OK;
}
