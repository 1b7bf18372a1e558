/*
 * Host-only C ABI over the mesh builder: lets a caller (or a test on a
 * machine without a GPU) read the numbering that the device path uses.
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include "mclg_host.h"

struct mclg_mesh_handle {
	mclg_mesh mesh;
	mclg_config cfg;
	mclg_qt_level qt[MCLG_MAX_LEVEL];   /* the refined-mesh solver's lists, built on first use */
	int qt_lo, qt_n;
};

static int mesh_new(mclg_mesh_handle **h, const mclg_config *cfg, const int *leaves, long n)
{
	int rc;
	mclg_mesh_handle *p;
	if (h == NULL || cfg == NULL)
		return MCLG_BAD_INPUT;
	*h = NULL;
	p = (mclg_mesh_handle *)calloc(1, sizeof *p);
	if (p == NULL)
		return MCLG_BAD_INPUT;
	p->cfg = *cfg;
	rc = leaves ? mclg_mesh_build_leaves(&p->mesh, cfg, leaves, n) : mclg_mesh_build(&p->mesh, cfg);
	if (rc != MCLG_OK) {
		mclg_mesh_free(&p->mesh);
		free(p);
		return rc;
	}
	*h = p;
	return MCLG_OK;
}

int mclg_mesh_new(mclg_mesh_handle **h, const mclg_config *cfg)
{
	return mesh_new(h, cfg, NULL, 0);
}

int mclg_mesh_new_leaves(mclg_mesh_handle **h, const mclg_config *cfg, const int *leaves, size_t n)
{
	if (leaves == NULL)
		return MCLG_BAD_INPUT;
	return mesh_new(h, cfg, leaves, (long)n);
}

int mclg_mesh_new_leaves_device(mclg_mesh_handle **h, const mclg_config *cfg, const int *leaves, size_t n)
{
	int rc;
	mclg_mesh_handle *p;
	if (h == NULL || cfg == NULL || leaves == NULL)
		return MCLG_BAD_INPUT;
	*h = NULL;
	p = (mclg_mesh_handle *)calloc(1, sizeof *p);
	if (p == NULL)
		return MCLG_BAD_INPUT;
	p->cfg = *cfg;
	rc = mclg_mesh_build_leaves_device(&p->mesh, cfg, leaves, (long)n, NULL);
	if (rc != MCLG_OK) {
		free(p);
		return rc;
	}
	*h = p;
	return MCLG_OK;
}

/* every array of every level, byte for byte (the lengths the builder fills) */
int mclg_mesh_diff(const mclg_mesh_handle *ha, const mclg_mesh_handle *hb, char *what, size_t cap)
{
	const mclg_mesh *a, *b;
	int lev;
	char buf[128];
	if (ha == NULL || hb == NULL)
		return MCLG_BAD_INPUT;
	a = &ha->mesh;
	b = &hb->mesh;
	buf[0] = 0;
	if (a->min_level != b->min_level || a->max_level != b->max_level || a->gnox != b->gnox ||
	    a->gnoz != b->gnoz || a->uniform != b->uniform)
		snprintf(buf, sizeof buf, "mesh frame");
	for (lev = a->min_level; lev < a->max_level && buf[0] == 0; lev++) {
		const mclg_level *A = &a->lev[lev], *B = &b->lev[lev];
		const size_t ne = (size_t)A->nel, nn = (size_t)A->nno, nh = (size_t)A->nh;
		const int fine = lev == a->max_level - 1;
		struct {
			const char *name;
			const void *x, *y;
			size_t bytes;
		} arr[] = {
			{"Mcode", A->Mcode, B->Mcode, ne * sizeof(int)},
			{"node", A->node, B->node, nn * sizeof(int)},
			{"node_lut", A->node_lut, B->node_lut, (size_t)A->lut_n * sizeof(int)},
			{"ien", A->ien, B->ien, 4 * ne * sizeof(int)},
			{"ienl", A->ienl, B->ienl, 4 * ne * sizeof(int)},
			{"elev", A->elev, B->elev, ne * sizeof(int)},
			{"id", A->id, B->id, 2 * nn * sizeof(int)},
			{"heat_id", A->heat_id, B->heat_id, nn * sizeof(int)},
			{"v_bc", A->v_bc, B->v_bc, 2 * nn},
			{"v_bc_val", A->v_bc_val, B->v_bc_val, 2 * nn * sizeof(double)},
			{"T_bc", A->T_bc, B->T_bc, nn},
			{"T_bc_val", A->T_bc_val, B->T_bc_val, nn * sizeof(double)},
			{"X", A->X, B->X, 2 * nn * sizeof(double)},
			{"dx_dxi", A->dx_dxi, B->dx_dxi, ne * sizeof(double)},
			{"dz_deta", A->dz_deta, B->dz_deta, ne * sizeof(double)},
			{"jacobi", A->jacobi, B->jacobi, ne * sizeof(double)},
			{"area", A->area, B->area, ne * sizeof(double)},
			{"hang_node", A->hang_node, B->hang_node, nh * sizeof(int)},
			{"hang_c0", A->hang_c0, B->hang_c0, nh * sizeof(int)},
			{"hang_c1", A->hang_c1, B->hang_c1, nh * sizeof(int)},
			{"hang_ni", A->hang_ni, B->hang_ni, nh * sizeof(int)},
			{"hang_ci0", A->hang_ci0, B->hang_ci0, nh * sizeof(int)},
			{"hang_ci1", A->hang_ci1, B->hang_ci1, nh * sizeof(int)},
			{"p2n_cnt", A->p2n_cnt, B->p2n_cnt, nn * sizeof(int)},
			{"p2n_el", A->p2n_el, B->p2n_el, 4 * nn * sizeof(int)},
			{"p2n_a", A->p2n_a, B->p2n_a, 4 * nn * sizeof(int)},
			{"nb", A->nb, B->nb, (size_t)A->nbw * nn * sizeof(int)},
			{"nb_cnt", A->nb_cnt, B->nb_cnt, nn * sizeof(int)},
			{"kslot", A->kslot, B->kslot, 16 * ne},
			{"cell_elem", fine ? A->cell_elem : NULL, fine ? B->cell_elem : NULL,
			 fine ? (size_t)(a->gnox - 1) * (size_t)(a->gnoz - 1) * sizeof(int) : 0},
		};
		size_t k;
		if (A->nel != B->nel || A->nno != B->nno || A->neq != B->neq || A->heat_neq != B->heat_neq ||
		    A->nh != B->nh || A->hang_chained != B->hang_chained || A->nbw != B->nbw || A->lut_n != B->lut_n) {
			snprintf(buf, sizeof buf, "level %d sizes", lev);
			break;
		}
		for (k = 0; k < sizeof arr / sizeof arr[0]; k++) {
			if (arr[k].bytes == 0)
				continue;
			if ((arr[k].x == NULL) != (arr[k].y == NULL) ||
			    (arr[k].x != NULL && memcmp(arr[k].x, arr[k].y, arr[k].bytes) != 0)) {
				snprintf(buf, sizeof buf, "level %d %s", lev, arr[k].name);
				break;
			}
		}
	}
	if (what != NULL && cap > 0)
		snprintf(what, cap, "%s", buf);
	return buf[0] == 0 ? 0 : 1;
}

void mclg_mesh_delete(mclg_mesh_handle *h)
{
	if (h == NULL)
		return;
	for (int k = 0; k < h->qt_n; k++)
		mclg_qt_free(&h->qt[k]);
	mclg_mesh_free(&h->mesh);
	free(h);
}

int mclg_mesh_qt_get(mclg_mesh_handle *h, int lev, int which, void *out, size_t n)
{
	const mclg_qt_level *q;
	size_t need;
	int top, k;
	if (h == NULL || out == NULL)
		return MCLG_BAD_INPUT;
	top = h->mesh.max_level - 1;
	if (h->qt_n == 0) {
		const int lo = h->mesh.min_level;
		int rc;
		if (lo >= top) {
			mclg_set_error("the refined-mesh lists need at least two levels (levels %d..%d)", lo, top);
			return MCLG_BAD_INPUT;
		}
		rc = mclg_qt_build(&h->mesh, lo, h->qt);
		if (rc != MCLG_OK) {
			for (k = 0; k <= top - lo; k++)
				mclg_qt_free(&h->qt[k]);
			return rc;
		}
		h->qt_lo = lo;
		h->qt_n = top - lo + 1;
	}
	if (lev < 0)
		lev = top;
	if (lev < h->qt_lo || lev > top) {
		mclg_set_error("level %d has no refined-mesh lists (levels %d..%d)", lev, h->qt_lo, top);
		return MCLG_BAD_INPUT;
	}
	q = &h->qt[lev - h->qt_lo];
	switch (which) {
	case MCLG_QT_SIZES: need = 4; break;
	case MCLG_QT_KIND: need = 2 * (size_t)q->nno; break;
	case MCLG_QT_RC_OFF: need = (size_t)q->nno + 1; break;
	case MCLG_QT_RC_TGT:
	case MCLG_QT_RC_SRC:
	case MCLG_QT_RC_W: need = (size_t)q->n_rc; break;
	case MCLG_QT_RNB: need = (size_t)q->rnbw * q->nno; break;
	case MCLG_QT_RCNT: need = (size_t)q->nno; break;
	default:
		mclg_set_error("unknown refined-mesh list %d", which);
		return MCLG_BAD_INPUT;
	}
	if (n != need) {
		mclg_set_error("refined-mesh list %d has %zu entries, buffer has %zu", which, need, n);
		return MCLG_BAD_INPUT;
	}
	switch (which) {
	case MCLG_QT_SIZES: {
		int *o = (int *)out;
		o[0] = q->nno; o[1] = q->rnbw; o[2] = q->n_rc; o[3] = q->n_ex;
		break;
	}
	case MCLG_QT_KIND:
		for (size_t i = 0; i < need; i++)
			((int *)out)[i] = q->kind[i];
		break;
	case MCLG_QT_RC_OFF: memcpy(out, q->rc_off, need * sizeof(int)); break;
	case MCLG_QT_RC_TGT: memcpy(out, q->rc_tgt, need * sizeof(int)); break;
	case MCLG_QT_RC_SRC: memcpy(out, q->rc_src, need * sizeof(int)); break;
	case MCLG_QT_RC_W: memcpy(out, q->rc_w, need * sizeof(double)); break;
	case MCLG_QT_RNB: memcpy(out, q->rnb, need * sizeof(int)); break;
	case MCLG_QT_RCNT:
		for (size_t i = 0; i < need; i++)
			((int *)out)[i] = q->rcnt[i];
		break;
	}
	return MCLG_OK;
}

static const mclg_level *pick_level(const mclg_mesh *m, int lev)
{
	if (lev < 0)
		lev = m->max_level - 1;
	if (lev < m->min_level || lev >= m->max_level)
		return NULL;
	return &m->lev[lev];
}

/* shared by mclg_mesh_get and mclg_get_mesh */
int mclg_host_mesh_get(const mclg_mesh *m, int which, int lev, int *out, size_t n)
{
	const mclg_level *L = pick_level(m, lev);
	size_t ne, nn, i, need;
	if (L == NULL || out == NULL) {
		mclg_set_error("level %d is not a level of this mesh", lev);
		return MCLG_BAD_INPUT;
	}
	ne = (size_t)L->nel;
	nn = (size_t)L->nno;
	switch (which) {
	case MCLG_M_SIZES: need = 8; break;
	case MCLG_M_MCODE: need = ne; break;
	case MCLG_M_NODE: need = nn; break;
	case MCLG_M_IEN: need = 4 * ne; break;
	case MCLG_M_ID: need = 2 * nn; break;
	case MCLG_M_HEAT_ID: need = nn; break;
	case MCLG_M_LM: need = 8 * ne; break;
	case MCLG_M_HANG: need = 3 * (size_t)L->nh; break;
	case MCLG_M_VBC: need = 2 * nn; break;
	case MCLG_M_TBC: need = nn; break;
	case MCLG_M_INTERP: need = 5 * (size_t)L->neq; break;
	case MCLG_M_PROJECT: need = (size_t)L->neq; break;
	case MCLG_M_GS_WAVE: need = nn; break;
	case MCLG_M_NB: need = (size_t)MCLG_NB_MAX * nn; break;
	case MCLG_M_KSLOT: need = 16 * ne; break;
	default:
		mclg_set_error("unknown mesh array %d", which);
		return MCLG_BAD_INPUT;
	}
	if (n != need) {
		mclg_set_error("mesh array %d has %zu entries, buffer has %zu", which, need, n);
		return MCLG_BAD_INPUT;
	}
	switch (which) {
	case MCLG_M_SIZES:
		out[0] = L->nel; out[1] = L->nno; out[2] = L->neq; out[3] = L->heat_neq;
		out[4] = L->nh; out[5] = m->gnox; out[6] = m->gnoz; out[7] = m->max_level;
		break;
	case MCLG_M_MCODE: memcpy(out, L->Mcode, ne * sizeof(int)); break;
	case MCLG_M_NODE: memcpy(out, L->node, nn * sizeof(int)); break;
	case MCLG_M_IEN: memcpy(out, L->ien, 4 * ne * sizeof(int)); break;
	case MCLG_M_ID: memcpy(out, L->id, 2 * nn * sizeof(int)); break;
	case MCLG_M_HEAT_ID: memcpy(out, L->heat_id, nn * sizeof(int)); break;
	case MCLG_M_LM: {
		size_t d, a, e;
		for (d = 0; d < 2; d++)
			for (a = 0; a < 4; a++)
				for (e = 0; e < ne; e++)
					out[(d * 4 + a) * ne + e] = L->id[d * nn + (size_t)L->ienl[a * ne + e]];
		break;
	}
	case MCLG_M_HANG:
		for (i = 0; i < (size_t)L->nh; i++) {
			out[i] = L->hang_node[i];
			out[L->nh + i] = L->hang_c0[i];
			out[2 * (size_t)L->nh + i] = L->hang_c1[i];
		}
		break;
	case MCLG_M_VBC:
		for (i = 0; i < 2 * nn; i++)
			out[i] = (unsigned char)L->v_bc[i];
		break;
	case MCLG_M_TBC:
		for (i = 0; i < nn; i++)
			out[i] = (unsigned char)L->T_bc[i];
		break;
	case MCLG_M_INTERP:
	case MCLG_M_PROJECT: {
		const int lv = (int)(L - m->lev);
		const int rc = which == MCLG_M_INTERP ? mclg_refmg_interp(m, lv, out, out + L->neq)
		                                      : mclg_refmg_project(m, lv, out);
		if (rc != MCLG_OK) {
			mclg_set_error("level %d has no %s map (levels %d..%d)", lv,
			               which == MCLG_M_INTERP ? "interpolation" : "projection", m->min_level,
			               m->max_level - 1);
			return rc;
		}
		break;
	}
	case MCLG_M_GS_WAVE: mclg_refmg_waves(L, out); break;
	case MCLG_M_NB:
		for (i = 0; i < nn; i++)
			for (size_t j = 0; j < MCLG_NB_MAX; j++)
				out[i * MCLG_NB_MAX + j] = (int)j < L->nb_cnt[i] ? L->nb[j * nn + i] : -1;
		break;
	case MCLG_M_KSLOT:
		for (i = 0; i < 16 * ne; i++)
			out[i] = L->kslot[i];
		break;
	}
	return MCLG_OK;
}

int mclg_mesh_get(const mclg_mesh_handle *h, int which, int lev, int *out, size_t n)
{
	if (h == NULL)
		return MCLG_BAD_INPUT;
	return mclg_host_mesh_get(&h->mesh, which, lev, out, n);
}

int mclg_mesh_get_real(const mclg_mesh_handle *h, int which, int lev, double *out, size_t n)
{
	const mclg_level *L;
	size_t need, ne, nn;
	if (h == NULL || out == NULL)
		return MCLG_BAD_INPUT;
	L = pick_level(&h->mesh, lev);
	if (L == NULL) {
		mclg_set_error("level %d is not a level of this mesh", lev);
		return MCLG_BAD_INPUT;
	}
	ne = (size_t)L->nel;
	nn = (size_t)L->nno;
	switch (which) {
	case MCLG_R_X: need = 2 * nn; break;
	case MCLG_R_JACOBI: need = ne; break;
	case MCLG_R_AREA: need = ne; break;
	case MCLG_R_VBCVAL: need = 2 * nn; break;
	case MCLG_R_TBCVAL: need = nn; break;
	default:
		mclg_set_error("unknown mesh array %d", which);
		return MCLG_BAD_INPUT;
	}
	if (n != need) {
		mclg_set_error("mesh array %d has %zu entries, buffer has %zu", which, need, n);
		return MCLG_BAD_INPUT;
	}
	switch (which) {
	case MCLG_R_X: memcpy(out, L->X, need * sizeof(double)); break;
	case MCLG_R_JACOBI: memcpy(out, L->jacobi, need * sizeof(double)); break;
	case MCLG_R_AREA: memcpy(out, L->area, need * sizeof(double)); break;
	case MCLG_R_VBCVAL: memcpy(out, L->v_bc_val, need * sizeof(double)); break;
	case MCLG_R_TBCVAL: memcpy(out, L->T_bc_val, need * sizeof(double)); break;
	}
	return MCLG_OK;
}

int mclg_mesh_initial_temperature(const mclg_mesh_handle *h, int lev, double *T, size_t n)
{
	const mclg_level *L;
	if (h == NULL || T == NULL)
		return MCLG_BAD_INPUT;
	if (lev < 0)
		lev = h->mesh.max_level - 1;
	L = pick_level(&h->mesh, lev);
	if (L == NULL || n != (size_t)L->nno) {
		mclg_set_error("bad level or buffer size");
		return MCLG_BAD_INPUT;
	}
	return mclg_host_initial_temperature(&h->mesh, &h->cfg, lev, T);
}

int mclg_mesh_write_output(const mclg_mesh_handle *h, const char *data_dir, int timestep,
                           const double *T, const double *V0, const double *V1,
                           const double *stress, const double *vis, size_t n)
{
	const mclg_level *L;
	if (h == NULL || T == NULL || V0 == NULL || V1 == NULL || stress == NULL || vis == NULL)
		return MCLG_BAD_INPUT;
	L = &h->mesh.lev[h->mesh.max_level - 1];
	if (n != (size_t)L->nno) {
		mclg_set_error("output fields have %zu entries, the finest level has %d nodes", n, L->nno);
		return MCLG_BAD_INPUT;
	}
	return mclg_write_output(data_dir ? data_dir : h->cfg.data_dir, timestep, L, T, V0, V1, stress, vis);
}

int mclg_mesh_amr_leaves(const mclg_mesh_handle *h, const unsigned char *flags, size_t nflags, int base_level,
                         int target_level, int *leaves, size_t cap, size_t *n)
{
	int *tmp = NULL;
	long cnt = 0;
	int rc;
	if (h == NULL || flags == NULL || leaves == NULL || n == NULL)
		return MCLG_BAD_INPUT;
	if (nflags != (size_t)h->mesh.lev[h->mesh.max_level - 1].nel) {
		mclg_set_error("flag buffer has %zu entries, the mesh %d elements", nflags,
		               h->mesh.lev[h->mesh.max_level - 1].nel);
		return MCLG_BAD_INPUT;
	}
	rc = mclg_amr_build_leaves(&h->mesh, flags, base_level, target_level, &tmp, &cnt);
	if (rc)
		return rc;
	*n = (size_t)cnt;
	if ((size_t)cnt > cap) {
		free(tmp);
		mclg_set_error("the refined tree has %ld leaves, the buffer holds %zu", cnt, cap);
		return MCLG_BAD_INPUT;
	}
	memcpy(leaves, tmp, (size_t)cnt * sizeof(int));
	free(tmp);
	return MCLG_OK;
}

int mclg_mesh_transfer_elem(const mclg_mesh_handle *from, const double *P_from, size_t n_from,
                            const mclg_mesh_handle *to, double *P_to, size_t n_to)
{
	if (from == NULL || to == NULL || P_from == NULL || P_to == NULL)
		return MCLG_BAD_INPUT;
	if (n_from != (size_t)from->mesh.lev[from->mesh.max_level - 1].nel ||
	    n_to != (size_t)to->mesh.lev[to->mesh.max_level - 1].nel) {
		mclg_set_error("field buffers do not match the meshes' element counts");
		return MCLG_BAD_INPUT;
	}
	return mclg_amr_transfer_elem(&from->mesh, P_from, &to->mesh, P_to);
}

int mclg_mesh_transfer(const mclg_mesh_handle *from, const double *T_from, size_t n_from,
                       const mclg_mesh_handle *to, double *T_to, size_t n_to)
{
	if (from == NULL || to == NULL || T_from == NULL || T_to == NULL)
		return MCLG_BAD_INPUT;
	if (n_from != (size_t)from->mesh.lev[from->mesh.max_level - 1].nno ||
	    n_to != (size_t)to->mesh.lev[to->mesh.max_level - 1].nno) {
		mclg_set_error("field buffers do not match the meshes' node counts");
		return MCLG_BAD_INPUT;
	}
	return mclg_amr_transfer(&from->mesh, T_from, &to->mesh, T_to);
}
