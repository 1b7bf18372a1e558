/*
 * Host-side mesh, numbering and I/O of the GB300 engine (C, no CUDA).
 *
 * One mclg_mesh holds what the reference keeps per MG level in its global G
 * (global_variables.h:315-422) for a single rank: Morton leaf codes, the
 * sorted node list, ien/id/lm numbering, boundary codes, hanging-node
 * constraints, element geometry and the node->element map.  Everything here
 * is built once per mesh on the host and then uploaded to the device.
 */
#ifndef MCLG_HOST_H
#define MCLG_HOST_H

#include "mclg.h"

#ifdef __cplusplus
extern "C" {
#endif

#define MCLG_LEVEL_BITS 4
#define MCLG_NB_MAX 25     /* max distinct neighbour nodes of a node (2:1 meshes need <= 21) */

typedef struct mclg_level {
	int nel, nno;
	int *Mcode;            /* [nel]  (morton << 4) | element level             Tree.c:340-358 */
	int *node;             /* [nno]  sorted global node ids                    Construct_ien_id_lm.c:43-66 */
	int *node_lut;         /* [lut_n] global id -> index or -1 (grids of up to 4M ids; else NULL) */
	long lut_n;
	int *ien;              /* [4*nel] global node ids, ien[a*nel + e]          Construct_ien_id_lm.c:3-41 */
	int *ienl;             /* [4*nel] local node indices (node_index(ien))     */
	int *elev;             /* [nel]  element level (Mcode_lev)                 */
	int *id;               /* [2*nno] velocity equation or -1, id[d*nno + A]   Construct_ien_id_lm.c:79-115 */
	int neq;
	int *heat_id;          /* [nno]  temperature equation or -1                Construct_ien_id_lm.c:117-144 */
	int heat_neq;
	char *v_bc;            /* [2*nno] velocity BC codes                        Boundary_condition.c:58-110 */
	double *v_bc_val;      /* [2*nno] */
	char *T_bc;            /* [nno]                                            Boundary_condition.c:10-56 */
	double *T_bc_val;      /* [nno] */
	double *X;             /* [2*nno] node coordinates, X[d*nno + A]           Mesh.c:430-452 */
	double *dx_dxi, *dz_deta, *jacobi, *area;  /* [nel] Shape_function.c:123-167, Construct_ien_id_lm.c:198-218 */
	int nh;                /* hanging nodes                                     Connection.c:59-276 */
	int *hang_node, *hang_c0, *hang_c1;   /* global ids */
	int *hang_ni, *hang_ci0, *hang_ci1;   /* local indices */
	int hang_chained;      /* 1 when a parent of some hanging node is itself hanging */
	int *p2n_cnt;          /* [nno] number of elements touching a node          Construct_ien_id_lm.c:220-244 */
	int *p2n_el;           /* [4*nno] element ids in ascending order, p2n_el[k*nno + A] */
	int *p2n_a;            /* [4*nno] local corner index of the node in that element */
	int nbw;               /* neighbour-list width (max over nodes) */
	int *nb;               /* [nbw*nno] sorted neighbour nodes, nb[k*nno + A], padded with A */
	int *nb_cnt;           /* [nno] */
	unsigned char *kslot;  /* [16*nel] slot of corner b in the neighbour list of corner a, kslot[(a*4+b)*nel + e] */
	int *cell_elem;        /* [(gnox-1)*(gnoz-1)] element covering fine cell (ix,iz), cell_elem[ix*(gnoz-1)+iz] */
} mclg_level;

typedef struct mclg_mesh {
	int min_level, max_level;   /* MG levels [min_level, max_level) */
	int gnox, gnoz;
	int max_elx[MCLG_MAX_LEVEL], max_nel[MCLG_MAX_LEVEL];
	double dx[MCLG_MAX_LEVEL], dz[MCLG_MAX_LEVEL];
	double length, height;
	int uniform;                /* finest level is a uniform grid (no hanging nodes) */
	mclg_level lev[MCLG_MAX_LEVEL];
} mclg_mesh;

/* Build the mesh the way Main.c:33-52 does on its first step, for one rank. */
int mclg_mesh_build(mclg_mesh *m, const mclg_config *cfg);
/* The same mesh stack from a given leaf set (finest-level Morton start codes). */
int mclg_mesh_build_leaves(mclg_mesh *m, const mclg_config *cfg, const int *leaves, long n);
/* The level-independent part (Mesh.c:396-428, one rank) and the configuration
 * checks; clears m first. */
int mclg_mesh_frame(mclg_mesh *m, const mclg_config *cfg);
/* A leaf list: at least 2 strictly increasing codes within the finest level. */
int mclg_mesh_check_leaves(const mclg_mesh *m, const int *leaves, long n);
/* The same mesh stack as mclg_mesh_build_leaves, numbered on the current CUDA
 * device (k_mesh.cu) and copied into host arrays that are equal byte for byte;
 * st is the stream the device work runs on (0: a stream of its own). */
int mclg_mesh_build_leaves_device(mclg_mesh *m, const mclg_config *cfg, const int *leaves, long n, void *st);
/* |grad T| refinement (mclg_amr.c): leaves of a new tree from per-element flags
 * of the finest level of m; *leaves is malloc'ed. */
int mclg_amr_build_leaves(const mclg_mesh *m, const unsigned char *flags, int base_level, int target_level,
                          int **leaves, long *n);
int mclg_amr_transfer(const mclg_mesh *from, const double *T_from, const mclg_mesh *to, double *T_to);
int mclg_amr_transfer_elem(const mclg_mesh *from, const double *P_from, const mclg_mesh *to, double *P_to);
/* fn(ctx, i0, i1) over [0, n) in chunks of at least `grain` items on up to 8
 * threads; for loops whose items write only their own results */
void mclg_parallel_for(long n, long grain, void (*fn)(void *, long, long), void *ctx);
void mclg_mesh_free(mclg_mesh *m);
/* The reference's multigrid maps and the Gauss-Seidel wavefronts (mclg_refmg.c).
 * interp: lev in (min_level, max_level); n[neq(lev)], src[4*neq(lev)] (src[i*neq + u]).
 * project: lev in [min_level, max_level-1); up_eq[neq(lev)].  waves: wave[nno]. */
int mclg_refmg_interp(const mclg_mesh *m, int lev, int *n, int *src);
int mclg_refmg_project(const mclg_mesh *m, int lev, int *up_eq);
int mclg_refmg_waves(const mclg_level *L, int *wave);
/* Constrained-space structure of one level for the converged solver on
 * quadtree meshes (mclg_qtmg.c).  Dofs are 2*node + component. */
typedef struct mclg_qt_level {
	int nno;
	unsigned char *kind;              /* [2*nno] 0 fixed, 1 reduced, 2 constrained */
	int *ex_off, *ex_src;             /* expand: constrained dof = sum ex_w * x[ex_src] */
	double *ex_w;
	int *fo_off, *fo_dof;             /* fold: reduced dof <- constrained dofs holding it */
	double *fo_w;
	int *p_off, *p_src;               /* prolongation from the level below (rows: this level's dofs) */
	double *p_w;
	int *r_off, *r_src;               /* restriction from the level above (rows: this level's dofs) */
	double *r_w;
	int *node_map;                    /* [nno] the same node on the level above (NULL on the finest) */
	int rnbw;                         /* C^T K C as node-block ELL over reduced columns: width, */
	int *rnb;                         /* [rnbw*nno] columns (padded with the row node), */
	unsigned char *rcnt;              /* [nno] columns per row, */
	int *rc_off, *rc_tgt, *rc_src;    /* per row: entry (4*slot + 2c + c') += rc_w * K[rc_src] (K as */
	double *rc_w;                     /* flat doubles, 4 per block) */
	int n_ex, n_fo, n_p, n_r, n_rc;
} mclg_qt_level;
/* levels lo..max_level-1 into q[0..]; lo > min_level-1 and below the finest */
int mclg_qt_build(const mclg_mesh *m, int lo, mclg_qt_level *q);
void mclg_qt_free(mclg_qt_level *q);
/* Binary search in the sorted node list (node_index, Array_work.c:106-129). */
int mclg_node_index(const mclg_level *L, int gid);

/* Initial temperature on one level (Initial_condition.c:3-136, plus T_ini=-2). */
int mclg_host_initial_temperature(const mclg_mesh *m, const mclg_config *cfg, int lev, double *T);

/* the step's directory, and one of the five files of mclg_write_output (0 coord, 1 temperature,
 * 2 stress, 3 viscosity, 4 velocity) */
int mclg_output_dirs(const char *data_dir, int timestep);
int mclg_write_output_file(const char *data_dir, int timestep, int which, const mclg_level *L,
                           const double *T, const double *V0, const double *V1, const double *stress,
                           const double *vis);
/* Output.c:31-156 text files for one step. */
int mclg_write_output(const char *data_dir, int timestep, const mclg_level *L,
                      const double *T, const double *V0, const double *V1,
                      const double *stress, const double *vis);

void mclg_set_error(const char *fmt, ...);

#ifdef __cplusplus
}
#endif
#endif
