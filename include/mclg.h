/*
 * mclg.h -- C ABI of the GB300 time-step engine for the 2-D mantle-convection
 * code (reference: mingming-li/Mantle_Convection_Lab).
 *
 * The reference has no plugin registry or FFI: its "operator API" is the fixed
 * call sequence of Main.c:58-64 over one global struct G
 * (global_variables.h:315-422):
 *     buoyancy_force(); viscosity(); velocity_pressure_KGF_matrix();
 *     solve_velocity_pressure(); output(); update_temperature();
 * This header exports the same sequence as plain C functions over an opaque
 * context that owns the device-resident mesh and fields.  Every function
 * returns an int status (MCLG_OK == 0); none of them exits the process.
 * Vectors that cross this boundary use the reference's own layouts:
 *   node arrays    [nno] in G.node order (sorted global node id, iz + ix*gnoz)
 *   element arrays [nel] in Morton (G.Mcode) order
 *   velocity dofs  [neq] in G.id order (u,w interleaved per node, 'V' dofs skipped)
 *   temperature dofs [heat neq] in G.heat.id order ('T' nodes skipped)
 * All arrays are plain host memory; the library copies in and out.
 * The context is stream-ordered on one CUDA stream and not thread-safe.
 */
#ifndef MCLG_H
#define MCLG_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------ */
enum {
	MCLG_OK = 0,
	MCLG_CAP_REACHED = 1,   /* an iteration cap was hit (the reference carries on too) */
	MCLG_NAN = 2,           /* a non-finite value appeared in a solver */
	MCLG_BREAKDOWN = 3,     /* CG breakdown: zero curvature d.Kd */
	MCLG_BAD_INPUT = 4,     /* malformed .input, bad sizes or unsupported option */
	MCLG_CUDA_ERROR = 5,    /* a CUDA call failed; see mclg_last_error() */
	MCLG_IO_ERROR = 6,      /* a file could not be read or written */
	MCLG_NO_DEVICE = 7      /* no CUDA device is visible */
};

#define MCLG_MAX_LEVEL 16

/*
 * Run configuration.  Field names and defaults follow the .input keys read by
 * read_input_file() (Input.c:3-99); mclg_config_from_input() parses a .input
 * file with the reference's getpar rules (Parsing.c:54-141: name=value tokens,
 * '#' comments, quoted values, last occurrence wins).
 */
typedef struct mclg_config {
	char data_dir[256];      /* data_dir (".")                         Input.c:7 */
	char solver[8];          /* solver: "cg" | "jc" | "gs" | "mg" ("jc") Input.c:10 */
	int level;               /* level: finest level + 1 (1)            Input.c:12 */
	int mg_min_level;        /* mg_min_level (1)                       Input.c:13 */
	int nprox, nproz;        /* nprox/nproz: must be 1 on one device   Input.c:20-21 */
	double model_length;     /* model_length (2.0)                     Input.c:23 */
	double model_height;     /* model_height (1.0)                     Input.c:24 */
	char top_v_bc[2], bot_v_bc[2], lef_v_bc[2], rig_v_bc[2];  /* "SV".. Input.c:26-29 */
	double top_v_bc_val[2], bot_v_bc_val[2], lef_v_bc_val[2], rig_v_bc_val[2];
	char top_T_bc, bot_T_bc, lef_T_bc, rig_T_bc;              /* 'T' / 'F' Input.c:35-38 */
	double top_T_bc_val, bot_T_bc_val, lef_T_bc_val, rig_T_bc_val;
	int T_ini;               /* T_ini (1); -2 = seeded synthetic field  Input.c:45 */
	double T_mantle, T_mantle_perturb;
	int T_wave_number;
	double Rayleigh;         /* Rayleigh (1e7)                         Input.c:51 */
	double A, refT, lower_mantle_jump;   /* Viscosity.c:13-16       Input.c:55-57 */
	int max_timestep, save_spacing;
	double Q, theta;         /* internal heating, time-integration theta */
	int AMR;
	int cg_precondition;     /* cg_precondition (0)                    Input.c:80 */
	double accuracy;         /* inner CG tolerance (0.001)              Input.c:83 */
	int auto_accuracy;
	double citcom_solver_accu; /* Uzawa tolerance (0.001)               Input.c:85 */
	int develop_mode;        /* static refinement pattern (1)           Input.c:86 */
	int check_v_only;
	int max_citcom_cycle;    /* (375) */
	int max_cg_cycle;        /* (200) */
	int zero_P;              /* (1) */
	int lg_mul, grain_damage; /* lg_mul must be 0 (the Lagrange-multiplier path is out of scope);
	                             grain_damage=1 runs the grain-size rheology after the viscosity,
	                             accepted on single-level meshes with precision=fp64 and solver
	                             "cg" or "jc" (Grain_size_evolution.c:3-152) */
	char old_T_file[1024];
	int old_T_timestep;
	/* seeded synthetic initial temperature (T_ini=-2), see mclg_ic.h */
	int ic_kind;
	uint64_t ic_seed;
	double ic_noise, ic_bl_thickness, ic_mode_amp;
	int ic_modes;
	/* GB300 solver options (not in the reference) */
	int precision;           /* 0 "fp64": FP64 replica of the reference's iteration;
	                            1 "mixed": FP32 multigrid-preconditioned inner CG inside the
	                                FP64 Uzawa loop and FP64 iterative refinement (on a refined mesh:
	                                MINRES with an FP32 V-cycle on the mesh's levels, conforming
	                                hanging-node space);
	                            2 "fp64mg": the same converged solver with FP64 inner solves */
	double stokes_rtol;      /* converged solvers: stop when |[F-Kd-Gp; G^T d]| / |F| < rtol (1e-8) */
	int warm_start;          /* converged solvers: 0 zero, 1 the previous step's (d,p), 2 d=0 and p kept
	                            (the reference's start), 3 linear extrapolation of the last two steps,
	                            4 (uniform meshes, stokes_method=1) the start of least FP64 residual in
	                            h1 + a (h1 - h2) + b (h1 - 2 h2 + h3) over the last three solutions
	                            (refined meshes treat 4 as 3) */
	double vis_min, vis_max; /* viscosity clip, applied when vis_max > 0 */
	int mg_smooth;           /* damped-Jacobi sweeps per V-cycle side (2) */
	double mg_omega;         /* Jacobi damping (0.6) */
	int mg_coarse;           /* elements per side of the coarsest grid (4; 2..8) */
	double outer_rtol;       /* Uzawa reduction per refinement pass (1e-3) */
	double inner_rtol;       /* inner CG reduction (1e-4) */
	int max_refine, max_outer, max_inner;  /* caps (20, 500, 200) */
	int mg_eta_avg;          /* coarse viscosity: 0 injection, 1 full-weighted mean, 2 log-mean (2) */
	int mg_block_n;          /* grids of at most this many elements per side run in one block (8) */
	int guess_smooth;        /* learned guess: binomial filter passes on the network's output (2) */
	int stokes_method;       /* converged solvers' correction solve: 0 Uzawa with inner MG-PCG (the
	                            reference's outer loop), 1 MINRES with a block-diagonal preconditioner (0) */
	/* the reference's multigrid inner solver, solver="mg" (Solver.c:668-768) */
	int mg_cycle;            /* V-cycles per inner solve (2)            Input.c:86 */
	int mg_finest_iteration; /* Gauss-Seidel sweeps before restriction (4)  Input.c:65 */
	int mg_coarse_iteration; /* Gauss-Seidel sweeps after prolongation (4)  Input.c:64 */
	/* grain-size rheology (grain_damage=1, Grain_size_evolution.c:3-123): the clip of
	 * the viscosity it sets */
	double lowest_vis, highest_vis;   /* (1.0, 1.0)  Input.c:58-59 */
	/* converged solvers on uniform meshes: smoothing sweeps per V-cycle side on the
	 * levels below the mg_fine_levels finest (0: mg_smooth) */
	int mg_smooth_coarse;
	/* converged solvers on uniform meshes with mg_smooth=2: 0 damped Jacobi (mg_omega),
	 * 1 the degree-2 Chebyshev polynomial of D^-1 K on [mg_cheb_lmax / mg_cheb_ratio,
	 * mg_cheb_lmax] (the same polynomial before and after the coarse correction, so
	 * the V-cycle stays symmetric) */
	int mg_smoother;
	double mg_cheb_lmax, mg_cheb_ratio;   /* (2.5, 4.0) */
	/* the number of finest levels that take mg_smooth sweeps per side; the coarser
	 * ones take mg_smooth_coarse (2) */
	int mg_fine_levels;
} mclg_config;

typedef struct mclg_step_stats {
	int timestep;
	int uzawa_cycles;        /* outer iterations (Solver.c:131-224) */
	int cg_cycles;           /* total inner CG iterations this step */
	int heat_cg_cycles;      /* Update_temperature.c:1140-1354 */
	int status;              /* worst status seen in this step */
	double dv, dp;           /* last Uzawa update sizes (Solver.c:202-204) */
	double dt, model_time;   /* Update_temperature.c:37-42 */
	double res_momentum;     /* |F - K d - G p|_2 / |F|_2 after the solve */
	double res_continuity;   /* |G^T d|_2 / |F|_2 after the solve */
	double ms_stokes, ms_heat, ms_total;  /* device time per phase */
	long long kernel_launches;            /* kernels launched by this step */
	double solver_kernel_ms; /* device time of the Stokes solver kernel(s) of this step (CUDA events) */
	long long solver_kernel_launches;
	int refine_passes;       /* converged solvers: FP64 refinement passes (0 for the replica) */
	int guess_used;          /* learned guess: 1 network, 0 previous solution, -1 not judged this step */
	double res_guess_learned, res_guess_prev;   /* relative FP64 residuals of the two candidate guesses */
	double ms_guess;         /* device time of the network and its feature kernels this step */
	double warm_alpha, warm_beta;   /* warm_start=4: the start h1 + alpha (h1-h2) + beta (h1-2h2+h3) chosen */
	/* the last remesh of this model (host wall clock, 0 before the first): the new
	 * mesh's numbering on the device (in begin), the refined-mesh solver's lists
	 * and the new device state (on the worker), the wait for the worker and the
	 * field carry-over (in end) */
	double remesh_ms_numbering, remesh_ms_lists, remesh_ms_state, remesh_ms_wait, remesh_ms_carry;
} mclg_step_stats;

typedef struct mclg_ctx mclg_ctx;

/* ---- configuration ----------------------------------------------------- */
/* Defaults of Input.c:3-99 (plus the GB300 options). */
void mclg_config_defaults(mclg_config *cfg);
/* sizeof(mclg_config), sizeof(mclg_step_stats): lets a binding check its layout. */
size_t mclg_config_sizeof(void);
size_t mclg_step_stats_sizeof(void);
/* setup_parser + read_input_file (Parsing.c:54-141, Input.c:3-99). */
int mclg_config_from_input(const char *path, mclg_config *cfg);

/* ---- life cycle -------------------------------------------------------- */
/* initial_data_structure + get_time_independent_variables (Mesh.c:3-428),
 * then the mesh block of Main.c:33-52 (build_quad_tree .. assign_matrix_memory)
 * on the host, and upload of the mesh to the device. */
int mclg_create(mclg_ctx **ctx, const mclg_config *cfg);
void mclg_destroy(mclg_ctx *ctx);
const char *mclg_status_string(int status);
const char *mclg_last_error(void);

/* ---- the per-step operator sequence (Main.c:55-64) --------------------- */
int mclg_initial_temperature(mclg_ctx *ctx);               /* Initial_condition.c:3-37 */
int mclg_buoyancy_force(mclg_ctx *ctx);                    /* Buoyancy.c:3-22 */
int mclg_viscosity(mclg_ctx *ctx);                         /* Viscosity.c:3-24 */
int mclg_velocity_pressure_KGF_matrix(mclg_ctx *ctx);      /* Build_matrix.c:4-40 */
int mclg_solve_velocity_pressure(mclg_ctx *ctx, mclg_step_stats *st); /* Solver.c:3-12 */
/* No counterpart in the reference (its solver mallocs its work vectors on
 * every call).  The same FP64 solve as mclg_solve_velocity_pressure (replica
 * mode, precision=fp64) for callers that must not allocate device memory at
 * solve time -- a host program that hands out all device memory up front, or
 * a time loop that cannot take cudaMalloc's latency and implicit device
 * synchronisation.  Its scratch is one device array built into the library,
 * sized for meshes of at most MCLG_NOALLOC_MAX_NODES nodes and
 * MCLG_NOALLOC_MAX_ELEMS elements (about 3.3 MB, held on every GPU that loads
 * the library until exit); larger meshes get MCLG_BAD_INPUT.  All calls share
 * the array: calls whose GPU work overlaps race.  The first call on a device
 * looks the array's device address up, so make it before any stream capture.
 * It updates d, P, V and the nodal stress of the context; the element stresses
 * and the solve counts that the context keeps for the regular solve are left
 * as they were (the counts come back in *st). */
#define MCLG_NOALLOC_MAX_NODES 16641
#define MCLG_NOALLOC_MAX_ELEMS 16384
int mclg_solve_velocity_pressure_noalloc(mclg_ctx *ctx, mclg_step_stats *st);
int mclg_update_temperature(mclg_ctx *ctx, mclg_step_stats *st);      /* Update_temperature.c:3-133 */
/* output(): Output.c:4-156 text files for the current G.timestep. */
int mclg_output(mclg_ctx *ctx, const char *data_dir, int timestep);
/* output() off the critical path: the fields are copied to pinned host memory
 * on the model's stream and a writer thread formats the files (one thread per
 * file) while the GPU carries on.  At most two outputs are in flight; a third
 * call waits for the oldest.  flags: MCLG_OUT_TEXT, Output.c's five text files
 * byte for byte; MCLG_OUT_BINARY, a full-precision side-car with pressure,
 * <data_dir>/<%07d>/fields.0.<%07d>.bin ("MCLGOUT1", int32 version, nno, nel,
 * timestep, double model_time, then X, Z, T, V0, V1 [nno], P [nel],
 * stress, vis [nno] as doubles).  A write error is returned by the next
 * output call or by mclg_output_wait. */
#define MCLG_OUT_TEXT 1
#define MCLG_OUT_BINARY 2
int mclg_output_async(mclg_ctx *ctx, const char *data_dir, int timestep, int flags);
/* every pending output written; the first error of any */
int mclg_output_wait(mclg_ctx *ctx);
/* One whole step: buoyancy .. solve, optional output (asynchronous, as
 * mclg_output_async with MCLG_OUT_TEXT), update_temperature. */
int mclg_step(mclg_ctx *ctx, int write_output, mclg_step_stats *st);
/* Same step with the host-buffer round trip a caller without device memory
 * makes: T (nno doubles, G.node order) is copied in before the step and
 * T, V (2*nno) and P (nel) are copied out after it. */
int mclg_step_host(mclg_ctx *ctx, const double *T_in, double *T_out, double *V_out,
                   double *P_out, mclg_step_stats *st);

/* ---- checkpoint / restart ----------------------------------------------
 * The reference restarts from a temperature file alone (T_ini=-1,
 * read_T_from_file, Initial_condition.c:171-195; mclg_create reads it too).
 * A checkpoint holds the whole state a continued run reads: the finest
 * level's leaves (so any develop_mode or remeshed tree is rebuilt), T, V,
 * stress, d, P, the model time and step counter, the converged solvers'
 * warm-start history and the learned guess's counters, in one binary file
 * closed by a checksum.  A run restarted from a checkpoint continues bit for
 * bit as the uninterrupted run; the network of a learned guess is attached
 * again by the caller (mclg_guess_set). */
int mclg_checkpoint_save(mclg_ctx *ctx, const char *path);
/* into a model on the same mesh (MCLG_BAD_INPUT otherwise; MCLG_IO_ERROR for
 * a truncated or corrupt file) */
int mclg_checkpoint_load(mclg_ctx *ctx, const char *path);
/* create a model on the checkpoint's mesh with this configuration, then load */
int mclg_restart(mclg_ctx **ctx, const mclg_config *cfg, const char *path);
/* G.timestep and G.model_time of the model */
int mclg_get_time(mclg_ctx *ctx, int *timestep, double *model_time);

/* ---- state access ------------------------------------------------------ */
enum {
	MCLG_F_T = 0,        /* [nno] temperature                     G.T[lev]          */
	MCLG_F_V0 = 1,       /* [nno] horizontal velocity             G.V[lev][0]       */
	MCLG_F_V1 = 2,       /* [nno] vertical velocity               G.V[lev][1]       */
	MCLG_F_P = 3,        /* [nel] pressure                        G.p[lev]          */
	MCLG_F_D = 4,        /* [neq] velocity solution vector        G.d[lev]          */
	MCLG_F_STRESS = 5,   /* [nno] second-invariant stress         G.stress[lev]     */
	MCLG_F_VIS = 6,      /* [nno] viscosity                       G.vis[lev]        */
	MCLG_F_BUOY = 7,     /* [nno] buoyancy                        G.buoyancy[lev]   */
	MCLG_F_F = 8,        /* [neq] Stokes right-hand side          G.F[lev]          */
	MCLG_F_KDIAG = 9,    /* [neq] diagonal of K                   G.Kdiag[lev]      */
	MCLG_F_BAB = 10,     /* [nel] sum_rows G^2/Kdiag              Solver.c:54-64    */
	MCLG_F_TAU0 = 11,    /* [nel] SUPG tau_x                      G.heat[lev].tau[0] */
	MCLG_F_TAU1 = 12,    /* [nel] SUPG tau_z                      G.heat[lev].tau[1] */
	MCLG_F_HEAT_F = 13,  /* [heat neq] heat right-hand side       G.heat[lev].F     */
	MCLG_F_X0 = 14,      /* [nno] node x                          G.X[lev][0]       */
	MCLG_F_X1 = 15,      /* [nno] node z                          G.X[lev][1]       */
	MCLG_F_GRAIN = 16    /* [nno] grain size (grain_damage=1; get only)  G.gs[lev]      */
};
enum {
	MCLG_M_SIZES = 0,    /* [8]: nel, nno, neq, heat_neq, nh, gnox, gnoz, max_level */
	MCLG_M_MCODE = 1,    /* [nel]      G.Mcode[lev]                                  */
	MCLG_M_NODE = 2,     /* [nno]      G.node[lev]                                   */
	MCLG_M_IEN = 3,      /* [4*nel]    G.ien[lev][a][e], a-major                      */
	MCLG_M_ID = 4,       /* [2*nno]    G.id[lev][d][A], d-major                       */
	MCLG_M_HEAT_ID = 5,  /* [nno]      G.heat[lev].id                                 */
	MCLG_M_LM = 6,       /* [8*nel]    G.lm[lev][d][a][e], (d,a)-major                */
	MCLG_M_HANG = 7,     /* [3*nh]     hanging node, parent 0, parent 1 (global ids)  */
	MCLG_M_VBC = 8,      /* [2*nno]    G.bc.v_bc[lev][d] codes ('V','S','N',...)       */
	MCLG_M_TBC = 9,      /* [nno]      G.bc.T_bc[lev] codes                           */
	/* the reference's multigrid transfer maps (solver="mg"), equation-indexed: */
	MCLG_M_INTERP = 10,  /* [5*neq]    lev > mg_min_level: G.interp[lev].local_eq_n, then
	                                   local_eq[0..3] (equations of lev-1, -1 unused or fixed)
	                                   Connection.c:708-930 */
	MCLG_M_PROJECT = 11, /* [neq]      lev < finest: the equation of lev+1 whose residual
	                                   equation l of lev takes (G.project[lev].local_u), -1 none
	                                   Connection.c:1051-1250 */
	MCLG_M_GS_WAVE = 12, /* [nno]      Gauss-Seidel wavefront of each node: nodes of one
	                                   wavefront share no matrix entry, and sweeping the
	                                   wavefronts in order reproduces the sequential sweep */
	/* the node-block operator's structure: */
	MCLG_M_NB = 13,      /* [25*nno]   node A's matrix neighbours (the distinct nodes of the
	                                   elements touching it, level-local indices, ascending)
	                                   in out[25A ..], -1 after the last */
	MCLG_M_KSLOT = 14    /* [16*nel]   slot of corner b in corner a's neighbour list,
	                                   out[(4a+b)*nel + e] */
};
/* lev < 0 selects the finest level.  n is the caller's buffer length; the
 * call fails with MCLG_BAD_INPUT when it does not match the array size. */
int mclg_get_field(mclg_ctx *ctx, int which, int lev, double *out, size_t n);
int mclg_set_field(mclg_ctx *ctx, int which, int lev, const double *in, size_t n);
int mclg_get_mesh(mclg_ctx *ctx, int which, int lev, int *out, size_t n);

/* ---- host-only mesh access (no device needed) ------------------------- */
/* The mesh block of Main.c:33-52 on the host: quadtree, numbering, BC codes,
 * hanging nodes.  Usable on a machine without a GPU. */
typedef struct mclg_mesh_handle mclg_mesh_handle;
int mclg_mesh_new(mclg_mesh_handle **h, const mclg_config *cfg);
void mclg_mesh_delete(mclg_mesh_handle *h);
int mclg_mesh_get(const mclg_mesh_handle *h, int which, int lev, int *out, size_t n);
enum {
	MCLG_R_X = 0,        /* [2*nno]  G.X[lev][d][A], d-major                    */
	MCLG_R_JACOBI = 1,   /* [nel]    G.jacobi[lev]                              */
	MCLG_R_AREA = 2,     /* [nel]    G.eco[lev].area                            */
	MCLG_R_VBCVAL = 3,   /* [2*nno]  G.bc.v_bc_val[lev][d]                      */
	MCLG_R_TBCVAL = 4    /* [nno]    G.bc.T_bc_val[lev]                         */
};
int mclg_mesh_get_real(const mclg_mesh_handle *h, int which, int lev, double *out, size_t n);
/* Initial_condition.c:3-136 on level lev (finest when lev < 0). */
int mclg_mesh_initial_temperature(const mclg_mesh_handle *h, int lev, double *T, size_t n);
/* Output.c:4-156 from host fields of the finest level (each nno long, G.node
 * order): the files mclg_output writes, for fields the caller holds. */
int mclg_mesh_write_output(const mclg_mesh_handle *h, const char *data_dir, int timestep,
                           const double *T, const double *V0, const double *V1,
                           const double *stress, const double *vis, size_t n);

/* ---- single operators, for parity tests (finest level unless lev >= 0) -- */
int mclg_stokes_matvec(mclg_ctx *ctx, int lev, const double *x, double *y);   /* K_prod_d, Solver.c:360-386 */
int mclg_stokes_G(mclg_ctx *ctx, int lev, const double *p, double *y);        /* G_prod_p, Solver.c:569-591 */
int mclg_stokes_GT(mclg_ctx *ctx, int lev, const double *x, double *p);       /* GT_prod_d, Solver.c:645-666 */
enum { MCLG_HEAT_K = 0, MCLG_HEAT_C = 1 };
int mclg_heat_matvec(mclg_ctx *ctx, int which, const double *x, double *y);   /* K_prod_d_heat, Update_temperature.c:935-962 */

/* ---- |grad T| adaptive refinement (no reference counterpart) --------------
 * The reference refines only by the fixed patterns of initial_refine
 * (Tree.c:184-300; adaptive_mesh_refine is empty, Tree.c:95-99).  Leaves are
 * finest-level Morton start codes (Mcode >> 4 of the finest level), sorted,
 * covering the box.
 *   mclg_create_leaves   a model on a given leaf set instead of develop_mode;
 *   mclg_amr_flags       per finest-level element (Morton order): |grad T| at
 *                        its centre > frac * max over elements (device, IEEE
 *                        rounding, bit-reproducible on the CPU);
 *   mclg_amr_leaves      flags (host buffer, one per finest-level element) ->
 *                        the new tree's leaves, built on the device: flagged
 *                        leaves' cells at target_level, the rest at
 *                        base_level, 2:1 balanced across edges and corners;
 *                        equal to mclg_mesh_amr_leaves on the same flags;
 *   mclg_amr_remesh      flags and the new tree on the device -> the model
 *                        rebuilt on it in place (numbering and hanging nodes
 *                        on the host), T carried over by bilinear
 *                        interpolation, time step and model time kept.
 *                        Refined meshes run the FP64 replica (precision=fp64)
 *                        or the converged refined-mesh solver (mixed, fp64mg).
 * Host-only counterparts for checking the tree and the transfers without a GPU:
 * mclg_mesh_new_leaves, mclg_mesh_amr_leaves, mclg_mesh_transfer (nodal fields,
 * bilinear) and mclg_mesh_transfer_elem (element fields such as the pressure:
 * the area mean of the old field over each new element, as a remesh carries
 * the converged solvers' pressure over). */
int mclg_create_leaves(mclg_ctx **ctx, const mclg_config *cfg, const int *leaves, size_t n);
int mclg_amr_flags(mclg_ctx *ctx, double frac, unsigned char *flags, size_t n, double *gmax);
int mclg_amr_leaves(mclg_ctx *ctx, const unsigned char *flags, size_t n, int base_level, int target_level, int *leaves,
                    size_t cap, size_t *nleaves);
int mclg_amr_remesh(mclg_ctx *ctx, double frac, int base_level, int target_level, size_t *nel);
/* The same in two halves, so that the host work overlaps the GPU's: begin takes
 * the flags of the current T, the new tree and the new mesh's numbering and
 * hanging nodes (device, on the model's stream), then builds the refined-mesh
 * solver's lists and the new device state on a worker thread and returns; the
 * caller may go on stepping the old mesh; end waits
 * for the worker and carries the current fields over (as mclg_amr_remesh).
 * One remesh may be pending at a time; mclg_destroy finishes a pending one. */
int mclg_amr_remesh_begin(mclg_ctx *ctx, double frac, int base_level, int target_level);
int mclg_amr_remesh_end(mclg_ctx *ctx, size_t *nel);
int mclg_mesh_new_leaves(mclg_mesh_handle **h, const mclg_config *cfg, const int *leaves, size_t n);
/* The same mesh numbered on the current CUDA device (k_mesh.cu: ien, node list,
 * BC codes, equation numbers, geometry, node->element map, hanging nodes,
 * neighbour lists), copied into host arrays equal to mclg_mesh_new_leaves's
 * byte for byte.  Rejects leaf lists that are not quadtree cells. */
int mclg_mesh_new_leaves_device(mclg_mesh_handle **h, const mclg_config *cfg, const int *leaves, size_t n);
/* 0 when every array of every level of a and b is equal byte for byte, else 1
 * and the first differing array's name in what[cap]. */
int mclg_mesh_diff(const mclg_mesh_handle *a, const mclg_mesh_handle *b, char *what, size_t cap);
int mclg_mesh_amr_leaves(const mclg_mesh_handle *h, const unsigned char *flags, size_t nflags, int base_level,
                         int target_level, int *leaves, size_t cap, size_t *n);
int mclg_mesh_transfer(const mclg_mesh_handle *from, const double *T_from, size_t n_from,
                       const mclg_mesh_handle *to, double *T_to, size_t n_to);
int mclg_mesh_transfer_elem(const mclg_mesh_handle *from, const double *P_from, size_t n_from,
                            const mclg_mesh_handle *to, double *P_to, size_t n_to);
/* The refined-mesh solver's host lists of one level (lev < 0: the finest), as
 * the converged solvers upload them, for checking without a GPU.  Built on
 * the first call for every level from mg_min_level up.  Dofs are 2*node + c.
 *   SIZES  int[4]       nno, width of C^T K C's node-block rows, contributions,
 *                       expansion entries
 *   KIND   int[2*nno]   0 fixed, 1 reduced, 2 constrained (hanging)
 *   RC_OFF int[nno+1], RC_TGT int[n], RC_SRC int[n], RC_W double[n]: row A of
 *          C^T K C gets, for i in RC_OFF[A] .. RC_OFF[A+1]-1, entry
 *          (slot RC_TGT>>2, component pair RC_TGT&3) += RC_W * K[RC_SRC], K the
 *          node-block operator as flat doubles: K[((k*nno + A)*4 + 2c + c')]
 *          couples (A,c) with (the k-th neighbour of A, c')
 *   RNB    int[width*nno] the row's reduced column nodes, slot-major
 *   RCNT   int[nno]       columns per row */
/* Grain-size rheology (grain_damage=1, Grain_size_evolution.c:3-152), host work:
 * one call per time step after the exponential viscosity, on the level the
 * reference evolves (a single-level mesh's only level).  The state holds the
 * routine's first-call flag, its clock and the nodal grain size.  The first
 * call sets the grain size to 1e-3; later calls scale `stress` (nodal,
 * nondimensional) to Pa in place and, while the clock is behind model_time,
 * take the reference's 100-year steps per node within 200 km of the top,
 * setting `vis` there (clipped to [lowest_vis, highest_vis]) and the stress of
 * the deeper nodes to 0.  X: [2*nno] node coordinates (x then z). */
typedef struct mclg_grain_state mclg_grain_state;
int mclg_grain_new(mclg_grain_state **g);
int mclg_grain_update(mclg_grain_state *g, int nno, const double *X, const double *T, double *stress,
                      double *vis, double model_time, double Ra, double lowest_vis, double highest_vis,
                      int threads);
int mclg_grain_get(const mclg_grain_state *g, double *grain_size, size_t n);
void mclg_grain_delete(mclg_grain_state *g);

enum { MCLG_QT_SIZES = 0, MCLG_QT_KIND = 1, MCLG_QT_RC_OFF = 2, MCLG_QT_RC_TGT = 3, MCLG_QT_RC_SRC = 4,
       MCLG_QT_RC_W = 5, MCLG_QT_RNB = 6, MCLG_QT_RCNT = 7 };
int mclg_mesh_qt_get(mclg_mesh_handle *h, int lev, int which, void *out, size_t n);

/* ---- batched ensembles (no reference counterpart) ------------------------
 * n independent models, each built from its own configuration (converged
 * solvers on uniform meshes, all with the same precision and element aspect
 * ratio), stepped together on one stream: per step the members' element
 * kernels, ONE launch of the batched converged solver (each thread block
 * solves one model; blocks take models from a queue ordered largest first),
 * then the members' stress and heat kernels.  In the batch launch a model is
 * solved by a thread-block cluster (cluster barriers, reductions through
 * distributed shared memory); the cluster size (1, 2, 4, 8 or, where the
 * device allows it, 16 blocks) is chosen by an autotuner that times each on
 * one of steps 2..6 and keeps the cheapest per inner iteration.  Results per member equal those of the member
 * stepped alone up to summation order. */
typedef struct mclg_ensemble mclg_ensemble;
int mclg_ensemble_create(mclg_ensemble **e, const mclg_config *cfgs, int n);
/* The same with refined members: member i's configuration gives its base grid
 * (level-1), refined up to amr_levels[i] levels by |grad T| > 0.2 max of its
 * initial temperature (2:1 balanced, hanging nodes; 0 = uniform).  Refined
 * members are solved by the refined-mesh solver, one launch each after the
 * batched launch of the uniform members. */
int mclg_ensemble_create_amr(mclg_ensemble **e, const mclg_config *cfgs, const int *amr_levels, int n);
/* 1 when steps replay a CUDA graph of the whole ensemble step: captured once the
 * cluster-size autotuner has chosen (step 7) and every member's warm start is
 * steady; until then, or where capture is refused, the step is issued launch by
 * launch. */
int mclg_ensemble_graph(const mclg_ensemble *e);
void mclg_ensemble_destroy(mclg_ensemble *e);
int mclg_ensemble_size(const mclg_ensemble *e);
/* Member i as a context (fields, mesh, single operators); owned by the ensemble. */
int mclg_ensemble_member(mclg_ensemble *e, int i, mclg_ctx **ctx);
int mclg_ensemble_initial_temperature(mclg_ensemble *e);
/* One time step of every member; stats (optional) has n entries, grid_used
 * (optional) receives the blocks of this step's batched launch.  ms_total and
 * solver_kernel_ms are the whole batch's.  cluster_used (optional) receives
 * the cluster size of this step's batched launch. */
int mclg_ensemble_step(mclg_ensemble *e, mclg_step_stats *stats, int *cluster_used);

/* ---- learned initial guess (no reference counterpart) -------------------
 * A fully convolutional network of `depth` 3x3 convolution layers (ReLU
 * between them, `width` channels) with BF16 weights and FP32 accumulation,
 * trained on the device by the library's own forward, backward and Adam
 * kernels.  Parameters are one flat FP32 array, layer by layer:
 * W[cout][cin][3][3] then b[cout].  Tensors are [batch][channel][h][w]. */
typedef struct mclg_cnn mclg_cnn;
int mclg_cnn_create(mclg_cnn **net, int cin, int width, int depth, int cout, unsigned long long seed);
void mclg_cnn_destroy(mclg_cnn *net);
size_t mclg_cnn_num_params(const mclg_cnn *net);
int mclg_cnn_shape(const mclg_cnn *net, int *cin, int *width, int *depth, int *cout);
int mclg_cnn_get_params(const mclg_cnn *net, float *out, size_t n);
int mclg_cnn_set_params(mclg_cnn *net, const float *in, size_t n);   /* also resets the Adam moments */
int mclg_cnn_forward(mclg_cnn *net, const float *x, int batch, int h, int w, float *y);
/* Mean squared error against target and its gradient (flat parameter layout). */
int mclg_cnn_gradient(mclg_cnn *net, const float *x, const float *target, int batch, int h, int w,
                      double *loss, float *grad, size_t n);
int mclg_cnn_adam_step(mclg_cnn *net, const float *grad, size_t n, float lr);   /* beta 0.9/0.999, eps 1e-8 */
/* Adam on the mean squared error over nsamples (x, target) pairs held on the
 * device; `iters` steps of `batch` samples drawn with a Philox stream. */
int mclg_cnn_train(mclg_cnn *net, const float *x, const float *target, int nsamples, int h, int w, int batch,
                   int iters, float lr, unsigned long long seed, float *loss_trace);
int mclg_cnn_save(const mclg_cnn *net, const char *path);
int mclg_cnn_load(mclg_cnn **net, const char *path);

/* The guess on a context (converged solvers, warm_start=1 or 3).  Features
 * live on the (grid+1)^2 node grid of a uniform mesh coarsened to `grid`
 * elements per side: T, 0.2 log10 eta, the last solution (u, w scaled by its
 * RMS speed, nodal p by its RMS) and the last change between solutions (scaled
 * by its own RMS).  The network predicts, in units of the last change, the
 * correction to the warm_start guess (the last solution, or its linear
 * extrapolation), prolonged bilinearly to the mesh.  The solver keeps
 * whichever of the corrected and the plain warm_start guess has the smaller
 * FP64 residual, and switches the network off for 16 steps after it fails to
 * save iterations on 3 steps in a row.  MCLG_GUESS_RECORD computes features
 * and targets without a network (training data, see mclg_guess_sample). */
enum { MCLG_GUESS_OFF = 0, MCLG_GUESS_RECORD = 1, MCLG_GUESS_LEARNED = 2,
       MCLG_GUESS_FORCED = 3 /* the network's guess on every step, never judged (for measurement) */ };
int mclg_guess_set(mclg_ctx *ctx, int mode, int grid, mclg_cnn *net);
/* Features x[8][grid+1][grid+1] and target y[3][grid+1][grid+1] of the last
 * solve; MCLG_BAD_INPUT when that solve had fewer than two solutions before it. */
int mclg_guess_sample(mclg_ctx *ctx, float *x, size_t nx, float *y, size_t ny);

#ifdef __cplusplus
}
#endif
#endif
