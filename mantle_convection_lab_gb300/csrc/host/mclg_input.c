/*
 * .input reader: the getpar dialect of Parsing.c:54-141 and the key table of
 * Input.c:3-99, restated for the C ABI.
 *
 * Tokenisation follows setup_parser (Parsing.c:83-125): on each line, after
 * blanks, a '#' ends the line; a name runs up to '=', a blank or the end of
 * line; a value is either quoted ('...' or "...", up to the matching quote)
 * or runs up to the next blank.  Several name=value pairs may share a line.
 * Lookups search the list backwards, so the last occurrence of a key wins
 * (Parsing.c:231-243).  Unlike the reference, nothing here exits the process:
 * errors come back as MCLG_IO_ERROR / MCLG_BAD_INPUT.
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include "mclg.h"
#include "mclg_host.h"

#define LINE_MAX_CHARS 1024
#define NAME_MAX_CHARS 64
#define VALUE_MAX_CHARS 1024

typedef struct par_entry {
	char name[NAME_MAX_CHARS];
	char value[VALUE_MAX_CHARS];
} par_entry;

typedef struct par_list {
	par_entry *e;
	int n, cap;
} par_list;

static int par_add(par_list *pl, const char *name, const char *value)
{
	if (pl->n == pl->cap) {
		int cap = pl->cap ? 2 * pl->cap : 64;
		par_entry *e = (par_entry *)realloc(pl->e, (size_t)cap * sizeof(par_entry));
		if (e == NULL)
			return -1;
		pl->e = e;
		pl->cap = cap;
	}
	snprintf(pl->e[pl->n].name, NAME_MAX_CHARS, "%s", name);
	snprintf(pl->e[pl->n].value, VALUE_MAX_CHARS, "%s", value);
	pl->n++;
	return 0;
}

static const char *par_find(const par_list *pl, const char *name)
{
	int i;
	for (i = pl->n - 1; i >= 0; i--)
		if (strcmp(pl->e[i].name, name) == 0)
			return pl->e[i].value;
	return NULL;
}

static int par_read_file(par_list *pl, const char *path)
{
	char line[LINE_MAX_CHARS];
	FILE *fp = fopen(path, "r");
	if (fp == NULL)
		return MCLG_IO_ERROR;
	while (fgets(line, sizeof line, fp) != NULL) {
		const char *c = line;
		for (;;) {
			char name[NAME_MAX_CHARS], value[VALUE_MAX_CHARS];
			int nn = 0, nv = 0;
			char stop1, stop2;
			while (*c == ' ' || *c == '\t')
				c++;
			if (*c == '\0' || *c == '\n' || *c == '#')
				break;
			while (*c != '=' && *c != '\0' && *c != ' ' && *c != '\n' && *c != '\t') {
				if (nn < NAME_MAX_CHARS - 1)
					name[nn++] = *c;
				c++;
			}
			name[nn] = '\0';
			if (*c == '=')
				c++;
			if (*c == '"' || *c == '\'') {
				stop1 = stop2 = *c;
				c++;
			} else {
				stop1 = ' ';
				stop2 = '\t';
			}
			while (*c != stop1 && *c != stop2 && *c != '\0' && *c != '\n') {
				if (nv < VALUE_MAX_CHARS - 1)
					value[nv++] = *c;
				c++;
			}
			value[nv] = '\0';
			if (*c == '"' || *c == '\'')
				c++;
			if (par_add(pl, name, value) != 0) {
				fclose(fp);
				return MCLG_BAD_INPUT;
			}
		}
	}
	fclose(fp);
	return MCLG_OK;
}

static void get_int(const par_list *pl, const char *name, int *v, int dflt)
{
	const char *s = par_find(pl, name);
	*v = dflt;
	if (s != NULL)
		sscanf(s, "%d", v);
}

static void get_double(const par_list *pl, const char *name, double *v, double dflt)
{
	const char *s = par_find(pl, name);
	*v = dflt;
	if (s != NULL)
		sscanf(s, "%lf", v);
}

static void get_string(const par_list *pl, const char *name, char *v, size_t cap, const char *dflt)
{
	const char *s = par_find(pl, name);
	snprintf(v, cap, "%s", s != NULL ? s : dflt);
}

/* Comma-separated doubles; entries missing from the value keep their old
 * contents, as input_double_vector (Parsing.c:694-741) leaves them. */
static void get_double_vector(const par_list *pl, const char *name, int n, double *v)
{
	const char *s = par_find(pl, name);
	int k;
	if (s == NULL)
		return;
	for (k = 0; k < n; k++) {
		char *end;
		double x;
		while (*s == ' ' || *s == '\t')
			s++;
		x = strtod(s, &end);
		if (end == s)
			return;
		v[k] = x;
		s = end;
		if (*s != ',')
			return;
		s++;
	}
}

size_t mclg_config_sizeof(void)
{
	return sizeof(mclg_config);
}

size_t mclg_step_stats_sizeof(void)
{
	return sizeof(mclg_step_stats);
}

void mclg_config_defaults(mclg_config *c)
{
	memset(c, 0, sizeof *c);
	snprintf(c->data_dir, sizeof c->data_dir, ".");
	snprintf(c->solver, sizeof c->solver, "jc");
	c->level = 1;
	c->mg_min_level = 1;
	c->nprox = c->nproz = 2;
	c->model_length = 2.0;
	c->model_height = 1.0;
	memcpy(c->top_v_bc, "sv", 2);
	memcpy(c->bot_v_bc, "sv", 2);
	memcpy(c->lef_v_bc, "vs", 2);
	memcpy(c->rig_v_bc, "vs", 2);
	c->top_T_bc = 'T';
	c->bot_T_bc = 'T';
	c->lef_T_bc = 'F';
	c->rig_T_bc = 'F';
	c->top_T_bc_val = 0.0;
	c->bot_T_bc_val = 1.0;
	c->T_ini = 1;
	c->T_mantle = 0.5;
	c->T_mantle_perturb = 0.01;
	c->T_wave_number = 6;
	c->Rayleigh = 1e7;
	c->A = 0.0;
	c->refT = 0.5;
	c->lower_mantle_jump = 1.0;
	c->max_timestep = 0;
	c->save_spacing = 1;
	c->Q = 0.0;
	c->theta = 0.0;
	c->cg_precondition = 0;
	c->accuracy = 0.001;
	c->citcom_solver_accu = 0.001;
	c->develop_mode = 1;
	c->max_citcom_cycle = 375;
	c->max_cg_cycle = 200;
	c->zero_P = 1;
	c->ic_kind = 1;
	c->ic_bl_thickness = 0.02;
	c->ic_modes = 8;
	c->ic_mode_amp = 0.005;
	c->precision = 0;
	c->stokes_rtol = 1e-8;
	c->mg_smooth = 2;
	c->mg_omega = 0.6;
	c->mg_coarse = 4;
	c->outer_rtol = 1e-3;
	c->inner_rtol = 1e-4;
	c->max_refine = 20;
	c->max_outer = 500;
	c->max_inner = 200;
	c->mg_eta_avg = 2;
	c->mg_block_n = 8;
	c->guess_smooth = 2;
	c->stokes_method = 0;
	c->mg_cycle = 2;
	c->mg_finest_iteration = 4;
	c->mg_coarse_iteration = 4;
	c->lowest_vis = 1.0;
	c->highest_vis = 1.0;
	c->mg_smoother = 0;
	c->mg_cheb_lmax = 2.5;
	c->mg_cheb_ratio = 4.0;
	c->mg_fine_levels = 2;
}

int mclg_config_from_input(const char *path, mclg_config *c)
{
	par_list pl = {0};
	char buf[VALUE_MAX_CHARS];
	int rc;
	mclg_config_defaults(c);
	rc = par_read_file(&pl, path);
	if (rc != MCLG_OK) {
		free(pl.e);
		mclg_set_error("cannot read input file %s", path);
		return rc;
	}
	get_string(&pl, "data_dir", c->data_dir, sizeof c->data_dir, ".");
	get_string(&pl, "solver", c->solver, sizeof c->solver, "jc");
	get_int(&pl, "level", &c->level, 1);
	get_int(&pl, "mg_min_level", &c->mg_min_level, 1);
	get_int(&pl, "nprox", &c->nprox, 2);
	get_int(&pl, "nproz", &c->nproz, 2);
	get_double(&pl, "model_length", &c->model_length, 2.0);
	get_double(&pl, "model_height", &c->model_height, 1.0);
	/* v_bc strings keep their first two characters (char[NSD], global_variables.h:256-259) */
	get_string(&pl, "top_v_bc", buf, sizeof buf, "sv"); c->top_v_bc[0] = buf[0]; c->top_v_bc[1] = buf[0] ? buf[1] : 0;
	get_string(&pl, "bot_v_bc", buf, sizeof buf, "sv"); c->bot_v_bc[0] = buf[0]; c->bot_v_bc[1] = buf[0] ? buf[1] : 0;
	get_string(&pl, "lef_v_bc", buf, sizeof buf, "vs"); c->lef_v_bc[0] = buf[0]; c->lef_v_bc[1] = buf[0] ? buf[1] : 0;
	get_string(&pl, "rig_v_bc", buf, sizeof buf, "vs"); c->rig_v_bc[0] = buf[0]; c->rig_v_bc[1] = buf[0] ? buf[1] : 0;
	get_double_vector(&pl, "top_v_bc_val", 2, c->top_v_bc_val);
	get_double_vector(&pl, "bot_v_bc_val", 2, c->bot_v_bc_val);
	get_double_vector(&pl, "lef_v_bc_val", 2, c->lef_v_bc_val);
	get_double_vector(&pl, "rig_v_bc_val", 2, c->rig_v_bc_val);
	get_string(&pl, "top_T_bc", buf, sizeof buf, "T"); c->top_T_bc = buf[0];
	get_string(&pl, "bot_T_bc", buf, sizeof buf, "T"); c->bot_T_bc = buf[0];
	get_string(&pl, "lef_T_bc", buf, sizeof buf, "F"); c->lef_T_bc = buf[0];
	get_string(&pl, "rig_T_bc", buf, sizeof buf, "F"); c->rig_T_bc = buf[0];
	get_double(&pl, "top_T_bc_val", &c->top_T_bc_val, 0.0);
	get_double(&pl, "bot_T_bc_val", &c->bot_T_bc_val, 1.0);
	get_double(&pl, "lef_T_bc_val", &c->lef_T_bc_val, 0.0);
	get_double(&pl, "rig_T_bc_val", &c->rig_T_bc_val, 0.0);
	get_int(&pl, "T_ini", &c->T_ini, 1);
	get_double(&pl, "T_mantle", &c->T_mantle, 0.5);
	get_double(&pl, "T_mantle_perturb", &c->T_mantle_perturb, 0.01);
	get_int(&pl, "T_wave_number", &c->T_wave_number, 6);
	get_double(&pl, "Rayleigh", &c->Rayleigh, 1e7);
	get_double(&pl, "A", &c->A, 0.0);
	get_double(&pl, "refT", &c->refT, 0.5);
	get_double(&pl, "lower_mantle_jump", &c->lower_mantle_jump, 1.0);
	get_int(&pl, "max_timestep", &c->max_timestep, 0);
	get_int(&pl, "save_spacing", &c->save_spacing, 1);
	get_double(&pl, "Q", &c->Q, 0.0);
	get_double(&pl, "theta", &c->theta, 0.0);
	get_int(&pl, "AMR", &c->AMR, 0);
	get_int(&pl, "cg_precondition", &c->cg_precondition, 0);
	get_double(&pl, "accuracy", &c->accuracy, 0.001);
	get_int(&pl, "auto_accuracy", &c->auto_accuracy, 0);
	get_double(&pl, "citcom_solver_accu", &c->citcom_solver_accu, 0.001);
	get_int(&pl, "develop_mode", &c->develop_mode, 1);
	get_int(&pl, "check_v_only", &c->check_v_only, 0);
	get_int(&pl, "max_citcom_cycle", &c->max_citcom_cycle, 375);
	get_int(&pl, "max_cg_cycle", &c->max_cg_cycle, 200);
	get_string(&pl, "old_T_file", c->old_T_file, sizeof c->old_T_file, "");
	get_int(&pl, "old_T_timestep", &c->old_T_timestep, 0);
	get_int(&pl, "lg_mul", &c->lg_mul, 0);
	get_int(&pl, "grain_damage", &c->grain_damage, 0);
	get_int(&pl, "zero_P", &c->zero_P, 1);
	/* seeded synthetic temperature (mclg_ic.h) */
	get_int(&pl, "ic_kind", &c->ic_kind, 1);
	get_string(&pl, "ic_seed", buf, sizeof buf, "0");
	c->ic_seed = strtoull(buf, NULL, 10);
	get_double(&pl, "ic_noise", &c->ic_noise, 0.0);
	get_double(&pl, "ic_bl_thickness", &c->ic_bl_thickness, 0.02);
	get_int(&pl, "ic_modes", &c->ic_modes, 8);
	get_double(&pl, "ic_mode_amp", &c->ic_mode_amp, 0.005);
	/* GB300 solver options */
	get_string(&pl, "precision", buf, sizeof buf, "fp64");
	c->precision = (strcmp(buf, "mixed") == 0) ? 1 : (strcmp(buf, "fp64mg") == 0) ? 2 : 0;
	get_double(&pl, "stokes_rtol", &c->stokes_rtol, 1e-8);
	get_int(&pl, "warm_start", &c->warm_start, 0);
	get_double(&pl, "vis_min", &c->vis_min, 0.0);
	get_double(&pl, "vis_max", &c->vis_max, 0.0);
	get_int(&pl, "mg_smooth", &c->mg_smooth, 2);
	get_double(&pl, "mg_omega", &c->mg_omega, 0.6);
	get_int(&pl, "mg_coarse", &c->mg_coarse, 4);
	get_double(&pl, "outer_rtol", &c->outer_rtol, 1e-3);
	get_double(&pl, "inner_rtol", &c->inner_rtol, 1e-4);
	get_int(&pl, "max_refine", &c->max_refine, 20);
	get_int(&pl, "max_outer", &c->max_outer, 500);
	get_int(&pl, "max_inner", &c->max_inner, 200);
	get_int(&pl, "mg_eta_avg", &c->mg_eta_avg, 2);
	get_int(&pl, "mg_block_n", &c->mg_block_n, 8);
	get_int(&pl, "guess_smooth", &c->guess_smooth, 2);
	get_int(&pl, "stokes_method", &c->stokes_method, 0);
	/* Input.c:64-65, 86 */
	get_int(&pl, "mg_cycle", &c->mg_cycle, 2);
	get_int(&pl, "mg_finest_iteration", &c->mg_finest_iteration, 4);
	get_int(&pl, "mg_coarse_iteration", &c->mg_coarse_iteration, 4);
	get_double(&pl, "lowest_vis", &c->lowest_vis, 1.0);
	get_double(&pl, "highest_vis", &c->highest_vis, 1.0);
	get_int(&pl, "mg_smooth_coarse", &c->mg_smooth_coarse, 0);
	get_int(&pl, "mg_smoother", &c->mg_smoother, 0);
	get_double(&pl, "mg_cheb_lmax", &c->mg_cheb_lmax, 2.5);
	get_double(&pl, "mg_cheb_ratio", &c->mg_cheb_ratio, 4.0);
	get_int(&pl, "mg_fine_levels", &c->mg_fine_levels, 2);
	free(pl.e);
	return MCLG_OK;
}
