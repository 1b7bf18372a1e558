/*
 * Output.c:4-156 text files, one set per saved step:
 *   <data_dir>/<%07d step>/{coord,temperature,stress,viscosity,velocity}.0.<%07d step>
 * one line per node of the finest level in G.node order, "%e" ("%+e" for
 * velocity), stress divided by 1e6 (Output.c:88).  The rank suffix is always
 * 0: one device holds the whole mesh.  Pressure is not written, as in the
 * reference.
 */
#include <stdio.h>
#include <string.h>
#include <sys/stat.h>
#include <sys/types.h>
#include <unistd.h>
#include "mclg_host.h"

static FILE *open_field(const char *dir, const char *name, int step)
{
	char path[2048];
	FILE *fp;
	snprintf(path, sizeof path, "%s/%07d/%s.%d.%07d", dir, step, name, 0, step);
	fp = fopen(path, "w");
	if (fp == NULL)
		mclg_set_error("cannot open file %s", path);
	return fp;
}

/* <dir>/<%07d step>/ */
int mclg_output_dirs(const char *dir, int step)
{
	char path[2048];
	if (access(dir, F_OK) == -1)
		mkdir(dir, 0700);
	snprintf(path, sizeof path, "%s/%07d", dir, step);
	if (access(path, F_OK) == -1)
		mkdir(path, 0700);
	return MCLG_OK;
}

/* One of the five files: which = 0 coord, 1 temperature, 2 stress, 3 viscosity, 4 velocity. */
int mclg_write_output_file(const char *dir, int step, int which, const mclg_level *L, const double *T,
                           const double *V0, const double *V1, const double *stress, const double *vis)
{
	static const char *names[5] = {"coord", "temperature", "stress", "viscosity", "velocity"};
	FILE *fp;
	int i, nn = L->nno, ok = 1;
	if (which < 0 || which > 4)
		return MCLG_BAD_INPUT;
	if ((fp = open_field(dir, names[which], step)) == NULL)
		return MCLG_IO_ERROR;
	for (i = 0; i < nn && ok; i++) {
		switch (which) {
		case 0: ok = fprintf(fp, "%e %e\n", L->X[i], L->X[nn + i]) > 0; break;
		case 1: ok = fprintf(fp, "%e\n", T[i]) > 0; break;
		case 2: ok = fprintf(fp, "%e\n", stress[i] / 1e6) > 0; break;
		case 3: ok = fprintf(fp, "%e\n", vis[i]) > 0; break;
		default: ok = fprintf(fp, "%+e %+e\n", V0[i], V1[i]) > 0; break;
		}
	}
	if (fclose(fp) != 0 || !ok) {
		mclg_set_error("writing %s of step %d under %s failed", names[which], step, dir);
		return MCLG_IO_ERROR;
	}
	return MCLG_OK;
}

int mclg_write_output(const char *dir, int step, const mclg_level *L, const double *T,
                      const double *V0, const double *V1, const double *stress, const double *vis)
{
	int which, rc;
	mclg_output_dirs(dir, step);
	for (which = 0; which < 5; which++)
		if ((rc = mclg_write_output_file(dir, step, which, L, T, V0, V1, stress, vis)) != MCLG_OK)
			return rc;
	return MCLG_OK;
}
