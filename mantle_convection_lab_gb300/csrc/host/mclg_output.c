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

int mclg_write_output(const char *dir, int step, const mclg_level *L, const double *T,
                      const double *V0, const double *V1, const double *stress, const double *vis)
{
	char path[2048];
	FILE *fp;
	int i, nn = L->nno;
	if (access(dir, F_OK) == -1)
		mkdir(dir, 0700);
	snprintf(path, sizeof path, "%s/%07d", dir, step);
	if (access(path, F_OK) == -1)
		mkdir(path, 0700);

	if ((fp = open_field(dir, "coord", step)) == NULL)
		return MCLG_IO_ERROR;
	for (i = 0; i < nn; i++)
		fprintf(fp, "%e %e\n", L->X[i], L->X[nn + i]);
	fclose(fp);

	if ((fp = open_field(dir, "temperature", step)) == NULL)
		return MCLG_IO_ERROR;
	for (i = 0; i < nn; i++)
		fprintf(fp, "%e\n", T[i]);
	fclose(fp);

	if ((fp = open_field(dir, "stress", step)) == NULL)
		return MCLG_IO_ERROR;
	for (i = 0; i < nn; i++)
		fprintf(fp, "%e\n", stress[i] / 1e6);
	fclose(fp);

	if ((fp = open_field(dir, "viscosity", step)) == NULL)
		return MCLG_IO_ERROR;
	for (i = 0; i < nn; i++)
		fprintf(fp, "%e\n", vis[i]);
	fclose(fp);

	if ((fp = open_field(dir, "velocity", step)) == NULL)
		return MCLG_IO_ERROR;
	for (i = 0; i < nn; i++)
		fprintf(fp, "%+e %+e\n", V0[i], V1[i]);
	fclose(fp);
	return MCLG_OK;
}
