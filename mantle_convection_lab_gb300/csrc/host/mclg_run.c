/*
 * mclg_run <file.input> -- the reference's driver (Main.c:3-80) over the C ABI.
 *
 * Same sequence and same files: the mesh is built once (AMR=1 rebuilds the
 * same static mesh in the reference, Tree.c:95-99, so once is equivalent),
 * the initial temperature is set on step 0, and each step runs
 *     buoyancy_force, viscosity, velocity_pressure_KGF_matrix,
 *     solve_velocity_pressure, output (every save_spacing steps), update_temperature
 * for timestep = 0 .. max_timestep (max_timestep + 1 solves, Main.c:28).
 * Per-step progress goes to stderr as in Main.c:30-31; the Uzawa and heat CG
 * iteration counts go to stdout as Solver.c:224-225 and
 * Update_temperature.c:1254-1255 print them.  Failures return a nonzero exit
 * code instead of the reference's exit(0).
 */
#include <stdio.h>
#include <stdlib.h>
#include <time.h>
#include "mclg.h"

static double now(void)
{
	struct timespec ts;
	clock_gettime(CLOCK_MONOTONIC, &ts);
	return (double)ts.tv_sec + 1e-9 * (double)ts.tv_nsec;
}

int main(int argc, char **argv)
{
	mclg_config cfg;
	mclg_ctx *ctx = NULL;
	mclg_step_stats st;
	int rc, ts;
	double t0;
	if (argc < 2) {
		fprintf(stderr, "Usage: mclg_run inputfile\n");
		return 10;
	}
	rc = mclg_config_from_input(argv[1], &cfg);
	if (rc != MCLG_OK) {
		fprintf(stderr, "File: %s is unreadable (%s)\n", argv[1], mclg_last_error());
		return 11;
	}
	t0 = now();
	rc = mclg_create(&ctx, &cfg);
	if (rc != MCLG_OK) {
		fprintf(stderr, "mclg_create: %s: %s\n", mclg_status_string(rc), mclg_last_error());
		return 20 + rc;
	}
	rc = mclg_initial_temperature(ctx);
	if (rc != MCLG_OK) {
		fprintf(stderr, "initial temperature: %s: %s\n", mclg_status_string(rc), mclg_last_error());
		mclg_destroy(ctx);
		return 20 + rc;
	}
	for (ts = 0; ts <= cfg.max_timestep; ts++) {
		fprintf(stderr, "\ntimestep = %d, CPU time = %.0fs, model time = %e\n", ts, now() - t0,
		        ts == 0 ? 0.0 : st.model_time);
		rc = mclg_step(ctx, 1, &st);
		if (rc != MCLG_OK && rc != MCLG_CAP_REACHED) {
			fprintf(stderr, "step %d: %s: %s\n", ts, mclg_status_string(rc), mclg_last_error());
			mclg_destroy(ctx);
			return 20 + rc;
		}
		printf("%d dv = %.10e dp = %.10e\n", st.uzawa_cycles, st.dv, st.dp);
		printf("Temperature CG cycle = %d\n", st.heat_cg_cycles);
		if (st.status == MCLG_NAN || st.status == MCLG_BREAKDOWN)
			fprintf(stderr, "step %d: solver status: %s\n", ts, mclg_status_string(st.status));
	}
	rc = mclg_output_wait(ctx);   /* the last steps' files */
	if (rc != MCLG_OK) {
		fprintf(stderr, "output: %s: %s\n", mclg_status_string(rc), mclg_last_error());
		mclg_destroy(ctx);
		return 20 + rc;
	}
	fprintf(stderr, "%f seconds of CPU time used in total\n", now() - t0);
	mclg_destroy(ctx);
	return 0;
}
