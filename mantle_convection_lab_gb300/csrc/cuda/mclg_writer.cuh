// Asynchronous output writer (mclg_writer.cu).
#pragma once
#include <stddef.h>
#include <cuda_runtime.h>
#include "../host/mclg_host.h"

namespace mclg {

struct OutWriter;

OutWriter *writer_new();
// Stage T, V (node double2), stress, vis, P and the model time into pinned
// memory on stream st and queue the files of `flags` (MCLG_OUT_TEXT,
// MCLG_OUT_BINARY) for <dir>/<timestep>/.  Waits while both slots are in use.
// L (the mesh level) must stay alive until writer_wait returns.
int writer_submit(OutWriter *w, cudaStream_t st, const mclg_level *L, const char *dir, int timestep, int flags,
                  const double *T, const double2 *V, const double *stress, const double *vis, const double *P,
                  size_t ne, const double *model_time);
// Every queued output written; returns (and clears) the first error of any.
int writer_wait(OutWriter *w);
void writer_free(OutWriter *w);

}  // namespace mclg
