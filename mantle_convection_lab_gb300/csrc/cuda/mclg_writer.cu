// Output off the critical path: the reference's output() (Output.c:4-156)
// formats five text files per saved step inside the time loop.  Here the
// fields are copied to pinned host memory on the model's stream (ordered
// before the kernels that next overwrite them), and a writer thread waits for
// the copies and formats the files -- one thread per file -- while the GPU
// carries on with the following steps.  Two staging slots bound the memory; a
// third output waits for the oldest.  The text is byte for byte Output.c's
// (the same printf formats); an optional binary side-car keeps every field at
// full precision, pressure included, which the text files lack.
#include <stdint.h>
#include <stdio.h>
#include <string.h>
#include <condition_variable>
#include <deque>
#include <mutex>
#include <string>
#include <thread>
#include <vector>
#include <cuda_runtime.h>
#include "mclg_writer.cuh"

namespace mclg {

namespace {

struct Slot {
	double *pin = nullptr;      // T | V (2 nn) | stress | vis | P | model_time
	size_t cap = 0;             // doubles
	cudaEvent_t ev = nullptr;
	bool busy = false;
};

struct Job {
	int slot, timestep, flags;
	std::string dir;
	const mclg_level *L;
	size_t nn, ne;
};

}  // namespace

struct OutWriter {
	Slot slot[2];
	std::deque<Job> q;
	std::mutex mu;
	std::condition_variable cv;
	std::thread th;
	bool stop = false;
	int pending = 0;
	int err = MCLG_OK;
	std::string err_msg;
};

static const char kBinMagic[8] = {'M', 'C', 'L', 'G', 'O', 'U', 'T', '1'};

static int write_binary(const Job &j, const double *h)
{
	const size_t nn = j.nn, ne = j.ne;
	char path[2048];
	snprintf(path, sizeof path, "%s/%07d/fields.%d.%07d.bin", j.dir.c_str(), j.timestep, 0, j.timestep);
	FILE *f = fopen(path, "wb");
	if (f == NULL) {
		mclg_set_error("cannot open file %s", path);
		return MCLG_IO_ERROR;
	}
	const int32_t hd[4] = {1, (int32_t)nn, (int32_t)ne, j.timestep};
	const double *T = h, *V = h + nn, *S = h + 3 * nn, *vis = h + 4 * nn, *P = h + 5 * nn;
	const double model_time = h[5 * nn + ne];
	std::vector<double> comp(nn);
	bool ok = fwrite(kBinMagic, 1, 8, f) == 8 && fwrite(hd, sizeof hd, 1, f) == 1 &&
	          fwrite(&model_time, sizeof(double), 1, f) == 1 && fwrite(j.L->X, sizeof(double), 2 * nn, f) == 2 * nn &&
	          fwrite(T, sizeof(double), nn, f) == nn;
	for (int c = 0; c < 2 && ok; c++) {
		for (size_t i = 0; i < nn; i++)
			comp[i] = V[2 * i + c];
		ok = fwrite(comp.data(), sizeof(double), nn, f) == nn;
	}
	ok = ok && fwrite(P, sizeof(double), ne, f) == ne && fwrite(S, sizeof(double), nn, f) == nn &&
	     fwrite(vis, sizeof(double), nn, f) == nn;
	if (fclose(f) != 0 || !ok) {
		mclg_set_error("writing %s failed", path);
		return MCLG_IO_ERROR;
	}
	return MCLG_OK;
}

static void run_job(OutWriter *w, const Job &j)
{
	Slot &s = w->slot[j.slot];
	int rc = MCLG_OK;
	std::string msg;
	cudaError_t e = cudaEventSynchronize(s.ev);
	if (e != cudaSuccess) {
		rc = MCLG_CUDA_ERROR;
		msg = std::string("output copy: ") + cudaGetErrorString(e);
	} else {
		const size_t nn = j.nn;
		const double *h = s.pin, *V = h + nn;
		std::vector<double> V0(nn), V1(nn);
		for (size_t i = 0; i < nn; i++) {
			V0[i] = V[2 * i];
			V1[i] = V[2 * i + 1];
		}
		mclg_output_dirs(j.dir.c_str(), j.timestep);
		int frc[6] = {MCLG_OK, MCLG_OK, MCLG_OK, MCLG_OK, MCLG_OK, MCLG_OK};
		std::string fmsg[6];
		std::vector<std::thread> files;
		if (j.flags & MCLG_OUT_TEXT)
			for (int k = 0; k < 5; k++)
				files.emplace_back([&, k]() {
					frc[k] = mclg_write_output_file(j.dir.c_str(), j.timestep, k, j.L, h, V0.data(), V1.data(),
					                                h + 3 * nn, h + 4 * nn);
					if (frc[k])
						fmsg[k] = mclg_last_error();
				});
		if (j.flags & MCLG_OUT_BINARY) {
			frc[5] = write_binary(j, h);
			if (frc[5])
				fmsg[5] = mclg_last_error();
		}
		for (auto &t : files)
			t.join();
		for (int k = 0; k < 6 && rc == MCLG_OK; k++)
			if (frc[k]) {
				rc = frc[k];
				msg = fmsg[k];
			}
	}
	std::lock_guard<std::mutex> lk(w->mu);
	if (rc && w->err == MCLG_OK) {
		w->err = rc;
		w->err_msg = msg;
	}
	s.busy = false;
	w->pending--;
	w->cv.notify_all();
}

static void writer_main(OutWriter *w)
{
	for (;;) {
		Job j;
		{
			std::unique_lock<std::mutex> lk(w->mu);
			w->cv.wait(lk, [w] { return w->stop || !w->q.empty(); });
			if (w->q.empty())
				return;
			j = w->q.front();
			w->q.pop_front();
		}
		run_job(w, j);
	}
}

OutWriter *writer_new()
{
	OutWriter *w = new OutWriter();
	w->th = std::thread(writer_main, w);
	return w;
}

int writer_submit(OutWriter *w, cudaStream_t st, const mclg_level *L, const char *dir, int timestep, int flags,
                  const double *T, const double2 *V, const double *stress, const double *vis, const double *P,
                  size_t ne, const double *model_time)
{
	const size_t nn = (size_t)L->nno, need = 5 * nn + ne + 1;
	int k;
	{
		std::unique_lock<std::mutex> lk(w->mu);
		if (w->err) {   // an earlier output failed: report it now
			const int rc = w->err;
			mclg_set_error("%s", w->err_msg.c_str());
			w->err = MCLG_OK;
			w->err_msg.clear();
			return rc;
		}
		w->cv.wait(lk, [w] { return !w->slot[0].busy || !w->slot[1].busy; });
		k = w->slot[0].busy ? 1 : 0;
		w->slot[k].busy = true;
	}
	Slot &s = w->slot[k];
	cudaError_t e = cudaSuccess;
	if (s.cap < need) {
		if (s.pin)
			cudaFreeHost(s.pin);
		s.pin = nullptr;
		s.cap = 0;
		e = cudaMallocHost((void **)&s.pin, need * sizeof(double));
		if (e == cudaSuccess)
			s.cap = need;
	}
	if (e == cudaSuccess && s.ev == nullptr)
		e = cudaEventCreateWithFlags(&s.ev, cudaEventDisableTiming);
	double *h = s.pin;
	const struct {
		double *dst;
		const void *src;
		size_t n;
	} cp[6] = {{h, T, nn}, {h + nn, V, 2 * nn}, {h + 3 * nn, stress, nn}, {h + 4 * nn, vis, nn},
	           {h + 5 * nn, P, ne}, {h + 5 * nn + ne, model_time, 1}};
	for (int i = 0; i < 6 && e == cudaSuccess; i++)
		e = cudaMemcpyAsync(cp[i].dst, cp[i].src, cp[i].n * sizeof(double), cudaMemcpyDeviceToHost, st);
	if (e == cudaSuccess)
		e = cudaEventRecord(s.ev, st);
	std::lock_guard<std::mutex> lk(w->mu);
	if (e != cudaSuccess) {
		s.busy = false;
		w->cv.notify_all();
		mclg_set_error("output staging: %s", cudaGetErrorString(e));
		return MCLG_CUDA_ERROR;
	}
	w->q.push_back(Job{k, timestep, flags, std::string(dir), L, nn, ne});
	w->pending++;
	w->cv.notify_all();
	return MCLG_OK;
}

int writer_wait(OutWriter *w)
{
	std::unique_lock<std::mutex> lk(w->mu);
	w->cv.wait(lk, [w] { return w->pending == 0; });
	const int rc = w->err;
	if (rc)
		mclg_set_error("%s", w->err_msg.c_str());
	w->err = MCLG_OK;
	w->err_msg.clear();
	return rc;
}

void writer_free(OutWriter *w)
{
	if (w == nullptr)
		return;
	writer_wait(w);
	{
		std::lock_guard<std::mutex> lk(w->mu);
		w->stop = true;
	}
	w->cv.notify_all();
	w->th.join();
	for (Slot &s : w->slot) {
		if (s.pin)
			cudaFreeHost(s.pin);
		if (s.ev)
			cudaEventDestroy(s.ev);
	}
	delete w;
}

}  // namespace mclg
