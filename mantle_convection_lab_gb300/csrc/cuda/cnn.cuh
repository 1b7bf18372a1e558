// Learned initial guess: the CNN (k_cnn.cu) as the context sees it.
#pragma once
#include <cuda_runtime.h>

struct mclg_cnn;

namespace mclg {

constexpr int kCnnMaxLayers = 8;
constexpr int kCnnMaxC = 48;       // widest layer the kernels take
constexpr int kGuessCin = 8;       // T, log10 eta, u1, w1, p1, u2, w2, p2
constexpr int kGuessCout = 3;      // du, dw, dp

// Activation buffers for one forward pass of batch B on an H x W grid.
struct CnnWork {
	int B, H, W;
	float *act[kCnnMaxLayers + 1];   // act[0] is the caller's input; act[nl] the output
};

int cnn_work_ensure(const mclg_cnn *net, CnnWork &w, int B, int H, int W);
void cnn_work_free(CnnWork &w);
int cnn_forward_dev(const mclg_cnn *net, CnnWork &w, const float *x, cudaStream_t st);
int cnn_channels(const mclg_cnn *net, int *cin, int *cout);
const float *cnn_output(const mclg_cnn *net, const CnnWork &w);
int cnn_layers(const mclg_cnn *net);

// Features and targets on the (Nc+1)^2 node grid of a uniform N0 x N0 mesh,
// s = N0 / Nc.  Node arrays are x-major (A = iz + ix*(N0+1)), pressures Morton.
void guess_features(cudaStream_t st, int N0, int s, const double *T, const double *vis, const double2 *d1,
                    const double *p1, const double2 *d2, const double *p2, float *X, double *scale);
void guess_smooth(cudaStream_t st, int nc, int passes, float *Y, float *tmp);   // 2 x passes filter sweeps
void guess_apply(cudaStream_t st, int N0, int s, const float *Y, const double *scale, const unsigned char *mask0,
                 const double2 *d1, const double *p1, double2 *d, double *p);
void guess_extrapolate(cudaStream_t st, int nn, int ne, const unsigned char *mask0, const double2 *d1,
                       const double *p1, const double2 *d2, const double *p2, double2 *d, double *p);
void guess_target(cudaStream_t st, int N0, int s, const double2 *d, const double *p, const double2 *d1,
                  const double *p1, const double2 *d2, const double *p2, const double *scale, float *Yt);

}  // namespace mclg
