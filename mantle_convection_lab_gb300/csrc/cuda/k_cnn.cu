// Learned initial guess for the Stokes solve: a small fully convolutional
// network (3x3 convolutions, ReLU between layers, linear last layer) with
// hand-written forward, backward and Adam kernels.  The reference has no
// counterpart; the solver refines whatever guess it gets to the same
// residual, so the network only changes how many iterations that takes.
//
// Precision: BF16 weights (rounded from FP32 master copies after every Adam
// step), FP32 activations, biases and accumulation.
//
// Tensors are [B][C][H][W] with W contiguous.  The convolutions (forward, and
// backward-data with flipped weights) run on the tensor cores: a block covers a
// 16 x 16 output tile as an implicit GEMM, M = 256 pixels, N = the output
// channels, K = 9 taps x the input channels, in mma.sync.m16n8k16 steps with
// BF16 operands and FP32 accumulation.  The input tile (with its halo) is
// staged in shared memory as BF16, channels innermost, and the weights as
// [tap][out][in]; both are padded so that the fragment loads of a warp fall
// in 32 different banks.  So the convolution inputs (activations forward,
// gradients backward) are rounded to BF16 as the weights are.
// The weight gradient (FP32 inputs) is reduced in two deterministic stages
// (per-block partials, then a fixed-order sum over blocks).
#include <cuda_bf16.h>
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include "cnn.cuh"
#include "../host/mclg_host.h"
#include "../host/mclg_ic.h"

struct mclg_cnn {
	int nl;
	int cin[mclg::kCnnMaxLayers], cout[mclg::kCnnMaxLayers];
	size_t off[mclg::kCnnMaxLayers];        // start of layer l in the flat parameter array: W[co][ci][9], b[co]
	size_t nparam;
	float *master, *grad, *m, *v;           // device, [nparam]
	__nv_bfloat16 *wf[mclg::kCnnMaxLayers]; // forward weights  [9][co_pad(cout)][ci_pad(cin)]
	__nv_bfloat16 *wb[mclg::kCnnMaxLayers]; // backward weights [9 flipped][co_pad(cin)][ci_pad(cout)]
	long long adam_t;
	float *part;                            // weight-gradient partials
	size_t part_cap;
	cudaStream_t st;
};

namespace mclg {

constexpr int kTile = 16;
constexpr int kHalo = kTile + 2;
constexpr int kChunk = 16;
constexpr int kWgradBlocks = 304;

static int pad_channels(int c)
{
	return c <= 4 ? 4 : c <= 8 ? 8 : c <= 16 ? 16 : c <= 32 ? 32 : 48;
}

// channel padding of the tensor-core convolution: K steps of 16 input
// channels, N tiles of 8 output channels
static int ci_pad(int c) { return c <= 16 ? 16 : 32; }
static int co_pad(int c) { return c <= 8 ? 8 : c <= 16 ? 16 : 32; }

static int cnn_fail(cudaError_t e, const char *what)
{
	mclg_set_error("%s: %s", what, cudaGetErrorString(e));
	return MCLG_CUDA_ERROR;
}

#define CKC(call)                                 \
	do {                                          \
		cudaError_t e_ = (call);                  \
		if (e_ != cudaSuccess)                    \
			return cnn_fail(e_, #call);           \
	} while (0)

// ---- convolution (forward, and backward-data with flipped weights) -----------
// out[b][o][y][x] = bias[o] + sum_c sum_k w[k][o][c] * in[b][c][y+ky-1][x+kx-1]
// (w and in rounded to BF16, FP32 accumulation), then ReLU (relu != 0) and/or
// a multiply by (mask > 0) (mask != null).  CI >= Cin input channels (a
// multiple of 16), CO >= Cout output channels (a multiple of 8).
__device__ __forceinline__ void mma_bf16_16816(float (&d)[4], unsigned a0, unsigned a1, unsigned a2, unsigned a3,
                                               unsigned b0, unsigned b1)
{
	asm volatile("mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
	             "{%0,%1,%2,%3};\n"
	             : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
	             : "r"(a0), "r"(a1), "r"(a2), "r"(a3), "r"(b0), "r"(b1));
}

template <int CI, int CO>
__global__ void __launch_bounds__(256) k_conv3x3(const float *__restrict__ in, int Cin,
                                                 const __nv_bfloat16 *__restrict__ w, const float *__restrict__ bias,
                                                 float *__restrict__ out, int Cout, int H, int W, int relu,
                                                 const float *__restrict__ mask)
{
	// channel stride of a pixel (and of an output channel's weights) in shared
	// memory: CI + 8 BF16 puts the 8 rows of a fragment in distinct banks
	constexpr int SI = CI + 8, NT = CO / 8;
	__shared__ __align__(16) __nv_bfloat16 s_in[kHalo * kHalo * SI];
	__shared__ __align__(16) __nv_bfloat16 s_w[9 * CO * SI];
	const int x0 = blockIdx.x * kTile, y0 = blockIdx.y * kTile, b = blockIdx.z;
	for (int i = threadIdx.x; i < CI * kHalo * kHalo; i += blockDim.x) {
		const int c = i / (kHalo * kHalo), r = i - c * kHalo * kHalo;
		const int yy = r / kHalo, xx = r - yy * kHalo;
		const int gy = y0 + yy - 1, gx = x0 + xx - 1;
		float v = 0.f;
		if (c < Cin && gy >= 0 && gy < H && gx >= 0 && gx < W)
			v = in[((size_t)(b * Cin + c) * H + gy) * W + gx];
		s_in[r * SI + c] = __float2bfloat16_rn(v);
	}
	for (int i = threadIdx.x; i < 9 * CO * CI; i += blockDim.x) {
		const int kc = i / CI, c = i - kc * CI;
		s_w[kc * SI + c] = w[i];
	}
	__syncthreads();
	const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
	const int g = lane >> 2, t2 = (lane & 3) * 2;
	float acc[2][NT][4];
#pragma unroll
	for (int m = 0; m < 2; m++)
#pragma unroll
		for (int j = 0; j < NT; j++)
#pragma unroll
			for (int q = 0; q < 4; q++)
				acc[m][j][q] = 0.f;
	// warp w: output rows 2w and 2w+1, each an M tile of 16 pixels
#pragma unroll 1
	for (int k = 0; k < 9; k++) {
		const int ky = k / 3, kx = k - 3 * (k / 3);
#pragma unroll
		for (int cb = 0; cb < CI; cb += 16) {
			unsigned bfr[NT][2];
#pragma unroll
			for (int j = 0; j < NT; j++) {
				const __nv_bfloat16 *wr = s_w + (k * CO + j * 8 + g) * SI + cb + t2;
				bfr[j][0] = *reinterpret_cast<const unsigned *>(wr);
				bfr[j][1] = *reinterpret_cast<const unsigned *>(wr + 8);
			}
#pragma unroll
			for (int m = 0; m < 2; m++) {
				const int py = 2 * warp + m;
				const __nv_bfloat16 *r0 = s_in + ((py + ky) * kHalo + g + kx) * SI + cb + t2;
				const __nv_bfloat16 *r1 = r0 + 8 * SI;
				const unsigned a0 = *reinterpret_cast<const unsigned *>(r0);
				const unsigned a1 = *reinterpret_cast<const unsigned *>(r1);
				const unsigned a2 = *reinterpret_cast<const unsigned *>(r0 + 8);
				const unsigned a3 = *reinterpret_cast<const unsigned *>(r1 + 8);
#pragma unroll
				for (int j = 0; j < NT; j++)
					mma_bf16_16816(acc[m][j], a0, a1, a2, a3, bfr[j][0], bfr[j][1]);
			}
		}
	}
	// D fragment: rows g (pixels x0+g) and g+8, columns t2, t2+1 of the N tile
#pragma unroll
	for (int m = 0; m < 2; m++) {
		const int y = y0 + 2 * warp + m;
		if (y >= H)
			continue;
#pragma unroll
		for (int j = 0; j < NT; j++)
#pragma unroll
			for (int q = 0; q < 4; q++) {
				const int x = x0 + g + (q >= 2 ? 8 : 0), o = j * 8 + t2 + (q & 1);
				if (x >= W || o >= Cout)
					continue;
				const size_t idx = ((size_t)(b * Cout + o) * H + y) * W + x;
				float v = acc[m][j][q] + (bias ? bias[o] : 0.f);
				if (relu)
					v = fmaxf(v, 0.f);
				if (mask && !(mask[idx] > 0.f))
					v = 0.f;
				out[idx] = v;
			}
	}
}

// ---- weight gradient: per-block partials ------------------------------------
// part[blk][(c*9 + k)*CO + o] = sum over the block's pixels of g[b][o][p] * in[b][c][p + k - 1],
// part[blk][Cin*9*CO + o]    = sum of g[b][o][p].
template <int CO>
__global__ void __launch_bounds__(256) k_conv3x3_wgrad(const float *__restrict__ in, int Cin,
                                                       const float *__restrict__ g, int Cout, int H, int W, int B,
                                                       float *__restrict__ part)
{
	extern __shared__ __align__(16) float smw[];
	float *s_in = smw;                              // [Cin][kHalo*kHalo]
	float *s_g = smw + Cin * kHalo * kHalo;         // [256][CO]
	constexpr int G = CO / 4;                        // float4 groups of output channels
	constexpr int U = (32 * 9 * G + 255) / 256;      // work units per thread (Cin <= 32)
	const int tilesx = (W + kTile - 1) / kTile, tilesy = (H + kTile - 1) / kTile;
	const int nitems = tilesx * tilesy * B;
	const int nunits = Cin * 9 * G;
	float acc[U][4];
	float bacc = 0.f;
#pragma unroll
	for (int u = 0; u < U; u++)
		acc[u][0] = acc[u][1] = acc[u][2] = acc[u][3] = 0.f;
	for (int item = blockIdx.x; item < nitems; item += gridDim.x) {
		const int b = item / (tilesx * tilesy), t = item - b * tilesx * tilesy;
		const int y0 = (t / tilesx) * kTile, x0 = (t - (t / tilesx) * tilesx) * kTile;
		__syncthreads();
		for (int i = threadIdx.x; i < Cin * kHalo * kHalo; i += blockDim.x) {
			const int ci = i / (kHalo * kHalo), r = i - ci * kHalo * kHalo;
			const int yy = r / kHalo, xx = r - yy * kHalo;
			const int gy = y0 + yy - 1, gx = x0 + xx - 1;
			float v = 0.f;
			if (gy >= 0 && gy < H && gx >= 0 && gx < W)
				v = in[((size_t)(b * Cin + ci) * H + gy) * W + gx];
			s_in[i] = v;
		}
		for (int i = threadIdx.x; i < kTile * kTile * CO; i += blockDim.x) {
			const int o = i / (kTile * kTile), px = i - o * kTile * kTile;
			const int y = y0 + px / kTile, x = x0 + (px & (kTile - 1));
			float v = 0.f;
			if (o < Cout && y < H && x < W)
				v = g[((size_t)(b * Cout + o) * H + y) * W + x];
			s_g[px * CO + o] = v;
		}
		__syncthreads();
#pragma unroll
		for (int u = 0; u < U; u++) {
			const int unit = threadIdx.x + 256 * u;
			if (unit < nunits) {
				const int pair = unit / G, grp = unit - pair * G;
				const int ci = pair / 9, k = pair - ci * 9, ky = k / 3, kx = k - 3 * ky;
				const float *sx = s_in + ci * kHalo * kHalo + ky * kHalo + kx;
				const float4 *sg = reinterpret_cast<const float4 *>(s_g) + grp;
				float a0 = acc[u][0], a1 = acc[u][1], a2 = acc[u][2], a3 = acc[u][3];
				for (int py = 0; py < kTile; py++)
#pragma unroll 4
					for (int px = 0; px < kTile; px++) {
						const float xv = sx[py * kHalo + px];
						const float4 gv = sg[(py * kTile + px) * G];
						a0 = fmaf(gv.x, xv, a0);
						a1 = fmaf(gv.y, xv, a1);
						a2 = fmaf(gv.z, xv, a2);
						a3 = fmaf(gv.w, xv, a3);
					}
				acc[u][0] = a0;
				acc[u][1] = a1;
				acc[u][2] = a2;
				acc[u][3] = a3;
			}
		}
		if (threadIdx.x < Cout)
			for (int px = 0; px < kTile * kTile; px++)
				bacc += s_g[px * CO + threadIdx.x];
	}
	float *pb = part + (size_t)blockIdx.x * (Cin * 9 * CO + CO);
#pragma unroll
	for (int u = 0; u < U; u++) {
		const int unit = threadIdx.x + 256 * u;
		if (unit < nunits) {
			const int pair = unit / G, grp = unit - pair * G;
#pragma unroll
			for (int q = 0; q < 4; q++)
				pb[pair * CO + grp * 4 + q] = acc[u][q];
		}
	}
	if (threadIdx.x < CO)
		pb[Cin * 9 * CO + threadIdx.x] = threadIdx.x < Cout ? bacc : 0.f;
}

// Fixed-order sum of the partials into the flat gradient W[o][c][k], b[o].
__global__ void k_wgrad_reduce(const float *__restrict__ part, int nblk, int Cin, int Cout, int CO,
                               float *__restrict__ grad)
{
	const int nw = Cout * Cin * 9, n = nw + Cout, stride = Cin * 9 * CO + CO;
	for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
		int src;
		if (i < nw) {
			const int o = i / (Cin * 9), r = i - o * Cin * 9;   // r = c*9 + k
			src = r * CO + o;
		} else {
			src = Cin * 9 * CO + (i - nw);
		}
		float s = 0.f;
		for (int bk = 0; bk < nblk; bk++)
			s += part[(size_t)bk * stride + src];
		grad[i] = s;
	}
}

// ---- loss, optimiser, weight packing ------------------------------------------
// Mean squared error over all entries; g = d loss / d y.  Per-block partial
// sums in double, then one block sums them in order.
__global__ void k_mse(const float *__restrict__ y, const float *__restrict__ t, size_t n, float *__restrict__ g,
                      double *__restrict__ part)
{
	__shared__ double sh[256];
	double s = 0.0;
	const float inv = 2.f / (float)n;
	for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
		const float d = y[i] - t[i];
		g[i] = inv * d;
		s += (double)d * (double)d;
	}
	sh[threadIdx.x] = s;
	__syncthreads();
	for (int w = blockDim.x / 2; w > 0; w >>= 1) {
		if (threadIdx.x < w)
			sh[threadIdx.x] += sh[threadIdx.x + w];
		__syncthreads();
	}
	if (threadIdx.x == 0)
		part[blockIdx.x] = sh[0];
}

__global__ void k_sum_partials(const double *__restrict__ part, int n, double scale, double *__restrict__ out)
{
	if (threadIdx.x == 0 && blockIdx.x == 0) {
		double s = 0.0;
		for (int i = 0; i < n; i++)
			s += part[i];
		out[0] = s * scale;
	}
}

__global__ void k_adam(float *__restrict__ w, const float *__restrict__ g, float *__restrict__ m,
                       float *__restrict__ v, size_t n, float lr, float b1, float b2, float eps, float c1, float c2)
{
	for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
		const float gi = g[i];
		const float mi = b1 * m[i] + (1.f - b1) * gi;
		const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
		m[i] = mi;
		v[i] = vi;
		w[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
	}
}

// Weights of the tensor-core convolutions, zero padded:
//   wf[k][o][c] = bf16(W[o][c][k])      o < co_pad(Cout) = NO, c < ci_pad(Cin) = NC
//   wb[k][c][o] = bf16(W[o][c][8 - k])  c < co_pad(Cin) = BO,  o < ci_pad(Cout) = BC
__global__ void k_pack(const float *__restrict__ W, int Cin, int Cout, int NO, int NC, int BO, int BC,
                       __nv_bfloat16 *__restrict__ wf, __nv_bfloat16 *__restrict__ wb)
{
	const int nf = 9 * NO * NC, nb = 9 * BO * BC;
	for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nf + nb; i += gridDim.x * blockDim.x) {
		if (i < nf) {
			const int k = i / (NO * NC), r = i - k * NO * NC, o = r / NC, c = r - o * NC;
			wf[i] = __float2bfloat16_rn(o < Cout && c < Cin ? W[(o * Cin + c) * 9 + k] : 0.f);
		} else {
			const int j = i - nf;
			const int k = j / (BO * BC), r = j - k * BO * BC, c = r / BC, o = r - c * BC;
			wb[j] = __float2bfloat16_rn(o < Cout && c < Cin ? W[(o * Cin + c) * 9 + (8 - k)] : 0.f);
		}
	}
}

// ---- launch helpers -----------------------------------------------------------
// w is packed for (ci_pad(Cin), co_pad(Cout)) as k_pack lays it out.
static void conv_launch(const float *in, int Cin, const __nv_bfloat16 *w, const float *bias, float *out, int Cout,
                        int B, int H, int W, int relu, const float *mask, cudaStream_t st)
{
	dim3 grid((W + kTile - 1) / kTile, (H + kTile - 1) / kTile, B);
	const int ci = ci_pad(Cin), co = co_pad(Cout);
#define CONV_TC(CI_, CO_) k_conv3x3<CI_, CO_><<<grid, 256, 0, st>>>(in, Cin, w, bias, out, Cout, H, W, relu, mask)
	if (ci == 16)
		co == 8 ? CONV_TC(16, 8) : co == 16 ? CONV_TC(16, 16) : CONV_TC(16, 32);
	else
		co == 8 ? CONV_TC(32, 8) : co == 16 ? CONV_TC(32, 16) : CONV_TC(32, 32);
#undef CONV_TC
}

static size_t wgrad_smem(int Cin, int CO)
{
	return (size_t)(Cin * kHalo * kHalo + kTile * kTile * CO) * sizeof(float);
}

static cudaError_t wgrad_launch(const float *in, int Cin, const float *g, int Cout, int CO, int B, int H, int W,
                                float *part, int nblk, cudaStream_t st)
{
	const size_t sm = wgrad_smem(Cin, CO);
	cudaError_t e;
	switch (CO) {
	case 4:
		e = cudaFuncSetAttribute(k_conv3x3_wgrad<4>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
		if (e == cudaSuccess)
			k_conv3x3_wgrad<4><<<nblk, 256, sm, st>>>(in, Cin, g, Cout, H, W, B, part);
		break;
	case 8:
		e = cudaFuncSetAttribute(k_conv3x3_wgrad<8>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
		if (e == cudaSuccess)
			k_conv3x3_wgrad<8><<<nblk, 256, sm, st>>>(in, Cin, g, Cout, H, W, B, part);
		break;
	case 16:
		e = cudaFuncSetAttribute(k_conv3x3_wgrad<16>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
		if (e == cudaSuccess)
			k_conv3x3_wgrad<16><<<nblk, 256, sm, st>>>(in, Cin, g, Cout, H, W, B, part);
		break;
	default:
		e = cudaFuncSetAttribute(k_conv3x3_wgrad<32>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
		if (e == cudaSuccess)
			k_conv3x3_wgrad<32><<<nblk, 256, sm, st>>>(in, Cin, g, Cout, H, W, B, part);
		break;
	}
	return e;
}

static int pack_all(mclg_cnn *n)
{
	for (int l = 0; l < n->nl; l++) {
		const int NO = co_pad(n->cout[l]), NC = ci_pad(n->cin[l]), BO = co_pad(n->cin[l]), BC = ci_pad(n->cout[l]);
		const int nb = 9 * (NO * NC + BO * BC);
		k_pack<<<(nb + 255) / 256, 256, 0, n->st>>>(n->master + n->off[l], n->cin[l], n->cout[l], NO, NC, BO, BC,
		                                            n->wf[l], n->wb[l]);
	}
	CKC(cudaGetLastError());
	return MCLG_OK;
}

int cnn_channels(const mclg_cnn *net, int *cin, int *cout)
{
	*cin = net->cin[0];
	*cout = net->cout[net->nl - 1];
	return MCLG_OK;
}

const float *cnn_output(const mclg_cnn *net, const CnnWork &w)
{
	return w.act[net->nl];
}

int cnn_layers(const mclg_cnn *net)
{
	return net->nl;
}

void cnn_work_free(CnnWork &w)
{
	for (int l = 1; l <= kCnnMaxLayers; l++) {
		cudaFree(w.act[l]);
		w.act[l] = nullptr;
	}
	w.B = w.H = w.W = 0;
}

int cnn_work_ensure(const mclg_cnn *net, CnnWork &w, int B, int H, int W)
{
	if (w.B == B && w.H == H && w.W == W && w.act[net->nl] != nullptr)
		return MCLG_OK;
	cnn_work_free(w);
	for (int l = 0; l < net->nl; l++)
		CKC(cudaMalloc((void **)&w.act[l + 1], (size_t)B * net->cout[l] * H * W * sizeof(float)));
	w.B = B;
	w.H = H;
	w.W = W;
	return MCLG_OK;
}

int cnn_forward_dev(const mclg_cnn *net, CnnWork &w, const float *x, cudaStream_t st)
{
	w.act[0] = const_cast<float *>(x);
	for (int l = 0; l < net->nl; l++)
		conv_launch(w.act[l], net->cin[l], net->wf[l], net->master + net->off[l] + (size_t)net->cout[l] * net->cin[l] * 9,
		            w.act[l + 1], net->cout[l], w.B, w.H, w.W, l + 1 < net->nl, nullptr, st);
	CKC(cudaGetLastError());
	return MCLG_OK;
}

// Backward pass for the loss gradient gy (= d loss / d output) of the last
// forward pass in w; accumulates nothing: writes the flat gradient.
static int cnn_backward_dev(mclg_cnn *net, CnnWork &w, const float *gy, float *gbuf0, float *gbuf1, cudaStream_t st)
{
	const float *gz = gy;
	float *bufs[2] = {gbuf0, gbuf1};
	for (int l = net->nl - 1; l >= 0; l--) {
		const int Cin = net->cin[l], Cout = net->cout[l], CO = pad_channels(Cout);
		const int tiles = ((w.W + kTile - 1) / kTile) * ((w.H + kTile - 1) / kTile) * w.B;
		const int nblk = tiles < kWgradBlocks ? tiles : kWgradBlocks;
		const size_t need = (size_t)nblk * (Cin * 9 * CO + CO);
		if (need > net->part_cap) {
			cudaFree(net->part);
			net->part = nullptr;
			CKC(cudaMalloc((void **)&net->part, need * sizeof(float)));
			net->part_cap = need;
		}
		CKC(wgrad_launch(w.act[l], Cin, gz, Cout, CO, w.B, w.H, w.W, net->part, nblk, st));
		const int n = Cout * Cin * 9 + Cout;
		k_wgrad_reduce<<<(n + 255) / 256, 256, 0, st>>>(net->part, nblk, Cin, Cout, CO, net->grad + net->off[l]);
		if (l > 0) {
			// d loss / d z_{l-1} = (W_l^T g_l) masked by ReLU'(z_{l-1}) = (act_l > 0)
			float *gin = bufs[l & 1];
			conv_launch(gz, Cout, net->wb[l], nullptr, gin, Cin, w.B, w.H, w.W, 0, w.act[l], st);
			gz = gin;
		}
	}
	CKC(cudaGetLastError());
	return MCLG_OK;
}

// ---- features of the learned guess ----------------------------------------------
__device__ __forceinline__ unsigned spread_bits_c(unsigned v)
{
	v &= 0xffffu;
	v = (v | (v << 8)) & 0x00ff00ffu;
	v = (v | (v << 4)) & 0x0f0f0f0fu;
	v = (v | (v << 2)) & 0x33333333u;
	v = (v | (v << 1)) & 0x55555555u;
	return v;
}

__device__ __forceinline__ int morton_c(int ex, int ez)
{
	return (int)((spread_bits_c((unsigned)ex) << 1) | spread_bits_c((unsigned)ez));
}

// Mean over the fine elements of the dual cell of coarse node (cx, cz) of
// p, p - q (q != null) or p - 2 q + r (q, r != null).
__device__ double dual_mean(const double *p, const double *q, const double *r, int N0, int s, int cx, int cz)
{
	const int ex0 = max(cx * s - s, 0), ex1 = min(cx * s + s, N0);
	const int ez0 = max(cz * s - s, 0), ez1 = min(cz * s + s, N0);
	double sum = 0.0;
	for (int ex = ex0; ex < ex1; ex++)
		for (int ez = ez0; ez < ez1; ez++) {
			const int e = morton_c(ex, ez);
			sum += r ? p[e] - 2.0 * q[e] + r[e] : q ? p[e] - q[e] : p[e];
		}
	return sum / (double)((ex1 - ex0) * (ez1 - ez0));
}

// X[c][cx][cz] before scaling: T, 0.2 log10 eta, u1, w1, p1, u1 - u2,
// w1 - w2, p1 - p2 (velocities injected, pressures dual-cell means).
// The differences are formed in FP64 here: in the network's FP32/BF16
// arithmetic they would vanish against u1 and u2.
__global__ void k_guess_raw(int N0, int s, const double *__restrict__ T, const double *__restrict__ vis,
                            const double2 *__restrict__ d1, const double *__restrict__ p1,
                            const double2 *__restrict__ d2, const double *__restrict__ p2, float *__restrict__ X)
{
	const int nc = N0 / s + 1, n0 = N0 + 1, plane = nc * nc;
	for (int A = blockIdx.x * blockDim.x + threadIdx.x; A < plane; A += gridDim.x * blockDim.x) {
		const int cx = A / nc, cz = A - cx * nc;
		const int F = cz * s + cx * s * n0;
		const double2 a = d1[F], b = d2[F];
		X[0 * plane + A] = (float)T[F];
		X[1 * plane + A] = (float)(0.2 * log10(vis[F]));
		X[2 * plane + A] = (float)a.x;
		X[3 * plane + A] = (float)a.y;
		X[4 * plane + A] = (float)dual_mean(p1, nullptr, nullptr, N0, s, cx, cz);
		X[5 * plane + A] = (float)(a.x - b.x);
		X[6 * plane + A] = (float)(a.y - b.y);
		X[7 * plane + A] = (float)dual_mean(p1, p2, nullptr, N0, s, cx, cz);
	}
}

// RMS of the (u, w) pair in channels c, c+1 and of the pressure in channel
// c+2, floored; those channels are divided by them.
// scale = {speed of the last solution, its pressure, speed of the last change, pressure of the last change}.
__global__ void __launch_bounds__(1024) k_guess_scale(float *__restrict__ X, int plane, double *__restrict__ scale)
{
	__shared__ double sh[4][1024];
	double a[4] = {0.0, 0.0, 0.0, 0.0};
	for (int A = threadIdx.x; A < plane; A += blockDim.x) {
		const double u = X[2 * plane + A], w = X[3 * plane + A], p = X[4 * plane + A];
		const double du = X[5 * plane + A], dw = X[6 * plane + A], dp = X[7 * plane + A];
		a[0] += u * u + w * w;
		a[1] += p * p;
		a[2] += du * du + dw * dw;
		a[3] += dp * dp;
	}
	for (int q = 0; q < 4; q++)
		sh[q][threadIdx.x] = a[q];
	__syncthreads();
	for (int k = blockDim.x / 2; k > 0; k >>= 1) {
		if (threadIdx.x < k)
			for (int q = 0; q < 4; q++)
				sh[q][threadIdx.x] += sh[q][threadIdx.x + k];
		__syncthreads();
	}
	double sc[4];
	for (int q = 0; q < 4; q++)
		sc[q] = fmax(sqrt(sh[q][0] / plane), 1e-30);
	__syncthreads();
	if (threadIdx.x < 4)
		scale[threadIdx.x] = sc[threadIdx.x];
	const float i0 = (float)(1.0 / sc[0]), i1 = (float)(1.0 / sc[1]), i2 = (float)(1.0 / sc[2]),
	            i3 = (float)(1.0 / sc[3]);
	for (int A = threadIdx.x; A < plane; A += blockDim.x) {
		X[2 * plane + A] *= i0;
		X[3 * plane + A] *= i0;
		X[4 * plane + A] *= i1;
		X[5 * plane + A] *= i2;
		X[6 * plane + A] *= i2;
		X[7 * plane + A] *= i3;
	}
}

// Bilinear value of channel c of Y at coarse coordinates (fx, fz) (node units).
__device__ __forceinline__ double bilin(const float *__restrict__ Y, int nc, double fx, double fz)
{
	int ix = (int)floor(fx), iz = (int)floor(fz);
	ix = min(max(ix, 0), nc - 2);
	iz = min(max(iz, 0), nc - 2);
	const double ax = fx - ix, az = fz - iz;
	const double v00 = Y[iz + ix * nc], v01 = Y[iz + 1 + ix * nc], v10 = Y[iz + (ix + 1) * nc],
	             v11 = Y[iz + 1 + (ix + 1) * nc];
	return (1 - ax) * ((1 - az) * v00 + az * v01) + ax * ((1 - az) * v10 + az * v11);
}

__global__ void k_guess_apply(int N0, int s, const float *__restrict__ Y, const double *__restrict__ scale,
                              const unsigned char *__restrict__ mask0, const double2 *__restrict__ d1,
                              const double *__restrict__ p1, double2 *__restrict__ d, double *__restrict__ p)
{
	const int nc = N0 / s + 1, n0 = N0 + 1, plane = nc * nc, nn = n0 * n0, ne = N0 * N0;
	const double s_u = scale[2], s_p = scale[3], is = 1.0 / s;
	for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nn + ne; i += gridDim.x * blockDim.x) {
		if (i < nn) {
			const int ix = i / n0, iz = i - ix * n0;
			const double fx = ix * is, fz = iz * is;
			const unsigned m = mask0[i];
			const double2 a = d1[i];
			d[i] = make_double2((m & 1u) ? 0.0 : a.x + s_u * bilin(Y, nc, fx, fz),
			                    (m & 2u) ? 0.0 : a.y + s_u * bilin(Y + plane, nc, fx, fz));
		} else {
			const int e = i - nn, ex = e / N0, ez = e - ex * N0;
			const int me = morton_c(ex, ez);
			p[me] = p1[me] + s_p * bilin(Y + 2 * plane, nc, (ex + 0.5) * is, (ez + 0.5) * is);
		}
	}
}

// Target: the converged solution minus the base guess, 2 d1 - d2 when d2 is
// given (extrapolation) and d1 otherwise, scaled like the features.
__global__ void k_guess_target(int N0, int s, const double2 *__restrict__ d, const double *__restrict__ p,
                               const double2 *__restrict__ d1, const double *__restrict__ p1,
                               const double2 *__restrict__ d2, const double *__restrict__ p2,
                               const double *__restrict__ scale, float *__restrict__ Yt)
{
	const int nc = N0 / s + 1, n0 = N0 + 1, plane = nc * nc;
	const double iu = 1.0 / scale[2], ip = 1.0 / scale[3];
	for (int A = blockIdx.x * blockDim.x + threadIdx.x; A < plane; A += gridDim.x * blockDim.x) {
		const int cx = A / nc, cz = A - cx * nc;
		const int F = cz * s + cx * s * n0;
		const double2 a = d[F], b = d1[F];
		double bx = b.x, by = b.y;
		if (d2) {
			const double2 c = d2[F];
			bx = 2.0 * b.x - c.x;
			by = 2.0 * b.y - c.y;
		}
		Yt[A] = (float)((a.x - bx) * iu);
		Yt[plane + A] = (float)((a.y - by) * iu);
		Yt[2 * plane + A] = (float)(dual_mean(p, p1, d2 ? p2 : nullptr, N0, s, cx, cz) * ip);
	}
}

// d = 2 d1 - d2, p = 2 p1 - p2 (linear extrapolation in time of the last two solutions).
__global__ void k_guess_extrapolate(int nn, int ne, const unsigned char *__restrict__ mask0,
                                    const double2 *__restrict__ d1, const double *__restrict__ p1,
                                    const double2 *__restrict__ d2, const double *__restrict__ p2,
                                    double2 *__restrict__ d, double *__restrict__ p)
{
	for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nn + ne; i += gridDim.x * blockDim.x) {
		if (i < nn) {
			const double2 a = d1[i], b = d2[i];
			const unsigned m = mask0[i];
			d[i] = make_double2((m & 1u) ? 0.0 : 2.0 * a.x - b.x, (m & 2u) ? 0.0 : 2.0 * a.y - b.y);
		} else {
			const int e = i - nn;
			p[e] = 2.0 * p1[e] - p2[e];
		}
	}
}

// One pass of the separable binomial filter [1 2 1] x [1 2 1] / 16 over the
// channels of Y (coarse node grid, edge values repeated): removes the
// grid-scale part of the network's output before it is prolonged.
__global__ void k_guess_smooth(const float *__restrict__ Y, float *__restrict__ Z, int nc, int nch)
{
	const int plane = nc * nc;
	for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nch * plane; i += gridDim.x * blockDim.x) {
		const int c = i / plane, A = i - c * plane, cx = A / nc, cz = A - cx * nc;
		const float *y = Y + (size_t)c * plane;
		float acc = 0.f;
#pragma unroll
		for (int dx = -1; dx <= 1; dx++)
#pragma unroll
			for (int dz = -1; dz <= 1; dz++) {
				const int x = min(max(cx + dx, 0), nc - 1), z = min(max(cz + dz, 0), nc - 1);
				acc += (dx == 0 ? 2.f : 1.f) * (dz == 0 ? 2.f : 1.f) * y[z + x * nc];
			}
		Z[i] = acc * (1.f / 16.f);
	}
}

static int blocks_for_n(long long n)
{
	long long b = (n + 255) / 256;
	return (int)(b < 4096 ? (b > 0 ? b : 1) : 4096);
}

void guess_features(cudaStream_t st, int N0, int s, const double *T, const double *vis, const double2 *d1,
                    const double *p1, const double2 *d2, const double *p2, float *X, double *scale)
{
	const int nc = N0 / s + 1;
	k_guess_raw<<<blocks_for_n((long long)nc * nc), 256, 0, st>>>(N0, s, T, vis, d1, p1, d2, p2, X);
	k_guess_scale<<<1, 1024, 0, st>>>(X, nc * nc, scale);
}

void guess_smooth(cudaStream_t st, int nc, int passes, float *Y, float *tmp)
{
	for (int k = 0; k < passes; k++) {
		k_guess_smooth<<<blocks_for_n((long long)kGuessCout * nc * nc), 256, 0, st>>>(Y, tmp, nc, kGuessCout);
		k_guess_smooth<<<blocks_for_n((long long)kGuessCout * nc * nc), 256, 0, st>>>(tmp, Y, nc, kGuessCout);
	}
}

void guess_apply(cudaStream_t st, int N0, int s, const float *Y, const double *scale, const unsigned char *mask0,
                 const double2 *d1, const double *p1, double2 *d, double *p)
{
	const long long n = (long long)(N0 + 1) * (N0 + 1) + (long long)N0 * N0;
	k_guess_apply<<<blocks_for_n(n), 256, 0, st>>>(N0, s, Y, scale, mask0, d1, p1, d, p);
}

void guess_extrapolate(cudaStream_t st, int nn, int ne, const unsigned char *mask0, const double2 *d1,
                       const double *p1, const double2 *d2, const double *p2, double2 *d, double *p)
{
	k_guess_extrapolate<<<blocks_for_n((long long)nn + ne), 256, 0, st>>>(nn, ne, mask0, d1, p1, d2, p2, d, p);
}

void guess_target(cudaStream_t st, int N0, int s, const double2 *d, const double *p, const double2 *d1,
                  const double *p1, const double2 *d2, const double *p2, const double *scale, float *Yt)
{
	const int nc = N0 / s + 1;
	k_guess_target<<<blocks_for_n((long long)nc * nc), 256, 0, st>>>(N0, s, d, p, d1, p1, d2, p2, scale, Yt);
}

}  // namespace mclg

using namespace mclg;

// ---- C ABI ------------------------------------------------------------------------
extern "C" {

int mclg_cnn_create(mclg_cnn **out, int cin, int width, int depth, int cout, unsigned long long seed)
{
	if (out == NULL)
		return MCLG_BAD_INPUT;
	*out = NULL;
	if (depth < 2 || depth > kCnnMaxLayers || cin < 1 || cin > 32 || width < 1 || width > 32 || cout < 1 ||
	    cout > 32) {
		mclg_set_error("network shape cin=%d width=%d depth=%d cout=%d: need 2 <= depth <= %d and channels in [1, 32]",
		               cin, width, depth, cout, kCnnMaxLayers);
		return MCLG_BAD_INPUT;
	}
	int ndev = 0;
	if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
		cudaGetLastError();
		mclg_set_error("no CUDA device visible");
		return MCLG_NO_DEVICE;
	}
	mclg_cnn *n = (mclg_cnn *)calloc(1, sizeof(mclg_cnn));
	if (n == NULL)
		return MCLG_BAD_INPUT;
	n->nl = depth;
	size_t off = 0;
	for (int l = 0; l < depth; l++) {
		n->cin[l] = l == 0 ? cin : width;
		n->cout[l] = l == depth - 1 ? cout : width;
		n->off[l] = off;
		off += (size_t)n->cout[l] * n->cin[l] * 9 + n->cout[l];
	}
	n->nparam = off;
	// He-uniform weights from a Philox stream, last layer and biases zero
	// (the untrained network predicts no change).
	float *h = (float *)calloc(off, sizeof(float));
	for (int l = 0; l + 1 < depth; l++) {
		const double a = sqrt(6.0 / (9.0 * n->cin[l]));
		const size_t nw = (size_t)n->cout[l] * n->cin[l] * 9;
		for (size_t i = 0; i < nw; i++)
			h[n->off[l] + i] = (float)(a * (2.0 * mclg_uniform01(seed, 7u + (uint32_t)l, (uint32_t)i) - 1.0));
	}
	int rc = MCLG_OK;
	cudaError_t e = cudaStreamCreateWithFlags(&n->st, cudaStreamNonBlocking);
	if (e == cudaSuccess) e = cudaMalloc((void **)&n->master, off * sizeof(float));
	if (e == cudaSuccess) e = cudaMalloc((void **)&n->grad, off * sizeof(float));
	if (e == cudaSuccess) e = cudaMalloc((void **)&n->m, off * sizeof(float));
	if (e == cudaSuccess) e = cudaMalloc((void **)&n->v, off * sizeof(float));
	for (int l = 0; l < depth && e == cudaSuccess; l++) {
		e = cudaMalloc((void **)&n->wf[l], (size_t)9 * co_pad(n->cout[l]) * ci_pad(n->cin[l]) * sizeof(__nv_bfloat16));
		if (e == cudaSuccess)
			e = cudaMalloc((void **)&n->wb[l], (size_t)9 * co_pad(n->cin[l]) * ci_pad(n->cout[l]) * sizeof(__nv_bfloat16));
	}
	if (e == cudaSuccess) e = cudaMemcpyAsync(n->master, h, off * sizeof(float), cudaMemcpyHostToDevice, n->st);
	if (e == cudaSuccess) e = cudaMemsetAsync(n->m, 0, off * sizeof(float), n->st);
	if (e == cudaSuccess) e = cudaMemsetAsync(n->v, 0, off * sizeof(float), n->st);
	if (e == cudaSuccess) rc = pack_all(n);
	if (e == cudaSuccess && rc == MCLG_OK) e = cudaStreamSynchronize(n->st);
	free(h);
	if (e != cudaSuccess)
		rc = cnn_fail(e, "mclg_cnn_create");
	if (rc != MCLG_OK) {
		mclg_cnn_destroy(n);
		return rc;
	}
	*out = n;
	return MCLG_OK;
}

void mclg_cnn_destroy(mclg_cnn *n)
{
	if (n == NULL)
		return;
	if (n->st)
		cudaStreamSynchronize(n->st);
	cudaFree(n->master);
	cudaFree(n->grad);
	cudaFree(n->m);
	cudaFree(n->v);
	cudaFree(n->part);
	for (int l = 0; l < kCnnMaxLayers; l++) {
		cudaFree(n->wf[l]);
		cudaFree(n->wb[l]);
	}
	if (n->st)
		cudaStreamDestroy(n->st);
	free(n);
}

size_t mclg_cnn_num_params(const mclg_cnn *n)
{
	return n ? n->nparam : 0;
}

int mclg_cnn_shape(const mclg_cnn *n, int *cin, int *width, int *depth, int *cout)
{
	if (n == NULL)
		return MCLG_BAD_INPUT;
	if (cin) *cin = n->cin[0];
	if (width) *width = n->nl > 1 ? n->cout[0] : 0;
	if (depth) *depth = n->nl;
	if (cout) *cout = n->cout[n->nl - 1];
	return MCLG_OK;
}

int mclg_cnn_get_params(const mclg_cnn *n, float *out, size_t count)
{
	if (n == NULL || out == NULL || count != n->nparam) {
		mclg_set_error("parameter buffer has %zu entries, the network %zu", count, n ? n->nparam : 0);
		return MCLG_BAD_INPUT;
	}
	CKC(cudaMemcpyAsync(out, n->master, count * sizeof(float), cudaMemcpyDeviceToHost, n->st));
	CKC(cudaStreamSynchronize(n->st));
	return MCLG_OK;
}

int mclg_cnn_set_params(mclg_cnn *n, const float *in, size_t count)
{
	if (n == NULL || in == NULL || count != n->nparam) {
		mclg_set_error("parameter buffer has %zu entries, the network %zu", count, n ? n->nparam : 0);
		return MCLG_BAD_INPUT;
	}
	CKC(cudaMemcpyAsync(n->master, in, count * sizeof(float), cudaMemcpyHostToDevice, n->st));
	CKC(cudaMemsetAsync(n->m, 0, count * sizeof(float), n->st));
	CKC(cudaMemsetAsync(n->v, 0, count * sizeof(float), n->st));
	n->adam_t = 0;
	int rc = pack_all(n);
	if (rc)
		return rc;
	CKC(cudaStreamSynchronize(n->st));
	return MCLG_OK;
}

static int check_grid(const mclg_cnn *n, int batch, int h, int w)
{
	if (n == NULL || batch < 1 || h < 1 || w < 1 || (size_t)batch * h * w > ((size_t)1 << 31) / kCnnMaxC) {
		mclg_set_error("bad batch/grid %d x %d x %d", batch, h, w);
		return MCLG_BAD_INPUT;
	}
	return MCLG_OK;
}

int mclg_cnn_forward(mclg_cnn *n, const float *x, int batch, int h, int w, float *y)
{
	int rc = check_grid(n, batch, h, w);
	if (rc)
		return rc;
	if (x == NULL || y == NULL)
		return MCLG_BAD_INPUT;
	CnnWork wk;
	memset(&wk, 0, sizeof wk);
	float *dx = NULL;
	const size_t nx = (size_t)batch * n->cin[0] * h * w, ny = (size_t)batch * n->cout[n->nl - 1] * h * w;
	cudaError_t e = cudaMalloc((void **)&dx, nx * sizeof(float));
	if (e == cudaSuccess) e = cudaMemcpyAsync(dx, x, nx * sizeof(float), cudaMemcpyHostToDevice, n->st);
	if (e == cudaSuccess) rc = cnn_work_ensure(n, wk, batch, h, w);
	if (e == cudaSuccess && rc == MCLG_OK) rc = cnn_forward_dev(n, wk, dx, n->st);
	if (e == cudaSuccess && rc == MCLG_OK)
		e = cudaMemcpyAsync(y, wk.act[n->nl], ny * sizeof(float), cudaMemcpyDeviceToHost, n->st);
	if (e == cudaSuccess && rc == MCLG_OK) e = cudaStreamSynchronize(n->st);
	cudaFree(dx);
	cnn_work_free(wk);
	if (e != cudaSuccess)
		return cnn_fail(e, "mclg_cnn_forward");
	return rc;
}

// Loss and gradient of the mean squared error for one batch (host buffers).
int mclg_cnn_gradient(mclg_cnn *n, const float *x, const float *target, int batch, int h, int w, double *loss,
                      float *grad, size_t count)
{
	int rc = check_grid(n, batch, h, w);
	if (rc)
		return rc;
	if (x == NULL || target == NULL || grad == NULL || count != n->nparam) {
		mclg_set_error("gradient buffer has %zu entries, the network %zu", count, n->nparam);
		return MCLG_BAD_INPUT;
	}
	CnnWork wk;
	memset(&wk, 0, sizeof wk);
	const size_t nx = (size_t)batch * n->cin[0] * h * w, ny = (size_t)batch * n->cout[n->nl - 1] * h * w;
	size_t ng = 0;
	for (int l = 0; l < n->nl; l++)
		ng = ng > (size_t)n->cout[l] ? ng : (size_t)n->cout[l];
	ng *= (size_t)batch * h * w;
	float *dx = NULL, *dt = NULL, *gy = NULL, *g0 = NULL, *g1 = NULL;
	double *part = NULL, *dl = NULL;
	const int nb = 256;
	cudaError_t e = cudaMalloc((void **)&dx, nx * sizeof(float));
	if (e == cudaSuccess) e = cudaMalloc((void **)&dt, ny * sizeof(float));
	if (e == cudaSuccess) e = cudaMalloc((void **)&gy, ny * sizeof(float));
	if (e == cudaSuccess) e = cudaMalloc((void **)&g0, ng * sizeof(float));
	if (e == cudaSuccess) e = cudaMalloc((void **)&g1, ng * sizeof(float));
	if (e == cudaSuccess) e = cudaMalloc((void **)&part, (nb + 1) * sizeof(double));
	dl = part + nb;
	if (e == cudaSuccess) e = cudaMemcpyAsync(dx, x, nx * sizeof(float), cudaMemcpyHostToDevice, n->st);
	if (e == cudaSuccess) e = cudaMemcpyAsync(dt, target, ny * sizeof(float), cudaMemcpyHostToDevice, n->st);
	if (e == cudaSuccess) rc = cnn_work_ensure(n, wk, batch, h, w);
	if (e == cudaSuccess && rc == MCLG_OK) rc = cnn_forward_dev(n, wk, dx, n->st);
	if (e == cudaSuccess && rc == MCLG_OK) {
		k_mse<<<nb, 256, 0, n->st>>>(wk.act[n->nl], dt, ny, gy, part);
		k_sum_partials<<<1, 32, 0, n->st>>>(part, nb, 1.0 / (double)ny, dl);
		rc = cnn_backward_dev(n, wk, gy, g0, g1, n->st);
	}
	if (e == cudaSuccess && rc == MCLG_OK)
		e = cudaMemcpyAsync(grad, n->grad, count * sizeof(float), cudaMemcpyDeviceToHost, n->st);
	if (e == cudaSuccess && rc == MCLG_OK && loss)
		e = cudaMemcpyAsync(loss, dl, sizeof(double), cudaMemcpyDeviceToHost, n->st);
	if (e == cudaSuccess && rc == MCLG_OK) e = cudaStreamSynchronize(n->st);
	cudaFree(dx);
	cudaFree(dt);
	cudaFree(gy);
	cudaFree(g0);
	cudaFree(g1);
	cudaFree(part);
	cnn_work_free(wk);
	if (e != cudaSuccess)
		return cnn_fail(e, "mclg_cnn_gradient");
	return rc;
}

// Adam on the mean squared error over a device-resident data set: samples
// x[nsamples][cin][h][w], targets y[nsamples][cout][h][w] (host buffers,
// uploaded once).  Each iteration draws `batch` samples with a Philox stream
// keyed by `seed`.  loss_trace (optional) receives the loss of every iteration.
int mclg_cnn_train(mclg_cnn *n, const float *x, const float *y, int nsamples, int h, int w, int batch, int iters,
                   float lr, unsigned long long seed, float *loss_trace)
{
	int rc = check_grid(n, batch, h, w);
	if (rc)
		return rc;
	if (x == NULL || y == NULL || nsamples < 1 || iters < 0 || !(lr > 0.f)) {
		mclg_set_error("bad training arguments");
		return MCLG_BAD_INPUT;
	}
	const int cin = n->cin[0], cout = n->cout[n->nl - 1];
	const size_t sx = (size_t)cin * h * w, sy = (size_t)cout * h * w;
	size_t ng = 0;
	for (int l = 0; l < n->nl; l++)
		ng = ng > (size_t)n->cout[l] ? ng : (size_t)n->cout[l];
	ng *= (size_t)batch * h * w;
	float *DX = NULL, *DY = NULL, *bx = NULL, *by = NULL, *gy = NULL, *g0 = NULL, *g1 = NULL;
	double *part = NULL, *dl = NULL, *hl = NULL;
	const int nb = 256;
	CnnWork wk;
	memset(&wk, 0, sizeof wk);
	cudaError_t e = cudaMalloc((void **)&DX, (size_t)nsamples * sx * sizeof(float));
	if (e == cudaSuccess) e = cudaMalloc((void **)&DY, (size_t)nsamples * sy * sizeof(float));
	if (e == cudaSuccess) e = cudaMalloc((void **)&bx, (size_t)batch * sx * sizeof(float));
	if (e == cudaSuccess) e = cudaMalloc((void **)&by, (size_t)batch * sy * sizeof(float));
	if (e == cudaSuccess) e = cudaMalloc((void **)&gy, (size_t)batch * sy * sizeof(float));
	if (e == cudaSuccess) e = cudaMalloc((void **)&g0, ng * sizeof(float));
	if (e == cudaSuccess) e = cudaMalloc((void **)&g1, ng * sizeof(float));
	if (e == cudaSuccess) e = cudaMalloc((void **)&part, (nb + 1) * sizeof(double));
	if (e == cudaSuccess) e = cudaMallocHost((void **)&hl, sizeof(double));
	dl = part + nb;
	if (e == cudaSuccess) e = cudaMemcpyAsync(DX, x, (size_t)nsamples * sx * sizeof(float), cudaMemcpyHostToDevice, n->st);
	if (e == cudaSuccess) e = cudaMemcpyAsync(DY, y, (size_t)nsamples * sy * sizeof(float), cudaMemcpyHostToDevice, n->st);
	if (e == cudaSuccess) rc = cnn_work_ensure(n, wk, batch, h, w);
	const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
	for (int it = 0; it < iters && e == cudaSuccess && rc == MCLG_OK; it++) {
		for (int j = 0; j < batch && e == cudaSuccess; j++) {
			int k = (int)(mclg_uniform01(seed, 11u, (uint32_t)(it * batch + j)) * nsamples);
			k = k < nsamples ? k : nsamples - 1;
			e = cudaMemcpyAsync(bx + j * sx, DX + (size_t)k * sx, sx * sizeof(float), cudaMemcpyDeviceToDevice, n->st);
			if (e == cudaSuccess)
				e = cudaMemcpyAsync(by + j * sy, DY + (size_t)k * sy, sy * sizeof(float), cudaMemcpyDeviceToDevice,
				                    n->st);
		}
		if (e != cudaSuccess)
			break;
		rc = cnn_forward_dev(n, wk, bx, n->st);
		if (rc)
			break;
		const size_t ny = (size_t)batch * sy;
		k_mse<<<nb, 256, 0, n->st>>>(wk.act[n->nl], by, ny, gy, part);
		k_sum_partials<<<1, 32, 0, n->st>>>(part, nb, 1.0 / (double)ny, dl);
		rc = cnn_backward_dev(n, wk, gy, g0, g1, n->st);
		if (rc)
			break;
		n->adam_t++;
		const float c1 = 1.f - powf(b1, (float)n->adam_t), c2 = 1.f - powf(b2, (float)n->adam_t);
		k_adam<<<blocks_for_n((long long)n->nparam), 256, 0, n->st>>>(n->master, n->grad, n->m, n->v, n->nparam, lr,
		                                                              b1, b2, eps, c1, c2);
		rc = pack_all(n);
		if (rc)
			break;
		if (loss_trace) {
			e = cudaMemcpyAsync(hl, dl, sizeof(double), cudaMemcpyDeviceToHost, n->st);
			if (e == cudaSuccess)
				e = cudaStreamSynchronize(n->st);
			loss_trace[it] = (float)*hl;
		}
	}
	if (e == cudaSuccess && rc == MCLG_OK)
		e = cudaStreamSynchronize(n->st);
	cudaFree(DX);
	cudaFree(DY);
	cudaFree(bx);
	cudaFree(by);
	cudaFree(gy);
	cudaFree(g0);
	cudaFree(g1);
	cudaFree(part);
	cudaFreeHost(hl);
	cnn_work_free(wk);
	if (e != cudaSuccess)
		return cnn_fail(e, "mclg_cnn_train");
	return rc;
}

// Adam step from a caller-supplied gradient (host buffer, flat layout).
int mclg_cnn_adam_step(mclg_cnn *n, const float *grad, size_t count, float lr)
{
	if (n == NULL || grad == NULL || count != n->nparam)
		return MCLG_BAD_INPUT;
	const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
	CKC(cudaMemcpyAsync(n->grad, grad, count * sizeof(float), cudaMemcpyHostToDevice, n->st));
	n->adam_t++;
	const float c1 = 1.f - powf(b1, (float)n->adam_t), c2 = 1.f - powf(b2, (float)n->adam_t);
	k_adam<<<blocks_for_n((long long)n->nparam), 256, 0, n->st>>>(n->master, n->grad, n->m, n->v, n->nparam, lr, b1,
	                                                              b2, eps, c1, c2);
	int rc = pack_all(n);
	if (rc)
		return rc;
	CKC(cudaStreamSynchronize(n->st));
	return MCLG_OK;
}

// File: "MCLGCNN1", int32 cin, width, depth, cout, int64 nparam, float32 params.
int mclg_cnn_save(const mclg_cnn *n, const char *path)
{
	if (n == NULL || path == NULL)
		return MCLG_BAD_INPUT;
	float *h = (float *)malloc(n->nparam * sizeof(float));
	int rc = h ? mclg_cnn_get_params(n, h, n->nparam) : MCLG_BAD_INPUT;
	if (rc) {
		free(h);
		return rc;
	}
	FILE *fp = fopen(path, "wb");
	if (fp == NULL) {
		free(h);
		mclg_set_error("cannot open file %s", path);
		return MCLG_IO_ERROR;
	}
	const int32_t hdr[4] = {n->cin[0], n->nl > 1 ? n->cout[0] : 0, n->nl, n->cout[n->nl - 1]};
	const int64_t np = (int64_t)n->nparam;
	int ok = fwrite("MCLGCNN1", 1, 8, fp) == 8 && fwrite(hdr, sizeof hdr, 1, fp) == 1 &&
	         fwrite(&np, sizeof np, 1, fp) == 1 && fwrite(h, sizeof(float), n->nparam, fp) == n->nparam;
	ok = (fclose(fp) == 0) && ok;
	free(h);
	if (!ok) {
		mclg_set_error("cannot write file %s", path);
		return MCLG_IO_ERROR;
	}
	return MCLG_OK;
}

int mclg_cnn_load(mclg_cnn **out, const char *path)
{
	if (out == NULL || path == NULL)
		return MCLG_BAD_INPUT;
	*out = NULL;
	FILE *fp = fopen(path, "rb");
	if (fp == NULL) {
		mclg_set_error("cannot open file %s", path);
		return MCLG_IO_ERROR;
	}
	char magic[8];
	int32_t hdr[4];
	int64_t np = 0;
	if (fread(magic, 1, 8, fp) != 8 || memcmp(magic, "MCLGCNN1", 8) != 0 || fread(hdr, sizeof hdr, 1, fp) != 1 ||
	    fread(&np, sizeof np, 1, fp) != 1 || np <= 0 || np > (1 << 24)) {
		fclose(fp);
		mclg_set_error("%s is not a network file", path);
		return MCLG_BAD_INPUT;
	}
	float *h = (float *)malloc((size_t)np * sizeof(float));
	if (h == NULL || fread(h, sizeof(float), (size_t)np, fp) != (size_t)np) {
		free(h);
		fclose(fp);
		mclg_set_error("%s is truncated", path);
		return MCLG_IO_ERROR;
	}
	fclose(fp);
	mclg_cnn *n = NULL;
	int rc = mclg_cnn_create(&n, hdr[0], hdr[1], hdr[2], hdr[3], 0);
	if (rc == MCLG_OK && (size_t)np != n->nparam) {
		mclg_set_error("%s: %lld parameters, its header implies %zu", path, (long long)np, n->nparam);
		rc = MCLG_BAD_INPUT;
	}
	if (rc == MCLG_OK)
		rc = mclg_cnn_set_params(n, h, (size_t)np);
	free(h);
	if (rc != MCLG_OK) {
		mclg_cnn_destroy(n);
		return rc;
	}
	*out = n;
	return MCLG_OK;
}

}  // extern "C"
