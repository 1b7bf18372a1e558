// Tiled matrix-free Q1 viscous operator on a uniform level (included by k_mg.cu).
//
// A tile owns TX x 32 nodes (x by z; z is the contiguous direction of the
// node numbering A = iz + ix*n).  Its patch of (TX+2) x 34 nodes -- velocity
// and viscosity -- is staged in shared memory; the three stress components
// at the 4 Gauss points of each of its (TX+1) x 33 elements go to shared
// memory; then each thread gathers the rows of its own nodes from their 4
// elements in a fixed order (deterministic, no atomics).
//
// The tile loop is software-pipelined: while a tile is being computed, the
// global loads of the next tile's patch and of this tile's epilogue operands
// are already in flight in registers, so each block keeps memory busy
// instead of waiting a full round trip per tile.
// Included inside namespace mclg after OpTab / tab<T>() are defined.
#pragma once

constexpr int TZN = 32;
template <class T> struct TileCfg;
template <> struct TileCfg<float> { static constexpr int TX = 16; };   // 512 nodes, 2 per thread
template <> struct TileCfg<double> { static constexpr int TX = 8; };   // 256 nodes, 1 per thread

template <class T>
struct TileSmem {
	static constexpr int TX = TileCfg<T>::TX, PX = TX + 2, PZ = TZN + 2, EX = TX + 1, EZ = TZN + 1;
	T u[PX][PZ], w[PX][PZ], e[PX][PZ];
	// 12 stress values per element, padded to 13 words so that the 32 elements
	// a warp touches at once fall in 32 different shared-memory banks (a
	// stride of 12 words put every 8th element in the same bank)
	T s[EX][EZ][13];
};
constexpr int kSmemBytes = sizeof(TileSmem<double>) > sizeof(TileSmem<float>) ? sizeof(TileSmem<double>)
                                                                                : sizeof(TileSmem<float>);

enum { PASS_MATVEC = 0, PASS_RESID = 1, PASS_SMOOTH = 2, PASS_STOKES = 3 };

// How a tile pass forms its input x at a node:
//   XS_PLAIN    x
//   XS_ZERO     omega D^-1 b         (the first Jacobi sweep from a zero guess)
//   XS_PROLONG  x + P xc             (coarse-grid correction, bilinear P)
//   XS_ZERO_R   omega D^-1 b with b = P^T r_f formed from the finer level's
//               residual (xc = r_f, nc = its nodes per side); the pass also
//               writes b for its own nodes (bout), for the level's later passes
// Fusing these into the next tile pass saves a grid barrier and a pass over
// memory on every multigrid level.
enum { XS_PLAIN = 0, XS_ZERO = 1, XS_PROLONG = 2, XS_ZERO_R = 3 };

// (P^T r_f) at coarse node (cx, cz): full weighting 1, 1/2, 1/4 over the 3 x 3
// fine nodes around (2 cx, 2 cz), in restrict_res's order; unmasked.
template <class T, class V>
__device__ __forceinline__ V restrict_at(const V *__restrict__ rf, int nf, int cx, int cz)
{
	T su = 0, sw = 0;
#pragma unroll
	for (int dx = -1; dx <= 1; dx++)
#pragma unroll
		for (int dz = -1; dz <= 1; dz++) {
			const int fx = 2 * cx + dx, fz = 2 * cz + dz;
			if (fx < 0 || fx >= nf || fz < 0 || fz >= nf)
				continue;
			const T wgt = (dx == 0 ? T(1) : T(0.5)) * (dz == 0 ? T(1) : T(0.5));
			const V r = rf[fz + fx * nf];
			su += wgt * r.x;
			sw += wgt * r.y;
		}
	V o;
	o.x = su;
	o.y = sw;
	return o;
}

template <class T, class V>
__device__ __forceinline__ V x_eff(int xs, int A, int gx, int gz, const V *__restrict__ x, const V *__restrict__ b,
                                   const V *__restrict__ invD, T omega, const V *__restrict__ xc, int nc)
{
	V v;
	if (xs == XS_ZERO || xs == XS_ZERO_R) {
		const V bv = xs == XS_ZERO ? b[A] : restrict_at<T, V>(xc, nc, gx, gz), dv = invD[A];
		v.x = omega * dv.x * bv.x;
		v.y = omega * dv.y * bv.y;
	} else {
		v = x[A];
		if (xs == XS_PROLONG) {
			const int x0 = gx >> 1, z0 = gz >> 1, x1 = (gx + 1) >> 1, z1 = (gz + 1) >> 1;
			const V a = xc[z0 + x0 * nc], bb = xc[z1 + x0 * nc], c = xc[z0 + x1 * nc], d = xc[z1 + x1 * nc];
			v.x += T(0.25) * ((a.x + bb.x) + (c.x + d.x));
			v.y += T(0.25) * ((a.y + bb.y) + (c.y + d.y));
		}
	}
	return v;
}

// One pass of y = A x over a level, with a fused epilogue:
//   MATVEC: out = A x            (*dot = this thread's share of x.(A x) when dot != nullptr)
//   RESID:  out = b - A x        (with xout, x as formed is stored there too)
//   SMOOTH: out = cx x - c0 x0 + omega D^-1 (b - A x)   (cx = 1, no x0: damped Jacobi;
//           the Chebyshev recurrence otherwise; with xout, x as formed is stored there)
//           (*dot = this thread's share of out.dotv when dot != nullptr)
//   STOKES: out64 = A x + G gp, with G gp in FP64 from the element pressures
//           gp (Morton order) and the corner coefficients gt of the fine
//           uniform mesh; *dot = this thread's share of x.out64 (the velocity
//           rows of the Stokes operator applied to (x, gp), and their product
//           with x).  G stays in FP64: applied in FP32 as well, it raised the
//           MINRES iterations per step by half.
// x at Dirichlet dofs is read as 0 and out is 0 there.  wload (when >= 0)
// replaces omega in the XS_ZERO / XS_ZERO_R formation of x.
template <class T, class V>
__device__ __noinline__ void tile_pass(unsigned char *smraw, Part pt, int N, const unsigned char *__restrict__ mask,
                                       const T *__restrict__ eta, const V *__restrict__ x,
                                       const V *__restrict__ b, const V *__restrict__ invD, V *__restrict__ out,
                                       int mode, T omega, double *dot, int xs = XS_PLAIN,
                                       const V *__restrict__ xc = nullptr, int nc = 0,
                                       const double2 *__restrict__ dotv = nullptr,
                                       const double *__restrict__ gp = nullptr, const GTab *gt = nullptr,
                                       double2 *__restrict__ out64 = nullptr, V *__restrict__ bout = nullptr,
                                       V *__restrict__ xout = nullptr, T wload = T(-1), T cx = T(1),
                                       const V *__restrict__ x0 = nullptr, T c0 = T(0))
{
	typedef TileSmem<T> SM;
	constexpr int TX = SM::TX, PX = SM::PX, PZ = SM::PZ, EX = SM::EX, EZ = SM::EZ;
	constexpr int PSLOTS = (PX * PZ + kBlock - 1) / kBlock;   // patch entries per thread
	constexpr int NPT = TX * TZN / kBlock;                      // owned nodes per thread
	SM &S = *reinterpret_cast<SM *>(smraw);
	const OpTab<T> &O = tab<T>();
	const int n = N + 1;
	const int tz_tiles = (n + TZN - 1) / TZN, tx_tiles = (n + TX - 1) / TX, ntiles = tz_tiles * tx_tiles;
	const int t0 = pt.rank, ts = pt.size;
	const int lz = threadIdx.x & 31, lx0 = threadIdx.x >> 5;
	const T wl = wload < T(0) ? omega : wload;
	double dacc = 0.0;
	T pu[PSLOTS], pw[PSLOTS], pe[PSLOTS];

	auto load_patch = [&](int t) {
		const int ix0 = (t / tz_tiles) * TX, iz0 = (t % tz_tiles) * TZN;
#pragma unroll
		for (int j = 0; j < PSLOTS; j++) {
			const int k = threadIdx.x + j * kBlock;
			T uu = 0, ww = 0, ee = 0;
			if (k < PX * PZ) {
				const int px = k / PZ, pz = k - px * PZ;
				const int gx = ix0 - 1 + px, gz = iz0 - 1 + pz;
				if (gx >= 0 && gx < n && gz >= 0 && gz < n) {
					const int A = gz + gx * n;
					const V xv = x_eff<T, V>(xs, A, gx, gz, x, b, invD, wl, xc, nc);
					const unsigned m = mask[A];
					uu = (m & 1u) ? T(0) : xv.x;
					ww = (m & 2u) ? T(0) : xv.y;
					ee = eta[A];
				}
			}
			pu[j] = uu;
			pw[j] = ww;
			pe[j] = ee;
		}
	};

	if (t0 < ntiles)
		load_patch(t0);
	for (int t = t0; t < ntiles; t += ts) {
		const int ix0 = (t / tz_tiles) * TX, iz0 = (t % tz_tiles) * TZN;
		__syncthreads();   // the previous tile is done with shared memory
#pragma unroll
		for (int j = 0; j < PSLOTS; j++) {
			const int k = threadIdx.x + j * kBlock;
			if (k < PX * PZ) {
				const int px = k / PZ, pz = k - px * PZ;
				S.u[px][pz] = pu[j];
				S.w[px][pz] = pw[j];
				S.e[px][pz] = pe[j];
			}
		}
		// epilogue operands of this tile, and the next tile's patch, go in flight now
		V eb[NPT], ed[NPT], e0[NPT];
#pragma unroll
		for (int j = 0; j < NPT; j++) {
			const int gx = ix0 + lx0 + 8 * j, gz = iz0 + lz;
			if (gx < n && gz < n && (mode == PASS_RESID || mode == PASS_SMOOTH)) {
				const int A = gz + gx * n;
				if (xs == XS_ZERO_R) {
					const unsigned m = mask[A];
					V bv = restrict_at<T, V>(xc, nc, gx, gz);
					bv.x = (m & 1u) ? T(0) : bv.x;
					bv.y = (m & 2u) ? T(0) : bv.y;
					eb[j] = bv;
					bout[A] = bv;
				} else {
					eb[j] = b[A];
				}
				if (mode == PASS_SMOOTH) {
					ed[j] = invD[A];
					if (x0 != nullptr)
						e0[j] = x0[A];
				}
			}
		}
		if (t + ts < ntiles)
			load_patch(t + ts);
		__syncthreads();
		for (int k = threadIdx.x; k < EX * EZ; k += kBlock) {
			const int pex = k / EZ, pez = k - pex * EZ;
			const int ex = ix0 - 1 + pex, ez = iz0 - 1 + pez;
			T *sv = S.s[pex][pez];
			if (ex < 0 || ex >= N || ez < 0 || ez >= N) {
#pragma unroll
				for (int q = 0; q < 12; q++)
					sv[q] = 0;
				continue;
			}
			// corners 0=(ex,ez) 1=(ex,ez+1) 2=(ex+1,ez+1) 3=(ex+1,ez)
			const T u[4] = {S.u[pex][pez], S.u[pex][pez + 1], S.u[pex + 1][pez + 1], S.u[pex + 1][pez]};
			const T w[4] = {S.w[pex][pez], S.w[pex][pez + 1], S.w[pex + 1][pez + 1], S.w[pex + 1][pez]};
			const T e[4] = {S.e[pex][pez], S.e[pex][pez + 1], S.e[pex + 1][pez + 1], S.e[pex + 1][pez]};
#pragma unroll
			for (int g = 0; g < 4; g++) {
				T eg = 0, ux = 0, uz = 0, wx = 0, wz = 0;
#pragma unroll
				for (int a = 0; a < 4; a++) {
					eg += O.N[a][g] * e[a];
					ux += O.Dx[a][g] * u[a];
					uz += O.Dz[a][g] * u[a];
					wx += O.Dx[a][g] * w[a];
					wz += O.Dz[a][g] * w[a];
				}
				sv[g] = 2 * eg * ux;
				sv[4 + g] = 2 * eg * wz;
				sv[8 + g] = eg * (uz + wx);
			}
		}
		__syncthreads();
#pragma unroll
		for (int j = 0; j < NPT; j++) {
			const int lx = lx0 + 8 * j;
			const int gx = ix0 + lx, gz = iz0 + lz;
			if (gx >= n || gz >= n)
				continue;
			const int px = lx + 1, pz = lz + 1;
			const int epx[4] = {px - 1, px - 1, px, px}, epz[4] = {pz - 1, pz, pz, pz - 1}, ea[4] = {2, 3, 0, 1};
			T fu = 0, fw = 0;
#pragma unroll
			for (int q = 0; q < 4; q++) {
				const T *sv = S.s[epx[q]][epz[q]];
				const int a = ea[q];
#pragma unroll
				for (int g = 0; g < 4; g++) {
					fu += O.Dx[a][g] * sv[g] + O.Dz[a][g] * sv[8 + g];
					fw += O.Dz[a][g] * sv[4 + g] + O.Dx[a][g] * sv[8 + g];
				}
			}
			const int A = gz + gx * n;
			const unsigned m = mask[A];
			if (m & 1u)
				fu = 0;
			if (m & 2u)
				fw = 0;
			const T xu = S.u[px][pz], xw = S.w[px][pz];   // x as this pass formed it (0 on Dirichlet dofs)
			V o;
			if (mode == PASS_STOKES) {
				// (G gp) at this node: its up to 4 elements, as gmul64
				double s0 = 0.0, s1 = 0.0;
				const int eox[4] = {gx - 1, gx - 1, gx, gx}, eoz[4] = {gz - 1, gz, gz, gz - 1};
#pragma unroll
				for (int q = 0; q < 4; q++) {
					const int ex = eox[q], ez = eoz[q];
					if (ex < 0 || ex >= N || ez < 0 || ez >= N)
						continue;
					const double se = gp[morton(ex, ez)];
					s0 += gt->g0[ea[q]] * se;
					s1 += gt->g1[ea[q]] * se;
				}
				const double2 az = make_double2((m & 1u) ? 0.0 : (double)fu + s0, (m & 2u) ? 0.0 : (double)fw + s1);
				out64[A] = az;
				dacc += az.x * (double)xu + az.y * (double)xw;
				continue;
			}
			if (mode == PASS_MATVEC) {
				o.x = fu;
				o.y = fw;
				if (dot)
					dacc += (double)xu * (double)fu + (double)xw * (double)fw;
			} else if (mode == PASS_RESID) {
				o.x = (m & 1u) ? T(0) : eb[j].x - fu;
				o.y = (m & 2u) ? T(0) : eb[j].y - fw;
				if (xout) {   // x as this pass formed it (the first sweep from zero)
					V xv;
					xv.x = xu;
					xv.y = xw;
					xout[A] = xv;
				}
			} else {
				T px = cx * xu, pw = cx * xw;
				if (x0 != nullptr) {
					px -= c0 * e0[j].x;
					pw -= c0 * e0[j].y;
				}
				o.x = (m & 1u) ? T(0) : px + omega * ed[j].x * (eb[j].x - fu);
				o.y = (m & 2u) ? T(0) : pw + omega * ed[j].y * (eb[j].y - fw);
				if (xout) {   // x as this pass formed it (the coarse-corrected iterate)
					V xv;
					xv.x = xu;
					xv.y = xw;
					xout[A] = xv;
				}
				if (dot) {
					const double2 v = dotv[A];
					dacc += (double)o.x * v.x + (double)o.y * v.y;
				}
			}
			out[A] = o;
		}
	}
	if (dot)
		*dot = dacc;
}
