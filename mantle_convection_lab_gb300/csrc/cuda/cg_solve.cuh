// Conjugate gradients inside a persistent cooperative kernel.
//
// The iteration is the reference's Conj_Grad (Solver.c:1589-1797) and
// Conj_Grad_heat (Update_temperature.c:1140-1354), step for step:
//   r = b - A x;  d = r / diag (or r);  delta0 = r.d
//   while cycle < max_cycle && delta > accu * delta0:
//       q = A d;  alpha = delta / d.q;  x += alpha d;  hanging-node overwrite of x
//       r = b - A x every 50th cycle, else r -= alpha q
//       s = r / diag;  delta = r.s;  d = s + (delta/delta_old) d;  cycle++
//       stop when max|alpha r| < accu  (the heat solver without a
//       preconditioner also needs cycle > 10)
// Every block computes the scalars from the same partial sums in the same
// order, so all blocks branch together; no loop runs past max_cycle.
#pragma once
#include "mclg_dev.cuh"

namespace mclg {

template <class Op>
__device__ int cg_solve(cg::grid_group &g, GridRed &red, const Op &op, const double *__restrict__ b,
                        double *__restrict__ x, double *__restrict__ r, double *__restrict__ s,
                        double *__restrict__ d, double *__restrict__ q, double accu, int max_cycle,
                        bool precond, bool plain_needs_10, int *status)
{
	constexpr int NC = Op::NC;
	const int n = op.nunits();
	const int tid = blockIdx.x * blockDim.x + threadIdx.x, nth = gridDim.x * blockDim.x;

	double a0[1] = {0.0};
	for (int A = tid; A < n; A += nth) {
		double y[NC];
		op.apply(x, A, y);
#pragma unroll
		for (int c = 0; c < NC; c++) {
			const int i = A * NC + c;
			if (op.is_free(A, c)) {
				const double rr = b[i] - y[c];
				const double dd = precond ? rr * op.inv_diag(A, c) : rr;
				r[i] = rr;
				d[i] = dd;
				a0[0] += rr * dd;
			} else {
				r[i] = 0.0;
				d[i] = 0.0;
				s[i] = 0.0;
				q[i] = 0.0;
			}
		}
	}
	grid_reduce<1>(g, red, a0, 0u);
	double delta_new = a0[0];
	const double delta0 = delta_new;
	int cycle = 0;
	while (cycle < max_cycle && delta_new > accu * delta0) {
		double a1[1] = {0.0};
		for (int A = tid; A < n; A += nth) {
			double y[NC];
			op.apply(d, A, y);
#pragma unroll
			for (int c = 0; c < NC; c++) {
				const int i = A * NC + c;
				if (op.is_free(A, c)) {
					q[i] = y[c];
					a1[0] += d[i] * y[c];
				}
			}
		}
		grid_reduce<1>(g, red, a1, 0u);
		const double alpha = delta_new / a1[0];
		const bool refresh = (cycle % 50) == 0;
		double a2[2] = {0.0, 0.0};
		for (int A = tid; A < n; A += nth) {
#pragma unroll
			for (int c = 0; c < NC; c++) {
				const int i = A * NC + c;
				if (!op.is_free(A, c))
					continue;
				x[i] += alpha * d[i];
				if (!refresh) {
					const double rr = r[i] - alpha * q[i];
					const double ss = precond ? rr * op.inv_diag(A, c) : rr;
					r[i] = rr;
					s[i] = ss;
					a2[0] += rr * ss;
					a2[1] = fmax(a2[1], fabs(alpha * rr));
				}
			}
		}
		if (op.nhang() > 0) {
			g.sync();
			op.constrain(x, tid, nth);
		}
		if (refresh) {
			g.sync();
			for (int A = tid; A < n; A += nth) {
				double y[NC];
				op.apply(x, A, y);
#pragma unroll
				for (int c = 0; c < NC; c++) {
					const int i = A * NC + c;
					if (!op.is_free(A, c))
						continue;
					const double rr = b[i] - y[c];
					const double ss = precond ? rr * op.inv_diag(A, c) : rr;
					r[i] = rr;
					s[i] = ss;
					a2[0] += rr * ss;
					a2[1] = fmax(a2[1], fabs(alpha * rr));
				}
			}
		}
		grid_reduce<2>(g, red, a2, 2u);
		const double delta_old = delta_new;
		delta_new = a2[0];
		const double beta = delta_new / delta_old;
		for (int A = tid; A < n; A += nth) {
#pragma unroll
			for (int c = 0; c < NC; c++) {
				const int i = A * NC + c;
				if (op.is_free(A, c))
					d[i] = s[i] + beta * d[i];
			}
		}
		cycle++;
		if (!isfinite(delta_new) || !isfinite(alpha)) {
			if (tid == 0)
				atomicOr(status, a1[0] == 0.0 ? kStatBreakdown : kStatNan);
			break;
		}
		if (a2[1] < accu && (!plain_needs_10 || cycle > 10))
			break;
		g.sync();
	}
	if (cycle >= max_cycle && tid == 0)
		atomicOr(status, kStatCap);
	g.sync();
	return cycle;
}

}  // namespace mclg
