// Internal declarations shared by the host setup (qpc_setup.cpp) and the CUDA
// engine (qpc_engine.cu).  The public C ABI is include/qpc_gb300.h.
#pragma once
#include "../../include/qpc_gb300.h"
#include <cstddef>
#include <cstdint>
#include <vector>

namespace qpc {
// B-spline basis of one radial grid with its Gauss-Legendre quadrature (nq points per knot
// interval, absolute interval index s over the knot vector t); built by build_basis.
struct radial_basis {
	int n, p, nq;
	std::vector<double> t;               // absolute knots t_0 .. t_{n+p+2}
	std::vector<double> xq, wq;          // [interval][nq]
	std::vector<double> b0, b1;          // [interval][p+1][nq], spline s-p+j at interval s
	int nint() const { return (int)t.size() - 1; }
};
void build_basis(radial_basis& B);
// values and first derivatives of the p+1 splines non-zero on interval [t_s, t_s+1) at x
void bspline_eval(const std::vector<double>& t, int s, int p, double x, double* out0, double* out1);

void set_error(const char* fmt, ...);
// bound of every host wait for the device, in seconds (qpc_set_wait_limit; the
// environment variable QPC_WAIT_LIMIT_S read at first use; default 600 s)
double wait_limit_s();
// t-SURFF accumulate inside a length-gauge run (qpc_momentum.cu): the surface values straight from
// the engine's resident state st (r-major [slot][m][r][l], instance i at slot_dev[i], a device
// array), a[2 i], a[2 i + 1] = f(t_i), f(t_i+1) of instance i (zeros for a field-free step: the
// accumulate of a z-linear step with zero field is the field-free one), act[i] = 1 for the
// instances that take it; enqueued on stream without a wait
int tsurff_check_grid(qpc_tsurff* t, const qpc_dims& d);
int tsurff_enqueue_engine(qpc_tsurff* t, const void* st, const int* slot_dev, const double* a, const int* act, double dt, void* stream);
// real symmetric form D^H Z_c D of a propagator_cn_hc_vgwr coupling (qpc_setup.cpp)
void vgwr_real_coupling(int n_l, int n_m, int m0, int comp, double* Zr);
}
