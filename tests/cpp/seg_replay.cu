// Host replay of the segmented recurrences of k_chain_seg (qpc_chain.cuh): the homogeneous solutions
// come from the same seg_spike the engine runs (on the host for the field-free factors, on the device
// for the coupling ones), the segment solves, carry chains and fix-ups follow the kernel's index
// arithmetic one lane at a time, and the result is compared with the sequential forward (L y = w) and
// backward (L^T x = y) solves on a random complex band.  Prints the relative L2 errors per case.
// Test infrastructure for tests/test_seg_solver.py.
#include <cstdio>
#include <cmath>
#include <vector>
#include <random>
#include "qpc_internal.h"
#include "qpc_chain.cuh"
namespace qpc { void set_error(const char*, ...) {} }
using namespace qpc;
template <int P> double run(int N, int Q)
{
	const int NE = P + 1, Ls = (N + Q - 1) / Q;
	std::mt19937 g(1); std::uniform_real_distribution<double> U(-0.15, 0.15);
	std::vector<double2> fs(N * NE);
	for (auto& v : fs) v = make_double2(U(g), U(g));
	std::vector<double2> w(N);
	for (auto& v : w) v = make_double2(U(g) * 5, U(g) * 5);
	auto L = [&](int r, int c) { return fs[r * NE + (r - c) - 1]; };	// L(r, c), c < r
	auto cm = [](double2 a, double2 b) { return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x); };
	// sequential forward then backward
	std::vector<double2> ys(w), xs;
	for (int r = 0; r < N; ++r) for (int k = 1; k <= P; ++k) if (r - k >= 0) { double2 t = cm(L(r, r - k), ys[r - k]); ys[r].x -= t.x; ys[r].y -= t.y; }
	xs = ys;
	for (int r = N - 1; r >= 0; --r) for (int k = 1; k <= P; ++k) if (r + k < N) { double2 t = cm(L(r + k, r), xs[r + k]); xs[r].x -= t.x; xs[r].y -= t.y; }
	// segmented, the kernel's formulas
	std::vector<double2> sf(N * P), sb(N * P);
	for (int sg = 0; sg < Q; ++sg) { int a = sg * Ls, b = std::min(N, a + Ls); for (int j = 1; j <= P; ++j) { seg_spike<P>(fs.data(), N, a, b, j, true, sf.data()); seg_spike<P>(fs.data(), N, a, b, j, false, sb.data()); } }
	std::vector<double2> y(w);
	for (int sg = 0; sg < Q; ++sg) { int a = sg * Ls, b = std::min(N, a + Ls);
		for (int r = a; r < b; ++r) for (int k = 1; k <= P; ++k) if (r - k >= a) { double2 t = cm(L(r, r - k), y[r - k]); y[r].x -= t.x; y[r].y -= t.y; } }
	std::vector<std::vector<double2>> xc(16, std::vector<double2>(P));
	for (int sg = 1; sg < Q; ++sg) for (int i = 0; i < P; ++i) { int r = sg * Ls - 1 - i; double2 v = y[r];
		if (sg >= 2) for (int jj = 0; jj < P; ++jj) { double2 t = cm(sf[r * P + jj], xc[sg - 1][jj]); v.x += t.x; v.y += t.y; }
		xc[sg][i] = v; }
	for (int r = 0; r < N; ++r) { int sg = r / Ls; if (sg >= 1) for (int jj = 0; jj < P; ++jj) { double2 t = cm(sf[r * P + jj], xc[sg][jj]); y[r].x += t.x; y[r].y += t.y; } }
	double ef = 0, nf = 0; for (int r = 0; r < N; ++r) { ef += pow(y[r].x - ys[r].x, 2) + pow(y[r].y - ys[r].y, 2); nf += ys[r].x * ys[r].x + ys[r].y * ys[r].y; }
	// backward on the exact y
	std::vector<double2> x(ys);
	for (int sg = 0; sg < Q; ++sg) { int a = sg * Ls, b = std::min(N, a + Ls);
		for (int r = b - 1; r >= a; --r) for (int k = 1; k <= P; ++k) if (r + k <= b - 1) { double2 t = cm(L(r + k, r), x[r + k]); x[r].x -= t.x; x[r].y -= t.y; } }
	for (int sg = Q - 2; sg >= 0; --sg) for (int i = 0; i < P; ++i) { int r = (sg + 1) * Ls + i; double2 v = x[r];
		if (sg + 1 <= Q - 2) for (int jj = 0; jj < P; ++jj) { double2 t = cm(sb[r * P + jj], xc[sg + 1][jj]); v.x += t.x; v.y += t.y; }
		xc[sg][i] = v; }
	for (int r = 0; r < N; ++r) { int sg = r / Ls; if (sg <= Q - 2) for (int jj = 0; jj < P; ++jj) { double2 t = cm(sb[r * P + jj], xc[sg][jj]); x[r].x += t.x; x[r].y += t.y; } }
	double eb = 0, nb = 0; for (int r = 0; r < N; ++r) { eb += pow(x[r].x - xs[r].x, 2) + pow(x[r].y - xs[r].y, 2); nb += xs[r].x * xs[r].x + xs[r].y * xs[r].y; }
	printf("%d %d %d %d %.3e %.3e\n", P, N, Q, Ls, sqrt(ef / nf), sqrt(eb / nb));
	return 0;
}
int main() { run<6>(400, 16); run<6>(800, 16); run<7>(2000, 16); run<5>(40, 3); run<8>(410, 16); return 0; }
