// Internal declarations shared by the host setup (qpc_setup.cpp) and the CUDA
// engine (qpc_engine.cu).  The public C ABI is include/qpc_gb300.h.
#pragma once
#include "../../include/qpc_gb300.h"
#include <cstddef>
#include <cstdint>

namespace qpc {
void set_error(const char* fmt, ...);
// real symmetric form D^H Z_c D of a propagator_cn_hc_vgwr coupling (qpc_setup.cpp)
void vgwr_real_coupling(int n_l, int n_m, int m0, int comp, double* Zr);
}
