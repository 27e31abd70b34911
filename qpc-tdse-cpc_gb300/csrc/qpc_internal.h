// Internal declarations shared by the host setup (qpc_setup.cpp) and the CUDA
// engine (qpc_engine.cu).  The public C ABI is include/qpc_gb300.h.
#pragma once
#include "../../include/qpc_gb300.h"
#include <cstddef>
#include <cstdint>

namespace qpc {
void set_error(const char* fmt, ...);
}
