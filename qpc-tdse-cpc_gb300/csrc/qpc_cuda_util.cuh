// Host-side CUDA helpers shared by the engine's translation units: error
// reporting, device check, allocation and the bounded stream wait.
#pragma once
#include "qpc_internal.h"
#include <cuda_runtime.h>
#include <algorithm>
#include <time.h>

namespace qpc {

#define QPC_CUDA(call) do { cudaError_t e_ = (call); if (e_ != cudaSuccess) { \
	set_error("%s failed: %s (%s:%d)", #call, cudaGetErrorString(e_), __FILE__, __LINE__); return QPC_ERR_CUDA; } } while (0)

// the current device, if it is Blackwell-class (sm_100 or later)
inline int check_device(int* dev)
{
	int n = 0;
	cudaError_t e = cudaGetDeviceCount(&n);
	if (e != cudaSuccess || n == 0) { set_error("no CUDA device: %s", cudaGetErrorString(e)); return QPC_ERR_NODEVICE; }
	QPC_CUDA(cudaGetDevice(dev));
	cudaDeviceProp prop;
	QPC_CUDA(cudaGetDeviceProperties(&prop, *dev));
	if (prop.major * 10 + prop.minor < 100) { set_error("device %s (sm_%d%d) is not Blackwell-class", prop.name, prop.major, prop.minor); return QPC_ERR_NODEVICE; }
	return QPC_OK;
}

template <class T> inline int dalloc(T** p, size_t n)
{
	cudaError_t e = cudaMalloc((void**)p, sizeof(T) * std::max<size_t>(n, 1));
	if (e != cudaSuccess) { *p = nullptr; set_error("cudaMalloc(%zu bytes): %s", sizeof(T) * n, cudaGetErrorString(e)); return QPC_ERR_NOMEM; }
	return QPC_OK;
}

// bounded wait: poll the stream, give up after ~600 s of wall time
inline int wait_on(cudaStream_t st)
{
	for (long it = 0;; ++it) {
		cudaError_t e = cudaStreamQuery(st);
		if (e == cudaSuccess) return QPC_OK;
		if (e != cudaErrorNotReady) { set_error("stream error: %s", cudaGetErrorString(e)); return QPC_ERR_CUDA; }
		if (it > 6000000) { set_error("timed out waiting for the device"); return QPC_ERR_TIMEOUT; }
		struct timespec ts = {0, 100000};
		nanosleep(&ts, nullptr);
	}
}

} // namespace qpc
