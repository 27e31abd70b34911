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

// bounded wait: poll the stream until its work is done, give up after
// wait_limit_s() seconds of wall time with QPC_ERR_TIMEOUT (the work stays
// queued; a later call on the same stream waits for it again)
inline int wait_on(cudaStream_t st)
{
	struct timespec t0, now;
	clock_gettime(CLOCK_MONOTONIC, &t0);
	const double limit = wait_limit_s();
	for (long it = 0;; ++it) {
		cudaError_t e = cudaStreamQuery(st);
		if (e == cudaSuccess) return QPC_OK;
		if (e != cudaErrorNotReady) { set_error("stream error: %s", cudaGetErrorString(e)); return QPC_ERR_CUDA; }
		clock_gettime(CLOCK_MONOTONIC, &now);
		if ((double)(now.tv_sec - t0.tv_sec) + 1e-9 * (double)(now.tv_nsec - t0.tv_nsec) > limit) {
			set_error("timed out after %.3g s waiting for the device", limit);
			return QPC_ERR_TIMEOUT;
		}
		struct timespec ts = {0, it < 100 ? 2000L : 100000L};
		nanosleep(&ts, nullptr);
	}
}

// device -> host copy of a result: wait (bounded) for the work queued before it, then
// copy.  Waiting first means the copy never blocks on queued work (a copy into pageable
// memory may block inside the driver until the stream reaches it, without a bound), and a
// wait that runs out leaves no copy pending into a host buffer the caller may free.
inline int copy_to_host(void* dst, const void* src, size_t bytes, cudaStream_t st)
{
	if (int rc = wait_on(st)) return rc;
	QPC_CUDA(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, st));
	return wait_on(st);
}

} // namespace qpc
