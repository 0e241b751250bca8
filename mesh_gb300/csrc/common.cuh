// Shared infrastructure of the sm_103a library: status codes, the per-context
// state (device, stream, FP64 reduction scratch), launch sizing.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <cstdio>
#include <stdexcept>
#include <string>

#include "../../include/mesh_gb300.h"

namespace meshgb {

// Error carrying a C-ABI status code; every extern "C" entry point catches it
// and returns the code (no exception crosses the ABI).
struct Error : std::runtime_error
{
	int code;
	Error(int c, std::string const &m) : std::runtime_error(m), code(c) {}
};

inline void cuda_check(cudaError_t e, char const *what)
{
	if (e != cudaSuccess)
		throw Error(MESH_ERR_CUDA, std::string("cuda error: ") + what + ": " + cudaGetErrorString(e));
}
#define MESH_CUDA(x) ::meshgb::cuda_check((x), #x)
#define MESH_LAUNCH_CHECK() ::meshgb::cuda_check(cudaGetLastError(), "kernel launch")

inline void require(bool ok, char const *msg, int code = MESH_ERR_ARG)
{
	if (!ok)
		throw Error(code, msg);
}

// Number of FP64 reduction slots a context owns; slots are used for the
// scalars of one HMC trajectory (S_old, S_new, K_old, K_new, ...) and by the
// synchronous one-off reductions.
constexpr int kSlots = 64;
// Maximum number of blocks of one reduction launch (partials per slot).
constexpr int kMaxRedBlocks = 4096;

struct Context
{
	// owners: the caller's handle plus every field and chain created on it;
	// the context is torn down when the last one is released
	int refs = 1;
	int device = 0;
	cudaStream_t stream = nullptr;
	bool own_stream = false;
	int num_sms = 0;
	// reduction scratch: partials [kSlots][kMaxRedBlocks] (double),
	// results [kSlots] (double), counters [kSlots] (unsigned)
	double *d_partials = nullptr;
	double *d_results = nullptr;
	unsigned *d_counters = nullptr;
	// device error word: kernels with bounded waits (the TMA-staged line march)
	// write a nonzero code here when a wait gives up; zero otherwise
	int *d_err = nullptr;
	// host staging for layout conversions
	void *d_stage = nullptr;
	size_t stage_bytes = 0;

	void *stage(size_t bytes)
	{
		if (bytes > stage_bytes)
		{
			if (d_stage)
				MESH_CUDA(cudaFreeAsync(d_stage, stream));
			MESH_CUDA(cudaMallocAsync(&d_stage, bytes, stream));
			stage_bytes = bytes;
		}
		return d_stage;
	}
};

// Makes the context's device current for the duration of a call.
struct DeviceGuard
{
	int prev = -1;
	explicit DeviceGuard(int dev)
	{
		cudaGetDevice(&prev);
		if (prev != dev)
			MESH_CUDA(cudaSetDevice(dev));
	}
	~DeviceGuard()
	{
		if (prev >= 0)
			cudaSetDevice(prev);
	}
};

// grid size for a grid-stride kernel over n items: at most `per_sm` resident
// blocks per SM worth of blocks, never more than needed.
inline unsigned grid_for(Context const &c, int64_t n, int block, int per_sm = 8)
{
	int64_t need = (n + block - 1) / block;
	int64_t cap = int64_t(c.num_sms) * per_sm;
	if (need < 1)
		need = 1;
	return unsigned(need < cap ? need : cap);
}

} // namespace meshgb
