// Deterministic FP64 grid reductions: warp shuffles, then a per-block sum in
// shared memory, then the last block to finish adds the block partials in a
// fixed order. The result depends only on the grid and block shape, not on
// block scheduling. This replaces the reference's per-block shared-memory
// tree + host-side serial sum of partials (src/lattice/device.h:185-212,
// 246-265), which needs a device synchronisation and a D2H copy per sum; here
// the scalar stays on the device (a result slot) for later kernels.
#pragma once

#include <cuda_runtime.h>

namespace meshgb {

struct RedSlot
{
	double *partials; // >= gridDim.x entries
	double *result;
	unsigned *counter; // zero between launches (reset by the last block)
};

__device__ __forceinline__ double warp_sum(double v)
{
#pragma unroll
	for (int o = 16; o > 0; o >>= 1)
		v += __shfl_down_sync(0xffffffffu, v, o);
	return v;
}

// Adds v of every thread of the grid into *slot.result (overwrites it).
// Must be called by all threads of every block (no early return before it).
template <int BLOCK> __device__ __forceinline__ void grid_sum(double v, RedSlot slot)
{
	static_assert(BLOCK % 32 == 0 && BLOCK <= 1024, "block size");
	constexpr int NW = BLOCK / 32;
	__shared__ double sw[NW];
	__shared__ bool is_last;
	int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
	v = warp_sum(v);
	if (lane == 0)
		sw[warp] = v;
	__syncthreads();
	if (warp == 0)
	{
		double t = lane < NW ? sw[lane] : 0.0;
		t = warp_sum(t);
		if (lane == 0)
		{
			slot.partials[blockIdx.x] = t;
			__threadfence();
			unsigned prev = atomicInc(slot.counter, gridDim.x - 1);
			is_last = (prev == gridDim.x - 1);
		}
	}
	__syncthreads();
	if (is_last)
	{
		double s = 0.0;
		for (unsigned i = threadIdx.x; i < gridDim.x; i += BLOCK)
			s += __ldcg(slot.partials + i);
		s = warp_sum(s);
		if (lane == 0)
			sw[warp] = s;
		__syncthreads();
		if (threadIdx.x == 0)
		{
			double r = 0.0;
#pragma unroll
			for (int w = 0; w < NW; ++w)
				r += sw[w];
			*slot.result = r;
		}
	}
}

} // namespace meshgb
