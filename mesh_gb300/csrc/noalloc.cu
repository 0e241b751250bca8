// Plaquette entry point that allocates no device memory.
//
// Who needs it: callers that cannot call cudaMalloc at the point where they
// measure the plaquette, e.g. a host application that hands all device
// memory to its own pool or arena at start-up and forbids further
// allocations, or code running under a memory cap where the library's
// context (which owns reduction scratch, streams and staging buffers) cannot
// be created. They keep the links in their own device buffer and call this
// function with plain pointers.
//
// The kernel is the one mesh_plaquette launches (k_plaquette), with the same
// grid, so the two entry points return the same bits. Its reduction scratch
// (one FP64 partial sum per block, the result and the last-block counter)
// lives in the file-scope device array below instead of context memory.
// The CUDA runtime places that array when it loads this library's module on
// a device; this file never calls cudaMalloc, cudaFree or any allocating
// routine.
#include <mutex>

#include "field.cuh"
#include "kernels.cuh"

namespace meshgb {
namespace {

// Maximum number of reduction blocks the static scratch holds.
constexpr int kNoAllocMaxBlocks = MESH_NOALLOC_MAX_BLOCKS;
// partials [0, kNoAllocMaxBlocks), result at kNoAllocMaxBlocks, counter (an
// unsigned in its own 8-byte word) at kNoAllocMaxBlocks + 1: 8 KiB + 16 B
static __device__ __align__(256) double g_noalloc_scratch[kNoAllocMaxBlocks + 2];

constexpr int kMaxDevices = 64;

struct NoAllocDevice
{
	std::mutex mu;
	bool ready = false; // set only by a set-up that succeeded
	double *scratch = nullptr;
	int num_sms = 0;
};
NoAllocDevice g_dev[kMaxDevices];

// Once per device, with that device current: resolve the scratch array's
// address and read the SM count. The first call on a device may also make
// the CUDA runtime create the device's primary context and load this
// module, which is the only device memory this path ever causes to exist.
// A set-up that fails leaves the device not ready, so the next call tries
// again (the cause, e.g. a device still busy being reset by its owner, may
// have cleared); the failing call returns the error. Returns the failure's
// message, or nullptr on success.
char const *setup(int device, NoAllocDevice &d)
{
	std::lock_guard<std::mutex> lk(d.mu);
	if (d.ready)
		return nullptr;
	double *p = nullptr;
	int n = 0;
	if (cudaGetSymbolAddress(reinterpret_cast<void **>(&p), g_noalloc_scratch) != cudaSuccess)
	{
		cudaGetLastError();
		return "cudaGetSymbolAddress of the no-allocation scratch failed";
	}
	if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, device) != cudaSuccess || n <= 0)
	{
		cudaGetLastError();
		return "cudaDeviceGetAttribute(multiProcessorCount) failed";
	}
	d.scratch = p;
	d.num_sms = n;
	d.ready = true;
	return nullptr;
}

// `links` must be device memory of `device` (or managed memory): a host
// pointer or another device's buffer is refused here, before any launch.
// cudaPointerGetAttributes allocates nothing.
void check_links(int device, void const *links)
{
	cudaPointerAttributes a{};
	cudaError_t e = cudaPointerGetAttributes(&a, links);
	if (e != cudaSuccess)
	{
		cudaGetLastError();
		throw Error(MESH_ERR_ARG, "links: not a pointer the CUDA runtime knows (device memory required)");
	}
	if (a.type != cudaMemoryTypeDevice && a.type != cudaMemoryTypeManaged)
		throw Error(MESH_ERR_ARG, "links: host memory given where device memory of `device` is required");
	if (a.device != device)
		throw Error(MESH_ERR_ARG, "links: the buffer belongs to another device");
}

template <int GRP, class T, int ND>
void launch(Geom const &g, void const *links, unsigned blocks, cudaStream_t st, RedSlot slot)
{
	k_plaquette<GRP, T, ND><<<blocks, kBlock, 0, st>>>(g, static_cast<T const *>(links), slot);
}

template <int GRP, class T>
void launch_nd(int nd, Geom const &g, void const *links, unsigned blocks, cudaStream_t st, RedSlot slot)
{
	if (nd == 2)
		launch<GRP, T, 2>(g, links, blocks, st, slot);
	else if (nd == 3)
		launch<GRP, T, 3>(g, links, blocks, st, slot);
	else
		launch<GRP, T, 4>(g, links, blocks, st, slot);
}

} // namespace
} // namespace meshgb

using namespace meshgb;

extern "C" int mesh_plaquette_noalloc(int device, int group, int precision, int nd, int32_t const *dims,
                                      void const *links, void *stream, double *out)
{
	return api_call([&] {
		require(device >= 0 && device < kMaxDevices, "device index out of range");
		require(group >= 1 && group <= 3, "unknown gauge group");
		require(precision == MESH_F32 || precision == MESH_F64, "invalid precision level");
		require(nd >= 2 && nd <= 4, "number of dimensions must be 2, 3 or 4");
		require(dims != nullptr, "null dims");
		require(links != nullptr, "null links");
		require(out != nullptr, "null output");
		int64_t V = 1;
		for (int i = 0; i < nd; ++i)
		{
			require(dims[i] >= 2 && dims[i] % 2 == 0, "every extent must be even and >= 2 (checkerboard layout)");
			require(dims[i] < 256, "every extent must be below 256");
			V *= dims[i];
			require(V < (int64_t(1) << 31), "volume must be below 2^31");
		}
		DeviceGuard dg(device);
		NoAllocDevice &d = g_dev[device];
		if (char const *why = setup(device, d))
			throw Error(MESH_ERR_CUDA, why);
		check_links(device, links);
		// the grid mesh_plaquette uses on this device (a function of the volume
		// and the SM count only); a grid beyond the scratch is refused rather
		// than shrunk, as a different grid would change the summation order
		int64_t need = (V + kBlock - 1) / kBlock;
		int64_t cap = int64_t(d.num_sms) * 4;
		int64_t blocks = need < cap ? need : cap;
		if (blocks > kMaxRedBlocks)
			blocks = kMaxRedBlocks;
		require(blocks <= kNoAllocMaxBlocks,
		        "mesh_plaquette_noalloc: the reduction needs more blocks than MESH_NOALLOC_MAX_BLOCKS");
		auto st = static_cast<cudaStream_t>(stream);
		RedSlot slot{d.scratch, d.scratch + kNoAllocMaxBlocks,
		             reinterpret_cast<unsigned *>(d.scratch + kNoAllocMaxBlocks + 1)};
		// the last-block counter must start at zero; a finished reduction
		// leaves it at zero, this also covers one cut short by an error
		MESH_CUDA(cudaMemsetAsync(slot.counter, 0, sizeof(unsigned), st));
		Geom g = make_geom(nd, dims);
		bool f32 = precision == MESH_F32;
		switch (group)
		{
		case 1:
			f32 ? launch_nd<1, float>(nd, g, links, unsigned(blocks), st, slot)
			    : launch_nd<1, double>(nd, g, links, unsigned(blocks), st, slot);
			break;
		case 2:
			f32 ? launch_nd<2, float>(nd, g, links, unsigned(blocks), st, slot)
			    : launch_nd<2, double>(nd, g, links, unsigned(blocks), st, slot);
			break;
		default:
			f32 ? launch_nd<3, float>(nd, g, links, unsigned(blocks), st, slot)
			    : launch_nd<3, double>(nd, g, links, unsigned(blocks), st, slot);
			break;
		}
		MESH_LAUNCH_CHECK();
		double s = 0.0;
		MESH_CUDA(cudaMemcpyAsync(&s, slot.result, sizeof(double), cudaMemcpyDeviceToHost, st));
		MESH_CUDA(cudaStreamSynchronize(st));
		double nplanes = double(nd) * double(nd - 1) / 2.0;
		*out = s / (double(V) * nplanes) / double(group_nc(group));
	});
}
