// mesh/lattice_apply.cuh — the generic lattice_apply / reduction layer for
// user functors, on the device layout of libmesh_gb300 (CUDA, header-only;
// compile with nvcc -std=c++20 for sm_103a).
//
// Counterpart of src/lattice/device.h:139-265 and lattice.h:256-273:
//   lattice_apply(f, a, as...)       f(T&, Ts const&...) on every site
//   lattice_sum_apply(f, a, as...)   sum over sites of f(T const&, Ts const&...)
//   lattice_sum(a)                   sum of the objects
//   cshift(nd, dims, dst, src, dir, offset)   dst[x] = src[x + offset e_dir]
// a, as... are FieldView<T> (device base pointer and V). The forms above run
// on the legacy default stream; lattice_apply_on / lattice_sum_apply_on take
// the stream first. Functors are __device__ lambdas (nvcc --extended-lambda)
// or structs with a __device__ operator().
//
// Storage. A field of V objects of type T (trivially copyable, sizeof(T) a
// multiple of 4) is held even/odd-ordered as structure-of-arrays "planes" of
// 16, 8 and 4 bytes: floor(sizeof(T)/16) planes of 16-byte words, then an
// 8-byte plane if (sizeof(T) % 16) >= 8, then a 4-byte plane if needed. This
// is exactly the layout of libmesh_gb300's fields (float4/float2/float and
// double2/double planes), so the functors can run on mesh_field_device_ptr()
// of a library field whose object type has the same byte size (one stacked
// component at offset c * sizeof(T) * V). Each warp reads 32 consecutive
// 16-byte words per plane: 128-bit coalesced accesses.
//
// Differences to the reference: no temporaries are allocated by the apply
// itself; launches go to a caller-given stream; sums accumulate in the
// functor's result type R with a deterministic order (per-thread grid-stride
// sums, warp/block tree, last-block combine), instead of the reference's
// 256-wide blocks in lexicographic order followed by a host loop.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <cstring>
#include <stdexcept>
#include <string>
#include <type_traits>

namespace mesh {
namespace device {

template <class T> struct Planes
{
	static_assert(std::is_trivially_copyable_v<T>, "lattice objects must be trivially copyable");
	static_assert(sizeof(T) % 4 == 0, "lattice objects must be a multiple of 4 bytes");
	static constexpr int N16 = int(sizeof(T) / 16);
	static constexpr int R = int(sizeof(T) % 16);
	static constexpr bool H8 = R >= 8;
	static constexpr bool H4 = (R % 8) == 4;
};

// typed view of V objects of T in the plane layout starting at `base`
template <class T> struct FieldView
{
	void *base;
	int64_t V;

	__device__ __forceinline__ T load(int64_t s) const
	{
		using P = Planes<T>;
		alignas(16) unsigned char buf[sizeof(T)];
		uint4 const *p16 = static_cast<uint4 const *>(base);
#pragma unroll
		for (int k = 0; k < P::N16; ++k)
			reinterpret_cast<uint4 *>(buf)[k] = p16[k * V + s];
		unsigned char const *tail = static_cast<unsigned char const *>(base) + size_t(P::N16) * 16 * size_t(V);
		int off = P::N16 * 16;
		if constexpr (P::H8)
		{
			*reinterpret_cast<uint2 *>(buf + off) = reinterpret_cast<uint2 const *>(tail)[s];
			tail += 8 * size_t(V);
			off += 8;
		}
		if constexpr (P::H4)
			*reinterpret_cast<unsigned *>(buf + off) = reinterpret_cast<unsigned const *>(tail)[s];
		T t;
		memcpy(&t, buf, sizeof(T));
		return t;
	}
	__device__ __forceinline__ void store(int64_t s, T const &t) const
	{
		using P = Planes<T>;
		alignas(16) unsigned char buf[sizeof(T)];
		memcpy(buf, &t, sizeof(T));
		uint4 *p16 = static_cast<uint4 *>(base);
#pragma unroll
		for (int k = 0; k < P::N16; ++k)
			p16[k * V + s] = reinterpret_cast<uint4 const *>(buf)[k];
		unsigned char *tail = static_cast<unsigned char *>(base) + size_t(P::N16) * 16 * size_t(V);
		int off = P::N16 * 16;
		if constexpr (P::H8)
		{
			reinterpret_cast<uint2 *>(tail)[s] = *reinterpret_cast<uint2 const *>(buf + off);
			tail += 8 * size_t(V);
			off += 8;
		}
		if constexpr (P::H4)
			reinterpret_cast<unsigned *>(tail)[s] = *reinterpret_cast<unsigned const *>(buf + off);
	}
};

template <class T> FieldView<T> view(void *base, int64_t V) { return {base, V}; }
template <class T> FieldView<T> view(void const *base, int64_t V) { return {const_cast<void *>(base), V}; }

inline void cuda_ok(cudaError_t e, char const *what)
{
	if (e != cudaSuccess)
		throw std::runtime_error(std::string("cuda error: ") + what + ": " + cudaGetErrorString(e));
}

inline unsigned grid_blocks(int64_t n, int block = 256)
{
	int dev = 0, sms = 0;
	cudaGetDevice(&dev);
	cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
	int64_t need = (n + block - 1) / block, cap = int64_t(sms > 0 ? sms : 1) * 8;
	return unsigned(need < 1 ? 1 : (need < cap ? need : cap));
}

template <class F, class T, class... Ts>
__global__ void apply_kernel(F f, int64_t V, FieldView<T> a, FieldView<Ts>... as)
{
	for (int64_t s = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; s < V; s += int64_t(gridDim.x) * blockDim.x)
	{
		T x = a.load(s);
		f(x, static_cast<Ts const &>(as.load(s))...);
		a.store(s, x);
	}
}

// lattice_apply (lattice.h:256-261, device.h:219-228)
template <class F, class T, class... Ts>
void lattice_apply_on(cudaStream_t stream, F f, FieldView<T> a, FieldView<Ts>... as)
{
	apply_kernel<<<grid_blocks(a.V), 256, 0, stream>>>(f, a.V, a, as...);
	cuda_ok(cudaGetLastError(), "lattice_apply launch");
}
template <class F, class T, class... Ts> void lattice_apply(F f, FieldView<T> a, FieldView<Ts>... as)
{
	lattice_apply_on(cudaStream_t(nullptr), f, a, as...);
}

template <int BLOCK, class R, class F, class T, class... Ts>
__global__ void sum_kernel(F f, int64_t V, R *partials, unsigned *counter, R *result, FieldView<T> a,
                           FieldView<Ts>... as)
{
	__shared__ R sm[BLOCK];
	__shared__ bool last;
	R acc{};
	for (int64_t s = int64_t(blockIdx.x) * BLOCK + threadIdx.x; s < V; s += int64_t(gridDim.x) * BLOCK)
		acc += f(a.load(s), as.load(s)...);
	sm[threadIdx.x] = acc;
	__syncthreads();
	for (int st = BLOCK / 2; st > 0; st /= 2)
	{
		if (int(threadIdx.x) < st)
			sm[threadIdx.x] += sm[threadIdx.x + st];
		__syncthreads();
	}
	if (threadIdx.x == 0)
	{
		partials[blockIdx.x] = sm[0];
		__threadfence();
		last = atomicInc(counter, gridDim.x - 1) == gridDim.x - 1;
	}
	__syncthreads();
	if (last && threadIdx.x == 0)
	{
		// the other blocks' partials, read past L1 (written by other SMs)
		R r{};
		for (unsigned b = 0; b < gridDim.x; ++b)
		{
			R v;
			unsigned char volatile const *src = reinterpret_cast<unsigned char volatile const *>(partials + b);
			unsigned char *dst = reinterpret_cast<unsigned char *>(&v);
			for (size_t k = 0; k < sizeof(R); ++k)
				dst[k] = src[k];
			r += v;
		}
		*result = r;
	}
}

// lattice_sum_apply (lattice.h:263-268, device.h:185-212,246-265); returns
// the sum on the host (synchronises the stream, as the reference does)
template <class F, class T, class... Ts>
auto lattice_sum_apply_on(cudaStream_t stream, F f, FieldView<T> a, FieldView<Ts>... as)
{
	using R = std::decay_t<decltype(f(std::declval<T const &>(), std::declval<Ts const &>()...))>;
	static_assert(std::is_trivially_copyable_v<R>, "sum type must be trivially copyable");
	constexpr int B = 256;
	int64_t V = a.V;
	unsigned blocks = grid_blocks(V, B);
	if (blocks > 1024)
		blocks = 1024;
	void *buf = nullptr;
	size_t bytes = sizeof(R) * (size_t(blocks) + 1) + sizeof(unsigned);
	cuda_ok(cudaMallocAsync(&buf, bytes, stream), "cudaMallocAsync");
	R *partials = static_cast<R *>(buf);
	R *result = partials + blocks;
	unsigned *counter = reinterpret_cast<unsigned *>(result + 1);
	cuda_ok(cudaMemsetAsync(counter, 0, sizeof(unsigned), stream), "cudaMemsetAsync");
	sum_kernel<B, R><<<blocks, B, 0, stream>>>(f, V, partials, counter, result, a, as...);
	cuda_ok(cudaGetLastError(), "lattice_sum_apply launch");
	R host{};
	cuda_ok(cudaMemcpyAsync(&host, result, sizeof(R), cudaMemcpyDeviceToHost, stream), "cudaMemcpyAsync");
	cuda_ok(cudaFreeAsync(buf, stream), "cudaFreeAsync");
	cuda_ok(cudaStreamSynchronize(stream), "cudaStreamSynchronize");
	return host;
}
template <class F, class T, class... Ts> auto lattice_sum_apply(F f, FieldView<T> a, FieldView<Ts>... as)
{
	return lattice_sum_apply_on(cudaStream_t(nullptr), f, a, as...);
}

// the functor of lattice_sum: the object itself
struct Identity
{
	template <class T> __device__ T operator()(T const &x) const { return x; }
};

// lattice_sum (lattice.h:270-273)
template <class T> T lattice_sum(FieldView<T> a, cudaStream_t stream = nullptr)
{
	return lattice_sum_apply_on(stream, Identity{}, a);
}

// geometry for cshift on the even/odd order (all extents even)
struct EoGrid
{
	int nd;
	int L[4];
	int64_t stride[4];
	int64_t V;
	static EoGrid make(int nd, int32_t const *dims)
	{
		EoGrid g{};
		g.nd = nd;
		g.V = 1;
		for (int i = nd - 1; i >= 0; --i)
		{
			g.L[i] = dims[i];
			g.stride[i] = g.V;
			g.V *= dims[i];
		}
		return g;
	}
};

template <class T>
__global__ void cshift_kernel(EoGrid g, int dir, int offset, FieldView<T> dst, FieldView<T> src)
{
	int64_t Vh = g.V / 2;
	for (int64_t s = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; s < g.V; s += int64_t(gridDim.x) * blockDim.x)
	{
		int p = s >= Vh;
		int64_t r = (s - p * Vh) * 2;
		int x[4] = {0, 0, 0, 0}, sum = 0;
		int64_t q = r;
		for (int i = g.nd - 1; i >= 0; --i)
		{
			x[i] = int(q % g.L[i]);
			q /= g.L[i];
			sum += x[i];
		}
		if ((sum & 1) != p)
		{
			x[g.nd - 1] += 1;
			r += 1;
		}
		int xn = ((x[dir] + offset) % g.L[dir] + g.L[dir]) % g.L[dir];
		int64_t rn = r + int64_t(xn - x[dir]) * g.stride[dir];
		int pn = (p + (xn - x[dir])) & 1;
		dst.store(s, src.load(int64_t(pn) * Vh + rn / 2));
	}
}

// cshift (lattice.h:366-389): dst[x] = src[x + offset * e_dir], periodic
template <class T>
void cshift(int nd, int32_t const *dims, FieldView<T> dst, FieldView<T> src, int dir, int offset,
            cudaStream_t stream = nullptr)
{
	EoGrid g = EoGrid::make(nd, dims);
	cshift_kernel<<<grid_blocks(g.V), 256, 0, stream>>>(g, dir, offset, dst, src);
	cuda_ok(cudaGetLastError(), "cshift launch");
}

} // namespace device
} // namespace mesh
