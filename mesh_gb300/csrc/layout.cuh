// Device data layout: even/odd (checkerboard) site order, structure-of-arrays
// planes read and written with 128-bit coalesced accesses.
//
// Site order. The reference indexes sites lexicographically with dimension 0
// slowest (src/lattice/grid.h:39-49): r = (((x0 L1 + x1) L2 + x2) L3 + x3).
// The device order puts all even sites (sum of coordinates even) first, then
// all odd sites, each parity in lexicographic order:
//     eo(r) = parity(r) * V/2 + floor(r / 2).
// This is a bijection when the last extent is even (sites 2k and 2k+1 differ
// in parity); every extent must be even for the checkerboard to be a proper
// two-colouring under periodic wrap-around, which the library requires.
//
// Field storage. A field holds `nstack` components (the directions mu of a
// gauge field) of V objects of NR reals. Component c occupies NR*V reals at
// offset c*NR*V; inside it the NR reals of every site are split into planes:
// float: floor(NR/4) float4 planes, then a float2 plane if NR%4 >= 2, then a
// float plane if NR is odd; double: floor(NR/2) double2 planes, then a double
// plane if NR is odd. Plane p of site s sits at plane_base + s, so a warp's
// 32 consecutive sites read 32 consecutive 16-byte words.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

namespace meshgb {

struct Geom
{
	int nd;
	int L[4];
	int64_t V, Vh;
	int64_t stride[4]; // lexicographic stride of dimension i
	// division by L[i] as a multiply and shift: n / L[i] == (n * dm[i]) >> ds[i]
	// for every n < 2^31 (ds = 31 + ceil(log2 L), dm = floor(2^ds / L) + 1 <
	// 2^33, so n * dm < 2^64; the rounding error n / 2^ds < 1 / L)
	uint64_t dm[4];
	int ds[4];

	// extent / stride of a runtime direction through selects on constant
	// offsets (indexing the kernel-parameter arrays with a runtime index
	// would copy the struct to local memory)
	__host__ __device__ __forceinline__ int Ld(int d) const
	{
		return d == 0 ? L[0] : d == 1 ? L[1] : d == 2 ? L[2] : L[3];
	}
	__host__ __device__ __forceinline__ int32_t Sd(int d) const
	{
		return int32_t(d == 0 ? stride[0] : d == 1 ? stride[1] : d == 2 ? stride[2] : stride[3]);
	}
};

inline Geom make_geom(int nd, int32_t const *dims)
{
	Geom g{};
	g.nd = nd;
	g.V = 1;
	for (int i = 0; i < 4; ++i)
		g.L[i] = i < nd ? dims[i] : 1;
	for (int i = nd - 1; i >= 0; --i)
	{
		g.stride[i] = g.V;
		g.V *= g.L[i];
	}
	for (int i = nd; i < 4; ++i)
		g.stride[i] = 0;
	for (int i = 0; i < 4; ++i)
	{
		int l = 0;
		while ((1 << l) < g.L[i])
			++l;
		g.ds[i] = 31 + l;
		g.dm[i] = (uint64_t(1) << g.ds[i]) / uint64_t(g.L[i]) + 1;
	}
	g.Vh = g.V / 2;
	return g;
}

// Coordinates, lexicographic index and parity of a site. The coordinates are
// packed 8 bits per dimension into one register (extents < 256), so that a
// runtime direction selects one with a shift: no local-memory arrays.
template <int ND> struct Site
{
	uint32_t px;  // coordinate i in bits [8i, 8i+8)
	int32_t lex;  // lexicographic index (V < 2^31)
	int par;      // parity of the coordinate sum
	__device__ __forceinline__ int x(int i) const { return int((px >> (8 * i)) & 0xffu); }
};

template <int ND> __device__ __forceinline__ Site<ND> site_from_eo(Geom const &g, int64_t s)
{
	Site<ND> st;
	int p = s >= g.Vh ? 1 : 0;
	// V < 2^31 is enforced at field creation: 32-bit division suffices
	uint32_t r = uint32_t(s - p * g.Vh) * 2u;
	int sum = 0;
	uint32_t px = 0;
#pragma unroll
	for (int i = ND - 1; i >= 0; --i)
	{
		uint32_t L = uint32_t(g.L[i]);
		uint32_t q = uint32_t((uint64_t(r) * g.dm[i]) >> g.ds[i]);
		uint32_t xi = r - q * L;
		px |= xi << (8 * i);
		r = q;
		sum += int(xi);
	}
	int32_t lex = int32_t(s - p * g.Vh) * 2;
	if ((sum & 1) != p)
	{
		px += 1u << (8 * (ND - 1));
		lex += 1;
	}
	st.px = px;
	st.lex = lex;
	st.par = p;
	return st;
}

// site with the given coordinates (each in range)
template <int ND> __device__ __forceinline__ Site<ND> site_from_coords(Geom const &g, int const *x)
{
	Site<ND> st;
	uint32_t px = 0;
	int32_t lex = 0;
	int sum = 0;
#pragma unroll
	for (int i = 0; i < ND; ++i)
	{
		px |= uint32_t(x[i]) << (8 * i);
		lex = lex * g.L[i] + x[i];
		sum += x[i];
	}
	st.px = px;
	st.lex = lex;
	st.par = sum & 1;
	return st;
}

template <int ND> __device__ __forceinline__ int64_t eo_of(Geom const &g, Site<ND> const &st)
{
	return int64_t(st.par) * g.Vh + (st.lex >> 1);
}

// lexicographic index after a step of `sign` (+-1) in direction dir
__device__ __forceinline__ int32_t lex_step(Geom const &g, uint32_t px, int32_t lex, int dir, int sign)
{
	int xd = int((px >> (8 * dir)) & 0xffu) + sign;
	int L = g.Ld(dir);
	int32_t st = g.Sd(dir);
	if (xd == L)
		return lex - (L - 1) * st;
	if (xd < 0)
		return lex + (L - 1) * st;
	return lex + sign * st;
}

// even/odd index of the neighbour x + sign e_dir (opposite parity)
template <int ND>
__device__ __forceinline__ int64_t eo_shift1(Geom const &g, Site<ND> const &st, int dir, int sign)
{
	int32_t lex = lex_step(g, st.px, st.lex, dir, sign);
	return int64_t(st.par ^ 1) * g.Vh + (lex >> 1);
}

// neighbour at x + s1 e_d1 + s2 e_d2 (d1 != d2); same parity as x
template <int ND>
__device__ __forceinline__ int64_t eo_shift2(Geom const &g, Site<ND> const &st, int d1, int s1, int d2, int s2)
{
	int32_t lex = lex_step(g, st.px, st.lex, d1, s1);
	lex = lex_step(g, st.px, lex, d2, s2);
	return int64_t(st.par) * g.Vh + (lex >> 1);
}

// host-side even/odd index of a lexicographic site (same formula)
inline int64_t eo_index_host(Geom const &g, int64_t r)
{
	int64_t q = r;
	int sum = 0;
	for (int i = g.nd - 1; i >= 0; --i)
	{
		sum += int(q % g.L[i]);
		q /= g.L[i];
	}
	return int64_t(sum & 1) * g.Vh + r / 2;
}

// ---------------------------------------------------------------------------
// cache-policy loads/stores: links are re-read by neighbouring sites (keep
// them in L1), momenta are touched once per kernel (stream them past L1)
// ---------------------------------------------------------------------------
enum CachePolicy
{
	CACHE_DEFAULT = 0,
	CACHE_KEEP = 1,   // read-only path, L1 evict_last
	CACHE_STREAM = 2, // evict-first streaming
};

template <int CP> __device__ __forceinline__ float4 ld4(float4 const *p)
{
	if constexpr (CP == CACHE_KEEP)
	{
		float4 r;
		asm volatile("ld.global.nc.L1::evict_last.v4.f32 {%0,%1,%2,%3}, [%4];"
		             : "=f"(r.x), "=f"(r.y), "=f"(r.z), "=f"(r.w)
		             : "l"(p));
		return r;
	}
	else if constexpr (CP == CACHE_STREAM)
		return __ldcs(p);
	else
		return *p;
}
template <int CP> __device__ __forceinline__ float2 ld2(float2 const *p)
{
	if constexpr (CP == CACHE_KEEP)
	{
		float2 r;
		asm volatile("ld.global.nc.L1::evict_last.v2.f32 {%0,%1}, [%2];" : "=f"(r.x), "=f"(r.y) : "l"(p));
		return r;
	}
	else if constexpr (CP == CACHE_STREAM)
		return __ldcs(p);
	else
		return *p;
}
template <int CP> __device__ __forceinline__ float ld1(float const *p)
{
	if constexpr (CP == CACHE_KEEP)
		return __ldg(p);
	else if constexpr (CP == CACHE_STREAM)
		return __ldcs(p);
	else
		return *p;
}
template <int CP> __device__ __forceinline__ double2 ld2d(double2 const *p)
{
	if constexpr (CP == CACHE_KEEP)
	{
		double2 r;
		asm volatile("ld.global.nc.L1::evict_last.v2.f64 {%0,%1}, [%2];" : "=d"(r.x), "=d"(r.y) : "l"(p));
		return r;
	}
	else if constexpr (CP == CACHE_STREAM)
		return __ldcs(p);
	else
		return *p;
}
template <int CP> __device__ __forceinline__ double ld1d(double const *p)
{
	if constexpr (CP == CACHE_KEEP)
		return __ldg(p);
	else if constexpr (CP == CACHE_STREAM)
		return __ldcs(p);
	else
		return *p;
}
template <int CP, class V> __device__ __forceinline__ void stv(V *p, V v)
{
	if constexpr (CP == CACHE_STREAM)
		__stcs(p, v);
	else
		*p = v;
}

// ---------------------------------------------------------------------------
// structure-of-arrays planes
// ---------------------------------------------------------------------------
template <class T, int NR> struct Soa;

template <int NR> struct Soa<float, NR>
{
	static constexpr int N4 = NR / 4;
	static constexpr int R = NR % 4;
	template <int CP = CACHE_DEFAULT>
	__device__ __forceinline__ static void load(float const *__restrict__ base, int64_t V, int64_t s, float *v)
	{
		float4 const *p4 = reinterpret_cast<float4 const *>(base);
#pragma unroll
		for (int k = 0; k < N4; ++k)
		{
			float4 t = ld4<CP>(p4 + (k * V + s));
			v[4 * k] = t.x;
			v[4 * k + 1] = t.y;
			v[4 * k + 2] = t.z;
			v[4 * k + 3] = t.w;
		}
		float const *tail = base + int64_t(4 * N4) * V;
		if constexpr (R >= 2)
		{
			float2 t = ld2<CP>(reinterpret_cast<float2 const *>(tail) + s);
			v[4 * N4] = t.x;
			v[4 * N4 + 1] = t.y;
			tail += 2 * V;
		}
		if constexpr (R & 1)
			v[NR - 1] = ld1<CP>(tail + s);
	}
	// the first K reals (K a multiple of 4, K <= 4 N4): the leading float4 planes
	template <int K, int CP = CACHE_DEFAULT>
	__device__ __forceinline__ static void load_head(float const *__restrict__ base, int64_t V, int64_t s, float *v)
	{
		static_assert(K % 4 == 0 && K <= 4 * N4, "head must be whole float4 planes");
		float4 const *p4 = reinterpret_cast<float4 const *>(base);
#pragma unroll
		for (int k = 0; k < K / 4; ++k)
		{
			float4 t = ld4<CP>(p4 + (k * V + s));
			v[4 * k] = t.x;
			v[4 * k + 1] = t.y;
			v[4 * k + 2] = t.z;
			v[4 * k + 3] = t.w;
		}
	}
	template <int CP = CACHE_DEFAULT>
	__device__ __forceinline__ static void store(float *__restrict__ base, int64_t V, int64_t s, float const *v)
	{
		float4 *p4 = reinterpret_cast<float4 *>(base);
#pragma unroll
		for (int k = 0; k < N4; ++k)
			stv<CP>(p4 + (k * V + s), make_float4(v[4 * k], v[4 * k + 1], v[4 * k + 2], v[4 * k + 3]));
		float *tail = base + int64_t(4 * N4) * V;
		if constexpr (R >= 2)
		{
			stv<CP>(reinterpret_cast<float2 *>(tail) + s, make_float2(v[4 * N4], v[4 * N4 + 1]));
			tail += 2 * V;
		}
		if constexpr (R & 1)
			stv<CP>(tail + s, v[NR - 1]);
	}
};

template <int NR> struct Soa<double, NR>
{
	static constexpr int N2 = NR / 2;
	template <int CP = CACHE_DEFAULT>
	__device__ __forceinline__ static void load(double const *__restrict__ base, int64_t V, int64_t s, double *v)
	{
		double2 const *p2 = reinterpret_cast<double2 const *>(base);
#pragma unroll
		for (int k = 0; k < N2; ++k)
		{
			double2 t = ld2d<CP>(p2 + (k * V + s));
			v[2 * k] = t.x;
			v[2 * k + 1] = t.y;
		}
		if constexpr (NR & 1)
			v[NR - 1] = ld1d<CP>(base + int64_t(2 * N2) * V + s);
	}
	// the first K reals (K even): the leading double2 planes
	template <int K, int CP = CACHE_DEFAULT>
	__device__ __forceinline__ static void load_head(double const *__restrict__ base, int64_t V, int64_t s, double *v)
	{
		static_assert(K % 2 == 0 && K <= 2 * N2, "head must be whole double2 planes");
		double2 const *p2 = reinterpret_cast<double2 const *>(base);
#pragma unroll
		for (int k = 0; k < K / 2; ++k)
		{
			double2 t = ld2d<CP>(p2 + (k * V + s));
			v[2 * k] = t.x;
			v[2 * k + 1] = t.y;
		}
	}
	template <int CP = CACHE_DEFAULT>
	__device__ __forceinline__ static void store(double *__restrict__ base, int64_t V, int64_t s, double const *v)
	{
		double2 *p2 = reinterpret_cast<double2 *>(base);
#pragma unroll
		for (int k = 0; k < N2; ++k)
			stv<CP>(p2 + (k * V + s), make_double2(v[2 * k], v[2 * k + 1]));
		if constexpr (NR & 1)
			stv<CP>(base + int64_t(2 * N2) * V + s, v[NR - 1]);
	}
};

// typed view of one component (direction) of a field
template <class T, int NR> struct View
{
	T *base;
	int64_t V;
	template <int CP = CACHE_DEFAULT> __device__ __forceinline__ void load(int64_t s, T *v) const
	{
		Soa<T, NR>::template load<CP>(base, V, s, v);
	}
	template <int CP = CACHE_DEFAULT> __device__ __forceinline__ void store(int64_t s, T const *v) const
	{
		Soa<T, NR>::template store<CP>(base, V, s, v);
	}
};

template <class T, int NR> __host__ __device__ __forceinline__ View<T, NR> comp(T *base, int64_t V, int c)
{
	return {base + int64_t(c) * NR * V, V};
}

} // namespace meshgb
