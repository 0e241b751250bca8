// Kernels of the lattice-gauge hot path, templated over group (U(1), SU(2),
// SU(3)), real type and number of dimensions, and their host launchers.
// Instantiated per group in inst_u1.cu / inst_su2.cu / inst_su3.cu.
#pragma once

#include "field.cuh"
#include "group.cuh"
#include "heatbath.cuh"
#include "rng.cuh"

#include <string>
#include <type_traits>

namespace meshgb {

constexpr int kBlock = 256;

template <class T> __device__ __forceinline__ T *tptr(void *p) { return static_cast<T *>(p); }
template <class T> __device__ __forceinline__ T const *tptr(void const *p) { return static_cast<T const *>(p); }

// grid-stride loop over n items
#define MESH_GRID_LOOP(i, n)                                                                                       \
	for (int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < (n); i += int64_t(gridDim.x) * blockDim.x)

// ---------------------------------------------------------------------------
// host <-> device layout conversion (Lattice::copy_from_host/copy_to_host)
// ---------------------------------------------------------------------------

// host layout: [c][lex][NRH]; device: component c, even/odd SoA of NR reals
template <int GRP, class T, int ND, bool ALG>
__global__ void __launch_bounds__(kBlock) k_import(Geom g, int nstack, T const *__restrict__ host, T *__restrict__ dev)
{
	using Gp = Group<GRP, T>;
	constexpr int NRH = Gp::NR;
	constexpr int NR = ALG ? Gp::NA : Gp::NR;
	int64_t n = int64_t(nstack) * g.V;
	MESH_GRID_LOOP(i, n)
	{
		int c = int(i / g.V);
		int64_t s = i - int64_t(c) * g.V;
		Site<ND> st = site_from_eo<ND>(g, s);
		T const *src = host + (int64_t(c) * g.V + st.lex) * NRH;
		T v[NR];
		if constexpr (!ALG)
		{
#pragma unroll
			for (int k = 0; k < NR; ++k)
				v[k] = src[k];
		}
		else if constexpr (GRP == U1)
			v[0] = src[1];
		else if constexpr (GRP == SU2)
		{
			v[0] = src[1];
			v[1] = src[2];
			v[2] = src[3];
		}
		else
		{
			// entries a00.im, a11.im, a01, a02, a12 of the antihermitian matrix
			v[0] = src[1];
			v[1] = src[9];
			v[2] = src[2];
			v[3] = src[3];
			v[4] = src[4];
			v[5] = src[5];
			v[6] = src[10];
			v[7] = src[11];
		}
		comp<T, NR>(dev, g.V, c).store(s, v);
	}
}

template <int GRP, class T, int ND, bool ALG>
__global__ void __launch_bounds__(kBlock) k_export(Geom g, int nstack, T const *__restrict__ dev, T *__restrict__ host)
{
	using Gp = Group<GRP, T>;
	constexpr int NRH = Gp::NR;
	constexpr int NR = ALG ? Gp::NA : Gp::NR;
	int64_t n = int64_t(nstack) * g.V;
	MESH_GRID_LOOP(i, n)
	{
		int c = int(i / g.V);
		int64_t s = i - int64_t(c) * g.V;
		Site<ND> st = site_from_eo<ND>(g, s);
		T v[NR];
		comp<T, NR>(const_cast<T *>(dev), g.V, c).load(s, v);
		T *dst = host + (int64_t(c) * g.V + st.lex) * NRH;
		if constexpr (!ALG)
		{
#pragma unroll
			for (int k = 0; k < NR; ++k)
				dst[k] = v[k];
		}
		else
		{
			typename Gp::E e = Gp::from_alg(v);
#pragma unroll
			for (int k = 0; k < NRH; ++k)
				dst[k] = e.v[k];
		}
	}
}

// Direct host transfers: the host buffer is mapped into the device's address
// space (pinned memory), so the conversion kernel reads or writes it over the
// host link itself, without a staging copy. A block moves kBlock consecutive
// host objects of one component as contiguous 16-byte words through shared
// memory (the host side stays coalesced) and the threads scatter them to (or
// gather them from) the even/odd device layout. The host buffer must be
// 16-byte aligned.
template <int ND> __device__ __forceinline__ int64_t eo_of_lex(Geom const &g, int64_t lex)
{
	uint32_t r = uint32_t(lex);
	int sum = 0;
#pragma unroll
	for (int i = ND - 1; i >= 0; --i)
	{
		uint32_t L = uint32_t(g.L[i]);
		uint32_t q = uint32_t((uint64_t(r) * g.dm[i]) >> g.ds[i]);
		sum += int(r - q * L);
		r = q;
	}
	return int64_t(sum & 1) * g.Vh + (lex >> 1);
}

template <int GRP, class T, int ND, bool ALG>
__global__ void __launch_bounds__(kBlock)
    k_import_direct(Geom g, int nstack, T const *__restrict__ host, T *__restrict__ dev)
{
	using Gp = Group<GRP, T>;
	constexpr int NRH = Gp::NR;
	constexpr int NR = ALG ? Gp::NA : Gp::NR;
	__shared__ __align__(16) T tile[kBlock * NRH];
	int64_t bpc = (g.V + kBlock - 1) / kBlock; // blocks per component
	for (int64_t b = blockIdx.x; b < int64_t(nstack) * bpc; b += gridDim.x)
	{
		int c = int(b / bpc);
		int64_t lex0 = (b - int64_t(c) * bpc) * kBlock;
		int cnt = int(g.V - lex0 < kBlock ? g.V - lex0 : kBlock);
		T const *src = host + (int64_t(c) * g.V + lex0) * NRH;
		int nreal = cnt * NRH;
		int nvec = int((size_t(nreal) * sizeof(T)) / 16);
		constexpr int PER = 16 / sizeof(T);
		__syncthreads();
		for (int k = threadIdx.x; k < nvec; k += kBlock)
			reinterpret_cast<uint4 *>(tile)[k] = __ldcs(reinterpret_cast<uint4 const *>(src) + k);
		for (int k = nvec * PER + threadIdx.x; k < nreal; k += kBlock)
			tile[k] = src[k];
		__syncthreads();
		if (threadIdx.x < cnt)
		{
			int64_t lex = lex0 + threadIdx.x;
			T const *o = tile + threadIdx.x * NRH;
			T v[NR];
			if constexpr (!ALG)
			{
#pragma unroll
				for (int k = 0; k < NR; ++k)
					v[k] = o[k];
			}
			else if constexpr (GRP == U1)
				v[0] = o[1];
			else if constexpr (GRP == SU2)
			{
				v[0] = o[1];
				v[1] = o[2];
				v[2] = o[3];
			}
			else
			{
				v[0] = o[1];
				v[1] = o[9];
				v[2] = o[2];
				v[3] = o[3];
				v[4] = o[4];
				v[5] = o[5];
				v[6] = o[10];
				v[7] = o[11];
			}
			comp<T, NR>(dev, g.V, c).store(eo_of_lex<ND>(g, lex), v);
		}
	}
}

template <int GRP, class T, int ND, bool ALG>
__global__ void __launch_bounds__(kBlock)
    k_export_direct(Geom g, int nstack, T const *__restrict__ dev, T *__restrict__ host)
{
	using Gp = Group<GRP, T>;
	constexpr int NRH = Gp::NR;
	constexpr int NR = ALG ? Gp::NA : Gp::NR;
	__shared__ __align__(16) T tile[kBlock * NRH];
	int64_t bpc = (g.V + kBlock - 1) / kBlock;
	for (int64_t b = blockIdx.x; b < int64_t(nstack) * bpc; b += gridDim.x)
	{
		int c = int(b / bpc);
		int64_t lex0 = (b - int64_t(c) * bpc) * kBlock;
		int cnt = int(g.V - lex0 < kBlock ? g.V - lex0 : kBlock);
		__syncthreads();
		if (threadIdx.x < cnt)
		{
			T v[NR];
			comp<T, NR>(const_cast<T *>(dev), g.V, c).load(eo_of_lex<ND>(g, lex0 + threadIdx.x), v);
			T *o = tile + threadIdx.x * NRH;
			if constexpr (!ALG)
			{
#pragma unroll
				for (int k = 0; k < NR; ++k)
					o[k] = v[k];
			}
			else
			{
				typename Gp::E e = Gp::from_alg(v);
#pragma unroll
				for (int k = 0; k < NRH; ++k)
					o[k] = e.v[k];
			}
		}
		__syncthreads();
		T *dst = host + (int64_t(c) * g.V + lex0) * NRH;
		int nreal = cnt * NRH;
		int nvec = int((size_t(nreal) * sizeof(T)) / 16);
		constexpr int PER = 16 / sizeof(T);
		for (int k = threadIdx.x; k < nvec; k += kBlock)
			__stcs(reinterpret_cast<uint4 *>(dst) + k, reinterpret_cast<uint4 const *>(tile)[k]);
		for (int k = nvec * PER + threadIdx.x; k < nreal; k += kBlock)
			dst[k] = tile[k];
	}
}

// ---------------------------------------------------------------------------
// initialisation and random fields
// ---------------------------------------------------------------------------
template <int GRP, class T>
__global__ void __launch_bounds__(kBlock) k_set_unit(int64_t n_total, int64_t V, T *__restrict__ dev)
{
	using Gp = Group<GRP, T>;
	MESH_GRID_LOOP(i, n_total)
	{
		int c = int(i / V);
		int64_t s = i - int64_t(c) * V;
		auto e = Gp::unit();
		comp<T, Gp::NR>(dev, V, c).store(s, e.v);
	}
}

template <int GRP, class T, int ND>
__global__ void __launch_bounds__(kBlock)
    k_random_group(Geom g, int nstack, uint64_t seed, uint64_t counter, uint32_t tag, T *__restrict__ dev)
{
	using Gp = Group<GRP, T>;
	int64_t n = int64_t(nstack) * g.V;
	MESH_GRID_LOOP(i, n)
	{
		int c = int(i / g.V);
		int64_t s = i - int64_t(c) * g.V;
		Site<ND> st = site_from_eo<ND>(g, s);
		T p[Gp::NNORM_GROUP];
		normals<T, Gp::NNORM_GROUP>(seed, tag, uint32_t(st.lex), uint32_t(c), counter, p);
		auto e = Gp::group_from_normals(p);
		comp<T, Gp::NR>(dev, g.V, c).store(s, e.v);
	}
}

// Gaussian momenta; also sums the kinetic energy norm2(P) in FP64
template <int GRP, class T, int ND>
__global__ void __launch_bounds__(kBlock)
    k_random_alg(Geom g, int nstack, uint64_t seed, uint64_t const *counter_dev, uint64_t counter, T *__restrict__ dev,
                 RedSlot kin)
{
	using Gp = Group<GRP, T>;
	uint64_t ctr = counter_dev ? *counter_dev : counter;
	int64_t n = int64_t(nstack) * g.V;
	double acc = 0.0;
	MESH_GRID_LOOP(i, n)
	{
		int c = int(i / g.V);
		int64_t s = i - int64_t(c) * g.V;
		Site<ND> st = site_from_eo<ND>(g, s);
		T p[Gp::DIM], o[Gp::NA];
		normals<T, Gp::DIM>(seed, TAG_MOMENTUM, uint32_t(st.lex), uint32_t(c), ctr, p);
		Gp::alg_from_normals(p, o);
		comp<T, Gp::NA>(dev, g.V, c).store(s, o);
		acc += double(Gp::kin(o));
	}
	if (kin.result)
		grid_sum<kBlock>(acc, kin);
}

// sum over all components of the (kinetic) norm2
template <int GRP, class T, bool ALG>
__global__ void __launch_bounds__(kBlock) k_norm2(int64_t n_total, int64_t V, T const *__restrict__ dev, RedSlot out)
{
	using Gp = Group<GRP, T>;
	constexpr int NR = ALG ? Gp::NA : Gp::NR;
	double acc = 0.0;
	MESH_GRID_LOOP(i, n_total)
	{
		int c = int(i / V);
		int64_t s = i - int64_t(c) * V;
		T v[NR];
		comp<T, NR>(const_cast<T *>(dev), V, c).load(s, v);
		if constexpr (ALG)
			acc += double(Gp::kin(v));
		else
		{
			T t = 0;
#pragma unroll
			for (int k = 0; k < NR; ++k)
				t += v[k] * v[k];
			acc += double(t);
		}
	}
	grid_sum<kBlock>(acc, out);
}

// ---------------------------------------------------------------------------
// lattice_apply layer (single-component group fields)
// ---------------------------------------------------------------------------
template <int GRP, class T, int ND>
__global__ void __launch_bounds__(kBlock)
    k_cshift(Geom g, int dir, int offset, T const *__restrict__ src, T *__restrict__ dst)
{
	using Gp = Group<GRP, T>;
	MESH_GRID_LOOP(s, g.V)
	{
		Site<ND> st = site_from_eo<ND>(g, s);
		int L = g.Ld(dir);
		int x0 = st.x(dir);
		int xn = ((x0 + offset) % L + L) % L;
		int64_t lex = st.lex + int64_t(xn - x0) * g.Sd(dir);
		int par = (st.par + (xn - x0)) & 1;
		int64_t sn = int64_t(par) * g.Vh + (lex >> 1);
		T v[Gp::NR];
		Soa<T, Gp::NR>::load(src, g.V, sn, v);
		Soa<T, Gp::NR>::store(dst, g.V, s, v);
	}
}

template <int GRP, class T>
__global__ void __launch_bounds__(kBlock)
    k_site_op(int op, int64_t V, T const *__restrict__ a, T const *__restrict__ b, T *__restrict__ dst)
{
	using Gp = Group<GRP, T>;
	using E = typename Gp::E;
	MESH_GRID_LOOP(s, V)
	{
		E x, y, r;
		if (op == SITE_EXP) // a holds packed algebra elements
		{
			T o[Gp::NA];
			Soa<T, Gp::NA>::load(a, V, s, o);
			r = Gp::exp_alg(o, T(1));
			Soa<T, Gp::NR>::store(dst, V, s, r.v);
			continue;
		}
		Soa<T, Gp::NR>::load(a, V, s, x.v);
		if (op == SITE_PROJ) // dst holds packed algebra elements
		{
			T o[Gp::NA];
			Gp::proj(x, o);
			Soa<T, Gp::NA>::store(dst, V, s, o);
			continue;
		}
		if (op == SITE_MUL)
		{
			Soa<T, Gp::NR>::load(b, V, s, y.v);
			r = Gp::mul(x, y);
		}
		else if (op == SITE_ADJ)
			r = Gp::adj(x);
		else
			r = x;
		Soa<T, Gp::NR>::store(dst, V, s, r.v);
	}
}

template <int GRP, class T>
__global__ void __launch_bounds__(kBlock) k_sum_real_trace(int64_t V, T const *__restrict__ a, RedSlot out)
{
	using Gp = Group<GRP, T>;
	double acc = 0.0;
	MESH_GRID_LOOP(s, V)
	{
		typename Gp::E x;
		Soa<T, Gp::NR>::load(a, V, s, x.v);
		acc += double(Gp::retr(x));
	}
	grid_sum<kBlock>(acc, out);
}

// ---------------------------------------------------------------------------
// gauge action and force
// ---------------------------------------------------------------------------
// Link loads of a gauge field. ROWS: SU(3) links are read as their rows 0
// and 1 (the first 12 reals: whole leading planes of the layout) and row 2
// is rebuilt as conj(row0 x row1), which is exact for special unitary
// matrices: a third less link traffic. Used only where the links are SU(3)
// by construction (the HMC trajectory and the batched replicas).
template <int GRP, class T, int ND, bool ROWS = false> struct LinkLoad
{
	using Gp = Group<GRP, T>;
	using E = typename Gp::E;
	T const *U;
	int64_t V;
	__device__ __forceinline__ E operator()(int mu, int64_t s) const
	{
		E e;
		if constexpr (ROWS && GRP == SU3)
		{
			Soa<T, Gp::NR>::template load_head<12, CACHE_KEEP>(U + int64_t(mu) * Gp::NR * V, V, s, e.v);
			Gp::complete_row2(e);
		}
		else
			Soa<T, Gp::NR>::template load<CACHE_KEEP>(U + int64_t(mu) * Gp::NR * V, V, s, e.v);
		return e;
	}
	// rows 0 and 1 only (row 2 left unset) where ROWS applies; else the link
	__device__ __forceinline__ E rows(int mu, int64_t s) const
	{
		if constexpr (ROWS && GRP == SU3)
		{
			E e;
			Soa<T, Gp::NR>::template load_head<12, CACHE_KEEP>(U + int64_t(mu) * Gp::NR * V, V, s, e.v);
			return e;
		}
		else
			return (*this)(mu, s);
	}
};

// SU(3) FP32 rows-0,1 loads with 32-bit offsets in float4 units (the
// thread-per-site kernel: one wide multiply-add per float4 instead of 64-bit
// index arithmetic); valid while 18 V < 2^32 float4s (V < 238 M sites)
struct LinkLoadSU3R32
{
	using E = Group<SU3, float>::E;
	float4 const *U4;
	uint32_t V, Vmu; // sites per parity plane pair; float4s per direction (4.5 V)
	__host__ __device__ static bool fits(int64_t V) { return 18 * V < (int64_t(1) << 32); }
	__device__ __forceinline__ E rows(int mu, int64_t s) const
	{
		uint32_t o = uint32_t(mu) * Vmu + uint32_t(s);
		E e;
#pragma unroll
		for (int k = 0; k < 3; ++k)
		{
			float4 t = ld4<CACHE_KEEP>(U4 + (o + uint32_t(k) * V));
			e.v[4 * k] = t.x;
			e.v[4 * k + 1] = t.y;
			e.v[4 * k + 2] = t.z;
			e.v[4 * k + 3] = t.w;
		}
		return e;
	}
	__device__ __forceinline__ E operator()(int mu, int64_t s) const
	{
		E e = rows(mu, s);
		Group<SU3, float>::complete_row2(e);
		return e;
	}
};

// rebuilt-row link loads for SU(3) in FP32 (the mixed-precision HMC links)
template <int GRP, class T> inline constexpr bool kRows = GRP == SU3 && sizeof(T) == 4;

// sum over the planes mu<nu at site s of ReTr(U_mu(x) U_nu(x+mu) U_mu(x+nu)^+ U_nu(x)^+)
template <int GRP, class T, int ND, class LD>
__device__ __forceinline__ T plaquette_site(Geom const &g, Site<ND> const &st, int64_t s, LD const &ld)
{
	using Gp = Group<GRP, T>;
	using E = typename Gp::E;
	T t = 0;
#pragma unroll
	for (int mu = 0; mu < ND; ++mu)
	{
		E a = ld(mu, s);
		int64_t xm = eo_shift1<ND>(g, st, mu, +1);
#pragma unroll
		for (int nu = mu + 1; nu < ND; ++nu)
		{
			E b = ld(nu, xm);
			E c = ld(mu, eo_shift1<ND>(g, st, nu, +1));
			E d = ld(nu, s);
			// ReTr((a b) (d c)^+)
			t += Gp::retr_nd(Gp::mul(a, b), Gp::mul(d, c));
		}
	}
	return t;
}

// sum over sites and planes of the plaquette traces
template <int GRP, class T, int ND, bool ROWS = false>
__global__ void __launch_bounds__(kBlock) k_plaquette(Geom g, T const *__restrict__ U, RedSlot out)
{
	LinkLoad<GRP, T, ND, ROWS> ld{U, g.V};
	double acc = 0.0;
	MESH_GRID_LOOP(s, g.V)
	{
		Site<ND> st = site_from_eo<ND>(g, s);
		acc += double(plaquette_site<GRP, T, ND>(g, st, s, ld));
	}
	grid_sum<kBlock>(acc, out);
}

// 3x3 products of the force: packed FP32x2 FMAs for SU(3) float when F2 = 1. mul_r2: the product of two
// special unitary matrices from rows 0 and 1 of the left one (row 2 of the
// result rebuilt); the plain product for the other groups.
template <int GRP, class T, int F2> struct Prod
{
	using Gp = Group<GRP, T>;
	using E = typename Gp::E;
	__device__ __forceinline__ static E mul(E const &a, E const &b) { return Gp::mul(a, b); }
	__device__ __forceinline__ static E mul_nd(E const &a, E const &b) { return Gp::mul_nd(a, b); }
	__device__ __forceinline__ static E mul_dn(E const &a, E const &b) { return Gp::mul_dn(a, b); }
	__device__ __forceinline__ static E mul_r2(E const &a, E const &b)
	{
		if constexpr (GRP == SU3)
			return Gp::mul_r2(a, b);
		else
			return Gp::mul(a, b);
	}
};
struct ProdF2
{
	using E = Group<SU3, float>::E;
	using S = Su3F2;
	__device__ __forceinline__ static E mul(E const &a, E const &b) { return S::template mul<3>(a, b); }
	__device__ __forceinline__ static E mul_nd(E const &a, E const &b) { return S::template mul_nd<3>(a, b); }
	// rows 0, 1 of a b and of a b^dagger (row 2 left unset)
	__device__ __forceinline__ static E mul_rows(E const &a, E const &b) { return S::template mul<2>(a, b); }
	// s + a^dagger b, the sum inside the products' FMA chains
	__device__ __forceinline__ static E add_dn(E const &s, E const &a, E const &b) { return S::add_dn(s, a, b); }
	__device__ __forceinline__ static E mul_nd_rows(E const &a, E const &b) { return S::template mul_nd<2>(a, b); }
	__device__ __forceinline__ static E mul_dn(E const &a, E const &b) { return S::mul_dn(a, b); }
	__device__ __forceinline__ static E mul_r2(E const &a, E const &b)
	{
		E r = S::template mul<2>(a, b);
		Group<SU3, float>::complete_row2(r);
		return r;
	}
};
template <> struct Prod<SU3, float, 1> : ProdF2
{
};

// staple sum for link (x, mu) in the reference's association and summation
// order (utils.h:119-137): for nu = 0..Nd-1, nu != mu, the upper staple
// U_nu(x+mu) (U_nu(x) U_mu(x+nu))^+ then the lower staple
// (U_mu(y) U_nu(y+mu))^+ U_nu(y) at y = x - nu. Runtime mu and a rolled nu
// loop keep one copy of the SU(3) body in the instruction cache.
template <int GRP, class T, int ND, bool F2 = false, class LD>
__device__ __forceinline__ typename Group<GRP, T>::E staple(Geom const &g, Site<ND> const &st, int64_t s, int mu,
                                                            LD const &ld)
{
	using Gp = Group<GRP, T>;
	using E = typename Gp::E;
	using Pr = Prod<GRP, T, F2>;
	E S = Gp::zero();
	int64_t xpm = eo_shift1<ND>(g, st, mu, +1);
#pragma unroll 1
	for (int nu = 0; nu < ND; ++nu)
	{
		if (nu == mu)
			continue;
		{
			E b = ld(nu, xpm);
			E c = ld(mu, eo_shift1<ND>(g, st, nu, +1));
			E d = ld(nu, s);
			Gp::add_to(S, Pr::mul_nd(b, Pr::mul(d, c)));
		}
		{
			int64_t y = eo_shift1<ND>(g, st, nu, -1);
			E e = ld(mu, y);
			E f = ld(nu, eo_shift2<ND>(g, st, nu, -1, mu, +1));
			E h = ld(nu, y);
			Gp::add_to(S, Pr::mul_dn(Pr::mul(e, f), h));
		}
	}
	return S;
}

// one link's momentum update: P_mu(x) -= coef proj(U_mu(x) S_mu(x)); returns
// the kinetic norm of the updated momentum
template <int GRP, class T, int ND, bool F2 = false, class LD>
__device__ __forceinline__ double force_item(Geom const &g, Site<ND> const &st, int64_t s, int mu, LD const &ld,
                                             T *__restrict__ P, T coef)
{
	using Gp = Group<GRP, T>;
	using E = typename Gp::E;
	E S = staple<GRP, T, ND, F2>(g, st, s, mu, ld);
	E W = Prod<GRP, T, F2>::mul(ld(mu, s), S);
	T f[Gp::NA], p[Gp::NA];
	Gp::proj(W, f);
	auto Pv = comp<T, Gp::NA>(P, g.V, mu);
	Pv.template load<CACHE_STREAM>(s, p);
#pragma unroll
	for (int k = 0; k < Gp::NA; ++k)
		p[k] -= coef * f[k];
	Pv.template store<CACHE_STREAM>(s, p);
	return double(Gp::kin(p));
}

// Momentum step, one thread per (site, mu) in even/odd order.
template <int GRP, class T, int ND, int NT, int MINB, bool ROWS = false>
__global__ void __launch_bounds__(NT, MINB)
    k_momentum_step(Geom g, T const *__restrict__ U, T *__restrict__ P, T coef, RedSlot kin)
{
	LinkLoad<GRP, T, ND, ROWS> ld{U, g.V};
	double acc = 0.0;
	int64_t n = int64_t(ND) * g.V;
	for (int64_t i = int64_t(blockIdx.x) * NT + threadIdx.x; i < n; i += int64_t(gridDim.x) * NT)
	{
		int mu = int(i / g.V);
		int64_t s = i - int64_t(mu) * g.V;
		Site<ND> st = site_from_eo<ND>(g, s);
		double k = force_item<GRP, T, ND>(g, st, s, mu, ld, P, coef);
		if (kin.result)
			acc += k;
	}
	if (kin.result)
		grid_sum<NT>(acc, kin);
}

// 4D tile of sites handled by one block: extents 2^lt[i], tiles per
// dimension nt[i]; a block walks its tile's sites lexicographically and all
// directions of each site, so neighbour links are reused from L1.
struct TileSpec
{
	int lt[4];
	int nt[4];
	int sites;  // sites per tile
	int ntiles; // tiles in the lattice
};

template <int GRP, class T, int ND, int NT, int MINB, bool F2 = false, bool ROWS = false>
__global__ void __launch_bounds__(NT, MINB)
    k_momentum_step_tiled(Geom g, TileSpec ts, T const *__restrict__ U, T *__restrict__ P, T coef, RedSlot kin)
{
	LinkLoad<GRP, T, ND, ROWS> ld{U, g.V};
	double acc = 0.0;
	for (int tile = blockIdx.x; tile < ts.ntiles; tile += gridDim.x)
	{
		int origin[ND];
		int r = tile;
#pragma unroll
		for (int i = ND - 1; i >= 0; --i)
		{
			int q = r / ts.nt[i];
			origin[i] = (r - q * ts.nt[i]) << ts.lt[i];
			r = q;
		}
		for (int t = threadIdx.x; t < ts.sites; t += NT)
		{
			int x[ND];
			int rr = t;
#pragma unroll
			for (int i = ND - 1; i >= 0; --i)
			{
				x[i] = origin[i] + (rr & ((1 << ts.lt[i]) - 1));
				rr >>= ts.lt[i];
			}
			Site<ND> st = site_from_coords<ND>(g, x);
			int64_t s = eo_of<ND>(g, st);
#pragma unroll 1
			for (int mu = 0; mu < ND; ++mu)
			{
				double k = force_item<GRP, T, ND, F2>(g, st, s, mu, ld, P, coef);
				if (kin.result)
					acc += k;
			}
		}
	}
	if (kin.result)
		grid_sum<NT>(acc, kin);
}

// site t of tile `tile` (TileSpec order: tiles lexicographic, sites of a tile
// lexicographic with the last dimension fastest)
template <int ND> __device__ __forceinline__ void tile_site(TileSpec const &ts, int tile, int t, int *x)
{
	int r = tile;
#pragma unroll
	for (int i = ND - 1; i >= 0; --i)
	{
		int q = r / ts.nt[i];
		x[i] = ((r - q * ts.nt[i]) << ts.lt[i]) + (t & ((1 << ts.lt[i]) - 1));
		t >>= ts.lt[i];
		r = q;
	}
}

// planes mu < nu numbered q = 0 .. ND(ND-1)/2 - 1 in the order (0,1), (0,2), ...
// (four dimensions: read from packed 4-bit tables, two integer operations for
// a runtime plane)
template <int ND> __host__ __device__ constexpr int plane_mu(int q)
{
	if constexpr (ND == 4)
		return (0x211000 >> (4 * q)) & 15;
	int mu = 0;
	while (q >= ND - 1 - mu)
	{
		q -= ND - 1 - mu;
		++mu;
	}
	return mu;
}
template <int ND> __host__ __device__ constexpr int plane_nu(int q)
{
	if constexpr (ND == 4)
		return (0x332321 >> (4 * q)) & 15;
	int mu = 0;
	while (q >= ND - 1 - mu)
	{
		q -= ND - 1 - mu;
		++mu;
	}
	return mu + 1 + q;
}

// F[mu] += x, F[nu] -= x for the plane q (a runtime index): a chain of
// branches on compile-time planes keeps F in registers
template <int ND, int NA, int K = 0, class T>
__device__ __forceinline__ void add_plane(T (&F)[ND][NA], int q, T const *x)
{
	if constexpr (K < ND * (ND - 1) / 2)
	{
		if (q == K)
		{
			constexpr int mu = plane_mu<ND>(K), nu = plane_nu<ND>(K);
#pragma unroll
			for (int a = 0; a < NA; ++a)
			{
				F[mu][a] += x[a];
				F[nu][a] -= x[a];
			}
		}
		else
			add_plane<ND, NA, K + 1>(F, q, x);
	}
}
template <int ND, int NA, class T> __device__ __forceinline__ void add_dir(T (&F)[ND][NA], int mu, T const *x)
{
#pragma unroll
	for (int k = 0; k < ND; ++k)
		if (k == mu)
		{
#pragma unroll
			for (int a = 0; a < NA; ++a)
				F[k][a] += x[a];
		}
}

// The per-site body for the small groups (U(1), SU(2)) in four dimensions:
// the same momentum step (and with FUSE link update) as site_md below,
// unrolled over planes and directions, with the site's four own links held in
// registers and the twenty neighbour indices (x + e_mu, x - e_nu,
// x - e_nu + e_mu) computed once per site instead of once per staple: for
// these groups the products are a few FMAs, and the index arithmetic, not the
// arithmetic of the staples, set the instruction count.
template <int GRP, class T, bool FUSE, class LD>
__device__ __forceinline__ double site_md_small(Geom const &g, Site<4> const &st, int64_t s, LD const &ld,
                                                T *__restrict__ P, T coef, T *__restrict__ Uout, T tu, int reunit,
                                                bool want_kin)
{
	using Gp = Group<GRP, T>;
	using E = typename Gp::E;
	constexpr int NA = Gp::NA;
	int32_t f[4], b[4], d[4][4];
#pragma unroll
	for (int mu = 0; mu < 4; ++mu)
	{
		f[mu] = int32_t(eo_shift1<4>(g, st, mu, +1));
		b[mu] = int32_t(eo_shift1<4>(g, st, mu, -1));
	}
#pragma unroll
	for (int nu = 0; nu < 4; ++nu)
#pragma unroll
		for (int mu = 0; mu < 4; ++mu)
			d[nu][mu] = mu == nu ? 0 : int32_t(eo_shift2<4>(g, st, nu, -1, mu, +1));
	E u[4];
#pragma unroll
	for (int mu = 0; mu < 4; ++mu)
		u[mu] = ld(mu, s);
	T F[4][NA];
#pragma unroll
	for (int mu = 0; mu < 4; ++mu)
#pragma unroll
		for (int a = 0; a < NA; ++a)
			F[mu][a] = T(0);
	// forward plaquette loops: (a b)(d c)^+ closes both forward staples
#pragma unroll
	for (int mu = 0; mu < 4; ++mu)
#pragma unroll
		for (int nu = mu + 1; nu < 4; ++nu)
		{
			E pl = Gp::mul_nd(Gp::mul(u[mu], ld(nu, f[mu])), Gp::mul(u[nu], ld(mu, f[nu])));
			T xa[NA];
			Gp::proj(pl, xa);
#pragma unroll
			for (int a = 0; a < NA; ++a)
			{
				F[mu][a] += xa[a];
				F[nu][a] -= xa[a];
			}
		}
	// lower staples, summed per link and closed with U_mu(x)
#pragma unroll
	for (int mu = 0; mu < 4; ++mu)
	{
		E S = Gp::zero();
#pragma unroll
		for (int nu = 0; nu < 4; ++nu)
		{
			if (nu == mu)
				continue;
			Gp::add_to(S, Gp::mul_dn(Gp::mul(ld(mu, b[nu]), ld(nu, d[nu][mu])), ld(nu, b[nu])));
		}
		T xa[NA];
		Gp::proj(Gp::mul(u[mu], S), xa);
#pragma unroll
		for (int a = 0; a < NA; ++a)
			F[mu][a] += xa[a];
	}
	T kacc = T(0); // the site's kinetic terms in the field precision, one FP64 add per site
#pragma unroll
	for (int mu = 0; mu < 4; ++mu)
	{
		auto Pv = comp<T, NA>(P, g.V, mu);
		T p[NA];
		Pv.template load<CACHE_STREAM>(s, p);
#pragma unroll
		for (int a = 0; a < NA; ++a)
			p[a] -= coef * F[mu][a];
		Pv.template store<CACHE_STREAM>(s, p);
		if (want_kin)
			kacc += Gp::kin(p);
		if constexpr (FUSE)
		{
			E r = Gp::mul(Gp::exp_alg(p, tu), u[mu]);
			if (reunit)
				r = Gp::reunit_fast(r);
			comp<T, Gp::NR>(Uout, g.V, mu).store(s, r.v);
		}
	}
	return double(kacc);
}

// Force accumulators F[mu][a] of the thread-per-site body: in registers, or
// (SM) in a block of shared memory private to the thread, element (mu, a) at
// sm[(mu NA + a) 32] past the thread's lane (a warp's 32 threads touch 32
// consecutive words: no bank conflicts). Shared memory frees the ND x NA
// registers for a higher occupancy at the cost of a load and a store per
// accumulated real.
template <class T, int ND, int NA, bool SM> struct SiteAcc;
template <class T, int ND, int NA> struct SiteAcc<T, ND, NA, false>
{
	T F[ND][NA];
	__device__ __forceinline__ explicit SiteAcc(T *)
	{
#pragma unroll
		for (int mu = 0; mu < ND; ++mu)
#pragma unroll
			for (int a = 0; a < NA; ++a)
				F[mu][a] = T(0);
	}
	__device__ __forceinline__ void plane(int q, T const *x) { add_plane<ND, NA>(F, q, x); }
	__device__ __forceinline__ void dir(int mu, T const *x) { add_dir<ND, NA>(F, mu, x); }
	__device__ __forceinline__ void get(int mu, T *f) const
	{
#pragma unroll
		for (int a = 0; a < NA; ++a)
		{
			f[a] = F[0][a];
#pragma unroll
			for (int k = 1; k < ND; ++k)
				f[a] = mu == k ? F[k][a] : f[a];
		}
	}
};
template <class T, int ND, int NA> struct SiteAcc<T, ND, NA, true>
{
	T *sm; // the thread's first element: warp block + lane
	__device__ __forceinline__ explicit SiteAcc(T *p) : sm(p)
	{
#pragma unroll
		for (int k = 0; k < ND * NA; ++k)
			sm[32 * k] = T(0);
	}
	__device__ __forceinline__ void add(int mu, T const *x, T sg)
	{
		T *b = sm + 32 * NA * mu;
#pragma unroll
		for (int a = 0; a < NA; ++a)
			b[32 * a] += sg * x[a];
	}
	__device__ __forceinline__ void plane(int q, T const *x)
	{
		add(plane_mu<ND>(q), x, T(1));
		add(plane_nu<ND>(q), x, T(-1));
	}
	__device__ __forceinline__ void dir(int mu, T const *x) { add(mu, x, T(1)); }
	__device__ __forceinline__ void get(int mu, T *f) const
	{
		T const *b = sm + 32 * NA * mu;
#pragma unroll
		for (int a = 0; a < NA; ++a)
			f[a] = b[32 * a];
	}
};

// Momentum step, one thread per site updating the momenta of all ND links of
// the site. With a = U_mu(x), b = U_nu(x+mu), c = U_mu(x+nu), d = U_nu(x),
// the forward staple of link (x, mu) in the plane (mu, nu) closes to the
// plaquette loop a b c^+ d^+ = (a b)(d c)^+ and the forward staple of link
// (x, nu) in the same plane closes to its adjoint, whose projection is the
// negative: both come from 3 products. The backward staples are summed per
// direction and multiplied by U_mu(x) once, as in staple(). For SU(3) that is
// 11.5 matrix products and 11 link loads per link, against 13 products and 19
// loads when each link is handled on its own. The sum over staples runs in a
// different order than the reference's (forward loops first), which changes
// results only at the rounding level.
//
// FUSE: the link update that follows the momentum step in the integrator is
// done in the same pass, out of place: Uout_mu(x) = exp(tu P_mu(x)) U_mu(x)
// with the updated momentum (and project_on_group_fast when `reunit`), which
// saves the separate link-update kernel's reads of U and P. The force of every
// link reads U only, so writing Uout is race free.
// The per-site body of the thread-per-site momentum step: the forces of the
// ND links of site s, P_mu(s) -= coef F_mu and, with FUSE, the link update
// Uout_mu(s) = exp(tu P_mu) U_mu(s); returns the kinetic norm of the updated
// momenta when want_kin (the FP64 sum costs FP64-pipe time: only the last
// momentum step of a trajectory asks for it). Shared by k_momentum_step_site
// and the batched replicas.
template <int GRP, class T, int ND, int F2, bool ROWS, bool FUSE, class LD, bool SM = false, bool PIPE = false,
          bool GENERIC = false>
__device__ __forceinline__ double site_md(Geom const &g, Site<ND> const &st, int64_t s, LD const &ld,
                                          T *__restrict__ P, T coef, T *__restrict__ Uout, T tu, int reunit,
                                          bool want_kin, T *acc_sm = nullptr)
{
	// GENERIC: the rolled plane/staple loops below for every group
	if constexpr (GRP != SU3 && ND == 4 && !SM && !PIPE && !GENERIC)
		return site_md_small<GRP, T, FUSE>(g, st, s, ld, P, coef, Uout, tu, reunit, want_kin);
	using Gp = Group<GRP, T>;
	using E = typename Gp::E;
	using Pr = Prod<GRP, T, F2>;
	constexpr int NA = Gp::NA;
	T kacc = T(0); // the site's kinetic terms in the field precision, one FP64 add per site
	SiteAcc<T, ND, NA, SM> F(acc_sm);
	// direction mu's force is complete (F_mu plus `last`, its lower-staple
	// term, when given): P_mu -= coef F_mu and, with FUSE, the link update
	// from u = U_mu(x) (a full link)
	auto finish = [&](int mu, E const &u, T const *last) {
		T f[NA];
		F.get(mu, f);
		if (last)
		{
#pragma unroll
			for (int a = 0; a < NA; ++a)
				f[a] += last[a];
		}
		auto Pv = comp<T, NA>(P, g.V, mu);
		T p[NA];
		Pv.template load<CACHE_STREAM>(s, p);
#pragma unroll
		for (int a = 0; a < NA; ++a)
			p[a] -= coef * f[a];
		Pv.template store<CACHE_STREAM>(s, p);
		if (want_kin)
			kacc += Gp::kin(p);
		if constexpr (FUSE)
		{
			E r;
			if constexpr (ROWS && GRP == SU3 && sizeof(T) == 4)
				r = Pr::mul_r2(Gp::exp_alg_rows01(p, tu), u); // mul_r2 reads rows 0, 1 of its left factor
			else if constexpr (ROWS)
				r = Pr::mul_r2(Gp::exp_alg(p, tu), u);
			else
				r = Gp::mul(Gp::exp_alg(p, tu), u);
			if (reunit)
				r = Gp::reunit_fast(r);
			comp<T, Gp::NR>(Uout, g.V, mu).store(s, r.v);
		}
	};
	if constexpr (PIPE && ROWS && GRP == SU3 && ND == 4)
	{
		// software-pipelined form: the neighbour rows of the next plane (of
		// the next lower staple) are loaded while the current one is
		// multiplied; row 2 is rebuilt once the rows have arrived
		E bn = ld.rows(1, eo_shift1<ND>(g, st, 0, +1)), cn = ld.rows(0, eo_shift1<ND>(g, st, 1, +1));
#pragma unroll 1
		for (int q = 0; q < 6; ++q)
		{
			int mu = plane_mu<ND>(q), nu = plane_nu<ND>(q);
			E b = bn, c = cn;
			if (q < 5)
			{
				int m2 = plane_mu<ND>(q + 1), n2 = plane_nu<ND>(q + 1);
				bn = ld.rows(n2, eo_shift1<ND>(g, st, m2, +1));
				cn = ld.rows(m2, eo_shift1<ND>(g, st, n2, +1));
			}
			Gp::complete_row2(b);
			Gp::complete_row2(c);
			E ab = Pr::mul_r2(ld.rows(mu, s), b);
			E dc = Pr::mul_r2(ld.rows(nu, s), c);
			E pl = Pr::mul_nd(ab, dc);
			T xa[NA];
			Gp::proj(pl, xa);
			F.plane(q, xa);
		}
		// lower staples: pair j = 3 mu + k, nu = k < mu ? k : k + 1
		auto pair_nu = [](int j) {
			int mu = j / 3, k = j - 3 * (j / 3);
			return k < mu ? k : k + 1;
		};
		E en, fn, hn;
		{
			int64_t y = eo_shift1<ND>(g, st, 1, -1);
			en = ld.rows(0, y);
			fn = ld.rows(1, eo_shift2<ND>(g, st, 1, -1, 0, +1));
			hn = ld.rows(1, y);
		}
		E S = Gp::zero();
#pragma unroll 1
		for (int j = 0; j < 12; ++j)
		{
			int mu = j / 3, nu = pair_nu(j);
			E e = en, f = fn, h = hn;
			if (j < 11)
			{
				int m2 = (j + 1) / 3, n2 = pair_nu(j + 1);
				int64_t y = eo_shift1<ND>(g, st, n2, -1);
				en = ld.rows(m2, y);
				fn = ld.rows(n2, eo_shift2<ND>(g, st, n2, -1, m2, +1));
				hn = ld.rows(n2, y);
			}
			Gp::complete_row2(f);
			Gp::complete_row2(h);
			Gp::add_to(S, Pr::mul_dn(Pr::mul_r2(e, f), h));
			if (j - 3 * mu == 2)
			{
				E W = Pr::mul(ld(mu, s), S);
				T xa[NA];
				Gp::proj(W, xa);
				F.dir(mu, xa);
				S = Gp::zero();
			}
		}
	}
	else
	{
	// the lexicographic indices of x + e_d and x - e_d, computed once per site
	// (each is used three times)
	int32_t fl[ND], bl[ND];
#pragma unroll
	for (int d = 0; d < ND; ++d)
	{
		fl[d] = lex_step(g, st.px, st.lex, d, +1);
		bl[d] = lex_step(g, st.px, st.lex, d, -1);
	}
	auto pick = [](int32_t const(&a)[ND], int d) {
		int32_t r = a[0];
#pragma unroll
		for (int k = 1; k < ND; ++k)
			r = d == k ? a[k] : r;
		return r;
	};
	int64_t const base_nb = int64_t(st.par ^ 1) * g.Vh, base_same = int64_t(st.par) * g.Vh;
	// forward plaquette loops, one per plane
#pragma unroll 1
	for (int q = 0; q < ND * (ND - 1) / 2; ++q)
	{
		int mu = plane_mu<ND>(q), nu = plane_nu<ND>(q);
		int64_t xpmu = base_nb + (pick(fl, mu) >> 1), xpnu = base_nb + (pick(fl, nu) >> 1);
		E ab, dc;
		T xa[NA];
		if constexpr (ROWS && F2 && GRP == SU3)
		{
			// the plaquette (a b)(d c)^+ is special unitary: rows 0, 1 of a b
			// and of the plaquette suffice, its row-2 entries that proj reads
			// follow from them
			ab = ProdF2::mul_rows(ld.rows(mu, s), ld(nu, xpmu));
			dc = Pr::mul_r2(ld.rows(nu, s), ld(mu, xpnu));
			Gp::proj_rows01(ProdF2::mul_nd_rows(ab, dc), xa);
		}
		else
		{
			if constexpr (ROWS)
			{
				// special unitary links: products from rows 0, 1 of the left factor
				ab = Pr::mul_r2(ld.rows(mu, s), ld(nu, xpmu));
				dc = Pr::mul_r2(ld.rows(nu, s), ld(mu, xpnu));
			}
			else
			{
				ab = Pr::mul(ld(mu, s), ld(nu, xpmu));
				dc = Pr::mul(ld(nu, s), ld(mu, xpnu));
			}
			Gp::proj(Pr::mul_nd(ab, dc), xa);
		}
		F.plane(q, xa);
	}
	// backward staples
#pragma unroll 1
	for (int mu = 0; mu < ND; ++mu)
	{
		E S = Gp::zero();
#pragma unroll 1
		for (int nu = 0; nu < ND; ++nu)
		{
			if (nu == mu)
				continue;
			int32_t lnu = pick(bl, nu);
			int64_t y = base_nb + (lnu >> 1);
			E f = ld(nu, base_same + (lex_step(g, st.px, lnu, mu, +1) >> 1));
			E ef;
			if constexpr (ROWS)
				ef = Pr::mul_r2(ld.rows(mu, y), f);
			else
				ef = Pr::mul(ld(mu, y), f);
			if constexpr (F2 && GRP == SU3)
				S = ProdF2::add_dn(S, ef, ld(nu, y));
			else
				Gp::add_to(S, Pr::mul_dn(ef, ld(nu, y)));
		}
		E u = ld(mu, s);
		T xa[NA];
		Gp::proj(Pr::mul(u, S), xa);
		// the planes came first: direction mu is complete
		finish(mu, u, xa);
	}
	}
	if constexpr (PIPE && ROWS && GRP == SU3 && ND == 4)
	{
		// one copy of the exp body: rolled direction loop
#pragma unroll 1
		for (int mu = 0; mu < ND; ++mu)
			finish(mu, ld(mu, s), nullptr);
	}
	return double(kacc);
}

} // namespace meshgb
#include "site_pair.cuh"
#include "site_async.cuh"
namespace meshgb {

template <int GRP, class T, int ND, int NT, int MINB, int F2 = 0, bool ROWS = false, bool FUSE = false,
          bool SM = false, bool PIPE = false, int PAIR = 0, bool ASYNC = false>
__global__ void __launch_bounds__(NT, MINB)
    k_momentum_step_site(Geom g, TileSpec ts, T const *__restrict__ U, T *__restrict__ P, T coef, RedSlot kin,
                         T *__restrict__ Uout = nullptr, T tu = T(0), int reunit = 0)
{
	constexpr bool kR32 = GRP == SU3 && ROWS && ND == 4 && sizeof(T) == 4;
	using LD = std::conditional_t<kR32, LinkLoadSU3R32, LinkLoad<GRP, T, ND, ROWS>>;
	LD ld = [&] {
		if constexpr (kR32)
			return LinkLoadSU3R32{reinterpret_cast<float4 const *>(U), uint32_t(g.V), uint32_t(g.V / 2 * 9)};
		else
			return LinkLoad<GRP, T, ND, ROWS>{U, g.V};
	}();
	constexpr int NA = Group<GRP, T>::NA;
	// SM: the threads' force accumulators, [warp][element][lane]
	__shared__ T sm_acc[SM ? NT * ND * NA : 1];
	// ASYNC: the threads' double buffers of neighbour-link rows (site_md_async)
	constexpr bool kAsync = ASYNC && GRP == SU3 && ROWS && ND == 4 && sizeof(T) == 4;
	__shared__ float4 abuf[kAsync ? kAsyncSmemFloat4<NT> : 1];
	T *my = SM ? sm_acc + (threadIdx.x >> 5) * (32 * ND * NA) + (threadIdx.x & 31) : nullptr;
	double acc = 0.0;
	for (int tile = blockIdx.x; tile < ts.ntiles; tile += gridDim.x)
	{
		for (int t = threadIdx.x; t < ts.sites; t += NT)
		{
			int x[ND];
			tile_site<ND>(ts, tile, t, x);
			Site<ND> st = site_from_coords<ND>(g, x);
			int64_t s = eo_of<ND>(g, st);
			if constexpr (kAsync)
				acc += site_md_async<NT, FUSE, decltype(ld), SM>(g, st, s, ld, U, P, coef, Uout, tu, reunit,
				                                                 kin.result != nullptr, my, abuf + threadIdx.x);
			else if constexpr (PAIR != 0 && GRP == SU3 && ROWS && ND == 4 && sizeof(T) == 4)
				acc += site_md_pair<FUSE, decltype(ld), SM, PAIR>(g, st, s, ld, P, coef, Uout, tu, reunit,
				                                            kin.result != nullptr, my);
			else
				acc += site_md<GRP, T, ND, F2, ROWS, FUSE, decltype(ld), SM, PIPE>(g, st, s, ld, P, coef, Uout, tu,
				                                                                  reunit, kin.result != nullptr, my);
		}
	}
	if (kin.result)
		grid_sum<NT>(acc, kin);
}

// ---------------------------------------------------------------------------
// heat-bath / overrelaxation (legacy src/old/wilson.cpp:15-60,
// src/old/mesh/gauge_action.h:42-73), checkerboard: the links (x, mu) of one
// parity do not enter each other's staples (those read U_mu only at x +- nu,
// of the other parity), so they are updated together
// ---------------------------------------------------------------------------
template <int GRP, class T, int ND, bool OR>
__global__ void __launch_bounds__(kBlock)
    k_gauge_update(Geom g, int mu, int parity, T *U, double beta, uint64_t seed, uint64_t ctr)
{
	using Gp = Group<GRP, T>;
	using E = typename Gp::E;
	LinkLoad<GRP, T, ND> ld{U, g.V};
	MESH_GRID_LOOP(i, g.Vh)
	{
		int64_t s = int64_t(parity) * g.Vh + i;
		Site<ND> st = site_from_eo<ND>(g, s);
		E S = staple<GRP, T, ND>(g, st, s, mu, ld);
		auto v = comp<T, Gp::NR>(U, g.V, mu);
		E u;
		v.load(s, u.v);
		if constexpr (OR)
			HbUpdate<GRP, T>::overrelax(u, S);
		else
			HbUpdate<GRP, T>::heatbath(u, S, T(beta), HbStream{seed, ctr, uint32_t(st.lex), uint32_t(mu), 0u});
		v.store(s, u.v);
	}
}

// ---------------------------------------------------------------------------
// Wilson loops (legacy src/old/mesh/wilson.cpp:40-75): straight lines of links
// built one link at a time, then the rectangular loops from four lines
// ---------------------------------------------------------------------------
// even/odd index of x + off e_dir for 0 <= off < L_dir (extents are even, so
// the parity changes with off whether or not the step wraps)
template <int ND> __device__ __forceinline__ int64_t eo_offset(Geom const &g, Site<ND> const &st, int dir, int off)
{
	int L = g.Ld(dir);
	int32_t lex = st.lex + (st.x(dir) + off >= L ? off - L : off) * g.Sd(dir);
	return int64_t(st.par ^ (off & 1)) * g.Vh + (lex >> 1);
}

// Lout(x) = Lprev(x) U_dir(x + (n - 1) dir): the line of n links from x
// (Lout may be Lprev: every site reads and writes only its own line)
template <int GRP, class T, int ND>
__global__ void __launch_bounds__(kBlock)
    k_line_extend(Geom g, int dir, int n, T const *Lprev, T const *__restrict__ U, T *Lout)
{
	using Gp = Group<GRP, T>;
	using E = typename Gp::E;
	int off = (n - 1) % g.Ld(dir);
	MESH_GRID_LOOP(s, g.V)
	{
		Site<ND> st = site_from_eo<ND>(g, s);
		E a, b;
		Soa<T, Gp::NR>::load(Lprev, g.V, s, a.v);
		Soa<T, Gp::NR>::load(U + int64_t(dir) * Gp::NR * g.V, g.V, eo_offset<ND>(g, st, dir, off), b.v);
		E c = Gp::mul(a, b);
		Soa<T, Gp::NR>::store(Lout, g.V, s, c.v);
	}
}

// sum over sites and mu < 3 of ReTr(S_mu(x) T(x + r mu) S_mu(x + t 3)^+ T(x)^+),
// S: the three spatial lines of r links (components 0..2), T: the line of t
// links in direction 3
template <int GRP, class T, int ND>
__global__ void __launch_bounds__(kBlock)
    k_wilson_rt(Geom g, int r, int t, T const *__restrict__ S, T const *__restrict__ Tt, RedSlot out)
{
	using Gp = Group<GRP, T>;
	using E = typename Gp::E;
	double acc = 0.0;
	MESH_GRID_LOOP(s, g.V)
	{
		Site<ND> st = site_from_eo<ND>(g, s);
		E d;
		Soa<T, Gp::NR>::load(Tt, g.V, s, d.v);
		int64_t xt = eo_offset<ND>(g, st, 3, t % g.Ld(3));
		T sum = T(0);
#pragma unroll 1
		for (int mu = 0; mu < 3; ++mu)
		{
			T const *Smu = S + int64_t(mu) * Gp::NR * g.V;
			E a, b, c;
			Soa<T, Gp::NR>::load(Smu, g.V, s, a.v);
			Soa<T, Gp::NR>::load(Tt, g.V, eo_offset<ND>(g, st, mu, r % g.Ld(mu)), b.v);
			Soa<T, Gp::NR>::load(Smu, g.V, xt, c.v);
			sum += Gp::retr_nd(Gp::mul(a, b), Gp::mul(d, c));
		}
		acc += double(sum);
	}
	grid_sum<kBlock>(acc, out);
}

template <int GRP, class T, int ND>
__global__ void __launch_bounds__(kBlock) k_staple_sum(Geom g, int mu, T const *__restrict__ U, T *__restrict__ S)
{
	using Gp = Group<GRP, T>;
	LinkLoad<GRP, T, ND> ld{U, g.V};
	MESH_GRID_LOOP(s, g.V)
	{
		Site<ND> st = site_from_eo<ND>(g, s);
		auto e = staple<GRP, T, ND>(g, st, s, mu, ld);
		Soa<T, Gp::NR>::store(S, g.V, s, e.v);
	}
}

template <int GRP, class T, int ND>
__global__ void __launch_bounds__(kBlock)
    k_wilson_deriv(Geom g, int mu, T scale, T const *__restrict__ U, T *__restrict__ F)
{
	using Gp = Group<GRP, T>;
	using E = typename Gp::E;
	LinkLoad<GRP, T, ND> ld{U, g.V};
	MESH_GRID_LOOP(s, g.V)
	{
		Site<ND> st = site_from_eo<ND>(g, s);
		E S = staple<GRP, T, ND>(g, st, s, mu, ld);
		E W = Gp::mul(ld(mu, s), S);
		T f[Gp::NA];
		Gp::proj(W, f);
#pragma unroll
		for (int k = 0; k < Gp::NA; ++k)
			f[k] *= scale;
		Soa<T, Gp::NA>::store(F, g.V, s, f);
	}
}

// U_dst = exp(t P) U_src for every (site, mu); optional project_on_group_fast
template <int GRP, class T, bool REUNIT, bool ROWS = false>
__global__ void __launch_bounds__(kBlock)
    k_evolve(int64_t n_total, int64_t V, T const *__restrict__ Usrc, T *__restrict__ Udst, T const *__restrict__ P,
             T t)
{
	using Gp = Group<GRP, T>;
	using E = typename Gp::E;
	MESH_GRID_LOOP(i, n_total)
	{
		int mu = int(i / V);
		int64_t s = i - int64_t(mu) * V;
		T p[Gp::NA];
		comp<T, Gp::NA>(const_cast<T *>(P), V, mu).load(s, p);
		E u;
		if constexpr (ROWS && GRP == SU3)
		{
			Soa<T, Gp::NR>::template load_head<12>(Usrc + int64_t(mu) * Gp::NR * V, V, s, u.v);
			Gp::complete_row2(u);
		}
		else
			comp<T, Gp::NR>(const_cast<T *>(Usrc), V, mu).load(s, u.v);
		E r = Gp::mul(Gp::exp_alg(p, t), u);
		if constexpr (REUNIT)
			r = Gp::reunit_fast(r);
		comp<T, Gp::NR>(Udst, V, mu).store(s, r.v);
	}
}

template <int GRP, class T, bool EXACT>
__global__ void __launch_bounds__(kBlock) k_reunit(int64_t n_total, int64_t V, T *__restrict__ U)
{
	using Gp = Group<GRP, T>;
	using E = typename Gp::E;
	MESH_GRID_LOOP(i, n_total)
	{
		int mu = int(i / V);
		int64_t s = i - int64_t(mu) * V;
		auto v = comp<T, Gp::NR>(U, V, mu);
		E u;
		v.load(s, u.v);
		u = EXACT ? Gp::reunit_exact(u) : Gp::reunit_fast(u);
		v.store(s, u.v);
	}
}

// ---------------------------------------------------------------------------
// Landau gauge fixing
// ---------------------------------------------------------------------------

// sum_x sum_mu ReTr(g(x) U_mu(x) g(x+mu)^+)
template <int GRP, class T, int ND>
__global__ void __launch_bounds__(kBlock)
    k_landau_functional(Geom g, T const *__restrict__ U, T const *__restrict__ G, RedSlot out)
{
	using Gp = Group<GRP, T>;
	using E = typename Gp::E;
	LinkLoad<GRP, T, ND> ld{U, g.V};
	double acc = 0.0;
	MESH_GRID_LOOP(s, g.V)
	{
		Site<ND> st = site_from_eo<ND>(g, s);
		E gx;
		Soa<T, Gp::NR>::load(G, g.V, s, gx.v);
		T t = 0;
#pragma unroll
		for (int mu = 0; mu < ND; ++mu)
		{
			E gf;
			Soa<T, Gp::NR>::load(G, g.V, eo_shift1<ND>(g, st, mu, +1), gf.v);
			t += Gp::retr_nd(Gp::mul(gx, ld(mu, s)), gf);
		}
		acc += double(t);
	}
	grid_sum<kBlock>(acc, out);
}

// Delta(x) = sum_mu [A_mu(x) - A_mu(x-mu)], A_mu(y) = proj(g(y) U_mu(y) g(y+mu)^+)
template <int GRP, class T, int ND>
__device__ __forceinline__ void divergence(Geom const &g, Site<ND> const &st, int64_t s, LinkLoad<GRP, T, ND> const &ld,
                                           T const *__restrict__ G, T *D)
{
	using Gp = Group<GRP, T>;
	using E = typename Gp::E;
#pragma unroll
	for (int k = 0; k < Gp::NA; ++k)
		D[k] = T(0);
	E gx;
	Soa<T, Gp::NR>::load(G, g.V, s, gx.v);
#pragma unroll
	for (int mu = 0; mu < ND; ++mu)
	{
		E gf, gb, ub;
		int64_t f = eo_shift1<ND>(g, st, mu, +1), b = eo_shift1<ND>(g, st, mu, -1);
		Soa<T, Gp::NR>::load(G, g.V, f, gf.v);
		Soa<T, Gp::NR>::load(G, g.V, b, gb.v);
		T a[Gp::NA];
		Gp::proj(Gp::mul_nd(Gp::mul(gx, ld(mu, s)), gf), a);
#pragma unroll
		for (int k = 0; k < Gp::NA; ++k)
			D[k] += a[k];
		Gp::proj(Gp::mul_nd(Gp::mul(gb, ld(mu, b)), gx), a);
#pragma unroll
		for (int k = 0; k < Gp::NA; ++k)
			D[k] -= a[k];
	}
}

template <int GRP, class T, int ND>
__global__ void __launch_bounds__(kBlock)
    k_landau_theta(Geom g, T const *__restrict__ U, T const *__restrict__ G, RedSlot out)
{
	using Gp = Group<GRP, T>;
	LinkLoad<GRP, T, ND> ld{U, g.V};
	double acc = 0.0;
	MESH_GRID_LOOP(s, g.V)
	{
		Site<ND> st = site_from_eo<ND>(g, s);
		T D[Gp::NA];
		divergence<GRP, T, ND>(g, st, s, ld, G, D);
		acc += double(Gp::kin(D));
	}
	grid_sum<kBlock>(acc, out);
}

// F(x) = proj(g(x) d(x)) * scale, d = sum_mu U_mu(x) g(x+mu)^+ + (g(x-mu) U_mu(x-mu))^+
// (Landau::deriv, landau.h:52-65)
template <int GRP, class T, int ND>
__global__ void __launch_bounds__(kBlock)
    k_landau_deriv(Geom g, T const *__restrict__ U, T const *__restrict__ G, T *__restrict__ F, T scale)
{
	using Gp = Group<GRP, T>;
	using E = typename Gp::E;
	LinkLoad<GRP, T, ND> ld{U, g.V};
	MESH_GRID_LOOP(s, g.V)
	{
		Site<ND> st = site_from_eo<ND>(g, s);
		E d = Gp::zero();
#pragma unroll
		for (int mu = 0; mu < ND; ++mu)
		{
			E gf, gb;
			int64_t f = eo_shift1<ND>(g, st, mu, +1), b = eo_shift1<ND>(g, st, mu, -1);
			Soa<T, Gp::NR>::load(G, g.V, f, gf.v);
			Soa<T, Gp::NR>::load(G, g.V, b, gb.v);
			Gp::add_to(d, Gp::mul_nd(ld(mu, s), gf));
			Gp::add_to(d, Gp::adj(Gp::mul(gb, ld(mu, b))));
		}
		E gx;
		Soa<T, Gp::NR>::load(G, g.V, s, gx.v);
		T o[Gp::NA];
		Gp::proj(Gp::mul(gx, d), o);
#pragma unroll
		for (int k = 0; k < Gp::NA; ++k)
			o[k] *= scale;
		Soa<T, Gp::NA>::store(F, g.V, s, o);
	}
}

// second-order binomial h^omega of a unit quaternion, renormalised
// (Mandula & Ogilvie, Phys. Lett. B 248 (1990) 156)
template <class T> __device__ __forceinline__ void or_power(T *h, T w)
{
	T c = w * (w - T(1)) * T(0.5);
	T a = h[0] - T(1);
	T v2 = h[1] * h[1] + h[2] * h[2] + h[3] * h[3];
	T r0 = T(1) + w * a + c * (a * a - v2);
	T f = w + T(2) * c * a;
	T r1 = h[1] * f, r2 = h[2] * f, r3 = h[3] * f;
	T n = m_rsqrt(r0 * r0 + r1 * r1 + r2 * r2 + r3 * r3);
	h[0] = r0 * n;
	h[1] = r1 * n;
	h[2] = r2 * n;
	h[3] = r3 * n;
}

template <int GRP, class T> struct OrUpdate;
template <class T> struct OrUpdate<U1, T>
{
	using E = typename Group<U1, T>::E;
	__device__ __forceinline__ static E apply(E W, E gx, T w)
	{
		T n2 = W.v[0] * W.v[0] + W.v[1] * W.v[1];
		if (n2 < T(1e-60))
			return gx;
		T phi = atan2(W.v[1], W.v[0]);
		T s, c;
		m_sincos(w * phi, &s, &c);
		E h = {{c, -s}};
		return Group<U1, T>::mul(h, gx);
	}
};
template <class T> struct OrUpdate<SU2, T>
{
	using E = typename Group<SU2, T>::E;
	__device__ __forceinline__ static E apply(E W, E gx, T w)
	{
		T n2 = W.v[0] * W.v[0] + W.v[1] * W.v[1] + W.v[2] * W.v[2] + W.v[3] * W.v[3];
		if (n2 < T(1e-60))
			return gx;
		T n = m_rsqrt(n2);
		T h[4] = {W.v[0] * n, -W.v[1] * n, -W.v[2] * n, -W.v[3] * n};
		or_power(h, w);
		E he = {{h[0], h[1], h[2], h[3]}};
		return Group<SU2, T>::mul(he, gx);
	}
};
template <class T> struct OrUpdate<SU3, T>
{
	using E = typename Group<SU3, T>::E;
	__device__ __forceinline__ static E apply(E W, E gx, T w)
	{
		constexpr int sub[3][2] = {{0, 1}, {0, 2}, {1, 2}};
#pragma unroll
		for (int sg = 0; sg < 3; ++sg)
		{
			int i = sub[sg][0], j = sub[sg][1];
			T q[4] = {(W.v[6 * i + 2 * i] + W.v[6 * j + 2 * j]) * T(0.5),
			          (W.v[6 * j + 2 * i + 1] + W.v[6 * i + 2 * j + 1]) * T(0.5),
			          (W.v[6 * i + 2 * j] - W.v[6 * j + 2 * i]) * T(0.5),
			          (W.v[6 * i + 2 * i + 1] - W.v[6 * j + 2 * j + 1]) * T(0.5)};
			T n2 = q[0] * q[0] + q[1] * q[1] + q[2] * q[2] + q[3] * q[3];
			if (n2 < T(1e-60))
				continue;
			T n = m_rsqrt(n2);
			T h[4] = {q[0] * n, -q[1] * n, -q[2] * n, -q[3] * n};
			or_power(h, w);
			cx<T> a = {h[0], h[3]}, b = {h[2], h[1]}, c = {-h[2], h[1]}, d = {h[0], -h[3]};
#pragma unroll
			for (int k = 0; k < 3; ++k)
			{
				cx<T> gi = gx.at(i, k), gj = gx.at(j, k);
				gx.set(i, k, cadd(cmul(a, gi), cmul(b, gj)));
				gx.set(j, k, cadd(cmul(c, gi), cmul(d, gj)));
				cx<T> wi = W.at(i, k), wj = W.at(j, k);
				W.set(i, k, cadd(cmul(a, wi), cmul(b, wj)));
				W.set(j, k, cadd(cmul(c, wi), cmul(d, wj)));
			}
		}
		return gx;
	}
};

// one checkerboard half-sweep of overrelaxation on the sites of `parity`
template <int GRP, class T, int ND>
__global__ void __launch_bounds__(kBlock)
    k_landau_or_half(Geom g, int parity, T omega, T const *__restrict__ U, T *__restrict__ G)
{
	using Gp = Group<GRP, T>;
	using E = typename Gp::E;
	LinkLoad<GRP, T, ND> ld{U, g.V};
	MESH_GRID_LOOP(h, g.Vh)
	{
		int64_t s = int64_t(parity) * g.Vh + h;
		Site<ND> st = site_from_eo<ND>(g, s);
		E K = Gp::zero();
#pragma unroll
		for (int mu = 0; mu < ND; ++mu)
		{
			E gf, gb;
			int64_t f = eo_shift1<ND>(g, st, mu, +1), b = eo_shift1<ND>(g, st, mu, -1);
			Soa<T, Gp::NR>::load(G, g.V, f, gf.v);
			Soa<T, Gp::NR>::load(G, g.V, b, gb.v);
			Gp::add_to(K, Gp::mul_nd(ld(mu, s), gf));
			// U_mu(x-mu)^+ g(x-mu)^+ = (g(x-mu) U_mu(x-mu))^+
			Gp::add_to(K, Gp::adj(Gp::mul(gb, ld(mu, b))));
		}
		E gx;
		Soa<T, Gp::NR>::load(G, g.V, s, gx.v);
		E r = OrUpdate<GRP, T>::apply(Gp::mul(gx, K), gx, omega);
		Soa<T, Gp::NR>::store(G, g.V, s, r.v);
	}
}

// sum_x <a(x), b(x)> for algebra fields (the kinetic bilinear form);
// sum_real_trace(a*b) of the reference equals minus this
template <int GRP, class T>
__global__ void __launch_bounds__(kBlock)
    k_alg_dot(int64_t n_total, int64_t V, T const *__restrict__ a, T const *__restrict__ b, RedSlot out)
{
	using Gp = Group<GRP, T>;
	double acc = 0.0;
	MESH_GRID_LOOP(i, n_total)
	{
		int c = int(i / V);
		int64_t s = i - int64_t(c) * V;
		T x[Gp::NA], y[Gp::NA];
		comp<T, Gp::NA>(const_cast<T *>(a), V, c).load(s, x);
		comp<T, Gp::NA>(const_cast<T *>(b), V, c).load(s, y);
		T pp[Gp::NA], mm[Gp::NA];
#pragma unroll
		for (int k = 0; k < Gp::NA; ++k)
		{
			pp[k] = x[k] + y[k];
			mm[k] = x[k] - y[k];
		}
		// polarisation: <x,y> = (|x+y|^2 - |x-y|^2)/4
		acc += double((Gp::kin(pp) - Gp::kin(mm)) * T(0.25));
	}
	grid_sum<kBlock>(acc, out);
}

// dst(x) = exp(eps F(x)) g(x)
template <int GRP, class T>
__global__ void __launch_bounds__(kBlock)
    k_exp_apply(int64_t V, T eps, T const *__restrict__ F, T const *__restrict__ G, T *__restrict__ dst)
{
	using Gp = Group<GRP, T>;
	using E = typename Gp::E;
	MESH_GRID_LOOP(s, V)
	{
		T f[Gp::NA];
		Soa<T, Gp::NA>::load(F, V, s, f);
		E gx;
		Soa<T, Gp::NR>::load(G, V, s, gx.v);
		E r = Gp::mul(Gp::exp_alg(f, eps), gx);
		Soa<T, Gp::NR>::store(dst, V, s, r.v);
	}
}

// y += a x (algebra fields)
template <int GRP, class T>
__global__ void __launch_bounds__(kBlock)
    k_axpy_alg(int64_t n_total, int64_t V, T a, T const *__restrict__ x, T *__restrict__ y)
{
	using Gp = Group<GRP, T>;
	MESH_GRID_LOOP(i, n_total)
	{
		int c = int(i / V);
		int64_t s = i - int64_t(c) * V;
		T xv[Gp::NA], yv[Gp::NA];
		comp<T, Gp::NA>(const_cast<T *>(x), V, c).load(s, xv);
		auto yc = comp<T, Gp::NA>(y, V, c);
		yc.load(s, yv);
#pragma unroll
		for (int k = 0; k < Gp::NA; ++k)
			yv[k] += a * xv[k];
		yc.store(s, yv);
	}
}

// U_mu(x) <- g(x) U_mu(x) g(x+mu)^+
template <int GRP, class T, int ND>
__global__ void __launch_bounds__(kBlock) k_gauge_transform(Geom g, T *__restrict__ U, T const *__restrict__ G)
{
	using Gp = Group<GRP, T>;
	using E = typename Gp::E;
	int64_t n = int64_t(ND) * g.V;
	MESH_GRID_LOOP(i, n)
	{
		int mu = int(i / g.V);
		int64_t s = i - int64_t(mu) * g.V;
		Site<ND> st = site_from_eo<ND>(g, s);
		E gx, gf, u;
		Soa<T, Gp::NR>::load(G, g.V, s, gx.v);
		Soa<T, Gp::NR>::load(G, g.V, eo_shift1<ND>(g, st, mu, +1), gf.v);
		auto v = comp<T, Gp::NR>(U, g.V, mu);
		v.load(s, u.v);
		E r = Gp::mul_nd(Gp::mul(gx, u), gf);
		v.store(s, r.v);
	}
}

} // namespace meshgb
#include "md_line.cuh"
namespace meshgb {

// ---------------------------------------------------------------------------
// host launchers
// ---------------------------------------------------------------------------
template <int GRP, class T, int ND> struct Ops
{
	using Gp = Group<GRP, T>;

	static unsigned blocks(Context const &c, int64_t n) { return grid_for(c, n, kBlock); }
	static unsigned red_blocks(Context const &c, int64_t n)
	{
		unsigned b = grid_for(c, n, kBlock, 4);
		return b < unsigned(kMaxRedBlocks) ? b : unsigned(kMaxRedBlocks);
	}

	static void import_(Field &f, void const *stage)
	{
		auto &c = *f.ctx;
		int64_t n = int64_t(f.nstack) * f.geom.V;
		if (f.kind == MESH_GROUP)
			k_import<GRP, T, ND, false><<<blocks(c, n), kBlock, 0, c.stream>>>(f.geom, f.nstack,
			                                                                     static_cast<T const *>(stage),
			                                                                     static_cast<T *>(f.d));
		else
			k_import<GRP, T, ND, true><<<blocks(c, n), kBlock, 0, c.stream>>>(f.geom, f.nstack,
			                                                                    static_cast<T const *>(stage),
			                                                                    static_cast<T *>(f.d));
		MESH_LAUNCH_CHECK();
	}
	// conversion straight from / to a device-accessible host buffer
	static void import_direct(Field &f, void const *host)
	{
		auto &c = *f.ctx;
		int64_t nb = int64_t(f.nstack) * ((f.geom.V + kBlock - 1) / kBlock);
		unsigned b = unsigned(nb < int64_t(c.num_sms) * 8 ? nb : int64_t(c.num_sms) * 8);
		if (f.kind == MESH_GROUP)
			k_import_direct<GRP, T, ND, false><<<b, kBlock, 0, c.stream>>>(f.geom, f.nstack, static_cast<T const *>(host),
			                                                               static_cast<T *>(f.d));
		else
			k_import_direct<GRP, T, ND, true><<<b, kBlock, 0, c.stream>>>(f.geom, f.nstack, static_cast<T const *>(host),
			                                                              static_cast<T *>(f.d));
		MESH_LAUNCH_CHECK();
	}
	static void export_direct(Field const &f, void *host)
	{
		auto &c = *f.ctx;
		int64_t nb = int64_t(f.nstack) * ((f.geom.V + kBlock - 1) / kBlock);
		unsigned b = unsigned(nb < int64_t(c.num_sms) * 8 ? nb : int64_t(c.num_sms) * 8);
		if (f.kind == MESH_GROUP)
			k_export_direct<GRP, T, ND, false><<<b, kBlock, 0, c.stream>>>(f.geom, f.nstack, static_cast<T const *>(f.d),
			                                                               static_cast<T *>(host));
		else
			k_export_direct<GRP, T, ND, true><<<b, kBlock, 0, c.stream>>>(f.geom, f.nstack, static_cast<T const *>(f.d),
			                                                              static_cast<T *>(host));
		MESH_LAUNCH_CHECK();
	}
	static void export_(Field const &f, void *stage)
	{
		auto &c = *f.ctx;
		int64_t n = int64_t(f.nstack) * f.geom.V;
		if (f.kind == MESH_GROUP)
			k_export<GRP, T, ND, false><<<blocks(c, n), kBlock, 0, c.stream>>>(f.geom, f.nstack,
			                                                                     static_cast<T const *>(f.d),
			                                                                     static_cast<T *>(stage));
		else
			k_export<GRP, T, ND, true><<<blocks(c, n), kBlock, 0, c.stream>>>(f.geom, f.nstack,
			                                                                    static_cast<T const *>(f.d),
			                                                                    static_cast<T *>(stage));
		MESH_LAUNCH_CHECK();
	}
	static void set_unit(Field &f)
	{
		auto &c = *f.ctx;
		int64_t n = int64_t(f.nstack) * f.geom.V;
		k_set_unit<GRP, T><<<blocks(c, n), kBlock, 0, c.stream>>>(n, f.geom.V, static_cast<T *>(f.d));
		MESH_LAUNCH_CHECK();
	}
	static void random(Field &f, uint64_t seed, uint64_t counter, RedSlot kin)
	{
		auto &c = *f.ctx;
		int64_t n = int64_t(f.nstack) * f.geom.V;
		if (f.kind == MESH_GROUP)
		{
			uint32_t tag = f.nstack == 1 ? TAG_TRANSFORM : TAG_GAUGE;
			k_random_group<GRP, T, ND><<<blocks(c, n), kBlock, 0, c.stream>>>(f.geom, f.nstack, seed, counter, tag,
			                                                                  static_cast<T *>(f.d));
		}
		else
			k_random_alg<GRP, T, ND><<<red_blocks(c, n), kBlock, 0, c.stream>>>(
			    f.geom, f.nstack, seed, nullptr, counter, static_cast<T *>(f.d), kin);
		MESH_LAUNCH_CHECK();
	}
	static void random_momenta_dev(Field &f, uint64_t seed, uint64_t const *counter_dev, RedSlot kin)
	{
		auto &c = *f.ctx;
		int64_t n = int64_t(f.nstack) * f.geom.V;
		k_random_alg<GRP, T, ND><<<red_blocks(c, n), kBlock, 0, c.stream>>>(f.geom, f.nstack, seed, counter_dev, 0,
		                                                                  static_cast<T *>(f.d), kin);
		MESH_LAUNCH_CHECK();
	}
	static void norm2(Field const &f, RedSlot out)
	{
		auto &c = *f.ctx;
		int64_t n = int64_t(f.nstack) * f.geom.V;
		if (f.kind == MESH_ALGEBRA)
			k_norm2<GRP, T, true><<<red_blocks(c, n), kBlock, 0, c.stream>>>(n, f.geom.V, static_cast<T const *>(f.d),
			                                                                 out);
		else
			k_norm2<GRP, T, false><<<red_blocks(c, n), kBlock, 0, c.stream>>>(n, f.geom.V,
			                                                                  static_cast<T const *>(f.d), out);
		MESH_LAUNCH_CHECK();
	}
	static void cshift(Field &dst, Field const &src, int dir, int offset)
	{
		auto &c = *dst.ctx;
		k_cshift<GRP, T, ND><<<blocks(c, dst.geom.V), kBlock, 0, c.stream>>>(
		    dst.geom, dir, offset, static_cast<T const *>(src.d), static_cast<T *>(dst.d));
		MESH_LAUNCH_CHECK();
	}
	static void site_op(int op, Field &dst, Field const &a, Field const *b)
	{
		auto &c = *dst.ctx;
		k_site_op<GRP, T><<<blocks(c, dst.geom.V), kBlock, 0, c.stream>>>(
		    op, dst.geom.V, static_cast<T const *>(a.d), b ? static_cast<T const *>(b->d) : nullptr,
		    static_cast<T *>(dst.d));
		MESH_LAUNCH_CHECK();
	}
	static void sum_real_trace(Field const &a, RedSlot out)
	{
		auto &c = *a.ctx;
		k_sum_real_trace<GRP, T><<<red_blocks(c, a.geom.V), kBlock, 0, c.stream>>>(
		    a.geom.V, static_cast<T const *>(a.d), out);
		MESH_LAUNCH_CHECK();
	}
	static void plaquette(Field const &U, RedSlot out)
	{
		auto &c = *U.ctx;
		k_plaquette<GRP, T, ND><<<red_blocks(c, U.geom.V), kBlock, 0, c.stream>>>(
		    U.geom, static_cast<T const *>(U.d), out);
		MESH_LAUNCH_CHECK();
	}
	// the HMC trajectory's versions: SU(3) FP32 links read as rows 0, 1
	static void hmc_plaquette(Field const &U, RedSlot out)
	{
		if constexpr (kRows<GRP, T>)
		{
			auto &c = *U.ctx;
			k_plaquette<GRP, T, ND, true><<<red_blocks(c, U.geom.V), kBlock, 0, c.stream>>>(
			    U.geom, static_cast<T const *>(U.d), out);
			MESH_LAUNCH_CHECK();
		}
		else
			plaquette(U, out);
	}
	static void staple_sum(Field &S, Field const &U, int mu)
	{
		auto &c = *U.ctx;
		k_staple_sum<GRP, T, ND><<<blocks(c, U.geom.V), kBlock, 0, c.stream>>>(
		    U.geom, mu, static_cast<T const *>(U.d), static_cast<T *>(S.d));
		MESH_LAUNCH_CHECK();
	}
	static void wilson_deriv(Field &F, Field const &U, int mu, double beta)
	{
		auto &c = *U.ctx;
		k_wilson_deriv<GRP, T, ND><<<blocks(c, U.geom.V), kBlock, 0, c.stream>>>(
		    U.geom, mu, T(beta / (2.0 * Gp::NC)), static_cast<T const *>(U.d), static_cast<T *>(F.d));
		MESH_LAUNCH_CHECK();
	}
	static void reunitize(Field &U)
	{
		auto &c = *U.ctx;
		int64_t n = int64_t(U.nstack) * U.geom.V;
		k_reunit<GRP, T, false><<<blocks(c, n), kBlock, 0, c.stream>>>(n, U.geom.V, static_cast<T *>(U.d));
		MESH_LAUNCH_CHECK();
	}
	static void reunit_exact(Field &U)
	{
		auto &c = *U.ctx;
		int64_t n = int64_t(U.nstack) * U.geom.V;
		k_reunit<GRP, T, true><<<blocks(c, n), kBlock, 0, c.stream>>>(n, U.geom.V, static_cast<T *>(U.d));
		MESH_LAUNCH_CHECK();
	}
	static void hmc_evolve(Field const &Usrc, Field &Udst, Field const &P, double t, bool reunit)
	{
		if constexpr (kRows<GRP, T>)
		{
			auto &c = *Udst.ctx;
			int64_t n = int64_t(Udst.nstack) * Udst.geom.V;
			if (reunit)
				k_evolve<GRP, T, true, true><<<blocks(c, n), kBlock, 0, c.stream>>>(
				    n, Udst.geom.V, static_cast<T const *>(Usrc.d), static_cast<T *>(Udst.d),
				    static_cast<T const *>(P.d), T(t));
			else
				k_evolve<GRP, T, false, true><<<blocks(c, n), kBlock, 0, c.stream>>>(
				    n, Udst.geom.V, static_cast<T const *>(Usrc.d), static_cast<T *>(Udst.d),
				    static_cast<T const *>(P.d), T(t));
			MESH_LAUNCH_CHECK();
		}
		else
			evolve(Usrc, Udst, P, t, reunit);
	}
	static void evolve(Field const &Usrc, Field &Udst, Field const &P, double t, bool reunit)
	{
		auto &c = *Udst.ctx;
		int64_t n = int64_t(Udst.nstack) * Udst.geom.V;
		if (reunit)
			k_evolve<GRP, T, true><<<blocks(c, n), kBlock, 0, c.stream>>>(
			    n, Udst.geom.V, static_cast<T const *>(Usrc.d), static_cast<T *>(Udst.d),
			    static_cast<T const *>(P.d), T(t));
		else
			k_evolve<GRP, T, false><<<blocks(c, n), kBlock, 0, c.stream>>>(
			    n, Udst.geom.V, static_cast<T const *>(Usrc.d), static_cast<T *>(Udst.d),
			    static_cast<T const *>(P.d), T(t));
		MESH_LAUNCH_CHECK();
	}
	// ---- momentum step: launch variants and their autotuning ----------------
	struct ForceVariant
	{
		int tiled;
		int lt[4]; // log2 tile extents
		int threads, minb;
		char const *name;
		int f2 = 0;        // packed FP32x2 products (SU(3) float only)
		int r2 = 0;        // line march: row 2 of whole-link loads read, not rebuilt
		int fsm = 0;       // line march: force accumulators in shared memory
		int pf = 0;        // line march: L1 prefetch of the next iteration's links
		int sm = 0;        // thread per site: force accumulators in shared memory
		int st = 0;        // line march: own line staged in shared memory by bulk copies (L3 = 32)
		int pipe = 0;      // thread per site: next neighbour rows loaded ahead (software pipeline)
		int pair = 0;      // thread per site: sections with two products per FP32x2 operation (site_md_pair)
		int async = 0;     // thread per site: next step's neighbour rows copied to shared memory (site_md_async)
	};
	static constexpr bool kF2 = GRP == SU3 && sizeof(T) == 4;
	// 0-10: thread per link (even/odd order or 4D tiles); 11-13: the same with
	// packed FP32x2 products; 14-17, 21-28: thread per site
	// (k_momentum_step_site) with FP32x2 products, tiles and launch shapes;
	// 18-20: thread per site, plain products (every group and precision);
	// 29-34: SU(3) line march (k_md_line: plaquettes computed once, lower
	// staples along x1 and x3 handed over), launch shapes, products and
	// whether row 2 of whole links is read or rebuilt; 35-36: thread per site
	// with the force accumulators in shared memory (five blocks per SM); 37:
	// line march with the warp's own line staged by bulk copies (TMA); 38-39:
	// thread per site, software-pipelined neighbour loads; 40-45: thread per
	// site with two products per FP32x2 operation in the sections `pair`
	// selects (1 forward loops, 2 lower staples, 4 link update); 46-48:
	// thread per site with the next step's neighbour rows copied to shared
	// memory by cp.async; 49-53, 54-57: thread per site, more tile shapes of
	// 512 and 256 sites
	static constexpr int kForceVariants = 58;
	static int n_force_variants() { return ND == 4 ? kForceVariants : 2; }
	static ForceVariant force_variant(int v)
	{
		static const ForceVariant t[kForceVariants] = {
		    {0, {0, 0, 0, 0}, 256, 1, "eo-order/256thr/1blk"},
		    {0, {0, 0, 0, 0}, 256, 2, "eo-order/256thr/2blk"},
		    {1, {2, 2, 2, 2}, 256, 1, "tile4x4x4x4/256thr/1blk"},
		    {1, {2, 2, 2, 2}, 256, 2, "tile4x4x4x4/256thr/2blk"},
		    {1, {1, 2, 2, 2}, 128, 3, "tile2x4x4x4/128thr/3blk"},
		    {1, {1, 2, 2, 2}, 128, 4, "tile2x4x4x4/128thr/4blk"},
		    {1, {2, 2, 2, 3}, 256, 2, "tile4x4x4x8/256thr/2blk"},
		    {1, {1, 1, 2, 3}, 128, 4, "tile2x2x4x8/128thr/4blk"},
		    {1, {1, 1, 1, 3}, 128, 4, "tile2x2x2x8/128thr/4blk"},
		    {1, {1, 1, 2, 4}, 128, 4, "tile2x2x4x16/128thr/4blk"},
		    {1, {0, 1, 2, 4}, 128, 4, "tile1x2x4x16/128thr/4blk"},
		    {1, {1, 1, 2, 3}, 128, 4, "tile2x2x4x8/128thr/4blk/f32x2", true},
		    {1, {1, 1, 2, 3}, 128, 3, "tile2x2x4x8/128thr/3blk/f32x2", true},
		    {1, {2, 2, 2, 3}, 256, 2, "tile4x4x4x8/256thr/2blk/f32x2", true},
		    {2, {1, 1, 2, 3}, 128, 4, "site/tile2x2x4x8/128thr/4blk/f32x2", true},
		    {2, {1, 1, 2, 3}, 128, 3, "site/tile2x2x4x8/128thr/3blk/f32x2", true},
		    {2, {1, 2, 2, 3}, 256, 2, "site/tile2x4x4x8/256thr/2blk/f32x2", true},
		    {2, {0, 1, 2, 4}, 128, 4, "site/tile1x2x4x16/128thr/4blk/f32x2", true},
		    {2, {1, 1, 2, 3}, 128, 4, "site/tile2x2x4x8/128thr/4blk"},
		    {2, {1, 1, 2, 3}, 128, 3, "site/tile2x2x4x8/128thr/3blk"},
		    {2, {1, 2, 2, 3}, 256, 2, "site/tile2x4x4x8/256thr/2blk"},
		    {2, {2, 2, 2, 3}, 512, 1, "site/tile4x4x4x8/512thr/1blk/f32x2", true},
		    {2, {1, 2, 3, 3}, 512, 1, "site/tile2x4x8x8/512thr/1blk/f32x2", true},
		    {2, {0, 1, 3, 3}, 128, 4, "site/tile1x2x8x8/128thr/4blk/f32x2", 1},
		    {2, {1, 2, 2, 2}, 128, 4, "site/tile2x4x4x4/128thr/4blk/f32x2", 1},
		    {2, {0, 2, 2, 3}, 128, 4, "site/tile1x4x4x8/128thr/4blk/f32x2", 1},
		    {2, {2, 1, 1, 3}, 128, 4, "site/tile4x2x2x8/128thr/4blk/f32x2", 1},
		    {2, {0, 0, 3, 4}, 128, 4, "site/tile1x1x8x16/128thr/4blk/f32x2", 1},
		    {2, {1, 1, 1, 4}, 128, 4, "site/tile2x2x2x16/128thr/4blk/f32x2", 1},
		    {3, {0, 0, 0, 0}, 128, 4, "line/128thr/4blk/f32x2", 1},
		    {3, {0, 0, 0, 0}, 128, 4, "line/128thr/4blk/f32x2/pf", 1, 0, 0, 1},
		    {3, {0, 0, 0, 0}, 128, 5, "line/128thr/5blk/f32x2/fsm/pf", 1, 0, 1, 1},
		    {3, {0, 0, 0, 0}, 128, 5, "line/128thr/5blk/f32x2/fsm", 1, 0, 1},
		    {3, {0, 0, 0, 0}, 128, 4, "line/128thr/4blk/f32x2/row2", 1, 1},
		    {3, {0, 0, 0, 0}, 128, 4, "line/128thr/4blk/f32x2/row2/pf", 1, 1, 0, 1},
		    {2, {1, 1, 2, 3}, 128, 5, "site/tile2x2x4x8/128thr/5blk/f32x2/smacc", 1, 0, 0, 0, 1},
		    {2, {0, 2, 2, 3}, 128, 5, "site/tile1x4x4x8/128thr/5blk/f32x2/smacc", 1, 0, 0, 0, 1},
		    {3, {0, 0, 0, 0}, 64, 8, "line/64thr/8blk/f32x2/tma", 1, 0, 0, 0, 0, 1},
		    {2, {1, 1, 2, 3}, 128, 4, "site/tile2x2x4x8/128thr/4blk/f32x2/smacc/pipe", 1, 0, 0, 0, 1, 0, 1},
		    {2, {1, 1, 2, 3}, 128, 4, "site/tile2x2x4x8/128thr/4blk/f32x2/pipe", 1, 0, 0, 0, 0, 0, 1},
		    {2, {1, 1, 2, 3}, 128, 4, "site/tile2x2x4x8/128thr/4blk/pair-update", 1, 0, 0, 0, 0, 0, 0, 4},
		    {2, {1, 1, 2, 3}, 128, 5, "site/tile2x2x4x8/128thr/5blk/smacc/pair-update", 1, 0, 0, 0, 1, 0, 0, 4},
		    {2, {1, 1, 2, 3}, 128, 4, "site/tile2x2x4x8/128thr/4blk/smacc/pair-loops-update", 1, 0, 0, 0, 1, 0, 0, 5},
		    {2, {1, 1, 2, 3}, 128, 3, "site/tile2x2x4x8/128thr/3blk/smacc/pair-all", 1, 0, 0, 0, 1, 0, 0, 7},
		    {2, {1, 1, 2, 3}, 128, 3, "site/tile2x2x4x8/128thr/3blk/smacc/pair-loops-update", 1, 0, 0, 0, 1, 0, 0, 5},
		    {2, {0, 2, 2, 3}, 128, 4, "site/tile1x4x4x8/128thr/4blk/pair-update", 1, 0, 0, 0, 0, 0, 0, 4},
		    {2, {1, 1, 2, 3}, 128, 4, "site/tile2x2x4x8/128thr/4blk/f32x2/async", 1, 0, 0, 0, 0, 0, 0, 0, 1},
		    {2, {0, 2, 2, 3}, 128, 4, "site/tile1x4x4x8/128thr/4blk/f32x2/async", 1, 0, 0, 0, 0, 0, 0, 0, 1},
		    {2, {1, 1, 2, 3}, 128, 3, "site/tile2x2x4x8/128thr/3blk/f32x2/async", 1, 0, 0, 0, 0, 0, 0, 0, 1},
		    {2, {0, 3, 3, 3}, 512, 1, "site/tile1x8x8x8/512thr/1blk/f32x2", 1},
		    {2, {1, 1, 3, 4}, 512, 1, "site/tile2x2x8x16/512thr/1blk/f32x2", 1},
		    {2, {0, 2, 3, 4}, 512, 1, "site/tile1x4x8x16/512thr/1blk/f32x2", 1},
		    {2, {1, 2, 2, 4}, 512, 1, "site/tile2x4x4x16/512thr/1blk/f32x2", 1},
		    {2, {1, 1, 3, 3}, 256, 2, "site/tile2x2x8x8/256thr/2blk/f32x2", 1},
		    {2, {0, 1, 4, 4}, 512, 1, "site/tile1x2x16x16/512thr/1blk/f32x2", 1},
		    {2, {1, 1, 2, 5}, 512, 1, "site/tile2x2x4x32/512thr/1blk/f32x2", 1},
		    {2, {0, 2, 2, 5}, 512, 1, "site/tile1x4x4x32/512thr/1blk/f32x2", 1},
		    {2, {0, 1, 3, 5}, 512, 1, "site/tile1x2x8x32/512thr/1blk/f32x2", 1}};
		return t[v];
	}
	static bool force_variant_valid(Geom const &g, int v)
	{
		if (v < 0 || v >= n_force_variants())
			return false;
		ForceVariant fv = force_variant(v);
		if (fv.f2 && !kF2)
			return false;
		if (!fv.tiled)
			return true;
		if (fv.tiled == 3)
			return GRP == SU3 && ND == 4 && line_supported(g) && (!fv.st || (kF2 && g.L[3] == 32));
		if (ND != 4)
			return false;
		if (fv.tiled == 2 && kF2 && !LinkLoadSU3R32::fits(g.V))
			return false; // the per-site kernel's 32-bit link offsets
		for (int i = 0; i < 4; ++i)
			if (g.L[i] % (1 << fv.lt[i]) != 0)
				return false;
		return true;
	}
	static void launch_force(int v, Field &P, Field const &U, T coef, RedSlot kin, bool rows = false)
	{
		if constexpr (kRows<GRP, T>)
			if (rows)
				return launch_force_t<true>(v, P, U, coef, kin);
		launch_force_t<false>(v, P, U, coef, kin);
	}
	template <bool ROWS> static void launch_force_t(int v, Field &P, Field const &U, T coef, RedSlot kin)
	{
		auto &c = *U.ctx;
		Geom const &g = U.geom;
		ForceVariant fv = force_variant(v);
		T const *u = static_cast<T const *>(U.d);
		T *p = static_cast<T *>(P.d);
		if (!fv.tiled)
		{
			int64_t n = int64_t(ND) * g.V;
			unsigned b = grid_for(c, n, fv.threads, fv.minb * 2);
			if (b > unsigned(kMaxRedBlocks))
				b = kMaxRedBlocks;
			if (fv.minb == 1)
				k_momentum_step<GRP, T, ND, 256, 1, ROWS><<<b, 256, 0, c.stream>>>(g, u, p, coef, kin);
			else
				k_momentum_step<GRP, T, ND, 256, 2, ROWS><<<b, 256, 0, c.stream>>>(g, u, p, coef, kin);
		}
		else if constexpr (ND == 4)
		{
			unsigned b = 0;
			if (fv.tiled == 3)
			{
				launch_line<ROWS, false>(fv, g, u, p, coef, kin, c, nullptr, T(0), 0);
				MESH_LAUNCH_CHECK();
				return;
			}
			TileSpec ts = tiles_for(g, fv, c, b);
			if (fv.tiled == 2)
				launch_force_site<ROWS>(fv, b, g, ts, u, p, coef, kin, c);
			else if (fv.f2)
			{
				if constexpr (kF2)
				{
					if (fv.threads == 128 && fv.minb == 4)
						k_momentum_step_tiled<GRP, T, 4, 128, 4, true, ROWS>
						    <<<b, 128, 0, c.stream>>>(g, ts, u, p, coef, kin);
					else if (fv.threads == 128)
						k_momentum_step_tiled<GRP, T, 4, 128, 3, true, ROWS>
						    <<<b, 128, 0, c.stream>>>(g, ts, u, p, coef, kin);
					else
						k_momentum_step_tiled<GRP, T, 4, 256, 2, true, ROWS>
						    <<<b, 256, 0, c.stream>>>(g, ts, u, p, coef, kin);
				}
			}
			else if (fv.threads == 256 && fv.minb == 1)
				k_momentum_step_tiled<GRP, T, 4, 256, 1, false, ROWS><<<b, 256, 0, c.stream>>>(g, ts, u, p, coef, kin);
			else if (fv.threads == 256 && fv.minb == 2)
				k_momentum_step_tiled<GRP, T, 4, 256, 2, false, ROWS><<<b, 256, 0, c.stream>>>(g, ts, u, p, coef, kin);
			else if (fv.threads == 128 && fv.minb == 3)
				k_momentum_step_tiled<GRP, T, 4, 128, 3, false, ROWS><<<b, 128, 0, c.stream>>>(g, ts, u, p, coef, kin);
			else
				k_momentum_step_tiled<GRP, T, 4, 128, 4, false, ROWS><<<b, 128, 0, c.stream>>>(g, ts, u, p, coef, kin);
		}
		MESH_LAUNCH_CHECK();
	}
	template <bool ROWS>
	static void launch_force_site(ForceVariant const &fv, unsigned b, Geom const &g, TileSpec const &ts, T const *u,
	                              T *p, T coef, RedSlot kin, Context &c)
	{
		if constexpr (ND == 4)
		{
			if constexpr (kF2)
			{
				if (fv.f2)
					return site_cfg<1, ROWS, false>(fv, b, g, ts, u, p, coef, kin, c, nullptr, T(0), 0);
			}
			site_cfg<0, ROWS, false>(fv, b, g, ts, u, p, coef, kin, c, nullptr, T(0), 0);
		}
	}
	// the launch configurations of the thread-per-site kernel
	template <int F2, bool ROWS, bool FUSE>
	static void site_cfg(ForceVariant const &fv, unsigned b, Geom const &g, TileSpec const &ts, T const *u, T *p,
	                     T coef, RedSlot kin, Context &c, T *uo, T tu, int reunit)
	{
		if constexpr (GRP == SU3 && ROWS && F2)
		{
			if (fv.pair)
				return site_pair_cfg<ROWS, FUSE>(fv, b, g, ts, u, p, coef, kin, c, uo, tu, reunit);
			if (fv.async)
			{
				if (fv.minb == 4)
					k_momentum_step_site<GRP, T, 4, 128, 4, F2, ROWS, FUSE, false, false, 0, true>
					    <<<b, 128, 0, c.stream>>>(g, ts, u, p, coef, kin, uo, tu, reunit);
				else
					k_momentum_step_site<GRP, T, 4, 128, 3, F2, ROWS, FUSE, false, false, 0, true>
					    <<<b, 128, 0, c.stream>>>(g, ts, u, p, coef, kin, uo, tu, reunit);
				return;
			}
			if (fv.pipe)
			{
				if (fv.sm)
					k_momentum_step_site<GRP, T, 4, 128, 4, F2, ROWS, FUSE, true, true>
					    <<<b, 128, 0, c.stream>>>(g, ts, u, p, coef, kin, uo, tu, reunit);
				else
					k_momentum_step_site<GRP, T, 4, 128, 4, F2, ROWS, FUSE, false, true>
					    <<<b, 128, 0, c.stream>>>(g, ts, u, p, coef, kin, uo, tu, reunit);
				return;
			}
			if (fv.sm)
			{
				k_momentum_step_site<GRP, T, 4, 128, 5, F2, ROWS, FUSE, true>
				    <<<b, 128, 0, c.stream>>>(g, ts, u, p, coef, kin, uo, tu, reunit);
				return;
			}
		}
		if (fv.threads == 512)
			k_momentum_step_site<GRP, T, 4, 512, 1, F2, ROWS, FUSE>
			    <<<b, 512, 0, c.stream>>>(g, ts, u, p, coef, kin, uo, tu, reunit);
		else if (fv.threads == 128 && fv.minb == 4)
			k_momentum_step_site<GRP, T, 4, 128, 4, F2, ROWS, FUSE>
			    <<<b, 128, 0, c.stream>>>(g, ts, u, p, coef, kin, uo, tu, reunit);
		else if (fv.threads == 128)
			k_momentum_step_site<GRP, T, 4, 128, 3, F2, ROWS, FUSE>
			    <<<b, 128, 0, c.stream>>>(g, ts, u, p, coef, kin, uo, tu, reunit);
		else
			k_momentum_step_site<GRP, T, 4, 256, 2, F2, ROWS, FUSE>
			    <<<b, 256, 0, c.stream>>>(g, ts, u, p, coef, kin, uo, tu, reunit);
	}
	// the paired thread-per-site kernel's configurations (variants 40-45)
	template <bool ROWS, bool FUSE>
	static void site_pair_cfg(ForceVariant const &fv, unsigned b, Geom const &g, TileSpec const &ts, T const *u,
	                          T *p, T coef, RedSlot kin, Context &c, T *uo, T tu, int reunit)
	{
		if constexpr (kF2 && ROWS)
		{
#define MESH_PAIR_LAUNCH(MB, SMA, PARTS)                                                                             \
	k_momentum_step_site<GRP, T, 4, 128, MB, 1, ROWS, FUSE, SMA, false, PARTS>                                     \
	    <<<b, 128, 0, c.stream>>>(g, ts, u, p, coef, kin, uo, tu, reunit)
			if (fv.pair == 4 && !fv.sm)
				MESH_PAIR_LAUNCH(4, false, 4);
			else if (fv.pair == 4)
				MESH_PAIR_LAUNCH(5, true, 4);
			else if (fv.pair == 5 && fv.minb == 4)
				MESH_PAIR_LAUNCH(4, true, 5);
			else if (fv.pair == 5)
				MESH_PAIR_LAUNCH(3, true, 5);
			else
				MESH_PAIR_LAUNCH(3, true, 7);
#undef MESH_PAIR_LAUNCH
		}
	}
	// the line-march kernel (SU(3), four dimensions): persistent grid of at
	// most minb blocks per SM, every warp one contiguous range of line steps
	template <bool ROWS, bool FUSE>
	static void launch_line(ForceVariant const &fv, Geom const &g, T const *u, T *p, T coef, RedSlot kin,
	                        Context &c, T *uo, T tu, int reunit)
	{
		if constexpr (GRP == SU3 && ND == 4)
		{
			LineSpec ls{};
			ls.ns = 32 / g.L[3];
			ls.ncol = g.L[0] * (g.L[2] / ls.ns);
			// FP64 slots take twice the shared memory: 64-thread blocks
			int threads = sizeof(T) == 8 ? 64 : fv.threads;
			int minb = sizeof(T) == 8 ? 6 : fv.minb;
			int wpb = threads / 32;
			// segments of the x1 march: as many as the resident warps allow
			int64_t resident = int64_t(c.num_sms) * minb * wpb;
			int64_t nseg = resident / ls.ncol;
			ls.nseg = int(nseg < 1 ? 1 : (nseg > g.L[1] ? g.L[1] : nseg));
			ls.nwork = ls.ncol * ls.nseg;
			ls.err = c.d_err;
			unsigned b = unsigned((ls.nwork + wpb - 1) / wpb);
			if constexpr (sizeof(T) == 8)
				k_md_line<T, 64, 6, 0, ROWS, FUSE><<<b, 64, 0, c.stream>>>(g, ls, u, p, coef, kin, uo, tu, reunit);
			else
			{
				if (fv.f2)
					line_cfg<1, ROWS, FUSE>(fv, b, g, ls, u, p, coef, kin, c, uo, tu, reunit);
				else
					line_cfg<0, ROWS, FUSE>(fv, b, g, ls, u, p, coef, kin, c, uo, tu, reunit);
			}
		}
	}
	template <int F2, bool ROWS, bool FUSE>
	static void line_cfg(ForceVariant const &fv, unsigned b, Geom const &g, LineSpec const &ls, T const *u, T *p,
	                     T coef, RedSlot kin, Context &c, T *uo, T tu, int reunit)
	{
		auto go = [&](auto kernel, int threads) {
			kernel<<<b, threads, 0, c.stream>>>(g, ls, u, p, coef, kin, uo, tu, reunit);
		};
		if constexpr (ROWS && F2)
		{
			if (fv.st)
			{
				go(k_md_line<T, 64, 8, F2, ROWS, FUSE, false, false, false, true>, 64);
				return;
			}
			if (fv.fsm)
			{
				if (fv.pf)
					go(k_md_line<T, 128, 5, F2, ROWS, FUSE, false, true, true>, 128);
				else
					go(k_md_line<T, 128, 5, F2, ROWS, FUSE, false, true>, 128);
				return;
			}
			if (fv.r2)
			{
				if (fv.pf)
					go(k_md_line<T, 128, 4, F2, ROWS, FUSE, true, false, true>, 128);
				else
					go(k_md_line<T, 128, 4, F2, ROWS, FUSE, true>, 128);
				return;
			}
			if (fv.pf)
			{
				go(k_md_line<T, 128, 4, F2, ROWS, FUSE, false, false, true>, 128);
				return;
			}
		}
		if (fv.threads == 64)
			go(k_md_line<T, 64, 8, F2, ROWS, FUSE>, 64);
		else if (fv.minb == 3)
			go(k_md_line<T, 128, 3, F2, ROWS, FUSE>, 128);
		else
			go(k_md_line<T, 128, 4, F2, ROWS, FUSE>, 128);
	}
	// tiles of variant fv over g and the grid size (at most minb blocks per SM)
	static TileSpec tiles_for(Geom const &g, ForceVariant const &fv, Context const &c, unsigned &b)
	{
		TileSpec ts{};
		ts.sites = 1;
		ts.ntiles = 1;
		for (int i = 0; i < 4; ++i)
		{
			ts.lt[i] = fv.lt[i];
			ts.nt[i] = g.L[i] >> fv.lt[i];
			ts.sites <<= fv.lt[i];
			ts.ntiles *= ts.nt[i];
		}
		int64_t cap = int64_t(c.num_sms) * fv.minb;
		b = unsigned(ts.ntiles < cap ? ts.ntiles : cap);
		return ts;
	}
	// ---- fused momentum step + link update (trajectory) ----------------------
	static constexpr int kMdFirst = 14, kMdLast = 57; // thread-per-site and line-march variants
	static bool md_supported(Geom const &g)
	{
		if constexpr (ND != 4)
			return false;
		for (int v = kMdFirst; v <= kMdLast; ++v)
			if (force_variant_valid(g, v))
				return true;
		return false;
	}
	static void launch_md(int v, Field &P, Field const &Uin, Field &Uout, T coef, T tu, int reunit, RedSlot kin)
	{
		launch_md_t<kRows<GRP, T>>(v, P, Uin, Uout, coef, tu, reunit, kin);
	}
	template <bool R>
	static void launch_md_t(int v, Field &P, Field const &Uin, Field &Uout, T coef, T tu, int reunit, RedSlot kin)
	{
		if constexpr (ND == 4)
		{
			auto &c = *Uin.ctx;
			Geom const &g = Uin.geom;
			ForceVariant fv = force_variant(v);
			unsigned b = 0;
			T const *u = static_cast<T const *>(Uin.d);
			T *p = static_cast<T *>(P.d);
			T *uo = static_cast<T *>(Uout.d);
			if (fv.tiled == 3)
			{
				launch_line<R, true>(fv, g, u, p, coef, kin, c, uo, tu, reunit);
				MESH_LAUNCH_CHECK();
				return;
			}
			TileSpec ts = tiles_for(g, fv, c, b);
			if constexpr (kF2)
			{
				if (fv.f2)
					site_cfg<1, R, true>(fv, b, g, ts, u, p, coef, kin, c, uo, tu, reunit);
				else
					site_cfg<0, R, true>(fv, b, g, ts, u, p, coef, kin, c, uo, tu, reunit);
			}
			else
				site_cfg<0, R, true>(fv, b, g, ts, u, p, coef, kin, c, uo, tu, reunit);
			MESH_LAUNCH_CHECK();
		}
	}
	// fastest thread-per-site variant of the fused step for this lattice, timed
	// once with coef = 0 and tu = 0 (P unchanged, Uout = Uin); not while the
	// stream is capturing
	static constexpr int kSeparate = 1000; // the two steps as separate kernels were faster
	static int choose_md(Field &P, Field const &Uin, Field &Uout)
	{
		int ov = force_override();
		if (ov >= kMdFirst && ov <= kMdLast && force_variant_valid(Uin.geom, ov))
			return ov;
		if (ov >= 0 && ov < kMdFirst)
			return kSeparate; // a thread-per-link variant pinned: no fusion
		std::string key = "md_step/group" + std::to_string(GRP) + "/" + (sizeof(T) == 4 ? "f32" : "f64") + "/";
		for (int i = 0; i < ND; ++i)
			key += (i ? "x" : "") + std::to_string(Uin.dims[i]);
		int v = tuned_variant(key);
		if (v >= 0)
			return v;
		int dflt = -1;
		for (int cand = kMdFirst; cand <= kMdLast && dflt < 0; ++cand)
			if (force_variant_valid(Uin.geom, cand))
				dflt = cand;
		cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
		cudaStreamIsCapturing(Uin.ctx->stream, &cs);
		if (cs != cudaStreamCaptureStatusNone || !autotune_enabled())
			return dflt;
		auto &c = *Uin.ctx;
		cudaEvent_t e0, e1;
		MESH_CUDA(cudaEventCreate(&e0));
		MESH_CUDA(cudaEventCreate(&e1));
		float best = 1e30f;
		int bestv = dflt;
		std::string report;
		for (int cand = kMdFirst; cand <= kMdLast; ++cand)
		{
			if (!force_variant_valid(Uin.geom, cand))
				continue;
			launch_md(cand, P, Uin, Uout, T(0), T(0), 0, RedSlot{});
			MESH_CUDA(cudaEventRecord(e0, c.stream));
			for (int r = 0; r < 3; ++r)
				launch_md(cand, P, Uin, Uout, T(0), T(0), 0, RedSlot{});
			MESH_CUDA(cudaEventRecord(e1, c.stream));
			MESH_CUDA(cudaEventSynchronize(e1));
			float ms = 0;
			MESH_CUDA(cudaEventElapsedTime(&ms, e0, e1));
			ms /= 3;
			report += std::string(report.empty() ? "" : ", ") + force_variant(cand).name + "=" +
			          std::to_string(ms * 1000.0f) + "us";
			if (ms < best)
			{
				best = ms;
				bestv = cand;
			}
		}
		// against the momentum step and the link update as two kernels
		{
			int fv = choose_force(P, Uin, true);
			auto pair = [&] {
				launch_force(fv, P, Uin, T(0), RedSlot{}, true);
				hmc_evolve(Uin, Uout, P, 0.0, false);
			};
			pair();
			MESH_CUDA(cudaEventRecord(e0, c.stream));
			for (int r = 0; r < 3; ++r)
				pair();
			MESH_CUDA(cudaEventRecord(e1, c.stream));
			MESH_CUDA(cudaEventSynchronize(e1));
			float ms = 0;
			MESH_CUDA(cudaEventElapsedTime(&ms, e0, e1));
			ms /= 3;
			report += std::string(", separate ") + force_variant(fv).name + " + link update=" +
			          std::to_string(ms * 1000.0f) + "us";
			if (ms < best)
			{
				best = ms;
				bestv = kSeparate;
			}
		}
		cudaEventDestroy(e0);
		cudaEventDestroy(e1);
		set_tuned_variant(key, bestv,
		                  std::string("chosen ") + (bestv == kSeparate ? "separate kernels" : force_variant(bestv).name) +
		                      " [" + report + "]");
		return bestv;
	}
	// momentum step P -= coef F(Uin) fused with the link update
	// Uout = exp(tu P) Uin; false (nothing launched) where no fused variant fits
	static bool hmc_md_step(Field &P, Field const &Uin, Field &Uout, double coef, double tu, bool reunit,
	                        RedSlot *kin)
	{
		if (!md_supported(Uin.geom))
			return false;
		int v = choose_md(P, Uin, Uout);
		if (v == kSeparate)
			return false;
		launch_md(v, P, Uin, Uout, T(coef), T(tu), reunit ? 1 : 0, kin ? *kin : RedSlot{});
		return true;
	}
	static void hmc_tune_md(Field &P, Field const &Uin, Field &Uout)
	{
		if (md_supported(Uin.geom))
			choose_md(P, Uin, Uout);
	}
	static std::string force_key(Field const &U, bool rows)
	{
		std::string k = "momentum_step/group" + std::to_string(GRP) + "/" + (sizeof(T) == 4 ? "f32" : "f64") + "/";
		for (int i = 0; i < ND; ++i)
			k += (i ? "x" : "") + std::to_string(U.dims[i]);
		if (rows && kRows<GRP, T>)
			k += "/rows01";
		return k;
	}
	// fastest valid variant for this lattice, timed once with coef = 0 (the
	// momenta are rewritten unchanged); not while the stream is capturing
	static int choose_force(Field &P, Field const &U, bool rows = false)
	{
		int ov = force_override();
		if (ov >= 0 && ov < n_force_variants() && force_variant_valid(U.geom, ov))
			return ov;
		std::string key = force_key(U, rows);
		int v = tuned_variant(key);
		if (v >= 0)
			return v;
		int dflt = force_variant_valid(U.geom, 3) ? 3 : 0;
		cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
		cudaStreamIsCapturing(U.ctx->stream, &cs);
		if (cs != cudaStreamCaptureStatusNone || !autotune_enabled())
			return dflt;
		auto &c = *U.ctx;
		cudaEvent_t e0, e1;
		MESH_CUDA(cudaEventCreate(&e0));
		MESH_CUDA(cudaEventCreate(&e1));
		float best = 1e30f;
		int bestv = dflt;
		std::string report;
		for (int cand = 0; cand < n_force_variants(); ++cand)
		{
			if (!force_variant_valid(U.geom, cand))
				continue;
			launch_force(cand, P, U, T(0), RedSlot{}, rows);
			MESH_CUDA(cudaEventRecord(e0, c.stream));
			for (int r = 0; r < 3; ++r)
				launch_force(cand, P, U, T(0), RedSlot{}, rows);
			MESH_CUDA(cudaEventRecord(e1, c.stream));
			MESH_CUDA(cudaEventSynchronize(e1));
			float ms = 0;
			MESH_CUDA(cudaEventElapsedTime(&ms, e0, e1));
			ms /= 3;
			report += std::string(report.empty() ? "" : ", ") + force_variant(cand).name + "=" +
			          std::to_string(ms * 1000.0f) + "us";
			if (ms < best)
			{
				best = ms;
				bestv = cand;
			}
		}
		cudaEventDestroy(e0);
		cudaEventDestroy(e1);
		set_tuned_variant(key, bestv, std::string("chosen ") + force_variant(bestv).name + " [" + report + "]");
		return bestv;
	}
	static void tune(Field &P, Field const &U) { choose_force(P, U); }
	static void momentum_step(Field &P, Field const &U, double coef, RedSlot *kin)
	{
		int v = choose_force(P, U);
		launch_force(v, P, U, T(coef), kin ? *kin : RedSlot{});
	}
	static void hmc_tune(Field &P, Field const &U) { choose_force(P, U, true); }
	static void hmc_momentum_step(Field &P, Field const &U, double coef, RedSlot *kin)
	{
		int v = choose_force(P, U, true);
		launch_force(v, P, U, T(coef), kin ? *kin : RedSlot{}, true);
	}
	static void landau_functional(Field const &U, Field const &g, RedSlot out)
	{
		auto &c = *U.ctx;
		k_landau_functional<GRP, T, ND><<<red_blocks(c, U.geom.V), kBlock, 0, c.stream>>>(
		    U.geom, static_cast<T const *>(U.d), static_cast<T const *>(g.d), out);
		MESH_LAUNCH_CHECK();
	}
	static void landau_theta(Field const &U, Field const &g, RedSlot out)
	{
		auto &c = *U.ctx;
		k_landau_theta<GRP, T, ND><<<red_blocks(c, U.geom.V), kBlock, 0, c.stream>>>(
		    U.geom, static_cast<T const *>(U.d), static_cast<T const *>(g.d), out);
		MESH_LAUNCH_CHECK();
	}
	static void landau_deriv(Field &F, Field const &U, Field const &g, double scale)
	{
		auto &c = *U.ctx;
		k_landau_deriv<GRP, T, ND><<<blocks(c, U.geom.V), kBlock, 0, c.stream>>>(
		    U.geom, static_cast<T const *>(U.d), static_cast<T const *>(g.d), static_cast<T *>(F.d), T(scale));
		MESH_LAUNCH_CHECK();
	}
	static void landau_or_half(Field const &U, Field &g, double omega, int parity)
	{
		auto &c = *U.ctx;
		k_landau_or_half<GRP, T, ND><<<blocks(c, U.geom.Vh), kBlock, 0, c.stream>>>(
		    U.geom, parity, T(omega), static_cast<T const *>(U.d), static_cast<T *>(g.d));
		MESH_LAUNCH_CHECK();
	}
	static void alg_dot(Field const &a, Field const &b, RedSlot out)
	{
		auto &c = *a.ctx;
		int64_t n = int64_t(a.nstack) * a.geom.V;
		k_alg_dot<GRP, T><<<red_blocks(c, n), kBlock, 0, c.stream>>>(n, a.geom.V, static_cast<T const *>(a.d),
		                                                            static_cast<T const *>(b.d), out);
		MESH_LAUNCH_CHECK();
	}
	static void exp_apply(Field &dst, Field const &F, double eps, Field const &g)
	{
		auto &c = *g.ctx;
		k_exp_apply<GRP, T><<<blocks(c, g.geom.V), kBlock, 0, c.stream>>>(
		    g.geom.V, T(eps), static_cast<T const *>(F.d), static_cast<T const *>(g.d), static_cast<T *>(dst.d));
		MESH_LAUNCH_CHECK();
	}
	static void axpy_alg(Field &y, double a, Field const &x)
	{
		auto &c = *y.ctx;
		int64_t n = int64_t(y.nstack) * y.geom.V;
		k_axpy_alg<GRP, T><<<blocks(c, n), kBlock, 0, c.stream>>>(n, y.geom.V, T(a), static_cast<T const *>(x.d),
		                                                         static_cast<T *>(y.d));
		MESH_LAUNCH_CHECK();
	}
	static void gauge_transform(Field &U, Field const &g)
	{
		auto &c = *U.ctx;
		int64_t n = int64_t(ND) * U.geom.V;
		k_gauge_transform<GRP, T, ND><<<blocks(c, n), kBlock, 0, c.stream>>>(U.geom, static_cast<T *>(U.d),
		                                                                     static_cast<T const *>(g.d));
		MESH_LAUNCH_CHECK();
	}

	// one heat-bath (or overrelaxation) sweep: every direction, both parities
	static void gauge_sweep(Field &U, double beta, uint64_t seed, uint64_t ctr, bool overrelax)
	{
		auto &c = *U.ctx;
		for (int mu = 0; mu < ND; ++mu)
			for (int par = 0; par < 2; ++par)
			{
				if (overrelax)
					k_gauge_update<GRP, T, ND, true><<<blocks(c, U.geom.Vh), kBlock, 0, c.stream>>>(
					    U.geom, mu, par, static_cast<T *>(U.d), beta, seed, ctr);
				else
					k_gauge_update<GRP, T, ND, false><<<blocks(c, U.geom.Vh), kBlock, 0, c.stream>>>(
					    U.geom, mu, par, static_cast<T *>(U.d), beta, seed, ctr);
				MESH_LAUNCH_CHECK();
			}
	}
	// Wilson loops: one line extension / the r x t loop sum (4D only)
	static void line_extend(Field const &U, int dir, int n, void const *Lprev, void *Lout)
	{
		if constexpr (ND == 4)
		{
			auto &c = *U.ctx;
			k_line_extend<GRP, T, ND><<<blocks(c, U.geom.V), kBlock, 0, c.stream>>>(
			    U.geom, dir, n, static_cast<T const *>(Lprev), static_cast<T const *>(U.d), static_cast<T *>(Lout));
			MESH_LAUNCH_CHECK();
		}
	}
	static void wilson_rt(Field const &U, int r, int t, void const *S, void const *Tt, RedSlot out)
	{
		if constexpr (ND == 4)
		{
			auto &c = *U.ctx;
			k_wilson_rt<GRP, T, ND><<<red_blocks(c, U.geom.V), kBlock, 0, c.stream>>>(
			    U.geom, r, t, static_cast<T const *>(S), static_cast<T const *>(Tt), out);
			MESH_LAUNCH_CHECK();
		}
	}
	static OpsTable const *table()
	{
		static const OpsTable t = {import_,      export_,       set_unit,       random,  random_momenta_dev,       norm2,
		                           cshift,       site_op,       sum_real_trace, plaquette,      staple_sum,
		                           wilson_deriv, reunitize,     evolve,         momentum_step,  landau_functional,
		                           landau_theta, landau_deriv,  landau_or_half, reunit_exact,   alg_dot,
		                           exp_apply,    axpy_alg,      gauge_transform, tune,
		                           hmc_plaquette, hmc_evolve,   hmc_momentum_step, hmc_tune,
		                           hmc_md_step,   hmc_tune_md,  line_extend,    wilson_rt,
		                           gauge_sweep,   import_direct, export_direct};
		return &t;
	}
};

#define MESH_OPS_GETTER(NAME, GRP)                                                                                  \
	OpsTable const *NAME(int prec, int nd)                                                                           \
	{                                                                                                                \
		if (prec == MESH_F32)                                                                                        \
		{                                                                                                            \
			if (nd == 2)                                                                                             \
				return Ops<GRP, float, 2>::table();                                                                  \
			if (nd == 3)                                                                                             \
				return Ops<GRP, float, 3>::table();                                                                  \
			if (nd == 4)                                                                                             \
				return Ops<GRP, float, 4>::table();                                                                  \
		}                                                                                                            \
		else if (prec == MESH_F64)                                                                                   \
		{                                                                                                            \
			if (nd == 2)                                                                                             \
				return Ops<GRP, double, 2>::table();                                                                 \
			if (nd == 3)                                                                                             \
				return Ops<GRP, double, 3>::table();                                                                 \
			if (nd == 4)                                                                                             \
				return Ops<GRP, double, 4>::table();                                                                 \
		}                                                                                                            \
		return nullptr;                                                                                              \
	}

} // namespace meshgb
