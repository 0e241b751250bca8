// Kernels of the lattice-gauge hot path, templated over group (U(1), SU(2),
// SU(3)), real type and number of dimensions, and their host launchers.
// Instantiated per group in inst_u1.cu / inst_su2.cu / inst_su3.cu.
#pragma once

#include "field.cuh"
#include "group.cuh"
#include "rng.cuh"

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
		int L = g.L[dir];
		int xn = ((st.x[dir] + offset) % L + L) % L;
		int64_t lex = st.lex + int64_t(xn - st.x[dir]) * g.stride[dir];
		int par = (st.par + (xn - st.x[dir])) & 1;
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
		Soa<T, Gp::NR>::load(a, V, s, x.v);
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
template <int GRP, class T, int ND> struct LinkLoad
{
	using Gp = Group<GRP, T>;
	using E = typename Gp::E;
	T const *U;
	int64_t V;
	__device__ __forceinline__ E operator()(int mu, int64_t s) const
	{
		E e;
		Soa<T, Gp::NR>::load(U + int64_t(mu) * Gp::NR * V, V, s, e.v);
		return e;
	}
};

// sum over sites and planes mu<nu of ReTr(U_mu(x) U_nu(x+mu) U_mu(x+nu)^+ U_nu(x)^+)
template <int GRP, class T, int ND>
__global__ void __launch_bounds__(kBlock) k_plaquette(Geom g, T const *__restrict__ U, RedSlot out)
{
	using Gp = Group<GRP, T>;
	using E = typename Gp::E;
	LinkLoad<GRP, T, ND> ld{U, g.V};
	double acc = 0.0;
	MESH_GRID_LOOP(s, g.V)
	{
		Site<ND> st = site_from_eo<ND>(g, s);
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
		acc += double(t);
	}
	grid_sum<kBlock>(acc, out);
}

// staple sum for link (x, mu) in the reference's association order
// (utils.h:129-136): upper U_nu(x+mu) (U_nu(x) U_mu(x+nu))^+, lower
// (U_mu(y) U_nu(y+mu))^+ U_nu(y) at y = x - nu. MU is a template argument so
// that every coordinate access is static (no local-memory indexing).
template <int GRP, class T, int ND, int MU>
__device__ __forceinline__ typename Group<GRP, T>::E staple(Geom const &g, Site<ND> const &st, int64_t s,
                                                            LinkLoad<GRP, T, ND> const &ld)
{
	using Gp = Group<GRP, T>;
	using E = typename Gp::E;
	E S = Gp::zero();
	int64_t xpm = eo_shift1<ND>(g, st, MU, +1);
#pragma unroll
	for (int nu = 0; nu < ND; ++nu)
	{
		if (nu == MU)
			continue;
		{
			E b = ld(nu, xpm);
			E c = ld(MU, eo_shift1<ND>(g, st, nu, +1));
			E d = ld(nu, s);
			Gp::add_to(S, Gp::mul_nd(b, Gp::mul(d, c)));
		}
		{
			int64_t y = eo_shift1<ND>(g, st, nu, -1);
			E e = ld(MU, y);
			E f = ld(nu, eo_shift2<ND>(g, st, nu, -1, MU, +1));
			E h = ld(nu, y);
			Gp::add_to(S, Gp::mul_dn(Gp::mul(e, f), h));
		}
	}
	return S;
}

// calls f(std::integral_constant<int, mu>) for a runtime direction mu < ND
template <int ND, class Fn> __device__ __forceinline__ void with_mu(int mu, Fn &&f)
{
	switch (mu)
	{
	case 0:
		f(std::integral_constant<int, 0>{});
		break;
	case 1:
		f(std::integral_constant<int, 1>{});
		break;
	case 2:
		if constexpr (ND > 2)
			f(std::integral_constant<int, 2>{});
		break;
	default:
		if constexpr (ND > 3)
			f(std::integral_constant<int, 3>{});
		break;
	}
}

// P_mu(x) -= coef * proj(U_mu(x) S_mu(x)) with coef = beta/(2 Nc) * delta,
// one thread per (site, mu); optionally sums norm2 of the updated momenta
template <int GRP, class T, int ND, bool KIN>
__global__ void __launch_bounds__(kBlock)
    k_momentum_step(Geom g, T const *__restrict__ U, T *__restrict__ P, T coef, RedSlot kin)
{
	using Gp = Group<GRP, T>;
	using E = typename Gp::E;
	LinkLoad<GRP, T, ND> ld{U, g.V};
	double acc = 0.0;
	int64_t n = int64_t(ND) * g.V;
	MESH_GRID_LOOP(i, n)
	{
		int mu = int(i / g.V);
		int64_t s = i - int64_t(mu) * g.V;
		Site<ND> st = site_from_eo<ND>(g, s);
		with_mu<ND>(mu, [&](auto MUc) {
			constexpr int MU = decltype(MUc)::value;
			E S = staple<GRP, T, ND, MU>(g, st, s, ld);
			E W = Gp::mul(ld(MU, s), S);
			T f[Gp::NA], p[Gp::NA];
			Gp::proj(W, f);
			auto Pv = comp<T, Gp::NA>(P, g.V, MU);
			Pv.load(s, p);
#pragma unroll
			for (int k = 0; k < Gp::NA; ++k)
				p[k] -= coef * f[k];
			Pv.store(s, p);
			if constexpr (KIN)
				acc += double(Gp::kin(p));
		});
	}
	if constexpr (KIN)
		grid_sum<kBlock>(acc, kin);
}

template <int GRP, class T, int ND>
__global__ void __launch_bounds__(kBlock) k_staple_sum(Geom g, int mu, T const *__restrict__ U, T *__restrict__ S)
{
	using Gp = Group<GRP, T>;
	LinkLoad<GRP, T, ND> ld{U, g.V};
	MESH_GRID_LOOP(s, g.V)
	{
		Site<ND> st = site_from_eo<ND>(g, s);
		with_mu<ND>(mu, [&](auto MUc) {
			auto e = staple<GRP, T, ND, decltype(MUc)::value>(g, st, s, ld);
			Soa<T, Gp::NR>::store(S, g.V, s, e.v);
		});
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
		with_mu<ND>(mu, [&](auto MUc) {
			constexpr int MU = decltype(MUc)::value;
			E S = staple<GRP, T, ND, MU>(g, st, s, ld);
			E W = Gp::mul(ld(MU, s), S);
			T f[Gp::NA];
			Gp::proj(W, f);
#pragma unroll
			for (int k = 0; k < Gp::NA; ++k)
				f[k] *= scale;
			Soa<T, Gp::NA>::store(F, g.V, s, f);
		});
	}
}

// U_dst = exp(t P) U_src for every (site, mu); optional project_on_group_fast
template <int GRP, class T, bool REUNIT>
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
	static void momentum_step(Field &P, Field const &U, double coef, RedSlot *kin)
	{
		auto &c = *U.ctx;
		int64_t n = int64_t(ND) * U.geom.V;
		if (kin)
			k_momentum_step<GRP, T, ND, true><<<red_blocks(c, n), kBlock, 0, c.stream>>>(
			    U.geom, static_cast<T const *>(U.d), static_cast<T *>(P.d), T(coef), *kin);
		else
			k_momentum_step<GRP, T, ND, false><<<blocks(c, n), kBlock, 0, c.stream>>>(
			    U.geom, static_cast<T const *>(U.d), static_cast<T *>(P.d), T(coef), RedSlot{});
		MESH_LAUNCH_CHECK();
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

	static OpsTable const *table()
	{
		static const OpsTable t = {import_,      export_,       set_unit,       random,  random_momenta_dev,       norm2,
		                           cshift,       site_op,       sum_real_trace, plaquette,      staple_sum,
		                           wilson_deriv, reunitize,     evolve,         momentum_step,  landau_functional,
		                           landau_theta, landau_deriv,  landau_or_half, reunit_exact,   alg_dot,
		                           exp_apply,    axpy_alg,      gauge_transform};
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
