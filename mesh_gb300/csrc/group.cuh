// Per-element group and algebra arithmetic for U(1), SU(2), SU(3) in float or
// double, for device (and host) code.
//
// Element layouts are the reference's object layouts (src/gauge/groups.h):
//   U(1):  complex      (re, im)                       2 reals
//   SU(2): quaternion   (re, im1, im2, im3)            4 reals, Hamilton product
//   SU(3): 3x3 complex  row-major (re, im) pairs      18 reals
// Algebra elements (momenta, forces) are stored packed:
//   U(1): 1 real a <-> (0, a);  SU(2): 3 reals <-> (0, v1, v2, v3);
//   SU(3): 8 reals (a0, a1, b01, b02, b12) <->
//          [[i a0, b01, b02], [-b01*, i a1, b12], [-b02*, -b12*, -i(a0+a1)]].
//
// Operations follow groups.h: adj (:55,135,214), real_trace (:59,137,219),
// project_on_algebra (:64,142,224), project_on_group_fast (:79,188,237),
// exp (:103,153,263). The SU(3) exponential of an algebra element uses the
// Cayley-Hamilton form exp(iQ) = f0 + f1 Q + f2 Q^2 of Morningstar & Peardon,
// Phys. Rev. D 69 (2004) 054501, eqs. (19)-(35), instead of util::exp.
#pragma once

#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>

#ifndef MESH_HD
#define MESH_HD __host__ __device__ __forceinline__
#endif

namespace meshgb {

template <class T> struct cx
{
	T re, im;
};

// cos x and sin(x)/x from x^2 for x^2 < 1/4 by their Taylor series through
// x^8 (remainders below x^10/10! < 3e-10): the small angles of FP32 link
// updates, without a range-reduced sincos
template <class T> MESH_HD void cos_sinc_small(T x2, T *c, T *sc)
{
	*c = T(1) - x2 * (T(1.0 / 2) - x2 * (T(1.0 / 24) - x2 * (T(1.0 / 720) - x2 * T(1.0 / 40320))));
	*sc = T(1) - x2 * (T(1.0 / 6) - x2 * (T(1.0 / 120) - x2 * (T(1.0 / 5040) - x2 * T(1.0 / 362880))));
}
template <class T> MESH_HD cx<T> cmul(cx<T> a, cx<T> b) { return {a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re}; }
template <class T> MESH_HD cx<T> cadd(cx<T> a, cx<T> b) { return {a.re + b.re, a.im + b.im}; }
template <class T> MESH_HD cx<T> csub(cx<T> a, cx<T> b) { return {a.re - b.re, a.im - b.im}; }
template <class T> MESH_HD cx<T> cconj(cx<T> a) { return {a.re, -a.im}; }
template <class T> MESH_HD cx<T> cscale(cx<T> a, T s) { return {a.re * s, a.im * s}; }

template <class T> MESH_HD T m_sqrt(T x) { return sqrt(x); }
template <class T> MESH_HD T m_rsqrt(T x) { return T(1) / sqrt(x); }
template <class T> MESH_HD void m_sincos(T x, T *s, T *c)
{
	*s = sin(x);
	*c = cos(x);
}
#ifdef __CUDA_ARCH__
template <> __device__ __forceinline__ void m_sincos<float>(float x, float *s, float *c) { sincosf(x, s, c); }
template <> __device__ __forceinline__ void m_sincos<double>(double x, double *s, double *c) { sincos(x, s, c); }
#endif

enum
{
	U1 = 1,
	SU2 = 2,
	SU3 = 3
};

template <int GRP, class T> struct Group;

// ---------------------------------------------------------------------------
// U(1)
// ---------------------------------------------------------------------------
template <class T> struct Group<U1, T>
{
	using real = T;
	static constexpr int NR = 2, NA = 1, NC = 1, DIM = 1;
	static constexpr int NNORM_GROUP = 2; // normals for a Haar element
	struct E
	{
		T v[2];
	};
	MESH_HD static E unit() { return {{T(1), T(0)}}; }
	MESH_HD static E zero() { return {{T(0), T(0)}}; }
	MESH_HD static E mul(E a, E b) { return {{a.v[0] * b.v[0] - a.v[1] * b.v[1], a.v[0] * b.v[1] + a.v[1] * b.v[0]}}; }
	// a * b^dagger
	MESH_HD static E mul_nd(E a, E b) { return {{a.v[0] * b.v[0] + a.v[1] * b.v[1], a.v[1] * b.v[0] - a.v[0] * b.v[1]}}; }
	// a^dagger * b
	MESH_HD static E mul_dn(E a, E b) { return {{a.v[0] * b.v[0] + a.v[1] * b.v[1], a.v[0] * b.v[1] - a.v[1] * b.v[0]}}; }
	MESH_HD static E adj(E a) { return {{a.v[0], -a.v[1]}}; }
	MESH_HD static void add_to(E &a, E b)
	{
		a.v[0] += b.v[0];
		a.v[1] += b.v[1];
	}
	MESH_HD static void sub_from(E &a, E b)
	{
		a.v[0] -= b.v[0];
		a.v[1] -= b.v[1];
	}
	MESH_HD static T retr(E a) { return a.v[0]; }
	// ReTr(a b^dagger)
	MESH_HD static T retr_nd(E a, E b) { return a.v[0] * b.v[0] + a.v[1] * b.v[1]; }
	MESH_HD static void proj(E a, T *o) { o[0] = a.v[1]; }
	MESH_HD static E from_alg(T const *o) { return {{T(0), o[0]}}; }
	MESH_HD static T kin(T const *o) { return o[0] * o[0]; }
	// exp(t X)
	MESH_HD static E exp_alg(T const *o, T t)
	{
		T x = o[0] * t;
		if constexpr (sizeof(T) == 4)
			if (x * x < T(0.25))
			{
				T c, sc;
				cos_sinc_small(x * x, &c, &sc);
				return {{c, x * sc}};
			}
		T s, c;
		m_sincos(x, &s, &c);
		return {{c, s}};
	}
	MESH_HD static E reunit_fast(E a)
	{
		if constexpr (sizeof(T) == 4)
		{
			// a - a (|a|^2 - 1) / 2 with |a|^2 - 1 accumulated from -1: no
			// quantity near 1.0 is rounded (the float grid is twice as fine
			// below 1 as above, which biases such roundings)
			T g = fmaf(a.v[0], a.v[0], fmaf(a.v[1], a.v[1], T(-1))) * T(-0.5);
			return {{fmaf(a.v[0], g, a.v[0]), fmaf(a.v[1], g, a.v[1])}};
		}
		T f = T(1.5) - (a.v[0] * a.v[0] + a.v[1] * a.v[1]) * T(0.5);
		return {{a.v[0] * f, a.v[1] * f}};
	}
	MESH_HD static E reunit_exact(E a)
	{
		T f = m_rsqrt(a.v[0] * a.v[0] + a.v[1] * a.v[1]);
		return {{a.v[0] * f, a.v[1] * f}};
	}
	MESH_HD static void alg_from_normals(T const *p, T *o) { o[0] = p[0] * T(0.70710678118654752440); }
	MESH_HD static E group_from_normals(T const *p)
	{
		T t = atan2(p[1], p[0]);
		T s, c;
		m_sincos(t, &s, &c);
		return {{c, s}};
	}
};

// ---------------------------------------------------------------------------
// SU(2) as unit quaternions
// ---------------------------------------------------------------------------
template <class T> struct Group<SU2, T>
{
	using real = T;
	static constexpr int NR = 4, NA = 3, NC = 2, DIM = 3;
	static constexpr int NNORM_GROUP = 4;
	struct E
	{
		T v[4];
	};
	MESH_HD static E unit() { return {{T(1), T(0), T(0), T(0)}}; }
	MESH_HD static E zero() { return {{T(0), T(0), T(0), T(0)}}; }
	MESH_HD static E mul(E a, E b)
	{
		return {{a.v[0] * b.v[0] - a.v[1] * b.v[1] - a.v[2] * b.v[2] - a.v[3] * b.v[3],
		         a.v[0] * b.v[1] + a.v[1] * b.v[0] + a.v[2] * b.v[3] - a.v[3] * b.v[2],
		         a.v[0] * b.v[2] - a.v[1] * b.v[3] + a.v[2] * b.v[0] + a.v[3] * b.v[1],
		         a.v[0] * b.v[3] + a.v[1] * b.v[2] - a.v[2] * b.v[1] + a.v[3] * b.v[0]}};
	}
	MESH_HD static E adj(E a) { return {{a.v[0], -a.v[1], -a.v[2], -a.v[3]}}; }
	MESH_HD static E mul_nd(E a, E b) { return mul(a, adj(b)); }
	MESH_HD static E mul_dn(E a, E b) { return mul(adj(a), b); }
	MESH_HD static void add_to(E &a, E b)
	{
#pragma unroll
		for (int i = 0; i < 4; ++i)
			a.v[i] += b.v[i];
	}
	MESH_HD static void sub_from(E &a, E b)
	{
#pragma unroll
		for (int i = 0; i < 4; ++i)
			a.v[i] -= b.v[i];
	}
	MESH_HD static T retr(E a) { return a.v[0] * T(2); }
	// ReTr(a b^dagger) = 2 Re(a conj(b)) = 2 a.b
	MESH_HD static T retr_nd(E a, E b)
	{
		return T(2) * (a.v[0] * b.v[0] + a.v[1] * b.v[1] + a.v[2] * b.v[2] + a.v[3] * b.v[3]);
	}
	MESH_HD static void proj(E a, T *o)
	{
		o[0] = a.v[1];
		o[1] = a.v[2];
		o[2] = a.v[3];
	}
	MESH_HD static E from_alg(T const *o) { return {{T(0), o[0], o[1], o[2]}}; }
	// 2x2 Frobenius norm of the algebra element
	MESH_HD static T kin(T const *o) { return T(2) * (o[0] * o[0] + o[1] * o[1] + o[2] * o[2]); }
	MESH_HD static E exp_alg(T const *o, T t)
	{
		T a1 = o[0] * t, a2 = o[1] * t, a3 = o[2] * t;
		if constexpr (sizeof(T) == 4)
		{
			T al2 = a1 * a1 + a2 * a2 + a3 * a3;
			if (al2 < T(0.25))
			{
				T c, sc;
				cos_sinc_small(al2, &c, &sc);
				return {{c, a1 * sc, a2 * sc, a3 * sc}};
			}
		}
		T al = m_sqrt(a1 * a1 + a2 * a2 + a3 * a3);
		T s, c;
		m_sincos(al, &s, &c);
		// sin(al)/al with its limit 1 at al == 0 (groups.h:153-164 divides)
		T f = al == T(0) ? T(1) : s / al;
		return {{c, a1 * f, a2 * f, a3 * f}};
	}
	MESH_HD static E reunit_fast(E a)
	{
		if constexpr (sizeof(T) == 4)
		{
			// a - a (|a|^2 - 1) / 2, no quantity near 1.0 rounded (see U(1))
			T g = fmaf(a.v[0], a.v[0], fmaf(a.v[1], a.v[1], fmaf(a.v[2], a.v[2], fmaf(a.v[3], a.v[3], T(-1))))) *
			      T(-0.5);
			return {{fmaf(a.v[0], g, a.v[0]), fmaf(a.v[1], g, a.v[1]), fmaf(a.v[2], g, a.v[2]),
			         fmaf(a.v[3], g, a.v[3])}};
		}
		T n = a.v[0] * a.v[0] + a.v[1] * a.v[1] + a.v[2] * a.v[2] + a.v[3] * a.v[3];
		T f = T(1.5) - n * T(0.5);
		return {{a.v[0] * f, a.v[1] * f, a.v[2] * f, a.v[3] * f}};
	}
	MESH_HD static E reunit_exact(E a)
	{
		T f = m_rsqrt(a.v[0] * a.v[0] + a.v[1] * a.v[1] + a.v[2] * a.v[2] + a.v[3] * a.v[3]);
		return {{a.v[0] * f, a.v[1] * f, a.v[2] * f, a.v[3] * f}};
	}
	MESH_HD static void alg_from_normals(T const *p, T *o)
	{
		o[0] = T(0.5) * p[0];
		o[1] = T(0.5) * p[1];
		o[2] = T(0.5) * p[2];
	}
	MESH_HD static E group_from_normals(T const *p) { return reunit_exact({{p[0], p[1], p[2], p[3]}}); }
};

// ---------------------------------------------------------------------------
// SU(3) as 3x3 complex matrices
// ---------------------------------------------------------------------------
template <class T> struct Group<SU3, T>
{
	using real = T;
	static constexpr int NR = 18, NA = 8, NC = 3, DIM = 8;
	static constexpr int NNORM_GROUP = 18;
	struct E
	{
		T v[18];
		MESH_HD cx<T> at(int i, int j) const { return {v[6 * i + 2 * j], v[6 * i + 2 * j + 1]}; }
		MESH_HD void set(int i, int j, cx<T> z)
		{
			v[6 * i + 2 * j] = z.re;
			v[6 * i + 2 * j + 1] = z.im;
		}
	};
	MESH_HD static E zero()
	{
		E r;
#pragma unroll
		for (int k = 0; k < 18; ++k)
			r.v[k] = T(0);
		return r;
	}
	MESH_HD static E unit()
	{
		E r = zero();
		r.v[0] = r.v[8] = r.v[16] = T(1);
		return r;
	}
	// c = a * b
	MESH_HD static E mul(E const &a, E const &b)
	{
		E r;
#pragma unroll
		for (int i = 0; i < 3; ++i)
#pragma unroll
			for (int j = 0; j < 3; ++j)
			{
				T re = a.v[6 * i] * b.v[2 * j] - a.v[6 * i + 1] * b.v[2 * j + 1];
				T im = a.v[6 * i] * b.v[2 * j + 1] + a.v[6 * i + 1] * b.v[2 * j];
#pragma unroll
				for (int k = 1; k < 3; ++k)
				{
					re += a.v[6 * i + 2 * k] * b.v[6 * k + 2 * j] - a.v[6 * i + 2 * k + 1] * b.v[6 * k + 2 * j + 1];
					im += a.v[6 * i + 2 * k] * b.v[6 * k + 2 * j + 1] + a.v[6 * i + 2 * k + 1] * b.v[6 * k + 2 * j];
				}
				r.v[6 * i + 2 * j] = re;
				r.v[6 * i + 2 * j + 1] = im;
			}
		return r;
	}
	// c = a * b for special unitary a, b: rows 0 and 1 of the product (only
	// rows 0 and 1 of a are read), row 2 rebuilt as conj(row 0 x row 1)
	MESH_HD static E mul_r2(E const &a, E const &b)
	{
		E r;
#pragma unroll
		for (int i = 0; i < 2; ++i)
#pragma unroll
			for (int j = 0; j < 3; ++j)
			{
				T re = 0, im = 0;
#pragma unroll
				for (int k = 0; k < 3; ++k)
				{
					re += a.v[6 * i + 2 * k] * b.v[6 * k + 2 * j] - a.v[6 * i + 2 * k + 1] * b.v[6 * k + 2 * j + 1];
					im += a.v[6 * i + 2 * k] * b.v[6 * k + 2 * j + 1] + a.v[6 * i + 2 * k + 1] * b.v[6 * k + 2 * j];
				}
				r.v[6 * i + 2 * j] = re;
				r.v[6 * i + 2 * j + 1] = im;
			}
		complete_row2(r);
		return r;
	}
	// c = a * b^dagger:  c_ij = sum_k a_ik conj(b_jk)
	MESH_HD static E mul_nd(E const &a, E const &b)
	{
		E r;
#pragma unroll
		for (int i = 0; i < 3; ++i)
#pragma unroll
			for (int j = 0; j < 3; ++j)
			{
				T re = 0, im = 0;
#pragma unroll
				for (int k = 0; k < 3; ++k)
				{
					T ar = a.v[6 * i + 2 * k], ai = a.v[6 * i + 2 * k + 1];
					T br = b.v[6 * j + 2 * k], bi = b.v[6 * j + 2 * k + 1];
					re += ar * br + ai * bi;
					im += ai * br - ar * bi;
				}
				r.v[6 * i + 2 * j] = re;
				r.v[6 * i + 2 * j + 1] = im;
			}
		return r;
	}
	// c = a^dagger * b:  c_ij = sum_k conj(a_ki) b_kj
	MESH_HD static E mul_dn(E const &a, E const &b)
	{
		E r;
#pragma unroll
		for (int i = 0; i < 3; ++i)
#pragma unroll
			for (int j = 0; j < 3; ++j)
			{
				T re = 0, im = 0;
#pragma unroll
				for (int k = 0; k < 3; ++k)
				{
					T ar = a.v[6 * k + 2 * i], ai = a.v[6 * k + 2 * i + 1];
					T br = b.v[6 * k + 2 * j], bi = b.v[6 * k + 2 * j + 1];
					re += ar * br + ai * bi;
					im += ar * bi - ai * br;
				}
				r.v[6 * i + 2 * j] = re;
				r.v[6 * i + 2 * j + 1] = im;
			}
		return r;
	}
	MESH_HD static E adj(E const &a)
	{
		E r;
#pragma unroll
		for (int i = 0; i < 3; ++i)
#pragma unroll
			for (int j = 0; j < 3; ++j)
			{
				r.v[6 * i + 2 * j] = a.v[6 * j + 2 * i];
				r.v[6 * i + 2 * j + 1] = -a.v[6 * j + 2 * i + 1];
			}
		return r;
	}
	MESH_HD static void add_to(E &a, E const &b)
	{
#pragma unroll
		for (int k = 0; k < 18; ++k)
			a.v[k] += b.v[k];
	}
	MESH_HD static void sub_from(E &a, E const &b)
	{
#pragma unroll
		for (int k = 0; k < 18; ++k)
			a.v[k] -= b.v[k];
	}
	MESH_HD static T retr(E const &a) { return a.v[0] + a.v[8] + a.v[16]; }
	MESH_HD static T retr_nd(E const &a, E const &b)
	{
		T s = 0;
#pragma unroll
		for (int k = 0; k < 18; ++k)
			s += a.v[k] * b.v[k];
		return s;
	}
	// antihermitian traceless part, packed
	MESH_HD static void proj(E const &a, T *o)
	{
		T t = (a.v[1] + a.v[9] + a.v[17]) * T(1.0 / 3.0);
		o[0] = a.v[1] - t;
		o[1] = a.v[9] - t;
		o[2] = (a.v[2] - a.v[6]) * T(0.5);
		o[3] = (a.v[3] + a.v[7]) * T(0.5);
		o[4] = (a.v[4] - a.v[12]) * T(0.5);
		o[5] = (a.v[5] + a.v[13]) * T(0.5);
		o[6] = (a.v[10] - a.v[14]) * T(0.5);
		o[7] = (a.v[11] + a.v[15]) * T(0.5);
	}
	MESH_HD static E from_alg(T const *o)
	{
		E r;
		r.v[0] = 0;
		r.v[1] = o[0];
		r.v[8] = 0;
		r.v[9] = o[1];
		r.v[16] = 0;
		r.v[17] = -(o[0] + o[1]);
		r.v[2] = o[2];
		r.v[3] = o[3];
		r.v[4] = o[4];
		r.v[5] = o[5];
		r.v[10] = o[6];
		r.v[11] = o[7];
		r.v[6] = -o[2];
		r.v[7] = o[3];
		r.v[12] = -o[4];
		r.v[13] = o[5];
		r.v[14] = -o[6];
		r.v[15] = o[7];
		return r;
	}
	// sum_ij |A_ij|^2 of the algebra element
	MESH_HD static T kin(T const *o)
	{
		T d = o[0] + o[1];
		return o[0] * o[0] + o[1] * o[1] + d * d +
		       T(2) * (o[2] * o[2] + o[3] * o[3] + o[4] * o[4] + o[5] * o[5] + o[6] * o[6] + o[7] * o[7]);
	}
	MESH_HD static cx<T> det(E const &m)
	{
		cx<T> a = cmul(m.at(1, 1), m.at(2, 2)), b = cmul(m.at(1, 2), m.at(2, 1));
		cx<T> c = cmul(m.at(1, 0), m.at(2, 2)), d = cmul(m.at(1, 2), m.at(2, 0));
		cx<T> e = cmul(m.at(1, 0), m.at(2, 1)), f = cmul(m.at(1, 1), m.at(2, 0));
		cx<T> r = cmul(m.at(0, 0), csub(a, b));
		r = csub(r, cmul(m.at(0, 1), csub(c, d)));
		return cadd(r, cmul(m.at(0, 2), csub(e, f)));
	}
	// X^2 for antihermitian X: hermitian, (X^2)_ii = -sum_k |X_ik|^2 and
	// (X^2)_ji = conj((X^2)_ij), so only the upper triangle is multiplied out
	MESH_HD static E sq_ah(E const &X)
	{
		E r;
#pragma unroll
		for (int i = 0; i < 3; ++i)
		{
			T d = 0;
#pragma unroll
			for (int k = 0; k < 3; ++k)
				d -= X.v[6 * i + 2 * k] * X.v[6 * i + 2 * k] + X.v[6 * i + 2 * k + 1] * X.v[6 * i + 2 * k + 1];
			r.v[6 * i + 2 * i] = d;
			r.v[6 * i + 2 * i + 1] = T(0);
#pragma unroll
			for (int j = i + 1; j < 3; ++j)
			{
				cx<T> z = {T(0), T(0)};
#pragma unroll
				for (int k = 0; k < 3; ++k)
					z = cadd(z, cmul(X.at(i, k), X.at(k, j)));
				r.set(i, j, z);
				r.set(j, i, cconj(z));
			}
		}
		return r;
	}
	// exp(X) for antihermitian traceless X with |X| < 1 (Frobenius norm), as
	// the power series truncated after X^N (N = 10: remainder below
	// |X|^11/11! = 2.5e-8; N = 6 for |X| < 0.2: below 0.2^7/7! = 2.5e-9) and
	// reduced to a polynomial u0 + u1 X + u2 X^2 with the Cayley-Hamilton
	// relation X^3 = -c1 X + i dim, c1 = |X|^2/2, i dim = det X; the series
	// is summed by Horner's rule on the three coefficients (M. Luscher,
	// "SU(3) matrix functions", openQCD notes). No transcendental functions:
	// the FP32 trajectory's link update.
	template <int N = 10> MESH_HD static E exp_series(E const &X, E const &X2, T c1, T dim)
	{
		static_assert(N >= 1 && N <= 10, "series order");
		// 1/k! for k = 0..N
		constexpr T inv_fact[11] = {T(1),
		                               T(1),
		                               T(1.0 / 2),
		                               T(1.0 / 6),
		                               T(1.0 / 24),
		                               T(1.0 / 120),
		                               T(1.0 / 720),
		                               T(1.0 / 5040),
		                               T(1.0 / 40320),
		                               T(1.0 / 362880),
		                               T(1.0 / 3628800)};
		cx<T> u0 = {inv_fact[N], T(0)}, u1 = {T(0), T(0)}, u2 = {T(0), T(0)};
#pragma unroll
		for (int k = N - 1; k >= 0; --k)
		{
			// X (u0 + u1 X + u2 X^2) + 1/k! = (i dim u2 + 1/k!) + (u0 - c1 u2) X + u1 X^2
			cx<T> n0 = {inv_fact[k] - dim * u2.im, dim * u2.re};
			cx<T> n1 = {u0.re - c1 * u2.re, u0.im - c1 * u2.im};
			u2 = u1;
			u1 = n1;
			u0 = n0;
		}
		E r;
#pragma unroll
		for (int i = 0; i < 3; ++i)
#pragma unroll
			for (int j = 0; j < 3; ++j)
			{
				cx<T> z = cadd(cmul(u1, X.at(i, j)), cmul(u2, X2.at(i, j)));
				if (i == j)
					z = cadd(z, u0);
				r.set(i, j, z);
			}
		return r;
	}
	// rows 0 and 1 of exp(t X) for X = from_alg(o), FP32, when |tX| < 0.2
	// (a molecular-dynamics step; row 2 of the result left unset): the order-6
	// series of exp_series with only the entries rows 0 and 1 read, each real
	// part one multiply and three fused multiply-adds; exp_alg otherwise
	MESH_HD static E exp_alg_rows01(T const *o, T t)
	{
		static_assert(sizeof(T) == 4, "FP32 only");
		T x[8];
#pragma unroll
		for (int k = 0; k < 8; ++k)
			x[k] = o[k] * t;
		T c1 = T(0.5) * kin(x);
		if (!(c1 < T(0.02)))
			return exp_alg(o, t);
		E X = from_alg(x);
		// X^2 rows 0, 1 (hermitian): diagonal -sum_k |X_ik|^2, (0,1), (0,2),
		// (1,2) multiplied out, (1,0) = conj (0,1)
		T d0 = 0, d1 = 0;
#pragma unroll
		for (int k = 0; k < 3; ++k)
		{
			d0 = fmaf(X.v[2 * k], X.v[2 * k], fmaf(X.v[2 * k + 1], X.v[2 * k + 1], d0));
			d1 = fmaf(X.v[6 + 2 * k], X.v[6 + 2 * k], fmaf(X.v[6 + 2 * k + 1], X.v[6 + 2 * k + 1], d1));
		}
		auto up = [&](int i, int j, T &re, T &im) {
			re = 0, im = 0;
#pragma unroll
			for (int k = 0; k < 3; ++k)
			{
				T ar = X.v[6 * i + 2 * k], ai = X.v[6 * i + 2 * k + 1];
				T br = X.v[6 * k + 2 * j], bi = X.v[6 * k + 2 * j + 1];
				re = fmaf(ar, br, fmaf(-ai, bi, re));
				im = fmaf(ar, bi, fmaf(ai, br, im));
			}
		};
		E X2;
		X2.v[0] = -d0, X2.v[1] = 0;
		X2.v[8] = -d1, X2.v[9] = 0;
		up(0, 1, X2.v[2], X2.v[3]);
		up(0, 2, X2.v[4], X2.v[5]);
		up(1, 2, X2.v[10], X2.v[11]);
		X2.v[6] = X2.v[2], X2.v[7] = -X2.v[3];
		// i dim = det X
		T dim = det(X).im;
		constexpr int N = 6;
		constexpr T inv_fact[N + 1] = {T(1), T(1), T(1.0 / 2), T(1.0 / 6), T(1.0 / 24), T(1.0 / 120), T(1.0 / 720)};
		T u0r = inv_fact[N], u0i = 0, u1r = 0, u1i = 0, u2r = 0, u2i = 0;
#pragma unroll
		for (int k = N - 1; k >= 0; --k)
		{
			T n0r = fmaf(-dim, u2i, inv_fact[k]), n0i = dim * u2r;
			T n1r = fmaf(-c1, u2r, u0r), n1i = fmaf(-c1, u2i, u0i);
			u2r = u1r, u2i = u1i;
			u1r = n1r, u1i = n1i;
			u0r = n0r, u0i = n0i;
		}
		E r;
#pragma unroll
		for (int k = 0; k < 6; ++k)
		{
			T xr = X.v[2 * k], xi = X.v[2 * k + 1], yr = X2.v[2 * k], yi = X2.v[2 * k + 1];
			T re = fmaf(u1r, xr, fmaf(-u1i, xi, fmaf(u2r, yr, -u2i * yi)));
			T im = fmaf(u1r, xi, fmaf(u1i, xr, fmaf(u2r, yi, u2i * yr)));
			if (k == 0 || k == 4)
			{
				re += u0r;
				im += u0i;
			}
			r.v[2 * k] = re;
			r.v[2 * k + 1] = im;
		}
		return r;
	}
	// exp(t X) for X = from_alg(o) (antihermitian traceless), Cayley-Hamilton
	MESH_HD static E exp_alg(T const *o, T t)
	{
		T x[8];
#pragma unroll
		for (int k = 0; k < 8; ++k)
			x[k] = o[k] * t;
		E X = from_alg(x);
		E X2 = sq_ah(X);
		// c1 = Tr(Q^2)/2 = |X|^2/2,  c0 = det(Q) = det(-iX) = -Im det(X)
		T c1 = T(0.5) * kin(x);
		T c0 = -det(X).im;
		if constexpr (sizeof(T) == 4)
		{
			// |X|^2 = 2 c1: |X| < 0.2 (a molecular-dynamics step) or < 1
			if (c1 < T(0.02))
				return exp_series<6>(X, X2, c1, -c0);
			if (c1 < T(0.5))
				return exp_series<10>(X, X2, c1, -c0);
		}
		cx<T> f0, f1, f2;
		T const tiny = sizeof(T) == 8 ? T(1e-11) : T(1e-5);
		if (c1 < tiny)
		{
			// exp(X) = 1 + X + X^2/2 + X^3/6; with X^3 = -i Q^3 and
			// Q^3 = c1 Q + c0: 1 + X + X^2/2 - i (c1 Q + c0)/6
			// -> f0 = 1 - i c0/6, f1 (on Q) = i - i c1/6, f2 (on Q^2) = -1/2
			f0 = {T(1), -c0 * T(1.0 / 6.0)};
			f1 = {T(0), T(1) - c1 * T(1.0 / 6.0)};
			f2 = {T(-0.5), T(0)};
		}
		else
		{
			bool neg = c0 < T(0);
			T c0a = neg ? -c0 : c0;
			T sq = m_sqrt(c1 * T(1.0 / 3.0));
			T c0max = T(2) * sq * sq * sq;
			T ratio = c0a / c0max;
			ratio = ratio > T(1) ? T(1) : ratio;
			T theta = acos(ratio);
			T st, ct;
			m_sincos(theta * T(1.0 / 3.0), &st, &ct);
			T u = sq * ct;
			T w = m_sqrt(c1) * st;
			T u2 = u * u, w2 = w * w;
			T s2u, c2u, su, cu, sw, cw;
			m_sincos(T(2) * u, &s2u, &c2u);
			m_sincos(u, &su, &cu);
			m_sincos(w, &sw, &cw);
			T xi0;
			if (w < T(0.05))
				xi0 = T(1) - w2 * T(1.0 / 6.0) * (T(1) - w2 * T(1.0 / 20.0) * (T(1) - w2 * T(1.0 / 42.0)));
			else
				xi0 = sw / w;
			cx<T> e2iu = {c2u, s2u};
			cx<T> emiu = {cu, -su};
			// h0 = (u^2 - w^2) e^{2iu} + e^{-iu} [8u^2 cos w + 2iu(3u^2 + w^2) xi0]
			cx<T> h0 = cadd(cscale(e2iu, u2 - w2),
			                cmul(emiu, cx<T>{T(8) * u2 * cw, T(2) * u * (T(3) * u2 + w2) * xi0}));
			// h1 = 2u e^{2iu} - e^{-iu} [2u cos w - i(3u^2 - w^2) xi0]
			cx<T> h1 = csub(cscale(e2iu, T(2) * u), cmul(emiu, cx<T>{T(2) * u * cw, -(T(3) * u2 - w2) * xi0}));
			// h2 = e^{2iu} - e^{-iu} [cos w + 3iu xi0]
			cx<T> h2 = csub(e2iu, cmul(emiu, cx<T>{cw, T(3) * u * xi0}));
			T inv = T(1) / (T(9) * u2 - w2);
			f0 = cscale(h0, inv);
			f1 = cscale(h1, inv);
			f2 = cscale(h2, inv);
			if (neg)
			{
				// f_j(-c0) = (-1)^j conj(f_j(c0))
				f0 = cconj(f0);
				f1 = {-f1.re, f1.im};
				f2 = cconj(f2);
			}
		}
		// exp(iQ) = f0 + f1 Q + f2 Q^2 with Q = -iX, Q^2 = -X^2:
		//         = f0 - i f1 X - f2 X^2
		cx<T> g1 = {f1.im, -f1.re}; // -i f1
		E r;
#pragma unroll
		for (int i = 0; i < 3; ++i)
#pragma unroll
			for (int j = 0; j < 3; ++j)
			{
				cx<T> z = csub(cmul(g1, X.at(i, j)), cmul(f2, X2.at(i, j)));
				if (i == j)
					z = cadd(z, f0);
				r.set(i, j, z);
			}
		return r;
	}
	// project_on_group_fast (groups.h:237-243):
	// r = 1.5 a - 0.5 a a^dagger a;  r (4/3 - det(r)/3)
	MESH_HD static E reunit_fast(E const &a)
	{
		E r;
		if constexpr (sizeof(T) == 4)
		{
			// FP32: the same r = a - (a a^dagger - 1) a / 2 with the deviation
			// a a^dagger - 1 accumulated from -1, so that no sum is rounded at
			// 1.0, where the float grid is twice as fine below as above and
			// rounding pulls the norms of nearly unitary rows down on average
			// (1.5 a - 0.5 (a a^dagger) a in FP32 leaves |det| 2e-8 above 1)
			E dev;
#pragma unroll
			for (int i = 0; i < 3; ++i)
#pragma unroll
				for (int j = 0; j < 3; ++j)
				{
					T re = i == j ? T(-1) : T(0), im = T(0);
#pragma unroll
					for (int k = 0; k < 3; ++k)
					{
						T ar = a.v[6 * i + 2 * k], ai = a.v[6 * i + 2 * k + 1];
						T br = a.v[6 * j + 2 * k], bi = a.v[6 * j + 2 * k + 1];
						re = fmaf(ar, br, fmaf(ai, bi, re));
						im = fmaf(ai, br, fmaf(-ar, bi, im));
					}
					dev.v[6 * i + 2 * j] = re;
					dev.v[6 * i + 2 * j + 1] = im;
				}
			E da = mul(dev, a);
#pragma unroll
			for (int k = 0; k < 18; ++k)
				r.v[k] = a.v[k] - da.v[k] * T(0.5);
		}
		else
		{
			E aa = mul_nd(a, a);
			E aaa = mul(aa, a);
#pragma unroll
			for (int k = 0; k < 18; ++k)
				r.v[k] = a.v[k] * T(1.5) - aaa.v[k] * T(0.5);
		}
		E o;
		if constexpr (sizeof(T) == 4)
		{
			// r (4/3 - det r / 3) = r + r g with g = -(det r - 1) / 3, det r - 1
			// accumulated from -1 (no quantity near 1.0 rounded)
			cx<T> A = csub(cmul(r.at(1, 1), r.at(2, 2)), cmul(r.at(1, 2), r.at(2, 1)));
			cx<T> B = csub(cmul(r.at(1, 0), r.at(2, 2)), cmul(r.at(1, 2), r.at(2, 0)));
			cx<T> Cc = csub(cmul(r.at(1, 0), r.at(2, 1)), cmul(r.at(1, 1), r.at(2, 0)));
			cx<T> t0 = cmul(r.at(0, 0), A), t1 = cmul(r.at(0, 1), B), t2 = cmul(r.at(0, 2), Cc);
			cx<T> dm1 = {((T(-1) + t0.re) - t1.re) + t2.re, (t0.im - t1.im) + t2.im};
			cx<T> g = {dm1.re * T(-1.0 / 3.0), dm1.im * T(-1.0 / 3.0)};
#pragma unroll
			for (int i = 0; i < 3; ++i)
#pragma unroll
				for (int j = 0; j < 3; ++j)
					o.set(i, j, cadd(r.at(i, j), cmul(r.at(i, j), g)));
		}
		else
		{
			cx<T> d = det(r);
			cx<T> f = {T(4.0 / 3.0) - d.re * T(1.0 / 3.0), -d.im * T(1.0 / 3.0)};
#pragma unroll
			for (int i = 0; i < 3; ++i)
#pragma unroll
				for (int j = 0; j < 3; ++j)
					o.set(i, j, cmul(r.at(i, j), f));
		}
		return o;
	}
	// proj of a special unitary matrix given by rows 0 and 1 only: the row-2
	// entries proj reads (a_20, a_21, Im a_22) from conj(row0 x row1)
	MESH_HD static void proj_rows01(E const &a, T *o)
	{
		cx<T> a20 = cconj(csub(cmul(a.at(0, 1), a.at(1, 2)), cmul(a.at(0, 2), a.at(1, 1))));
		cx<T> a21 = cconj(csub(cmul(a.at(0, 2), a.at(1, 0)), cmul(a.at(0, 0), a.at(1, 2))));
		// Im a_22 = -Im(a_00 a_11 - a_01 a_10)
		T im22 = -((a.v[0] * a.v[9] + a.v[1] * a.v[8]) - (a.v[2] * a.v[7] + a.v[3] * a.v[6]));
		T t = (a.v[1] + a.v[9] + im22) * T(1.0 / 3.0);
		o[0] = a.v[1] - t;
		o[1] = a.v[9] - t;
		o[2] = (a.v[2] - a.v[6]) * T(0.5);
		o[3] = (a.v[3] + a.v[7]) * T(0.5);
		o[4] = (a.v[4] - a20.re) * T(0.5);
		o[5] = (a.v[5] + a20.im) * T(0.5);
		o[6] = (a.v[10] - a21.re) * T(0.5);
		o[7] = (a.v[11] + a21.im) * T(0.5);
	}
	// row 2 of a special unitary matrix from rows 0 and 1: conj(row0 x row1)
	MESH_HD static void complete_row2(E &r)
	{
		if constexpr (sizeof(T) == 4)
		{
			// entry j = conj(a_0k a_1l - a_0l a_1k), (k, l) = (1, 2), (2, 0),
			// (0, 1): each real part one multiply and three fused multiply-adds
			auto entry = [&](int j, int k, int l) {
				T xr = r.v[2 * k], xi = r.v[2 * k + 1], yr = r.v[6 + 2 * l], yi = r.v[6 + 2 * l + 1];
				T ur = r.v[2 * l], ui = r.v[2 * l + 1], vr = r.v[6 + 2 * k], vi = r.v[6 + 2 * k + 1];
				// re(z) = xr yr - xi yi - ur vr + ui vi;  -im(z) = -xr yi - xi yr + ur vi + ui vr
				r.v[12 + 2 * j] = fmaf(xr, yr, fmaf(-xi, yi, fmaf(-ur, vr, ui * vi)));
				r.v[12 + 2 * j + 1] = fmaf(-xr, yi, fmaf(-xi, yr, fmaf(ur, vi, ui * vr)));
			};
			entry(0, 1, 2);
			entry(1, 2, 0);
			entry(2, 0, 1);
		}
		else
		{
			r.set(2, 0, cconj(csub(cmul(r.at(0, 1), r.at(1, 2)), cmul(r.at(0, 2), r.at(1, 1)))));
			r.set(2, 1, cconj(csub(cmul(r.at(0, 2), r.at(1, 0)), cmul(r.at(0, 0), r.at(1, 2)))));
			r.set(2, 2, cconj(csub(cmul(r.at(0, 0), r.at(1, 1)), cmul(r.at(0, 1), r.at(1, 0)))));
		}
	}
	// exact: Gram-Schmidt rows 0,1; row 2 = conj(row0 x row1)
	MESH_HD static E reunit_exact(E const &a)
	{
		E r;
		T n0 = 0;
#pragma unroll
		for (int k = 0; k < 6; ++k)
			n0 += a.v[k] * a.v[k];
		n0 = m_rsqrt(n0);
#pragma unroll
		for (int k = 0; k < 6; ++k)
			r.v[k] = a.v[k] * n0;
		cx<T> ip = {T(0), T(0)};
#pragma unroll
		for (int j = 0; j < 3; ++j)
			ip = cadd(ip, cmul(cconj(r.at(0, j)), a.at(1, j)));
#pragma unroll
		for (int j = 0; j < 3; ++j)
			r.set(1, j, csub(a.at(1, j), cmul(r.at(0, j), ip)));
		T n1 = 0;
#pragma unroll
		for (int k = 6; k < 12; ++k)
			n1 += r.v[k] * r.v[k];
		n1 = m_rsqrt(n1);
#pragma unroll
		for (int k = 6; k < 12; ++k)
			r.v[k] *= n1;
		r.set(2, 0, cconj(csub(cmul(r.at(0, 1), r.at(1, 2)), cmul(r.at(0, 2), r.at(1, 1)))));
		r.set(2, 1, cconj(csub(cmul(r.at(0, 2), r.at(1, 0)), cmul(r.at(0, 0), r.at(1, 2)))));
		r.set(2, 2, cconj(csub(cmul(r.at(0, 0), r.at(1, 1)), cmul(r.at(0, 1), r.at(1, 0)))));
		return r;
	}
	// Gaussian algebra element: i/2 sum_a p_a lambda_a (Gell-Mann)
	MESH_HD static void alg_from_normals(T const *p, T *o)
	{
		T const r3 = T(0.57735026918962576451);
		o[0] = T(0.5) * (p[2] + p[7] * r3);
		o[1] = T(0.5) * (-p[2] + p[7] * r3);
		o[2] = T(0.5) * p[1];
		o[3] = T(0.5) * p[0];
		o[4] = T(0.5) * p[4];
		o[5] = T(0.5) * p[3];
		o[6] = T(0.5) * p[6];
		o[7] = T(0.5) * p[5];
	}
	// Haar element: Gram-Schmidt of a complex normal matrix, row 0 divided
	// by the determinant (groups.h:255-261)
	MESH_HD static E group_from_normals(T const *p)
	{
		E r;
#pragma unroll
		for (int k = 0; k < 18; ++k)
			r.v[k] = p[k];
#pragma unroll
		for (int i = 0; i < 3; ++i)
		{
#pragma unroll
			for (int k = 0; k < i; ++k)
			{
				cx<T> ip = {T(0), T(0)};
#pragma unroll
				for (int j = 0; j < 3; ++j)
					ip = cadd(ip, cmul(cconj(r.at(k, j)), r.at(i, j)));
#pragma unroll
				for (int j = 0; j < 3; ++j)
					r.set(i, j, csub(r.at(i, j), cmul(r.at(k, j), ip)));
			}
			T n = 0;
#pragma unroll
			for (int j = 0; j < 6; ++j)
				n += r.v[6 * i + j] * r.v[6 * i + j];
			n = T(1) / m_sqrt(n);
#pragma unroll
			for (int j = 0; j < 6; ++j)
				r.v[6 * i + j] *= n;
		}
		cx<T> d = det(r);
		T dn = T(1) / (d.re * d.re + d.im * d.im);
		cx<T> inv = {d.re * dn, -d.im * dn};
#pragma unroll
		for (int j = 0; j < 3; ++j)
			r.set(0, j, cmul(r.at(0, j), inv));
		return r;
	}
};

// ---------------------------------------------------------------------------
// SU(3) float products on the packed FP32x2 FMA (fma.rn.f32x2, sm_100+): a
// complex multiply-accumulate c += a b is two packed FMAs,
//   (cr, ci) += (ar, ai) * (br, br);  (cr, ci) += (-ai, ar) * (bi, bi),
// halving the FMA instruction count of the 3x3 products.
// ---------------------------------------------------------------------------
struct Su3F2
{
	using E = Group<SU3, float>::E;
	__device__ __forceinline__ static unsigned long long pk(float a, float b)
	{
		unsigned long long r;
		asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(a), "f"(b));
		return r;
	}
	__device__ __forceinline__ static void upk(unsigned long long r, float &a, float &b)
	{
		asm("mov.b64 {%0, %1}, %2;" : "=f"(a), "=f"(b) : "l"(r));
	}
	__device__ __forceinline__ static unsigned long long fma2(unsigned long long a, unsigned long long b,
	                                                          unsigned long long c)
	{
		unsigned long long d;
		asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(d) : "l"(a), "l"(b), "l"(c));
		return d;
	}
	// generic product with operand access functors: c_ij = sum_k A(i,k) B(k,j)
	// for the rows i < NRW, where A(i,k) = (ar, ai) and B(k,j) = (br, bi):
	//   (cr, ci) += (ar, ai) * (br, br) + (-ai, ar) * (bi, bi)
	// (pairing the other way round, broadcast parts of A against (re, im)
	// pairs of B, measured slower)
	template <int NRW, class FA, class FB> __device__ __forceinline__ static E prod(FA fa, FB fb)
	{
		return prod_add<NRW, false>(E{}, fa, fb);
	}
	// c0 + a b (ADD) or a b, rows i < NRW: the sums start from c0's entries
	template <int NRW, bool ADD, class FA, class FB>
	__device__ __forceinline__ static E prod_add(E const &c0, FA fa, FB fb)
	{
		E r;
#pragma unroll
		for (int i = 0; i < NRW; ++i)
		{
			unsigned long long an[3], ar[3];
#pragma unroll
			for (int k = 0; k < 3; ++k)
			{
				float re, im;
				fa(i, k, re, im);
				an[k] = pk(re, im);
				ar[k] = pk(-im, re);
			}
#pragma unroll
			for (int j = 0; j < 3; ++j)
			{
				unsigned long long acc = ADD ? pk(c0.v[6 * i + 2 * j], c0.v[6 * i + 2 * j + 1]) : 0ull;
#pragma unroll
				for (int k = 0; k < 3; ++k)
				{
					float re, im;
					fb(k, j, re, im);
					acc = fma2(an[k], pk(re, re), acc);
					acc = fma2(ar[k], pk(im, im), acc);
				}
				upk(acc, r.v[6 * i + 2 * j], r.v[6 * i + 2 * j + 1]);
			}
		}
		return r;
	}
	template <int NRW = 3> __device__ __forceinline__ static E mul(E const &a, E const &b)
	{
		return prod<NRW>(
		    [&](int i, int k, float &re, float &im) { re = a.v[6 * i + 2 * k]; im = a.v[6 * i + 2 * k + 1]; },
		    [&](int k, int j, float &re, float &im) { re = b.v[6 * k + 2 * j]; im = b.v[6 * k + 2 * j + 1]; });
	}
	// a b^dagger: B(k,j) = conj(b_jk) (rows 0 .. NRW-1)
	template <int NRW = 3> __device__ __forceinline__ static E mul_nd(E const &a, E const &b)
	{
		return prod<NRW>(
		    [&](int i, int k, float &re, float &im) { re = a.v[6 * i + 2 * k]; im = a.v[6 * i + 2 * k + 1]; },
		    [&](int k, int j, float &re, float &im) { re = b.v[6 * j + 2 * k]; im = -b.v[6 * j + 2 * k + 1]; });
	}
	// s + a^dagger b
	__device__ __forceinline__ static E add_dn(E const &s, E const &a, E const &b)
	{
		return prod_add<3, true>(
		    s, [&](int i, int k, float &re, float &im) { re = a.v[6 * k + 2 * i]; im = -a.v[6 * k + 2 * i + 1]; },
		    [&](int k, int j, float &re, float &im) { re = b.v[6 * k + 2 * j]; im = b.v[6 * k + 2 * j + 1]; });
	}
	// a^dagger b: A(i,k) = conj(a_ki)
	__device__ __forceinline__ static E mul_dn(E const &a, E const &b)
	{
		return prod<3>(
		    [&](int i, int k, float &re, float &im) { re = a.v[6 * k + 2 * i]; im = -a.v[6 * k + 2 * i + 1]; },
		    [&](int k, int j, float &re, float &im) { re = b.v[6 * k + 2 * j]; im = b.v[6 * k + 2 * j + 1]; });
	}
};


} // namespace meshgb
