// TEST INFRASTRUCTURE — NOT PART OF THE PRODUCT.
//
// CPU oracle: a plain C++ restatement of krox/mesh's lattice-gauge hot path,
// used only by tests/, __graft_entry__.smoke() and bench.py's CPU legs as the
// checker. The product (mesh_gb300/) never includes, links or calls this.
//
// It follows the reference's data layout (lexicographic site order, dim 0
// slowest, one array-of-structs buffer per direction mu; src/lattice/grid.h:39-49,
// src/lattice/lattice.h:159-192) and its algorithms op for op:
//   group element math ........ src/gauge/groups.h:33-268
//   cshift ..................... src/lattice/lattice.h:366-389, device.h:55-110
//   reductions ................. src/lattice/device.h:185-212,246-265
//                                (256-wide pairwise tree per block, serial
//                                combine of the block partials, in the
//                                object's real type)
//   plaquette/staples/force .... src/gauge/utils.h:80-153
//   evolve/runHmd/makeDeltas ... src/gauge/hmc.h:26-59, hmc.cpp:7-51
//   runHmcUpdate ............... src/gauge/hmc.cpp:74-106
//   Landau functional/CG ....... src/gauge/landau.h:23-136
// Items with no reference counterpart (checkerboard overrelaxation, Fourier
// acceleration, counter-based RNG) are written from the published methods
// named where they are defined.
//
// The reference's arithmetic library (krox/util @ de3e57e3b98d1bd9954c1aae5d6cd2d8f7f97e21,
// fetched by CPM in CMakeLists.txt:19-24) is not available, so complex,
// quaternion (Hamilton product) and 3x3 matrix arithmetic, util::exp (here:
// Taylor series with scaling and squaring) and the random-number generators are
// restated from their mathematical definitions.
//
// Pinning: the restatement is checked against the reference's own templates
// (groups.h, utils.h, hmc.h, hmc.cpp, lattice.h, grid.h) compiled in place with
// a project-written util shim (oracle/ref_shim, recipe in oracle/Makefile), and
// against the identities the reference's test prints (tests/lattice_gauge.cpp).
#pragma once

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <stdexcept>
#include <string>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

namespace oracle {

// --------------------------------------------------------------------------
// scalar types
// --------------------------------------------------------------------------

template <class T> struct cplx
{
	T re, im;
};
template <class T> inline cplx<T> operator+(cplx<T> a, cplx<T> b) { return {a.re + b.re, a.im + b.im}; }
template <class T> inline cplx<T> operator-(cplx<T> a, cplx<T> b) { return {a.re - b.re, a.im - b.im}; }
template <class T> inline cplx<T> operator-(cplx<T> a) { return {-a.re, -a.im}; }
template <class T> inline cplx<T> operator*(cplx<T> a, cplx<T> b)
{
	return {a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re};
}
template <class T> inline cplx<T> operator*(cplx<T> a, T s) { return {a.re * s, a.im * s}; }
template <class T> inline cplx<T> conj(cplx<T> a) { return {a.re, -a.im}; }
template <class T> inline T norm2(cplx<T> a) { return a.re * a.re + a.im * a.im; }
template <class T> inline cplx<T> &operator+=(cplx<T> &a, cplx<T> b) { return a = a + b; }
template <class T> inline cplx<T> &operator-=(cplx<T> &a, cplx<T> b) { return a = a - b; }

// quaternion re + im1*I + im2*J + im3*K, Hamilton product (groups.h:114-133)
template <class T> struct quat
{
	T re, im1, im2, im3;
};
template <class T> inline quat<T> operator+(quat<T> a, quat<T> b)
{
	return {a.re + b.re, a.im1 + b.im1, a.im2 + b.im2, a.im3 + b.im3};
}
template <class T> inline quat<T> operator-(quat<T> a, quat<T> b)
{
	return {a.re - b.re, a.im1 - b.im1, a.im2 - b.im2, a.im3 - b.im3};
}
template <class T> inline quat<T> operator*(quat<T> a, quat<T> b)
{
	return {a.re * b.re - a.im1 * b.im1 - a.im2 * b.im2 - a.im3 * b.im3,
	        a.re * b.im1 + a.im1 * b.re + a.im2 * b.im3 - a.im3 * b.im2,
	        a.re * b.im2 - a.im1 * b.im3 + a.im2 * b.re + a.im3 * b.im1,
	        a.re * b.im3 + a.im1 * b.im2 - a.im2 * b.im1 + a.im3 * b.re};
}
template <class T> inline quat<T> operator*(quat<T> a, T s)
{
	return {a.re * s, a.im1 * s, a.im2 * s, a.im3 * s};
}
template <class T> inline quat<T> conj(quat<T> a) { return {a.re, -a.im1, -a.im2, -a.im3}; }
template <class T> inline quat<T> &operator+=(quat<T> &a, quat<T> b) { return a = a + b; }
template <class T> inline quat<T> &operator-=(quat<T> &a, quat<T> b) { return a = a - b; }

// 3x3 complex matrix, row-major
template <class T> struct mat3
{
	cplx<T> m[3][3];
};
template <class T> inline mat3<T> operator+(mat3<T> const &a, mat3<T> const &b)
{
	mat3<T> r;
	for (int i = 0; i < 3; ++i)
		for (int j = 0; j < 3; ++j)
			r.m[i][j] = a.m[i][j] + b.m[i][j];
	return r;
}
template <class T> inline mat3<T> operator-(mat3<T> const &a, mat3<T> const &b)
{
	mat3<T> r;
	for (int i = 0; i < 3; ++i)
		for (int j = 0; j < 3; ++j)
			r.m[i][j] = a.m[i][j] - b.m[i][j];
	return r;
}
template <class T> inline mat3<T> operator*(mat3<T> const &a, mat3<T> const &b)
{
	mat3<T> r;
	for (int i = 0; i < 3; ++i)
		for (int j = 0; j < 3; ++j)
		{
			cplx<T> s = a.m[i][0] * b.m[0][j];
			s += a.m[i][1] * b.m[1][j];
			s += a.m[i][2] * b.m[2][j];
			r.m[i][j] = s;
		}
	return r;
}
template <class T> inline mat3<T> operator*(mat3<T> const &a, T s)
{
	mat3<T> r;
	for (int i = 0; i < 3; ++i)
		for (int j = 0; j < 3; ++j)
			r.m[i][j] = a.m[i][j] * s;
	return r;
}
template <class T> inline mat3<T> operator*(mat3<T> const &a, cplx<T> s)
{
	mat3<T> r;
	for (int i = 0; i < 3; ++i)
		for (int j = 0; j < 3; ++j)
			r.m[i][j] = a.m[i][j] * s;
	return r;
}
template <class T> inline mat3<T> &operator+=(mat3<T> &a, mat3<T> const &b) { return a = a + b; }
template <class T> inline mat3<T> &operator-=(mat3<T> &a, mat3<T> const &b) { return a = a - b; }
template <class T> inline mat3<T> adjm(mat3<T> const &a)
{
	mat3<T> r;
	for (int i = 0; i < 3; ++i)
		for (int j = 0; j < 3; ++j)
			r.m[i][j] = conj(a.m[j][i]);
	return r;
}
template <class T> inline mat3<T> unit3()
{
	mat3<T> r;
	for (int i = 0; i < 3; ++i)
		for (int j = 0; j < 3; ++j)
			r.m[i][j] = {T(i == j), T(0)};
	return r;
}
template <class T> inline cplx<T> trace(mat3<T> const &a)
{
	return a.m[0][0] + a.m[1][1] + a.m[2][2];
}
template <class T> inline cplx<T> determinant(mat3<T> const &a)
{
	auto const &m = a.m;
	return m[0][0] * (m[1][1] * m[2][2] - m[1][2] * m[2][1]) -
	       m[0][1] * (m[1][0] * m[2][2] - m[1][2] * m[2][0]) +
	       m[0][2] * (m[1][0] * m[2][1] - m[1][1] * m[2][0]);
}
template <class T> inline T norm2(mat3<T> const &a)
{
	T s = 0;
	for (int i = 0; i < 3; ++i)
		for (int j = 0; j < 3; ++j)
			s += norm2(a.m[i][j]);
	return s;
}
template <class T> inline T norm1(mat3<T> const &a)
{
	// maximum absolute column sum
	T best = 0;
	for (int j = 0; j < 3; ++j)
	{
		T s = 0;
		for (int i = 0; i < 3; ++i)
			s += std::sqrt(norm2(a.m[i][j]));
		best = std::max(best, s);
	}
	return best;
}

// --------------------------------------------------------------------------
// gauge groups (groups.h). Group element types:
//   U1  -> cplx<T>   SU2 -> quat<T>   SU3 -> mat3<T>
// --------------------------------------------------------------------------

template <class G> struct traits;
template <class T> struct traits<cplx<T>>
{
	using real = T;
	static constexpr int Nc = 1, dim = 1, nreal = 2, nalg = 1;
};
template <class T> struct traits<quat<T>>
{
	using real = T;
	static constexpr int Nc = 2, dim = 3, nreal = 4, nalg = 3;
};
template <class T> struct traits<mat3<T>>
{
	using real = T;
	static constexpr int Nc = 3, dim = 8, nreal = 18, nalg = 8;
};

template <class G> inline G unit();
template <> inline cplx<float> unit() { return {1, 0}; }
template <> inline cplx<double> unit() { return {1, 0}; }
template <> inline quat<float> unit() { return {1, 0, 0, 0}; }
template <> inline quat<double> unit() { return {1, 0, 0, 0}; }
template <> inline mat3<float> unit() { return unit3<float>(); }
template <> inline mat3<double> unit() { return unit3<double>(); }

template <class G> inline G zero()
{
	G r;
	std::memset(&r, 0, sizeof(G));
	return r;
}

// adj (groups.h:55,135,214)
template <class T> inline cplx<T> adj(cplx<T> a) { return conj(a); }
template <class T> inline quat<T> adj(quat<T> a) { return conj(a); }
template <class T> inline mat3<T> adj(mat3<T> const &a) { return adjm(a); }

// real_trace (groups.h:59,137-140,219-222)
template <class T> inline T real_trace(cplx<T> a) { return a.re; }
template <class T> inline T real_trace(quat<T> a) { return a.re * T(2.0); }
template <class T> inline T real_trace(mat3<T> const &a) { return trace(a).re; }

// project_on_algebra (groups.h:64-67,142-145,224-228)
template <class T> inline cplx<T> project_on_algebra(cplx<T> a) { return {T(0), a.im}; }
template <class T> inline quat<T> project_on_algebra(quat<T> a) { return {T(0), a.im1, a.im2, a.im3}; }
template <class T> inline mat3<T> project_on_algebra(mat3<T> const &a)
{
	// antihermitian_traceless: (a - a^dagger)/2 minus the trace part
	mat3<T> r;
	for (int i = 0; i < 3; ++i)
		for (int j = 0; j < 3; ++j)
			r.m[i][j] = (a.m[i][j] - conj(a.m[j][i])) * T(0.5);
	cplx<T> tr = trace(r) * T(1.0 / 3.0);
	for (int i = 0; i < 3; ++i)
		r.m[i][i] -= tr;
	return r;
}

// kinetic-energy norm of an algebra element: the Frobenius norm of the
// defining representation, sum_ij |a_ij|^2. For U(1) and SU(3) this is
// util's norm2 on the object. For SU(2) as a quaternion the 2x2 matrix norm
// is 2|q|^2; this is the only normalisation under which the momentum
// distribution (groups.h:166-176), the force (utils.h:148-153) and
// H = S + norm2(P) (hmc.cpp:85) conserve H along the trajectory, and under
// which the identity printed at tests/lattice_gauge.cpp:23-25 equals 1.
template <class T> inline T alg_norm2(cplx<T> a) { return norm2(a); }
template <class T> inline T alg_norm2(quat<T> a)
{
	return T(2) * (a.re * a.re + a.im1 * a.im1 + a.im2 * a.im2 + a.im3 * a.im3);
}
template <class T> inline T alg_norm2(mat3<T> const &a) { return norm2(a); }

// project_on_group_fast (groups.h:79-83,188-192,237-243). For the
// quaternion the quaternion norm |q|^2 is used (the linearised 1/sqrt(|q|^2)).
template <class T> inline cplx<T> project_on_group_fast(cplx<T> a)
{
	return a * (T(1.5) - norm2(a) * T(0.5));
}
template <class T> inline quat<T> project_on_group_fast(quat<T> a)
{
	T n = a.re * a.re + a.im1 * a.im1 + a.im2 * a.im2 + a.im3 * a.im3;
	return a * (T(1.5) - n * T(0.5));
}
template <class T> inline mat3<T> project_on_group_fast(mat3<T> const &a)
{
	mat3<T> r = a * T(1.5) - a * adjm(a) * a * T(0.5);
	cplx<T> d = determinant(r);
	cplx<T> f = {T(4.0 / 3.0) - d.re * T(1.0 / 3.0), -d.im * T(1.0 / 3.0)};
	return r * f;
}

// exact projection onto the group (used for the gauge transforms of the
// gauge-fixing code, which are applied many times): U(1)/SU(2) normalise,
// SU(3) Gram-Schmidt on the first two rows and the third row as the
// conjugated cross product.
template <class T> inline cplx<T> project_on_group_exact(cplx<T> a)
{
	T n = std::sqrt(norm2(a));
	return a * (T(1) / n);
}
template <class T> inline quat<T> project_on_group_exact(quat<T> a)
{
	T n = std::sqrt(a.re * a.re + a.im1 * a.im1 + a.im2 * a.im2 + a.im3 * a.im3);
	return a * (T(1) / n);
}
template <class T> inline mat3<T> project_on_group_exact(mat3<T> const &a)
{
	mat3<T> r;
	T n0 = 0;
	for (int j = 0; j < 3; ++j)
		n0 += norm2(a.m[0][j]);
	n0 = T(1) / std::sqrt(n0);
	for (int j = 0; j < 3; ++j)
		r.m[0][j] = a.m[0][j] * n0;
	cplx<T> ip = {T(0), T(0)};
	for (int j = 0; j < 3; ++j)
		ip += conj(r.m[0][j]) * a.m[1][j];
	for (int j = 0; j < 3; ++j)
		r.m[1][j] = a.m[1][j] - r.m[0][j] * ip;
	T n1 = 0;
	for (int j = 0; j < 3; ++j)
		n1 += norm2(r.m[1][j]);
	n1 = T(1) / std::sqrt(n1);
	for (int j = 0; j < 3; ++j)
		r.m[1][j] = r.m[1][j] * n1;
	r.m[2][0] = conj(r.m[0][1] * r.m[1][2] - r.m[0][2] * r.m[1][1]);
	r.m[2][1] = conj(r.m[0][2] * r.m[1][0] - r.m[0][0] * r.m[1][2]);
	r.m[2][2] = conj(r.m[0][0] * r.m[1][1] - r.m[0][1] * r.m[1][0]);
	return r;
}

// exp: algebra -> group (groups.h:103-108,153-164,263-268)
template <class T> inline cplx<T> gexp(cplx<T> a) { return {std::cos(a.im), std::sin(a.im)}; }
template <class T> inline quat<T> gexp(quat<T> a)
{
	T alpha = std::sqrt(a.im1 * a.im1 + a.im2 * a.im2 + a.im3 * a.im3);
	// groups.h:161-163 divides sin(alpha)/alpha (NaN at alpha == 0); the
	// limit value 1 is used there instead.
	T f = alpha == T(0) ? T(1) : std::sin(alpha) / alpha;
	return {std::cos(alpha), a.im1 * f, a.im2 * f, a.im3 * f};
}
// matrix exponential (util::exp, absent): scaling and squaring with a
// Taylor polynomial evaluated by Horner's rule (Moler & Van Loan, "Nineteen
// dubious ways", method 3). ||X/2^s||_1 <= 1/2 and K terms give a truncation
// error below 0.5^(K+1)/(K+1)!.
template <class T> inline mat3<T> gexp(mat3<T> const &a)
{
	constexpr int K = sizeof(T) == 8 ? 18 : 10;
	T n = norm1(a);
	int s = 0;
	while (n > T(0.5))
	{
		n *= T(0.5);
		++s;
	}
	T scale = std::ldexp(T(1), -s);
	mat3<T> x = a * scale;
	mat3<T> e = unit3<T>();
	for (int k = K; k >= 1; --k)
		e = unit3<T>() + (x * e) * (T(1) / T(k));
	for (int i = 0; i < s; ++i)
		e = e * e;
	return e;
}

// --------------------------------------------------------------------------
// algebra packing shared with the device representation of momenta:
//   U(1):  1 real  a           <-> (0, a)
//   SU(2): 3 reals (v1,v2,v3)  <-> (0, v1, v2, v3)
//   SU(3): 8 reals (a0, a1, Re b01, Im b01, Re b02, Im b02, Re b12, Im b12)
//          <-> [[i a0, b01, b02], [-b01*, i a1, b12], [-b02*, -b12*, -i(a0+a1)]]
// --------------------------------------------------------------------------
template <class T> inline void pack_alg(cplx<T> a, T *o) { o[0] = a.im; }
template <class T> inline void pack_alg(quat<T> a, T *o)
{
	o[0] = a.im1;
	o[1] = a.im2;
	o[2] = a.im3;
}
template <class T> inline void pack_alg(mat3<T> const &a, T *o)
{
	o[0] = a.m[0][0].im;
	o[1] = a.m[1][1].im;
	o[2] = a.m[0][1].re;
	o[3] = a.m[0][1].im;
	o[4] = a.m[0][2].re;
	o[5] = a.m[0][2].im;
	o[6] = a.m[1][2].re;
	o[7] = a.m[1][2].im;
}
template <class T> inline void unpack_alg(T const *o, cplx<T> &a) { a = {T(0), o[0]}; }
template <class T> inline void unpack_alg(T const *o, quat<T> &a) { a = {T(0), o[0], o[1], o[2]}; }
template <class T> inline void unpack_alg(T const *o, mat3<T> &a)
{
	a.m[0][0] = {T(0), o[0]};
	a.m[1][1] = {T(0), o[1]};
	a.m[2][2] = {T(0), -(o[0] + o[1])};
	a.m[0][1] = {o[2], o[3]};
	a.m[0][2] = {o[4], o[5]};
	a.m[1][2] = {o[6], o[7]};
	a.m[1][0] = {-o[2], o[3]};
	a.m[2][0] = {-o[4], o[5]};
	a.m[2][1] = {-o[6], o[7]};
}

// --------------------------------------------------------------------------
// Philox4x32-10 counter-based generator (Salmon, Moraes, Dror, Shaw,
// "Parallel random numbers: as easy as 1, 2, 3", SC'11), restated from the
// paper. Used for momenta, hot starts, Haar-random gauge transforms and the
// Metropolis uniform, with the stream layout the device uses:
//   key = (seed & 0xffffffff, seed >> 32)
//   ctr = (lexicographic site, tag << 24 | mu << 8 | block, n & 0xffffffff, n >> 32)
// --------------------------------------------------------------------------
struct philox_out
{
	uint32_t v[4];
};
inline philox_out philox4x32_10(uint32_t c0, uint32_t c1, uint32_t c2, uint32_t c3, uint32_t k0,
                                uint32_t k1)
{
	for (int r = 0; r < 10; ++r)
	{
		uint64_t p0 = uint64_t(0xD2511F53u) * c0;
		uint64_t p1 = uint64_t(0xCD9E8D57u) * c2;
		uint32_t hi0 = uint32_t(p0 >> 32), lo0 = uint32_t(p0);
		uint32_t hi1 = uint32_t(p1 >> 32), lo1 = uint32_t(p1);
		uint32_t n0 = hi1 ^ c1 ^ k0;
		uint32_t n2 = hi0 ^ c3 ^ k1;
		c0 = n0;
		c1 = lo1;
		c2 = n2;
		c3 = lo0;
		k0 += 0x9E3779B9u;
		k1 += 0xBB67AE85u;
	}
	return {{c0, c1, c2, c3}};
}

enum : uint32_t
{
	TAG_MOMENTUM = 1,
	TAG_GAUGE = 2,
	TAG_METROPOLIS = 3,
	TAG_TRANSFORM = 4,
};

// uniforms in the open interval (0,1)
inline float u24(uint32_t x) { return (float(x >> 8) + 0.5f) * (1.0f / 16777216.0f); }
inline double u53(uint32_t a, uint32_t b)
{
	uint64_t m = (uint64_t(a) << 21) ^ uint64_t(b >> 11);
	return (double(m) + 0.5) * (1.0 / 9007199254740992.0);
}

// n standard normals (n <= 18) for (site, mu) under a tag, by Box-Muller on
// pairs of uniforms in the precision T.
template <class T>
inline void normals(uint64_t seed, uint32_t tag, uint32_t site, uint32_t mu, uint64_t n_ctr, int n,
                    T *out)
{
	uint32_t k0 = uint32_t(seed), k1 = uint32_t(seed >> 32);
	uint32_t c2 = uint32_t(n_ctr), c3 = uint32_t(n_ctr >> 32);
	if constexpr (sizeof(T) == 4)
	{
		// 4 uniforms per Philox call -> 4 normals
		for (int blk = 0; 4 * blk < n; ++blk)
		{
			auto r = philox4x32_10(site, (tag << 24) | (mu << 8) | uint32_t(blk), c2, c3, k0, k1);
			for (int h = 0; h < 2; ++h)
			{
				float ua = u24(r.v[2 * h]), ub = u24(r.v[2 * h + 1]);
				float rad = std::sqrt(-2.0f * std::log(ua));
				float s = std::sin(float(2.0 * M_PI) * ub), c = std::cos(float(2.0 * M_PI) * ub);
				int i = 4 * blk + 2 * h;
				if (i < n)
					out[i] = rad * c;
				if (i + 1 < n)
					out[i + 1] = rad * s;
			}
		}
	}
	else
	{
		// 2 uniforms (53 bit) per Philox call -> 2 normals
		for (int blk = 0; 2 * blk < n; ++blk)
		{
			auto r = philox4x32_10(site, (tag << 24) | (mu << 8) | uint32_t(blk), c2, c3, k0, k1);
			double ua = u53(r.v[0], r.v[1]), ub = u53(r.v[2], r.v[3]);
			double rad = std::sqrt(-2.0 * std::log(ua));
			double s = std::sin(2.0 * M_PI * ub), c = std::cos(2.0 * M_PI * ub);
			int i = 2 * blk;
			if (i < n)
				out[i] = rad * c;
			if (i + 1 < n)
				out[i + 1] = rad * s;
		}
	}
}

inline double metropolis_uniform(uint64_t seed, uint64_t traj)
{
	auto r = philox4x32_10(0u, TAG_METROPOLIS << 24, uint32_t(traj), uint32_t(traj >> 32),
	                       uint32_t(seed), uint32_t(seed >> 32));
	return u53(r.v[0], r.v[1]);
}

// Gaussian algebra element with tr(T^a T^b) = delta^ab / 2 and unit-variance
// coefficients (groups.h:86-91,166-176,245-253): same distribution as the
// reference's generators, built from dim independent normals.
template <class T> inline void alg_from_normals(T const *p, cplx<T> &a)
{
	a = {T(0), p[0] * T(M_SQRT1_2)};
}
template <class T> inline void alg_from_normals(T const *p, quat<T> &a)
{
	a = {T(0), T(0.5) * p[0], T(0.5) * p[1], T(0.5) * p[2]};
}
template <class T> inline void alg_from_normals(T const *p, mat3<T> &a)
{
	// i/2 * sum_a p_a lambda_a (Gell-Mann matrices)
	T const r3 = T(0.57735026918962576451); // 1/sqrt(3)
	T o[8];
	o[0] = T(0.5) * (p[2] + p[7] * r3);
	o[1] = T(0.5) * (-p[2] + p[7] * r3);
	o[2] = T(0.5) * p[1];
	o[3] = T(0.5) * p[0];
	o[4] = T(0.5) * p[4];
	o[5] = T(0.5) * p[3];
	o[6] = T(0.5) * p[6];
	o[7] = T(0.5) * p[5];
	unpack_alg(o, a);
}

// uniform (Haar) group element from normals (groups.h:94-100,178-186,255-261)
template <class T> inline void group_from_normals(T const *p, cplx<T> &a)
{
	// angle from the Box-Muller pair direction: atan2 of two normals is uniform
	T t = std::atan2(p[1], p[0]);
	a = {std::cos(t), std::sin(t)};
}
template <class T> inline void group_from_normals(T const *p, quat<T> &a)
{
	quat<T> q = {p[0], p[1], p[2], p[3]};
	a = project_on_group_exact(q);
}
template <class T> inline void group_from_normals(T const *p, mat3<T> &a)
{
	mat3<T> m;
	for (int i = 0; i < 3; ++i)
		for (int j = 0; j < 3; ++j)
			m.m[i][j] = {p[6 * i + 2 * j], p[6 * i + 2 * j + 1]};
	// Gram-Schmidt on the rows, then divide row 0 by the determinant
	mat3<T> r;
	for (int i = 0; i < 3; ++i)
	{
		for (int j = 0; j < 3; ++j)
			r.m[i][j] = m.m[i][j];
		for (int k = 0; k < i; ++k)
		{
			cplx<T> ip = {T(0), T(0)};
			for (int j = 0; j < 3; ++j)
				ip += conj(r.m[k][j]) * r.m[i][j];
			for (int j = 0; j < 3; ++j)
				r.m[i][j] -= r.m[k][j] * ip;
		}
		T n = 0;
		for (int j = 0; j < 3; ++j)
			n += norm2(r.m[i][j]);
		n = T(1) / std::sqrt(n);
		for (int j = 0; j < 3; ++j)
			r.m[i][j] = r.m[i][j] * n;
	}
	cplx<T> d = determinant(r);
	// r(0) /= det: multiply by conj(d)/|d|^2
	T dn = T(1) / norm2(d);
	cplx<T> inv = {d.re * dn, -d.im * dn};
	for (int j = 0; j < 3; ++j)
		r.m[0][j] = r.m[0][j] * inv;
	a = r;
}

// --------------------------------------------------------------------------
// grid (grid.h:11-58), lexicographic with dim 0 slowest
// --------------------------------------------------------------------------
struct Grid
{
	int nd = 0;
	int L[4] = {0, 0, 0, 0};
	size_t V = 0;
	Grid() = default;
	Grid(int nd_, int const *dims) : nd(nd_), V(1)
	{
		if (nd < 1 || nd > 4)
			throw std::runtime_error("grid dimension must be 1..4");
		for (int i = 0; i < nd; ++i)
		{
			L[i] = dims[i];
			if (L[i] <= 0)
				throw std::runtime_error("grid extents must be positive");
			V *= size_t(L[i]);
		}
	}
	size_t flat_index(int const *x) const
	{
		size_t r = 0;
		for (int i = 0; i < nd; ++i)
			r = r * size_t(L[i]) + size_t(x[i]);
		return r;
	}
	void coords(size_t r, int *x) const
	{
		for (int i = nd - 1; i >= 0; --i)
		{
			x[i] = int(r % size_t(L[i]));
			r /= size_t(L[i]);
		}
	}
	// even/odd (checkerboard) index used by the device layout: all even
	// sites first, each parity in lexicographic order.
	size_t eo_index(size_t r) const
	{
		int x[4];
		coords(r, x);
		int p = 0;
		for (int i = 0; i < nd; ++i)
			p += x[i];
		return size_t(p & 1) * (V / 2) + r / 2;
	}
	size_t shift(size_t r, int dir, int off) const
	{
		int x[4];
		coords(r, x);
		x[dir] = ((x[dir] + off) % L[dir] + L[dir]) % L[dir];
		return flat_index(x);
	}
};

// --------------------------------------------------------------------------
// lattice_apply layer (lattice.h:254-389) over host vectors
// --------------------------------------------------------------------------
template <class T> using Field = std::vector<T>;

template <class F> inline void site_loop(size_t n, F f)
{
#pragma omp parallel for schedule(static)
	for (long long i = 0; i < (long long)n; ++i)
		f(size_t(i));
}

// device_sum_apply_kernel (device.h:185-212) + host combine (device.h:259-264):
// blocks of 256, pairwise tree in shared memory, serial sum of block partials.
template <class R, class F> inline R tree_sum(size_t n, F f)
{
	constexpr size_t B = 256;
	size_t nb = (n + B - 1) / B;
	std::vector<R> part(nb);
#pragma omp parallel for schedule(static)
	for (long long b = 0; b < (long long)nb; ++b)
	{
		R s[B];
		for (size_t l = 0; l < B; ++l)
		{
			size_t g = size_t(b) * B + l;
			if (g < n)
				s[l] = f(g);
		}
		for (size_t stride = B / 2; stride > 0; stride /= 2)
			for (size_t l = 0; l < stride; ++l)
			{
				size_t g = size_t(b) * B + l;
				if (g + stride < n)
					s[l] += s[l + stride];
			}
		part[b] = s[0];
	}
	R r = part[0];
	for (size_t i = 1; i < nb; ++i)
		r += part[i];
	return r;
}

// cshift (lattice.h:366-389): dst[x] = src[x + offset * e_dir], periodic
template <class T> inline Field<T> cshift(Grid const &g, Field<T> const &a, int dir, int offset)
{
	size_t slow = 1, fast = 1;
	for (int i = 0; i < dir; ++i)
		slow *= size_t(g.L[i]);
	size_t s = size_t(g.L[dir]);
	for (int i = dir + 1; i < g.nd; ++i)
		fast *= size_t(g.L[i]);
	size_t width = s * fast;
	long long shift = (long long)offset * (long long)fast;
	Field<T> r(a.size());
#pragma omp parallel for schedule(static)
	for (long long row = 0; row < (long long)slow; ++row)
		for (size_t j = 0; j < width; ++j)
		{
			long long src = ((long long)j + shift) % (long long)width;
			if (src < 0)
				src += (long long)width;
			r[size_t(row) * width + j] = a[size_t(row) * width + size_t(src)];
		}
	return r;
}

template <class G> using GaugeField = std::vector<Field<G>>;

template <class G> inline Field<G> mul(Field<G> const &a, Field<G> const &b)
{
	Field<G> r(a.size());
	site_loop(a.size(), [&](size_t i) { r[i] = a[i] * b[i]; });
	return r;
}
template <class G> inline Field<G> adjf(Field<G> const &a)
{
	Field<G> r(a.size());
	site_loop(a.size(), [&](size_t i) { r[i] = adj(a[i]); });
	return r;
}
template <class G, class S> inline Field<G> scale(Field<G> const &a, S s)
{
	using T = typename traits<G>::real;
	Field<G> r(a.size());
	site_loop(a.size(), [&](size_t i) { r[i] = a[i] * T(s); });
	return r;
}
template <class G> inline Field<G> proj_alg(Field<G> const &a)
{
	Field<G> r(a.size());
	site_loop(a.size(), [&](size_t i) { r[i] = project_on_algebra(a[i]); });
	return r;
}
template <class G> inline Field<G> expf_(Field<G> const &a)
{
	Field<G> r(a.size());
	site_loop(a.size(), [&](size_t i) { r[i] = gexp(a[i]); });
	return r;
}
template <class G> inline typename traits<G>::real sum_real_trace(Field<G> const &a)
{
	using T = typename traits<G>::real;
	return tree_sum<T>(a.size(), [&](size_t i) { return real_trace(a[i]); });
}
template <class G> inline typename traits<G>::real norm2f(Field<G> const &a)
{
	using T = typename traits<G>::real;
	return tree_sum<T>(a.size(), [&](size_t i) { return alg_norm2(a[i]); });
}

// --------------------------------------------------------------------------
// gauge utilities (utils.h)
// --------------------------------------------------------------------------
template <class G> inline double norm2(GaugeField<G> const &P)
{
	double s = 0;
	for (auto const &p : P)
		s += norm2f(p);
	return s;
}

template <class G> inline void reunitize(Field<G> &U)
{
	site_loop(U.size(), [&](size_t i) { U[i] = project_on_group_fast(U[i]); });
}
template <class G> inline void reunitize(GaugeField<G> &U)
{
	for (auto &u : U)
		reunitize(u);
}

// plaquette (utils.h:94-108), normalised to [0,1]
template <class G> inline double plaquette(Grid const &g, GaugeField<G> const &U)
{
	double vol = double(g.V);
	double s = 0;
	int Nd = g.nd;
	for (int mu = 0; mu < Nd; ++mu)
		for (int nu = mu + 1; nu < Nd; ++nu)
		{
			auto a = cshift(g, U[nu], mu, 1);
			auto b = cshift(g, U[mu], nu, 1);
			auto tmp = mul(mul(mul(U[mu], a), adjf(b)), adjf(U[nu]));
			s += sum_real_trace(tmp);
		}
	return s / (vol * Nd * (Nd - 1) * 0.5) / traits<G>::Nc;
}

// stapleSum (utils.h:114-139), the "optimized" form op for op
template <class G> inline Field<G> stapleSum(Grid const &g, GaugeField<G> const &U, int mu)
{
	Field<G> S(g.V, zero<G>());
	int Nd = g.nd;
	for (int nu = 0; nu < Nd; ++nu)
	{
		if (nu == mu)
			continue;
		auto tmp = cshift(g, U[nu], mu, 1);
		auto c = cshift(g, U[mu], nu, 1);
		auto const &d = U[nu];
		site_loop(g.V, [&](size_t i) { S[i] += tmp[i] * adj(d[i] * c[i]); });
		auto const &um = U[mu];
		site_loop(g.V, [&](size_t i) { tmp[i] = adj(um[i] * tmp[i]) * d[i]; });
		auto sh = cshift(g, tmp, nu, -1);
		site_loop(g.V, [&](size_t i) { S[i] += sh[i]; });
	}
	return S;
}

template <class G> inline double wilsonAction(Grid const &g, GaugeField<G> const &U, double beta)
{
	int Nd = g.nd;
	double vol = double(g.V);
	return (1.0 - plaquette(g, U)) * (beta * Nd * (Nd - 1) * 0.5 * vol);
}

// wilsonDeriv (utils.h:148-153)
template <class G> inline Field<G> wilsonDeriv(Grid const &g, GaugeField<G> const &U, int mu, double beta)
{
	auto S = stapleSum(g, U, mu);
	return proj_alg(scale(mul(U[mu], S), beta / (2 * traits<G>::Nc)));
}

// --------------------------------------------------------------------------
// HMC (hmc.h, hmc.cpp)
// --------------------------------------------------------------------------
inline std::vector<double> makeDeltas(std::string const &scheme, double epsilon, int substeps)
{
	double delta = std::sqrt(2 * epsilon) / substeps;
	std::vector<double> raw;
	if (scheme == "2lf")
		raw = {0.5, 1.0, 0.5};
	else if (scheme == "2mn")
	{
		double lamb = 0.19318332750378361;
		raw = {lamb, 0.5, 1.0 - 2.0 * lamb, 0.5, lamb};
	}
	else if (scheme == "4mn")
	{
		double rho = 0.1786178958448091;
		double theta = -0.06626458266981843;
		double lamb = 0.7123418310626056;
		raw = {rho, lamb, theta, 0.5 - lamb, 1.0 - 2.0 * (rho + theta), 0.5 - lamb, theta, lamb, rho};
	}
	else
		throw std::runtime_error("unknown scheme '" + scheme + "'");
	std::vector<double> d;
	for (int i = 0; i < substeps; ++i)
	{
		if (i == 0)
			d.insert(d.end(), raw.begin(), raw.end());
		else
		{
			d.back() *= 2;
			d.insert(d.end(), raw.begin() + 1, raw.end());
		}
	}
	for (double &x : d)
		x *= delta;
	return d;
}

// evolve (hmc.h:26-36): U = exp(project_on_algebra(P) * t) * U
template <class G> inline void evolve(Field<G> &U, Field<G> const &P, double t)
{
	using T = typename traits<G>::real;
	site_loop(U.size(), [&](size_t i) { U[i] = gexp(project_on_algebra(P[i]) * T(t)) * U[i]; });
}

// runHmd (hmc.h:38-59)
template <class G>
inline void runHmd(Grid const &g, GaugeField<G> &U, GaugeField<G> &P, double beta,
                   std::vector<double> const &deltas)
{
	using T = typename traits<G>::real;
	int Nd = g.nd;
	for (size_t i = 0; i < deltas.size(); ++i)
		if (i % 2 == 0)
		{
			for (int mu = 0; mu < Nd; ++mu)
				evolve(U[mu], P[mu], deltas[i]);
		}
		else
		{
			for (int mu = 0; mu < Nd; ++mu)
			{
				auto F = scale(wilsonDeriv(g, U, mu, beta), deltas[i]);
				auto &p = P[mu];
				site_loop(g.V, [&](size_t k) { p[k] -= F[k]; });
			}
		}
	(void)sizeof(T);
}

struct HmcRecord
{
	double plaq, dH, accept, H_old, H_new;
};

// runHmcUpdate (hmc.cpp:73-107) with the momenta and the Metropolis
// uniform supplied by the caller instead of drawn from util::xoshiro256.
template <class G>
inline HmcRecord runHmcUpdate(Grid const &g, GaugeField<G> &U, GaugeField<G> const &P_in, double beta,
                              std::vector<double> const &deltas, double uniform)
{
	GaugeField<G> P = P_in;
	double H_old = wilsonAction(g, U, beta) + norm2(P);
	GaugeField<G> U_new = U;
	runHmd(g, U_new, P, beta, deltas);
	reunitize(U_new);
	double H_new = wilsonAction(g, U_new, beta) + norm2(P);
	double dH = H_new - H_old;
	HmcRecord rec;
	if (uniform < std::exp(-dH))
	{
		rec.accept = 1.0;
		std::swap(U, U_new);
	}
	else
		rec.accept = 0.0;
	rec.plaq = plaquette(g, U);
	rec.dH = dH;
	rec.H_old = H_old;
	rec.H_new = H_new;
	return rec;
}

// momenta from the counter-based stream (layout independent)
template <class G>
inline void random_momenta(Grid const &g, GaugeField<G> &P, uint64_t seed, uint64_t counter)
{
	using T = typename traits<G>::real;
	constexpr int dim = traits<G>::dim;
	for (int mu = 0; mu < g.nd; ++mu)
	{
		auto &p = P[mu];
		site_loop(g.V, [&](size_t r) {
			T n[8];
			normals<T>(seed, TAG_MOMENTUM, uint32_t(r), uint32_t(mu), counter, dim, n);
			alg_from_normals(n, p[r]);
		});
	}
}

template <class G> inline void random_gauge(Grid const &g, GaugeField<G> &U, uint64_t seed)
{
	using T = typename traits<G>::real;
	constexpr int nn = traits<G>::nreal;
	for (int mu = 0; mu < g.nd; ++mu)
	{
		auto &u = U[mu];
		site_loop(g.V, [&](size_t r) {
			T n[18];
			normals<T>(seed, TAG_GAUGE, uint32_t(r), uint32_t(mu), 0, nn, n);
			group_from_normals(n, u[r]);
		});
	}
}

template <class G> inline void random_transform(Grid const &g, Field<G> &h, uint64_t seed)
{
	using T = typename traits<G>::real;
	constexpr int nn = traits<G>::nreal;
	site_loop(g.V, [&](size_t r) {
		T n[18];
		normals<T>(seed, TAG_TRANSFORM, uint32_t(r), 0, 0, nn, n);
		group_from_normals(n, h[r]);
	});
}

// U^h_mu(x) = h(x) U_mu(x) h(x+mu)^dagger
template <class G> inline void gauge_transform(Grid const &g, GaugeField<G> &U, Field<G> const &h)
{
	for (int mu = 0; mu < g.nd; ++mu)
	{
		auto hs = cshift(g, h, mu, 1);
		auto &u = U[mu];
		site_loop(g.V, [&](size_t i) { u[i] = h[i] * u[i] * adj(hs[i]); });
	}
}

// --------------------------------------------------------------------------
// Landau gauge fixing (landau.h)
// --------------------------------------------------------------------------
template <class G> struct Landau
{
	Grid const &grid;
	GaugeField<G> const &U;
	Field<G> g;

	Landau(Grid const &gr, GaugeField<G> const &U_) : grid(gr), U(U_), g(gr.V, unit<G>()) {}

	// landau.h:23-32
	double functional(Field<G> const &h) const
	{
		int Nd = grid.nd;
		double vol = double(grid.V);
		double s = 0;
		for (int mu = 0; mu < Nd; ++mu)
			s += sum_real_trace(mul(mul(h, U[mu]), adjf(cshift(grid, h, mu, 1))));
		return s / (traits<G>::Nc * Nd * vol);
	}
	double functional() const { return functional(g); }

	Field<G> dfield() const
	{
		int Nd = grid.nd;
		Field<G> d(grid.V, zero<G>());
		for (int mu = 0; mu < Nd; ++mu)
		{
			auto a = mul(U[mu], adjf(cshift(grid, g, mu, 1)));
			site_loop(grid.V, [&](size_t i) { d[i] += a[i]; });
			auto b = adjf(cshift(grid, mul(g, U[mu]), mu, -1));
			site_loop(grid.V, [&](size_t i) { d[i] += b[i]; });
		}
		return d;
	}

	// landau.h:37-49 (theta_ref)
	double condition() const
	{
		int Nd = grid.nd;
		double vol = double(grid.V);
		auto d = dfield();
		return double(norm2f(proj_alg(mul(g, d)))) * (1.0 / (Nd * vol));
	}

	// landau.h:52-65
	Field<G> deriv() const
	{
		int Nd = grid.nd;
		double vol = double(grid.V);
		auto d = dfield();
		return scale(proj_alg(mul(g, d)), -0.5 / (traits<G>::Nc * Nd * vol));
	}

	static double solve_quadratic(double x1, double x2, double x3, double y1, double y2, double y3)
	{
		return 0.5 * ((x2 * x2 - x3 * x3) * y1 - (x1 * x1 - x3 * x3) * y2 + (x1 * x1 - x2 * x2) * y3) /
		       ((x2 - x3) * y1 - (x1 - x3) * y2 + (x1 - x2) * y3);
	}

	Field<G> stepped(Field<G> const &F, double eps) const { return mul(expf_(scale(F, eps)), g); }

	// landau.h:77-98
	double line_search(Field<G> const &F, double eps, int *n_evals) const
	{
		double base = functional();
		double y1 = functional(stepped(F, eps));
		++*n_evals;
		while (y1 <= base)
		{
			eps *= 0.5;
			y1 = functional(stepped(F, eps));
			++*n_evals;
			if (eps < 1e-10)
				return 0.0;
		}
		double y2 = functional(stepped(F, eps * 1.2));
		++*n_evals;
		if (y2 > y1)
			return 1.2 * eps;
		double y3 = functional(stepped(F, eps * 0.8));
		++*n_evals;
		return solve_quadratic(eps, 1.2 * eps, 0.8 * eps, y1, y2, y3);
	}

	// landau.h:100-136, with the stopping threshold as a parameter (the
	// reference hard-codes 1e-10). Returns the iteration count.
	int run(int max_iter, double tol, double *theta_out, int *n_evals)
	{
		double eps = 3000.0;
		Field<G> last(grid.V, zero<G>());
		double lastNorm = 0.0;
		*n_evals = 0;
		for (int iter = 0; iter < max_iter; ++iter)
		{
			double cond = condition();
			*theta_out = cond;
			if (cond < tol)
				return iter;
			auto F = deriv();
			double norm = sum_real_trace(mul(F, F));
			double beta = (norm - double(sum_real_trace(mul(F, last)))) / lastNorm;
			last = F;
			if (iter > 20 && beta > 0)
			{
				// landau.h:126-128 adds last*beta after last = F
				auto lb = scale(last, beta);
				site_loop(grid.V, [&](size_t i) { F[i] += lb[i]; });
			}
			eps = line_search(F, eps, n_evals);
			g = stepped(F, eps);
			reunitize(g);
			lastNorm = norm;
		}
		*theta_out = condition();
		return max_iter;
	}
};

} // namespace oracle
