// TEST INFRASTRUCTURE: quaternion and small-matrix stand-ins for krox/util
// (absent), written from the definitions (Hamilton product; matrix product,
// adjoint, trace, cofactor determinant, antihermitian-traceless projection,
// Gram-Schmidt, and the matrix exponential by scaling and squaring of a
// Taylor polynomial).
#pragma once
#include "util/complex.h"
#include <cmath>
#include <cstring>

namespace util {

// ---- quaternion ----
template <class T> struct quaternion
{
	T re, im1, im2, im3;
};
template <class T> inline quaternion<T> operator+(quaternion<T> a, quaternion<T> b)
{
	return {a.re + b.re, a.im1 + b.im1, a.im2 + b.im2, a.im3 + b.im3};
}
template <class T> inline quaternion<T> operator-(quaternion<T> a, quaternion<T> b)
{
	return {a.re - b.re, a.im1 - b.im1, a.im2 - b.im2, a.im3 - b.im3};
}
template <class T> inline quaternion<T> operator*(quaternion<T> a, quaternion<T> b)
{
	return {a.re * b.re - a.im1 * b.im1 - a.im2 * b.im2 - a.im3 * b.im3,
	        a.re * b.im1 + a.im1 * b.re + a.im2 * b.im3 - a.im3 * b.im2,
	        a.re * b.im2 - a.im1 * b.im3 + a.im2 * b.re + a.im3 * b.im1,
	        a.re * b.im3 + a.im1 * b.im2 - a.im2 * b.im1 + a.im3 * b.re};
}
template <class T, class S>
    requires is_scalar_v<S>
inline quaternion<T> operator*(quaternion<T> a, S s)
{
	return {T(a.re * s), T(a.im1 * s), T(a.im2 * s), T(a.im3 * s)};
}
template <class T> inline quaternion<T> &operator+=(quaternion<T> &a, quaternion<T> b) { return a = a + b; }
template <class T> inline quaternion<T> &operator-=(quaternion<T> &a, quaternion<T> b) { return a = a - b; }
template <class T, class S>
    requires is_scalar_v<S>
inline quaternion<T> &operator*=(quaternion<T> &a, S s)
{
	return a = a * s;
}
template <class T> inline quaternion<T> conj(quaternion<T> a) { return {a.re, -a.im1, -a.im2, -a.im3}; }
// quaternion norm |q|^2 (the choice under which project_on_group_fast of
// src/gauge/groups.h:188-192 is a reunitarisation)
template <class T> inline T norm2(quaternion<T> a)
{
	return a.re * a.re + a.im1 * a.im1 + a.im2 * a.im2 + a.im3 * a.im3;
}

// ---- N x N matrix ----
template <class T, int N> struct Vector
{
	T v[N];
	T &operator[](int i) { return v[i]; }
	T const &operator[](int i) const { return v[i]; }
	template <class S> Vector &operator/=(S const &s)
	{
		for (int i = 0; i < N; ++i)
			v[i] /= s;
		return *this;
	}
};

template <class T, int N> struct Matrix
{
	Vector<T, N> rows[N];
	T &operator()(int i, int j) { return rows[i][j]; }
	T const &operator()(int i, int j) const { return rows[i][j]; }
	Vector<T, N> &operator()(int i) { return rows[i]; }
	static Matrix zero()
	{
		Matrix r;
		std::memset((void *)&r, 0, sizeof(r));
		return r;
	}
	static Matrix identity()
	{
		Matrix r = zero();
		for (int i = 0; i < N; ++i)
			r(i, i) = T{1, 0};
		return r;
	}
	template <class Rng> static Matrix random_normal(Rng &rng)
	{
		using R = decltype(T{}.re);
		Matrix r;
		for (int i = 0; i < N; ++i)
			for (int j = 0; j < N; ++j)
			{
				R a = rng.template normal<R>();
				R b = rng.template normal<R>();
				r(i, j) = T{a, b};
			}
		return r;
	}
};

template <class T, int N> inline Matrix<T, N> operator+(Matrix<T, N> const &a, Matrix<T, N> const &b)
{
	Matrix<T, N> r;
	for (int i = 0; i < N; ++i)
		for (int j = 0; j < N; ++j)
			r(i, j) = a(i, j) + b(i, j);
	return r;
}
template <class T, int N> inline Matrix<T, N> operator-(Matrix<T, N> const &a, Matrix<T, N> const &b)
{
	Matrix<T, N> r;
	for (int i = 0; i < N; ++i)
		for (int j = 0; j < N; ++j)
			r(i, j) = a(i, j) - b(i, j);
	return r;
}
template <class T, int N> inline Matrix<T, N> operator*(Matrix<T, N> const &a, Matrix<T, N> const &b)
{
	Matrix<T, N> r;
	for (int i = 0; i < N; ++i)
		for (int j = 0; j < N; ++j)
		{
			T s = a(i, 0) * b(0, j);
			for (int k = 1; k < N; ++k)
				s += a(i, k) * b(k, j);
			r(i, j) = s;
		}
	return r;
}
template <class T, int N, class S>
    requires is_scalar_v<S>
inline Matrix<T, N> operator*(Matrix<T, N> const &a, S s)
{
	Matrix<T, N> r;
	for (int i = 0; i < N; ++i)
		for (int j = 0; j < N; ++j)
			r(i, j) = a(i, j) * s;
	return r;
}
template <class T, int N> inline Matrix<T, N> operator*(Matrix<T, N> const &a, T s)
{
	Matrix<T, N> r;
	for (int i = 0; i < N; ++i)
		for (int j = 0; j < N; ++j)
			r(i, j) = a(i, j) * s;
	return r;
}
template <class T, int N> inline Matrix<T, N> &operator+=(Matrix<T, N> &a, Matrix<T, N> const &b)
{
	return a = a + b;
}
template <class T, int N> inline Matrix<T, N> &operator-=(Matrix<T, N> &a, Matrix<T, N> const &b)
{
	return a = a - b;
}
template <class T, int N, class S>
    requires is_scalar_v<S>
inline Matrix<T, N> &operator*=(Matrix<T, N> &a, S s)
{
	return a = a * s;
}
template <class T, int N> inline Matrix<T, N> &operator*=(Matrix<T, N> &a, Matrix<T, N> const &b)
{
	return a = a * b;
}

template <class T, int N> inline Matrix<T, N> adj(Matrix<T, N> const &a)
{
	Matrix<T, N> r;
	for (int i = 0; i < N; ++i)
		for (int j = 0; j < N; ++j)
			r(i, j) = conj(a(j, i));
	return r;
}
template <class T, int N> inline T trace(Matrix<T, N> const &a)
{
	T s = a(0, 0);
	for (int i = 1; i < N; ++i)
		s += a(i, i);
	return s;
}
template <class T, int N> inline T norm2(Matrix<complex<T>, N> const &a)
{
	T s = 0;
	for (int i = 0; i < N; ++i)
		for (int j = 0; j < N; ++j)
			s += norm2(a(i, j));
	return s;
}
template <class T> inline complex<T> determinant(Matrix<complex<T>, 3> const &a)
{
	return a(0, 0) * (a(1, 1) * a(2, 2) - a(1, 2) * a(2, 1)) - a(0, 1) * (a(1, 0) * a(2, 2) - a(1, 2) * a(2, 0)) +
	       a(0, 2) * (a(1, 0) * a(2, 1) - a(1, 1) * a(2, 0));
}
template <class T, int N> inline Matrix<complex<T>, N> antihermitian_traceless(Matrix<complex<T>, N> const &a)
{
	Matrix<complex<T>, N> r;
	for (int i = 0; i < N; ++i)
		for (int j = 0; j < N; ++j)
			r(i, j) = (a(i, j) - conj(a(j, i))) * T(0.5);
	complex<T> tr = trace(r) * T(1.0 / N);
	for (int i = 0; i < N; ++i)
		r(i, i) -= tr;
	return r;
}
template <class T, int N> inline Matrix<complex<T>, N> gram_schmidt(Matrix<complex<T>, N> a)
{
	for (int i = 0; i < N; ++i)
	{
		for (int k = 0; k < i; ++k)
		{
			complex<T> ip = {T(0), T(0)};
			for (int j = 0; j < N; ++j)
				ip += conj(a(k, j)) * a(i, j);
			for (int j = 0; j < N; ++j)
				a(i, j) -= a(k, j) * ip;
		}
		T n = 0;
		for (int j = 0; j < N; ++j)
			n += norm2(a(i, j));
		n = T(1) / std::sqrt(n);
		for (int j = 0; j < N; ++j)
			a(i, j) = a(i, j) * n;
	}
	return a;
}
template <class T, int N> inline Matrix<complex<T>, N> exp(Matrix<complex<T>, N> const &a)
{
	constexpr int K = sizeof(T) == 8 ? 18 : 10;
	T n = 0;
	for (int j = 0; j < N; ++j)
	{
		T s = 0;
		for (int i = 0; i < N; ++i)
			s += std::sqrt(norm2(a(i, j)));
		n = std::max(n, s);
	}
	int sq = 0;
	while (n > T(0.5))
	{
		n *= T(0.5);
		++sq;
	}
	auto x = a * std::ldexp(T(1), -sq);
	auto id = Matrix<complex<T>, N>::identity();
	auto e = id;
	for (int k = K; k >= 1; --k)
		e = id + (x * e) * (T(1) / T(k));
	for (int i = 0; i < sq; ++i)
		e = e * e;
	return e;
}
} // namespace util
