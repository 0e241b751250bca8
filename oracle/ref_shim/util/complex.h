// TEST INFRASTRUCTURE: complex-number stand-in for krox/util (absent),
// written from the definition of complex arithmetic.
#pragma once
#include <cassert>
#include <cmath>
#include <string>
#include <string_view>
#include <type_traits>
#include <utility>
#include "fmt/format.h"

#ifndef UTIL_DEVICE
#define UTIL_DEVICE
#endif

namespace util {
template <class T> struct complex
{
	T re, im;
};
template <class S> inline constexpr bool is_scalar_v = std::is_arithmetic_v<S>;

template <class T> inline complex<T> operator+(complex<T> a, complex<T> b) { return {a.re + b.re, a.im + b.im}; }
template <class T> inline complex<T> operator-(complex<T> a, complex<T> b) { return {a.re - b.re, a.im - b.im}; }
template <class T> inline complex<T> operator-(complex<T> a) { return {-a.re, -a.im}; }
template <class T> inline complex<T> operator*(complex<T> a, complex<T> b)
{
	return {a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re};
}
template <class T> inline complex<T> operator/(complex<T> a, complex<T> b)
{
	T n = b.re * b.re + b.im * b.im;
	return {(a.re * b.re + a.im * b.im) / n, (a.im * b.re - a.re * b.im) / n};
}
template <class T, class S>
    requires is_scalar_v<S>
inline complex<T> operator*(complex<T> a, S s)
{
	return {T(a.re * s), T(a.im * s)};
}
template <class T, class S>
    requires is_scalar_v<S>
inline complex<T> operator*(S s, complex<T> a)
{
	return {T(s * a.re), T(s * a.im)};
}
template <class T, class S>
    requires is_scalar_v<S>
inline complex<T> operator/(complex<T> a, S s)
{
	return {T(a.re / s), T(a.im / s)};
}
template <class T, class S>
    requires is_scalar_v<S>
inline complex<T> operator-(S s, complex<T> a)
{
	return {T(s - a.re), T(-a.im)};
}
template <class T, class S>
    requires is_scalar_v<S>
inline complex<T> operator+(complex<T> a, S s)
{
	return {T(a.re + s), a.im};
}
template <class T> inline complex<T> &operator+=(complex<T> &a, complex<T> b) { return a = a + b; }
template <class T> inline complex<T> &operator-=(complex<T> &a, complex<T> b) { return a = a - b; }
template <class T> inline complex<T> &operator*=(complex<T> &a, complex<T> b) { return a = a * b; }
template <class T> inline complex<T> &operator/=(complex<T> &a, complex<T> b) { return a = a / b; }
template <class T, class S>
    requires is_scalar_v<S>
inline complex<T> &operator*=(complex<T> &a, S s)
{
	return a = a * s;
}
template <class T> inline complex<T> conj(complex<T> a) { return {a.re, -a.im}; }
template <class T> inline T norm2(complex<T> a) { return a.re * a.re + a.im * a.im; }
template <class T> inline T real(complex<T> a) { return a.re; }
} // namespace util
