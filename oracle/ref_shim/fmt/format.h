// TEST INFRASTRUCTURE: minimal {fmt} stand-in (format/print with "{}" fields;
// format specs are accepted and applied for floating-point precision only).
#pragma once
#include <cstdio>
#include <span>
#include <sstream>
#include <string>
#include <string_view>
#include <iomanip>

namespace fmt {
namespace detail {
template <class T> void put(std::ostringstream &os, std::string_view spec, T const &v)
{
	if constexpr (std::is_floating_point_v<T>)
	{
		auto dot = spec.find('.');
		if (dot != std::string_view::npos)
		{
			int prec = 0;
			for (size_t i = dot + 1; i < spec.size() && spec[i] >= '0' && spec[i] <= '9'; ++i)
				prec = prec * 10 + (spec[i] - '0');
			os << std::fixed << std::setprecision(prec) << v;
			os.unsetf(std::ios::fixed);
			return;
		}
		os << std::setprecision(17) << v;
	}
	else if constexpr (requires { v.begin(); v.end(); } && !std::is_convertible_v<T, std::string_view>)
	{
		os << "[";
		bool first = true;
		for (auto const &x : v)
		{
			if (!first)
				os << ", ";
			first = false;
			os << x;
		}
		os << "]";
	}
	else
		os << v;
}
inline void emit(std::ostringstream &os, std::string_view f)
{
	os << f;
}
template <class A, class... As> void emit(std::ostringstream &os, std::string_view f, A const &a, As const &...as)
{
	auto open = f.find('{');
	if (open == std::string_view::npos)
	{
		os << f;
		return;
	}
	auto close = f.find('}', open);
	os << f.substr(0, open);
	auto inner = f.substr(open + 1, close - open - 1);
	auto colon = inner.find(':');
	put(os, colon == std::string_view::npos ? std::string_view{} : inner.substr(colon + 1), a);
	emit(os, f.substr(close + 1), as...);
}
} // namespace detail

template <class... As> std::string format(std::string_view f, As const &...as)
{
	std::ostringstream os;
	detail::emit(os, f, as...);
	return os.str();
}
template <class... As> void print(std::string_view f, As const &...as)
{
	std::fputs(format(f, as...).c_str(), stdout);
}
} // namespace fmt
