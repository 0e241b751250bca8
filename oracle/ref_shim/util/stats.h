// TEST INFRASTRUCTURE: statistics helpers used by Hmc::print_summary.
#pragma once
#include <algorithm>
#include <cmath>
#include <span>
#include <vector>
namespace util {
inline double mean(std::span<const double> xs)
{
	double s = 0;
	for (double x : xs)
		s += x;
	return xs.empty() ? 0.0 : s / double(xs.size());
}
template <class F> double mean(std::span<const double> xs, F f)
{
	double s = 0;
	for (double x : xs)
		s += f(x);
	return xs.empty() ? 0.0 : s / double(xs.size());
}
inline double variance(std::span<const double> xs)
{
	double m = mean(xs), s = 0;
	for (double x : xs)
		s += (x - m) * (x - m);
	return xs.size() < 2 ? 0.0 : s / double(xs.size() - 1);
}
inline double min(std::span<const double> xs) { return xs.empty() ? 0.0 : *std::min_element(xs.begin(), xs.end()); }
inline double max(std::span<const double> xs) { return xs.empty() ? 0.0 : *std::max_element(xs.begin(), xs.end()); }
} // namespace util
