// TEST INFRASTRUCTURE: host replacement of src/lattice/device.h (whose apply
// and sum kernels exist only under __CUDACC__). Same interface; device_apply
// is a loop over sites and the sums keep the reference's reduction order:
// blocks of 256, pairwise tree per block (device.h:185-212), serial combine of
// the block partials in the result type (device.h:246-265).
#pragma once
#include "util/memory.h"
#include "util/span.h"
#include <cassert>
#include <cstddef>
#include <cstring>
#include <memory>
#include <span>
#include <stdexcept>
#include <type_traits>
#include <vector>

namespace mesh {

template <class T> class device_buffer
{
	std::vector<T> v_;

  public:
	device_buffer() = default;
	explicit device_buffer(size_t n) : v_(n) {}
	std::span<T> get() { return {v_.data(), v_.size()}; }
	std::span<const T> get() const { return {v_.data(), v_.size()}; }
};

template <class T> device_buffer<T> device_allocate(size_t n) { return device_buffer<T>(n); }

inline void device_synchronize() {}

template <class T> void device_copy(std::span<T> dst, std::span<const T> src)
{
	assert(dst.size() == src.size());
	if (!dst.empty())
		std::memcpy((void *)dst.data(), (void const *)src.data(), dst.size() * sizeof(T));
}
template <class T> void device_clear(std::span<T> data)
{
	if (!data.empty())
		std::memset((void *)data.data(), 0, data.size() * sizeof(T));
}
template <class T> void device_copy_from_host(std::span<T> dst, std::span<const T> src) { device_copy(dst, src); }
template <class T> void device_copy_to_host(std::vector<T> &dst, std::span<const T> src)
{
	device_copy(std::span<T>(dst), src);
}

// dst[i, j] = src[i, j + offset] (periodic in j)
template <class T> void device_cshift(util::span_2d<T> dst, util::span_2d<const T> src, int64_t offset)
{
	if ((void const *)dst.data() == (void const *)src.data())
		throw std::runtime_error("inplace cshift(2d) not supported");
	int64_t w = int64_t(dst.width());
	for (size_t i = 0; i < dst.height(); ++i)
		for (int64_t j = 0; j < w; ++j)
		{
			int64_t s = ((j + offset) % w + w) % w;
			dst(i, size_t(j)) = src(i, size_t(s));
		}
}

template <class F, class T, class... Ts> void device_apply(F f, std::span<T> a, std::span<const Ts>... as)
{
	assert(((a.size() == as.size()) && ...));
	long long n = (long long)a.size();
#pragma omp parallel for schedule(static)
	for (long long i = 0; i < n; ++i)
		f(a[size_t(i)], as[size_t(i)]...);
}

template <class R, class G> R tree_reduce(size_t n, G gen)
{
	constexpr size_t B = 256;
	size_t nb = (n + B - 1) / B;
	std::vector<R> part(nb);
#pragma omp parallel for schedule(static)
	for (long long b = 0; b < (long long)nb; ++b)
	{
		std::vector<R> s(B);
		for (size_t l = 0; l < B; ++l)
		{
			size_t g = size_t(b) * B + l;
			if (g < n)
				s[l] = gen(g);
		}
		for (size_t stride = B / 2; stride > 0; stride /= 2)
			for (size_t l = 0; l < stride; ++l)
				if (size_t(b) * B + l + stride < n)
					s[l] += s[l + stride];
		part[size_t(b)] = s[0];
	}
	R r = part[0];
	for (size_t i = 1; i < nb; ++i)
		r += part[i];
	return r;
}

template <class T> T device_sum(std::span<const T> a)
{
	return tree_reduce<T>(a.size(), [&](size_t i) { return a[i]; });
}

template <class F, class T, class... Ts>
auto device_sum_apply(F f, std::span<const T> a, std::span<const Ts>... as) -> decltype(f(a[0], as[0]...))
{
	using R = decltype(f(a[0], as[0]...));
	return tree_reduce<R>(a.size(), [&](size_t i) { return f(a[i], as[i]...); });
}

} // namespace mesh
