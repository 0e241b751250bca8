// TEST INFRASTRUCTURE: row-major 2-D span stand-in (lattice.h cshift).
#pragma once
#include <cstddef>
#include <span>
namespace util {
template <class T> class span_2d
{
	T *data_;
	size_t h_, w_;

  public:
	span_2d(T *d, size_t h, size_t w) : data_(d), h_(h), w_(w) {}
	T *data() const { return data_; }
	size_t height() const { return h_; }
	size_t width() const { return w_; }
	size_t size() const { return h_ * w_; }
	T &operator()(size_t i, size_t j) const { return data_[i * w_ + j]; }
};
template <class T> span_2d(T *, size_t, size_t) -> span_2d<T>;
} // namespace util
