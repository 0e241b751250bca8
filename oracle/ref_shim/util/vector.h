// TEST INFRASTRUCTURE: fixed-capacity vector stand-in (Coordinate).
#pragma once
#include <cassert>
#include <cstddef>
#include <initializer_list>
namespace util {
template <class T, size_t N> class static_vector
{
	T data_[N] = {};
	size_t size_ = 0;

  public:
	static_vector() = default;
	static_vector(std::initializer_list<T> l)
	{
		for (auto const &x : l)
			data_[size_++] = x;
	}
	template <class It> static_vector(It b, It e)
	{
		for (; b != e; ++b)
			data_[size_++] = T(*b);
	}
	size_t size() const { return size_; }
	T &operator[](size_t i) { return data_[i]; }
	T const &operator[](size_t i) const { return data_[i]; }
	T const *begin() const { return data_; }
	T const *end() const { return data_ + size_; }
	bool operator==(static_vector const &o) const
	{
		if (size_ != o.size_)
			return false;
		for (size_t i = 0; i < size_; ++i)
			if (data_[i] != o.data_[i])
				return false;
		return true;
	}
};
} // namespace util
