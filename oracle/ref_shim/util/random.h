// TEST INFRASTRUCTURE: stand-in for util::xoshiro256 that plays back
// caller-supplied normals and uniforms (so the reference's own
// random_algebra_field / runHmcUpdate consume known inputs).
#pragma once
#include <cstddef>
#include <stdexcept>
#include <vector>

namespace util {
struct playback
{
	std::vector<double> normals, uniforms;
	size_t in = 0, iu = 0;
};
inline playback &playback_state()
{
	static playback p;
	return p;
}
class xoshiro256
{
  public:
	template <class S> void seed(S const &) {}
	template <class T = double> T normal()
	{
		auto &p = playback_state();
		if (p.in >= p.normals.size())
			throw std::runtime_error("playback: out of normals");
		return T(p.normals[p.in++]);
	}
	template <class T = double> T uniform()
	{
		auto &p = playback_state();
		if (p.iu >= p.uniforms.size())
			throw std::runtime_error("playback: out of uniforms");
		return T(p.uniforms[p.iu++]);
	}
};
} // namespace util
