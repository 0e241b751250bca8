// Counter-based random numbers on the device: Philox4x32-10 (Salmon, Moraes,
// Dror, Shaw, "Parallel random numbers: as easy as 1, 2, 3", SC'11), written
// from the paper's round function and constants. Every draw is addressed by
// (seed, lexicographic site, direction, tag, counter), so a stream does not
// depend on the device layout, the launch shape or the number of GPUs.
//   key = (seed & 0xffffffff, seed >> 32)
//   ctr = (site, tag << 24 | mu << 8 | block, n & 0xffffffff, n >> 32)
#pragma once

#include <cstdint>

#include "group.cuh"

namespace meshgb {

enum : uint32_t
{
	TAG_MOMENTUM = 1,
	TAG_GAUGE = 2,
	TAG_METROPOLIS = 3,
	TAG_TRANSFORM = 4,
};

struct U4
{
	uint32_t v[4];
};

MESH_HD U4 philox4x32_10(uint32_t c0, uint32_t c1, uint32_t c2, uint32_t c3, uint32_t k0, uint32_t k1)
{
#pragma unroll
	for (int r = 0; r < 10; ++r)
	{
#ifdef __CUDA_ARCH__
		uint32_t lo0 = 0xD2511F53u * c0, hi0 = __umulhi(0xD2511F53u, c0);
		uint32_t lo1 = 0xCD9E8D57u * c2, hi1 = __umulhi(0xCD9E8D57u, c2);
#else
		uint64_t p0 = uint64_t(0xD2511F53u) * c0, p1 = uint64_t(0xCD9E8D57u) * c2;
		uint32_t lo0 = uint32_t(p0), hi0 = uint32_t(p0 >> 32);
		uint32_t lo1 = uint32_t(p1), hi1 = uint32_t(p1 >> 32);
#endif
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

MESH_HD float u24(uint32_t x) { return (float(x >> 8) + 0.5f) * (1.0f / 16777216.0f); }
MESH_HD double u53(uint32_t a, uint32_t b)
{
	uint64_t m = (uint64_t(a) << 21) ^ uint64_t(b >> 11);
	return (double(m) + 0.5) * (1.0 / 9007199254740992.0);
}

// n standard normals by Box-Muller in the precision T (float: 4 per Philox
// call from 24-bit uniforms; double: 2 per call from 53-bit uniforms)
template <class T, int N>
MESH_HD void normals(uint64_t seed, uint32_t tag, uint32_t site, uint32_t mu, uint64_t n_ctr, T *out)
{
	uint32_t k0 = uint32_t(seed), k1 = uint32_t(seed >> 32);
	uint32_t c2 = uint32_t(n_ctr), c3 = uint32_t(n_ctr >> 32);
	if constexpr (sizeof(T) == 4)
	{
#pragma unroll
		for (int blk = 0; 4 * blk < N; ++blk)
		{
			U4 r = philox4x32_10(site, (tag << 24) | (mu << 8) | uint32_t(blk), c2, c3, k0, k1);
#pragma unroll
			for (int h = 0; h < 2; ++h)
			{
				float ua = u24(r.v[2 * h]), ub = u24(r.v[2 * h + 1]);
				float rad = sqrtf(-2.0f * logf(ua));
				float s, c;
#ifdef __CUDA_ARCH__
				sincospif(2.0f * ub, &s, &c);
#else
				s = std::sin(float(2.0 * M_PI) * ub);
				c = std::cos(float(2.0 * M_PI) * ub);
#endif
				int i = 4 * blk + 2 * h;
				if (i < N)
					out[i] = rad * c;
				if (i + 1 < N)
					out[i + 1] = rad * s;
			}
		}
	}
	else
	{
#pragma unroll
		for (int blk = 0; 2 * blk < N; ++blk)
		{
			U4 r = philox4x32_10(site, (tag << 24) | (mu << 8) | uint32_t(blk), c2, c3, k0, k1);
			double ua = u53(r.v[0], r.v[1]), ub = u53(r.v[2], r.v[3]);
			double rad = sqrt(-2.0 * log(ua));
			double s, c;
#ifdef __CUDA_ARCH__
			sincospi(2.0 * ub, &s, &c);
#else
			s = std::sin(2.0 * M_PI * ub);
			c = std::cos(2.0 * M_PI * ub);
#endif
			int i = 2 * blk;
			if (i < N)
				out[i] = T(rad * c);
			if (i + 1 < N)
				out[i + 1] = T(rad * s);
		}
	}
}

MESH_HD double metropolis_uniform(uint64_t seed, uint64_t traj)
{
	U4 r = philox4x32_10(0u, TAG_METROPOLIS << 24, uint32_t(traj), uint32_t(traj >> 32), uint32_t(seed),
	                     uint32_t(seed >> 32));
	return u53(r.v[0], r.v[1]);
}

} // namespace meshgb
