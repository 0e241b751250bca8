// Multi-dimensional complex FFT of lattice fields, FP32, hand-written.
//
// Layout: nf complex fields, each V points in lexicographic site order
// (dimension 0 slowest), buf[f * V + r]. One kernel launch per axis: one
// thread per line along that axis keeps the line in registers and runs a
// mixed-radix decimation-in-time DFT (radix 2 and 3, so extents 2^a 3^b up to
// 32 cover the lattices 4..32 including 12 and 24). Twiddle factors are
// compile-time constants from a constexpr Taylor series (no runtime sin/cos).
//
// Sign convention: forward X[k] = sum_x x e^{-2 pi i k x / L}; backward uses
// e^{+...}; both unnormalised (the caller divides by V).
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <type_traits>

namespace meshgb {
namespace fft {

// ---- compile-time sin/cos (Taylor series after reduction to [-pi/4, pi/4]) ----
constexpr double kPi = 3.14159265358979323846264338327950288;
__host__ __device__ constexpr double taylor_sin(double x)
{
	double t = x, s = x;
	for (int n = 1; n < 14; ++n)
	{
		t *= -x * x / double((2 * n) * (2 * n + 1));
		s += t;
	}
	return s;
}
__host__ __device__ constexpr double taylor_cos(double x)
{
	double t = 1.0, s = 1.0;
	for (int n = 1; n < 14; ++n)
	{
		t *= -x * x / double((2 * n - 1) * (2 * n));
		s += t;
	}
	return s;
}
// cos / sin of an angle in [0, pi], reduced to [0, pi/4]
__host__ __device__ constexpr double cos_a(double a)
{
	if (a > kPi / 2)
		return -cos_a(kPi - a);
	if (a > kPi / 4)
		return taylor_sin(kPi / 2 - a);
	return taylor_cos(a);
}
__host__ __device__ constexpr double sin_a(double a)
{
	if (a > kPi / 2)
		return sin_a(kPi - a);
	if (a > kPi / 4)
		return taylor_cos(kPi / 2 - a);
	return taylor_sin(a);
}
// cos and sin of 2 pi j / L for integers j, L
__host__ __device__ constexpr double cos2pi(int j, int L)
{
	j = ((j % L) + L) % L;
	if (2 * j > L)
		return cos2pi(L - j, L);
	return cos_a(2.0 * kPi * double(j) / double(L));
}
__host__ __device__ constexpr double sin2pi(int j, int L)
{
	j = ((j % L) + L) % L;
	if (2 * j > L)
		return -sin2pi(L - j, L);
	return sin_a(2.0 * kPi * double(j) / double(L));
}
static_assert(cos2pi(1, 4) > -1e-15 && cos2pi(1, 4) < 1e-15, "twiddle table");
static_assert(sin2pi(1, 12) > 0.4999999999999 && sin2pi(1, 12) < 0.5000000000001, "twiddle table");

template <int L, int SIGN> struct Twiddle
{
	// W^j = e^{SIGN 2 pi i j / L}
	__host__ __device__ static constexpr float re(int j) { return float(cos2pi(j, L)); }
	__host__ __device__ static constexpr float im(int j) { return float(double(SIGN) * sin2pi(j, L)); }
};

// compile-time loop: f(std::integral_constant<int, I>) for I in [B, E)
template <int B, int E, class F> __device__ __forceinline__ void static_for(F &&f)
{
	if constexpr (B < E)
	{
		f(std::integral_constant<int, B>{});
		static_for<B + 1, E>(f);
	}
}

__device__ __forceinline__ float2 cmulf(float2 a, float2 b)
{
	return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}

// in-place DFT of a register array of length L (2^a 3^b), decimation in time
template <int L, int SIGN> __device__ __forceinline__ void dft(float2 (&x)[L])
{
	if constexpr (L == 1)
		return;
	else
	{
		constexpr int R = (L % 2 == 0) ? 2 : 3;
		constexpr int M = L / R;
		static_assert(R * M == L && (L % 2 == 0 || L % 3 == 0), "FFT extents must be 2^a 3^b");
		float2 sub[R][M];
#pragma unroll
		for (int r = 0; r < R; ++r)
#pragma unroll
			for (int m = 0; m < M; ++m)
				sub[r][m] = x[r + R * m];
#pragma unroll
		for (int r = 0; r < R; ++r)
			dft<M, SIGN>(sub[r]);
		static_for<0, L>([&](auto kc) {
			constexpr int k = decltype(kc)::value;
			float2 acc = sub[0][k % M];
			static_for<1, R>([&](auto rc) {
				constexpr int r = decltype(rc)::value;
				constexpr int e = (r * k) % L;
				constexpr float wr = Twiddle<L, SIGN>::re(e);
				constexpr float wi = Twiddle<L, SIGN>::im(e);
				float2 t = cmulf(make_float2(wr, wi), sub[r][k % M]);
				acc.x += t.x;
				acc.y += t.y;
			});
			x[k] = acc;
		});
	}
}

// one axis pass: every line of length L along axis `d` (lexicographic
// stride `stride`), for nf fields of V points
template <int L, int SIGN>
__global__ void __launch_bounds__(128) k_fft_axis(float2 *__restrict__ buf, int64_t V, int nf, int64_t stride)
{
	int64_t lines_per_field = V / L;
	int64_t nlines = lines_per_field * nf;
	int64_t block = int64_t(L) * stride;
	for (int64_t l = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; l < nlines; l += int64_t(gridDim.x) * blockDim.x)
	{
		int64_t f = l / lines_per_field;
		int64_t r = l - f * lines_per_field;
		int64_t inner = r % stride;
		int64_t outer = r / stride;
		float2 *p = buf + f * V + outer * block + inner;
		float2 x[L];
#pragma unroll
		for (int j = 0; j < L; ++j)
			x[j] = p[j * stride];
		dft<L, SIGN>(x);
#pragma unroll
		for (int j = 0; j < L; ++j)
			p[j * stride] = x[j];
	}
}

inline bool supported_extent(int L)
{
	switch (L)
	{
	case 2:
	case 4:
	case 6:
	case 8:
	case 12:
	case 16:
	case 24:
	case 32:
		return true;
	default:
		return false;
	}
}

// full transform over the nd axes of a lattice with extents dims[]
template <int SIGN>
inline void fft_nd(float2 *buf, int nd, int32_t const *dims, int nf, int num_sms, cudaStream_t stream)
{
	int64_t V = 1;
	for (int i = 0; i < nd; ++i)
		V *= dims[i];
	int64_t stride = 1;
	for (int d = nd - 1; d >= 0; --d)
	{
		int L = dims[d];
		int64_t nlines = (V / L) * nf;
		int64_t need = (nlines + 127) / 128;
		int64_t cap = int64_t(num_sms) * 16;
		unsigned blocks = unsigned(need < cap ? need : cap);
		switch (L)
		{
		case 2:
			k_fft_axis<2, SIGN><<<blocks, 128, 0, stream>>>(buf, V, nf, stride);
			break;
		case 4:
			k_fft_axis<4, SIGN><<<blocks, 128, 0, stream>>>(buf, V, nf, stride);
			break;
		case 6:
			k_fft_axis<6, SIGN><<<blocks, 128, 0, stream>>>(buf, V, nf, stride);
			break;
		case 8:
			k_fft_axis<8, SIGN><<<blocks, 128, 0, stream>>>(buf, V, nf, stride);
			break;
		case 12:
			k_fft_axis<12, SIGN><<<blocks, 128, 0, stream>>>(buf, V, nf, stride);
			break;
		case 16:
			k_fft_axis<16, SIGN><<<blocks, 128, 0, stream>>>(buf, V, nf, stride);
			break;
		case 24:
			k_fft_axis<24, SIGN><<<blocks, 128, 0, stream>>>(buf, V, nf, stride);
			break;
		case 32:
			k_fft_axis<32, SIGN><<<blocks, 128, 0, stream>>>(buf, V, nf, stride);
			break;
		default:
			break;
		}
		stride *= L;
	}
}

} // namespace fft
} // namespace meshgb
