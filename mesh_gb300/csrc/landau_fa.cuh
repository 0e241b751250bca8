// Fourier-accelerated steepest descent for Landau gauge (Davies et al.,
// Phys. Rev. D 37 (1988) 1581), with the fixed spectral multiplier
// alpha p_max^2 / p^2 or a learned multiplier table, and the per-momentum
// response probe that produces the learned multiplier's training targets.
// No counterpart in the reference (its solver is the CG of landau.h:100-136).
//
// One step on the gauge transform g (FP64), links U fixed:
//   A_mu(x)   = proj(g(x) U_mu(x) g(x+mu)^+)                 k_fa_links (FP64;
//               optionally the FP64 sum of Re tr g(x) U_mu(x) g(x+mu)^+,
//               the gauge functional up to its normalisation)
//   Delta(x)  = sum_mu A_mu(x) - A_mu(x-mu)                   k_fa_div   (FP64;
//               theta_ref = sum |Delta|^2/(Nd V) in FP64; Delta packed
//               pairwise into FP32 complex fields, lexicographic order)
//   X         = F^-1[ m(p) F[Delta] ] / V                     FP32 FFT
//   g(x)     <- reunit( exp(-X(x)) g(x) )                     k_fa_update (FP64)
// The FFT only shapes the step direction; theta and g stay FP64, so the
// stopping criterion is unaffected by the FP32 transform.
#pragma once

#include "fft.cuh"
#include "kernels.cuh"

namespace meshgb {

// lattice momentum tables: s_d[n] = 4 sin^2(pi n / L_d)
struct MomTables
{
	float s[4][32];
	int nd;
	int L[4];
	int64_t stride[4];
	float p2max;
};

// multiplier: mode 0: alpha p2max/p2 (0 at p=0); mode 1: exp(table) with the
// table sampled uniformly in log p^2 over [lo, hi] and interpolated linearly
struct Multiplier
{
	int mode;
	float alpha;
	float lo, hi;
	int n;
	float const *table; // device, n entries (log multiplier)
};

__device__ __forceinline__ float phat2_of(MomTables const &mt, int64_t r)
{
	float p2 = 0.f;
#pragma unroll
	for (int d = 0; d < 4; ++d)
	{
		if (d >= mt.nd)
			break;
		int64_t q = r / mt.stride[d];
		int x = int(q % mt.L[d]);
		p2 += mt.s[d][x];
	}
	return p2;
}

__device__ __forceinline__ float mult_of(Multiplier const &m, MomTables const &mt, float p2)
{
	if (p2 <= 0.f)
		return 0.f;
	if (m.mode == 0)
		return m.alpha * mt.p2max / p2;
	float t = (logf(p2) - m.lo) / (m.hi - m.lo) * float(m.n - 1);
	t = fminf(fmaxf(t, 0.f), float(m.n - 1));
	int i = int(t);
	if (i >= m.n - 1)
		i = m.n - 2;
	float f = t - float(i);
	return expf(m.table[i] * (1.f - f) + m.table[i + 1] * f);
}

// A_mu(x) for every link, packed algebra, SoA per direction
template <int GRP, class T, int ND>
__global__ void __launch_bounds__(256) k_fa_links(Geom g, T const *__restrict__ U, T const *__restrict__ G,
                                                   T *__restrict__ A, RedSlot func)
{
	double acc = 0.0;
	using Gp = Group<GRP, T>;
	using E = typename Gp::E;
	LinkLoad<GRP, T, ND> ld{U, g.V};
	int64_t n = int64_t(ND) * g.V;
	for (int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x)
	{
		int mu = int(i / g.V);
		int64_t s = i - int64_t(mu) * g.V;
		Site<ND> st = site_from_eo<ND>(g, s);
		E gx, gf;
		Soa<T, Gp::NR>::load(G, g.V, s, gx.v);
		Soa<T, Gp::NR>::load(G, g.V, eo_shift1<ND>(g, st, mu, +1), gf.v);
		T a[Gp::NA];
		E w = Gp::mul_nd(Gp::mul(gx, ld(mu, s)), gf);
		if (func.result)
			acc += double(Gp::retr(w));
		Gp::proj(w, a);
		comp<T, Gp::NA>(A, g.V, mu).store(s, a);
	}
	if (func.result) // uniform over the grid (a kernel argument)
		grid_sum<256>(acc, func);
}

// Delta(x), theta sum, and the FP32 complex FFT input (lexicographic order)
template <int GRP, class T, int ND>
__global__ void __launch_bounds__(256) k_fa_div(Geom g, T const *__restrict__ A, float2 *__restrict__ buf,
                                                 RedSlot theta)
{
	using Gp = Group<GRP, T>;
	constexpr int NF = (Gp::NA + 1) / 2;
	double acc = 0.0;
	for (int64_t s = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; s < g.V; s += int64_t(gridDim.x) * blockDim.x)
	{
		Site<ND> st = site_from_eo<ND>(g, s);
		T D[Gp::NA];
#pragma unroll
		for (int k = 0; k < Gp::NA; ++k)
			D[k] = T(0);
#pragma unroll
		for (int mu = 0; mu < ND; ++mu)
		{
			T a[Gp::NA], b[Gp::NA];
			comp<T, Gp::NA>(const_cast<T *>(A), g.V, mu).load(s, a);
			comp<T, Gp::NA>(const_cast<T *>(A), g.V, mu).load(eo_shift1<ND>(g, st, mu, -1), b);
#pragma unroll
			for (int k = 0; k < Gp::NA; ++k)
				D[k] += a[k] - b[k];
		}
		acc += double(Gp::kin(D));
		if (buf)
		{
#pragma unroll
			for (int f = 0; f < NF; ++f)
			{
				float re = float(D[2 * f]);
				float im = (2 * f + 1 < Gp::NA) ? float(D[2 * f + 1]) : 0.f;
				buf[int64_t(f) * g.V + st.lex] = make_float2(re, im);
			}
		}
	}
	grid_sum<256>(acc, theta);
}

// multiply every momentum mode by the spectral multiplier
__global__ void __launch_bounds__(256) k_fa_scale(float2 *__restrict__ buf, int64_t V, int nf, MomTables mt,
                                                  Multiplier m)
{
	for (int64_t r = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; r < V; r += int64_t(gridDim.x) * blockDim.x)
	{
		float f = mult_of(m, mt, phat2_of(mt, r));
		for (int k = 0; k < nf; ++k)
		{
			float2 v = buf[int64_t(k) * V + r];
			buf[int64_t(k) * V + r] = make_float2(v.x * f, v.y * f);
		}
	}
}

// g_out(x) = reunit(exp(-X(x)/V) g_in(x)), X from the transformed buffer
template <int GRP, class T, int ND>
__global__ void __launch_bounds__(256) k_fa_update(Geom g, float2 const *__restrict__ buf, T const *__restrict__ Gin,
                                                    T *__restrict__ Gout, T scale)
{
	using Gp = Group<GRP, T>;
	using E = typename Gp::E;
	constexpr int NF = (Gp::NA + 1) / 2;
	for (int64_t s = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; s < g.V; s += int64_t(gridDim.x) * blockDim.x)
	{
		Site<ND> st = site_from_eo<ND>(g, s);
		T X[Gp::NA];
#pragma unroll
		for (int f = 0; f < NF; ++f)
		{
			float2 v = buf[int64_t(f) * g.V + st.lex];
			X[2 * f] = T(v.x);
			if (2 * f + 1 < Gp::NA)
				X[2 * f + 1] = T(v.y);
		}
		E gx;
		Soa<T, Gp::NR>::load(Gin, g.V, s, gx.v);
		E r = Gp::reunit_exact(Gp::mul(Gp::exp_alg(X, -scale), gx));
		Soa<T, Gp::NR>::store(Gout, g.V, s, r.v);
	}
}

// per-bin response of the modes to a probe step:
// lambda_b = sum_{p in b} (|F_old|^2 - Re<F_new, F_old>) / m0(p) / sum |F_old|^2
__global__ void __launch_bounds__(256) k_fa_shell(float2 const *__restrict__ Fold, float2 const *__restrict__ Fnew,
                                                  int64_t V, int nf, MomTables mt, Multiplier m0, int nbins,
                                                  float blo, float bhi, double *__restrict__ num,
                                                  double *__restrict__ den, double *__restrict__ p2sum,
                                                  double *__restrict__ cnt)
{
	extern __shared__ double sh[];
	double *snum = sh, *sden = sh + nbins, *sp2 = sh + 2 * nbins, *scnt = sh + 3 * nbins;
	for (int b = threadIdx.x; b < 4 * nbins; b += blockDim.x)
		sh[b] = 0.0;
	__syncthreads();
	for (int64_t r = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; r < V; r += int64_t(gridDim.x) * blockDim.x)
	{
		float p2 = phat2_of(mt, r);
		if (p2 <= 0.f)
			continue;
		float mm = mult_of(m0, mt, p2);
		int b = int((logf(p2) - blo) / (bhi - blo) * float(nbins));
		b = b < 0 ? 0 : (b >= nbins ? nbins - 1 : b);
		double o2 = 0, on = 0;
		for (int k = 0; k < nf; ++k)
		{
			float2 a = Fold[int64_t(k) * V + r], c = Fnew[int64_t(k) * V + r];
			o2 += double(a.x) * a.x + double(a.y) * a.y;
			on += double(a.x) * c.x + double(a.y) * c.y;
		}
		atomicAdd(&snum[b], (o2 - on) / double(mm));
		atomicAdd(&sden[b], o2);
		atomicAdd(&sp2[b], double(p2));
		atomicAdd(&scnt[b], 1.0);
	}
	__syncthreads();
	for (int b = threadIdx.x; b < nbins; b += blockDim.x)
	{
		atomicAdd(&num[b], snum[b]);
		atomicAdd(&den[b], sden[b]);
		atomicAdd(&p2sum[b], sp2[b]);
		atomicAdd(&cnt[b], scnt[b]);
	}
}

// features of the learned multiplier on its table grid:
// (log p^2 - log p2max, 5 (beta - 6), (log10 theta + 7) / 5)
__global__ void k_fa_features(int n, float lo, float hi, float logp2max, float f1, float f2, float *__restrict__ x)
{
	for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < n; j += gridDim.x * blockDim.x)
	{
		float lp = lo + (hi - lo) * float(j) / float(n - 1);
		x[3 * j] = lp - logp2max;
		x[3 * j + 1] = f1;
		x[3 * j + 2] = f2;
	}
}

} // namespace meshgb
