// TEST INFRASTRUCTURE — NOT PART OF THE PRODUCT.
//
// Oracle parts with no counterpart in the reference, restated from published
// methods (the reference's Landau solver is the nonlinear CG of
// src/gauge/landau.h:100-136; its only relaxation code is the legacy,
// non-compiling src/old/gauge_fixing.cpp:33-79, whose site update
// "g(a) = normalize(sum_b u g(b)^dagger)^dagger" and block-of-sweeps stopping
// rule these follow):
//   * checkerboard overrelaxation for Landau gauge (Mandula & Ogilvie,
//     Phys. Lett. B 248 (1990) 156): local maximisation of
//     ReTr(g(x) K(x)), SU(3) through its three SU(2) subgroups
//     (Cabibbo & Marinari, Phys. Lett. B 119 (1982) 387), overrelaxed by the
//     second-order binomial expansion of h^omega, renormalised;
//   * Fourier-accelerated steepest descent (Davies et al., Phys. Rev. D 37
//     (1988) 1581) with a per-momentum multiplier table;
//   * a direct multi-dimensional DFT;
//   * the 3-layer tanh MLP of the learned spectral multiplier, with its
//     mean-squared-error loss and gradient in double precision;
//   * rectangular Wilson loops r x t in the planes (mu, 3), mu < 3, as in the
//     legacy src/old/mesh/wilson.cpp:40-75 (spatial line of r links, temporal
//     line of t links; sum over sites and the three spatial directions),
//     normalised like the plaquette (ReTr / Nc), every loop walked link by
//     link.
#pragma once

#include "oracle.hpp"

#include <complex>

namespace oracle {

// ---- Wilson loops ------------------------------------------------------------

// W(r, t) = sum_x sum_{mu<3} ReTr(S_mu^r(x) T^t(x + r mu) S_mu^r(x + t 3)^+ T^t(x)^+) / (3 V Nc)
// for r = 1..R, t = 1..T (out[(r-1) T + (t-1)]); S^r: product of r links in
// direction mu, T^t: product of t links in direction 3. Each loop is walked
// link by link (no shared line products), in double precision.
template <class G>
inline void wilson_loops(Grid const &g, GaugeField<G> const &U, int R, int T, double *out)
{
	using real = typename traits<G>::real;
	std::vector<double> acc(size_t(R) * T, 0.0);
	for (size_t x = 0; x < g.V; ++x)
		for (int mu = 0; mu < 3; ++mu)
			for (int r = 1; r <= R; ++r)
				for (int t = 1; t <= T; ++t)
				{
					G w = unit<G>();
					size_t y = x;
					for (int k = 0; k < r; ++k, y = g.shift(y, mu, 1))
						w = w * U[mu][y];
					for (int k = 0; k < t; ++k, y = g.shift(y, 3, 1))
						w = w * U[3][y];
					for (int k = 0; k < r; ++k)
					{
						y = g.shift(y, mu, -1);
						w = w * adj(U[mu][y]);
					}
					for (int k = 0; k < t; ++k)
					{
						y = g.shift(y, 3, -1);
						w = w * adj(U[3][y]);
					}
					acc[size_t(r - 1) * T + (t - 1)] += double(real(real_trace(w)));
				}
	double norm = 3.0 * double(g.V) * double(traits<G>::Nc);
	for (size_t k = 0; k < acc.size(); ++k)
		out[k] = acc[k] / norm;
}

// ---- gauge-fixed links and the Landau-gauge divergence --------------------

// A_mu(x) = proj(g(x) U_mu(x) g(x+mu)^dagger);
// Delta(x) = sum_mu [A_mu(x) - A_mu(x-mu)]  (== proj(g d) of landau.h:37-49)
template <class G> inline Field<G> divergence(Grid const &g, GaugeField<G> const &U, Field<G> const &h)
{
	Field<G> D(g.V, zero<G>());
	for (int mu = 0; mu < g.nd; ++mu)
	{
		Field<G> A(g.V);
		site_loop(g.V, [&](size_t r) {
			size_t f = g.shift(r, mu, 1);
			A[r] = project_on_algebra(h[r] * U[mu][r] * adj(h[f]));
		});
		site_loop(g.V, [&](size_t r) {
			size_t b = g.shift(r, mu, -1);
			D[r] = D[r] + A[r] - A[b];
		});
	}
	return D;
}

template <class G> inline double theta_fast(Grid const &g, GaugeField<G> const &U, Field<G> const &h)
{
	auto D = divergence(g, U, h);
	double s = tree_sum<double>(g.V, [&](size_t r) { return double(alg_norm2(D[r])); });
	return s / (double(g.nd) * double(g.V));
}

template <class G> inline double functional_fast(Grid const &g, GaugeField<G> const &U, Field<G> const &h)
{
	double s = tree_sum<double>(g.V, [&](size_t r) {
		double t = 0;
		for (int mu = 0; mu < g.nd; ++mu)
			t += double(real_trace(h[r] * U[mu][r] * adj(h[g.shift(r, mu, 1)])));
		return t;
	});
	return s / (double(traits<G>::Nc) * g.nd * double(g.V));
}

// ---- overrelaxation -------------------------------------------------------

// second-order binomial approximation of h^omega for a unit quaternion h,
// renormalised: 1 + w(h-1) + w(w-1)/2 (h-1)^2
template <class T> inline quat<T> or_power(quat<T> h, T w)
{
	T c = w * (w - T(1)) * T(0.5);
	T a = h.re - T(1);
	T v2 = h.im1 * h.im1 + h.im2 * h.im2 + h.im3 * h.im3;
	T r0 = T(1) + w * a + c * (a * a - v2);
	T f = w + T(2) * c * a;
	quat<T> r = {r0, h.im1 * f, h.im2 * f, h.im3 * f};
	T n = std::sqrt(r.re * r.re + r.im1 * r.im1 + r.im2 * r.im2 + r.im3 * r.im3);
	return r * (T(1) / n);
}

// the update of g(x) given W = g(x) K(x)
template <class T> inline cplx<T> or_update(cplx<T> W, cplx<T> gx, T w)
{
	T n = std::sqrt(norm2(W));
	if (n < T(1e-30))
		return gx;
	// h = conj(W)/|W| = e^{-i phi}; h^w = e^{-i w phi}
	T phi = std::atan2(W.im, W.re);
	cplx<T> hw = {std::cos(w * phi), -std::sin(w * phi)};
	return hw * gx;
}
template <class T> inline quat<T> or_update(quat<T> W, quat<T> gx, T w)
{
	T n = std::sqrt(W.re * W.re + W.im1 * W.im1 + W.im2 * W.im2 + W.im3 * W.im3);
	if (n < T(1e-30))
		return gx;
	quat<T> h = conj(W) * (T(1) / n);
	return or_power(h, w) * gx;
}
template <class T> inline mat3<T> or_update(mat3<T> W, mat3<T> gx, T w)
{
	static const int sub[3][2] = {{0, 1}, {0, 2}, {1, 2}};
	for (int s = 0; s < 3; ++s)
	{
		int i = sub[s][0], j = sub[s][1];
		// SU(2) projection of the (i,j) block of W
		quat<T> q = {(W.m[i][i].re + W.m[j][j].re) * T(0.5), (W.m[j][i].im + W.m[i][j].im) * T(0.5),
		             (W.m[i][j].re - W.m[j][i].re) * T(0.5), (W.m[i][i].im - W.m[j][j].im) * T(0.5)};
		T n = std::sqrt(q.re * q.re + q.im1 * q.im1 + q.im2 * q.im2 + q.im3 * q.im3);
		if (n < T(1e-30))
			continue;
		quat<T> h = or_power(conj(q) * (T(1) / n), w);
		// 2x2 matrix of h: [[h0 + i h3, h2 + i h1], [-h2 + i h1, h0 - i h3]]
		cplx<T> a = {h.re, h.im3}, b = {h.im2, h.im1}, c = {-h.im2, h.im1}, d = {h.re, -h.im3};
		for (int k = 0; k < 3; ++k)
		{
			cplx<T> gi = gx.m[i][k], gj = gx.m[j][k];
			gx.m[i][k] = a * gi + b * gj;
			gx.m[j][k] = c * gi + d * gj;
			cplx<T> wi = W.m[i][k], wj = W.m[j][k];
			W.m[i][k] = a * wi + b * wj;
			W.m[j][k] = c * wi + d * wj;
		}
	}
	return gx;
}

// one sweep: all even sites, then all odd sites. Sites of one parity do not
// interact, so the order inside a parity is immaterial.
template <class G> inline void or_sweep(Grid const &g, GaugeField<G> const &U, Field<G> &h, double omega)
{
	using T = typename traits<G>::real;
	for (int p = 0; p < 2; ++p)
	{
		site_loop(g.V, [&](size_t r) {
			int x[4];
			g.coords(r, x);
			int par = 0;
			for (int i = 0; i < g.nd; ++i)
				par += x[i];
			if ((par & 1) != p)
				return;
			G K = zero<G>();
			for (int mu = 0; mu < g.nd; ++mu)
			{
				size_t f = g.shift(r, mu, 1), b = g.shift(r, mu, -1);
				K += U[mu][r] * adj(h[f]);
				K += adj(U[mu][b]) * adj(h[b]);
			}
			h[r] = or_update(h[r] * K, h[r], T(omega));
		});
	}
}

template <class G> inline void reunitize_exact(Field<G> &h)
{
	site_loop(h.size(), [&](size_t i) { h[i] = project_on_group_exact(h[i]); });
}

// sweeps in blocks of check_every, exact reunitarisation and theta_ref after
// each block; stops when theta_ref < tol. Returns the number of sweeps.
template <class G>
inline int or_run(Grid const &g, GaugeField<G> const &U, Field<G> &h, double omega, double tol,
                  int max_sweeps, int check_every, double *theta)
{
	*theta = theta_fast(g, U, h);
	if (*theta < tol)
		return 0;
	int s = 0;
	while (s < max_sweeps)
	{
		for (int k = 0; k < check_every && s < max_sweeps; ++k, ++s)
			or_sweep(g, U, h, omega);
		reunitize_exact(h);
		*theta = theta_fast(g, U, h);
		if (*theta < tol)
			break;
	}
	return s;
}

// ---- DFT and Fourier acceleration -----------------------------------------

// unnormalised DFT along every axis of ncomp interleaved complex components;
// sign -1: forward (e^{-2 pi i k x / L}), +1: backward
inline void fft_nd(Grid const &g, int ncomp, double *data, int sign)
{
	using C = std::complex<double>;
	C *d = reinterpret_cast<C *>(data);
	for (int dir = 0; dir < g.nd; ++dir)
	{
		int L = g.L[dir];
		size_t stride = 1;
		for (int i = dir + 1; i < g.nd; ++i)
			stride *= size_t(g.L[i]);
		size_t outer = g.V / (size_t(L) * stride);
		std::vector<C> tw(L);
		for (int k = 0; k < L; ++k)
			tw[k] = std::polar(1.0, sign * 2.0 * M_PI * double(k) / double(L));
#pragma omp parallel for schedule(static)
		for (long long o = 0; o < (long long)outer; ++o)
		{
			std::vector<C> line(L), res(L);
			for (size_t in = 0; in < stride; ++in)
				for (int c = 0; c < ncomp; ++c)
				{
					size_t base = (size_t(o) * size_t(L) * stride + in) * size_t(ncomp) + size_t(c);
					for (int x = 0; x < L; ++x)
						line[x] = d[base + size_t(x) * stride * size_t(ncomp)];
					for (int k = 0; k < L; ++k)
					{
						C s = 0;
						for (int x = 0; x < L; ++x)
							s += line[x] * tw[(size_t(k) * size_t(x)) % size_t(L)];
						res[k] = s;
					}
					for (int k = 0; k < L; ++k)
						d[base + size_t(k) * stride * size_t(ncomp)] = res[k];
				}
		}
	}
}

// lattice momentum squared phat^2(k) = sum_mu 4 sin^2(pi k_mu / L_mu)
inline double phat2(Grid const &g, size_t r)
{
	int x[4];
	g.coords(r, x);
	double s = 0;
	for (int mu = 0; mu < g.nd; ++mu)
	{
		double t = std::sin(M_PI * double(x[mu]) / double(g.L[mu]));
		s += 4.0 * t * t;
	}
	return s;
}

// g <- exp(-alpha X) g with X = F^-1[mult * F[Delta]], then exact
// reunitarisation. Algebra reals are packed pairwise into complex fields.
template <class G>
inline void fa_step(Grid const &g, GaugeField<G> const &U, Field<G> &h, double const *mult, double alpha)
{
	using T = typename traits<G>::real;
	constexpr int na = traits<G>::nalg;
	constexpr int nc = (na + 1) / 2;
	auto D = divergence(g, U, h);
	std::vector<double> buf(g.V * nc * 2, 0.0);
	for (size_t r = 0; r < g.V; ++r)
	{
		T o[8];
		pack_alg(D[r], o);
		for (int a = 0; a < na; ++a)
			buf[(r * nc) * 2 + a] = double(o[a]);
	}
	fft_nd(g, nc, buf.data(), -1);
	for (size_t r = 0; r < g.V; ++r)
		for (int c = 0; c < 2 * nc; ++c)
			buf[r * nc * 2 + c] *= mult[r];
	fft_nd(g, nc, buf.data(), +1);
	double inv = 1.0 / double(g.V);
	site_loop(g.V, [&](size_t r) {
		T o[8];
		for (int a = 0; a < na; ++a)
			o[a] = T(-alpha * buf[(r * nc) * 2 + a] * inv);
		G X;
		unpack_alg(o, X);
		h[r] = project_on_group_exact(gexp(X) * h[r]);
	});
}

// ---- MLP of the learned multiplier -----------------------------------------
// params (float32): W1[w][3] b1[w] W2[w][w] b2[w] W3[w] b3
// h1 = tanh(W1 x + b1), h2 = tanh(W2 h1 + b2), y = W3 . h2 + b3
inline void mlp_forward(int n, float const *x, float const *p, int w, float *y)
{
	float const *W1 = p, *b1 = W1 + 3 * w, *W2 = b1 + w, *b2 = W2 + w * w, *W3 = b2 + w, *b3 = W3 + w;
	for (int s = 0; s < n; ++s)
	{
		std::vector<double> h1(w), h2(w);
		for (int i = 0; i < w; ++i)
		{
			double a = b1[i];
			for (int k = 0; k < 3; ++k)
				a += double(W1[3 * i + k]) * double(x[3 * s + k]);
			h1[i] = std::tanh(a);
		}
		double out = b3[0];
		for (int i = 0; i < w; ++i)
		{
			double a = b2[i];
			for (int k = 0; k < w; ++k)
				a += double(W2[w * i + k]) * h1[k];
			h2[i] = std::tanh(a);
			out += double(W3[i]) * h2[i];
		}
		y[s] = float(out);
	}
}

// mean squared error over n samples and its gradient (double) w.r.t. params
inline double mlp_loss_grad(int n, float const *x, float const *t, float const *p, int w, double *grad)
{
	float const *W1 = p, *b1 = W1 + 3 * w, *W2 = b1 + w, *b2 = W2 + w * w, *W3 = b2 + w, *b3 = W3 + w;
	int np = 3 * w + w + w * w + w + w + 1;
	std::fill(grad, grad + np, 0.0);
	double *gW1 = grad, *gb1 = gW1 + 3 * w, *gW2 = gb1 + w, *gb2 = gW2 + w * w, *gW3 = gb2 + w, *gb3 = gW3 + w;
	double loss = 0;
	std::vector<double> h1(w), h2(w), d2(w), d1(w);
	for (int s = 0; s < n; ++s)
	{
		for (int i = 0; i < w; ++i)
		{
			double a = b1[i];
			for (int k = 0; k < 3; ++k)
				a += double(W1[3 * i + k]) * double(x[3 * s + k]);
			h1[i] = std::tanh(a);
		}
		double out = b3[0];
		for (int i = 0; i < w; ++i)
		{
			double a = b2[i];
			for (int k = 0; k < w; ++k)
				a += double(W2[w * i + k]) * h1[k];
			h2[i] = std::tanh(a);
			out += double(W3[i]) * h2[i];
		}
		double e = out - double(t[s]);
		loss += e * e;
		double dy = 2.0 * e / n;
		gb3[0] += dy;
		for (int i = 0; i < w; ++i)
		{
			gW3[i] += dy * h2[i];
			d2[i] = dy * double(W3[i]) * (1.0 - h2[i] * h2[i]);
			gb2[i] += d2[i];
		}
		for (int k = 0; k < w; ++k)
		{
			double a = 0;
			for (int i = 0; i < w; ++i)
			{
				gW2[w * i + k] += d2[i] * h1[k];
				a += d2[i] * double(W2[w * i + k]);
			}
			d1[k] = a * (1.0 - h1[k] * h1[k]);
		}
		for (int i = 0; i < w; ++i)
		{
			gb1[i] += d1[i];
			for (int k = 0; k < 3; ++k)
				gW1[3 * i + k] += d1[i] * double(x[3 * s + k]);
		}
	}
	return loss / n;
}

} // namespace oracle
