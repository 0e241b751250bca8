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
//   * heat-bath and overrelaxation sweeps of the Wilson action, checkerboard
//     order (direction, then parity), with the per-link updates of the legacy
//     src/old/wilson.cpp:15-60 and src/old/mesh/gauge_action.h:42-73: SU(2)
//     Kennedy & Pendleton (Phys. Lett. B 156 (1985) 393) / Creutz (Phys. Rev.
//     D 21 (1980) 2308), U(1) von Mises by Best & Fisher (Appl. Statist. 28
//     (1979) 152), SU(3) by Cabibbo-Marinari subgroups; the same Philox streams
//     as the device;
//   * rectangular Wilson loops r x t in the planes (mu, 3), mu < 3, as in the
//     legacy src/old/mesh/wilson.cpp:40-75 (spatial line of r links, temporal
//     line of t links; sum over sites and the three spatial directions),
//     normalised like the plaquette (ReTr / Nc), every loop walked link by
//     link.
#pragma once

#include "oracle.hpp"

#include <complex>

namespace oracle {

// ---- heat-bath and overrelaxation -------------------------------------------

constexpr uint32_t TAG_HEATBATH = 5;
constexpr int HB_TRIES = 24;

struct hb_stream
{
	uint64_t seed, ctr;
	uint32_t site, mu, sub;
	void draw(uint32_t call, double *u) const
	{
		auto r = philox4x32_10(site, (TAG_HEATBATH << 24) | (mu << 8) | (sub << 6) | call, uint32_t(ctr),
		                       uint32_t(ctr >> 32), uint32_t(seed), uint32_t(seed >> 32));
		u[0] = u53(r.v[0], r.v[1]);
		u[1] = u53(r.v[2], r.v[3]);
	}
};

// X = (x0, x1, x2, x3) in SU(2) with density exp(alpha x0) (Haar measure)
inline bool hb_su2(double alpha, hb_stream const &rs, double *x)
{
	double x0 = 0;
	bool ok = false;
	for (int a = 0; a < HB_TRIES && !ok; ++a)
	{
		double u[4];
		rs.draw(uint32_t(1 + 2 * a), u);
		rs.draw(uint32_t(2 + 2 * a), u + 2);
		if (alpha < 1.0)
		{
			// Creutz: x from the density exp(alpha x) by inversion, accepted
			// with probability sqrt(1 - x^2)
			double t = alpha < 1e-8 ? 2.0 * u[0] - 1.0
			                        : 1.0 + std::log(u[0] + (1.0 - u[0]) * std::exp(-2.0 * alpha)) / alpha;
			if (u[1] * u[1] <= 1.0 - t * t)
				x0 = t, ok = true;
		}
		else
		{
			// Kennedy-Pendleton in delta = 1 - x0
			double c = std::cos(M_PI * 2.0 * u[1]);
			double d = -(std::log(u[0]) + c * c * std::log(u[2])) / alpha;
			if (u[3] * u[3] <= 1.0 - 0.5 * d)
				x0 = 1.0 - d, ok = true;
		}
	}
	if (!ok)
		return false;
	double u[2];
	rs.draw(0, u);
	double ct = 2.0 * u[0] - 1.0, st = std::sqrt(std::max(0.0, 1.0 - ct * ct));
	double sp = std::sin(M_PI * 2.0 * u[1]), cp = std::cos(M_PI * 2.0 * u[1]);
	double r = std::sqrt(std::max(0.0, 1.0 - x0 * x0));
	x[0] = x0;
	x[1] = r * st * cp;
	x[2] = r * st * sp;
	x[3] = r * ct;
	return true;
}

// von Mises angle, density exp(kappa cos theta) (Best & Fisher), returned
// as its cosine and sine
inline bool hb_u1(double kappa, hb_stream const &rs, double *cs, double *sn)
{
	if (kappa < 1e-8)
	{
		double u[2];
		rs.draw(1, u);
		*sn = std::sin(M_PI * (2.0 * u[0] - 1.0));
		*cs = std::cos(M_PI * (2.0 * u[0] - 1.0));
		return true;
	}
	double tau = 1.0 + std::sqrt(1.0 + 4.0 * kappa * kappa);
	double rho = (tau - std::sqrt(2.0 * tau)) / (2.0 * kappa);
	double r = (1.0 + rho * rho) / (2.0 * rho);
	for (int a = 0; a < HB_TRIES; ++a)
	{
		double u[4];
		rs.draw(uint32_t(1 + 2 * a), u);
		rs.draw(uint32_t(2 + 2 * a), u + 2);
		double z = std::cos(M_PI * u[0]);
		double f = (1.0 + r * z) / (r + z);
		double c = kappa * (r - f);
		if (c * (2.0 - c) - u[1] > 0.0 || std::log(c / u[1]) + 1.0 - c >= 0.0)
		{
			f = std::min(1.0, std::max(-1.0, f));
			*cs = f;
			*sn = (u[2] > 0.5 ? 1.0 : -1.0) * std::sqrt(std::max(0.0, 1.0 - f * f));
			return true;
		}
	}
	return false;
}

// one link: heat-bath (or, with OR, the action-keeping reflection) from the
// staple sum S
template <class T> inline void hb_link(cplx<T> &u, cplx<T> const &S, double beta, hb_stream rs, bool OR)
{
	double sr = S.re, si = S.im, k = std::sqrt(sr * sr + si * si);
	if (OR)
	{
		if (!(k > 0))
			return;
		// U' = conj(v)^2 conj(U)
		std::complex<double> v(sr / k, si / k), uu(u.re, u.im);
		std::complex<double> r = std::conj(v) * std::conj(v) * std::conj(uu);
		u = {T(r.real()), T(r.imag())};
		return;
	}
	double cs, sn;
	if (!hb_u1(beta * k, rs, &cs, &sn))
		return;
	std::complex<double> v = k > 0 ? std::complex<double>(sr / k, si / k) : std::complex<double>(1, 0);
	std::complex<double> r = std::complex<double>(cs, sn) * std::conj(v);
	u = {T(r.real()), T(r.imag())};
}
template <class T> inline void hb_link(quat<T> &u, quat<T> const &S, double beta, hb_stream rs, bool OR)
{
	double k = std::sqrt(double(S.re) * S.re + double(S.im1) * S.im1 + double(S.im2) * S.im2 + double(S.im3) * S.im3);
	if (OR)
	{
		if (!(k > 0))
			return;
		quat<T> vd = conj(quat<T>{T(S.re / k), T(S.im1 / k), T(S.im2 / k), T(S.im3 / k)});
		u = project_on_group_fast(vd * conj(u) * vd);
		return;
	}
	double x[4];
	if (!hb_su2(beta * k, rs, x))
		return;
	quat<T> X{T(x[0]), T(x[1]), T(x[2]), T(x[3])};
	quat<T> v = k > 0 ? quat<T>{T(S.re / k), T(S.im1 / k), T(S.im2 / k), T(S.im3 / k)} : unit<quat<T>>();
	u = project_on_group_fast(X * conj(v));
}
template <class T> inline void hb_link(mat3<T> &u, mat3<T> const &S, double beta, hb_stream rs, bool OR)
{
	using C = std::complex<double>;
	auto W = u * S;
	static const int SI[3] = {0, 1, 0}, SJ[3] = {1, 2, 2};
	for (int sg = 0; sg < 3; ++sg)
	{
		int i = SI[sg], j = SJ[sg];
		// SU(2)-like part [[A, B], [-B*, A*]] of the block (i, j) of W
		C A = 0.5 * (C(W.m[i][i].re, W.m[i][i].im) + std::conj(C(W.m[j][j].re, W.m[j][j].im)));
		C B = 0.5 * (C(W.m[i][j].re, W.m[i][j].im) - std::conj(C(W.m[j][i].re, W.m[j][i].im)));
		double k = std::sqrt(std::norm(A) + std::norm(B));
		if (!(k > 0))
			continue;
		A /= k;
		B /= k;
		C xp, xq; // X = [[xp, xq], [-xq*, xp*]]
		if (OR)
		{
			xp = std::conj(A); // X = v^dagger
			xq = -B;
		}
		else
		{
			rs.sub = uint32_t(sg);
			double x[4];
			if (!hb_su2(2.0 * beta * k / 3.0, rs, x))
				continue;
			xp = C(x[0], x[3]);
			xq = C(x[2], x[1]);
		}
		// R = X v^dagger, v^dagger = [[A*, -B], [B*, A]]
		C p = xp * std::conj(A) + xq * std::conj(B);
		C q = -xp * B + xq * A;
		auto left = [&](mat3<T> &M) {
			for (int c = 0; c < 3; ++c)
			{
				C x(M.m[i][c].re, M.m[i][c].im), y(M.m[j][c].re, M.m[j][c].im);
				C nx = p * x + q * y, ny = -std::conj(q) * x + std::conj(p) * y;
				M.m[i][c] = {T(nx.real()), T(nx.imag())};
				M.m[j][c] = {T(ny.real()), T(ny.imag())};
			}
		};
		left(u);
		left(W);
	}
	u = project_on_group_fast(u);
}

// one sweep: for mu, for parity (0, 1), every link (x, mu) with parity(x) =
// parity from the staples of the current links; counter = sweep number
template <class G>
inline void gauge_sweep(Grid const &g, GaugeField<G> &U, double beta, uint64_t seed, uint64_t ctr, bool OR)
{
	for (int mu = 0; mu < g.nd; ++mu)
		for (int par = 0; par < 2; ++par)
		{
			auto S = stapleSum(g, U, mu);
			site_loop(g.V, [&](size_t r) {
				int x[4];
				g.coords(r, x);
				int p = 0;
				for (int i = 0; i < g.nd; ++i)
					p += x[i];
				if ((p & 1) != par)
					return;
				hb_link(U[mu][r], S[r], beta, hb_stream{seed, ctr, uint32_t(r), uint32_t(mu), 0}, OR);
			});
		}
}

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
