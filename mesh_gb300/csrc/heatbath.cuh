// Heat-bath and overrelaxation link updates of the Wilson action: the
// legacy WilsonAction::sweep (src/old/wilson.cpp:15-60) and
// GaugeAction::thermalize / overrelax (src/old/mesh/gauge_action.h:42-73),
// which update one link at a time from its staple sum S:
//   U(1), SU(2): U' = X v^dagger with v = S / |S| and X drawn with density
//                exp(alpha Re X) (alpha = beta |S|);
//   SU(3):       three SU(2) subgroups in turn (Cabibbo & Marinari, Phys.
//                Lett. B 119 (1982) 387): with W = U S and the SU(2)-like
//                part k v of a 2x2 block of W, U' = (X v^dagger) U with
//                alpha = 2 beta k / 3, then project_on_group_fast;
//   overrelaxation: the reflection that keeps ReTr(U S): U(1)/SU(2)
//                U' = v^dagger U^dagger v^dagger, SU(3) per subgroup
//                U' = (v^dagger)^2 U (the legacy applies the SU(2) formula to
//                the whole SU(3) matrix, which does not keep the action; the
//                subgroup form does).
// Samplers, written from the published methods: SU(2) X_0 with density
// sqrt(1 - x^2) exp(alpha x) by Kennedy & Pendleton, Phys. Lett. B 156 (1985)
// 393 for alpha >= 1 and by Creutz, Phys. Rev. D 21 (1980) 2308 (inverse CDF
// of exp(alpha x), accepted with sqrt(1 - x^2)) below; U(1) angles from the
// von Mises distribution by Best & Fisher, Appl. Statist. 28 (1979) 152.
// The decisions run in double precision for every link precision.
//
// Random numbers: Philox with the tag 5, the lexicographic site, the
// direction, the SU(2) subgroup and a call index (0: the direction of X,
// 1 + 2a and 2 + 2a: the four uniforms of attempt a), counter = the sweep
// number, so a sweep is reproducible and independent of the launch shape.
// After kHbTries rejected attempts the subgroup update is skipped (the link
// keeps its value, which leaves the heat-bath distribution invariant).
#pragma once

#include "group.cuh"
#include "rng.cuh"

namespace meshgb {

constexpr uint32_t TAG_HEATBATH = 5;
constexpr int kHbTries = 24;

MESH_HD void hb_uniforms(uint64_t seed, uint32_t site, uint32_t mu, uint32_t sub, uint32_t call, uint64_t ctr,
                         double *u)
{
	U4 r = philox4x32_10(site, (TAG_HEATBATH << 24) | (mu << 8) | (sub << 6) | call, uint32_t(ctr),
	                     uint32_t(ctr >> 32), uint32_t(seed), uint32_t(seed >> 32));
	u[0] = u53(r.v[0], r.v[1]);
	u[1] = u53(r.v[2], r.v[3]);
}

MESH_HD double hb_cospi(double x)
{
#ifdef __CUDA_ARCH__
	return cospi(x);
#else
	return std::cos(M_PI * x);
#endif
}
MESH_HD void hb_sincospi(double x, double *s, double *c)
{
#ifdef __CUDA_ARCH__
	sincospi(x, s, c);
#else
	*s = std::sin(M_PI * x);
	*c = std::cos(M_PI * x);
#endif
}

struct HbStream
{
	uint64_t seed, ctr;
	uint32_t site, mu, sub;
	MESH_HD void draw(uint32_t call, double *u) const { hb_uniforms(seed, site, mu, sub, call, ctr, u); }
};

// X in SU(2) as (x0, x1, x2, x3) with density exp(alpha x0) under the Haar
// measure; false when every attempt was rejected
MESH_HD bool su2_sample(double alpha, HbStream const &rs, double *x)
{
	double x0 = 0;
	bool ok = false;
	for (int a = 0; a < kHbTries && !ok; ++a)
	{
		double u[4];
		rs.draw(uint32_t(1 + 2 * a), u);
		rs.draw(uint32_t(2 + 2 * a), u + 2);
		if (alpha < 1.0)
		{
			double t = alpha < 1e-8 ? 2.0 * u[0] - 1.0 : 1.0 + log(u[0] + (1.0 - u[0]) * exp(-2.0 * alpha)) / alpha;
			if (u[1] * u[1] <= 1.0 - t * t)
			{
				x0 = t;
				ok = true;
			}
		}
		else
		{
			double c = hb_cospi(2.0 * u[1]);
			double d = -(log(u[0]) + c * c * log(u[2])) / alpha;
			if (u[3] * u[3] <= 1.0 - 0.5 * d)
			{
				x0 = 1.0 - d;
				ok = true;
			}
		}
	}
	if (!ok)
		return false;
	double u[2];
	rs.draw(0, u);
	double ct = 2.0 * u[0] - 1.0;
	double st = sqrt(fmax(0.0, 1.0 - ct * ct));
	double sp, cp;
	hb_sincospi(2.0 * u[1], &sp, &cp);
	double r = sqrt(fmax(0.0, 1.0 - x0 * x0));
	x[0] = x0;
	x[1] = r * st * cp;
	x[2] = r * st * sp;
	x[3] = r * ct;
	return true;
}

// angle with density exp(kappa cos theta) on (-pi, pi]
MESH_HD bool u1_sample(double kappa, HbStream const &rs, double *theta)
{
	if (kappa < 1e-8)
	{
		double u[2];
		rs.draw(1, u);
		*theta = M_PI * (2.0 * u[0] - 1.0);
		return true;
	}
	double tau = 1.0 + sqrt(1.0 + 4.0 * kappa * kappa);
	double rho = (tau - sqrt(2.0 * tau)) / (2.0 * kappa);
	double r = (1.0 + rho * rho) / (2.0 * rho);
	for (int a = 0; a < kHbTries; ++a)
	{
		double u[4];
		rs.draw(uint32_t(1 + 2 * a), u);
		rs.draw(uint32_t(2 + 2 * a), u + 2);
		double z = hb_cospi(u[0]);
		double f = (1.0 + r * z) / (r + z);
		double c = kappa * (r - f);
		if (c * (2.0 - c) - u[1] > 0.0 || log(c / u[1]) + 1.0 - c >= 0.0)
		{
			f = fmin(1.0, fmax(-1.0, f));
			*theta = (u[2] > 0.5 ? 1.0 : -1.0) * acos(f);
			return true;
		}
	}
	return false;
}

template <int GRP, class T> struct HbUpdate;

template <class T> struct HbUpdate<U1, T>
{
	using E = typename Group<U1, T>::E;
	MESH_HD static void heatbath(E &u, E const &S, double beta, HbStream rs)
	{
		double sr = double(S.v[0]), si = double(S.v[1]);
		double k = sqrt(sr * sr + si * si);
		double th;
		if (!u1_sample(beta * k, rs, &th))
			return;
		double s, c;
		hb_sincospi(th / M_PI, &s, &c);
		// U' = e^{i th} conj(v), v = S / k (k = 0: v = 1)
		double vr = k > 0 ? sr / k : 1.0, vi = k > 0 ? si / k : 0.0;
		u.v[0] = T(c * vr + s * vi);
		u.v[1] = T(s * vr - c * vi);
	}
	MESH_HD static void overrelax(E &u, E const &S)
	{
		double sr = double(S.v[0]), si = double(S.v[1]);
		double k = sqrt(sr * sr + si * si);
		if (!(k > 0))
			return;
		// U' = conj(v)^2 conj(U)
		double vr = sr / k, vi = -si / k;
		double wr = vr * vr - vi * vi, wi = 2 * vr * vi;
		double ur = double(u.v[0]), ui = -double(u.v[1]);
		u.v[0] = T(wr * ur - wi * ui);
		u.v[1] = T(wr * ui + wi * ur);
	}
};

template <class T> struct HbUpdate<SU2, T>
{
	using Gp = Group<SU2, T>;
	using E = typename Gp::E;
	MESH_HD static void heatbath(E &u, E const &S, double beta, HbStream rs)
	{
		double s[4] = {double(S.v[0]), double(S.v[1]), double(S.v[2]), double(S.v[3])};
		double k = sqrt(s[0] * s[0] + s[1] * s[1] + s[2] * s[2] + s[3] * s[3]);
		double x[4];
		if (!su2_sample(beta * k, rs, x))
			return;
		E X = {{T(x[0]), T(x[1]), T(x[2]), T(x[3])}};
		E v = k > 0 ? E{{T(s[0] / k), T(s[1] / k), T(s[2] / k), T(s[3] / k)}} : Gp::unit();
		u = Gp::reunit_fast(Gp::mul(X, Gp::adj(v)));
	}
	MESH_HD static void overrelax(E &u, E const &S)
	{
		double k = sqrt(double(S.v[0]) * S.v[0] + double(S.v[1]) * S.v[1] + double(S.v[2]) * S.v[2] +
		                double(S.v[3]) * S.v[3]);
		if (!(k > 0))
			return;
		E vd = Gp::adj(E{{T(S.v[0] / k), T(S.v[1] / k), T(S.v[2] / k), T(S.v[3] / k)}});
		u = Gp::reunit_fast(Gp::mul(Gp::mul(vd, Gp::adj(u)), vd));
	}
};

template <class T> struct HbUpdate<SU3, T>
{
	using Gp = Group<SU3, T>;
	using E = typename Gp::E;
	// rows (i, j) of the three SU(2) subgroups
	MESH_HD static void sub_rows(int k, int &i, int &j)
	{
		i = k == 1 ? 1 : 0;
		j = k == 0 ? 1 : 2;
	}
	// SU(2)-like part (a, b) of the 2x2 block (i, j) of W: [[a, b], [-b*, a*]]
	MESH_HD static void block(E const &W, int i, int j, double *a, double *b)
	{
		a[0] = 0.5 * (double(W.v[6 * i + 2 * i]) + double(W.v[6 * j + 2 * j]));
		a[1] = 0.5 * (double(W.v[6 * i + 2 * i + 1]) - double(W.v[6 * j + 2 * j + 1]));
		b[0] = 0.5 * (double(W.v[6 * i + 2 * j]) - double(W.v[6 * j + 2 * i]));
		b[1] = 0.5 * (double(W.v[6 * i + 2 * j + 1]) + double(W.v[6 * j + 2 * i + 1]));
	}
	// rows i, j of M <- R rows, R = [[p, q], [-q*, p*]]
	MESH_HD static void left_mul(E &M, int i, int j, double const *p, double const *q)
	{
#pragma unroll
		for (int c = 0; c < 3; ++c)
		{
			double xr = M.v[6 * i + 2 * c], xi = M.v[6 * i + 2 * c + 1];
			double yr = M.v[6 * j + 2 * c], yi = M.v[6 * j + 2 * c + 1];
			M.v[6 * i + 2 * c] = T(p[0] * xr - p[1] * xi + q[0] * yr - q[1] * yi);
			M.v[6 * i + 2 * c + 1] = T(p[0] * xi + p[1] * xr + q[0] * yi + q[1] * yr);
			// -q* x + p* y
			M.v[6 * j + 2 * c] = T(-(q[0] * xr + q[1] * xi) + p[0] * yr + p[1] * yi);
			M.v[6 * j + 2 * c + 1] = T(-(q[0] * xi - q[1] * xr) + p[0] * yi - p[1] * yr);
		}
	}
	// R = X v^dagger for X = (x0..x3) <-> [[x0 + i x3, x2 + i x1], ...] and
	// v = (a, b) / k
	MESH_HD static void times_vdag(double const *x, double const *a, double const *b, double k, double *p, double *q)
	{
		double xp[2] = {x[0], x[3]}, xq[2] = {x[2], x[1]};
		double ar = a[0] / k, ai = a[1] / k, br = b[0] / k, bi = b[1] / k;
		// v^dagger = [[a*, -b], [b*, a]]: p = xp a* + xq b*, q = -xp b + xq a
		p[0] = xp[0] * ar + xp[1] * ai + xq[0] * br + xq[1] * bi;
		p[1] = xp[1] * ar - xp[0] * ai + xq[1] * br - xq[0] * bi;
		q[0] = -(xp[0] * br - xp[1] * bi) + xq[0] * ar - xq[1] * ai;
		q[1] = -(xp[0] * bi + xp[1] * br) + xq[0] * ai + xq[1] * ar;
	}
	MESH_HD static void heatbath(E &u, E const &S, double beta, HbStream rs)
	{
		E W = Gp::mul(u, S);
		for (int sg = 0; sg < 3; ++sg)
		{
			int i, j;
			sub_rows(sg, i, j);
			double a[2], b[2];
			block(W, i, j, a, b);
			double k = sqrt(a[0] * a[0] + a[1] * a[1] + b[0] * b[0] + b[1] * b[1]);
			rs.sub = uint32_t(sg);
			double x[4];
			if (!(k > 0) || !su2_sample(2.0 * beta * k / 3.0, rs, x))
				continue;
			double p[2], q[2];
			times_vdag(x, a, b, k, p, q);
			left_mul(u, i, j, p, q);
			left_mul(W, i, j, p, q);
		}
		u = Gp::reunit_fast(u);
	}
	MESH_HD static void overrelax(E &u, E const &S)
	{
		E W = Gp::mul(u, S);
		for (int sg = 0; sg < 3; ++sg)
		{
			int i, j;
			sub_rows(sg, i, j);
			double a[2], b[2];
			block(W, i, j, a, b);
			double k = sqrt(a[0] * a[0] + a[1] * a[1] + b[0] * b[0] + b[1] * b[1]);
			if (!(k > 0))
				continue;
			// R = (v^dagger)^2 = X v^dagger with X = v^dagger
			double x[4] = {a[0] / k, -b[1] / k, -b[0] / k, -a[1] / k};
			double p[2], q[2];
			times_vdag(x, a, b, k, p, q);
			left_mul(u, i, j, p, q);
			left_mul(W, i, j, p, q);
		}
		u = Gp::reunit_fast(u);
	}
};

} // namespace meshgb
