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
// The samplers and the subgroup arithmetic run in the links' precision
// (FP64 links: double, matching the oracle draw for draw; FP32 links: float,
// as the GPU's FP64 rate is a small fraction of its FP32 rate).
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

template <class R> MESH_HD R hb_cospi(R x)
{
#ifdef __CUDA_ARCH__
	if constexpr (sizeof(R) == 4)
		return cospif(x);
	else
		return cospi(x);
#else
	return R(std::cos(M_PI * double(x)));
#endif
}
template <class R> MESH_HD void hb_sincospi(R x, R *s, R *c)
{
#ifdef __CUDA_ARCH__
	if constexpr (sizeof(R) == 4)
		sincospif(x, s, c);
	else
		sincospi(x, s, c);
#else
	*s = R(std::sin(M_PI * double(x)));
	*c = R(std::cos(M_PI * double(x)));
#endif
}

struct HbStream
{
	uint64_t seed, ctr;
	uint32_t site, mu, sub;
	template <class R> MESH_HD void draw(uint32_t call, R *u) const
	{
		double d[2];
		hb_uniforms(seed, site, mu, sub, call, ctr, d);
		u[0] = R(d[0]);
		u[1] = R(d[1]);
	}
};

// X in SU(2) as (x0, x1, x2, x3) with density exp(alpha x0) under the Haar
// measure; false when every attempt was rejected
template <class R> MESH_HD bool su2_sample(R alpha, HbStream const &rs, R *x)
{
	R x0 = 0;
	bool ok = false;
	for (int a = 0; a < kHbTries && !ok; ++a)
	{
		R u[4];
		rs.draw(uint32_t(1 + 2 * a), u);
		rs.draw(uint32_t(2 + 2 * a), u + 2);
		if (alpha < R(1))
		{
			R t = alpha < R(1e-8) ? R(2) * u[0] - R(1) : R(1) + log(u[0] + (R(1) - u[0]) * exp(R(-2) * alpha)) / alpha;
			if (u[1] * u[1] <= R(1) - t * t)
			{
				x0 = t;
				ok = true;
			}
		}
		else
		{
			R c = hb_cospi(R(2) * u[1]);
			R d = -(log(u[0]) + c * c * log(u[2])) / alpha;
			if (u[3] * u[3] <= R(1) - R(0.5) * d)
			{
				x0 = R(1) - d;
				ok = true;
			}
		}
	}
	if (!ok)
		return false;
	R u[2];
	rs.draw(0, u);
	R ct = R(2) * u[0] - R(1);
	R st = sqrt(fmax(R(0), R(1) - ct * ct));
	R sp, cp;
	hb_sincospi(R(2) * u[1], &sp, &cp);
	R r = sqrt(fmax(R(0), R(1) - x0 * x0));
	x[0] = x0;
	x[1] = r * st * cp;
	x[2] = r * st * sp;
	x[3] = r * ct;
	return true;
}

// angle with density exp(kappa cos theta) on (-pi, pi], returned as its
// cosine and sine
template <class R> MESH_HD bool u1_sample(R kappa, HbStream const &rs, R *cs, R *sn)
{
	if (kappa < R(1e-8))
	{
		R u[2];
		rs.draw(1, u);
		hb_sincospi(R(2) * u[0] - R(1), sn, cs);
		return true;
	}
	R tau = R(1) + sqrt(R(1) + R(4) * kappa * kappa);
	R rho = (tau - sqrt(R(2) * tau)) / (R(2) * kappa);
	R r = (R(1) + rho * rho) / (R(2) * rho);
	for (int a = 0; a < kHbTries; ++a)
	{
		R u[4];
		rs.draw(uint32_t(1 + 2 * a), u);
		rs.draw(uint32_t(2 + 2 * a), u + 2);
		R z = hb_cospi(u[0]);
		R f = (R(1) + r * z) / (r + z);
		R c = kappa * (r - f);
		if (c * (R(2) - c) - u[1] > R(0) || log(c / u[1]) + R(1) - c >= R(0))
		{
			f = fmin(R(1), fmax(R(-1), f));
			*cs = f;
			*sn = (u[2] > R(0.5) ? R(1) : R(-1)) * sqrt(fmax(R(0), R(1) - f * f));
			return true;
		}
	}
	return false;
}

template <int GRP, class T> struct HbUpdate;

template <class T> struct HbUpdate<U1, T>
{
	using E = typename Group<U1, T>::E;
	MESH_HD static void heatbath(E &u, E const &S, T beta, HbStream rs)
	{
		T sr = S.v[0], si = S.v[1];
		T k = sqrt(sr * sr + si * si);
		T c, s;
		if (!u1_sample(beta * k, rs, &c, &s))
			return;
		// U' = e^{i th} conj(v), v = S / k (k = 0: v = 1)
		T vr = k > T(0) ? sr / k : T(1), vi = k > T(0) ? si / k : T(0);
		u.v[0] = c * vr + s * vi;
		u.v[1] = s * vr - c * vi;
	}
	MESH_HD static void overrelax(E &u, E const &S)
	{
		T sr = S.v[0], si = S.v[1];
		T k = sqrt(sr * sr + si * si);
		if (!(k > T(0)))
			return;
		// U' = conj(v)^2 conj(U)
		T vr = sr / k, vi = -si / k;
		T wr = vr * vr - vi * vi, wi = T(2) * vr * vi;
		T ur = u.v[0], ui = -u.v[1];
		u.v[0] = wr * ur - wi * ui;
		u.v[1] = wr * ui + wi * ur;
	}
};

template <class T> struct HbUpdate<SU2, T>
{
	using Gp = Group<SU2, T>;
	using E = typename Gp::E;
	MESH_HD static void heatbath(E &u, E const &S, T beta, HbStream rs)
	{
		T k = sqrt(S.v[0] * S.v[0] + S.v[1] * S.v[1] + S.v[2] * S.v[2] + S.v[3] * S.v[3]);
		T x[4];
		if (!su2_sample(beta * k, rs, x))
			return;
		E X = {{x[0], x[1], x[2], x[3]}};
		E v = k > T(0) ? E{{S.v[0] / k, S.v[1] / k, S.v[2] / k, S.v[3] / k}} : Gp::unit();
		u = Gp::reunit_fast(Gp::mul(X, Gp::adj(v)));
	}
	MESH_HD static void overrelax(E &u, E const &S)
	{
		T k = sqrt(S.v[0] * S.v[0] + S.v[1] * S.v[1] + S.v[2] * S.v[2] + S.v[3] * S.v[3]);
		if (!(k > T(0)))
			return;
		E vd = Gp::adj(E{{S.v[0] / k, S.v[1] / k, S.v[2] / k, S.v[3] / k}});
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
	MESH_HD static void block(E const &W, int i, int j, T *a, T *b)
	{
		a[0] = T(0.5) * (T(W.v[6 * i + 2 * i]) + T(W.v[6 * j + 2 * j]));
		a[1] = T(0.5) * (T(W.v[6 * i + 2 * i + 1]) - T(W.v[6 * j + 2 * j + 1]));
		b[0] = T(0.5) * (T(W.v[6 * i + 2 * j]) - T(W.v[6 * j + 2 * i]));
		b[1] = T(0.5) * (T(W.v[6 * i + 2 * j + 1]) + T(W.v[6 * j + 2 * i + 1]));
	}
	// rows i, j of M <- R rows, R = [[p, q], [-q*, p*]]
	MESH_HD static void left_mul(E &M, int i, int j, T const *p, T const *q)
	{
#pragma unroll
		for (int c = 0; c < 3; ++c)
		{
			T xr = M.v[6 * i + 2 * c], xi = M.v[6 * i + 2 * c + 1];
			T yr = M.v[6 * j + 2 * c], yi = M.v[6 * j + 2 * c + 1];
			M.v[6 * i + 2 * c] = p[0] * xr - p[1] * xi + q[0] * yr - q[1] * yi;
			M.v[6 * i + 2 * c + 1] = p[0] * xi + p[1] * xr + q[0] * yi + q[1] * yr;
			// -q* x + p* y
			M.v[6 * j + 2 * c] = -(q[0] * xr + q[1] * xi) + p[0] * yr + p[1] * yi;
			M.v[6 * j + 2 * c + 1] = -(q[0] * xi - q[1] * xr) + p[0] * yi - p[1] * yr;
		}
	}
	// R = X v^dagger for X = (x0..x3) <-> [[x0 + i x3, x2 + i x1], ...] and
	// v = (a, b) / k
	MESH_HD static void times_vdag(T const *x, T const *a, T const *b, T k, T *p, T *q)
	{
		T xp[2] = {x[0], x[3]}, xq[2] = {x[2], x[1]};
		T ar = a[0] / k, ai = a[1] / k, br = b[0] / k, bi = b[1] / k;
		// v^dagger = [[a*, -b], [b*, a]]: p = xp a* + xq b*, q = -xp b + xq a
		p[0] = xp[0] * ar + xp[1] * ai + xq[0] * br + xq[1] * bi;
		p[1] = xp[1] * ar - xp[0] * ai + xq[1] * br - xq[0] * bi;
		q[0] = -(xp[0] * br - xp[1] * bi) + xq[0] * ar - xq[1] * ai;
		q[1] = -(xp[0] * bi + xp[1] * br) + xq[0] * ai + xq[1] * ar;
	}
	MESH_HD static void heatbath(E &u, E const &S, T beta, HbStream rs)
	{
		E W = Gp::mul(u, S);
		for (int sg = 0; sg < 3; ++sg)
		{
			int i, j;
			sub_rows(sg, i, j);
			T a[2], b[2];
			block(W, i, j, a, b);
			T k = sqrt(a[0] * a[0] + a[1] * a[1] + b[0] * b[0] + b[1] * b[1]);
			rs.sub = uint32_t(sg);
			T x[4];
			if (!(k > T(0)) || !su2_sample(T(2) * beta * k / T(3), rs, x))
				continue;
			T p[2], q[2];
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
			T a[2], b[2];
			block(W, i, j, a, b);
			T k = sqrt(a[0] * a[0] + a[1] * a[1] + b[0] * b[0] + b[1] * b[1]);
			if (!(k > T(0)))
				continue;
			// R = (v^dagger)^2 = X v^dagger with X = v^dagger
			T x[4] = {a[0] / k, -b[1] / k, -b[0] / k, -a[1] / k};
			T p[2], q[2];
			times_vdag(x, a, b, k, p, q);
			left_mul(u, i, j, p, q);
			left_mul(W, i, j, p, q);
		}
		u = Gp::reunit_fast(u);
	}
};

} // namespace meshgb
