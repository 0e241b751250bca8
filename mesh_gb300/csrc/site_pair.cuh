// Thread-per-site momentum step for SU(3) in FP32 with two independent
// matrix products in the two lanes of every FP32x2 operation.
//
// The same operation as site_md (the reference's momentum step of runHmd,
// src/gauge/hmc.h:54-58, with wilsonDeriv/stapleSum of
// src/gauge/utils.h:114-153, fused with evolve, src/gauge/hmc.h:26-36), with
// the site's work paired:
//   * forward plaquette loops: planes q and q + 3 ((0,1)&(1,2), (0,2)&(1,3),
//     (0,3)&(2,3));
//   * lower staples: links (x, mu) and (x, mu + 2), the three staples of each
//     in step;
//   * link update: directions mu and mu + 2.
// A pair matrix holds the real parts of both products' entries in float2
// lanes (x: first, y: second) and the imaginary parts likewise, so every
// complex multiply-add is FP32x2 FMAs on whole registers: no lane broadcast
// or swap is built per product, as the one-product FP32x2 form
// (Su3F2::prod) must. The cost is one packing of the two loaded links per
// pair. Projections are formed from the entries they read only (9 of the 18
// reals of a product). Results differ from site_md's only by rounding.
#pragma once

namespace meshgb {
namespace pair {

struct M2
{
	float2 r[9], i[9]; // entry (row a, column b) at 3a + b; x: first product, y: second
};

__device__ __forceinline__ float2 fma2(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }
__device__ __forceinline__ float2 mul2(float2 a, float2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ float2 add2(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 neg2(float2 a) { return __fmul2_rn(a, make_float2(-1.f, -1.f)); }
__device__ __forceinline__ float2 sub2(float2 a, float2 b) { return __ffma2_rn(b, make_float2(-1.f, -1.f), a); }
__device__ __forceinline__ float2 bc(float v) { return make_float2(v, v); }

using E = Group<SU3, float>::E;

// rows 0 and 1 of a and b into the lanes of a pair matrix
__device__ __forceinline__ M2 pack_rows(E const &a, E const &b)
{
	M2 m;
#pragma unroll
	for (int k = 0; k < 6; ++k)
	{
		m.r[k] = make_float2(a.v[2 * k], b.v[2 * k]);
		m.i[k] = make_float2(a.v[2 * k + 1], b.v[2 * k + 1]);
	}
	return m;
}
__device__ __forceinline__ void unpack(M2 const &m, E &a, E &b)
{
#pragma unroll
	for (int k = 0; k < 9; ++k)
	{
		a.v[2 * k] = m.r[k].x;
		a.v[2 * k + 1] = m.i[k].x;
		b.v[2 * k] = m.r[k].y;
		b.v[2 * k + 1] = m.i[k].y;
	}
}

// row 2 of special unitary matrices: conj(row 0 x row 1)
__device__ __forceinline__ void row2(M2 &m)
{
	float2 nr[3], ni[3];
#pragma unroll
	for (int k = 0; k < 3; ++k)
	{
		nr[k] = neg2(m.r[k]);
		ni[k] = neg2(m.i[k]);
	}
#pragma unroll
	for (int j = 0; j < 3; ++j)
	{
		int k = (j + 1) % 3, l = (j + 2) % 3;
		// z = a_0k a_1l - a_0l a_1k;  row 2 entry j = conj(z)
		float2 re = mul2(m.i[l], m.i[3 + k]);
		re = fma2(nr[l], m.r[3 + k], re);
		re = fma2(ni[k], m.i[3 + l], re);
		re = fma2(m.r[k], m.r[3 + l], re);
		float2 nim = mul2(m.i[l], m.r[3 + k]);
		nim = fma2(m.r[l], m.i[3 + k], nim);
		nim = fma2(ni[k], m.r[3 + l], nim);
		nim = fma2(nr[k], m.i[3 + l], nim);
		m.r[6 + j] = re;
		m.i[6 + j] = nim;
	}
}

// rows 0 .. NRW-1 of a b
template <int NRW> __device__ __forceinline__ M2 mul(M2 const &a, M2 const &b)
{
	M2 c;
#pragma unroll
	for (int i = 0; i < NRW; ++i)
	{
		float2 ni[3];
#pragma unroll
		for (int k = 0; k < 3; ++k)
			ni[k] = neg2(a.i[3 * i + k]);
#pragma unroll
		for (int j = 0; j < 3; ++j)
		{
			float2 re = mul2(a.r[3 * i], b.r[j]);
			float2 im = mul2(a.r[3 * i], b.i[j]);
			re = fma2(ni[0], b.i[j], re);
			im = fma2(a.i[3 * i], b.r[j], im);
#pragma unroll
			for (int k = 1; k < 3; ++k)
			{
				re = fma2(a.r[3 * i + k], b.r[3 * k + j], re);
				re = fma2(ni[k], b.i[3 * k + j], re);
				im = fma2(a.r[3 * i + k], b.i[3 * k + j], im);
				im = fma2(a.i[3 * i + k], b.r[3 * k + j], im);
			}
			c.r[3 * i + j] = re;
			c.i[3 * i + j] = im;
		}
	}
	return c;
}

// s += a^+ b:  s_ij += sum_k conj(a_ki) b_kj
__device__ __forceinline__ void add_dn(M2 &s, M2 const &a, M2 const &b)
{
	float2 ni[9];
#pragma unroll
	for (int k = 0; k < 9; ++k)
		ni[k] = neg2(a.i[k]);
#pragma unroll
	for (int i = 0; i < 3; ++i)
#pragma unroll
		for (int j = 0; j < 3; ++j)
		{
			float2 re = s.r[3 * i + j], im = s.i[3 * i + j];
#pragma unroll
			for (int k = 0; k < 3; ++k)
			{
				re = fma2(a.r[3 * k + i], b.r[3 * k + j], re);
				re = fma2(a.i[3 * k + i], b.i[3 * k + j], re);
				im = fma2(a.r[3 * k + i], b.i[3 * k + j], im);
				im = fma2(ni[3 * k + i], b.r[3 * k + j], im);
			}
			s.r[3 * i + j] = re;
			s.i[3 * i + j] = im;
		}
}

// the antihermitian traceless part of W (packed as Group<SU3>::proj) from the
// entries of W it reads, W_ij = sum_k A(i,k) B(k,j) with the entry functors
// returning (re, im) pairs
template <class FA, class FB> __device__ __forceinline__ void proj_prod(FA A, FB B, float2 *o)
{
	// Re W_ij, Im W_ij for the entries proj reads
	auto re = [&](int i, int j) {
		float2 acc = bc(0.f);
#pragma unroll
		for (int k = 0; k < 3; ++k)
		{
			float2 ar, ai, br, bi;
			A(i, k, ar, ai);
			B(k, j, br, bi);
			acc = fma2(ar, br, acc);
			acc = fma2(neg2(ai), bi, acc);
		}
		return acc;
	};
	auto im = [&](int i, int j) {
		float2 acc = bc(0.f);
#pragma unroll
		for (int k = 0; k < 3; ++k)
		{
			float2 ar, ai, br, bi;
			A(i, k, ar, ai);
			B(k, j, br, bi);
			acc = fma2(ar, bi, acc);
			acc = fma2(ai, br, acc);
		}
		return acc;
	};
	float2 d0 = im(0, 0), d1 = im(1, 1), d2 = im(2, 2);
	float2 t = mul2(add2(add2(d0, d1), d2), bc(1.f / 3.f));
	o[0] = sub2(d0, t);
	o[1] = sub2(d1, t);
	o[2] = mul2(sub2(re(0, 1), re(1, 0)), bc(0.5f));
	o[3] = mul2(add2(im(0, 1), im(1, 0)), bc(0.5f));
	o[4] = mul2(sub2(re(0, 2), re(2, 0)), bc(0.5f));
	o[5] = mul2(add2(im(0, 2), im(2, 0)), bc(0.5f));
	o[6] = mul2(sub2(re(1, 2), re(2, 1)), bc(0.5f));
	o[7] = mul2(add2(im(1, 2), im(2, 1)), bc(0.5f));
}

// proj(a b^+) and proj(a b)
__device__ __forceinline__ void proj_nd(M2 const &a, M2 const &b, float2 *o)
{
	proj_prod([&](int i, int k, float2 &r, float2 &im) { r = a.r[3 * i + k], im = a.i[3 * i + k]; },
	          [&](int k, int j, float2 &r, float2 &im) { r = b.r[3 * j + k], im = neg2(b.i[3 * j + k]); }, o);
}
__device__ __forceinline__ void proj_nn(M2 const &a, M2 const &b, float2 *o)
{
	proj_prod([&](int i, int k, float2 &r, float2 &im) { r = a.r[3 * i + k], im = a.i[3 * i + k]; },
	          [&](int k, int j, float2 &r, float2 &im) { r = b.r[3 * k + j], im = b.i[3 * k + j]; }, o);
}

__device__ __forceinline__ M2 zero()
{
	M2 m;
#pragma unroll
	for (int k = 0; k < 9; ++k)
		m.r[k] = m.i[k] = bc(0.f);
	return m;
}

// exp(t X) for the algebra elements oa, ob (X = from_alg), both lanes by the
// FP32 power series of Group<SU3, float>::exp_series (Cayley-Hamilton
// reduced, Horner on the three coefficients) when |X|^2/2 < 1/2 in both
// lanes; otherwise each lane by Group<SU3, float>::exp_alg
__device__ __forceinline__ M2 exp_alg(float const *oa, float const *ob, float t)
{
	using Gp = Group<SU3, float>;
	float2 x[8];
#pragma unroll
	for (int k = 0; k < 8; ++k)
		x[k] = mul2(make_float2(oa[k], ob[k]), bc(t));
	// c1 = |X|^2 / 2 (Group::kin / 2)
	float2 dsum = add2(x[0], x[1]);
	float2 kin = mul2(x[0], x[0]);
	kin = fma2(x[1], x[1], kin);
	kin = fma2(dsum, dsum, kin);
	float2 off = mul2(x[2], x[2]);
#pragma unroll
	for (int k = 3; k < 8; ++k)
		off = fma2(x[k], x[k], off);
	kin = fma2(bc(2.f), off, kin);
	float2 c1 = mul2(bc(0.5f), kin);
	if (!(c1.x < 0.5f && c1.y < 0.5f))
	{
		E ea = Gp::exp_alg(oa, t), eb = Gp::exp_alg(ob, t);
		M2 m;
#pragma unroll
		for (int k = 0; k < 9; ++k)
		{
			m.r[k] = make_float2(ea.v[2 * k], eb.v[2 * k]);
			m.i[k] = make_float2(ea.v[2 * k + 1], eb.v[2 * k + 1]);
		}
		return m;
	}
	// X = from_alg(x): diagonal i x0, i x1, -i (x0 + x1); X_01 = (x2, x3),
	// X_02 = (x4, x5), X_12 = (x6, x7), X_ji = -conj(X_ij)
	M2 X;
	X.r[0] = X.r[4] = X.r[8] = bc(0.f);
	X.i[0] = x[0];
	X.i[4] = x[1];
	X.i[8] = neg2(dsum);
	X.r[1] = x[2], X.i[1] = x[3];
	X.r[2] = x[4], X.i[2] = x[5];
	X.r[5] = x[6], X.i[5] = x[7];
	X.r[3] = neg2(x[2]), X.i[3] = x[3];
	X.r[6] = neg2(x[4]), X.i[6] = x[5];
	X.r[7] = neg2(x[6]), X.i[7] = x[7];
	// X^2 (hermitian): diagonal -sum_k |X_ik|^2, upper triangle multiplied out
	M2 X2;
#pragma unroll
	for (int i = 0; i < 3; ++i)
	{
		float2 d = bc(0.f);
#pragma unroll
		for (int k = 0; k < 3; ++k)
		{
			d = fma2(X.r[3 * i + k], X.r[3 * i + k], d);
			d = fma2(X.i[3 * i + k], X.i[3 * i + k], d);
		}
		X2.r[4 * i] = neg2(d);
		X2.i[4 * i] = bc(0.f);
#pragma unroll
		for (int j = i + 1; j < 3; ++j)
		{
			float2 re = bc(0.f), im = bc(0.f);
#pragma unroll
			for (int k = 0; k < 3; ++k)
			{
				re = fma2(X.r[3 * i + k], X.r[3 * k + j], re);
				re = fma2(neg2(X.i[3 * i + k]), X.i[3 * k + j], re);
				im = fma2(X.r[3 * i + k], X.i[3 * k + j], im);
				im = fma2(X.i[3 * i + k], X.r[3 * k + j], im);
			}
			X2.r[3 * i + j] = re;
			X2.i[3 * i + j] = im;
			X2.r[3 * j + i] = re;
			X2.i[3 * j + i] = neg2(im);
		}
	}
	// i dim = det X: Im det X by the cofactors of row 0
	auto cm = [](float2 ar, float2 ai, float2 br, float2 bi, float2 &rr, float2 &ri) {
		rr = fma2(neg2(ai), bi, mul2(ar, br));
		ri = fma2(ai, br, mul2(ar, bi));
	};
	auto cof = [&](int a, int b, int c, int d, float2 &rr, float2 &ri) {
		float2 pr, pi, qr, qi;
		cm(X.r[a], X.i[a], X.r[b], X.i[b], pr, pi);
		cm(X.r[c], X.i[c], X.r[d], X.i[d], qr, qi);
		rr = sub2(pr, qr);
		ri = sub2(pi, qi);
	};
	float2 Ar, Ai, Br, Bi, Cr, Ci;
	cof(4, 8, 5, 7, Ar, Ai); // X11 X22 - X12 X21
	cof(3, 8, 5, 6, Br, Bi); // X10 X22 - X12 X20
	cof(3, 7, 4, 6, Cr, Ci); // X10 X21 - X11 X20
	// Im(X00 A - X01 B + X02 C)
	float2 dim = fma2(X.r[0], Ai, mul2(X.i[0], Ar));
	dim = fma2(neg2(X.r[1]), Bi, dim);
	dim = fma2(neg2(X.i[1]), Br, dim);
	dim = fma2(X.r[2], Ci, dim);
	dim = fma2(X.i[2], Cr, dim);
	// Horner on (u0, u1, u2): X (u0 + u1 X + u2 X^2) + 1/k!
	//   = (i dim u2 + 1/k!) + (u0 - c1 u2) X + u1 X^2
	constexpr int N = 10;
	constexpr float inv_fact[N + 1] = {1.f,
	                                   1.f,
	                                   float(1.0 / 2),
	                                   float(1.0 / 6),
	                                   float(1.0 / 24),
	                                   float(1.0 / 120),
	                                   float(1.0 / 720),
	                                   float(1.0 / 5040),
	                                   float(1.0 / 40320),
	                                   float(1.0 / 362880),
	                                   float(1.0 / 3628800)};
	float2 u0r = bc(inv_fact[N]), u0i = bc(0.f), u1r = bc(0.f), u1i = bc(0.f), u2r = bc(0.f), u2i = bc(0.f);
	float2 nc1 = neg2(c1), ndim = neg2(dim);
#pragma unroll
	for (int k = N - 1; k >= 0; --k)
	{
		float2 n0r = fma2(ndim, u2i, bc(inv_fact[k]));
		float2 n0i = mul2(dim, u2r);
		float2 n1r = fma2(nc1, u2r, u0r);
		float2 n1i = fma2(nc1, u2i, u0i);
		u2r = u1r, u2i = u1i;
		u1r = n1r, u1i = n1i;
		u0r = n0r, u0i = n0i;
	}
	M2 r;
	float2 nu1i = neg2(u1i), nu2i = neg2(u2i);
#pragma unroll
	for (int k = 0; k < 9; ++k)
	{
		float2 re = fma2(u1r, X.r[k], mul2(nu1i, X.i[k]));
		re = fma2(u2r, X2.r[k], re);
		re = fma2(nu2i, X2.i[k], re);
		float2 im = fma2(u1r, X.i[k], mul2(u1i, X.r[k]));
		im = fma2(u2r, X2.i[k], im);
		im = fma2(u2i, X2.r[k], im);
		if (k % 4 == 0)
		{
			re = add2(re, u0r);
			im = add2(im, u0i);
		}
		r.r[k] = re;
		r.i[k] = im;
	}
	return r;
}

} // namespace pair

// The per-site body (see the file comment). LD: rows-only link loads
// (LinkLoad<SU3, float, 4, true>); F: the site's force accumulators. PARTS
// selects the paired sections (the others run one product at a time with
// the one-product FP32x2 form, as site_md): 1 the forward plaquette loops,
// 2 the lower staples, 4 the link update.
template <bool FUSE, class LD, bool SM, int PARTS>
__device__ __forceinline__ double site_md_pair(Geom const &g, Site<4> const &st, int64_t s, LD const &ld,
                                               float *__restrict__ P, float coef, float *__restrict__ Uout, float tu,
                                               int reunit, bool want_kin, float *acc_sm)
{
	using Gp = Group<SU3, float>;
	using E = Gp::E;
	using Pr = Prod<SU3, float, 1>;
	using pair::M2;
	constexpr int NA = 8;
	SiteAcc<float, 4, NA, SM> F(acc_sm);
	if constexpr (PARTS & 1)
	{
		// forward plaquette loops (a b)(d c)^+, planes q and q + 3
#pragma unroll 1
		for (int q = 0; q < 3; ++q)
		{
			int ma = plane_mu<4>(q), na = plane_nu<4>(q), mb = plane_mu<4>(q + 3), nb = plane_nu<4>(q + 3);
			M2 ab;
			{
				M2 a = pair::pack_rows(ld.rows(ma, s), ld.rows(mb, s));
				M2 b = pair::pack_rows(ld.rows(na, eo_shift1<4>(g, st, ma, +1)),
				                       ld.rows(nb, eo_shift1<4>(g, st, mb, +1)));
				pair::row2(b);
				ab = pair::mul<2>(a, b);
				pair::row2(ab);
			}
			M2 dc;
			{
				M2 d = pair::pack_rows(ld.rows(na, s), ld.rows(nb, s));
				M2 c = pair::pack_rows(ld.rows(ma, eo_shift1<4>(g, st, na, +1)),
				                       ld.rows(mb, eo_shift1<4>(g, st, nb, +1)));
				pair::row2(c);
				dc = pair::mul<2>(d, c);
				pair::row2(dc);
			}
			float2 o[NA];
			pair::proj_nd(ab, dc, o);
			float xa[NA], xb[NA];
#pragma unroll
			for (int k = 0; k < NA; ++k)
				xa[k] = o[k].x, xb[k] = o[k].y;
			F.plane(q, xa);
			F.plane(q + 3, xb);
		}
	}
	else
	{
#pragma unroll 1
		for (int q = 0; q < 6; ++q)
		{
			int mu = plane_mu<4>(q), nu = plane_nu<4>(q);
			E ab = Pr::mul_r2(ld.rows(mu, s), ld(nu, eo_shift1<4>(g, st, mu, +1)));
			E dc = Pr::mul_r2(ld.rows(nu, s), ld(mu, eo_shift1<4>(g, st, nu, +1)));
			float xa[NA];
			Gp::proj(Pr::mul_nd(ab, dc), xa);
			F.plane(q, xa);
		}
	}
	// lower staples (U_mu(y) U_nu(y+mu))^+ U_nu(y), y = x - nu, summed per link
	if constexpr (PARTS & 2)
	{
		// links (x, m) and (x, m + 2)
#pragma unroll 1
		for (int m = 0; m < 2; ++m)
		{
			M2 S = pair::zero();
#pragma unroll 1
			for (int k = 0; k < 3; ++k)
			{
				int mb = m + 2;
				int na = k < m ? k : k + 1, nb = k < mb ? k : k + 1;
				int64_t ya = eo_shift1<4>(g, st, na, -1), yb = eo_shift1<4>(g, st, nb, -1);
				M2 ef;
				{
					M2 e = pair::pack_rows(ld.rows(m, ya), ld.rows(mb, yb));
					M2 f = pair::pack_rows(ld.rows(na, eo_shift2<4>(g, st, na, -1, m, +1)),
					                       ld.rows(nb, eo_shift2<4>(g, st, nb, -1, mb, +1)));
					pair::row2(f);
					ef = pair::mul<2>(e, f);
					pair::row2(ef);
				}
				M2 h = pair::pack_rows(ld.rows(na, ya), ld.rows(nb, yb));
				pair::row2(h);
				pair::add_dn(S, ef, h);
			}
			M2 u = pair::pack_rows(ld.rows(m, s), ld.rows(m + 2, s));
			pair::row2(u);
			float2 o[NA];
			pair::proj_nn(u, S, o);
			float xa[NA], xb[NA];
#pragma unroll
			for (int k = 0; k < NA; ++k)
				xa[k] = o[k].x, xb[k] = o[k].y;
			F.dir(m, xa);
			F.dir(m + 2, xb);
		}
	}
	else
	{
#pragma unroll 1
		for (int mu = 0; mu < 4; ++mu)
		{
			E S = Gp::zero();
#pragma unroll 1
			for (int nu = 0; nu < 4; ++nu)
			{
				if (nu == mu)
					continue;
				int64_t y = eo_shift1<4>(g, st, nu, -1);
				E f = ld(nu, eo_shift2<4>(g, st, nu, -1, mu, +1));
				Gp::add_to(S, Pr::mul_dn(Pr::mul_r2(ld.rows(mu, y), f), ld(nu, y)));
			}
			float xa[NA];
			Gp::proj(Pr::mul(ld(mu, s), S), xa);
			F.dir(mu, xa);
		}
	}
	float kacc = 0.f; // the site's kinetic terms in FP32, one FP64 add per site
	if constexpr (PARTS & 4)
	{
		// directions m and m + 2
#pragma unroll 1
		for (int m = 0; m < 2; ++m)
		{
			float pa[NA], pb[NA], fa[NA], fb[NA];
			F.get(m, fa);
			F.get(m + 2, fb);
			auto Pa = comp<float, NA>(P, g.V, m), Pb = comp<float, NA>(P, g.V, m + 2);
			Pa.template load<CACHE_STREAM>(s, pa);
			Pb.template load<CACHE_STREAM>(s, pb);
#pragma unroll
			for (int a = 0; a < NA; ++a)
			{
				pa[a] -= coef * fa[a];
				pb[a] -= coef * fb[a];
			}
			Pa.template store<CACHE_STREAM>(s, pa);
			Pb.template store<CACHE_STREAM>(s, pb);
			if (want_kin)
				kacc += Gp::kin(pa) + Gp::kin(pb);
			if constexpr (FUSE)
			{
				M2 ex = pair::exp_alg(pa, pb, tu);
				M2 u = pair::pack_rows(ld.rows(m, s), ld.rows(m + 2, s));
				pair::row2(u);
				M2 r = pair::mul<2>(ex, u);
				pair::row2(r);
				E ra, rb;
				pair::unpack(r, ra, rb);
				if (reunit)
				{
					ra = Gp::reunit_fast(ra);
					rb = Gp::reunit_fast(rb);
				}
				comp<float, Gp::NR>(Uout, g.V, m).store(s, ra.v);
				comp<float, Gp::NR>(Uout, g.V, m + 2).store(s, rb.v);
			}
		}
	}
	else
	{
#pragma unroll 1
		for (int mu = 0; mu < 4; ++mu)
		{
			float f[NA], p[NA];
			F.get(mu, f);
			auto Pv = comp<float, NA>(P, g.V, mu);
			Pv.template load<CACHE_STREAM>(s, p);
#pragma unroll
			for (int a = 0; a < NA; ++a)
				p[a] -= coef * f[a];
			Pv.template store<CACHE_STREAM>(s, p);
			if (want_kin)
				kacc += Gp::kin(p);
			if constexpr (FUSE)
			{
				E r = Pr::mul_r2(Gp::exp_alg(p, tu), ld(mu, s));
				if (reunit)
					r = Gp::reunit_fast(r);
				comp<float, Gp::NR>(Uout, g.V, mu).store(s, r.v);
			}
		}
	}
	return double(kacc);
}

} // namespace meshgb
