// Momentum step (optionally fused with the link update after it) for SU(3) in
// four dimensions, organised by lattice lines: one warp holds the L3 sites
// x3 = 0..L3-1 of 32/L3 neighbouring lines (fixed x0, x1, x2), and marches
// along x1. The operation is the reference's momentum step of runHmd
// (src/gauge/hmc.h:54-58: P_mu -= wilsonDeriv(U, mu, beta) dt, with
// wilsonDeriv = project_on_algebra(U_mu stapleSum_mu) beta/(2 Nc),
// src/gauge/utils.h:114-153), followed, when fused, by evolve
// (src/gauge/hmc.h:26-36).
//
// The force on link (x, mu) is the sum over the six plaquettes that contain
// it of the projection of the loop that starts with that link. A plaquette
// P = U_mu(x) U_nu(x+mu) U_mu(x+nu)^+ U_nu(x)^+ (mu < nu), A = proj(P),
// contributes
//     +A                      to (x, mu)      (its upper staple),
//     -A                      to (x, nu),
//     -U_nu(x)^+ A U_nu(x)    to (x+nu, mu)   (the lower staple of that link),
//     +U_mu(x)^+ A U_mu(x)    to (x+mu, nu),
// because proj(V^+ M V) = V^+ proj(M) V for unitary V and the lower-staple
// loop of (x+nu, mu) is U_nu(x)^+ P^+ U_nu(x). Each site computes its six
// plaquettes once (3 products each, from rows 0 and 1 where the links are
// special unitary) and hands the lower-staple contributions along the two
// directions the warp can reach cheaply as 8-real algebra elements:
//   * along x3 to the next lane of the same warp, through shared memory;
//   * along x1 to the next line of the march, carried by the same thread.
// The lower staples along x0 and x2 are summed as in the reference
// (U_nu(y+mu)^+ U_mu(y)^+ U_nu(y) at y = x - nu, one product U_mu(x) S_mu
// for the sum). Against computing every staple per link this saves six of
// the twelve lower-staple products of a site and most neighbour loads: a
// site reads its own four links, the twelve forward neighbours
// U_nu(x + mu) and the links of the x0 and x2 lower staples.
//
// Work assignment: a "column" is the set of lines (x0, x2-group) along x1;
// its x1 march is cut into nseg segments, and every warp of the launch takes
// one (column, segment), warp w the column w mod ncol, so that the warps of
// a block hold neighbouring columns and all warps march in step: the lines
// being read at one time are a few x1 slices of the lattice, which stay in
// L2. At the first step of a segment the carry along x1 is computed for the
// line behind (three plaquettes and their contributions).
//
// The sum runs in a different order than the reference's staple sum, which
// changes the force only at the rounding level.
//
// Included by kernels.cuh after the thread-per-site kernels, whose helpers
// (LinkLoad, Prod, add_plane, plane_mu/nu, comp, grid_sum) it uses.
#pragma once

namespace meshgb {

struct LineSpec
{
	int ns;   // lines per warp = 32 / L3
	int ncol; // columns of lines along x1: L0 * L2 / ns
	int nseg; // segments of the x1 march per column
	int nwork; // warps with work: ncol * nseg
	int *err;  // the context's device error word (bounded waits of the staged variant)
};

inline bool line_supported(Geom const &g)
{
	if (g.nd != 4)
		return false;
	int l3 = g.L[3];
	if (l3 < 2 || l3 > 32 || 32 % l3 != 0)
		return false;
	int ns = 32 / l3;
	return g.L[2] % ns == 0;
}

template <class T, int F2> struct LineProd
{
	using Gp = Group<SU3, T>;
	using E = typename Gp::E;
	// rows 0, 1 of a b (rows 0, 1 of a read)
	__device__ __forceinline__ static E mul01(E const &a, E const &b)
	{
		if constexpr (F2)
			return Su3F2::template mul<2>(a, b);
		else
		{
			E r;
#pragma unroll
			for (int i = 0; i < 2; ++i)
#pragma unroll
				for (int j = 0; j < 3; ++j)
				{
					T re = 0, im = 0;
#pragma unroll
					for (int k = 0; k < 3; ++k)
					{
						re += a.v[6 * i + 2 * k] * b.v[6 * k + 2 * j] - a.v[6 * i + 2 * k + 1] * b.v[6 * k + 2 * j + 1];
						im += a.v[6 * i + 2 * k] * b.v[6 * k + 2 * j + 1] + a.v[6 * i + 2 * k + 1] * b.v[6 * k + 2 * j];
					}
					r.v[6 * i + 2 * j] = re;
					r.v[6 * i + 2 * j + 1] = im;
				}
			return r;
		}
	}
	// rows 0, 1 of a b^+ (rows 0, 1 of a and all of b read)
	__device__ __forceinline__ static E mul01_nd(E const &a, E const &b)
	{
		if constexpr (F2)
			return Su3F2::template prod<2>(
			    [&](int i, int k, float &re, float &im) {
				    re = a.v[6 * i + 2 * k];
				    im = a.v[6 * i + 2 * k + 1];
			    },
			    [&](int k, int j, float &re, float &im) {
				    re = b.v[6 * j + 2 * k];
				    im = -b.v[6 * j + 2 * k + 1];
			    });
		else
		{
			E r;
#pragma unroll
			for (int i = 0; i < 2; ++i)
#pragma unroll
				for (int j = 0; j < 3; ++j)
				{
					T re = 0, im = 0;
#pragma unroll
					for (int k = 0; k < 3; ++k)
					{
						T ar = a.v[6 * i + 2 * k], ai = a.v[6 * i + 2 * k + 1];
						T br = b.v[6 * j + 2 * k], bi = b.v[6 * j + 2 * k + 1];
						re += ar * br + ai * bi;
						im += ai * br - ar * bi;
					}
					r.v[6 * i + 2 * j] = re;
					r.v[6 * i + 2 * j + 1] = im;
				}
			return r;
		}
	}
	// proj (antihermitian traceless part, packed) of a special unitary matrix
	// given by rows 0 and 1: the row-2 entries it needs come from
	// row 2 = conj(row 0 x row 1)
	__device__ __forceinline__ static void proj01(E const &p, T *o)
	{
		cx<T> p20 = cconj(csub(cmul(p.at(0, 1), p.at(1, 2)), cmul(p.at(0, 2), p.at(1, 1))));
		cx<T> p21 = cconj(csub(cmul(p.at(0, 2), p.at(1, 0)), cmul(p.at(0, 0), p.at(1, 2))));
		// Im conj(p00 p11 - p01 p10)
		T i22 = -((p.v[0] * p.v[9] + p.v[1] * p.v[8]) - (p.v[2] * p.v[7] + p.v[3] * p.v[6]));
		T t = (p.v[1] + p.v[9] + i22) * T(1.0 / 3.0);
		o[0] = p.v[1] - t;
		o[1] = p.v[9] - t;
		o[2] = (p.v[2] - p.v[6]) * T(0.5);
		o[3] = (p.v[3] + p.v[7]) * T(0.5);
		o[4] = (p.v[4] - p20.re) * T(0.5);
		o[5] = (p.v[5] + p20.im) * T(0.5);
		o[6] = (p.v[10] - p21.re) * T(0.5);
		o[7] = (p.v[11] + p21.im) * T(0.5);
	}
	// proj(a b) (antihermitian traceless part, packed) from the nine entries
	// of the product it needs
	__device__ __forceinline__ static void proj_mul(E const &a, E const &b, T *o)
	{
		auto c = [&](int i, int j) {
			cx<T> z = cmul(a.at(i, 0), b.at(0, j));
			z = cadd(z, cmul(a.at(i, 1), b.at(1, j)));
			return cadd(z, cmul(a.at(i, 2), b.at(2, j)));
		};
		auto ci = [&](int i) {
			T z = T(0);
#pragma unroll
			for (int k = 0; k < 3; ++k)
				z += a.v[6 * i + 2 * k] * b.v[6 * k + 2 * i + 1] + a.v[6 * i + 2 * k + 1] * b.v[6 * k + 2 * i];
			return z;
		};
		T i0 = ci(0), i1 = ci(1), i2 = ci(2);
		T t = (i0 + i1 + i2) * T(1.0 / 3.0);
		cx<T> c01 = c(0, 1), c10 = c(1, 0), c02 = c(0, 2), c20 = c(2, 0), c12 = c(1, 2), c21 = c(2, 1);
		o[0] = i0 - t;
		o[1] = i1 - t;
		o[2] = (c01.re - c10.re) * T(0.5);
		o[3] = (c01.im + c10.im) * T(0.5);
		o[4] = (c02.re - c20.re) * T(0.5);
		o[5] = (c02.im + c20.im) * T(0.5);
		o[6] = (c12.re - c21.re) * T(0.5);
		o[7] = (c12.im + c21.im) * T(0.5);
	}
	// sg V^+ A V for A = from_alg(o) and unitary V, packed (upper triangle
	// and the imaginary diagonal of the exactly antihermitian traceless
	// result)
	__device__ __forceinline__ static void adjoint(E const &V, T const *o, T sg, T *out)
	{
		// B = A V with A_ii = i a_i, A_ij = -conj(A_ji)
		T a0 = o[0], a1 = o[1], a2 = -(o[0] + o[1]);
		cx<T> A01 = {o[2], o[3]}, A02 = {o[4], o[5]}, A12 = {o[6], o[7]};
		cx<T> A10 = {-o[2], o[3]}, A20 = {-o[4], o[5]}, A21 = {-o[6], o[7]};
		cx<T> B[3][3];
#pragma unroll
		for (int j = 0; j < 3; ++j)
		{
			cx<T> v0 = V.at(0, j), v1 = V.at(1, j), v2 = V.at(2, j);
			B[0][j] = cadd(cx<T>{-a0 * v0.im, a0 * v0.re}, cadd(cmul(A01, v1), cmul(A02, v2)));
			B[1][j] = cadd(cx<T>{-a1 * v1.im, a1 * v1.re}, cadd(cmul(A10, v0), cmul(A12, v2)));
			B[2][j] = cadd(cx<T>{-a2 * v2.im, a2 * v2.re}, cadd(cmul(A20, v0), cmul(A21, v1)));
		}
		// C = V^+ B: C_ij = sum_k conj(V_ki) B_kj
		auto cij = [&](int i, int j) {
			cx<T> z = {T(0), T(0)};
#pragma unroll
			for (int k = 0; k < 3; ++k)
				z = cadd(z, cmul(cconj(V.at(k, i)), B[k][j]));
			return z;
		};
		auto cii_im = [&](int i) {
			T z = T(0);
#pragma unroll
			for (int k = 0; k < 3; ++k)
			{
				cx<T> v = V.at(k, i);
				z += v.re * B[k][i].im - v.im * B[k][i].re;
			}
			return z;
		};
		cx<T> c01 = cij(0, 1), c02 = cij(0, 2), c12 = cij(1, 2);
		out[0] = sg * cii_im(0);
		out[1] = sg * cii_im(1);
		out[2] = sg * c01.re;
		out[3] = sg * c01.im;
		out[4] = sg * c02.re;
		out[5] = sg * c02.im;
		out[6] = sg * c12.re;
		out[7] = sg * c12.im;
	}
};

// link loads of the line march: rows() reads rows 0 and 1 (the left factor
// of a product of special unitary links); operator() reads the whole link,
// with row 2 rebuilt from rows 0, 1 (R2 = false: 48 bytes read, 24 FMAs) or
// read from memory (R2 = true: 72 bytes, no arithmetic). FP64 links and
// ROWS = false read every real.
template <class T, bool ROWS, bool R2> struct LineLoad;
template <bool ROWS, bool R2> struct LineLoad<float, ROWS, R2>
{
	// component mu: float4 planes k = 0..3 at mu 9 V/2 + k V (in float4
	// units), the float2 plane at mu 9 V + 8 V (in float2 units); 32-bit
	// indices (the library keeps 72 V < 2^32 reals per field)
	using Gp = Group<SU3, float>;
	using E = typename Gp::E;
	float const *U;
	uint32_t V;
	__device__ __forceinline__ void head(int mu, uint32_t s, E &e) const
	{
		float4 const *p = reinterpret_cast<float4 const *>(U) + (uint32_t(mu) * 9u * (V >> 1) + s);
#pragma unroll
		for (int k = 0; k < 3; ++k)
		{
			float4 t = ld4<CACHE_KEEP>(p + k * V);
			e.v[4 * k] = t.x;
			e.v[4 * k + 1] = t.y;
			e.v[4 * k + 2] = t.z;
			e.v[4 * k + 3] = t.w;
		}
	}
	__device__ __forceinline__ E operator()(int mu, uint32_t s) const
	{
		E e;
		head(mu, s, e);
		if constexpr (ROWS && !R2)
			Gp::complete_row2(e);
		else
		{
			float4 t = ld4<CACHE_KEEP>(reinterpret_cast<float4 const *>(U) + (uint32_t(mu) * 9u * (V >> 1) + 3 * V + s));
			e.v[12] = t.x;
			e.v[13] = t.y;
			e.v[14] = t.z;
			e.v[15] = t.w;
			float2 u = ld2<CACHE_KEEP>(reinterpret_cast<float2 const *>(U) + (uint32_t(mu) * 9u * V + 8 * V + s));
			e.v[16] = u.x;
			e.v[17] = u.y;
		}
		return e;
	}
	__device__ __forceinline__ E rows(int mu, uint32_t s) const
	{
		if constexpr (ROWS)
		{
			E e;
			head(mu, s, e);
			return e;
		}
		else
			return (*this)(mu, s);
	}
	// L1 prefetch of what rows() / operator() will read (one 128-byte line
	// per plane of the warp's addresses)
	__device__ __forceinline__ static void pf(void const *p) { asm volatile("prefetch.global.L1 [%0];" ::"l"(p)); }
	__device__ __forceinline__ void prefetch_rows(int mu, uint32_t s) const
	{
		float4 const *p = reinterpret_cast<float4 const *>(U) + (uint32_t(mu) * 9u * (V >> 1) + s);
#pragma unroll
		for (int k = 0; k < 3; ++k)
			pf(p + k * V);
	}
	__device__ __forceinline__ void prefetch(int mu, uint32_t s) const
	{
		prefetch_rows(mu, s);
		if constexpr (!(ROWS && !R2))
		{
			pf(reinterpret_cast<float4 const *>(U) + (uint32_t(mu) * 9u * (V >> 1) + 3 * V + s));
			pf(reinterpret_cast<float2 const *>(U) + (uint32_t(mu) * 9u * V + 8 * V + s));
		}
	}
};
template <bool ROWS, bool R2> struct LineLoad<double, ROWS, R2>
{
	// component mu: double2 planes k = 0..8 at mu 9 V + k V
	using Gp = Group<SU3, double>;
	using E = typename Gp::E;
	double const *U;
	uint32_t V;
	template <int K> __device__ __forceinline__ void planes(int mu, uint32_t s, E &e) const
	{
		double2 const *p = reinterpret_cast<double2 const *>(U) + (uint32_t(mu) * 9u * V + s);
#pragma unroll
		for (int k = 0; k < K; ++k)
		{
			double2 t = ld2d<CACHE_KEEP>(p + k * V);
			e.v[2 * k] = t.x;
			e.v[2 * k + 1] = t.y;
		}
	}
	__device__ __forceinline__ E operator()(int mu, uint32_t s) const
	{
		E e;
		planes<9>(mu, s, e);
		return e;
	}
	__device__ __forceinline__ E rows(int mu, uint32_t s) const
	{
		E e;
		planes<6>(mu, s, e);
		return e;
	}
	__device__ __forceinline__ void prefetch_rows(int, uint32_t) const {}
	__device__ __forceinline__ void prefetch(int, uint32_t) const {}
};

// site coordinates of the line march (x3 of the lane, x2 of its sub-line)
struct LineSite
{
	int x0, x1, x2, x3;
};

__device__ __forceinline__ int wrap_add(int x, int d, int L)
{
	x += d;
	return x >= L ? x - L : (x < 0 ? x + L : x);
}

// even/odd index of the site (a0, a1, a2, a3) (coordinates in range)
__device__ __forceinline__ uint32_t line_eo(Geom const &g, int a0, int a1, int a2, int a3)
{
	uint32_t lex = uint32_t(((a0 * g.L[1] + a1) * g.L[2] + a2) * g.L[3] + a3);
	uint32_t p = uint32_t(a0 + a1 + a2 + a3) & 1u;
	return p * uint32_t(g.Vh) + (lex >> 1);
}

// site x shifted by s1 along d1 and s2 along d2 (s = 0: no shift)
__device__ __forceinline__ uint32_t line_nb(Geom const &g, LineSite const &x, int d1, int s1, int d2 = 0, int s2 = 0)
{
	int c[4] = {x.x0, x.x1, x.x2, x.x3};
#pragma unroll
	for (int i = 0; i < 4; ++i)
	{
		int d = (i == d1 ? s1 : 0) + (i == d2 ? s2 : 0);
		c[i] = wrap_add(c[i], d, g.L[i]);
	}
	return line_eo(g, c[0], c[1], c[2], c[3]);
}

// lexicographic index after a step of `sign` along d, for coordinate xd
__device__ __forceinline__ uint32_t lex_shift(uint32_t lex, int xd, int Ld, uint32_t str, int sign)
{
	if (sign > 0)
		return xd == Ld - 1 ? lex - uint32_t(Ld - 1) * str : lex + str;
	return xd == 0 ? lex + uint32_t(Ld - 1) * str : lex - str;
}

// even/odd indices of the neighbours one step of the march reads, computed
// once per site: x + e_mu, x - e_0, x - e_2 and x - e_nu + e_mu (nu = 0, 2)
struct LineNb
{
	uint32_t f[4];                // x + e_mu (opposite parity)
	uint32_t b0, b2;              // x - e_0, x - e_2 (opposite parity)
	uint32_t d01, d02, d03;       // x - e_0 + e_mu, mu = 1, 2, 3 (x's parity)
	uint32_t d20, d21, d23;       // x - e_2 + e_mu, mu = 0, 1, 3
	// selects on constant members (a runtime index into f would go to local memory)
	__device__ __forceinline__ uint32_t fwd(int mu) const
	{
		return mu == 0 ? f[0] : mu == 1 ? f[1] : mu == 2 ? f[2] : f[3];
	}
	__device__ __forceinline__ uint32_t diag(int nu, int mu) const
	{
		if (nu == 0)
			return mu == 1 ? d01 : mu == 2 ? d02 : d03;
		return mu == 0 ? d20 : mu == 1 ? d21 : d23;
	}
};

__device__ __forceinline__ LineNb line_neighbours(Geom const &g, LineSite const &x)
{
	int c[4] = {x.x0, x.x1, x.x2, x.x3};
	uint32_t str[4] = {uint32_t(g.stride[0]), uint32_t(g.stride[1]), uint32_t(g.stride[2]), uint32_t(g.stride[3])};
	uint32_t lex = ((uint32_t(c[0]) * g.L[1] + c[1]) * g.L[2] + c[2]) * g.L[3] + c[3];
	uint32_t par = uint32_t(c[0] + c[1] + c[2] + c[3]) & 1u;
	uint32_t Vh = uint32_t(g.Vh);
	uint32_t po = (par ^ 1u) * Vh, ps = par * Vh;
	LineNb n;
#pragma unroll
	for (int mu = 0; mu < 4; ++mu)
		n.f[mu] = po + (lex_shift(lex, c[mu], g.L[mu], str[mu], +1) >> 1);
	uint32_t y0 = lex_shift(lex, c[0], g.L[0], str[0], -1);
	uint32_t y2 = lex_shift(lex, c[2], g.L[2], str[2], -1);
	n.b0 = po + (y0 >> 1);
	n.b2 = po + (y2 >> 1);
	n.d01 = ps + (lex_shift(y0, c[1], g.L[1], str[1], +1) >> 1);
	n.d02 = ps + (lex_shift(y0, c[2], g.L[2], str[2], +1) >> 1);
	n.d03 = ps + (lex_shift(y0, c[3], g.L[3], str[3], +1) >> 1);
	n.d20 = ps + (lex_shift(y2, c[0], g.L[0], str[0], +1) >> 1);
	n.d21 = ps + (lex_shift(y2, c[1], g.L[1], str[1], +1) >> 1);
	n.d23 = ps + (lex_shift(y2, c[3], g.L[3], str[3], +1) >> 1);
	return n;
}

// A = proj of the plaquette (mu, nu) at site x (mu < nu, runtime) from the
// forward neighbours x + e_mu (fmu) and x + e_nu (fnu)
template <class T, int F2, class LD>
__device__ __forceinline__ void plaquette_at(uint32_t s, uint32_t fmu, uint32_t fnu, int mu, int nu, LD const &ld,
                                             T *o)
{
	using Pr = LineProd<T, F2>;
	using Gp = Group<SU3, T>;
	using E = typename Gp::E;
	E M1 = Pr::mul01(ld.rows(mu, s), ld(nu, fmu));
	E M2 = Pr::mul01(ld.rows(nu, s), ld(mu, fnu));
	Gp::complete_row2(M2);
	Pr::proj01(Pr::mul01_nd(M1, M2), o);
}

// A = proj of the plaquette (mu, nu) at site x (mu < nu, runtime)
template <class T, int F2, class LD>
__device__ __forceinline__ void line_plaquette(Geom const &g, LineSite const &x, uint32_t s, int mu, int nu,
                                               LD const &ld, T *o)
{
	using Pr = LineProd<T, F2>;
	using Gp = Group<SU3, T>;
	using E = typename Gp::E;
	E M1 = Pr::mul01(ld.rows(mu, s), ld(nu, line_nb(g, x, mu, +1)));
	E M2 = Pr::mul01(ld.rows(nu, s), ld(mu, line_nb(g, x, nu, +1)));
	Gp::complete_row2(M2);
	Pr::proj01(Pr::mul01_nd(M1, M2), o);
}

// the three planes that send along x1: (0,1) to link 0 with -U_1^+ A U_1,
// (1,2) to link 2 and (1,3) to link 3 with +U_1^+ A U_1; along x3: (0,3),
// (1,3), (2,3) to links 0, 1, 2 with -U_3^+ A U_3
__device__ __forceinline__ int plane_q(int mu, int nu) { return mu == 0 ? nu - 1 : (mu == 1 ? nu + 1 : 5); }

// shared-memory hand-over slots of one warp: 8 reals per (link k, lane) as
// 16-byte words, [k][word][lane], so that a warp's access is contiguous
template <class T> struct Slot16;
template <> struct Slot16<float>
{
	using W = float4;
	static constexpr int N = 2; // words per algebra element
	__device__ __forceinline__ static W pack(float const *o) { return W{o[0], o[1], o[2], o[3]}; }
	__device__ __forceinline__ static void unpack(W w, float *o)
	{
		o[0] = w.x;
		o[1] = w.y;
		o[2] = w.z;
		o[3] = w.w;
	}
};
template <> struct Slot16<double>
{
	using W = double2;
	static constexpr int N = 4;
	__device__ __forceinline__ static W pack(double const *o) { return W{o[0], o[1]}; }
	__device__ __forceinline__ static void unpack(W w, double *o)
	{
		o[0] = w.x;
		o[1] = w.y;
	}
};

template <class T> __device__ __forceinline__ void slot_store(typename Slot16<T>::W *sl, int k, int lane, T const *o)
{
	using S = Slot16<T>;
#pragma unroll
	for (int w = 0; w < S::N; ++w)
		sl[(S::N * k + w) * 32 + lane] = S::pack(o + w * (8 / S::N));
}
template <class T>
__device__ __forceinline__ void slot_load(typename Slot16<T>::W const *sl, int k, int lane, T *o)
{
	using S = Slot16<T>;
#pragma unroll
	for (int w = 0; w < S::N; ++w)
		S::unpack(sl[(S::N * k + w) * 32 + lane], o + w * (8 / S::N));
}

// F[mu] += x for a runtime mu (selects keep F in registers)
template <int NA, class T> __device__ __forceinline__ void add_link(T (&F)[4][NA], int mu, T const *x, T sg = T(1))
{
#pragma unroll
	for (int k = 0; k < 4; ++k)
		if (k == mu)
		{
#pragma unroll
			for (int a = 0; a < NA; ++a)
				F[k][a] += sg * x[a];
		}
}

// the force accumulators F[mu] (8 reals for each of the four links of a
// site): in registers, or (FSM) in shared-memory slots of the thread, which
// frees 32 registers for a higher occupancy
template <class T, bool FSM> struct FAcc;
template <class T> struct FAcc<T, false>
{
	T F[4][8];
	__device__ __forceinline__ FAcc(typename Slot16<T>::W *, int) {}
	__device__ __forceinline__ void set(int k, T const *o)
	{
#pragma unroll
		for (int j = 0; j < 4; ++j)
			if (j == k)
#pragma unroll
				for (int a = 0; a < 8; ++a)
					F[j][a] = o[a];
	}
	__device__ __forceinline__ void add(int k, T const *o, T sg) { add_link<8>(F, k, o, sg); }
	__device__ __forceinline__ void get(int k, T *o) const
	{
#pragma unroll
		for (int a = 0; a < 8; ++a)
		{
			o[a] = F[0][a];
#pragma unroll
			for (int j = 1; j < 4; ++j)
				o[a] = k == j ? F[j][a] : o[a];
		}
	}
};
template <class T> struct FAcc<T, true>
{
	typename Slot16<T>::W *sl;
	int lane;
	__device__ __forceinline__ FAcc(typename Slot16<T>::W *s, int l) : sl(s), lane(l) {}
	__device__ __forceinline__ void set(int k, T const *o) { slot_store<T>(sl, k, lane, o); }
	__device__ __forceinline__ void add(int k, T const *o, T sg)
	{
		T f[8];
		slot_load<T>(sl, k, lane, f);
#pragma unroll
		for (int a = 0; a < 8; ++a)
			f[a] += sg * o[a];
		slot_store<T>(sl, k, lane, f);
	}
	__device__ __forceinline__ void get(int k, T *o) const { slot_load<T>(sl, k, lane, o); }
};

// carry of the line behind x (x - e_1): the contributions of its planes
// (0,1), (1,2), (1,3) to links 0, 2, 3 of x, into the carry slots
template <class T, int F2, class LD>
__device__ __forceinline__ void line_carry(Geom const &g, LineSite const &x, LD const &ld,
                                           typename Slot16<T>::W *carry, int lane)
{
	using Pr = LineProd<T, F2>;
	using Gp = Group<SU3, T>;
	using E = typename Gp::E;
	LineSite y = x;
	y.x1 = wrap_add(x.x1, -1, g.L[1]);
	uint32_t sy = line_eo(g, y.x0, y.x1, y.x2, y.x3);
#pragma unroll 1
	for (int k = 0; k < 3; ++k)
	{
		int mu = k == 0 ? 0 : 1, nu = k == 0 ? 1 : k + 1;
		T o[8], c[8];
		line_plaquette<T, F2>(g, y, sy, mu, nu, ld, o);
		E V = ld(1, sy);
		Pr::adjoint(V, o, k == 0 ? T(-1) : T(1), c);
		slot_store<T>(carry, k, lane, c);
	}
}

// One momentum step (and with FUSE the link update after it) of every link,
// line-marching. P -= coef F(U); Uout = exp(tu P) U (reunitised when reunit).
// ---- bulk copies (TMA) into shared memory with an mbarrier ------------------
// One warp stages its own line (rows 0, 1 of the four links: per link 3
// float4 planes x 2 parities, each a contiguous 256-byte run of the even/odd
// layout when L3 = 32) with 24 cp.async.bulk copies issued by lane 0, which
// complete on the warp's mbarrier. Every wait is bounded in time; a wait that
// gives up writes a code to the context's device error word and the warp
// stops working (the host reports MESH_ERR_TIMEOUT).
__device__ __forceinline__ uint32_t smem_addr(void const *p) { return uint32_t(__cvta_generic_to_shared(p)); }
__device__ __forceinline__ void mbar_init(unsigned long long *b)
{
	asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_addr(b)) : "memory");
	asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ void mbar_expect(unsigned long long *b, uint32_t bytes)
{
	asm volatile("{\n\t.reg .b64 st;\n\tmbarrier.arrive.expect_tx.shared::cta.b64 st, [%0], %1;\n\t}" ::"r"(
	                 smem_addr(b)),
	             "r"(bytes)
	             : "memory");
}
__device__ __forceinline__ void bulk_to_smem(void *dst, void const *src, uint32_t bytes, unsigned long long *b)
{
	asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
	                 smem_addr(dst)),
	             "l"(src), "r"(bytes), "r"(smem_addr(b))
	             : "memory");
}
__device__ __forceinline__ bool mbar_try(unsigned long long *b, uint32_t parity)
{
	uint32_t ok;
	asm volatile("{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, "
	             "p;\n\t}"
	             : "=r"(ok)
	             : "r"(smem_addr(b)), "r"(parity)
	             : "memory");
	return ok != 0;
}
__device__ __forceinline__ uint64_t global_ns()
{
	uint64_t t;
	asm volatile("mov.u64 %0, %globaltimer;" : "=l"(t));
	return t;
}
// waits for the phase `parity` of b for at most `limit_ns`; false on timeout
__device__ __forceinline__ bool mbar_wait_bounded(unsigned long long *b, uint32_t parity, uint64_t limit_ns)
{
	uint64_t t0 = global_ns();
	while (!mbar_try(b, parity))
		if (global_ns() - t0 > limit_ns)
			return false;
	return true;
}
constexpr uint64_t kWaitLimitNs = 200000000ull; // 0.2 s: a line copy takes microseconds

template <class T, int NT, int MINB, int F2, bool ROWS, bool FUSE, bool R2 = false, bool FSM = false,
          bool PF = false, bool ST = false>
__global__ void __launch_bounds__(NT, MINB)
    k_md_line(Geom g, LineSpec ls, T const *__restrict__ U, T *__restrict__ P, T coef, RedSlot kin,
              T *__restrict__ Uout, T tu, int reunit)
{
	using Gp = Group<SU3, T>;
	using E = typename Gp::E;
	using Pr = LineProd<T, F2>;
	using PrO = Prod<SU3, T, F2>;
	using SW = typename Slot16<T>::W;
	constexpr int NA = 8;
	constexpr int NW = NT / 32;
	constexpr int NS = 3 * Slot16<T>::N * 32;
	// per warp: hand-over along x3 (3 links) and the carry along x1 (3 links)
	__shared__ SW sm_x3[NW][NS];
	__shared__ SW sm_x1[NW][NS];
	// FSM: the force accumulators of the warp's threads, [link][word][lane]
	__shared__ SW sm_f[FSM ? NW : 1][FSM ? 4 * Slot16<T>::N * 32 : 1];
	// ST (float, L3 = 32): the warp's own line, rows 0, 1 of the four links,
	// [link][plane][parity][x3 / 2] float4, filled by bulk copies
	static_assert(!ST || (sizeof(T) == 4 && ROWS), "staged lines: FP32 links read as rows 0, 1");
	__shared__ __align__(128) float4 sm_own[ST ? NW : 1][ST ? 24 * 16 : 1];
	__shared__ __align__(8) unsigned long long sm_bar[ST ? NW : 1];
	LineLoad<T, ROWS, R2> ld{U, uint32_t(g.V)};
	int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
	SW *s3 = sm_x3[wib];
	SW *s1 = sm_x1[wib];
	int wid = int(blockIdx.x) * NW + wib;
	int L1 = g.L[1], L3 = g.L[3];
	int sub = lane / L3;
	int lane_prev = sub * L3 + (lane % L3 == 0 ? L3 - 1 : lane % L3 - 1);
	int ngrp = g.L[2] / ls.ns;
	int col = wid % ls.ncol, seg = wid / ls.ncol;
	int t0 = seg * L1 / ls.nseg, t1 = wid < ls.nwork ? (seg + 1) * L1 / ls.nseg : t0;
	double acc = 0.0;
	// ST: copy the line (x0, t, x2) of every link's rows 0, 1 into sm_own
	float4 *own = ST ? sm_own[wib] : nullptr;
	unsigned long long *bar = ST ? &sm_bar[wib] : nullptr;
	uint32_t phase = 0;
	bool bad = false;
	auto stage = [&](int t) {
		if constexpr (ST)
		{
			if (lane == 0)
			{
				int x0 = col / ngrp, x2 = col - x0 * ngrp;
				uint32_t lbh = uint32_t((x0 * L1 + t) * g.L[2] + x2) * 16u;
				uint32_t V = uint32_t(g.V), Vh = uint32_t(g.Vh);
				float4 const *U4 = reinterpret_cast<float4 const *>(U);
				// the generic-proxy reads of the previous line come before the
				// copies overwrite it
				asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
				mbar_expect(bar, 24u * 256u);
#pragma unroll 1
				for (int c = 0; c < 24; ++c)
				{
					int mu = c / 6, k = (c / 2) % 3, p = c & 1;
					bulk_to_smem(own + c * 16, U4 + (uint32_t(mu) * 9u * (V >> 1) + uint32_t(k) * V + p * Vh + lbh),
					             256u, bar);
				}
			}
		}
	};
	if constexpr (ST)
	{
		if (lane == 0)
			mbar_init(bar);
		__syncwarp();
		if (t0 < t1)
			stage(t0);
	}
	for (int t = t0; t < t1 && !bad; ++t)
	{
		LineSite x;
		x.x1 = t;
		x.x0 = col / ngrp;
		x.x2 = (col - x.x0 * ngrp) * ls.ns + sub;
		x.x3 = lane % L3;
		uint32_t s = line_eo(g, x.x0, x.x1, x.x2, x.x3);
		if constexpr (ST)
		{
			// the line's copies (issued at the end of the previous step)
			// a warp-uniform decision: all lanes leave together or none
			bool ok = __all_sync(0xffffffffu, mbar_wait_bounded(bar, phase, kWaitLimitNs));
			if (!ok)
			{
				if (lane == 0 && ls.err)
					atomicExch(ls.err, 1);
				bad = true;
				break;
			}
			phase ^= 1u;
		}
		// own links from the staged line: lane xl of the warp's line, rows 0, 1
		auto own_rows = [&](int mu, int xl) {
			E e;
			if constexpr (ST)
			{
				int pl = (x.x0 + x.x1 + x.x2 + xl) & 1;
#pragma unroll
				for (int k = 0; k < 3; ++k)
				{
					float4 w = own[((mu * 3 + k) * 2 + pl) * 16 + (xl >> 1)];
					e.v[4 * k] = w.x;
					e.v[4 * k + 1] = w.y;
					e.v[4 * k + 2] = w.z;
					e.v[4 * k + 3] = w.w;
				}
			}
			return e;
		};
		auto own_full = [&](int mu, int xl) {
			E e = own_rows(mu, xl);
			Gp::complete_row2(e);
			return e;
		};
		int lane_next = (lane + 1) & 31;
		if (t == t0)
			line_carry<T, F2>(g, x, ld, s1, lane);
		LineNb nb = line_neighbours(g, x);
		FAcc<T, FSM> F(sm_f[FSM ? wib : 0], lane);
		// the carry from x - e_1: links 0, 2, 3
		{
			T z[NA], c[NA];
#pragma unroll
			for (int a = 0; a < NA; ++a)
				z[a] = T(0);
			F.set(1, z);
			slot_load<T>(s1, 0, lane, c);
			F.set(0, c);
			slot_load<T>(s1, 1, lane, c);
			F.set(2, c);
			slot_load<T>(s1, 2, lane, c);
			F.set(3, c);
		}
		__syncwarp();
		// the six plaquettes of x
#pragma unroll 1
		for (int q = 0; q < 6; ++q)
		{
			int mu = plane_mu<4>(q), nu = plane_nu<4>(q);
			if constexpr (PF)
			{
				// the neighbour links of the next plane (or, after the last
				// plane, of the first lower staple) into L1 while this one runs
				if (q < 5)
				{
					int m2 = plane_mu<4>(q + 1), n2 = plane_nu<4>(q + 1);
					ld.prefetch(n2, nb.fwd(m2));
					ld.prefetch(m2, nb.fwd(n2));
				}
				else
				{
					ld.prefetch_rows(0, nb.b2);
					ld.prefetch(2, nb.diag(2, 0));
					ld.prefetch(2, nb.b2);
				}
			}
			T o[8];
			if constexpr (ST)
			{
				// rows of U_mu(x), U_nu(x) and U_mu(x + e_3) from the staged line
				E M1 = Pr::mul01(own_rows(mu, lane), ld(nu, nb.fwd(mu)));
				E M2 = Pr::mul01(own_rows(nu, lane), nu == 3 ? own_full(mu, lane_next) : ld(mu, nb.fwd(nu)));
				Gp::complete_row2(M2);
				Pr::proj01(Pr::mul01_nd(M1, M2), o);
			}
			else
				plaquette_at<T, F2>(s, nb.fwd(mu), nb.fwd(nu), mu, nu, ld, o);
			F.add(mu, o, T(1));
			F.add(nu, o, T(-1));
			// hand-overs: along x1 (planes with mu or nu = 1), along x3 (nu = 3)
#pragma unroll 1
			for (int r = 0; r < 2; ++r)
			{
				int dir = r == 0 ? 1 : 3;
				bool send = r == 0 ? (mu == 1 || nu == 1) : (nu == 3);
				if (!send)
					continue;
				// the receiving link and the sign: (mu, nu) with dir == nu goes
				// to link mu with -V^+ A V, dir == mu to link nu with +
				int k = dir == nu ? mu : nu;
				T sg = dir == nu ? T(-1) : T(1);
				T c[8];
				Pr::adjoint(ST ? own_full(dir, lane) : ld(dir, s), o, sg, c);
				if (r == 0)
					slot_store<T>(s1, k == 0 ? 0 : k - 1, lane, c);
				else
					slot_store<T>(s3, k, lane, c);
			}
		}
		// lower staples along x0 and x2, summed per link and closed with U_mu(x)
#pragma unroll 1
		for (int mu = 0; mu < 4; ++mu)
		{
			E S = Gp::zero();
#pragma unroll 1
			for (int r = 0; r < 2; ++r)
			{
				int nu = r == 0 ? 0 : 2;
				if (nu == mu)
					continue;
				uint32_t y = nu == 0 ? nb.b0 : nb.b2;
				if constexpr (PF)
				{
					// the next lower staple's links: (mu, 2) after (mu, 0); else
					// the next link's first staple
					int mn = r == 0 && mu != 2 ? mu : mu + 1, nn = r == 0 && mu != 2 ? 2 : (mu + 1 == 0 ? 2 : 0);
					if (mn < 4)
					{
						uint32_t yn = nn == 0 ? nb.b0 : nb.b2;
						ld.prefetch_rows(mn, yn);
						ld.prefetch(nn, nb.diag(nn, mn));
						ld.prefetch(nn, yn);
					}
				}
				E f = ld(nu, nb.diag(nu, mu));
				E ef = PrO::mul_r2(ld.rows(mu, y), f);
				Gp::add_to(S, PrO::mul_dn(ef, ld(nu, y)));
			}
			T xa[NA];
			Pr::proj_mul(ST ? own_full(mu, lane) : ld(mu, s), S, xa);
			F.add(mu, xa, T(1));
		}
		// contributions from x - e_3 (the previous lane): links 0, 1, 2
		__syncwarp();
		{
			T c[8];
#pragma unroll
			for (int k = 0; k < 3; ++k)
			{
				slot_load<T>(s3, k, lane_prev, c);
				F.add(k, c, T(1));
			}
		}
		__syncwarp();
		// momentum update and (FUSE) the link update
#pragma unroll 1
		for (int mu = 0; mu < 4; ++mu)
		{
			T f[NA];
			F.get(mu, f);
			auto Pv = comp<T, NA>(P, g.V, mu);
			T p[NA];
			Pv.template load<CACHE_STREAM>(s, p);
#pragma unroll
			for (int a = 0; a < NA; ++a)
				p[a] -= coef * f[a];
			Pv.template store<CACHE_STREAM>(s, p);
			if (kin.result)
				acc += double(Gp::kin(p));
			if constexpr (FUSE)
			{
				E r;
				if constexpr (ROWS)
					r = PrO::mul_r2(Gp::exp_alg(p, tu), ST ? own_full(mu, lane) : ld(mu, s));
				else
					r = Gp::mul(Gp::exp_alg(p, tu), ld(mu, s));
				if (reunit)
					r = Gp::reunit_fast(r);
				comp<T, Gp::NR>(Uout, g.V, mu).store(s, r.v);
			}
		}
		if constexpr (ST)
		{
			// every lane is done with this line: copy the next one
			__syncwarp();
			if (t + 1 < t1)
				stage(t + 1);
		}
	}
	if constexpr (ST)
	{
		// after a wait gave up, the copies still in flight land before the
		// block's shared memory is released (bounded as well)
		if (bad)
			mbar_wait_bounded(bar, phase, kWaitLimitNs);
	}
	if (kin.result)
		grid_sum<NT>(acc, kin);
}

} // namespace meshgb
