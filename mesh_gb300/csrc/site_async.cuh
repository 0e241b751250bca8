// Thread-per-site momentum step for SU(3) in FP32 with the neighbour links
// of the next step copied into shared memory asynchronously (cp.async) while
// the current step is multiplied.
//
// The same operation and summation order as site_md's ROWS/F2 body (the
// reference's momentum step of runHmd, src/gauge/hmc.h:54-58, with
// wilsonDeriv/stapleSum of src/gauge/utils.h:114-153, fused with evolve,
// src/gauge/hmc.h:26-36). The site's work is a sequence of 18 steps: the six
// forward plaquette loops (two neighbour links each: U_nu(x+mu), U_mu(x+nu))
// and the twelve lower staples (three links each: U_mu(y), U_nu(y+mu),
// U_nu(y), y = x - nu). Rows 0 and 1 of the links of step t+1 are copied
// global -> shared by the thread's own cp.async (16 bytes each, L1-allocating)
// into the other half of a private double buffer before step t is computed;
// the wait for a step's copies (cp.async.wait_group 1) comes one step of
// arithmetic after they were issued. Unlike loads into registers issued
// ahead (site_md PIPE), the copies in flight hold no registers. A thread's
// buffer is [stage][link][16-byte chunk] with the threads of the block
// innermost, so that a warp's reads of one chunk are 512 contiguous bytes.
#pragma once

namespace meshgb {
namespace async_copy {

__device__ __forceinline__ void cp16(void *smem_dst, void const *gmem_src)
{
	uint32_t d = uint32_t(__cvta_generic_to_shared(smem_dst));
	asm volatile("cp.async.ca.shared.global [%0], [%1], 16;" ::"r"(d), "l"(gmem_src) : "memory");
}
__device__ __forceinline__ void commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N> __device__ __forceinline__ void wait_group() { asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory"); }

} // namespace async_copy

// the shared-memory floats a block of NT threads needs
template <int NT> inline constexpr int kAsyncSmemFloat4 = 2 * 3 * 3 * NT;

template <int NT, bool FUSE, class LD, bool SM>
__device__ __forceinline__ double site_md_async(Geom const &g, Site<4> const &st, int64_t s, LD const &ld,
                                                float const *__restrict__ U, float *__restrict__ P, float coef,
                                                float *__restrict__ Uout, float tu, int reunit, bool want_kin,
                                                float *acc_sm, float4 *buf)
{
	using Gp = Group<SU3, float>;
	using E = Gp::E;
	using Pr = Prod<SU3, float, 1>;
	constexpr int NA = 8;
	constexpr int64_t NR = Gp::NR;
	SiteAcc<float, 4, NA, SM> F(acc_sm);
	float4 const *U4 = reinterpret_cast<float4 const *>(U);
	int64_t const V = g.V;
	// chunk k of link l in stage b of this thread
	auto slot = [&](int b, int l, int k) { return buf + ((b * 3 + l) * 3 + k) * NT; };
	// rows 0, 1 of link (mu, idx) into slot (b, l)
	auto fetch = [&](int b, int l, int mu, int64_t idx) {
		float4 const *src = U4 + (int64_t(mu) * NR * V) / 4 + idx;
#pragma unroll
		for (int k = 0; k < 3; ++k)
			async_copy::cp16(slot(b, l, k), src + k * V);
	};
	auto read = [&](int b, int l) {
		E e;
#pragma unroll
		for (int k = 0; k < 3; ++k)
		{
			float4 t = *slot(b, l, k);
			e.v[4 * k] = t.x;
			e.v[4 * k + 1] = t.y;
			e.v[4 * k + 2] = t.z;
			e.v[4 * k + 3] = t.w;
		}
		return e;
	};
	// lower staple j = 3 mu + k: nu = k < mu ? k : k + 1
	auto staple_nu = [](int j) {
		int mu = j / 3, k = j - 3 * (j / 3);
		return k < mu ? k : k + 1;
	};
	// issue the copies of step t into stage b
	auto issue = [&](int t, int b) {
		if (t < 6)
		{
			int mu = plane_mu<4>(t), nu = plane_nu<4>(t);
			fetch(b, 0, nu, eo_shift1<4>(g, st, mu, +1));
			fetch(b, 1, mu, eo_shift1<4>(g, st, nu, +1));
		}
		else
		{
			int j = t - 6, mu = j / 3, nu = staple_nu(j);
			int64_t y = eo_shift1<4>(g, st, nu, -1);
			fetch(b, 0, mu, y);
			fetch(b, 1, nu, eo_shift2<4>(g, st, nu, -1, mu, +1));
			fetch(b, 2, nu, y);
		}
	};
	issue(0, 0);
	async_copy::commit();
	E S = Gp::zero();
#pragma unroll 1
	for (int t = 0; t < 18; ++t)
	{
		int b = t & 1;
		if (t + 1 < 18)
			issue(t + 1, b ^ 1);
		async_copy::commit();
		async_copy::wait_group<1>();
		if (t < 6)
		{
			int mu = plane_mu<4>(t), nu = plane_nu<4>(t);
			E nb = read(b, 0), nc = read(b, 1);
			Gp::complete_row2(nb);
			Gp::complete_row2(nc);
			E ab = Pr::mul_r2(ld.rows(mu, s), nb);
			E dc = Pr::mul_r2(ld.rows(nu, s), nc);
			float xa[NA];
			Gp::proj(Pr::mul_nd(ab, dc), xa);
			F.plane(t, xa);
		}
		else
		{
			int j = t - 6, mu = j / 3;
			E e = read(b, 0), f = read(b, 1), h = read(b, 2);
			Gp::complete_row2(f);
			Gp::complete_row2(h);
			Gp::add_to(S, Pr::mul_dn(Pr::mul_r2(e, f), h));
			if (j - 3 * mu == 2)
			{
				float xa[NA];
				Gp::proj(Pr::mul(ld(mu, s), S), xa);
				F.dir(mu, xa);
				S = Gp::zero();
			}
		}
	}
	float kacc = 0.f; // the site's kinetic terms in FP32, one FP64 add per site
#pragma unroll 1
	for (int mu = 0; mu < 4; ++mu)
	{
		float f[NA], p[NA];
		F.get(mu, f);
		auto Pv = comp<float, NA>(P, V, mu);
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
			comp<float, Gp::NR>(Uout, V, mu).store(s, r.v);
		}
	}
	return double(kacc);
}

} // namespace meshgb
