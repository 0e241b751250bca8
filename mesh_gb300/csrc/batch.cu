// Batched replicas: many independent 4D lattices of one group and precision,
// each with its own extents, beta and seed, advanced together by the HMC
// trajectory sequence of runHmcUpdate (src/gauge/hmc.cpp:73-107) in which
// every step is ONE persistent launch over all replicas.
//
// Layout in HBM: one allocation per field kind (U, U_new, P) holding the
// replicas' segments back to back (each 256-byte aligned), every segment in
// the single-lattice layout (even/odd structure of arrays). A device table of
// BatchRep descriptors holds each replica's geometry, pointers and seed.
//
// Work decomposition: the items of a launch (links: 4 planes of V_r per
// replica, or sites: one plane of V_r) are cut into chunks of 256 items that
// never straddle two planes or two replicas (a plane has ceil(V_r/256)
// chunks). A chunk is 256 consecutive sites of the even/odd order; as an
// option (tiles_ok) a chunk can be a 4x4x4x4 tile of sites (tiles in
// lexicographic order, sites of a tile lexicographic).
// The persistent grid walks the chunks grid-stride, so all blocks sweep the
// batch together and neighbouring links are shared in L2. A block's replica
// changes only at chunk boundaries (a block-uniform event), which is where
// per-replica FP64 sums are flushed: block sum -> partial [b][r] -> the last
// block adds, for each replica, the partials of exactly the blocks that
// covered it (deterministic for a given batch).
//
// MD steps: each momentum step runs fused with the link update after it in
// one launch over the sites of every replica (the single-lattice
// thread-per-site body, site_md), reading the proposal from Unew or Ut and
// writing it to the other; a one-thread-per-replica kernel swaps the two
// pointers when the proposal ends in Ut.
//
// Accept: the Metropolis kernel (one thread per replica) swaps the
// replica's U and U_new pointers in the descriptor table instead of copying
// the proposal, so an accepted trajectory costs no link traffic.
//
// Every per-link and per-site body is the single-lattice trajectory's one
// (force_item, the exp update, plaquette_site, the Philox momentum stream,
// SU(3) FP32 links read as rows 0 and 1), so replica r follows the same
// trajectory as a single chain with the same seed.
#include "field.cuh"
#include "kernels.cuh"
#include "rng.cuh"

#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <limits>
#include <string>
#include <vector>

namespace meshgb {
namespace {

constexpr int kChunk = 256; // items per chunk = threads per block
constexpr int kBND = 4;     // batches are 4D

struct BatchRep
{
	Geom g;
	void *U;       // accepted links
	void *Unew;    // proposal (swapped with U on accept)
	void *Ut;      // second proposal buffer of the fused MD steps (swapped with Unew)
	void *P;       // momenta
	uint64_t seed; // Philox key of the replica's momentum and Metropolis streams
	int64_t lchunk0, schunk0; // first chunk of the replica's links / sites
	int32_t cpp;              // chunks per plane: ceil(V / 256)
	int32_t tile;             // 1: a chunk is a 4^4 tile of sites (every extent a multiple of 4)
};

// one item space (links or sites) of a batch and its persistent grid
struct BatchSpace
{
	BatchRep const *reps;
	int R;
	bool sites;
	int64_t nchunks; // total chunks over all replicas
};

struct BatchRed
{
	double *part;      // [gridDim][R]
	double *result;    // [R]
	unsigned *counter; // zero between launches
};

__device__ __forceinline__ int64_t chunk0_of(BatchSpace const &sp, int r)
{
	if (r >= sp.R)
		return sp.nchunks;
	return sp.sites ? sp.reps[r].schunk0 : sp.reps[r].lchunk0;
}

__device__ __forceinline__ int find_rep(BatchSpace const &sp, int64_t c)
{
	int lo = 0, hi = sp.R - 1;
	while (lo < hi)
	{
		int mid = (lo + hi + 1) >> 1;
		if (chunk0_of(sp, mid) <= c)
			lo = mid;
		else
			hi = mid - 1;
	}
	return lo;
}

// a replica is walked in 4^4 tiles only when MESH_BATCH_TILES=1 is set in
// the environment and every extent is a multiple of 4. Measured on the
// 64-replica SU(2) workload (10 trajectories, GB300): 17.4 G link updates/s
// in tiles against 25.4 G in the even/odd chunk order, which stays the
// default (consecutive chunks of all blocks share neighbour lines in L2)
bool tiles_ok(int32_t const *d)
{
	static_assert(kChunk == 256, "a tile of 4^4 sites is one chunk");
	char const *e = std::getenv("MESH_BATCH_TILES");
	if (!(e && e[0] == '1'))
		return false;
	for (int i = 0; i < kBND; ++i)
		if (d[i] % 4 != 0)
			return false;
	return true;
}

// sum over the block (valid in thread 0); every thread must call it
__device__ __forceinline__ double block_sum(double v)
{
	__shared__ double sw[kChunk / 32];
	v = warp_sum(v);
	__syncthreads(); // sw may still be read by a previous call
	if ((threadIdx.x & 31) == 0)
		sw[threadIdx.x >> 5] = v;
	__syncthreads();
	double t = 0.0;
	if (threadIdx.x == 0)
		for (int i = 0; i < kChunk / 32; ++i)
			t += sw[i];
	return t;
}

// Runs body(r, rep, mu, s) -> double for the chunks c = blockIdx.x + k
// gridDim.x (the whole grid sweeps the batch together, as a grid-stride loop
// over one lattice does, so neighbouring links are shared in L2) with mu the
// direction plane (0 for sites) and s the even/odd site. The replica only
// grows along a block's chunks; the descriptor is reloaded when it changes.
// With RED, a block's sum over one replica's chunks is flushed when the
// replica changes (each (block, replica) pair once), and the last block adds
// for replica q the partials of the blocks that covered q's chunks [a, b):
// all blocks when b - a >= gridDim.x, else blocks a mod G .. (b-1) mod G
// (one warp per replica, in a fixed order: deterministic for a given batch).
//
// ACC: the type a thread sums the body's values in between two flushes (a
// replica's chunks of one block, a few items): the field's FP32 where the
// values are FP32 (FP64 adds cost FP64-pipe time on this part), FP64 for
// the block sums and the final reduction either way.
template <bool RED, class ACC = double, class Body>
__device__ __forceinline__ void batch_loop(BatchSpace const &sp, BatchRed red, Body &&body)
{
	int64_t const G = gridDim.x;
	int64_t c = blockIdx.x;
	int r = c < sp.nchunks ? find_rep(sp, c) : 0;
	int64_t first = chunk0_of(sp, r), next = chunk0_of(sp, r + 1);
	BatchRep rep = sp.reps[r];
	int cur = r;
	bool touched = false;
	ACC acc = ACC(0);
	for (; c < sp.nchunks; c += G)
	{
		if (c >= next)
		{
			if constexpr (RED)
			{
				double t = block_sum(double(acc));
				if (threadIdx.x == 0)
					red.part[int64_t(blockIdx.x) * sp.R + cur] = t;
				acc = ACC(0);
			}
			while (c >= next)
			{
				++r;
				first = next;
				next = chunk0_of(sp, r + 1);
			}
			rep = sp.reps[r];
			cur = r;
		}
		touched = true;
		uint32_t local = uint32_t(c - first);
		uint32_t mu = local / uint32_t(rep.cpp);
		uint32_t k = local - mu * uint32_t(rep.cpp);
		if (rep.tile)
		{
			// tile k of the replica, site threadIdx.x of the tile
			int x[kBND];
			uint32_t t = k, a = threadIdx.x;
#pragma unroll
			for (int i = kBND - 1; i >= 0; --i)
			{
				uint32_t n = uint32_t(rep.g.L[i]) >> 2;
				uint32_t q = t / n;
				x[i] = int((t - q * n) << 2) + int(a & 3u);
				t = q;
				a >>= 2;
			}
			Site<kBND> st = site_from_coords<kBND>(rep.g, x);
			acc += body(r, rep, int(mu), eo_of<kBND>(rep.g, st), st);
		}
		else
		{
			int64_t s = int64_t(k) * kChunk + threadIdx.x;
			if (s < rep.g.V)
				acc += body(r, rep, int(mu), s, site_from_eo<kBND>(rep.g, s));
		}
	}
	if constexpr (RED)
	{
		if (touched)
		{
			double t = block_sum(double(acc));
			if (threadIdx.x == 0)
				red.part[int64_t(blockIdx.x) * sp.R + cur] = t;
		}
		__shared__ bool is_last;
		if (threadIdx.x == 0)
		{
			__threadfence();
			unsigned prev = atomicInc(red.counter, gridDim.x - 1);
			is_last = (prev == gridDim.x - 1);
		}
		__syncthreads();
		if (is_last)
		{
			// one warp per replica: lane l adds the covering blocks' partials
			// l, l + 32, ... (blocks a mod G, a+1 mod G, ... in that order),
			// then the warp's shuffle tree: a fixed order, and the partials'
			// load latency paid once per 32 instead of once per partial
			__threadfence();
			int lane = threadIdx.x & 31;
			for (int q = threadIdx.x >> 5; q < sp.R; q += kChunk / 32)
			{
				int64_t a = chunk0_of(sp, q), b = chunk0_of(sp, q + 1);
				int64_t n = b - a >= G ? G : b - a;
				int64_t k0 = b - a >= G ? 0 : a % G;
				double sum = 0.0;
				for (int64_t i = lane; i < n; i += 32)
				{
					int64_t k = k0 + i;
					sum += __ldcg(red.part + (k < G ? k : k - G) * sp.R + q);
				}
				sum = warp_sum(sum);
				if (lane == 0)
					red.result[q] = sum;
			}
		}
	}
}

// Haar-random links (the stream of a single chain's randomize_gauge_field)
template <int GRP, class T> __global__ void __launch_bounds__(kChunk) kb_random_links(BatchSpace sp)
{
	using Gp = Group<GRP, T>;
	batch_loop<false>(sp, BatchRed{}, [&](int, BatchRep const &rep, int mu, int64_t s, Site<kBND> const &st) {
		T p[Gp::NNORM_GROUP];
		normals<T, Gp::NNORM_GROUP>(rep.seed, TAG_GAUGE, uint32_t(st.lex), uint32_t(mu), 0, p);
		auto e = Gp::group_from_normals(p);
		comp<T, Gp::NR>(static_cast<T *>(rep.U), rep.g.V, mu).store(s, e.v);
		return 0.0;
	});
}

template <int GRP, class T> __global__ void __launch_bounds__(kChunk) kb_unit_links(BatchSpace sp)
{
	using Gp = Group<GRP, T>;
	batch_loop<false>(sp, BatchRed{}, [&](int, BatchRep const &rep, int mu, int64_t s, Site<kBND> const &) {
		auto e = Gp::unit();
		comp<T, Gp::NR>(static_cast<T *>(rep.U), rep.g.V, mu).store(s, e.v);
		return 0.0;
	});
}

// momentum refresh from the replica's stream at its trajectory counter and the
// kinetic energy, fused with the trajectory's first link update U_new =
// exp(t P) U (optionally reunitised): the momenta are not read back
template <int GRP, class T, bool REUNIT>
__global__ void __launch_bounds__(kChunk)
    kb_refresh_evolve(BatchSpace sp, HmcDev const *__restrict__ dev, BatchRed kin, T t)
{
	using Gp = Group<GRP, T>;
	using E = typename Gp::E;
	batch_loop<true, T>(sp, kin, [&](int r, BatchRep const &rep, int mu, int64_t s, Site<kBND> const &st) {
		int64_t V = rep.g.V;
		T p[Gp::DIM], o[Gp::NA];
		normals<T, Gp::DIM>(rep.seed, TAG_MOMENTUM, uint32_t(st.lex), uint32_t(mu), dev[r].traj, p);
		Gp::alg_from_normals(p, o);
		comp<T, Gp::NA>(static_cast<T *>(rep.P), V, mu).store(s, o);
		E u;
		T const *src = static_cast<T const *>(rep.U);
		if constexpr (kRows<GRP, T>)
		{
			Soa<T, Gp::NR>::template load_head<12>(src + int64_t(mu) * Gp::NR * V, V, s, u.v);
			Gp::complete_row2(u);
		}
		else
			comp<T, Gp::NR>(const_cast<T *>(src), V, mu).load(s, u.v);
		E x = Gp::mul(Gp::exp_alg(o, t), u);
		if constexpr (REUNIT)
			x = Gp::reunit_fast(x);
		comp<T, Gp::NR>(static_cast<T *>(rep.Unew), V, mu).store(s, x.v);
		return Gp::kin(o);
	});
}

// U_new = exp(t P) U_new, optionally reunitised (the later link updates of a
// trajectory; the first is fused with the momentum refresh)
template <int GRP, class T, bool REUNIT>
__global__ void __launch_bounds__(kChunk) kb_evolve(BatchSpace sp, T t)
{
	using Gp = Group<GRP, T>;
	using E = typename Gp::E;
	batch_loop<false>(sp, BatchRed{}, [&](int, BatchRep const &rep, int mu, int64_t s, Site<kBND> const &) {
		int64_t V = rep.g.V;
		T p[Gp::NA];
		comp<T, Gp::NA>(static_cast<T *>(rep.P), V, mu).load(s, p);
		E u;
		T const *src = static_cast<T const *>(rep.Unew);
		if constexpr (kRows<GRP, T>)
		{
			Soa<T, Gp::NR>::template load_head<12>(src + int64_t(mu) * Gp::NR * V, V, s, u.v);
			Gp::complete_row2(u);
		}
		else
			comp<T, Gp::NR>(const_cast<T *>(src), V, mu).load(s, u.v);
		E x = Gp::mul(Gp::exp_alg(p, t), u);
		if constexpr (REUNIT)
			x = Gp::reunit_fast(x);
		comp<T, Gp::NR>(static_cast<T *>(rep.Unew), V, mu).store(s, x.v);
		return 0.0;
	});
}

// P -= (beta_r / (2 Nc)) delta proj(U_new S); with KIN also the kinetic sums
template <int GRP, class T, bool KIN>
__global__ void __launch_bounds__(kChunk)
    kb_force(BatchSpace sp, double const *__restrict__ beta, double delta, BatchRed kin)
{
	using Gp = Group<GRP, T>;
	batch_loop<KIN>(sp, kin, [&](int r, BatchRep const &rep, int mu, int64_t s, Site<kBND> const &st) {
		int64_t V = rep.g.V;
		LinkLoad<GRP, T, kBND, kRows<GRP, T>> ld{static_cast<T const *>(rep.Unew), V};
		T coef = T(beta[r] / (2.0 * Gp::NC) * delta);
		double k = force_item<GRP, T, kBND>(rep.g, st, s, mu, ld, static_cast<T *>(rep.P), coef);
		return KIN ? k : 0.0;
	});
}

// launch variants of the fused MD kernel. U(1)/SU(2) in FP32: 0 the
// unrolled per-site body (whose loads the compiler hoists) under a cap of 128
// registers (2 resident blocks of 256 per SM), 1 the same body under 80
// registers (3 blocks, spilling), 2 the rolled generic body under 128. One
// variant (1 block, the unrolled body for the small groups) otherwise.
// Measured on the 64-replica SU(2) workload: 41.9, 44.5-45.7 and 22.9 G link
// updates/s; the unrolled body under 64 registers (4 blocks, 908 bytes of
// spills) 30.2 G, not offered.
template <int GRP, class T> inline constexpr int kMdVariants = GRP != SU3 && sizeof(T) == 4 ? 3 : 1;
template <int GRP, class T> constexpr int md_min_blocks(int v)
{
	constexpr int mb[3] = {2, 3, 2};
	return kMdVariants<GRP, T> == 1 ? 1 : mb[v];
}
template <int GRP, class T> constexpr bool md_generic(int v) { return kMdVariants<GRP, T> > 1 && v == 2; }

// P -= (beta_r / (2 Nc)) dp proj(U S) fused with U' = exp(du P) U for the four
// links of every site; reads the proposal from Unew (flip = 0) or Ut (flip =
// 1) and writes it to the other; with KIN also the kinetic sums
template <int GRP, class T, bool KIN, int MB, bool GENERIC>
__global__ void __launch_bounds__(kChunk, MB)
    kb_md(BatchSpace sp, double const *__restrict__ beta, double dp, double du, int flip, int reunit, BatchRed kin)
{
	using Gp = Group<GRP, T>;
	constexpr int F2 = (GRP == SU3 && sizeof(T) == 4) ? 1 : 0;
	batch_loop<KIN, T>(sp, kin, [&](int r, BatchRep const &rep, int, int64_t s, Site<kBND> const &st) {
		LinkLoad<GRP, T, kBND, kRows<GRP, T>> ld{static_cast<T const *>(flip ? rep.Ut : rep.Unew), rep.g.V};
		T coef = T(beta[r] / (2.0 * Gp::NC) * dp);
		double k = site_md<GRP, T, kBND, F2, kRows<GRP, T>, true, decltype(ld), false, false, GENERIC>(
		    rep.g, st, s, ld, static_cast<T *>(rep.P), coef, static_cast<T *>(flip ? rep.Unew : rep.Ut), T(du),
		    reunit, KIN);
		return KIN ? T(k) : T(0); // k is the site's sum in T, exactly
	});
}

// the proposal back in Unew after an odd number of fused steps
__global__ void kb_swap_proposal(BatchRep *reps, int R)
{
	int r = blockIdx.x * blockDim.x + threadIdx.x;
	if (r >= R)
		return;
	void *t = reps[r].Unew;
	reps[r].Unew = reps[r].Ut;
	reps[r].Ut = t;
}

// per-replica plaquette trace sums of U (NEW: of U_new)
template <int GRP, class T, bool NEW> __global__ void __launch_bounds__(kChunk) kb_plaquette(BatchSpace sp, BatchRed out)
{
	batch_loop<true>(sp, out, [&](int, BatchRep const &rep, int, int64_t s, Site<kBND> const &st) {
		LinkLoad<GRP, T, kBND, kRows<GRP, T>> ld{static_cast<T const *>(NEW ? rep.Unew : rep.U), rep.g.V};
		return double(plaquette_site<GRP, T, kBND>(rep.g, st, s, ld));
	});
}

// Metropolis test per replica (k_metropolis for every replica); an accepted
// proposal becomes the replica's links by a pointer swap
__global__ void kb_metropolis(BatchRep *reps, int R, HmcDev *dev, HmcRecordDev *hist, int hist_cap,
                              double const *beta, double *S_cur, double const *K_old, double const *S_new,
                              double const *K_new, double Nc)
{
	int r = blockIdx.x * blockDim.x + threadIdx.x;
	if (r >= R)
		return;
	double nplanes_V = 6.0 * double(reps[r].g.V);
	double b = beta[r];
	double plaq_old = S_cur[r] / nplanes_V / Nc;
	double plaq_new = S_new[r] / nplanes_V / Nc;
	double H_old = (1.0 - plaq_old) * (b * nplanes_V) + K_old[r];
	double H_new = (1.0 - plaq_new) * (b * nplanes_V) + K_new[r];
	double dH = H_new - H_old;
	uint64_t traj = dev[r].traj;
	double u = metropolis_uniform(reps[r].seed, traj);
	bool finite = isfinite(H_old) && isfinite(H_new);
	bool acc = finite && (u < exp(-dH));
	if (!finite)
		dev[r].bad = 1;
	if (traj < uint64_t(hist_cap))
	{
		HmcRecordDev rec;
		rec.plaq = acc ? plaq_new : plaq_old;
		rec.dH = dH;
		rec.accept = acc ? 1.0 : 0.0;
		rec.H_old = H_old;
		rec.H_new = H_new;
		hist[int64_t(r) * hist_cap + int64_t(traj)] = rec;
	}
	if (acc)
	{
		S_cur[r] = S_new[r];
		void *t = reps[r].U;
		reps[r].U = reps[r].Unew;
		reps[r].Unew = t;
	}
	dev[r].accept_last = acc ? 1 : 0;
	dev[r].traj = traj + 1;
}

// launchers per (group, real type)
struct BatchOps
{
	void (*random_links)(cudaStream_t, unsigned, BatchSpace);
	void (*unit_links)(cudaStream_t, unsigned, BatchSpace);
	// momentum refresh + kinetic sums + the first link update U_new = exp(t P) U
	void (*refresh)(cudaStream_t, unsigned, BatchSpace, HmcDev const *, BatchRed, double t, bool reunit);
	void (*evolve)(cudaStream_t, unsigned, BatchSpace, double, bool reunit);
	void (*force)(cudaStream_t, unsigned, BatchSpace, double const *, double, BatchRed, bool kin);
	void (*plaquette)(cudaStream_t, unsigned, BatchSpace, BatchRed, bool on_new);
	void (*md)(cudaStream_t, unsigned, BatchSpace, double const *, double dp, double du, bool flip, bool reunit,
	           BatchRed, bool kin, int variant);
	// resident blocks per SM of kernel `which` (0 links-type, 1 force, 2 sites,
	// 3 + v the fused MD kernel in launch variant v)
	int (*occupancy)(int which);
	int md_variants;
	int (*md_bound)(int v); // the minimum resident blocks per SM variant v is compiled for
};

template <int GRP, class T> struct BatchImpl
{
	static void random_links(cudaStream_t st, unsigned g, BatchSpace sp)
	{
		kb_random_links<GRP, T><<<g, kChunk, 0, st>>>(sp);
		MESH_LAUNCH_CHECK();
	}
	static void unit_links(cudaStream_t st, unsigned g, BatchSpace sp)
	{
		kb_unit_links<GRP, T><<<g, kChunk, 0, st>>>(sp);
		MESH_LAUNCH_CHECK();
	}
	static void refresh(cudaStream_t st, unsigned g, BatchSpace sp, HmcDev const *dev, BatchRed kin, double t,
	                    bool reunit)
	{
		if (reunit)
			kb_refresh_evolve<GRP, T, true><<<g, kChunk, 0, st>>>(sp, dev, kin, T(t));
		else
			kb_refresh_evolve<GRP, T, false><<<g, kChunk, 0, st>>>(sp, dev, kin, T(t));
		MESH_LAUNCH_CHECK();
	}
	static void evolve(cudaStream_t st, unsigned g, BatchSpace sp, double t, bool reunit)
	{
		if (reunit)
			kb_evolve<GRP, T, true><<<g, kChunk, 0, st>>>(sp, T(t));
		else
			kb_evolve<GRP, T, false><<<g, kChunk, 0, st>>>(sp, T(t));
		MESH_LAUNCH_CHECK();
	}
	static void force(cudaStream_t st, unsigned g, BatchSpace sp, double const *beta, double delta, BatchRed kin,
	                  bool with_kin)
	{
		if (with_kin)
			kb_force<GRP, T, true><<<g, kChunk, 0, st>>>(sp, beta, delta, kin);
		else
			kb_force<GRP, T, false><<<g, kChunk, 0, st>>>(sp, beta, delta, kin);
		MESH_LAUNCH_CHECK();
	}
	static void plaquette(cudaStream_t st, unsigned g, BatchSpace sp, BatchRed out, bool on_new)
	{
		if (on_new)
			kb_plaquette<GRP, T, true><<<g, kChunk, 0, st>>>(sp, out);
		else
			kb_plaquette<GRP, T, false><<<g, kChunk, 0, st>>>(sp, out);
		MESH_LAUNCH_CHECK();
	}
	template <int V>
	static void md_v(cudaStream_t st, unsigned g, BatchSpace sp, double const *beta, double dp, double du, bool flip,
	                 bool reunit, BatchRed kin, bool with_kin)
	{
		constexpr int MB = md_min_blocks<GRP, T>(V);
		constexpr bool GEN = md_generic<GRP, T>(V);
		if (with_kin)
			kb_md<GRP, T, true, MB, GEN><<<g, kChunk, 0, st>>>(sp, beta, dp, du, flip ? 1 : 0, reunit ? 1 : 0, kin);
		else
			kb_md<GRP, T, false, MB, GEN><<<g, kChunk, 0, st>>>(sp, beta, dp, du, flip ? 1 : 0, reunit ? 1 : 0, kin);
		MESH_LAUNCH_CHECK();
	}
	static void md(cudaStream_t st, unsigned g, BatchSpace sp, double const *beta, double dp, double du, bool flip,
	               bool reunit, BatchRed kin, bool with_kin, int v)
	{
		if constexpr (kMdVariants<GRP, T> > 1)
		{
			if (v == 1)
				return md_v<1>(st, g, sp, beta, dp, du, flip, reunit, kin, with_kin);
			if (v == 2)
				return md_v<2>(st, g, sp, beta, dp, du, flip, reunit, kin, with_kin);
		}
		md_v<0>(st, g, sp, beta, dp, du, flip, reunit, kin, with_kin);
	}
	template <int V> static int md_occupancy()
	{
		int n = 0;
		MESH_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, kb_md<GRP, T, true, md_min_blocks<GRP, T>(V), md_generic<GRP, T>(V)>,
		                                                        kChunk, 0));
		return n;
	}
	static int occupancy(int which)
	{
		int n = 0;
		cudaError_t e;
		if (which >= 3)
		{
			if constexpr (kMdVariants<GRP, T> > 1)
			{
				if (which == 4)
					return md_occupancy<1>();
				if (which == 5)
					return md_occupancy<2>();
			}
			return md_occupancy<0>();
		}
		if (which == 1)
			e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, kb_force<GRP, T, true>, kChunk, 0);
		else if (which == 2)
			e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, kb_plaquette<GRP, T, true>, kChunk, 0);
		else
			e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, kb_evolve<GRP, T, true>, kChunk, 0);
		MESH_CUDA(e);
		return n;
	}
	static int md_bound(int v) { return md_min_blocks<GRP, T>(v); }
	static constexpr BatchOps ops{random_links, unit_links, refresh, evolve, force, plaquette, md, occupancy,
	                              kMdVariants<GRP, T>, md_bound};
};

BatchOps const &batch_ops(int group, int prec)
{
	static BatchOps const t[3][2] = {{BatchImpl<U1, float>::ops, BatchImpl<U1, double>::ops},
	                                 {BatchImpl<SU2, float>::ops, BatchImpl<SU2, double>::ops},
	                                 {BatchImpl<SU3, float>::ops, BatchImpl<SU3, double>::ops}};
	return t[group - 1][prec == MESH_F32 ? 0 : 1];
}

} // namespace
} // namespace meshgb

using namespace meshgb;

struct mesh_batch_s
{
	Context *ctx = nullptr;
	int group = 0, prec = 0, R = 0;
	std::vector<int32_t> dims;  // R x 4
	std::vector<BatchRep> reps; // host copy at creation (initial pointers)
	void *bufU = nullptr, *bufUnew = nullptr, *bufUt = nullptr, *bufP = nullptr;
	BatchRep *d_reps = nullptr;
	HmcDev *d_dev = nullptr;
	HmcRecordDev *d_hist = nullptr;
	int hist_cap = 0;
	double *d_beta = nullptr;
	double *d_part = nullptr, *d_res = nullptr; // partials [G][R]; results [4][R]
	unsigned *d_cnt = nullptr;
	BatchSpace links{}, sites{};
	unsigned g_links = 0, g_force = 0, g_sites = 0; // grids (links space uses g_links/g_force chunks)
	unsigned g_md[3] = {};                          // grid of each launch variant of the fused MD kernel
	BatchSpace md_sp[3]{};
	int use_md = -1; // fused MD steps (1) or separate kernels (0), timed at the first run; -1 not yet
	int md_var = 0;  // the fused kernel's launch variant (timed with use_md)
	BatchSpace force_sp{};
	int64_t count = 0;
	bool S_valid = false;
	cudaGraphExec_t graph = nullptr;
	std::vector<double> graph_deltas;
	HmcRecordDev *graph_hist = nullptr;

	enum
	{
		S_CUR = 0,
		K_OLD = 1,
		S_NEW = 2,
		K_NEW = 3,
	};
	BatchRed red(int k) { return {d_part, d_res + size_t(k) * R, d_cnt + k}; }
	BatchOps const &ops() const { return batch_ops(group, prec); }

	void drop_graph()
	{
		if (graph)
			cudaGraphExecDestroy(graph);
		graph = nullptr;
	}

	~mesh_batch_s()
	{
		if (!ctx)
			return;
		cudaSetDevice(ctx->device);
		cudaStreamSynchronize(ctx->stream);
		drop_graph();
		for (void *p : {bufU, bufUnew, bufUt, bufP, static_cast<void *>(d_reps), static_cast<void *>(d_dev),
		                static_cast<void *>(d_hist), static_cast<void *>(d_beta), static_cast<void *>(d_part),
		                static_cast<void *>(d_res), static_cast<void *>(d_cnt)})
			if (p)
				cudaFree(p);
		ctx_release(ctx);
	}

	// space with its persistent grid: G = min(resident blocks, chunks)
	static BatchSpace make_space(BatchRep const *reps, int R, bool sites, int64_t nchunks, int64_t target,
	                             unsigned *grid)
	{
		int64_t G = std::max<int64_t>(1, std::min<int64_t>(target, nchunks));
		*grid = unsigned(G);
		return BatchSpace{reps, R, sites, nchunks};
	}

	void ensure_history(int64_t need)
	{
		if (need <= hist_cap)
			return;
		int cap = hist_cap ? hist_cap : 256;
		while (cap < need)
			cap *= 2;
		HmcRecordDev *nh = nullptr;
		MESH_CUDA(cudaMalloc(&nh, size_t(cap) * R * sizeof(HmcRecordDev)));
		MESH_CUDA(cudaStreamSynchronize(ctx->stream));
		if (d_hist)
		{
			MESH_CUDA(cudaMemcpy2D(nh, size_t(cap) * sizeof(HmcRecordDev), d_hist, size_t(hist_cap) * sizeof(HmcRecordDev),
			                       size_t(hist_cap) * sizeof(HmcRecordDev), R, cudaMemcpyDeviceToDevice));
			cudaFree(d_hist);
		}
		d_hist = nh;
		hist_cap = cap;
		drop_graph();
	}

	// one trajectory of every replica (runHmcUpdate, hmc.cpp:73-107)
	void enqueue(double const *deltas, int n)
	{
		cudaStream_t st = ctx->stream;
		auto const &o = ops();
		if (!S_valid)
		{
			o.plaquette(st, g_sites, sites, red(S_CUR), false);
			S_valid = true;
		}
		// the momenta and the first link update (step 0) in one pass
		o.refresh(st, g_links, links, d_dev, red(K_OLD), deltas[0], n == 1);
		int last_p = n >= 3 ? n - 2 : -1;
		bool flip = false; // the proposal is in Ut
		auto unflip = [&] {
			if (flip)
			{
				kb_swap_proposal<<<(R + 127) / 128, 128, 0, st>>>(d_reps, R);
				MESH_LAUNCH_CHECK();
				flip = false;
			}
		};
		for (int i = 0; i < n; ++i)
		{
			if (i % 2 == 0)
			{
				unflip();
				if (i > 0)
					o.evolve(st, g_links, links, deltas[i], i == n - 1);
			}
			else if (i + 1 < n && use_md == 1)
			{
				// momentum step i fused with the link update i + 1
				o.md(st, g_md[md_var], md_sp[md_var], d_beta, deltas[i], deltas[i + 1], flip, i + 1 == n - 1,
				     red(K_NEW), i == last_p, md_var);
				flip = !flip;
				++i;
			}
			else
			{
				unflip();
				o.force(st, g_force, force_sp, d_beta, deltas[i], red(K_NEW), i == last_p);
			}
		}
		unflip();
		o.plaquette(st, g_sites, sites, red(S_NEW), true);
		kb_metropolis<<<(R + 127) / 128, 128, 0, st>>>(d_reps, R, d_dev, d_hist, hist_cap, d_beta, d_res + size_t(S_CUR) * R,
		                                             d_res + size_t(K_OLD) * R, d_res + size_t(S_NEW) * R,
		                                             d_res + size_t(K_NEW) * R, double(group_nc(group)));
		MESH_LAUNCH_CHECK();
		++count;
	}

	// fused or separate MD steps: whichever is faster on this batch, timed once
	// (dp = du = 0: the momenta and the proposal keep their values; the first
	// trajectory's momentum refresh and link update overwrite both anyway)
	void tune_md()
	{
		if (use_md >= 0)
			return;
		cudaStream_t st = ctx->stream;
		auto const &o = ops();
		// MESH_BATCH_MD pins the choice instead: "sep", or a fused launch variant
		if (char const *pin = std::getenv("MESH_BATCH_MD"); pin && pin[0])
		{
			if (std::string(pin) == "sep")
			{
				use_md = 0;
				return;
			}
			int v = std::atoi(pin);
			require(v >= 0 && v < o.md_variants, "MESH_BATCH_MD: no such fused launch variant");
			use_md = 1;
			md_var = v;
			return;
		}
		cudaEvent_t e0, e1;
		MESH_CUDA(cudaEventCreate(&e0));
		MESH_CUDA(cudaEventCreate(&e1));
		auto timed = [&](auto &&f) {
			f();
			MESH_CUDA(cudaEventRecord(e0, st));
			for (int r = 0; r < 3; ++r)
				f();
			MESH_CUDA(cudaEventRecord(e1, st));
			MESH_CUDA(cudaEventSynchronize(e1));
			float ms = 0;
			MESH_CUDA(cudaEventElapsedTime(&ms, e0, e1));
			return ms;
		};
		float t_md = 0.f;
		for (int v = 0; v < o.md_variants; ++v)
		{
			float t = timed([&] {
				o.md(st, g_md[v], md_sp[v], d_beta, 0.0, 0.0, false, false, red(K_NEW), false, v);
				o.md(st, g_md[v], md_sp[v], d_beta, 0.0, 0.0, true, false, red(K_NEW), false, v);
			});
			if (v == 0 || t < t_md)
			{
				t_md = t;
				md_var = v;
			}
		}
		float t_sep = timed([&] {
			for (int k = 0; k < 2; ++k)
			{
				o.force(st, g_force, force_sp, d_beta, 0.0, red(K_NEW), false);
				o.evolve(st, g_links, links, 0.0, false);
			}
		});
		cudaEventDestroy(e0);
		cudaEventDestroy(e1);
		use_md = t_md < t_sep ? 1 : 0;
	}

	// the replica's current link buffer (the descriptor table is updated on
	// the device by accepted trajectories)
	void *current_links(int r)
	{
		BatchRep rep;
		MESH_CUDA(cudaMemcpyAsync(&rep, d_reps + r, sizeof(rep), cudaMemcpyDeviceToHost, ctx->stream));
		MESH_CUDA(cudaStreamSynchronize(ctx->stream));
		return rep.U;
	}

	Field view(int r, void *d)
	{
		Field f;
		f.ctx = ctx;
		f.kind = MESH_GROUP;
		f.group = group;
		f.prec = prec;
		f.nd = kBND;
		f.nstack = kBND;
		for (int i = 0; i < kBND; ++i)
			f.dims[i] = dims[size_t(r) * kBND + i];
		f.geom = make_geom(kBND, f.dims);
		f.nr = group_nr(group);
		f.nr_host = group_nr(group);
		f.real_bytes = prec == MESH_F32 ? 4 : 8;
		f.bytes = size_t(kBND) * size_t(f.geom.V) * f.nr * f.real_bytes;
		f.d = d;
		return f;
	}
};

namespace {
int batch_api_fail(char const *msg)
{
	set_last_error(msg);
	return MESH_ERR_ARG;
}
} // namespace

extern "C" {

int mesh_batch_create(mesh_ctx ctxh, int group, int precision, int nrep, int32_t const *dims, uint64_t const *seeds,
                      mesh_batch *out)
{
	if (!out)
		return batch_api_fail("null output handle");
	*out = nullptr;
	if (!ctxh)
		return batch_api_fail("null context");
	auto *h = new mesh_batch_s();
	int rc = api_call([&] {
		require(group >= 1 && group <= 3, "unknown gauge group");
		require(precision == MESH_F32 || precision == MESH_F64, "invalid precision level");
		require(nrep >= 1 && nrep <= 4096, "number of replicas must be in [1, 4096]");
		require(dims != nullptr && seeds != nullptr, "null dims or seeds");
		Context &c = ctxh->c;
		DeviceGuard dg(c.device);
		h->group = group;
		h->prec = precision;
		h->R = nrep;
		h->dims.assign(dims, dims + size_t(nrep) * kBND);
		size_t rb = precision == MESH_F32 ? 4 : 8;
		size_t nr = size_t(group_nr(group)), na = size_t(group_na(group));
		auto align = [](size_t x) { return (x + 255) & ~size_t(255); };
		std::vector<size_t> offU(nrep), offP(nrep);
		size_t totU = 0, totP = 0;
		int64_t lch = 0, sch = 0;
		h->reps.resize(nrep);
		for (int r = 0; r < nrep; ++r)
		{
			int64_t V = 1;
			for (int i = 0; i < kBND; ++i)
			{
				int32_t L = dims[size_t(r) * kBND + i];
				require(L >= 2 && L % 2 == 0, "every extent must be even and >= 2 (checkerboard layout)");
				require(L < 256, "every extent must be below 256");
				V *= L;
				require(V < (int64_t(1) << 31), "volume must be below 2^31");
			}
			BatchRep &rep = h->reps[r];
			rep.g = make_geom(kBND, dims + size_t(r) * kBND);
			rep.seed = seeds[r];
			rep.lchunk0 = lch;
			rep.schunk0 = sch;
			rep.cpp = int32_t((V + kChunk - 1) / kChunk);
			rep.tile = tiles_ok(dims + size_t(r) * kBND) ? 1 : 0;
			lch += int64_t(kBND) * rep.cpp;
			sch += rep.cpp;
			offU[r] = totU;
			offP[r] = totP;
			totU += align(size_t(kBND) * size_t(V) * nr * rb);
			totP += align(size_t(kBND) * size_t(V) * na * rb);
		}
		MESH_CUDA(cudaMalloc(&h->bufU, totU));
		MESH_CUDA(cudaMalloc(&h->bufUnew, totU));
		MESH_CUDA(cudaMalloc(&h->bufUt, totU));
		MESH_CUDA(cudaMalloc(&h->bufP, totP));
		for (int r = 0; r < nrep; ++r)
		{
			h->reps[r].U = static_cast<char *>(h->bufU) + offU[r];
			h->reps[r].Unew = static_cast<char *>(h->bufUnew) + offU[r];
			h->reps[r].Ut = static_cast<char *>(h->bufUt) + offU[r];
			h->reps[r].P = static_cast<char *>(h->bufP) + offP[r];
		}
		MESH_CUDA(cudaMalloc(&h->d_reps, sizeof(BatchRep) * nrep));
		MESH_CUDA(cudaMemcpy(h->d_reps, h->reps.data(), sizeof(BatchRep) * nrep, cudaMemcpyHostToDevice));
		MESH_CUDA(cudaMalloc(&h->d_dev, sizeof(HmcDev) * nrep));
		MESH_CUDA(cudaMemset(h->d_dev, 0, sizeof(HmcDev) * nrep));
		MESH_CUDA(cudaMalloc(&h->d_beta, sizeof(double) * nrep));
		MESH_CUDA(cudaMemset(h->d_beta, 0, sizeof(double) * nrep));
		auto const &o = batch_ops(group, precision);
		int64_t sms = c.num_sms;
		h->links = mesh_batch_s::make_space(h->d_reps, nrep, false, lch, sms * std::min(8, o.occupancy(0)), &h->g_links);
		h->force_sp =
		    mesh_batch_s::make_space(h->d_reps, nrep, false, lch, sms * std::min(8, o.occupancy(1)), &h->g_force);
		h->sites = mesh_batch_s::make_space(h->d_reps, nrep, true, sch, sms * std::min(8, o.occupancy(2)), &h->g_sites);
		unsigned G = std::max({h->g_links, h->g_force, h->g_sites});
		for (int v = 0; v < o.md_variants; ++v)
		{
			h->md_sp[v] = mesh_batch_s::make_space(h->d_reps, nrep, true, sch, sms * std::min(8, o.occupancy(3 + v)),
			                                       &h->g_md[v]);
			G = std::max(G, h->g_md[v]);
		}
		MESH_CUDA(cudaMalloc(&h->d_part, sizeof(double) * size_t(G) * nrep));
		MESH_CUDA(cudaMalloc(&h->d_res, sizeof(double) * 4 * size_t(nrep)));
		MESH_CUDA(cudaMemset(h->d_res, 0, sizeof(double) * 4 * size_t(nrep)));
		MESH_CUDA(cudaMalloc(&h->d_cnt, sizeof(unsigned) * 4));
		MESH_CUDA(cudaMemset(h->d_cnt, 0, sizeof(unsigned) * 4));
		h->ctx = &c;
		ctx_retain(c);
		// unit links until the caller chooses a start
		o.unit_links(c.stream, h->g_links, h->links);
		MESH_CUDA(cudaStreamSynchronize(c.stream));
	});
	if (rc != MESH_OK)
	{
		if (!h->ctx)
		{
			for (void *p : {h->bufU, h->bufUnew, h->bufUt, h->bufP, static_cast<void *>(h->d_reps), static_cast<void *>(h->d_dev),
			                static_cast<void *>(h->d_beta), static_cast<void *>(h->d_part),
			                static_cast<void *>(h->d_res), static_cast<void *>(h->d_cnt)})
				if (p)
					cudaFree(p);
		}
		delete h;
		return rc;
	}
	*out = h;
	return MESH_OK;
}

int mesh_batch_destroy(mesh_batch h)
{
	delete h;
	return MESH_OK;
}

int mesh_batch_size(mesh_batch h, int *nrep)
{
	return api_call([&] {
		require(h != nullptr && nrep != nullptr, "null argument");
		*nrep = h->R;
	});
}

int mesh_batch_randomize(mesh_batch h)
{
	return api_call([&] {
		require(h != nullptr, "null batch");
		DeviceGuard dg(h->ctx->device);
		// descriptors back to the creation pointers, so that U is the buffer
		// the random links go to whatever earlier trajectories swapped
		MESH_CUDA(cudaMemcpyAsync(h->d_reps, h->reps.data(), sizeof(BatchRep) * h->R, cudaMemcpyHostToDevice,
		                          h->ctx->stream));
		h->ops().random_links(h->ctx->stream, h->g_links, h->links);
		h->S_valid = false;
		MESH_CUDA(cudaStreamSynchronize(h->ctx->stream));
	});
}

int mesh_batch_cold_start(mesh_batch h)
{
	return api_call([&] {
		require(h != nullptr, "null batch");
		DeviceGuard dg(h->ctx->device);
		MESH_CUDA(cudaMemcpyAsync(h->d_reps, h->reps.data(), sizeof(BatchRep) * h->R, cudaMemcpyHostToDevice,
		                          h->ctx->stream));
		h->ops().unit_links(h->ctx->stream, h->g_links, h->links);
		h->S_valid = false;
		MESH_CUDA(cudaStreamSynchronize(h->ctx->stream));
	});
}

int mesh_batch_import(mesh_batch h, int r, void const *host, size_t bytes)
{
	return api_call([&] {
		require(h != nullptr, "null batch");
		require(r >= 0 && r < h->R, "replica index out of range");
		DeviceGuard dg(h->ctx->device);
		Field f = h->view(r, h->current_links(r));
		field_import_host(f, host, bytes);
		h->S_valid = false;
	});
}

int mesh_batch_export(mesh_batch h, int r, void *host, size_t bytes)
{
	return api_call([&] {
		require(h != nullptr, "null batch");
		require(r >= 0 && r < h->R, "replica index out of range");
		DeviceGuard dg(h->ctx->device);
		Field f = h->view(r, h->current_links(r));
		field_export_host(f, host, bytes);
	});
}

int mesh_batch_run(mesh_batch h, double const *betas, double const *deltas, int n, int count, int use_graph)
{
	return api_call([&] {
		require(h != nullptr, "null batch");
		require(betas != nullptr, "null betas");
		require(deltas != nullptr && n >= 1, "empty step table");
		require(n % 2 == 1, "step table must alternate position/momentum steps and have odd length");
		require(count >= 0, "count must be >= 0");
		for (int r = 0; r < h->R; ++r)
			require(std::isfinite(betas[r]), "non-finite beta");
		DeviceGuard dg(h->ctx->device);
		cudaStream_t st = h->ctx->stream;
		h->ensure_history(h->count + count);
		// betas are read by the kernels from device memory: a captured
		// trajectory stays valid when they change
		MESH_CUDA(cudaMemcpyAsync(h->d_beta, betas, sizeof(double) * h->R, cudaMemcpyHostToDevice, st));
		h->tune_md();
		if (!use_graph)
		{
			for (int k = 0; k < count; ++k)
				h->enqueue(deltas, n);
			MESH_CUDA(cudaStreamSynchronize(st));
			return;
		}
		if (!h->S_valid)
		{
			h->ops().plaquette(st, h->g_sites, h->sites, h->red(mesh_batch_s::S_CUR), false);
			h->S_valid = true;
		}
		std::vector<double> dv(deltas, deltas + n);
		if (!h->graph || h->graph_deltas != dv || h->graph_hist != h->d_hist)
		{
			h->drop_graph();
			cudaGraph_t g = nullptr;
			MESH_CUDA(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
			int64_t saved = h->count;
			try
			{
				h->enqueue(deltas, n);
			}
			catch (...)
			{
				cudaStreamEndCapture(st, &g);
				if (g)
					cudaGraphDestroy(g);
				throw;
			}
			h->count = saved;
			MESH_CUDA(cudaStreamEndCapture(st, &g));
			cudaGraphExec_t exec = nullptr;
			cudaError_t e = cudaGraphInstantiate(&exec, g, 0);
			cudaGraphDestroy(g);
			MESH_CUDA(e);
			h->graph = exec;
			h->graph_deltas = dv;
			h->graph_hist = h->d_hist;
		}
		for (int k = 0; k < count; ++k)
			MESH_CUDA(cudaGraphLaunch(h->graph, st));
		h->count += count;
		MESH_CUDA(cudaStreamSynchronize(st));
	});
}

int mesh_batch_count(mesh_batch h, int *n)
{
	return api_call([&] {
		require(h != nullptr && n != nullptr, "null argument");
		*n = int(h->count);
	});
}

int mesh_batch_history(mesh_batch h, int r, int first, int count, double *plaquette, double *dH, double *accept)
{
	return api_call([&] {
		require(h != nullptr, "null batch");
		require(r >= 0 && r < h->R, "replica index out of range");
		require(first >= 0 && count >= 0 && int64_t(first) + count <= h->count, "history range out of bounds");
		DeviceGuard dg(h->ctx->device);
		std::vector<HmcRecordDev> buf(static_cast<size_t>(count));
		if (count)
		{
			MESH_CUDA(cudaMemcpyAsync(buf.data(), h->d_hist + int64_t(r) * h->hist_cap + first,
			                          sizeof(HmcRecordDev) * size_t(count), cudaMemcpyDeviceToHost, h->ctx->stream));
			MESH_CUDA(cudaStreamSynchronize(h->ctx->stream));
		}
		for (int k = 0; k < count; ++k)
		{
			if (plaquette)
				plaquette[k] = buf[k].plaq;
			if (dH)
				dH[k] = buf[k].dH;
			if (accept)
				accept[k] = buf[k].accept;
		}
	});
}

int mesh_batch_plaquettes(mesh_batch h, double *out)
{
	return api_call([&] {
		require(h != nullptr && out != nullptr, "null argument");
		DeviceGuard dg(h->ctx->device);
		cudaStream_t st = h->ctx->stream;
		// S_CUR's slot is the trajectory's running action: use S_NEW's
		h->ops().plaquette(st, h->g_sites, h->sites, h->red(mesh_batch_s::S_NEW), false);
		std::vector<double> s(static_cast<size_t>(h->R));
		MESH_CUDA(cudaMemcpyAsync(s.data(), h->d_res + size_t(mesh_batch_s::S_NEW) * h->R, sizeof(double) * h->R,
		                          cudaMemcpyDeviceToHost, st));
		MESH_CUDA(cudaStreamSynchronize(st));
		for (int r = 0; r < h->R; ++r)
		{
			double V = double(h->reps[r].g.V);
			out[r] = s[r] / (6.0 * V) / double(group_nc(h->group));
		}
	});
}

int mesh_batch_launch_info(mesh_batch h, int *launches_per_trajectory, int n_deltas, int *grid_links, int *grid_sites)
{
	return api_call([&] {
		require(h != nullptr, "null batch");
		require(n_deltas >= 1 && n_deltas % 2 == 1, "step table length must be odd");
		// fused: refresh with the first link update + (n - 1) / 2 fused MD
		// steps (+ the pointer swap when that count is odd) + plaquette +
		// Metropolis; separate: refresh with the first link update + the other
		// n - 1 MD steps + plaquette + Metropolis
		int n_md = (n_deltas - 1) / 2;
		if (launches_per_trajectory)
			*launches_per_trajectory = h->use_md == 1 ? 1 + n_md + (n_md % 2) + 1 + 1 : n_deltas + 2;
		if (grid_links)
			*grid_links = int(h->g_force);
		if (grid_sites)
			*grid_sites = int(h->g_sites);
	});
}

int mesh_batch_md_launch(mesh_batch h, int *fused, int *variant, int *min_blocks, int *grid)
{
	return api_call([&] {
		require(h != nullptr, "null batch");
		int v = h->md_var;
		if (fused)
			*fused = h->use_md;
		if (variant)
			*variant = v;
		if (min_blocks)
			*min_blocks = h->ops().md_bound(v);
		if (grid)
			*grid = int(h->g_md[v]);
	});
}

} // extern "C"
