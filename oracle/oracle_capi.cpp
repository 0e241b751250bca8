// TEST INFRASTRUCTURE — NOT PART OF THE PRODUCT.
//
// C entry points of the CPU oracle (oracle.hpp) for ctypes. Every buffer is in
// the reference's host layout: lexicographic sites (grid.h:39-49), one
// array-of-structs block of V objects per direction mu (lattice.h:159-192),
// objects as util would pack them (complex: re,im; quaternion: re,i,j,k;
// 3x3 complex matrix: row-major re,im pairs). Group codes follow
// dispatchByGroup (utils.h:156-186): 1=u1, 2=su2, 3=su3; precision 1=float,
// 2=double. Functions return 0 on success and -1 on error (message via
// oracle_last_error).
#include "oracle.hpp"
#include "oracle_ext.hpp"

#include <cstdio>
#include <exception>
#include <string>

using namespace oracle;

namespace {
thread_local std::string g_err;

template <class G> GaugeField<G> load_stack(Grid const &g, int n, void const *p)
{
	GaugeField<G> U(n, Field<G>(g.V));
	auto const *src = static_cast<G const *>(p);
	for (int mu = 0; mu < n; ++mu)
		std::memcpy(U[mu].data(), src + size_t(mu) * g.V, g.V * sizeof(G));
	return U;
}
template <class G> void store_stack(Grid const &g, GaugeField<G> const &U, void *p)
{
	auto *dst = static_cast<G *>(p);
	for (size_t mu = 0; mu < U.size(); ++mu)
		std::memcpy(dst + mu * g.V, U[mu].data(), g.V * sizeof(G));
}
template <class G> Field<G> load_field(Grid const &g, void const *p)
{
	Field<G> f(g.V);
	std::memcpy(f.data(), p, g.V * sizeof(G));
	return f;
}
template <class G> void store_field(Field<G> const &f, void *p)
{
	std::memcpy(p, f.data(), f.size() * sizeof(G));
}

template <class F> int guarded(F f)
{
	try
	{
		f();
		return 0;
	}
	catch (std::exception const &e)
	{
		g_err = e.what();
		return -1;
	}
}

// dispatch over (group, precision) to a generic lambda taking a G value
template <class F> void dispatch(int group, int prec, F f)
{
	if (prec == 1)
	{
		if (group == 1)
			f(cplx<float>{});
		else if (group == 2)
			f(quat<float>{});
		else if (group == 3)
			f(mat3<float>{});
		else
			throw std::runtime_error("unknown gauge group");
	}
	else if (prec == 2)
	{
		if (group == 1)
			f(cplx<double>{});
		else if (group == 2)
			f(quat<double>{});
		else if (group == 3)
			f(mat3<double>{});
		else
			throw std::runtime_error("unknown gauge group");
	}
	else
		throw std::runtime_error("invalid precision level");
}
} // namespace

extern "C" {

char const *oracle_last_error() { return g_err.c_str(); }

int oracle_set_threads(int n)
{
#ifdef _OPENMP
	if (n > 0)
		omp_set_num_threads(n);
	return omp_get_max_threads();
#else
	(void)n;
	return 1;
#endif
}

int oracle_make_deltas(char const *scheme, double eps, int substeps, double *out, int cap)
{
	int n = -1;
	int rc = guarded([&] {
		auto d = makeDeltas(scheme, eps, substeps);
		if ((int)d.size() > cap)
			throw std::runtime_error("deltas buffer too small");
		std::copy(d.begin(), d.end(), out);
		n = (int)d.size();
	});
	return rc ? -1 : n;
}

int oracle_plaquette(int grp, int prec, int nd, int const *dims, void const *U, double *out)
{
	return guarded([&] {
		Grid g(nd, dims);
		dispatch(grp, prec, [&](auto tag) {
			using G = decltype(tag);
			*out = plaquette(g, load_stack<G>(g, nd, U));
		});
	});
}

int oracle_wilson_action(int grp, int prec, int nd, int const *dims, void const *U, double beta,
                         double *out)
{
	return guarded([&] {
		Grid g(nd, dims);
		dispatch(grp, prec, [&](auto tag) {
			using G = decltype(tag);
			*out = wilsonAction(g, load_stack<G>(g, nd, U), beta);
		});
	});
}

int oracle_staple_sum(int grp, int prec, int nd, int const *dims, void const *U, int mu, void *S)
{
	return guarded([&] {
		Grid g(nd, dims);
		dispatch(grp, prec, [&](auto tag) {
			using G = decltype(tag);
			store_field(stapleSum(g, load_stack<G>(g, nd, U), mu), S);
		});
	});
}

int oracle_wilson_deriv(int grp, int prec, int nd, int const *dims, void const *U, int mu, double beta,
                        void *F)
{
	return guarded([&] {
		Grid g(nd, dims);
		dispatch(grp, prec, [&](auto tag) {
			using G = decltype(tag);
			store_field(wilsonDeriv(g, load_stack<G>(g, nd, U), mu, beta), F);
		});
	});
}

int oracle_evolve(int grp, int prec, int nd, int const *dims, void *U, void const *P, double t)
{
	return guarded([&] {
		Grid g(nd, dims);
		dispatch(grp, prec, [&](auto tag) {
			using G = decltype(tag);
			auto u = load_stack<G>(g, nd, U);
			auto p = load_stack<G>(g, nd, P);
			for (int mu = 0; mu < nd; ++mu)
				evolve(u[mu], p[mu], t);
			store_stack(g, u, U);
		});
	});
}

int oracle_momentum_step(int grp, int prec, int nd, int const *dims, void const *U, void *P, double beta,
                         double delta)
{
	return guarded([&] {
		Grid g(nd, dims);
		dispatch(grp, prec, [&](auto tag) {
			using G = decltype(tag);
			auto u = load_stack<G>(g, nd, U);
			auto p = load_stack<G>(g, nd, P);
			std::vector<double> d = {0.0, delta, 0.0};
			runHmd(g, u, p, beta, d);
			store_stack(g, p, P);
		});
	});
}

int oracle_run_hmd(int grp, int prec, int nd, int const *dims, void *U, void *P, double beta,
                   double const *deltas, int n)
{
	return guarded([&] {
		Grid g(nd, dims);
		dispatch(grp, prec, [&](auto tag) {
			using G = decltype(tag);
			auto u = load_stack<G>(g, nd, U);
			auto p = load_stack<G>(g, nd, P);
			runHmd(g, u, p, beta, std::vector<double>(deltas, deltas + n));
			store_stack(g, u, U);
			store_stack(g, p, P);
		});
	});
}

int oracle_reunitize(int grp, int prec, int nd, int const *dims, void *U, int n_stack)
{
	return guarded([&] {
		Grid g(nd, dims);
		dispatch(grp, prec, [&](auto tag) {
			using G = decltype(tag);
			auto u = load_stack<G>(g, n_stack, U);
			reunitize(u);
			store_stack(g, u, U);
		});
	});
}

int oracle_norm2(int grp, int prec, int nd, int const *dims, void const *P, int n_stack, double *out)
{
	return guarded([&] {
		Grid g(nd, dims);
		dispatch(grp, prec, [&](auto tag) {
			using G = decltype(tag);
			*out = norm2(load_stack<G>(g, n_stack, P));
		});
	});
}

int oracle_sum_real_trace(int grp, int prec, int nd, int const *dims, void const *A, double *out)
{
	return guarded([&] {
		Grid g(nd, dims);
		dispatch(grp, prec, [&](auto tag) {
			using G = decltype(tag);
			*out = double(sum_real_trace(load_field<G>(g, A)));
		});
	});
}

// one trajectory on supplied momenta and Metropolis uniform;
// rec = {plaquette, dH, accept, H_old, H_new}
int oracle_hmc_update(int grp, int prec, int nd, int const *dims, void *U, void const *P, double beta,
                      double const *deltas, int n, double uniform, double *rec)
{
	return guarded([&] {
		Grid g(nd, dims);
		dispatch(grp, prec, [&](auto tag) {
			using G = decltype(tag);
			auto u = load_stack<G>(g, nd, U);
			auto p = load_stack<G>(g, nd, P);
			auto r = runHmcUpdate(g, u, p, beta, std::vector<double>(deltas, deltas + n), uniform);
			store_stack(g, u, U);
			rec[0] = r.plaq;
			rec[1] = r.dH;
			rec[2] = r.accept;
			rec[3] = r.H_old;
			rec[4] = r.H_new;
		});
	});
}

// a Markov chain with momenta and uniforms drawn from the counter-based
// streams: trajectory t uses counter first + t. recs = ntraj x 5.
int oracle_hmc_chain(int grp, int prec, int nd, int const *dims, void *U, double beta,
                     double const *deltas, int n, uint64_t seed, uint64_t first, int ntraj,
                     double *recs)
{
	return guarded([&] {
		Grid g(nd, dims);
		dispatch(grp, prec, [&](auto tag) {
			using G = decltype(tag);
			auto u = load_stack<G>(g, nd, U);
			GaugeField<G> p(nd, Field<G>(g.V));
			std::vector<double> d(deltas, deltas + n);
			for (int t = 0; t < ntraj; ++t)
			{
				random_momenta(g, p, seed, first + t);
				auto r = runHmcUpdate(g, u, p, beta, d, metropolis_uniform(seed, first + t));
				double *o = recs + 5 * t;
				o[0] = r.plaq;
				o[1] = r.dH;
				o[2] = r.accept;
				o[3] = r.H_old;
				o[4] = r.H_new;
			}
			store_stack(g, u, U);
		});
	});
}

int oracle_random_momenta(int grp, int prec, int nd, int const *dims, uint64_t seed, uint64_t counter,
                          void *P)
{
	return guarded([&] {
		Grid g(nd, dims);
		dispatch(grp, prec, [&](auto tag) {
			using G = decltype(tag);
			GaugeField<G> p(nd, Field<G>(g.V));
			random_momenta(g, p, seed, counter);
			store_stack(g, p, P);
		});
	});
}

int oracle_random_gauge(int grp, int prec, int nd, int const *dims, uint64_t seed, void *U)
{
	return guarded([&] {
		Grid g(nd, dims);
		dispatch(grp, prec, [&](auto tag) {
			using G = decltype(tag);
			GaugeField<G> u(nd, Field<G>(g.V));
			random_gauge(g, u, seed);
			store_stack(g, u, U);
		});
	});
}

int oracle_random_transform(int grp, int prec, int nd, int const *dims, uint64_t seed, void *h)
{
	return guarded([&] {
		Grid g(nd, dims);
		dispatch(grp, prec, [&](auto tag) {
			using G = decltype(tag);
			Field<G> f(g.V);
			random_transform(g, f, seed);
			store_field(f, h);
		});
	});
}

int oracle_gauge_transform(int grp, int prec, int nd, int const *dims, void *U, void const *h)
{
	return guarded([&] {
		Grid g(nd, dims);
		dispatch(grp, prec, [&](auto tag) {
			using G = decltype(tag);
			auto u = load_stack<G>(g, nd, U);
			gauge_transform(g, u, load_field<G>(g, h));
			store_stack(g, u, U);
		});
	});
}

double oracle_metropolis_uniform(uint64_t seed, uint64_t traj) { return metropolis_uniform(seed, traj); }

void oracle_philox(uint32_t const *ctr, uint32_t const *key, uint32_t *out)
{
	auto r = philox4x32_10(ctr[0], ctr[1], ctr[2], ctr[3], key[0], key[1]);
	for (int i = 0; i < 4; ++i)
		out[i] = r.v[i];
}

int oracle_normals(int prec, uint64_t seed, uint32_t tag, uint32_t site, uint32_t mu, uint64_t ctr, int n,
                   void *out)
{
	return guarded([&] {
		if (n > 18)
			throw std::runtime_error("at most 18 normals per call");
		if (prec == 1)
			normals<float>(seed, tag, site, mu, ctr, n, static_cast<float *>(out));
		else
			normals<double>(seed, tag, site, mu, ctr, n, static_cast<double *>(out));
	});
}

// perm[r] = even/odd index of lexicographic site r
int oracle_eo_index(int nd, int const *dims, uint64_t *perm)
{
	return guarded([&] {
		Grid g(nd, dims);
		for (size_t r = 0; r < g.V; ++r)
			perm[r] = g.eo_index(r);
	});
}

int oracle_cshift(int grp, int prec, int nd, int const *dims, void const *src, int dir, int off, void *dst)
{
	return guarded([&] {
		Grid g(nd, dims);
		dispatch(grp, prec, [&](auto tag) {
			using G = decltype(tag);
			store_field(cshift(g, load_field<G>(g, src), dir, off), dst);
		});
	});
}

// site-wise product c = a * b of two site fields (the lattice '*' operator)
int oracle_site_mul(int grp, int prec, int nd, int const *dims, void const *a, void const *b, void *c)
{
	return guarded([&] {
		Grid g(nd, dims);
		dispatch(grp, prec, [&](auto tag) {
			using G = decltype(tag);
			store_field(mul(load_field<G>(g, a), load_field<G>(g, b)), c);
		});
	});
}

// algebra packing helpers: full objects <-> packed algebra reals
int oracle_pack_algebra(int grp, int prec, size_t n, void const *full, void *packed)
{
	return guarded([&] {
		dispatch(grp, prec, [&](auto tag) {
			using G = decltype(tag);
			using T = typename traits<G>::real;
			constexpr int na = traits<G>::nalg;
			auto const *f = static_cast<G const *>(full);
			auto *p = static_cast<T *>(packed);
			for (size_t i = 0; i < n; ++i)
				pack_alg(f[i], p + na * i);
		});
	});
}
int oracle_unpack_algebra(int grp, int prec, size_t n, void const *packed, void *full)
{
	return guarded([&] {
		dispatch(grp, prec, [&](auto tag) {
			using G = decltype(tag);
			using T = typename traits<G>::real;
			constexpr int na = traits<G>::nalg;
			auto *f = static_cast<G *>(full);
			auto const *p = static_cast<T const *>(packed);
			for (size_t i = 0; i < n; ++i)
				unpack_alg(p + na * i, f[i]);
		});
	});
}

// ---- Landau (landau.h) ----
int oracle_landau_functional(int grp, int prec, int nd, int const *dims, void const *U, void const *gt,
                             double *out)
{
	return guarded([&] {
		Grid g(nd, dims);
		dispatch(grp, prec, [&](auto tag) {
			using G = decltype(tag);
			auto u = load_stack<G>(g, nd, U);
			Landau<G> l(g, u);
			l.g = load_field<G>(g, gt);
			*out = l.functional();
		});
	});
}

int oracle_landau_condition(int grp, int prec, int nd, int const *dims, void const *U, void const *gt,
                            double *out)
{
	return guarded([&] {
		Grid g(nd, dims);
		dispatch(grp, prec, [&](auto tag) {
			using G = decltype(tag);
			auto u = load_stack<G>(g, nd, U);
			Landau<G> l(g, u);
			l.g = load_field<G>(g, gt);
			*out = l.condition();
		});
	});
}

int oracle_landau_deriv(int grp, int prec, int nd, int const *dims, void const *U, void const *gt, void *F)
{
	return guarded([&] {
		Grid g(nd, dims);
		dispatch(grp, prec, [&](auto tag) {
			using G = decltype(tag);
			auto u = load_stack<G>(g, nd, U);
			Landau<G> l(g, u);
			l.g = load_field<G>(g, gt);
			store_field(l.deriv(), F);
		});
	});
}

// line_search (landau.h:77-98) from the transform gt along F
int oracle_landau_line_search(int grp, int prec, int nd, int const *dims, void const *U, void const *gt,
                              void const *F, double eps, double *out)
{
	return guarded([&] {
		Grid g(nd, dims);
		dispatch(grp, prec, [&](auto tag) {
			using G = decltype(tag);
			auto u = load_stack<G>(g, nd, U);
			Landau<G> l(g, u);
			l.g = load_field<G>(g, gt);
			int n = 0;
			*out = l.line_search(load_field<G>(g, F), eps, &n);
		});
	});
}

// reference CG + line search (landau.h:100-136), threshold as a parameter
int oracle_landau_cg(int grp, int prec, int nd, int const *dims, void const *U, void *gt, int max_iter,
                     double tol, int *iters, double *theta, int *n_evals)
{
	return guarded([&] {
		Grid g(nd, dims);
		dispatch(grp, prec, [&](auto tag) {
			using G = decltype(tag);
			auto u = load_stack<G>(g, nd, U);
			Landau<G> l(g, u);
			l.g = load_field<G>(g, gt);
			*iters = l.run(max_iter, tol, theta, n_evals);
			store_field(l.g, gt);
		});
	});
}

// ---- overrelaxation, Fourier acceleration (oracle_ext.hpp) ----
int oracle_landau_or_sweeps(int grp, int prec, int nd, int const *dims, void const *U, void *gt, double omega,
                            int nsweeps)
{
	return guarded([&] {
		Grid g(nd, dims);
		dispatch(grp, prec, [&](auto tag) {
			using G = decltype(tag);
			auto u = load_stack<G>(g, nd, U);
			auto h = load_field<G>(g, gt);
			for (int s = 0; s < nsweeps; ++s)
				or_sweep(g, u, h, omega);
			store_field(h, gt);
		});
	});
}

int oracle_landau_or(int grp, int prec, int nd, int const *dims, void const *U, void *gt, double omega,
                     double tol, int max_sweeps, int check_every, int *sweeps, double *theta)
{
	return guarded([&] {
		Grid g(nd, dims);
		dispatch(grp, prec, [&](auto tag) {
			using G = decltype(tag);
			auto u = load_stack<G>(g, nd, U);
			auto h = load_field<G>(g, gt);
			*sweeps = or_run(g, u, h, omega, tol, max_sweeps, check_every, theta);
			store_field(h, gt);
		});
	});
}

int oracle_landau_theta(int grp, int prec, int nd, int const *dims, void const *U, void const *gt,
                        double *theta_ref, double *functional)
{
	return guarded([&] {
		Grid g(nd, dims);
		dispatch(grp, prec, [&](auto tag) {
			using G = decltype(tag);
			auto u = load_stack<G>(g, nd, U);
			auto h = load_field<G>(g, gt);
			*theta_ref = theta_fast(g, u, h);
			*functional = functional_fast(g, u, h);
		});
	});
}

// divergence of the gauge-fixed field, packed algebra reals [V][nalg]
int oracle_landau_divergence(int grp, int prec, int nd, int const *dims, void const *U, void const *gt,
                             void *D)
{
	return guarded([&] {
		Grid g(nd, dims);
		dispatch(grp, prec, [&](auto tag) {
			using G = decltype(tag);
			using T = typename traits<G>::real;
			auto u = load_stack<G>(g, nd, U);
			auto h = load_field<G>(g, gt);
			auto d = divergence(g, u, h);
			auto *o = static_cast<T *>(D);
			for (size_t i = 0; i < g.V; ++i)
				pack_alg(d[i], o + traits<G>::nalg * i);
		});
	});
}

// 4D (nd-dimensional) complex FFT of ncomp interleaved complex components
// per site, sign -1 forward / +1 backward, unnormalised.
int oracle_fft(int nd, int const *dims, int ncomp, double *data, int sign)
{
	return guarded([&] {
		Grid g(nd, dims);
		fft_nd(g, ncomp, data, sign);
	});
}

// one Fourier-accelerated steepest-descent step with multiplier table
// mult[V] (per lexicographic momentum), g <- exp(-alpha * F^-1[m F[D]]) g
int oracle_landau_fa_step(int grp, int prec, int nd, int const *dims, void const *U, void *gt,
                          double const *mult, double alpha)
{
	return guarded([&] {
		Grid g(nd, dims);
		dispatch(grp, prec, [&](auto tag) {
			using G = decltype(tag);
			auto u = load_stack<G>(g, nd, U);
			auto h = load_field<G>(g, gt);
			fa_step(g, u, h, mult, alpha);
			store_field(h, gt);
		});
	});
}

int oracle_mlp_forward(int n, float const *x, float const *params, int width, float *y)
{
	return guarded([&] { mlp_forward(n, x, params, width, y); });
}

int oracle_mlp_grad(int n, float const *x, float const *target, float const *params, int width,
                    double *loss, double *grad)
{
	return guarded([&] { *loss = mlp_loss_grad(n, x, target, params, width, grad); });
}

int oracle_gauge_sweep(int grp, int prec, int nd, int const *dims, void *U, double beta, uint64_t seed,
                       uint64_t ctr, int overrelax)
{
	return guarded([&] {
		Grid g(nd, dims);
		dispatch(grp, prec, [&](auto tag) {
			using G = decltype(tag);
			auto F = load_stack<G>(g, nd, U);
			gauge_sweep(g, F, beta, seed, ctr, overrelax != 0);
			store_stack(g, F, U);
		});
	});
}

int oracle_wilson_loops(int grp, int prec, int nd, int const *dims, void const *U, int R, int T, double *out)
{
	return guarded([&] {
		Grid g(nd, dims);
		if (nd != 4 || R < 1 || T < 1)
			throw std::runtime_error("Wilson loops need a 4D grid and R, T >= 1");
		dispatch(grp, prec, [&](auto tag) {
			using G = decltype(tag);
			wilson_loops(g, load_stack<G>(g, nd, U), R, T, out);
		});
	});
}

} // extern "C"

// ---- timing of the restated reference path (CPU baseline) ------------------
// Times, on the host cores, one momentum step (P -= wilsonDeriv * delta for
// all mu), one link update (evolve for all mu) and one plaquette of the
// reference's algorithm on supplied fields; seconds per operation, best of
// `reps`.
#include <chrono>
extern "C" int oracle_bench_md(int grp, int prec, int nd, int const *dims, void const *U, void const *P, double beta,
                               double delta, int reps, double *t_force, double *t_evolve, double *t_plaq)
{
	return guarded([&] {
		Grid g(nd, dims);
		dispatch(grp, prec, [&](auto tag) {
			using G = decltype(tag);
			using clk = std::chrono::steady_clock;
			auto u = load_stack<G>(g, nd, U);
			auto p = load_stack<G>(g, nd, P);
			double bf = 1e300, be = 1e300, bp = 1e300;
			for (int r = 0; r < reps; ++r)
			{
				auto t0 = clk::now();
				runHmd(g, u, p, beta, std::vector<double>{0.0, delta, 0.0});
				auto t1 = clk::now();
				// runHmd above also ran two evolve steps of length 0; time one
				// evolve separately and subtract it twice
				for (int mu = 0; mu < nd; ++mu)
					evolve(u[mu], p[mu], delta);
				auto t2 = clk::now();
				double pl = plaquette(g, u);
				auto t3 = clk::now();
				(void)pl;
				double te = std::chrono::duration<double>(t2 - t1).count();
				double tf = std::chrono::duration<double>(t1 - t0).count() - 2 * te;
				bf = std::min(bf, tf > 0 ? tf : std::chrono::duration<double>(t1 - t0).count());
				be = std::min(be, te);
				bp = std::min(bp, std::chrono::duration<double>(t3 - t2).count());
			}
			*t_force = bf;
			*t_evolve = be;
			*t_plaq = bp;
		});
	});
}
