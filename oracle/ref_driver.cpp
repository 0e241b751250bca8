// TEST INFRASTRUCTURE — NOT PART OF THE PRODUCT.
//
// Drives the reference's own templates, compiled in place from the reference
// tree (src/lattice/grid.h, lattice.h, tensor.h; src/gauge/groups.h, utils.h,
// hmc.h, hmc.cpp, landau.h) against the project-written stand-ins in
// oracle/ref_shim.
// Built by `make -C oracle ref` into oracle/_ref/libref.so (x86 or Arm, never
// committed); only the tests that pin the restated oracle load it.
#include "gauge/hmc.h"
#include "gauge/landau.h"

#include <exception>
#include <string>

using namespace mesh;

// Landau<G>::reset() is the one line of src/gauge/landau.h (:14, g.fill(G(1)))
// that does not compile as shipped: Lattice::fill is commented out in
// src/lattice/lattice.h:59. It is replaced here, for the six instantiations
// used, by an explicit specialisation that sets g to the unit element through
// copy_from_host; the primary definition is then never instantiated and every
// other member of Landau<G> (landau.h:23-136) is the reference's own.
namespace {
template <class T> util::complex<T> unit_of(util::complex<T> *) { return {T(1), T(0)}; }
template <class T> util::quaternion<T> unit_of(util::quaternion<T> *) { return {T(1), T(0), T(0), T(0)}; }
template <class T, int N> util::Matrix<T, N> unit_of(util::Matrix<T, N> *) { return util::Matrix<T, N>::identity(); }
template <class G> void set_unit(Lattice<G> &g)
{
	std::vector<G> h(g.grid().size(), unit_of(static_cast<G *>(nullptr)));
	g.copy_from_host(std::span<const G>(h.data(), h.size()));
}
} // namespace
namespace mesh {
template <> void Landau<U1<float>>::reset() { set_unit(g); }
template <> void Landau<U1<double>>::reset() { set_unit(g); }
template <> void Landau<SU2<float>>::reset() { set_unit(g); }
template <> void Landau<SU2<double>>::reset() { set_unit(g); }
template <> void Landau<SU3<float>>::reset() { set_unit(g); }
template <> void Landau<SU3<double>>::reset() { set_unit(g); }
} // namespace mesh

namespace {
thread_local std::string g_err;

Grid make_grid(int nd, int const *dims) { return Grid(Coordinate(dims, dims + nd)); }

template <class G> void load(GaugeField<G> &U, int nd, size_t V, void const *p)
{
	auto const *src = static_cast<G const *>(p);
	for (int mu = 0; mu < nd; ++mu)
		U[mu].copy_from_host(std::span<const G>(src + size_t(mu) * V, V));
}
template <class G> void store(GaugeField<G> const &U, int nd, size_t V, void *p)
{
	auto *dst = static_cast<G *>(p);
	for (int mu = 0; mu < nd; ++mu)
	{
		auto h = U[mu].copy_to_host();
		std::memcpy((void *)(dst + size_t(mu) * V), h.data(), V * sizeof(G));
	}
}
template <class G> void store1(Lattice<G> const &L, void *p)
{
	auto h = L.copy_to_host();
	std::memcpy(p, (void const *)h.data(), h.size() * sizeof(G));
}

template <class G> void load1(Lattice<G> &L, void const *p)
{
	L.copy_from_host(std::span<const G>(static_cast<G const *>(p), L.grid().size()));
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

template <class F> void dispatch(int group, int prec, F f)
{
	if (prec == 1)
	{
		if (group == 1)
			f.template operator()<U1<float>>();
		else if (group == 2)
			f.template operator()<SU2<float>>();
		else if (group == 3)
			f.template operator()<SU3<float>>();
		else
			throw std::runtime_error("unknown gauge group");
	}
	else if (prec == 2)
	{
		if (group == 1)
			f.template operator()<U1<double>>();
		else if (group == 2)
			f.template operator()<SU2<double>>();
		else if (group == 3)
			f.template operator()<SU3<double>>();
		else
			throw std::runtime_error("unknown gauge group");
	}
	else
		throw std::runtime_error("invalid precision");
}
} // namespace

extern "C" {
char const *ref_last_error() { return g_err.c_str(); }

int ref_make_deltas(char const *scheme, double eps, int substeps, double *out, int cap)
{
	int n = -1;
	int rc = guarded([&] {
		auto d = makeDeltas(scheme, eps, substeps);
		if ((int)d.size() > cap)
			throw std::runtime_error("buffer too small");
		std::copy(d.begin(), d.end(), out);
		n = (int)d.size();
	});
	return rc ? -1 : n;
}

int ref_plaquette(int grp, int prec, int nd, int const *dims, void const *Up, double *out)
{
	return guarded([&] {
		auto g = make_grid(nd, dims);
		dispatch(grp, prec, [&]<class G>() {
			GaugeField<G> U(g);
			load(U, nd, g.size(), Up);
			*out = plaquette(U);
		});
	});
}

int ref_wilson_action(int grp, int prec, int nd, int const *dims, void const *Up, double beta, double *out)
{
	return guarded([&] {
		auto g = make_grid(nd, dims);
		dispatch(grp, prec, [&]<class G>() {
			GaugeField<G> U(g);
			load(U, nd, g.size(), Up);
			*out = wilsonAction(U, beta);
		});
	});
}

int ref_staple_sum(int grp, int prec, int nd, int const *dims, void const *Up, int mu, void *S)
{
	return guarded([&] {
		auto g = make_grid(nd, dims);
		dispatch(grp, prec, [&]<class G>() {
			GaugeField<G> U(g);
			load(U, nd, g.size(), Up);
			store1(stapleSum(U, mu), S);
		});
	});
}

int ref_wilson_deriv(int grp, int prec, int nd, int const *dims, void const *Up, int mu, double beta, void *F)
{
	return guarded([&] {
		auto g = make_grid(nd, dims);
		dispatch(grp, prec, [&]<class G>() {
			GaugeField<G> U(g);
			load(U, nd, g.size(), Up);
			store1(wilsonDeriv(U, mu, beta), F);
		});
	});
}

int ref_evolve(int grp, int prec, int nd, int const *dims, void *Up, void const *Pp, double t)
{
	return guarded([&] {
		auto g = make_grid(nd, dims);
		dispatch(grp, prec, [&]<class G>() {
			GaugeField<G> U(g), P(g);
			load(U, nd, g.size(), Up);
			load(P, nd, g.size(), Pp);
			for (int mu = 0; mu < nd; ++mu)
				evolve(U[mu], P[mu], t);
			store(U, nd, g.size(), Up);
		});
	});
}

int ref_run_hmd(int grp, int prec, int nd, int const *dims, void *Up, void *Pp, double beta,
                double const *deltas, int n)
{
	return guarded([&] {
		auto g = make_grid(nd, dims);
		dispatch(grp, prec, [&]<class G>() {
			GaugeField<G> U(g), P(g);
			load(U, nd, g.size(), Up);
			load(P, nd, g.size(), Pp);
			runHmd(U, P, beta, std::vector<double>(deltas, deltas + n));
			store(U, nd, g.size(), Up);
			store(P, nd, g.size(), Pp);
		});
	});
}

int ref_reunitize(int grp, int prec, int nd, int const *dims, void *Up)
{
	return guarded([&] {
		auto g = make_grid(nd, dims);
		dispatch(grp, prec, [&]<class G>() {
			GaugeField<G> U(g);
			load(U, nd, g.size(), Up);
			reunitize(U);
			store(U, nd, g.size(), Up);
		});
	});
}

int ref_norm2(int grp, int prec, int nd, int const *dims, void const *Pp, double *out)
{
	return guarded([&] {
		auto g = make_grid(nd, dims);
		dispatch(grp, prec, [&]<class G>() {
			GaugeField<G> P(g);
			load(P, nd, g.size(), Pp);
			*out = norm2(P);
		});
	});
}

int ref_cshift(int grp, int prec, int nd, int const *dims, void const *src, int dir, int off, void *dst)
{
	return guarded([&] {
		auto g = make_grid(nd, dims);
		dispatch(grp, prec, [&]<class G>() {
			Lattice<G> a(g);
			a.copy_from_host(std::span<const G>(static_cast<G const *>(src), g.size()));
			store1(cshift(a, dir, off), dst);
		});
	});
}

// random_algebra_field (utils.h:72-78) fed with supplied normals
int ref_random_algebra_field(int grp, int prec, int nd, int const *dims, double const *normals, size_t nn,
                             void *Pp)
{
	return guarded([&] {
		auto &pb = util::playback_state();
		pb.normals.assign(normals, normals + nn);
		pb.in = 0;
		auto g = make_grid(nd, dims);
		dispatch(grp, prec, [&]<class G>() {
			GaugeField<G> P(g);
			util::xoshiro256 rng;
			random_algebra_field(P, rng);
			store(P, nd, g.size(), Pp);
		});
	});
}

// Hmc<G>::runHmcUpdate (hmc.cpp:73-107) with the momenta normals and the
// Metropolis uniform played back; rec = {plaquette, dH, accept}
int ref_hmc_update(int grp, int prec, int nd, int const *dims, void *Up, double const *normals, size_t nn,
                   double uniform, double beta, double const *deltas, int n, double *rec)
{
	return guarded([&] {
		auto &pb = util::playback_state();
		pb.normals.assign(normals, normals + nn);
		pb.in = 0;
		pb.uniforms.assign(1, uniform);
		pb.iu = 0;
		auto g = make_grid(nd, dims);
		dispatch(grp, prec, [&]<class G>() {
			Hmc<G> hmc(g);
			load(hmc.U, nd, g.size(), Up);
			hmc.runHmcUpdate(beta, std::vector<double>(deltas, deltas + n));
			store(hmc.U, nd, g.size(), Up);
			rec[0] = hmc.plaq_history.back();
			rec[1] = hmc.deltaH_history.back();
			rec[2] = hmc.accept_history.back();
		});
	});
}

// ---- Landau<G> (src/gauge/landau.h) on supplied links U and transform g ----
// operator() (landau.h:23-34), condition() (:37-49), deriv() (:52-65)
int ref_landau_eval(int grp, int prec, int nd, int const *dims, void const *Up, void const *gp, double *functional,
                    double *condition, void *deriv)
{
	return guarded([&] {
		auto gr = make_grid(nd, dims);
		dispatch(grp, prec, [&]<class G>() {
			GaugeField<G> U(gr);
			load(U, nd, gr.size(), Up);
			Landau<G> L(U);
			load1(L.g, gp);
			*functional = L();
			*condition = L.condition();
			store1(L.deriv(), deriv);
		});
	});
}

// line_search(F, eps) (landau.h:77-98) from the transform g
int ref_landau_line_search(int grp, int prec, int nd, int const *dims, void const *Up, void const *gp,
                           void const *Fp, double eps, double *out)
{
	return guarded([&] {
		auto gr = make_grid(nd, dims);
		dispatch(grp, prec, [&]<class G>() {
			GaugeField<G> U(gr);
			load(U, nd, gr.size(), Up);
			Landau<G> L(U);
			load1(L.g, gp);
			Lattice<G> F(gr);
			load1(F, Fp);
			*out = L.line_search(F, eps);
		});
	});
}

// run(max_iter) (landau.h:100-136) from the transform g (g updated in place)
int ref_landau_run(int grp, int prec, int nd, int const *dims, void const *Up, void *gp, int max_iter)
{
	return guarded([&] {
		auto gr = make_grid(nd, dims);
		dispatch(grp, prec, [&]<class G>() {
			GaugeField<G> U(gr);
			load(U, nd, gr.size(), Up);
			Landau<G> L(U);
			load1(L.g, gp);
			L.run(max_iter);
			store1(L.g, gp);
		});
	});
}
}

