// mesh/mesh.hpp — header-only C++ drop-in for krox/mesh's lattice-gauge call
// surface, implemented on the C ABI of libmesh_gb300.so (mesh_gb300.h).
//
// Reference names kept (namespace mesh):
//   Grid, Coordinate .................... src/lattice/grid.h:11-58
//   Lattice<G>, LatticeStack<G> ......... src/lattice/lattice.h:23-192
//   GaugeField<G> = LatticeStack<G> ..... src/gauge/utils.h:21
//   U1<T>, SU2<T>, SU3<T>, GaugeTraits .. src/gauge/groups.h:33-212
//   plaquette, wilsonAction, stapleSum,
//   wilsonDeriv, reunitize, norm2,
//   random_gauge_field, random_algebra_field,
//   dispatchByGroup ..................... src/gauge/utils.h:35-186
//   makeDeltas, evolve, runHmd, Hmc<G> .. src/gauge/hmc.h, hmc.cpp
//   Landau<G> ........................... src/gauge/landau.h
// Semantics as in the reference: owning RAII device buffers, deep copy on
// copy, std::runtime_error on failure. Differences: random fields take a
// (seed, counter) pair of the device counter-based generator instead of a
// util::xoshiro256&; a GaugeField is one allocation holding all directions.
#pragma once

#include "../mesh_gb300.h"

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <initializer_list>
#include <memory>
#include <span>
#include <stdexcept>
#include <string>
#include <string_view>
#include <tuple>
#include <type_traits>
#include <vector>

namespace mesh {

inline void check(int rc)
{
	if (rc != MESH_OK)
		throw std::runtime_error(std::string("mesh: ") + mesh_last_error());
}

// ---- groups (host object layouts of groups.h) -------------------------------
template <class T> struct U1
{
	T re, im;
};
template <class T> struct SU2
{
	T re, im1, im2, im3;
};
template <class T> struct SU3
{
	T v[18]; // row-major 3x3 complex, (re, im) pairs
};

template <class G> struct GaugeTraits;
template <class T> struct GaugeTraits<U1<T>>
{
	using real = T;
	static constexpr int group = MESH_U1, precision = sizeof(T) == 4 ? MESH_F32 : MESH_F64;
	static constexpr std::string_view name() { return "u1"; }
	static constexpr int dim() { return 1; }
	static constexpr int Nc() { return 1; }
};
template <class T> struct GaugeTraits<SU2<T>>
{
	using real = T;
	static constexpr int group = MESH_SU2, precision = sizeof(T) == 4 ? MESH_F32 : MESH_F64;
	static constexpr std::string_view name() { return "su2"; }
	static constexpr int dim() { return 3; }
	static constexpr int Nc() { return 2; }
};
template <class T> struct GaugeTraits<SU3<T>>
{
	using real = T;
	static constexpr int group = MESH_SU3, precision = sizeof(T) == 4 ? MESH_F32 : MESH_F64;
	static constexpr std::string_view name() { return "su3"; }
	static constexpr int dim() { return 8; }
	static constexpr int Nc() { return 3; }
};

// ---- context: the implicit "current device + stream" of the reference --------
class Context
{
	mesh_ctx h_ = nullptr;

  public:
	explicit Context(int device = 0, void *stream = nullptr) { check(mesh_ctx_create(device, stream, &h_)); }
	~Context() { mesh_ctx_destroy(h_); }
	Context(Context const &) = delete;
	Context &operator=(Context const &) = delete;
	mesh_ctx get() const { return h_; }
	void synchronize() const { check(mesh_ctx_synchronize(h_)); }
	// process-wide default context on device 0 (what the reference's free
	// functions implicitly use)
	static Context &current()
	{
		static Context c(0);
		return c;
	}
};

// ---- grid ---------------------------------------------------------------------
using Coordinate = std::vector<int32_t>;

class Grid
{
	size_t size_ = 0;
	Coordinate shape_ = {0};

  public:
	Grid() = default;
	explicit Grid(Coordinate shape) : size_(1), shape_(std::move(shape))
	{
		for (auto s : shape_)
			size_ *= size_t(s);
	}
	Grid(std::initializer_list<int32_t> l) : Grid(Coordinate(l)) {}
	int ndim() const { return int(shape_.size()); }
	size_t size() const { return size_; }
	Coordinate const &shape() const { return shape_; }
	int32_t shape(size_t i) const { return shape_[i]; }
	size_t flat_index(Coordinate const &x) const
	{
		size_t r = 0;
		for (int i = 0; i < ndim(); ++i)
			r = r * size_t(shape_[size_t(i)]) + size_t(x[size_t(i)]);
		return r;
	}
	bool operator==(Grid const &) const = default;
};

// ---- fields -------------------------------------------------------------------
namespace detail {
// owned fields are destroyed with their object; borrowed ones (a chain's U and P)
// belong to the chain
struct FieldDeleter
{
	bool owned = true;
	void operator()(mesh_field_s *f) const
	{
		if (owned)
			mesh_field_destroy(f);
	}
};
struct borrow_t
{
};
using FieldPtr = std::unique_ptr<mesh_field_s, FieldDeleter>;

inline FieldPtr make_field(Context &c, int kind, int group, int prec, Grid const &g, int nstack)
{
	mesh_field f = nullptr;
	check(mesh_field_create(c.get(), kind, group, prec, g.ndim(), g.shape().data(), nstack, &f));
	return FieldPtr(f);
}
} // namespace detail

// A field of nstack x V objects of G; `algebra` fields hold momenta/forces
// (full G objects on the host, packed on the device).
template <class G> class BasicField
{
  protected:
	Grid grid_;
	int nstack_ = 1;
	int kind_ = MESH_GROUP;
	detail::FieldPtr h_;

  public:
	using value_type = G;
	using Traits = GaugeTraits<G>;

	BasicField() = default;
	BasicField(Grid const &g, int nstack, int kind, Context &c = Context::current())
	    : grid_(g), nstack_(nstack), kind_(kind),
	      h_(detail::make_field(c, kind, Traits::group, Traits::precision, g, nstack))
	{}
	// a view of a field owned elsewhere (Hmc<G>::U and P)
	BasicField(Grid const &g, int nstack, int kind, mesh_field borrowed, detail::borrow_t)
	    : grid_(g), nstack_(nstack), kind_(kind), h_(borrowed, detail::FieldDeleter{false})
	{}
	BasicField(BasicField const &o) : BasicField(o.grid_, o.nstack_, o.kind_) { check(mesh_field_copy(get(), o.get())); }
	BasicField(BasicField &&) noexcept = default;
	// assignment copies the contents (deep copy, as the reference); a borrowed
	// field keeps its buffer, so `hmc.U = readConfig<G>(...)` sets the chain's links
	BasicField &operator=(BasicField const &o)
	{
		if (this != &o)
		{
			bool same = h_ && grid_ == o.grid_ && nstack_ == o.nstack_ && kind_ == o.kind_;
			if (!same && borrowed())
				throw std::runtime_error("mesh: a chain's field can only be assigned a field of its own shape");
			if (!same)
				*this = BasicField(o.grid_, o.nstack_, o.kind_);
			check(mesh_field_copy(get(), o.get()));
		}
		return *this;
	}
	BasicField &operator=(BasicField &&o)
	{
		if (borrowed())
			return *this = static_cast<BasicField const &>(o);
		grid_ = std::move(o.grid_);
		nstack_ = o.nstack_;
		kind_ = o.kind_;
		h_ = std::move(o.h_);
		return *this;
	}
	bool borrowed() const { return h_ && !h_.get_deleter().owned; }

	mesh_field get() const { return h_.get(); }
	Grid const &grid() const { return grid_; }
	size_t size() const { return size_t(nstack_) * grid_.size(); }
	bool is_algebra() const { return kind_ == MESH_ALGEBRA; }

	void fill_zeros() { check(mesh_field_set_zero(get())); }
	void copy_from_host(std::span<const G> data)
	{
		if (data.size() != size())
			throw std::runtime_error("mesh: copy_from_host size mismatch");
		check(mesh_field_import(get(), data.data(), data.size_bytes()));
	}
	std::vector<G> copy_to_host() const
	{
		std::vector<G> r(size());
		check(mesh_field_export(get(), r.data(), r.size() * sizeof(G)));
		return r;
	}
};

// Lattice<G> (lattice.h:23-143): one object per site
template <class G> class Lattice : public BasicField<G>
{
  public:
	Lattice() = default;
	explicit Lattice(Grid const &g, bool algebra = false, Context &c = Context::current())
	    : BasicField<G>(g, 1, algebra ? MESH_ALGEBRA : MESH_GROUP, c)
	{}
	static Lattice zeros(Grid const &g)
	{
		Lattice a(g);
		a.fill_zeros();
		return a;
	}
	static Lattice identity(Grid const &g)
	{
		Lattice a(g);
		check(mesh_field_set_unit(a.get()));
		return a;
	}
};

// LatticeStack<G> / GaugeField<G> (lattice.h:159-192, utils.h:21)
template <class G> class LatticeStack : public BasicField<G>
{
  public:
	LatticeStack() = default;
	explicit LatticeStack(Grid const &g, bool algebra = false, Context &c = Context::current())
	    : BasicField<G>(g, g.ndim(), algebra ? MESH_ALGEBRA : MESH_GROUP, c)
	{}
	LatticeStack(Grid const &g, bool algebra, mesh_field borrowed, detail::borrow_t b)
	    : BasicField<G>(g, g.ndim(), algebra ? MESH_ALGEBRA : MESH_GROUP, borrowed, b)
	{}
	size_t ndirs() const { return size_t(this->nstack_); }
	void set_unit() { check(mesh_field_set_unit(this->get())); }
};
template <class G> using GaugeField = LatticeStack<G>;
template <class G> GaugeField<G> Momenta(Grid const &g) { return GaugeField<G>(g, true); }

// ---- lattice operations (lattice.h:256-389, utils.h:28-33) -------------------
template <class G> Lattice<G> cshift(Lattice<G> const &a, int dir, int offset)
{
	Lattice<G> r(a.grid());
	check(mesh_site_cshift(r.get(), a.get(), dir, offset));
	return r;
}
template <class G> Lattice<G> operator*(Lattice<G> const &a, Lattice<G> const &b)
{
	Lattice<G> r(a.grid());
	check(mesh_site_mul(r.get(), a.get(), b.get()));
	return r;
}
template <class G> Lattice<G> adj(Lattice<G> const &a)
{
	Lattice<G> r(a.grid());
	check(mesh_site_adj(r.get(), a.get()));
	return r;
}
// exp of an algebra field, and the algebra projection of a group-type field
// (MESH_DEFINE_LATTICE_UNARY(exp / project_on_algebra), utils.h:32-33)
template <class G> Lattice<G> exp(Lattice<G> const &a)
{
	Lattice<G> r(a.grid());
	check(mesh_site_exp(r.get(), a.get()));
	return r;
}
template <class G> Lattice<G> project_on_algebra(Lattice<G> const &a)
{
	Lattice<G> r(a.grid(), true);
	check(mesh_site_project(r.get(), a.get()));
	return r;
}
template <class G> double sum_real_trace(Lattice<G> const &a)
{
	double s = 0;
	check(mesh_site_sum_real_trace(a.get(), &s));
	return s;
}
template <class G> double norm2(BasicField<G> const &a)
{
	double s = 0;
	check(mesh_field_norm2(a.get(), &s));
	return s;
}

// linear operations on Lattice<G> and GaugeField<G> (MESH_DEFINE_LATTICE_BINARY
// +, -, lattice.h:289-327,337-338; operator*(Lattice, double), lattice.h:348-356;
// add_mul, lattice.h:358-364): a new field of the operands' shape, or in place
template <class L>
concept MeshField = std::is_base_of_v<BasicField<typename L::value_type>, L>;
template <MeshField L> L axpby(double a, L const &x, double b, L const *y)
{
	L r(x.grid(), x.is_algebra());
	check(mesh_field_axpby(r.get(), a, x.get(), b, y ? y->get() : nullptr));
	return r;
}
template <MeshField L> L operator+(L const &x, L const &y) { return axpby(1.0, x, 1.0, &y); }
template <MeshField L> L operator-(L const &x, L const &y) { return axpby(1.0, x, -1.0, &y); }
template <MeshField L> L operator*(L const &x, double s) { return axpby<L>(s, x, 0.0, nullptr); }
template <MeshField L> L operator*(double s, L const &x) { return axpby<L>(s, x, 0.0, nullptr); }
template <MeshField L> L &operator+=(L &x, L const &y)
{
	check(mesh_field_axpby(x.get(), 1.0, x.get(), 1.0, y.get()));
	return x;
}
template <MeshField L> L &operator-=(L &x, L const &y)
{
	check(mesh_field_axpby(x.get(), 1.0, x.get(), -1.0, y.get()));
	return x;
}
template <MeshField L> L &operator*=(L &x, double s)
{
	check(mesh_field_axpby(x.get(), s, x.get(), 0.0, nullptr));
	return x;
}
// lhs += m * rhs for a real m
template <MeshField L> void add_mul(L &lhs, double m, L const &rhs)
{
	check(mesh_field_axpby(lhs.get(), 1.0, lhs.get(), m, rhs.get()));
}

// ---- gauge utilities (utils.h) -------------------------------------------------
template <class G> double plaquette(GaugeField<G> const &U)
{
	double p = 0;
	check(mesh_plaquette(U.get(), &p));
	return p;
}
template <class G> double wilsonAction(GaugeField<G> const &U, double beta)
{
	double s = 0;
	check(mesh_wilson_action(U.get(), beta, &s));
	return s;
}
// WilsonAction<G>::sweep / GaugeAction<G>::thermalize and overrelax
// (src/old/wilson.cpp:15-60, src/old/mesh/gauge_action.h:42-73): one
// heat-bath or overrelaxation sweep over every link
template <class G> void thermalize(GaugeField<G> &U, double beta, uint64_t seed, uint64_t sweep)
{
	check(mesh_heatbath_sweep(U.get(), beta, seed, sweep));
}
template <class G> void overrelax(GaugeField<G> &U) { check(mesh_overrelax_sweep(U.get())); }
// wilson(const Mesh<G>&, int maxN) of src/old/mesh/wilson.cpp:40-75: the
// rectangular loops (n, t, W) for n = 1..maxN, t = 1..maxT (default: L3)
template <class G>
std::vector<std::tuple<int, int, double>> wilson(GaugeField<G> const &U, int maxN, int maxT = -1)
{
	if (maxT < 0)
		maxT = U.grid().shape(3);
	std::vector<double> w(size_t(maxN) * size_t(maxT));
	check(mesh_wilson_loops(U.get(), maxN, maxT, w.data()));
	std::vector<std::tuple<int, int, double>> r;
	for (int n = 1; n <= maxN; ++n)
		for (int t = 1; t <= maxT; ++t)
			r.emplace_back(n, t, w[size_t(n - 1) * maxT + (t - 1)]);
	return r;
}
template <class G> Lattice<G> stapleSum(GaugeField<G> const &U, int mu)
{
	Lattice<G> S(U.grid());
	check(mesh_staple_sum(S.get(), U.get(), mu));
	return S;
}
template <class G> Lattice<G> wilsonDeriv(GaugeField<G> const &U, int mu, double beta)
{
	Lattice<G> F(U.grid(), true);
	check(mesh_wilson_deriv(F.get(), U.get(), mu, beta));
	return F;
}
template <class G> void reunitize(GaugeField<G> &U) { check(mesh_reunitize(U.get())); }
template <class G> void reunitize(Lattice<G> &g) { check(mesh_reunitize(g.get())); }
template <class G> void random_gauge_field(BasicField<G> &U, uint64_t seed, uint64_t counter = 0)
{
	check(mesh_field_random(U.get(), seed, counter));
}
template <class G> void random_algebra_field(GaugeField<G> &P, uint64_t seed, uint64_t counter = 0)
{
	check(mesh_field_random(P.get(), seed, counter));
}

// ---- HMC (hmc.h, hmc.cpp) --------------------------------------------------------
inline std::vector<double> makeDeltas(std::string_view scheme, double epsilon, int substeps)
{
	int n = 0;
	std::string s(scheme);
	std::vector<double> d(size_t(8 * substeps + 16));
	check(mesh_make_deltas(s.c_str(), epsilon, substeps, d.data(), int(d.size()), &n));
	d.resize(size_t(n));
	return d;
}
template <class G> void evolve(GaugeField<G> &U, GaugeField<G> const &P, double t)
{
	check(mesh_evolve(U.get(), P.get(), t));
}
template <class G> void runHmd(GaugeField<G> &U, GaugeField<G> &P, double beta, std::vector<double> const &deltas)
{
	check(mesh_run_hmd(U.get(), P.get(), beta, deltas.data(), int(deltas.size())));
}

template <class G> class Hmc
{
	struct Del
	{
		void operator()(mesh_hmc_s *h) const { mesh_hmc_destroy(h); }
	};
	std::unique_ptr<mesh_hmc_s, Del> h_;
	static mesh_hmc create(Grid const &grid, uint64_t seed, Context &c)
	{
		mesh_hmc h = nullptr;
		check(mesh_hmc_create(c.get(), GaugeTraits<G>::group, GaugeTraits<G>::precision, grid.ndim(),
		                      grid.shape().data(), seed, &h));
		return h;
	}
	static mesh_field state(mesh_hmc h, int which)
	{
		mesh_field f = nullptr;
		check(mesh_hmc_field(h, which, &f));
		return f;
	}
	uint64_t momentum_draws_ = 0;

  public:
	Grid const &g;
	uint64_t seed;
	// the chain's gauge field and momenta (hmc.h:71-72): views of its device
	// fields; assigning to U (e.g. U = readConfig<G>(path)) sets the chain's links
	GaugeField<G> U, P;
	std::vector<double> plaq_history, deltaH_history, accept_history, time_history;

	explicit Hmc(Grid const &grid, uint64_t seed_ = 0, Context &c = Context::current())
	    : h_(create(grid, seed_, c)), g(grid), seed(seed_), U(grid, false, state(h_.get(), 0), detail::borrow_t{}),
	      P(grid, true, state(h_.get(), 1), detail::borrow_t{})
	{}
	mesh_hmc get() const { return h_.get(); }
	// the gauge field and momenta in the reference's host layout
	std::vector<G> U_to_host() const
	{
		mesh_field f = nullptr;
		check(mesh_hmc_field(get(), 0, &f));
		std::vector<G> r(size_t(g.ndim()) * g.size());
		check(mesh_field_export(f, r.data(), r.size() * sizeof(G)));
		return r;
	}
	void U_from_host(std::span<const G> data)
	{
		mesh_field f = nullptr;
		check(mesh_hmc_field(get(), 0, &f));
		check(mesh_field_import(f, data.data(), data.size_bytes()));
	}
	void reset_observables()
	{
		plaq_history.clear();
		deltaH_history.clear();
		accept_history.clear();
		time_history.clear();
	}
	void randomizeGaugeField() { check(mesh_hmc_randomize(get())); }
	// new Gaussian momenta in P (hmc.cpp:65-74); runHmcUpdate draws its own, as
	// the reference's does, from the trajectory's stream
	void randomizeMomenta() { random_algebra_field(P, seed, (uint64_t(1) << 40) + momentum_draws_++); }
	void coldStart() { check(mesh_hmc_cold_start(get())); }
	// checkpoint / resume (links, trajectory counter, seed)
	void save(std::string const &path) const { check(mesh_hmc_save(get(), path.c_str())); }
	void load(std::string const &path) { check(mesh_hmc_load(get(), path.c_str())); }
	// generate momenta -> run a trajectory -> accept/reject -> measure
	// (hmc.cpp:76-107; the action of U is recomputed every trajectory, as there,
	// since U may have been written through the view)
	void runHmcUpdate(double beta, std::vector<double> const &deltas)
	{
		auto t0 = std::chrono::steady_clock::now();
		state(get(), 0); // marks the chain's cached action of U stale
		mesh_hmc_record r{};
		check(mesh_hmc_update(get(), beta, deltas.data(), int(deltas.size()), &r));
		plaq_history.push_back(r.plaquette);
		deltaH_history.push_back(r.dH);
		accept_history.push_back(r.accept);
		time_history.push_back(std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count());
	}
	void print_summary() const
	{
		auto mean = [](std::vector<double> const &v, auto f) {
			double s = 0;
			for (double x : v)
				s += f(x);
			return v.empty() ? 0.0 : s / double(v.size());
		};
		auto id = [](double x) { return x; };
		double m = mean(plaq_history, id);
		double var = 0;
		for (double x : plaq_history)
			var += (x - m) * (x - m);
		var = plaq_history.size() > 1 ? var / double(plaq_history.size() - 1) : 0.0;
		std::printf("========== HMC summary ==========\n");
		if (!time_history.empty())
			std::printf("time per step = %.3f s (min = %.3f, max = %.3f)\n", mean(time_history, id),
			            *std::min_element(time_history.begin(), time_history.end()),
			            *std::max_element(time_history.begin(), time_history.end()));
		std::printf("plaquette = %.4f +- %.4f\n", m, std::sqrt(var / double(plaq_history.size())));
		std::printf("acceptance = %.2f\n", mean(accept_history, id));
		std::printf("<exp(-dH)> = %.4f\n", mean(deltaH_history, [](double x) { return std::exp(-x); }));
	}
};

// ---- configuration files (writeToFile/readFromFile, lattice.h:205-252;
// readConfig, utils.h:188-219) -----------------------------------------------------
template <class G> void writeToFile(std::string const &path, BasicField<G> const &a)
{
	check(mesh_field_save(a.get(), path.c_str()));
}
template <class G> void readFromFile(std::string const &path, BasicField<G> &a)
{
	check(mesh_field_load(a.get(), path.c_str()));
}
// a gauge field with the file's grid; throws on a group mismatch, and on a
// grid mismatch when expected_grid is given
template <class G> GaugeField<G> readConfig(std::string const &path, Grid const *expected_grid = nullptr)
{
	int kind = 0, group = 0, prec = 0, nd = 0, nstack = 0;
	int32_t dims[4] = {0, 0, 0, 0};
	check(mesh_config_info(path.c_str(), &kind, &group, &prec, &nd, dims, &nstack, nullptr, nullptr));
	if (group != GaugeTraits<G>::group || prec != GaugeTraits<G>::precision || kind != MESH_GROUP)
		throw std::runtime_error("group mismatch on load");
	Grid grid(std::vector<int32_t>(dims, dims + nd));
	if (expected_grid && !(*expected_grid == grid))
		throw std::runtime_error("grid mismatch on load");
	GaugeField<G> U(grid);
	readFromFile(path, U);
	return U;
}

// ---- Landau (landau.h) -------------------------------------------------------------
template <class G> struct Landau
{
	GaugeField<G> const &U;
	Lattice<G> g;
	bool verbose = false;

	explicit Landau(GaugeField<G> const &U_) : U(U_), g(Lattice<G>::identity(U_.grid())) {}
	void reset() { check(mesh_field_set_unit(g.get())); }
	// the functional at the transform h (landau.h:23-32), or at g
	double operator()(Lattice<G> const &h) const
	{
		double s = 0;
		check(mesh_landau_functional(U.get(), h.get(), &s));
		return s;
	}
	double operator()() const { return (*this)(g); }
	// the step along the algebra field F from g that run() takes (landau.h:77-98)
	double line_search(Lattice<G> const &F, double eps) const
	{
		double step = 0;
		check(mesh_landau_line_search(U.get(), g.get(), F.get(), eps, &step));
		return step;
	}
	double condition() const
	{
		double t = 0;
		check(mesh_landau_theta(U.get(), g.get(), &t));
		return t;
	}
	Lattice<G> deriv() const
	{
		Lattice<G> F(U.grid(), true);
		check(mesh_landau_deriv(F.get(), U.get(), g.get()));
		return F;
	}
	// the reference's CG (threshold 1e-10 as in landau.h:113 unless given)
	int run(int max_iter, double tol = 1e-10)
	{
		int it = 0;
		double th = 0;
		int rc = mesh_landau_cg(U.get(), g.get(), max_iter, tol, &it, &th);
		if (rc != MESH_OK && rc != MESH_ERR_NOCONV)
			check(rc);
		return it;
	}
	// checkerboard overrelaxation; throws if it does not converge
	// (as the legacy relaxation, src/old/gauge_fixing.cpp:78)
	int overrelax(double omega, double tol, int max_sweeps, int check_every = 10)
	{
		int s = 0;
		double th = 0;
		check(mesh_landau_or(U.get(), g.get(), omega, tol, max_sweeps, check_every, &s, &th));
		return s;
	}
};

// ---- Fourier-accelerated Landau gauge fixing (no reference counterpart) ------------
// Steepest descent with a spectral multiplier (plain alpha p2max/p^2, or the learned
// MLP) on FP64 links; a step that fails the acceptance test (theta by default, or the
// gauge functional) is undone and overrelaxation sweeps run instead. g is the gauge
// transform, e.g. Landau<G>::g.
template <class G> class LandauFA
{
  public:
	static_assert(GaugeTraits<G>::precision == MESH_F64, "Fourier-accelerated gauge fixing runs on FP64 links");
	struct Result
	{
		int iterations = 0, fallbacks = 0;
		double theta = 0;
	};

	explicit LandauFA(GaugeField<G> const &U) { check(mesh_landau_fa_create(U.get(), &h_)); }
	~LandauFA() { mesh_landau_fa_destroy(h_); }
	LandauFA(LandauFA const &) = delete;
	LandauFA &operator=(LandauFA const &) = delete;

	void set_plain(double alpha = 0.08) { check(mesh_landau_fa_set_plain(h_, alpha)); }
	// network parameters in the library's layout: width^2 + 6 width + 1 floats
	void set_mlp(std::vector<float> const &params, int width, double beta, bool bf16 = true)
	{
		if (params.size() != size_t(width) * width + 6 * size_t(width) + 1)
			throw std::runtime_error("MLP parameter count does not match the width");
		check(mesh_landau_fa_set_mlp(h_, params.data(), width, beta, bf16 ? 1 : 0));
	}
	void accept_on_functional(bool on) { check(mesh_landau_fa_set_accept(h_, on ? 1 : 0)); }
	double theta(Lattice<G> const &g) const
	{
		double t = 0;
		check(mesh_landau_fa_theta(h_, g.get(), &t));
		return t;
	}
	// steps until theta < tol; throws if max_iter steps do not reach it
	Result run(Lattice<G> &g, double tol = 1e-12, int max_iter = 20000, double omega = 1.7, int or_sweeps = 10)
	{
		Result r;
		check(mesh_landau_fa_run(h_, g.get(), tol, max_iter, omega, or_sweeps, &r.iterations, &r.fallbacks,
		                         &r.theta));
		return r;
	}

  private:
	mesh_landau_fa h_ = nullptr;
};

// the committed network (mesh_gb300/landau_mlp_su3.f32): raw little-endian FP32 parameters
inline std::vector<float> readMlpParams(std::string const &path)
{
	std::FILE *f = std::fopen(path.c_str(), "rb");
	if (!f)
		throw std::runtime_error("cannot open " + path);
	std::vector<float> p;
	float buf[1024];
	size_t n;
	while ((n = std::fread(buf, sizeof(float), 1024, f)) > 0)
		p.insert(p.end(), buf, buf + n);
	std::fclose(f);
	return p;
}

// ---- runtime dispatch (utils.h:156-186) ------------------------------------------
template <typename F> void dispatchByGroup(F f, std::string const &group, int precision)
{
	if (precision == 1)
	{
		if (group == "u1")
			f.template operator()<U1<float>>();
		else if (group == "su2")
			f.template operator()<SU2<float>>();
		else if (group == "su3")
			f.template operator()<SU3<float>>();
		else
			throw std::runtime_error("unknown gauge group '" + group + "'");
	}
	else if (precision == 2)
	{
		if (group == "u1")
			f.template operator()<U1<double>>();
		else if (group == "su2")
			f.template operator()<SU2<double>>();
		else if (group == "su3")
			f.template operator()<SU3<double>>();
		else
			throw std::runtime_error("unknown gauge group '" + group + "'");
	}
	else // the reference's message, verbatim (utils.h:185)
		throw std::runtime_error("invlid precision level '" + std::to_string(precision) + "'");
}

} // namespace mesh
