// Coupling scan of pure gauge theory, the counterpart of krox/mesh's
// src/apps/sweep_beta.cpp (same options, defaults and output lines). The
// reference sweeps one chain through the couplings one after another; here
// every coupling is one replica of a batch (mesh_batch_*, C ABI), all
// replicas advance together in one persistent launch per integrator step,
// so the whole scan costs about as much GPU time as one coupling. Each
// replica starts from Haar-random links (the reference's randomizeGaugeField
// of its single chain) with its own seed; the plaquette reported is the mean
// over the last 90% of its `count` trajectories (sweep_beta.cpp:75-78).
//
//   g++ -std=c++20 -O2 -I include mesh_gb300/apps/sweep_beta.cpp
//       -L mesh_gb300 -lmesh_gb300 -Wl,-rpath,$PWD/mesh_gb300 -o sweep_beta
//   ./sweep_beta --group su3 --geom 4 4 4 4 --beta-min 0 --beta-max 8
//                --beta-count 30 --count 50 --scheme 4mn --epsilon 2.0
//                --substeps 8 --precision 2 --seed 1
//                [--digits N]   decimals of the printed values (default 3,
//                               the reference's format); with N > 3 the
//                               standard error of the plaquette mean (bins of
//                               5 trajectories) is printed too
// The 4D batch needs four even extents below 256.
#include "mesh/mesh.hpp"

#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <random>
#include <string>
#include <vector>

using namespace mesh;

int main(int argc, char **argv)
{
	std::string group = "su3", scheme = "4mn";
	std::vector<int32_t> geom = {4, 4, 4, 4};
	double beta_min = 0, beta_max = 8, epsilon = 2.0;
	int beta_count = 30, substeps = 8, count = 50, precision = 2, digits = 3;
	uint64_t seed = 0;
	bool have_seed = false;
	for (int i = 1; i < argc; ++i)
	{
		std::string a = argv[i];
		auto next = [&]() -> char const * {
			if (i + 1 >= argc)
			{
				std::fprintf(stderr, "missing value for %s\n", a.c_str());
				std::exit(2);
			}
			return argv[++i];
		};
		if (a == "--group")
			group = next();
		else if (a == "--geom")
		{
			geom.clear();
			while (i + 1 < argc && std::strncmp(argv[i + 1], "--", 2) != 0)
				geom.push_back(int32_t(std::atoi(argv[++i])));
		}
		else if (a == "--beta-min")
			beta_min = std::atof(next());
		else if (a == "--beta-max")
			beta_max = std::atof(next());
		else if (a == "--beta-count")
			beta_count = std::atoi(next());
		else if (a == "--seed")
		{
			seed = std::strtoull(next(), nullptr, 10);
			have_seed = true;
		}
		else if (a == "--count")
			count = std::atoi(next());
		else if (a == "--scheme")
			scheme = next();
		else if (a == "--epsilon")
			epsilon = std::atof(next());
		else if (a == "--substeps")
			substeps = std::atoi(next());
		else if (a == "--precision")
			precision = std::atoi(next());
		else if (a == "--digits")
			digits = std::atoi(next());
		else
		{
			std::fprintf(stderr, "unknown option %s\n", a.c_str());
			return 2;
		}
	}
	if (!have_seed)
		seed = uint64_t(std::random_device()());
	if (geom.size() != 4 || beta_count < 1 || count < 1)
	{
		std::fprintf(stderr, "sweep_beta: --geom needs 4 extents, --beta-count and --count must be >= 1\n");
		return 2;
	}
	try
	{
		int g = group == "u1" ? MESH_U1 : group == "su2" ? MESH_SU2 : group == "su3" ? MESH_SU3 : 0;
		if (g == 0)
			throw std::runtime_error("unknown gauge group '" + group + "'");
		auto deltas = makeDeltas(scheme, epsilon, substeps);
		std::vector<double> betas(static_cast<size_t>(beta_count));
		std::vector<int32_t> dims;
		std::vector<uint64_t> seeds;
		for (int iter = 0; iter < beta_count; ++iter)
		{
			betas[size_t(iter)] =
			    beta_count > 1 ? beta_min + (beta_max - beta_min) / (beta_count - 1) * iter : beta_min;
			dims.insert(dims.end(), geom.begin(), geom.end());
			seeds.push_back(seed * 1000003u + uint64_t(iter));
		}
		Context &ctx = Context::current();
		mesh_batch b = nullptr;
		check(mesh_batch_create(ctx.get(), g, precision, beta_count, dims.data(), seeds.data(), &b));
		struct Del
		{
			mesh_batch b;
			~Del() { mesh_batch_destroy(b); }
		} del{b};
		check(mesh_batch_randomize(b));
		check(mesh_batch_run(b, betas.data(), deltas.data(), int(deltas.size()), count, 1));
		std::vector<double> plaq(static_cast<size_t>(count)), acc(static_cast<size_t>(count));
		for (int r = 0; r < beta_count; ++r)
		{
			check(mesh_batch_history(b, r, 0, count, plaq.data(), nullptr, acc.data()));
			size_t first = size_t(count) / 10, m = size_t(count) - first;
			double sp = 0, sa = 0;
			for (size_t k = first; k < size_t(count); ++k)
				sp += plaq[k];
			for (size_t k = 0; k < size_t(count); ++k)
				sa += acc[k];
			double mean = sp / double(m);
			if (digits <= 3)
				std::printf("beta = %.3f, acc = %.3f, plaq = %.3f\n", betas[size_t(r)], sa / count, mean);
			else
			{
				// standard error from bins of 5 consecutive trajectories
				size_t nb = m / 5;
				double s2 = 0;
				for (size_t bi = 0; bi < nb; ++bi)
				{
					double bm = 0;
					for (size_t k = 0; k < 5; ++k)
						bm += plaq[first + 5 * bi + k];
					bm /= 5;
					s2 += (bm - mean) * (bm - mean);
				}
				double err = nb > 1 ? std::sqrt(s2 / double(nb - 1) / double(nb)) : 0.0;
				std::printf("beta = %.*f, acc = %.*f, plaq = %.*f +- %.*f\n", digits, betas[size_t(r)], digits,
				            sa / count, digits, mean, digits, err);
			}
		}
	}
	catch (std::exception const &e)
	{
		std::fprintf(stderr, "%s\n", e.what());
		return 1;
	}
	return 0;
}
