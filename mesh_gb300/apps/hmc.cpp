// Pure-gauge HMC driver on the drop-in C++ API (include/mesh/mesh.hpp), the
// counterpart of krox/mesh's src/apps/hmc.cpp: same options and flow
// (makeDeltas, dispatchByGroup, Hmc<G>, runHmcUpdate loop, print_summary).
//
//   g++ -std=c++20 -O2 -I include mesh_gb300/apps/hmc.cpp
//       -L mesh_gb300 -lmesh_gb300 -Wl,-rpath,$PWD/mesh_gb300 -o hmc
//   ./hmc --group su3 --geom 8 8 8 8 --beta 5.7 --start cold --scheme 2lf
//         --epsilon 0.5 --substeps 10 --count 20 --seed 1234 --precision 2
//         (--start random | cold | FILE: a configuration file, as the reference's
//          hmc.U = readConfig<G>(start, &g))
//         [--checkpoint chain.bin]   links + trajectory counter at the end
//         [--resume chain.bin]       continue a chain (same --seed) from a checkpoint
#include "mesh/mesh.hpp"

#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

using namespace mesh;

int main(int argc, char **argv)
{
	std::string group = "su3", scheme = "4mn", start = "random", resume, checkpoint;
	std::vector<int32_t> geom = {8, 8, 8, 8};
	double beta = 6.0, epsilon = 1.0;
	int substeps = 8, count = 100, precision = 2;
	uint64_t seed = 0;
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
		else if (a == "--beta")
			beta = std::atof(next());
		else if (a == "--start")
			start = next();
		else if (a == "--seed")
			seed = std::strtoull(next(), nullptr, 10);
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
		else if (a == "--resume")
			resume = next();
		else if (a == "--checkpoint")
			checkpoint = next();
		else
		{
			std::fprintf(stderr, "unknown option %s\n", a.c_str());
			return 2;
		}
	}
	try
	{
		auto deltas = makeDeltas(scheme, epsilon, substeps);
		dispatchByGroup(
		    [&]<typename G>() {
			    Grid g{Coordinate(geom.begin(), geom.end())};
			    Hmc<G> hmc(g, seed);
			    if (!resume.empty())
				    hmc.load(resume);
			    else if (start == "random")
				    hmc.randomizeGaugeField();
			    else if (start == "cold")
				    hmc.coldStart();
			    else
				    hmc.U = readConfig<G>(start, &g);
			    auto t0 = std::chrono::steady_clock::now();
			    for (int iter = 0; iter < count; ++iter)
				    hmc.runHmcUpdate(beta, deltas);
			    double secs = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
			    if (!checkpoint.empty())
				    hmc.save(checkpoint);
			    hmc.print_summary();
			    for (size_t k = 0; k < hmc.plaq_history.size(); ++k)
				    std::printf("traj %zu plaq %.15f dH %.15e accept %.0f\n", k, hmc.plaq_history[k],
				                hmc.deltaH_history[k], hmc.accept_history[k]);
			    std::printf("time per trajectory = %.6f s\n", secs / count);
		    },
		    group, precision);
	}
	catch (std::exception const &e)
	{
		std::fprintf(stderr, "error: %s\n", e.what());
		return 1;
	}
	return 0;
}
