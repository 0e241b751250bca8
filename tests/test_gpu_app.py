"""The converted HMC driver (mesh_gb300/apps/hmc.cpp on include/mesh/mesh.hpp)
runs the reference app's own small chain (SU(3) 8^4 beta 5.7, cold start, 2lf
eps 0.5 n 10, seed 1234, FP64) and matches the FP64 oracle chain; a run cut
in two by --checkpoint / --resume prints the same trajectories."""
import os
import re
import subprocess

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def build_app(tmp_path):
    import mesh_gb300.build as b

    lib = b.build()
    exe = tmp_path / "hmc"
    subprocess.run(["g++", "-std=c++20", "-O2", "-I", os.path.join(ROOT, "include"),
                    os.path.join(ROOT, "mesh_gb300", "apps", "hmc.cpp"), "-L", os.path.dirname(lib), "-lmesh_gb300",
                    "-Wl,-rpath," + os.path.dirname(lib), "-o", str(exe)], check=True)
    return str(exe)


def run(exe, *args):
    r = subprocess.run([exe, *args], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    recs = re.findall(r"traj (\d+) plaq (\S+) dH (\S+) accept (\S+)", r.stdout)
    return np.array([[float(p), float(d), float(a)] for _, p, d, a in recs])


def test_app_matches_oracle_and_resumes(oracle, tmp_path):
    exe = build_app(tmp_path)
    common = ["--group", "su3", "--geom", "8", "8", "8", "8", "--beta", "5.7", "--scheme", "2lf", "--epsilon",
              "0.5", "--substeps", "10", "--seed", "1234", "--precision", "2"]
    full = run(exe, *common, "--start", "cold", "--count", "6")
    dims = [8, 8, 8, 8]
    _, recs = oracle.hmc_chain(3, 2, dims, oracle.unit_gauge(3, 2, dims), 5.7, oracle.make_deltas("2lf", 0.5, 10),
                               1234, 0, 6)
    np.testing.assert_array_equal(full[:, 2], recs[:, 2])
    np.testing.assert_allclose(full[:, 0], recs[:, 0], rtol=1e-10)
    ck = str(tmp_path / "chain.bin")
    first = run(exe, *common, "--start", "cold", "--count", "3", "--checkpoint", ck)
    second = run(exe, *common, "--resume", ck, "--count", "3")
    np.testing.assert_array_equal(np.vstack([first, second]), full)
    # --start FILE (the reference's hmc.U = readConfig<G>(start, &g)): a new
    # chain, trajectory counter 0, from the checkpointed links
    from_file = run(exe, *common, "--start", ck, "--count", "2")
    deltas = oracle.make_deltas("2lf", 0.5, 10)
    U3, _ = oracle.hmc_chain(3, 2, dims, oracle.unit_gauge(3, 2, dims), 5.7, deltas, 1234, 0, 3)
    _, recs2 = oracle.hmc_chain(3, 2, dims, U3, 5.7, deltas, 1234, 0, 2)
    np.testing.assert_array_equal(from_file[:, 2], recs2[:, 2])
    np.testing.assert_allclose(from_file[:, 0], recs2[:, 0], rtol=1e-10)


LANDAU_FA_CPP = r"""
#include "mesh/mesh.hpp"
#include <cstdio>
// Fourier-accelerated Landau gauge fixing through the C++ wrapper, with the
// committed network, against the reference-style overrelaxation
int main(int argc, char **argv)
{
	using G = mesh::SU3<double>;
	if (argc < 2)
		return 2;
	mesh::Grid grid({8, 8, 8, 8});
	mesh::GaugeField<G> U(grid);
	U.set_unit();
	for (uint64_t s = 0; s < 20; ++s)
		mesh::thermalize(U, 6.0, 11, s);
	mesh::Landau<G> L(U);
	mesh::LandauFA<G> fa(U);
	fa.set_mlp(mesh::readMlpParams(argv[1]), 64, 6.0);
	auto r = fa.run(L.g);
	std::printf("fa %d %d %.6e %.15f\n", r.iterations, r.fallbacks, r.theta, L());
	mesh::Landau<G> L2(U);
	int sweeps = L2.overrelax(1.7, 1e-12, 20000);
	std::printf("or %d %.6e %.15f\n", sweeps, L2.condition(), L2());
	return 0;
}
"""


def test_cpp_landau_fa_learned(tmp_path):
    import mesh_gb300.build as b

    lib = b.build()
    src = tmp_path / "fa.cpp"
    src.write_text(LANDAU_FA_CPP)
    exe = tmp_path / "fa"
    subprocess.run(["g++", "-std=c++20", "-O2", "-I", os.path.join(ROOT, "include"), str(src), "-L",
                    os.path.dirname(lib), "-lmesh_gb300", "-Wl,-rpath," + os.path.dirname(lib), "-o", str(exe)],
                   check=True)
    r = subprocess.run([str(exe), os.path.join(ROOT, "mesh_gb300", "landau_mlp_su3.f32")], capture_output=True,
                       text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    fa = re.search(r"fa (\d+) (\d+) (\S+) (\S+)", r.stdout)
    orr = re.search(r"or (\d+) (\S+) (\S+)", r.stdout)
    assert float(fa.group(3)) < 1e-12
    f_fa, f_or = float(fa.group(4)), float(orr.group(3))
    # both gauge-fixed: maxima of the functional near 1 (Gribov copies may differ)
    assert 0.5 < f_fa < 1.0 and abs(f_fa - f_or) < 1e-3
