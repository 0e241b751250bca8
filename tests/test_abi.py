"""CPU checks of the drop-in boundary: the C-ABI library loads without a GPU
and exports every function include/mesh_gb300.h declares; the header compiles
as C and as C++; the Python binding covers every symbol."""
import ctypes
import os
import re
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADERS = [os.path.join(ROOT, "include", "mesh_gb300.h")]


def declared_symbols():
    names = []
    for h in HEADERS:
        txt = open(h).read()
        txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
        names += re.findall(r"^[A-Za-z_][\w\s\*]*?\b(mesh_\w+)\s*\(", txt, flags=re.M)
    return sorted(set(names))


@pytest.fixture(scope="module")
def libpath():
    import mesh_gb300.build as b

    return b.build()


def test_library_exports_every_declared_symbol(libpath):
    L = ctypes.CDLL(libpath)
    syms = declared_symbols()
    assert len(syms) > 40
    missing = [s for s in syms if not hasattr(L, s)]
    assert not missing, missing


def test_python_binding_covers_header():
    import mesh_gb300 as mg

    assert set(declared_symbols()) <= set(mg.SIGNATURES)


@pytest.mark.parametrize("lang,cc", [("c", "gcc"), ("c++", "g++")])
def test_header_compiles(lang, cc, tmp_path):
    src = tmp_path / ("t.c" if lang == "c" else "t.cpp")
    src.write_text('#include "mesh_gb300.h"\nint main(void){ return mesh_version() > 0 ? 0 : 1; }\n')
    r = subprocess.run([cc, "-fsyntax-only", "-Wall", "-Werror", "-I", os.path.join(ROOT, "include"), str(src)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


def test_version_and_errors_without_gpu(libpath):
    import mesh_gb300 as mg

    L = mg.load()
    assert L.mesh_version() >= 100
    # argument errors are reported, not thrown (no GPU needed for these)
    n = ctypes.c_int()
    rc = L.mesh_make_deltas(b"3xx", 0.5, 4, None, 0, ctypes.byref(n))
    assert rc == 1 and b"unknown scheme" in L.mesh_last_error()
    buf = (ctypes.c_double * 64)()
    assert L.mesh_make_deltas(b"2mn", 0.5, 4, buf, 64, ctypes.byref(n)) == 0 and n.value == 17
    # null handles are argument errors, checked before any device work
    d = ctypes.c_double()
    assert L.mesh_field_axpby(None, 1.0, None, 0.0, None) != 0
    assert L.mesh_site_exp(None, None) != 0 and b"null" in L.mesh_last_error()
    assert L.mesh_site_project(None, None) != 0
    assert L.mesh_landau_line_search(None, None, None, 1.0, ctypes.byref(d)) != 0
    assert L.mesh_landau_fa_set_accept(None, 1) != 0


def test_noalloc_plaquette_refuses_without_launching(libpath):
    """mesh_plaquette_noalloc given a host buffer (here, without a GPU, any
    buffer): an error status and a message, no crash; argument errors come
    before any CUDA call"""
    import mesh_gb300 as mg

    L = mg.load()
    host = np.ones(4 * 256 * 18, dtype=np.float32)
    d = (ctypes.c_int32 * 4)(4, 4, 4, 4)
    out = ctypes.c_double(-1.0)
    p = host.ctypes.data_as(ctypes.c_void_p)
    assert L.mesh_plaquette_noalloc(0, 3, 1, 4, d, p, None, ctypes.byref(out)) != 0
    assert L.mesh_last_error() and out.value == -1.0
    bad = (ctypes.c_int32 * 4)(4, 4, 4, 5)
    assert L.mesh_plaquette_noalloc(0, 3, 1, 4, bad, p, None, ctypes.byref(out)) == 1
    assert b"even" in L.mesh_last_error()


def test_make_deltas_matches_oracle(oracle, libpath):
    import mesh_gb300 as mg
    import numpy as np

    for sch, eps, n in (("2lf", 0.5, 10), ("2mn", 0.5, 20), ("4mn", 1.0, 8), ("2lf", 0.5, 16)):
        np.testing.assert_array_equal(mg.make_deltas(sch, eps, n), oracle.make_deltas(sch, eps, n))


def test_config_header_format_without_gpu(libpath, tmp_path):
    """the configuration file header is read on the host: a file written
    here by hand in the documented format is understood, a file with a wrong
    magic is refused"""
    import struct

    import mesh_gb300 as mg

    dims = [4, 6, 8, 2]
    data = np.arange(4 * 4 * 6 * 8 * 2 * 4, dtype=np.float64)  # SU(2) FP64, 4 components
    hdr = b"MESHCFG1" + struct.pack("<6i4iQQQ", 1, 2, 2, 0, 4, 4, *dims, 17, 99, 0)
    assert len(hdr) == 72
    path = tmp_path / "c.bin"
    path.write_bytes(hdr + data.tobytes())
    assert mg.config_info(str(path)) == {"kind": 0, "group": 2, "precision": 2, "dims": dims, "nstack": 4,
                                         "trajectory": 17, "seed": 99}
    bad = tmp_path / "bad.bin"
    bad.write_bytes(b"NOTMESH!" + hdr[8:] + data.tobytes())
    with pytest.raises(mg.MeshError):
        mg.config_info(str(bad))


def test_cpp_dropin_app_compiles(libpath, tmp_path):
    """the converted src/apps/hmc.cpp builds on the C++ drop-in header and
    links against the library (running it needs a GPU: test_gpu_app)"""
    exe = tmp_path / "hmc"
    r = subprocess.run(["g++", "-std=c++20", "-O1", "-Wall", "-Werror", "-I", os.path.join(ROOT, "include"),
                        os.path.join(ROOT, "mesh_gb300", "apps", "hmc.cpp"), "-L", os.path.dirname(libpath),
                        "-lmesh_gb300", "-Wl,-rpath," + os.path.dirname(libpath), "-o", str(exe)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


DISPATCH_CPP = r"""
#include "mesh/mesh.hpp"
#include <cstdio>
struct Show
{
	template <class G> void operator()() const
	{
		std::printf("%s %d %zu\n", std::string(mesh::GaugeTraits<G>::name()).c_str(),
		            int(mesh::GaugeTraits<G>::precision), sizeof(typename mesh::GaugeTraits<G>::real));
	}
};
int main()
{
	for (int p : {1, 2})
		for (char const *g : {"u1", "su2", "su3"})
			mesh::dispatchByGroup(Show{}, g, p);
	for (auto [g, p] : {std::pair{"su4", 1}, std::pair{"su3", 3}})
		try
		{
			mesh::dispatchByGroup(Show{}, g, p);
		}
		catch (std::runtime_error const &e)
		{
			std::printf("error: %s\n", e.what());
		}
	return 0;
}
"""


def test_cpp_dispatch_by_group_without_gpu(libpath, tmp_path):
    """dispatchByGroup (src/gauge/utils.h:156-186): the group names and
    precision levels of the reference select the same instantiations, and
    unknown ones raise the reference's messages"""
    src = tmp_path / "d.cpp"
    src.write_text(DISPATCH_CPP)
    exe = tmp_path / "d"
    r = subprocess.run(["g++", "-std=c++20", "-O1", "-Wall", "-Werror", "-I", os.path.join(ROOT, "include"), str(src),
                        "-L", os.path.dirname(libpath), "-lmesh_gb300", "-Wl,-rpath," + os.path.dirname(libpath),
                        "-o", str(exe)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    out = subprocess.run([str(exe)], capture_output=True, text=True, timeout=60).stdout.splitlines()
    assert out[:6] == ["u1 1 4", "su2 1 4", "su3 1 4", "u1 2 8", "su2 2 8", "su3 2 8"]
    assert out[6] == "error: unknown gauge group 'su4'"
    assert out[7] == "error: invlid precision level '3'"


def test_cpp_landau_fa_instantiate(libpath, tmp_path):
    """the C++ wrapper of the Fourier-accelerated solver compiles (FP64
    groups only) and the raw FP32 copy of the committed network matches the
    .npz the Python side loads"""
    import numpy as np

    src = tmp_path / "fa.cpp"
    src.write_text('#include "mesh/mesh.hpp"\n'
                   "template class mesh::LandauFA<mesh::SU3<double>>;\n"
                   "template class mesh::LandauFA<mesh::U1<double>>;\n"
                   "template struct mesh::Landau<mesh::SU3<float>>;\n"
                   "auto lin(mesh::Lattice<mesh::SU3<float>> const &a, mesh::Lattice<mesh::SU3<float>> const &b)\n"
                   "{ auto c = a + b; c -= a; c *= 2.0; c += b; mesh::add_mul(c, 0.5, b);\n"
                   "  return 3.0 * (c - b) * 1.0 * (a * b) * mesh::exp(mesh::project_on_algebra(a)); }\n"
                   "auto lin2(mesh::GaugeField<mesh::U1<double>> &U, mesh::GaugeField<mesh::U1<double>> const &P)\n"
                   "{ U += 0.5 * P; mesh::add_mul(U, -1.0, P); return U - P; }\n"
                   "std::vector<float> f() { return mesh::readMlpParams(\"x.f32\"); }\n")
    r = subprocess.run(["g++", "-std=c++20", "-O1", "-Wall", "-Werror", "-c", "-I", os.path.join(ROOT, "include"),
                        str(src), "-o", str(tmp_path / "fa.o")], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    z = np.load(os.path.join(ROOT, "mesh_gb300", "landau_mlp_su3.npz"))
    raw = np.fromfile(os.path.join(ROOT, "mesh_gb300", "landau_mlp_su3.f32"), dtype="<f4")
    w = int(z["width"])
    assert raw.size == w * w + 6 * w + 1
    assert np.array_equal(raw, z["params"].astype(np.float32))


def test_cpp_wilson_loops_instantiate(libpath, tmp_path):
    """the drop-in wilson(), thermalize() and overrelax() (legacy
    src/old/mesh/wilson.cpp:40-75, src/old/wilson.cpp, gauge_action.h)
    compile"""
    src = tmp_path / "w.cpp"
    src.write_text('#include "mesh/mesh.hpp"\n'
                   "template std::vector<std::tuple<int, int, double>> mesh::wilson(mesh::GaugeField<mesh::U1<float>> const &, int, int);\n"
                   "template std::vector<std::tuple<int, int, double>> mesh::wilson(mesh::GaugeField<mesh::SU2<double>> const &, int, int);\n"
                   "template std::vector<std::tuple<int, int, double>> mesh::wilson(mesh::GaugeField<mesh::SU3<float>> const &, int, int);\n"
                   "template void mesh::thermalize(mesh::GaugeField<mesh::SU3<double>> &, double, uint64_t, uint64_t);\n"
                   "template void mesh::overrelax(mesh::GaugeField<mesh::U1<float>> &);\n")
    r = subprocess.run(["g++", "-std=c++20", "-O1", "-Wall", "-Werror", "-c", "-I", os.path.join(ROOT, "include"),
                        str(src), "-o", str(tmp_path / "w.o")], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


def test_functor_layer_compiles_with_user_functors(tmp_path):
    """include/mesh/lattice_apply.cuh compiles for sm_103a with the user
    functors of the GPU test (a __device__ lambda, functor structs, a struct
    sum type, cshift); no GPU needed to compile"""
    import shutil

    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(nvcc):
        pytest.skip("nvcc not found")
    import test_gpu_functor_layer as t

    src = tmp_path / "user_functors.cu"
    src.write_text(t.SRC)
    r = subprocess.run([nvcc, "-gencode", "arch=compute_103a,code=sm_103a", "-std=c++20", "--extended-lambda",
                        "-c", "-Xcompiler", "-fPIC", "-I", os.path.join(ROOT, "include"), str(src), "-o",
                        str(tmp_path / "u.o")], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr

