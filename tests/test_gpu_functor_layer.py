"""The generic functor layer include/mesh/lattice_apply.cuh (the reference's
lattice_apply / lattice_sum_apply / lattice_sum / cshift for user functors,
src/lattice/device.h:139-265, src/lattice/lattice.h:256-273,366-389),
compiled here with nvcc as a user would compile it, run on library fields
(mesh_field_device_ptr) and compared with the oracle: elementwise functors
exactly, sums to the FP64 rounding of their order, cshift bit for bit."""
import ctypes as C
import os
import shutil
import subprocess

import numpy as np
import pytest

import mesh_gb300 as mg

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

SRC = r"""
#include "mesh/lattice_apply.cuh"
using namespace mesh::device;

struct SU3f { float v[18]; };
struct Sum18 {
	double v[18];
	__host__ __device__ Sum18 &operator+=(Sum18 const &o) { for (int k = 0; k < 18; ++k) v[k] += o.v[k]; return *this; }
};
// a = b c (3x3 complex product, row-major (re, im) pairs)
struct Mul {
	__device__ void operator()(SU3f &a, SU3f const &b, SU3f const &c) const {
		for (int i = 0; i < 3; ++i)
			for (int j = 0; j < 3; ++j) {
				float re = 0.f, im = 0.f;
				for (int k = 0; k < 3; ++k) {
					float br = b.v[6 * i + 2 * k], bi = b.v[6 * i + 2 * k + 1];
					float cr = c.v[6 * k + 2 * j], ci = c.v[6 * k + 2 * j + 1];
					re += br * cr - bi * ci;
					im += br * ci + bi * cr;
				}
				a.v[6 * i + 2 * j] = re;
				a.v[6 * i + 2 * j + 1] = im;
			}
	}
};
struct RealTrace {
	__device__ double operator()(SU3f const &a) const { return double(a.v[0]) + double(a.v[8]) + double(a.v[16]); }
};
struct Widen {
	__device__ Sum18 operator()(SU3f const &a) const { Sum18 r; for (int k = 0; k < 18; ++k) r.v[k] = a.v[k]; return r; }
};

extern "C" int fl_axpy(void *a, void const *b, long long V, float alpha) {
	try {
		lattice_apply([=] __device__(SU3f & x, SU3f const &y) { for (int k = 0; k < 18; ++k) x.v[k] += alpha * y.v[k]; },
		              view<SU3f>(a, V), view<SU3f>(b, V));
		return cudaDeviceSynchronize() == cudaSuccess ? 0 : 2;
	} catch (...) { return 1; }
}
extern "C" int fl_mul(void *a, void const *b, void const *c, long long V) {
	try {
		lattice_apply(Mul{}, view<SU3f>(a, V), view<SU3f>(b, V), view<SU3f>(c, V));
		return cudaDeviceSynchronize() == cudaSuccess ? 0 : 2;
	} catch (...) { return 1; }
}
extern "C" int fl_sum_retr(void const *a, long long V, double *out) {
	try { *out = lattice_sum_apply(RealTrace{}, view<SU3f>(a, V)); return 0; } catch (...) { return 1; }
}
extern "C" int fl_sum18(void const *a, long long V, double *out) {
	try {
		Sum18 s = lattice_sum_apply(Widen{}, view<SU3f>(a, V));
		for (int k = 0; k < 18; ++k) out[k] = s.v[k];
		return 0;
	} catch (...) { return 1; }
}
extern "C" int fl_sum_f(void const *a, long long V, float *out) {
	try { *out = lattice_sum(view<float>(a, V)); return 0; } catch (...) { return 1; }
}
extern "C" int fl_cshift(int nd, int const *dims, void *dst, void const *src, int dir, int off) {
	try {
		long long V = 1;
		for (int i = 0; i < nd; ++i) V *= dims[i];
		cshift(nd, dims, view<SU3f>(dst, V), view<SU3f>(src, V), dir, off);
		return cudaDeviceSynchronize() == cudaSuccess ? 0 : 2;
	} catch (...) { return 1; }
}
"""


@pytest.fixture(scope="module")
def fl(tmp_path_factory):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(nvcc):
        pytest.skip("nvcc not found")
    d = tmp_path_factory.mktemp("functor")
    src = d / "user_functors.cu"
    src.write_text(SRC)
    so = d / "libuser_functors.so"
    cmd = [nvcc, "-gencode", "arch=compute_103a,code=sm_103a", "-std=c++20", "--extended-lambda", "-O2", "-shared",
           "-Xcompiler", "-fPIC", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(so)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    L = C.CDLL(str(so))
    P, LL = C.c_void_p, C.c_longlong
    L.fl_axpy.argtypes = [P, P, LL, C.c_float]
    L.fl_mul.argtypes = [P, P, P, LL]
    L.fl_sum_retr.argtypes = [P, LL, C.POINTER(C.c_double)]
    L.fl_sum18.argtypes = [P, LL, C.POINTER(C.c_double)]
    L.fl_sum_f.argtypes = [P, LL, C.POINTER(C.c_float)]
    L.fl_cshift.argtypes = [C.c_int, C.POINTER(C.c_int), P, P, C.c_int, C.c_int]
    return L


DIMS = [4, 6, 4, 8]


def field(ctx, arr):
    return mg.Lattice(ctx, 3, mg.F32, mg.Grid(DIMS)).import_(arr)


def test_lattice_apply_lambda_and_functor(ctx, oracle, fl):
    V = int(np.prod(DIMS))
    A = oracle.random_gauge(3, 1, DIMS, 31)
    a, b, c = field(ctx, A[0]), field(ctx, A[1]), field(ctx, A[2])
    ctx.synchronize()
    assert fl.fl_axpy(a.device_ptr, b.device_ptr, V, C.c_float(0.25)) == 0
    np.testing.assert_array_equal(a.export(), (A[0] + np.float32(0.25) * A[1]).astype(np.float32))
    out = field(ctx, np.zeros_like(A[0]))
    ctx.synchronize()
    assert fl.fl_mul(out.device_ptr, b.device_ptr, c.device_ptr, V) == 0
    ref = oracle.site_mul(3, 2, DIMS, A[1].astype(np.float64), A[2].astype(np.float64))
    assert np.max(np.abs(out.export() - ref)) < 2e-6


def test_lattice_sum_apply_and_sum(ctx, oracle, fl):
    V = int(np.prod(DIMS))
    A = oracle.random_gauge(3, 1, DIMS, 32)
    a = field(ctx, A[0])
    ctx.synchronize()
    s = C.c_double()
    assert fl.fl_sum_retr(a.device_ptr, V, C.byref(s)) == 0
    ref = oracle.sum_real_trace(3, 2, DIMS, A[0].astype(np.float64))
    assert s.value == pytest.approx(ref, rel=1e-12, abs=1e-12)
    s18 = (C.c_double * 18)()
    assert fl.fl_sum18(a.device_ptr, V, s18) == 0
    np.testing.assert_allclose(np.array(s18), A[0].astype(np.float64).sum(axis=0), rtol=1e-12, atol=1e-12)
    # lattice_sum of a plain float field (one plane of 4-byte words)
    x = np.arange(V, dtype=np.float32) * np.float32(0.5)
    f = mg.Lattice(ctx, 1, mg.F32, mg.Grid(DIMS))
    # a U(1) field holds 2 floats per site; view its first V floats as a
    # float field (the first float plane of the float2 plane: interleaved)
    f.import_(np.stack([x, np.zeros(V, dtype=np.float32)], -1))
    ctx.synchronize()
    fs = C.c_float()
    assert fl.fl_sum_f(f.device_ptr, 2 * V, C.byref(fs)) == 0
    assert float(fs.value) == pytest.approx(float(x.astype(np.float64).sum()), rel=1e-6)


@pytest.mark.parametrize("dir,off", [(0, 1), (1, -1), (3, 3), (2, -2), (3, -7)])
def test_cshift_matches_library_and_oracle(ctx, oracle, fl, dir, off):
    A = oracle.random_gauge(3, 1, DIMS, 33)
    src = field(ctx, A[0])
    dst = field(ctx, np.zeros_like(A[0]))
    ctx.synchronize()
    d = (C.c_int * 4)(*DIMS)
    assert fl.fl_cshift(4, d, dst.device_ptr, src.device_ptr, dir, off) == 0
    ref = oracle.cshift(3, 1, DIMS, A[0], dir, off)
    np.testing.assert_array_equal(dst.export(), ref)
    lib = field(ctx, np.zeros_like(A[0]))
    mg.cshift(lib, src, dir, off)
    np.testing.assert_array_equal(lib.export(), dst.export())
