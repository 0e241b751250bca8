"""The SU(3) FP32 helpers of the trajectory kernels, compiled for the host
(they are __host__ __device__) and checked against their FP64 forms on random
special unitary matrices and algebra elements: the row-2 rebuild
conj(row 0 x row 1) with fused multiply-adds, the projection from rows 0, 1
(proj_rows01), the order-6/order-10 exponential series and the rows-0,1
exponential of the fused link update, and the four-dimensional plane tables.
FP32 results within 4e-7 of FP64; the row-2-free projection within 1e-14 in
FP64. No GPU needed."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

SRC = r"""
#include "csrc/kernels.cuh"
#include <cmath>
#include <cstdio>
#include <random>
using namespace meshgb;
int main()
{
	using F = Group<SU3, float>;
	using D = Group<SU3, double>;
	std::mt19937 rng(17);
	std::normal_distribution<double> nd;
	double e_row2 = 0, e_proj01 = 0, e_exp = 0, e_exp_rows = 0;
	for (int t = 0; t < 4000; ++t)
	{
		double o[8], o2[8];
		float of[8];
		double sc = 0.005 + 0.04 * (t % 6);
		for (int k = 0; k < 8; ++k)
		{
			o[k] = nd(rng) * sc;
			of[k] = float(o[k]);
			o2[k] = nd(rng);
		}
		// a random special unitary matrix (FP64), its FP32 copy with row 2 rebuilt
		D::E u = D::mul(D::exp_alg(o2, 0.8), D::exp_alg(o, 1.3));
		F::E uf;
		for (int k = 0; k < 18; ++k)
			uf.v[k] = float(u.v[k]);
		F::complete_row2(uf);
		for (int k = 12; k < 18; ++k)
			e_row2 = std::fmax(e_row2, std::fabs(double(uf.v[k]) - u.v[k]));
		// projection from rows 0, 1 against the full projection (FP64)
		double a[8], b[8];
		D::proj(u, a);
		D::proj_rows01(u, b);
		for (int k = 0; k < 8; ++k)
			e_proj01 = std::fmax(e_proj01, std::fabs(a[k] - b[k]));
		// exponentials: FP32 forms against FP64
		D::E x = D::exp_alg(o, 1.0);
		F::E y = F::exp_alg(of, 1.0f), z = F::exp_alg_rows01(of, 1.0f);
		for (int k = 0; k < 18; ++k)
			e_exp = std::fmax(e_exp, std::fabs(double(y.v[k]) - x.v[k]));
		for (int k = 0; k < 12; ++k)
			e_exp_rows = std::fmax(e_exp_rows, std::fabs(double(z.v[k]) - x.v[k]));
	}
	// the four-dimensional plane tables against the enumeration (0,1), (0,2), ...
	int q = 0, bad_planes = 0;
	for (int mu = 0; mu < 4; ++mu)
		for (int nu = mu + 1; nu < 4; ++nu, ++q)
			bad_planes += plane_mu<4>(q) != mu || plane_nu<4>(q) != nu;
	std::printf("%.3e %.3e %.3e %.3e %d\n", e_row2, e_proj01, e_exp, e_exp_rows, bad_planes);
	return 0;
}
"""


def test_su3_fp32_helpers_against_fp64(tmp_path):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(nvcc):
        pytest.skip("nvcc not found")
    src = tmp_path / "group_math.cu"
    src.write_text(SRC)
    exe = tmp_path / "group_math"
    r = subprocess.run([nvcc, "-gencode", "arch=compute_103a,code=sm_103a", "-std=c++20", "--extended-lambda", "-O2",
                        "-I", os.path.join(ROOT, "mesh_gb300"),
                        "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    out = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120)
    assert out.returncode == 0, out.stderr
    e_row2, e_proj01, e_exp, e_exp_rows, bad_planes = (float(v) for v in out.stdout.split())
    assert bad_planes == 0
    assert e_row2 < 4e-7
    assert e_proj01 < 1e-14
    assert e_exp < 4e-7
    assert e_exp_rows < 4e-7
