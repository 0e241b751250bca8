"""The coupling scan on the GPU: the converted sweep_beta app
(mesh_gb300/apps/sweep_beta.cpp; the reference's src/apps/sweep_beta.cpp),
every coupling a replica of one batched persistent launch. At strong coupling
the SU(3) plaquette follows the expansion the reference plots,
beta/18 (sweep_beta.cpp:91), with the next order beta^2/216; SU(2) follows
beta/4 and U(1) beta/2 at leading order. The app's output lines keep the
reference's format."""
import os
import re
import subprocess

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def app(tmp_path_factory):
    import mesh_gb300.build as b

    lib = b.build()
    exe = tmp_path_factory.mktemp("sweep") / "sweep_beta"
    subprocess.run(["g++", "-std=c++20", "-O2", "-I", os.path.join(ROOT, "include"),
                    os.path.join(ROOT, "mesh_gb300", "apps", "sweep_beta.cpp"), "-L", os.path.dirname(lib),
                    "-lmesh_gb300", "-Wl,-rpath," + os.path.dirname(lib), "-o", str(exe)], check=True)
    return str(exe)


def run(exe, *args):
    r = subprocess.run([exe, *args], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    return r.stdout


def test_reference_output_format(app):
    out = run(app, "--group", "su3", "--geom", "4", "4", "4", "4", "--beta-count", "4", "--count", "10",
              "--seed", "1")
    lines = out.strip().splitlines()
    assert len(lines) == 4
    for ln, beta in zip(lines, (0.0, 8 / 3, 16 / 3, 8.0)):
        m = re.fullmatch(r"beta = (\d+\.\d{3}), acc = (\d\.\d{3}), plaq = (-?\d\.\d{3})", ln)
        assert m, ln
        assert float(m.group(1)) == pytest.approx(beta, abs=1e-3)


@pytest.mark.parametrize("group,lead,second", [("su3", 1 / 18, 1 / 216), ("su2", 1 / 4, 0.0), ("u1", 1 / 2, 0.0)])
def test_strong_coupling_slope(app, group, lead, second):
    """small couplings, 8^4, 60 trajectories per coupling (the first 6
    dropped), all couplings in one batch: the plaquette against the strong-
    coupling series within 4 standard errors plus the size of the first
    neglected order"""
    betas_max = {"su3": 1.2, "su2": 0.4, "u1": 0.2}[group]
    out = run(app, "--group", group, "--geom", "8", "8", "8", "8", "--beta-min", "0", "--beta-max", str(betas_max),
              "--beta-count", "7", "--count", "60", "--scheme", "2mn", "--epsilon", "1.0", "--substeps", "6",
              "--precision", "2", "--seed", "5", "--digits", "6")
    rows = re.findall(r"beta = (\S+), acc = (\S+), plaq = (\S+) \+- (\S+)", out)
    assert len(rows) == 7, out
    b, acc, p, e = (np.array([float(r[i]) for r in rows]) for i in range(4))
    assert np.all(acc > 0.5), out
    expect = lead * b + second * b * b
    # size of the first neglected order at the largest coupling, per group
    slack = {"su3": 2e-3, "su2": 2e-3, "u1": 2e-3}[group]
    assert np.all(np.abs(p - expect) < 4 * e + slack), (out, expect)
    # the slope itself: a straight-line fit through the origin
    slope = float(np.sum(b * (p - second * b * b)) / np.sum(b * b))
    assert slope == pytest.approx(lead, rel=0.05), out
