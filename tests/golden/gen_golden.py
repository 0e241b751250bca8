"""Generates the golden fixtures of tests/golden/ from the REFERENCE ITSELF:
krox/mesh's own src/lattice + src/gauge templates and src/gauge/hmc.cpp,
compiled in place by `make -C oracle ref` (oracle/_ref/libref.so, with the
project-written util stand-ins of oracle/ref_shim). Inputs are seeded and
drawn with numpy; outputs are whatever the reference code computes on them.

    python tests/golden/gen_golden.py

Needs the reference tree (only present where the fixtures are generated);
the committed .npz files travel with the repository.
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
# this script reads the reference checkout in place
os.environ.setdefault("MESH_REF_SRC", "/root/reference/src")

import pyref  # noqa: E402

NREAL = {1: 2, 2: 4, 3: 18}
NNORM = {1: 1, 2: 3, 3: 18}  # normals the reference draws per algebra element


def haar(group, n, rng):
    """Haar-random group elements built with numpy (inputs only)."""
    if group == 1:
        t = rng.uniform(0, 2 * np.pi, n)
        return np.stack([np.cos(t), np.sin(t)], -1)
    if group == 2:
        q = rng.standard_normal((n, 4))
        return q / np.linalg.norm(q, axis=1, keepdims=True)
    m = rng.standard_normal((n, 3, 3)) + 1j * rng.standard_normal((n, 3, 3))
    q, r = np.linalg.qr(m)
    d = np.diagonal(r, axis1=1, axis2=2)
    q = q * (d / np.abs(d))[:, None, :]
    det = np.linalg.det(q)
    q[:, :, 0] /= det[:, None]
    out = np.zeros((n, 18))
    out[:, 0::2] = q.reshape(n, 9).real
    out[:, 1::2] = q.reshape(n, 9).imag
    return out


CASES = [
    # (name, group, dims, beta)
    ("su3", 3, [4, 4, 2, 4], 5.7),
    ("su2", 2, [4, 4, 4, 4], 2.3),
    ("u1", 1, [4, 4, 4, 4], 1.0),
    ("su3_3d", 3, [4, 4, 4], 5.0),
]


def main():
    for name, grp, dims, beta in CASES:
        rng = np.random.default_rng(sum(map(ord, name)))
        nd, V = len(dims), int(np.prod(dims))
        U = haar(grp, nd * V, rng).reshape(nd, V, NREAL[grp]).astype(np.float64)
        normals = rng.standard_normal(nd * V * NNORM[grp])
        P = pyref.random_algebra_field(grp, 2, dims, normals, NREAL[grp])
        d2lf = pyref.make_deltas("2lf", 0.5, 2)
        d2mn = pyref.make_deltas("2mn", 0.5, 2)
        out = dict(group=grp, dims=np.array(dims), beta=beta, U=U, P=P, normals=normals)
        out["plaquette"] = pyref.plaquette(grp, 2, dims, U)
        out["action"] = pyref.wilson_action(grp, 2, dims, U, beta)
        out["staple_mu1"] = pyref.staple_sum(grp, 2, dims, U, 1)
        out["deriv_mu2"] = pyref.wilson_deriv(grp, 2, dims, U, 2 % nd, beta)
        out["evolve_t0p1"] = pyref.evolve(grp, 2, dims, U, P, 0.1)
        out["reunit"] = pyref.reunitize(grp, 2, dims, U * 1.0005)
        out["cshift_d1_p1"] = pyref.cshift(grp, 2, dims, np.ascontiguousarray(U[0]), 1, 1)
        out["cshift_d0_m1"] = pyref.cshift(grp, 2, dims, np.ascontiguousarray(U[1]), 0, -1)
        out["hmd2lf_U"], out["hmd2lf_P"] = pyref.run_hmd(grp, 2, dims, U, P, beta, d2lf)
        out["hmd2mn_U"], out["hmd2mn_P"] = pyref.run_hmd(grp, 2, dims, U, P, beta, d2mn)
        out["deltas_2lf"], out["deltas_2mn"] = d2lf, d2mn
        out["deltas_4mn"] = pyref.make_deltas("4mn", 1.0, 3)
        if grp != 2:
            # full Hmc<G>::runHmcUpdate with the momenta normals played back
            Uh, rec = pyref.hmc_update(grp, 2, dims, U, normals, 0.25, beta, d2lf)
            out["hmc_U"] = Uh
            out["hmc_rec"] = np.array([rec["plaq"], rec["dH"], rec["accept"]])
        # Landau<G> (landau.h:23-136, reset() replaced by a unit fill): the
        # functional, condition and deriv at a Haar-random transform g, the
        # line search along that deriv from the reference's starting step,
        # and g after 25 iterations of run() (the Polak-Ribiere steps start
        # after iteration 20)
        g = haar(grp, V, rng).astype(np.float64)
        out["landau_g"] = g
        f, c, F = pyref.landau_eval(grp, 2, dims, U, g)
        out["landau_functional"], out["landau_condition"], out["landau_deriv"] = f, c, F
        out["landau_line_search"] = pyref.landau_line_search(grp, 2, dims, U, g, F, 3000.0)
        out["landau_run25_g"] = pyref.landau_run(grp, 2, dims, U, g, 25)
        np.savez_compressed(os.path.join(HERE, f"ref_{name}.npz"), **out)
        print(name, "plaquette", out["plaquette"])


if __name__ == "__main__":
    main()
