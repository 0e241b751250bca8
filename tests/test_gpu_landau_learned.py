"""What the trained spectral multiplier gains over the plain one: on eight
thermalised SU(3) 24^4 beta = 6.0 configurations (the lattice size the
committed network, mesh_gb300/landau_mlp_su3.npz, was trained on; HMC chains
with seeds 1..8, 100 trajectories, Haar-random gauge transform with seed 5),
Fourier-accelerated descent with the network and with the plain multiplier
0.08 p2max/p^2 both reach theta < 1e-12; the learned one does it at lower
total cost. The cost of a single configuration is dominated by where the
fallbacks fall and varies by up to 4x between configurations for either
multiplier, so the comparison is over the sum of eight (measured: 17019
against 23933). Cost = descent steps + 11 per
overrelaxation fallback (a fallback is 10 sweeps plus the rejected step; a
sweep and a step take about the same time), so the comparison does not
depend on timing noise."""
import numpy as np
import pytest

import mesh_gb300 as mg
from mesh_gb300 import landau_learn as ll

pytestmark = pytest.mark.gpu


def test_trained_multiplier_beats_plain(ctx):
    params, _ = ll.load_weights()
    cost = {"plain": 0, "learned": 0}
    for beta, Uh in ll.hmc_configs(ctx, 24, [6.0] * 8, list(range(1, 9)), 100, 1, 0):
        for method in ("plain", "learned"):
            U = ll.prepared_links(ctx, Uh, transform_seed=5)
            r = ll.solve(ctx, U, method, params, beta)
            assert r["theta"] < 1e-12
            # a gauge-fixed configuration: the functional is a maximum near 1
            assert 0.5 < r["functional"] < 1.0
            cost[method] += r["iterations"] + 11 * r["fallbacks"]
    assert cost["learned"] < cost["plain"], cost
