"""What the trained spectral multiplier gives on thermalised SU(3) 24^4
beta = 6.0 configurations (the lattice size the committed network,
mesh_gb300/landau_mlp_su3.npz, was trained on; HMC chains with seeds 1..8,
100 trajectories, Haar-random gauge transform with seed 5).

Cost = descent steps + 11 per overrelaxation fallback (a fallback is 10
sweeps plus the rejected step); overrelaxation costs one per sweep. A sweep
and a descent step take about the same time, so the comparisons do not depend
on timing noise.

* Fourier-accelerated descent with the network reaches theta < 1e-12 on
  every configuration, at under half the cost of FP64 overrelaxation
  (measured: about a fifth, on seeds 1..3).
* Against the plain multiplier 0.08 p2max/p^2 the network is not a robust
  win: the cost of one configuration is set by where the fallbacks fall and
  varies by up to 4x between configurations for either multiplier, and sums
  over eight configurations have come out 1.39x in the network's favour on
  one set of chains and 0.94x on another (the chains differ at the rounding
  level between builds of the HMC kernels). The test only guards against a
  broken network: the learned sum stays within 1.25x of the plain one."""
import pytest

from mesh_gb300 import landau_learn as ll

pytestmark = pytest.mark.gpu


def test_trained_multiplier_vs_plain_and_overrelaxation(ctx):
    params, _ = ll.load_weights()
    cost = {"plain": 0, "learned": 0, "or": 0, "learned_or_set": 0}
    for k, (beta, Uh) in enumerate(ll.hmc_configs(ctx, 24, [6.0] * 8, list(range(1, 9)), 100, 1, 0)):
        methods = ("plain", "learned", "or") if k < 3 else ("plain", "learned")
        for method in methods:
            U = ll.prepared_links(ctx, Uh, transform_seed=5)
            r = ll.solve(ctx, U, method, params, beta)
            assert r["theta"] < 1e-12, (k, method, r)
            # a gauge-fixed configuration: the functional is a maximum near 1
            assert 0.5 < r["functional"] < 1.0
            c = r["iterations"] + 11 * r["fallbacks"]
            cost[method] += c
            if method == "learned" and k < 3:
                cost["learned_or_set"] += c
    assert 2 * cost["learned_or_set"] < cost["or"], cost
    assert cost["learned"] < 1.25 * cost["plain"], cost
