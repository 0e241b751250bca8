"""What the trained spectral multiplier gives on thermalised SU(3) 24^4
beta = 6.0 configurations (the lattice size the committed network,
mesh_gb300/landau_mlp_su3.npz, was trained on: 96 configurations of 16 HMC
chains with beta uniform in [5.8, 6.2]; evaluated here on other chains, HMC
seeds 1..8, 100 trajectories, Haar-random gauge transform with seed 5).
Fourier-accelerated steps are accepted on the gauge functional (the test the
network was trained under); a step that lowers the functional is undone and
replaced by 10 overrelaxation sweeps.

Cost = descent steps + 11 per fallback (a fallback is 10 sweeps plus the
rejected step); overrelaxation costs one per sweep. A sweep and a descent
step take about the same time, so the comparisons do not depend on timing
noise. Measured on a GB300 on these eight configurations when the network
was committed: overrelaxation 55200, plain multiplier 16317, the best fixed
member of the training family (alpha 0.08, high-mode factor 0.6) 20431, the
network 18910 (the configurations depend on the HMC kernels' rounding, so a
later build generates slightly different ones).

* Fourier-accelerated descent with the network reaches theta < 1e-12 on
  every configuration, at a third of the cost of FP64 overrelaxation (the
  target is at least 2x less).
* The network does beat the fixed family member it was trained against on
  the sum (0.93x its cost) but not the plain multiplier (1.16x): the cost of
  one configuration varies up to 4x with either multiplier, the per-decade
  choices the network learned do not carry over, and the sums it loses or
  wins by are within that spread. The test asserts the overrelaxation gain
  and guards against a broken network (the learned sum within 1.35x of the
  plain one); it makes no claim of a gain over plain descent."""
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
            r = ll.solve(ctx, U, method, params, beta, accept="functional")
            U.close()
            assert r["theta"] < 1e-12, (k, method, r)
            # a gauge-fixed configuration: the functional is a maximum near 1
            assert 0.5 < r["functional"] < 1.0
            c = r["iterations"] + 11 * r["fallbacks"] if method != "or" else r["iterations"]
            cost[method] += c
            if method == "learned" and k < 3:
                cost["learned_or_set"] += c
    print(cost)
    assert cost["learned_or_set"] < 0.6 * cost["or"], cost
    assert cost["learned"] < 1.35 * cost["plain"], cost
