"""GPU tests of the Fourier-accelerated Landau path and the learned
multiplier's network, through the C ABI, against the CPU oracle.

Tolerances: the FFT is FP32 (1e-5 relative to the oracle's FP64 DFT); a
Fourier-accelerated step uses that FFT for its direction only, so g after
one step agrees with the FP64 oracle to 1e-5; theta and the convergence
criterion are FP64. Network: FP32 forward to 1e-5, BF16 inference to 2e-2
(relative to the output scale), gradients to 1e-3 relative of the oracle's
FP64 backward pass.
"""
import numpy as np
import pytest

import mesh_gb300 as mg

pytestmark = pytest.mark.gpu

BETA = {1: 2.0, 2: 2.5, 3: 6.0}


def rel(a, b):
    a, b = np.asarray(a), np.asarray(b)
    return float(np.max(np.abs(a - b)) / max(1e-300, float(np.max(np.abs(b)))))


def fixed_problem(oracle, g, dims, ntraj=20, seed=5):
    """thermalised links with a random gauge transform applied (FP64)"""
    U = oracle.unit_gauge(g, 2, dims)
    U, _ = oracle.hmc_chain(g, 2, dims, U, BETA[g], oracle.make_deltas("2lf", 0.5, 10), seed, 0, ntraj)
    h = oracle.random_transform(g, 2, dims, seed)
    return oracle.gauge_transform(g, 2, dims, U, h)


def plain_mult(dims, alpha):
    x = np.indices(dims).reshape(len(dims), -1).T
    p2 = np.sum(4 * np.sin(np.pi * x / np.array(dims)) ** 2, axis=1)
    p2max = 4.0 * len(dims)
    return np.where(p2 > 0, alpha * p2max / np.where(p2 > 0, p2, 1), 0.0)


@pytest.mark.parametrize("dims", [[8, 8, 8, 8], [4, 6, 8, 12], [24, 4, 4, 2], [8, 32], [6, 4, 16]])
def test_lattice_fft_vs_oracle(ctx, oracle, dims):
    rng = np.random.default_rng(0)
    V = int(np.prod(dims))
    data = (rng.standard_normal((3, V)) + 1j * rng.standard_normal((3, V))).astype(np.complex64)
    for sign in (-1, 1):
        got = mg.lattice_fft(ctx, dims, data, sign)
        ref = oracle.fft(dims, data.T.astype(np.complex128), sign).T
        assert rel(got, ref) < 2e-6 * np.log2(V)
    back = mg.lattice_fft(ctx, dims, mg.lattice_fft(ctx, dims, data, -1), 1) / V
    assert rel(back, data) < 1e-5


@pytest.mark.parametrize("g", [1, 2, 3])
def test_fa_step_vs_oracle(ctx, oracle, g):
    dims = [8, 8, 4, 8]
    U64 = fixed_problem(oracle, g, dims, ntraj=5)
    U = mg.GaugeField(ctx, g, mg.F64, mg.Grid(dims)).import_(U64)
    fa = mg.LandauFA(U)
    fa.set_plain(0.06)
    gt = mg.Lattice(ctx, g, mg.F64, mg.Grid(dims)).set_unit()
    g64 = oracle.unit_transform(g, 2, dims)
    mult = plain_mult(dims, 0.06)
    for k in range(3):
        th = fa.step(gt)
        th_ref, _ = oracle.landau_theta(g, 2, dims, U64, g64)
        # theta is FP64 on both sides; after the first step the two g differ
        # at the FP32-FFT level, ~1e-7
        assert th == pytest.approx(th_ref, rel=1e-12 if k == 0 else 1e-5)
        g64 = oracle.landau_fa_step(g, 2, dims, U64, g64, mult, 1.0)
        assert rel(gt.export(), g64) < 2e-5
    assert fa.theta(gt) == pytest.approx(oracle.landau_theta(g, 2, dims, U64, g64)[0], rel=1e-3)


def test_fa_run_converges_like_oracle(ctx, oracle):
    dims = [8, 8, 8, 8]
    U64 = fixed_problem(oracle, 3, dims)
    U = mg.GaugeField(ctx, 3, mg.F64, mg.Grid(dims)).import_(U64)
    fa = mg.LandauFA(U)
    fa.set_plain(0.08)
    gt = mg.Lattice(ctx, 3, mg.F64, mg.Grid(dims)).set_unit()
    it, fb, th = fa.run(gt, tol=1e-12, max_iter=400)
    assert th < 1e-12
    # the oracle's plain Fourier-accelerated descent on the same problem
    g64, mult, n_ref = oracle.unit_transform(3, 2, dims), plain_mult(dims, 0.08), 0
    while oracle.landau_theta(3, 2, dims, U64, g64)[0] >= 1e-12 and n_ref < 400:
        g64 = oracle.landau_fa_step(3, 2, dims, U64, g64, mult, 1.0)
        n_ref += 1
    if fb == 0:
        assert abs(it - n_ref) <= 3
    # gauge-fixed: same functional as the oracle's solution (same Gribov copy)
    L = mg.Landau(U)
    L.g.import_(gt.export())
    assert L() == pytest.approx(oracle.landau_theta(3, 2, dims, U64, g64)[1], rel=1e-9)


def test_fa_fallback_to_overrelaxation(ctx, oracle):
    """an unstable step size is caught: failed steps are undone and
    overrelaxation runs instead, and the run still converges"""
    dims = [8, 8, 8, 8]
    U64 = fixed_problem(oracle, 3, dims)
    U = mg.GaugeField(ctx, 3, mg.F64, mg.Grid(dims)).import_(U64)
    fa = mg.LandauFA(U)
    fa.set_plain(0.3)
    gt = mg.Lattice(ctx, 3, mg.F64, mg.Grid(dims)).set_unit()
    it, fb, th = fa.run(gt, tol=1e-12, max_iter=3000, omega=1.7, or_sweeps=10)
    assert th < 1e-12 and fb > 0


def test_fa_functional_acceptance(ctx, oracle):
    """steps accepted on the gauge functional instead of theta: the stable
    step size converges to the same functional as the theta-accepted run (a
    Gribov copy may differ at 1e-4), and an unstable one is still caught
    (fallbacks) and converges"""
    dims = [8, 8, 8, 8]
    U64 = fixed_problem(oracle, 3, dims)
    U = mg.GaugeField(ctx, 3, mg.F64, mg.Grid(dims)).import_(U64)
    L = mg.Landau(U)
    func = {}
    for accept in (False, True):
        for alpha in (0.08, 0.3):
            fa = mg.LandauFA(U)
            fa.set_plain(alpha)
            fa.set_accept(accept)
            gt = mg.Lattice(ctx, 3, mg.F64, mg.Grid(dims)).set_unit()
            it, fb, th = fa.run(gt, tol=1e-12, max_iter=3000, omega=1.7, or_sweeps=10)
            fa.close()
            assert th < 1e-12
            if alpha == 0.3:
                assert fb > 0
            L.g.import_(gt.export())
            func[accept, alpha] = L()
    assert func[True, 0.08] == pytest.approx(func[False, 0.08], rel=1e-4)
    assert 0.5 < func[True, 0.3] < 1.0


def test_fa_probe_response_is_physical(ctx, oracle):
    dims = [8, 8, 8, 8]
    U64 = fixed_problem(oracle, 3, dims)
    U = mg.GaugeField(ctx, 3, mg.F64, mg.Grid(dims)).import_(U64)
    fa = mg.LandauFA(U)
    fa.set_plain(0.08)
    gt = mg.Lattice(ctx, 3, mg.F64, mg.Grid(dims)).set_unit()
    for _ in range(25):
        fa.step(gt)
    pr = fa.probe(gt, 0.02, nbins=16)
    ok = pr["count"] > 0
    lam = pr["lambda"][ok]
    # every mode contracts under the probe step, at a finite rate
    assert np.all(lam > 0) and np.all(np.isfinite(lam))
    assert pr["theta"] > 0


def test_mlp_forward_grad_vs_oracle(ctx, oracle):
    rng = np.random.default_rng(3)
    for width in (32, 64):
        params = mg.mlp_init(width, seed=1) + rng.normal(0, 0.05, mg.mlp_nparams(width)).astype(np.float32)
        x = rng.normal(0, 1, (1000, 3)).astype(np.float32)
        t = rng.normal(0, 1, 1000).astype(np.float32)
        y = mg.mlp_forward(ctx, x, params, width)
        yo = oracle.mlp_forward(x, params, width)
        assert rel(y, yo) < 1e-5
        yb = mg.mlp_forward(ctx, x, params, width, bf16=True)
        assert np.max(np.abs(yb - yo)) < 2e-2 * max(1.0, np.max(np.abs(yo)))
        loss, grad = mg.mlp_grad(ctx, x, t, params, width)
        lo, go = oracle.mlp_grad(x, t, params, width)
        assert loss == pytest.approx(lo, rel=1e-5)
        assert rel(grad, go) < 1e-3


def test_mlp_training_fits_a_function(ctx):
    rng = np.random.default_rng(4)
    x = rng.uniform(-1, 1, (20000, 3)).astype(np.float32)
    t = (np.sin(2 * x[:, 0]) - 0.5 * x[:, 1] * x[:, 2]).astype(np.float32)
    p0 = mg.mlp_init(64, seed=2)
    p, losses = mg.mlp_train(ctx, x, t, p0, 64, epochs=30, batch=512, lr=3e-3, seed=1)
    assert losses[-1] < 0.05 * losses[0]
    assert np.mean((mg.mlp_forward(ctx, x, p, 64) - t) ** 2) < 1e-2


def test_fa_learned_mode_runs(ctx, oracle):
    """a network that reproduces the plain multiplier gives a converging run"""
    dims = [8, 8, 8, 8]
    U64 = fixed_problem(oracle, 3, dims)
    U = mg.GaugeField(ctx, 3, mg.F64, mg.Grid(dims)).import_(U64)
    fa = mg.LandauFA(U)
    # fit log m = log(0.07 p2max/p2) = log 0.07 - f0  (f0 = log p2 - log p2max)
    rng = np.random.default_rng(0)
    x = np.stack([rng.uniform(-4.5, 0, 8000), rng.uniform(-1, 1, 8000), rng.uniform(-2, 1.5, 8000)], 1)
    t = np.log(0.07) - x[:, 0]
    p, _ = mg.mlp_train(ctx, x.astype(np.float32), t.astype(np.float32), mg.mlp_init(64, 3), 64, epochs=40,
                        batch=256, lr=3e-3)
    fa.set_mlp(p, 64, beta=6.0, bf16=True)
    gt = mg.Lattice(ctx, 3, mg.F64, mg.Grid(dims)).set_unit()
    it, fb, th = fa.run(gt, tol=1e-12, max_iter=500)
    assert th < 1e-12
