"""GPU parity of the line-march MD kernel (k_md_line) on every lattice shape
class it takes, and parity at the headline configuration (SU(3) 32^4,
beta = 6.0, 2mn eps = 0.5 n = 20) with the launch the autotuner picks there.

Tolerances: FP32 links/momenta/force against the FP64 oracle on the same
supplied inputs, 2e-5 relative at link level for one MD step; after a whole
trajectory (40 momentum steps) 5e-5 relative on the links, 1e-6 absolute on
the plaquette, |dH(FP32) - dH(FP64)| < 0.1 on the 6.3e6 sites-by-planes of
the lattice; FP64: 1e-12 relative.
"""
import numpy as np
import pytest

import mesh_gb300 as mg

pytestmark = pytest.mark.gpu

LINE_VARIANTS = (29, 30, 31, 32, 33, 34, 37)


def rel(a, b):
    a, b = np.asarray(a, dtype=np.float64), np.asarray(b, dtype=np.float64)
    return float(np.max(np.abs(a - b)) / max(1e-300, float(np.max(np.abs(b)))))


def pinned(variant, fn):
    try:
        mg.force_variant(variant)
        return fn()
    finally:
        mg.force_variant(-1)


@pytest.mark.parametrize("dims", [[4, 6, 4, 32], [6, 4, 8, 16], [4, 4, 4, 8], [16, 32, 16, 32]])
@pytest.mark.parametrize("p", [1, 2])
def test_line_md_step_vs_oracle(ctx, oracle, dims, p):
    """one fused MD step (momentum step + the link update after it) and one
    momentum step alone of the line-march kernel, every launch variant,
    against the oracle's momentum step followed by evolve. The shapes cover
    one, two and four lines per warp and, at 16x32x16x32, warps whose range
    of line steps crosses into the next column (the x1 carry recomputed)."""
    grid = mg.Grid(dims)
    dt = mg.real_dtype(p)
    beta, dp, du = 6.0, 0.05, 0.05
    U64 = oracle.random_gauge(3, 2, dims, 21)
    P64 = oracle.random_momenta(3, 2, dims, 22, 0)
    P_o = oracle.momentum_step(3, 2, dims, U64, P64, beta, dp)
    U_o = oracle.evolve(3, 2, dims, U64, P_o, du)
    tol = 2e-5 if p == 1 else 1e-12
    for v in (LINE_VARIANTS if p == 1 else LINE_VARIANTS[:1]):
        h = mg.Hmc(ctx, 3, p, grid, seed=1)
        h.U.import_(U64.astype(dt))
        h.P.import_(P64.astype(dt))
        pinned(v, lambda: h.md_step(beta, dp, du))
        assert rel(h.P.export(), P_o) < tol, v
        assert rel(h.U.export(), U_o) < tol, v
        h.close()
        # the momentum step alone (mesh_momentum_step through the variant)
        U = mg.GaugeField(ctx, 3, p, grid).import_(U64.astype(dt))
        P = mg.Momenta(ctx, 3, p, grid).import_(P64.astype(dt))
        pinned(v, lambda: mg.momentum_step(P, U, beta, dp))
        assert rel(P.export(), P_o) < tol, v


def test_headline_32x4_md_step_and_trajectory(ctx, oracle):
    """SU(3) 32^4 at beta = 6.0 with the autotuner's own launch choice: one
    fused MD step, then one whole mixed-precision trajectory (2mn, eps = 0.5,
    n = 20; uniform 0 so that both sides accept) on links from the GPU's own
    mixed chain (30 trajectories from a hot start, seed 7) and momenta from
    the oracle, against the FP64 oracle on the same inputs."""
    dims = [32, 32, 32, 32]
    grid = mg.Grid(dims)
    beta = 6.0
    d = oracle.make_deltas("2mn", 0.5, 20)
    hm = mg.Hmc(ctx, 3, mg.F32, grid, seed=7)
    hm.randomize_gauge_field()
    hm.run(beta, d, 30, use_graph=True)
    U32 = hm.U.export()
    hm.close()
    U64 = U32.astype(np.float64)
    P64 = oracle.random_momenta(3, 2, dims, 3, 0)
    P32 = P64.astype(np.float32)
    mg.force_variant(-1)

    # one fused MD step with the autotuned launch
    h = mg.Hmc(ctx, 3, mg.F32, grid, seed=1)
    h.U.import_(U32)
    h.P.import_(P32)
    dp, du = float(d[1]), float(d[2])
    h.md_step(beta, dp, du)
    report = mg.tune_report()
    assert "md_step/group3/f32/32x32x32x32" in report
    P_o = oracle.momentum_step(3, 2, dims, U64, P64, beta, dp)
    U_o = oracle.evolve(3, 2, dims, U64, P_o, du)
    err_p, err_u = rel(h.P.export(), P_o), rel(h.U.export(), U_o)
    print(f"32^4 md step ({[ln for ln in report.splitlines() if 'md_step/group3/f32/32x' in ln][0][:90]}): "
          f"P {err_p:.2e}, U {err_u:.2e}")
    assert err_p < 2e-5 and err_u < 2e-5
    h.close()

    # one whole trajectory
    h = mg.Hmc(ctx, 3, mg.F32, grid, seed=1)
    h.U.import_(U32)
    P0 = mg.Momenta(ctx, 3, mg.F32, grid).import_(P32)
    rec = h.update_supplied(P0, 0.0, beta, d)
    U_new, ro = oracle.hmc_update(3, 2, dims, U64, P64, beta, d, 0.0)
    err_u = rel(h.U.export(), U_new)
    ddh = abs(rec["dH"] - ro["dH"])
    print(f"32^4 trajectory: links {err_u:.2e}, plaquette {abs(rec['plaquette'] - ro['plaq']):.2e}, "
          f"dH {rec['dH']:.5f} (FP32) vs {ro['dH']:.5f} (FP64), |ddH| = {ddh:.2e}")
    assert rec["accept"] == ro["accept"] == 1
    assert err_u < 5e-5
    assert abs(rec["plaquette"] - ro["plaq"]) < 1e-6
    assert ddh < 0.1
    h.close()
