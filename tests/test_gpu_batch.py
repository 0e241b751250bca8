"""Batched replicas (mesh_batch_*) through the C ABI: every replica against
the FP64 oracle's chain with the replica's seed and beta (1e-12 relative, as
the single-chain parity tests), and against a single chain (mesh_hmc_*) with
the same seed in mixed precision: the same accept decisions, links to 1e-5
relative and plaquettes to 1e-6 (the FP32 per-link code of the two kernels
may be contracted differently by the compiler)."""
import numpy as np
import pytest

import mesh_gb300 as mg

pytestmark = pytest.mark.gpu

TOL64 = 1e-12


def rel(a, b):
    a, b = np.asarray(a, dtype=np.float64), np.asarray(b, dtype=np.float64)
    return float(np.max(np.abs(a - b)) / max(1e-300, float(np.max(np.abs(b)))))


DIMS = [[4, 4, 4, 8], [6, 4, 4, 4], [8, 4, 4, 4], [4, 4, 4, 4], [8, 8, 4, 6]]
SEEDS = [3, 7, 11, 5, 19]


@pytest.mark.parametrize("g,beta", [(1, [1.0, 1.1, 0.9, 1.2, 1.05]), (2, [2.2, 2.4, 2.6, 2.3, 2.5]),
                                    (3, [5.7, 5.9, 6.1, 5.8, 6.0])])
def test_batch_replicas_match_oracle_chains(ctx, oracle, g, beta):
    d = mg.make_deltas("2lf", 0.5, 8)
    b = mg.HmcBatch(ctx, g, mg.F64, DIMS, SEEDS)
    b.randomize_gauge_field()
    U0 = [b.export(r) for r in range(b.R)]
    ntraj = 4
    b.run(beta, d, 2, use_graph=False)
    b.run(beta, d, ntraj - 2, use_graph=True)
    assert b.count == ntraj
    for r, dims in enumerate(DIMS):
        # hot start: the single chain's randomize_gauge_field stream
        assert rel(U0[r], oracle.random_gauge(g, 2, dims, SEEDS[r])) < 1e-13
        U_ref, recs = oracle.hmc_chain(g, 2, dims, U0[r], beta[r], d, SEEDS[r], 0, ntraj)
        h = b.history(r)
        np.testing.assert_array_equal(h["accept_history"], recs[:, 2])
        np.testing.assert_allclose(h["plaq_history"], recs[:, 0], rtol=1e-10)
        np.testing.assert_allclose(h["deltaH_history"], recs[:, 1], rtol=1e-6, atol=1e-7)
        assert rel(b.export(r), U_ref) < TOL64
    pl = b.plaquettes()
    for r, dims in enumerate(DIMS):
        assert pl[r] == pytest.approx(oracle.plaquette(g, 2, dims, b.export(r)), rel=1e-13)


@pytest.mark.parametrize("g", [2, 3])
def test_batch_matches_single_chains_fp32(ctx, g):
    """mixed precision: each replica follows a single chain with its seed;
    the two builds of the same FP32 per-link code agree to the FP32 level
    (the compiler may contract the FP32 sums differently in the two kernels),
    and their FP64 records agree to that level too"""
    d = mg.make_deltas("2lf", 0.5, 16)
    beta = [2.25, 2.45, 2.35, 2.55, 2.4] if g == 2 else [5.8, 6.0, 5.9, 6.1, 6.2]
    b = mg.HmcBatch(ctx, g, mg.F32, DIMS, SEEDS)
    b.cold_start()
    b.run(beta, d, 5, use_graph=True)
    for r, dims in enumerate(DIMS):
        h = mg.Hmc(ctx, g, mg.F32, mg.Grid(dims), seed=SEEDS[r])
        h.cold_start()
        h.run(beta[r], d, 5, use_graph=True)
        hs, hb = h.history(), b.history(r)
        np.testing.assert_array_equal(hb["accept_history"], hs["accept_history"])
        np.testing.assert_allclose(hb["plaq_history"], hs["plaq_history"], rtol=1e-6)
        np.testing.assert_allclose(hb["deltaH_history"], hs["deltaH_history"], atol=2e-3)
        assert rel(b.export(r), h.U.export()) < 1e-5
        h.close()


@pytest.mark.parametrize("g", [1, 2])
@pytest.mark.parametrize("pin", ["sep", "0", "1", "2"])
def test_batch_md_launch_variants_match_single_chains(ctx, monkeypatch, g, pin):
    """every MD-step form of the FP32 small-group batch (separate kernels, and
    the fused kernel's launch variants: unrolled per-site body under 128 and
    80 registers, rolled body), pinned through MESH_BATCH_MD, against single
    chains with the same seeds"""
    monkeypatch.setenv("MESH_BATCH_MD", pin)
    d = mg.make_deltas("2lf", 0.5, 16)
    beta = [1.0, 1.1, 0.9, 1.2, 1.05] if g == 1 else [2.25, 2.45, 2.35, 2.55, 2.4]
    b = mg.HmcBatch(ctx, g, mg.F32, DIMS, SEEDS)
    b.cold_start()
    b.run(beta, d, 3, use_graph=True)
    ml = b.md_launch()
    assert ml["fused"] == (0 if pin == "sep" else 1)
    if pin != "sep":
        assert ml["variant"] == int(pin) and ml["min_blocks"] == {"0": 2, "1": 3, "2": 2}[pin]
        assert ml["grid"] > 0
    for r, dims in enumerate(DIMS):
        h = mg.Hmc(ctx, g, mg.F32, mg.Grid(dims), seed=SEEDS[r])
        h.cold_start()
        h.run(beta[r], d, 3, use_graph=True)
        hs, hb = h.history(), b.history(r)
        np.testing.assert_array_equal(hb["accept_history"], hs["accept_history"])
        np.testing.assert_allclose(hb["plaq_history"], hs["plaq_history"], rtol=1e-6)
        assert rel(b.export(r), h.U.export()) < 1e-5
        h.close()
    b.close()


def test_batch_graph_equals_eager_and_cold_start(ctx):
    d = mg.make_deltas("2lf", 0.5, 16)
    beta = [2.2, 2.6, 2.4, 2.3, 2.5]
    runs = []
    for graph in (False, True):
        b = mg.HmcBatch(ctx, 2, mg.F32, DIMS, SEEDS)
        b.cold_start()
        assert np.all(b.plaquettes() == 1.0)
        b.run(beta, d, 6, use_graph=graph)
        runs.append(([b.export(r) for r in range(b.R)], [b.history(r) for r in range(b.R)]))
        b.close()
    for r in range(len(DIMS)):
        np.testing.assert_array_equal(runs[0][0][r], runs[1][0][r])
        for k in ("plaq_history", "deltaH_history", "accept_history"):
            np.testing.assert_array_equal(runs[0][1][r][k], runs[1][1][r][k])


def test_batch_import_and_argument_errors(ctx, oracle):
    b = mg.HmcBatch(ctx, 2, mg.F64, DIMS[:2], SEEDS[:2])
    U = oracle.random_gauge(2, 2, DIMS[1], 99)
    b.import_(1, U)
    np.testing.assert_array_equal(b.export(1), U)
    assert b.plaquettes()[1] == pytest.approx(oracle.plaquette(2, 2, DIMS[1], U), rel=1e-13)
    with pytest.raises(mg.MeshError):
        mg.HmcBatch(ctx, 2, mg.F32, [[4, 4, 4, 5]], [1])
    with pytest.raises(ValueError):
        b.run([2.3], mg.make_deltas("2lf", 0.5, 4), 1)
    with pytest.raises(mg.MeshError):
        b.run([2.3, 2.4], mg.make_deltas("2lf", 0.5, 4)[:-1], 1)  # even-length step table
