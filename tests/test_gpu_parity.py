"""GPU parity tests: the sm_103a kernels, called through the C ABI
(mesh_gb300 ctypes binding), against the CPU oracle on identical supplied
inputs.

Tolerances (written here, per the precision of the GPU path):
  * index and layout work (even/odd permutation, import/export, cshift):
    bit-exact;
  * plain FP64 path against the FP64 oracle: 1e-12 relative (the oracle is
    itself bit-exact against the reference's templates);
  * FP32 links/momenta against the FP64 oracle: 2e-5 relative on link-level
    quantities, 1e-6 on plaquettes (FP64 accumulation on the device).
"""
import ctypes
import ctypes.util
import os

import numpy as np
import pytest

import mesh_gb300 as mg

pytestmark = pytest.mark.gpu

TOL64 = 1e-12
TOL32 = 2e-5
BETA = {1: 1.0, 2: 2.3, 3: 5.7}
CASES = [(g, p) for g in (1, 2, 3) for p in (2, 1)]


def rel(a, b):
    a, b = np.asarray(a, dtype=np.float64), np.asarray(b, dtype=np.float64)
    return float(np.max(np.abs(a - b)) / max(1e-300, float(np.max(np.abs(b)))))


def tol(p):
    return TOL64 if p == 2 else TOL32


def gauge(ctx, g, p, dims, arr):
    return mg.GaugeField(ctx, g, p, mg.Grid(dims)).import_(arr)


def momenta(ctx, g, p, dims, arr):
    return mg.Momenta(ctx, g, p, mg.Grid(dims)).import_(arr)


def thermal(oracle, g, dims, seed=3, ntraj=3):
    """A partly thermalised FP64 configuration: a few trajectories of the
    oracle's chain from a cold start (plaquette well away from 0 and 1)."""
    U = oracle.unit_gauge(g, 2, dims)
    U, _ = oracle.hmc_chain(g, 2, dims, U, BETA[g], oracle.make_deltas("2lf", 0.5, 8), seed, 0, ntraj)
    return U


def _cudart():
    for name in ("libcudart.so", "libcudart.so.13", ctypes.util.find_library("cudart")):
        if not name:
            continue
        for base in ("", "/usr/local/cuda/lib64/"):
            try:
                return ctypes.CDLL(base + name)
            except OSError:
                pass
    pytest.skip("libcudart not found for raw device reads")


# ---------------------------------------------------------------------------
# layout
# ---------------------------------------------------------------------------
@pytest.mark.parametrize("dims", [[8, 8, 8, 8], [4, 6, 2, 8], [8, 8, 8], [6, 4]])
@pytest.mark.parametrize("g,p", CASES)
def test_import_export_roundtrip_bit_exact(ctx, g, p, dims):
    rng = np.random.default_rng(1)
    V, nd = int(np.prod(dims)), len(dims)
    dt = mg.real_dtype(p)
    host = rng.standard_normal((nd, V, mg.NREAL[g])).astype(dt)
    U = mg.GaugeField(ctx, g, p, mg.Grid(dims)).import_(host)
    np.testing.assert_array_equal(U.export(), host)
    # algebra: packed on the device, full antihermitian objects on the host
    import pyoracle

    packed = rng.standard_normal((nd, V, mg.NALG[g])).astype(dt)
    full = pyoracle.unpack_algebra(g, p, packed)
    P = mg.Momenta(ctx, g, p, mg.Grid(dims)).import_(full)
    np.testing.assert_array_equal(P.export(), full)


@pytest.mark.parametrize("dims", [[8, 8, 8, 8], [4, 6, 2, 8], [4, 4, 6]])
def test_even_odd_order_matches_oracle(ctx, oracle, dims):
    """site r lives at device index eo(r) = parity * V/2 + r // 2"""
    V = int(np.prod(dims))
    host = np.zeros((1, V, 2))
    host[0, :, 0] = np.arange(V)
    host[0, :, 1] = -np.arange(V)
    f = mg.Lattice(ctx, 1, 2, mg.Grid(dims)).import_(host[0])
    raw = np.zeros(2 * V)
    rt = _cudart()
    rt.cudaMemcpy.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t, ctypes.c_int]
    assert rt.cudaMemcpy(raw.ctypes.data_as(ctypes.c_void_p), ctypes.c_void_p(f.device_ptr), raw.nbytes, 2) == 0
    eo = oracle.eo_index(dims).astype(np.int64)
    got = np.empty(V, dtype=np.int64)
    got[eo] = np.arange(V)
    np.testing.assert_array_equal(raw[0::2][eo], np.arange(V, dtype=np.float64))
    assert sorted(eo.tolist()) == list(range(V))


# ---------------------------------------------------------------------------
# lattice layer
# ---------------------------------------------------------------------------
@pytest.mark.parametrize("g,p", CASES)
def test_cshift_mul_adj_sum_vs_oracle(ctx, oracle, g, p):
    dims = [4, 6, 4, 8]
    grid = mg.Grid(dims)
    dt = mg.real_dtype(p)
    U = oracle.random_gauge(g, p, dims, 5)
    a = mg.Lattice(ctx, g, p, grid).import_(U[0])
    b = mg.Lattice(ctx, g, p, grid).import_(U[1])
    out = mg.Lattice(ctx, g, p, grid)
    for d, off in ((0, 1), (1, -1), (3, 3), (2, -2), (3, -7)):
        mg.cshift(out, a, d, off)
        np.testing.assert_array_equal(out.export(), oracle.cshift(g, p, dims, U[0], d, off))
    mg.site_mul(out, a, b)
    assert rel(out.export(), oracle.site_mul(g, p, dims, U[0], U[1])) < (1e-15 if p == 2 else 1e-6)
    mg.site_adj(out, a)
    ref = mg.Lattice(ctx, g, p, grid).import_(U[0])
    mg.site_mul(out, ref, mg.site_adj(mg.Lattice(ctx, g, p, grid), a))
    assert mg.sum_real_trace(out) == pytest.approx(float(mg.NC[g]) * np.prod(dims), rel=1e-12 if p == 2 else 1e-5)
    assert mg.sum_real_trace(a) == pytest.approx(oracle.sum_real_trace(g, 2, dims, U[0].astype(np.float64)),
                                                 rel=1e-12 if p == 2 else 1e-5, abs=1e-9 if p == 2 else 1e-3)


# ---------------------------------------------------------------------------
# gauge kernels
# ---------------------------------------------------------------------------
@pytest.mark.parametrize("dims", [[8, 8, 8, 8], [4, 6, 2, 8], [8, 8, 8]])
@pytest.mark.parametrize("g,p", CASES)
def test_plaquette_action_vs_oracle(ctx, oracle, g, p, dims):
    U64 = thermal(oracle, g, dims)
    U = gauge(ctx, g, p, dims, U64.astype(mg.real_dtype(p)))
    ref = oracle.plaquette(g, 2, dims, U64)
    assert mg.plaquette(U) == pytest.approx(ref, rel=1e-13, abs=1e-15) if p == 2 else \
        mg.plaquette(U) == pytest.approx(ref, abs=1e-6)
    hot = oracle.random_gauge(g, p, dims, 8)
    U_hot = gauge(ctx, g, p, dims, hot)
    assert mg.plaquette(U_hot) == pytest.approx(oracle.plaquette(g, 2, dims, hot.astype(np.float64)),
                                                abs=1e-14 if p == 2 else 1e-6)
    S = oracle.wilson_action(g, 2, dims, U64, BETA[g])
    assert mg.wilson_action(U, BETA[g]) == pytest.approx(S, rel=1e-12 if p == 2 else 1e-5)
    cold = mg.GaugeField(ctx, g, p, mg.Grid(dims)).set_unit()
    assert mg.plaquette(cold) == 1.0 and mg.wilson_action(cold, 6.0) == 0.0


@pytest.mark.parametrize("g,p", CASES)
def test_staples_force_evolve_reunit_vs_oracle(ctx, oracle, g, p):
    dims = [4, 6, 4, 8]
    nd = 4
    grid = mg.Grid(dims)
    U64 = thermal(oracle, g, dims)
    P64 = oracle.random_momenta(g, 2, dims, 9, 0)
    dt = mg.real_dtype(p)
    U = gauge(ctx, g, p, dims, U64.astype(dt))
    S = mg.Lattice(ctx, g, p, grid)
    F = mg.Lattice(ctx, g, p, grid, algebra=True)
    for mu in range(nd):
        mg.staple_sum(S, U, mu)
        assert rel(S.export(), oracle.staple_sum(g, 2, dims, U64, mu)) < tol(p)
        mg.wilson_deriv(F, U, mu, BETA[g])
        assert rel(F.export(), oracle.wilson_deriv(g, 2, dims, U64, mu, BETA[g])) < tol(p)
    P = momenta(ctx, g, p, dims, P64.astype(dt))
    mg.evolve(U, P, 0.1)
    assert rel(U.export(), oracle.evolve(g, 2, dims, U64, P64, 0.1)) < tol(p)
    Uw = gauge(ctx, g, p, dims, (U64 * 1.0005).astype(dt))
    mg.reunitize(Uw)
    assert rel(Uw.export(), oracle.reunitize(g, 2, dims, U64 * 1.0005)) < tol(p)
    U = gauge(ctx, g, p, dims, U64.astype(dt))
    mg.momentum_step(P, U, BETA[g], 0.05)
    assert rel(P.export(), oracle.momentum_step(g, 2, dims, U64, P64, BETA[g], 0.05)) < tol(p)


@pytest.mark.parametrize("t", [0.01, 0.05, 0.2, 0.6, 2.0])
@pytest.mark.parametrize("g", [1, 2, 3])
def test_exp_fp32_series_and_closed_form(ctx, oracle, g, t):
    """FP32 link update exp(t P) U: small arguments by truncated series (SU(3):
    the power series reduced by Cayley-Hamilton for |t P| < 1; U(1), SU(2):
    the Taylor series of cos and sin(x)/x for |x| < 1/2), larger ones by the
    closed forms; against the FP64 oracle (groups.h exp; SU(3) Taylor with
    scaling and squaring)"""
    dims = [4, 4, 4, 8]
    U64 = thermal(oracle, g, dims)
    P64 = oracle.random_momenta(g, 2, dims, 9, 0)
    U = gauge(ctx, g, 1, dims, U64.astype(np.float32))
    P = momenta(ctx, g, 1, dims, P64.astype(np.float32))
    mg.evolve(U, P, t)
    assert rel(U.export(), oracle.evolve(g, 2, dims, U64, P64, t)) < TOL32


@pytest.mark.parametrize("variant", list(range(58)))
@pytest.mark.parametrize("g,p", [(3, 1), (3, 2), (2, 1), (1, 1)])
def test_every_force_launch_variant_vs_oracle(ctx, oracle, g, p, variant):
    """each launch variant the autotuner can choose (thread per link in
    even/odd order or 4D tiles, thread per site with shared plaquette loops,
    packed FP32x2 products) computes the same momentum step"""
    dims = [8, 8, 8, 16]
    U64 = thermal(oracle, g, dims, ntraj=1)
    P64 = oracle.random_momenta(g, 2, dims, 9, 0)
    dt = mg.real_dtype(p)
    U = gauge(ctx, g, p, dims, U64.astype(dt))
    P = momenta(ctx, g, p, dims, P64.astype(dt))
    try:
        mg.force_variant(variant)
        mg.momentum_step(P, U, BETA[g], 0.05)
    finally:
        mg.force_variant(-1)
    assert rel(P.export(), oracle.momentum_step(g, 2, dims, U64, P64, BETA[g], 0.05)) < tol(p)


@pytest.mark.parametrize("scheme", ["2lf", "2mn", "4mn"])
@pytest.mark.parametrize("g,p", CASES)
def test_run_hmd_vs_oracle(ctx, oracle, g, p, scheme):
    dims = [4, 4, 4, 8]
    U64 = thermal(oracle, g, dims)
    P64 = oracle.random_momenta(g, 2, dims, 9, 0)
    dt = mg.real_dtype(p)
    d = oracle.make_deltas(scheme, 0.5, 3)
    U = gauge(ctx, g, p, dims, U64.astype(dt))
    P = momenta(ctx, g, p, dims, P64.astype(dt))
    mg.run_hmd(U, P, BETA[g], d)
    Uo, Po = oracle.run_hmd(g, 2, dims, U64, P64, BETA[g], d)
    assert rel(U.export(), Uo) < (1e-12 if p == 2 else 1e-4)
    assert rel(P.export(), Po) < (1e-11 if p == 2 else 1e-4)


# ---------------------------------------------------------------------------
# HMC
# ---------------------------------------------------------------------------
@pytest.mark.parametrize("g", [1, 2, 3])
def test_hmc_update_fp64_matches_oracle_on_supplied_inputs(ctx, oracle, g):
    """runHmcUpdate on identical supplied links, momenta and uniform:
    H_old, H_new, dH, plaquette and the new links to 1e-12 relative."""
    dims = [8, 8, 8, 8]
    U64 = thermal(oracle, g, dims)
    d = oracle.make_deltas("2lf", 0.5, 10)
    h = mg.Hmc(ctx, g, 2, mg.Grid(dims), seed=1)
    for t in range(3):
        P64 = oracle.random_momenta(g, 2, dims, 100 + t, 0)
        u = 0.3
        h.U.import_(U64)
        P0 = momenta(ctx, g, 2, dims, P64)
        rec = h.update_supplied(P0, u, BETA[g], d)
        U64, ro = oracle.hmc_update(g, 2, dims, U64, P64, BETA[g], d, u)
        assert rec["H_old"] == pytest.approx(ro["H_old"], rel=TOL64)
        assert rec["H_new"] == pytest.approx(ro["H_new"], rel=TOL64)
        assert abs(rec["dH"] - ro["dH"]) <= TOL64 * abs(ro["H_old"])
        assert rec["accept"] == ro["accept"]
        assert rec["plaquette"] == pytest.approx(ro["plaq"], rel=TOL64)
        assert rel(h.U.export(), U64) < TOL64


def test_fp64_8x4_cold_chain_matches_oracle(ctx, oracle):
    """SU(3) 8^4, beta=5.7, cold start, 20 trajectories of 2lf n=10 (tau=1),
    momenta from seed 1234: plaquette, dH and accept per trajectory. Momenta
    and uniforms come from each side's own counter-based streams (same
    algorithm, transcendental rounding may differ by an ulp)."""
    dims = [8, 8, 8, 8]
    d = oracle.make_deltas("2lf", 0.5, 10)
    _, recs = oracle.hmc_chain(3, 2, dims, oracle.unit_gauge(3, 2, dims), 5.7, d, 1234, 0, 20)
    h = mg.Hmc(ctx, 3, 2, mg.Grid(dims), seed=1234)
    h.cold_start()
    got = [h.update(5.7, d) for _ in range(20)]
    np.testing.assert_array_equal([r["accept"] for r in got], recs[:, 2])
    np.testing.assert_allclose([r["plaquette"] for r in got], recs[:, 0], rtol=1e-10)
    np.testing.assert_allclose([r["dH"] for r in got], recs[:, 1], rtol=1e-6, atol=1e-7)
    hist = h.history()
    np.testing.assert_array_equal(hist["accept_history"], recs[:, 2])


@pytest.mark.parametrize("g,p", CASES)
def test_device_momenta_match_oracle_stream(ctx, oracle, g, p):
    dims = [4, 6, 4, 8]
    P = mg.Momenta(ctx, g, p, mg.Grid(dims)).random(77, 5)
    ref = oracle.random_momenta(g, p, dims, 77, 5)
    assert rel(P.export(), ref) < (1e-14 if p == 2 else 2e-6)
    U = mg.GaugeField(ctx, g, p, mg.Grid(dims)).random(78)
    ref = oracle.random_gauge(g, p, dims, 78)
    # FP32 Gram-Schmidt amplifies last-ulp differences of the transcendental
    # functions in Box-Muller (device sincospif/logf vs host libm)
    assert rel(U.export(), ref) < (1e-13 if p == 2 else 1e-4)


def test_graph_replay_equals_eager(ctx):
    dims = [8, 8, 8, 8]
    d = mg.make_deltas("2mn", 0.5, 4)
    out = []
    for use_graph in (False, True):
        h = mg.Hmc(ctx, 3, 1, mg.Grid(dims), seed=42)
        h.randomize_gauge_field()
        h.run(6.0, d, 4, use_graph=use_graph)
        out.append((h.history(), h.U.export()))
    for k in ("plaq_history", "deltaH_history", "accept_history"):
        np.testing.assert_array_equal(out[0][0][k], out[1][0][k])
    np.testing.assert_array_equal(out[0][1], out[1][1])


def test_run_host_roundtrip(ctx, oracle):
    dims = [8, 8, 8, 8]
    d = mg.make_deltas("2lf", 0.5, 10)
    host = np.ascontiguousarray(oracle.unit_gauge(3, 1, dims))
    h = mg.Hmc(ctx, 3, 1, mg.Grid(dims), seed=5)
    rec = h.run_host(host, 5.7, d, count=2)
    assert 0.5 < rec["plaquette"] < 1.0
    assert rel(host, h.U.export()) == 0.0


@pytest.mark.parametrize("dims", [[4, 6, 4, 8], [4, 6, 2, 6]])
@pytest.mark.parametrize("g,p", CASES)
def test_pinned_host_transfers_match_staged(ctx, oracle, monkeypatch, g, p, dims):
    """gauge fields and momenta through pinned host buffers (converted by the
    kernels that read and write the mapped host memory directly, 256 objects
    per block; V = 768 and V = 288, a partial last block) equal the path
    through a staging copy, bit for bit, and so do pinned buffers sent through
    the staging copy (MESH_HOST_PATH=staged)"""
    torch = pytest.importorskip("torch")
    dt = mg.real_dtype(p)
    tdt = torch.float64 if p == 2 else torch.float32
    U64 = thermal(oracle, g, dims)
    P64 = oracle.random_momenta(g, 2, dims, 9, 0)
    for arr, ctor in ((U64, mg.GaugeField), (P64, mg.Momenta)):
        host = arr.astype(dt)
        pin = torch.empty(host.shape, dtype=tdt, pin_memory=True)
        pin.numpy()[...] = host
        F = ctor(ctx, g, p, mg.Grid(dims)).import_(pin.numpy())
        Fs = ctor(ctx, g, p, mg.Grid(dims)).import_(host)  # pageable: staged
        staged = Fs.export()
        assert np.array_equal(F.export(), staged)
        out = torch.zeros(host.shape, dtype=tdt, pin_memory=True)
        Fs.export(out.numpy())
        assert np.array_equal(out.numpy(), staged)
        if ctor is mg.GaugeField:
            assert np.array_equal(staged, host)
        monkeypatch.setenv("MESH_HOST_PATH", "staged")
        Fp = ctor(ctx, g, p, mg.Grid(dims)).import_(pin.numpy())
        out2 = torch.zeros(host.shape, dtype=tdt, pin_memory=True)
        Fp.export(out2.numpy())
        monkeypatch.delenv("MESH_HOST_PATH")
        assert np.array_equal(out2.numpy(), staged)


@pytest.mark.parametrize("variant", [-1, 11, 13, 14, 15, 16, 17, 18, 20, 21, 22, 23, 25, 29, 30, 31, 32, 33, 34, 35, 36, 37, 38, 39, 40, 41, 42, 43, 44, 45, 46, 47, 48, 49, 50, 51, 52, 53, 54, 55, 56, 57])
@pytest.mark.parametrize("g", [2, 3])
def test_trajectory_momentum_step_matches_generic(ctx, oracle, g, variant):
    """the trajectory's momentum step (SU(3) FP32 links read as rows 0, 1 with
    row 2 rebuilt), in every launch variant, against the generic one and the
    FP64 oracle"""
    dims = [8, 8, 8, 8]
    U64 = thermal(oracle, g, dims)
    P64 = oracle.random_momenta(g, 2, dims, 5, 0)
    h = mg.Hmc(ctx, g, 1, mg.Grid(dims), seed=1)
    h.U.import_(U64.astype(np.float32))
    h.P.import_(P64.astype(np.float32))
    try:
        mg.force_variant(variant)
        h.momentum_step(BETA[g], 0.1)
    finally:
        mg.force_variant(-1)
    P_ref = momenta(ctx, g, 1, dims, P64.astype(np.float32))
    mg.momentum_step(P_ref, h.U, BETA[g], 0.1)
    assert rel(h.P.export(), P_ref.export()) < 2e-6
    assert rel(h.P.export(), oracle.momentum_step(g, 2, dims, U64, P64, BETA[g], 0.1)) < TOL32


@pytest.mark.parametrize("g,p", [(3, 1), (2, 1), (1, 1), (3, 2)])
def test_md_step_vs_oracle(ctx, oracle, g, p):
    """the momentum step fused with the link update after it (FP32: one
    thread-per-site kernel; FP64: the two kernels) against the oracle's
    momentum step followed by evolve"""
    dims = [8, 8, 8, 16]
    U64 = thermal(oracle, g, dims)
    P64 = oracle.random_momenta(g, 2, dims, 5, 0)
    dt = mg.real_dtype(p)
    h = mg.Hmc(ctx, g, p, mg.Grid(dims), seed=1)
    h.U.import_(U64.astype(dt))
    h.P.import_(P64.astype(dt))
    h.md_step(BETA[g], 0.1, 0.07)
    P_o = oracle.momentum_step(g, 2, dims, U64, P64, BETA[g], 0.1)
    U_o = oracle.evolve(g, 2, dims, U64, P_o, 0.07)
    assert rel(h.P.export(), P_o) < tol(p)
    assert rel(h.U.export(), U_o) < tol(p)
    # a second step from the swapped buffers
    h.md_step(BETA[g], 0.1, 0.07)
    P_o = oracle.momentum_step(g, 2, dims, U_o, P_o, BETA[g], 0.1)
    U_o = oracle.evolve(g, 2, dims, U_o, P_o, 0.07)
    assert rel(h.P.export(), P_o) < 2 * tol(p)
    assert rel(h.U.export(), U_o) < 2 * tol(p)


MD_VARIANTS = [(3, v) for v in (-1, 14, 15, 16, 17, 18, 19, 20, 21, 22, 23, 24, 25, 26, 27, 28, 29, 30, 31, 32, 33, 34, 35, 36, 37, 38, 39, 40, 41, 42, 43, 44, 45, 46, 47, 48, 49, 50, 51, 52, 53, 54, 55, 56, 57)] + [(g, v) for g in (1, 2) for v in (-1, 18, 20)]


@pytest.mark.parametrize("g,variant", MD_VARIANTS)
def test_mixed_precision_error_vs_fp64(ctx, oracle, g, variant):
    """FP32 links/momenta/force with FP64 sums against the FP64 oracle on the
    same supplied inputs: plaquette and dH errors. On this lattice every
    momentum step of the trajectory runs fused with the link update after it
    (thread-per-site kernel, each launch variant pinned in turn)."""
    dims = [8, 8, 8, 8]
    U64 = thermal(oracle, g, dims, ntraj=4)
    P64 = oracle.random_momenta(g, 2, dims, 11, 0)
    d = oracle.make_deltas("2mn", 0.5, 5)
    U_new, ro = oracle.hmc_update(g, 2, dims, U64, P64, BETA[g], d, 0.5)
    h = mg.Hmc(ctx, g, 1, mg.Grid(dims), seed=1)
    h.U.import_(U64.astype(np.float32))
    try:
        mg.force_variant(variant)
        rec = h.update_supplied(momenta(ctx, g, 1, dims, P64.astype(np.float32)), 0.5, BETA[g], d)
    finally:
        mg.force_variant(-1)
    assert abs(rec["dH"] - ro["dH"]) < 0.05
    assert rec["plaquette"] == pytest.approx(ro["plaq"], abs=1e-5)
    # the trajectory reads SU(3) FP32 links as rows 0, 1 and rebuilds row 2:
    # the links after it still agree with the FP64 oracle at the FP32 level
    assert rec["accept"] == ro["accept"]
    assert rel(h.U.export(), U_new) < 2e-5


# ---------------------------------------------------------------------------
# Landau
# ---------------------------------------------------------------------------
@pytest.mark.parametrize("g,p", CASES)
def test_landau_pieces_vs_oracle(ctx, oracle, g, p):
    dims = [4, 6, 4, 8]
    grid = mg.Grid(dims)
    dt = mg.real_dtype(p)
    U64 = thermal(oracle, g, dims)
    h64 = oracle.random_transform(g, 2, dims, 5)
    U = gauge(ctx, g, p, dims, U64.astype(dt))
    L = mg.Landau(U)
    L.g.import_(h64.astype(dt))
    t = 1e-12 if p == 2 else 1e-5
    assert L() == pytest.approx(oracle.landau_functional(g, 2, dims, U64, h64), rel=t)
    assert L.condition() == pytest.approx(oracle.landau_condition(g, 2, dims, U64, h64), rel=t * 10)
    assert rel(L.deriv().export(), oracle.landau_deriv(g, 2, dims, U64, h64)) < (1e-12 if p == 2 else 1e-4)
    if p == 2:
        L.overrelax(1.7, tol=0.0, max_sweeps=3, check_every=3)
        ref = oracle.landau_or_sweeps(g, 2, dims, U64, h64, 1.7, 3)
        assert rel(L.g.export(), ref) < 1e-11


@pytest.mark.parametrize("g", [1, 2, 3])
def test_landau_or_converges_fp64(ctx, oracle, g):
    dims = [8, 8, 8, 8]
    U64 = thermal(oracle, g, dims, ntraj=5)
    U = gauge(ctx, g, 2, dims, U64)
    L = mg.Landau(U)
    f0 = L()
    sweeps, theta = L.overrelax(1.7, tol=1e-12, max_sweeps=20000, check_every=10)
    assert theta < 1e-12 and L() > f0
    go, so, to = oracle.landau_or(g, 2, dims, U64, oracle.unit_transform(g, 2, dims), 1.7, 1e-12, 20000, 10)
    assert abs(sweeps - so) <= 20
    assert L() == pytest.approx(oracle.landau_theta(g, 2, dims, U64, go)[1], rel=1e-9)


@pytest.mark.parametrize("g", [1, 3])
def test_landau_cg_matches_oracle(ctx, oracle, g):
    dims = [4, 4, 4, 8]
    U64 = thermal(oracle, g, dims)
    U = gauge(ctx, g, 2, dims, U64)
    L = mg.Landau(U)
    it, th = L.run(8, tol=1e-30)
    go, ito, tho, _ = oracle.landau_cg(g, 2, dims, U64, oracle.unit_transform(g, 2, dims), 8, 1e-30)
    assert it == ito
    assert th == pytest.approx(tho, rel=1e-6)
    assert rel(L.g.export(), go) < 1e-9


def test_errors_are_status_codes(ctx):
    a = mg.GaugeField(ctx, 3, 2, mg.Grid([4, 4, 4, 4]))
    b = mg.GaugeField(ctx, 3, 2, mg.Grid([4, 4, 4, 6]))
    with pytest.raises(mg.MeshError) as e:
        a.copy_from(b)
    assert e.value.code == 3
    with pytest.raises(mg.MeshError) as e:
        mg.GaugeField(ctx, 3, 2, mg.Grid([4, 4, 4, 5]))
    assert e.value.code == 1
    with pytest.raises(mg.MeshError):
        mg.run_hmd(a, mg.Momenta(ctx, 3, 2, mg.Grid([4, 4, 4, 4])), 6.0, [0.1, 0.1])


# ---------------------------------------------------------------------------
# Wilson loops (legacy src/old/mesh/wilson.cpp:40-75)
# ---------------------------------------------------------------------------
@pytest.mark.parametrize("g,p", CASES)
def test_wilson_loops_vs_oracle(ctx, oracle, g, p):
    """W(r, t) for r = 1..4, t = 1..6 on an asymmetric lattice (lines that
    wrap around the spatial extents included) against the oracle, which walks
    every loop link by link"""
    dims = [4, 6, 4, 6]
    U64 = thermal(oracle, g, dims)
    U = gauge(ctx, g, p, dims, U64.astype(mg.real_dtype(p)))
    W = mg.wilson_loops(U, 4, 6)
    Wo = oracle.wilson_loops(g, 2, dims, U64, 4, 6)
    assert np.max(np.abs(W - Wo)) < (1e-13 if p == 2 else 2e-6)
    assert mg.wilson_loops(U, 1, 1)[0, 0] == pytest.approx(W[0, 0], abs=1e-15 if p == 2 else 1e-7)


def test_wilson_loops_argument_errors(ctx):
    U = mg.GaugeField(ctx, 3, 1, mg.Grid([4, 4, 4, 4]))
    for r, t in ((0, 1), (5, 1), (1, 0), (1, 5)):
        with pytest.raises(mg.MeshError):
            mg.wilson_loops(U, r, t)


# ---------------------------------------------------------------------------
# heat-bath and overrelaxation (legacy src/old/wilson.cpp:15-60,
# src/old/mesh/gauge_action.h:42-73)
# ---------------------------------------------------------------------------
@pytest.mark.parametrize("g", [1, 2, 3])
def test_heatbath_and_overrelaxation_fp64_vs_oracle(ctx, oracle, g):
    """FP64 heat-bath sweeps (same Philox streams, same checkerboard order)
    and an overrelaxation sweep against the oracle; the overrelaxation sweep
    keeps the action"""
    dims = [4, 4, 4, 6]
    U64 = thermal(oracle, g, dims)
    U = gauge(ctx, g, 2, dims, U64)
    for k in range(2):
        mg.heatbath_sweep(U, BETA[g], 21, k)
        U64 = oracle.gauge_sweep(g, 2, dims, U64, BETA[g], 21, k)
    assert rel(U.export(), U64) < 1e-12
    p0 = mg.plaquette(U)
    mg.overrelax_sweep(U)
    U64 = oracle.gauge_sweep(g, 2, dims, U64, BETA[g], 0, 0, overrelax=True)
    assert rel(U.export(), U64) < 1e-12
    assert abs(mg.plaquette(U) - p0) < 1e-13


@pytest.mark.parametrize("g", [1, 2, 3])
def test_overrelaxation_keeps_action_fp32(ctx, oracle, g):
    dims = [8, 8, 8, 8]
    U = gauge(ctx, g, 1, dims, thermal(oracle, g, dims).astype(np.float32))
    p0 = mg.plaquette(U)
    mg.overrelax_sweep(U)
    assert abs(mg.plaquette(U) - p0) < 2e-6


def test_heatbath_equilibrium_matches_hmc(ctx):
    """SU(3) 8^4 beta = 5.7, FP32: the equilibrium plaquette of heat-bath +
    overrelaxation sweeps and of HMC trajectories agree within their
    statistical errors (two Markov chains with the same distribution)"""
    dims = [8, 8, 8, 8]
    U = mg.GaugeField(ctx, 3, 1, mg.Grid(dims)).set_unit()
    ph = []
    for k in range(160):
        mg.heatbath_sweep(U, 5.7, 3, k)
        for _ in range(3):
            mg.overrelax_sweep(U)
        if k >= 60:
            ph.append(mg.plaquette(U))
    # HMC from a hot start (from a cold start at this beta the first
    # trajectories have dH ~ +9 and are all rejected)
    h = mg.Hmc(ctx, 3, 1, mg.Grid(dims), seed=4)
    h.randomize_gauge_field()
    h.run(5.7, mg.make_deltas("2mn", 0.5, 10), 160, use_graph=True)
    pm = h.history()["plaq_history"][60:]
    assert h.history()["accept_history"][60:].mean() > 0.5
    ph, pm = np.array(ph), np.array(pm)
    # errors from blocks of 20 (autocorrelations)
    err = np.hypot(ph.reshape(5, 20).mean(1).std() / np.sqrt(5), pm.reshape(5, 20).mean(1).std() / np.sqrt(5))
    assert abs(ph.mean() - pm.mean()) < 4 * err + 1e-3, (ph.mean(), pm.mean(), err)
