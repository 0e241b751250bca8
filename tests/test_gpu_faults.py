"""Numeric faults injected on the host: HMC trajectories given NaN momenta,
links with a NaN entry, or links so far from unitary that the products
overflow, end with MESH_ERR_NUMERIC (the reference has no such check: its
Metropolis test `rng.uniform() < exp(-deltaH)` rejects a NaN dH silently,
src/gauge/hmc.cpp:92-99). The trajectory is rejected (the links are left as
they were), the history records it with accept 0, and with good inputs the
chain goes on. Every fault is in the inputs prepared on the host; no device
code is made to fail."""
import numpy as np
import pytest

import mesh_gb300 as mg

pytestmark = pytest.mark.gpu

MESH_ERR_NUMERIC = 5
DIMS = [4, 4, 4, 8]
BETA = 5.7


def chain(ctx, p):
    h = mg.Hmc(ctx, 3, p, mg.Grid(DIMS), seed=3)
    h.cold_start()
    h.run(BETA, mg.make_deltas("2lf", 0.5, 4), 2, use_graph=False)
    return h


@pytest.mark.parametrize("p", [1, 2])
def test_nan_momenta_reject_the_trajectory(ctx, oracle, p):
    d = mg.make_deltas("2lf", 0.5, 4)
    h = chain(ctx, p)
    U0 = h.U.export()
    n0 = h.count
    P = oracle.random_momenta(3, p, DIMS, 9, 0).astype(mg.real_dtype(p))
    P[1, 17, :] = np.nan
    P0 = mg.Momenta(ctx, 3, p, mg.Grid(DIMS)).import_(P)
    with pytest.raises(mg.MeshError) as e:
        h.update_supplied(P0, 0.5, BETA, d)
    assert e.value.code == MESH_ERR_NUMERIC
    np.testing.assert_array_equal(h.U.export(), U0)
    hist = h.history()
    assert h.count == n0 + 1 and hist["accept_history"][-1] == 0.0
    # good momenta: the chain goes on
    rec = h.update(BETA, d)
    assert np.isfinite(rec["dH"]) and np.isfinite(rec["plaquette"])
    h.close()


@pytest.mark.parametrize("p", [1, 2])
@pytest.mark.parametrize("fault", ["nan", "overflow"])
def test_bad_links_reject_the_trajectory(ctx, p, fault):
    d = mg.make_deltas("2lf", 0.5, 4)
    h = chain(ctx, p)
    U = h.U.export()
    if fault == "nan":
        U[2, 5, 4] = np.nan
    else:
        # far from unitary: FP32 products of 1e30 overflow, FP64 of 1e200
        U[0, 9, :] *= 1e30 if p == 1 else 1e200
    h.U.import_(U)
    with pytest.raises(mg.MeshError) as e:
        h.update(BETA, d)
    assert e.value.code == MESH_ERR_NUMERIC
    np.testing.assert_array_equal(h.U.export(), U)
    assert h.history()["accept_history"][-1] == 0.0
    # the same through the host-buffer entry point
    host = np.ascontiguousarray(U)
    with pytest.raises(mg.MeshError) as e:
        h.run_host(host, BETA, d, 1)
    assert e.value.code == MESH_ERR_NUMERIC
    np.testing.assert_array_equal(host, U)
    # good links again: the chain goes on
    h.cold_start()
    rec = h.update(BETA, d)
    assert np.isfinite(rec["dH"]) and rec["plaquette"] <= 1.0
    h.close()


def test_bounded_wait_expires_and_the_context_stays_usable(ctx):
    """a device-side wait on a flag that nothing sets gives up after its
    limit and reports MESH_ERR_TIMEOUT through the context's error word; the
    next launches on the same context run normally"""
    import time
    t0 = time.perf_counter()
    with pytest.raises(mg.MeshError) as e:
        ctx.wait_probe(0.05, flag_set=False)
    assert e.value.code == 4  # MESH_ERR_TIMEOUT
    assert time.perf_counter() - t0 < 5.0
    ctx.wait_probe(0.05, flag_set=True)  # the flag is set: no wait, no error
    ctx.synchronize()
    U = mg.GaugeField(ctx, 3, mg.F32, mg.Grid([4, 4, 4, 4])).set_unit()
    assert mg.plaquette(U) == pytest.approx(1.0)
