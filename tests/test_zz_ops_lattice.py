"""GPU tests of the generic lattice layer beyond the hot path's fused
kernels, through the C ABI: linear combinations (the reference's lattice +,
-, scalar * and add_mul), exp and project_on_algebra of a lattice, and the
Landau line search as its own entry point. Tolerances are written in each
test."""
import numpy as np
import pytest

import mesh_gb300 as mg
from test_gpu_parity import CASES, gauge, rel, thermal, tol

pytestmark = pytest.mark.gpu


def np_project_on_algebra(g, a):
    """project_on_algebra (groups.h:64-67,142-145,224-228) on host-layout
    objects: U(1) (re, im) -> (0, im); SU(2) quaternions (re, im1, im2, im3)
    -> (0, im1, im2, im3); SU(3) row-major complex 3x3 -> (A - A^+)/2 minus
    its trace part"""
    a = np.asarray(a, dtype=np.float64)
    r = a.copy()
    if g in (1, 2):
        r[..., 0] = 0.0
        return r
    m = (a[..., 0::2] + 1j * a[..., 1::2]).reshape(*a.shape[:-1], 3, 3)
    h = 0.5 * (m - np.conj(np.swapaxes(m, -1, -2)))
    h -= np.trace(h, axis1=-2, axis2=-1)[..., None, None] / 3.0 * np.eye(3)
    h = h.reshape(*a.shape[:-1], 9)
    r[..., 0::2], r[..., 1::2] = h.real, h.imag
    return r


@pytest.mark.parametrize("g,p", CASES)
def test_site_exp_and_project_vs_oracle(ctx, oracle, g, p):
    """exp of an algebra field (utils.h:32) against the oracle's evolve of
    unit links by t = 1, and project_on_algebra of a group field (utils.h:33)
    against its restatement on the host objects"""
    dims = [4, 6, 2, 4]
    grid = mg.Grid(dims)
    P = oracle.random_momenta(g, p, dims, 7, 0)
    U = oracle.random_gauge(g, p, dims, 8)
    a = mg.Lattice(ctx, g, p, grid, algebra=True).import_(P[0])
    e = mg.site_exp(mg.Lattice(ctx, g, p, grid), a)
    ref = oracle.evolve(g, 2, dims, oracle.unit_gauge(g, 2, dims), P.astype(np.float64), 1.0)[0]
    assert rel(e.export(), ref) < tol(p)
    u = mg.Lattice(ctx, g, p, grid).import_(U[0])
    pr = mg.site_project(mg.Lattice(ctx, g, p, grid, algebra=True), u)
    assert rel(pr.export(), np_project_on_algebra(g, U[0])) < (1e-14 if p == 2 else 1e-6)
    with pytest.raises(mg.MeshError):
        mg.site_exp(mg.Lattice(ctx, g, p, grid), u)


@pytest.mark.parametrize("algebra", [False, True])
@pytest.mark.parametrize("g,p", CASES)
def test_linear_combinations_vs_host(ctx, oracle, g, p, algebra):
    """out = a x + b y (mesh_field_axpby: the reference's lattice +, -,
    scalar * and add_mul, lattice.h:289-364) on gauge fields and momenta of
    every group: exported, it is the same combination of the exported
    operands (import and export are linear maps); also without y and in place
    (out = x). FP64 to 1e-14, FP32 to 1e-6 relative (a few roundings)."""
    dims = [4, 6, 2, 4]
    grid = mg.Grid(dims)
    if algebra:
        xh, yh = oracle.random_momenta(g, p, dims, 5, 0), oracle.random_momenta(g, p, dims, 6, 0)
        make = mg.Momenta
    else:
        xh, yh = oracle.random_gauge(g, p, dims, 5), oracle.random_gauge(g, p, dims, 6)
        make = mg.GaugeField
    x = make(ctx, g, p, grid).import_(xh)
    y = make(ctx, g, p, grid).import_(yh)
    out = make(ctx, g, p, grid)
    X, Y = xh.astype(np.float64), yh.astype(np.float64)
    t = 1e-14 if p == 2 else 1e-6
    mg.axpby(out, 0.75, x, -1.5, y)
    assert rel(out.export(), 0.75 * X - 1.5 * Y) < t
    mg.axpby(out, 2.0, x)
    assert rel(out.export(), 2.0 * X) < t
    mg.axpby(x, 1.0, x, 0.5, y)
    assert rel(x.export(), X + 0.5 * Y) < t
    with pytest.raises(mg.MeshError):
        mg.axpby(out, 1.0, mg.Lattice(ctx, g, p, grid), 1.0, y)


@pytest.mark.parametrize("g", [1, 3])
def test_landau_line_search_is_the_cg_step(ctx, oracle, g):
    """Landau::line_search (landau.h:77-98) through its own entry point: the
    first CG iteration from g = 1 is g <- reunit(exp(s F) g) with F = deriv()
    and s = line_search(F, 3000)"""
    dims = [4, 4, 4, 8]
    grid = mg.Grid(dims)
    U64 = thermal(oracle, g, dims)
    U = gauge(ctx, g, 2, dims, U64)
    L = mg.Landau(U)
    F = L.deriv()
    s = L.line_search(F, 3000.0)
    assert s > 0
    # the step itself against the oracle's line search (pinned to the
    # reference's Landau<G>::line_search by the golden fixtures)
    g1 = oracle.unit_transform(g, 2, dims)
    s_o = oracle.landau_line_search(g, 2, dims, U64, g1, oracle.landau_deriv(g, 2, dims, U64, g1), 3000.0)
    assert s == pytest.approx(s_o, rel=1e-10)
    X = mg.axpby(mg.Lattice(ctx, g, 2, grid, algebra=True), s, F)
    h = mg.site_mul(mg.Lattice(ctx, g, 2, grid), mg.site_exp(mg.Lattice(ctx, g, 2, grid), X), L.g)
    mg.reunitize(h)
    f_h = L(h)
    L.run(1, tol=1e-30)
    assert rel(L.g.export(), h.export()) < 1e-12
    assert L() == pytest.approx(f_h, rel=1e-12)
