"""mesh_plaquette_noalloc (no device allocation, static scratch) against
mesh_plaquette, through the C ABI, on two calls in a row each, with the
tolerance of the plaquette tests (FP64 accumulation: 1e-13 relative).

The file name sorts last so that pytest collects it after every other test:
it must pass both there and alone in a fresh process, where its first call
does the per-device set-up."""
import ctypes as C

import pytest

import mesh_gb300 as mg

pytestmark = pytest.mark.gpu

MESH_OK, MESH_ERR_ARG = 0, 1  # include/mesh_gb300.h status codes


def noalloc(L, group, prec, dims, links, stream=None):
    d = (C.c_int32 * len(dims))(*dims)
    out = C.c_double()
    rc = L.mesh_plaquette_noalloc(0, group, prec, len(dims), d, links, stream, C.byref(out))
    return rc, out.value


@pytest.mark.parametrize("group,prec,dims", [(3, mg.F32, [8, 8, 8, 16]), (3, mg.F64, [8, 8, 8, 8]),
                                             (2, mg.F64, [6, 4, 8]), (2, mg.F32, [32, 32, 32, 32]),
                                             (1, mg.F32, [16, 32])])
def test_noalloc_plaquette_matches_plaquette(ctx, group, prec, dims):
    L = mg.load()
    U = mg.GaugeField(ctx, group, prec, mg.Grid(dims)).random(seed=11)
    links = U.device_ptr
    for state in ("hot", "cold"):
        if state == "cold":
            U.set_unit()
        ref = mg.plaquette(U)
        for _ in range(2):
            rc, got = noalloc(L, group, prec, dims, links)
            assert rc == MESH_OK, L.mesh_last_error()
            assert got == pytest.approx(ref, rel=1e-13, abs=1e-15)
    assert ref == 1.0


def test_noalloc_plaquette_argument_errors(ctx):
    L = mg.load()
    U = mg.GaugeField(ctx, 3, mg.F32, mg.Grid([4, 4, 4, 4])).set_unit()
    links = U.device_ptr
    assert noalloc(L, 3, mg.F32, [4, 4, 4, 5], links)[0] == MESH_ERR_ARG
    assert noalloc(L, 4, mg.F32, [4, 4, 4, 4], links)[0] == MESH_ERR_ARG
    assert noalloc(L, 3, mg.F32, [4, 4, 4, 4], None)[0] == MESH_ERR_ARG
    d = (C.c_int32 * 4)(4, 4, 4, 4)
    assert L.mesh_plaquette_noalloc(-1, 3, mg.F32, 4, d, links, None, None) == MESH_ERR_ARG
    # a host buffer where device memory is required: refused before any launch
    import numpy as np

    host = np.ones(4 * 256 * 18, dtype=np.float32)
    assert noalloc(L, 3, mg.F32, [4, 4, 4, 4], host.ctypes.data_as(C.c_void_p))[0] == MESH_ERR_ARG
    assert b"host memory" in L.mesh_last_error() or b"not a pointer" in L.mesh_last_error()
    # a valid call after the refused ones
    rc, got = noalloc(L, 3, mg.F32, [4, 4, 4, 4], links)
    assert rc == MESH_OK and got == 1.0
