"""TEST INFRASTRUCTURE — NOT PART OF THE PRODUCT.

ctypes wrapper of oracle/_ref/libref.so: the reference's own src/lattice and
src/gauge templates (plus src/gauge/hmc.cpp) compiled in place against the
project-written util stand-ins in oracle/ref_shim. Used only by the tests that
pin the restated oracle, and only where the reference tree is present
(``available()``); the library is never committed.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_ref", "libref.so")
# the reference's src/ directory, given by the environment (the build recipe
# sets it where the reference tree is present); unset: nothing is built here
REF_SRC = os.environ.get("MESH_REF_SRC", "")

_lib = None


def available() -> bool:
    return os.path.exists(LIB_PATH) or bool(REF_SRC and os.path.isdir(REF_SRC))


def build():
    if not (REF_SRC and os.path.isdir(REF_SRC)):
        raise RuntimeError("MESH_REF_SRC does not name the reference's src/ directory")
    out = subprocess.run(["make", "-C", HERE, "ref", f"REF_SRC={REF_SRC}"], capture_output=True, text=True)
    if out.returncode != 0:
        raise RuntimeError("reference build failed:\n" + out.stdout + out.stderr)


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        L = C.CDLL(LIB_PATH)
        P, I, D = C.c_void_p, C.c_int, C.c_double
        IP, DP = C.POINTER(C.c_int), C.POINTER(C.c_double)
        sig = {
            "ref_last_error": (C.c_char_p, []),
            "ref_make_deltas": (I, [C.c_char_p, D, I, DP, I]),
            "ref_plaquette": (I, [I, I, I, IP, P, DP]),
            "ref_wilson_action": (I, [I, I, I, IP, P, D, DP]),
            "ref_staple_sum": (I, [I, I, I, IP, P, I, P]),
            "ref_wilson_deriv": (I, [I, I, I, IP, P, I, D, P]),
            "ref_evolve": (I, [I, I, I, IP, P, P, D]),
            "ref_run_hmd": (I, [I, I, I, IP, P, P, D, DP, I]),
            "ref_reunitize": (I, [I, I, I, IP, P]),
            "ref_norm2": (I, [I, I, I, IP, P, DP]),
            "ref_cshift": (I, [I, I, I, IP, P, I, I, P]),
            "ref_random_algebra_field": (I, [I, I, I, IP, DP, C.c_size_t, P]),
            "ref_hmc_update": (I, [I, I, I, IP, P, DP, C.c_size_t, D, D, DP, I, DP]),
            "ref_landau_eval": (I, [I, I, I, IP, P, P, DP, DP, P]),
            "ref_landau_line_search": (I, [I, I, I, IP, P, P, P, D, DP]),
            "ref_landau_run": (I, [I, I, I, IP, P, P, I]),
        }
        for name, (res, args) in sig.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def _chk(rc):
    if rc != 0:
        raise RuntimeError("reference: " + lib().ref_last_error().decode())


def _dims(dims):
    return len(dims), (C.c_int * len(dims))(*dims)


def _p(a):
    assert a.flags["C_CONTIGUOUS"]
    return a.ctypes.data_as(C.c_void_p)


def _dp(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def make_deltas(scheme, eps, substeps):
    buf = (C.c_double * 4096)()
    n = lib().ref_make_deltas(scheme.encode(), eps, substeps, buf, 4096)
    if n < 0:
        raise RuntimeError(lib().ref_last_error().decode())
    return np.array(buf[:n])


def plaquette(grp, prec, dims, U):
    nd, d = _dims(dims)
    o = C.c_double()
    _chk(lib().ref_plaquette(grp, prec, nd, d, _p(U), C.byref(o)))
    return o.value


def wilson_action(grp, prec, dims, U, beta):
    nd, d = _dims(dims)
    o = C.c_double()
    _chk(lib().ref_wilson_action(grp, prec, nd, d, _p(U), beta, C.byref(o)))
    return o.value


def staple_sum(grp, prec, dims, U, mu):
    nd, d = _dims(dims)
    S = np.zeros(U.shape[1:], dtype=U.dtype)
    _chk(lib().ref_staple_sum(grp, prec, nd, d, _p(U), mu, _p(S)))
    return S


def wilson_deriv(grp, prec, dims, U, mu, beta):
    nd, d = _dims(dims)
    F = np.zeros(U.shape[1:], dtype=U.dtype)
    _chk(lib().ref_wilson_deriv(grp, prec, nd, d, _p(U), mu, beta, _p(F)))
    return F


def evolve(grp, prec, dims, U, P, t):
    nd, d = _dims(dims)
    U = np.ascontiguousarray(U.copy())
    _chk(lib().ref_evolve(grp, prec, nd, d, _p(U), _p(np.ascontiguousarray(P)), t))
    return U


def run_hmd(grp, prec, dims, U, P, beta, deltas):
    nd, d = _dims(dims)
    U = np.ascontiguousarray(U.copy())
    P = np.ascontiguousarray(P.copy())
    dl = np.ascontiguousarray(deltas, dtype=np.float64)
    _chk(lib().ref_run_hmd(grp, prec, nd, d, _p(U), _p(P), beta, _dp(dl), len(dl)))
    return U, P


def reunitize(grp, prec, dims, U):
    nd, d = _dims(dims)
    U = np.ascontiguousarray(U.copy())
    _chk(lib().ref_reunitize(grp, prec, nd, d, _p(U)))
    return U


def norm2(grp, prec, dims, P):
    nd, d = _dims(dims)
    o = C.c_double()
    _chk(lib().ref_norm2(grp, prec, nd, d, _p(np.ascontiguousarray(P)), C.byref(o)))
    return o.value


def cshift(grp, prec, dims, a, dir, off):
    nd, d = _dims(dims)
    out = np.zeros_like(a)
    _chk(lib().ref_cshift(grp, prec, nd, d, _p(np.ascontiguousarray(a)), dir, off, _p(out)))
    return out


def random_algebra_field(grp, prec, dims, normals, nreal):
    nd, d = _dims(dims)
    V = int(np.prod(dims))
    P = np.zeros((nd, V, nreal), dtype=np.float32 if prec == 1 else np.float64)
    nrm = np.ascontiguousarray(normals, dtype=np.float64)
    _chk(lib().ref_random_algebra_field(grp, prec, nd, d, _dp(nrm), nrm.size, _p(P)))
    return P


def hmc_update(grp, prec, dims, U, normals, uniform, beta, deltas):
    nd, d = _dims(dims)
    U = np.ascontiguousarray(U.copy())
    nrm = np.ascontiguousarray(normals, dtype=np.float64)
    dl = np.ascontiguousarray(deltas, dtype=np.float64)
    rec = np.zeros(3)
    _chk(lib().ref_hmc_update(grp, prec, nd, d, _p(U), _dp(nrm), nrm.size, uniform, beta, _dp(dl), len(dl),
                              _dp(rec)))
    return U, dict(plaq=rec[0], dH=rec[1], accept=rec[2])


def landau_eval(group, prec, dims, U, g):
    """the reference's Landau<G> on (U, g): (functional, condition, deriv)"""
    nd, d = _dims(dims)
    f, c = C.c_double(), C.c_double()
    g = np.ascontiguousarray(g)
    F = np.zeros_like(g)
    _chk(lib().ref_landau_eval(group, prec, nd, d, _p(np.ascontiguousarray(U)), _p(g), C.byref(f), C.byref(c), _p(F)))
    return f.value, c.value, F


def landau_line_search(group, prec, dims, U, g, F, eps):
    nd, d = _dims(dims)
    out = C.c_double()
    g = np.ascontiguousarray(g)
    _chk(lib().ref_landau_line_search(group, prec, nd, d, _p(np.ascontiguousarray(U)), _p(g), _p(np.ascontiguousarray(F)), eps, C.byref(out)))
    return out.value


def landau_run(group, prec, dims, U, g, max_iter):
    """the reference's Landau<G>::run(max_iter) from g; returns the new g"""
    nd, d = _dims(dims)
    g = np.ascontiguousarray(g.copy())
    _chk(lib().ref_landau_run(group, prec, nd, d, _p(np.ascontiguousarray(U)), _p(g), max_iter))
    return g

