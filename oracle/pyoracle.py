"""TEST INFRASTRUCTURE — NOT PART OF THE PRODUCT.

ctypes wrapper of the CPU oracle (oracle/liboracle.so, a C++ restatement of
krox/mesh's src/gauge and src/lattice hot path). Only tests/, the smoke check
and bench.py's CPU legs import this module, as the checker.

Arrays are numpy views of the reference's host layout: a gauge field is
``(nd, V, nreal)`` (one lexicographic array-of-structs block per direction,
src/lattice/lattice.h:159-192), a site field ``(V, nreal)``.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liboracle.so")

GROUPS = {"u1": 1, "su2": 2, "su3": 3}
NREAL = {1: 2, 2: 4, 3: 18}
NALG = {1: 1, 2: 3, 3: 8}
NC = {1: 1, 2: 2, 3: 3}
DIM = {1: 1, 2: 3, 3: 8}


def build(quiet: bool = True) -> str:
    """Compile liboracle.so with its Makefile (g++ -fopenmp)."""
    out = subprocess.run(["make", "-C", HERE], capture_output=True, text=True)
    if out.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + out.stdout + out.stderr)
    return LIB_PATH


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        L = C.CDLL(LIB_PATH)
        P, I, D, U64, U32 = C.c_void_p, C.c_int, C.c_double, C.c_uint64, C.c_uint32
        IP, DP = C.POINTER(C.c_int), C.POINTER(C.c_double)
        sig = {
            "oracle_last_error": (C.c_char_p, []),
            "oracle_set_threads": (I, [I]),
            "oracle_make_deltas": (I, [C.c_char_p, D, I, DP, I]),
            "oracle_plaquette": (I, [I, I, I, IP, P, DP]),
            "oracle_wilson_action": (I, [I, I, I, IP, P, D, DP]),
            "oracle_wilson_loops": (I, [I, I, I, IP, P, I, I, P]),
            "oracle_gauge_sweep": (I, [I, I, I, IP, P, D, U64, U64, I]),
            "oracle_staple_sum": (I, [I, I, I, IP, P, I, P]),
            "oracle_wilson_deriv": (I, [I, I, I, IP, P, I, D, P]),
            "oracle_evolve": (I, [I, I, I, IP, P, P, D]),
            "oracle_momentum_step": (I, [I, I, I, IP, P, P, D, D]),
            "oracle_run_hmd": (I, [I, I, I, IP, P, P, D, DP, I]),
            "oracle_reunitize": (I, [I, I, I, IP, P, I]),
            "oracle_norm2": (I, [I, I, I, IP, P, I, DP]),
            "oracle_sum_real_trace": (I, [I, I, I, IP, P, DP]),
            "oracle_hmc_update": (I, [I, I, I, IP, P, P, D, DP, I, D, DP]),
            "oracle_hmc_chain": (I, [I, I, I, IP, P, D, DP, I, U64, U64, I, DP]),
            "oracle_random_momenta": (I, [I, I, I, IP, U64, U64, P]),
            "oracle_random_gauge": (I, [I, I, I, IP, U64, P]),
            "oracle_random_transform": (I, [I, I, I, IP, U64, P]),
            "oracle_gauge_transform": (I, [I, I, I, IP, P, P]),
            "oracle_metropolis_uniform": (D, [U64, U64]),
            "oracle_philox": (None, [C.POINTER(U32), C.POINTER(U32), C.POINTER(U32)]),
            "oracle_normals": (I, [I, U64, U32, U32, U32, U64, I, P]),
            "oracle_eo_index": (I, [I, IP, C.POINTER(U64)]),
            "oracle_cshift": (I, [I, I, I, IP, P, I, I, P]),
            "oracle_site_mul": (I, [I, I, I, IP, P, P, P]),
            "oracle_pack_algebra": (I, [I, I, C.c_size_t, P, P]),
            "oracle_unpack_algebra": (I, [I, I, C.c_size_t, P, P]),
            "oracle_landau_functional": (I, [I, I, I, IP, P, P, DP]),
            "oracle_landau_condition": (I, [I, I, I, IP, P, P, DP]),
            "oracle_landau_deriv": (I, [I, I, I, IP, P, P, P]),
            "oracle_landau_cg": (I, [I, I, I, IP, P, P, I, D, IP, DP, IP]),
            "oracle_landau_line_search": (I, [I, I, I, IP, P, P, P, D, DP]),
            "oracle_landau_or_sweeps": (I, [I, I, I, IP, P, P, D, I]),
            "oracle_landau_or": (I, [I, I, I, IP, P, P, D, D, I, I, IP, DP]),
            "oracle_landau_theta": (I, [I, I, I, IP, P, P, DP, DP]),
            "oracle_landau_divergence": (I, [I, I, I, IP, P, P, P]),
            "oracle_fft": (I, [I, IP, I, DP, I]),
            "oracle_landau_fa_step": (I, [I, I, I, IP, P, P, DP, D]),
            "oracle_bench_md": (I, [I, I, I, IP, P, P, D, D, I, DP, DP, DP]),
            "oracle_mlp_forward": (I, [I, C.POINTER(C.c_float), C.POINTER(C.c_float), I, C.POINTER(C.c_float)]),
            "oracle_mlp_grad": (I, [I, C.POINTER(C.c_float), C.POINTER(C.c_float), C.POINTER(C.c_float), I, DP, DP]),
        }
        for name, (res, args) in sig.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def _chk(rc):
    if rc != 0:
        raise RuntimeError("oracle: " + lib().oracle_last_error().decode())


def _dims(dims):
    a = (C.c_int * len(dims))(*dims)
    return len(dims), a


def _ptr(a: np.ndarray):
    assert a.flags["C_CONTIGUOUS"]
    return a.ctypes.data_as(C.c_void_p)


def dtype(prec: int):
    return np.float32 if prec == 1 else np.float64


def volume(dims) -> int:
    v = 1
    for d in dims:
        v *= int(d)
    return v


def set_threads(n: int = 0) -> int:
    return lib().oracle_set_threads(n)


def make_deltas(scheme: str, eps: float, substeps: int):
    buf = (C.c_double * 4096)()
    n = lib().oracle_make_deltas(scheme.encode(), eps, substeps, buf, 4096)
    if n < 0:
        raise RuntimeError("oracle: " + lib().oracle_last_error().decode())
    return np.array(buf[:n])


def unit_gauge(group: int, prec: int, dims) -> np.ndarray:
    V = volume(dims)
    U = np.zeros((len(dims), V, NREAL[group]), dtype=dtype(prec))
    if group == 1 or group == 2:
        U[..., 0] = 1
    else:
        for i in range(3):
            U[..., 6 * i + 2 * i] = 1
    return U


def random_gauge(group, prec, dims, seed):
    nd, d = _dims(dims)
    U = np.zeros((nd, volume(dims), NREAL[group]), dtype=dtype(prec))
    _chk(lib().oracle_random_gauge(group, prec, nd, d, seed, _ptr(U)))
    return U


def random_momenta(group, prec, dims, seed, counter):
    nd, d = _dims(dims)
    P = np.zeros((nd, volume(dims), NREAL[group]), dtype=dtype(prec))
    _chk(lib().oracle_random_momenta(group, prec, nd, d, seed, counter, _ptr(P)))
    return P


def random_transform(group, prec, dims, seed):
    nd, d = _dims(dims)
    h = np.zeros((volume(dims), NREAL[group]), dtype=dtype(prec))
    _chk(lib().oracle_random_transform(group, prec, nd, d, seed, _ptr(h)))
    return h


def gauge_transform(group, prec, dims, U, h):
    nd, d = _dims(dims)
    U = np.ascontiguousarray(U.copy())
    _chk(lib().oracle_gauge_transform(group, prec, nd, d, _ptr(U), _ptr(np.ascontiguousarray(h))))
    return U


def plaquette(group, prec, dims, U):
    nd, d = _dims(dims)
    out = C.c_double()
    _chk(lib().oracle_plaquette(group, prec, nd, d, _ptr(np.ascontiguousarray(U)), C.byref(out)))
    return out.value


def gauge_sweep(group, prec, dims, U, beta, seed, counter, overrelax=False):
    """one heat-bath (or overrelaxation) sweep in checkerboard order; returns
    the new links"""
    nd, d = _dims(dims)
    U = np.ascontiguousarray(U.copy())
    _chk(lib().oracle_gauge_sweep(group, prec, nd, d, _ptr(U), beta, seed, counter, 1 if overrelax else 0))
    return U


def wilson_loops(group, prec, dims, U, R, T):
    """W(r, t), r = 1..R, t = 1..T: rectangular loops in the planes (mu, 3),
    ReTr / Nc averaged over sites and mu < 3 (array [R, T])"""
    nd, d = _dims(dims)
    out = np.zeros((R, T), dtype=np.float64)
    _chk(lib().oracle_wilson_loops(group, prec, nd, d, _ptr(np.ascontiguousarray(U)), R, T, _ptr(out)))
    return out


def wilson_action(group, prec, dims, U, beta):
    nd, d = _dims(dims)
    out = C.c_double()
    _chk(lib().oracle_wilson_action(group, prec, nd, d, _ptr(np.ascontiguousarray(U)), beta, C.byref(out)))
    return out.value


def staple_sum(group, prec, dims, U, mu):
    nd, d = _dims(dims)
    S = np.zeros((volume(dims), NREAL[group]), dtype=dtype(prec))
    _chk(lib().oracle_staple_sum(group, prec, nd, d, _ptr(np.ascontiguousarray(U)), mu, _ptr(S)))
    return S


def wilson_deriv(group, prec, dims, U, mu, beta):
    nd, d = _dims(dims)
    F = np.zeros((volume(dims), NREAL[group]), dtype=dtype(prec))
    _chk(lib().oracle_wilson_deriv(group, prec, nd, d, _ptr(np.ascontiguousarray(U)), mu, beta, _ptr(F)))
    return F


def evolve(group, prec, dims, U, P, t):
    nd, d = _dims(dims)
    U = np.ascontiguousarray(U.copy())
    _chk(lib().oracle_evolve(group, prec, nd, d, _ptr(U), _ptr(np.ascontiguousarray(P)), t))
    return U


def momentum_step(group, prec, dims, U, P, beta, delta):
    nd, d = _dims(dims)
    P = np.ascontiguousarray(P.copy())
    _chk(lib().oracle_momentum_step(group, prec, nd, d, _ptr(np.ascontiguousarray(U)), _ptr(P), beta, delta))
    return P


def run_hmd(group, prec, dims, U, P, beta, deltas):
    nd, d = _dims(dims)
    U = np.ascontiguousarray(U.copy())
    P = np.ascontiguousarray(P.copy())
    dl = np.ascontiguousarray(deltas, dtype=np.float64)
    _chk(lib().oracle_run_hmd(group, prec, nd, d, _ptr(U), _ptr(P), beta,
                              dl.ctypes.data_as(C.POINTER(C.c_double)), len(dl)))
    return U, P


def reunitize(group, prec, dims, U):
    nd, d = _dims(dims)
    U = np.ascontiguousarray(U.copy())
    n_stack = U.shape[0] if U.ndim == 3 else 1
    _chk(lib().oracle_reunitize(group, prec, nd, d, _ptr(U), n_stack))
    return U


def norm2(group, prec, dims, P):
    nd, d = _dims(dims)
    out = C.c_double()
    n_stack = P.shape[0] if P.ndim == 3 else 1
    _chk(lib().oracle_norm2(group, prec, nd, d, _ptr(np.ascontiguousarray(P)), n_stack, C.byref(out)))
    return out.value


def sum_real_trace(group, prec, dims, A):
    nd, d = _dims(dims)
    out = C.c_double()
    _chk(lib().oracle_sum_real_trace(group, prec, nd, d, _ptr(np.ascontiguousarray(A)), C.byref(out)))
    return out.value


def hmc_update(group, prec, dims, U, P, beta, deltas, uniform):
    """One trajectory of runHmcUpdate on supplied momenta/uniform.
    Returns (U_after, dict(plaq, dH, accept, H_old, H_new))."""
    nd, d = _dims(dims)
    U = np.ascontiguousarray(U.copy())
    dl = np.ascontiguousarray(deltas, dtype=np.float64)
    rec = (C.c_double * 5)()
    _chk(lib().oracle_hmc_update(group, prec, nd, d, _ptr(U), _ptr(np.ascontiguousarray(P)), beta,
                                 dl.ctypes.data_as(C.POINTER(C.c_double)), len(dl), uniform, rec))
    keys = ("plaq", "dH", "accept", "H_old", "H_new")
    return U, dict(zip(keys, list(rec)))


def hmc_chain(group, prec, dims, U, beta, deltas, seed, first, ntraj):
    nd, d = _dims(dims)
    U = np.ascontiguousarray(U.copy())
    dl = np.ascontiguousarray(deltas, dtype=np.float64)
    recs = np.zeros((ntraj, 5), dtype=np.float64)
    _chk(lib().oracle_hmc_chain(group, prec, nd, d, _ptr(U), beta, dl.ctypes.data_as(C.POINTER(C.c_double)),
                                len(dl), seed, first, ntraj, recs.ctypes.data_as(C.POINTER(C.c_double))))
    return U, recs


def metropolis_uniform(seed, traj):
    return lib().oracle_metropolis_uniform(seed, traj)


def philox(ctr, key):
    c = (C.c_uint32 * 4)(*ctr)
    k = (C.c_uint32 * 2)(*key)
    o = (C.c_uint32 * 4)()
    lib().oracle_philox(c, k, o)
    return list(o)


def normals(prec, seed, tag, site, mu, ctr, n):
    out = np.zeros(n, dtype=dtype(prec))
    _chk(lib().oracle_normals(prec, seed, tag, site, mu, ctr, n, _ptr(out)))
    return out


def eo_index(dims):
    nd, d = _dims(dims)
    perm = np.zeros(volume(dims), dtype=np.uint64)
    _chk(lib().oracle_eo_index(nd, d, perm.ctypes.data_as(C.POINTER(C.c_uint64))))
    return perm


def cshift(group, prec, dims, a, dir, off):
    nd, d = _dims(dims)
    out = np.zeros_like(a)
    _chk(lib().oracle_cshift(group, prec, nd, d, _ptr(np.ascontiguousarray(a)), dir, off, _ptr(out)))
    return out


def site_mul(group, prec, dims, a, b):
    nd, d = _dims(dims)
    out = np.zeros_like(a)
    _chk(lib().oracle_site_mul(group, prec, nd, d, _ptr(np.ascontiguousarray(a)),
                               _ptr(np.ascontiguousarray(b)), _ptr(out)))
    return out


def pack_algebra(group, prec, full):
    full = np.ascontiguousarray(full)
    n = full.size // NREAL[group]
    out = np.zeros(full.shape[:-1] + (NALG[group],), dtype=dtype(prec))
    _chk(lib().oracle_pack_algebra(group, prec, n, _ptr(full), _ptr(out)))
    return out


def unpack_algebra(group, prec, packed):
    packed = np.ascontiguousarray(packed)
    n = packed.size // NALG[group]
    out = np.zeros(packed.shape[:-1] + (NREAL[group],), dtype=dtype(prec))
    _chk(lib().oracle_unpack_algebra(group, prec, n, _ptr(packed), _ptr(out)))
    return out


def unit_transform(group, prec, dims):
    return unit_gauge(group, prec, dims)[0].copy()


def landau_functional(group, prec, dims, U, g):
    nd, d = _dims(dims)
    out = C.c_double()
    _chk(lib().oracle_landau_functional(group, prec, nd, d, _ptr(np.ascontiguousarray(U)),
                                        _ptr(np.ascontiguousarray(g)), C.byref(out)))
    return out.value


def landau_condition(group, prec, dims, U, g):
    nd, d = _dims(dims)
    out = C.c_double()
    _chk(lib().oracle_landau_condition(group, prec, nd, d, _ptr(np.ascontiguousarray(U)),
                                       _ptr(np.ascontiguousarray(g)), C.byref(out)))
    return out.value


def landau_deriv(group, prec, dims, U, g):
    nd, d = _dims(dims)
    F = np.zeros((volume(dims), NREAL[group]), dtype=dtype(prec))
    _chk(lib().oracle_landau_deriv(group, prec, nd, d, _ptr(np.ascontiguousarray(U)),
                                   _ptr(np.ascontiguousarray(g)), _ptr(F)))
    return F


def landau_line_search(group, prec, dims, U, g, F, eps):
    nd, d = _dims(dims)
    out = C.c_double()
    _chk(lib().oracle_landau_line_search(group, prec, nd, d, _ptr(np.ascontiguousarray(U)),
                                         _ptr(np.ascontiguousarray(g)), _ptr(np.ascontiguousarray(F)), eps,
                                         C.byref(out)))
    return out.value


def landau_cg(group, prec, dims, U, g, max_iter, tol):
    nd, d = _dims(dims)
    g = np.ascontiguousarray(g.copy())
    it, th, ne = C.c_int(), C.c_double(), C.c_int()
    _chk(lib().oracle_landau_cg(group, prec, nd, d, _ptr(np.ascontiguousarray(U)), _ptr(g), max_iter, tol,
                                C.byref(it), C.byref(th), C.byref(ne)))
    return g, it.value, th.value, ne.value


def landau_or_sweeps(group, prec, dims, U, g, omega, nsweeps):
    nd, d = _dims(dims)
    g = np.ascontiguousarray(g.copy())
    _chk(lib().oracle_landau_or_sweeps(group, prec, nd, d, _ptr(np.ascontiguousarray(U)), _ptr(g), omega,
                                       nsweeps))
    return g


def landau_or(group, prec, dims, U, g, omega, tol, max_sweeps, check_every):
    nd, d = _dims(dims)
    g = np.ascontiguousarray(g.copy())
    s, th = C.c_int(), C.c_double()
    _chk(lib().oracle_landau_or(group, prec, nd, d, _ptr(np.ascontiguousarray(U)), _ptr(g), omega, tol,
                                max_sweeps, check_every, C.byref(s), C.byref(th)))
    return g, s.value, th.value


def landau_theta(group, prec, dims, U, g):
    nd, d = _dims(dims)
    th, fn = C.c_double(), C.c_double()
    _chk(lib().oracle_landau_theta(group, prec, nd, d, _ptr(np.ascontiguousarray(U)),
                                   _ptr(np.ascontiguousarray(g)), C.byref(th), C.byref(fn)))
    return th.value, fn.value


def landau_divergence(group, prec, dims, U, g):
    nd, d = _dims(dims)
    D = np.zeros((volume(dims), NALG[group]), dtype=dtype(prec))
    _chk(lib().oracle_landau_divergence(group, prec, nd, d, _ptr(np.ascontiguousarray(U)),
                                        _ptr(np.ascontiguousarray(g)), _ptr(D)))
    return D


def fft(dims, data, sign):
    """data: complex128 array (V, ncomp); returns the unnormalised DFT."""
    nd, d = _dims(dims)
    a = np.ascontiguousarray(data.astype(np.complex128))
    ncomp = a.shape[1] if a.ndim == 2 else 1
    _chk(lib().oracle_fft(nd, d, ncomp, a.ctypes.data_as(C.POINTER(C.c_double)), sign))
    return a


def landau_fa_step(group, prec, dims, U, g, mult, alpha):
    nd, d = _dims(dims)
    g = np.ascontiguousarray(g.copy())
    m = np.ascontiguousarray(mult, dtype=np.float64)
    _chk(lib().oracle_landau_fa_step(group, prec, nd, d, _ptr(np.ascontiguousarray(U)), _ptr(g),
                                     m.ctypes.data_as(C.POINTER(C.c_double)), alpha))
    return g


def mlp_nparams(width):
    return 3 * width + width + width * width + width + width + 1


def mlp_forward(x, params, width):
    x = np.ascontiguousarray(x, dtype=np.float32)
    p = np.ascontiguousarray(params, dtype=np.float32)
    y = np.zeros(x.shape[0], dtype=np.float32)
    fp = C.POINTER(C.c_float)
    _chk(lib().oracle_mlp_forward(x.shape[0], x.ctypes.data_as(fp), p.ctypes.data_as(fp), width,
                                  y.ctypes.data_as(fp)))
    return y


def mlp_grad(x, t, params, width):
    x = np.ascontiguousarray(x, dtype=np.float32)
    t = np.ascontiguousarray(t, dtype=np.float32)
    p = np.ascontiguousarray(params, dtype=np.float32)
    g = np.zeros(mlp_nparams(width), dtype=np.float64)
    loss = C.c_double()
    fp = C.POINTER(C.c_float)
    _chk(lib().oracle_mlp_grad(x.shape[0], x.ctypes.data_as(fp), t.ctypes.data_as(fp), p.ctypes.data_as(fp),
                               width, C.byref(loss), g.ctypes.data_as(C.POINTER(C.c_double))))
    return loss.value, g


def bench_md(group, prec, dims, U, P, beta, delta, reps=1):
    """Seconds per momentum step, link update and plaquette of the restated
    reference algorithm on the host cores (best of reps)."""
    nd, d = _dims(dims)
    tf, te, tp = C.c_double(), C.c_double(), C.c_double()
    _chk(lib().oracle_bench_md(group, prec, nd, d, _ptr(np.ascontiguousarray(U)), _ptr(np.ascontiguousarray(P)),
                               beta, delta, reps, C.byref(tf), C.byref(te), C.byref(tp)))
    return tf.value, te.value, tp.value
