"""mesh_gb300 — GB300 (sm_103a) implementation of krox/mesh's lattice-gauge
hot path, behind a C ABI (include/mesh_gb300.h).

This package is the Python host side used by the tests and the benchmark: a
ctypes binding of libmesh_gb300.so with classes named after the reference's
C++ API (src/lattice/lattice.h, src/gauge/utils.h, hmc.h, landau.h):
``Grid``, ``Lattice``, ``GaugeField``, ``Hmc``, ``Landau``, ``make_deltas``,
``plaquette``, ``wilson_action``, ``staple_sum``, ``wilson_deriv``,
``reunitize``, ``evolve``, ``run_hmd``, ``cshift``.

Host arrays use the reference's host layout: a gauge field is a numpy array
``(nd, V, nreal)`` (sites lexicographic, dimension 0 slowest), a single
lattice ``(V, nreal)``; momenta/forces are full group-type objects on the host
(complex / quaternion / 3x3 complex matrix), packed algebra on the device.

There is no CPU fallback: if the CUDA library is missing or no GPU is present,
creating a ``Context`` raises.
"""
from __future__ import annotations

import ctypes as C
import math
import os
from dataclasses import dataclass

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libmesh_gb300.so")

U1, SU2, SU3 = 1, 2, 3
F32, F64 = 1, 2
GROUP, ALGEBRA = 0, 1
GROUP_NAMES = {"u1": U1, "su2": SU2, "su3": SU3}
NREAL = {U1: 2, SU2: 4, SU3: 18}
NALG = {U1: 1, SU2: 3, SU3: 8}
NC = {U1: 1, SU2: 2, SU3: 3}

STATUS = {
    0: "MESH_OK", 1: "MESH_ERR_ARG", 2: "MESH_ERR_CUDA", 3: "MESH_ERR_STATE", 4: "MESH_ERR_TIMEOUT",
    5: "MESH_ERR_NUMERIC", 6: "MESH_ERR_NOCONV", 7: "MESH_ERR_UNSUPPORTED",
}

# every symbol declared in include/mesh_gb300.h, with its ctypes signature
_P, _I, _D, _U64, _SZ = C.c_void_p, C.c_int, C.c_double, C.c_uint64, C.c_size_t
_IP, _DP, _I32P = C.POINTER(C.c_int), C.POINTER(C.c_double), C.POINTER(C.c_int32)
_PP = C.POINTER(C.c_void_p)


class HmcRecord(C.Structure):
    _fields_ = [("plaquette", C.c_double), ("dH", C.c_double), ("accept", C.c_double),
                ("H_old", C.c_double), ("H_new", C.c_double)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


SIGNATURES = {
    "mesh_last_error": (C.c_char_p, []),
    "mesh_version": (_I, []),
    "mesh_tune_report": (_SZ, [C.c_char_p, _SZ]),
    "mesh_tune_force_variant": (_I, [_I]),
    "mesh_ctx_create": (_I, [_I, _P, _PP]),
    "mesh_ctx_destroy": (_I, [_P]),
    "mesh_ctx_synchronize": (_I, [_P]),
    "mesh_ctx_stream": (_P, [_P]),
    "mesh_ctx_wait_probe": (_I, [_P, C.c_double, _I]),
    "mesh_field_create": (_I, [_P, _I, _I, _I, _I, _I32P, _I, _PP]),
    "mesh_field_destroy": (_I, [_P]),
    "mesh_field_info": (_I, [_P, _IP, _IP, _IP, _IP, _I32P, _IP]),
    "mesh_field_host_bytes": (_SZ, [_P]),
    "mesh_field_import": (_I, [_P, _P, _SZ]),
    "mesh_field_export": (_I, [_P, _P, _SZ]),
    "mesh_field_copy": (_I, [_P, _P]),
    "mesh_field_save": (_I, [_P, C.c_char_p]),
    "mesh_field_load": (_I, [_P, C.c_char_p]),
    "mesh_config_info": (_I, [C.c_char_p, _IP, _IP, _IP, _IP, _I32P, _IP, C.POINTER(C.c_uint64),
                              C.POINTER(C.c_uint64)]),
    "mesh_hmc_save": (_I, [_P, C.c_char_p]),
    "mesh_hmc_momentum_step": (_I, [_P, _D, _D]),
    "mesh_hmc_md_step": (_I, [_P, _D, _D, _D]),
    "mesh_hmc_load": (_I, [_P, C.c_char_p]),
    "mesh_field_set_zero": (_I, [_P]),
    "mesh_field_set_unit": (_I, [_P]),
    "mesh_field_random": (_I, [_P, _U64, _U64]),
    "mesh_field_device_ptr": (_P, [_P]),
    "mesh_site_cshift": (_I, [_P, _P, _I, _I]),
    "mesh_site_mul": (_I, [_P, _P, _P]),
    "mesh_site_adj": (_I, [_P, _P]),
    "mesh_field_axpby": (_I, [_P, _D, _P, _D, _P]),
    "mesh_site_exp": (_I, [_P, _P]),
    "mesh_site_project": (_I, [_P, _P]),
    "mesh_site_sum_real_trace": (_I, [_P, _DP]),
    "mesh_field_norm2": (_I, [_P, _DP]),
    "mesh_plaquette": (_I, [_P, _DP]),
    "mesh_wilson_action": (_I, [_P, _D, _DP]),
    "mesh_wilson_loops": (_I, [_P, _I, _I, _DP]),
    "mesh_heatbath_sweep": (_I, [_P, _D, C.c_uint64, C.c_uint64]),
    "mesh_overrelax_sweep": (_I, [_P]),
    "mesh_plaquette_noalloc": (_I, [_I, _I, _I, _I, _I32P, _P, _P, _DP]),
    "mesh_staple_sum": (_I, [_P, _P, _I]),
    "mesh_wilson_deriv": (_I, [_P, _P, _I, _D]),
    "mesh_reunitize": (_I, [_P]),
    "mesh_evolve": (_I, [_P, _P, _D]),
    "mesh_momentum_step": (_I, [_P, _P, _D, _D]),
    "mesh_run_hmd": (_I, [_P, _P, _D, _DP, _I]),
    "mesh_make_deltas": (_I, [C.c_char_p, _D, _I, _DP, _I, _IP]),
    "mesh_hmc_create": (_I, [_P, _I, _I, _I, _I32P, _U64, _PP]),
    "mesh_hmc_destroy": (_I, [_P]),
    "mesh_hmc_field": (_I, [_P, _I, _PP]),
    "mesh_hmc_randomize": (_I, [_P]),
    "mesh_hmc_cold_start": (_I, [_P]),
    "mesh_hmc_update": (_I, [_P, _D, _DP, _I, C.POINTER(HmcRecord)]),
    "mesh_hmc_update_supplied": (_I, [_P, _P, _D, _D, _DP, _I, C.POINTER(HmcRecord)]),
    "mesh_hmc_run": (_I, [_P, _D, _DP, _I, _I, _I]),
    "mesh_hmc_count": (_I, [_P, _IP]),
    "mesh_hmc_history": (_I, [_P, _I, _I, _DP, _DP, _DP]),
    "mesh_hmc_run_host": (_I, [_P, _P, _SZ, _D, _DP, _I, _I, C.POINTER(HmcRecord)]),
    "mesh_batch_create": (_I, [_P, _I, _I, _I, _I32P, C.POINTER(C.c_uint64), _PP]),
    "mesh_batch_destroy": (_I, [_P]),
    "mesh_batch_size": (_I, [_P, _IP]),
    "mesh_batch_randomize": (_I, [_P]),
    "mesh_batch_cold_start": (_I, [_P]),
    "mesh_batch_import": (_I, [_P, _I, _P, _SZ]),
    "mesh_batch_export": (_I, [_P, _I, _P, _SZ]),
    "mesh_batch_run": (_I, [_P, _DP, _DP, _I, _I, _I]),
    "mesh_batch_count": (_I, [_P, _IP]),
    "mesh_batch_history": (_I, [_P, _I, _I, _I, _DP, _DP, _DP]),
    "mesh_batch_plaquettes": (_I, [_P, _DP]),
    "mesh_batch_launch_info": (_I, [_P, _IP, _I, _IP, _IP]),
    "mesh_batch_md_launch": (_I, [_P, _IP, _IP, _IP, _IP]),
    "mesh_landau_functional": (_I, [_P, _P, _DP]),
    "mesh_landau_line_search": (_I, [_P, _P, _P, _D, _DP]),
    "mesh_landau_theta": (_I, [_P, _P, _DP]),
    "mesh_landau_deriv": (_I, [_P, _P, _P]),
    "mesh_landau_cg": (_I, [_P, _P, _I, _D, _IP, _DP]),
    "mesh_landau_or": (_I, [_P, _P, _D, _D, _I, _I, _IP, _DP]),
    "mesh_gauge_transform": (_I, [_P, _P]),
    "mesh_landau_fa_create": (_I, [_P, _PP]),
    "mesh_landau_fa_destroy": (_I, [_P]),
    "mesh_landau_fa_set_plain": (_I, [_P, _D]),
    "mesh_landau_fa_set_table": (_I, [_P, C.POINTER(C.c_float), _I, _D, _D]),
    "mesh_landau_fa_set_mlp": (_I, [_P, C.POINTER(C.c_float), _I, _D, _I]),
    "mesh_landau_fa_p2range": (_I, [_P, _DP, _DP]),
    "mesh_landau_fa_theta": (_I, [_P, _P, _DP]),
    "mesh_landau_fa_step": (_I, [_P, _P, _DP]),
    "mesh_landau_fa_run": (_I, [_P, _P, _D, _I, _D, _I, _IP, _IP, _DP]),
    "mesh_landau_fa_set_accept": (_I, [_P, _I]),
    "mesh_landau_fa_probe": (_I, [_P, _P, _D, _I, _DP, _DP, _DP, _DP, _DP]),
    "mesh_landau_fa_trial": (_I, [_P, _P, _D, _DP, _DP]),
    "mesh_lattice_fft": (_I, [_P, _I, _I32P, _I, C.POINTER(C.c_float), _I]),
    "mesh_mlp_nparams": (_I, [_I]),
    "mesh_mlp_forward": (_I, [_P, _I, C.POINTER(C.c_float), C.POINTER(C.c_float), _I, _I, C.POINTER(C.c_float)]),
    "mesh_mlp_grad": (_I, [_P, _I, C.POINTER(C.c_float), C.POINTER(C.c_float), C.POINTER(C.c_float), _I, _DP,
                           C.POINTER(C.c_float)]),
    "mesh_mlp_train": (_I, [_P, _I, C.POINTER(C.c_float), C.POINTER(C.c_float), C.POINTER(C.c_float), _I, _I, _I,
                            C.c_float, _U64, C.POINTER(C.c_float)]),
}

_lib = None


class MeshError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"{STATUS.get(code, code)}: {msg}")
        self.code = code


def tune_report() -> str:
    """Launch variants chosen by the autotuner so far (one line per key)."""
    L = load()
    n = L.mesh_tune_report(None, 0)
    buf = C.create_string_buffer(n)
    L.mesh_tune_report(buf, n)
    return buf.value.decode()


def force_variant(v: int) -> None:
    """Force launch variant v of the momentum-step kernel (-1: autotune)."""
    _chk(load().mesh_tune_force_variant(v))


def lib_path() -> str:
    return LIB_PATH


def load(build_if_missing: bool = False):
    """Load libmesh_gb300.so (in-tree). Raises if it is missing."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        if not build_if_missing:
            raise RuntimeError(f"{LIB_PATH} is missing: build it with `python -m mesh_gb300.build`")
        from . import build as _b
        _b.build()
    L = C.CDLL(LIB_PATH)
    for name, (res, args) in SIGNATURES.items():
        f = getattr(L, name)
        f.restype = res
        f.argtypes = args
    _lib = L
    return L


def _chk(rc):
    if rc != 0:
        raise MeshError(rc, load().mesh_last_error().decode())


def _dims(shape):
    return (C.c_int32 * len(shape))(*[int(x) for x in shape])


def _darr(x):
    a = np.ascontiguousarray(np.asarray(x, dtype=np.float64))
    return a, a.ctypes.data_as(_DP)


def group_code(g) -> int:
    return GROUP_NAMES[g] if isinstance(g, str) else int(g)


def real_dtype(prec):
    return np.float32 if prec == F32 else np.float64


# ---------------------------------------------------------------------------
class Context:
    """Device + stream + reduction scratch (mesh_ctx)."""

    def __init__(self, device: int = 0, stream: int | None = None):
        L = load()
        h = C.c_void_p()
        _chk(L.mesh_ctx_create(device, C.c_void_p(stream) if stream else None, C.byref(h)))
        self.h = h
        self.device = device

    @property
    def stream(self) -> int:
        return load().mesh_ctx_stream(self.h) or 0

    def synchronize(self):
        _chk(load().mesh_ctx_synchronize(self.h))

    def wait_probe(self, seconds: float, flag_set: bool) -> None:
        """a device-side wait bounded at `seconds` on a flag set before the
        launch (flag_set) or never: raises MeshError(MESH_ERR_TIMEOUT) when
        the wait expired"""
        _chk(load().mesh_ctx_wait_probe(self.h, float(seconds), 1 if flag_set else 0))

    def close(self):
        if getattr(self, "h", None):
            load().mesh_ctx_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


@dataclass(frozen=True)
class Grid:
    """Lattice shape, lexicographic with dimension 0 slowest (grid.h:11-58)."""
    shape: tuple

    def __init__(self, shape):
        object.__setattr__(self, "shape", tuple(int(x) for x in shape))

    @property
    def ndim(self):
        return len(self.shape)

    @property
    def size(self):
        return int(np.prod(self.shape))


class Field:
    """A device field: nstack components of V group or algebra objects."""

    def __init__(self, ctx: Context, kind: int, group, prec: int, grid: Grid, nstack: int):
        self.ctx, self.kind, self.group, self.prec = ctx, kind, group_code(group), prec
        self.grid, self.nstack = grid, nstack
        h = C.c_void_p()
        _chk(load().mesh_field_create(ctx.h, kind, self.group, prec, grid.ndim, _dims(grid.shape), nstack,
                                      C.byref(h)))
        self.h = h

    def _host_shape(self):
        return (self.nstack, self.grid.size, NREAL[self.group])

    def import_(self, arr):
        a = np.ascontiguousarray(np.asarray(arr, dtype=real_dtype(self.prec)))
        assert a.size == int(np.prod(self._host_shape())), "host array size does not match the field"
        _chk(load().mesh_field_import(self.h, a.ctypes.data_as(C.c_void_p), a.nbytes))
        return self

    def export(self, out=None):
        """the field in the reference's host layout; into `out` (a contiguous
        array of the host shape, e.g. a view of pinned memory) when given"""
        if out is None:
            a = np.zeros(self._host_shape(), dtype=real_dtype(self.prec))
        else:
            a = out
            assert a.flags["C_CONTIGUOUS"] and a.dtype == real_dtype(self.prec)
            assert a.size == int(np.prod(self._host_shape())), "host array size does not match the field"
        _chk(load().mesh_field_export(self.h, a.ctypes.data_as(C.c_void_p), a.nbytes))
        if out is not None:
            return out
        return a if self.nstack > 1 else a[0]

    def copy_from(self, other: "Field"):
        _chk(load().mesh_field_copy(self.h, other.h))
        return self

    def save(self, path: str):
        """writeToFile (lattice.h:205-252): the host-layout dataset behind a
        self-describing header"""
        _chk(load().mesh_field_save(self.h, os.fsencode(path)))
        return self

    def load(self, path: str):
        """readFromFile; refuses files of another group, precision or grid"""
        _chk(load().mesh_field_load(self.h, os.fsencode(path)))
        return self

    def set_zero(self):
        _chk(load().mesh_field_set_zero(self.h))
        return self

    def set_unit(self):
        _chk(load().mesh_field_set_unit(self.h))
        return self

    def random(self, seed: int, counter: int = 0):
        _chk(load().mesh_field_random(self.h, seed, counter))
        return self

    def norm2(self) -> float:
        out = C.c_double()
        _chk(load().mesh_field_norm2(self.h, C.byref(out)))
        return out.value

    @property
    def device_ptr(self) -> int:
        return load().mesh_field_device_ptr(self.h) or 0

    def close(self):
        if getattr(self, "h", None):
            load().mesh_field_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def GaugeField(ctx, group, prec, grid) -> Field:
    """GaugeField<G> = LatticeStack<G> (utils.h:21): nd link components."""
    return Field(ctx, GROUP, group, prec, grid, grid.ndim)


def Momenta(ctx, group, prec, grid) -> Field:
    """Conjugate momenta: nd algebra components."""
    return Field(ctx, ALGEBRA, group, prec, grid, grid.ndim)


def config_info(path: str) -> dict:
    """header of a configuration file"""
    kind, group, prec, nd, nstack = (C.c_int() for _ in range(5))
    dims = (C.c_int32 * 4)()
    traj, seed = C.c_uint64(), C.c_uint64()
    _chk(load().mesh_config_info(os.fsencode(path), C.byref(kind), C.byref(group), C.byref(prec), C.byref(nd), dims,
                                 C.byref(nstack), C.byref(traj), C.byref(seed)))
    return {"kind": kind.value, "group": group.value, "precision": prec.value, "dims": list(dims[:nd.value]),
            "nstack": nstack.value, "trajectory": traj.value, "seed": seed.value}


def read_config(ctx, path: str, expected_grid: "Grid | None" = None) -> Field:
    """readConfig (utils.h:188-219): a new field with the file's grid and
    group; refuses a file on another grid than `expected_grid`"""
    info = config_info(path)
    grid = Grid(info["dims"])
    if expected_grid is not None and expected_grid != grid:
        raise MeshError(3, f"grid mismatch on load. Expected {expected_grid.shape}, got {grid.shape}")
    f = Field(ctx, info["kind"], info["group"], info["precision"], grid, info["nstack"])
    return f.load(path)


def Lattice(ctx, group, prec, grid, algebra: bool = False) -> Field:
    """Lattice<G> (lattice.h:23-143): one object per site."""
    return Field(ctx, ALGEBRA if algebra else GROUP, group, prec, grid, 1)


# ---- lattice layer ----------------------------------------------------------
def cshift(dst: Field, src: Field, dir: int, offset: int) -> Field:
    _chk(load().mesh_site_cshift(dst.h, src.h, dir, offset))
    return dst


def site_mul(dst: Field, a: Field, b: Field) -> Field:
    _chk(load().mesh_site_mul(dst.h, a.h, b.h))
    return dst


def axpby(out: Field, a: float, x: Field, b: float = 0.0, y: Field = None) -> Field:
    """out = a x + b y object by object (y optional; out may be x or y)"""
    _chk(load().mesh_field_axpby(out.h, a, x.h, b, y.h if y is not None else None))
    return out


def site_exp(dst: Field, a: Field) -> Field:
    """dst (group) = exp(a) for an algebra field a"""
    _chk(load().mesh_site_exp(dst.h, a.h))
    return dst


def site_project(dst: Field, a: Field) -> Field:
    """dst (algebra) = project_on_algebra(a) for a group-type field a"""
    _chk(load().mesh_site_project(dst.h, a.h))
    return dst


def site_adj(dst: Field, a: Field) -> Field:
    _chk(load().mesh_site_adj(dst.h, a.h))
    return dst


def sum_real_trace(a: Field) -> float:
    out = C.c_double()
    _chk(load().mesh_site_sum_real_trace(a.h, C.byref(out)))
    return out.value


def norm2(a: Field) -> float:
    return a.norm2()


# ---- gauge ------------------------------------------------------------------
def plaquette(U: Field) -> float:
    out = C.c_double()
    _chk(load().mesh_plaquette(U.h, C.byref(out)))
    return out.value


def wilson_action(U: Field, beta: float) -> float:
    out = C.c_double()
    _chk(load().mesh_wilson_action(U.h, beta, C.byref(out)))
    return out.value


def heatbath_sweep(U: Field, beta: float, seed: int, sweep: int) -> Field:
    """one heat-bath sweep of the Wilson action (checkerboard order; the
    random numbers are addressed by seed and sweep number)"""
    _chk(load().mesh_heatbath_sweep(U.h, beta, seed, sweep))
    return U


def overrelax_sweep(U: Field) -> Field:
    """one overrelaxation sweep (keeps the action)"""
    _chk(load().mesh_overrelax_sweep(U.h))
    return U


def wilson_loops(U: Field, max_r: int, max_t: int) -> np.ndarray:
    """Rectangular Wilson loops W(r, t) (r = 1..max_r spatial, t = 1..max_t
    in direction 3), ReTr / Nc averaged over sites and the three spatial
    directions: array [max_r, max_t]"""
    out = np.zeros((max_r, max_t), dtype=np.float64)
    _chk(load().mesh_wilson_loops(U.h, max_r, max_t, out.ctypes.data_as(_DP)))
    return out


def staple_sum(S: Field, U: Field, mu: int) -> Field:
    _chk(load().mesh_staple_sum(S.h, U.h, mu))
    return S


def wilson_deriv(F: Field, U: Field, mu: int, beta: float) -> Field:
    _chk(load().mesh_wilson_deriv(F.h, U.h, mu, beta))
    return F


def reunitize(U: Field) -> Field:
    _chk(load().mesh_reunitize(U.h))
    return U


def evolve(U: Field, P: Field, t: float) -> Field:
    _chk(load().mesh_evolve(U.h, P.h, t))
    return U


def momentum_step(P: Field, U: Field, beta: float, delta: float) -> Field:
    _chk(load().mesh_momentum_step(P.h, U.h, beta, delta))
    return P


def run_hmd(U: Field, P: Field, beta: float, deltas) -> None:
    a, p = _darr(deltas)
    _chk(load().mesh_run_hmd(U.h, P.h, beta, p, len(a)))


def make_deltas(scheme: str, epsilon: float, substeps: int) -> np.ndarray:
    n = C.c_int()
    cap = 8 * substeps + 16
    buf = (C.c_double * cap)()
    _chk(load().mesh_make_deltas(scheme.encode(), epsilon, substeps, buf, cap, C.byref(n)))
    return np.array(buf[: n.value])


def gauge_transform(U: Field, g: Field) -> Field:
    _chk(load().mesh_gauge_transform(U.h, g.h))
    return U


# ---- HMC --------------------------------------------------------------------
class Hmc:
    """Hmc<G> (hmc.h:66-115): U, P, proposal, histories; momenta and the
    Metropolis uniform from counter-based device streams keyed by `seed`."""

    def __init__(self, ctx: Context, group, prec: int, grid: Grid, seed: int):
        self.ctx, self.group, self.prec, self.grid = ctx, group_code(group), prec, grid
        h = C.c_void_p()
        _chk(load().mesh_hmc_create(ctx.h, self.group, prec, grid.ndim, _dims(grid.shape), seed, C.byref(h)))
        self.h = h
        self._U = self._borrow(0)
        self._P = self._borrow(1)

    def _borrow(self, which):
        out = C.c_void_p()
        _chk(load().mesh_hmc_field(self.h, which, C.byref(out)))
        f = Field.__new__(Field)
        f.ctx, f.kind, f.group, f.prec, f.grid = self.ctx, GROUP if which == 0 else ALGEBRA, self.group, self.prec, \
            self.grid
        f.nstack = self.grid.ndim
        f.h = out
        f.close = lambda: None  # borrowed: owned by the chain
        return f

    @property
    def U(self) -> Field:
        # writes through the handle invalidate the cached action
        _chk(load().mesh_hmc_field(self.h, 0, C.byref(C.c_void_p())))
        return self._U

    @property
    def P(self) -> Field:
        return self._P

    def randomize_gauge_field(self):
        _chk(load().mesh_hmc_randomize(self.h))

    def cold_start(self):
        _chk(load().mesh_hmc_cold_start(self.h))

    def update(self, beta: float, deltas) -> dict:
        a, p = _darr(deltas)
        rec = HmcRecord()
        _chk(load().mesh_hmc_update(self.h, beta, p, len(a), C.byref(rec)))
        return rec.as_dict()

    def update_supplied(self, P0: Field, uniform: float, beta: float, deltas) -> dict:
        a, p = _darr(deltas)
        rec = HmcRecord()
        _chk(load().mesh_hmc_update_supplied(self.h, P0.h, uniform, beta, p, len(a), C.byref(rec)))
        return rec.as_dict()

    def run(self, beta: float, deltas, count: int, use_graph: bool = True):
        a, p = _darr(deltas)
        _chk(load().mesh_hmc_run(self.h, beta, p, len(a), count, 1 if use_graph else 0))

    def momentum_step(self, beta: float, delta: float):
        """the trajectory's momentum step on the chain's own U and P"""
        _chk(load().mesh_hmc_momentum_step(self.h, beta, delta))

    def md_step(self, beta: float, dp: float, du: float):
        """one momentum step (dp) and the link update (du) after it on the
        chain's own U and P, fused in one kernel where the trajectory fuses
        them"""
        _chk(load().mesh_hmc_md_step(self.h, beta, dp, du))

    def save(self, path: str):
        """checkpoint: links, trajectory counter and seed"""
        _chk(load().mesh_hmc_save(self.h, os.fsencode(path)))

    def load(self, path: str):
        """resume from a checkpoint written by a chain with the same seed"""
        _chk(load().mesh_hmc_load(self.h, os.fsencode(path)))

    def run_host(self, host_U: np.ndarray, beta: float, deltas, count: int = 1) -> dict:
        a, p = _darr(deltas)
        rec = HmcRecord()
        assert host_U.flags["C_CONTIGUOUS"]
        _chk(load().mesh_hmc_run_host(self.h, host_U.ctypes.data_as(C.c_void_p), host_U.nbytes, beta, p, len(a),
                                      count, C.byref(rec)))
        return rec.as_dict()

    @property
    def count(self) -> int:
        n = C.c_int()
        _chk(load().mesh_hmc_count(self.h, C.byref(n)))
        return n.value

    def history(self, first: int = 0, count: int | None = None):
        if count is None:
            count = self.count - first
        pl, dh, ac = (np.zeros(count) for _ in range(3))
        _chk(load().mesh_hmc_history(self.h, first, count, pl.ctypes.data_as(_DP), dh.ctypes.data_as(_DP),
                                     ac.ctypes.data_as(_DP)))
        return {"plaq_history": pl, "deltaH_history": dh, "accept_history": ac}

    def close(self):
        if getattr(self, "h", None):
            load().mesh_hmc_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class HmcBatch:
    """Independent 4D replicas (own extents, beta, seed) advanced together,
    one persistent launch per trajectory step over all of them. Replica r
    follows the trajectory of Hmc(ctx, group, prec, Grid(dims[r]), seeds[r])."""

    def __init__(self, ctx: Context, group, prec: int, dims, seeds):
        self.ctx, self.group, self.prec = ctx, group_code(group), prec
        self.dims = [list(map(int, d)) for d in dims]
        assert all(len(d) == 4 for d in self.dims), "replicas are 4D"
        self.R = len(self.dims)
        flat = (C.c_int32 * (4 * self.R))(*[x for d in self.dims for x in d])
        sd = (C.c_uint64 * self.R)(*[int(x) for x in seeds])
        h = C.c_void_p()
        _chk(load().mesh_batch_create(ctx.h, self.group, prec, self.R, flat, sd, C.byref(h)))
        self.h = h

    def randomize_gauge_field(self):
        _chk(load().mesh_batch_randomize(self.h))

    def cold_start(self):
        _chk(load().mesh_batch_cold_start(self.h))

    def _host_shape(self, r):
        return (4, int(np.prod(self.dims[r])), NREAL[self.group])

    def export(self, r: int) -> np.ndarray:
        out = np.zeros(self._host_shape(r), dtype=np.float32 if self.prec == F32 else np.float64)
        _chk(load().mesh_batch_export(self.h, r, out.ctypes.data_as(C.c_void_p), out.nbytes))
        return out

    def import_(self, r: int, host: np.ndarray):
        a = np.ascontiguousarray(host, dtype=np.float32 if self.prec == F32 else np.float64)
        assert a.shape == self._host_shape(r)
        _chk(load().mesh_batch_import(self.h, r, a.ctypes.data_as(C.c_void_p), a.nbytes))
        return self

    def run(self, betas, deltas, count: int, use_graph: bool = True):
        b, pb = _darr(betas)
        if b.shape != (self.R,):
            raise ValueError(f"expected {self.R} betas, one per replica")
        a, p = _darr(deltas)
        _chk(load().mesh_batch_run(self.h, pb, p, len(a), count, 1 if use_graph else 0))

    @property
    def count(self) -> int:
        n = C.c_int()
        _chk(load().mesh_batch_count(self.h, C.byref(n)))
        return n.value

    def history(self, r: int, first: int = 0, count: int | None = None):
        if count is None:
            count = self.count - first
        pl, dh, ac = (np.zeros(count) for _ in range(3))
        _chk(load().mesh_batch_history(self.h, r, first, count, pl.ctypes.data_as(_DP), dh.ctypes.data_as(_DP),
                                       ac.ctypes.data_as(_DP)))
        return {"plaq_history": pl, "deltaH_history": dh, "accept_history": ac}

    def plaquettes(self) -> np.ndarray:
        out = np.zeros(self.R)
        _chk(load().mesh_batch_plaquettes(self.h, out.ctypes.data_as(_DP)))
        return out

    def launch_info(self, n_deltas: int):
        lpt, gl, gs = C.c_int(), C.c_int(), C.c_int()
        _chk(load().mesh_batch_launch_info(self.h, C.byref(lpt), n_deltas, C.byref(gl), C.byref(gs)))
        return {"launches_per_trajectory": lpt.value, "grid_links": gl.value, "grid_sites": gs.value}

    def md_launch(self):
        """the MD-step form the first run chose: fused (1) or separate kernels
        (0; -1 before the first run), the fused kernel's launch variant, its
        minimum resident blocks per SM and its grid"""
        f, v, mb, g = C.c_int(), C.c_int(), C.c_int(), C.c_int()
        _chk(load().mesh_batch_md_launch(self.h, C.byref(f), C.byref(v), C.byref(mb), C.byref(g)))
        return {"fused": f.value, "variant": v.value, "min_blocks": mb.value, "grid": g.value}

    def close(self):
        if getattr(self, "h", None):
            load().mesh_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


# ---- Landau -----------------------------------------------------------------
class Landau:
    """Landau<G> (landau.h:8-137): gauge transform g for fixed links U."""

    def __init__(self, U: Field):
        self.U = U
        self.g = Lattice(U.ctx, U.group, U.prec, U.grid).set_unit()

    def reset(self):
        self.g.set_unit()

    def __call__(self, h: Field = None) -> float:
        """the functional at g, or at the transform h (landau.h:23-34)"""
        out = C.c_double()
        _chk(load().mesh_landau_functional(self.U.h, (self.g if h is None else h).h, C.byref(out)))
        return out.value

    def line_search(self, F: Field, eps: float) -> float:
        """the CG's step along the algebra field F from g (landau.h:77-98)"""
        out = C.c_double()
        _chk(load().mesh_landau_line_search(self.U.h, self.g.h, F.h, eps, C.byref(out)))
        return out.value

    def condition(self) -> float:
        out = C.c_double()
        _chk(load().mesh_landau_theta(self.U.h, self.g.h, C.byref(out)))
        return out.value

    def deriv(self) -> Field:
        F = Lattice(self.U.ctx, self.U.group, self.U.prec, self.U.grid, algebra=True)
        _chk(load().mesh_landau_deriv(F.h, self.U.h, self.g.h))
        return F

    def run(self, max_iter: int, tol: float = 1e-10, raise_on_noconv: bool = False):
        it, th = C.c_int(), C.c_double()
        rc = load().mesh_landau_cg(self.U.h, self.g.h, max_iter, tol, C.byref(it), C.byref(th))
        if rc != 0 and (rc != 6 or raise_on_noconv):
            _chk(rc)
        return it.value, th.value

    def overrelax(self, omega: float = 1.7, tol: float = 1e-12, max_sweeps: int = 100000, check_every: int = 10,
                  raise_on_noconv: bool = False):
        s, th = C.c_int(), C.c_double()
        rc = load().mesh_landau_or(self.U.h, self.g.h, omega, tol, max_sweeps, check_every, C.byref(s), C.byref(th))
        if rc != 0 and (rc != 6 or raise_on_noconv):
            _chk(rc)
        return s.value, th.value


# ---- Fourier-accelerated Landau fixing, FFT, MLP -------------------------------
def _fp(a):
    return a.ctypes.data_as(C.POINTER(C.c_float))


class LandauFA:
    """Fourier-accelerated steepest descent for Landau gauge on FP64 links,
    with the plain multiplier alpha p2max/p^2 or the learned MLP multiplier."""

    def __init__(self, U: Field):
        self.U = U
        h = C.c_void_p()
        _chk(load().mesh_landau_fa_create(U.h, C.byref(h)))
        self.h = h

    def set_plain(self, alpha: float):
        _chk(load().mesh_landau_fa_set_plain(self.h, alpha))

    def set_table(self, log_mult, log_p2_lo: float, log_p2_hi: float):
        a = np.ascontiguousarray(log_mult, dtype=np.float32)
        _chk(load().mesh_landau_fa_set_table(self.h, _fp(a), len(a), log_p2_lo, log_p2_hi))

    def set_mlp(self, params, width: int, beta: float, bf16: bool = True):
        a = np.ascontiguousarray(params, dtype=np.float32)
        _chk(load().mesh_landau_fa_set_mlp(self.h, _fp(a), width, beta, 1 if bf16 else 0))

    def p2range(self):
        a, b = C.c_double(), C.c_double()
        _chk(load().mesh_landau_fa_p2range(self.h, C.byref(a), C.byref(b)))
        return a.value, b.value

    def theta(self, g: Field) -> float:
        t = C.c_double()
        _chk(load().mesh_landau_fa_theta(self.h, g.h, C.byref(t)))
        return t.value

    def step(self, g: Field) -> float:
        t = C.c_double()
        _chk(load().mesh_landau_fa_step(self.h, g.h, C.byref(t)))
        return t.value

    def set_accept(self, functional: bool):
        """acceptance test of run(): on theta (default) or on the gauge functional"""
        _chk(load().mesh_landau_fa_set_accept(self.h, 1 if functional else 0))

    def run(self, g: Field, tol=1e-12, max_iter=100000, omega=1.7, or_sweeps=10, raise_on_noconv=False):
        it, fb, th = C.c_int(), C.c_int(), C.c_double()
        rc = load().mesh_landau_fa_run(self.h, g.h, tol, max_iter, omega, or_sweeps, C.byref(it), C.byref(fb),
                                       C.byref(th))
        if rc != 0 and (rc != 6 or raise_on_noconv):
            _chk(rc)
        return it.value, fb.value, th.value

    def trial(self, g: Field, alpha: float = 0.0):
        """theta before and after a step that leaves g unchanged (plain
        multiplier alpha if alpha > 0, else the current one)"""
        a, b = C.c_double(), C.c_double()
        _chk(load().mesh_landau_fa_trial(self.h, g.h, alpha, C.byref(a), C.byref(b)))
        return a.value, b.value

    def probe(self, g: Field, probe_alpha: float, nbins: int = 64):
        p2, lam, w, cnt = (np.zeros(nbins) for _ in range(4))
        th = C.c_double()
        _chk(load().mesh_landau_fa_probe(self.h, g.h, probe_alpha, nbins, p2.ctypes.data_as(_DP),
                                         lam.ctypes.data_as(_DP), w.ctypes.data_as(_DP), cnt.ctypes.data_as(_DP),
                                         C.byref(th)))
        return {"p2": p2, "lambda": lam, "weight": w, "count": cnt, "theta": th.value}

    def close(self):
        if getattr(self, "h", None):
            load().mesh_landau_fa_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def lattice_fft(ctx: Context, dims, data, sign: int) -> np.ndarray:
    """data: complex64 array (nf, V) in lexicographic order; returns the
    unnormalised transform over all axes (sign -1 forward, +1 backward)."""
    a = np.array(data, dtype=np.complex64, order="C", copy=True)
    nf = a.shape[0] if a.ndim == 2 else 1
    f = a.view(np.float32)
    _chk(load().mesh_lattice_fft(ctx.h, len(dims), _dims(dims), nf, _fp(f), sign))
    return a


def mlp_nparams(width: int) -> int:
    return load().mesh_mlp_nparams(width)


def mlp_forward(ctx: Context, x, params, width: int, bf16: bool = False) -> np.ndarray:
    x = np.ascontiguousarray(x, dtype=np.float32)
    p = np.ascontiguousarray(params, dtype=np.float32)
    y = np.zeros(x.shape[0], dtype=np.float32)
    _chk(load().mesh_mlp_forward(ctx.h, x.shape[0], _fp(x), _fp(p), width, 1 if bf16 else 0, _fp(y)))
    return y


def mlp_grad(ctx: Context, x, t, params, width: int):
    x = np.ascontiguousarray(x, dtype=np.float32)
    t = np.ascontiguousarray(t, dtype=np.float32)
    p = np.ascontiguousarray(params, dtype=np.float32)
    g = np.zeros(mlp_nparams(width), dtype=np.float32)
    loss = C.c_double()
    _chk(load().mesh_mlp_grad(ctx.h, x.shape[0], _fp(x), _fp(t), _fp(p), width, C.byref(loss), _fp(g)))
    return loss.value, g


def mlp_train(ctx: Context, x, t, params, width: int, epochs: int, batch: int = 1024, lr: float = 1e-3,
              seed: int = 0):
    x = np.ascontiguousarray(x, dtype=np.float32)
    t = np.ascontiguousarray(t, dtype=np.float32)
    p = np.ascontiguousarray(params, dtype=np.float32).copy()
    losses = np.zeros(max(epochs, 1), dtype=np.float32)
    _chk(load().mesh_mlp_train(ctx.h, x.shape[0], _fp(x), _fp(t), _fp(p), width, epochs, batch, lr, seed,
                               _fp(losses)))
    return p, losses[:epochs]


def mlp_init(width: int, seed: int = 0) -> np.ndarray:
    """Glorot-style initial parameters in the library's layout."""
    rng = np.random.default_rng(seed)
    w = width
    parts = [rng.normal(0, np.sqrt(1 / 3), (w, 3)), np.zeros(w), rng.normal(0, np.sqrt(1 / w), (w, w)), np.zeros(w),
             rng.normal(0, np.sqrt(1 / w), w), np.zeros(1)]
    return np.concatenate([p.ravel() for p in parts]).astype(np.float32)
