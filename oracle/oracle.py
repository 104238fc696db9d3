"""ctypes front end of the oracle (CPU restatement of the reference SEM step).

TEST INFRASTRUCTURE ONLY: imported by tests/, ``__graft_entry__.smoke()`` and the CPU-baseline
leg of ``bench.py`` as the checker.  The product (libsemgb) never imports this module.

Two back ends share one calling convention:

* ``liboracle.so`` -- the C restatement in this directory (sem_oracle.c), built by ``make`` on
  any machine;
* ``_ref/libsemref_q<order>.so`` -- the reference's own sources compiled by ``build_ref.sh``
  (only where the reference checkout exists).
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from dataclasses import dataclass, field

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
_I64P = C.POINTER(C.c_int64)
_I32P = C.POINTER(C.c_int32)
_F32P = C.POINTER(C.c_float)
_F64P = C.POINTER(C.c_double)


class OrConfig(C.Structure):
    """Mirror of ``or_config`` in sem_oracle.h."""

    _fields_ = [
        ("ex", C.c_int), ("ey", C.c_int), ("ez", C.c_int), ("order", C.c_int),
        ("lx", C.c_float), ("ly", C.c_float), ("lz", C.c_float),
        ("dt", C.c_float),
        ("nsteps", C.c_int), ("step0", C.c_int),
        ("xi", _F64P), ("w", _F64P), ("dphi", _F64P),
        ("vel", _F32P),
        ("nsrc", C.c_int), ("src_elem", _I64P), ("wavelet", _F32P), ("nsamples", C.c_int),
        ("sx", C.c_void_p), ("sy", C.c_void_p), ("sz", C.c_void_p),
        ("nrec", C.c_int), ("rec_node", _I64P),
        ("nthreads", C.c_int),
    ]


def _ptr(a, t):
    return a.ctypes.data_as(t) if a is not None else None


_LIB = None


def lib() -> C.CDLL:
    """Load (building on first use) liboracle.so."""
    global _LIB
    if _LIB is not None:
        return _LIB
    path = os.path.join(HERE, "liboracle.so")
    srcs = [os.path.join(HERE, f) for f in ("sem_oracle.c", "sem_oracle_impl.h", "sem_oracle.h")]
    if not os.path.exists(path) or any(os.path.getmtime(s) > os.path.getmtime(path) for s in srcs):
        build()
    L = C.CDLL(path)
    L.or_box_counts.argtypes = [C.c_int] * 4 + [_I64P] * 3
    L.or_connectivity.argtypes = [C.c_int] * 4 + [_I32P]
    L.or_interior_nodes.argtypes = [C.c_int] * 4 + [_I32P]
    L.or_element_from_point.argtypes = [C.c_int] * 3 + [C.c_float] * 6
    L.or_element_from_point.restype = C.c_int64
    L.or_nearest_node.argtypes = [C.c_int] * 3 + [C.c_float] * 3 + [C.c_int] + [C.c_float] * 3
    L.or_nearest_node.restype = C.c_int64
    L.or_element_coords.argtypes = [C.c_int] * 3 + [C.c_float] * 3 + [C.c_int] + [_F32P] * 3
    L.or_gll_tables.argtypes = [C.c_int, _F64P, _F64P, _F64P]
    L.or_ricker.argtypes = [C.c_float, C.c_float, C.c_int]
    L.or_ricker.restype = C.c_float
    L.or_source_term.argtypes = [C.c_int, C.c_float, C.c_float, C.c_int, _F32P]
    L.or_sponge_profile.argtypes = ([C.c_int] * 3 + [C.c_float] * 3 + [C.c_int, C.c_int, C.c_float]
                                    + [_F32P] * 3 + [_F64P] * 3)
    L.or_run_f32.argtypes = [C.POINTER(OrConfig), _F32P, _F32P, _F32P]
    L.or_run_f64.argtypes = [C.POINTER(OrConfig), _F64P, _F64P, _F64P]
    L.or_element_apply_f32.argtypes = [C.POINTER(OrConfig), C.c_int64, _F32P, _F32P, _F32P]
    _LIB = L
    return L


def build() -> str:
    subprocess.run(["make", "-s", "-C", HERE], check=True)
    return os.path.join(HERE, "liboracle.so")


_REFS: dict[int, C.CDLL] = {}


def ref_available(order: int) -> bool:
    return os.path.exists(os.path.join(HERE, "_ref", f"libsemref_q{order}.so"))


def ref(order: int) -> C.CDLL:
    """The compiled reference for one polynomial order (built by build_ref.sh)."""
    if order in _REFS:
        return _REFS[order]
    L = C.CDLL(os.path.join(HERE, "_ref", f"libsemref_q{order}.so"))
    L.semref_order.restype = C.c_int
    L.semref_tables.argtypes = [_F64P, _F64P, _F64P]
    L.semref_source_term.argtypes = [C.c_int, C.c_float, C.c_float, C.c_int, _F32P]
    L.semref_mesh.argtypes = [C.c_int] * 3 + [C.c_float] * 3 + [_I64P, _I32P, _I32P, _F32P, _F32P, _F32P]
    L.semref_element_from_point.argtypes = [C.c_int] * 3 + [C.c_float] * 6
    L.semref_element_from_point.restype = C.c_int64
    L.semref_run.argtypes = [C.POINTER(OrConfig), _F32P, _F32P, _F32P]
    L.semref_element_apply.argtypes = [C.POINTER(OrConfig), C.c_int64, _F32P, _F32P, _F32P]
    assert L.semref_order() == order
    _REFS[order] = L
    return L


# ---------------------------------------------------------------------------------------------
# host-side helpers
# ---------------------------------------------------------------------------------------------

def box_counts(ex, ey, ez, order):
    a, b, c = C.c_int64(), C.c_int64(), C.c_int64()
    lib().or_box_counts(ex, ey, ez, order, C.byref(a), C.byref(b), C.byref(c))
    return a.value, b.value, c.value


def connectivity(ex, ey, ez, order):
    _, ne, _ = box_counts(ex, ey, ez, order)
    out = np.empty((ne, (order + 1) ** 3), np.int32)
    lib().or_connectivity(ex, ey, ez, order, _ptr(out, _I32P))
    return out


def interior_nodes(ex, ey, ez, order):
    _, _, ni = box_counts(ex, ey, ez, order)
    out = np.empty(max(ni, 0), np.int32)
    if ni > 0:
        lib().or_interior_nodes(ex, ey, ez, order, _ptr(out, _I32P))
    return out


def element_coords(ex, ey, ez, lx, ly, lz, order):
    _, ne, _ = box_counts(ex, ey, ez, order)
    X, Z, Y = (np.empty((ne, (order + 1) ** 3), np.float32) for _ in range(3))
    lib().or_element_coords(ex, ey, ez, lx, ly, lz, order, _ptr(X, _F32P), _ptr(Z, _F32P), _ptr(Y, _F32P))
    return X, Z, Y


def element_from_point(ex, ey, ez, lx, ly, lz, x, y, z):
    return lib().or_element_from_point(ex, ey, ez, lx, ly, lz, x, y, z)


def nearest_node(ex, ey, ez, lx, ly, lz, order, x, y, z):
    return lib().or_nearest_node(ex, ey, ez, lx, ly, lz, order, x, y, z)


def gll_tables(order):
    n = order + 1
    xi, w, d = np.empty(n), np.empty(n), np.empty(n * n)
    assert lib().or_gll_tables(order, _ptr(xi, _F64P), _ptr(w, _F64P), _ptr(d, _F64P)) == 0
    return xi, w, d.reshape(n, n)


def ref_tables(order):
    n = order + 1
    xi, w, d = np.empty(n), np.empty(n), np.empty(n * n)
    ref(order).semref_tables(_ptr(xi, _F64P), _ptr(w, _F64P), _ptr(d, _F64P))
    return xi, w, d.reshape(n, n)


def source_term(n, dt, f0, order=1):
    out = np.empty(n, np.float32)
    lib().or_source_term(n, dt, f0, order, _ptr(out, _F32P))
    return out


def sponge_profile(ex, ey, ez, lx, ly, lz, order, thickness, sigma):
    """Per-axis sponge factors (x, y, z) as float32 and float64 arrays."""
    nx, ny, nz = ex * order + 1, ey * order + 1, ez * order + 1
    f = [np.empty(n, np.float32) for n in (nx, ny, nz)]
    d = [np.empty(n, np.float64) for n in (nx, ny, nz)]
    lib().or_sponge_profile(ex, ey, ez, lx, ly, lz, order, thickness, sigma,
                            *[_ptr(a, _F32P) for a in f], *[_ptr(a, _F64P) for a in d])
    return tuple(f), tuple(d)


# ---------------------------------------------------------------------------------------------
# problem description and runs
# ---------------------------------------------------------------------------------------------

@dataclass
class Problem:
    """One SEM run: a box mesh, per-element velocity, sources, receivers, sponge, dt, steps."""

    ex: int
    ey: int
    ez: int
    order: int
    lx: float
    ly: float
    lz: float
    dt: float
    nsteps: int
    vel: np.ndarray                      # float32 [n_elem]
    src_elem: np.ndarray                 # int64 [nsrc]
    wavelet: np.ndarray                  # float32 [nsrc, nsamples]
    rec_node: np.ndarray = field(default_factory=lambda: np.zeros(0, np.int64))
    sponge32: tuple | None = None        # (sx, sy, sz) float32 or None
    sponge64: tuple | None = None        # (sx, sy, sz) float64 or None
    step0: int = 0

    @property
    def n_nodes(self):
        return box_counts(self.ex, self.ey, self.ez, self.order)[0]


def _config(p: Problem, tables, keep: list, nthreads: int, real=np.float32) -> OrConfig:
    xi, w, d = (np.ascontiguousarray(t, np.float64) for t in tables)
    vel = np.ascontiguousarray(p.vel, np.float32)
    src = np.ascontiguousarray(p.src_elem, np.int64)
    wav = np.ascontiguousarray(p.wavelet, np.float32).reshape(len(src), -1) if len(src) else np.zeros((0, 1), np.float32)
    rec = np.ascontiguousarray(p.rec_node, np.int64)
    sp = p.sponge32 if real == np.float32 else p.sponge64
    sp = tuple(np.ascontiguousarray(a, real) for a in sp) if sp is not None else None
    keep += [xi, w, d, vel, src, wav, rec, sp]
    c = OrConfig()
    c.ex, c.ey, c.ez, c.order = p.ex, p.ey, p.ez, p.order
    c.lx, c.ly, c.lz, c.dt = p.lx, p.ly, p.lz, p.dt
    c.nsteps, c.step0 = p.nsteps, p.step0
    c.xi, c.w, c.dphi = _ptr(xi, _F64P), _ptr(w, _F64P), _ptr(d, _F64P)
    c.vel = _ptr(vel, _F32P)
    c.nsrc, c.src_elem, c.wavelet, c.nsamples = len(src), _ptr(src, _I64P), _ptr(wav, _F32P), wav.shape[1]
    if sp is not None:
        c.sx, c.sy, c.sz = (a.ctypes.data for a in sp)
    c.nrec, c.rec_node = len(rec), _ptr(rec, _I64P)
    c.nthreads = nthreads
    return c


def run(p: Problem, p_cur=None, p_prev=None, *, backend: str = "oracle", real=np.float32,
        tables: str = "own", nthreads: int = 1):
    """Run ``p.nsteps`` steps.  backend: "oracle" (C restatement) or "ref" (compiled reference,
    float only).  tables: "own" (or_gll_tables) or "ref" (the reference's literals).
    Returns (p_cur, p_prev, traces[nsteps, nrec])."""
    N = p.n_nodes
    pc = np.zeros(N, real) if p_cur is None else np.array(p_cur, real, copy=True)
    pp = np.zeros(N, real) if p_prev is None else np.array(p_prev, real, copy=True)
    tr = np.zeros((p.nsteps, max(len(p.rec_node), 1)), real)
    tabs = ref_tables(p.order) if tables == "ref" else gll_tables(p.order)
    keep: list = []
    cfg = _config(p, tabs, keep, nthreads, real)
    if backend == "ref":
        assert real == np.float32
        rc = ref(p.order).semref_run(C.byref(cfg), _ptr(pc, _F32P), _ptr(pp, _F32P), _ptr(tr, _F32P))
    elif real == np.float32:
        rc = lib().or_run_f32(C.byref(cfg), _ptr(pc, _F32P), _ptr(pp, _F32P), _ptr(tr, _F32P))
    else:
        rc = lib().or_run_f64(C.byref(cfg), _ptr(pc, _F64P), _ptr(pp, _F64P), _ptr(tr, _F64P))
    if rc != 0:
        raise RuntimeError(f"oracle run failed: {rc}")
    return pc, pp, tr[:, : len(p.rec_node)]


def element_apply(p: Problem, e: int, p_local, *, backend="oracle", tables="own"):
    tabs = ref_tables(p.order) if tables == "ref" else gll_tables(p.order)
    keep: list = []
    cfg = _config(p, tabs, keep, 1)
    npe = (p.order + 1) ** 3
    pl = np.ascontiguousarray(p_local, np.float32)
    M, Y = np.empty(npe, np.float32), np.empty(npe, np.float32)
    if backend == "ref":
        rc = ref(p.order).semref_element_apply(C.byref(cfg), e, _ptr(pl, _F32P), _ptr(M, _F32P), _ptr(Y, _F32P))
        assert rc == 0
    else:
        lib().or_element_apply_f32(C.byref(cfg), e, _ptr(pl, _F32P), _ptr(M, _F32P), _ptr(Y, _F32P))
    return M, Y


def rel_l2(a, b) -> float:
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    den = np.linalg.norm(b)
    return float(np.linalg.norm(a - b) / den) if den > 0 else float(np.linalg.norm(a - b))


def problem_from_workload(wl, nsteps=None) -> Problem:
    """Resolve a ``semgb.workloads.Workload`` (positions) into an oracle Problem (indices) with
    the oracle's own host logic."""
    n = wl.nsteps if nsteps is None else nsteps
    src = np.array([element_from_point(wl.ex, wl.ey, wl.ez, wl.lx, wl.ly, wl.lz, *map(float, s))
                    for s in wl.src_xyz], np.int64)
    wav = np.stack([source_term(n, wl.dt, float(f), wl.ricker_order) for f in wl.f0]) if len(src) else np.zeros((0, n), np.float32)
    rec = np.array([nearest_node(wl.ex, wl.ey, wl.ez, wl.lx, wl.ly, wl.lz, wl.order, *map(float, r))
                    for r in wl.rec_xyz], np.int64)
    sp32 = sp64 = None
    if wl.sponge_thickness > 0:
        sp32, sp64 = sponge_profile(wl.ex, wl.ey, wl.ez, wl.lx, wl.ly, wl.lz, wl.order,
                                    wl.sponge_thickness, wl.sponge_sigma)
    return Problem(wl.ex, wl.ey, wl.ez, wl.order, wl.lx, wl.ly, wl.lz, wl.dt, n,
                   np.ascontiguousarray(wl.vel, np.float32), src, wav, rec, sp32, sp64)
