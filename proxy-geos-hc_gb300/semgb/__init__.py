"""Python binding of libsemgb (the GB300 SEM acoustic step) over its C ABI (include/semgb.h).

The binding loads ``semgb/_lib/libsemgb.so`` (built by ``proxy-geos-hc_gb300/build.py``) and
raises if it is missing; there is no other implementation behind it.

Classes mirror the reference's objects: :class:`Mesh` (SEMmesh + the mesh half of
SEMsolver::computeFEInit) and :class:`Solver` (SEMsolver::computeOneStep in a time loop, with
source and receiver I/O).
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
# SEMGB_LIBRARY selects another build of the library (same ABI), e.g. one with other tile sizes
LIB_PATH = os.environ.get("SEMGB_LIBRARY") or os.path.join(_HERE, "_lib", "libsemgb.so")

SEM_OK, SEM_ERR_ARG, SEM_ERR_CUDA, SEM_ERR_OOM, SEM_ERR_TIMEOUT, SEM_ERR_UNSTABLE, SEM_ERR_STATE = range(7)
KERNEL_AUTO, KERNEL_ELEMENT, KERNEL_STENCIL = 0, 1, 2
FORM_DIRECT, FORM_DIFFERENCE = 0, 1
ROUNDING_DEFAULT, ROUNDING_REFERENCE = 0, 1
TILE_AUTO, TILE_DEFAULT, TILE_SQUARE = -1, 0, 1
GROUP_ONE_LAUNCH, GROUP_BRANCHES = 0, 1
LEVEL_CURRENT, LEVEL_PREVIOUS = 0, 1

_I64P = C.POINTER(C.c_int64)
_I32P = C.POINTER(C.c_int32)
_F32P = C.POINTER(C.c_float)
_F64P = C.POINTER(C.c_double)
_VP = C.c_void_p


class SemError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"semgb error {code}: {msg}")
        self.code = code


# name -> argtypes (all functions return int unless listed in _RESTYPE)
_SIGS = {
    "sem_last_error_string": [],
    "sem_version": [],
    "sem_selftest_bounded_wait": [C.c_double, C.POINTER(C.c_double)],
    "sem_gll_tables": [C.c_int, _F64P, _F64P, _F64P],
    "sem_ricker": [C.c_int, C.c_float, C.c_float, C.c_int, _F32P],
    "sem_box_counts": [C.c_int, C.c_int, C.c_int, C.c_int, _I64P, _I64P, _I64P],
    "sem_box_connectivity": [C.c_int, C.c_int, C.c_int, C.c_int, C.c_int64, C.c_int64, _I64P],
    "sem_box_element_from_point": [C.c_int] * 3 + [C.c_float] * 6 + [_I64P],
    "sem_box_nearest_node": [C.c_int] * 3 + [C.c_float] * 3 + [C.c_int] + [C.c_float] * 3 + [_I64P],
    "sem_box_sponge_profile": [C.c_int] * 3 + [C.c_float] * 3 + [C.c_int, C.c_int, C.c_float, _F32P, _F32P, _F32P],
    "sem_box_refround_rows": [C.c_int] * 3 + [C.c_float] * 3 + [C.c_int, _F32P],
    "sem_box_refround_class_table": [C.c_int] * 3 + [C.c_float] * 3 + [C.c_int, _F32P],
    "sem_mesh_create_box": [C.c_int] * 3 + [C.c_float] * 3 + [C.c_int, C.POINTER(_VP)],
    "sem_mesh_destroy": [_VP],
    "sem_mesh_info": [_VP, _I64P, _I64P, C.POINTER(C.c_int), _I64P],
    "sem_mesh_get_connectivity": [_VP, _I32P],
    "sem_model_set_element_velocity": [_VP, _F32P],
    "sem_model_set_node_slowness2": [_VP, _F32P],
    "sem_solver_create": [_VP, C.c_float, C.POINTER(_VP)],
    "sem_solver_destroy": [_VP],
    "sem_solver_set_stream": [_VP, _VP],
    "sem_solver_set_kernel": [_VP, C.c_int],
    "sem_solver_set_operator_form": [_VP, C.c_int],
    "sem_solver_set_rounding": [_VP, C.c_int],
    "sem_solver_set_tile_shape": [_VP, C.c_int],
    "sem_solver_get_tile_shape": [_VP, _I32P],
    "sem_solver_set_sponge": [_VP, C.c_int, C.c_float],
    "sem_solver_set_sponge_profile": [_VP, _F32P, _F32P, _F32P],
    "sem_solver_set_sources": [_VP, C.c_int, _I64P, _F32P, C.c_int],
    "sem_solver_set_source_points": [_VP, C.c_int, _F32P, _F32P, C.c_int],
    "sem_solver_set_receiver_nodes": [_VP, C.c_int, _I64P],
    "sem_solver_set_receivers": [_VP, C.c_int, _F32P],
    "sem_solver_step": [_VP, C.c_int],
    "sem_solver_step_host": [_VP, C.c_int, _F32P, _F32P],
    "sem_solver_steps_done": [_VP, _I64P],
    "sem_solver_get_traces": [_VP, _F32P],
    "sem_solver_get_pressure": [_VP, C.c_int, _F32P],
    "sem_solver_set_pressure": [_VP, C.c_int, _F32P],
    "sem_solver_reset": [_VP],
    "sem_solver_synchronize": [_VP],
    "sem_solver_time_kernels": [_VP, C.c_int, _F32P],
    "sem_element_step_noalloc": [C.c_int] * 3 + [C.c_float] * 3 + [C.c_int] + [_VP] * 8,
    "sem_batch_create": [_VP, C.c_float, C.c_int, C.POINTER(_VP)],
    "sem_batch_destroy": [_VP],
    "sem_batch_set_stream": [_VP, _VP],
    "sem_batch_set_sponge": [_VP, C.c_int, C.c_float],
    "sem_batch_set_sponge_profile": [_VP, _F32P, _F32P, _F32P],
    "sem_batch_set_sources": [_VP, _I64P, _F32P, C.c_int],
    "sem_batch_set_source_points": [_VP, _F32P, _F32P, C.c_int],
    "sem_batch_set_receiver_nodes": [_VP, C.c_int, _I64P],
    "sem_batch_set_receivers": [_VP, C.c_int, _F32P],
    "sem_batch_step": [_VP, C.c_int],
    "sem_batch_synchronize": [_VP],
    "sem_batch_get_traces": [_VP, _F32P],
    "sem_batch_get_pressure": [_VP, C.c_int, C.c_int, _F32P],
    "sem_batch_time_step": [_VP, C.c_int, _F32P],
    "sem_batch_autotune": [_VP, C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_int)],
    "sem_mlp_create": [C.c_uint64, C.POINTER(_VP)],
    "sem_mlp_destroy": [_VP],
    "sem_mlp_n_params": [],
    "sem_mlp_set_params": [_VP, _F32P],
    "sem_mlp_get_params": [_VP, _F32P],
    "sem_mlp_forward": [_VP, C.c_int64, _F32P, _F32P],
    "sem_mlp_loss_grad": [_VP, C.c_int64, _F32P, _F32P, _F64P, _F32P],
    "sem_mlp_train": [_VP, C.c_int64, _F32P, _F32P, C.c_int, C.c_int, C.c_float, C.c_uint64, _F64P],
    "sem_abc_create": [_VP, _VP, C.c_int, C.POINTER(_VP)],
    "sem_abc_destroy": [_VP],
    "sem_abc_info": [_VP, _I64P, _I64P],
    "sem_abc_nodes": [_VP, _I64P],
    "sem_abc_step": [_VP, C.c_int],
    "sem_abc_correct": [_VP],
    "sem_abc_reset": [_VP],
    "sem_abc_set_history": [_VP, _F32P],
    "sem_abc_features": [_VP, _F32P, _F32P],
    "sem_traces_write": [C.c_char_p, C.c_int, C.c_int, _F32P, C.c_float, _F32P, C.c_int, _F32P, C.c_char_p],
    "sem_traces_read_info": [C.c_char_p, C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_float)],
    "sem_traces_read": [C.c_char_p, _F32P],
    "sem_solver_write_snapshot": [_VP, C.c_int, C.c_int, C.c_char_p],
    "sem_snapshot_read_info": [C.c_char_p, C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_int)],
    "sem_snapshot_read": [C.c_char_p, _F32P],
    "sem_group_create": [C.c_int, C.POINTER(_VP), C.POINTER(_VP)],
    "sem_group_destroy": [_VP],
    "sem_group_step": [_VP, C.c_int],
    "sem_group_synchronize": [_VP],
    "sem_group_time_step": [_VP, C.c_int, C.POINTER(C.c_float)],
    "sem_group_set_launch": [_VP, C.c_int],
    "sem_abc_bptt": [_VP, C.c_int, C.c_int, C.POINTER(C.c_int64), C.POINTER(C.c_float), C.POINTER(C.c_double),
                     C.POINTER(C.c_float)],
    "sem_mlp_adam_step": [_VP, C.POINTER(C.c_float), C.c_float],
    "sem_group_get_launch": [_VP, C.POINTER(C.c_int)],
    "sem_adjoint_create": [_VP, C.c_float, C.c_int, C.c_int, C.POINTER(_VP)],
    "sem_adjoint_destroy": [_VP],
    "sem_adjoint_set_sponge": [_VP, C.c_int, C.c_float],
    "sem_adjoint_set_sponge_profile": [_VP, _F32P, _F32P, _F32P],
    "sem_adjoint_set_sources": [_VP, C.c_int, _I64P, _F32P, C.c_int],
    "sem_adjoint_set_source_points": [_VP, C.c_int, _F32P, _F32P, C.c_int],
    "sem_adjoint_set_receiver_nodes": [_VP, C.c_int, _I64P],
    "sem_adjoint_set_receivers": [_VP, C.c_int, _F32P],
    "sem_adjoint_forward": [_VP, _F32P],
    "sem_adjoint_backward": [_VP, _F32P, _F32P],
    "sem_adjoint_gradient": [_VP, _F32P, _F64P, _F32P],
    "sem_adjoint_set_adjoint_receiver_nodes": [_VP, C.c_int, _I64P],
    "sem_adjoint_get_adjoint_traces": [_VP, _F32P],
}
_RESTYPE = {"sem_last_error_string": C.c_char_p}

_lib: C.CDLL | None = None


def lib() -> C.CDLL:
    """The loaded libsemgb.so; raises if it has not been built."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(f"libsemgb.so not built ({LIB_PATH}); run proxy-geos-hc_gb300/build.py")
        L = C.CDLL(LIB_PATH)
        for name, args in _SIGS.items():
            f = getattr(L, name)
            f.argtypes = args
            f.restype = _RESTYPE.get(name, C.c_int)
        _lib = L
    return _lib


def exported_symbols() -> list[str]:
    return list(_SIGS)


def _check(rc: int):
    if rc != SEM_OK:
        raise SemError(rc, lib().sem_last_error_string().decode())


def _p(a, t):
    return a.ctypes.data_as(t)


def _f32(a):
    return np.ascontiguousarray(a, np.float32)


def _i64(a):
    return np.ascontiguousarray(a, np.int64)


# ---- host-only utilities ---------------------------------------------------------------------

def gll_tables(order: int):
    n = order + 1
    xi, w, d = np.empty(n), np.empty(n), np.empty(n * n)
    _check(lib().sem_gll_tables(order, _p(xi, _F64P), _p(w, _F64P), _p(d, _F64P)))
    return xi, w, d.reshape(n, n)


def ricker(nsamples: int, dt: float, f0: float, order: int = 1) -> np.ndarray:
    out = np.empty(nsamples, np.float32)
    _check(lib().sem_ricker(nsamples, dt, f0, order, _p(out, _F32P)))
    return out


def box_counts(ex, ey, ez, order):
    a, b, c = C.c_int64(), C.c_int64(), C.c_int64()
    _check(lib().sem_box_counts(ex, ey, ez, order, C.byref(a), C.byref(b), C.byref(c)))
    return a.value, b.value, c.value


def box_connectivity(ex, ey, ez, order, e0=0, count=None):
    _, ne, _ = box_counts(ex, ey, ez, order)
    count = ne - e0 if count is None else count
    out = np.empty((count, (order + 1) ** 3), np.int64)
    _check(lib().sem_box_connectivity(ex, ey, ez, order, e0, count, _p(out, _I64P)))
    return out


def element_from_point(ex, ey, ez, lx, ly, lz, x, y, z) -> int:
    e = C.c_int64()
    _check(lib().sem_box_element_from_point(ex, ey, ez, lx, ly, lz, x, y, z, C.byref(e)))
    return e.value


def nearest_node(ex, ey, ez, lx, ly, lz, order, x, y, z) -> int:
    n = C.c_int64()
    _check(lib().sem_box_nearest_node(ex, ey, ez, lx, ly, lz, order, x, y, z, C.byref(n)))
    return n.value


def sponge_profile(ex, ey, ez, lx, ly, lz, order, thickness, sigma):
    f = [np.empty(n * order + 1, np.float32) for n in (ex, ey, ez)]
    _check(lib().sem_box_sponge_profile(ex, ey, ez, lx, ly, lz, order, thickness, sigma,
                                        *[_p(a, _F32P) for a in f]))
    return tuple(f)


def refround_rows(ex, ey, ez, lx, ly, lz, order):
    """The reference's float-rounded element rows, [3][(o+1)^3][o+1] (see semgb.h)."""
    o1 = order + 1
    out = np.empty(3 * o1 ** 4, np.float32)
    _check(lib().sem_box_refround_rows(ex, ey, ez, lx, ly, lz, order, _p(out, _F32P)))
    return out.reshape(3, o1 ** 3, o1)


def refround_class_table(ex, ey, ez, lx, ly, lz, order):
    """Node-class coefficients of the reference's assembled operator, [3][ly][lz][2o+1][lx]."""
    o = order
    out = np.empty(3 * o * o * (2 * o + 1) * o, np.float32)
    _check(lib().sem_box_refround_class_table(ex, ey, ez, lx, ly, lz, order, _p(out, _F32P)))
    return out.reshape(3, o, o, 2 * o + 1, o)


# ---- device objects ---------------------------------------------------------------------------

class Mesh:
    """Structured hex box on the GPU (SEMmesh + the FE set-up of SEMsolver::computeFEInit)."""

    def __init__(self, ex, ey, ez, lx, ly, lz, order):
        h = _VP()
        _check(lib().sem_mesh_create_box(ex, ey, ez, lx, ly, lz, order, C.byref(h)))
        self._h = h
        self.ex, self.ey, self.ez, self.order = ex, ey, ez, order
        self.lx, self.ly, self.lz = lx, ly, lz
        n, e, npe, ni = C.c_int64(), C.c_int64(), C.c_int(), C.c_int64()
        _check(lib().sem_mesh_info(h, C.byref(n), C.byref(e), C.byref(npe), C.byref(ni)))
        self.n_nodes, self.n_elem, self.nodes_per_elem, self.n_interior = n.value, e.value, npe.value, ni.value

    def close(self):
        if getattr(self, "_h", None):
            lib().sem_mesh_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def connectivity(self) -> np.ndarray:
        out = np.empty((self.n_elem, self.nodes_per_elem), np.int32)
        _check(lib().sem_mesh_get_connectivity(self._h, _p(out, _I32P)))
        return out

    def set_velocity(self, vel):
        v = _f32(vel)
        assert v.size == self.n_elem
        _check(lib().sem_model_set_element_velocity(self._h, _p(v, _F32P)))

    def set_slowness2(self, m):
        v = _f32(m)
        assert v.size == self.n_nodes
        _check(lib().sem_model_set_node_slowness2(self._h, _p(v, _F32P)))


class Solver:
    """Time stepper over a :class:`Mesh` (SEMsolver::computeOneStep + SEMproxy::run's loop)."""

    def __init__(self, mesh: Mesh, dt: float):
        h = _VP()
        _check(lib().sem_solver_create(mesh._h, dt, C.byref(h)))
        self._h = h
        self.mesh = mesh
        self.dt = dt
        self.nrec = 0
        self.nsrc = 0

    def close(self):
        if getattr(self, "_h", None):
            lib().sem_solver_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_stream(self, stream_handle: int | None):
        _check(lib().sem_solver_set_stream(self._h, stream_handle))

    def set_kernel(self, kernel: int):
        _check(lib().sem_solver_set_kernel(self._h, kernel))

    def set_operator_form(self, form: int):
        """FORM_DIRECT (default, fastest) or FORM_DIFFERENCE (exact on constant fields)."""
        _check(lib().sem_solver_set_operator_form(self._h, form))

    def set_rounding(self, rounding: int):
        """ROUNDING_DEFAULT or ROUNDING_REFERENCE (the reference's float-rounded element rows)."""
        _check(lib().sem_solver_set_rounding(self._h, rounding))

    def set_tile_shape(self, shape: int):
        """TILE_AUTO (default, chosen per box), TILE_DEFAULT or TILE_SQUARE (order 4): the
        stencil pass's tile; the same bits with every shape."""
        _check(lib().sem_solver_set_tile_shape(self._h, shape))

    @property
    def tile_shape(self) -> int:
        """Shape of the built stencil tables (TILE_AUTO before the first stencil step)."""
        v = C.c_int32(0)
        _check(lib().sem_solver_get_tile_shape(self._h, C.byref(v)))
        return v.value

    def set_sponge(self, thickness: int, sigma: float):
        _check(lib().sem_solver_set_sponge(self._h, thickness, sigma))

    def set_sponge_profile(self, sx, sy, sz):
        a, b, c = _f32(sx), _f32(sy), _f32(sz)
        _check(lib().sem_solver_set_sponge_profile(self._h, _p(a, _F32P), _p(b, _F32P), _p(c, _F32P)))

    def set_sources(self, elements, wavelet):
        e = _i64(elements)
        w = _f32(wavelet).reshape(len(e), -1) if len(e) else np.zeros((0, 0), np.float32)
        _check(lib().sem_solver_set_sources(self._h, len(e), _p(e, _I64P), _p(w, _F32P), w.shape[1]))
        self.nsrc = len(e)

    def set_source_points(self, xyz, wavelet):
        x = _f32(xyz).reshape(-1, 3)
        w = _f32(wavelet).reshape(len(x), -1)
        _check(lib().sem_solver_set_source_points(self._h, len(x), _p(x, _F32P), _p(w, _F32P), w.shape[1]))
        self.nsrc = len(x)

    def set_receiver_nodes(self, nodes):
        n = _i64(nodes)
        _check(lib().sem_solver_set_receiver_nodes(self._h, len(n), _p(n, _I64P)))
        self.nrec = len(n)

    def set_receivers(self, xyz):
        x = _f32(xyz).reshape(-1, 3)
        _check(lib().sem_solver_set_receivers(self._h, len(x), _p(x, _F32P)))
        self.nrec = len(x)

    def step(self, n: int = 1):
        _check(lib().sem_solver_step(self._h, n))

    def step_host(self, n: int, wavelet_samples=None, traces_out=None):
        w = _f32(wavelet_samples) if wavelet_samples is not None else None
        _check(lib().sem_solver_step_host(self._h, n, _p(w, _F32P) if w is not None else None,
                                          _p(traces_out, _F32P) if traces_out is not None else None))

    @property
    def steps_done(self) -> int:
        n = C.c_int64()
        _check(lib().sem_solver_steps_done(self._h, C.byref(n)))
        return n.value

    def traces(self) -> np.ndarray:
        out = np.zeros((self.steps_done, self.nrec), np.float32)
        _check(lib().sem_solver_get_traces(self._h, _p(out, _F32P)))
        return out

    def pressure(self, level: int = LEVEL_CURRENT) -> np.ndarray:
        out = np.empty(self.mesh.n_nodes, np.float32)
        _check(lib().sem_solver_get_pressure(self._h, level, _p(out, _F32P)))
        return out

    def set_pressure(self, level: int, values):
        v = _f32(values)
        _check(lib().sem_solver_set_pressure(self._h, level, _p(v, _F32P)))

    def reset(self):
        _check(lib().sem_solver_reset(self._h))

    def synchronize(self):
        _check(lib().sem_solver_synchronize(self._h))

    def write_snapshot(self, path, level: int = LEVEL_CURRENT, y_index: int = -1):
        """One x-z plane of a level to a SEMSNP01 container (y_index -1: ny/2 - 1)."""
        _check(lib().sem_solver_write_snapshot(self._h, level, y_index, str(path).encode()))

    def time_kernels(self, n: int) -> np.ndarray:
        ms = np.zeros(3, np.float32)
        _check(lib().sem_solver_time_kernels(self._h, n, _p(ms, _F32P)))
        return ms


def write_traces(path, traces, dt, rec_xyz=None, src_xyz=None, extra_json=None):
    """Write traces [n_steps][n_rec] to a SEMTRC01 container (sem_traces_write)."""
    t = _f32(traces)
    ns, nr = t.shape
    r = _f32(rec_xyz).reshape(nr, 3) if rec_xyz is not None else None
    s = _f32(src_xyz).reshape(-1, 3) if src_xyz is not None else np.zeros((0, 3), np.float32)
    _check(lib().sem_traces_write(str(path).encode(), ns, nr, _p(t, _F32P), dt,
                                  _p(r, _F32P) if r is not None else None, len(s), _p(s, _F32P),
                                  extra_json.encode() if extra_json else None))


def read_traces(path):
    """Traces [n_steps][n_rec] and dt from a SEMTRC01 container (sem_traces_read)."""
    ns, nr, dt = C.c_int(), C.c_int(), C.c_float()
    _check(lib().sem_traces_read_info(str(path).encode(), C.byref(ns), C.byref(nr), C.byref(dt)))
    out = np.zeros((ns.value, nr.value), np.float32)
    _check(lib().sem_traces_read(str(path).encode(), _p(out, _F32P)))
    return out, dt.value


def read_snapshot(path):
    """(plane [nz][nx], y_index) from a SEMSNP01 container (sem_snapshot_read)."""
    nx, nz, y = C.c_int(), C.c_int(), C.c_int()
    _check(lib().sem_snapshot_read_info(str(path).encode(), C.byref(nx), C.byref(nz), C.byref(y)))
    out = np.zeros((nz.value, nx.value), np.float32)
    _check(lib().sem_snapshot_read(str(path).encode(), _p(out, _F32P)))
    return out, y.value


def solver_from_workload(wl, kernel: int = KERNEL_AUTO):
    """Build (mesh, solver) for a :class:`semgb.workloads.Workload`, resolving positions with
    the library's own host logic."""
    mesh = Mesh(wl.ex, wl.ey, wl.ez, wl.lx, wl.ly, wl.lz, wl.order)
    mesh.set_velocity(wl.vel)
    s = Solver(mesh, wl.dt)
    s.set_kernel(kernel)
    if wl.sponge_thickness > 0:
        s.set_sponge(wl.sponge_thickness, wl.sponge_sigma)
    wav = np.stack([ricker(wl.nsteps, wl.dt, float(f), wl.ricker_order) for f in wl.f0])
    s.set_source_points(wl.src_xyz, wav)
    s.set_receivers(wl.rec_xyz)
    return mesh, s


class Batch:
    """Many shots on one mesh (sem_batch_*): shared mesh, model, sponge and receivers."""

    def __init__(self, mesh: Mesh, dt: float, n_shots: int):
        h = _VP()
        _check(lib().sem_batch_create(mesh._h, dt, n_shots, C.byref(h)))
        self._h = h
        self.mesh = mesh
        self.n_shots = n_shots
        self.nrec = 0
        self.steps = 0

    def close(self):
        if getattr(self, "_h", None):
            lib().sem_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_stream(self, stream_handle):
        _check(lib().sem_batch_set_stream(self._h, stream_handle))

    def set_sponge(self, thickness, sigma):
        _check(lib().sem_batch_set_sponge(self._h, thickness, sigma))

    def set_sponge_profile(self, sx, sy, sz):
        a, b, c = _f32(sx), _f32(sy), _f32(sz)
        _check(lib().sem_batch_set_sponge_profile(self._h, _p(a, _F32P), _p(b, _F32P), _p(c, _F32P)))

    def set_sources(self, elements, wavelet):
        e = _i64(elements)
        w = _f32(wavelet).reshape(self.n_shots, -1)
        _check(lib().sem_batch_set_sources(self._h, _p(e, _I64P), _p(w, _F32P), w.shape[1]))

    def set_source_points(self, xyz, wavelet):
        x = _f32(xyz).reshape(self.n_shots, 3)
        w = _f32(wavelet).reshape(self.n_shots, -1)
        _check(lib().sem_batch_set_source_points(self._h, _p(x, _F32P), _p(w, _F32P), w.shape[1]))

    def set_receiver_nodes(self, nodes):
        n = _i64(nodes)
        _check(lib().sem_batch_set_receiver_nodes(self._h, len(n), _p(n, _I64P)))
        self.nrec = len(n)

    def set_receivers(self, xyz):
        x = _f32(xyz).reshape(-1, 3)
        _check(lib().sem_batch_set_receivers(self._h, len(x), _p(x, _F32P)))
        self.nrec = len(x)

    def step(self, n=1):
        _check(lib().sem_batch_step(self._h, n))
        self.steps += n

    def synchronize(self):
        _check(lib().sem_batch_synchronize(self._h))

    def traces(self):
        out = np.zeros((self.steps, self.nrec, self.n_shots), np.float32)
        _check(lib().sem_batch_get_traces(self._h, _p(out, _F32P)))
        return out

    def pressure(self, shot, level=LEVEL_CURRENT):
        out = np.empty(self.mesh.n_nodes, np.float32)
        _check(lib().sem_batch_get_pressure(self._h, shot, level, _p(out, _F32P)))
        return out

    def time_step(self, n):
        ms = C.c_float()
        _check(lib().sem_batch_time_step(self._h, n, C.byref(ms)))
        self.steps += n
        return ms.value

    def autotune(self):
        a, b, c = C.c_int(), C.c_int(), C.c_int()
        _check(lib().sem_batch_autotune(self._h, C.byref(a), C.byref(b), C.byref(c)))
        return {"shots_per_cluster": a.value, "warps_per_cta": b.value, "ychunk": c.value}


class Group:
    """Independent solvers of uneven size advanced together (sem_group_*), one CUDA graph per
    two steps: by default one launch per step over every member's tiles (GROUP_ONE_LAUNCH),
    or each member's own launches as parallel branches (GROUP_BRANCHES)."""

    def __init__(self, solvers, launch: int = 0):
        self.solvers = list(solvers)  # keeps the members alive while the group exists
        arr = (_VP * len(self.solvers))(*[s._h for s in self.solvers])
        h = _VP()
        _check(lib().sem_group_create(len(self.solvers), arr, C.byref(h)))
        self._h = h
        if launch != GROUP_ONE_LAUNCH:
            _check(lib().sem_group_set_launch(self._h, launch))

    @property
    def launch(self) -> int:
        """Launch form of the last step (GROUP_ONE_LAUNCH or GROUP_BRANCHES)."""
        v = C.c_int()
        _check(lib().sem_group_get_launch(self._h, C.byref(v)))
        return v.value

    def close(self):
        if getattr(self, "_h", None):
            lib().sem_group_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def step(self, n=1):
        _check(lib().sem_group_step(self._h, n))

    def synchronize(self):
        _check(lib().sem_group_synchronize(self._h))

    def time_step(self, n):
        ms = C.c_float()
        _check(lib().sem_group_time_step(self._h, n, C.byref(ms)))
        return ms.value


class Mlp:
    """The boundary network (sem_mlp_*): 81 -> 64 -> 64 -> 1, GELU, BF16 weights on the tensor
    cores with FP32 accumulation, FP32 master parameters and Adam."""

    N_IN = 81

    def __init__(self, seed: int = 0):
        h = _VP()
        _check(lib().sem_mlp_create(seed, C.byref(h)))
        self._h = h
        self.n_params = lib().sem_mlp_n_params()

    def close(self):
        if getattr(self, "_h", None):
            lib().sem_mlp_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def params(self) -> np.ndarray:
        out = np.zeros(self.n_params, np.float32)
        _check(lib().sem_mlp_get_params(self._h, _p(out, _F32P)))
        return out

    @params.setter
    def params(self, p):
        v = _f32(p).reshape(-1)
        assert v.size == self.n_params
        _check(lib().sem_mlp_set_params(self._h, _p(v, _F32P)))

    def forward(self, x):
        x = _f32(x).reshape(-1, self.N_IN)
        y = np.zeros(len(x), np.float32)
        _check(lib().sem_mlp_forward(self._h, len(x), _p(x, _F32P), _p(y, _F32P)))
        return y

    def loss_grad(self, x, t):
        x = _f32(x).reshape(-1, self.N_IN)
        t = _f32(t).reshape(-1)
        loss = C.c_double()
        g = np.zeros(self.n_params, np.float32)
        _check(lib().sem_mlp_loss_grad(self._h, len(x), _p(x, _F32P), _p(t, _F32P), C.byref(loss), _p(g, _F32P)))
        return loss.value, g

    def train(self, x, t, epochs, batch=4096, lr=1e-3, seed=0):
        x = _f32(x).reshape(-1, self.N_IN)
        t = _f32(t).reshape(-1)
        losses = np.zeros(max(epochs, 1), np.float64)
        _check(lib().sem_mlp_train(self._h, len(x), _p(x, _F32P), _p(t, _F32P), epochs, batch, lr, seed,
                                   _p(losses, _F64P)))
        return losses[:epochs]

    def adam_step(self, grad, lr=1e-3):
        """One Adam step with a given gradient (e.g. from Abc.bptt)."""
        g = _f32(grad).reshape(-1)
        assert g.size == self.n_params
        _check(lib().sem_mlp_adam_step(self._h, _p(g, _F32P), lr))


class Abc:
    """Learned absorbing boundary on a solver (sem_abc_*): after every step the network corrects
    the new level on the interior nodes within `layer` elements of a face."""

    def __init__(self, solver: Solver, net: Mlp, layer: int = 1):
        h = _VP()
        _check(lib().sem_abc_create(solver._h, net._h, layer, C.byref(h)))
        self._h = h
        self.solver = solver
        self.net = net
        n, m = C.c_int64(), C.c_int64()
        _check(lib().sem_abc_info(h, C.byref(n), C.byref(m)))
        self.n_nodes = n.value
        self.n_history = m.value

    def close(self):
        if getattr(self, "_h", None):
            lib().sem_abc_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def nodes(self):
        out = np.zeros(self.n_nodes, np.int64)
        _check(lib().sem_abc_nodes(self._h, _p(out, _I64P)))
        return out

    def step(self, n=1):
        _check(lib().sem_abc_step(self._h, n))

    def correct(self):
        _check(lib().sem_abc_correct(self._h))

    def reset(self):
        _check(lib().sem_abc_reset(self._h))

    def set_history(self, p_prev):
        v = _f32(p_prev)
        _check(lib().sem_abc_set_history(self._h, _p(v, _F32P)))

    def features(self):
        x = np.zeros((self.n_nodes, Mlp.N_IN), np.float32)
        sc = np.zeros(self.n_nodes, np.float32)
        _check(lib().sem_abc_features(self._h, _p(x, _F32P), _p(sc, _F32P)))
        return x, sc

    def bptt(self, roi_nodes, ref, grad: bool = True):
        """Loss sum_m sum_r (p^m_r - ref[m-1][r])^2 of n_steps = len(ref) corrected steps from rest
        and (grad=True) its gradient with respect to the network's parameters through the adjoint
        of the whole time loop (sem_abc_bptt).  Returns (loss, gradient or None)."""
        roi = np.ascontiguousarray(np.asarray(roi_nodes, np.int64).reshape(-1))
        r = _f32(ref).reshape(-1, len(roi))
        loss = C.c_double()
        g = np.zeros(self.net.n_params, np.float32) if grad else None
        _check(lib().sem_abc_bptt(self._h, len(r), len(roi), _p(roi, _I64P), _p(r, _F32P), C.byref(loss),
                                  _p(g, _F32P) if grad else None))
        return loss.value, g


class Adjoint:
    """Trace-misfit gradient with respect to per-node squared slowness (sem_adjoint_*): one shot,
    n_steps plain steps, forward levels checkpointed every `checkpoint_every` steps."""

    def __init__(self, mesh: Mesh, dt: float, n_steps: int, checkpoint_every: int = 50):
        h = _VP()
        _check(lib().sem_adjoint_create(mesh._h, dt, n_steps, checkpoint_every, C.byref(h)))
        self._h = h
        self.mesh = mesh
        self.n_steps = n_steps
        self.nrec = 0
        self.n_adj_rec = 0

    def close(self):
        if getattr(self, "_h", None):
            lib().sem_adjoint_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_sponge(self, thickness, sigma):
        _check(lib().sem_adjoint_set_sponge(self._h, thickness, sigma))

    def set_sponge_profile(self, sx, sy, sz):
        a, b, c = _f32(sx), _f32(sy), _f32(sz)
        _check(lib().sem_adjoint_set_sponge_profile(self._h, _p(a, _F32P), _p(b, _F32P), _p(c, _F32P)))

    def set_sources(self, elements, wavelet):
        e = _i64(elements)
        w = _f32(wavelet).reshape(len(e), -1)
        _check(lib().sem_adjoint_set_sources(self._h, len(e), _p(e, _I64P), _p(w, _F32P), w.shape[1]))

    def set_source_points(self, xyz, wavelet):
        x = _f32(xyz).reshape(-1, 3)
        w = _f32(wavelet).reshape(len(x), -1)
        _check(lib().sem_adjoint_set_source_points(self._h, len(x), _p(x, _F32P), _p(w, _F32P), w.shape[1]))

    def set_receiver_nodes(self, nodes):
        n = _i64(nodes)
        _check(lib().sem_adjoint_set_receiver_nodes(self._h, len(n), _p(n, _I64P)))
        self.nrec = len(n)

    def set_receivers(self, xyz):
        x = _f32(xyz).reshape(-1, 3)
        _check(lib().sem_adjoint_set_receivers(self._h, len(x), _p(x, _F32P)))
        self.nrec = len(x)

    def forward(self):
        """Forward run from rest; returns the traces [n_steps][n_rec]."""
        out = np.zeros((self.n_steps, self.nrec), np.float32)
        _check(lib().sem_adjoint_forward(self._h, _p(out, _F32P)))
        return out

    def backward(self, residual):
        """Gradient of 1/2 |residual|^2 with respect to squared slowness, [n_nodes]."""
        r = _f32(residual).reshape(self.n_steps, self.nrec)
        g = np.zeros(self.mesh.n_nodes, np.float32)
        _check(lib().sem_adjoint_backward(self._h, _p(r, _F32P), _p(g, _F32P)))
        return g

    def gradient(self, observed):
        """(loss, gradient) for the last forward run against observed traces [n_steps][n_rec]."""
        o = _f32(observed).reshape(self.n_steps, self.nrec)
        loss = C.c_double()
        g = np.zeros(self.mesh.n_nodes, np.float32)
        _check(lib().sem_adjoint_gradient(self._h, _p(o, _F32P), C.byref(loss), _p(g, _F32P)))
        return loss.value, g

    def set_adjoint_receiver_nodes(self, nodes):
        n = _i64(nodes)
        _check(lib().sem_adjoint_set_adjoint_receiver_nodes(self._h, len(n), _p(n, _I64P)))
        self.n_adj_rec = len(n)

    def adjoint_traces(self):
        out = np.zeros((self.n_steps, self.n_adj_rec), np.float32)
        _check(lib().sem_adjoint_get_adjoint_traces(self._h, _p(out, _F32P)))
        return out


def selftest_bounded_wait(limit_seconds: float = 0.05):
    """Run the bounded-wait self-test (sem_selftest_bounded_wait): a device wait on an mbarrier
    phase that nothing completes.  Returns (status code, seconds waited); the expected code is
    SEM_ERR_TIMEOUT."""
    waited = C.c_double(0.0)
    rc = lib().sem_selftest_bounded_wait(float(limit_seconds), C.byref(waited))
    return int(rc), float(waited.value)
