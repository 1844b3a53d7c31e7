"""Python face of the GB300 Demo4 SPH step, over the C ABI of
``include/sph_gb300.h``.

``Simulation`` mirrors the reference's ``BaseSimulation`` interface
(NBodySimulation/base.h:8-38) method by method, in snake_case, with the same
argument meaning.  The only compute path is the CUDA library
``libsph_gb300.so``; if it cannot be loaded or no CUDA device is present the
constructor raises -- there is no CPU fallback.
"""
from __future__ import annotations

import ctypes
import os
from typing import Dict, Optional, Sequence, Tuple

import numpy as np

from . import _build

_c = ctypes

SPH_OK = 0
SPH_ERR_INVALID_ARGUMENT = 1
SPH_ERR_CAPACITY = 2
SPH_ERR_CUDA = 3
SPH_ERR_DEVICE_OVERFLOW = 4
SPH_ERR_TIMEOUT = 5
SPH_ERR_NOT_SUPPORTED = 6
SPH_ERR_NO_DEVICE = 7


class Vec2(ctypes.Structure):
    _fields_ = [("x", _c.c_float), ("y", _c.c_float)]


class Domain(ctypes.Structure):
    """``sph_domain``: the reference's compile-time constants (sph.h:15-72)."""

    _fields_ = [
        ("width", _c.c_float), ("height", _c.c_float), ("cell_size", _c.c_float),
        ("max_particles", _c.c_uint32), ("max_cell_particles", _c.c_uint32), ("max_neighbors", _c.c_uint32),
        ("particle_radius", _c.c_float), ("collision_margin", _c.c_float),
        ("jitter_kernel_height", _c.c_float), ("jitter_scale", _c.c_float),
    ]

    def grid(self) -> Tuple[int, int]:
        w, h, cs = np.float32(self.width), np.float32(self.height), np.float32(self.cell_size)
        return int(w / cs), int(h / cs)


class Params(ctypes.Structure):
    """``sph_params`` = SPHParameters (sph.h:77-86), same member order."""

    _fields_ = [(name, _c.c_float) for name in (
        "kernel_height", "cell_size", "particle_spacing", "inv_kernel_height", "rest_density",
        "stiffness", "near_stiffness", "linear_viscosity", "quadratic_viscosity")]

    def as_array(self) -> np.ndarray:
        return np.array([getattr(self, f) for f, _ in self._fields_], np.float32)

    @classmethod
    def from_array(cls, a) -> "Params":
        p = cls()
        for (f, _), v in zip(cls._fields_, np.asarray(a, np.float32)):
            setattr(p, f, float(v))
        return p


class Stats(ctypes.Structure):
    """``sph_stats`` = SPHStatistics (sph.h:125-141)."""

    _fields_ = [
        ("min_particle_neighbor_count", _c.c_uint64), ("max_particle_neighbor_count", _c.c_uint64),
        ("min_cell_particle_count", _c.c_uint64), ("max_cell_particle_count", _c.c_uint64),
    ] + [(name, _c.c_float) for name in (
        "time_emitters", "time_integration", "time_viscosity_forces", "time_predict", "time_update_grid",
        "time_neighbor_search", "time_density_and_pressure", "time_delta_positions", "time_collisions")]


class StateView(ctypes.Structure):
    _fields_ = [
        ("count", _c.c_size_t), ("canonical_count", _c.c_size_t),
        ("grid_x", _c.c_int), ("grid_y", _c.c_int),
        ("pos", _c.c_void_p), ("prev", _c.c_void_p), ("vel", _c.c_void_p), ("acc", _c.c_void_p),
        ("dens", _c.c_void_p), ("press", _c.c_void_p),
        ("id", _c.c_void_p), ("cell", _c.c_void_p), ("cell_start", _c.c_void_p), ("cell_count", _c.c_void_p),
    ]


class ScenarioBody(ctypes.Structure):
    """``sph_scenario_body``: one AddPlane/AddCircle/AddLineSegment/AddPolygon."""

    _fields_ = [("type", _c.c_int), ("vertex_count", _c.c_int), ("normal", Vec2), ("distance", _c.c_float),
                ("center", Vec2), ("radius", _c.c_float), ("verts", Vec2 * 8)]


class ScenarioVolume(ctypes.Structure):
    _fields_ = [("center", Vec2), ("force", Vec2), ("count_x", _c.c_int), ("count_y", _c.c_int),
                ("spacing", _c.c_float)]


class ScenarioEmitter(ctypes.Structure):
    _fields_ = [("position", Vec2), ("direction", Vec2), ("radius", _c.c_float), ("speed", _c.c_float),
                ("rate", _c.c_float), ("duration", _c.c_float)]


class ScenarioDesc(ctypes.Structure):
    """``sph_scenario_desc``: the calls DemoApplication::LoadScenario
    (app.cpp:477-534) makes for one built-in scenario (sph.h:315-437)."""

    _fields_ = [("name", _c.c_char * 100), ("gravity", Vec2), ("params", Params),
                ("body_count", _c.c_uint32), ("bodies", ScenarioBody * 32),
                ("volume_count", _c.c_uint32), ("volumes", ScenarioVolume * 32),
                ("emitter_count", _c.c_uint32), ("emitters", ScenarioEmitter * 8)]


SPH_BODY_PLANE, SPH_BODY_CIRCLE, SPH_BODY_LINE_SEGMENT, SPH_BODY_POLYGON = 1, 2, 3, 4


class SpringParams(ctypes.Structure):
    """``sph_spring_params``: viscoelastic springs (Clavet et al. 2005)."""

    _fields_ = [("enabled", _c.c_int), ("yield_ratio", _c.c_float), ("plasticity", _c.c_float),
                ("stiffness", _c.c_float), ("max_per_particle", _c.c_int)]


SPRING_SLOTS = 16
#: Warps per task of the ordered sweeps' launch shapes, (wide, lean) and for
#: the delta sweep (wide, lean, mid, tri, quad, dense): the values
#: ``sph_set_sweep_shape`` accepts (csrc/sph_kernels.cuh).
VISC_WARPS = (4, 5)
DELTA_WARPS = (12, 2, 8, 3, 4, 16)


class BodyDesc(ctypes.Structure):
    """``sph_body_desc``: one collision body of a batched scene."""

    _fields_ = [("type", _c.c_int), ("vertex_count", _c.c_size_t), ("a", Vec2), ("b", Vec2),
                ("value", _c.c_float), ("verts", Vec2 * 8)]


class SceneDesc(ctypes.Structure):
    """``sph_scene_desc``: one scene of a batch (domain, parameters, gravity,
    particles in AddParticle order, bodies)."""

    _fields_ = [("domain", Domain), ("params", Params), ("gravity", Vec2), ("particle_count", _c.c_size_t),
                ("positions", _c.c_void_p), ("forces", _c.c_void_p), ("body_count", _c.c_size_t),
                ("bodies", _c.c_void_p)]


SPH_BODY_PLANE, SPH_BODY_CIRCLE, SPH_BODY_SEGMENT, SPH_BODY_POLYGON = 1, 2, 3, 4


class SphError(RuntimeError):
    def __init__(self, status: int, what: str):
        self.status = status
        detail = ""
        if status == SPH_ERR_CUDA and _LIB is not None:
            detail = ": " + _LIB.sph_last_error().decode(errors="replace")
        super().__init__("%s failed: %s (status %d)%s" % (what, _status_string(status), status, detail))


_LIB = None


def _status_string(status: int) -> str:
    if _LIB is None:
        return "status"
    return _LIB.sph_status_string(status).decode()


def library_path() -> str:
    return _build.LIB_PATH


def load_library(build_if_missing: bool = True):
    """Load ``libsph_gb300.so`` (building it first if allowed)."""
    global _LIB
    if _LIB is not None:
        return _LIB
    path = _build.LIB_PATH
    if not os.path.exists(path) or not _build.up_to_date():
        if not build_if_missing:
            raise FileNotFoundError(path)
        _build.build()
    lib = ctypes.CDLL(path)
    P = _c.POINTER
    vp = _c.c_void_p
    sig = {
        "sph_reference_domain": [P(Domain)],
        "sph_default_params": [P(Params)],
        "sph_create": [P(Domain), _c.c_int, P(vp)],
        "sph_destroy": [vp],
        "sph_reset_stats": [vp],
        "sph_clear_bodies": [vp],
        "sph_clear_particles": [vp],
        "sph_clear_emitters": [vp],
        "sph_add_plane": [vp, Vec2, _c.c_float],
        "sph_add_circle": [vp, Vec2, _c.c_float],
        "sph_add_line_segment": [vp, Vec2, Vec2],
        "sph_add_polygon": [vp, _c.c_size_t, vp],
        "sph_add_particle": [vp, Vec2, Vec2, P(_c.c_size_t)],
        "sph_add_particles": [vp, _c.c_size_t, vp, vp, P(_c.c_size_t)],
        "sph_add_volume": [vp, Vec2, Vec2, _c.c_int, _c.c_int, _c.c_float],
        "sph_add_emitter": [vp, Vec2, Vec2, _c.c_float, _c.c_float, _c.c_float, _c.c_float],
        "sph_update": [vp, _c.c_float],
        "sph_add_external_forces": [vp, Vec2],
        "sph_clear_external_force": [vp],
        "sph_get_particle_count": [vp, P(_c.c_size_t)],
        "sph_set_gravity": [vp, Vec2],
        "sph_get_params": [vp, P(Params)],
        "sph_get_stats": [vp, P(Stats)],
        "sph_set_params": [vp, P(Params)],
        "sph_set_multithreading": [vp, _c.c_int],
        "sph_is_multithreading_supported": [vp, P(_c.c_int)],
        "sph_is_multithreading": [vp, P(_c.c_int)],
        "sph_get_worker_thread_count": [vp, P(_c.c_size_t)],
        "sph_read_particles": [vp, _c.c_size_t, vp, vp, vp, vp, vp, vp],
        "sph_state_info": [vp, P(_c.c_size_t), P(_c.c_size_t), P(_c.c_int), P(_c.c_int)],
        "sph_dump_state": [vp, P(StateView)],
        "sph_load_state": [vp, P(StateView)],
        "sph_get_stream": [vp, P(vp)],
        "sph_device_arrays": [vp, P(vp), P(vp), P(vp), P(vp)],
        "sph_particle_colors": [vp, _c.c_size_t, vp],
        "sph_render_points": [vp, _c.c_int, _c.c_int, vp],
        "sph_scenario_count": [P(_c.c_int)],
        "sph_scenario_describe": [_c.c_int, P(ScenarioDesc)],
        "sph_load_scenario": [vp, _c.c_int],
        "sph_synchronize": [vp],
        "sph_kernel_launches": [vp, P(_c.c_uint64)],
        "sph_use_graphs": [vp, _c.c_int],
        "sph_set_reference_order": [vp, _c.c_int],
        "sph_get_reference_order": [vp, P(_c.c_int)],
        "sph_set_wait_limit": [vp, _c.c_double],
        "sph_test_hold_task": [vp, _c.c_int, _c.c_int],
        "sph_autotune": [vp, _c.c_float, vp],
        "sph_get_sweep_shape": [vp, vp],
        "sph_set_sweep_shape": [vp, vp],
        "sph_set_adaptive_shapes": [vp, _c.c_int],
        "sph_last_sweep_shape": [vp, vp],
        "sph_set_springs": [vp, P(SpringParams)],
        "sph_get_spring_count": [vp, P(_c.c_uint64)],
        "sph_dump_springs": [vp, _c.c_size_t, vp, vp, vp],
        "sph_load_springs": [vp, _c.c_size_t, vp, vp, vp],
        "sph_mpnn_create": [_c.c_int, _c.c_size_t, _c.c_uint64, P(vp)],
        "sph_mpnn_destroy": [vp],
        "sph_mpnn_param_count": [P(_c.c_size_t)],
        "sph_mpnn_get_params": [vp, vp],
        "sph_mpnn_set_params": [vp, vp],
        "sph_mpnn_set_edge_path": [vp, _c.c_int],
        "sph_mpnn_get_edge_path": [vp, P(_c.c_int)],
        "sph_mpnn_capture": [vp, vp, _c.c_float, _c.c_int],
        "sph_mpnn_sample_count": [vp, P(_c.c_size_t)],
        "sph_mpnn_clear_samples": [vp],
        "sph_mpnn_sample_info": [vp, _c.c_size_t, P(_c.c_size_t), P(_c.c_int), P(_c.c_int), P(_c.c_float)],
        "sph_mpnn_read_sample": [vp, _c.c_size_t, vp, vp, vp, vp, vp],
        "sph_mpnn_eval": [vp, _c.c_size_t, P(_c.c_float), vp],
        "sph_mpnn_gradient": [vp, _c.c_size_t, P(_c.c_float), vp],
        "sph_mpnn_train_step": [vp, _c.c_size_t, _c.c_float, P(_c.c_float)],
        "sph_learned_frame": [vp, vp, _c.c_float, _c.c_int, _c.c_float, P(_c.c_int), P(_c.c_float)],
        "sph_batch_create": [vp, _c.c_size_t, _c.c_int, P(vp)],
        "sph_batch_scene_count": [vp, P(_c.c_size_t)],
        "sph_batch_read_particles": [vp, _c.c_size_t, _c.c_size_t, vp, vp, vp, vp],
        "sph_batch_get_stats": [vp, _c.c_size_t, P(Stats)],
        "sph_batch_state_info": [vp, _c.c_size_t, P(_c.c_size_t), P(_c.c_size_t), P(_c.c_int), P(_c.c_int)],
        "sph_batch_dump_state": [vp, _c.c_size_t, P(StateView)],
    }
    for name, args in sig.items():
        fn = getattr(lib, name)
        fn.argtypes = args
        fn.restype = _c.c_int
    lib.sph_status_string.argtypes = [_c.c_int]
    lib.sph_status_string.restype = _c.c_char_p
    lib.sph_last_error.argtypes = []
    lib.sph_last_error.restype = _c.c_char_p
    _LIB = lib
    return lib


#: Exported C symbols, in the order include/sph_gb300.h declares them.
C_SYMBOLS = (
    "sph_reference_domain", "sph_default_params", "sph_status_string", "sph_last_error", "sph_create",
    "sph_destroy",
    "sph_reset_stats", "sph_clear_bodies", "sph_clear_particles", "sph_clear_emitters", "sph_add_plane",
    "sph_add_circle", "sph_add_line_segment", "sph_add_polygon", "sph_add_particle", "sph_add_particles",
    "sph_add_volume", "sph_add_emitter", "sph_update", "sph_add_external_forces", "sph_clear_external_force",
    "sph_get_particle_count", "sph_set_gravity", "sph_get_params", "sph_get_stats", "sph_set_params",
    "sph_set_multithreading", "sph_is_multithreading_supported", "sph_is_multithreading",
    "sph_get_worker_thread_count", "sph_read_particles", "sph_state_info", "sph_dump_state", "sph_load_state",
    "sph_get_stream", "sph_device_arrays", "sph_particle_colors", "sph_render_points", "sph_scenario_count",
    "sph_scenario_describe", "sph_load_scenario", "sph_synchronize",
    "sph_kernel_launches",
    "sph_use_graphs", "sph_autotune", "sph_set_reference_order", "sph_get_reference_order",
    "sph_set_wait_limit", "sph_test_hold_task", "sph_get_sweep_shape", "sph_set_sweep_shape",
    "sph_set_adaptive_shapes", "sph_last_sweep_shape", "sph_set_springs", "sph_get_spring_count", "sph_dump_springs", "sph_load_springs",
    "sph_mpnn_create", "sph_mpnn_destroy", "sph_mpnn_param_count", "sph_mpnn_get_params", "sph_mpnn_set_params",
    "sph_mpnn_set_edge_path", "sph_mpnn_get_edge_path", "sph_mpnn_capture", "sph_mpnn_sample_count", "sph_mpnn_clear_samples", "sph_mpnn_sample_info",
    "sph_mpnn_read_sample", "sph_mpnn_eval", "sph_mpnn_gradient", "sph_mpnn_train_step", "sph_learned_frame",
    "sph_batch_create", "sph_batch_scene_count", "sph_batch_read_particles", "sph_batch_get_stats",
    "sph_batch_state_info", "sph_batch_dump_state",
)


def _check(status: int, what: str) -> None:
    if status != SPH_OK:
        raise SphError(status, what)


def scenario_count() -> int:
    """Number of the reference's built-in scenarios (SPHScenarios[], sph.h:315-437)."""
    n = _c.c_int()
    _check(load_library().sph_scenario_count(_c.byref(n)), "sph_scenario_count")
    return n.value


def scenario_describe(index: int) -> ScenarioDesc:
    """The calls LoadScenario (app.cpp:477-534) makes for scenario ``index``."""
    d = ScenarioDesc()
    _check(load_library().sph_scenario_describe(int(index), _c.byref(d)), "sph_scenario_describe")
    return d


def reference_domain() -> Domain:
    d = Domain()
    _check(load_library().sph_reference_domain(_c.byref(d)), "sph_reference_domain")
    return d


def default_params() -> Params:
    p = Params()
    _check(load_library().sph_default_params(_c.byref(p)), "sph_default_params")
    return p


def _v(x, y) -> Vec2:
    return Vec2(float(x), float(y))


def _f2(a: np.ndarray) -> np.ndarray:
    return np.ascontiguousarray(a, dtype=np.float32).reshape(-1, 2)


def _state_arrays(n: int, n0: int, gx: int, gy: int):
    """Host arrays for one dump and the ``StateView`` pointing at them."""
    st = {k: np.zeros((n, 2), np.float32) for k in ("pos", "prev", "vel", "acc", "dens", "press")}
    st["id"] = np.zeros(n, np.int32)
    st["cell"] = np.zeros(n, np.int32)
    st["cell_start"] = np.zeros(gx * gy, np.int32)
    st["cell_count"] = np.zeros(gx * gy, np.int32)
    v = StateView(count=n, canonical_count=n0, grid_x=gx, grid_y=gy)
    for k in ("pos", "prev", "vel", "acc", "dens", "press", "id", "cell", "cell_start", "cell_count"):
        setattr(v, k, st[k].ctypes.data)
    st["canonical_count"] = n0
    st["grid"] = (gx, gy)
    return st, v


def _state_view_of(out: Dict[str, np.ndarray], n: int, n0: int, gx: int, gy: int):
    """The ``StateView`` of caller-given host arrays for one dump (checked
    against the state's sizes)."""
    shapes = {k: ((n, 2), np.float32) for k in ("pos", "prev", "vel", "acc", "dens", "press")}
    shapes.update(id=((n,), np.int32), cell=((n,), np.int32), cell_start=((gx * gy,), np.int32),
                  cell_count=((gx * gy,), np.int32))
    v = StateView(count=n, canonical_count=n0, grid_x=gx, grid_y=gy)
    for k, (shape, dtype) in shapes.items():
        a = out[k]
        if a.shape != shape or a.dtype != dtype or not a.flags["C_CONTIGUOUS"] or not a.flags["WRITEABLE"]:
            raise ValueError("dump_state out[%r]: want a writeable contiguous %s array of shape %s"
                             % (k, np.dtype(dtype).name, shape))
        setattr(v, k, a.ctypes.data)
    out["canonical_count"] = n0
    out["grid"] = (gx, gy)
    return out, v


class Simulation:
    """GB300 Demo4 particle simulation (``BaseSimulation``, base.h:8-38)."""

    def __init__(self, domain: Optional[Domain] = None, device: int = 0):
        self._lib = load_library()
        self.domain = domain if domain is not None else reference_domain()
        h = _c.c_void_p()
        _check(self._lib.sph_create(_c.byref(self.domain), int(device), _c.byref(h)), "sph_create")
        self._h = h
        self.grid = self.domain.grid()

    def close(self) -> None:
        if getattr(self, "_h", None):
            self._lib.sph_destroy(self._h)
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _call(self, name: str, *args) -> None:
        _check(getattr(self._lib, name)(self._h, *args), name)

    # --- BaseSimulation ------------------------------------------------------
    def reset_stats(self):
        self._call("sph_reset_stats")

    def clear_bodies(self):
        self._call("sph_clear_bodies")

    def clear_particles(self):
        self._call("sph_clear_particles")

    def clear_emitters(self):
        self._call("sph_clear_emitters")

    def add_plane(self, normal, distance):
        self._call("sph_add_plane", _v(*normal), float(distance))

    def add_circle(self, pos, radius):
        self._call("sph_add_circle", _v(*pos), float(radius))

    def add_line_segment(self, a, b):
        self._call("sph_add_line_segment", _v(*a), _v(*b))

    def add_polygon(self, verts):
        v = _f2(verts)
        self._call("sph_add_polygon", len(v), v.ctypes.data_as(_c.c_void_p))

    def add_particle(self, position, force=(0.0, 0.0)) -> int:
        out = _c.c_size_t()
        self._call("sph_add_particle", _v(*position), _v(*force), _c.byref(out))
        return out.value

    def add_particles(self, positions, forces=None) -> int:
        p = _f2(positions)
        f = _f2(forces) if forces is not None else None
        first = _c.c_size_t()
        self._call("sph_add_particles", len(p), p.ctypes.data_as(_c.c_void_p),
                   f.ctypes.data_as(_c.c_void_p) if f is not None else None, _c.byref(first))
        return first.value

    def add_volume(self, center, force, count_x, count_y, spacing):
        self._call("sph_add_volume", _v(*center), _v(*force), int(count_x), int(count_y), float(spacing))

    def add_emitter(self, position, direction, radius, speed, rate, duration):
        self._call("sph_add_emitter", _v(*position), _v(*direction), float(radius), float(speed), float(rate),
                   float(duration))

    def update(self, delta_time: float):
        self._call("sph_update", float(np.float32(delta_time)))

    def add_external_forces(self, force):
        self._call("sph_add_external_forces", _v(*force))

    def clear_external_force(self):
        self._call("sph_clear_external_force")

    def get_particle_count(self) -> int:
        out = _c.c_size_t()
        self._call("sph_get_particle_count", _c.byref(out))
        return out.value

    def set_gravity(self, gravity):
        self._call("sph_set_gravity", _v(*gravity))

    def get_params(self) -> Params:
        p = Params()
        self._call("sph_get_params", _c.byref(p))
        return p

    def set_params(self, params: Params):
        self._call("sph_set_params", _c.byref(params))

    def get_stats(self) -> Stats:
        s = Stats()
        self._call("sph_get_stats", _c.byref(s))
        return s

    def set_multithreading(self, value: bool):
        self._call("sph_set_multithreading", 1 if value else 0)

    def is_multithreading_supported(self) -> bool:
        out = _c.c_int()
        self._call("sph_is_multithreading_supported", _c.byref(out))
        return bool(out.value)

    def is_multithreading(self) -> bool:
        out = _c.c_int()
        self._call("sph_is_multithreading", _c.byref(out))
        return bool(out.value)

    def get_worker_thread_count(self) -> int:
        out = _c.c_size_t()
        self._call("sph_get_worker_thread_count", _c.byref(out))
        return out.value

    # --- data access ------------------------------------------------------------
    def read_particles(self, fields: Sequence[str] = ("pos", "prev", "vel", "acc", "dens", "press")
                       ) -> Dict[str, np.ndarray]:
        """Particle arrays in AddParticle order, as (n, 2) float32 arrays."""
        n = self.get_particle_count()
        out = {f: np.zeros((n, 2), np.float32) for f in fields}
        ptr = lambda f: out[f].ctypes.data_as(_c.c_void_p) if f in out else None
        self._call("sph_read_particles", n, ptr("pos"), ptr("prev"), ptr("vel"), ptr("acc"), ptr("dens"),
                   ptr("press"))
        return out

    def state_info(self) -> Tuple[int, int, int, int]:
        n, n0 = _c.c_size_t(), _c.c_size_t()
        gx, gy = _c.c_int(), _c.c_int()
        self._call("sph_state_info", _c.byref(n), _c.byref(n0), _c.byref(gx), _c.byref(gy))
        return n.value, n0.value, gx.value, gy.value

    def dump_state(self, out: Optional[Dict[str, np.ndarray]] = None) -> Dict[str, np.ndarray]:
        """Full state in the internal numbering (see sph_dump_state).  With
        ``out`` (arrays of a previous dump's keys, shapes and types, e.g. in
        pinned host memory) the state is copied into those arrays."""
        n, n0, gx, gy = self.state_info()
        st, v = _state_arrays(n, n0, gx, gy) if out is None else _state_view_of(out, n, n0, gx, gy)
        self._call("sph_dump_state", _c.byref(v))
        return st

    def load_state(self, st: Dict[str, np.ndarray]) -> None:
        n = len(st["pos"])
        gx, gy = self.grid
        arrs = {k: np.ascontiguousarray(st[k], np.float32).reshape(-1, 2)
                for k in ("pos", "prev", "vel", "acc", "dens", "press")}
        for k in ("id", "cell", "cell_start", "cell_count"):
            arrs[k] = np.ascontiguousarray(st[k], np.int32)
        v = StateView(count=n, canonical_count=int(st["canonical_count"]), grid_x=gx, grid_y=gy)
        for k, a in arrs.items():
            setattr(v, k, a.ctypes.data)
        self._call("sph_load_state", _c.byref(v))

    def load_scenario(self, index: int):
        """DemoApplication::LoadScenario (app.cpp:477-534) for built-in
        scenario ``index``; use the reference domain."""
        self._call("sph_load_scenario", int(index))

    def particle_colors(self) -> np.ndarray:
        """RGBA of every particle in AddParticle order: SPHGetParticleColor
        (sph.h:683-695), as Demo4's Render colours its points."""
        n = self.get_particle_count()
        out = np.zeros((n, 4), np.float32)
        self._call("sph_particle_colors", n, out.ctypes.data)
        return out

    def render_points(self, width: int, height: int) -> np.ndarray:
        """Headless point image of the box: (height, width, 4) uint8, row 0 at
        the top; each particle colours the pixel under it."""
        out = np.zeros((height, width, 4), np.uint8)
        self._call("sph_render_points", int(width), int(height), out.ctypes.data)
        return out

    def stream(self) -> int:
        out = _c.c_void_p()
        self._call("sph_get_stream", _c.byref(out))
        return out.value or 0

    def synchronize(self):
        self._call("sph_synchronize")

    def kernel_launches(self) -> int:
        out = _c.c_uint64()
        self._call("sph_kernel_launches", _c.byref(out))
        return out.value

    def use_graphs(self, enable: bool = True):
        """Replay repeated updates from a per-step CUDA graph (default on)."""
        self._call("sph_use_graphs", 1 if enable else 0)

    def set_reference_order(self, enable: bool = True) -> None:
        """Visit particles in AddParticle order in both ordered passes and the
        grid update, as the reference's own Update does, so that free runs
        reproduce the reference's trajectory (see sph_set_reference_order)."""
        self._call("sph_set_reference_order", 1 if enable else 0)

    def reference_order(self) -> bool:
        out = _c.c_int()
        self._call("sph_get_reference_order", _c.byref(out))
        return bool(out.value)

    def set_wait_limit(self, seconds: float) -> None:
        """Device-side waits of the ordered sweeps give up after ``seconds``
        (default 2); a wait that runs out makes the next synchronising call
        raise with SPH_ERR_TIMEOUT (see sph_set_wait_limit)."""
        self._call("sph_set_wait_limit", float(seconds))

    def test_hold_task(self, sweep: int, claim: int) -> None:
        """Tests of the timeout path only: the task claimed at position
        ``claim`` of sweep ``sweep`` (0 viscosity, 1 delta) never publishes
        that it is done; -1 turns it off (sph_test_hold_task)."""
        self._call("sph_test_hold_task", int(sweep), int(claim))

    def autotune(self, delta_time: float) -> Tuple[int, int, int, int]:
        """Pick the sweeps' launch shapes by timing (state kept); returns
        (viscosity warps, viscosity blocks, delta warps, delta blocks)."""
        shape = np.zeros(4, np.int32)
        self._call("sph_autotune", float(np.float32(delta_time)), shape.ctypes.data)
        return tuple(int(v) for v in shape)

    def sweep_shape(self) -> Tuple[int, int, int, int]:
        """(viscosity warps, viscosity blocks, delta warps, delta blocks); the
        warp counts name the shapes (``VISC_WARPS``, ``DELTA_WARPS``)."""
        shape = np.zeros(4, np.int32)
        self._call("sph_get_sweep_shape", shape.ctypes.data)
        return tuple(int(v) for v in shape)

    def set_sweep_shape(self, shape) -> None:
        a = np.ascontiguousarray(shape, np.int32)
        self._call("sph_set_sweep_shape", a.ctypes.data)

    def set_adaptive_shapes(self, enable: bool = True) -> None:
        """Dense states run the staging-safe sweep shapes (on by default)."""
        self._call("sph_set_adaptive_shapes", 1 if enable else 0)

    def last_sweep_shape(self) -> Tuple[int, int, int, int]:
        """The sweep shapes the last update ran with."""
        shape = np.zeros(4, np.int32)
        self._call("sph_last_sweep_shape", shape.ctypes.data)
        return tuple(int(v) for v in shape)

    # --- viscoelastic springs (no reference counterpart) ----------------------
    def set_springs(self, enabled: bool = True, yield_ratio: float = 0.1, plasticity: float = 0.3,
                    stiffness: float = 0.3, max_per_particle: int = SPRING_SLOTS):
        p = SpringParams(1 if enabled else 0, float(yield_ratio), float(plasticity), float(stiffness),
                         int(max_per_particle))
        self._call("sph_set_springs", _c.byref(p))

    def spring_count(self) -> int:
        out = _c.c_uint64()
        self._call("sph_get_spring_count", _c.byref(out))
        return out.value

    def dump_springs(self, out: Optional[Dict[str, np.ndarray]] = None):
        """(count (n,), partner (n, 16) internal numbers or -1, rest (n, 16)).
        With ``out`` (keys count, partner, rest of those shapes and types,
        e.g. in pinned host memory) the tables are copied into those arrays."""
        n = self.get_particle_count()
        if out is not None:
            count, partner, rest = out["count"], out["partner"], out["rest"]
            for a, shape, dtype in ((count, (n,), np.int32), (partner, (n, SPRING_SLOTS), np.int32),
                                    (rest, (n, SPRING_SLOTS), np.float32)):
                if a.shape != shape or a.dtype != dtype or not a.flags["C_CONTIGUOUS"] or not a.flags["WRITEABLE"]:
                    raise ValueError("dump_springs out: want writeable contiguous %s arrays of shape %s"
                                     % (np.dtype(dtype).name, shape))
        else:
            count = np.zeros(n, np.int32)
            partner = np.zeros((n, SPRING_SLOTS), np.int32)
            rest = np.zeros((n, SPRING_SLOTS), np.float32)
        self._call("sph_dump_springs", n, count.ctypes.data, partner.ctypes.data, rest.ctypes.data)
        return count, partner, rest

    def learned_frame(self, model: "Mpnn", frame_dt: float, substeps: int = 4, bound: float = 0.01):
        """One frame by the network, judged by the plain method (see
        ``sph_learned_frame``); returns (learned frame used, density error)."""
        used = _c.c_int()
        err = _c.c_float()
        self._call("sph_learned_frame", model._h, float(np.float32(frame_dt)), int(substeps), float(bound),
                   _c.byref(used), _c.byref(err))
        return bool(used.value), float(err.value)

    def load_springs(self, count, partner, rest):
        n = len(count)
        count = np.ascontiguousarray(count, np.int32)
        partner = np.ascontiguousarray(partner, np.int32).reshape(n, SPRING_SLOTS)
        rest = np.ascontiguousarray(rest, np.float32).reshape(n, SPRING_SLOTS)
        self._call("sph_load_springs", n, count.ctypes.data, partner.ctypes.data, rest.ctypes.data)


def _scene_desc(scene, keep: list) -> SceneDesc:
    """A ``SceneDesc`` for an object with the ``scenes.Scene`` fields; the
    arrays it points into are appended to ``keep``."""
    d = SceneDesc()
    d.domain = scene.domain()
    d.params = Params.from_array(scene.params)
    d.gravity = _v(*scene.gravity)
    pos = _f2(scene.positions)
    keep.append(pos)
    d.particle_count = len(pos)
    d.positions = pos.ctypes.data if len(pos) else None
    d.forces = None
    bodies = []
    for nx, ny, dist in scene.planes:
        bodies.append(BodyDesc(type=SPH_BODY_PLANE, a=_v(nx, ny), value=float(dist)))
    for x, y, r in scene.circles:
        bodies.append(BodyDesc(type=SPH_BODY_CIRCLE, a=_v(x, y), value=float(r)))
    for ax, ay, bx, by in scene.segments:
        bodies.append(BodyDesc(type=SPH_BODY_SEGMENT, a=_v(ax, ay), b=_v(bx, by)))
    for verts in getattr(scene, "polygons", ()):
        b = BodyDesc(type=SPH_BODY_POLYGON, vertex_count=len(verts))
        for k, (x, y) in enumerate(verts):
            b.verts[k] = _v(x, y)
        bodies.append(b)
    arr = (BodyDesc * max(len(bodies), 1))(*bodies)
    keep.append(arr)
    d.body_count = len(bodies)
    d.bodies = _c.addressof(arr) if bodies else None
    return d


class BatchSimulation:
    """Many independent Demo4 scenes advanced by one update (the batched
    form of the step; no single reference counterpart).  Each scene's update
    equals a single-scene ``Simulation`` holding the same state, bit for bit.
    Scenes are fixed at creation: bodies first in the order planes, circles,
    segments, polygons (as ``Scene.apply`` adds them), then particles."""

    def __init__(self, scenes, device: int = 0):
        self._lib = load_library()
        keep: list = []
        descs = [_scene_desc(sc, keep) for sc in scenes]
        arr = (SceneDesc * len(descs))(*descs)
        h = _c.c_void_p()
        _check(self._lib.sph_batch_create(_c.addressof(arr), len(descs), int(device), _c.byref(h)),
               "sph_batch_create")
        self._h = h
        self.counts = [int(d.particle_count) for d in descs]
        self.grids = [d.domain.grid() for d in descs]

    def close(self) -> None:
        if getattr(self, "_h", None):
            self._lib.sph_destroy(self._h)
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _call(self, name: str, *args) -> None:
        _check(getattr(self._lib, name)(self._h, *args), name)

    @property
    def scene_count(self) -> int:
        out = _c.c_size_t()
        self._call("sph_batch_scene_count", _c.byref(out))
        return out.value

    def update(self, delta_time: float):
        self._call("sph_update", float(np.float32(delta_time)))

    def get_particle_count(self) -> int:
        out = _c.c_size_t()
        self._call("sph_get_particle_count", _c.byref(out))
        return out.value

    def get_stats(self, scene: int) -> Stats:
        s = Stats()
        self._call("sph_batch_get_stats", int(scene), _c.byref(s))
        return s

    def read_particles(self, scene: int, fields: Sequence[str] = ("pos", "vel", "dens", "press")
                       ) -> Dict[str, np.ndarray]:
        """One scene's arrays in its AddParticle order, as (n, 2) float32."""
        n = self.counts[scene]
        out = {f: np.zeros((n, 2), np.float32) for f in fields}
        ptr = lambda f: out[f].ctypes.data_as(_c.c_void_p) if f in out else None
        self._call("sph_batch_read_particles", int(scene), n, ptr("pos"), ptr("vel"), ptr("dens"), ptr("press"))
        return out

    def state_info(self, scene: int) -> Tuple[int, int, int, int]:
        n, n0 = _c.c_size_t(), _c.c_size_t()
        gx, gy = _c.c_int(), _c.c_int()
        self._call("sph_batch_state_info", int(scene), _c.byref(n), _c.byref(n0), _c.byref(gx), _c.byref(gy))
        return n.value, n0.value, gx.value, gy.value

    def dump_state(self, scene: int) -> Dict[str, np.ndarray]:
        """One scene's state in scene-local numbers and cells (the layout of
        ``Simulation.dump_state``)."""
        n, n0, gx, gy = self.state_info(scene)
        st, v = _state_arrays(n, n0, gx, gy)
        self._call("sph_batch_dump_state", int(scene), _c.byref(v))
        return st

    def stream(self) -> int:
        out = _c.c_void_p()
        self._call("sph_get_stream", _c.byref(out))
        return out.value or 0

    def synchronize(self):
        self._call("sph_synchronize")

    def kernel_launches(self) -> int:
        out = _c.c_uint64()
        self._call("sph_kernel_launches", _c.byref(out))
        return out.value

    def use_graphs(self, enable: bool = True):
        """Replay repeated updates from a per-step CUDA graph (default on)."""
        self._call("sph_use_graphs", 1 if enable else 0)

    def autotune(self, delta_time: float) -> Tuple[int, int, int, int]:
        """Pick the sweeps' launch shapes by timing (state kept); returns
        (viscosity warps, viscosity blocks, delta warps, delta blocks)."""
        shape = np.zeros(4, np.int32)
        self._call("sph_autotune", float(np.float32(delta_time)), shape.ctypes.data)
        return tuple(int(v) for v in shape)

    def sweep_shape(self) -> Tuple[int, int, int, int]:
        shape = np.zeros(4, np.int32)
        self._call("sph_get_sweep_shape", shape.ctypes.data)
        return tuple(int(v) for v in shape)

    def set_sweep_shape(self, shape) -> None:
        a = np.ascontiguousarray(shape, np.int32)
        self._call("sph_set_sweep_shape", a.ctypes.data)


class Mpnn:
    """The learned frame's message-passing network (``include/sph_mpnn.h``):
    parameters, training samples captured from plain frames, and training on
    the GPU by the library's own forward and backward kernels."""

    def __init__(self, max_particles: int, device: int = 0, seed: int = 1):
        self._lib = load_library()
        h = _c.c_void_p()
        _check(self._lib.sph_mpnn_create(int(device), int(max_particles), int(seed), _c.byref(h)), "sph_mpnn_create")
        self._h = h

    def close(self) -> None:
        if getattr(self, "_h", None):
            self._lib.sph_mpnn_destroy(self._h)
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _call(self, name: str, *args) -> None:
        _check(getattr(self._lib, name)(self._h, *args), name)

    @staticmethod
    def param_count() -> int:
        out = _c.c_size_t()
        _check(load_library().sph_mpnn_param_count(_c.byref(out)), "sph_mpnn_param_count")
        return out.value

    def get_params(self) -> np.ndarray:
        p = np.zeros(self.param_count(), np.float32)
        self._call("sph_mpnn_get_params", p.ctypes.data)
        return p

    def set_params(self, p) -> None:
        p = np.ascontiguousarray(p, np.float32)
        assert p.size == self.param_count()
        self._call("sph_mpnn_set_params", p.ctypes.data)

    #: Edge-layer paths of ``sph_mpnn_set_edge_path``.
    EDGE_TENSOR_CORES, EDGE_CUDA_CORES = 0, 1

    @property
    def edge_path(self) -> int:
        out = _c.c_int()
        self._call("sph_mpnn_get_edge_path", _c.byref(out))
        return out.value

    @edge_path.setter
    def edge_path(self, path: int) -> None:
        self._call("sph_mpnn_set_edge_path", int(path))

    def capture(self, sim: Simulation, frame_dt: float, substeps: int = 4) -> None:
        _check(self._lib.sph_mpnn_capture(sim._h, self._h, float(np.float32(frame_dt)), int(substeps)),
               "sph_mpnn_capture")

    @property
    def sample_count(self) -> int:
        out = _c.c_size_t()
        self._call("sph_mpnn_sample_count", _c.byref(out))
        return out.value

    def clear_samples(self) -> None:
        self._call("sph_mpnn_clear_samples")

    def sample(self, index: int) -> Dict[str, np.ndarray]:
        n, gx, gy, h = _c.c_size_t(), _c.c_int(), _c.c_int(), _c.c_float()
        self._call("sph_mpnn_sample_info", int(index), _c.byref(n), _c.byref(gx), _c.byref(gy), _c.byref(h))
        n = n.value
        out = {k: np.zeros((n, 2), np.float32) for k in ("pos", "z0", "target")}
        out["cell_start"] = np.zeros(gx.value * gy.value, np.int32)
        out["cell_count"] = np.zeros(gx.value * gy.value, np.int32)
        self._call("sph_mpnn_read_sample", int(index), out["pos"].ctypes.data, out["z0"].ctypes.data,
                   out["target"].ctypes.data, out["cell_start"].ctypes.data, out["cell_count"].ctypes.data)
        out["grid"] = (gx.value, gy.value)
        out["h"] = h.value
        return out

    def eval(self, index: int, want_u: bool = False):
        loss = _c.c_float()
        u = None
        if want_u:
            n = _c.c_size_t()
            self._call("sph_mpnn_sample_info", int(index), _c.byref(n), None, None, None)
            u = np.zeros((n.value, 2), np.float32)
        self._call("sph_mpnn_eval", int(index), _c.byref(loss), u.ctypes.data if u is not None else None)
        return (loss.value, u) if want_u else loss.value

    def gradient(self, index: int):
        loss = _c.c_float()
        g = np.zeros(self.param_count(), np.float32)
        self._call("sph_mpnn_gradient", int(index), _c.byref(loss), g.ctypes.data)
        return loss.value, g

    def train_step(self, index: int, lr: float) -> float:
        loss = _c.c_float()
        self._call("sph_mpnn_train_step", int(index), float(lr), _c.byref(loss))
        return loss.value
