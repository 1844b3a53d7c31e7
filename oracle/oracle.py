"""Test infrastructure: ctypes front end of the two CPU oracles.

Only tests, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline leg may
import this module; the product never does.

* ``ReferenceSim`` drives the reference's own ``Demo4::ParticleSimulation``
  (NBodySimulation/demo4.cpp), compiled headless into ``oracle/_ref/libsphref.so``
  by ``oracle/Makefile`` where the reference tree exists.
* ``OracleSim`` drives the CPU restatement of the same step
  (``oracle/sph_oracle.cpp``) in FP32 or FP64, with the domain and capacities
  as runtime values.

Both expose the reference's ``BaseSimulation`` calls (base.h:8-38) plus full
state get/set for teacher forcing.  The state dictionary used everywhere in
the tests is::

    pos, prev, acc, vel, dens, press : (n, 2) float arrays
    cell          : (n, 2) int32   -- ParticleIndex::cellIndex
    index_in_cell : (n,)   uint64  -- ParticleIndex::indexInCell
    nb_count      : (n,)   uint64  -- ParticleIndex::neighborCount
    nb_flat       : (sum nb_count,) uint64, lists in particle order
    cell_count    : (gx*gy,) uint64 -- Cell::count, cells numbered y*gx+x
    cell_flat     : (sum cell_count,) uint64, cell arrays in cell order
"""
from __future__ import annotations

import ctypes
import os
import subprocess
from typing import Dict, Optional

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REF_DIR = os.path.join(HERE, "_ref")


def _reference_tree() -> str:
    """The reference's source tree: $SPH_REFERENCE_TREE, else the Makefile's
    REF default (the one recipe that names where the tree lies)."""
    env = os.environ.get("SPH_REFERENCE_TREE")
    if env:
        return env
    try:
        with open(os.path.join(HERE, "Makefile")) as f:
            for line in f:
                if line.startswith("REF ?="):
                    return line.split("?=", 1)[1].strip()
    except OSError:
        pass
    return ""


REFERENCE_TREE = _reference_tree()


def reference_tree_present() -> bool:
    return bool(REFERENCE_TREE) and os.path.isdir(os.path.join(REFERENCE_TREE, "NBodySimulation"))

_c = ctypes
_vp = _c.c_void_p
_f = _c.c_float
_u64 = _c.c_uint64
_i = _c.c_int
_fp = _c.POINTER(_c.c_float)
_dp = _c.POINTER(_c.c_double)
_ip = _c.POINTER(_c.c_int)
_u64p = _c.POINTER(_c.c_uint64)


class DomainStruct(ctypes.Structure):
    _fields_ = [
        ("width", _f), ("height", _f), ("cell_size", _f),
        ("max_particles", _u64), ("max_cell_particles", _u64), ("max_neighbors", _u64),
        ("stats_min_init", _u64), ("max_neighbors_stat", _u64),
        ("particle_radius", _f), ("collision_margin", _f), ("jitter_kernel_height", _f),
    ]


def build(reference: bool = True) -> None:
    """Build the restatement, and the reference harness where the tree exists."""
    targets = ["all"]
    if reference and reference_tree_present():
        targets.append("reference")
    subprocess.run(["make", "-s", "-C", HERE, "REF=" + (REFERENCE_TREE or ".")] + targets, check=True)


def reference_available() -> bool:
    return os.path.exists(os.path.join(REF_DIR, "libsphref.so"))


def _ptr(a, ctype):
    return a.ctypes.data_as(_c.POINTER(ctype)) if a is not None else None


def _setup(lib, prefix: str, real):
    realp = _c.POINTER(real)
    sig = {
        "destroy": (None, [_vp]),
        "reset_stats": (None, [_vp]),
        "clear_bodies": (None, [_vp]),
        "clear_particles": (None, [_vp]),
        "clear_emitters": (None, [_vp]),
        "set_gravity": (None, [_vp, _f, _f]),
        "add_external_force": (None, [_vp, _f, _f]),
        "clear_external_force": (None, [_vp]),
        "set_params": (None, [_vp, _fp]),
        "get_params": (None, [_vp, _fp]),
        "add_polygon": (None, [_vp, _u64, _fp]),
        "add_volume": (None, [_vp, _f, _f, _f, _f, _i, _i, _f]),
        "add_emitter": (None, [_vp, _f, _f, _f, _f, _f, _f, _f, _f]),
        "update": (None, [_vp, _f]),
        "particle_count": (_u64, [_vp]),
        "get_particles": (None, [_vp] + [realp] * 6),
        "get_index": (None, [_vp, _ip, _u64p, _u64p]),
        "get_neighbors": (None, [_vp, _u64, _u64p]),
        "get_cell": (_u64, [_vp, _i, _u64p]),
        "set_state": (_i, [_vp, _u64] + [realp] * 6 + [_ip, _u64p, _u64p, _u64p, _u64p, _u64p]),
        "get_stats": (None, [_vp, _u64p, _fp]),
        "srand": (None, [_c.c_uint]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(lib, prefix + name)
        fn.restype = res
        fn.argtypes = args


class _CpuSim:
    """Common Python face of both oracles (BaseSimulation + state I/O)."""

    _prefix = ""
    _real = np.float32

    def __init__(self, lib, handle, gx: int, gy: int):
        self._lib = lib
        self._h = _vp(handle)
        self.gx, self.gy = gx, gy
        self._p = lambda name: getattr(lib, self._prefix + name)

    def close(self):
        if self._h:
            self._p("destroy")(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # --- BaseSimulation -------------------------------------------------
    def reset_stats(self):
        self._p("reset_stats")(self._h)

    def clear_bodies(self):
        self._p("clear_bodies")(self._h)

    def clear_particles(self):
        self._p("clear_particles")(self._h)

    def clear_emitters(self):
        self._p("clear_emitters")(self._h)

    def set_gravity(self, x, y):
        self._p("set_gravity")(self._h, x, y)

    def add_external_force(self, x, y):
        self._p("add_external_force")(self._h, x, y)

    def clear_external_force(self):
        self._p("clear_external_force")(self._h)

    def set_params(self, p):
        a = np.asarray(p, dtype=np.float32)
        self._p("set_params")(self._h, _ptr(a, _c.c_float))

    def get_params(self):
        a = np.zeros(9, np.float32)
        self._p("get_params")(self._h, _ptr(a, _c.c_float))
        return a

    def add_plane(self, nx, ny, d):
        self._p("add_plane")(self._h, nx, ny, d)

    def add_circle(self, x, y, r):
        self._p("add_circle")(self._h, x, y, r)

    def add_segment(self, ax, ay, bx, by):
        self._p("add_segment")(self._h, ax, ay, bx, by)

    def add_polygon(self, verts):
        v = np.ascontiguousarray(verts, dtype=np.float32).reshape(-1)
        self._p("add_polygon")(self._h, len(v) // 2, _ptr(v, _c.c_float))

    def add_particle(self, x, y, fx=0.0, fy=0.0):
        return int(self._p("add_particle")(self._h, x, y, fx, fy))

    def add_particles(self, pos, force=None):
        pos = np.asarray(pos, np.float32)
        f = np.zeros_like(pos) if force is None else np.asarray(force, np.float32)
        for k in range(len(pos)):
            self.add_particle(float(pos[k, 0]), float(pos[k, 1]), float(f[k, 0]), float(f[k, 1]))

    def add_volume(self, cx, cy, fx, fy, nx, ny, spacing):
        self._p("add_volume")(self._h, cx, cy, fx, fy, nx, ny, spacing)

    def add_emitter(self, px, py, dx, dy, radius, speed, rate, duration):
        self._p("add_emitter")(self._h, px, py, dx, dy, radius, speed, rate, duration)

    def update(self, dt):
        return self._p("update")(self._h, dt)

    def particle_count(self) -> int:
        return int(self._p("particle_count")(self._h))

    def srand(self, seed: int):
        self._p("srand")(seed)

    # --- state I/O ------------------------------------------------------
    def get_state(self, lists: bool = True) -> Dict[str, np.ndarray]:
        n = self.particle_count()
        r = self._real
        st = {k: np.zeros((n, 2), r) for k in ("pos", "prev", "acc", "vel", "dens", "press")}
        ct = _c.c_float if r == np.float32 else _c.c_double
        self._p("get_particles")(self._h, *[_ptr(st[k], ct) for k in ("pos", "prev", "acc", "vel", "dens", "press")])
        cell = np.zeros((n, 2), np.int32)
        ic = np.zeros(n, np.uint64)
        nbc = np.zeros(n, np.uint64)
        self._p("get_index")(self._h, _ptr(cell, _c.c_int), _ptr(ic, _c.c_uint64), _ptr(nbc, _c.c_uint64))
        st.update(cell=cell, index_in_cell=ic, nb_count=nbc)
        if lists:
            flat = np.zeros(int(nbc.sum()), np.uint64)
            off = 0
            for i in range(n):
                c = int(nbc[i])
                if c:
                    view = flat[off:off + c]
                    self._p("get_neighbors")(self._h, i, _ptr(view, _c.c_uint64))
                off += c
            st["nb_flat"] = flat
        g = self.gx * self.gy
        cc = np.zeros(g, np.uint64)
        parts = []
        for c in range(g):
            cnt = int(self._p("get_cell")(self._h, c, None))
            buf = np.zeros(cnt, np.uint64)
            if cnt:
                self._p("get_cell")(self._h, c, _ptr(buf, _c.c_uint64))
            cc[c] = cnt
            parts.append(buf)
        st["cell_count"] = cc
        st["cell_flat"] = np.concatenate(parts) if parts else np.zeros(0, np.uint64)
        return st

    def set_state(self, st: Dict[str, np.ndarray]) -> None:
        r = self._real
        ct = _c.c_float if r == np.float32 else _c.c_double
        n = len(st["pos"])
        arrs = [np.ascontiguousarray(st[k], dtype=r) for k in ("pos", "prev", "acc", "vel", "dens", "press")]
        cell = np.ascontiguousarray(st["cell"], dtype=np.int32)
        ic = np.ascontiguousarray(st["index_in_cell"], dtype=np.uint64)
        nbc = np.ascontiguousarray(st["nb_count"], dtype=np.uint64)
        nbf = np.ascontiguousarray(st["nb_flat"], dtype=np.uint64)
        cc = np.ascontiguousarray(st["cell_count"], dtype=np.uint64)
        cf = np.ascontiguousarray(st["cell_flat"], dtype=np.uint64)
        if len(nbf) == 0:
            nbf = np.zeros(1, np.uint64)
        if len(cf) == 0:
            cf = np.zeros(1, np.uint64)
        rc = self._p("set_state")(self._h, n, *[_ptr(a, ct) for a in arrs], _ptr(cell, _c.c_int),
                                  _ptr(ic, _c.c_uint64), _ptr(nbc, _c.c_uint64), _ptr(nbf, _c.c_uint64),
                                  _ptr(cc, _c.c_uint64), _ptr(cf, _c.c_uint64))
        if rc != 0:
            raise ValueError("oracle set_state: capacity exceeded")

    def get_stats(self):
        counts = np.zeros(4, np.uint64)
        times = np.zeros(9, np.float32)
        self._p("get_stats")(self._h, _ptr(counts, _c.c_uint64), _ptr(times, _c.c_float))
        return counts, times


class ReferenceSim(_CpuSim):
    """The reference's own Demo4 solver (FP32, its fixed 33x18 grid)."""

    _prefix = "sphref_"
    _real = np.float32
    _lib = None
    _libname = "libsphref.so"

    @classmethod
    def load(cls):
        if cls._lib is None:
            path = os.path.join(REF_DIR, cls._libname)
            if not os.path.exists(path):
                raise FileNotFoundError(path)
            lib = ctypes.CDLL(path)
            _setup(lib, cls._prefix, _c.c_float)
            lib.sphref_create.restype = _vp
            lib.sphref_add_plane.argtypes = [_vp, _f, _f, _f]
            lib.sphref_add_circle.argtypes = [_vp, _f, _f, _f]
            lib.sphref_add_segment.argtypes = [_vp, _f, _f, _f, _f]
            lib.sphref_add_particle.argtypes = [_vp, _f, _f, _f, _f]
            lib.sphref_add_particle.restype = _u64
            lib.sphref_set_multithreading.argtypes = [_vp, _i]
            lib.sphref_worker_count.restype = _u64
            lib.sphref_worker_count.argtypes = [_vp]
            lib.sphref_limits.argtypes = [_ip, _ip, _fp, _fp, _fp, _u64p, _u64p, _u64p]
            lib.sphref_params_from_ctor8.argtypes = [_fp, _fp]
            cls._lib = lib
        return cls._lib

    @classmethod
    def limits(cls):
        lib = cls.load()
        gx, gy = _c.c_int(), _c.c_int()
        cs, hw, hh = _c.c_float(), _c.c_float(), _c.c_float()
        a, b, c = _c.c_uint64(), _c.c_uint64(), _c.c_uint64()
        lib.sphref_limits(_c.byref(gx), _c.byref(gy), _c.byref(cs), _c.byref(hw), _c.byref(hh),
                          _c.byref(a), _c.byref(b), _c.byref(c))
        return dict(gx=gx.value, gy=gy.value, cell_size=cs.value, half_width=hw.value, half_height=hh.value,
                    max_particles=a.value, max_cell=b.value, max_neighbors=c.value)

    def __init__(self, multithreading: bool = False):
        lib = self.load()
        lim = self.limits()
        super().__init__(lib, lib.sphref_create(), lim["gx"], lim["gy"])
        self.set_multithreading(multithreading)

    def set_multithreading(self, on: bool):
        self._lib.sphref_set_multithreading(self._h, 1 if on else 0)

    def worker_count(self) -> int:
        return int(self._lib.sphref_worker_count(self._h))

    @classmethod
    def params_from_ctor8(cls, args):
        lib = cls.load()
        a = np.asarray(args, np.float32)
        out = np.zeros(9, np.float32)
        lib.sphref_params_from_ctor8(_ptr(a, _c.c_float), _ptr(out, _c.c_float))
        return out


class ReferenceSimBox51(ReferenceSim):
    """The reference's own Demo4 solver built with raised compile-time
    constants (oracle/Makefile target ``reference``): a 51.2-wide box
    (kSPHBoundaryWidth; the height follows from the reference's 16:9 aspect,
    170 x 96 cells) holding up to 65,536 particles, for the 65,536-particle
    scene.  Cell and neighbour capacities are the reference's."""

    _lib = None
    _libname = "libsphref_box51.so"

    @classmethod
    def available(cls) -> bool:
        return os.path.exists(os.path.join(REF_DIR, cls._libname))

    @classmethod
    def oracle_domain(cls):
        """The restatement's domain with exactly this build's box and
        capacities."""
        lim = cls.limits()
        d = OracleSim.reference_domain()
        d.width = float(np.float32(lim["half_width"]) * np.float32(2.0))
        d.height = float(np.float32(lim["half_height"]) * np.float32(2.0))
        d.max_particles = lim["max_particles"]
        d.max_cell_particles = lim["max_cell"]
        d.max_neighbors = lim["max_neighbors"]
        return d


class ReferenceSimBox205(ReferenceSimBox51):
    """The reference's own solver with a 204.8-wide box (682 x 384 cells)
    holding up to 1,048,576 particles, for the 1,048,576-particle block
    (about 9.5 GB of host memory: the reference's fixed 1,000-entry
    neighbour arrays)."""

    _lib = None
    _libname = "libsphref_box205.so"


class OracleSim(_CpuSim):
    """CPU restatement of the Demo4 step (sph_oracle.cpp), FP32 or FP64."""

    _prefix = "sph_oracle_"

    @staticmethod
    def reference_domain() -> DomainStruct:
        d = DomainStruct()
        OracleSim._raw_lib().sph_oracle_reference_domain(_c.byref(d))
        return d

    @classmethod
    def _raw_lib(cls):
        if not hasattr(cls, "_raw"):
            path = os.path.join(REF_DIR, "liboracle.so")
            build(reference=False)  # make: rebuilds only when a source changed
            cls._raw = ctypes.CDLL(path)
        return cls._raw

    @staticmethod
    def default_params():
        a = np.zeros(9, np.float32)
        OracleSim._raw_lib().sph_oracle_default_params(_ptr(a, _c.c_float))
        return a

    def __init__(self, domain: Optional[DomainStruct] = None, fp64: bool = False, workers: int = 1):
        raw = self._raw_lib()
        _setup(raw, self._prefix, _c.c_double)
        raw.sph_oracle_create.restype = _vp
        raw.sph_oracle_create.argtypes = [_c.POINTER(DomainStruct), _i]
        raw.sph_oracle_add_plane.argtypes = [_vp, _f, _f, _f]
        raw.sph_oracle_add_circle.argtypes = [_vp, _f, _f, _f]
        raw.sph_oracle_add_segment.argtypes = [_vp, _f, _f, _f, _f]
        raw.sph_oracle_add_particle.argtypes = [_vp, _f, _f, _f, _f]
        raw.sph_oracle_add_particle.restype = _c.c_int64
        raw.sph_oracle_update.restype = _i
        raw.sph_oracle_set_workers.argtypes = [_vp, _u64]
        raw.sph_oracle_workers.argtypes = [_vp]
        raw.sph_oracle_workers.restype = _u64
        raw.sph_oracle_hardware_threads.restype = _u64
        if domain is None:
            domain = self.reference_domain()
        self.domain = domain
        gx = int(np.float32(domain.width) / np.float32(domain.cell_size))
        gy = int(np.float32(domain.height) / np.float32(domain.cell_size))
        super().__init__(raw, raw.sph_oracle_create(_c.byref(domain), 1 if fp64 else 0), gx, gy)
        self.fp64 = fp64
        self._real = np.float64
        self.set_workers(workers)

    def set_workers(self, w: int):
        self._lib.sph_oracle_set_workers(self._h, int(w))

    @classmethod
    def hardware_threads(cls) -> int:
        return int(cls._raw_lib().sph_oracle_hardware_threads())

    # --- viscoelastic springs (restated from Clavet et al. 2005) -------------
    SPRING_SLOTS = 16

    def set_springs(self, enabled: bool, yield_ratio: float = 0.1, plasticity: float = 0.3,
                    stiffness: float = 0.3, max_per_particle: int = 16, serial: bool = False):
        """Springs on or off.  ``serial`` applies the spring displacements as
        the paper's loop does (Clavet et al. 2005, Algorithm 3: one spring at
        a time, positions updated at once, springs in order of their lower
        end's number); otherwise every particle moves by its springs'
        displacements from the positions before the phase (the library's
        form)."""
        fn = self._lib.sph_oracle_set_springs
        fn.argtypes = [_vp, _i, _f, _f, _f, _i]
        fn.restype = None
        fn(self._h, 1 if enabled else 0, float(yield_ratio), float(plasticity), float(stiffness),
           int(max_per_particle))
        fs = self._lib.sph_oracle_set_spring_serial
        fs.argtypes = [_vp, _i]
        fs.restype = None
        fs(self._h, 1 if serial else 0)

    def set_spring_state(self, count, partner, rest, tag=None):
        """Springs per particle: count (n,), partner (n, 16) particle
        indices, rest (n, 16) lengths; tag (n,) the AddParticle indices used
        to order candidates with equal distances."""
        n = len(count)
        count = np.ascontiguousarray(count, np.int32)
        partner = np.ascontiguousarray(partner, np.int32).reshape(n, self.SPRING_SLOTS)
        rest = np.ascontiguousarray(rest, np.float32).reshape(n, self.SPRING_SLOTS)
        tg = np.ascontiguousarray(tag, np.int64) if tag is not None else None
        fn = self._lib.sph_oracle_set_spring_state
        fn.argtypes = [_vp, _u64, _c.POINTER(_c.c_int32), _c.POINTER(_c.c_int32), _c.POINTER(_c.c_float),
                       _c.POINTER(_c.c_int64)]
        fn.restype = _i
        rc = fn(self._h, n, _ptr(count, _c.c_int32), _ptr(partner, _c.c_int32), _ptr(rest, _c.c_float),
                _ptr(tg, _c.c_int64))
        if rc != 0:
            raise ValueError("oracle set_spring_state: invalid spring state")

    def get_spring_state(self):
        n = self.particle_count()
        count = np.zeros(n, np.int32)
        partner = np.zeros((n, self.SPRING_SLOTS), np.int32)
        rest = np.zeros((n, self.SPRING_SLOTS), np.float32)
        fn = self._lib.sph_oracle_get_spring_state
        fn.argtypes = [_vp, _c.POINTER(_c.c_int32), _c.POINTER(_c.c_int32), _c.POINTER(_c.c_float)]
        fn.restype = None
        fn(self._h, _ptr(count, _c.c_int32), _ptr(partner, _c.c_int32), _ptr(rest, _c.c_float))
        return count, partner, rest

    def spring_total(self) -> int:
        fn = self._lib.sph_oracle_spring_total
        fn.argtypes = [_vp]
        fn.restype = _u64
        return int(fn(self._h))

