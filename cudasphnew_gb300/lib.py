"""ctypes binding of libsph_gb300.so (include/sph.h) and a Python mirror of the
reference's ``ParticleSimulation`` class (CUDASPHNEW/particle_simulation.h:113-324).

There is no CPU fallback: if the shared library has not been built this module
raises on first use.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

from .params import BoundaryDesc, Options, SdfGrid, SimulationParameters

PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(PKG, "_build", "libsph_gb300.so")

SPH_STEP_PLAIN, SPH_STEP_TWO_SCALE, SPH_STEP_SUB_ONLY, SPH_STEP_LEARNED = 0, 1, 2, 3
CORRECTOR_FEATURES, CORRECTOR_OUTPUTS, CORRECTOR_WEIGHTS, CORRECTOR_FLOATS = 24, 6, 7312, 7378
(FIELD_VERTEX_DATA, FIELD_SIMULATION_DATA, FIELD_VELOCITY, FIELD_ACCELERATION,
 FIELD_DENSITY, FIELD_PRESSURE, FIELD_STATE, FIELD_SUB_VERTEX_DATA, FIELD_SUB_SIMULATION_DATA,
 FIELD_SUB_IDS, FIELD_SPLIT_IDS, FIELD_BOUNDARY_IDS, FIELD_DEFAULT_IDS) = range(13)

STATUS = {0: "SPH_OK", 1: "SPH_ERR_INVALID_ARGUMENT", 2: "SPH_ERR_CUDA",
          3: "SPH_ERR_OUT_OF_MEMORY", 4: "SPH_ERR_OUT_OF_DOMAIN", 5: "SPH_ERR_DEVICE_WAIT",
          6: "SPH_ERR_NOT_SUPPORTED", 7: "SPH_ERR_NON_FINITE"}

# Every function include/sph.h declares, with its ctypes signature.
_vp = ctypes.c_void_p
_u = ctypes.c_uint
_i = ctypes.c_int
SIGNATURES = {
    "sph_default_options": (None, [_vp]),
    "sph_create": (_i, [_vp, _vp, _vp, _vp, _vp, _vp]),
    "sph_create_batch": (_i, [_vp, _i, _vp, _vp]),
    "sph_batch_info": (_i, [_vp, _vp, _vp, _vp]),
    "sph_destroy": (_i, [_vp]),
    "sph_bind": (_i, [_vp, _vp]),
    "sph_set_stream": (_i, [_vp, _vp]),
    "sph_step": (_i, [_vp, _i]),
    "sph_step_many": (_i, [_vp, _i, _i]),
    "sph_synchronize": (_i, [_vp]),
    "sph_read": (_i, [_vp, _i, _vp, ctypes.c_size_t]),
    "sph_read_async": (_i, [_vp, _i, _vp, ctypes.c_size_t]),
    "sph_write": (_i, [_vp, _i, _vp, ctypes.c_size_t]),
    "sph_read_cells": (_i, [_vp, _i, _vp, _vp, _vp, _vp]),
    "sph_get_counts": (_i, [_vp, _vp]),
    "sph_get_diagnostics": (_i, [_vp, _vp]),
    "sph_device_pointer": (_i, [_vp, _i, _vp]),
    "sph_boundary_dims": (_i, [_vp, _vp]),
    "sph_boundary_maps": (_i, [_vp, _vp, _vp, _vp]),
    "sph_get_tuning": (_i, [_vp, _vp]),
    "sph_set_tuning": (_i, [_vp, _vp]),
    "sph_autotune": (_i, [_vp, _i, _vp]),
    "sph_set_stage_timing": (_i, [_vp, _i]),
    "sph_stage_times": (_i, [_vp, _vp, _vp, _i, _vp]),
    "sph_stage_name": (ctypes.c_char_p, [_i]),
    "sph_cell_tables_noalloc": (_i, [_vp, _vp, _u, _vp, _vp, _vp, _vp, _vp]),
    "sph_corrector_default_config": (None, [_vp]),
    "sph_corrector_train": (_i, [_vp, _vp]),
    "sph_corrector_load": (_i, [_vp, _vp, _vp, ctypes.c_size_t]),
    "sph_corrector_save": (_i, [_vp, _vp, ctypes.c_size_t]),
    "sph_corrector_get_report": (_i, [_vp, _vp]),
    "sph_corrector_predict": (_i, [_vp, _vp, _i, _vp]),
    "sph_corrector_gradient": (_i, [_vp, _vp, _vp, _i, _vp, _vp]),
    "sph_read_features": (_i, [_vp, _vp, ctypes.c_size_t]),
    "sph_corrector_record_features": (_i, [_vp, ctypes.c_int]),
    "sph_obj_load": (_i, [ctypes.c_char_p, _vp]),
    "sph_mesh_free": (None, [_vp]),
    "sph_sdf_from_mesh": (_i, [_vp, ctypes.c_float, ctypes.c_float, ctypes.c_float, _vp]),
    "sph_sdf_from_mesh_on_grid": (_i, [_vp, _vp, ctypes.c_float, _vp, ctypes.c_float, ctypes.c_float, _vp]),
    "sph_sdf_save": (_i, [_vp, ctypes.c_char_p]),
    "sph_sdf_load": (_i, [ctypes.c_char_p, _vp]),
    "sph_sdf_free": (None, [_vp]),
    "sph_surface_particles": (_i, [_vp, _vp]),
    "sph_time_kernel": (_i, [_vp, ctypes.c_int, ctypes.c_int, _vp]),
    "sph_neighbour_builds": (_i, [_vp, _vp]),
    "sph_camera_look_at": (_i, [_vp, _vp, _vp, _vp]),
    "sph_camera_perspective": (_i, [_vp, ctypes.c_float, ctypes.c_float, ctypes.c_float, ctypes.c_float]),
    "sph_render": (_i, [_vp, _vp, ctypes.c_int, ctypes.c_int, ctypes.c_int, _vp, _vp]),
    "sph_image_save_ppm": (_i, [ctypes.c_char_p, _vp, ctypes.c_int, ctypes.c_int]),
    "sph_last_error": (ctypes.c_char_p, []),
    "sph_status_string": (ctypes.c_char_p, [_i]),
}


class Counts(ctypes.Structure):
    _fields_ = [(name, ctypes.c_uint) for name in (
        "numParticles", "numParticlesDefault", "numParticlesSplit", "numParticlesBoundary",
        "numSubParticles", "numTimeSteps", "numCells", "numSubCells")]


SPH_RENDER_PARTICLES, SPH_RENDER_TWO_SCALE, SPH_RENDER_SUB_PARTICLES = 0, 1, 2


class Camera(ctypes.Structure):
    """sph_camera: column-major view and projection matrices."""

    _fields_ = [("view", ctypes.c_float * 16), ("proj", ctypes.c_float * 16)]

    @classmethod
    def look(cls, eye, centre, up, fovy, aspect, znear, zfar):
        """cgtkGLLookAt + cgtkGLPerspective, as the reference's renderers set them."""
        c = cls()
        f3 = ctypes.c_float * 3
        check(load().sph_camera_look_at(ctypes.byref(c), f3(*eye), f3(*centre), f3(*up)))
        check(load().sph_camera_perspective(ctypes.byref(c), fovy, aspect, znear, zfar))
        return c


def save_ppm(path: str, rgba: np.ndarray) -> None:
    """PortablePixmap's ASCII P3 layout of an (H, W, 4) uint8 image."""
    img = np.ascontiguousarray(rgba, np.uint8)
    h, w = img.shape[:2]
    check(load().sph_image_save_ppm(path.encode(), img.ctypes.data, w, h))


class Diagnostics(ctypes.Structure):
    """sph_diagnostics: FP64 conservation terms of the coarse particles."""

    _fields_ = [("mass", ctypes.c_double), ("momentum", ctypes.c_double * 3),
                ("kineticEnergy", ctypes.c_double), ("potentialEnergy", ctypes.c_double),
                ("densityMean", ctypes.c_double), ("densityMaxRelError", ctypes.c_double)]


class CorrectorConfig(ctypes.Structure):
    """sph_corrector_config."""

    _fields_ = [("trainSteps", ctypes.c_int), ("stride", ctypes.c_int), ("epochs", ctypes.c_int),
                ("batchTiles", ctypes.c_int), ("learningRate", ctypes.c_float),
                ("densityTolerance", ctypes.c_float), ("auditInterval", ctypes.c_int), ("seed", ctypes.c_uint),
                ("targetScale", ctypes.c_float)]

    @classmethod
    def default(cls, **kw) -> "CorrectorConfig":
        c = cls()
        load().sph_corrector_default_config(ctypes.byref(c))
        for k, v in kw.items():
            setattr(c, k, v)
        return c


class CorrectorReport(ctypes.Structure):
    """sph_corrector_report."""

    _fields_ = [("samples", ctypes.c_uint), ("optimizerSteps", ctypes.c_uint),
                ("firstEpochLoss", ctypes.c_float), ("lastEpochLoss", ctypes.c_float),
                ("trainMilliseconds", ctypes.c_float), ("learnedSteps", ctypes.c_uint),
                ("audits", ctypes.c_uint), ("rollbacks", ctypes.c_uint),
                ("lastAuditError", ctypes.c_float), ("maxAuditError", ctypes.c_float)]


class Tuning(ctypes.Structure):
    _fields_ = [(name, ctypes.c_int) for name in (
        "densityBlock", "forceBlock", "forceVariant", "prune", "kahan")]

    def as_dict(self):
        return {name: getattr(self, name) for name, _ in self._fields_}


class SphError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(f"{STATUS.get(status, status)}: {message}")
        self.status = status


_lib = None


def load(path: str = LIB_PATH):
    """Loads the shared library; raises if it has not been built."""
    global _lib
    if _lib is None:
        if not os.path.exists(path):
            raise RuntimeError(
                f"{path} is missing: build it with `python -c 'import __graft_entry__ as g; g.build()'`")
        L = ctypes.CDLL(path)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def check(status: int) -> None:
    if status != 0:
        raise SphError(status, load().sph_last_error().decode(errors="replace"))


def _p(a: np.ndarray):
    return a.ctypes.data_as(ctypes.c_void_p)


def boundary_maps(desc: BoundaryDesc):
    """Boundary maps built on the GPU: (distance, density, viscosity) as
    (nz, ny, nx) float32 arrays."""
    L = load()
    dims = np.zeros(3, np.uint32)
    check(L.sph_boundary_dims(ctypes.byref(desc), _p(dims)))
    shape = (int(dims[2]), int(dims[1]), int(dims[0]))
    out = [np.zeros(shape, np.float32) for _ in range(3)]
    check(L.sph_boundary_maps(ctypes.byref(desc), *[_p(a) for a in out]))
    return tuple(out)


class Mesh(ctypes.Structure):
    """sph_mesh: triangle mesh (0-based faces)."""

    _fields_ = [("vertices", ctypes.POINTER(ctypes.c_float)), ("numVertices", ctypes.c_uint),
                ("faces", ctypes.POINTER(ctypes.c_uint)), ("numFaces", ctypes.c_uint)]


def load_obj(path: str):
    """sph_obj_load: (vertices float32 [nv, 3], faces uint32 [nf, 3])."""
    L = load()
    m = Mesh()
    check(L.sph_obj_load(path.encode(), ctypes.byref(m)))
    try:
        v = np.ctypeslib.as_array(m.vertices, (m.numVertices, 3)).copy()
        f = np.ctypeslib.as_array(m.faces, (m.numFaces, 3)).copy()
    finally:
        L.sph_mesh_free(ctypes.byref(m))
    return v, f


def _grid_arrays(g: SdfGrid):
    n = int(g.dims[0]) * int(g.dims[1]) * int(g.dims[2])
    shape = (int(g.dims[2]), int(g.dims[1]), int(g.dims[0]))
    d = np.ctypeslib.as_array(g.distance, (n,)).copy().reshape(shape)
    nrm = np.ctypeslib.as_array(g.normal, (3 * n,)).copy().reshape(shape + (3,)) if g.normal else None
    return d, nrm


class SignedDistanceGrid:
    """A signed distance grid (host copy): distance[k, j, i] (negative inside),
    normal[k, j, i, 3], origin, dx, restDistance, compactSupport, maxDist."""

    def __init__(self, g: SdfGrid):
        self.origin = np.array(g.origin[:], np.float32)
        self.dx = float(g.dx)
        self.restDistance, self.compactSupport, self.maxDist = (float(g.restDistance), float(g.compactSupport),
                                                                float(g.maxDist))
        self.distance, self.normal = _grid_arrays(g)

    @property
    def dims(self):
        return tuple(int(v) for v in self.distance.shape[::-1])

    def struct(self) -> SdfGrid:
        """An sph_sdf_grid viewing this object's arrays (keep the object alive)."""
        g = SdfGrid()
        for a in range(3):
            g.origin[a] = float(self.origin[a])
            g.dims[a] = self.dims[a]
        g.dx, g.restDistance, g.compactSupport, g.maxDist = self.dx, self.restDistance, self.compactSupport, \
            self.maxDist
        self._d = np.ascontiguousarray(self.distance, np.float32)
        g.distance = self._d.ctypes.data_as(ctypes.POINTER(ctypes.c_float))
        if self.normal is not None:
            self._n = np.ascontiguousarray(self.normal, np.float32)
            g.normal = self._n.ctypes.data_as(ctypes.POINTER(ctypes.c_float))
        return g

    @classmethod
    def _take(cls, g: SdfGrid) -> "SignedDistanceGrid":
        try:
            return cls(g)
        finally:
            load().sph_sdf_free(ctypes.byref(g))

    @classmethod
    def from_mesh(cls, vertices, faces, rest_distance: float, compact_support: float, dx: float,
                  origin=None, dims=None) -> "SignedDistanceGrid":
        """sph_sdf_from_mesh (or _on_grid when origin and dims are given)."""
        L = load()
        v = np.ascontiguousarray(vertices, np.float32).reshape(-1, 3)
        f = np.ascontiguousarray(faces, np.uint32).reshape(-1, 3)
        m = Mesh(v.ctypes.data_as(ctypes.POINTER(ctypes.c_float)), len(v),
                 f.ctypes.data_as(ctypes.POINTER(ctypes.c_uint)), len(f))
        g = SdfGrid()
        if origin is None:
            check(L.sph_sdf_from_mesh(ctypes.byref(m), rest_distance, compact_support, dx, ctypes.byref(g)))
        else:
            o = (ctypes.c_float * 3)(*origin)
            dm = (ctypes.c_uint * 3)(*dims)
            check(L.sph_sdf_from_mesh_on_grid(ctypes.byref(m), o, dx, dm, rest_distance, compact_support,
                                              ctypes.byref(g)))
        return cls._take(g)

    @classmethod
    def load_file(cls, path: str) -> "SignedDistanceGrid":
        """sph_sdf_load: the reference's boundary-map text file."""
        g = SdfGrid()
        check(load().sph_sdf_load(path.encode(), ctypes.byref(g)))
        return cls._take(g)

    def save(self, path: str) -> None:
        g = self.struct()
        check(load().sph_sdf_save(ctypes.byref(g), path.encode()))


class Scene(ctypes.Structure):
    """sph_scene: one scene of a batched handle."""

    _fields_ = [("params", _vp), ("vertexData", _vp), ("simulationData", _vp), ("boundary", _vp)]


class ParticleSimulation:
    """Headless ``ParticleSimulation``: Init + Bind happen in the constructor
    (sph_create); the OpenGL buffer getters are replaced by device pointers
    and host reads."""

    def __init__(self, params: SimulationParameters, positions: np.ndarray,
                 velocities: np.ndarray | None = None, options: Options | None = None,
                 boundary: BoundaryDesc | None = None, simulation_data: np.ndarray | None = None):
        L = load()
        n = int(params.numParticles)
        vd = np.ascontiguousarray(positions, np.float32).reshape(n, 3)
        if simulation_data is None and velocities is not None:
            simulation_data = np.zeros((n, 10), np.float32)
            simulation_data[:, 6:9] = np.asarray(velocities, np.float32).reshape(n, 3)
        sd = None if simulation_data is None else np.ascontiguousarray(simulation_data, np.float32)
        self._params = params
        self.options = options if options is not None else Options()
        if options is None:
            L.sph_default_options(ctypes.byref(self.options))
        self.n = n
        h = ctypes.c_void_p()
        check(L.sph_create(ctypes.byref(params), ctypes.byref(self.options), _p(vd),
                           None if sd is None else _p(sd),
                           None if boundary is None else ctypes.byref(boundary), ctypes.byref(h)))
        self._h = h

    @classmethod
    def batch(cls, scenes, options: Options | None = None) -> "ParticleSimulation":
        """A batched handle over `scenes` (objects with params, positions,
        velocities, boundary): sph_create_batch.  Fields read back scene after
        scene; `scene_ranges()` gives each scene's particle range."""
        L = load()
        self = cls.__new__(cls)
        keep = []
        arr = (Scene * len(scenes))()
        for k, sc in enumerate(scenes):
            n = int(sc.params.numParticles)
            vd = np.ascontiguousarray(sc.positions, np.float32).reshape(n, 3)
            sd = np.zeros((n, 10), np.float32)
            sd[:, 6:9] = np.asarray(sc.velocities, np.float32).reshape(n, 3)
            keep += [vd, sd]
            arr[k].params = ctypes.addressof(sc.params)
            arr[k].vertexData = vd.ctypes.data
            arr[k].simulationData = sd.ctypes.data
            arr[k].boundary = ctypes.addressof(sc.boundary) if sc.boundary is not None else None
        self.options = options if options is not None else Options()
        if options is None:
            L.sph_default_options(ctypes.byref(self.options))
        self._params = scenes[0].params
        self.n = sum(int(sc.params.numParticles) for sc in scenes)
        h = ctypes.c_void_p()
        check(L.sph_create_batch(arr, len(scenes), ctypes.byref(self.options), ctypes.byref(h)))
        self._h = h
        return self

    def scene_ranges(self):
        """(first particle, first cell) arrays of numScenes + 1 entries."""
        L = load()
        k = ctypes.c_int()
        check(L.sph_batch_info(self._h, ctypes.byref(k), None, None))
        fp = np.zeros(k.value + 1, np.uint32)
        fc = np.zeros(k.value + 1, np.uint32)
        check(L.sph_batch_info(self._h, None, fp.ctypes.data, fc.ctypes.data))
        return fp, fc

    # -- lifetime ----------------------------------------------------------
    def close(self) -> None:
        if getattr(self, "_h", None) and self._h.value:
            load().sph_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    # -- reference API -------------------------------------------------------
    def Bind(self, params: SimulationParameters | None = None) -> None:
        if params is not None:
            self._params = params
        check(load().sph_bind(self._h, ctypes.byref(self._params)))

    def Advance(self) -> None:
        check(load().sph_step(self._h, SPH_STEP_PLAIN))

    def AdvanceTwoScale(self) -> None:
        check(load().sph_step(self._h, SPH_STEP_TWO_SCALE))

    def AdvanceSubParticles(self) -> None:
        check(load().sph_step(self._h, SPH_STEP_SUB_ONLY))

    def GetNumParticles(self) -> int:
        return self.counts().numParticles

    def GetNumTimesSteps(self) -> int:
        return self.counts().numTimeSteps

    def GetParticleRadius(self) -> float:
        """(3V/(4 pi N))^(1/3) (particle_simulation.cu:2227-2231)."""
        p = self._params
        return float(np.float32((3.0 * p.fluidVolume) / (4.0 * np.pi * p.numParticles)) ** np.float32(1.0 / 3.0))

    def GetSubParticleRadius(self) -> float:
        return 0.5 * self.GetParticleRadius()

    # -- extended API --------------------------------------------------------
    def step(self, mode: int = SPH_STEP_PLAIN, count: int = 1) -> None:
        L = load()
        if count == 1:
            check(L.sph_step(self._h, mode))
        else:
            check(L.sph_step_many(self._h, mode, count))

    def synchronize(self) -> None:
        check(load().sph_synchronize(self._h))

    def counts(self) -> Counts:
        c = Counts()
        check(load().sph_get_counts(self._h, ctypes.byref(c)))
        return c

    # -- learned step corrector ------------------------------------------------
    def train_corrector(self, cfg: CorrectorConfig | None = None, **kw) -> CorrectorReport:
        cfg = cfg or CorrectorConfig.default(**kw)
        check(load().sph_corrector_train(self._h, ctypes.byref(cfg)))
        return self.corrector_report()

    def load_corrector(self, model: np.ndarray, cfg: CorrectorConfig | None = None, **kw) -> None:
        cfg = cfg or CorrectorConfig.default(**kw)
        m = np.ascontiguousarray(model, np.float32)
        check(load().sph_corrector_load(self._h, ctypes.byref(cfg), m.ctypes.data, m.size))

    def save_corrector(self) -> np.ndarray:
        m = np.zeros(CORRECTOR_FLOATS, np.float32)
        check(load().sph_corrector_save(self._h, m.ctypes.data, m.size))
        return m

    def corrector_report(self) -> CorrectorReport:
        r = CorrectorReport()
        check(load().sph_corrector_get_report(self._h, ctypes.byref(r)))
        return r

    def corrector_predict(self, features: np.ndarray) -> np.ndarray:
        f = np.ascontiguousarray(features, np.float32).reshape(-1, CORRECTOR_FEATURES)
        out = np.zeros((len(f), CORRECTOR_OUTPUTS), np.float32)
        check(load().sph_corrector_predict(self._h, f.ctypes.data, len(f), out.ctypes.data))
        return out

    def corrector_gradient(self, features: np.ndarray, targets: np.ndarray):
        f = np.ascontiguousarray(features, np.float32).reshape(-1, CORRECTOR_FEATURES)
        t = np.zeros((len(f), 8), np.float32)
        t[:, :CORRECTOR_OUTPUTS] = np.asarray(targets, np.float32).reshape(len(f), CORRECTOR_OUTPUTS)
        g = np.zeros(CORRECTOR_WEIGHTS, np.float32)
        loss = np.zeros(1, np.float32)
        check(load().sph_corrector_gradient(self._h, f.ctypes.data, t.ctypes.data, len(f), g.ctypes.data,
                                            loss.ctypes.data))
        return g, float(loss[0])

    def record_features(self, enable: bool = True) -> None:
        """Learned steps also write their input features (96 bytes per particle)."""
        check(load().sph_corrector_record_features(self._h, 1 if enable else 0))

    def features(self) -> np.ndarray:
        """Features the last learned step with recording on computed (particle order)."""
        out = np.zeros((self.n, CORRECTOR_FEATURES), np.float32)
        check(load().sph_read_features(self._h, out.ctypes.data, out.nbytes))
        return out

    def render(self, camera: "Camera", width: int, height: int, what: int = 0, depth: bool = False):
        """sph_render: (height, width, 4) uint8 RGBA, rows top to bottom (and
        the (height, width) float depth when asked)."""
        img = np.zeros((height, width, 4), np.uint8)
        dep = np.zeros((height, width), np.float32) if depth else None
        check(load().sph_render(self._h, ctypes.byref(camera), width, height, what, img.ctypes.data,
                                dep.ctypes.data if dep is not None else None))
        return (img, dep) if depth else img

    def time_kernel(self, stage: str, reps: int = 20) -> float:
        """sph_time_kernel: microseconds per launch of 'density' or 'force'."""
        us = ctypes.c_float()
        check(load().sph_time_kernel(self._h, {"density": 4, "force": 5}[stage], reps, ctypes.byref(us)))
        return us.value

    def neighbour_builds(self) -> int:
        """How many times the plain and learned steps have built the reused neighbour lists."""
        b = ctypes.c_uint()
        check(load().sph_neighbour_builds(self._h, ctypes.byref(b)))
        return int(b.value)

    def surface_particles(self) -> np.ndarray:
        """CreateIsParticleSurfaceList: 1 for surface particles (particle order)."""
        out = np.zeros(self.n, np.int32)
        check(load().sph_surface_particles(self._h, out.ctypes.data))
        return out

    def diagnostics(self) -> Diagnostics:
        d = Diagnostics()
        check(load().sph_get_diagnostics(self._h, ctypes.byref(d)))
        return d

    def read(self, field: int) -> np.ndarray:
        n = self.n
        shapes = {FIELD_VERTEX_DATA: ((n, 3), np.float32), FIELD_VELOCITY: ((n, 3), np.float32),
                  FIELD_ACCELERATION: ((n, 3), np.float32), FIELD_SIMULATION_DATA: ((n, 10), np.float32),
                  FIELD_DENSITY: ((n,), np.float32), FIELD_PRESSURE: ((n,), np.float32),
                  FIELD_STATE: ((n,), np.uint8), FIELD_SUB_VERTEX_DATA: ((8 * n, 3), np.float32),
                  FIELD_SUB_SIMULATION_DATA: ((8 * n, 10), np.float32)}
        if field in (FIELD_SUB_IDS, FIELD_SPLIT_IDS, FIELD_BOUNDARY_IDS, FIELD_DEFAULT_IDS):
            c = self.counts()
            count = {FIELD_SUB_IDS: c.numSubParticles, FIELD_SPLIT_IDS: c.numParticlesSplit,
                     FIELD_BOUNDARY_IDS: c.numParticlesBoundary, FIELD_DEFAULT_IDS: c.numParticlesDefault}[field]
            shapes[field] = ((count,), np.int32)
        shape, dt = shapes[field]
        out = np.zeros(shape, dt)
        check(load().sph_read(self._h, field, _p(out), out.nbytes))
        return out

    def write_state(self, positions: np.ndarray, velocities: np.ndarray) -> None:
        self.write(FIELD_VERTEX_DATA, np.asarray(positions, np.float32).reshape(-1, 3))
        self.write(FIELD_VELOCITY, np.asarray(velocities, np.float32).reshape(-1, 3))

    def write(self, field: int, data: np.ndarray) -> None:
        a = np.ascontiguousarray(data, np.float32)
        check(load().sph_write(self._h, field, _p(a), a.nbytes))

    def positions(self) -> np.ndarray:
        return self.read(FIELD_VERTEX_DATA)

    def velocities(self) -> np.ndarray:
        return self.read(FIELD_VELOCITY)

    def cells(self, level: int = 0):
        """(sorted hash, sorted ids, cell start, cell end) of the last step."""
        c = self.counts()
        n = self.n if level == 0 else c.numSubParticles
        C = c.numCells if level == 0 else c.numSubCells
        h = np.zeros(n, np.int32)
        ids = np.zeros(n, np.int32)
        s = np.zeros(C, np.int32)
        e = np.zeros(C, np.int32)
        check(load().sph_read_cells(self._h, level, _p(h), _p(ids), _p(s), _p(e)))
        return h, ids, s, e

    def device_pointer(self, which: int) -> int:
        p = ctypes.c_void_p()
        check(load().sph_device_pointer(self._h, which, ctypes.byref(p)))
        return int(p.value or 0)

    def set_stream(self, stream_handle: int | None) -> None:
        check(load().sph_set_stream(self._h, ctypes.c_void_p(stream_handle or 0)))

    def tuning(self) -> Tuning:
        t = Tuning()
        check(load().sph_get_tuning(self._h, ctypes.byref(t)))
        return t

    def set_tuning(self, **kw) -> None:
        t = self.tuning()
        for k, v in kw.items():
            setattr(t, k, int(v))
        check(load().sph_set_tuning(self._h, ctypes.byref(t)))

    def autotune(self, reps: int = 5) -> Tuning:
        t = Tuning()
        check(load().sph_autotune(self._h, int(reps), ctypes.byref(t)))
        return t

    def set_stage_timing(self, capacity_steps: int) -> None:
        check(load().sph_set_stage_timing(self._h, int(capacity_steps)))

    def stage_times(self):
        """{stage name: (total ms, launches)} since the last call."""
        L = load()
        ms = np.zeros(32, np.float32)
        cnt = np.zeros(32, np.int32)
        k = ctypes.c_int()
        check(L.sph_stage_times(self._h, _p(ms), _p(cnt), 32, ctypes.byref(k)))
        return {L.sph_stage_name(i).decode(): (float(ms[i]), int(cnt[i])) for i in range(k.value)}
