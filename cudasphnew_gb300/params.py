"""Parameter structures of the SPH step and the parameter sets of the scenes.

``SimulationParameters`` is byte-for-byte the reference's POD struct
(CUDASPHNEW/particle_simulation.h:54-111); ``Options`` and ``BoundaryDesc``
mirror ``sph_options`` and ``sph_boundary_desc`` of include/sph.h.
"""
from __future__ import annotations

import ctypes
import math

import numpy as np

F3 = ctypes.c_float * 3
I3 = ctypes.c_int * 3


class SimulationParameters(ctypes.Structure):
    """particle_simulation.h:54-111, same field order and types."""

    _fields_ = [
        ("gridOrigin", F3),
        ("gridSpacing", ctypes.c_float),
        ("gridDim", I3),
        ("gridSpacingSubParticles", ctypes.c_float),
        ("gridDimSubParticles", I3),
        ("numParticles", ctypes.c_uint),
        ("compactSupport", ctypes.c_float),
        ("compactSupportSub", ctypes.c_float),
        ("kernelParticles", ctypes.c_int),
        ("timeStep", ctypes.c_float),
        ("timeStepSubParticles", ctypes.c_float),
        ("particleMass", ctypes.c_float),
        ("subParticleMass", ctypes.c_float),
        ("gasStiffness", ctypes.c_float),
        ("restDensity", ctypes.c_float),
        ("dynamicViscosity", ctypes.c_float),
        ("gravity", ctypes.c_float),
        ("tensionCoefficient", ctypes.c_float),
        ("normThresh", ctypes.c_float),
        ("fluidVolume", ctypes.c_float),
        ("poly6", ctypes.c_float),
        ("gradPoly6", ctypes.c_float),
        ("laplPoly6", ctypes.c_float),
        ("gradSpiky", ctypes.c_float),
        ("laplVisc", ctypes.c_float),
        ("poly6Sub", ctypes.c_float),
        ("gradPoly6Sub", ctypes.c_float),
        ("laplPoly6Sub", ctypes.c_float),
        ("gradSpikySub", ctypes.c_float),
        ("laplViscSub", ctypes.c_float),
        ("cmDistanceThresh", ctypes.c_float),
        ("nPartTresh", ctypes.c_float),
        ("boxDim", F3),
        ("boxCen", F3),
        ("restitution", ctypes.c_float),
    ]

    @property
    def num_cells(self) -> int:
        d = self.gridDim
        return int(d[0]) * int(d[1]) * int(d[2])

    @property
    def num_sub_cells(self) -> int:
        d = self.gridDimSubParticles
        return int(d[0]) * int(d[1]) * int(d[2])


class Options(ctypes.Structure):
    """sph_options (include/sph.h): what the reference hard-codes."""

    _fields_ = [
        ("gravityAxis", ctypes.c_int),
        ("boxCollision", ctypes.c_int),
        ("childMode", ctypes.c_int),
        ("cellRelative", ctypes.c_int),
        ("splitMin", F3),
        ("splitMax", F3),
        ("neighbourSkin", ctypes.c_float),
    ]


class Shape(ctypes.Structure):
    """sph_shape: 1 sphere obstacle, 2 cone obstacle, 3 box container."""

    _fields_ = [("kind", ctypes.c_int), ("p", ctypes.c_float * 7)]


SHAPE_SPHERE = 1
SHAPE_CONE = 2
SHAPE_BOX = 3
SHAPE_MESH = 4


class SdfGrid(ctypes.Structure):
    """sph_sdf_grid: a signed distance grid (negative inside), x fastest."""

    _fields_ = [("origin", F3), ("dx", ctypes.c_float), ("dims", ctypes.c_uint * 3),
                ("restDistance", ctypes.c_float), ("compactSupport", ctypes.c_float),
                ("maxDist", ctypes.c_float), ("distance", ctypes.POINTER(ctypes.c_float)),
                ("normal", ctypes.POINTER(ctypes.c_float))]


class BoundaryDesc(ctypes.Structure):
    """sph_boundary_desc: SphInComplexShapes' constructor arguments + solids."""

    _fields_ = [
        ("gridStart", F3),
        ("gridEnd", F3),
        ("gridSpacing", ctypes.c_float),
        ("restDistance", ctypes.c_float),
        ("compactSupport", ctypes.c_float),
        ("particleMass", ctypes.c_float),
        ("restDensity", ctypes.c_float),
        ("viscosity", ctypes.c_float),
        ("particleSpacing", ctypes.c_float),
        ("numShapes", ctypes.c_int),
        ("shapes", Shape * 8),
        ("sdfGrids", ctypes.c_void_p),
        ("numSdfGrids", ctypes.c_int),
    ]

    def dims(self):
        return tuple(
            int(np.uint32(np.float32(np.float32(self.gridEnd[a]) - np.float32(self.gridStart[a]))
                          / np.float32(self.gridSpacing))) + 1
            for a in range(3))


def _f32(x) -> float:
    return float(np.float32(x))


def kernel_constants(p: SimulationParameters, h: float) -> None:
    """Kernel coefficients as Example01 forms them (particle_simulation.cu:1777-1788).

    The reference evaluates ``315.0f/(64.0f*M_PI*h*...)`` with M_PI a double, so
    the value is computed in double and rounded once to float.
    """
    hf = float(np.float32(h))

    def prod(c, k):  # c * h * h * ... (k factors), left to right in double
        v = c
        for _ in range(k):
            v = v * hf
        return v

    p.compactSupport = hf
    p.compactSupportSub = _f32(np.float32(hf) / np.float32(2.0))
    p.poly6 = _f32(315.0 / prod(64.0 * math.pi, 9))
    p.gradPoly6 = _f32(-945.0 / prod(32.0 * math.pi, 9))
    p.laplPoly6 = _f32(-945.0 / prod(32.0 * math.pi, 9))
    p.gradSpiky = _f32(-45.0 / prod(math.pi, 6))
    p.laplVisc = _f32(45.0 / prod(math.pi, 6))
    p.poly6Sub = _f32(np.float32(p.poly6) * np.float32(512.0))
    p.gradPoly6Sub = _f32(np.float32(p.gradPoly6) * np.float32(512.0))
    p.laplPoly6Sub = _f32(np.float32(p.laplPoly6) * np.float32(512.0))
    p.gradSpikySub = _f32(np.float32(p.gradSpiky) * np.float32(64.0))
    p.laplViscSub = _f32(np.float32(p.laplVisc) * np.float32(64.0))


def set_simulation_domain(p: SimulationParameters, lo, hi, spacing: float, spacing_sub: float) -> None:
    """set_simulation_domain (particle_simulation.cu:2919-2941)."""
    for a in range(3):
        p.gridOrigin[a] = _f32(lo[a])
        ext = np.float32(np.float32(hi[a]) - np.float32(lo[a]))
        p.gridDim[a] = int(float(ext / np.float32(spacing)) + 0.5)
        p.gridDimSubParticles[a] = int(float(ext / np.float32(spacing_sub)) + 0.5)
    p.gridSpacing = _f32(spacing)
    p.gridSpacingSubParticles = _f32(spacing_sub)


def example01_params(num_particles: int = 39304) -> SimulationParameters:
    """Example01's parameter set (particle_simulation.cu:1745-1817)."""
    p = SimulationParameters()
    p.numParticles = num_particles
    p.kernelParticles = 20
    p.restDensity = _f32(998.648)
    p.particleMass = _f32(np.float32(p.restDensity) * np.float32(0.5) * np.float32(0.5)
                          * np.float32(0.5) / np.float32(num_particles))
    p.subParticleMass = _f32(np.float32(p.particleMass) / np.float32(8.0))
    p.gasStiffness = 3.0
    p.dynamicViscosity = 3.0
    p.gravity = _f32(9.81)
    p.tensionCoefficient = _f32(0.0728)
    p.normThresh = _f32(15.065)
    # powf of the float argument, as particle_simulation.cu:1774-1775 evaluates it
    h = float(np.power(np.float32((3.0 * 0.5 * 0.5 * 0.5 * 20) / (4.0 * math.pi * num_particles)),
                       np.float32(1.0 / 3.0)))
    kernel_constants(p, h)
    p.timeStep = _f32(0.003)
    p.timeStepSubParticles = _f32(0.001)
    set_simulation_domain(p, (-1, -1, -1), (1, 1, 1), h, _f32(np.float32(h) / np.float32(2)))
    p.fluidVolume = 0.125
    p.restitution = 0.0
    for a, v in enumerate((0.7, 0.5, 0.3)):
        p.boxDim[a] = v
        p.boxCen[a] = 0.0
    p.cmDistanceThresh = 0.5
    p.nPartTresh = 20.0
    return p


def example01_boundary(p: SimulationParameters) -> BoundaryDesc:
    """setUpSphInComplexShapes (particle_simulation.cu:2592-2612): the box
    container of centre 0 and extents (0.7, 0.5, 0.3), grid spacing h/4."""
    d = BoundaryDesc()
    h = np.float32(p.compactSupport)
    for a, (s, e) in enumerate(zip((-0.8, -0.6, -0.4), (0.8, 0.6, 0.4))):
        d.gridStart[a] = s
        d.gridEnd[a] = e
    d.gridSpacing = _f32(h / np.float32(4.0))
    d.restDistance = _f32(h)
    d.compactSupport = _f32(h)
    d.particleMass = p.particleMass
    d.restDensity = p.restDensity
    d.viscosity = p.dynamicViscosity
    # std::powf(mass/restDensity, 1.0f/3.0f), particle_simulation.cu:2603
    d.particleSpacing = float(np.power(np.float32(p.particleMass) / np.float32(p.restDensity), np.float32(1.0 / 3.0)))
    d.numShapes = 1
    d.shapes[0].kind = SHAPE_BOX
    for a, v in enumerate((0.0, 0.0, 0.0, 0.7, 0.5, 0.3)):
        d.shapes[0].p[a] = v
    return d


# ---------------------------------------------------------------------------
# Dam-break scenes (synthetic inputs of the benchmark configurations)
# ---------------------------------------------------------------------------
H = 0.025            # smoothing length
SPACING = 0.5 * H    # lattice pitch
REST_DENSITY = 1000.0


def dam_break_params(box_lo, box_hi, num_particles: int, dt: float = 1e-4,
                     stiffness: float = 3.0, viscosity: float = 0.02,
                     restitution: float = 0.0) -> SimulationParameters:
    """WCSPH dam break: h = 0.025, lattice pitch h/2, m = rho0*(h/2)^3,
    p = k(rho - rho0), gravity 9.81, tension off.  The cell grid has cell size
    h and is padded by two cells on every side of the container box: with one
    cell, a particle resting on an upper wall has (x + h - origin)/h == dim and
    compute_grid_coordinate's `% dim` (particle_simulation.cu:1249) wraps its
    neighbour range to nothing."""
    p = SimulationParameters()
    p.numParticles = num_particles
    p.kernelParticles = 34
    p.restDensity = REST_DENSITY
    p.particleMass = _f32(REST_DENSITY * SPACING ** 3)
    p.subParticleMass = _f32(np.float32(p.particleMass) / np.float32(8.0))
    p.gasStiffness = stiffness
    p.dynamicViscosity = viscosity
    p.gravity = _f32(9.81)
    p.tensionCoefficient = 0.0
    p.normThresh = _f32(15.065)
    kernel_constants(p, H)
    p.timeStep = _f32(dt)
    p.timeStepSubParticles = _f32(dt)
    lo = [float(np.float32(b) - np.float32(2 * H)) for b in box_lo]
    hi = [float(np.float32(b) + np.float32(2 * H)) for b in box_hi]
    set_simulation_domain(p, lo, hi, H, H / 2)
    p.fluidVolume = _f32(num_particles * SPACING ** 3)
    p.restitution = restitution
    for a in range(3):
        p.boxCen[a] = _f32(0.5 * (box_lo[a] + box_hi[a]))
        p.boxDim[a] = _f32(0.5 * (box_hi[a] - box_lo[a]))
    p.cmDistanceThresh = 0.5
    p.nPartTresh = 20.0
    return p


# Default skin of the reused neighbour lists, as a fraction of compactSupport
# (sph_options.neighbourSkin; the C default of sph_default_options).
NEIGHBOUR_SKIN = 0.1


def default_options(gravity_axis: int = 1, box_collision: bool = True) -> Options:
    o = Options()
    o.gravityAxis = gravity_axis
    o.boxCollision = 1 if box_collision else 0
    for a, (lo, hi) in enumerate(zip((0.2, -3.0e38, -3.0e38), (0.5, 3.0e38, 3.0e38))):
        o.splitMin[a] = lo
        o.splitMax[a] = hi
    o.neighbourSkin = NEIGHBOUR_SKIN
    return o


def obstacle_boundary(p: SimulationParameters, grid_start, n_nodes: int, shapes) -> BoundaryDesc:
    """Boundary maps of analytic obstacles on an ``n_nodes``^3 grid of pitch h/4
    (the reference's boundary-grid pitch, particle_simulation.cu:2606)."""
    d = BoundaryDesc()
    sp = np.float32(np.float32(p.compactSupport) / np.float32(4.0))
    for a in range(3):
        d.gridStart[a] = grid_start[a]
        d.gridEnd[a] = _f32(np.float32(grid_start[a]) + sp * np.float32(n_nodes - 1 + 0.5))
    d.gridSpacing = float(sp)
    d.restDistance = p.compactSupport
    d.compactSupport = p.compactSupport
    d.particleMass = p.particleMass
    d.restDensity = p.restDensity
    d.viscosity = p.dynamicViscosity
    d.particleSpacing = float(np.power(np.float32(p.particleMass) / np.float32(p.restDensity), np.float32(1.0 / 3.0)))
    d.numShapes = len(shapes)
    for i, (kind, vals) in enumerate(shapes):
        d.shapes[i].kind = kind
        for a, v in enumerate(vals):
            d.shapes[i].p[a] = v
    return d


def sphere_boundary(p: SimulationParameters, centre, radius: float, n_nodes: int = 64) -> BoundaryDesc:
    """Boundary maps of a solid sphere on an ``n_nodes``^3 grid centred on it,
    reaching 2h beyond its surface (pitch max(h/4, 2(r + 2h)/(n_nodes - 1)))."""
    h = float(np.float32(p.compactSupport))
    half = radius + 2.0 * h
    pitch = max(h / 4.0, 2.0 * half / (n_nodes - 1))
    sp = np.float32(pitch)
    d = obstacle_boundary(p, [c - half for c in centre], n_nodes, [(SHAPE_SPHERE, (*centre, radius))])
    for a in range(3):
        d.gridEnd[a] = _f32(np.float32(d.gridStart[a]) + sp * np.float32(n_nodes - 1 + 0.5))
    d.gridSpacing = float(sp)
    return d

