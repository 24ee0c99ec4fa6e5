"""ctypes binding of the CPU oracle (oracle/sph_oracle.cpp).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and the
CPU legs of bench.py, never by the cudasphnew_gb300 package.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

from cudasphnew_gb300.params import BoundaryDesc, Options, SimulationParameters

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libsph_oracle.so")


def build() -> str:
    subprocess.run(["sh", os.path.join(HERE, "build_oracle.sh")], check=True)
    return LIB_PATH


class Maps(ctypes.Structure):
    _fields_ = [
        ("origin", ctypes.c_float * 3),
        ("spacing", ctypes.c_float),
        ("dims", ctypes.c_uint * 3),
        ("restDistance", ctypes.c_float),
        ("dist", ctypes.c_void_p),
        ("dens", ctypes.c_void_p),
        ("visc", ctypes.c_void_p),
    ]


_P = ctypes.POINTER
_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        L = ctypes.CDLL(LIB_PATH)
        vp = ctypes.c_void_p
        L.orc_set_threads.argtypes = [ctypes.c_int]
        L.orc_max_threads.restype = ctypes.c_int
        L.orc_hash.argtypes = [_P(SimulationParameters), vp, ctypes.c_int, vp, vp]
        L.orc_hash.restype = ctypes.c_int
        L.orc_sort.argtypes = [vp, vp, ctypes.c_int, ctypes.c_int]
        L.orc_sort.restype = ctypes.c_int
        L.orc_cells.argtypes = [vp, ctypes.c_int, ctypes.c_int, vp, vp]
        L.orc_step_plain_f32.argtypes = [_P(SimulationParameters), _P(Options), _P(Maps),
                                         ctypes.c_int] + [vp] * 9
        L.orc_step_plain_f32.restype = ctypes.c_int
        L.orc_step_plain_f64.argtypes = [_P(SimulationParameters), _P(Options), _P(Maps),
                                         ctypes.c_int] + [vp] * 12
        L.orc_step_plain_f64.restype = ctypes.c_int
        L.orc_tex3d.argtypes = [_P(Maps), ctypes.c_int, vp, ctypes.c_int, vp]
        L.orc_boundary_dims.argtypes = [_P(BoundaryDesc), vp]
        L.orc_boundary_maps.argtypes = [_P(BoundaryDesc), vp, vp, vp]
        L.orc_boundary_maps.restype = ctypes.c_int
        _lib = L
    return _lib


def _ptr(a: np.ndarray):
    return a.ctypes.data_as(ctypes.c_void_p)


def set_threads(n: int) -> None:
    lib().orc_set_threads(int(n))


def max_threads() -> int:
    return int(lib().orc_max_threads())


class BoundaryMaps:
    """Dense x-fastest grids (distance, density, viscosity) + texture metadata."""

    def __init__(self, desc: BoundaryDesc, dist, dens, visc):
        self.desc = desc
        self.dims = tuple(int(d) for d in dist.shape[::-1])
        self.dist, self.dens, self.visc = dist, dens, visc
        m = Maps()
        for a in range(3):
            m.origin[a] = desc.gridStart[a]
            m.dims[a] = self.dims[a]
        m.spacing = desc.gridSpacing
        m.restDistance = desc.restDistance
        m.dist = self.dist.ctypes.data
        m.dens = self.dens.ctypes.data
        m.visc = self.visc.ctypes.data
        self.maps = m


def boundary_maps(desc: BoundaryDesc) -> BoundaryMaps:
    dims = np.zeros(3, np.uint32)
    lib().orc_boundary_dims(ctypes.byref(desc), _ptr(dims))
    shape = (int(dims[2]), int(dims[1]), int(dims[0]))
    dist = np.zeros(shape, np.float32)
    dens = np.zeros(shape, np.float32)
    visc = np.zeros(shape, np.float32)
    rc = lib().orc_boundary_maps(ctypes.byref(desc), _ptr(dist), _ptr(dens), _ptr(visc))
    assert rc == 0
    return BoundaryMaps(desc, dist, dens, visc)


def tex3d(bm: BoundaryMaps, which: int, xyz: np.ndarray) -> np.ndarray:
    xyz = np.ascontiguousarray(xyz, np.float64)
    out = np.zeros(len(xyz), np.float64)
    lib().orc_tex3d(ctypes.byref(bm.maps), which, _ptr(xyz), len(xyz), _ptr(out))
    return out


def hash_sort_cells(p: SimulationParameters, pos: np.ndarray):
    """compute_particle_hash + sort_by_key + compute_cell_start_end (FP32)."""
    n = len(pos)
    pos = np.ascontiguousarray(pos, np.float32)
    h = np.zeros(n, np.int32)
    ids = np.zeros(n, np.int32)
    bad = lib().orc_hash(ctypes.byref(p), _ptr(pos), n, _ptr(h), _ptr(ids))
    if bad:
        raise ValueError(f"{bad} particles outside the hash range")
    C = p.num_cells
    if lib().orc_sort(_ptr(h), _ptr(ids), n, C):
        raise ValueError("hash outside [0, numCells)")
    start = np.zeros(C, np.int32)
    end = np.zeros(C, np.int32)
    lib().orc_cells(_ptr(h), n, C, _ptr(start), _ptr(end))
    return h, ids, start, end


def step_plain(p: SimulationParameters, o: Options, bm: BoundaryMaps | None,
               pos: np.ndarray, vel: np.ndarray, fp64: bool = False):
    """One plain step.  Returns a dict with the step's outputs; ``pos``/``vel``
    in the dict are the updated state (inputs are not modified)."""
    n = len(pos)
    dt = np.float64 if fp64 else np.float32
    pos = np.array(pos, dt, order="C", copy=True)
    vel = np.array(vel, dt, order="C", copy=True)
    rho = np.zeros(n, dt)
    prs = np.zeros(n, dt)
    acc = np.zeros((n, 3), dt)
    C = p.num_cells
    h = np.zeros(n, np.int32)
    ids = np.zeros(n, np.int32)
    start = np.zeros(C, np.int32)
    end = np.zeros(C, np.int32)
    mp = ctypes.byref(bm.maps) if bm is not None else None
    out = dict(pos=pos, vel=vel, rho=rho, p=prs, acc=acc, hash=h, ids=ids, start=start, end=end)
    if fp64:
        srho = np.zeros(n, np.float64)
        sacc = np.zeros(n, np.float64)
        sdir = np.zeros(n, np.float64)
        rc = lib().orc_step_plain_f64(ctypes.byref(p), ctypes.byref(o), mp, n, _ptr(pos), _ptr(vel),
                                      _ptr(rho), _ptr(prs), _ptr(acc), _ptr(srho), _ptr(sacc),
                                      _ptr(sdir), _ptr(h), _ptr(ids), _ptr(start), _ptr(end))
        out.update(scale_rho=srho, scale_acc=sacc, scale_acc_direct=sdir)
    else:
        rc = lib().orc_step_plain_f32(ctypes.byref(p), ctypes.byref(o), mp, n, _ptr(pos), _ptr(vel),
                                      _ptr(rho), _ptr(prs), _ptr(acc), _ptr(h), _ptr(ids),
                                      _ptr(start), _ptr(end))
    if rc:
        raise ValueError(f"oracle step failed ({rc})")
    return out


def jet_slice(values: np.ndarray, scale: float) -> np.ndarray:
    """PortablePixmap::setJET over a (W, H) slice (portable_pixmap.cpp:49-62),
    returned as the P3 file's value order (rows top to bottom, RGB)."""
    s = (values.astype(np.float32) / np.float32(scale)).astype(np.float32)
    t = (s * np.float32(4.0)).astype(np.float32)
    r = np.minimum(t - np.float32(1.5), -t + np.float32(4.5))
    g = np.minimum(t - np.float32(0.5), -t + np.float32(3.5))
    b = np.minimum(t + np.float32(0.5), -t + np.float32(2.5))
    rgb = [np.clip(c, 0.0, 1.0).astype(np.float32) for c in (r, g, b)]
    px = [np.floor(np.float32(255.0) * c).astype(np.int64) for c in rgb]
    img = np.stack(px, axis=-1)          # (W, H, 3) indexed [i, j]
    img = img[:, ::-1, :]                # set() stores row H-j-1
    return np.transpose(img, (1, 0, 2))  # (H, W, 3) row-major like the file


class TwoScale:
    """Two-scale state of the oracle (particle states, lists and 8n child slots)."""

    WHAT = {"state": 0, "split": 1, "boundary": 2, "default": 3, "sub_ids": 4, "sub_hash": 5,
            "sorted_sub_ids": 6, "sub_start": 7, "sub_end": 8, "sub_pos": 10, "sub_vel": 11,
            "sub_acc": 12, "sub_rho": 13, "sub_p": 14, "sub_scale_acc": 15}

    def __init__(self, n: int, fp64: bool = False):
        L = lib()
        vp = ctypes.c_void_p
        L.orc_ts_new.restype = vp
        L.orc_ts_new.argtypes = [ctypes.c_int, ctypes.c_int]
        L.orc_ts_free.argtypes = [vp, ctypes.c_int]
        for name in ("orc_ts_step_f32", "orc_ts_step_f64"):
            getattr(L, name).argtypes = [vp, _P(SimulationParameters), _P(Options), _P(Maps)] + [vp] * 9
            getattr(L, name).restype = ctypes.c_int
        for name in ("orc_ts_part_f32", "orc_ts_part_f64"):
            getattr(L, name).argtypes = [vp, _P(SimulationParameters), _P(Options)] + [vp] * 7
            getattr(L, name).restype = ctypes.c_int
        for name in ("orc_ts_sub_only_f32", "orc_ts_sub_only_f64"):
            getattr(L, name).argtypes = [vp, _P(SimulationParameters), _P(Options)] + [vp] * 6
            getattr(L, name).restype = ctypes.c_int
        L.orc_ts_counts.argtypes = [vp, ctypes.c_int, vp]
        L.orc_ts_get.argtypes = [vp, ctypes.c_int, ctypes.c_int, vp]
        self.n, self.fp64 = n, fp64
        self.dt = np.float64 if fp64 else np.float32
        self._h = ctypes.c_void_p(L.orc_ts_new(n, 1 if fp64 else 0))

    def __del__(self):
        try:
            lib().orc_ts_free(self._h, 1 if self.fp64 else 0)
        except Exception:
            pass

    def counts(self):
        c = np.zeros(5, np.int32)
        lib().orc_ts_counts(self._h, 1 if self.fp64 else 0, _ptr(c))
        return dict(split=int(c[0]), boundary=int(c[1]), default=int(c[2]), sub=int(c[3]), sub_cells=int(c[4]))

    def get(self, what: str) -> np.ndarray:
        c = self.counts()
        n = self.n
        sizes = {"state": (n, np.uint8), "split": (c["split"], np.int32), "boundary": (c["boundary"], np.int32),
                 "default": (c["default"], np.int32), "sub_ids": (c["sub"], np.int32),
                 "sub_hash": (c["sub"], np.int32), "sorted_sub_ids": (c["sub"], np.int32),
                 "sub_start": (c["sub_cells"], np.int32), "sub_end": (c["sub_cells"], np.int32),
                 "sub_pos": ((8 * n, 3), self.dt), "sub_vel": ((8 * n, 3), self.dt),
                 "sub_acc": ((8 * n, 3), self.dt), "sub_rho": (8 * n, self.dt), "sub_p": (8 * n, self.dt),
                 "sub_scale_acc": (8 * n, self.dt)}
        shape, dt = sizes[what]
        out = np.zeros(shape, dt)
        if out.size:
            lib().orc_ts_get(self._h, 1 if self.fp64 else 0, self.WHAT[what], _ptr(out))
        return out

    def set_state(self, state: np.ndarray) -> None:
        a = np.ascontiguousarray(state, np.uint8)
        lib().orc_ts_get(self._h, 1 if self.fp64 else 0, 20, _ptr(a))

    def set_children(self, pos: np.ndarray, vel: np.ndarray) -> None:
        """Overwrites the 8n child positions and velocities (slot order)."""
        for what, a in ((21, pos), (22, vel)):
            a = np.ascontiguousarray(np.asarray(a).reshape(8 * self.n, 3), self.dt)
            lib().orc_ts_get(self._h, 1 if self.fp64 else 0, what, _ptr(a))

    def step(self, p, o, bm, pos, vel):
        """AdvanceTwoScale; returns the coarse outputs like step_plain."""
        n = self.n
        dt = self.dt
        pos = np.array(pos, dt, order="C", copy=True)
        vel = np.array(vel, dt, order="C", copy=True)
        rho, prs, acc = np.zeros(n, dt), np.zeros(n, dt), np.zeros((n, 3), dt)
        C = p.num_cells
        h, ids = np.zeros(n, np.int32), np.zeros(n, np.int32)
        start, end = np.zeros(C, np.int32), np.zeros(C, np.int32)
        fn = lib().orc_ts_step_f64 if self.fp64 else lib().orc_ts_step_f32
        mp = ctypes.byref(bm.maps) if bm is not None else None
        rc = fn(self._h, ctypes.byref(p), ctypes.byref(o), mp, _ptr(pos), _ptr(vel), _ptr(rho), _ptr(prs),
                _ptr(acc), _ptr(h), _ptr(ids), _ptr(start), _ptr(end))
        if rc:
            raise ValueError(f"oracle two-scale step failed ({rc})")
        return dict(pos=pos, vel=vel, rho=rho, p=prs, acc=acc, hash=h, ids=ids, start=start, end=end)

    def part(self, p, o, pos, vel, rho, prs, ids, start, end):
        """The two-scale part of AdvanceTwoScale from given coarse results."""
        dt = self.dt
        arrs = [np.ascontiguousarray(a, dt) for a in (pos, vel, rho, prs)]
        ints = [np.ascontiguousarray(a, np.int32) for a in (ids, start, end)]
        fn = lib().orc_ts_part_f64 if self.fp64 else lib().orc_ts_part_f32
        rc = fn(self._h, ctypes.byref(p), ctypes.byref(o), *[_ptr(a) for a in arrs], *[_ptr(a) for a in ints])
        if rc:
            raise ValueError(f"oracle two-scale part failed ({rc})")


def mesh_sdf(vertices, faces, origin, dx, dims, max_dist):
    """The oracle's mesh signed distance grid: (distance [k, j, i], normal [k, j, i, 3])."""
    L = lib()
    fn = L.orc_mesh_sdf
    fn.restype = None
    fn.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p, ctypes.c_float,
                   ctypes.c_void_p, ctypes.c_float, ctypes.c_void_p, ctypes.c_void_p]
    v = np.ascontiguousarray(vertices, np.float32).reshape(-1, 3)
    f = np.ascontiguousarray(faces, np.uint32).reshape(-1, 3)
    o = np.ascontiguousarray(origin, np.float32)
    d = np.ascontiguousarray(dims, np.uint32)
    dist = np.zeros((int(d[2]), int(d[1]), int(d[0])), np.float32)
    nrm = np.zeros(dist.shape + (3,), np.float32)
    fn(_ptr(v), len(v), _ptr(f), len(f), _ptr(o), float(dx), _ptr(d), float(max_dist), _ptr(dist), _ptr(nrm))
    return dist, nrm


def look_at(eye, centre, up):
    """cgtkGLLookAt (cgtk/src/opengl.c:10-46): column-major view matrix, float64."""
    e, c, u0 = (np.asarray(a, np.float64) for a in (eye, centre, up))
    n = c - e
    n /= np.linalg.norm(n)
    u = np.cross(n, u0)
    u /= np.linalg.norm(u)
    v = np.cross(u, n)
    m = np.zeros(16)
    for a in range(3):
        m[4 * a:4 * a + 3] = (u[a], v[a], -n[a])
    m[12], m[13], m[14], m[15] = -u @ e, -v @ e, n @ e, 1.0
    return m


def perspective(fovy, aspect, znear, zfar):
    """cgtkGLPerspective + cgtkGLFrustum (cgtk/src/opengl.c:48-78), float64."""
    t = np.tan((fovy / 2.0) * (3.141593 / 180.0))
    h = znear * t
    w = h * aspect
    m = np.zeros(16)
    m[0] = 2 * znear / (2 * w)
    m[5] = 2 * znear / (2 * h)
    m[10] = (zfar + znear) / (znear - zfar)
    m[11] = -1.0
    m[14] = -2 * zfar * znear / (zfar - znear)
    return m


def render_splats(view, proj, passes, width, height):
    """The TwoScaleStateSub shaders (twoscalestatesub_{v,g,f}.glsl) restated in
    float64 with GL's rasterisation: a pixel is covered when its centre lies
    inside a particle's quad, the fragment is kept when inside the unit disk,
    depth -proj[2][2] - proj[2][3]/zEye clamped to [0, 1] and stored as 24-bit
    fixed point, GL_LESS (the first drawn fragment keeps a tie), white clear.
    passes: [(positions (k, 3), radius, (r, g, b)), ...] in draw order.
    Returns (rgba uint8 (H, W, 4) rows top to bottom, winner draw index or -1)."""
    V = np.asarray(view, np.float64).reshape(4, 4).T  # column-major -> math
    Pm = np.asarray(proj, np.float64).reshape(4, 4).T
    key = np.full((height, width), np.iinfo(np.int64).max, np.int64)
    shade = np.zeros((height, width, 4))
    base = 0
    info = []
    for pos, R, rgb in passes:
        pos = np.asarray(pos, np.float64).reshape(-1, 3)
        for k in range(len(pos)):
            eye = V @ np.append(pos[k], 1.0)
            w = -eye[2]
            clip = Pm @ eye
            if not (w > 0 and abs(clip[2] / w) <= 1):
                continue
            cx, cy = clip[0] / w, clip[1] / w
            dx, dy = Pm[0, 0] * R / w, Pm[1, 1] * R / w
            i0 = max(int(np.ceil((cx - dx + 1) * 0.5 * width - 0.5)), 0)
            i1 = min(int(np.ceil((cx + dx + 1) * 0.5 * width - 0.5)) - 1, width - 1)
            j0 = max(int(np.ceil((cy - dy + 1) * 0.5 * height - 0.5)), 0)
            j1 = min(int(np.ceil((cy + dy + 1) * 0.5 * height - 0.5)) - 1, height - 1)
            if i1 < i0 or j1 < j0:
                continue
            ii, jj = np.meshgrid(np.arange(i0, i1 + 1), np.arange(j0, j1 + 1))
            u = ((ii + 0.5) * 2 / width - 1 - cx) / dx
            v = ((jj + 0.5) * 2 / height - 1 - cy) / dy
            norm = u * u + v * v
            inside = norm <= 1
            nz = np.sqrt(np.maximum(1 - norm, 0))
            zeye = eye[2] + R * nz
            z = np.clip(-Pm[2, 2] - Pm[3, 2] / zeye, 0, 1)
            d24 = np.rint(z * 16777215).astype(np.int64)
            kk = (d24 << 32) | (base + k)
            rows = height - 1 - jj
            cur = key[rows, ii]
            win = inside & (kk < cur)
            key[rows[win], ii[win]] = kk[win]
            atten = 0.9 + 0.1 * np.maximum(0, nz)
            col = np.stack([atten * rgb[0], atten * rgb[1], atten * rgb[2], atten], -1)
            shade[rows[win], ii[win]] = col[win]
        info.append(base)
        base += len(pos)
    empty = key == np.iinfo(np.int64).max
    rgba = np.rint(np.clip(shade, 0, 1) * 255).astype(np.uint8)
    rgba[empty] = 255
    winner = np.where(empty, -1, key & 0xFFFFFFFF)
    return rgba, winner


# ---------------------------------------------------------------------------
# The reference's own plain-step code on the host (oracle/_ref/libsph_ref.so,
# built by oracle/build_ref.py where the reference checkout is present).
# ---------------------------------------------------------------------------
REF_LIB_PATH = os.path.join(HERE, "_ref", "libsph_ref.so")
_ref = None


def ref_build() -> str | None:
    """Builds the reference harness if the checkout is present; its path or None."""
    import build_ref
    return build_ref.build()


def ref_available() -> bool:
    return os.path.exists(REF_LIB_PATH) or ref_build() is not None


def ref_lib():
    global _ref
    if _ref is None:
        if not os.path.exists(REF_LIB_PATH) and ref_build() is None:
            raise RuntimeError("the reference checkout is absent: oracle/_ref cannot be built")
        L = ctypes.CDLL(REF_LIB_PATH)
        vp = ctypes.c_void_p
        L.ref_step_plain.argtypes = [vp] * 8 + [ctypes.c_float, ctypes.c_float, ctypes.c_int] + [vp] * 4
        L.ref_step_plain.restype = ctypes.c_int
        L.ref_set_threads.argtypes = [ctypes.c_int]
        _ref = L
    return _ref


def ref_step_plain(p: SimulationParameters, bm: BoundaryMaps | None, pos: np.ndarray, vel: np.ndarray,
                   collide: bool) -> dict:
    """One plain step of the reference's own code (Advance, plus
    handleCollisions when `collide`): the cell tables and the new state."""
    n = int(p.numParticles)
    vd = np.ascontiguousarray(pos, np.float32).reshape(n, 3).copy()
    sd = np.zeros((n, 10), np.float32)
    sd[:, 6:9] = np.asarray(vel, np.float32).reshape(n, 3)
    C = p.num_cells
    h, ids = np.zeros(n, np.int32), np.zeros(n, np.int32)
    start, end = np.zeros(C, np.int32), np.zeros(C, np.int32)
    if bm is not None:
        dims = np.asarray(bm.dims, np.uint32)
        origin = np.asarray([bm.desc.gridStart[a] for a in range(3)], np.float32)
        maps = [_ptr(bm.dist), _ptr(bm.dens), _ptr(bm.visc), _ptr(dims), _ptr(origin)]
        spacing, rest = float(bm.desc.gridSpacing), float(bm.desc.restDistance)
    else:
        maps, spacing, rest = [None] * 5, 1.0, 0.0
    rc = ref_lib().ref_step_plain(ctypes.byref(p), _ptr(vd), _ptr(sd), *maps, spacing, rest, 1 if collide else 0,
                                  _ptr(h), _ptr(ids), _ptr(start), _ptr(end))
    if rc:
        raise ValueError("a particle hashed outside the reference's cell tables")
    return dict(hash=h, ids=ids, start=start, end=end, rho=sd[:, 1].copy(), p=sd[:, 2].copy(),
                acc=sd[:, 3:6].copy(), pos=vd, vel=sd[:, 6:9].copy())


def ref_set_threads(n: int) -> None:
    """Host threads the reference harness spreads a kernel's threads over."""
    ref_lib().ref_set_threads(int(n))
