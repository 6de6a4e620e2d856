"""Python binding of the CPU oracle.  TEST INFRASTRUCTURE ONLY.

``Oracle`` wraps the C restatement (``oracle/liborc.so`` built from ``efs_oracle.c``); ``RefOracle`` wraps the
reference's own CPU backend compiled from its sources (``oracle/_ref/libefs_ref.so``, only where the
reference tree exists).  Both expose the same calls as the product binding so tests can run the three side by
side: ``set_field`` / ``field`` (reference layout), ``stage``, ``step``, ``stats``.

Only ``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline leg use this module.
"""
import ctypes
import os
import subprocess

import numpy as np

from eulerianfluidsimulation_gb300.abi import (EfsParams, EfsStats, FIELD_COUNT, VECTOR_FIELDS)

HERE = os.path.dirname(os.path.abspath(__file__))
LIBORC = os.path.join(HERE, "liborc.so")
LIBREF = os.path.join(HERE, "_ref", "libefs_ref.so")

DOTS_FP64 = 1
SHARPEN_PARALLEL = 2
REVERSE_SUMS = 4


def reference_tree():
    """Where the reference's source tree is: $EFS_REFERENCE_TREE, else the build recipe's default (the REF
    variable of oracle/Makefile).  The path may not exist (machines without the reference)."""
    env = os.environ.get("EFS_REFERENCE_TREE")
    if env:
        return env
    with open(os.path.join(HERE, "Makefile")) as fh:
        for line in fh:
            if line.startswith("REF ?="):
                return line.split("?=", 1)[1].strip()
    return ""


def reference_tree_present():
    t = reference_tree()
    return bool(t) and os.path.isdir(os.path.join(t, "src"))


def build(reference=True):
    """Build liborc.so and, when the reference tree is present, _ref/libefs_ref.so."""
    subprocess.check_call(["make", "-s", "-C", HERE, "oracle"])
    if reference and reference_tree_present():
        subprocess.check_call(["make", "-s", "-C", HERE, "ref", "REF=" + reference_tree()])


def reference_available():
    return os.path.exists(LIBREF)


def dropin_driver():
    """Build _ref/dropin_driver (tests/dropin_driver.cpp: the C++ drop-in backend and the reference's
    CPUSimulator3D behind its ISimulator3D interface) and return its path.  Needs the reference tree and
    libefs_gb300.so."""
    build(reference=True)
    subprocess.check_call(["make", "-s", "-C", HERE, "dropin", "REF=" + reference_tree()])
    return os.path.join(HERE, "_ref", "dropin_driver")


def dropin_reference(n, frames):
    """The reference's CPUSimulator3D::update() for `frames` frames on the driver's seeded n^3 dam break, with
    the Properties set as the application does: {"steps", "paused"} per frame, "params" (the efs_params the C++
    drop-in derives from those Properties) and the fields after the last frame, keyed by field id."""
    import tempfile
    from eulerianfluidsimulation_gb300 import abi
    with tempfile.TemporaryDirectory() as d:
        out = os.path.join(d, "ref.bin")
        subprocess.check_call([dropin_driver(), "reference", str(n), str(frames), out])
        raw = open(out, "rb").read()
    head = np.frombuffer(raw[:8], np.int32)
    assert head[0] == n and head[1] == frames
    off = 8
    steps = np.frombuffer(raw[off:off + 4 * frames], np.int32).copy()
    off += 4 * frames
    paused = np.frombuffer(raw[off:off + 4 * frames], np.int32).copy()
    off += 4 * frames
    psize = ctypes.sizeof(EfsParams)
    prm = EfsParams.from_buffer_copy(raw[off:off + psize])
    off += psize
    N = n * n * n
    fl = np.frombuffer(raw[off:], np.float32)
    assert fl.size == 8 * N
    fields = {abi.FIELD_VEL: fl[:3 * N].reshape(n, n, n, 3).copy()}
    for k, f in enumerate((abi.FIELD_RHO, abi.FIELD_GAMMA, abi.FIELD_BETA, abi.FIELD_DIVERGENCE, abi.FIELD_PRESSURE)):
        fields[f] = fl[(3 + k) * N:(4 + k) * N].reshape(n, n, n).copy()
    return {"steps": steps, "paused": paused, "params": prm, "fields": fields}


_orc = None
_ref = None
_FP = ctypes.POINTER(ctypes.c_float)


def _load_orc():
    global _orc
    if _orc is None:
        if not os.path.exists(LIBORC):
            build(reference=False)
        lib = ctypes.CDLL(LIBORC)
        lib.orc_create.restype = ctypes.c_void_p
        lib.orc_create.argtypes = [ctypes.c_int] * 4 + [ctypes.POINTER(EfsParams)]
        lib.orc_destroy.argtypes = [ctypes.c_void_p]
        lib.orc_set_params.argtypes = [ctypes.c_void_p, ctypes.POINTER(EfsParams)]
        lib.orc_set_mode.argtypes = [ctypes.c_void_p, ctypes.c_int]
        lib.orc_field.restype = _FP
        lib.orc_field.argtypes = [ctypes.c_void_p, ctypes.c_int]
        lib.orc_reset.argtypes = [ctypes.c_void_p]
        lib.orc_stage.argtypes = [ctypes.c_void_p, ctypes.c_int]
        lib.orc_step.argtypes = [ctypes.c_void_p, ctypes.c_int]
        lib.orc_solve.restype = ctypes.c_float
        lib.orc_solve.argtypes = [ctypes.c_void_p]
        lib.orc_stats.argtypes = [ctypes.c_void_p, ctypes.POINTER(EfsStats)]
        lib.orc_solve_fp64.restype = ctypes.c_int
        lib.orc_solve_fp64.argtypes = [ctypes.c_void_p, ctypes.c_double, ctypes.c_int, ctypes.POINTER(ctypes.c_double)]
        lib.orc_relres_fp64.restype = ctypes.c_double
        lib.orc_relres_fp64.argtypes = [ctypes.c_void_p, _FP]
        lib.orc_total_mass.restype = ctypes.c_double
        lib.orc_total_mass.argtypes = [ctypes.c_void_p]
        lib.orc_params_default.argtypes = [ctypes.POINTER(EfsParams)]
        lib.orc_scene_dam3d.restype = ctypes.c_int
        lib.orc_scene_dam3d.argtypes = [ctypes.c_int] * 5 + [ctypes.c_uint64, _FP, _FP]
        lib.orc_scene_dam2d.restype = ctypes.c_int
        lib.orc_scene_dam2d.argtypes = [ctypes.c_int, ctypes.c_int, _FP, _FP]
        lib.orc_scene_batch2d.restype = ctypes.c_int
        lib.orc_scene_batch2d.argtypes = [ctypes.c_uint64, ctypes.POINTER(ctypes.c_int), _FP, _FP]
        lib.orc_mesh_label.argtypes = [ctypes.c_int] * 3 + [_FP, ctypes.c_int, _FP, _FP, ctypes.c_float,
                                                            ctypes.c_float, _FP]
        lib.orc_query_box.restype = ctypes.c_longlong
        lib.orc_query_box.argtypes = [ctypes.c_int] * 4 + [_FP] * 5 + [ctypes.POINTER(ctypes.c_int)] * 2 + \
            [ctypes.c_int, _FP]
        _orc = lib
    return _orc


def _load_ref():
    global _ref
    if _ref is None:
        lib = ctypes.CDLL(LIBREF)
        lib.ref_create.restype = ctypes.c_void_p
        lib.ref_create.argtypes = [ctypes.c_int] * 4 + [ctypes.POINTER(EfsParams)]
        lib.ref_destroy.argtypes = [ctypes.c_void_p]
        lib.ref_set_params.argtypes = [ctypes.c_void_p, ctypes.POINTER(EfsParams)]
        lib.ref_field.restype = _FP
        lib.ref_field.argtypes = [ctypes.c_void_p, ctypes.c_int]
        lib.ref_step.argtypes = [ctypes.c_void_p, ctypes.c_int]
        lib.ref_stage.argtypes = [ctypes.c_void_p, ctypes.c_int]
        lib.ref_stats.argtypes = [ctypes.c_void_p, ctypes.POINTER(EfsStats)]
        lib.ref_query_box.restype = ctypes.c_longlong
        lib.ref_query_box.argtypes = [ctypes.c_void_p, _FP, _FP, ctypes.c_int, _FP]
        _ref = lib
    return _ref


def _fptr(a):
    return a.ctypes.data_as(_FP)


def scene_dam3d(w, h, d, n_min, n_max, seed):
    """Seeded 3D dam break with spheres (include/efs_scene.h) -> (boundary, rho) float32 arrays (d, h, w)."""
    lib = _load_orc()
    b = np.zeros((d, h, w), np.float32)
    r = np.zeros((d, h, w), np.float32)
    n = lib.orc_scene_dam3d(w, h, d, n_min, n_max, seed, _fptr(b), _fptr(r))
    if n < 0:
        raise ValueError("bad scene arguments")
    return b, r


def scene_dam2d(w, h):
    lib = _load_orc()
    b = np.zeros((h, w), np.float32)
    r = np.zeros((h, w), np.float32)
    if lib.orc_scene_dam2d(w, h, _fptr(b), _fptr(r)) < 0:
        raise ValueError("bad scene arguments")
    return b, r


def scene_batch2d(seed):
    lib = _load_orc()
    side = ctypes.c_int(0)
    lib.orc_scene_batch2d(seed, ctypes.byref(side), None, None)
    s = side.value
    b = np.zeros((s, s), np.float32)
    r = np.zeros((s, s), np.float32)
    lib.orc_scene_batch2d(seed, ctypes.byref(side), _fptr(b), _fptr(r))
    return b, r


class _Base:
    def __init__(self, dim, w, h, d, params):
        self.dim, self.w, self.h = dim, w, h
        self.d = d if dim == 3 else 1
        self.shape = (self.d, h, w) if dim == 3 else (h, w)
        self.params = params.copy()

    def _shape(self, f):
        return self.shape + (self.dim,) if f in VECTOR_FIELDS else self.shape

    def field(self, f):
        n = int(np.prod(self._shape(f)))
        ptr = self._ptr(f)
        return np.ctypeslib.as_array(ptr, shape=(n,)).reshape(self._shape(f)).copy()

    def set_field(self, f, arr):
        n = int(np.prod(self._shape(f)))
        src = np.ascontiguousarray(arr, dtype=np.float32).reshape(-1)
        if src.size != n:
            raise ValueError("field size mismatch")
        ctypes.memmove(self._ptr(f), src.ctypes.data, n * 4)

    def fields(self):
        return {f: self.field(f) for f in range(FIELD_COUNT)}

    def set_fields(self, fields):
        for f, a in fields.items():
            self.set_field(f, a)


class Oracle(_Base):
    """The C restatement of the reference CPU path (efs_oracle.c)."""

    def __init__(self, dim, w, h, d=1, params=None, mode=0):
        lib = _load_orc()
        if params is None:
            params = EfsParams()
            lib.orc_params_default(ctypes.byref(params))
        super().__init__(dim, w, h, d, params)
        self._lib = lib
        self._h = lib.orc_create(dim, w, h, self.d, ctypes.byref(self.params))
        if not self._h:
            raise ValueError("orc_create failed")
        lib.orc_set_mode(self._h, mode)

    def __del__(self):
        if getattr(self, "_h", None):
            self._lib.orc_destroy(self._h)
            self._h = None

    def _ptr(self, f):
        return self._lib.orc_field(self._h, f)

    def set_params(self, params):
        self.params = params.copy()
        self._lib.orc_set_params(self._h, ctypes.byref(self.params))

    def set_mode(self, mode):
        self._lib.orc_set_mode(self._h, mode)

    def reset(self):
        self._lib.orc_reset(self._h)

    def stage(self, s):
        self._lib.orc_stage(self._h, s)

    def step(self, n=1):
        self._lib.orc_step(self._h, n)

    def solve(self):
        return self._lib.orc_solve(self._h)

    def stats(self):
        s = EfsStats()
        self._lib.orc_stats(self._h, ctypes.byref(s))
        return s

    def solve_fp64(self, tol=1e-12, maxit=100000):
        p = np.zeros(self.shape, np.float64)
        it = self._lib.orc_solve_fp64(self._h, tol, maxit, p.ctypes.data_as(ctypes.POINTER(ctypes.c_double)))
        return p, it

    def relres_fp64(self, p):
        p = np.ascontiguousarray(p, dtype=np.float32)
        return self._lib.orc_relres_fp64(self._h, _fptr(p))

    def total_mass(self):
        return self._lib.orc_total_mass(self._h)


class RefOracle(_Base):
    """The reference's own CPUSimulator2D/3D compiled from its sources with the shim include directory."""

    def __init__(self, dim, w, h, d=1, params=None):
        if not reference_available():
            raise RuntimeError("oracle/_ref/libefs_ref.so is not built (needs the reference tree)")
        lib = _load_ref()
        super().__init__(dim, w, h, d, params)
        self._lib = lib
        self._h = lib.ref_create(dim, w, h, self.d, ctypes.byref(self.params))

    def __del__(self):
        if getattr(self, "_h", None):
            self._lib.ref_destroy(self._h)
            self._h = None

    def _ptr(self, f):
        return self._lib.ref_field(self._h, f)

    def set_params(self, params):
        self.params = params.copy()
        self._lib.ref_set_params(self._h, ctypes.byref(self.params))

    def stage(self, s):
        self._lib.ref_stage(self._h, s)

    def step(self, n=1):
        self._lib.ref_step(self._h, n)

    def stats(self):
        s = EfsStats()
        self._lib.ref_stats(self._h, ctypes.byref(s))
        return s

    def query_box(self, position, scale, only_fluid=True):
        """QueryNode::update's metric loop (the reference's own lines) on this 3D grid -> (metrics, count)."""
        pos = np.asarray(position, np.float32)
        scl = np.asarray(scale, np.float32)
        out = np.zeros(13, np.float32)
        n = self._lib.ref_query_box(self._h, _fptr(pos), _fptr(scl), int(only_fluid), _fptr(out))
        m = {"max_position": out[0:3].copy(), "min_position": out[3:6].copy(), "avg_position": out[6:9].copy(),
             "velocity": out[9:12].copy(), "pressure": float(out[12])}
        return m, int(n)


def mesh_label(shape, triangles, center, size, value_inside=1.0, value_outside=0.0, out=None):
    """sdf.comp's label of every cell of [0, W-1) x [0, H-1) x [0, D-1) (restated in scene_oracle.c).
    shape = (D, H, W); triangles: [n, 3, 3] world coordinates; other cells of `out` (default zeros) kept."""
    D, H, W = shape
    t = np.zeros((len(triangles), 3, 4), np.float32)
    t[:, :, :3] = np.asarray(triangles, np.float32).reshape(-1, 3, 3)
    o = np.zeros(shape, np.float32) if out is None else np.ascontiguousarray(out, np.float32).copy()
    c = np.asarray(center, np.float32)
    s = np.asarray(size, np.float32)
    _load_orc().orc_mesh_label(W, H, D, _fptr(t), len(t), _fptr(c), _fptr(s), value_inside, value_outside, _fptr(o))
    return o


def query_box(rho, vel, pressure, position, scale, only_fluid=True):
    """QueryNode::update's metrics (restated in scene_oracle.c).  rho, pressure: [D, H, W] or [H, W];
    vel: [..., dim].  Returns (dict of floats, count)."""
    rho = np.ascontiguousarray(rho, np.float32)
    dim = rho.ndim
    shape = rho.shape if dim == 3 else (1,) + rho.shape
    vel = np.asarray(vel, np.float32)
    u = np.ascontiguousarray(vel[..., 0])
    v = np.ascontiguousarray(vel[..., 1])
    w = np.ascontiguousarray(vel[..., 2]) if dim == 3 else None
    p = np.ascontiguousarray(pressure, np.float32)
    out = np.zeros(13, np.float32)
    pos = (ctypes.c_int * 3)(*[int(x) for x in position])
    sc = (ctypes.c_int * 3)(*[int(x) for x in scale])
    n = _load_orc().orc_query_box(dim, shape[2], shape[1], shape[0], _fptr(rho), _fptr(u), _fptr(v),
                                  _fptr(w) if w is not None else None, _fptr(p), pos, sc, int(only_fluid), _fptr(out))
    m = {"max_position": out[0:3].copy(), "min_position": out[3:6].copy(), "avg_position": out[6:9].copy(),
         "velocity": out[9:12].copy(), "pressure": float(out[12])}
    return m, int(n)
