"""Host-side mirror of the reference's simulator-backend interface, over the C ABI.

``GB300Simulator3D`` / ``GB300Simulator2D`` stand where the reference's ``CPUSimulator3D`` / ``CudaSimulator3D``
stand (include/simulation/simulator/ISimulator.h:8-53): ``update()`` runs the seven stages in the reference
order with the ``DISABLE_*`` gates of ``params.disable_mask``; the protected stage virtuals are exposed under
their reference names; ``solve()`` is ``ISolver::solve``; the grid accessors of ``IGrid3D``
(include/simulation/data/IGrid.h:44-68) return host copies in the reference layout and the ``set_*``
methods write them back, as the reference editor writes ``rho`` / ``boundary`` through those references.
"""
import ctypes

import numpy as np

from . import abi
from ._lib import EfsError, check, fptr, lib


class _GB300Simulator:
    def __init__(self, dim, width, height, depth, params=None):
        self.dim = dim
        self.width, self.height = width, height
        self.depth = depth if dim == 3 else 1
        self.shape = (self.depth, height, width) if dim == 3 else (height, width)
        if params is None:
            params = abi.params_default()
        self._params = params.copy()
        h = ctypes.c_void_p()
        L = lib()
        st = L.efs_create(dim, width, height, self.depth, ctypes.byref(self._params), ctypes.byref(h))
        if st != 0:
            raise EfsError(st, L.efs_last_error(None).decode())
        self._h = h

    def close(self):
        if getattr(self, "_h", None):
            lib().efs_destroy(self._h)
            self._h = None

    def __del__(self):
        self.close()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    # ---- parameters (Properties values) ----
    @property
    def params(self):
        return self._params.copy()

    def set_params(self, params):
        check(lib().efs_set_params(self._h, ctypes.byref(params)), self._h)
        self._params = params.copy()

    # ---- ISimulator ----
    def update(self, n=1):
        """ISimulator::update() n times (asynchronous; fields and stats synchronise)."""
        check(lib().efs_step(self._h, n), self._h)

    def stage(self, s):
        check(lib().efs_stage(self._h, s), self._h)

    def vel_decay(self):
        self.stage(abi.STAGE_VEL_DECAY)

    def vel_extrapolate(self):
        self.stage(abi.STAGE_VEL_EXTRAPOLATE)

    def rho_sharpen(self):
        self.stage(abi.STAGE_RHO_SHARPEN)

    def rho_advect(self):
        self.stage(abi.STAGE_RHO_ADVECT)

    def vel_advect(self):
        self.stage(abi.STAGE_VEL_ADVECT)

    def add_force(self):
        self.stage(abi.STAGE_ADD_FORCE)

    def project(self):
        self.stage(abi.STAGE_PROJECT)

    # ---- ISolver ----
    def solve(self):
        """ISolver::solve on the current divergence; returns the stats (raises EfsError if not converged)."""
        s = abi.EfsStats()
        check(lib().efs_solve(self._h, ctypes.byref(s)), self._h)
        return s

    def synchronize(self):
        check(lib().efs_synchronize(self._h), self._h)

    def stats(self):
        s = abi.EfsStats()
        check(lib().efs_get_stats(self._h, ctypes.byref(s)), self._h)
        return s

    def total_mass(self):
        m = ctypes.c_double()
        check(lib().efs_total_mass(self._h, ctypes.byref(m)), self._h)
        return m.value

    # ---- IGrid ----
    def _fshape(self, f):
        return self.shape + (self.dim,) if f in abi.VECTOR_FIELDS else self.shape

    def field(self, f):
        out = np.empty(self._fshape(f), np.float32)
        check(lib().efs_download_field(self._h, f, fptr(out)), self._h)
        return out

    def set_field(self, f, arr):
        a = np.ascontiguousarray(arr, dtype=np.float32)
        if a.size != int(np.prod(self._fshape(f))):
            raise ValueError(f"{abi.FIELD_NAMES[f]}: expected {self._fshape(f)}, got {a.shape}")
        check(lib().efs_upload_field(self._h, f, fptr(a)), self._h)

    def fields(self):
        return {f: self.field(f) for f in range(abi.FIELD_COUNT)}

    def set_fields(self, fields):
        if abi.FIELD_BOUNDARY in fields:
            self.set_field(abi.FIELD_BOUNDARY, fields[abi.FIELD_BOUNDARY])
        for f, a in fields.items():
            if f != abi.FIELD_BOUNDARY:
                self.set_field(f, a)

    def reset(self):
        check(lib().efs_reset_fields(self._h), self._h)

    # ---- scene construction and queries (Editor / scene nodes) ----
    @staticmethod
    def _tris(triangles):
        """[n, 3, 3] world-space vertices -> the reference Triangle layout (12 floats per triangle)."""
        t = np.asarray(triangles, np.float32).reshape(-1, 3, 3)
        out = np.zeros((len(t), 3, 4), np.float32)
        out[:, :, :3] = t
        return out

    @staticmethod
    def _vec3(v):
        return np.ascontiguousarray(np.asarray(v, np.float32).reshape(3))

    @staticmethod
    def _ivec3(v):
        return (ctypes.c_int * 3)(*[int(x) for x in v])

    def mesh_label(self, field, triangles, domain_center, domain_size, value_inside=1.0, value_outside=0.0):
        t = self._tris(triangles)
        c, s = self._vec3(domain_center), self._vec3(domain_size)
        check(lib().efs_mesh_label(self._h, field, fptr(t), len(t), fptr(c), fptr(s), value_inside, value_outside),
              self._h)

    def mesh_cells(self, triangles, domain_center, domain_size, capacity=None):
        """Inside cells (ascending linear indices) and their total number (which may exceed capacity)."""
        t = self._tris(triangles)
        c, s = self._vec3(domain_center), self._vec3(domain_size)
        cap = int(np.prod(self.shape)) if capacity is None else int(capacity)
        cells = np.zeros(max(cap, 1), np.int32)
        n = ctypes.c_longlong()
        check(lib().efs_mesh_cells(self._h, fptr(t), len(t), fptr(c), fptr(s),
                                   cells.ctypes.data_as(ctypes.POINTER(ctypes.c_int)), cap, ctypes.byref(n)), self._h)
        return cells[:min(n.value, cap)], n.value

    def _value(self, field, value):
        comps = self.dim if field in abi.VECTOR_FIELDS else 1
        v = np.zeros(3, np.float32)
        v[:comps] = np.broadcast_to(np.asarray(value, np.float32), (comps,))
        return v

    def fill_box(self, field, lo, hi, value):
        v = self._value(field, value)
        check(lib().efs_fill_box(self._h, field, self._ivec3(lo), self._ivec3(hi), fptr(v)), self._h)

    def set_cells(self, field, cells, value):
        idx = np.ascontiguousarray(np.asarray(cells, np.int64).astype(np.int32))
        v = self._value(field, value)
        check(lib().efs_set_cells(self._h, field, idx.ctypes.data_as(ctypes.POINTER(ctypes.c_int)), len(idx), fptr(v)),
              self._h)

    def seal_boundary(self):
        check(lib().efs_seal_boundary(self._h), self._h)

    def query_box(self, position, scale, only_fluid=True):
        m = abi.EfsQueryMetrics()
        check(lib().efs_query_box(self._h, self._ivec3(position), self._ivec3(scale), int(only_fluid), ctypes.byref(m)),
              self._h)
        return m

    def vel(self):
        return self.field(abi.FIELD_VEL)

    def rho(self):
        return self.field(abi.FIELD_RHO)

    def gamma(self):
        return self.field(abi.FIELD_GAMMA)

    def beta(self):
        return self.field(abi.FIELD_BETA)

    def divergence(self):
        return self.field(abi.FIELD_DIVERGENCE)

    def pressure(self):
        return self.field(abi.FIELD_PRESSURE)

    def forces(self):
        return self.field(abi.FIELD_FORCES)

    def boundary(self):
        return self.field(abi.FIELD_BOUNDARY)

    def kernels_per_step(self):
        n = ctypes.c_int()
        check(lib().efs_step_kernel_count(self._h, ctypes.byref(n)), self._h)
        return n.value

    def mark(self, slot):
        """Record CUDA event `slot` on the simulator's stream."""
        check(lib().efs_timer_mark(self._h, slot), self._h)

    def elapsed_ms(self, a, b):
        ms = ctypes.c_double()
        check(lib().efs_timer_elapsed(self._h, a, b, ctypes.byref(ms)), self._h)
        return ms.value

    def upload_fields(self, vel=None, rho=None, gamma=None, boundary=None, forces=None):
        """efs_upload_fields (CudaGrid3D::upload): host arrays in the reference layout; None skips."""
        check(lib().efs_upload_fields(self._h, fptr(vel), fptr(rho), fptr(gamma), fptr(boundary), fptr(forces)), self._h)

    def download_fields(self, vel=None, rho=None, gamma=None, beta=None, divergence=None, pressure=None):
        """efs_download_fields (CudaGrid3D::download) into host arrays; None skips."""
        check(lib().efs_download_fields(self._h, fptr(vel), fptr(rho), fptr(gamma), fptr(beta), fptr(divergence),
                                        fptr(pressure)), self._h)

    def step_host(self, vel=None, rho=None, gamma=None, boundary=None, forces=None, vel_out=None, rho_out=None,
                  gamma_out=None, beta_out=None, divergence_out=None, pressure_out=None):
        """efs_step_host: upload, one step, download in one call (transfers overlap the step when the buffers
        are page-locked); None skips a field."""
        check(lib().efs_step_host(self._h, fptr(vel), fptr(rho), fptr(gamma), fptr(boundary), fptr(forces),
                                  fptr(vel_out), fptr(rho_out), fptr(gamma_out), fptr(beta_out), fptr(divergence_out),
                                  fptr(pressure_out)), self._h)

    def pressure_fp64(self):
        """efs_download_pressure_fp64: the FP64 pressure of the last CG solve, shaped like the fields."""
        out = np.empty(self._fshape(abi.FIELD_PRESSURE), np.float64)
        check(lib().efs_download_pressure_fp64(self._h, out.ctypes.data_as(ctypes.POINTER(ctypes.c_double))), self._h)
        return out

    # ---- learned preconditioner (3D) ----
    def unet_init(self, seed=0, sample_capacity=0):
        check(lib().efs_unet_init(self._h, seed, sample_capacity), self._h)

    def unet_grid(self):
        """(width, height, depth, level): the grid the network works on, `level` aggregation levels below the
        context's grid (the FCG preconditioner's bottom level; 0 = the context's own grid)."""
        v = [ctypes.c_int() for _ in range(4)]
        check(lib().efs_unet_grid(self._h, *[ctypes.byref(x) for x in v]), self._h)
        return tuple(x.value for x in v)

    def unet_weights(self):
        out = np.empty(unet_param_count(), np.float32)
        check(lib().efs_unet_get_weights(self._h, fptr(out), out.size), self._h)
        return out

    def unet_set_weights(self, w):
        a = np.ascontiguousarray(w, dtype=np.float32)
        check(lib().efs_unet_set_weights(self._h, fptr(a), a.size), self._h)

    def unet_apply(self, r):
        """z = net(r) for a field of the network's grid (unet_grid)."""
        a = np.ascontiguousarray(r, dtype=np.float32)
        z = np.empty_like(a)
        check(lib().efs_unet_apply(self._h, fptr(a), fptr(z)), self._h)
        return z

    def unet_loss_grad(self, b, p, grads=True, loss_kind=0):
        bb = np.ascontiguousarray(b, dtype=np.float32)
        pp = np.ascontiguousarray(p, dtype=np.float32)
        loss = ctypes.c_float()
        g = np.empty(unet_param_count(), np.float32) if grads else None
        check(lib().efs_unet_loss_grad(self._h, loss_kind, fptr(bb), fptr(pp), ctypes.byref(loss), fptr(g)), self._h)
        return loss.value, g

    def unet_time_forward(self, reps=5):
        """(ms per forward pass, ms per convolution layer [6]) on the device."""
        ms = np.zeros(1, np.float32)
        lay = np.zeros(6, np.float32)
        check(lib().efs_unet_time_forward(self._h, reps, fptr(ms), fptr(lay)), self._h)
        return float(ms[0]), lay

    def fcg_time_vcycle(self, reps=5):
        """efs_fcg_time_vcycle: (ms per preconditioner application launched kernel by kernel, ms per replay of
        one captured application) on the current divergence."""
        d = np.zeros(1, np.float32)
        g = np.zeros(1, np.float32)
        check(lib().efs_fcg_time_vcycle(self._h, reps, fptr(d), fptr(g)), self._h)
        return float(d[0]), float(g[0])

    def unet_add_sample(self):
        check(lib().efs_unet_add_sample(self._h), self._h)

    def unet_sample_count(self):
        n = ctypes.c_int()
        check(lib().efs_unet_sample_count(self._h, ctypes.byref(n)), self._h)
        return n.value

    def unet_train(self, iterations, batch=4, lr=1e-3, synthetic=0.5, seed=0, loss_kind=1):
        loss = ctypes.c_float()
        check(lib().efs_unet_train(self._h, loss_kind, iterations, batch, lr, synthetic, seed, ctypes.byref(loss)),
              self._h)
        return loss.value

    # ---- timing of the pressure solve ----
    def solve_timing_arm(self, capacity):
        check(lib().efs_solve_timing_arm(self._h, capacity), self._h)

    def solve_timing_read(self):
        n = ctypes.c_int()
        ms = ctypes.c_double()
        ri = ctypes.c_double()
        rs = ctypes.c_double()
        check(lib().efs_solve_timing_read(self._h, ctypes.byref(n), ctypes.byref(ms), ctypes.byref(ri), ctypes.byref(rs)), self._h)
        return n.value, ms.value, ri.value, rs.value


class GB300Simulator3D(_GB300Simulator):
    """Drop-in for the reference's 3D backends (ISimulator3D(w, h, d), ISimulator3D.h:6-14)."""

    def __init__(self, width, height, depth, params=None):
        super().__init__(3, width, height, depth, params)


class GB300Simulator2D(_GB300Simulator):
    """Drop-in for the reference's 2D backends (ISimulator2D(w, h), ISimulator2D.h:6-13)."""

    def __init__(self, width, height, params=None):
        super().__init__(2, width, height, 1, params)


class GB300Batch2D:
    """Many independent 2D scenes of uneven sizes advanced together (efs_batch_*): scene s is a
    ``widths[s] x heights[s]`` grid (border included); all share ``params`` except the optional per-scene
    ``gravity`` (GRAVITY_FORCE in cells/s^2)."""

    def __init__(self, widths, heights, params, gravity=None):
        self.widths = [int(w) for w in widths]
        self.heights = [int(h) for h in heights]
        n = len(self.widths)
        W = (ctypes.c_int * n)(*self.widths)
        H = (ctypes.c_int * n)(*self.heights)
        g = None if gravity is None else np.ascontiguousarray(gravity, np.float32)
        self._params = params.copy()
        h = ctypes.c_void_p()
        L = lib()
        st = L.efs_batch_create(n, W, H, ctypes.byref(self._params), fptr(g), ctypes.byref(h))
        if st != 0:
            raise EfsError(st, L.efs_batch_last_error(None).decode())
        self._h = h

    def _check(self, st):
        if st != 0:
            raise EfsError(st, lib().efs_batch_last_error(self._h).decode())

    def close(self):
        if getattr(self, "_h", None):
            lib().efs_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        self.close()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    @property
    def n(self):
        return len(self.widths)

    def _shape(self, s, f):
        shp = (self.heights[s], self.widths[s])
        return shp + (2,) if f in abi.VECTOR_FIELDS else shp

    def set_field(self, s, f, arr):
        a = np.ascontiguousarray(arr, dtype=np.float32)
        if a.size != int(np.prod(self._shape(s, f))):
            raise ValueError(f"scene {s} {abi.FIELD_NAMES[f]}: expected {self._shape(s, f)}, got {a.shape}")
        self._check(lib().efs_batch_upload_field(self._h, s, f, fptr(a)))

    def field(self, s, f):
        out = np.empty(self._shape(s, f), np.float32)
        self._check(lib().efs_batch_download_field(self._h, s, f, fptr(out)))
        return out

    def stage(self, st):
        self._check(lib().efs_batch_stage(self._h, st))

    def update(self, n=1):
        self._check(lib().efs_batch_step(self._h, n))

    def synchronize(self):
        self._check(lib().efs_batch_synchronize(self._h))

    def time_steps(self, n):
        """n steps timed with CUDA events on the batch's stream; device milliseconds."""
        ms = np.zeros(1, np.float32)
        self._check(lib().efs_batch_time_steps(self._h, n, fptr(ms)))
        return float(ms[0])

    def stats(self, s):
        out = abi.EfsStats()
        self._check(lib().efs_batch_stats(self._h, s, ctypes.byref(out)))
        return out

    def kernels_per_step(self):
        n = ctypes.c_int()
        self._check(lib().efs_batch_kernel_count(self._h, ctypes.byref(n)))
        return n.value

    def tuning(self):
        t = abi.EfsBatchTuning()
        self._check(lib().efs_batch_get_tuning(self._h, ctypes.byref(t)))
        return t

    def set_tuning(self, t):
        self._check(lib().efs_batch_set_tuning(self._h, ctypes.byref(t)))

    def autotune(self, trial_steps=3):
        t = abi.EfsBatchTuning()
        self._check(lib().efs_batch_autotune(self._h, trial_steps, ctypes.byref(t)))
        return t


def unet_param_count():
    n = ctypes.c_int64()
    check(lib().efs_unet_param_count(ctypes.byref(n)))
    return n.value


def device_count():
    n = ctypes.c_int()
    check(lib().efs_device_count(ctypes.byref(n)))
    return n.value


def scene_dam3d(w, h, d, n_min, n_max, seed):
    b = np.zeros((d, h, w), np.float32)
    r = np.zeros((d, h, w), np.float32)
    check(lib().efs_scene_dam3d(w, h, d, n_min, n_max, seed, fptr(b), fptr(r)))
    return b, r


def scene_dam2d(w, h):
    b = np.zeros((h, w), np.float32)
    r = np.zeros((h, w), np.float32)
    check(lib().efs_scene_dam2d(w, h, fptr(b), fptr(r)))
    return b, r


def scene_batch2d(seed):
    s = ctypes.c_int()
    check(lib().efs_scene_batch2d(seed, ctypes.byref(s), None, None, 0))
    b = np.zeros((s.value, s.value), np.float32)
    r = np.zeros((s.value, s.value), np.float32)
    check(lib().efs_scene_batch2d(seed, ctypes.byref(s), fptr(b), fptr(r), b.size))
    return b, r


def params_dam(cell_size, dt, solver=abi.SOLVER_CG, tol_rel=1e-6):
    """efs_params_dam from the library (the C preset)."""
    p = abi.EfsParams()
    lib().efs_params_dam(ctypes.byref(p), cell_size, dt, solver, tol_rel)
    return p
