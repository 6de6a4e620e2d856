"""ctypes mirror of ``include/efs_gb300.h``: enums, ``efs_params`` / ``efs_stats`` and the parameter presets.

Pure Python (no library is loaded here), so both the CUDA binding and the test harness can share it.
The presets restate the C ones in ``efs_api.cu`` (``efs_params_default`` / ``efs_params_dam``); a test checks
that the two agree field by field.
"""
import ctypes

# stages, in ISimulator::update order (include/simulation/simulator/ISimulator.h:15-35)
STAGE_VEL_DECAY = 0
STAGE_VEL_EXTRAPOLATE = 1
STAGE_RHO_SHARPEN = 2
STAGE_RHO_ADVECT = 3
STAGE_VEL_ADVECT = 4
STAGE_ADD_FORCE = 5
STAGE_PROJECT = 6
STAGE_COUNT = 7
STAGE_NAMES = ("vel_decay", "vel_extrapolate", "rho_sharpen", "rho_advect", "vel_advect", "add_force", "project")

SOLVER_JACOBI = 0
SOLVER_CG = 1
SOLVER_FCG_UNET = 2

FCG_BOTTOM_UNET = 0
FCG_BOTTOM_JACOBI = 1

SHARPEN_PARALLEL = 0
SHARPEN_SEQUENTIAL = 1

CG_MIXED = 0
CG_REFERENCE = 1
CG_MIXED_RECURRENCE = 2
CG_FP64 = 3
CG_PIPELINED = 4

FIELD_VEL = 0
FIELD_RHO = 1
FIELD_GAMMA = 2
FIELD_BETA = 3
FIELD_DIVERGENCE = 4
FIELD_PRESSURE = 5
FIELD_FORCES = 6
FIELD_BOUNDARY = 7
FIELD_COUNT = 8
FIELD_NAMES = ("vel", "rho", "gamma", "beta", "divergence", "pressure", "forces", "boundary")
VECTOR_FIELDS = (FIELD_VEL, FIELD_FORCES)

EFS_OK = 0
EFS_ERR_ARG = 1
EFS_ERR_CUDA = 2
EFS_ERR_STATE = 3
EFS_ERR_NO_DEVICE = 4
EFS_ERR_DEVICE_FAULT = 5
EFS_ERR_NOT_CONVERGED = 6
STATUS_NAMES = {0: "EFS_OK", 1: "EFS_ERR_ARG", 2: "EFS_ERR_CUDA", 3: "EFS_ERR_STATE", 4: "EFS_ERR_NO_DEVICE",
                5: "EFS_ERR_DEVICE_FAULT", 6: "EFS_ERR_NOT_CONVERGED"}


class EfsParams(ctypes.Structure):
    """``efs_params``: the values of the reference Properties the step reads (Properties.h:141-162)."""
    _fields_ = [
        ("dt", ctypes.c_float),
        ("gravity_force", ctypes.c_float),
        ("gravity_enabled", ctypes.c_int),
        ("vel_decay", ctypes.c_float),
        ("lambda_minus", ctypes.c_float),
        ("lambda_plus", ctypes.c_float),
        ("eta", ctypes.c_float),
        ("liquid_threshold", ctypes.c_float),
        ("rho_d", ctypes.c_float),
        ("solver", ctypes.c_int),
        ("max_steps", ctypes.c_int),
        ("solver_threshold", ctypes.c_float),
        ("tol_rel", ctypes.c_float),
        ("disable_mask", ctypes.c_uint),
        ("re_calc_div", ctypes.c_int),
        ("sharpen_mode", ctypes.c_int),
        ("cg_variant", ctypes.c_int),
        ("fcg_levels", ctypes.c_int),
        ("fcg_bottom", ctypes.c_int),
        ("reserved", ctypes.c_int * 3),
    ]

    def as_dict(self):
        return {name: getattr(self, name) for name, _ in self._fields_ if name != "reserved"}

    def copy(self):
        c = EfsParams()
        ctypes.memmove(ctypes.byref(c), ctypes.byref(self), ctypes.sizeof(EfsParams))
        return c


class EfsStats(ctypes.Structure):
    """``efs_stats``: SIMULATION_FRAMES / SOLVE_STEPS / PAUSED and solve diagnostics."""
    _fields_ = [
        ("frames", ctypes.c_int64),
        ("solve_steps", ctypes.c_int),
        ("converged", ctypes.c_int),
        ("paused", ctypes.c_int),
        ("device_error", ctypes.c_int),
        ("rr", ctypes.c_double),
        ("bb", ctypes.c_double),
        ("threshold", ctypes.c_double),
        ("active_cells", ctypes.c_int64),
        ("total_solve_steps", ctypes.c_int64),
        ("solves", ctypes.c_int64),
        ("precond_steps", ctypes.c_int64),
    ]

    def as_dict(self):
        return {name: getattr(self, name) for name, _ in self._fields_}


class EfsBatchTuning(ctypes.Structure):
    """``efs_batch_tuning``: launch configuration of a batch of 2D scenes."""
    _fields_ = [
        ("tile_x", ctypes.c_int),
        ("tile_y", ctypes.c_int),
        ("blocks_per_sm", ctypes.c_int),
        ("solver_threads", ctypes.c_int),
        ("solver_cluster", ctypes.c_int),
        ("ms_per_step", ctypes.c_float),
    ]

    def as_dict(self):
        return {name: getattr(self, name) for name, _ in self._fields_}


class EfsQueryMetrics(ctypes.Structure):
    """``efs_query_metrics``: QueryNode's Metrics (include/simulation/scene/nodes/QueryNode.h:10-17) plus the
    number of cells that counted."""
    _fields_ = [
        ("max_position", ctypes.c_float * 3),
        ("min_position", ctypes.c_float * 3),
        ("avg_position", ctypes.c_float * 3),
        ("velocity", ctypes.c_float * 3),
        ("pressure", ctypes.c_float),
        ("pad", ctypes.c_int),
        ("count", ctypes.c_longlong),
    ]

    def as_dict(self):
        return {"max_position": list(self.max_position), "min_position": list(self.min_position),
                "avg_position": list(self.avg_position), "velocity": list(self.velocity),
                "pressure": self.pressure, "count": self.count}


def _f32(x):
    return ctypes.c_float(x).value


def params_default():
    """Reference Properties defaults (Properties.h:141-162): gravity 10 cells/s^2 at cell size 1."""
    p = EfsParams()
    p.dt = 0.0167
    p.gravity_force = 10.0
    p.gravity_enabled = 1
    p.vel_decay = 0.8
    p.lambda_minus = 0.5
    p.lambda_plus = 0.1
    p.eta = 1.0
    p.liquid_threshold = 0.5
    p.rho_d = 3.0
    p.solver = SOLVER_CG
    p.max_steps = 2000
    p.solver_threshold = 1e-5
    p.tol_rel = 0.0
    p.disable_mask = 0
    p.re_calc_div = 0
    p.sharpen_mode = 0
    p.cg_variant = CG_MIXED_RECURRENCE
    p.fcg_levels = -1
    p.fcg_bottom = FCG_BOTTOM_UNET
    return p


def params_dam(cell_size, dt, solver=SOLVER_CG, tol_rel=1e-6):
    """The reference dam-break constants (assets/scenes/Dam128.json "properties"): lambda- 50, lambda+ 10,
    eta 100, D 32, velocity decay disabled, gravity 9.81 / cell size (float division, Application.cpp:89)."""
    p = params_default()
    p.dt = dt
    p.gravity_force = _f32(_f32(9.81) / _f32(cell_size))
    p.lambda_minus = 50.0
    p.lambda_plus = 10.0
    p.eta = 100.0
    p.rho_d = 32.0
    p.solver = solver
    p.tol_rel = tol_rel
    p.disable_mask = 1 << STAGE_VEL_DECAY
    return p
