"""FP64 pressure solves on the GPU and the precision study of the step.

- EFS_CG_FP64 (the study solver) against the oracle's FP64 CG of the same system: both solved to a relative
  residual of 1e-12, their pressures agree to relative L2 1e-8 on the matrix rows (the remaining difference
  is the conditioning times the tolerance);
- the mixed variants' FP64 pressure (efs_download_pressure_fp64) is the FP32 field before rounding;
- the precision study on small grids: every step converges, the FP32 pressure and the projected velocity
  are within relative L2 1e-5 of the FP64 solve of the same right-hand side, and liquid mass stays within
  1e-5 of the first step.
"""
import numpy as np
import pytest

from eulerianfluidsimulation_gb300 import abi
from tests.helpers import rel_l2
from tests.test_gpu_parity import GPU_MODE, gpu_sim, make_params, warm_state

pytestmark = pytest.mark.gpu

gb = pytest.importorskip("eulerianfluidsimulation_gb300")
from oracle import oracle  # noqa: E402


def _system(dim, n, prm):
    state = warm_state(dim, n, prm, 2)
    o = oracle.Oracle(dim, n, n, n, prm, mode=GPU_MODE)
    o.set_fields(state)
    o.stage(abi.STAGE_PROJECT)
    div = o.field(abi.FIELD_DIVERGENCE)
    rows = (state[abi.FIELD_RHO] > 0.5) & (state[abi.FIELD_BOUNDARY] == 0.0)   # the CG matrix's row test
    return state, o, div, rows


@pytest.mark.parametrize("dim,n", [(3, 32), (2, 64)])
def test_fp64_study_solver_matches_oracle_fp64(dim, n):
    prm = make_params(dim, n, variant=abi.CG_FP64, tol=1e-12)
    prm.max_steps = 100000
    state, o, div, rows = _system(dim, n, prm)
    pstar, _ = o.solve_fp64(1e-12)
    with gpu_sim(dim, n, prm) as s:
        s.set_fields(state)
        s.set_field(abi.FIELD_DIVERGENCE, div)
        st = s.solve()
        p64 = s.pressure_fp64()
        p32 = s.pressure()
    assert st.converged and st.rr < st.threshold
    assert np.sqrt(st.rr / st.bb) < 1e-12
    assert rel_l2(p64[rows], pstar[rows]) < 1e-8
    assert np.array_equal(p32[rows], p64[rows].astype(np.float32))


@pytest.mark.parametrize("variant", [abi.CG_MIXED, abi.CG_MIXED_RECURRENCE])
def test_mixed_fp64_pressure_is_the_unrounded_field(variant):
    dim, n = 3, 32
    prm = make_params(dim, n, variant=variant)
    state, o, div, rows = _system(dim, n, prm)
    pstar, _ = o.solve_fp64(1e-13)
    with gpu_sim(dim, n, prm) as s:
        s.set_fields(state)
        s.set_field(abi.FIELD_DIVERGENCE, div)
        s.solve()
        p64 = s.pressure_fp64()
        p32 = s.pressure()
    assert np.array_equal(p32[rows], p64[rows].astype(np.float32))
    assert rel_l2(p64[rows], pstar[rows]) < 1e-5


def test_fp64_pressure_refused_without_an_fp64_accumulator():
    prm = make_params(3, 16, variant=abi.CG_REFERENCE)
    with gpu_sim(3, 16, prm) as s:
        with pytest.raises(gb.EfsError):
            s.pressure_fp64()


@pytest.mark.parametrize("dim,n,steps", [(3, 32, 6), (2, 64, 6)])
def test_precision_study_small(dim, n, steps):
    from eulerianfluidsimulation_gb300.precision import precision_study
    rep = precision_study(dim, n, steps, spheres=8, seed=1, dt=0.004 if dim == 3 else 0.005)
    m = rep["max"]
    assert m["all_converged"]
    assert m["relres_b"] < 1e-11
    assert m["relres_a"] < 1e-6
    assert m["p_rel"] < 1e-5 and m["p64_rel"] < 1e-5
    assert m["vel_rel"] < 1e-5
    assert m["mass_rel_max_abs"] < 1e-5
