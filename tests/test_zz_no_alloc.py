"""efs_solve_noalloc: the pressure solve for callers that cannot allocate device memory.

Such callers (a host that owns every device allocation of its plug-ins, a real-time loop that may not
synchronise the device, work recorded into a CUDA graph) pass their own device buffers and the library works
in one fixed file-scope device array.  This test drives the entry point through the C ABI with device buffers
it allocates itself (PyTorch), twice in a row on different right-hand sides, and checks each result against
the existing entry point (efs_solve through a GB300Simulator3D context) on the same inputs, within the
pressure tolerance the other GPU tests use (relative L2 1e-5).  It also checks the solve against the CPU oracle
in 3D and 2D, for CG (both arithmetic variants) and for Jacobi started from a non-zero caller pressure; a
smaller grid right after a larger one (the scratch then holds the larger call's data past the new grid); and
that grids beyond the fixed maximum are refused.  This file is collected last so that a failure here stops a run only after every other
test has run.
"""
import ctypes

import numpy as np
import pytest

from eulerianfluidsimulation_gb300 import abi

pytestmark = pytest.mark.gpu


def _rel(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


def _state(n, seed):
    from oracle import oracle
    prm = abi.params_dam(1.0 / n, 0.004, abi.SOLVER_CG, 1e-6)
    b, r = oracle.scene_dam3d(n, n, n, 6, 6, seed)
    o = oracle.Oracle(3, n, n, n, prm, mode=oracle.SHARPEN_PARALLEL | oracle.DOTS_FP64)
    o.set_field(abi.FIELD_BOUNDARY, b)
    o.set_field(abi.FIELD_RHO, r)
    o.step(2)
    o.stage(abi.STAGE_PROJECT)
    return prm, o.field(abi.FIELD_BOUNDARY), o.field(abi.FIELD_RHO), o.field(abi.FIELD_DIVERGENCE)


def _reference_solve(n, prm, boundary, rho, div):
    import eulerianfluidsimulation_gb300 as gb
    with gb.GB300Simulator3D(n, n, n, prm) as s:
        s.set_field(abi.FIELD_BOUNDARY, boundary)
        s.set_field(abi.FIELD_RHO, rho)
        s.set_field(abi.FIELD_DIVERGENCE, div)
        st = s.solve()
        return s.pressure(), st


def test_noalloc_solve_matches_efs_solve_twice():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from eulerianfluidsimulation_gb300._lib import lib
    L = lib()
    n = 40                                    # 64,000 cells, within EFS_NOALLOC_MAX_CELLS
    for call, seed in enumerate((3, 9)):      # two calls in a row share the fixed scratch
        prm, boundary, rho, div = _state(n, seed)
        if call == 1:
            div = div * 2.0                   # a different right-hand side on the second call
        want, want_st = _reference_solve(n, prm, boundary, rho, div)
        dev = torch.device("cuda:0")
        t_rho = torch.from_numpy(rho.copy()).to(dev)
        t_bnd = torch.from_numpy(boundary.copy()).to(dev)
        t_div = torch.from_numpy(div.copy()).to(dev)
        t_p = torch.full_like(t_div, 123.0)   # whatever the caller left there: CG starts from p = b
        torch.cuda.synchronize()
        st = abi.EfsStats()
        rc = L.efs_solve_noalloc(3, n, n, n, ctypes.byref(prm), t_rho.data_ptr(), t_bnd.data_ptr(), t_div.data_ptr(),
                                 t_p.data_ptr(), None, ctypes.byref(st))
        assert rc == 0, L.efs_noalloc_last_error().decode()
        got = t_p.cpu().numpy()
        assert st.converged and st.solve_steps == want_st.solve_steps
        assert _rel(got, want) <= 1e-5, (call, _rel(got, want))


def _oracle_state(dim, n, solver, variant, seed):
    """A state 2 steps into a seeded dam break, its divergence, and a non-zero start pressure (Jacobi starts
    from the caller's pressure; CG ignores it)."""
    from oracle import oracle
    if dim == 3:
        prm = abi.params_dam(1.0 / n, 0.004, solver, 0.0 if variant == abi.CG_REFERENCE else 1e-6)
        b, r = oracle.scene_dam3d(n, n, n, 6, 6, seed)
    else:
        prm = abi.params_dam(1.0 / n, 0.005, solver, 0.0 if variant == abi.CG_REFERENCE else 1e-6)
        b, r = oracle.scene_dam2d(n, n)
    prm.cg_variant = variant
    if solver == abi.SOLVER_JACOBI:
        prm.max_steps = 200
    o = oracle.Oracle(dim, n, n, n, prm, mode=oracle.SHARPEN_PARALLEL | oracle.DOTS_FP64)
    o.set_field(abi.FIELD_BOUNDARY, b)
    o.set_field(abi.FIELD_RHO, r)
    o.step(2)
    o.stage(abi.STAGE_PROJECT)
    p_in = (o.field(abi.FIELD_PRESSURE) * 0.5).astype(np.float32)
    return prm, o, p_in


def _noalloc(L, torch, dim, n, prm, o, p_in):
    dev = torch.device("cuda:0")
    t = {f: torch.from_numpy(o.field(f).copy()).to(dev) for f in (abi.FIELD_RHO, abi.FIELD_BOUNDARY, abi.FIELD_DIVERGENCE)}
    t_p = torch.from_numpy(p_in.copy()).to(dev)
    torch.cuda.synchronize()
    st = abi.EfsStats()
    rc = L.efs_solve_noalloc(dim, n, n, n if dim == 3 else 1, ctypes.byref(prm), t[abi.FIELD_RHO].data_ptr(),
                             t[abi.FIELD_BOUNDARY].data_ptr(), t[abi.FIELD_DIVERGENCE].data_ptr(), t_p.data_ptr(),
                             None, ctypes.byref(st))
    assert rc == 0, L.efs_noalloc_last_error().decode()
    return t_p.cpu().numpy(), st


def _oracle_solve(o, p_in):
    o.set_field(abi.FIELD_PRESSURE, p_in)
    o.solve()
    return o.field(abi.FIELD_PRESSURE), o.stats()


# (dim, side, solver, variant): 3D and 2D, the recurrence CG (default), the reference-arithmetic CG and Jacobi
CASES = [(3, 40, abi.SOLVER_CG, abi.CG_MIXED_RECURRENCE), (3, 40, abi.SOLVER_CG, abi.CG_REFERENCE),
         (3, 40, abi.SOLVER_JACOBI, abi.CG_MIXED), (2, 96, abi.SOLVER_CG, abi.CG_MIXED_RECURRENCE),
         (2, 96, abi.SOLVER_JACOBI, abi.CG_MIXED), (2, 96, abi.SOLVER_CG, abi.CG_MIXED)]


@pytest.mark.parametrize("dim,n,solver,variant", CASES)
def test_noalloc_matches_oracle(dim, n, solver, variant):
    """The solve against the CPU oracle's solver on the same system: Jacobi (from a non-zero caller pressure)
    bit-exact, CG within relative L2 1e-5 and the same iteration count within 2."""
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from eulerianfluidsimulation_gb300._lib import lib
    L = lib()
    prm, o, p_in = _oracle_state(dim, n, solver, variant, seed=5)
    got, st = _noalloc(L, torch, dim, n, prm, o, p_in)
    want, ost = _oracle_solve(o, p_in)
    if solver == abi.SOLVER_JACOBI:
        assert np.array_equal(got, want), _rel(got, want)
        assert st.solve_steps == prm.max_steps // 2
    else:
        assert st.converged and ost.converged
        assert abs(st.solve_steps - ost.solve_steps) <= 2, (st.solve_steps, ost.solve_steps)
        assert _rel(got, want) <= 1e-5, _rel(got, want)


def test_noalloc_smaller_grid_after_larger():
    """The scratch keeps what the last call left.  A 60^3 call, then a 40^3 call, then a 2D 64^2 call: each
    smaller call finds the larger call's data past its own cells, and must still match the oracle and
    efs_solve."""
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from eulerianfluidsimulation_gb300._lib import lib
    import eulerianfluidsimulation_gb300 as gb
    L = lib()
    for dim, n in ((3, 60), (3, 40), (2, 64)):
        prm, o, p_in = _oracle_state(dim, n, abi.SOLVER_CG, abi.CG_MIXED_RECURRENCE, seed=7)
        got, st = _noalloc(L, torch, dim, n, prm, o, p_in)
        sim = gb.GB300Simulator3D(n, n, n, prm) if dim == 3 else gb.GB300Simulator2D(n, n, prm)
        with sim as s:
            for f in (abi.FIELD_BOUNDARY, abi.FIELD_RHO, abi.FIELD_DIVERGENCE):
                s.set_field(f, o.field(f))
            want_st = s.solve()
            want = s.pressure()
        orc, _ = _oracle_solve(o, p_in)
        assert st.converged and st.solve_steps == want_st.solve_steps, (dim, n, st.solve_steps, want_st.solve_steps)
        assert _rel(got, want) <= 1e-5, (dim, n, _rel(got, want))
        assert _rel(got, orc) <= 1e-5, (dim, n, _rel(got, orc))


def test_noalloc_rejects_grids_beyond_its_scratch():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from eulerianfluidsimulation_gb300._lib import lib
    L = lib()
    prm = abi.params_dam(1.0 / 80, 0.004, abi.SOLVER_CG, 1e-6)
    buf = torch.zeros(8, device="cuda:0")
    p = buf.data_ptr()
    rc = L.efs_solve_noalloc(3, 80, 80, 80, ctypes.byref(prm), p, p, p, p, None, None)   # 512,000 cells
    assert rc == 1
    assert b"at most" in L.efs_noalloc_last_error()
