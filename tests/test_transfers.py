"""Host transfers: page-locked host buffers are read and written by the GPU directly (the split, interleave,
boundary and copy kernels address them over the host link), pageable ones through the staging buffer and
the copy engine.  Both give the same fields, bit for bit, in 2D and 3D, for single fields and the
batched upload/download calls, and a step between them gives the same result."""
import numpy as np
import pytest

from eulerianfluidsimulation_gb300 import abi
from eulerianfluidsimulation_gb300._lib import check, fptr, lib

pytestmark = pytest.mark.gpu

gb = pytest.importorskip("eulerianfluidsimulation_gb300")
torch = pytest.importorskip("torch")


def _pinned(shape):
    return torch.empty(shape, dtype=torch.float32, pin_memory=True).numpy()


@pytest.mark.parametrize("dim", [2, 3])
def test_pinned_and_pageable_transfers_agree(dim):
    n = 40
    shape = (n, n) if dim == 2 else (n, n, n)
    if dim == 3:
        b, r = gb.scene_dam3d(n, n, n, 2, 2, 3)
        mk = lambda: gb.GB300Simulator3D(n, n, n, abi.params_dam(1.0 / n, 0.004, abi.SOLVER_CG, 1e-6))
    else:
        b, r = gb.scene_dam2d(n, n)
        mk = lambda: gb.GB300Simulator2D(n, n, abi.params_dam(1.0 / n, 0.005, abi.SOLVER_CG, 1e-6))
    rng = np.random.default_rng(dim)
    vel = rng.normal(size=shape + (dim,)).astype(np.float32)
    frc = rng.normal(size=shape + (dim,)).astype(np.float32)
    gam = (1.0 + 0.1 * rng.random(shape)).astype(np.float32)
    with mk() as A, mk() as B:
        # A: pageable numpy arrays; B: page-locked copies of the same values
        A.upload_fields(vel=vel, rho=r, gamma=gam, boundary=b, forces=frc)
        pv, pr, pg, pb, pf = _pinned(vel.shape), _pinned(shape), _pinned(shape), _pinned(shape), _pinned(frc.shape)
        pv[...], pr[...], pg[...], pb[...], pf[...] = vel, r, gam, b, frc
        B.upload_fields(vel=pv, rho=pr, gamma=pg, boundary=pb, forces=pf)
        for f in (abi.FIELD_VEL, abi.FIELD_RHO, abi.FIELD_GAMMA, abi.FIELD_BOUNDARY, abi.FIELD_FORCES):
            assert np.array_equal(A.field(f), B.field(f)), abi.FIELD_NAMES[f]
        A.update(1)
        B.update(1)
        # the step sums with float atomics: A and B agree to rounding, and A's own fields read back through
        # page-locked buffers equal A's fields read back through pageable ones bit for bit
        for f in (abi.FIELD_VEL, abi.FIELD_RHO, abi.FIELD_PRESSURE):
            a, bb = A.field(f).astype(np.float64), B.field(f).astype(np.float64)
            assert np.linalg.norm(a - bb) <= 1e-5 * np.linalg.norm(a), abi.FIELD_NAMES[f]
        outs = {}
        for key, s in (("vel", vel.shape), ("rho", shape), ("gamma", shape), ("beta", shape), ("divergence", shape),
                       ("pressure", shape)):
            outs[key] = _pinned(s)
        A.download_fields(vel=outs["vel"], rho=outs["rho"], gamma=outs["gamma"], beta=outs["beta"],
                          divergence=outs["divergence"], pressure=outs["pressure"])
        for key, f in (("vel", abi.FIELD_VEL), ("rho", abi.FIELD_RHO), ("gamma", abi.FIELD_GAMMA),
                       ("beta", abi.FIELD_BETA), ("divergence", abi.FIELD_DIVERGENCE), ("pressure", abi.FIELD_PRESSURE)):
            assert np.array_equal(outs[key], A.field(f)), key
        one = _pinned(shape)
        check(lib().efs_download_field(A._h, abi.FIELD_BOUNDARY, fptr(one)), A._h)
        assert np.array_equal(one, A.field(abi.FIELD_BOUNDARY))


def test_step_host_overlapped_equals_the_separate_calls():
    """efs_step_host with page-locked buffers (transfers overlapping the step on a second stream) writes
    the step's fields: the outputs equal the context's own fields after the call, and the step equals the
    separate upload / step / download calls on a second context to rounding (the step sums with atomics)."""
    n = 48
    b, r = gb.scene_dam3d(n, n, n, 3, 3, 5)
    prm = abi.params_dam(1.0 / n, 0.004, abi.SOLVER_CG, 1e-6)
    shape = (n, n, n)
    rng = np.random.default_rng(9)
    frc = (0.1 * rng.normal(size=shape + (3,))).astype(np.float32)
    with gb.GB300Simulator3D(n, n, n, prm) as A, gb.GB300Simulator3D(n, n, n, prm) as B:
        for S in (A, B):
            S.set_field(abi.FIELD_BOUNDARY, b)
            S.set_field(abi.FIELD_RHO, r)
            S.update(2)                                  # a state with motion; graphs already captured
        st = A.fields()
        h = {k: _pinned(st[f].shape) for k, f in (("vel", abi.FIELD_VEL), ("rho", abi.FIELD_RHO),
                                                  ("gamma", abi.FIELD_GAMMA), ("boundary", abi.FIELD_BOUNDARY))}
        h["vel"][...], h["rho"][...], h["gamma"][...], h["boundary"][...] = (st[abi.FIELD_VEL], st[abi.FIELD_RHO],
                                                                            st[abi.FIELD_GAMMA], st[abi.FIELD_BOUNDARY])
        h["forces"] = _pinned(frc.shape)
        h["forces"][...] = frc
        out = {k: _pinned(s) for k, s in (("vel", shape + (3,)), ("rho", shape), ("gamma", shape), ("beta", shape),
                                          ("div", shape), ("p", shape))}
        for _ in range(2):
            A.step_host(vel=h["vel"], rho=h["rho"], gamma=h["gamma"], boundary=h["boundary"], forces=h["forces"],
                        vel_out=out["vel"], rho_out=out["rho"], gamma_out=out["gamma"], beta_out=out["beta"],
                        divergence_out=out["div"], pressure_out=out["p"])
            for k, f in (("vel", abi.FIELD_VEL), ("rho", abi.FIELD_RHO), ("gamma", abi.FIELD_GAMMA),
                         ("beta", abi.FIELD_BETA), ("div", abi.FIELD_DIVERGENCE), ("p", abi.FIELD_PRESSURE)):
                assert np.array_equal(out[k], A.field(f)), k
            B.upload_fields(vel=h["vel"].copy(), rho=h["rho"].copy(), gamma=h["gamma"].copy(),
                            boundary=h["boundary"].copy(), forces=frc)
            B.update(1)
            for k, f in (("vel", abi.FIELD_VEL), ("rho", abi.FIELD_RHO), ("p", abi.FIELD_PRESSURE)):
                want = B.field(f).astype(np.float64)
                assert np.linalg.norm(out[k] - want) <= 1e-5 * np.linalg.norm(want), k
            # feed the step's output back in, as a host-mirrored simulator does
            for k in ("vel", "rho", "gamma"):
                h[k][...] = out[k]
        assert A.stats().converged
