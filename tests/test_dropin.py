"""The C++ drop-in backend's update() (eulerianfluidsimulation_gb300/host/GB300Simulator.cpp) against the
reference's CPUSimulator3D::update() on the same scene.

The adapter compiles against the reference's headers, which exist only where the reference tree does; these
tests repeat its calls through the C ABI, call for call: efs_create with the Properties' parameters, then per
frame efs_set_params (syncParams), efs_step_host with the grid's host storage as both inputs and outputs
(vel, rho, gamma in place; boundary and forces in; beta, divergence, pressure out) and efs_get_stats
(SOLVE_STEPS, PAUSED).  The fixture ref_dropin_dam32.npz is the reference's own run, made by
tests/dropin_driver.cpp through the ISimulator3D interface with the application's Properties, and holds the
efs_params the adapter derived from those Properties (tests/test_abi.py checks them)."""
import os

import numpy as np
import pytest

from eulerianfluidsimulation_gb300 import abi
from tests.helpers import GOLDEN, rel_l2

pytestmark = pytest.mark.gpu

gb = pytest.importorskip("eulerianfluidsimulation_gb300")
torch = pytest.importorskip("torch")


def _fixture():
    z = np.load(os.path.join(GOLDEN, "ref_dropin_dam32.npz"))
    n, frames, smin, smax, seed = [int(v) for v in z["meta"]]
    prm = abi.EfsParams.from_buffer_copy(z["params"].tobytes())
    fields = {f: z[f"field_{f}"] for f in range(abi.FIELD_COUNT) if f"field_{f}" in z}
    return n, frames, (smin, smax, seed), prm, z["steps"], z["paused"], fields


def _host(n, scene, pinned):
    """The adapter's grid storage after the application wrote the scene (GB300Grid3D's construction state:
    zero velocity and forces, gamma 1; boundary and rho from the scene)."""
    def arr(shape):
        if pinned:
            return torch.zeros(shape, dtype=torch.float32, pin_memory=True).numpy()
        return np.zeros(shape, np.float32)
    b, r = gb.scene_dam3d(n, n, n, *scene)
    h = {k: arr((n, n, n)) for k in ("rho", "gamma", "beta", "divergence", "pressure", "boundary")}
    h["vel"], h["forces"] = arr((n, n, n, 3)), arr((n, n, n, 3))
    h["gamma"][...] = 1.0
    h["boundary"][...] = b
    h["rho"][...] = r
    return h


def _run_adapter_sequence(n, frames, scene, prm, pinned):
    h = _host(n, scene, pinned)
    steps, paused = [], []
    with gb.GB300Simulator3D(n, n, n, prm) as s:
        for _ in range(frames):
            s.set_params(prm)
            s.step_host(vel=h["vel"], rho=h["rho"], gamma=h["gamma"], boundary=h["boundary"], forces=h["forces"],
                        vel_out=h["vel"], rho_out=h["rho"], gamma_out=h["gamma"], beta_out=h["beta"],
                        divergence_out=h["divergence"], pressure_out=h["pressure"])
            st = s.stats()
            steps.append(st.solve_steps)
            paused.append(int(st.paused))
    got = {abi.FIELD_VEL: h["vel"], abi.FIELD_RHO: h["rho"], abi.FIELD_GAMMA: h["gamma"], abi.FIELD_BETA: h["beta"],
           abi.FIELD_DIVERGENCE: h["divergence"], abi.FIELD_PRESSURE: h["pressure"]}
    return got, np.array(steps), np.array(paused)


# Relative L2 after the fixture's 4 frames.  The CG stops at the reference's absolute threshold (r.r < 1e-5), so
# two correct solves whose dot products round differently stop at different points, and the frames carry that on.
# The oracle with the reference's summation order lands within 1.2e-6 of the fixture; the oracle with FP64 dot
# products (another valid order) at vel 4.4e-6, beta 6.5e-5, pressure 2.0e-5, divergence 8.3e-5; the GPU's tree
# ordered float dot products at vel 1.5e-5, rho 3.8e-6, gamma 1.8e-6, beta 9.7e-5, pressure 4.6e-5, divergence
# 1.5e-4.  The bounds are about 3x the larger of the two spreads.
TOL = {abi.FIELD_VEL: 5e-5, abi.FIELD_RHO: 2e-5, abi.FIELD_GAMMA: 1e-5, abi.FIELD_BETA: 3e-4, abi.FIELD_PRESSURE: 1.5e-4,
       abi.FIELD_DIVERGENCE: 5e-4}


@pytest.mark.parametrize("pinned", [False, True], ids=["pageable", "page-locked"])
def test_adapter_update_matches_reference_cpusimulator(pinned):
    """Pageable storage (the reference's std::vector fields) takes efs_step_host's upload / step / download
    branch; page-locked storage the overlapped one.  Both, with the outputs aliasing the inputs as the adapter
    passes them, match the reference's frames: fields within TOL, SOLVE_STEPS within one iteration per frame,
    PAUSED identical."""
    n, frames, scene, prm, ref_steps, ref_paused, want = _fixture()
    got, steps, paused = _run_adapter_sequence(n, frames, scene, prm, pinned)
    print(f"{'page-locked' if pinned else 'pageable'}: steps {steps.tolist()} (reference {ref_steps.tolist()}); " +
          ", ".join(f"{abi.FIELD_NAMES[f]} {rel_l2(got[f], want[f]):.2e}" for f in TOL))
    assert np.array_equal(paused, ref_paused)
    assert np.all(np.abs(steps - ref_steps) <= 1), (steps, ref_steps)
    for f, tol in TOL.items():
        assert np.all(np.isfinite(got[f])), abi.FIELD_NAMES[f]
        assert rel_l2(got[f], want[f]) <= tol, (abi.FIELD_NAMES[f], rel_l2(got[f], want[f]))
