"""QueryNode's metrics (src/simulation/scene/nodes/QueryNode.cpp:52-81) pinned to the reference's own code.

tests/golden/ref_query.npz holds, for seven boxes on a stepped 32^3 dam break, the output of the reference's
own metric loop: its lines compiled unmodified into the reference build (oracle/Makefile cuts them from
QueryNode.cpp, whose scene-node headers cannot be compiled here).  The boxes cover the whole grid, a box in the
liquid, boxes clipped at the far faces and at negative coordinates, a box without liquid, every cell counted,
and an empty box.

- the C restatement (oracle/scene_oracle.c, the checker of efs_query_box) against the fixture: bit-exact
  (count, positions, averages, velocity and pressure, all summed in float in the reference's order);
- where the reference tree is present, the reference build against the fixture (the fixture is current);
- efs_query_box on the GPU (tests marked gpu): count, minimum and maximum positions exact; the averages of
  position, velocity and pressure within the reference's own float rounding (twice its distance from the
  FP64 average of the same cells) plus 1e-6 relative: the GPU sums exactly or in FP64 in a fixed block order,
  the reference in float, cell by cell.
"""
import numpy as np
import pytest

from eulerianfluidsimulation_gb300 import abi
from oracle import oracle
from tests.helpers import GOLDEN

import os


def _fixture():
    return np.load(os.path.join(GOLDEN, "ref_query.npz"))


def _vec(m, n):
    return np.concatenate([m["max_position"], m["min_position"], m["avg_position"], m["velocity"],
                           [m["pressure"], n]]).astype(np.float32)


def test_restatement_matches_reference_loop():
    z = _fixture()
    for q, want in zip(z["queries"], z["results"]):
        m, n = oracle.query_box(z["rho"], z["vel"], z["pressure"], q[:3], q[3:6], bool(q[6]))
        assert np.array_equal(_vec(m, n), want.astype(np.float32)), (q, _vec(m, n), want)


@pytest.mark.skipif(not oracle.reference_available(), reason="reference build not present")
def test_reference_build_reproduces_fixture():
    z = _fixture()
    n = 32
    prm = abi.params_dam(1.0 / n, 0.004, abi.SOLVER_CG, 1e-6)
    ref = oracle.RefOracle(3, n, n, n, prm)
    ref.set_field(abi.FIELD_RHO, z["rho"])
    ref.set_field(abi.FIELD_VEL, z["vel"])
    ref.set_field(abi.FIELD_PRESSURE, z["pressure"])
    for q, want in zip(z["queries"], z["results"]):
        m, cnt = ref.query_box(q[:3], q[3:6], bool(q[6]))
        assert np.array_equal(_vec(m, cnt), want.astype(np.float32)), q


@pytest.mark.gpu
def test_efs_query_box_matches_reference_loop():
    gb = pytest.importorskip("eulerianfluidsimulation_gb300")
    z = _fixture()
    n = 32
    with gb.GB300Simulator3D(n, n, n, abi.params_dam(1.0 / n, 0.004)) as s:
        s.set_field(abi.FIELD_RHO, z["rho"])
        s.set_field(abi.FIELD_VEL, z["vel"])
        s.set_field(abi.FIELD_PRESSURE, z["pressure"])
        for q, want in zip(z["queries"], z["results"]):
            m = s.query_box(q[:3], q[3:6], bool(q[6]))
            assert m.count == int(want[13]), (q, m.count, want[13])
            assert list(m.max_position) == list(want[0:3]) and list(m.min_position) == list(want[3:6]), q
            got = np.array(list(m.avg_position) + list(m.velocity) + [m.pressure], np.float64)
            ref = want[6:13]
            exact = _fp64_means(z, q)
            tol = 2 * np.abs(ref - exact) + 1e-6 * np.maximum(np.abs(exact), 1.0)
            assert np.all(np.abs(got - ref) <= tol), (q, got, ref, exact)


def _fp64_means(z, q):
    """The box's averages of position, velocity and pressure in FP64 (the loop's cells, QueryNode.cpp:58-70)."""
    rho, vel, p = z["rho"], z["vel"].astype(np.float64), z["pressure"].astype(np.float64)
    D, H, W = rho.shape
    pos, scl, only = q[:3], q[3:6], bool(q[6])
    lo = [max(0, int(pos[k])) for k in range(3)]
    hi = [min(n - 1, int(pos[k] + scl[k])) for k, n in enumerate((W, H, D))]
    if any(hi[k] <= lo[k] for k in range(3)):
        return np.zeros(7)
    zz, yy, xx = np.meshgrid(np.arange(lo[2], hi[2]), np.arange(lo[1], hi[1]), np.arange(lo[0], hi[0]), indexing="ij")
    sel = np.ones(zz.shape, bool) if not only else rho[zz, yy, xx] >= 0.5
    if not sel.any():
        return np.zeros(7)
    x, y, zc = xx[sel], yy[sel], zz[sel]
    return np.concatenate([[x.mean(), y.mean(), zc.mean()], vel[zc, y, x].mean(axis=0), [p[zc, y, x].mean()]])
