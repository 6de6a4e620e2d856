"""Solve timing: the event pool of efs_solve_timing_arm can be re-armed (larger, smaller, or 0) between replayed
steps, and the counts and times it reports follow the latest arming."""
import numpy as np
import pytest

from eulerianfluidsimulation_gb300 import abi

pytestmark = pytest.mark.gpu

gb = pytest.importorskip("eulerianfluidsimulation_gb300")


def test_rearming_the_solve_timing_pool():
    n = 32
    b, r = gb.scene_dam3d(n, n, n, 2, 2, 1)
    with gb.GB300Simulator3D(n, n, n, abi.params_dam(1.0 / n, 0.004)) as s:
        s.set_field(abi.FIELD_BOUNDARY, b)
        s.set_field(abi.FIELD_RHO, r)
        for capacity, steps in ((2, 1), (1, 3), (3, 2), (0, 1), (2, 2)):
            s.solve_timing_arm(capacity)
            s.update(steps)
            s.synchronize()
            launches, ms, _, _ = s.solve_timing_read()
            assert launches == min(capacity, steps), (capacity, steps, launches)
            assert (ms > 0) == (launches > 0) and np.isfinite(ms)
        assert s.stats().frames == 9 and s.stats().converged
