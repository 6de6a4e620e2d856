"""The U-Net oracle's own gradient (CPU): its exact float64 backward pass against central differences of its
loss along random directions in parameter space, on a tiny grid with odd dimensions (partial pooling
windows).  This pins the oracle that the GPU gradients are checked against."""
import numpy as np
import pytest

from oracle import unet_oracle as U


def test_param_count():
    assert U.param_count() == 152064 + 176


@pytest.mark.parametrize("kind", [0, 1])
def test_oracle_gradient_matches_finite_differences(kind):
    rng = np.random.default_rng(7)
    shape = (5, 6, 7)
    flat = rng.normal(0, 0.15, U.param_count()).astype(np.float64)
    for name, sl in U.layer_slices():
        if name.startswith("b"):
            flat[sl] = rng.normal(0, 0.05, sl.stop - sl.start)
    rho = (rng.random(shape) < 0.8).astype(np.float32)
    bnd = np.zeros(shape, np.float32)
    bnd[0], bnd[-1], bnd[:, 0], bnd[:, -1], bnd[:, :, 0], bnd[:, :, -1] = 1, 1, 1, 1, 1, 1
    apply_L, rows = U.matrix(rho, bnd)
    p = np.where(rows, rng.normal(size=shape), 0.0).astype(np.float32)
    b = apply_L(p).astype(np.float32) if kind == 1 else rng.normal(size=shape).astype(np.float32)
    kw = dict(bf16=False, kind=kind, apply_L=apply_L)
    loss, g = U.loss_grad(flat, b, p, rows, **kw)
    assert np.isfinite(loss) and g.shape == flat.shape
    h = 1e-6
    for _ in range(3):
        v = rng.normal(size=flat.shape)
        v /= np.linalg.norm(v)
        lp, _ = U.loss_grad(flat + h * v, b, p, rows, **kw)
        lm, _ = U.loss_grad(flat - h * v, b, p, rows, **kw)
        fd = (lp - lm) / (2 * h)
        an = float(g @ v)
        assert abs(fd - an) <= 1e-5 * max(abs(fd), abs(an), 1e-6), (fd, an)


def test_bf16_rounding_is_nearest_even():
    x = np.array([1.0, 1.00390625, 1.0078125, 1.01171875, -2.5, 3.0e-39], np.float32)
    got = U.to_bf16(x)
    assert got[0] == 1.0 and got[1] == 1.0          # halfway rounds to even (1.0)
    assert got[2] == 1.0078125                       # representable
    assert got[3] == 1.015625                        # halfway rounds to even (odd lower neighbour)
    assert got[4] == -2.5
