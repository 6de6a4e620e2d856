"""CPU oracle of the U-Net preconditioner (test infrastructure only): forward pass, training loss and the
gradient of every parameter, in float64 numpy.

It restates the network and the loss that ``efs_unet.cu`` computes (three levels, 16/32/64 channels, 3x3x3
zero-padded convolutions, 2x2x2 mean pooling, nearest up-sampling, additive skips; loss
sum_rows (y - p/rms(p))^2 / rows).  With ``bf16=True`` every tensor the GPU stores in BF16 is rounded to
BF16 (round to nearest even) at the same point, so the remaining GPU/oracle difference is the FP32 order
of the tensor-core and atomic sums.  With ``bf16=False`` it is the exact float64 function, whose gradient
``tests/test_unet_oracle.py`` checks against finite differences.

Parameter layout (flat float32, as efs_unet_get_weights): per layer, weights [27][cin][cout] (tap =
(dz+1)*9 + (dy+1)*3 + (dx+1)) then bias [cout].
"""
import numpy as np

LAYERS = [(16, 16, 0), (16, 32, 1), (32, 64, 2), (64, 32, 1), (32, 16, 0), (16, 16, 0)]
TAPS = [(t // 9 - 1, (t // 3) % 3 - 1, t % 3 - 1) for t in range(27)]


def param_count():
    return sum(27 * ci * co + co for ci, co, _ in LAYERS)


def unpack(flat):
    out, off = [], 0
    for ci, co, _ in LAYERS:
        w = np.asarray(flat[off:off + 27 * ci * co], np.float64).reshape(27, ci, co)
        off += 27 * ci * co
        b = np.asarray(flat[off:off + co], np.float64)
        off += co
        out.append((w, b))
    return out


def pack(grads):
    return np.concatenate([np.concatenate([w.ravel(), b.ravel()]) for w, b in grads])


def to_bf16(x):
    """Round to BF16 (nearest even), returned as float64."""
    a = np.ascontiguousarray(np.asarray(x, np.float32))
    u = a.view(np.uint32).astype(np.uint64)
    u = ((u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000).astype(np.uint32)
    return u.view(np.float32).astype(np.float64)


def _shift(x, d):
    """y[z, y, x] = x[z + dz, y + dy, x + dx], zero outside."""
    dz, dy, dx = d
    D, H, W = x.shape[:3]
    y = np.zeros_like(x)
    y[max(0, -dz):min(D, D - dz), max(0, -dy):min(H, H - dy), max(0, -dx):min(W, W - dx)] = \
        x[max(0, dz):min(D, D + dz), max(0, dy):min(H, H + dy), max(0, dx):min(W, W + dx)]
    return y


def conv(x, w, b=None):
    out = sum(_shift(x, TAPS[t]) @ w[t] for t in range(27))
    return out + b if b is not None else out


def conv_dgrad(g, w):
    return sum(_shift(g, tuple(-k for k in TAPS[t])) @ w[t].T for t in range(27))


def conv_wgrad(x, g):
    C, N = x.shape[-1], g.shape[-1]
    return np.stack([_shift(x, TAPS[t]).reshape(-1, C).T @ g.reshape(-1, N) for t in range(27)])


def _children(shape):
    D, H, W = shape[:3]
    return ((D + 1) // 2, (H + 1) // 2, (W + 1) // 2)


def pool(x):
    Dp, Hp, Wp = _children(x.shape)
    s = np.zeros((Dp, Hp, Wp, x.shape[-1]))
    n = np.zeros((Dp, Hp, Wp, 1))
    for dz in (0, 1):
        for dy in (0, 1):
            for dx in (0, 1):
                sub = x[dz::2, dy::2, dx::2]
                s[:sub.shape[0], :sub.shape[1], :sub.shape[2]] += sub
                n[:sub.shape[0], :sub.shape[1], :sub.shape[2]] += 1
    return s / n, n


def up(x, shape):
    y = x.repeat(2, 0).repeat(2, 1).repeat(2, 2)
    return y[:shape[0], :shape[1], :shape[2]]


def up_bwd(g, pshape):
    s = np.zeros(tuple(pshape[:3]) + (g.shape[-1],))
    for dz in (0, 1):
        for dy in (0, 1):
            for dx in (0, 1):
                sub = g[dz::2, dy::2, dx::2]
                s[:sub.shape[0], :sub.shape[1], :sub.shape[2]] += sub
    return s


def pool_bwd(gp, cnt, shape):
    return up(gp / cnt, shape)


def forward(flat, r, rows, bf16=True):
    """r: float32 field [D, H, W]; rows: bool mask of matrix rows.  Returns (y float64 [D, H, W], cache)."""
    R = to_bf16 if bf16 else (lambda a: np.asarray(a, np.float64))
    P = unpack(flat)
    Wq = [(R(w), b) for w, b in P]
    r64 = np.asarray(r, np.float64)
    s = np.sum(r64[rows] ** 2)
    cnt = np.count_nonzero(rows)
    inv = 1.0 / np.sqrt(s / cnt) if s > 0 and cnt > 0 else 1.0
    x0 = np.zeros(r.shape + (16,))
    x0[..., 0] = np.where(rows, R(np.float32(r64 * inv)) if bf16 else r64 * inv, 0.0)
    x0[..., 1] = rows.astype(np.float64)

    def layer(k, x, relu, skip=None):
        t = conv(x, Wq[k][0], Wq[k][1])
        pre = R(t)
        if relu:
            t = np.maximum(t, 0.0)
        if skip is not None:
            t = t + skip
        return R(t), pre, t

    e0, a0, _ = layer(0, x0, True)
    p0, n0 = pool(e0)
    p0 = R(p0)
    e1, a1, _ = layer(1, p0, True)
    p1, n1 = pool(e1)
    p1 = R(p1)
    e2, a2, _ = layer(2, p1, True)
    u2 = up(e2, e1.shape)
    d1, a3, _ = layer(3, u2, True, e1)
    u1 = up(d1, e0.shape)
    d0, a4, _ = layer(4, u1, True, e0)
    _, _, y32 = layer(5, d0, False)
    cache = dict(Wq=Wq, x0=x0, a0=a0, e0=e0, p0=p0, n0=n0, a1=a1, e1=e1, p1=p1, n1=n1, a2=a2, e2=e2, u2=u2,
                 a3=a3, d1=d1, u1=u1, a4=a4, d0=d0, y32=y32, R=R)
    return y32[..., 0], cache


def matrix(rho, boundary):
    """The pressure matrix of the CG solvers as a function z -> L z (rows: rho > 0.5 and not solid; a
    neighbour counts when it is interior and not solid, and is summed when it is liquid; L z = sum - count z),
    restated from CGSolver.cpp:467-497 as the library builds it (rowinfo of k_solver_prep)."""
    rho = np.asarray(rho)
    solid = np.asarray(boundary) != 0.0
    rows = (rho > 0.5) & ~solid
    D, H, W = rho.shape
    zz, yy, xx = np.meshgrid(np.arange(D), np.arange(H), np.arange(W), indexing="ij")
    terms = []
    cnt = np.zeros(rho.shape)
    for dz, dy, dx in ((0, 0, -1), (0, 0, 1), (0, -1, 0), (0, 1, 0), (-1, 0, 0), (1, 0, 0)):
        nz, ny, nx = zz + dz, yy + dy, xx + dx
        inside = (nx > 0) & (nx < W - 1) & (ny > 0) & (ny < H - 1) & (nz > 0) & (nz < D - 1)
        nzc, nyc, nxc = np.clip(nz, 0, D - 1), np.clip(ny, 0, H - 1), np.clip(nx, 0, W - 1)
        ok = inside & ~solid[nzc, nyc, nxc]
        cnt += ok
        summed = ok & (rho[nzc, nyc, nxc] > 0.5)
        terms.append((summed, (nzc, nyc, nxc)))

    def apply(z):
        z = np.asarray(z, np.float64)
        out = -cnt * z
        for summed, idx in terms:
            out = out + np.where(summed, z[idx], 0.0)
        return np.where(rows, out, 0.0)
    return apply, rows


def loss_grad(flat, b, p, rows, bf16=True, kind=0, apply_L=None):
    """Loss of efs_unet_loss_grad (kind 0: normalised pressure MSE; kind 1: energy-norm alignment, which
    needs apply_L = matrix(rho, boundary)[0]) and the gradient of every parameter (flat, float64)."""
    y, c = forward(flat, b, rows, bf16)
    R, Wq = c["R"], c["Wq"]
    p64 = np.asarray(p, np.float64)
    cnt = np.count_nonzero(rows)
    g5 = np.zeros(y.shape + (16,))
    if kind == 0:
        sp = np.sum(p64[rows] ** 2)
        invp = 1.0 / np.sqrt(sp / cnt) if sp > 0 else 1.0
        d = np.where(rows, y - p64 * invp, 0.0)
        loss = np.sum(d[rows] ** 2) / cnt
        g = 2.0 * d / cnt
    else:
        r64 = np.where(rows, np.asarray(b, np.float64), 0.0)
        z = np.where(rows, y, 0.0)
        q = apply_L(z)
        a, cz, k = np.sum(z * r64), np.sum(z * q), np.sum(np.where(rows, p64, 0.0) * r64)
        loss = 1.0 - a * a / (cz * k)
        g = -2.0 * a / (cz * k) * r64 + 2.0 * a * a / (cz * cz * k) * q
    g5[..., 0] = np.where(rows, R(np.float32(g)) if bf16 else g, 0.0)
    grads = [None] * 6
    grads[5] = (conv_wgrad(c["d0"], g5), g5.sum(axis=(0, 1, 2)))
    gd0 = R(conv_dgrad(g5, Wq[5][0]))
    ga4 = np.where(c["a4"] > 0, gd0, 0.0)
    grads[4] = (conv_wgrad(c["u1"], ga4), ga4.sum(axis=(0, 1, 2)))
    gu1 = R(conv_dgrad(ga4, Wq[4][0]))
    gd1 = R(up_bwd(gu1, c["d1"].shape))
    ga3 = np.where(c["a3"] > 0, gd1, 0.0)
    grads[3] = (conv_wgrad(c["u2"], ga3), ga3.sum(axis=(0, 1, 2)))
    gu2 = R(conv_dgrad(ga3, Wq[3][0]))
    ge2 = R(up_bwd(gu2, c["e2"].shape))
    ga2 = np.where(c["a2"] > 0, ge2, 0.0)
    grads[2] = (conv_wgrad(c["p1"], ga2), ga2.sum(axis=(0, 1, 2)))
    gp1 = R(conv_dgrad(ga2, Wq[2][0]))
    ge1 = R(pool_bwd(gp1, c["n1"], c["e1"].shape) + gd1)
    ga1 = np.where(c["a1"] > 0, ge1, 0.0)
    grads[1] = (conv_wgrad(c["p0"], ga1), ga1.sum(axis=(0, 1, 2)))
    gp0 = R(conv_dgrad(ga1, Wq[1][0]))
    ge0 = R(pool_bwd(gp0, c["n0"], c["e0"].shape) + gd0)
    ga0 = np.where(c["a0"] > 0, ge0, 0.0)
    grads[0] = (conv_wgrad(c["x0"], ga0), ga0.sum(axis=(0, 1, 2)))
    return loss, pack(grads)


def layer_slices():
    """(name, slice) of each layer's weights and bias in the flat parameter vector."""
    out, off = [], 0
    for k, (ci, co, _) in enumerate(LAYERS):
        out.append((f"w{k}", slice(off, off + 27 * ci * co)))
        off += 27 * ci * co
        out.append((f"b{k}", slice(off, off + co)))
        off += co
    return out
