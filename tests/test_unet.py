"""The learned preconditioner on the GPU (through the C ABI), against the CPU oracle of the network.

- forward pass: the GPU output against the oracle with BF16 rounding at the same points, relative L2 1e-2
  on the matrix rows (what remains is the FP32 order of tensor-core sums, which can flip a BF16 rounding);
- gradients: the loss within 1e-3 relative and every layer's weight and bias gradient within 3e-2
  relative L2 of the oracle's;
- training on the device lowers the loss on the samples it was given;
- FCG with the trained network reaches the same stop rule as CG, its pressure within 1e-5 of CG's, in
  fewer iterations than plain CG;
- FCG with the multilevel preconditioner (the network as its coarsest-level solve): the same stop rule and
  pressure bound; with a trained network it takes fewer iterations than the same V-cycle without the network
  (20 Jacobi sweeps at the bottom), which is the network's gain; a network that outputs zeros makes FCG break
  down at once and the plain-CG fallback finishes the solve; steps with FCG replay one captured graph and
  match the CG steps.
"""
import numpy as np
import pytest

from eulerianfluidsimulation_gb300 import abi
from tests.helpers import rel_l2

pytestmark = pytest.mark.gpu

gb = pytest.importorskip("eulerianfluidsimulation_gb300")
from oracle import oracle, unet_oracle as U  # noqa: E402


def _scene(n, seed=3):
    b, r = oracle.scene_dam3d(n, n, n, 4, 4, seed)
    rows = (r > 0.5) & (b == 0.0)
    return b, r, rows


def _ctx(n, seed=11, cap=0, solver=abi.SOLVER_CG):
    prm = abi.params_dam(1.0 / n, 0.004, solver, 1e-6)
    prm.max_steps = 20000
    s = gb.GB300Simulator3D(n, n, n, prm)
    s.unet_init(seed, cap)
    return s


def test_unet_forward_matches_oracle():
    n = 12
    bnd, rho, rows = _scene(n)
    rng = np.random.default_rng(1)
    r = rng.normal(size=(n, n, n)).astype(np.float32)
    with _ctx(n) as s:
        s.set_field(abi.FIELD_BOUNDARY, bnd)
        s.set_field(abi.FIELD_RHO, rho)
        z = s.unet_apply(r)
        w = s.unet_weights()
    y, _ = U.forward(w, r, rows, bf16=True)
    assert np.all(z[~rows] == 0)
    assert rel_l2(z[rows], y[rows]) < 1e-2, rel_l2(z[rows], y[rows])


@pytest.mark.parametrize("kind", [0, 1])
def test_unet_gradients_match_oracle(kind):
    n = 12
    bnd, rho, rows = _scene(n)
    apply_L, rows_l = U.matrix(rho, bnd)
    assert np.array_equal(rows, rows_l)
    rng = np.random.default_rng(2)
    p = np.where(rows, rng.normal(size=(n, n, n)), 0.0).astype(np.float32)
    b = apply_L(p).astype(np.float32) if kind == 1 else rng.normal(size=(n, n, n)).astype(np.float32)
    with _ctx(n, seed=5) as s:
        s.set_field(abi.FIELD_BOUNDARY, bnd)
        s.set_field(abi.FIELD_RHO, rho)
        loss, g = s.unet_loss_grad(b, p, loss_kind=kind)
        w = s.unet_weights()
    lo, go = U.loss_grad(w, b, p, rows, bf16=True, kind=kind, apply_L=apply_L)
    assert abs(loss - lo) <= 1e-3 * lo, (loss, lo)
    for name, sl in U.layer_slices():
        assert rel_l2(g[sl], go[sl]) < 3e-2, (name, rel_l2(g[sl], go[sl]))


def test_unet_halo_tile_path_matches_oracle():
    """Grids at least 96 voxels wide take the halo-tile convolution (TMA input box, one descriptor per tap) for
    32 and 64 input channels: here levels 0 and 1 (widths 200 and 100: a partial second segment, COUT 16/32/64
    in the forward and input-gradient passes).  Their 16-channel convolutions, and level 2 (width 50), take the
    slab kernel on these wide grids."""
    W, H, D = 200, 12, 10
    bnd, rho = oracle.scene_dam3d(W, H, D, 3, 3, 6)
    rows = (rho > 0.5) & (bnd == 0.0)
    apply_L, _ = U.matrix(rho, bnd)
    rng = np.random.default_rng(7)
    r = rng.normal(size=(D, H, W)).astype(np.float32)
    p = np.where(rows, rng.normal(size=(D, H, W)), 0.0).astype(np.float32)
    b = apply_L(p).astype(np.float32)
    prm = abi.params_dam(1.0 / W, 0.004, abi.SOLVER_CG, 1e-6)
    prm.fcg_levels = 0                      # the network on the context's own grid
    with gb.GB300Simulator3D(W, H, D, prm) as s:
        s.unet_init(13, 0)
        s.set_field(abi.FIELD_BOUNDARY, bnd)
        s.set_field(abi.FIELD_RHO, rho)
        z = s.unet_apply(r)
        loss, g = s.unet_loss_grad(b, p, loss_kind=1)
        w = s.unet_weights()
    y, _ = U.forward(w, r, rows, bf16=True)
    assert np.all(z[~rows] == 0)
    assert rel_l2(z[rows], y[rows]) < 1e-2, rel_l2(z[rows], y[rows])
    lo, go = U.loss_grad(w, b, p, rows, bf16=True, kind=1, apply_L=apply_L)
    assert abs(loss - lo) <= 1e-3 * lo, (loss, lo)
    for name, sl in U.layer_slices():
        assert rel_l2(g[sl], go[sl]) < 3e-2, (name, rel_l2(g[sl], go[sl]))


def test_unet_slab_path_matches_oracle():
    """Grids narrower than the halo-tile kernel's take the slab convolution (input brick and weights in shared
    memory, one descriptor per tap): here levels 0 and 1 in whole 8 x 16 slabs (16 x 32 x 6 and 8 x 16 x 3:
    16/32/64 input channels, COUT 16/32/64, the up-sampled inputs read in place, the forward and
    input-gradient passes) and level 2 (4 x 8 x 2) in one partial slab.  The 12^3 tests above run every
    level in partial slabs."""
    W, H, D = 16, 32, 6
    bnd, rho = oracle.scene_dam3d(W, H, D, 2, 2, 8)
    rows = (rho > 0.5) & (bnd == 0.0)
    apply_L, _ = U.matrix(rho, bnd)
    rng = np.random.default_rng(17)
    r = rng.normal(size=(D, H, W)).astype(np.float32)
    p = np.where(rows, rng.normal(size=(D, H, W)), 0.0).astype(np.float32)
    b = apply_L(p).astype(np.float32)
    prm = abi.params_dam(1.0 / W, 0.004, abi.SOLVER_CG, 1e-6)
    prm.fcg_levels = 0                      # the network on the context's own grid
    with gb.GB300Simulator3D(W, H, D, prm) as s:
        s.unet_init(19, 0)
        s.set_field(abi.FIELD_BOUNDARY, bnd)
        s.set_field(abi.FIELD_RHO, rho)
        z = s.unet_apply(r)
        loss, g = s.unet_loss_grad(b, p, loss_kind=1)
        w = s.unet_weights()
    y, _ = U.forward(w, r, rows, bf16=True)
    assert np.all(z[~rows] == 0)
    assert rel_l2(z[rows], y[rows]) < 1e-2, rel_l2(z[rows], y[rows])
    lo, go = U.loss_grad(w, b, p, rows, bf16=True, kind=1, apply_L=apply_L)
    assert abs(loss - lo) <= 1e-3 * lo, (loss, lo)
    for name, sl in U.layer_slices():
        assert rel_l2(g[sl], go[sl]) < 3e-2, (name, rel_l2(g[sl], go[sl]))


def _collect(s, steps):
    for _ in range(steps):
        s.update(1)
        s.unet_add_sample()
    s.synchronize()


def test_training_lowers_the_loss():
    n = 32
    bnd, rho, _ = _scene(n, seed=4)
    with _ctx(n, seed=9, cap=16) as s:
        s.set_field(abi.FIELD_BOUNDARY, bnd)
        s.set_field(abi.FIELD_RHO, rho)
        _collect(s, 16)
        assert s.unet_sample_count() == 16
        first = s.unet_train(1, batch=8, lr=1e-3, synthetic=0.0, seed=1, loss_kind=0)
        last = s.unet_train(150, batch=4, lr=1e-3, synthetic=0.0, seed=2, loss_kind=0)
    assert np.isfinite(last) and last < 0.7 * first, (first, last)


def test_fcg_converges_and_the_trained_network_saves_iterations():
    n = 32
    bnd, rho, rows0 = _scene(n, seed=4)
    with _ctx(n, seed=9, cap=24) as s:
        s.set_field(abi.FIELD_BOUNDARY, bnd)
        s.set_field(abi.FIELD_RHO, rho)
        _collect(s, 24)
        s.unet_train(400, batch=4, lr=1e-3, synthetic=0.5, seed=3)
        s.update(2)                                  # a state the network was not trained on
        state = s.fields()
        cg = s.params
        s.project()
        st_cg = s.stats()
        p_cg = s.pressure()
        fcg = cg.copy()
        fcg.solver = abi.SOLVER_FCG_UNET
        s.set_params(fcg)
        s.set_fields(state)
        s.project()
        st_fcg = s.stats()
        p_fcg = s.pressure()
    rows = (state[abi.FIELD_RHO] > 0.5) & (state[abi.FIELD_BOUNDARY] == 0.0)
    assert st_cg.converged and st_fcg.converged
    assert st_fcg.rr < st_fcg.threshold
    assert rel_l2(p_fcg[rows], p_cg[rows]) < 1e-5
    print(f"\nFCG {st_fcg.solve_steps} iterations ({st_fcg.precond_steps} preconditioned), CG {st_cg.solve_steps}")
    assert st_fcg.solve_steps < st_cg.solve_steps, (st_fcg.solve_steps, st_fcg.precond_steps, st_cg.solve_steps)


def _dam_ctx(n, spheres=4, seed=4, levels=-1, bottom=abi.FCG_BOTTOM_UNET, solver=abi.SOLVER_CG):
    prm = abi.params_dam(1.0 / n, 0.004, solver, 1e-6)
    prm.max_steps = 20000
    prm.fcg_levels = levels
    prm.fcg_bottom = bottom
    s = gb.GB300Simulator3D(n, n, n, prm)
    b, r = oracle.scene_dam3d(n, n, n, spheres, spheres, seed)
    s.set_field(abi.FIELD_BOUNDARY, b)
    s.set_field(abi.FIELD_RHO, r)
    return s


def _solve_with(s, state, **kw):
    p = s.params.copy()
    for k, v in kw.items():
        setattr(p, k, v)
    s.set_params(p)
    s.set_fields(state)
    s.project()
    return s.stats(), s.pressure()


def test_multilevel_fcg_without_network_matches_cg():
    """64^3 (one aggregation level, 32^3 bottom solved by Jacobi sweeps): FCG meets CG's stop rule, its
    pressure within 1e-5 of CG's on the rows, in a fraction of CG's iterations."""
    n = 64
    with _dam_ctx(n, bottom=abi.FCG_BOTTOM_JACOBI) as s:
        s.update(3)
        state = s.fields()
        st_cg, p_cg = _solve_with(s, state, solver=abi.SOLVER_CG)
        st, p = _solve_with(s, state, solver=abi.SOLVER_FCG_UNET)
    rows = (state[abi.FIELD_RHO] > 0.5) & (state[abi.FIELD_BOUNDARY] == 0.0)
    print(f"\nFCG (V-cycle, Jacobi bottom) {st.solve_steps} iterations, CG {st_cg.solve_steps}")
    assert st.converged and st_cg.converged and st.rr < st.threshold
    assert rel_l2(p[rows], p_cg[rows]) < 1e-5
    assert st.solve_steps * 4 < st_cg.solve_steps


def test_fcg_breakdown_falls_back_to_cg():
    """A network whose output is zero gives z = 0, so d.Ad = 0 in the first iteration: FCG stops there and the
    persistent CG kernel solves the remaining system; the pressure still meets the stop rule."""
    n = 32
    with _dam_ctx(n, levels=0) as s:
        s.update(2)
        state = s.fields()
        st_cg, p_cg = _solve_with(s, state, solver=abi.SOLVER_CG)
        s.unet_init(3, 0)
        s.unet_set_weights(np.zeros(gb.unet_param_count(), np.float32))
        st, p = _solve_with(s, state, solver=abi.SOLVER_FCG_UNET)
    rows = (state[abi.FIELD_RHO] > 0.5) & (state[abi.FIELD_BOUNDARY] == 0.0)
    assert st.converged and st.precond_steps == 1 and st.solve_steps > 1
    assert rel_l2(p[rows], p_cg[rows]) < 1e-5


def test_trained_network_beats_the_v_cycle_without_it():
    """64^3 with the network on the 32^3 bottom grid, trained on samples of another seed's trajectory: on a state
    it was not trained on, FCG takes fewer iterations with the network than with 20 Jacobi sweeps in its place,
    and both meet the stop rule with the CG pressure's accuracy."""
    n = 64
    with _dam_ctx(n, seed=9) as t:
        t.unet_init(5, 24)
        assert t.unet_grid() == (32, 32, 32, 1)
        for _ in range(24):
            t.update(1)
            t.unet_add_sample()
        t.unet_train(600, batch=8, lr=1e-3, synthetic=0.5, seed=3)
        w = t.unet_weights()
    with _dam_ctx(n, seed=4) as s:
        s.update(3)
        state = s.fields()
        st_cg, p_cg = _solve_with(s, state, solver=abi.SOLVER_CG)
        st_j, p_j = _solve_with(s, state, solver=abi.SOLVER_FCG_UNET, fcg_bottom=abi.FCG_BOTTOM_JACOBI)
        s.unet_init(0, 0)
        s.unet_set_weights(w)
        st_n, p_n = _solve_with(s, state, solver=abi.SOLVER_FCG_UNET, fcg_bottom=abi.FCG_BOTTOM_UNET)
    rows = (state[abi.FIELD_RHO] > 0.5) & (state[abi.FIELD_BOUNDARY] == 0.0)
    print(f"\nFCG: network bottom {st_n.solve_steps}, Jacobi bottom {st_j.solve_steps}, plain CG {st_cg.solve_steps}")
    assert st_n.converged and st_j.converged
    assert rel_l2(p_n[rows], p_cg[rows]) < 1e-5 and rel_l2(p_j[rows], p_cg[rows]) < 1e-5
    assert st_n.solve_steps < st_j.solve_steps < st_cg.solve_steps


def test_fcg_steps_replay_one_graph_and_match_cg_steps():
    """Whole steps with FCG (Jacobi bottom, no network needed) through efs_step: the step is one captured graph
    (the solve's conditional nodes inside it) and two steps match two CG steps within 1e-5."""
    n = 48
    with _dam_ctx(n, bottom=abi.FCG_BOTTOM_JACOBI) as s:
        s.update(1)
        state = s.fields()
        s.update(2)
        want = s.fields()
        p = s.params.copy()
        p.solver = abi.SOLVER_FCG_UNET
        s.set_params(p)
        assert s.kernels_per_step() > 0
        s.set_fields(state)
        s.update(2)
        got = s.fields()
        st = s.stats()
    assert st.converged and not st.paused and st.precond_steps == st.solve_steps
    for f in (abi.FIELD_VEL, abi.FIELD_RHO, abi.FIELD_PRESSURE):
        assert rel_l2(got[f], want[f]) < 1e-5, (abi.FIELD_NAMES[f], rel_l2(got[f], want[f]))


def test_preconditioner_timing_entry_point():
    """efs_fcg_time_vcycle times one preconditioner application (64^3: one aggregation level, the committed
    network's grid at the bottom) kernel by kernel and as a graph replay; it refuses a context whose solver is
    not FCG, and a solve afterwards still converges."""
    from eulerianfluidsimulation_gb300 import unet_weights
    n = 64
    with _dam_ctx(n, solver=abi.SOLVER_CG) as s:
        s.update(2)
        with pytest.raises(gb.EfsError) as ei:
            s.fcg_time_vcycle(2)
        assert ei.value.status == abi.EFS_ERR_STATE
        p = s.params.copy()
        p.solver = abi.SOLVER_FCG_UNET
        s.set_params(p)
        if unet_weights.available():
            unet_weights.load_into(s)
        else:
            s.unet_init(1, 0)
        direct, graph = s.fcg_time_vcycle(3)
        print(f"\npreconditioner at 64^3: {direct:.3f} ms kernel by kernel, {graph:.3f} ms as a graph replay")
        assert np.isfinite(direct) and np.isfinite(graph) and direct > 0 and graph > 0
        s.update(1)
        assert s.stats().converged
