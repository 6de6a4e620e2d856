"""CPU checks of the boundary: the C-ABI library loads without a GPU and exports every function that
include/*.h declares; the presets agree between C and Python; the C++ drop-in backend compiles and links
against the reference's own headers (where the reference tree is present)."""
import os
import re
import subprocess
import tempfile

import pytest

from oracle import oracle

ROOT = os.path.abspath(os.path.join(os.path.dirname(__file__), ".."))


def _lib():
    from eulerianfluidsimulation_gb300 import build
    build.build()
    from eulerianfluidsimulation_gb300._lib import lib
    return lib()


def declared_functions():
    names = set()
    for h in os.listdir(os.path.join(ROOT, "include")):
        if not h.endswith(".h"):
            continue
        text = open(os.path.join(ROOT, "include", h)).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        text = re.sub(r"static inline[^{;]*\{", "{", text)   # header-only helpers are not exported
        for m in re.finditer(r"^\s*(?:const\s+)?[A-Za-z_][\w\s\*]*?\b(efs_\w+)\s*\(", text, flags=re.M):
            names.add(m.group(1))
    return sorted(names)


def test_library_exports_every_declared_function():
    L = _lib()
    names = declared_functions()
    assert len(names) >= 25
    missing = [n for n in names if not hasattr(L, n)]
    assert not missing, missing
    from eulerianfluidsimulation_gb300._lib import SIGNATURES
    assert set(SIGNATURES) == set(names)


def test_library_loads_without_device():
    import eulerianfluidsimulation_gb300 as gb
    L = _lib()
    assert L.efs_abi_version() == 1
    if gb.device_count() == 0:
        with pytest.raises(gb.EfsError) as ei:
            gb.GB300Simulator3D(16, 16, 16)
        assert ei.value.status == 4   # EFS_ERR_NO_DEVICE


def test_presets_match_between_c_and_python():
    import eulerianfluidsimulation_gb300 as gb
    from eulerianfluidsimulation_gb300 import abi
    _lib()
    for cs, dt in ((1 / 128, 0.004), (1 / 256, 0.004), (1 / 64, 0.005)):
        assert gb.params_dam(cs, dt).as_dict() == abi.params_dam(cs, dt).as_dict()


def test_scene_generators_match_the_oracle():
    import numpy as np
    import eulerianfluidsimulation_gb300 as gb
    from oracle import oracle
    _lib()
    for seed in range(6):
        a = gb.scene_dam3d(48, 48, 48, 4, 24, seed)
        b = oracle.scene_dam3d(48, 48, 48, 4, 24, seed)
        assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])
        c = gb.scene_batch2d(seed)
        d = oracle.scene_batch2d(seed)
        assert np.array_equal(c[0], d[0]) and np.array_equal(c[1], d[1])


@pytest.mark.skipif(not os.path.isdir(os.path.join(oracle.reference_tree(), "include")), reason="reference tree not present")
def test_drop_in_backend_builds_against_reference_headers():
    _lib()
    REFERENCE = oracle.reference_tree()
    inc = ["-I", os.path.join(ROOT, "oracle", "shim"), "-I", os.path.join(REFERENCE, "include"), "-I", os.path.join(ROOT, "include")]
    srcs = [os.path.join(REFERENCE, "src/simulation/simulator/ISimulator.cpp")] + \
        [os.path.join(REFERENCE, f"src/simulation/data/{k}.cpp") for k in ("ScalField3D", "ScalField2D", "VecField3D", "VecField2D")]
    with tempfile.TemporaryDirectory() as d:
        out = os.path.join(d, "libgb300backend.so")
        cmd = ["g++", "-std=c++20", "-O1", "-fPIC", "-w", "-shared", "-Wl,--no-undefined"] + inc + \
              ["-o", out, os.path.join(ROOT, "eulerianfluidsimulation_gb300/host/GB300Simulator.cpp")] + srcs + \
              ["-L", os.path.join(ROOT, "eulerianfluidsimulation_gb300"), "-lefs_gb300"]
        res = subprocess.run(cmd, capture_output=True, text=True)
        assert res.returncode == 0, res.stderr[-2000:]


def _dropin_expected(n):
    """The efs_params the C++ drop-in must derive from tests/dropin_driver.cpp's Properties (an n^3 dam break
    with the reference's CG): the reference semantics of the solver (absolute r.r threshold, float dot products)
    and velocity decay disabled."""
    from eulerianfluidsimulation_gb300 import abi
    p = abi.params_dam(1.0 / n, 0.004, abi.SOLVER_CG, 1e-5)
    p.tol_rel = 0.0
    p.cg_variant = abi.CG_REFERENCE
    p.max_steps = 2000
    p.disable_mask = 1 << abi.STAGE_VEL_DECAY
    return p


def test_dropin_fixture_params_are_the_adapter_mapping():
    """ref_dropin_dam32.npz holds the efs_params GB300ParamsFromProperties() returned beside the reference's run."""
    import numpy as np
    from eulerianfluidsimulation_gb300 import abi
    from tests.helpers import GOLDEN
    z = np.load(os.path.join(GOLDEN, "ref_dropin_dam32.npz"))
    got = abi.EfsParams.from_buffer_copy(z["params"].tobytes()).as_dict()
    assert got == _dropin_expected(int(z["meta"][0])).as_dict()
    assert not z["paused"].any() and (z["steps"] > 0).all()


@pytest.mark.skipif(not oracle.reference_tree_present(), reason="reference tree not present")
def test_dropin_driver_runs_the_adapter():
    """tests/dropin_driver.cpp, built against the reference's headers and its CPU build: the Properties the
    application sets map to the expected efs_params, and without a CUDA device GB300Simulator3D reports the
    backend's error instead of stepping (the reference-side construction and update() calls still run)."""
    _lib()
    exe = oracle.dropin_driver()
    res = subprocess.run([exe, "params"], capture_output=True, text=True, timeout=60)
    assert res.returncode == 0, res.stderr
    got = dict(kv.split("=") for kv in res.stdout.split())
    want = _dropin_expected(64).as_dict()
    for k, v in got.items():
        assert float(v) == pytest.approx(float(want[k]), rel=1e-7), (k, v, want[k])
    assert set(got) <= set(want)
    import torch
    if not torch.cuda.is_available():
        res = subprocess.run([exe, "run", "32", "2"], capture_output=True, text=True, timeout=120)
        assert res.returncode == 0, res.stderr
        assert res.stdout.startswith("no-device"), res.stdout
