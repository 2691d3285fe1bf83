"""The tensor-core (3xTF32 tcgen05) DFT patch solve against the CPU oracle.

Tolerances (infinity-norm relative to the FP64 oracle):
  FP32 DFT patch solve on the tensor cores: 2e-5 (FP32 data, ~22-bit products)
  FP32 V-cycle with tensor-core solves on every level: 5e-5
  tensor-core vs SIMT FP32 V-cycle: 2e-5
  GMG-preconditioned BiCGStab with the tensor-core cycle: 1e-10 FP64 residual
"""
import os

import numpy as np
import pytest

from conftest import rel_err

pytestmark = pytest.mark.gpu


def _meshes():
    from thunderegg_gb300 import mesh as M

    return {
        "2d_uniform_n16": (M.uniform_mesh(2, 2, 16), 0),
        "2d_uniform_n32": (M.uniform_mesh(2, 2, 32), 1),
        "2d_uniform_n64": (M.uniform_mesh(2, 1, 64), 1),
        "2d_circle_n16": (M.circle_mesh(n=16, lo=2, hi=4), 1),
        "2d_random_n32": (M.random_mesh(7, n=32, lo=1, hi=3), 0),
        "3d_uniform_n16": (M.uniform_mesh(3, 1, 16), 2),
        "3d_random_n16": (M.random_mesh(8, n=16, dim=3, lo=1, hi=2), 2),
    }


MESHES = None


def meshes():
    global MESHES
    if MESHES is None:
        MESHES = _meshes()
    return MESHES


def _filler(te, scheme):
    return [te.BiLinearGhostFiller, te.BiQuadraticGhostFiller, te.TriLinearGhostFiller][scheme]


def _inner(lv):
    g = lv.num_ghost
    return (Ellipsis,) + tuple(slice(g, -g) for _ in range(lv.dim))


@pytest.mark.parametrize("name", sorted(["2d_uniform_n16", "2d_uniform_n32", "2d_uniform_n64", "2d_circle_n16",
                                         "2d_random_n32", "3d_uniform_n16", "3d_random_n16"]))
def test_tc_patch_solve(te, oracle, name):
    """PatchSolver::apply in FP32 runs on the tensor cores and matches the FP64 oracle."""
    levels, sc = meshes()[name]
    lv = levels[0]
    dom = te.Domain(lv)
    op = te.PoissonStarPatchOperator(dom, _filler(te, sc)(dom))
    ps = te.DFTPatchSolver(op)
    assert ps.uses_tensor_cores
    rng = np.random.default_rng(11)
    f = rng.standard_normal(lv.padded_shape(1))
    u = rng.standard_normal(lv.padded_shape(1))
    want, _ = oracle.patch_solver(lv, f, u, sc, smoother=0, mode=1)
    f32 = te.Vector.from_numpy(dom, f, dtype=te.TE_F32)
    u32 = te.Vector.from_numpy(dom, u, dtype=te.TE_F32)
    ps.apply(f32, u32)
    got = u32.numpy()
    inner = _inner(lv)
    assert rel_err(got[inner], want[inner]) <= 2e-5
    # apply zeroes the ghost cells (u.setWithGhost(0))
    ghosts = np.ones(got.shape, bool)
    ghosts[inner] = False
    assert np.all(got[ghosts] == 0)


def test_tc_patch_solve_large_level(te, oracle):
    """Many CTA passes over patch groups (persistent loop), including a partial last group."""
    from thunderegg_gb300 import mesh as M

    lv = M.random_mesh(12, n=32, lo=3, hi=6)[0]
    dom = te.Domain(lv)
    op = te.PoissonStarPatchOperator(dom, te.BiQuadraticGhostFiller(dom))
    ps = te.DFTPatchSolver(op)
    assert ps.uses_tensor_cores
    f = np.random.default_rng(12).standard_normal(lv.padded_shape(1))
    want, _ = oracle.patch_solver(lv, f, np.zeros_like(f), 1, smoother=0, mode=1)
    f32 = te.Vector.from_numpy(dom, f, dtype=te.TE_F32)
    u32 = te.Vector(dom, dtype=te.TE_F32)
    ps.apply(f32, u32)
    inner = _inner(lv)
    assert rel_err(u32.numpy()[inner], want[inner]) <= 2e-5


def test_tc_off_switch(te):
    from thunderegg_gb300 import mesh as M

    lv = M.uniform_mesh(2, 1, 32)[0]
    dom = te.Domain(lv)
    op = te.PoissonStarPatchOperator(dom, te.BiLinearGhostFiller(dom))
    os.environ["TE_NO_TC"] = "1"
    try:
        assert not te.DFTPatchSolver(op).uses_tensor_cores
    finally:
        del os.environ["TE_NO_TC"]
    assert te.DFTPatchSolver(op).uses_tensor_cores
    # sizes without a tensor-core shape fall back to the SIMT transforms
    lv8 = M.uniform_mesh(2, 1, 8)[0]
    d8 = te.Domain(lv8)
    assert not te.DFTPatchSolver(te.PoissonStarPatchOperator(d8, te.BiLinearGhostFiller(d8))).uses_tensor_cores


@pytest.mark.parametrize("name", ["2d_circle_n16", "2d_random_n32", "3d_uniform_n16"])
def test_tc_vcycle(te, oracle, name):
    """The FP32 fused V-cycle with tensor-core solves on every level against the FP64 oracle cycle,
    and against the same cycle with SIMT FP32 transforms."""
    from oracle import gmg_config
    from thunderegg_gb300.gmg import GmgOptions, GmgSolver

    levels, sc = meshes()[name]
    f = np.random.default_rng(13).standard_normal(levels[0].padded_shape(1))
    want = oracle.vcycle(levels, f, gmg_config(scheme=sc, smoother=0))
    inner = _inner(levels[0])
    s = GmgSolver(levels, GmgOptions(scheme=sc, smoother=0, cycle_dtype=te.TE_F32))
    assert all(ps.uses_tensor_cores for ps in s.smoothers)
    fv = te.Vector.from_numpy(s.finest, f)
    uv = te.Vector(s.finest)
    for _ in range(2):  # the second application replays the captured graph
        s.cycle.apply(fv, uv)
        got = uv.numpy()
        assert rel_err(got[inner], want[inner]) <= 5e-5
    os.environ["TE_NO_TC"] = "1"
    try:
        s2 = GmgSolver(levels, GmgOptions(scheme=sc, smoother=0, cycle_dtype=te.TE_F32))
    finally:
        del os.environ["TE_NO_TC"]
    assert not any(ps.uses_tensor_cores for ps in s2.smoothers)
    uv2 = te.Vector(s2.finest)
    s2.cycle.apply(te.Vector.from_numpy(s2.finest, f), uv2)
    assert rel_err(got[inner], uv2.numpy()[inner]) <= 2e-5


@pytest.mark.parametrize("name", ["2d_circle_n16", "3d_uniform_n16"])
def test_tc_solve_reaches_tolerance(te, oracle, name):
    """Mixed precision (tensor-core FP32 cycle, FP64 BiCGStab) reaches 1e-10 and matches the FP64 oracle solve."""
    from oracle import gmg_config
    from thunderegg_gb300.gmg import GmgOptions, GmgSolver

    levels, sc = meshes()[name]
    f = np.random.default_rng(14).standard_normal(levels[0].padded_shape(1))
    u_o, its_o, _, rc = oracle.solve(levels, f, gmg_config(scheme=sc, smoother=0, tol=1e-12))
    s = GmgSolver(levels, GmgOptions(scheme=sc, smoother=0, cycle_dtype=te.TE_F32, bicgstab_flags=1))
    fv, uv = te.Vector.from_numpy(s.finest, f), te.Vector(s.finest)
    its = s.solve(fv, uv)
    assert its <= its_o + 3
    assert s.residual(fv, uv) <= 1e-10
    inner = _inner(levels[0])
    # solution error <= cond(A) * relative residual; cond ~ 1e3 here (random right-hand side)
    assert rel_err(uv.numpy()[inner], u_o[inner]) <= 1e-6


_CYCLE_SCRIPT = r"""
import sys, numpy as np
sys.path.insert(0, {root!r})
import thunderegg_gb300 as te
from thunderegg_gb300 import mesh as M
from thunderegg_gb300.gmg import GmgOptions, GmgSolver
levels = {mesh}
s = GmgSolver(levels, GmgOptions(scheme={scheme}, smoother=0, cycle_dtype=te.TE_F32))
f = np.random.default_rng(31).standard_normal(levels[0].padded_shape(1))
fv, uv = te.Vector.from_numpy(s.finest, f), te.Vector(s.finest)
s.cycle.apply(fv, uv)
np.save({out!r}, uv.numpy())
"""


@pytest.mark.parametrize("mesh,scheme", [("M.circle_mesh(n=32, lo=2, hi=4)", 1), ("M.uniform_mesh(3, 2, 16)", 2)])
def test_fine_restrict_matches_coarse_centric(tmp_path, mesh, scheme):
    """The fine-patch-centric residual+restriction gives the same cycle as the coarse-patch-centric kernel."""
    import subprocess
    import sys

    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    outs = []
    for off in ("0", "1"):
        out = str(tmp_path / f"u{off}.npy")
        env = dict(os.environ, TE_NO_FINE_RESTRICT=off)
        code = _CYCLE_SCRIPT.format(root=root, mesh=mesh, scheme=scheme, out=out)
        subprocess.run([sys.executable, "-c", code], check=True, env=env, timeout=300)
        outs.append(np.load(out))
    assert rel_err(outs[0], outs[1]) <= 1e-6


@pytest.mark.parametrize("name", ["2d_circle_n16", "3d_uniform_n16"])
@pytest.mark.parametrize("cycle_type", ("W", "F"))
def test_tc_w_and_fmg_cycles(te, oracle, name, cycle_type):
    """The FP32 W and FMG cycles on the tensor-core path (mid smooth, second coarse visit
    from the first visit's result) against the FP64 oracle cycles (pinned to the
    reference's own), against the same cycles on the general kernels, and a mixed
    precision solve with them reaching 1e-10."""
    from oracle import gmg_config
    from thunderegg_gb300.gmg import GmgOptions, GmgSolver

    levels, sc = meshes()[name]
    f = np.random.default_rng(15).standard_normal(levels[0].padded_shape(1))
    want = oracle.vcycle(levels, f, gmg_config(scheme=sc, smoother=0, cycle_type=cycle_type))
    inner = _inner(levels[0])
    opts = dict(scheme=sc, smoother=0, cycle_type=cycle_type, cycle_dtype=te.TE_F32)
    s = GmgSolver(levels, GmgOptions(**opts))
    assert all(ps.uses_tensor_cores for ps in s.smoothers)
    fv = te.Vector.from_numpy(s.finest, f)
    uv = te.Vector(s.finest)
    for _ in range(2):
        s.cycle.apply(fv, uv)
        got = uv.numpy()
        assert rel_err(got[inner], want[inner]) <= 5e-5
    os.environ["TE_NO_TC"] = "1"
    try:
        s2 = GmgSolver(levels, GmgOptions(**opts))
    finally:
        del os.environ["TE_NO_TC"]
    uv2 = te.Vector(s2.finest)
    s2.cycle.apply(te.Vector.from_numpy(s2.finest, f), uv2)
    assert rel_err(got[inner], uv2.numpy()[inner]) <= 2e-5
    s3 = GmgSolver(levels, GmgOptions(bicgstab_flags=1, **opts))
    uv3 = te.Vector(s3.finest)
    s3.solve(fv, uv3)
    assert s3.residual(fv, uv3) <= 1e-10


def test_tc_kernel_variants_give_the_same_bits(te, monkeypatch):
    """The autotuner may run the 3xTF32 solve with its operands in shared memory or in tensor
    memory, at any resident-CTA count: every choice computes the same products in the same order,
    so results are bit-identical (which keeps a batched solve equal to the same solve alone)."""
    from thunderegg_gb300 import mesh as M

    outs = []
    for mode in ("smem", "tmem"):
        monkeypatch.setenv("TE_TC_OPERANDS", mode)
        for levels in (M.circle_mesh(n=32, lo=2, hi=4), M.uniform_mesh(3, 1, 16)):
            lv = levels[0]
            dom = te.Domain(lv)
            sc = 1 if lv.dim == 2 else 2
            op = te.PoissonStarPatchOperator(dom, _filler(te, sc)(dom))
            ps = te.DFTPatchSolver(op)
            f = np.random.default_rng(80 + lv.dim).standard_normal(lv.padded_shape(1))
            u = te.Vector(dom, 1, te.TE_F32)
            ps.apply(te.Vector.from_numpy(dom, f, dtype=te.TE_F32), u)
            outs.append(u.numpy())
    assert np.array_equal(outs[0], outs[2]) and np.array_equal(outs[1], outs[3])


def test_autotuner_report(te):
    """After a tensor-core solve the tuner names its choice per shape, with every candidate's time."""
    import ctypes
    import json

    from thunderegg_gb300 import mesh as M

    lv = M.uniform_mesh(2, 4, 32)[0]
    dom = te.Domain(lv)
    op = te.PoissonStarPatchOperator(dom, te.BiLinearGhostFiller(dom))
    ps = te.DFTPatchSolver(op)
    u = te.Vector(dom, 1, te.TE_F32)
    ps.apply(te.Vector.from_numpy(dom, np.ones(lv.padded_shape(1)), dtype=te.TE_F32), u)
    need = ctypes.c_int(0)
    te.capi.check(te.capi.lib().te_tune_report(None, 0, ctypes.byref(need)))
    buf = ctypes.create_string_buffer(need.value)
    te.capi.check(te.capi.lib().te_tune_report(buf, need.value, ctypes.byref(need)))
    rep = json.loads(buf.value.decode())
    mine = [r for r in rep if "|dft_tc|D=2 n=32 P~2^8 " in r["key"]]
    assert mine, rep
    r = mine[0]
    assert r["choice"] in r["ms"] and len(r["ms"]) >= 2
    assert all(v is None or v > 0 for v in r["ms"].values())

