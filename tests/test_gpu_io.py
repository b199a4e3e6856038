"""Checkpoint / restart (binary state + bed + time, checksummed), the exact
and error vertex views (plot_exact / plot_error, conserv_kernels.cu:1310-1369)
and the CLI's --checkpoint / --restart."""
import os
import re
import subprocess

import numpy as np
import pytest

from conftest import ROOT

pytestmark = pytest.mark.gpu
VTX = (5.0, 5.0, 5.0, 1.0, 1.0, 10.0)


def vortex(dg, p=2):
    mesh = dg.Mesh.square(12, 12, box=(0, 10, 0, 10), jitter=0.15, seed=3)
    s = dg.Solver(mesh, dg.EULER, p, problem="euler_vortex", prm=VTX, cfl=0.2)
    s.init_conditions()
    return mesh, s


def test_restart_continues_bit_for_bit(dglib, tmp_path):
    dg = dglib
    mesh, s = vortex(dg)
    t = s.step(10, dg.SSP_RK3, 0.0)
    ck = str(tmp_path / "a.ckpt")
    s.save_checkpoint(ck, t)
    ta = s.step(10, dg.SSP_RK3, t)
    a = s.get_state()
    _, s2 = vortex(dg)
    t2 = s2.load_checkpoint(ck)
    assert t2 == t
    tb = s2.step(10, dg.SSP_RK3, t2)
    assert tb == ta and np.array_equal(s2.get_state(), a)


def test_checkpoint_keeps_the_bed_and_rejects_mismatches(dglib, tmp_path):
    dg = dglib
    mesh = dg.Mesh.square(8, 8, jitter=0.1, seed=4, bc=(-1, -1, -1, -1))
    s = dg.Solver(mesh, dg.SHALLOW_WATER, 2, problem="sw_hump", prm=(1.0, 0.1, 0.1, 0.5, 0.5))
    s.bathymetry_project("sine", (0.1, 1.0, 1.0))
    s.init_conditions()
    ck = str(tmp_path / "sw.ckpt")
    s.save_checkpoint(ck, 0.25)
    s2 = dg.Solver(mesh, dg.SHALLOW_WATER, 2, problem="sw_hump", prm=(1.0, 0.1, 0.1, 0.5, 0.5))
    assert s2.load_checkpoint(ck) == 0.25
    assert np.array_equal(s2.get_bathymetry(), s.get_bathymetry())
    assert np.array_equal(s2.get_state(), s.get_state())
    with pytest.raises(dg.DGError, match="another equation"):
        dg.Solver(mesh, dg.SHALLOW_WATER, 1).load_checkpoint(ck)
    raw = bytearray(open(ck, "rb").read())
    raw[100] ^= 1
    bad = str(tmp_path / "bad.ckpt")
    open(bad, "wb").write(bytes(raw))
    with pytest.raises(dg.DGError, match="checksum"):
        s2.load_checkpoint(bad)
    open(bad, "wb").write(bytes(raw[:-20]))
    with pytest.raises(dg.DGError, match="truncated"):
        s2.load_checkpoint(bad)


def test_exact_and_error_views(dglib):
    dg = dglib
    mesh = dg.Mesh.square(10, 10, jitter=0.1, seed=1)
    s = dg.Solver(mesh, dg.ADVECTION, 3, problem="adv_sine", cfl=0.3)
    s.init_conditions()
    t = s.step(5, dg.SSP_RK3, 0.0)
    V = mesh.arrays()[0]
    ex = np.stack([np.sin(2 * np.pi * (V[2 * v] - 1.0 * t)) * np.sin(2 * np.pi * (V[2 * v + 1] - 0.5 * t))
                   for v in range(3)])
    np.testing.assert_allclose(s.plot_exact(0, t), ex, rtol=0, atol=1e-13)
    err = s.plot_error(0, t)
    np.testing.assert_allclose(err, s.eval_u(0) - s.plot_exact(0, t), rtol=0, atol=1e-15)
    assert 0 < np.abs(err).max() < 1e-2


def test_cli_checkpoint_restart(dglib, tmp_path):
    dg = dglib
    cli = os.path.join(ROOT, "dgcuda_gb300", "dgcuda")
    mesh = dg.Mesh.square(10, 10, box=(0, 10, 0, 10), jitter=0.15, seed=3)
    path = str(tmp_path / "v.pmsh")
    mesh.write(path)
    base = [cli, "-n", "2", "--eq", "euler", "--problem", "euler_vortex", "--prm",
            ",".join(map(str, VTX)), "--scheme", "ssprk3", "--cfl", "0.2"]
    ck = str(tmp_path / "v.ckpt")
    runs = [base + ["-t", "8", "-o", str(tmp_path / "o1"), "--checkpoint", ck, path],
            base + ["-t", "8", "-o", str(tmp_path / "o2"), "--restart", ck, path],
            base + ["-t", "16", "-o", str(tmp_path / "o3"), path]]
    for r in runs:
        p = subprocess.run(r, capture_output=True, text=True)
        assert p.returncode == 0, p.stderr
    a = open(str(tmp_path / "o2" / "U0-final.pos")).read()
    b = open(str(tmp_path / "o3" / "U0-final.pos")).read()
    assert a == b


@pytest.mark.parametrize("eq,p,n", [(1, 3, 200), (2, 2, 260)])
def test_large_state_round_trip_in_chunks(dglib, eq, p, n):
    """States above 16 MB move in chunks of rows (copies overlapping the
    permutation): a round trip is exact, from pinned and from pageable
    memory, also when the row count (18 for shallow water p = 2) does not
    split evenly."""
    import torch
    dg = dglib
    mesh = dg.Mesh.square(n, n, jitter=0.1, seed=6)
    s = dg.Solver(mesh, eq, p)
    shape = (s.N, s.n_p, s.K)
    assert s.N * s.n_p * s.K * 8 > 16 << 20
    rng = np.random.default_rng(p)
    x = rng.standard_normal(shape)
    s.set_state(x)
    assert np.array_equal(s.get_state(), x)
    pinned = torch.empty(shape, dtype=torch.float64, pin_memory=True).numpy()
    pinned[...] = -x
    s.set_state(pinned)
    out = torch.empty(shape, dtype=torch.float64, pin_memory=True).numpy()
    s.get_state(out=out)
    assert np.array_equal(out, -x)
