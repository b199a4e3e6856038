"""The dgcuda command line (run_dgcuda's flags, main.cu:481-599)."""
import os
import re
import subprocess

import numpy as np
import pytest

from conftest import ROOT

CLI = os.path.join(ROOT, "dgcuda_gb300", "dgcuda")


def test_usage_and_bad_options(dglib):
    r = subprocess.run([CLI, "-h"], capture_output=True, text=True)
    assert r.returncode == 1 and "Usage: dgcuda" in r.stdout
    r = subprocess.run([CLI, "--bogus", "x", "m.pmsh"], capture_output=True, text=True)
    assert r.returncode == 1
    r = subprocess.run([CLI, "-n", "9", "m.pmsh"], capture_output=True, text=True)
    assert r.returncode == 1


def test_missing_mesh_is_an_error_not_a_crash(dglib, tmp_path):
    r = subprocess.run([CLI, "-n", "1", "-t", "1", str(tmp_path / "none.pmsh")],
                       capture_output=True, text=True)
    assert r.returncode == 1 and "mesh file not found" in r.stderr


@pytest.mark.gpu
def test_cli_matches_library(dglib, tmp_path):
    dg = dglib
    vtx = (5.0, 5.0, 5.0, 1.0, 1.0, 10.0)
    mesh = dg.Mesh.square(16, 16, box=(0, 10, 0, 10), jitter=0.15, seed=3)
    path = str(tmp_path / "v.pmsh")
    mesh.write(path)
    out = str(tmp_path / "out")
    r = subprocess.run([CLI, "-n", "2", "-T", "0.1", "-e", "--eq", "euler", "--problem",
                        "euler_vortex", "--prm", ",".join(map(str, vtx)), "--scheme", "ssprk3",
                        "--cfl", "0.2", "-o", out, path], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    errs = [float(x) for x in re.findall(r"L2 U\d error\s+= (\S+)", r.stdout)]
    s = dg.Solver(mesh, dg.EULER, 2, problem="euler_vortex", prm=vtx, cfl=0.2)
    s.init_conditions()
    t, _ = s.advance_to(0.1, dg.SSP_RK3)
    np.testing.assert_allclose(errs, s.eval_error_L2(t), rtol=1e-6)
    lines = open(os.path.join(out, "U0-final.pos")).read().splitlines()
    assert lines[0].startswith('View "U0 "') and len(lines) == mesh.K + 2
    uv = s.eval_u(0)
    first = [float(x) for x in re.findall(r"\{([^}]*)\}", lines[1])[0].split(",")]
    np.testing.assert_allclose(first, uv[:, 0], rtol=1e-12)


@pytest.mark.gpu
def test_cli_runs_a_gmsh_file(dglib, tmp_path):
    """A Gmsh .msh given to the CLI is converted as genmesh.py would and run."""
    dg = dglib
    msh = os.path.join(ROOT, "tests", "golden", "gmsh_square6.msh")
    out = str(tmp_path / "out")
    r = subprocess.run([CLI, "-n", "1", "-t", "5", "--eq", "advection", "--problem", "adv_sine",
                        "-o", out, msh], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    mesh = dg.Mesh.read_gmsh(msh)
    s = dg.Solver(mesh, dg.ADVECTION, 1, problem="adv_sine", cfl=0.5)
    s.init_conditions()
    s.step(5, dg.RK4, 0.0)
    uv = s.eval_u(0)
    lines = open(os.path.join(out, "U0-final.pos")).read().splitlines()
    vals = np.array([[float(x) for x in re.findall(r"\{([^}]*)\}", l)[0].split(",")]
                     for l in lines[1:1 + mesh.K]])
    np.testing.assert_allclose(vals, uv.T, rtol=0, atol=1e-12)


def test_new_options_reject_bad_arguments(dglib, tmp_path):
    """--field wants 4 numbers, --series t0 and whole (amp, omega, phase)
    triples (at most 16), --reference-settings a known --problem."""
    mesh = str(tmp_path / "none.pmsh")
    for args in (["--field", "1,2,3"], ["--series", "0.5,1,2"],
                 ["--series", ",".join(["1"] * 50)], ["--reference-settings"],
                 ["--reference-settings", "--problem", "no_such_problem"]):
        r = subprocess.run([CLI, "-n", "1", "-t", "1"] + args + [mesh], capture_output=True,
                           text=True)
        assert r.returncode == 1 and "Usage: dgcuda" in r.stdout, args


def _pos_values(path, K):
    lines = open(path).read().splitlines()
    return np.array([[float(x) for x in re.findall(r"\{([^}]*)\}", l)[0].split(",")]
                     for l in lines[1:1 + K]])


@pytest.mark.gpu
def test_cli_reference_settings_and_field(dglib, tmp_path):
    """--reference-settings takes the problem file's settings (here spin:
    its rotation, RK2, no limiter); --field replaces the velocity; both as
    the library runs them."""
    dg = dglib
    mesh = dg.Mesh.square(12, 12, jitter=0.1, seed=8, bc=(-3, -3, -3, -3))
    path = str(tmp_path / "m.pmsh")
    mesh.write(path)
    out = str(tmp_path / "a")
    r = subprocess.run([CLI, "-n", "2", "-t", "6", "--eq", "advection", "--problem", "adv_spin",
                        "--reference-settings", "-o", out, path], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    P, scheme = dg.params_for_problem("adv_spin")
    assert scheme == dg.RK2
    P.cfl = 0.7  # the CLI's default CFL for RK2
    s = dg.Solver(mesh, dg.ADVECTION, 2, params=P)
    s.init_conditions()
    s.step(6, scheme, 0.0)
    np.testing.assert_allclose(_pos_values(os.path.join(out, "U0-final.pos"), mesh.K),
                               s.eval_u(0).T, rtol=0, atol=1e-12)
    out = str(tmp_path / "b")
    r = subprocess.run([CLI, "-n", "1", "-t", "6", "--eq", "advection", "--problem", "adv_sine",
                        "--velocity", "0.3,-0.2", "--field", "0.1,-1.5,1.5,0.2", "-o", out, path],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    s = dg.Solver(mesh, dg.ADVECTION, 1, problem="adv_sine", cfl=0.5)
    s.set_velocity_field(0.3, -0.2, (0.1, -1.5, 1.5, 0.2))
    s.init_conditions()
    s.step(6, dg.RK4, 0.0)
    np.testing.assert_allclose(_pos_values(os.path.join(out, "U0-final.pos"), mesh.K),
                               s.eval_u(0).T, rtol=0, atol=1e-12)


def test_new_options_are_accepted(dglib, tmp_path):
    """Well-formed --reference-settings, --field and --series pass the
    argument checks (the run then stops at the missing mesh)."""
    mesh = str(tmp_path / "none.pmsh")
    for args in (["--problem", "adv_spin", "--reference-settings", "--eq", "advection"],
                 ["--eq", "advection", "--problem", "adv_sine", "--field", "0,-1,1,0"],
                 ["--problem", "euler_pulse", "--series", "0.9,0.05,4.4,2.9,0.03,8.9,2.6"]):
        r = subprocess.run([CLI, "-n", "1", "-t", "1"] + args + [mesh], capture_output=True,
                           text=True)
        assert r.returncode == 1 and "mesh file not found" in r.stderr, (args, r.stdout)
