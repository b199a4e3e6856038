"""Accuracy against exact solutions: the L2 error converges at order p+1
for linear advection and the isentropic Euler vortex (SSP-RK3), and the
benchmark configurations 1 and 2 run as specified."""
import numpy as np
import pytest

from conftest import relerr

pytestmark = pytest.mark.gpu

VORTEX = (5.0, 5.0, 5.0, 1.0, 1.0, 10.0)  # beta, x0, y0, uinf, vinf, L


def rates(errs):
    return [np.log2(errs[i] / errs[i + 1]) for i in range(len(errs) - 1)]


@pytest.mark.parametrize("p", [1, 2, 3])
def test_advection_order(dglib, p):
    dg = dglib
    errs = []
    for n in (8, 16, 32):
        mesh = dg.Mesh.square(n, n, jitter=0.1, seed=11)
        s = dg.Solver(mesh, dg.ADVECTION, p, problem="adv_sine", cfl=0.3 if p < 3 else 0.1)
        s.init_conditions()
        t, _ = s.advance_to(0.5, dg.SSP_RK3)
        errs.append(s.eval_error_L2(t)[0])
    r = rates(errs)
    assert r[-1] >= p + 1 - 0.35, (errs, r)


@pytest.mark.parametrize("p", [1, 2, 3])
def test_vortex_order(dglib, p):
    dg = dglib
    errs = []
    for n in (16, 32, 64):
        mesh = dg.Mesh.square(n, n, box=(0, 10, 0, 10), jitter=0.15, seed=13)
        s = dg.Solver(mesh, dg.EULER, p, problem="euler_vortex", prm=VORTEX,
                      cfl=0.2 if p < 3 else 0.1)
        s.init_conditions()
        t, _ = s.advance_to(0.5, dg.SSP_RK3)
        errs.append(s.eval_error_L2(t)[0])
    r = rates(errs)
    assert r[-1] >= p + 1 - 0.5, (errs, r)


def test_config1_advection_to_T1(dglib):
    """32x32 periodic squares, jitter 0.1, p=1, upwind, SSP-RK3 CFL 0.3 to T=1."""
    dg = dglib
    mesh = dg.Mesh.square(32, 32, jitter=0.1, seed=1)
    s = dg.Solver(mesh, dg.ADVECTION, 1, problem="adv_sine", cfl=0.3, ax=1.0, ay=0.5)
    s.init_conditions()
    e0 = s.eval_error_L2(0.0)[0]
    t, n = s.advance_to(1.0, dg.SSP_RK3)
    e1 = s.eval_error_L2(t)[0]
    assert t == 1.0 and n > 100
    assert e1 < 0.05 and e0 < e1


@pytest.mark.parametrize("p", [2, 3])
def test_config2_vortex_matches_oracle(dglib, oracle_mod, p):
    """128x128 squares on [0,10]^2, jitter 0.15, Rusanov, SSP-RK3 CFL 0.2:
    50 steps against the oracle (state 1e-10), then the error stays small."""
    dg = dglib
    mesh = dg.Mesh.square(128, 128, box=(0, 10, 0, 10), jitter=0.15, seed=2)
    s = dg.Solver(mesh, dg.EULER, p, problem="euler_vortex", prm=VORTEX, cfl=0.2)
    s.init_conditions()
    c0 = s.get_state()
    t = s.step(50, dg.SSP_RK3, 0.0)
    o = oracle_mod.Oracle.from_mesh(mesh, dg.EULER, p, oracle_mod.prm_vec(extra=VORTEX),
                                    dg.PROBLEMS["euler_vortex"])
    c, to, _ = o.step(c0, 50, 0, 0, 0.2)
    assert abs(t - to) <= 1e-12 * to
    assert relerr(s.get_state(), c, 4) <= 1e-10
    err = s.eval_error_L2(t)
    assert err[0] < 1e-3
