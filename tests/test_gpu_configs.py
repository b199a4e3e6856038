"""Parity at the benchmark configurations' own sizes, against the oracle.

* Four-quadrant Riemann problem (the throughput configuration): 1024 x 1024
  squares cut into 2,097,152 triangles jittered by +-0.1h (seed 3),
  transmissive sides, Rusanov flux, Barth-Jespersen limiter, SSP-RK3 at CFL
  0.2, FP64, p = 1..4 -- each order with the element stage the bench runs
  (tensor-core contractions from p = 2, the FP64-FMA kernel at p = 1): 3
  steps against the oracle (state 1e-10, time 1e-12), then the right-hand
  side of the stepped state against the oracle's (1e-12).
* Isentropic vortex (beta 5 at (5, 5), free stream 1): 128 x 128 squares on
  [0, 10]^2 (32,768 triangles, jitter 0.15, seed 2), periodic, p = 2 and 3,
  SSP-RK3 at CFL 0.2, all 1000 steps against the oracle (state 1e-10), and
  the L2 error against the advected exact vortex.

Tolerances are norm-wise per variable block, as in the other parity tests.
"""
import numpy as np
import pytest

from conftest import relerr

pytestmark = pytest.mark.gpu

STATE_TOL = 1e-10
RHS_TOL = 1e-12
VORTEX = (5.0, 5.0, 5.0, 1.0, 1.0, 10.0)  # beta, x0, y0, uinf, vinf, L


@pytest.fixture(scope="module")
def riemann_mesh(dglib):
    return dglib.Mesh.square(1024, 1024, jitter=0.1, seed=3, bc=(-4, -4, -4, -4))


@pytest.mark.parametrize("p", [1, 2, 3, 4])
def test_riemann4_full_size_matches_oracle(dglib, oracle_mod, riemann_mesh, p):
    dg = dglib
    mesh = riemann_mesh
    assert mesh.K == 2097152
    s = dg.Solver(mesh, dg.EULER, p, problem="euler_riemann4", limiter=1, cfl=0.2, gamma=1.4)
    assert s.tensor_contractions == (p >= 2)
    s.init_conditions()
    c0 = s.get_state()
    t = s.step(3, dg.SSP_RK3, 0.0)
    o = oracle_mod.Oracle.from_mesh(mesh, dg.EULER, p, oracle_mod.prm_vec(gamma=1.4),
                                    dg.PROBLEMS["euler_riemann4"])
    c, to, n = o.step(c0, 3, 0, 1, 0.2)
    assert n == 3 and abs(t - to) <= 1e-12 * to
    cg = s.get_state()
    assert relerr(cg, c, 4) <= STATE_TOL
    # the operator itself on the stepped (limited) state
    r_gpu = s.eval_rhs(cg, t)
    r_ref = o.rhs(cg, t)
    assert relerr(r_gpu, r_ref, 4) <= RHS_TOL
    s.close()


@pytest.mark.parametrize("p", [2, 3])
def test_vortex_1000_steps_matches_oracle(dglib, oracle_mod, p):
    dg = dglib
    mesh = dg.Mesh.square(128, 128, box=(0, 10, 0, 10), jitter=0.15, seed=2)
    assert mesh.K == 32768
    s = dg.Solver(mesh, dg.EULER, p, problem="euler_vortex", prm=VORTEX, cfl=0.2)
    assert s.tensor_contractions
    s.init_conditions()
    c0 = s.get_state()
    e0 = s.eval_error_L2(0.0)[0]
    t = s.step(1000, dg.SSP_RK3, 0.0)
    o = oracle_mod.Oracle.from_mesh(mesh, dg.EULER, p, oracle_mod.prm_vec(extra=VORTEX),
                                    dg.PROBLEMS["euler_vortex"])
    c, to, n = o.step(c0, 1000, 0, 0, 0.2)
    assert n == 1000 and abs(t - to) <= 1e-12 * to
    assert relerr(s.get_state(), c, 4) <= STATE_TOL
    # the advected vortex stays resolved
    e1 = s.eval_error_L2(t)[0]
    assert e0 < 1e-3 and e1 < 1e-3
    s.close()
