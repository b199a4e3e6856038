"""SSP-RK3 time stepping (not in the reference; restated in the oracle) on
the GPU against the oracle, plus size-independent properties at full size."""
import numpy as np
import pytest

from conftest import relerr

pytestmark = pytest.mark.gpu


def vortex_params(dg, **kw):
    P = dg.Params()
    import ctypes
    dg.load_library().dg_params_default(ctypes.byref(P))
    P.problem = dg.PROBLEMS["euler_vortex"]
    for i, v in enumerate((5.0, 5.0, 5.0, 1.0, 1.0, 10.0)):
        P.prm[i] = v
    P.cfl = 0.2
    for k, v in kw.items():
        setattr(P, k, v)
    return P


CASES = [
    # eq, problem, box, bc, p, limiter, cfl, nsteps, extra prm
    ("adv_sine", 0, "adv_sine", (0, 1, 0, 1), (0, 0, 0, 0), 2, 0, 0.3, 20, ()),
    ("euler_vortex", 1, "euler_vortex", (0, 10, 0, 10), (0, 0, 0, 0), 3, 0, 0.2, 10,
     (5.0, 5.0, 5.0, 1.0, 1.0, 10.0)),
    ("euler_riemann4_lim", 1, "euler_riemann4", (0, 1, 0, 1), (-4, -4, -4, -4), 1, 1, 0.3, 10, ()),
    ("euler_riemann4_p2_lim", 1, "euler_riemann4", (0, 1, 0, 1), (-4, -4, -4, -4), 2, 1, 0.2, 6, ()),
    ("sw_hump_wall", 2, "sw_hump", (0, 1, 0, 1), (-1, -1, -1, -1), 2, 0, 0.3, 10,
     (1.0, 0.1, 0.1, 0.45, 0.55)),
    ("maxwell_plane", 3, "maxwell_plane", (0, 1, 0, 1), (0, 0, 0, 0), 3, 0, 0.3, 10, ()),
]


@pytest.mark.parametrize("case", CASES, ids=[c[0] for c in CASES])
def test_ssp_rk3_matches_oracle(dglib, oracle_mod, case):
    name, eq, pb, box, bc, p, lim, cfl, nsteps, extra = case
    dg = dglib
    mesh = dg.Mesh.square(10, 10, box=box, jitter=0.1, seed=5, bc=bc)
    s = dg.Solver(mesh, eq, p, problem=pb, limiter=lim, cfl=cfl, gravity=9.81, prm=extra)
    s.init_conditions()
    c0 = s.get_state()
    t = s.step(nsteps, dg.SSP_RK3, 0.0)
    prm = oracle_mod.prm_vec(g=9.81, extra=extra)
    o = oracle_mod.Oracle.from_mesh(mesh, eq, p, prm, dg.PROBLEMS[pb])
    c, to, n = o.step(c0, nsteps, 0, lim, cfl)
    assert n == nsteps
    assert abs(t - to) <= 1e-12 * to
    assert relerr(s.get_state(), c, s.N) <= 1e-10


def test_advance_to_lands_on_end_time(dglib):
    dg = dglib
    mesh = dg.Mesh.square(8, 8, jitter=0.1, seed=3)
    s = dg.Solver(mesh, dg.ADVECTION, 1, problem="adv_sine", cfl=0.3)
    s.init_conditions()
    t, n = s.advance_to(0.25, dg.SSP_RK3, 0.0)
    assert t == 0.25 and n > 0


def test_free_stream_preserved_full_size(dglib):
    """A uniform state has zero right-hand side on any mesh (metric identities)."""
    dg = dglib
    mesh = dg.Mesh.square(512, 512, jitter=0.1, seed=3, bc=(-4, -4, -4, -4))
    s = dg.Solver(mesh, dg.EULER, 3, problem="none")
    N, npm, K = s.shape
    c = np.zeros(s.shape)
    rho, u, v, p = 1.3, 0.4, -0.2, 0.9
    U = [rho, rho * u, rho * v, p / 0.4 + 0.5 * rho * (u * u + v * v)]
    for n in range(4):
        c[n, 0, :] = U[n] / np.sqrt(2.0)
    r = s.eval_rhs(c, 0.0)
    assert np.abs(r).max() < 1e-10


def test_periodic_conservation_and_determinism(dglib):
    """Periodic Euler p=3: cell-mean mass sum_e J_e c0_e is conserved to
    round-off, and two runs are bitwise identical."""
    dg = dglib
    mesh = dg.Mesh.square(128, 128, box=(0, 10, 0, 10), jitter=0.15, seed=2)
    V, _, _, _ = mesh.arrays()
    J = (V[2] - V[0]) * (V[5] - V[1]) - (V[4] - V[0]) * (V[3] - V[1])
    outs = []
    for _ in range(2):
        s = dg.Solver(mesh, dg.EULER, 3, params=vortex_params(dg))
        s.init_conditions()
        m0 = (s.get_state()[:, 0, :] * J).sum(axis=1)
        s.step(20, dg.SSP_RK3, 0.0)
        c = s.get_state()
        outs.append(c)
        m1 = (c[:, 0, :] * J).sum(axis=1)
        assert np.all(np.abs(m1 - m0) <= 1e-11 * np.abs(m0).max())
    assert np.array_equal(outs[0], outs[1])
