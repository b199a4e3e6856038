"""The reference's formula-defined problems (initial state, inflow/outflow
states, wall rules, the advection velocity fields) on the GPU against the
oracle's restatement of the same plugins, stepped with each problem's
scheme."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SERIES = (np.array([0.05, 0.03]), np.array([4.47, 8.95]), np.array([2.9, 2.66]), 0.9197)

CASES = [
    # name, eq, box, bc (left, right, bottom, top), p, limiter, scheme, cfl, steps
    ("euler_cylinder", 1, (1, 3, 1, 3), (-3, -2, -1, -1), 2, 0, 0, 0.3, 10),
    ("euler_lshock", 1, (0, 1, 0, 1), (-3, -2, -1, -1), 3, 0, 0, 0.3, 10),
    ("euler_doublemach", 1, (0, 4, 0, 1), (-3, -2, -1, -3), 1, 1, 2, 0.3, 6),
    ("euler_doublemach", 1, (0, 4, 0, 1), (-3, -2, -1, -3), 2, 1, 0, 0.2, 4),
    ("euler_airfoil", 1, (0, 1, 0, 1), (-3, -2, -1, -1), 2, 1, 0, 0.3, 10),
    ("euler_pulse", 1, (0, 4, 0, 1), (-3, -2, -1, -1), 2, 0, 1, 0.3, 10),
    ("adv_rotatinghill", 0, (-1, 1, -1, 1), (-3, -3, -3, -3), 2, 0, 1, 0.3, 20),
    ("adv_spin", 0, (0, 1, 0, 1), (-3, -3, -3, -3), 1, 0, 2, 0.3, 20),
    ("adv_squarehill", 0, (-1, 1, -1, 1), (-3, -2, -2, -2), 2, 1, 1, 0.3, 20),
    ("maxwell_cmirror", 3, (0, 1, 0, 1), (-3, -2, -1, -1), 2, 0, 1, 0.3, 20),
    ("maxwell_wscatter", 3, (-.5, .5, -.5, .5), (-3, -2, -1, -1), 2, 0, 0, 0.3, 20),
]


def close(a, b, tol):
    """Norm-wise over the whole state: in uniform flows and states at rest
    some variables are zero up to rounding, where a per-variable relative
    error would compare rounding with rounding."""
    return np.linalg.norm(a - b) <= tol * max(np.linalg.norm(b), 1e-300)


@pytest.mark.parametrize("case", CASES, ids=["%s_p%d_s%d" % (c[0], c[4], c[6]) for c in CASES])
def test_problem_matches_oracle(dglib, oracle_mod, case):
    pb, eq, box, bc, p, lim, scheme, cfl, nsteps = case
    dg = dglib
    mesh = dg.Mesh.square(24, 8 if box[1] == 4 else 12, box=box, jitter=0.1, seed=9, bc=bc)
    s = dg.Solver(mesh, eq, p, problem=pb, limiter=lim, cfl=cfl)
    o = oracle_mod.Oracle.from_mesh(mesh, eq, p, oracle_mod.prm_vec(), dg.PROBLEMS[pb])
    if pb == "euler_pulse":
        s.set_inflow_series(*SERIES)
        o.set_series(*SERIES)
    s.init_conditions()
    c0 = s.get_state()
    assert close(c0, o.init(), 1e-14)
    t = s.step(nsteps, scheme, 0.0)
    c, to, n = o.step(c0, nsteps, scheme, lim, cfl)
    assert n == nsteps and abs(t - to) <= 1e-12 * to
    g = s.get_state()
    assert np.all(np.isfinite(g))
    assert np.abs(g).max() > 0
    assert close(g, c, 1e-10)


@pytest.mark.parametrize("scheme", [0, 1])
def test_affine_velocity_field_matches_oracle(dglib, oracle_mod, scheme):
    """A general affine field (shear, stretch and rotation together) through
    the element, face and CFL paths: the step sizes agree, so the host's
    element-speed maximum is the oracle's."""
    dg = dglib
    mesh = dg.Mesh.square(16, 16, box=(-1, 1, -1, 1), jitter=0.1, seed=4, bc=(-3, -2, -2, -3))
    ax, ay, grad = 0.4, -0.3, (0.25, -1.7, 1.9, -0.1)
    s = dg.Solver(mesh, dg.ADVECTION, 2, problem="adv_sine", cfl=0.3)
    s.set_velocity_field(ax, ay, grad)
    o = oracle_mod.Oracle.from_mesh(mesh, dg.ADVECTION, 2, oracle_mod.prm_vec(ax=ax, ay=ay),
                                    dg.PROBLEMS["adv_sine"])
    o.set_field(ax, ay, grad)
    lam, _ = o.lambdas(np.zeros((1, 6, mesh.K)), 0.0)
    assert abs(s.velocity_field()[3] - lam.max()) <= 1e-14 * lam.max()
    s.init_conditions()
    c0 = s.get_state()
    t = s.step(15, scheme, 0.0)
    c, to, n = o.step(c0, 15, scheme, 0, 0.3)
    assert n == 15 and abs(t - to) <= 1e-13 * to
    assert close(s.get_state(), c, 1e-10)


def test_constant_field_is_the_constant_velocity(dglib):
    """A field with zero gradient is the constant-velocity path, bit for
    bit."""
    dg = dglib
    mesh = dg.Mesh.square(12, 12, jitter=0.1, seed=5)
    a = dg.Solver(mesh, dg.ADVECTION, 3, problem="adv_sine", ax=0.7, ay=-0.2)
    b = dg.Solver(mesh, dg.ADVECTION, 3, problem="adv_sine")
    b.set_velocity_field(0.7, -0.2, None)
    for s in (a, b):
        s.init_conditions()
        s.step(10, 0, 0.0)
    assert np.array_equal(a.get_state(), b.get_state())


def test_rotating_problems_set_their_rotation(dglib):
    dg = dglib
    mesh = dg.Mesh.square(4, 4, box=(-1, 1, -1, 1))
    for pb, w in (("adv_rotatinghill", 2 * 3.14159265358979323), ("adv_spin", 2 * 3.14159)):
        s = dg.Solver(mesh, dg.ADVECTION, 1, problem=pb)
        ax, ay, grad, _ = s.velocity_field()
        assert ax == 0 and ay == 0 and list(grad) == [0, -w, w, 0]
