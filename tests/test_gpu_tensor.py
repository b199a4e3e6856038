"""The fused element stage with its basis contractions on the tensor cores
(exact integer slices, Euler p = 1..4) against the FP64-FMA kernel and the
oracle: same steps, results equal to FP64 rounding."""
import numpy as np
import pytest

from conftest import ref_tables, relerr, split_tables

pytestmark = pytest.mark.gpu
VTX = (5.0, 5.0, 5.0, 1.0, 1.0, 10.0)


def vortex(dg, p, n=24):
    mesh = dg.Mesh.square(n, n, box=(0, 10, 0, 10), jitter=0.15, seed=2)
    s = dg.Solver(mesh, dg.EULER, p, problem="euler_vortex", prm=VTX, cfl=0.2)
    s.init_conditions()
    return mesh, s


@pytest.mark.parametrize("p", [1, 2, 3, 4])
def test_tensor_path_matches_fp64_path(dglib, p):
    dg = dglib
    _, a = vortex(dg, p)
    _, b = vortex(dg, p)
    assert a.tensor_contractions == (p >= 2)  # default: on from p = 2
    a.tensor_contractions = True
    b.tensor_contractions = False
    assert not b.tensor_contractions
    ta = a.step(20, dg.SSP_RK3, 0.0)
    tb = b.step(20, dg.SSP_RK3, 0.0)
    assert abs(ta - tb) <= 1e-14 * tb
    assert relerr(a.get_state(), b.get_state(), 4) <= 1e-12


@pytest.mark.parametrize("p", [2, 3, 4])
def test_tensor_path_matches_oracle(dglib, oracle_mod, p):
    dg = dglib
    mesh, s = vortex(dg, p, n=12)
    c0 = s.get_state()
    o = oracle_mod.Oracle.from_mesh(mesh, dg.EULER, p, oracle_mod.prm_vec(extra=VTX),
                                    dg.PROBLEMS["euler_vortex"])
    t = s.step(10, dg.SSP_RK3, 0.0)
    c, to, _ = o.step(c0, 10, 0, 0, 0.2)
    assert abs(t - to) <= 1e-12 * to
    assert relerr(s.get_state(), c, 4) <= 1e-10


def test_tensor_path_limiter_and_transmissive(dglib):
    dg = dglib
    mesh = dg.Mesh.square(48, 48, jitter=0.1, seed=3, bc=(-4, -4, -4, -4))
    kw = dict(problem="euler_riemann4", limiter=1, cfl=0.2)
    a = dg.Solver(mesh, dg.EULER, 3, **kw)
    b = dg.Solver(mesh, dg.EULER, 3, **kw)
    b.tensor_contractions = False
    for s in (a, b):
        s.init_conditions()
    ta, tb = a.step(10, dg.SSP_RK3, 0.0), b.step(10, dg.SSP_RK3, 0.0)
    assert abs(ta - tb) <= 1e-13 * tb
    assert relerr(a.get_state(), b.get_state(), 4) <= 1e-10


def test_tensor_path_unsupported_elsewhere(dglib):
    dg = dglib
    mesh = dg.Mesh.square(4, 4, jitter=0.1, seed=1)
    s = dg.Solver(mesh, dg.ADVECTION, 2, problem="adv_sine")
    assert not s.tensor_contractions
    with pytest.raises(dg.DGError):
        s.tensor_contractions = True
    s.tensor_contractions = False


@pytest.mark.parametrize("limiter", [0, 1])
def test_split_runs_equal_one_run(dglib, limiter):
    """dg_step(10) twice gives the bits of dg_step(20): the second call
    continues from the traces the first one left."""
    dg = dglib
    mesh = dg.Mesh.square(24, 24, jitter=0.1, seed=3, bc=(-4, -4, -4, -4))
    kw = dict(problem="euler_riemann4", limiter=limiter, cfl=0.2)
    a, b = dg.Solver(mesh, dg.EULER, 3, **kw), dg.Solver(mesh, dg.EULER, 3, **kw)
    for s in (a, b):
        s.init_conditions()
    t = a.step(10, dg.SSP_RK3, 0.0)
    ta = a.step(10, dg.SSP_RK3, t)
    tb = b.step(20, dg.SSP_RK3, 0.0)
    assert ta == tb and np.array_equal(a.get_state(), b.get_state())


def test_restart_from_state_equals_one_run(dglib):
    """A fresh solver given the state after 10 steps continues bit for bit:
    the start-of-run traces use the same tensor contraction as the stage."""
    dg = dglib
    _, a = vortex(dg, 3)
    _, b = vortex(dg, 3)
    t = a.step(10, dg.SSP_RK3, 0.0)
    c = a.get_state()
    ta = a.step(10, dg.SSP_RK3, t)
    b.set_state(c)
    tb = b.step(10, dg.SSP_RK3, t)
    assert ta == tb and np.array_equal(a.get_state(), b.get_state())


def test_flux_reciprocal_within_one_ulp(dglib):
    """The flux kernels' Newton-Raphson reciprocal against IEEE division on
    the GPU, over 12 decades and both signs."""
    dg = dglib
    rng = np.random.default_rng(7)
    x = 10.0 ** rng.uniform(-6, 6, 200000) * rng.choice([-1.0, 1.0], 200000)
    x = np.concatenate([x, [1.0, 2.0, 0.5, 3.0, 1.4, 1e-3, 7.0e5]])
    r, q = dg.probe_reciprocal(x)
    ulp = np.abs(r - q) / np.spacing(np.abs(q))
    assert ulp.max() <= 1.0
    assert np.array_equal(q, 1.0 / x)


def _oracle_run(dg, oracle_mod, mesh, p, prm, pb, c0, nsteps, lim, cfl, tables=None):
    o = oracle_mod.Oracle.from_mesh(mesh, dg.EULER, p, oracle_mod.prm_vec(extra=prm),
                                    dg.PROBLEMS[pb])
    if tables is not None:
        o.set_tables(tables)
    return o.step(c0, nsteps, 0, lim, cfl)


def test_tensor_path_limiter_matches_oracle(dglib, oracle_mod):
    """Four-quadrant Riemann problem, p = 3, limiter on, transmissive sides."""
    dg = dglib
    mesh = dg.Mesh.square(16, 16, jitter=0.1, seed=3, bc=(-4, -4, -4, -4))
    s = dg.Solver(mesh, dg.EULER, 3, problem="euler_riemann4", limiter=1, cfl=0.2)
    assert s.tensor_contractions
    s.init_conditions()
    c0 = s.get_state()
    t = s.step(8, dg.SSP_RK3, 0.0)
    c, to, n = _oracle_run(dg, oracle_mod, mesh, 3, (), "euler_riemann4", c0, 8, 1, 0.2)
    assert n == 8 and abs(t - to) <= 1e-12 * to
    assert relerr(s.get_state(), c, 4) <= 1e-10


def test_tensor_path_reflecting_walls_and_reference_tables(dglib, oracle_mod):
    """Slip walls (reflected ghost states) and the reference's own basis
    tabulation loaded through dg_solver_set_tables: the tensor tables are
    rebuilt from it, and the run matches the oracle with the same tables."""
    dg = dglib
    mesh = dg.Mesh.square(12, 12, box=(0, 10, 0, 10), jitter=0.15, seed=6, bc=(-1, -1, -1, -1))
    s = dg.Solver(mesh, dg.EULER, 3, problem="euler_vortex", prm=VTX, cfl=0.2)
    tab = ref_tables(3)
    s.set_tables(*split_tables(tab, 3))
    assert s.tensor_contractions
    s.init_conditions()
    c0 = s.get_state()
    t = s.step(10, dg.SSP_RK3, 0.0)
    c, to, _ = _oracle_run(dg, oracle_mod, mesh, 3, VTX, "euler_vortex", c0, 10, 0, 0.2, tab)
    assert abs(t - to) <= 1e-12 * to
    assert relerr(s.get_state(), c, 4) <= 1e-10


def test_full_size_conservation_determinism_and_fp64_agreement(dglib):
    """The bench problem at its full size (1024 x 1024 squares, 2,097,152
    triangles, p = 3, limiter on) with periodic sides, so that the element
    means' total is conserved: 3 steps on the tensor path conserve every
    variable to rounding, repeat bit for bit, and agree with the FP64
    kernel to rounding."""
    dg = dglib
    mesh = dg.Mesh.square(1024, 1024, jitter=0.1, seed=3)
    V = mesh.arrays()[0]
    J = (V[2] - V[0]) * (V[5] - V[1]) - (V[4] - V[0]) * (V[3] - V[1])
    outs = []
    for tensor in (True, True, False):
        s = dg.Solver(mesh, dg.EULER, 3, problem="euler_riemann4", limiter=1, cfl=0.2)
        s.tensor_contractions = tensor
        s.init_conditions()
        m0 = (s.get_state()[:, 0, :] * J).sum(axis=1)
        s.step(3, dg.SSP_RK3, 0.0)
        c = s.get_state()
        m1 = (c[:, 0, :] * J).sum(axis=1)
        assert np.all(np.abs(m1 - m0) <= 1e-12 * np.abs(m0).max())
        outs.append(c)
        s.close()
    assert np.array_equal(outs[0], outs[1])
    assert relerr(outs[0], outs[2], 4) <= 1e-12


def test_state_round_trip_through_the_host_is_invisible(dglib):
    """Reading the state out and handing it back unchanged between steps
    (what a caller that checkpoints or plots every step does) gives the bits
    of an uninterrupted run; handing back a changed state restarts."""
    dg = dglib
    mesh = dg.Mesh.square(24, 24, jitter=0.1, seed=3, bc=(-4, -4, -4, -4))
    kw = dict(problem="euler_riemann4", limiter=1, cfl=0.2)
    a, b, c = (dg.Solver(mesh, dg.EULER, 3, **kw) for _ in range(3))
    for s in (a, b, c):
        s.init_conditions()
    t = 0.0
    for _ in range(6):
        t = a.step(2, dg.SSP_RK3, t)
        a.set_state(a.get_state())
    tb = b.step(12, dg.SSP_RK3, 0.0)
    assert t == tb and np.array_equal(a.get_state(), b.get_state())
    # a changed state: same as a fresh solver started from it
    x = b.get_state()
    x[0, 1, 5] += 1e-6
    b.set_state(x)
    c.set_state(x)
    assert b.step(3, dg.SSP_RK3, tb) == c.step(3, dg.SSP_RK3, tb)
    assert np.array_equal(b.get_state(), c.get_state())


@pytest.mark.parametrize("p", [1, 2, 4])
def test_fused_limiter_matches_oracle(dglib, oracle_mod, p):
    """The limiter in the tensor-core element stage's epilogue at the orders
    the full-size test does not run on small meshes: p = 1 (no free shared-
    memory slot: the limiter rereads modes 1 and 2 from the output), p = 2,
    p = 4; four-quadrant Riemann problem, transmissive sides, 8 steps."""
    dg = dglib
    mesh = dg.Mesh.square(20, 20, jitter=0.1, seed=3, bc=(-4, -4, -4, -4))
    s = dg.Solver(mesh, dg.EULER, p, problem="euler_riemann4", limiter=1, cfl=0.2)
    s.tensor_contractions = True
    s.init_conditions()
    c0 = s.get_state()
    t = s.step(8, dg.SSP_RK3, 0.0)
    c, to, n = _oracle_run(dg, oracle_mod, mesh, p, (), "euler_riemann4", c0, 8, 1, 0.2)
    assert n == 8 and abs(t - to) <= 1e-12 * to
    assert relerr(s.get_state(), c, 4) <= 1e-10


@pytest.mark.parametrize("n", [1, 3])
def test_tensor_path_on_tiny_meshes(dglib, oracle_mod, n):
    """K = 2 and K = 18 (one partial tile of the 64-element blocks, lanes
    past the last element), slip walls, p = 3, limiter on: against the
    oracle."""
    dg = dglib
    mesh = dg.Mesh.square(n, n, jitter=0.0, seed=1, bc=(-1, -1, -1, -1))
    assert mesh.K == 2 * n * n
    s = dg.Solver(mesh, dg.EULER, 3, problem="euler_riemann4", limiter=1, cfl=0.2)
    assert s.tensor_contractions
    s.init_conditions()
    c0 = s.get_state()
    t = s.step(5, dg.SSP_RK3, 0.0)
    c, to, nst = _oracle_run(dg, oracle_mod, mesh, 3, (), "euler_riemann4", c0, 5, 1, 0.2)
    assert nst == 5 and abs(t - to) <= 1e-12 * to
    assert relerr(s.get_state(), c, 4) <= 1e-10
    r = s.eval_rhs(s.get_state(), t)
    o = oracle_mod.Oracle.from_mesh(mesh, dg.EULER, 3, oracle_mod.prm_vec(gamma=1.4),
                                    dg.PROBLEMS["euler_riemann4"])
    assert relerr(r, o.rhs(s.get_state(), t), 4) <= 1e-12
