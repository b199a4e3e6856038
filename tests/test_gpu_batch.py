"""Batched ensembles (per stage one face launch for all members, one
element launch per (order, mesh-size) group), the shallow-water bed source,
and the autotuners."""
import numpy as np
import pytest

from conftest import relerr

pytestmark = pytest.mark.gpu


def test_batched_shallow_water_bitwise_equals_one_at_a_time(dglib):
    from dgcuda_gb300.ensemble import build_member, ensemble_specs
    dg = dglib
    specs = ensemble_specs(9, seed=7, tri_min=200, tri_max=20000)
    assert {sp["p"] for sp in specs} == {1, 2, 3}
    assert {sp["bed"] for sp in specs} == {"flat", "sine"}
    a = [build_member(sp) for sp in specs]
    b = [build_member(sp) for sp in specs]
    batch = dg.Batch(a)
    ta = batch.step(12)
    tb = [s.step(12, dg.SSP_RK3, 0.0) for s in b]
    assert list(ta) == tb
    for sa, sb in zip(a, b):
        assert np.array_equal(sa.get_state(), sb.get_state())
    # a second call continues from the members' states and times
    ta2 = batch.step(3, ta)
    tb2 = [s.step(3, dg.SSP_RK3, t) for s, t in zip(b, tb)]
    assert list(ta2) == tb2
    for sa, sb in zip(a, b):
        assert np.array_equal(sa.get_state(), sb.get_state())
    assert batch.launches() > 0


def test_batched_euler_with_limiter_bitwise(dglib):
    dg = dglib
    members, singles = [], []
    for n, p in ((12, 1), (20, 2), (9, 3), (16, 2)):
        for lst in (members, singles):
            m = dg.Mesh.square(n, n, jitter=0.1, seed=n, bc=(-4, -4, -4, -4))
            s = dg.Solver(m, dg.EULER, p, problem="euler_riemann4", limiter=1, cfl=0.2)
            s.init_conditions()
            lst.append(s)
    # the batched kernels contract in FP64: compare with solvers doing the same
    for s in singles:
        s.tensor_contractions = False
    dg.Batch(members).step(8)
    for a, b in zip(members, singles):
        b.step(8, dg.SSP_RK3, 0.0)
        assert np.array_equal(a.get_state(), b.get_state())


def test_bed_projection_reproduces_linear_bed(dglib):
    dg = dglib
    mesh = dg.Mesh.square(6, 6, jitter=0.1, seed=4, bc=(-1, -1, -1, -1))
    s = dg.Solver(mesh, dg.SHALLOW_WATER, 2)
    s.bathymetry_project("linear", (0.2, 0.3, -0.1))
    b = s.get_bathymetry()
    s.set_state(np.concatenate([b[None], np.zeros((2, s.n_p, s.K))]))
    uv = s.eval_u(0)
    V = mesh.arrays()[0]
    exact = np.stack([0.2 + 0.3 * V[2 * v] - 0.1 * V[2 * v + 1] for v in range(3)])
    assert np.abs(uv - exact).max() < 1e-14
    assert np.abs(b[3:]).max() < 1e-15


def test_bathymetry_source_matches_oracle(dglib, oracle_mod):
    dg = dglib
    mesh = dg.Mesh.square(12, 12, jitter=0.1, seed=3, bc=(-1, -1, -1, -1))
    hump = (1.0, 0.1, 0.1, 0.45, 0.55)
    s = dg.Solver(mesh, dg.SHALLOW_WATER, 2, problem="sw_hump", prm=hump, gravity=9.81, cfl=0.3)
    s.bathymetry_project("sine", (0.1, 1.0, 1.0))
    s.init_conditions()
    c0 = s.get_state()
    o = oracle_mod.Oracle.from_mesh(mesh, dg.SHALLOW_WATER, 2,
                                    oracle_mod.prm_vec(g=9.81, extra=hump),
                                    dg.PROBLEMS["sw_hump"])
    o.set_bathymetry(s.get_bathymetry())
    assert relerr(s.eval_rhs(c0, 0.0), o.rhs(c0, 0.0), 3) <= 1e-12
    t = s.step(10, dg.SSP_RK3, 0.0)
    c, to, _ = o.step(c0, 10, 0, 0, 0.3)
    assert abs(t - to) <= 1e-12 * to
    assert relerr(s.get_state(), c, 3) <= 1e-10


def test_lake_at_rest_over_linear_bed(dglib):
    """h + b = const and u = 0 over a linear bed is a discrete steady state."""
    dg = dglib
    mesh = dg.Mesh.square(10, 10, jitter=0.1, seed=4, bc=(-1, -1, -1, -1))
    s = dg.Solver(mesh, dg.SHALLOW_WATER, 2, gravity=9.81)
    s.bathymetry_project("linear", (0.2, 0.3, -0.1))
    c = np.zeros(s.shape)
    c[0] = -s.get_bathymetry()
    c[0, 0] += 2.0 / np.sqrt(2.0)
    r = s.eval_rhs(c, 0.0)
    assert np.abs(r).max() < 1e-11
    s.set_state(c)
    t = s.step(20, dg.SSP_RK3, 0.0)
    assert t > 0 and np.abs(s.get_state() - c).max() < 1e-12


def test_autotune_keeps_results(dglib):
    dg = dglib
    m = dg.Mesh.square(48, 48, box=(0, 10, 0, 10), jitter=0.15, seed=5)
    vtx = (5.0, 5.0, 5.0, 1.0, 1.0, 10.0)
    a = dg.Solver(m, dg.EULER, 2, problem="euler_vortex", prm=vtx, cfl=0.2)
    b = dg.Solver(m, dg.EULER, 2, problem="euler_vortex", prm=vtx, cfl=0.2)
    for s in (a, b):
        s.init_conditions()
    blk = a.autotune()
    assert blk in (64, 128, 256)
    a.step(5, dg.SSP_RK3, 0.0)
    b.step(5, dg.SSP_RK3, 0.0)
    assert np.array_equal(a.get_state(), b.get_state())


def test_batch_autotune_keeps_results(dglib):
    """Block sizes tuned per (order, mesh-size) group of the element stage:
    the results stay those of the untuned batch and of the members stepped
    one at a time."""
    from dgcuda_gb300.ensemble import build_member, ensemble_specs
    dg = dglib
    specs = ensemble_specs(8, seed=3, tri_min=2000, tri_max=40000)
    a = [build_member(sp) for sp in specs]
    b = [build_member(sp) for sp in specs]
    c = [build_member(sp) for sp in specs]
    assert {s.K >= 16384 for s in a} == {False, True}
    ba = dg.Batch(a)
    assert ba.autotune() in (64, 128, 256)
    shared, groups = ba.blocks()
    assert shared in (64, 128, 256) and all(g in (64, 128, 256) for g in groups)
    ba.step(4)
    dg.Batch(b).step(4)
    for s in c:
        s.step(4, dg.SSP_RK3, 0.0)
    for sa, sb, sc in zip(a, b, c):
        assert np.array_equal(sa.get_state(), sb.get_state())
        assert np.array_equal(sa.get_state(), sc.get_state())


def test_autotune_stage_choice_restores_state_and_matches_oracle(dglib, oracle_mod):
    """Euler p = 3 with the limiter: the tuner picks a block size and the
    element stage (threads per element 1: FP64, 2: tensor cores), restores
    the state, and the run it leaves matches the oracle."""
    dg = dglib
    m = dg.Mesh.square(64, 64, jitter=0.1, seed=3, bc=(-4, -4, -4, -4))
    s = dg.Solver(m, dg.EULER, 3, problem="euler_riemann4", limiter=1, cfl=0.2)
    s.init_conditions()
    c0 = s.get_state()
    blk, tpe = s.autotune_stage()
    assert blk in (64, 128, 256) and tpe in (1, 2)
    assert s.tensor_contractions == (tpe == 2)
    assert np.array_equal(s.get_state(), c0)
    t = s.step(5, dg.SSP_RK3, 0.0)
    o = oracle_mod.Oracle.from_mesh(m, dg.EULER, 3, oracle_mod.prm_vec(gamma=1.4),
                                    dg.PROBLEMS["euler_riemann4"])
    c, to, _ = o.step(c0, 5, 0, 1, 0.2)
    assert abs(t - to) <= 1e-12 * to
    assert relerr(s.get_state(), c, 4) <= 1e-10
