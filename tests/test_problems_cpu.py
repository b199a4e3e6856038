"""Initial data of the added Euler problems in the oracle (no GPU):
uniform Mach flows, and the double Mach reflection's 60-degree shock."""
import numpy as np


def means(dg, oracle_mod, pb, box, nx, ny, prm=()):
    mesh = dg.Mesh.square(nx, ny, box=box, jitter=0.0, seed=1, bc=(-3, -2, -1, -3))
    o = oracle_mod.Oracle.from_mesh(mesh, dg.EULER, 1, oracle_mod.prm_vec(extra=prm), dg.PROBLEMS[pb])
    V = mesh.arrays()[0]
    xc, yc = (V[0] + V[2] + V[4]) / 3, (V[1] + V[3] + V[5]) / 3
    return xc, yc, o.init()[:, 0, :] * np.sqrt(2.0)   # cell means


def test_uniform_mach_states(dglib, oracle_mod):
    dg = dglib
    for pb, mach in (("euler_cylinder", 0.38), ("euler_lshock", 2.0)):
        _, _, m = means(dg, oracle_mod, pb, (1, 2, 1, 2), 4, 4)
        rho, ru, rv, E = m.mean(axis=1)
        assert abs(rho - 1.4) < 1e-14 and abs(ru / rho - mach) < 1e-14 and abs(rv) < 1e-14
        p = 0.4 * (E - 0.5 * ru * ru / rho)
        assert abs(p - 1.0) < 1e-13
    _, _, m = means(dg, oracle_mod, "euler_lshock", (1, 2, 1, 2), 4, 4, prm=(3.0,))
    assert abs(m[1].mean() / m[0].mean() - 3.0) < 1e-14


def test_double_mach_initial_shock(dglib, oracle_mod):
    dg = dglib
    xc, yc, m = means(dg, oracle_mod, "euler_doublemach", (0, 4, 0, 1), 64, 16)
    x0 = 1.0 / 6.0
    behind = (xc < x0) | (xc - x0 < yc / np.sqrt(3.0) - 0.1)
    ahead = (xc > x0) & (xc - x0 > yc / np.sqrt(3.0) + 0.1)
    assert behind.sum() > 10 and ahead.sum() > 100
    assert np.allclose(m[0][behind], 8.0, rtol=0, atol=1e-12)
    assert np.allclose(m[1][behind] / 8.0, 8.25 * np.cos(np.pi / 6), rtol=0, atol=1e-12)
    assert np.allclose(m[0][ahead], 1.4, rtol=0, atol=1e-12)
    assert np.allclose(m[1][ahead], 0.0, rtol=0, atol=1e-12)


def test_airfoil_and_pulse_initial_states(dglib, oracle_mod):
    dg = dglib
    _, _, m = means(dg, oracle_mod, "euler_airfoil", (0, 1, 0, 1), 4, 4)
    rho, ru, rv, E = m.mean(axis=1)
    a = np.deg2rad(5.0)
    assert abs(rho - 1.4) < 1e-14
    assert abs(ru / rho - 0.98 * np.cos(a)) < 1e-14 and abs(rv / rho - 0.98 * np.sin(a)) < 1e-14
    _, _, m = means(dg, oracle_mod, "euler_pulse", (0, 4, 0, 1), 8, 2)
    assert np.allclose(m[0], 1.4, rtol=0, atol=1e-14) and np.allclose(m[1:3], 0, atol=1e-15)
    assert np.allclose(0.4 * m[3], 1.0, rtol=0, atol=1e-14)


def test_advection_hills(dglib, oracle_mod):
    """Cell means of the rotating hill (centre (0.2, 0)), the spin hill
    (centre (0.5, 0.5)) and the square hill's box."""
    dg = dglib
    for pb, box, centre, peak in (("adv_rotatinghill", (-1, 1, -1, 1), (0.2, 0.0), 5.0),
                                  ("adv_spin", (0, 1, 0, 1), (0.5, 0.5), 1.0)):
        mesh = dg.Mesh.square(40, 40, box=box, jitter=0.0, seed=1, bc=(-3, -3, -3, -3))
        o = oracle_mod.Oracle.from_mesh(mesh, dg.ADVECTION, 2, oracle_mod.prm_vec(),
                                        dg.PROBLEMS[pb])
        V = mesh.arrays()[0]
        xc, yc = (V[0] + V[2] + V[4]) / 3, (V[1] + V[3] + V[5]) / 3
        c = o.init()[0, 0, :] * np.sqrt(2.0)
        k = int(np.argmax(c))
        assert np.hypot(xc[k] - centre[0], yc[k] - centre[1]) < 0.06
        assert 0.8 * peak < c[k] <= peak
    mesh = dg.Mesh.square(20, 20, box=(-1, 1, -1, 1), jitter=0.0, seed=1, bc=(-3, -2, -2, -2))
    o = oracle_mod.Oracle.from_mesh(mesh, dg.ADVECTION, 0, oracle_mod.prm_vec(),
                                    dg.PROBLEMS["adv_squarehill"])
    V = mesh.arrays()[0]
    xc, yc = (V[0] + V[2] + V[4]) / 3, (V[1] + V[3] + V[5]) / 3
    c = o.init()[0, 0, :] * np.sqrt(2.0)
    inside = (xc > -0.75) & (xc < -0.25) & (yc > -0.45) & (yc < 0.05)
    outside = (xc < -0.85) | (xc > -0.15) | (yc < -0.55) | (yc > 0.15)
    assert np.all(c[outside] == 0) and np.all(np.abs(c[inside] - 1) < 1e-13)


def test_params_for_problem(dglib):
    """Each reference problem file's settings (limiter, time integrator,
    Mach number, angle, velocity, g)."""
    dg = dglib
    want = {
        "adv_linear": dict(limiter=1, ax=1.0, ay=1.0, scheme=dg.RK4),
        "adv_squarehill": dict(limiter=1, ax=1.0, ay=0.0, scheme=dg.RK4),
        "adv_rotatinghill": dict(limiter=0, ax=0.0, ay=0.0, scheme=dg.RK4),
        "adv_spin": dict(limiter=0, scheme=dg.RK2),
        "euler_supersonic": dict(limiter=1, scheme=dg.RK4),
        "euler_doublemach": dict(limiter=1, scheme=dg.RK2),
        "euler_airfoil": dict(limiter=1, prm0=0.98, prm1=5.0, scheme=dg.RK4),
        "euler_cylinder": dict(limiter=0, prm0=0.38, scheme=dg.RK4),
        "euler_lshock": dict(limiter=0, prm0=2.0, scheme=dg.RK4),
        "sw_test": dict(gravity=9.8, scheme=dg.RK4),
        "maxwell_cmirror": dict(limiter=0, mu=1.0, eps=1.0, scheme=dg.RK4),
    }
    for name, w in want.items():
        P, sc = dg.params_for_problem(name)
        assert P.problem == dg.PROBLEMS[name] and sc == w.pop("scheme")
        for k, v in w.items():
            got = P.prm[int(k[3])] if k.startswith("prm") else getattr(P, k)
            assert got == v, (name, k, got, v)
    import pytest
    with pytest.raises(dg.DGError):
        dg.params_for_problem(99)
