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
