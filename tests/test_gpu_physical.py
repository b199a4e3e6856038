"""The Euler positivity test's single-precision filter on the GPU: it may
only ever accept a state the FP64 test accepts (so every flatten decision
of the kernels is the FP64 test's), and it settles ordinary states by
itself."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def states(rho, u, v, p, gamma=1.4):
    E = p / (gamma - 1) + 0.5 * rho * (u * u + v * v)
    return np.stack([rho, rho * u, rho * v, E], axis=1)


def test_filter_never_accepts_what_fp64_rejects(dglib):
    dg = dglib
    rng = np.random.default_rng(11)
    n = 400000
    rho = 10.0 ** rng.uniform(-12, 12, n)
    u, v = rng.standard_normal(n) * 10.0 ** rng.uniform(-3, 3, n), rng.standard_normal(n)
    kin = 0.5 * rho * (u * u + v * v)
    # pressures hugging p = 0 from both sides, relative to the kinetic energy
    p = kin * rng.choice([-1.0, 1.0], n) * 10.0 ** rng.uniform(-18, 0, n)
    U = [states(rho, u, v, p)]
    # E perturbed by a few ulp around 2 rho E = |m|^2 exactly
    m = np.stack([rho * u, rho * v], axis=1)
    E0 = (m ** 2).sum(axis=1) / (2 * rho)
    for k in range(-4, 5):
        U.append(np.column_stack([rho, m, E0 + k * np.spacing(E0)]))
    # signs, zeros, extremes, NaN and infinities in every slot
    special = np.array([0.0, -0.0, 1e-320, -1e-320, 1e-310, 1e-40, 1e-38, 3e38, 1e39, 1e300,
                        -1e300, np.inf, -np.inf, np.nan, 1.0, -1.0, 2.5])
    g = np.array(np.meshgrid(special, special, special, special)).reshape(4, -1).T
    U.append(g)
    U = np.concatenate(U)
    fast, exact = dg.probe_physical(U)
    assert not np.any(fast & ~exact)


def test_filter_settles_ordinary_states(dglib):
    dg = dglib
    rng = np.random.default_rng(12)
    n = 200000
    rho = 10.0 ** rng.uniform(-3, 3, n)
    u, v = rng.uniform(-20, 20, n), rng.uniform(-20, 20, n)
    kin = 0.5 * rho * (u * u + v * v)
    p = np.maximum(kin, rho) * 10.0 ** rng.uniform(-3, 1, n)
    fast, exact = dg.probe_physical(states(rho, u, v, p))
    assert exact.all() and fast.all()
    fast, exact = dg.probe_physical(states(rho, u, v, -p))
    assert not exact.any() and not fast.any()
    # gas at rest along one axis or both (an exact zero momentum component,
    # as in the uniform quadrants of a Riemann problem) is settled too
    zero = np.zeros(n)
    for uu, vv in ((zero, v), (u, zero), (zero, zero)):
        fast, exact = dg.probe_physical(states(rho, uu, vv, p))
        assert exact.all() and fast.all()


def test_sound_speed_sqrt_within_one_ulp(dglib):
    """The face kernel's square root against IEEE sqrt on the GPU, over the
    whole positive normal range and the special values (which take IEEE
    sqrt)."""
    dg = dglib
    rng = np.random.default_rng(13)
    x = 10.0 ** rng.uniform(-300, 300, 300000)
    x = np.concatenate([x, rng.uniform(0.5, 2.0, 100000), 2.0 ** np.arange(-1022, 1024, 1.0),
                        np.nextafter(2.0 ** np.arange(-1021, 1023, 1.0), 0),
                        [0.0, -0.0, 5e-324, 1e-310, np.inf, np.nan, -1.0, 1.4, 2.0, 4.0]])
    r, q = dg.probe_sqrt(x)
    ok = np.isfinite(q) & (q > 0)
    ulp = np.abs(r[ok] - q[ok]) / np.spacing(q[ok])
    assert ulp.max() <= 1.0
    assert np.array_equal(r[~ok], q[~ok], equal_nan=True)
    with np.errstate(invalid="ignore"):
        assert np.array_equal(q, np.sqrt(x), equal_nan=True)
