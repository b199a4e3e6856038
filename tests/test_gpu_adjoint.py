"""Discrete adjoint of the shallow-water RK-DG model: hand-derived
tangent-linear and adjoint operators, checked by dot-product tests and by
central finite differences (the reference has no derivatives)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

HUMP = (1.0, 0.1, 0.1, 0.45, 0.55)


def sw_solver(dg, n=10, p=2, seed=4):
    mesh = dg.Mesh.square(n, n, jitter=0.1, seed=seed, bc=(-1, -1, -1, -1))
    s = dg.Solver(mesh, dg.SHALLOW_WATER, p, problem="sw_hump", prm=HUMP, gravity=9.81, cfl=0.3)
    s.bathymetry_project("sine", (0.1, 1.0, 1.0))
    s.init_conditions()
    return s


def rnd_state(s, rng, scale=0.01):
    """The projected hump with small random higher modes and momenta; the
    water height stays well above zero everywhere, so the forward operator
    never takes its positivity fallback (which the derivatives exclude)."""
    c = s.get_state().copy()
    c[:, 1:, :] += scale * rng.standard_normal(c[:, 1:, :].shape)
    c[1:, 0, :] += scale * rng.standard_normal(c[1:, 0, :].shape)
    s.set_state(c)
    assert s.eval_u(0).min() > 0.5
    return c


def test_operator_dot_product(dglib):
    dg = dglib
    rng = np.random.default_rng(1)
    s = sw_solver(dg)
    c = rnd_state(s, rng)
    du = rng.standard_normal(s.shape)
    db = rng.standard_normal((s.n_p, s.K))
    lbar = rng.standard_normal(s.shape)
    dl = s.rhs_tl(c, du, db)
    cb, bb = s.rhs_adjoint(c, lbar)
    lhs = np.sum(lbar * dl)
    rhs = np.sum(cb * du) + np.sum(bb * db)
    assert abs(lhs - rhs) <= 1e-12 * max(abs(lhs), abs(rhs))


def test_operator_tangent_matches_central_differences(dglib):
    dg = dglib
    rng = np.random.default_rng(2)
    s = sw_solver(dg)
    c = rnd_state(s, rng)
    b0 = s.get_bathymetry()
    du = rng.standard_normal(s.shape) * 0.1
    db = rng.standard_normal((s.n_p, s.K)) * 0.1
    dl = s.rhs_tl(c, du, db)
    eps = 1e-6
    s.set_bathymetry(b0 + eps * db)
    lp = s.eval_rhs(c + eps * du, 0.0)
    s.set_bathymetry(b0 - eps * db)
    lm = s.eval_rhs(c - eps * du, 0.0)
    s.set_bathymetry(b0)
    fd = (lp - lm) / (2 * eps)
    assert np.linalg.norm(fd - dl) <= 1e-7 * np.linalg.norm(dl)


def model(dg, n=10, p=2, nrec=8, seed=5):
    s = sw_solver(dg, n, p)
    rng = np.random.default_rng(seed)
    rx, ry = rng.uniform(0.05, 0.95, nrec), rng.uniform(0.05, 0.95, nrec)
    return s, dg.Adjoint(s, rx, ry)


def test_model_dot_product(dglib):
    dg = dglib
    s, adj = model(dg)
    dt = 0.2 * s.cfl()[0]
    samples = adj.forward(60, dt, 10, 20)
    assert samples.shape == (6, 8)
    rng = np.random.default_rng(3)
    sbar = rng.standard_normal(samples.shape)
    du0 = rng.standard_normal(s.shape) * 0.01
    db = rng.standard_normal((s.n_p, s.K)) * 0.01
    gu, gb = adj.backward(sbar)
    ds = adj.tangent(du0, db)
    lhs = np.sum(sbar * ds)
    rhs = np.sum(gu * du0) + np.sum(gb * db)
    assert abs(lhs - rhs) <= 1e-10 * max(abs(lhs), abs(rhs))


def test_stored_stages_and_checkpoints_give_the_same_bits(dglib):
    """The reverse sweep from stage states kept in device memory and from
    recomputed checkpoint segments: identical gradients, and the solver is
    left at the forward run's final state either way."""
    dg = dglib
    s, adj = model(dg)
    dt = 0.2 * s.cfl()[0]
    c0, b0 = s.get_state(), s.get_bathymetry()
    sbar = np.random.default_rng(9).standard_normal((6, 8))
    out = []
    for keep in (True, False):
        s.set_state(c0)
        s.set_bathymetry(b0)
        adj.set_storage(keep)
        smp = adj.forward(60, dt, 10, 20)
        assert adj.stored == keep
        c_end = s.get_state()
        gu, gb = adj.backward(sbar)
        assert np.array_equal(s.get_state(), c_end)
        out.append((smp, gu, gb, c_end))
    for a, b in zip(out[0], out[1]):
        assert np.array_equal(a, b)


def test_misfit_gradient_matches_central_differences_16_directions(dglib):
    """J = sum (h - h_obs)^2 over receivers and sample times, h_obs from a
    run with the bed perturbed by 0.02 N(0,1) per mode; the adjoint gradient
    against central differences along 16 seeded directions (1e-6).

    The model is only piecewise smooth (|u.n| and the max of the two wave
    speeds in the Rusanov flux), and the derivatives follow the branch the
    forward run took.  A central difference whose step straddles a switch
    of branch is not a derivative of either branch, so each direction uses
    the first step of 1e-6, 5e-7, ... at which it agrees with the next
    smaller step to 1e-7: no branch switch lies inside it."""
    dg = dglib
    s, adj = model(dg, n=8, p=2, nrec=16)
    dt = 0.3 * s.cfl()[0]
    c0 = s.get_state()
    b0 = s.get_bathymetry()
    rng = np.random.default_rng(11)
    s.set_bathymetry(b0 + 0.02 * rng.standard_normal(b0.shape))
    obs = adj.forward(40, dt, 4, 10)
    s.set_bathymetry(b0)

    def J(h0, b):
        c = c0.copy()
        c[0] = h0
        s.set_state(c)
        s.set_bathymetry(b)
        smp = adj.forward(40, dt, 4, 10)
        return np.sum((smp - obs) ** 2), smp

    J0, smp = J(c0[0], b0)
    gu, gb = adj.backward(2 * (smp - obs))
    worst = 0.0
    for k in range(16):
        dh = rng.standard_normal(c0[0].shape)
        dbd = rng.standard_normal(b0.shape)
        dh /= np.linalg.norm(dh)
        dbd /= np.linalg.norm(dbd)

        def fd_at(eps):
            return (J(c0[0] + eps * dh, b0 + eps * dbd)[0]
                    - J(c0[0] - eps * dh, b0 - eps * dbd)[0]) / (2 * eps)

        eps = 1e-6
        fd, fd_half = fd_at(eps), fd_at(eps / 2)
        for _ in range(6):
            if abs(fd - fd_half) <= 1e-7 * abs(fd_half):
                break
            eps /= 2
            fd, fd_half = fd_half, fd_at(eps / 2)
        ad = np.sum(gu[0] * dh) + np.sum(gb * dbd)
        worst = max(worst, abs(fd - ad) / max(abs(ad), 1e-300))
    assert worst <= 1e-6, worst


def test_torch_autograd_function(dglib):
    torch = pytest.importorskip("torch")
    from dgcuda_gb300.torch_binding import DGShallowWater
    dg = dglib
    s, adj = model(dg, n=8, p=2, nrec=4)
    dt = 0.3 * s.cfl()[0]
    c0 = s.get_state()
    h0 = torch.tensor(c0[0], dtype=torch.float64, requires_grad=True)
    b = torch.tensor(s.get_bathymetry(), dtype=torch.float64, requires_grad=True)
    out = DGShallowWater.apply(h0, b, adj, 20, dt, 5, 10)
    loss = (out ** 2).sum()
    loss.backward()
    gu, gb = adj.backward(2 * out.detach().numpy())
    assert np.allclose(h0.grad.numpy(), gu[0], rtol=0, atol=0)
    assert np.allclose(b.grad.numpy(), gb, rtol=0, atol=0)
