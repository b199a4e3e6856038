"""GPU parity: the sm_103a kernels through the C ABI against (a) the golden
vectors of the reference's own kernels, with the reference's basis
tabulation loaded via dg_solver_set_tables, and (b) the C oracle with the
exact basis.  Tolerances (norm-wise per variable block, as the task states):
right-hand side 1e-12, state after N steps 1e-10."""
import numpy as np
import pytest

from conftest import (PB_PULSE, golden_names, load_golden, pulse_series, ref_tables, relerr,
                      split_tables)

pytestmark = pytest.mark.gpu

RHS_TOL = 1e-12
STATE_TOL = 1e-10


def params_from(dg, d):
    prm = d["prm"]
    P = dg.Params()
    dg.load_library().dg_params_default(__import__("ctypes").byref(P))
    P.gamma, P.ax, P.ay, P.mu, P.eps, P.gravity = prm[1], prm[2], prm[3], prm[4], prm[5], prm[6]
    P.cfl = prm[7]
    P.problem = int(d["problem"])
    for i in range(8):
        P.prm[i] = prm[8 + i]
    return P


def solver_for(dg, d, ref_tab=True, limiter=0):
    mesh = dg.Mesh.from_arrays(d["V"], d["es"], d["sxy"], d["se"])
    P = params_from(dg, d)
    P.limiter = limiter
    s = dg.Solver(mesh, int(d["eq"]), int(d["p"]), params=P)
    if int(d["problem"]) == PB_PULSE:
        s.set_inflow_series(*pulse_series(d))
    if ref_tab:
        s.set_tables(*split_tables(ref_tables(int(d["p"])), int(d["p"])))
    return s


@pytest.mark.parametrize("name", golden_names("rhs_"))
def test_rhs_matches_reference(dglib, name):
    d = load_golden(name)
    s = solver_for(dglib, d)
    r = s.eval_rhs(d["C"].reshape(s.shape), float(d["prm"][0]))
    assert relerr(r, d["out"], s.N) <= RHS_TOL


@pytest.mark.parametrize("name", golden_names("rhs_"))
def test_rhs_exact_basis_matches_oracle(dglib, oracle_mod, name):
    d = load_golden(name)
    s = solver_for(dglib, d, ref_tab=False)
    o = oracle_mod.Oracle(int(d["eq"]), int(d["p"]), d["V"], d["es"], d["sxy"], d["se"], d["prm"],
                          int(d["problem"]))
    if int(d["problem"]) == PB_PULSE:
        o.set_series(*pulse_series(d))
    t = float(d["prm"][0])
    assert relerr(s.eval_rhs(d["C"].reshape(s.shape), t), o.rhs(d["C"], t), s.N) <= RHS_TOL


def _euler_tensor_goldens():
    out = []
    for name in golden_names("rhs_euler"):
        p = int(load_golden(name)["p"])
        if 1 <= p <= 4:
            out.append(name)
    return out


@pytest.mark.parametrize("tensor", [True, False], ids=["tensor", "fp64"])
@pytest.mark.parametrize("name", _euler_tensor_goldens())
def test_euler_rhs_both_element_paths_match_reference(dglib, name, tensor):
    """The element stage the bench times (basis contractions on the tensor
    cores, k_element_oz, with its start-of-run traces k_trace_oz) and the
    FP64-FMA one, each through dg_rhs, against the reference kernels'
    right-hand side with the reference tabulation: 1e-12 norm-wise."""
    d = load_golden(name)
    s = solver_for(dglib, d)
    s.tensor_contractions = tensor
    assert s.tensor_contractions == tensor
    r = s.eval_rhs(d["C"].reshape(s.shape), float(d["prm"][0]))
    assert relerr(r, d["out"], s.N) <= RHS_TOL


@pytest.mark.parametrize("name", golden_names("init_"))
def test_projection_matches_reference(dglib, name):
    d = load_golden(name)
    s = solver_for(dglib, d)
    s.init_conditions()
    assert relerr(s.get_state(), d["out"], s.N) <= RHS_TOL


@pytest.mark.parametrize("name", golden_names("limit_"))
def test_limiter_matches_reference(dglib, name):
    d = load_golden(name)
    s = solver_for(dglib, d, limiter=1)
    s.set_state(d["C"])
    s.limit_c()
    assert relerr(s.get_state(), d["out"], s.N) <= RHS_TOL


@pytest.mark.parametrize("name", golden_names("rk"))
def test_reference_rk_loops(dglib, name):
    d = load_golden(name)
    s = solver_for(dglib, d, limiter=int(d["hdr"][6]))
    s.set_state(d["C"])
    scheme = dglib.RK4 if int(d["hdr"][8]) == 4 else dglib.RK2
    t = s.step(int(d["hdr"][5]), scheme, 0.0)
    assert abs(t - d["out"][-1]) <= 1e-12 * abs(d["out"][-1])
    assert relerr(s.get_state(), d["out"][:-1], s.N) <= STATE_TOL


@pytest.mark.parametrize("name", golden_names("l2err_"))
def test_l2_error_matches_reference(dglib, name):
    d = load_golden(name)
    s = solver_for(dglib, d)
    s.set_state(d["C"])
    err = s.eval_error_L2(float(d["prm"][0]))
    np.testing.assert_allclose(err ** 2, d["out"], rtol=1e-12)


@pytest.mark.parametrize("name", golden_names("cfl_"))
def test_cfl_matches_reference(dglib, name):
    d = load_golden(name)
    s = solver_for(dglib, d)
    s.set_state(d["C"])
    dt, lam, dmin = s.cfl()
    np.testing.assert_allclose(lam, d["out"][:-1].max(), rtol=1e-14)
    np.testing.assert_allclose(dmin, d["out"][-1], rtol=1e-14)
    p = int(d["p"])
    np.testing.assert_allclose(dt, d["prm"][7] * dmin / lam / (2 * p + 1), rtol=1e-14)
