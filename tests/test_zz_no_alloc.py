"""dg_rhs_device_noalloc: the right-hand side for callers that may not
allocate device memory during the call (a host application that owns all
device memory and forbids allocation after set-up, or a latency-critical
loop where a cudaMalloc would synchronise the device).  Its working
memory is a static array inside the library; the test checks, through the C
ABI, that two calls in a row give dg_rhs's result within the right-hand-side
tolerance of the other parity tests (1e-12, norm-wise per variable), and that
a problem too big for the array is rejected.  The device buffers below are
allocated by the test, never by the entry point."""
import ctypes

import numpy as np
import pytest

from conftest import relerr

pytestmark = pytest.mark.gpu

RHS_TOL = 1e-12
DG_UNSUPPORTED = 8


def entry(dg):
    fn = dg.load_library().dg_rhs_device_noalloc
    fn.restype = ctypes.c_int
    fn.argtypes = [ctypes.c_void_p, ctypes.c_double, ctypes.c_void_p, ctypes.c_void_p]
    return fn


def perturbed(c, seed):
    rng = np.random.default_rng(seed)
    out = c.copy()
    out[:, 1:, :] += 0.01 * np.abs(c[:, :1, :]) * rng.standard_normal(out[:, 1:, :].shape)
    return out


def test_noalloc_rhs_matches_dg_rhs_twice(dglib):
    torch = pytest.importorskip("torch")
    dg = dglib
    fn = entry(dg)
    mesh = dg.Mesh.square(24, 24, box=(0, 10, 0, 10), jitter=0.15, seed=9)
    s = dg.Solver(mesh, dg.EULER, 3, problem="euler_vortex", prm=(5.0, 5.0, 5.0, 1.0, 1.0, 10.0))
    s.init_conditions()
    c0 = s.get_state()
    for call, seed in enumerate((1, 2)):
        c = perturbed(c0, seed)
        ref = s.eval_rhs(c, 0.25)
        dev_in = torch.from_numpy(c).cuda()
        dev_out = torch.full_like(dev_in, float("nan"))
        # the entry point works on the solver's own stream: the copy and the
        # NaN fill above must be finished before it starts
        torch.cuda.synchronize()
        rc = fn(s._h, 0.25, dev_in.data_ptr(), dev_out.data_ptr())
        assert rc == 0, dg.load_library().dg_last_error().decode()
        got = dev_out.cpu().numpy()
        assert np.isfinite(got).all(), "call %d left entries unwritten" % call
        assert relerr(got, ref, s.N) <= RHS_TOL, "call %d" % call


def test_noalloc_rejects_problem_larger_than_scratch(dglib):
    torch = pytest.importorskip("torch")
    dg = dglib
    fn = entry(dg)
    mesh = dg.Mesh.square(128, 128, jitter=0.1, seed=4, bc=(-4, -4, -4, -4))
    s = dg.Solver(mesh, dg.EULER, 3, problem="euler_riemann4")
    buf = torch.zeros(s.N * s.n_p * s.K, dtype=torch.float64, device="cuda")
    rc = fn(s._h, 0.0, buf.data_ptr(), buf.data_ptr())
    assert rc == DG_UNSUPPORTED
    assert "scratch" in dg.load_library().dg_last_error().decode()
