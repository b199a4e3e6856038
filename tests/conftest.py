import glob
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)
GOLDEN = os.path.join(ROOT, "tests", "golden")
from oracle.reference_tree import conservation_tree  # noqa: E402

# the reference's src/2d/conservation tree where it is mounted, else None
REF_TREE = conservation_tree()


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


def golden_names(prefix):
    return sorted(os.path.basename(f)[:-4] for f in glob.glob(os.path.join(GOLDEN, prefix + "*.npz")))


def load_golden(name):
    return dict(np.load(os.path.join(GOLDEN, name + ".npz")))


def ref_tables(p):
    return np.load(os.path.join(GOLDEN, "tables_p%d.npz" % p))["out"]


def split_tables(tab, p):
    """Split a flat reference tabulation into the dg_solver_set_tables arrays."""
    npm, nq, n1 = (p + 1) * (p + 2) // 2, [1, 3, 6, 12, 16, 25][p], p + 1
    sizes = [npm * nq, npm * nq, npm * nq, 3 * npm * n1, 3 * npm, nq, nq, nq, n1, n1]
    out, o = [], 0
    for s in sizes:
        out.append(np.ascontiguousarray(tab[o:o + s]))
        o += s
    return out


PB_PULSE = 18


def pulse_series(d):
    """(amp, omega, phase, t0) of a euler_pulse fixture: prm 8 holds t0 and
    prm 9..14 two (amp, omega, phase) terms."""
    prm = d["prm"]
    return prm[[9, 12]], prm[[10, 13]], prm[[11, 14]], float(prm[8])


def relerr(a, b, N):
    """max over variables of ||a_n - b_n|| / ||b_n|| (norm-wise, per variable block)."""
    a = np.asarray(a).reshape(N, -1)
    b = np.asarray(b).reshape(N, -1)
    return max(np.linalg.norm(a[n] - b[n]) / max(np.linalg.norm(b[n]), 1e-300) for n in range(N))


@pytest.fixture(scope="session")
def dglib():
    """The native library, built in-tree if needed."""
    from dgcuda_gb300 import build as b
    b.build()
    import dgcuda_gb300 as dg
    dg.load_library()
    return dg


@pytest.fixture(scope="session")
def oracle_mod():
    from oracle import oracle as o
    o.build()
    return o


def has_gpu():
    try:
        import ctypes
        rt = ctypes.CDLL("libcudart.so")
    except OSError:
        rt = None
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False
