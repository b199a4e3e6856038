"""The C ABI: the library loads and exports every function include/dg.h
declares; without a GPU the solver fails loudly instead of falling back."""
import ctypes
import os
import re

import pytest

from conftest import ROOT


def declared(header="dg.h"):
    src = open(os.path.join(ROOT, "include", header)).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(dg_\w+)\s*\(", src)))


def test_every_declared_symbol_is_exported(dglib):
    lib = ctypes.CDLL(dglib.lib_path())
    names = declared()
    assert len(names) >= 30
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_test_header_symbols_are_exported_and_kept_apart(dglib):
    """The arithmetic checks live in include/dg_test.h, not in the drop-in
    interface."""
    lib = ctypes.CDLL(dglib.lib_path())
    probes = declared("dg_test.h")
    assert probes == ["dg_probe_physical", "dg_probe_reciprocal", "dg_probe_sqrt"]
    assert not set(probes) & set(declared())
    assert all(hasattr(lib, n) for n in probes)


def test_version_and_defaults(dglib):
    L = dglib.load_library()
    assert b"sm_103a" in L.dg_version()
    p = dglib.Params()
    L.dg_params_default(ctypes.byref(p))
    assert p.gamma == 1.4 and p.gravity == 9.81 and p.cfl == 0.3


def test_solver_without_gpu_fails_loudly(dglib):
    try:
        import torch
        if torch.cuda.is_available():
            pytest.skip("a GPU is present")
    except ImportError:
        pass
    m = dglib.Mesh.square(4, 4)
    with pytest.raises(dglib.DGError) as ei:
        dglib.Solver(m, dglib.EULER, 1)
    assert ei.value.status == 5  # CUDA_ERROR


def test_bad_arguments_are_status_codes(dglib):
    m = dglib.Mesh.square(4, 4)
    with pytest.raises(dglib.DGError) as ei:
        dglib.Solver(m, dglib.EULER, 7)
    assert ei.value.status == 1
