"""Meshes: .pmsh reader/writer (the reference's format, main.cu:205-277),
validation errors as status codes, the synthetic jittered generator."""
import os

import numpy as np
import pytest

from conftest import REF_TREE


def test_config_mesh_sizes(dglib):
    dg = dglib
    m = dg.Mesh.square(32, 32, jitter=0.1, seed=1)
    assert (m.K, m.S) == (2048, 3072)
    n = 64
    m = dg.Mesh.square(n, n, jitter=0.1, seed=3, bc=(-4, -4, -4, -4))
    assert (m.K, m.S) == (2 * n * n, 3 * n * n + 2 * n)
    V, es, sxy, se = m.arrays()
    assert np.sum(se[1] < 0) == 4 * n and np.all(se[1][:4 * n] == -4)  # boundary first


def test_boundary_sides_first_and_codes(dglib):
    dg = dglib
    m = dg.Mesh.square(5, 4, jitter=0.1, seed=2, bc=(-1, -2, -3, -4))
    _, _, _, se = m.arrays()
    codes = se[1][se[1] < 0]
    nb = len(codes)
    assert np.all(se[1][:nb] < 0) and np.all(se[1][nb:] >= 0)
    assert list(codes) == sorted(codes, reverse=True)
    assert {int(c): int(np.sum(codes == c)) for c in set(codes)} == {-1: 4, -2: 4, -3: 5, -4: 5}


def test_jitter_interior_only(dglib):
    dg = dglib
    n, d = 8, 0.1
    m = dg.Mesh.square(n, n, jitter=d, seed=5, bc=(-2, -2, -2, -2))
    V = m.arrays()[0]
    xs, ys = V[0::2].ravel(), V[1::2].ravel()
    h = 1.0 / n
    gx, gy = np.round(xs / h) * h, np.round(ys / h) * h
    assert np.all(np.abs(xs - gx) <= d * h + 1e-15) and np.all(np.abs(ys - gy) <= d * h + 1e-15)
    on_boundary = (np.isclose(gx, 0) | np.isclose(gx, 1) | np.isclose(gy, 0) | np.isclose(gy, 1))
    assert np.all(xs[on_boundary] == gx[on_boundary]) and np.all(ys[on_boundary] == gy[on_boundary])


def test_periodic_mesh_is_closed(dglib):
    dg = dglib
    m = dg.Mesh.square(6, 5, jitter=0.15, seed=8)
    V, es, sxy, se = m.arrays()
    assert np.all(se[1] >= 0)
    K = m.K
    for e in range(K):
        nb = set()
        for f in range(3):
            s = es[f][e]
            nb.add(se[1][s] if se[0][s] == e else se[0][s])
        assert len(nb) == 3 and e not in nb


def test_pmsh_round_trip(dglib, tmp_path):
    dg = dglib
    m = dg.Mesh.square(7, 5, box=(0, 10, -1, 1), jitter=0.12, seed=4, bc=(-1, -2, 0, 0))
    path = str(tmp_path / "m.pmsh")
    m.write(path)
    m2 = dg.Mesh.read_mesh(path)
    for a, b in zip(m.arrays(), m2.arrays()):
        assert np.array_equal(a, b)


def test_bad_meshes_are_status_codes(dglib, tmp_path):
    dg = dglib
    with pytest.raises(dg.DGError) as ei:
        dg.Mesh.read_mesh(str(tmp_path / "missing.pmsh"))
    assert ei.value.status == 7  # IO_ERROR
    m = dg.Mesh.square(4, 4, jitter=0.1, seed=1)
    path = str(tmp_path / "m.pmsh")
    m.write(path)
    lines = open(path).read().splitlines()
    open(str(tmp_path / "trunc.pmsh"), "w").write("\n".join(lines[:10]) + "\n")
    with pytest.raises(dg.DGError) as ei:
        dg.Mesh.read_mesh(str(tmp_path / "trunc.pmsh"))
    assert ei.value.status == 2  # BAD_MESH
    V, es, sxy, se = m.arrays()
    es2 = es.copy()
    es2[0, 3] = m.S + 5
    with pytest.raises(dg.DGError):
        dg.Mesh.from_arrays(V, es2, sxy, se)
    V2 = V.copy()
    V2[[0, 1, 2, 3]] = V[[2, 3, 0, 1]]  # swap vertices 1 and 2: clockwise
    with pytest.raises(dg.DGError) as ei:
        dg.Mesh.from_arrays(V2, es, sxy, se)
    assert "CCW" in str(ei.value)
    with pytest.raises(dg.DGError):
        dg.Mesh.square(4, 4, bc=(0, -1, 0, 0))  # unpaired periodic side


@pytest.mark.skipif(REF_TREE is None, reason="reference tree not mounted")
@pytest.mark.parametrize("name,K,S", [("A", 180, 293), ("B", 720, 1126), ("C", 2880, 4412),
                                      ("D", 11520, 17464)])
def test_reads_reference_supersonic_ladder(dglib, name, K, S):
    m = dglib.Mesh.read_mesh(os.path.join(REF_TREE, "euler/supersonic/mesh/%s.pmsh" % name))
    assert (m.K, m.S) == (K, S)
