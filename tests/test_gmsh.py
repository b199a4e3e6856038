"""Gmsh .msh import (genmesh.py:13-315 restated in C++): the converted mesh
matches what the reference's own converter writes for the same files
(fixtures made by tests/golden/make_gmsh_golden.py), and the importer's
error handling."""
import os

import numpy as np
import pytest

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def read_pmsh_text(path):
    L = open(path).read().split("\n")
    K = int(L[0])
    el = np.array([[float(x) for x in l.split()] for l in L[1:1 + K]])
    S = int(L[1 + K])
    sd = np.array([[float(x) for x in l.split()] for l in L[2 + K:2 + K + S]])
    return el, sd


@pytest.mark.parametrize("name", ["square6", "square9_mixed"])
def test_gmsh_matches_reference_converter(dglib, name, tmp_path):
    dg = dglib
    m = dg.Mesh.read_gmsh(os.path.join(GOLD, "gmsh_%s.msh" % name))
    el, sd = read_pmsh_text(os.path.join(GOLD, "gmsh_%s.pmsh" % name))
    V, es, sxy, se = m.arrays()
    assert (m.K, m.S) == (len(el), len(sd))
    # genmesh.py writes %.015lf: coordinates agree to its rounding
    assert np.abs(V.T - el[:, :6]).max() <= 1e-15
    assert np.array_equal(es.T, el[:, 6:].astype(int))
    assert np.abs(sxy.T - sd[:, :4]).max() <= 1e-15
    assert np.array_equal(se.T, sd[:, 4:].astype(int))
    # and the converted mesh survives the .pmsh round trip
    p = str(tmp_path / "m.pmsh")
    m.write(p)
    m2 = dg.Mesh.read_mesh(p)
    for a, b in zip(m.arrays(), m2.arrays()):
        assert np.array_equal(a, b)


def _write(path, text):
    with open(path, "w") as f:
        f.write(text)
    return str(path)


HEAD = "$MeshFormat\n2.2 0 8\n$EndMeshFormat\n$Nodes\n4\n1 0 0 0\n2 1 0 0\n3 1 1 0\n4 0 1 0\n$EndNodes\n"


def test_gmsh_clockwise_triangles_are_reoriented(dglib, tmp_path):
    dg = dglib
    lines = ["1 1 2 10000 1 1 2", "2 1 2 20000 1 2 3", "3 1 2 30000 1 3 4", "4 1 2 10000 1 4 1"]
    # both triangles listed clockwise, node ids not starting at 1 are fine too
    body = "$Elements\n6\n" + "\n".join(lines) + "\n5 2 2 100 1 1 3 2\n6 2 2 100 1 1 4 3\n$EndElements\n"
    m = dg.Mesh.read_gmsh(_write(tmp_path / "cw.msh", HEAD + body))
    V, es, sxy, se = m.arrays()
    J = (V[2] - V[0]) * (V[5] - V[1]) - (V[4] - V[0]) * (V[3] - V[1])
    assert (m.K, m.S) == (2, 5) and np.all(J > 0)
    assert sorted(se[1][:4]) == [-3, -2, -1, -1] and list(se[1][:4]) == [-1, -1, -2, -3]


def test_gmsh_errors(dglib, tmp_path):
    dg = dglib
    # a boundary side with no tagged line
    body = "$Elements\n2\n1 1 2 10000 1 1 2\n2 2 2 100 1 1 2 3\n$EndElements\n"
    with pytest.raises(dg.DGError, match="tagged line"):
        dg.Mesh.read_gmsh(_write(tmp_path / "untagged.msh", HEAD + body))
    with pytest.raises(dg.DGError):
        dg.Mesh.read_gmsh(str(tmp_path / "missing.msh"))
    with pytest.raises(dg.DGError, match="format"):
        dg.Mesh.read_gmsh(_write(tmp_path / "v4.msh", "$MeshFormat\n4.1 0 8\n$EndMeshFormat\n"))
    body = "$Elements\n1\n1 2 2 100 1 1 2 9\n$EndElements\n"
    with pytest.raises(dg.DGError, match="triangle"):
        dg.Mesh.read_gmsh(_write(tmp_path / "badnode.msh", HEAD + body))
