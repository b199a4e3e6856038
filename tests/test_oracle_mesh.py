"""The oracle's own square-mesh generator (which bench.py's reference arm
uses, so that it never loads the product library) builds the same arrays,
bit for bit, as the library's dg_mesh_square: same vertices, jitter, side
numbering and boundary order.  Host code only (no GPU)."""
import numpy as np
import pytest

CASES = [
    # nx, ny, box, jitter, seed, bc
    (32, 32, (0.0, 1.0, 0.0, 1.0), 0.1, 1, (0, 0, 0, 0)),
    (24, 17, (0.0, 10.0, 0.0, 10.0), 0.15, 2, (0, 0, 0, 0)),
    (40, 40, (0.0, 1.0, 0.0, 1.0), 0.1, 3, (-4, -4, -4, -4)),
    (9, 13, (-1.0, 2.0, 0.5, 1.5), 0.1, 4005, (-1, -1, -1, -1)),
    (7, 5, (0.0, 1.0, 0.0, 1.0), 0.1, 5, (-1, -2, -3, -4)),
    (6, 8, (0.0, 1.0, 0.0, 1.0), 0.0, 0, (0, 0, -1, -3)),
    (6, 8, (0.0, 1.0, 0.0, 1.0), 0.2, 9, (-2, -2, 0, 0)),
]


@pytest.mark.parametrize("case", CASES, ids=[str(i) for i in range(len(CASES))])
def test_oracle_mesh_equals_library_mesh(dglib, oracle_mod, case):
    nx, ny, box, jitter, seed, bc = case
    got = oracle_mod.mesh_square(nx, ny, box=box, jitter=jitter, seed=seed, bc=bc)
    want = dglib.Mesh.square(nx, ny, box=box, jitter=jitter, seed=seed, bc=bc).arrays()
    for g, w in zip(got, want):
        assert g.shape == w.shape and g.dtype == w.dtype
        assert np.array_equal(g, w)


def test_oracle_mesh_full_config_size(oracle_mod):
    """The 1024 x 1024 throughput mesh: 2,097,152 triangles, 3,147,776 sides
    (4096 transmissive, listed first)."""
    V, es, sxy, se = oracle_mod.mesh_square(1024, 1024, jitter=0.1, seed=3, bc=(-4, -4, -4, -4))
    assert V.shape == (6, 2097152) and sxy.shape == (4, 3147776)
    assert np.all(se[1][:4096] == -4) and np.all(se[1][4096:] >= 0)
    assert es.min() == 0 and es.max() == 3147775
