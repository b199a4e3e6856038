"""Golden fixtures for the Gmsh importer: small seeded .msh files written by
this script, and the .pmsh files the reference's own converter
(src/2d/conservation/genmesh.py) makes from them.

genmesh.py is Python 2; it is loaded as text and its `print` statements and
`xrange` are rewritten for Python 3 in memory (nothing else changes), then
its genmesh(infile, outfile) is called.  Run once in a tree that has the
reference checked out:

    python tests/golden/make_gmsh_golden.py /path/to/DGCUDA

Output: tests/golden/gmsh_<name>.msh and gmsh_<name>.pmsh.
"""
import os
import re
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def write_msh(path, n, seed, tags=(30000, 20000, 10000, 10000), jitter=0.15):
    """n x n squares on [0,1]^2, each cut into two CCW triangles, interior
    nodes jittered, triangles shuffled and their vertex lists rotated, node
    ids shuffled (still 1..nn, as genmesh.py requires); boundary lines
    tagged bottom/right/top/left = tags; one point element that the
    converters must skip."""
    rng = np.random.default_rng(seed)
    nn = (n + 1) * (n + 1)
    xy = np.zeros((nn, 2))
    for j in range(n + 1):
        for i in range(n + 1):
            x, y = i / n, j / n
            if 0 < i < n and 0 < j < n:
                x += jitter / n * rng.uniform(-1, 1)
                y += jitter / n * rng.uniform(-1, 1)
            xy[j * (n + 1) + i] = (x, y)
    ids = rng.permutation(nn) + 1          # node k has file id ids[k]
    tris = []
    for j in range(n):
        for i in range(n):
            a = j * (n + 1) + i
            b, c, d = a + 1, a + n + 2, a + n + 1
            tris.append((a, b, c))
            tris.append((a, c, d))
    tris = [tris[k] for k in rng.permutation(len(tris))]
    tris = [t[r:] + t[:r] for t, r in zip(tris, rng.integers(0, 3, len(tris)))]
    lines = []
    for i in range(n):
        lines.append((tags[0], i, i + 1))                                  # bottom
        lines.append((tags[1], i * (n + 1) + n, (i + 1) * (n + 1) + n))    # right
        lines.append((tags[2], n * (n + 1) + i + 1, n * (n + 1) + i))      # top
        lines.append((tags[3], (i + 1) * (n + 1), i * (n + 1)))            # left
    with open(path, "w") as f:
        f.write("$MeshFormat\n2.2 0 8\n$EndMeshFormat\n$Nodes\n%d\n" % nn)
        order = np.argsort(ids)
        for k in order:
            f.write("%d %.16g %.16g 0\n" % (ids[k], xy[k, 0], xy[k, 1]))
        f.write("$EndNodes\n$Elements\n%d\n" % (1 + len(lines) + len(tris)))
        num = 1
        f.write("%d 15 2 0 1 %d\n" % (num, ids[0]))
        for tag, a, b in lines:
            num += 1
            f.write("%d 1 2 %d 1 %d %d\n" % (num, tag, ids[a], ids[b]))
        for a, b, c in tris:
            num += 1
            f.write("%d 2 2 100 1 %d %d %d\n" % (num, ids[a], ids[b], ids[c]))
        f.write("$EndElements\n")


def load_genmesh(ref_root):
    src = open(os.path.join(ref_root, "src/2d/conservation/genmesh.py")).read()
    src = re.sub(r'^(\s*)print (.*)$', r'\1print(\2)', src, flags=re.M)
    src = src.replace("xrange", "range").replace('"rb"', '"r"').replace('"wb"', '"w"')
    ns = {"__name__": "genmesh_py2"}
    exec(compile(src, "genmesh.py", "exec"), ns)
    return ns["genmesh"]


CASES = {"square6": dict(n=6, seed=7), "square9_mixed": dict(n=9, seed=11,
                                                            tags=(10000, 20000, 30000, 20000))}

if __name__ == "__main__":
    genmesh = load_genmesh(sys.argv[1])
    for name, kw in CASES.items():
        msh = os.path.join(HERE, "gmsh_%s.msh" % name)
        write_msh(msh, **kw)
        genmesh(msh, os.path.join(HERE, "gmsh_%s.pmsh" % name))
