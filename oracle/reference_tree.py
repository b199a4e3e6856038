"""Where the reference repository is, for the recipes that read it (test
infrastructure only: the host build of the reference kernels, the golden
generator, the reference-mesh tests and the CPU timing of the reference's
shipped program).

The location is the environment variable DG_REFERENCE_ROOT when it is set,
else the default of REF_ROOT in oracle/ref_host/Makefile (the one place that
names it).  None when neither points at an existing directory, as on a
machine without the reference tree.
"""
import os
import re

HERE = os.path.dirname(os.path.abspath(__file__))
MAKEFILE = os.path.join(HERE, "ref_host", "Makefile")


def reference_root():
    root = os.environ.get("DG_REFERENCE_ROOT")
    if not root:
        try:
            m = re.search(r"^REF_ROOT\s*\?=\s*(\S+)", open(MAKEFILE).read(), re.M)
        except OSError:
            m = None
        root = m.group(1) if m else None
    return root if root and os.path.isdir(root) else None


def conservation_tree():
    """The reference's src/2d/conservation directory, or None."""
    root = reference_root()
    if root is None:
        return None
    tree = os.path.join(root, "src", "2d", "conservation")
    return tree if os.path.isdir(tree) else None
