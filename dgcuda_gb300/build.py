"""Build the native library libdg_gb300.so (and the dgcuda CLI) in-tree.

Every CUDA translation unit is compiled for sm_103a only
(``-gencode arch=compute_103a,code=sm_103a``); host C++ goes through nvcc as
well so one toolchain links everything.  Objects land in ``_build/`` beside
this file and are rebuilt when a source or any header is newer, or when
they were built on another host architecture or with other flags (a stamp
in ``_build/``).  Translation units compile in parallel.
"""
import hashlib
import os
import platform
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libdg_gb300.so")
CLI = os.path.join(HERE, "dgcuda")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc():
    for c in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def _sources():
    srcs = sorted(f for f in os.listdir(CSRC) if f.endswith((".cu", ".cpp")))
    lib = [s for s in srcs if s != "dg_cli.cpp"]
    return lib


def _headers():
    hs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    hs.append(os.path.join(ROOT, "include", "dg.h"))
    return hs


def _compile(src, flags):
    obj = os.path.join(BUILD, src + ".o")
    path = os.path.join(CSRC, src)
    newest = max([os.path.getmtime(path), os.path.getmtime(__file__)] +
                 [os.path.getmtime(h) for h in _headers()])
    if os.path.exists(obj) and os.path.getmtime(obj) >= newest:
        return obj
    cmd = [nvcc()] + ARCH + flags + ["-c", path, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("compile failed: %s\n%s\n%s" % (" ".join(cmd), r.stdout, r.stderr))
    return obj


def _check_stamp(flags):
    """Drops objects and outputs built on another machine architecture or
    with other flags: a newer mtime alone does not make them usable here."""
    stamp = os.path.join(BUILD, "STAMP")
    want = "%s %s" % (platform.machine(),
                      hashlib.sha1(" ".join(ARCH + flags).encode()).hexdigest())
    have = open(stamp).read().strip() if os.path.exists(stamp) else None
    if have == want:
        return
    for f in os.listdir(BUILD):
        if f.endswith(".o"):
            os.remove(os.path.join(BUILD, f))
    for f in (LIB, CLI):
        if os.path.exists(f):
            os.remove(f)
    with open(stamp, "w") as fh:
        fh.write(want + "\n")


def build(verbose=False, jobs=None):
    os.makedirs(BUILD, exist_ok=True)
    # host code: no contraction of a*b+c into FMAs the source does not write,
    # so meshes and geometry have the same bits on x86 and Arm
    common = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC,-O2,-ffp-contract=off",
              "-I" + CSRC,
              "-I" + os.path.join(ROOT, "include")]
    cuflags = common + ["-Xptxas", "-O3", "--expt-relaxed-constexpr"]
    _check_stamp(cuflags)
    srcs = _sources()
    jobs = jobs or min(len(srcs), os.cpu_count() or 4)
    with ThreadPoolExecutor(jobs) as ex:
        objs = list(ex.map(lambda s: _compile(s, cuflags), srcs))
    newest = max(os.path.getmtime(o) for o in objs)
    if not os.path.exists(LIB) or os.path.getmtime(LIB) < newest:
        cmd = [nvcc()] + ARCH + ["-shared", "-o", LIB] + objs + ["-lcudart_static", "-lrt",
                                                                   "-ldl", "-lpthread"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("link failed: %s\n%s" % (r.stdout, r.stderr))
    cli_src = os.path.join(CSRC, "dg_cli.cpp")
    if os.path.exists(cli_src):
        cobj = _compile("dg_cli.cpp", common)
        if not os.path.exists(CLI) or os.path.getmtime(CLI) < max(os.path.getmtime(cobj),
                                                                  os.path.getmtime(LIB)):
            cmd = [nvcc()] + ARCH + ["-o", CLI, cobj, "-L" + HERE, "-ldg_gb300",
                                     "-Xlinker", "-rpath,$ORIGIN"]
            r = subprocess.run(cmd, capture_output=True, text=True)
            if r.returncode != 0:
                raise RuntimeError("CLI link failed: %s\n%s" % (r.stdout, r.stderr))
    if verbose:
        print("built", LIB)
    return LIB


if __name__ == "__main__":
    build(verbose=True)
    sys.exit(0)
