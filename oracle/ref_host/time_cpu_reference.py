"""Times the reference's own CPU code (src/2d/cpu-conservation, the shipped
supersonic-vortex program, gcc -O2, one thread) against the C oracle port on
the same cores, mesh, order and scheme (RK4, no limiter), in DOF-stage
updates per second.  Needs the reference tree, so it runs where that tree
is (the build container); the binary goes to oracle/_ref/.

    python oracle/ref_host/time_cpu_reference.py [REF_ROOT] [STEPS]

The reference program writes into ./output and crashes when that directory
is missing, so it runs inside a scratch directory that has one.
"""
import os
import subprocess
import sys
import tempfile
import time

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
from oracle.reference_tree import reference_root  # noqa: E402

REF = sys.argv[1] if len(sys.argv) > 1 else reference_root()
STEPS = int(sys.argv[2]) if len(sys.argv) > 2 else 100
MESH = os.path.join(REF, "src/2d/conservation/euler/supersonic/mesh/sv-large.pmsh")


def build():
    out = os.path.join(ROOT, "oracle", "_ref")
    os.makedirs(out, exist_ok=True)
    exe = os.path.join(out, "cpu_supersonic")
    src = os.path.join(REF, "src/2d/cpu-conservation/euler/supersonic/supersonic.c")
    subprocess.run(["gcc", "-O2", "-w", src, "-lm", "-o", exe], check=True)
    return exe


def main():
    exe = build()
    os.environ["OMP_NUM_THREADS"] = "1"
    sys.path.insert(0, ROOT)
    import dgcuda_gb300 as dg
    from oracle import oracle as orc
    mesh = dg.Mesh.read_mesh(MESH)
    for p in (1, 3):
        npm = (p + 1) * (p + 2) // 2
        units = mesh.K * 4 * npm * 4 * STEPS  # 4 RK4 stages per step
        with tempfile.TemporaryDirectory() as d:
            os.makedirs(os.path.join(d, "output"))
            t0 = time.perf_counter()
            subprocess.run([exe, "-n", str(p), "-t", str(STEPS), MESH], cwd=d, check=True,
                           stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL)
            ref = units / (time.perf_counter() - t0)
        o = orc.Oracle.from_mesh(mesh, dg.EULER, p, orc.prm_vec(gamma=1.4),
                                 dg.PROBLEMS["euler_supersonic"])
        c = o.init()
        t0 = time.perf_counter()
        o.step(c, STEPS, 1, 0, 0.5)
        port = units / (time.perf_counter() - t0)
        print("p=%d K=%d steps=%d: reference CPU %.3e, oracle port %.3e DOF-stage/s (1 thread)"
              % (p, mesh.K, STEPS, ref, port))


if __name__ == "__main__":
    main()
