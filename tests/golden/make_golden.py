#!/usr/bin/env python3
"""Generate the golden vectors in this directory from the reference itself.

The reference's own DG kernels (src/2d/conservation: conserv_kernels.cu,
the four equation modules, quadrature.cu, basis.cu) are compiled as host
programs by oracle/ref_host/Makefile into oracle/_ref/ (this needs the
reference tree, so it only runs where that tree is mounted).  This script
feeds them small meshes made by the library's own mesh generator (and the
reference's supersonic mesh A, read from the reference tree), and stores
inputs + outputs as .npz fixtures that the tests read on any machine.

Each fixture holds: eq, p, mode, problem, hdr (int32[16]), prm (float64[16]),
mesh arrays V[6,K], es[3,K], sxy[4,S], se[4,S], C (input state, reference
layout [var][mode][elem]) and out (the reference's result).  Modes: 0 RHS
(du/dt), 1 RK steps (final state + final t), 2 limiter, 3 L2 projection of
the initial condition, 5 per-variable squared L2 error, 6 wave speeds + min
diameter.  tables_p{p}.npz holds the reference's basis/quadrature tabulation
for order p (mode 4).

Run from the repository root:  python tests/golden/make_golden.py
"""
import os
import subprocess
import sys
import tempfile

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
import dgcuda_gb300 as dg  # noqa: E402

from oracle.reference_tree import conservation_tree, reference_root  # noqa: E402

REF_TREE = conservation_tree()
OUT = os.path.join(ROOT, "tests", "golden")
TMP = tempfile.mkdtemp(prefix="dg_golden_")
REF = os.path.join(ROOT, "oracle", "_ref")
EQ_BIN = {dg.ADVECTION: "ref_advection", dg.EULER: "ref_euler",
          dg.SHALLOW_WATER: "ref_shallowwater", dg.MAXWELL: "ref_maxwells"}
PB = dg.PROBLEMS


def build_ref():
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle", "ref_host"),
                    "REF_ROOT=" + reference_root()], check=True)


def run_ref(eq, p, mode, problem, mesh, C, prm, nsteps=0, limiter=0, rk=4):
    V, es, sxy, se = mesh.arrays()
    hdr = np.zeros(16, dtype=np.int32)
    hdr[:9] = [eq, p, mesh.K, mesh.S, mode, nsteps, limiter, problem, rk]
    prm = np.asarray(prm, dtype=np.float64)
    os.makedirs(TMP, exist_ok=True)
    fin, fout = os.path.join(TMP, "in.bin"), os.path.join(TMP, "out.bin")
    with open(fin, "wb") as f:
        for a in (hdr, prm, V, es, sxy, se, np.ascontiguousarray(C, dtype=np.float64)):
            f.write(np.ascontiguousarray(a).tobytes())
    subprocess.run([os.path.join(REF, EQ_BIN[eq]), fin, fout], check=True)
    out = np.fromfile(fout, dtype=np.float64)
    return dict(eq=eq, p=p, mode=mode, problem=problem, hdr=hdr, prm=prm, V=V, es=es, sxy=sxy,
                se=se, C=np.asarray(C, dtype=np.float64), out=out)


def prm_vec(t=0.0, gamma=1.4, ax=1.0, ay=0.5, mu=1.0, eps=1.0, cfl=0.5, extra=()):
    # 0 t, 1 gamma, 2 ax, 3 ay, 4 mu, 5 eps, 6 g (the reference hard-codes
    # 9.8, shallowwater.cu:7), 7 cfl, 8.. problem parameters
    v = np.zeros(16)
    v[0], v[1], v[2], v[3], v[4], v[5], v[6], v[7] = t, gamma, ax, ay, mu, eps, 9.8, cfl
    for i, x in enumerate(extra):
        v[8 + i] = x
    return v


def perturbed_ic(eq, p, problem, mesh, prm, seed, amp=0.02):
    """L2 projection of the problem's IC (by the reference) plus a small
    seeded perturbation of every mode, so all modes are exercised."""
    N, npm = dg.n_vars(eq), dg.n_modes(p)
    zero = np.zeros((N, npm, mesh.K))
    C = run_ref(eq, p, 3, problem, mesh, zero, prm)["out"].reshape(N, npm, mesh.K)
    rng = np.random.default_rng(seed)
    # higher modes only, scaled by each element's own mean, so cell means
    # (and with them positivity) are untouched
    scale = np.abs(C[:, :1, :]) + 1e-3 * np.abs(C[:, :1, :]).mean()
    pert = amp * scale * rng.standard_normal(C.shape) / (1 + np.arange(npm))[None, :, None]
    pert[:, 0, :] = 0
    return C + pert


def save(name, d):
    np.savez_compressed(os.path.join(OUT, name + ".npz"), **d)


def main():
    build_ref()
    os.makedirs(OUT, exist_ok=True)
    # reference tabulation of basis + quadrature, p = 0..5
    for p in range(6):
        m = dg.Mesh.square(3, 3, jitter=0.0, seed=0)
        d = run_ref(dg.ADVECTION, p, 4, 0, m, np.zeros((1, dg.n_modes(p), m.K)), prm_vec())
        save("tables_p%d" % p, d)

    m_adv = dg.Mesh.square(6, 6, jitter=0.1, seed=11)
    m_lin = dg.Mesh.square(5, 5, jitter=0.1, seed=12, bc=(-3, -2, -3, -2))
    m_vtx = dg.Mesh.square(6, 6, box=(0, 10, 0, 10), jitter=0.15, seed=13)
    m_r4 = dg.Mesh.square(6, 6, jitter=0.1, seed=14, bc=(-2, -2, -2, -2))
    m_wall = dg.Mesh.square(5, 5, box=(0, 10, 0, 10), jitter=0.1, seed=15,
                            bc=(-1, -1, -1, -1))
    m_sw = dg.Mesh.square(6, 6, jitter=0.1, seed=16, bc=(-1, -1, -1, -1))
    m_swp = dg.Mesh.square(6, 6, jitter=0.1, seed=17)
    m_mx = dg.Mesh.square(6, 6, jitter=0.1, seed=18)
    m_mxw = dg.Mesh.square(5, 5, jitter=0.1, seed=19, bc=(-1, -1, -1, -1))
    m_ss = dg.Mesh.read_mesh(os.path.join(REF_TREE, "euler/supersonic/mesh/A.pmsh"))

    vtx = (5.0, 5.0, 5.0, 1.0, 1.0, 10.0)  # beta, x0, y0, uinf, vinf, L
    hump = (1.0, 0.1, 0.1, 0.45, 0.55)      # h0, A, sigma, x0, y0
    cases = [
        # name, eq, problem, mesh, prm, p list
        ("adv_sine", dg.ADVECTION, PB["adv_sine"], m_adv, prm_vec(), range(6)),
        ("adv_linear", dg.ADVECTION, PB["adv_linear"], m_lin, prm_vec(ax=1, ay=1), [1, 2, 3]),
        ("euler_vortex", dg.EULER, PB["euler_vortex"], m_vtx, prm_vec(extra=vtx), range(6)),
        ("euler_riemann4", dg.EULER, PB["euler_riemann4"], m_r4, prm_vec(), [1, 2]),
        ("euler_wall", dg.EULER, PB["euler_vortex"], m_wall,
         prm_vec(extra=(5.0, 5.0, 5.0, 0.3, -0.2, 0.0)), [2]),
        ("euler_supersonic", dg.EULER, PB["euler_supersonic"], m_ss, prm_vec(), [1, 2, 3, 4]),
        ("sw_test", dg.SHALLOW_WATER, PB["sw_test"], m_sw, prm_vec(), range(6)),
        ("sw_hump", dg.SHALLOW_WATER, PB["sw_hump"], m_swp, prm_vec(extra=hump), [2]),
        ("maxwell_plane", dg.MAXWELL, PB["maxwell_plane"], m_mx, prm_vec(mu=1.3, eps=0.7),
         [1, 2, 3, 4]),
        ("maxwell_wall", dg.MAXWELL, PB["maxwell_plane"], m_mxw, prm_vec(), [2]),
    ]
    seed = 100
    for name, eq, pb, mesh, prm, plist in cases:
        for p in plist:
            seed += 1
            C = perturbed_ic(eq, p, pb, mesh, prm, seed)
            prm_t = prm.copy()
            prm_t[0] = 0.05
            save("rhs_%s_p%d" % (name, p), run_ref(eq, p, 0, pb, mesh, C, prm_t))
        # initial-condition projection at the middle order
        p = list(plist)[len(list(plist)) // 2]
        N = dg.n_vars(eq)
        save("init_%s_p%d" % (name, p),
             run_ref(eq, p, 3, pb, mesh, np.zeros((N, dg.n_modes(p), mesh.K)), prm))

    # problems whose boundary data are the point of the case: each RHS at a
    # time where its inflow is active
    pulse = (0.9197, 0.05, 4.47, 2.9, 0.03, 8.95, 2.66)  # t0, (amp, omega, phase) x 2
    m_rot = dg.Mesh.square(6, 6, box=(-1, 1, -1, 1), jitter=0.1, seed=31, bc=(-3, -3, -3, -3))
    m_spin = dg.Mesh.square(6, 6, jitter=0.1, seed=32, bc=(-3, -3, -3, -3))
    m_sq = dg.Mesh.square(6, 6, box=(-1, 1, -1, 1), jitter=0.1, seed=33, bc=(-3, -2, -2, -2))
    m_cm = dg.Mesh.square(6, 6, jitter=0.1, seed=34, bc=(-3, -2, -1, -1))
    m_ws = dg.Mesh.square(6, 6, box=(-.5, .5, -.5, .5), jitter=0.1, seed=35, bc=(-3, -2, -1, -1))
    m_af = dg.Mesh.square(5, 5, jitter=0.1, seed=36, bc=(-2, -2, -1, -1))
    m_pu = dg.Mesh.square(8, 3, box=(0, 4, 0, 1), jitter=0.1, seed=37, bc=(-3, -2, -1, -1))
    bcases = [
        # name, eq, problem, mesh, prm (t in prm[0]), p list
        ("adv_rotatinghill", dg.ADVECTION, PB["adv_rotatinghill"], m_rot,
         prm_vec(t=0.1, ax=0, ay=0), [1, 2, 3]),
        ("adv_spin", dg.ADVECTION, PB["adv_spin"], m_spin, prm_vec(t=0.1, ax=0, ay=0), [2]),
        ("adv_squarehill", dg.ADVECTION, PB["adv_squarehill"], m_sq, prm_vec(t=0.1, ax=1, ay=0),
         [1, 2]),
        ("maxwell_cmirror", dg.MAXWELL, PB["maxwell_cmirror"], m_cm, prm_vec(t=0.02), [2]),
        ("maxwell_wscatter", dg.MAXWELL, PB["maxwell_wscatter"], m_ws, prm_vec(t=0.2), [2]),
        ("euler_airfoil", dg.EULER, PB["euler_airfoil"], m_af, prm_vec(t=0.1), [2]),
        ("euler_pulse", dg.EULER, PB["euler_pulse"], m_pu, prm_vec(t=0.3, extra=pulse), [2]),
    ]
    for name, eq, pb, mesh, prm, plist in bcases:
        for p in plist:
            seed += 1
            C = perturbed_ic(eq, p, pb, mesh, prm, seed)
            save("rhs_%s_p%d" % (name, p), run_ref(eq, p, 0, pb, mesh, C, prm))
        p = list(plist)[len(list(plist)) // 2]
        N = dg.n_vars(eq)
        save("init_%s_p%d" % (name, p),
             run_ref(eq, p, 3, pb, mesh, np.zeros((N, dg.n_modes(p), mesh.K)), prm))
    # wave speeds of the rotating fields (each element's speed at its middle
    # quadrature point) and reference RK loops driven by them
    for name, pb, mesh, p in [("adv_rotatinghill", PB["adv_rotatinghill"], m_rot, 2),
                              ("adv_spin", PB["adv_spin"], m_spin, 1)]:
        C = perturbed_ic(dg.ADVECTION, p, pb, mesh, prm_vec(ax=0, ay=0), 6)
        save("cfl_%s_p%d" % (name, p), run_ref(dg.ADVECTION, p, 6, pb, mesh, C,
                                               prm_vec(ax=0, ay=0)))
    for name, pb, mesh, p, ns, rk, cfl in [
            ("rk4_adv_rotatinghill_p2", PB["adv_rotatinghill"], m_rot, 2, 5, 4, 0.5),
            ("rk2_adv_spin_p1", PB["adv_spin"], m_spin, 1, 5, 2, 0.7)]:
        prm = prm_vec(ax=0, ay=0, cfl=cfl)
        C = run_ref(dg.ADVECTION, p, 3, pb, mesh, np.zeros((1, dg.n_modes(p), mesh.K)), prm)["out"]
        save(name, run_ref(dg.ADVECTION, p, 1, pb, mesh, C.reshape(1, -1, mesh.K), prm,
                           nsteps=ns, rk=rk))

    # limiter (p = 1): discontinuous Euler data, noisy advection data
    m8 = dg.Mesh.square(8, 8, jitter=0.1, seed=21, bc=(-2, -2, -2, -2))
    C = perturbed_ic(dg.EULER, 1, PB["euler_riemann4"], m8, prm_vec(), 7, amp=0.05)
    save("limit_euler_riemann4_p1", run_ref(dg.EULER, 1, 2, PB["euler_riemann4"], m8, C,
                                            prm_vec()))
    C = perturbed_ic(dg.ADVECTION, 1, PB["adv_sine"], m_adv, prm_vec(), 8, amp=0.5)
    save("limit_adv_sine_p1", run_ref(dg.ADVECTION, 1, 2, PB["adv_sine"], m_adv, C, prm_vec()))

    # reference RK loops (CFL dt from eval_global_lambda, t advanced first)
    steps = [
        ("rk4_adv_sine_p2", dg.ADVECTION, PB["adv_sine"], m_adv, prm_vec(cfl=0.5), 2, 10, 0, 4),
        ("rk4_euler_vortex_p1_lim", dg.EULER, PB["euler_vortex"], m_vtx,
         prm_vec(cfl=0.5, extra=vtx), 1, 5, 1, 4),
        ("rk4_euler_vortex_p3", dg.EULER, PB["euler_vortex"], m_vtx,
         prm_vec(cfl=0.5, extra=vtx), 3, 4, 0, 4),
        ("rk4_sw_test_p1", dg.SHALLOW_WATER, PB["sw_test"], m_sw, prm_vec(cfl=0.5), 1, 5, 0, 4),
        ("rk4_euler_supersonic_p1_lim", dg.EULER, PB["euler_supersonic"], m_ss,
         prm_vec(cfl=0.5), 1, 3, 1, 4),
        ("rk4_maxwell_plane_p2", dg.MAXWELL, PB["maxwell_plane"], m_mx, prm_vec(cfl=0.5), 2, 5,
         0, 4),
        ("rk2_adv_sine_p1", dg.ADVECTION, PB["adv_sine"], m_adv, prm_vec(cfl=0.7), 1, 6, 0, 2),
        ("rk2_euler_vortex_p1_lim", dg.EULER, PB["euler_vortex"], m_vtx,
         prm_vec(cfl=0.7, extra=vtx), 1, 4, 1, 2),
    ]
    for name, eq, pb, mesh, prm, p, ns, lim, rk in steps:
        N = dg.n_vars(eq)
        C = run_ref(eq, p, 3, pb, mesh, np.zeros((N, dg.n_modes(p), mesh.K)), prm)["out"]
        save(name, run_ref(eq, p, 1, pb, mesh, C.reshape(N, -1, mesh.K), prm, nsteps=ns,
                           limiter=lim, rk=rk))

    # L2 error and CFL inputs
    for name, eq, pb, mesh, prm, p in [
            ("euler_vortex", dg.EULER, PB["euler_vortex"], m_vtx, prm_vec(t=0.3, extra=vtx), 2),
            ("adv_sine", dg.ADVECTION, PB["adv_sine"], m_adv, prm_vec(t=0.2), 3)]:
        C = perturbed_ic(eq, p, pb, mesh, prm_vec(extra=prm[8:]), 5)
        save("l2err_%s_p%d" % (name, p), run_ref(eq, p, 5, pb, mesh, C, prm))
        save("cfl_%s_p%d" % (name, p), run_ref(eq, p, 6, pb, mesh, C, prm))
    print("golden fixtures written to", OUT)


if __name__ == "__main__":
    main()
