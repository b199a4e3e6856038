"""Seeded shallow-water ensembles (independent problems stepped together).

The ensemble of the batched benchmark: `n` problems on the unit square with
reflecting walls, each a jittered square-split mesh whose triangle count is
log-uniform in [tri_min, tri_max] (n_side = round(sqrt(T / 2))), order p
uniform in {1, 2, 3}, still water with a Gaussian hump
h = 1 + A exp(-|x - x0|^2 / sigma^2) (A ~ U[0.05, 0.2], sigma ~ U[0.05, 0.15],
x0 uniform in [0.2, 0.8]^2), bed flat or b = 0.1 sin(2 pi x) sin(2 pi y)
(even odds), g = 9.81, Rusanov flux, SSP-RK3.
"""
import numpy as np

from .api import Mesh, Solver, SHALLOW_WATER, BC_REFLECT

WALLS = (BC_REFLECT, BC_REFLECT, BC_REFLECT, BC_REFLECT)


def ensemble_specs(n, seed, tri_min=1000, tri_max=200000):
    rng = np.random.default_rng(seed)
    specs = []
    for i in range(n):
        T = float(np.exp(rng.uniform(np.log(tri_min), np.log(tri_max))))
        side = max(3, int(round(np.sqrt(T / 2.0))))
        specs.append(dict(
            side=side, p=int(rng.integers(1, 4)), A=float(rng.uniform(0.05, 0.2)),
            sigma=float(rng.uniform(0.05, 0.15)), x0=float(rng.uniform(0.2, 0.8)),
            y0=float(rng.uniform(0.2, 0.8)), bed="sine" if rng.uniform() < 0.5 else "flat",
            seed=int(rng.integers(0, 2 ** 31))))
    return specs


def build_member(spec, device=0, cfl=0.3):
    mesh = Mesh.square(spec["side"], spec["side"], jitter=0.1, seed=spec["seed"], bc=WALLS)
    s = Solver(mesh, SHALLOW_WATER, spec["p"], device=device, problem="sw_hump", gravity=9.81,
               cfl=cfl, prm=(1.0, spec["A"], spec["sigma"], spec["x0"], spec["y0"]))
    if spec["bed"] == "sine":
        s.bathymetry_project("sine", (0.1, 1.0, 1.0))
    s.init_conditions()
    return s


def dofs(solvers):
    return sum(s.N * s.n_p * s.K for s in solvers)
