"""ctypes wrapper and build recipe of the C oracle (dg_oracle.c).

Test infrastructure only: the reference results of the parity tests and the timed
CPU baseline of bench.py.  ``build()`` compiles dg_oracle.c with OpenMP into
oracle/_build/liboracle.so.
"""
import ctypes as C
import os
import shutil
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "liboracle.so")
SRC = os.path.join(HERE, "dg_oracle.c")
TABLES = os.path.join(os.path.dirname(HERE), "dgcuda_gb300", "csrc", "dg_tables_data.h")

NV = {0: 1, 1: 4, 2: 3, 3: 3}


def build():
    os.makedirs(BUILD, exist_ok=True)
    newest = max(os.path.getmtime(SRC), os.path.getmtime(TABLES))
    if os.path.exists(LIB) and os.path.getmtime(LIB) >= newest:
        return LIB
    cc = shutil.which("gcc") or "cc"
    # no contraction of a*b+c into FMAs the source does not write: the same
    # bits on x86 and Arm
    cmd = [cc, "-O2", "-ffp-contract=off", "-fopenmp", "-shared", "-fPIC", SRC, "-o", LIB, "-lm"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + r.stderr)
    return LIB


_L = None
_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int)


def lib():
    global _L
    if _L is None:
        build()
        L = C.CDLL(LIB)
        L.or_create.restype = C.c_void_p
        L.or_create.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int, _dp, _ip, _dp, _ip, _dp,
                                C.c_int]
        L.or_destroy.argtypes = [C.c_void_p]
        L.or_set_tables.argtypes = [C.c_void_p, C.c_int, C.c_int] + [_dp] * 10
        L.or_rhs.argtypes = [C.c_void_p, _dp, C.c_double, _dp]
        L.or_limit.argtypes = [C.c_void_p, _dp]
        L.or_init.argtypes = [C.c_void_p, _dp]
        L.or_l2err.argtypes = [C.c_void_p, _dp, C.c_double, _dp]
        L.or_lambda.argtypes = [C.c_void_p, _dp, C.c_double, _dp, _dp]
        L.or_step.argtypes = [C.c_void_p, _dp, C.c_int, C.c_int, C.c_int, C.c_double, C.c_double,
                              C.c_double, _dp]
        L.or_min_diameter.restype = C.c_double
        L.or_min_diameter.argtypes = [C.c_void_p]
        L.or_flattened.argtypes = [C.c_void_p]
        L.or_set_threads.argtypes = [C.c_int]
        L.or_get_tables.argtypes = [C.c_void_p, _dp]
        L.or_mesh_square_sizes.argtypes = [C.c_int, C.c_int, _ip, _ip, _ip]
        L.or_mesh_square.argtypes = [C.c_int, C.c_int, C.c_double, C.c_double, C.c_double,
                                     C.c_double, C.c_double, C.c_ulonglong, _ip, _dp, _ip, _dp,
                                     _ip]
        L.or_set_bathymetry.argtypes = [C.c_void_p, _dp]
        L.or_set_field.argtypes = [C.c_void_p, C.c_double, C.c_double, _dp]
        L.or_set_series.argtypes = [C.c_void_p, C.c_int, _dp, _dp, _dp, C.c_double]
        _L = L
    return _L


def _d(a):
    return a.ctypes.data_as(_dp)


def prm_vec(t=0.0, gamma=1.4, ax=1.0, ay=0.5, mu=1.0, eps=1.0, g=9.8, cfl=0.5, extra=()):
    """Parameter vector: 0 t, 1 gamma, 2 ax, 3 ay, 4 mu, 5 eps, 6 g, 7 cfl, 8.. problem."""
    v = np.zeros(16)
    v[:8] = [t, gamma, ax, ay, mu, eps, g, cfl]
    for i, x in enumerate(extra):
        v[8 + i] = x
    return v


class Oracle:
    def __init__(self, eq, p, V, es, sxy, se, prm, problem=0):
        L = lib()
        self.L = L
        self.eq, self.p = int(eq), int(p)
        self.N, self.np = NV[self.eq], (p + 1) * (p + 2) // 2
        V = np.ascontiguousarray(V, dtype=np.float64)
        es = np.ascontiguousarray(es, dtype=np.int32)
        sxy = np.ascontiguousarray(sxy, dtype=np.float64)
        se = np.ascontiguousarray(se, dtype=np.int32)
        self.K, self.S = V.shape[-1], sxy.shape[-1]
        self.prm = np.ascontiguousarray(prm, dtype=np.float64)
        self.h = L.or_create(self.eq, self.p, self.K, self.S, _d(V),
                             es.ctypes.data_as(_ip), _d(sxy), se.ctypes.data_as(_ip),
                             _d(self.prm), int(problem))
        if not self.h:
            raise ValueError("or_create failed")

    @classmethod
    def from_mesh(cls, mesh, eq, p, prm, problem=0):
        V, es, sxy, se = mesh.arrays()
        return cls(eq, p, V, es, sxy, se, prm, problem)

    def set_tables(self, tab):
        """tab: the flat reference tabulation (mode-4 golden output)."""
        np_, nq, n1 = self.np, self.nq_for(), self.p + 1
        tab = np.asarray(tab, dtype=np.float64)
        sizes = [np_ * nq, np_ * nq, np_ * nq, 3 * np_ * n1, 3 * np_, nq, nq, nq, n1, n1]
        parts, o = [], 0
        for s in sizes:
            parts.append(np.ascontiguousarray(tab[o:o + s]))
            o += s
        self._tab = parts
        rc = self.L.or_set_tables(self.h, nq, n1, *[_d(a) for a in parts])
        if rc:
            raise ValueError("table size mismatch")

    def set_bathymetry(self, b):
        """Bed modes [mode][elem] (shallow water), or None for flat."""
        if b is None:
            self.L.or_set_bathymetry(self.h, None)
        else:
            self._bathy = np.ascontiguousarray(b, dtype=np.float64).reshape(self.np, self.K)
            self.L.or_set_bathymetry(self.h, _d(self._bathy))

    def set_field(self, ax, ay, grad=None):
        """Advection velocity a = (ax, ay) + grad (x, y); grad = (dax/dx,
        dax/dy, day/dx, day/dy) or None for a constant velocity."""
        self._grad = None if grad is None else np.ascontiguousarray(grad, dtype=np.float64)
        self.L.or_set_field(self.h, float(ax), float(ay),
                            None if self._grad is None else _d(self._grad))

    def set_series(self, amp, omega, phase, t0=0.0):
        """Inflow pressure series of the pulse problem."""
        self._ser = [np.ascontiguousarray(a, dtype=np.float64) for a in (amp, omega, phase)]
        if self.L.or_set_series(self.h, len(self._ser[0]), *[_d(a) for a in self._ser],
                                float(t0)):
            raise ValueError("at most 16 series terms")

    def tables(self):
        """The oracle's tabulation in the reference's flat layout."""
        npm, nq, n1 = self.np, self.nq_for(), self.p + 1
        out = np.empty(3 * npm * nq + 3 * npm * n1 + 3 * npm + 3 * nq + 2 * n1)
        n = self.L.or_get_tables(self.h, _d(out))
        return out[:n]

    def nq_for(self):
        return [1, 3, 6, 12, 16, 25][self.p]

    def shape(self):
        return (self.N, self.np, self.K)

    def rhs(self, Cin, t=0.0):
        Cin = np.ascontiguousarray(Cin, dtype=np.float64).reshape(self.shape())
        out = np.empty(self.shape())
        self.L.or_rhs(self.h, _d(Cin), t, _d(out))
        return out

    def limit(self, Cin):
        c = np.array(Cin, dtype=np.float64).reshape(self.shape())
        self.L.or_limit(self.h, _d(c))
        return c

    def init(self):
        c = np.empty(self.shape())
        self.L.or_init(self.h, _d(c))
        return c

    def l2err2(self, Cin, t):
        Cin = np.ascontiguousarray(Cin, dtype=np.float64).reshape(self.shape())
        out = np.empty(self.N)
        self.L.or_l2err(self.h, _d(Cin), t, _d(out))
        return out

    def lambdas(self, Cin, t=0.0):
        Cin = np.ascontiguousarray(Cin, dtype=np.float64).reshape(self.shape())
        lam = np.empty(self.K)
        mr = C.c_double()
        self.L.or_lambda(self.h, _d(Cin), t, _d(lam), C.byref(mr))
        return lam, mr.value

    def step(self, Cin, nsteps, scheme, limiter, cfl, t=0.0, fixed_dt=0.0, endtime=0.0):
        c = np.array(Cin, dtype=np.float64).reshape(self.shape())
        tt = C.c_double(t)
        n = self.L.or_step(self.h, _d(c), nsteps, scheme, limiter, cfl, fixed_dt, endtime,
                           C.byref(tt))
        return c, tt.value, n

    def flattened(self):
        return self.L.or_flattened(self.h)

    def __del__(self):
        if getattr(self, "h", None):
            self.L.or_destroy(self.h)
            self.h = None


def mesh_square(nx, ny, box=(0.0, 1.0, 0.0, 1.0), jitter=0.0, seed=0, bc=(0, 0, 0, 0)):
    """The jittered square-split mesh of the benchmark configurations, built
    by the oracle (same arrays as the library's dg_mesh_square): V[6,K],
    elem_sides[3,K], side_xy[4,S], side_elems[4,S] in .pmsh column order."""
    L = lib()
    b = np.ascontiguousarray(bc, dtype=np.int32)
    K, S = C.c_int(), C.c_int()
    if L.or_mesh_square_sizes(nx, ny, b.ctypes.data_as(_ip), C.byref(K), C.byref(S)):
        raise ValueError("bad mesh size")
    V = np.empty((6, K.value))
    es = np.empty((3, K.value), dtype=np.int32)
    sxy = np.empty((4, S.value))
    se = np.empty((4, S.value), dtype=np.int32)
    rc = L.or_mesh_square(nx, ny, box[0], box[1], box[2], box[3], jitter, seed,
                          b.ctypes.data_as(_ip), _d(V), es.ctypes.data_as(_ip), _d(sxy),
                          se.ctypes.data_as(_ip))
    if rc:
        raise ValueError("or_mesh_square failed (%d)" % rc)
    return V, es, sxy, se


def set_threads(n):
    lib().or_set_threads(int(n))
