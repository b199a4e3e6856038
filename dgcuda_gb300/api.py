"""ctypes binding of include/dg.h (see the package docstring)."""
import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))

ADVECTION, EULER, SHALLOW_WATER, MAXWELL = 0, 1, 2, 3
SSP_RK3, RK4, RK2 = 0, 1, 2
BC_REFLECT, BC_OUTFLOW, BC_INFLOW, BC_TRANSMISSIVE, PERIODIC = -1, -2, -3, -4, 0
PROBLEMS = {
    "none": 0, "adv_sine": 1, "adv_linear": 2, "euler_vortex": 3, "euler_riemann4": 4,
    "euler_supersonic": 5, "sw_hump": 6, "sw_test": 7, "maxwell_plane": 8,
    "euler_cylinder": 9, "euler_lshock": 10, "euler_doublemach": 11, "euler_airfoil": 12,
    "adv_squarehill": 13, "adv_rotatinghill": 14, "adv_spin": 15, "maxwell_cmirror": 16,
    "maxwell_wscatter": 17, "euler_pulse": 18,
}
_NVARS = {ADVECTION: 1, EULER: 4, SHALLOW_WATER: 3, MAXWELL: 3}
_STATUS = ["OK", "BAD_ARG", "BAD_MESH", "NONPHYSICAL", "NAN", "CUDA_ERROR", "TIMEOUT",
           "IO_ERROR", "UNSUPPORTED"]


def n_modes(p):
    return (p + 1) * (p + 2) // 2


def n_vars(eq):
    return _NVARS[eq]


class DGError(RuntimeError):
    def __init__(self, status, msg):
        self.status = status
        name = _STATUS[status] if 0 <= status < len(_STATUS) else str(status)
        super().__init__("%s: %s" % (name, msg))


class Params(C.Structure):
    _fields_ = [("gamma", C.c_double), ("gravity", C.c_double), ("ax", C.c_double),
                ("ay", C.c_double), ("mu", C.c_double), ("eps", C.c_double),
                ("problem", C.c_int), ("limiter", C.c_int), ("cfl", C.c_double),
                ("prm", C.c_double * 8)]


def lib_path():
    return os.path.join(HERE, "libdg_gb300.so")


_LIB = None


def load_library():
    """Load libdg_gb300.so; raises when it has not been built."""
    global _LIB
    if _LIB is None:
        path = lib_path()
        if not os.path.exists(path):
            raise ImportError("libdg_gb300.so not built: run "
                              "`python -c 'import __graft_entry__ as g; g.build()'`")
        _LIB = C.CDLL(path)
        _declare(_LIB)
    return _LIB


_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int)


def _declare(L):
    sigs = {
        "dg_version": (C.c_char_p, []),
        "dg_last_error": (C.c_char_p, []),
        "dg_params_default": (None, [C.POINTER(Params)]),
        "dg_params_for_problem": (C.c_int, [C.POINTER(Params), C.c_int, _ip]),
        "dg_set_velocity_field": (C.c_int, [C.c_void_p, C.c_double, C.c_double, _dp]),
        "dg_get_velocity_field": (C.c_int, [C.c_void_p, _dp]),
        "dg_set_inflow_series": (C.c_int, [C.c_void_p, C.c_int, _dp, _dp, _dp, C.c_double]),
        "dg_mesh_read_pmsh": (C.c_int, [C.c_char_p, C.POINTER(C.c_void_p)]),
        "dg_mesh_write_pmsh": (C.c_int, [C.c_void_p, C.c_char_p]),
        "dg_mesh_read_gmsh": (C.c_int, [C.c_char_p, C.POINTER(C.c_void_p)]),
        "dg_mesh_from_arrays": (C.c_int, [C.c_int, _dp, _ip, C.c_int, _dp, _ip,
                                          C.POINTER(C.c_void_p)]),
        "dg_mesh_get_arrays": (C.c_int, [C.c_void_p, _dp, _ip, _dp, _ip]),
        "dg_mesh_sizes": (C.c_int, [C.c_void_p, _ip, _ip]),
        "dg_mesh_square": (C.c_int, [C.c_int, C.c_int, C.c_double, C.c_double, C.c_double,
                                     C.c_double, C.c_double, C.c_uint64, _ip,
                                     C.POINTER(C.c_void_p)]),
        "dg_mesh_destroy": (None, [C.c_void_p]),
        "dg_solver_create": (C.c_int, [C.c_void_p, C.c_int, C.c_int, C.POINTER(Params), C.c_int,
                                       C.POINTER(C.c_void_p)]),
        "dg_solver_destroy": (None, [C.c_void_p]),
        "dg_solver_sizes": (C.c_int, [C.c_void_p, _ip, _ip, _ip, _ip]),
        "dg_solver_stream": (C.c_void_p, [C.c_void_p]),
        "dg_solver_set_tables": (C.c_int, [C.c_void_p, C.c_int, C.c_int] + [_dp] * 10),
        "dg_init": (C.c_int, [C.c_void_p]),
        "dg_set_state": (C.c_int, [C.c_void_p, _dp]),
        "dg_get_state": (C.c_int, [C.c_void_p, _dp]),
        "dg_set_state_device": (C.c_int, [C.c_void_p, C.c_void_p]),
        "dg_get_state_device": (C.c_int, [C.c_void_p, C.c_void_p]),
        "dg_rhs": (C.c_int, [C.c_void_p, C.c_double, _dp, _dp]),
        "dg_limit": (C.c_int, [C.c_void_p]),
        "dg_step": (C.c_int, [C.c_void_p, C.c_int, C.c_int, C.c_double, _dp]),
        "dg_advance_to": (C.c_int, [C.c_void_p, C.c_double, C.c_int, _dp, _ip]),
        "dg_cfl": (C.c_int, [C.c_void_p, _dp, _dp, _dp]),
        "dg_l2_error": (C.c_int, [C.c_void_p, C.c_double, _dp]),
        "dg_profile_enable": (C.c_int, [C.c_void_p, C.c_int]),
        "dg_profile_get": (C.c_int, [C.c_void_p, C.c_char_p, C.POINTER(C.c_longlong), _dp]),
        "dg_profile_reset": (C.c_int, [C.c_void_p]),
        "dg_kernel_launches": (C.c_longlong, [C.c_void_p]),
        "dg_measure_fp64_peak": (C.c_int, [C.c_int, _dp]),
        "dg_probe_reciprocal": (C.c_int, [C.c_int, C.c_int, _dp, _dp, _dp]),
        "dg_probe_physical": (C.c_int, [C.c_int, C.c_int, _dp, _ip, _ip]),
        "dg_probe_sqrt": (C.c_int, [C.c_int, C.c_int, _dp, _dp, _dp]),
        "dg_eval_vertices": (C.c_int, [C.c_void_p, C.c_int, _dp]),
        "dg_eval_vertices_view": (C.c_int, [C.c_void_p, C.c_int, C.c_int, C.c_double, _dp]),
        "dg_save_checkpoint": (C.c_int, [C.c_void_p, C.c_char_p, C.c_double]),
        "dg_set_tensor_contractions": (C.c_int, [C.c_void_p, C.c_int]),
        "dg_oz_table_image": (C.c_int, [C.c_int, C.c_void_p, C.c_size_t, _dp]),
        "dg_get_tensor_contractions": (C.c_int, [C.c_void_p, _ip]),
        "dg_load_checkpoint": (C.c_int, [C.c_void_p, C.c_char_p, _dp]),
        "dg_set_bathymetry": (C.c_int, [C.c_void_p, _dp]),
        "dg_bathymetry_project": (C.c_int, [C.c_void_p, C.c_int, _dp]),
        "dg_get_bathymetry": (C.c_int, [C.c_void_p, _dp]),
        "dg_autotune": (C.c_int, [C.c_void_p, _ip]),
        "dg_autotune_stage": (C.c_int, [C.c_void_p, _ip, _ip]),
        "dg_batch_create": (C.c_int, [C.c_int, C.POINTER(C.c_void_p), C.POINTER(C.c_void_p)]),
        "dg_batch_blocks": (C.c_int, [C.c_void_p, _ip]),
        "dg_batch_step": (C.c_int, [C.c_void_p, C.c_int, _dp]),
        "dg_batch_autotune": (C.c_int, [C.c_void_p, _ip]),
        "dg_batch_launches": (C.c_longlong, [C.c_void_p]),
        "dg_batch_destroy": (None, [C.c_void_p]),
        "dg_rhs_tl": (C.c_int, [C.c_void_p, C.c_double, _dp, _dp, _dp, _dp]),
        "dg_rhs_adjoint": (C.c_int, [C.c_void_p, C.c_double, _dp, _dp, _dp, _dp]),
        "dg_adjoint_create": (C.c_int, [C.c_void_p, C.c_int, _dp, _dp, C.POINTER(C.c_void_p)]),
        "dg_adjoint_forward": (C.c_int, [C.c_void_p, C.c_int, C.c_double, C.c_int, C.c_int,
                                         C.c_double, _dp]),
        "dg_adjoint_backward": (C.c_int, [C.c_void_p, _dp, _dp, _dp]),
        "dg_adjoint_tangent": (C.c_int, [C.c_void_p, _dp, _dp, _dp]),
        "dg_adjoint_destroy": (None, [C.c_void_p]),
        "dg_adjoint_set_storage": (C.c_int, [C.c_void_p, C.c_int]),
        "dg_adjoint_stored": (C.c_int, [C.c_void_p, _ip]),
    }
    for name, (res, args) in sigs.items():
        fn = getattr(L, name, None)
        if fn is None:
            continue
        fn.restype = res
        fn.argtypes = args


class Batch:
    """Independent problems stepped together (dg_batch): one launch per
    kernel per RK stage for all members, one CUDA graph per ensemble step."""

    def __init__(self, solvers):
        self._L = load_library()
        self.solvers = list(solvers)
        arr = (C.c_void_p * len(self.solvers))(*[s._h.value for s in self.solvers])
        h = C.c_void_p()
        _check(self._L.dg_batch_create(len(self.solvers), arr, C.byref(h)))
        self._h = h

    def step(self, nsteps, t=None):
        tt = np.zeros(len(self.solvers)) if t is None else np.array(t, dtype=np.float64)
        _check(self._L.dg_batch_step(self._h, nsteps, _dptr(tt)))
        return tt

    def blocks(self):
        """(shared block size, element-stage block size of each (order,
        mesh-size) group: 2 (p - 1) + (K >= 16384))."""
        v = np.zeros(7, dtype=np.int32)
        _check(self._L.dg_batch_blocks(self._h, _iptr(v)))
        return int(v[0]), [int(x) for x in v[1:]]

    def autotune(self):
        b = C.c_int()
        _check(self._L.dg_batch_autotune(self._h, C.byref(b)))
        return b.value

    def launches(self):
        return self._L.dg_batch_launches(self._h)

    def close(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            self._L.dg_batch_destroy(h)
            self._h = None

    def __del__(self):
        self.close()


class Adjoint:
    """Discrete adjoint of the shallow-water SSP-RK3 model (dg_adjoint):
    samples of h at receivers, checkpointed reverse sweep."""

    def __init__(self, solver, rx, ry):
        self._L = load_library()
        self.solver = solver
        rx = np.ascontiguousarray(rx, dtype=np.float64)
        ry = np.ascontiguousarray(ry, dtype=np.float64)
        self.nrec = len(rx)
        h = C.c_void_p()
        _check(self._L.dg_adjoint_create(solver._h, self.nrec, _dptr(rx), _dptr(ry), C.byref(h)))
        self._h = h
        self.nsamp = 0

    def forward(self, nsteps, dt, every, ckpt=50, t0=0.0):
        self.nsamp = nsteps // every
        out = np.empty((max(self.nsamp, 1), max(self.nrec, 1)))
        _check(self._L.dg_adjoint_forward(self._h, nsteps, dt, every, ckpt, t0, _dptr(out)))
        return out[:self.nsamp, :self.nrec]

    def set_storage(self, keep_stages):
        """True: keep every step's stage states in device memory when they
        fit (the default; the reverse sweep then recomputes nothing); False:
        the checkpoints only."""
        _check(self._L.dg_adjoint_set_storage(self._h, int(bool(keep_stages))))

    @property
    def stored(self):
        """True when the last forward run kept every stage state."""
        v = np.zeros(1, dtype=np.int32)
        _check(self._L.dg_adjoint_stored(self._h, _iptr(v)))
        return bool(v[0])

    def backward(self, sbar):
        s = self.solver
        sbar = np.ascontiguousarray(sbar, dtype=np.float64).reshape(self.nsamp, self.nrec)
        gu = np.empty(s.shape)
        gb = np.empty((s.n_p, s.K))
        _check(self._L.dg_adjoint_backward(self._h, _dptr(sbar), _dptr(gu), _dptr(gb)))
        return gu, gb

    def tangent(self, du0=None, db=None):
        s = self.solver
        out = np.empty((max(self.nsamp, 1), max(self.nrec, 1)))
        a = None if du0 is None else np.ascontiguousarray(du0, dtype=np.float64).reshape(s.shape)
        b = None if db is None else np.ascontiguousarray(db, dtype=np.float64).reshape(s.n_p, s.K)
        _check(self._L.dg_adjoint_tangent(self._h, None if a is None else _dptr(a),
                                          None if b is None else _dptr(b), _dptr(out)))
        return out[:self.nsamp, :self.nrec]

    def close(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            self._L.dg_adjoint_destroy(h)
            self._h = None

    def __del__(self):
        self.close()


def probe_sqrt(x, device=0):
    """(r, q): the sound speeds' square root and IEEE sqrt on the GPU."""
    L = load_library()
    x = np.ascontiguousarray(x, dtype=np.float64)
    r, q = np.empty_like(x), np.empty_like(x)
    _check(L.dg_probe_sqrt(device, len(x), _dptr(x), _dptr(r), _dptr(q)))
    return r, q


def probe_physical(U, device=0):
    """(fast, exact) decisions of the Euler positivity test for states U of
    shape (n, 4) on the GPU: the single-precision filter and the FP64 test."""
    L = load_library()
    U = np.ascontiguousarray(U, dtype=np.float64).reshape(-1, 4)
    n = U.shape[0]
    fast, exact = np.zeros(n, dtype=np.int32), np.zeros(n, dtype=np.int32)
    _check(L.dg_probe_physical(device, n, _dptr(U), _iptr(fast), _iptr(exact)))
    return fast.astype(bool), exact.astype(bool)


def params_for_problem(problem):
    """(Params, scheme): the defaults with the reference problem's own
    settings (limiter, Mach, angle, velocity, g) and its time integrator."""
    L = load_library()
    if isinstance(problem, str):
        problem = PROBLEMS[problem]
    prm = Params()
    sc = np.zeros(1, dtype=np.int32)
    _check(L.dg_params_for_problem(C.byref(prm), int(problem), _iptr(sc)))
    return prm, int(sc[0])


def probe_reciprocal(x, device=0):
    """(rcp(x), 1/x) computed on the device: the flux kernels' reciprocal and
    IEEE division."""
    L = load_library()
    x = np.ascontiguousarray(x, dtype=np.float64)
    r, q = np.empty_like(x), np.empty_like(x)
    _check(L.dg_probe_reciprocal(device, x.size, _dptr(x), _dptr(r), _dptr(q)))
    return r, q


def oz_table_image(p):
    """(words uint32[2240, 2], colexp int32[3, 16], dense float64[5, 16, 16])
    of the tensor-core digit tables of order p: the digit words, the column
    exponents and the tables they were split from (host-built; no GPU
    needed)."""
    L = load_library()
    buf = np.zeros(18176 // 4, dtype=np.uint32)
    dense = np.zeros((5, 16, 16))
    _check(L.dg_oz_table_image(p, buf.ctypes.data_as(C.c_void_p), buf.nbytes, _dptr(dense)))
    return (buf[:4480].reshape(2240, 2).copy(),
            buf[4480:4528].view(np.int32).reshape(3, 16).copy(), dense)


def measure_fp64_peak(device=0):
    """FP64 FMA throughput of the GPU in TFLOP/s."""
    L = load_library()
    v = C.c_double()
    _check(L.dg_measure_fp64_peak(device, C.byref(v)))
    return v.value


def _check(st):
    if st != 0:
        raise DGError(st, load_library().dg_last_error().decode())


def _dptr(a):
    return a.ctypes.data_as(_dp)


def _iptr(a):
    return a.ctypes.data_as(_ip)


class Mesh:
    """A .pmsh triangle mesh (host object)."""

    def __init__(self, handle):
        self._h = C.c_void_p(handle) if not isinstance(handle, C.c_void_p) else handle
        self._L = load_library()
        K, S = C.c_int(), C.c_int()
        _check(self._L.dg_mesh_sizes(self._h, C.byref(K), C.byref(S)))
        self.K, self.S = K.value, S.value

    @classmethod
    def read_mesh(cls, path):
        """Read a .pmsh file (main.cu:205-277)."""
        L = load_library()
        h = C.c_void_p()
        _check(L.dg_mesh_read_pmsh(os.fsencode(path), C.byref(h)))
        return cls(h)

    @classmethod
    def read_gmsh(cls, path):
        """Gmsh ASCII 2.x .msh, converted as genmesh.py converts it."""
        L = load_library()
        h = C.c_void_p()
        _check(L.dg_mesh_read_gmsh(os.fsencode(path), C.byref(h)))
        return cls(h)

    @classmethod
    def square(cls, nx, ny, box=(0.0, 1.0, 0.0, 1.0), jitter=0.0, seed=0,
               bc=(PERIODIC, PERIODIC, PERIODIC, PERIODIC)):
        L = load_library()
        h = C.c_void_p()
        b = np.asarray(bc, dtype=np.int32)
        _check(L.dg_mesh_square(nx, ny, box[0], box[1], box[2], box[3], jitter, seed, _iptr(b),
                                C.byref(h)))
        return cls(h)

    @classmethod
    def from_arrays(cls, V, elem_sides, side_xy, side_elems):
        L = load_library()
        V = np.ascontiguousarray(V, dtype=np.float64)
        es = np.ascontiguousarray(elem_sides, dtype=np.int32)
        sxy = np.ascontiguousarray(side_xy, dtype=np.float64)
        se = np.ascontiguousarray(side_elems, dtype=np.int32)
        K, S = V.shape[-1], sxy.shape[-1]
        h = C.c_void_p()
        _check(L.dg_mesh_from_arrays(K, _dptr(V), _iptr(es), S, _dptr(sxy), _iptr(se),
                                     C.byref(h)))
        return cls(h)

    def arrays(self):
        """(V[6,K], elem_sides[3,K], side_xy[4,S], side_elems[4,S]) in .pmsh column order."""
        V = np.empty((6, self.K))
        es = np.empty((3, self.K), dtype=np.int32)
        sxy = np.empty((4, self.S))
        se = np.empty((4, self.S), dtype=np.int32)
        _check(self._L.dg_mesh_get_arrays(self._h, _dptr(V), _iptr(es), _dptr(sxy), _iptr(se)))
        return V, es, sxy, se

    def write(self, path):
        _check(self._L.dg_mesh_write_pmsh(self._h, os.fsencode(path)))

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            self._L.dg_mesh_destroy(h)
            self._h = None


class Solver:
    """One RK-DG problem on one GPU (wraps dg_solver)."""

    def __init__(self, mesh, eq, p, params=None, device=0, **kw):
        self._L = load_library()
        prm = Params()
        self._L.dg_params_default(C.byref(prm))
        if params is not None:
            prm = params
        for k, v in kw.items():
            if k == "problem" and isinstance(v, str):
                v = PROBLEMS[v]
            if k == "prm":
                for i, x in enumerate(v):
                    prm.prm[i] = x
                continue
            setattr(prm, k, v)
        self.params = prm
        self.mesh = mesh
        h = C.c_void_p()
        _check(self._L.dg_solver_create(mesh._h, eq, p, C.byref(prm), device, C.byref(h)))
        self._h = h
        N, npm, K, S = C.c_int(), C.c_int(), C.c_int(), C.c_int()
        _check(self._L.dg_solver_sizes(h, C.byref(N), C.byref(npm), C.byref(K), C.byref(S)))
        self.N, self.n_p, self.K, self.S = N.value, npm.value, K.value, S.value
        self.eq, self.p = eq, p

    @property
    def shape(self):
        return (self.N, self.n_p, self.K)

    def set_tables(self, basis, grad_x, grad_y, side, vertex, w, r1, r2, r_oned, w_oned):
        arrs = [np.ascontiguousarray(a, dtype=np.float64) for a in
                (basis, grad_x, grad_y, side, vertex, w, r1, r2, r_oned, w_oned)]
        _check(self._L.dg_solver_set_tables(self._h, len(arrs[5]), len(arrs[8]),
                                            *[_dptr(a) for a in arrs]))

    def init_conditions(self):
        _check(self._L.dg_init(self._h))

    def set_state(self, c):
        c = np.ascontiguousarray(c, dtype=np.float64).reshape(self.shape)
        _check(self._L.dg_set_state(self._h, _dptr(c)))

    def get_state(self, out=None):
        """State in the reference layout [var][mode][elem]; fills `out` (a
        C-contiguous float64 array, e.g. over pinned memory) when given."""
        if out is None:
            out = np.empty(self.shape)
        elif (out.dtype != np.float64 or not out.flags["C_CONTIGUOUS"]
              or out.size != self.N * self.n_p * self.K):
            raise ValueError("out must be a C-contiguous float64 array of the state's size")
        _check(self._L.dg_get_state(self._h, _dptr(out)))
        return out

    def eval_rhs(self, c, t=0.0):
        c = np.ascontiguousarray(c, dtype=np.float64).reshape(self.shape)
        out = np.empty(self.shape)
        _check(self._L.dg_rhs(self._h, t, _dptr(c), _dptr(out)))
        return out

    def limit_c(self):
        _check(self._L.dg_limit(self._h))

    def step(self, nsteps, scheme=SSP_RK3, t=0.0, dt=0.0):
        tt = C.c_double(t)
        _check(self._L.dg_step(self._h, nsteps, scheme, dt, C.byref(tt)))
        return tt.value

    def advance_to(self, T, scheme=SSP_RK3, t=0.0):
        tt, n = C.c_double(t), C.c_int()
        _check(self._L.dg_advance_to(self._h, T, scheme, C.byref(tt), C.byref(n)))
        return tt.value, n.value

    def time_integrate_rk4(self, nsteps, t=0.0):
        return self.step(nsteps, RK4, t)

    def time_integrate_rk2(self, nsteps, t=0.0):
        return self.step(nsteps, RK2, t)

    def time_integrate_ssp_rk3(self, nsteps, t=0.0):
        return self.step(nsteps, SSP_RK3, t)

    def cfl(self):
        dt, lam, dmin = C.c_double(), C.c_double(), C.c_double()
        _check(self._L.dg_cfl(self._h, C.byref(dt), C.byref(lam), C.byref(dmin)))
        return dt.value, lam.value, dmin.value

    def eval_error_L2(self, t):
        err = np.empty(self.N)
        _check(self._L.dg_l2_error(self._h, t, _dptr(err)))
        return err

    def eval_u(self, var):
        """Values of variable `var` at the vertices V1, V2, V3 of every element,
        shape (3, K) (eval_u, conserv_kernels.cu:1284)."""
        out = np.empty((3, self.K))
        _check(self._L.dg_eval_vertices(self._h, var, _dptr(out)))
        return out

    @property
    def tensor_contractions(self):
        """True when the fused element stage runs its contractions on the
        tensor cores (Euler, p = 1..4; on by default from p = 2)."""
        v = np.zeros(1, dtype=np.int32)
        _check(self._L.dg_get_tensor_contractions(self._h, _iptr(v)))
        return bool(v[0])

    @tensor_contractions.setter
    def tensor_contractions(self, on):
        _check(self._L.dg_set_tensor_contractions(self._h, int(bool(on))))

    def set_velocity_field(self, ax, ay, grad=None):
        """Advection velocity a(x, y) = (ax, ay) + grad (x, y), grad =
        (dax/dx, dax/dy, day/dx, day/dy) or None (the problem's get_velocity,
        advection.cu:12)."""
        g = None if grad is None else np.ascontiguousarray(grad, dtype=np.float64)
        _check(self._L.dg_set_velocity_field(self._h, float(ax), float(ay),
                                             None if g is None else _dptr(g)))

    def velocity_field(self):
        """(ax, ay, grad[4], CFL wave speed)."""
        out = np.zeros(7)
        _check(self._L.dg_get_velocity_field(self._h, _dptr(out)))
        return out[0], out[1], out[2:6].copy(), out[6]

    def set_inflow_series(self, amp, omega, phase, t0=0.0):
        """Inflow pressure series of euler_pulse: p(t) = 1 + sum amp_k
        cos(omega_k (t + t0) + phase_k) (the tube / trumpet inflow)."""
        a, w, f = (np.ascontiguousarray(v, dtype=np.float64) for v in (amp, omega, phase))
        if not (len(a) == len(w) == len(f)):
            raise ValueError("amp, omega and phase differ in length")
        _check(self._L.dg_set_inflow_series(self._h, len(a), _dptr(a), _dptr(w), _dptr(f),
                                            float(t0)))

    def save_checkpoint(self, path, t):
        """Binary state (+ bed) with the time t and a checksum."""
        _check(self._L.dg_save_checkpoint(self._h, os.fsencode(path), t))

    def load_checkpoint(self, path):
        """Restore a checkpoint written for this equation, order and mesh;
        returns its time."""
        t = np.zeros(1)
        _check(self._L.dg_load_checkpoint(self._h, os.fsencode(path), _dptr(t)))
        return float(t[0])

    def plot_exact(self, var, t):
        """The problem's exact solution of `var` at the vertices at time t,
        shape (3, K) (plot_exact, conserv_kernels.cu:1310)."""
        out = np.empty((3, self.K))
        _check(self._L.dg_eval_vertices_view(self._h, var, 1, t, _dptr(out)))
        return out

    def plot_error(self, var, t):
        """Solution minus exact solution of `var` at the vertices, shape (3, K)
        (plot_error, conserv_kernels.cu:1334)."""
        out = np.empty((3, self.K))
        _check(self._L.dg_eval_vertices_view(self._h, var, 2, t, _dptr(out)))
        return out

    def set_bathymetry(self, b):
        """Shallow-water bed modes [mode][elem] (.pmsh order) or None (flat)."""
        if b is None:
            _check(self._L.dg_set_bathymetry(self._h, None))
            return
        b = np.ascontiguousarray(b, dtype=np.float64).reshape(self.n_p, self.K)
        _check(self._L.dg_set_bathymetry(self._h, _dptr(b)))

    def get_bathymetry(self):
        b = np.empty((self.n_p, self.K))
        _check(self._L.dg_get_bathymetry(self._h, _dptr(b)))
        return b

    def bathymetry_project(self, kind, prm=(0.0, 0.0, 0.0)):
        """kind: 'flat', 'sine' (A, kx, ky) or 'linear' (b0, bx, by)."""
        k = {"flat": 0, "sine": 1, "linear": 2}[kind]
        a = np.ascontiguousarray(prm, dtype=np.float64)
        _check(self._L.dg_bathymetry_project(self._h, k, _dptr(a)))

    def blocks(self):
        """(shared block size, element-stage block size of each (order,
        mesh-size) group: 2 (p - 1) + (K >= 16384))."""
        v = np.zeros(7, dtype=np.int32)
        _check(self._L.dg_batch_blocks(self._h, _iptr(v)))
        return int(v[0]), [int(x) for x in v[1:]]

    def autotune(self):
        b = C.c_int()
        _check(self._L.dg_autotune(self._h, C.byref(b)))
        return b.value

    def autotune_stage(self):
        """(block size, threads per element): the stage kernels' block size
        and, where the solver has both, the element stage (1: FP64 FMAs, one
        thread per element; 2: tensor cores, a lane quad per two elements),
        chosen by timing SSP-RK3 steps; the state is restored."""
        b, tpe = C.c_int(), C.c_int()
        _check(self._L.dg_autotune_stage(self._h, C.byref(b), C.byref(tpe)))
        return b.value, tpe.value

    def rhs_tl(self, c, dc, db=None, t=0.0):
        """Tangent-linear right-hand side (shallow water)."""
        c = np.ascontiguousarray(c, dtype=np.float64).reshape(self.shape)
        dc = np.ascontiguousarray(dc, dtype=np.float64).reshape(self.shape)
        out = np.empty(self.shape)
        dbp = None
        if db is not None:
            db = np.ascontiguousarray(db, dtype=np.float64).reshape(self.n_p, self.K)
            dbp = _dptr(db)
        _check(self._L.dg_rhs_tl(self._h, t, _dptr(c), _dptr(dc), dbp, _dptr(out)))
        return out

    def rhs_adjoint(self, c, lbar, t=0.0):
        """(dL/du)^T lbar and (dL/db)^T lbar (shallow water)."""
        c = np.ascontiguousarray(c, dtype=np.float64).reshape(self.shape)
        lbar = np.ascontiguousarray(lbar, dtype=np.float64).reshape(self.shape)
        cb = np.empty(self.shape)
        bb = np.empty((self.n_p, self.K))
        _check(self._L.dg_rhs_adjoint(self._h, t, _dptr(c), _dptr(lbar), _dptr(cb), _dptr(bb)))
        return cb, bb

    def stream(self):
        return self._L.dg_solver_stream(self._h)

    def profile(self, on=True):
        _check(self._L.dg_profile_enable(self._h, 1 if on else 0))

    def profile_reset(self):
        _check(self._L.dg_profile_reset(self._h))

    def profile_get(self, kernel):
        n, ms = C.c_longlong(), C.c_double()
        _check(self._L.dg_profile_get(self._h, kernel.encode(), C.byref(n), C.byref(ms)))
        return n.value, ms.value

    def kernel_launches(self):
        return self._L.dg_kernel_launches(self._h)

    def close(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            self._L.dg_solver_destroy(h)
            self._h = None

    def __del__(self):
        self.close()

