/* dg.h -- C ABI of the GB300 RK-DG solver (dgcuda_gb300).
 *
 * A drop-in for the RK-DG hot path of DGCUDA (src/2d/conservation): read a
 * .pmsh triangle mesh, pick an equation module and order p, project the
 * initial condition, evaluate the DG right-hand side, step with SSP-RK3 (or
 * the reference's RK4 / midpoint RK2) with the optional slope limiter, and
 * measure the L2 error.  Every call returns a dg_status and never exits the
 * process; dg_last_error() gives the message of the last failure on the
 * calling thread.
 *
 * Data layout at the boundary is the reference's: a state array is
 * C[var][mode][elem] (conserv_kernels.cu:224), elements and sides in .pmsh
 * order.  Internally elements are renumbered along a space-filling curve;
 * the permutation is applied at the boundary.
 *
 * All pointers are plain host pointers unless a name says _device.
 */
#ifndef DG_GB300_H
#define DG_GB300_H
#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
  DG_OK = 0,
  DG_BAD_ARG = 1,
  DG_BAD_MESH = 2,     /* replaces read_mesh's printf + exit (main.cu:242-245, 272-275) */
  DG_NONPHYSICAL = 3,
  DG_NAN = 4,          /* replaces the NaN-dt early return (time_integrator.cu:219-223) */
  DG_CUDA_ERROR = 5,   /* replaces checkCudaError's exit(-1) (main.cu:196-203) */
  DG_TIMEOUT = 6,
  DG_IO_ERROR = 7,
  DG_UNSUPPORTED = 8
} dg_status;

/* equation modules (src/2d/conservation/{advection,euler,shallowwater,maxwells}) */
typedef enum { DG_ADVECTION = 0, DG_EULER = 1, DG_SHALLOW_WATER = 2, DG_MAXWELL = 3 } dg_equation;

/* time integrators: the reference's RK4 = 1 and RK2 = 2 (main.cu:35-36), plus SSP-RK3 */
typedef enum { DG_SSP_RK3 = 0, DG_RK4 = 1, DG_RK2 = 2 } dg_scheme;

/* problem plugins: initial condition, boundary ghost states and exact
 * solution (the reference's per-problem U0 / U_inflow / U_outflow /
 * U_reflection / U_exact device functions, e.g. supersonic.cu:27-97) */
typedef enum {
  DG_PB_NONE = 0,           /* state set by the caller; ghost states zero */
  DG_PB_ADV_SINE = 1,       /* u0 = sin(2 pi x) sin(2 pi y), exact = translated */
  DG_PB_ADV_LINEAR = 2,     /* u0 = x - y (advection/exact/exact.cu) */
  DG_PB_EULER_VORTEX = 3,   /* isentropic vortex: prm beta, x0, y0, uinf, vinf, L */
  DG_PB_EULER_RIEMANN4 = 4, /* four-quadrant Riemann problem on [0,1]^2 */
  DG_PB_EULER_SUPERSONIC = 5, /* supersonic vortex (euler/supersonic/supersonic.cu) */
  DG_PB_SW_HUMP = 6,        /* still water hump: prm h0, A, sigma, x0, y0 */
  DG_PB_SW_TEST = 7,        /* shallowwater/test/test.cu hump */
  DG_PB_MAXWELL_PLANE = 8,  /* plane TM wave along x */
  DG_PB_EULER_CYLINDER = 9, /* uniform flow past a cylinder at the origin (euler/cylinder):
                               prm[0] Mach (0: 0.38); walls are the circle through the point */
  DG_PB_EULER_LSHOCK = 10,  /* uniform flow with slip walls (euler/lshock): prm[0] Mach (0: 2) */
  DG_PB_EULER_DOUBLEMACH = 11, /* double Mach reflection (euler/doublemach): a Mach 10 shock
                               at 60 degrees; the wall reflects from x = 1/6 on */
  DG_PB_EULER_AIRFOIL = 12, /* uniform flow (euler/airfoil): prm[0] Mach (0: 0.98), prm[1]
                               angle of attack in degrees (0: 5) */
  DG_PB_ADV_SQUAREHILL = 13, /* box (-0.8,-0.2) x (-0.5,0.1) translated by a t
                               (advection/rotatinghill/squarehill.cu); inflow 0 */
  DG_PB_ADV_ROTATINGHILL = 14, /* Gaussian hill carried by the rotation (-2 pi y, 2 pi x)
                               (advection/rotatinghill); the problem sets that velocity */
  DG_PB_ADV_SPIN = 15,      /* advection/spin: its hill and rotation (with pi = 3.14159);
                               inflow 0 */
  DG_PB_MAXWELL_CMIRROR = 16, /* maxwells/cmirror: rest; inflow E_z = 2 sin(20 pi t) for
                               t <= 1/20 */
  DG_PB_MAXWELL_WSCATTER = 17, /* maxwells/wscatter: rest; inflow E_z = sin(2 pi t) through
                               |y| < 0.15 for t < 1/2 */
  DG_PB_EULER_PULSE = 18    /* euler/tube and euler/trumpet: gas at rest; inflow and outflow
                               the pressure series of dg_set_inflow_series */
} dg_problem;

/* boundary codes in the .pmsh right-element column (genmesh.py:166-174) */
#define DG_BC_REFLECT (-1)
#define DG_BC_OUTFLOW (-2)
#define DG_BC_INFLOW (-3)
#define DG_BC_TRANSMISSIVE (-4) /* new: ghost = interior trace */

typedef struct {
  double gamma;   /* Euler ratio of specific heats (get_GAMMA, supersonic.cu:105) */
  double gravity; /* shallow water g (the reference hard-codes 9.8, shallowwater.cu:7) */
  double ax, ay;  /* advection velocity (get_velocity, exact.cu:34-37) */
  double mu, eps; /* Maxwell material constants (get_mu/get_eps, cmirror.cu) */
  int problem;    /* dg_problem */
  int limiter;    /* 1 = Barth-Jespersen limiter (limit_c, conserv_kernels.cu:640) */
  double cfl;     /* dt = cfl * d_min / lambda_max / (2p + 1) (time_integrator.cu:217) */
  double prm[8];  /* problem parameters, see dg_problem */
} dg_params;

typedef struct dg_mesh dg_mesh;
typedef struct dg_solver dg_solver;

const char *dg_version(void);
const char *dg_last_error(void);
/* fills *p with the defaults: gamma 1.4, g 9.81, a = (1, 0.5), mu = eps = 1,
 * cfl 0.3, limiter off, problem DG_PB_NONE */
void dg_params_default(dg_params *p);
/* the defaults, then the reference problem's own settings (its limiter,
 * Mach number, angle, velocity, g); *scheme (may be NULL) receives its time
 * integrator (DG_RK4 or DG_RK2), the problem file's time_integrator global */
dg_status dg_params_for_problem(dg_params *p, int problem, int *scheme);

/* ---- meshes (host only; no GPU needed) ---------------------------------
 * replaces read_mesh (main.cu:205-277) and genmesh.py's .pmsh writer
 * (genmesh.py:286-313) */
dg_status dg_mesh_read_pmsh(const char *path, dg_mesh **out);
dg_status dg_mesh_write_pmsh(const dg_mesh *m, const char *path);
/* Gmsh ASCII 2.x .msh -> mesh, as genmesh.py converts it (genmesh.py:13-315):
 * triangles in file order, sides in first-visit order, boundary sides first
 * by code; line physical tags 10000/20000/30000 -> -1/-2/-3 (40000 -> -4 is
 * an addition).  Writing the result with dg_mesh_write_pmsh gives the
 * .pmsh genmesh.py writes. */
dg_status dg_mesh_read_gmsh(const char *path, dg_mesh **out);
/* arrays in .pmsh column order: V = 6*K doubles as V1x[K],V1y[K],V2x[K],
 * V2y[K],V3x[K],V3y[K]; elem_sides = 3*K ints s1[K],s2[K],s3[K];
 * side_xy = 4*S doubles x1[S],y1[S],x2[S],y2[S]; side_elems = 4*S ints
 * left[S],right[S],left_side[S],right_side[S] */
dg_status dg_mesh_from_arrays(int K, const double *V, const int *elem_sides, int S,
                              const double *side_xy, const int *side_elems, dg_mesh **out);
dg_status dg_mesh_get_arrays(const dg_mesh *m, double *V, int *elem_sides, double *side_xy,
                             int *side_elems);
dg_status dg_mesh_sizes(const dg_mesh *m, int *K, int *S);
/* nx x ny squares on [x0,x1]x[y0,y1], each cut along the (0,0)-(1,1)
 * diagonal into two CCW triangles; interior vertices jittered uniformly by
 * +-jitter*h (splitmix64, seed).  bc = {left, right, bottom, top}: 0 means
 * periodic (both sides of a pair must be 0), else a DG_BC_* code. */
dg_status dg_mesh_square(int nx, int ny, double x0, double x1, double y0, double y1,
                         double jitter, uint64_t seed, const int bc[4], dg_mesh **out);
void dg_mesh_destroy(dg_mesh *m);

/* ---- solver -------------------------------------------------------------
 * replaces run_dgcuda's set-up (init_gpu, set_quadrature, preval_* and
 * preval_basis; main.cu:600-806).  p = 0..5.  device = CUDA ordinal. */
dg_status dg_solver_create(const dg_mesh *m, dg_equation eq, int p, const dg_params *prm,
                           int device, dg_solver **out);
void dg_solver_destroy(dg_solver *s);
/* number of variables N and modes n_p */
dg_status dg_solver_sizes(const dg_solver *s, int *N, int *n_p, int *K, int *S);
/* the CUDA stream all work is issued on (a cudaStream_t) */
void *dg_solver_stream(dg_solver *s);

/* Override the basis / quadrature tabulation with the caller's, in the
 * reference's constant-table layouts (conserv_kernels.cu:42-76,
 * basis.cu:196-214): basis[i*n_q+j], grad_x/grad_y[i*n_q+j] (weights
 * folded in), side[f*n_p*n_1 + i*n_1 + j], vertex[i*3+v], w[n_q],
 * r1[n_q], r2[n_q], r_oned[n_1], w_oned[n_1].  n_q, n_1 must match p. */
dg_status dg_solver_set_tables(dg_solver *s, int n_q, int n_1, const double *basis,
                               const double *grad_x, const double *grad_y, const double *side,
                               const double *vertex, const double *w, const double *r1,
                               const double *r2, const double *r_oned, const double *w_oned);

/* L2 projection of the problem's initial condition (init_conditions,
 * conserv_kernels.cu:201-228) */
dg_status dg_init(dg_solver *s);
/* state copy in / out, reference layout C[var][mode][elem], .pmsh order */
dg_status dg_set_state(dg_solver *s, const double *C);
dg_status dg_get_state(dg_solver *s, double *C);
/* same, with device pointers (no host staging) */
dg_status dg_set_state_device(dg_solver *s, const double *C_device);
dg_status dg_get_state_device(dg_solver *s, double *C_device);

/* du/dt of the DG operator at time t for state C (host arrays, reference
 * layout): eval_surface + eval_volume + eval_rhs with dt = 1
 * (conserv_kernels.cu:899-1083, time_integrator.cu:26-101) */
dg_status dg_rhs(dg_solver *s, double t, const double *C, double *dCdt);

/* apply the slope limiter to the current state (limit_c) */
dg_status dg_limit(dg_solver *s);

/* nsteps time steps of `scheme` from the current state; each step takes
 * dt from the CFL condition on the device (eval_global_lambda + max,
 * time_integrator.cu:200-217) unless fixed_dt > 0.  *t is read and
 * advanced. */
dg_status dg_step(dg_solver *s, int nsteps, dg_scheme scheme, double fixed_dt, double *t);
/* step until t == T (the last step is shortened to land on T). */
dg_status dg_advance_to(dg_solver *s, double T, dg_scheme scheme, double *t, int *nsteps);

/* current CFL time step and the quantities it is built from */
dg_status dg_cfl(dg_solver *s, double *dt, double *lambda_max, double *d_min);

/* per-variable L2 error against the problem's exact solution at time t:
 * err[n] = sqrt(sum_e int_e (u_n - u_exact,n)^2) (eval_error_L2 + host sum,
 * conserv_kernels.cu:1432-1479, main.cu:859-875) */
dg_status dg_l2_error(dg_solver *s, double t, double *err);

/* values of variable `var` of the current state at the three vertices of
 * every element: uv[0*K + e], uv[1*K + e], uv[2*K + e] at V1, V2, V3 of
 * element e (.pmsh order) -- eval_u + the copies of write_U
 * (conserv_kernels.cu:1284-1307, main.cu:69-116) */
dg_status dg_eval_vertices(dg_solver *s, int var, double *uv);
/* the same layout for other views: DG_VIEW_SOLUTION (= dg_eval_vertices),
 * DG_VIEW_EXACT (the problem's exact solution at time t, plot_exact,
 * conserv_kernels.cu:1310-1331), DG_VIEW_ERROR (solution - exact,
 * plot_error, :1334-1369) */
#define DG_VIEW_SOLUTION 0
#define DG_VIEW_EXACT 1
#define DG_VIEW_ERROR 2
dg_status dg_eval_vertices_view(dg_solver *s, int var, int view, double t, double *uv);

/* advection velocity a(x, y) = (ax, ay) + grad (x, y), grad = {d a_x/dx,
 * d a_x/dy, d a_y/dx, d a_y/dy} (NULL: constant).  Replaces the problem's
 * get_velocity (advection.cu:12, rotatinghill.cu:37-40): the flux, the upwind
 * flux and the CFL wave speed take it at each point, the wave speed of an
 * element at its middle quadrature point (eval_global_lambda,
 * advection.cu:157-183).  Advection only (else DG_UNSUPPORTED).  The
 * rotating problems set their rotation when the solver is created; the
 * exact solutions of the translating problems (adv_sine, adv_linear,
 * adv_squarehill) move with (ax, ay) and do not follow grad. */
dg_status dg_set_velocity_field(dg_solver *s, double ax, double ay, const double *grad);
/* out[0..1] = (ax, ay), out[2..5] = grad, out[6] = the CFL wave speed */
dg_status dg_get_velocity_field(const dg_solver *s, double out[7]);
/* inflow pressure series of DG_PB_EULER_PULSE (tube.cu:52-97): p(t) = 1 +
 * sum_k amp[k] cos(omega[k] (t + t0) + phase[k]), k < n <= 16; the ghost
 * state is rho = gamma p^(1/gamma), u = (p - 1) / gamma, v = 0.  The tube and
 * trumpet problems are this with their own coefficient tables (amp = twice
 * each printed amplitude, omega = 2 PI times each frequency, t0 = 0.9197). */
dg_status dg_set_inflow_series(dg_solver *s, int n, const double *amp, const double *omega,
                               const double *phase, double t0);

/* The fused SSP-RK3 element stage computes its basis contractions (area
 * values, volume and surface projections, next-stage traces) either with
 * FP64 FMAs or on the tensor cores as exact integer slices (Ozaki-style
 * FP64 emulation; per-output error of the order of an FP64 dot product's
 * rounding).  The tensor path exists for Euler at p = 1..4 and is on by
 * default at p = 2..4 (at p = 1 the FP64 kernel is faster); DG_UNSUPPORTED
 * elsewhere.  No reference counterpart. */
dg_status dg_set_tensor_contractions(dg_solver *s, int on);
/* the digit tables of that path for order p = 1..4, built on the host from
 * the library's basis tables (for checks; no GPU needed): 2240 pairs of
 * 32-bit words, each two f16 digits, then 3 x 16 int column exponents and 16
 * ints of padding -- bytes >= 18176.  dense (optional, 1280 doubles): the
 * tables that were split, as [K block][K slot][N slot] matrices (EVAL,
 * PROJ x 3, TRACE) */
dg_status dg_oz_table_image(int p, void *out, size_t bytes, double *dense);
dg_status dg_get_tensor_contractions(dg_solver *s, int *on);

/* binary checkpoint / restart (no reference counterpart: the reference's
 * output is vertex values only).  The file holds the equation, order,
 * sizes, the time t, the state in .pmsh order, the shallow-water bed when
 * one is set, and a checksum; loading into a solver of another equation,
 * order or mesh size is DG_BAD_ARG, a damaged file DG_IO_ERROR. */
dg_status dg_save_checkpoint(dg_solver *s, const char *path, double t);
dg_status dg_load_checkpoint(dg_solver *s, const char *path, double *t);

/* ---- shallow-water bed (the reference's source_term hook,
 * conserv_kernels.cu:1063; its modules define no bed) -----------------------
 * source (0, -g h b_x, -g h b_y) with b a DG field of the solver's order:
 * b = modes [mode][elem] (.pmsh order, n_p x K), or NULL for a flat bed */
dg_status dg_set_bathymetry(dg_solver *s, const double *b);
/* the bed modes in the same layout (zeros for a flat bed) */
dg_status dg_get_bathymetry(dg_solver *s, double *b);
#define DG_BED_FLAT 0
#define DG_BED_SINE 1   /* b = prm[0] sin(2 pi prm[1] x) sin(2 pi prm[2] y) */
#define DG_BED_LINEAR 2 /* b = prm[0] + prm[1] x + prm[2] y */
/* L2 projection of an analytic bed onto the basis, then dg_set_bathymetry */
dg_status dg_bathymetry_project(dg_solver *s, int kind, const double *prm);

/* Block size (elements per block, one thread per element) of the stage
 * kernels, chosen by timing SSP-RK3 steps with 64, 128 and 256; the state is
 * restored afterwards.  *block receives the choice. */
dg_status dg_autotune(dg_solver *s, int *block);
/* dg_autotune that also chooses the element stage, where a solver has two:
 * the FP64-FMA kernel, one thread per element, or the tensor-core kernel,
 * whose quad of lanes holds two elements (two threads per element; Euler,
 * p = 1..4).  *threads_per_element receives 1 or 2.  The two agree to FP64
 * rounding, not bit for bit, so a run's last bits follow the choice. */
dg_status dg_autotune_stage(dg_solver *s, int *block, int *threads_per_element);

/* ---- batched ensembles: independent problems stepped together -----------
 * Per RK stage one face launch covers every member (concatenated element
 * and side ranges; each member keeps its own mesh, order p in 1..3, CFL time
 * step and time) and the element stage is one launch per group of members
 * of one order and mesh-size class (dg_batch_autotune), the groups running
 * concurrently; one SSP-RK3 step of the whole ensemble is one CUDA graph.
 * Members must share device, equation and limiter setting; they
 * stay owned by the caller and must outlive the batch.  No reference
 * counterpart (DGCUDA runs one problem per process). */
typedef struct dg_batch dg_batch;
dg_status dg_batch_create(int n, dg_solver *const *members, dg_batch **out);
/* nsteps SSP-RK3 steps of every member; t[i] is member i's time (read and
 * advanced) */
dg_status dg_batch_step(dg_batch *b, int nsteps, double *t);
/* block sizes of the batch's launches, timed on SSP-RK3 steps (states
 * restored): the one shared by the face, trace and limiter launches (*block),
 * then the element stage's per group -- group g = 2 (p - 1) + (K >= 16384):
 * members of order p on meshes below or from 16384 triangles, each its own
 * launch -- each from 64, 128 and 256 elements per block */
dg_status dg_batch_autotune(dg_batch *b, int *block);
/* blocks[0] = the shared block size, blocks[1 + g] = group g's (7 ints) */
dg_status dg_batch_blocks(const dg_batch *b, int *blocks);
long long dg_batch_launches(const dg_batch *b);
void dg_batch_destroy(dg_batch *b);

/* ---- derivatives (shallow water, p = 1..4, no limiter; reflect,
 * transmissive and periodic sides; no reference counterpart) -------------
 * Tangent-linear right-hand side: dL = dL/du dC + dL/db db (db may be NULL)
 * and its adjoint: Cbar = (dL/du)^T Lbar, bbar = (dL/db)^T Lbar.  Arrays in
 * the reference layout, .pmsh order; the flux Jacobians are hand-derived
 * (Rusanov: the branch of the max taken at C). */
dg_status dg_rhs_tl(dg_solver *s, double t, const double *C, const double *dC, const double *db,
                    double *dL);
dg_status dg_rhs_adjoint(dg_solver *s, double t, const double *C, const double *Lbar,
                         double *Cbar, double *bbar);

/* Discrete adjoint of SSP-RK3 time stepping with a fixed dt.  Samples are
 * the water height h at receiver points (rx, ry) after every `every` steps.
 * dg_adjoint_forward runs nsteps from the solver's current state and bed,
 * keeping the state every `ckpt` steps; dg_adjoint_backward recomputes each
 * segment from its checkpoint and sweeps back, returning the gradients of
 * sum_k,r sbar[k][r] sample[k][r] with respect to the initial state
 * ([var][mode][elem]) and the bed modes ([mode][elem]); dg_adjoint_tangent
 * returns the directional derivative of the samples along (du0, db). */
typedef struct dg_adjoint dg_adjoint;
dg_status dg_adjoint_create(dg_solver *s, int nrec, const double *rx, const double *ry,
                            dg_adjoint **out);
dg_status dg_adjoint_forward(dg_adjoint *a, int nsteps, double dt, int every, int ckpt,
                             double t0, double *samples);
/* What dg_adjoint_forward keeps for the reverse sweep: keep_stages = 0, the
 * checkpoints only (each segment is recomputed by dg_adjoint_backward); 1
 * (the default), also the three stage states u^n, u1, u2 of every step,
 * 3 * nsteps states of the solver's size, when they fit in free device
 * memory with 4 GiB to spare -- then the reverse sweep recomputes nothing --
 * and the checkpoints only otherwise.  dg_adjoint_stored: *kept = 1 when the
 * last forward run kept the stage states. */
dg_status dg_adjoint_set_storage(dg_adjoint *a, int keep_stages);
dg_status dg_adjoint_stored(const dg_adjoint *a, int *kept);
dg_status dg_adjoint_backward(dg_adjoint *a, const double *sbar, double *grad_u0,
                              double *grad_b);
dg_status dg_adjoint_tangent(dg_adjoint *a, const double *du0, const double *db,
                             double *dsamples);
void dg_adjoint_destroy(dg_adjoint *a);

/* Timing of the solver's own kernels (CUDA events around each launch on the
 * solver stream).  When enabled, dg_step launches kernels directly instead
 * of replaying a CUDA graph. */
dg_status dg_profile_enable(dg_solver *s, int on);
/* names: "trace", "face", "element", "limit", "cfl", "rk", "means" (the
 * fused limiter's cell means); fills launches and the
 * summed milliseconds since the last reset */
dg_status dg_profile_get(dg_solver *s, const char *kernel, long long *launches, double *ms);
dg_status dg_profile_reset(dg_solver *s);
/* launches of the solver's kernels since creation (all kinds) */
long long dg_kernel_launches(const dg_solver *s);

/* du/dt like dg_rhs, for callers that may not allocate device memory while
 * evaluating it (an application that owns all device memory and forbids
 * allocation after set-up, or a latency-critical loop where a cudaMalloc
 * would synchronise the device).  C_device and dCdt_device are the caller's
 * device buffers in the reference layout, ready with respect to the
 * solver's stream; the call returns when that stream has finished.  All
 * working memory comes from a static 32 MiB array that every GPU loading the
 * library holds until exit.  Larger problems get DG_UNSUPPORTED.  The first
 * call on a device looks up that array's address and keeps it (make it
 * before any stream capture; after cudaDeviceReset the kept address is
 * stale).  Calls that overlap on the GPU race on the array.  No counterpart
 * in the reference. */
dg_status dg_rhs_device_noalloc(dg_solver *s, double t, const double *C_device,
                                double *dCdt_device);

/* FP64 FMA throughput of `device` in TFLOP/s (the binding roof of the DG
 * kernels on GB300), timed with CUDA events; no reference counterpart */
dg_status dg_measure_fp64_peak(int device, double *tflops);
#ifdef __cplusplus
}
#endif
#endif
