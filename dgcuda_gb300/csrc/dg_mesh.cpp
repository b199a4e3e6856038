// dg_mesh.cpp -- .pmsh triangle meshes: read, write, validate, generate.
//
// The .pmsh text format is the reference's (read_mesh, main.cu:205-277;
// writer genmesh.py:286-313): the element count, one line per element
// "V1x V1y V2x V2y V3x V3y s1 s2 s3", the side count, one line per side
// "x1 y1 x2 y2 left right left_side right_side".  right < 0 marks a boundary
// side with code -1 reflect, -2 outflow, -3 inflow (genmesh.py:166-174);
// this library adds -4 transmissive.  Element face k joins vertices k and
// k+1 (mod 3); the element that first visits a side is its left element and
// boundary sides come first (genmesh.py:100-278).
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <unordered_map>
#include <numeric>

#include "dg_internal.h"

static thread_local std::string g_last_error;

namespace dg {
dg_status fail(dg_status st, const std::string &msg) {
  g_last_error = msg;
  return st;
}
}  // namespace dg

extern "C" const char *dg_last_error(void) { return g_last_error.c_str(); }
extern "C" const char *dg_version(void) { return "dgcuda_gb300 0.1 (sm_103a, FP64)"; }

extern "C" void dg_params_default(dg_params *p) {
  if (!p) return;
  std::memset(p, 0, sizeof *p);
  p->gamma = 1.4;
  p->gravity = 9.81;
  p->ax = 1.0;
  p->ay = 0.5;
  p->mu = 1.0;
  p->eps = 1.0;
  p->problem = DG_PB_NONE;
  p->limiter = 0;
  p->cfl = 0.3;
}

// the reference problem's own settings: each problem file's limiter and
// time_integrator globals, its GAMMA / MACH / ALPHA defines and its
// get_velocity (e.g. airfoil.cu:9-14, squarehill.cu:11-12, spin.cu:11-12)
extern "C" dg_status dg_params_for_problem(dg_params *p, int problem, int *scheme) {
  if (!p) return dg::fail(DG_BAD_ARG, "null argument");
  if (problem < DG_PB_NONE || problem > DG_PB_EULER_PULSE)
    return dg::fail(DG_BAD_ARG, "unknown problem");
  dg_params_default(p);
  p->problem = problem;
  int sc = DG_RK4;
  switch (problem) {
    case DG_PB_ADV_LINEAR:  // exact.cu:11-12, 34-37
      p->ax = p->ay = 1.0;
      p->limiter = 1;
      break;
    case DG_PB_ADV_SQUAREHILL:  // squarehill.cu:11-12, 35-38
      p->ax = 1.0;
      p->ay = 0.0;
      p->limiter = 1;
      break;
    case DG_PB_ADV_ROTATINGHILL:  // the rotation is set by the problem
      p->ax = p->ay = 0.0;
      break;
    case DG_PB_ADV_SPIN:  // spin.cu:11-12
      p->ax = p->ay = 0.0;
      sc = DG_RK2;
      break;
    case DG_PB_EULER_SUPERSONIC:  // supersonic.cu:10-14
      p->limiter = 1;
      break;
    case DG_PB_EULER_CYLINDER:  // cylinder.cu:10
      p->prm[0] = 0.38;
      break;
    case DG_PB_EULER_LSHOCK:  // lshock.cu:10
      p->prm[0] = 2.0;
      break;
    case DG_PB_EULER_DOUBLEMACH:  // doublemach.cu:18-19
      p->limiter = 1;
      sc = DG_RK2;
      break;
    case DG_PB_EULER_AIRFOIL:  // airfoil.cu:10-14
      p->prm[0] = 0.98;
      p->prm[1] = 5.0;
      p->limiter = 1;
      break;
    case DG_PB_SW_TEST:  // shallowwater.cu:7 hard-codes g = 9.8
      p->gravity = 9.8;
      break;
    default:
      break;
  }
  if (scheme) *scheme = sc;
  return DG_OK;
}

namespace dg {

dg_status validate_mesh(const dg_mesh &m) {
  if (m.K <= 0 || m.S <= 0) return fail(DG_BAD_MESH, "mesh has no elements or no sides");
  for (int k = 0; k < 6; k++)
    if ((int)m.V[k].size() != m.K) return fail(DG_BAD_MESH, "element array size mismatch");
  std::vector<int> refs(m.S, 0);
  for (int e = 0; e < m.K; e++) {
    for (int k = 0; k < 6; k++)
      if (!std::isfinite(m.V[k][e]))
        return fail(DG_BAD_MESH, "non-finite vertex in element " + std::to_string(e));
    double J = (m.V[2][e] - m.V[0][e]) * (m.V[5][e] - m.V[1][e]) -
               (m.V[4][e] - m.V[0][e]) * (m.V[3][e] - m.V[1][e]);
    if (!(J > 0)) return fail(DG_BAD_MESH, "element " + std::to_string(e) + " is not CCW (J <= 0)");
    for (int f = 0; f < 3; f++) {
      int s = m.es[f][e];
      if (s < 0 || s >= m.S)
        return fail(DG_BAD_MESH, "element " + std::to_string(e) + " has side index out of range");
      bool isl = m.left[s] == e && m.lsn[s] == f;
      bool isr = m.right[s] == e && m.rsn[s] == f;
      if (!isl && !isr)
        return fail(DG_BAD_MESH, "element " + std::to_string(e) + " face " + std::to_string(f) +
                                     " is not linked back from side " + std::to_string(s));
      refs[s]++;
    }
  }
  for (int s = 0; s < m.S; s++) {
    if (m.left[s] < 0 || m.left[s] >= m.K)
      return fail(DG_BAD_MESH, "side " + std::to_string(s) + " has no valid left element");
    if (m.lsn[s] < 0 || m.lsn[s] > 2)
      return fail(DG_BAD_MESH, "side " + std::to_string(s) + " left face out of range");
    int r = m.right[s];
    if (r >= 0) {
      if (r >= m.K) return fail(DG_BAD_MESH, "side " + std::to_string(s) + " right out of range");
      if (m.rsn[s] < 0 || m.rsn[s] > 2)
        return fail(DG_BAD_MESH, "side " + std::to_string(s) + " right face out of range");
      if (refs[s] != 2)
        return fail(DG_BAD_MESH, "interior side " + std::to_string(s) + " not shared by two faces");
    } else {
      if (r < -4) return fail(DG_BAD_MESH, "side " + std::to_string(s) + " has unknown code");
      if (refs[s] != 1)
        return fail(DG_BAD_MESH, "boundary side " + std::to_string(s) + " referenced twice");
    }
  }
  return DG_OK;
}

std::vector<int> sfc_order(const dg_mesh &m) {
  int K = m.K;
  std::vector<double> cx(K), cy(K);
  double xmin = 1e300, xmax = -1e300, ymin = 1e300, ymax = -1e300;
  for (int e = 0; e < K; e++) {
    cx[e] = (m.V[0][e] + m.V[2][e] + m.V[4][e]) / 3;
    cy[e] = (m.V[1][e] + m.V[3][e] + m.V[5][e]) / 3;
    xmin = std::min(xmin, cx[e]);
    xmax = std::max(xmax, cx[e]);
    ymin = std::min(ymin, cy[e]);
    ymax = std::max(ymax, cy[e]);
  }
  double sx = xmax > xmin ? (xmax - xmin) : 1, sy = ymax > ymin ? (ymax - ymin) : 1;
  auto spread = [](uint64_t v) {
    v &= 0xFFFFF;
    v = (v | (v << 16)) & 0x0000FFFF0000FFFFull;
    v = (v | (v << 8)) & 0x00FF00FF00FF00FFull;
    v = (v | (v << 4)) & 0x0F0F0F0F0F0F0F0Full;
    v = (v | (v << 2)) & 0x3333333333333333ull;
    v = (v | (v << 1)) & 0x5555555555555555ull;
    return v;
  };
  std::vector<uint64_t> key(K);
  for (int e = 0; e < K; e++) {
    uint64_t qx = (uint64_t)std::min(1048575.0, std::floor((cx[e] - xmin) / sx * 1048575.0));
    uint64_t qy = (uint64_t)std::min(1048575.0, std::floor((cy[e] - ymin) / sy * 1048575.0));
    key[e] = spread(qx) | (spread(qy) << 1);
  }
  std::vector<int> perm(K);
  std::iota(perm.begin(), perm.end(), 0);
  std::stable_sort(perm.begin(), perm.end(), [&](int a, int b) { return key[a] < key[b]; });
  return perm;
}

}  // namespace dg

using dg::fail;

extern "C" dg_status dg_mesh_read_pmsh(const char *path, dg_mesh **out) {
  if (!path || !out) return fail(DG_BAD_ARG, "null argument");
  *out = nullptr;
  FILE *f = std::fopen(path, "r");
  if (!f) return fail(DG_IO_ERROR, std::string("mesh file not found: ") + path);
  dg_mesh *m = new dg_mesh();
  char line[1000];
  auto bad = [&](const std::string &msg) {
    std::fclose(f);
    delete m;
    return fail(DG_BAD_MESH, msg);
  };
  if (!std::fgets(line, sizeof line, f) || std::sscanf(line, "%d", &m->K) != 1 || m->K <= 0)
    return bad("cannot read the element count");
  for (int k = 0; k < 6; k++) m->V[k].resize(m->K);
  for (int k = 0; k < 3; k++) m->es[k].resize(m->K);
  for (int i = 0; i < m->K; i++) {
    if (!std::fgets(line, sizeof line, f)) return bad("file ends inside the element list");
    int items = std::sscanf(line, "%lf %lf %lf %lf %lf %lf %d %d %d", &m->V[0][i], &m->V[1][i],
                            &m->V[2][i], &m->V[3][i], &m->V[4][i], &m->V[5][i], &m->es[0][i],
                            &m->es[1][i], &m->es[2][i]);
    if (items != 9)
      return bad("not enough items (" + std::to_string(items) + ") while reading element " +
                 std::to_string(i));
  }
  if (!std::fgets(line, sizeof line, f) || std::sscanf(line, "%d", &m->S) != 1 || m->S <= 0)
    return bad("cannot read the side count");
  m->sx1.resize(m->S);
  m->sy1.resize(m->S);
  m->sx2.resize(m->S);
  m->sy2.resize(m->S);
  m->left.resize(m->S);
  m->right.resize(m->S);
  m->lsn.resize(m->S);
  m->rsn.resize(m->S);
  for (int i = 0; i < m->S; i++) {
    if (!std::fgets(line, sizeof line, f)) return bad("file ends inside the side list");
    int items = std::sscanf(line, "%lf %lf %lf %lf %d %d %d %d", &m->sx1[i], &m->sy1[i],
                            &m->sx2[i], &m->sy2[i], &m->left[i], &m->right[i], &m->lsn[i],
                            &m->rsn[i]);
    if (items != 8)
      return bad("not enough items (" + std::to_string(items) + ") while reading side " +
                 std::to_string(i));
  }
  std::fclose(f);
  dg_status st = dg::validate_mesh(*m);
  if (st != DG_OK) {
    delete m;
    return st;
  }
  *out = m;
  return DG_OK;
}

extern "C" dg_status dg_mesh_write_pmsh(const dg_mesh *m, const char *path) {
  if (!m || !path) return fail(DG_BAD_ARG, "null argument");
  FILE *f = std::fopen(path, "w");
  if (!f) return fail(DG_IO_ERROR, std::string("cannot write ") + path);
  std::fprintf(f, "%d\n", m->K);
  for (int i = 0; i < m->K; i++)
    std::fprintf(f, "%.17g %.17g %.17g %.17g %.17g %.17g %d %d %d\n", m->V[0][i], m->V[1][i],
                 m->V[2][i], m->V[3][i], m->V[4][i], m->V[5][i], m->es[0][i], m->es[1][i],
                 m->es[2][i]);
  std::fprintf(f, "%d\n", m->S);
  for (int i = 0; i < m->S; i++)
    std::fprintf(f, "%.17g %.17g %.17g %.17g %d %d %d %d\n", m->sx1[i], m->sy1[i], m->sx2[i],
                 m->sy2[i], m->left[i], m->right[i], m->lsn[i], m->rsn[i]);
  bool ok = std::fclose(f) == 0;
  return ok ? DG_OK : fail(DG_IO_ERROR, "write failed");
}

extern "C" dg_status dg_mesh_from_arrays(int K, const double *V, const int *elem_sides, int S,
                                         const double *side_xy, const int *side_elems,
                                         dg_mesh **out) {
  if (!out || !V || !elem_sides || !side_xy || !side_elems || K <= 0 || S <= 0)
    return fail(DG_BAD_ARG, "bad mesh arrays");
  *out = nullptr;
  dg_mesh *m = new dg_mesh();
  m->K = K;
  m->S = S;
  for (int k = 0; k < 6; k++) m->V[k].assign(V + (size_t)k * K, V + (size_t)(k + 1) * K);
  for (int k = 0; k < 3; k++)
    m->es[k].assign(elem_sides + (size_t)k * K, elem_sides + (size_t)(k + 1) * K);
  m->sx1.assign(side_xy, side_xy + S);
  m->sy1.assign(side_xy + S, side_xy + 2 * (size_t)S);
  m->sx2.assign(side_xy + 2 * (size_t)S, side_xy + 3 * (size_t)S);
  m->sy2.assign(side_xy + 3 * (size_t)S, side_xy + 4 * (size_t)S);
  m->left.assign(side_elems, side_elems + S);
  m->right.assign(side_elems + S, side_elems + 2 * (size_t)S);
  m->lsn.assign(side_elems + 2 * (size_t)S, side_elems + 3 * (size_t)S);
  m->rsn.assign(side_elems + 3 * (size_t)S, side_elems + 4 * (size_t)S);
  dg_status st = dg::validate_mesh(*m);
  if (st != DG_OK) {
    delete m;
    return st;
  }
  *out = m;
  return DG_OK;
}

extern "C" dg_status dg_mesh_get_arrays(const dg_mesh *m, double *V, int *elem_sides,
                                        double *side_xy, int *side_elems) {
  if (!m) return fail(DG_BAD_ARG, "null mesh");
  size_t K = m->K, S = m->S;
  if (V)
    for (int k = 0; k < 6; k++) std::copy(m->V[k].begin(), m->V[k].end(), V + k * K);
  if (elem_sides)
    for (int k = 0; k < 3; k++) std::copy(m->es[k].begin(), m->es[k].end(), elem_sides + k * K);
  if (side_xy) {
    std::copy(m->sx1.begin(), m->sx1.end(), side_xy);
    std::copy(m->sy1.begin(), m->sy1.end(), side_xy + S);
    std::copy(m->sx2.begin(), m->sx2.end(), side_xy + 2 * S);
    std::copy(m->sy2.begin(), m->sy2.end(), side_xy + 3 * S);
  }
  if (side_elems) {
    std::copy(m->left.begin(), m->left.end(), side_elems);
    std::copy(m->right.begin(), m->right.end(), side_elems + S);
    std::copy(m->lsn.begin(), m->lsn.end(), side_elems + 2 * S);
    std::copy(m->rsn.begin(), m->rsn.end(), side_elems + 3 * S);
  }
  return DG_OK;
}

extern "C" dg_status dg_mesh_sizes(const dg_mesh *m, int *K, int *S) {
  if (!m) return fail(DG_BAD_ARG, "null mesh");
  if (K) *K = m->K;
  if (S) *S = m->S;
  return DG_OK;
}

extern "C" void dg_mesh_destroy(dg_mesh *m) { delete m; }

static inline uint64_t splitmix64(uint64_t &s) {
  uint64_t z = (s += 0x9E3779B97F4A7C15ull);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}
static inline double unif01(uint64_t &s) { return (double)(splitmix64(s) >> 11) * 0x1.0p-53; }

extern "C" dg_status dg_mesh_square(int nx, int ny, double x0, double x1, double y0, double y1,
                                    double jitter, uint64_t seed, const int bc[4],
                                    dg_mesh **out) {
  if (!out || !bc) return fail(DG_BAD_ARG, "null argument");
  *out = nullptr;
  bool px = bc[0] == 0 || bc[1] == 0, py = bc[2] == 0 || bc[3] == 0;
  if ((bc[0] == 0) != (bc[1] == 0) || (bc[2] == 0) != (bc[3] == 0))
    return fail(DG_BAD_ARG, "periodic boundaries must be paired (left/right, bottom/top)");
  for (int k = 0; k < 4; k++)
    if (bc[k] > 0 || bc[k] < -4) return fail(DG_BAD_ARG, "unknown boundary code");
  if (nx < 1 || ny < 1 || (px && nx < 3) || (py && ny < 3))
    return fail(DG_BAD_ARG, "need nx, ny >= 1 (>= 3 along periodic directions)");
  if (!(x1 > x0) || !(y1 > y0) || !(jitter >= 0) || jitter >= 0.5)
    return fail(DG_BAD_ARG, "bad box or jitter");
  if ((double)nx * ny * 2 > 2.0e9) return fail(DG_BAD_ARG, "mesh too large");
  double hx = (x1 - x0) / nx, hy = (y1 - y0) / ny;
  int vx = nx + 1, vy = ny + 1;
  std::vector<double> X((size_t)vx * vy), Y((size_t)vx * vy);
  uint64_t st = seed;
  for (int j = 0; j < vy; j++)
    for (int i = 0; i < vx; i++) {
      double x = x0 + i * hx, y = y0 + j * hy;
      if (i > 0 && i < nx && j > 0 && j < ny) {
        double ux = unif01(st), uy = unif01(st);
        x += (2 * ux - 1) * jitter * hx;
        y += (2 * uy - 1) * jitter * hy;
      }
      X[(size_t)j * vx + i] = x;
      Y[(size_t)j * vx + i] = y;
    }
  // connectivity ids identify periodic images
  auto vid = [&](int i, int j) -> int64_t {
    if (px) i %= nx;
    if (py) j %= ny;
    return (int64_t)j * vx + i;
  };
  dg_mesh *m = new dg_mesh();
  int K = 2 * nx * ny;
  m->K = K;
  for (int k = 0; k < 6; k++) m->V[k].resize(K);
  for (int k = 0; k < 3; k++) m->es[k].resize(K);
  struct Tmp {
    double x1, y1, x2, y2;
    int left, right, lsn, rsn;
    int box;  // -1 interior, else box edge 0..3
  };
  std::vector<Tmp> sides;
  sides.reserve((size_t)3 * K / 2 + 2 * (nx + ny));
  std::unordered_map<uint64_t, int> smap;
  smap.reserve((size_t)2 * K);
  const uint64_t nv = (uint64_t)vx * vy;
  int e = 0;
  for (int j = 0; j < ny; j++)
    for (int i = 0; i < nx; i++) {
      int tri[2][3][2] = {{{i, j}, {i + 1, j}, {i + 1, j + 1}},
                          {{i, j}, {i + 1, j + 1}, {i, j + 1}}};
      for (int t = 0; t < 2; t++, e++) {
        for (int k = 0; k < 3; k++) {
          size_t g = (size_t)tri[t][k][1] * vx + tri[t][k][0];
          m->V[2 * k][e] = X[g];
          m->V[2 * k + 1][e] = Y[g];
        }
        for (int k = 0; k < 3; k++) {
          int a = k, b = (k + 1) % 3;
          int ia = tri[t][a][0], ja = tri[t][a][1], ib = tri[t][b][0], jb = tri[t][b][1];
          int64_t ka = vid(ia, ja), kb = vid(ib, jb);
          uint64_t key = (uint64_t)std::min(ka, kb) * nv + (uint64_t)std::max(ka, kb);
          auto it = smap.find(key);
          if (it == smap.end()) {
            Tmp s;
            s.x1 = m->V[2 * a][e];
            s.y1 = m->V[2 * a + 1][e];
            s.x2 = m->V[2 * b][e];
            s.y2 = m->V[2 * b + 1][e];
            s.left = e;
            s.lsn = k;
            s.right = -1;
            s.rsn = 0;
            s.box = -1;
            if (ia == 0 && ib == 0) s.box = 0;
            else if (ia == nx && ib == nx) s.box = 1;
            else if (ja == 0 && jb == 0) s.box = 2;
            else if (ja == ny && jb == ny) s.box = 3;
            if (s.box >= 0 && bc[s.box] == 0) s.box = -1;  // periodic: will be matched
            smap.emplace(key, (int)sides.size());
            m->es[k][e] = (int)sides.size();
            sides.push_back(s);
          } else {
            Tmp &s = sides[it->second];
            s.right = e;
            s.rsn = k;
            m->es[k][e] = it->second;
          }
        }
      }
    }
  for (auto &s : sides)
    if (s.right < 0) {
      if (s.box < 0) {
        delete m;
        return fail(DG_BAD_MESH, "unmatched interior side while generating mesh");
      }
      s.right = bc[s.box];
    }
  // boundary sides first, by code -1, -2, -3, -4, then interior (stable)
  std::vector<int> order(sides.size());
  std::iota(order.begin(), order.end(), 0);
  auto rank = [&](int i) { return sides[i].right < 0 ? -sides[i].right : 100; };
  std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return rank(a) < rank(b); });
  std::vector<int> newidx(sides.size());
  for (size_t n = 0; n < order.size(); n++) newidx[order[n]] = (int)n;
  int S = (int)sides.size();
  m->S = S;
  m->sx1.resize(S);
  m->sy1.resize(S);
  m->sx2.resize(S);
  m->sy2.resize(S);
  m->left.resize(S);
  m->right.resize(S);
  m->lsn.resize(S);
  m->rsn.resize(S);
  for (int n = 0; n < S; n++) {
    const Tmp &s = sides[order[n]];
    m->sx1[n] = s.x1;
    m->sy1[n] = s.y1;
    m->sx2[n] = s.x2;
    m->sy2[n] = s.y2;
    m->left[n] = s.left;
    m->right[n] = s.right;
    m->lsn[n] = s.lsn;
    m->rsn[n] = s.rsn;
  }
  for (int k = 0; k < 3; k++)
    for (int el = 0; el < K; el++) m->es[k][el] = newidx[m->es[k][el]];
  dg_status vs = dg::validate_mesh(*m);
  if (vs != DG_OK) {
    delete m;
    return vs;
  }
  *out = m;
  return DG_OK;
}

// ---------------------------------------------------------------------------
// Gmsh ASCII .msh (format 2.2) -> mesh, the conversion genmesh.py performs
// (genmesh.py:13-315):
//  * nodes keep their (x, y); line elements (type 1) carry the boundary code
//    in their first (physical) tag: 10000 -> -1 reflect, 20000 -> -2 outflow,
//    30000 -> -3 inflow (genmesh.py:166-174), and, as an addition of this
//    library, 40000 -> -4 transmissive; triangles (type 2) are the elements,
//    in file order; other element types are skipped;
//  * sides are created element by element, faces (v1,v2), (v2,v3), (v3,v1):
//    the first element to visit a side is its left element, the second its
//    right element with its face number (genmesh.py:86-222);
//  * boundary sides are then moved to the front, code -1 first, then -2 and
//    -3, by swapping each one found (in side order) with the next free front
//    slot (genmesh.py:226-268), and the element -> side links follow.
// Deliberate differences, where genmesh.py would write an inconsistent
// mesh: a clockwise triangle is reoriented (its first two vertices swapped)
// before its sides are made, not only in the written coordinates
// (genmesh.py:284-288); a side with one element and no tagged line is an
// error (genmesh.py leaves element 0 as its right neighbour); node numbers
// need not be consecutive.
extern "C" dg_status dg_mesh_read_gmsh(const char *path, dg_mesh **out) {
  using dg::fail;
  if (!path || !out) return fail(DG_BAD_ARG, "null argument");
  *out = nullptr;
  FILE *f = std::fopen(path, "r");
  if (!f) return fail(DG_IO_ERROR, std::string("cannot open ") + path);
  struct Closer {
    FILE *f;
    ~Closer() { std::fclose(f); }
  } closer{f};
  char buf[4096];
  auto seek = [&](const char *tag) {
    while (std::fgets(buf, sizeof buf, f))
      if (std::strncmp(buf, tag, std::strlen(tag)) == 0) return true;
    return false;
  };
  if (!seek("$MeshFormat")) return fail(DG_BAD_MESH, "no $MeshFormat section");
  double version = 0;
  int ftype = -1;
  if (!std::fgets(buf, sizeof buf, f) || std::sscanf(buf, "%lf %d", &version, &ftype) != 2)
    return fail(DG_BAD_MESH, "bad $MeshFormat line");
  if (version < 2.0 || version >= 3.0 || ftype != 0)
    return fail(DG_UNSUPPORTED, "only ASCII Gmsh format 2.x is read");
  if (!seek("$Nodes")) return fail(DG_BAD_MESH, "no $Nodes section");
  long nn = 0;
  if (!std::fgets(buf, sizeof buf, f) || std::sscanf(buf, "%ld", &nn) != 1 || nn <= 0)
    return fail(DG_BAD_MESH, "bad node count");
  std::unordered_map<long, int> node_index;
  std::vector<double> nx(nn), ny(nn);
  for (long i = 0; i < nn; i++) {
    long id;
    double x, y, z;
    if (!std::fgets(buf, sizeof buf, f) || std::sscanf(buf, "%ld %lf %lf %lf", &id, &x, &y, &z) != 4)
      return fail(DG_BAD_MESH, "bad node line " + std::to_string(i + 1));
    node_index[id] = (int)i;
    nx[i] = x;
    ny[i] = y;
  }
  if (!seek("$Elements")) return fail(DG_BAD_MESH, "no $Elements section");
  long ne = 0;
  if (!std::fgets(buf, sizeof buf, f) || std::sscanf(buf, "%ld", &ne) != 1 || ne < 0)
    return fail(DG_BAD_MESH, "bad element count");
  auto edge_key = [](int a, int b) {
    const unsigned lo = (unsigned)std::min(a, b), hi = (unsigned)std::max(a, b);
    return ((uint64_t)hi << 32) | lo;
  };
  std::unordered_map<uint64_t, int> bcode;  // node pair -> boundary code
  std::vector<int> tri;                      // 3 node indices per element
  for (long i = 0; i < ne; i++) {
    if (!std::fgets(buf, sizeof buf, f)) return fail(DG_BAD_MESH, "truncated $Elements");
    std::vector<long> v;
    char *p = buf, *end;
    for (;;) {
      long x = std::strtol(p, &end, 10);
      if (end == p) break;
      v.push_back(x);
      p = end;
    }
    if (v.size() < 3 || (long)v.size() < 3 + v[2])
      return fail(DG_BAD_MESH, "bad element line " + std::to_string(i + 1));
    const long type = v[1], ntags = v[2];
    const size_t n0 = 3 + (size_t)ntags;
    auto node = [&](size_t k, int *o) {
      auto it = node_index.find(v[k]);
      if (it == node_index.end()) return false;
      *o = it->second;
      return true;
    };
    if (type == 1) {
      int a, b;
      if (v.size() < n0 + 2 || !node(n0, &a) || !node(n0 + 1, &b))
        return fail(DG_BAD_MESH, "bad line element " + std::to_string(v[0]));
      const long tag = ntags > 0 ? v[3] : 0;
      const int code = tag == 10000 ? -1 : tag == 20000 ? -2 : tag == 30000 ? -3 : tag == 40000 ? -4 : 0;
      if (code) bcode[edge_key(a, b)] = code;
    } else if (type == 2) {
      int a, b, c;
      if (v.size() < n0 + 3 || !node(n0, &a) || !node(n0 + 1, &b) || !node(n0 + 2, &c))
        return fail(DG_BAD_MESH, "bad triangle " + std::to_string(v[0]));
      const double J = (nx[b] - nx[a]) * (ny[c] - ny[a]) - (nx[c] - nx[a]) * (ny[b] - ny[a]);
      if (J < 0) std::swap(a, b);
      tri.push_back(a);
      tri.push_back(b);
      tri.push_back(c);
    }
  }
  const int K = (int)(tri.size() / 3);
  if (K == 0) return fail(DG_BAD_MESH, "no triangles in the mesh");
  struct Side {
    int a, b, left, right, lsn, rsn;
  };
  std::vector<Side> sides;
  sides.reserve((size_t)K * 3 / 2 + 16);
  std::unordered_map<uint64_t, int> smap;
  for (int e = 0; e < K; e++)
    for (int k = 0; k < 3; k++) {
      const int a = tri[3 * e + k], b = tri[3 * e + (k + 1) % 3];
      const uint64_t key = edge_key(a, b);
      auto it = smap.find(key);
      if (it != smap.end()) {
        Side &s = sides[it->second];
        if (s.right >= 0 && s.right != INT32_MAX)
          return fail(DG_BAD_MESH, "a side is shared by more than two triangles");
        s.right = e;
        s.rsn = k;
      } else {
        smap[key] = (int)sides.size();
        auto bc = bcode.find(key);
        sides.push_back({a, b, e, bc != bcode.end() ? bc->second : INT32_MAX, k, 0});
      }
    }
  for (const Side &s : sides)
    if (s.right == INT32_MAX)
      return fail(DG_BAD_MESH, "boundary side without a tagged line (10000/20000/30000/40000)");
  int front = 0;
  for (int code = -1; code >= -4; code--)
    for (size_t i = 0; i < sides.size(); i++)
      if (sides[i].right == code) std::swap(sides[i], sides[front++]);
  dg_mesh *m = new dg_mesh();
  m->K = K;
  m->S = (int)sides.size();
  for (int k = 0; k < 6; k++) m->V[k].resize(K);
  for (int k = 0; k < 3; k++) m->es[k].assign(K, -1);
  for (int e = 0; e < K; e++)
    for (int v = 0; v < 3; v++) {
      m->V[2 * v][e] = nx[tri[3 * e + v]];
      m->V[2 * v + 1][e] = ny[tri[3 * e + v]];
    }
  for (int j = 0; j < m->S; j++) {
    const Side &s = sides[j];
    m->sx1.push_back(nx[s.a]);
    m->sy1.push_back(ny[s.a]);
    m->sx2.push_back(nx[s.b]);
    m->sy2.push_back(ny[s.b]);
    m->left.push_back(s.left);
    m->right.push_back(s.right);
    m->lsn.push_back(s.lsn);
    m->rsn.push_back(s.rsn);
    m->es[s.lsn][s.left] = j;
    if (s.right >= 0) m->es[s.rsn][s.right] = j;
  }
  dg_status st = dg::validate_mesh(*m);
  if (st != DG_OK) {
    delete m;
    return st;
  }
  *out = m;
  return DG_OK;
}
