// dg_internal.h -- host-side structures shared by the library's C++ files.
#pragma once
#include <cstdint>
#include <string>
#include <vector>

#include "../../include/dg.h"

struct dg_mesh {
  int K = 0, S = 0;
  // .pmsh column order (main.cu:205-277): per element V1x V1y V2x V2y V3x V3y
  // s1 s2 s3, per side x1 y1 x2 y2 left right left_side right_side.
  std::vector<double> V[6];
  std::vector<int> es[3];
  std::vector<double> sx1, sy1, sx2, sy2;
  std::vector<int> left, right, lsn, rsn;
};

namespace dg {

// records the message for dg_last_error() and returns the status
dg_status fail(dg_status st, const std::string &msg);

// checks the connectivity invariants of a .pmsh mesh
dg_status validate_mesh(const dg_mesh &m);

// Morton order of the element centroids (space-filling-curve renumbering):
// perm[new] = old
std::vector<int> sfc_order(const dg_mesh &m);

}  // namespace dg
