// Host compilation of one CGSEM problem (topology groups, gather indices, folded factors, Jacobi
// diagonal), shared by the single-problem handle and the batched solver.
#pragma once

#include <vector>

#include "internal.hpp"

namespace selfgpu {
namespace cg {

struct HostCompiled {
  int N = 0, n = 0, nEl = 0, ngroups = 0;
  size_t nl = 0;
  std::vector<int> src, gptr, gidx;
  std::vector<unsigned char> gdir;
  std::vector<double> fac;   // 4 n^2 per element: G11, G12, G22, M
  std::vector<double> dinv;  // 1 / assembled diagonal, 1 at masked copies
  std::vector<double> Jww;   // J w_i w_j per node (load assembly)
  std::vector<double> D;     // GLL derivative matrix
};

int compile_host(self_ctx* ctx, const self_cg2d_desc* d, HostCompiled& out);

}  // namespace cg
}  // namespace selfgpu
