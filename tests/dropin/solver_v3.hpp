// Stand-in for the reference's src/v3_cuda_opt/solver_v3.hpp, used when the reference's own v3
// test programs (tests/test_v3_vs_v0.cu, test_poiseuille_v3.cu, test_cylinder_v3.cu) are built
// against this library: placed first on the include path, it makes lbm::SolverV3 the drop-in
// lbm::SolverB200 (include/lbm_b200.hpp), so the programs run unmodified on the GB300 kernels.
// This is the one-line binding a maintainer of the reference adds to switch its consumers over.
// The programs set LBM_V3_VARIANT to pick one of the reference's kernel variants; the drop-in
// ignores it (every kernel of the library gives the same results).
#pragma once

#include "lbm_b200.hpp"

namespace lbm {
using SolverV3 = SolverB200;
}  // namespace lbm
