// adapters_drive.cpp -- TEST INFRASTRUCTURE ONLY: the C++ adapters
// (include/thunderegg_gb300/adapters.hpp) inside ThunderEgg's own solver
// classes, compiled from the reference sources by oracle/Makefile (target
// "adapt") into oracle/_ref/libteadapt.so with the host stand-in of the C ABI
// (fake_abi.cpp).  One GMG-preconditioned BiCGStab solve per call, wired the
// way a ThunderEgg application wires it, along one of these paths:
//   0  GMG::CycleBuilder<D> handed the GPU parts; its getCycle() (ThunderEgg's
//      own VCycle) is the Mr of ThunderEgg's Iterative::BiCGStab<D>
//   1  the same CycleBuilder's level chain turned into a GpuCycle<D>
//      (getCycle()->getFinestLevel()), solved by GpuBiCGStab<D>
//   2  GpuCycleBuilder<D> -> GpuCycle<D> as the Mr of ThunderEgg's BiCGStab
// smoother 0: GpuDFTPatchSolver, 1: GpuBiCGStabPatchSolver (inner 1e-12, 1000,
// continue on breakdown).

#include <ThunderEgg/GMG/CycleBuilder.h>
#include <ThunderEgg/Iterative/BiCGStab.h>

#include <cstring>
#include <memory>
#include <string>
#include <type_traits>
#include <vector>

#include "te_gpu.h"
#include "te_oracle.h"
#include "teref_domain.hpp"
#include "thunderegg_gb300/adapters.hpp"

namespace {
std::string g_err;
using namespace ThunderEgg;
namespace tg = thunderegg_gb300;

template <int D>
int solve(const te_level_desc* levels, int nlevels, int scheme, int smoother, int path, double tol, const double* f,
          double* u, int* iterations) {
  std::vector<std::shared_ptr<tg::GpuDomain<D>>> gd;
  std::vector<std::unique_ptr<tg::GpuGhostFiller<D>>> gf;
  std::vector<std::unique_ptr<tg::GpuStarPatchOperator<D>>> op;
  std::vector<std::unique_ptr<tg::GpuPatchSolver<D>>> sm;
  std::vector<std::unique_ptr<tg::GpuLinearRestrictor<D>>> rs;
  std::vector<std::unique_ptr<tg::GpuDirectInterpolator<D>>> in;
  for (int k = 0; k < nlevels; k++) {
    gd.push_back(std::make_shared<tg::GpuDomain<D>>(teref_tables::make_domain<D>(&levels[k], k)));
    gf.push_back(std::make_unique<tg::GpuGhostFiller<D>>(gd[k], scheme));
    op.push_back(std::make_unique<tg::GpuStarPatchOperator<D>>(*gf[k]));
    if (smoother == 0)
      sm.push_back(std::make_unique<tg::GpuDFTPatchSolver<D>>(*op[k]));
    else
      sm.push_back(std::make_unique<tg::GpuBiCGStabPatchSolver<D>>(*op[k], 1e-12, 1000, true));
  }
  for (int k = 0; k + 1 < nlevels; k++) rs.push_back(std::make_unique<tg::GpuLinearRestrictor<D>>(gd[k], gd[k + 1]));
  for (int k = 1; k < nlevels; k++) in.push_back(std::make_unique<tg::GpuDirectInterpolator<D>>(gd[k], gd[k - 1]));

  GMG::CycleOpts opts;
  auto build = [&](auto& b) {
    b.addFinestLevel(*op[0], *sm[0], *rs[0]);
    for (int k = 1; k + 1 < nlevels; k++) b.addIntermediateLevel(*op[k], *sm[k], *rs[k], *in[k - 1]);
    b.addCoarsestLevel(*op[nlevels - 1], *sm[nlevels - 1], *in[nlevels - 2]);
    return b.getCycle();
  };
  auto fv = gd[0]->makeVector();
  auto uv = gd[0]->makeVector();
  const size_t n = (size_t)levels[0].num_patches * gd[0]->patchStride(1);
  std::memcpy(fv.mem.get(), f, n * sizeof(double));
  int its = 0;
  if (path == 0) {
    GMG::CycleBuilder<D> b(opts);
    std::shared_ptr<GMG::Cycle<D>> cycle = build(b);
    Iterative::BiCGStab<D> solver;
    solver.setTolerance(tol);
    solver.setMaxIterations(1000);
    its = solver.solve(*op[0], uv.vec, fv.vec, cycle.get());
  } else if (path == 1) {
    GMG::CycleBuilder<D> b(opts);
    std::shared_ptr<GMG::Cycle<D>> ref_cycle = build(b);
    tg::GpuCycle<D> cycle(ref_cycle->getFinestLevel(), opts, TE_F64);
    tg::GpuBiCGStab<D> solver;
    solver.tolerance = tol;
    solver.flags = 0;  // the reference's update rule
    its = solver.solve(*op[0], uv.vec, fv.vec, &cycle);
  } else {
    tg::GpuCycleBuilder<D> b(opts, TE_F64);
    std::shared_ptr<GMG::Cycle<D>> cycle = build(b);
    Iterative::BiCGStab<D> solver;
    solver.setTolerance(tol);
    solver.setMaxIterations(1000);
    its = solver.solve(*op[0], uv.vec, fv.vec, cycle.get());
  }
  std::memcpy(u, uv.mem.get(), n * sizeof(double));
  *iterations = its;
  return TE_OK;
}
}  // namespace

extern "C" {
const char* teadapt_last_error(void) { return g_err.c_str(); }

int teadapt_solve(const te_level_desc* levels, int nlevels, int scheme, int smoother, int path, double tol,
                  const double* f, double* u, int* iterations) {
  try {
    if (nlevels < 2) throw std::runtime_error("at least two levels");
    if (levels[0].dim == 2) return solve<2>(levels, nlevels, scheme, smoother, path, tol, f, u, iterations);
    return solve<3>(levels, nlevels, scheme, smoother, path, tol, f, u, iterations);
  } catch (const std::exception& e) {
    g_err = e.what();
    return TE_ERR_INVALID;
  }
}

// the adapters' error translation: a failing ABI call throws ThunderEgg::RuntimeError (whose
// message carries te_last_error_message), a Krylov breakdown Iterative::BreakdownError
int teadapt_error_paths(void) {
  int ok = 0;
  try {
    thunderegg_gb300::check(TE_ERR_INVALID);
  } catch (const RuntimeError&) {
    ok |= 1;
  }
  try {
    thunderegg_gb300::check(TE_ERR_BREAKDOWN);
  } catch (const Iterative::BreakdownError&) {
    ok |= 2;
  }
  return ok;
}
}
