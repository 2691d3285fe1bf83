// te_ir.cu -- FP64 iterative refinement around a multigrid cycle.
//
// The outer loop of a mixed-precision solve whose preconditioner runs in a
// lower precision (an FP32 V-cycle, possibly with BF16 tensor-core
// transforms):
//
//   r = b - A x                                  (FP64, one pass)
//   while ||r|| / ||b|| > tol and its < max_iterations:
//     c = M r                                    (the cycle, its own precision)
//     x += c ; r = b - A x                       (FP64)
//
// The reference offers Krylov solvers only (Iterative/BiCGStab.h, CG.h); this
// solver sits behind the same Iterative::Solver<D>::solve(A, x, b, Mr)
// signature (Iterative/Solver.h:64-69) and stopping test ||r||/||b|| <= tol,
// on the true FP64 residual at every iteration.  M may not be NULL.  One host
// synchronisation per iteration reads ||r||^2.  A zero right-hand side returns
// at once with x unchanged; a non-finite residual returns TE_ERR_BREAKDOWN.

#include <cmath>
#include <memory>
#include <string>

#include "te_gmg.cuh"
#include "te_ops.cuh"

namespace te {
namespace {

struct IrWork {
  DevBuf<double> r, c;
};

double ir_dot(const te_domain* d, int nc, const void* x, const void* y) {
  reduce_dot(d, nc, TE_F64, x, y, d->d_result.p, d->stream);
  TE_CUDA(cudaMemcpyAsync(d->h_result, d->d_result.p, sizeof(double), cudaMemcpyDeviceToHost, d->stream));
  TE_CUDA(cudaStreamSynchronize(d->stream));
  return *d->h_result;
}

}  // namespace
}  // namespace te

using namespace te;

extern "C" int te_ir_solve(const te_operator* A, int nc, void* xv, const void* bv, const te_cycle* M, double tol,
                           int max_iterations, int* iterations, double* final_residual) {
  int status = TE_OK;
  int rc = guard([&] {
    require(A && xv && bv && M && iterations, "null argument (iterative refinement needs a cycle)");
    require(nc >= 1, "ncomp must be >= 1");
    const te_domain* d = A->dom;
    require(M->levels[0].op->dom->stream == d->stream, "the cycle and the operator must share a stream");
    const size_t n = (size_t)d->lay.P * d->lay.pstride(nc);
    auto& slot = A->krylov[std::make_pair(nc, std::vector<int>{-2})];
    if (!slot) {
      auto w = std::make_shared<IrWork>();
      w->r.alloc(n);
      w->c.alloc(n);
      slot = w;
    }
    IrWork& W = *std::static_pointer_cast<IrWork>(slot);
    cudaStream_t st = d->stream;
    te_cycle* m = const_cast<te_cycle*>(M);
    m->ensure(nc);
    *iterations = 0;
    if (final_residual) *final_residual = 0.0;
    const double r0 = std::sqrt(ir_dot(d, nc, bv, bv));
    if (!std::isfinite(r0)) {
      status = TE_ERR_BREAKDOWN;
      set_error("iterative refinement: the right-hand side is not finite");
      return;
    }
    if (r0 == 0) return;
    operator_residual(A, nc, xv, bv, W.r.p, st);
    double residual = std::sqrt(ir_dot(d, nc, W.r.p, W.r.p)) / r0;
    int its = 0;
    while (residual > tol && its < max_iterations) {
      if (!std::isfinite(residual)) {
        status = TE_ERR_BREAKDOWN;
        set_error("iterative refinement: the residual is not finite on iteration " + std::to_string(its));
        break;
      }
      m->apply_on(W.r.p, W.c.p, st);  // c = M r (Cycle::apply clears c first)
      vec_dispatch(d, nc, TE_F64, OP_ADD, xv, W.c.p, nullptr, 0.0, 0.0, 0.0);
      operator_residual(A, nc, xv, bv, W.r.p, st);
      its++;
      residual = std::sqrt(ir_dot(d, nc, W.r.p, W.r.p)) / r0;
    }
    *iterations = its;
    if (final_residual) *final_residual = residual;
  });
  return rc != TE_OK ? rc : status;
}
