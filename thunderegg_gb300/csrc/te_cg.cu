// te_cg.cu -- Iterative::CG (Iterative/CG.h:126-194) on FP64 device vectors.
//
// The reference's right-preconditioned form: r = b - A x; the iteration runs
// on a correction y started at zero (x.set(0)), with search directions p
// mapped through the preconditioner before A (A M p), and at the end
// x = M y + x0.  Every vector operation is one level kernel (te_runtime.cu);
// each iteration reads p.ap and r.r back to the host (two synchronisations),
// which sets alpha and beta exactly as the reference computes them.  The
// residual ||r|| / ||b|| reuses r.r: Vector::twoNorm and Vector::dot sum the
// same products in the same order here.
//
// A zero right-hand side returns at once with x's interior set to zero (the
// initial guess is not restored, as in the reference).  rho == 0 inside the
// loop returns TE_ERR_BREAKDOWN (the reference throws BreakdownError).

#include <cmath>
#include <memory>
#include <string>

#include "te_gmg.cuh"
#include "te_ops.cuh"

namespace te {
namespace {

struct CgWork {
  DevBuf<double> resid, p, ap, tmp, init;
};

double host_dot(const te_domain* d, int nc, const void* x, const void* y) {
  reduce_dot(d, nc, TE_F64, x, y, d->d_result.p, d->stream);
  TE_CUDA(cudaMemcpyAsync(d->h_result, d->d_result.p, sizeof(double), cudaMemcpyDeviceToHost, d->stream));
  TE_CUDA(cudaStreamSynchronize(d->stream));
  return *d->h_result;
}

// u = M f through the cycle (Cycle::apply clears u first)
void cycle_apply(const te_cycle* M, int nc, const void* f, void* u) {
  te_cycle* m = const_cast<te_cycle*>(M);
  m->ensure(nc);
  m->apply_on(f, u, m->stream);
}

}  // namespace
}  // namespace te

using namespace te;

extern "C" int te_cg_solve(const te_operator* A, int nc, void* xv, const void* bv, const te_cycle* M, double tol,
                           int max_iterations, int* iterations, double* final_residual) {
  int status = TE_OK;
  int rc = guard([&] {
    require(A && xv && bv && iterations, "null argument");
    require(nc >= 1, "ncomp must be >= 1");
    const te_domain* d = A->dom;
    require(!M || M->levels[0].op->dom->stream == d->stream, "the cycle and the operator must share a stream");
    const size_t n = (size_t)d->lay.P * d->lay.pstride(nc);
    // work vectors live with the operator, per component count
    auto& slot = A->krylov[std::make_pair(nc, std::vector<int>{-1})];
    if (!slot) {
      auto w = std::make_shared<CgWork>();
      w->resid.alloc(n);
      w->p.alloc(n);
      w->ap.alloc(n);
      w->tmp.alloc(n);
      w->init.alloc(n);
      slot = w;
    }
    CgWork& W = *std::static_pointer_cast<CgWork>(slot);
    cudaStream_t st = d->stream;
    double* x = (double*)xv;
    // resid = b - A x
    operator_residual(A, nc, x, bv, W.resid.p, st);
    // initial_guess = x (a copy with ghosts); x.set(0)
    TE_CUDA(cudaMemcpyAsync(W.init.p, x, n * sizeof(double), cudaMemcpyDeviceToDevice, st));
    vec_dispatch(d, nc, TE_F64, OP_SET, x, nullptr, nullptr, 0.0, 0.0, 0.0);
    const double r0 = std::sqrt(host_dot(d, nc, bv, bv));
    TE_CUDA(cudaMemcpyAsync(W.p.p, W.resid.p, n * sizeof(double), cudaMemcpyDeviceToDevice, st));
    double rho = host_dot(d, nc, W.resid.p, W.resid.p);
    int its = 0;
    *iterations = 0;
    if (final_residual) *final_residual = 0.0;
    if (r0 == 0) return;
    double residual = std::sqrt(rho) / r0;
    while (residual > tol && its < max_iterations) {
      if (rho == 0) {
        status = TE_ERR_BREAKDOWN;
        set_error("CG broke down, rho was 0 on iteration " + std::to_string(its));
        break;
      }
      if (M) {
        cycle_apply(M, nc, W.p.p, W.tmp.p);
        operator_apply(A, nc, TE_F64, W.tmp.p, W.ap.p, st);
      } else {
        operator_apply(A, nc, TE_F64, W.p.p, W.ap.p, st);
      }
      const double alpha = rho / host_dot(d, nc, W.p.p, W.ap.p);
      vec_dispatch(d, nc, TE_F64, OP_ADD_SCALED, x, W.p.p, nullptr, alpha, 0.0, 0.0);
      vec_dispatch(d, nc, TE_F64, OP_ADD_SCALED, W.resid.p, W.ap.p, nullptr, -alpha, 0.0, 0.0);
      const double rho_new = host_dot(d, nc, W.resid.p, W.resid.p);
      const double beta = rho_new / rho;
      vec_dispatch(d, nc, TE_F64, OP_SCALE_THEN_ADD, W.p.p, W.resid.p, nullptr, beta, 0.0, 0.0);
      its++;
      rho = rho_new;
      residual = std::sqrt(rho) / r0;
    }
    *iterations = its;
    if (final_residual) *final_residual = residual;
    if (status != TE_OK) return;
    if (M) {
      cycle_apply(M, nc, x, W.resid.p);
      vec_dispatch(d, nc, TE_F64, OP_COPY, x, W.resid.p, nullptr, 0.0, 0.0, 0.0);
    }
    vec_dispatch(d, nc, TE_F64, OP_ADD, x, W.init.p, nullptr, 0.0, 0.0, 0.0);
    TE_CUDA(cudaStreamSynchronize(st));
  });
  return rc != TE_OK ? rc : status;
}
