// fake_abi.cpp -- TEST INFRASTRUCTURE ONLY: the te_gpu C ABI (include/te_gpu.h)
// implemented on the host by the oracle restatement (te_oracle.cpp), for
// running the C++ adapters (include/thunderegg_gb300/adapters.hpp) inside
// ThunderEgg's own solver classes on a machine without a GPU.  "Device"
// buffers are host memory.  Only the entry points the adapters call exist;
// the level operations forward to the oracle with the level tables saved at
// creation, so results are the oracle's bit for bit.  Linked into
// oracle/_ref/libteadapt.so together with the reference objects and
// adapters_drive.cpp; nothing on the product path uses it.

#include <cmath>
#include <cstdlib>
#include <cstring>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "te_gpu.h"
#include "te_oracle.h"

extern "C" {
int teo_ghost_fill(const te_level_desc* d, int scheme, int fill_type, int nc, double* u);
int teo_operator_apply(const te_level_desc* d, int scheme, int fill_type, int kind, int neumann,
                       const double* coeffs, int nc, double* u, double* f);
int teo_modify_rhs(const te_level_desc* d, int scheme, int fill_type, int kind, const double* coeffs, int nc,
                   const double* u, double* f);
int teo_patch_solver(const te_level_desc* d, int scheme, int fill_type, int kind, const double* coeffs,
                     int smoother, int dft_neumann_mask, double tol, int max_it, int cont, int mode, int nc,
                     const double* f, double* u, long long* inner_its);
int teo_restrict(const te_level_desc* fine, const te_level_desc* coarse, int extrapolate, int nc, const double* f,
                 double* c);
int teo_interpolate(const te_level_desc* coarse, const te_level_desc* fine, int nc, const double* c, double* f);
int teo_vcycle_apply(const te_level_desc* levels, int nlevels, const teo_gmg_config* cfg,
                     const double* const* coeffs, int nc, const double* f, double* u);
int teo_gmg_solve(const te_level_desc* levels, int nlevels, const teo_gmg_config* cfg, const double* const* coeffs,
                  int nc, double* u, const double* f, int* iterations, double* final_residual);
const char* teo_last_error(void);
}

namespace {
std::string g_msg;

int fail(int code, const std::string& m) {
  g_msg = m;
  return code;
}
int wrap_rc(int rc) {
  if (rc != TE_OK) g_msg = teo_last_error();
  return rc;
}
}  // namespace

// owned copies of the level tables
struct te_domain {
  std::vector<int> id, refine_level, parent_id, orth_on_parent, child_ids, nbr_type, nbr_ids, nbr_orth;
  std::vector<double> starts, spacings;
  te_level_desc desc{};
  long long cs = 1;
  explicit te_domain(const te_level_desc* d) : desc(*d) {
    const int P = d->num_patches, D = d->dim, F = D == 2 ? 8 : 26;
    auto cp = [](auto& v, const auto* p, size_t n) { v.assign(p, p + n); };
    cp(id, d->id, P);
    cp(refine_level, d->refine_level, P);
    cp(parent_id, d->parent_id, P);
    cp(orth_on_parent, d->orth_on_parent, P);
    cp(child_ids, d->child_ids, (size_t)P << D);
    cp(starts, d->starts, (size_t)P * D);
    cp(spacings, d->spacings, (size_t)P * D);
    cp(nbr_type, d->nbr_type, (size_t)P * F);
    cp(nbr_ids, d->nbr_ids, (size_t)P * F * 4);
    cp(nbr_orth, d->nbr_orth, (size_t)P * F);
    desc.id = id.data();
    desc.refine_level = refine_level.data();
    desc.parent_id = parent_id.data();
    desc.orth_on_parent = orth_on_parent.data();
    desc.child_ids = child_ids.data();
    desc.starts = starts.data();
    desc.spacings = spacings.data();
    desc.nbr_type = nbr_type.data();
    desc.nbr_ids = nbr_ids.data();
    desc.nbr_orth = nbr_orth.data();
    for (int a = 0; a < D; a++) cs *= d->ns[a] + 2 * d->num_ghost;
  }
};
struct te_ghost_filler {
  const te_domain* d;
  int scheme, fill_type;
};
struct te_operator {
  const te_domain* d;
  const te_ghost_filler* g;
  int kind, neumann;
};
struct te_patch_solver {
  const te_operator* op;
  int kind;  // 0 DFT, 1 BiCGStab patch solver
  int neumann_mask;
  double tol;
  int max_it, cont;
};
struct te_restrictor {
  const te_domain *fine, *coarse;
  int extrapolate;
};
struct te_interpolator {
  const te_domain *coarse, *fine;
};
struct te_cycle {
  std::vector<te_level_desc> descs;
  teo_gmg_config cfg{};
  const te_operator* finest_op = nullptr;
};

extern "C" {

const char* te_last_error_message(void) { return g_msg.c_str(); }

int te_domain_create(const te_level_desc* desc, te_domain** out) {
  if (!desc || !out) return fail(TE_ERR_INVALID, "null argument");
  *out = new te_domain(desc);
  return TE_OK;
}
int te_domain_destroy(te_domain* d) {
  delete d;
  return TE_OK;
}
long long te_domain_patch_stride(const te_domain* d, int ncomp) { return d ? d->cs * ncomp : -1; }
int te_domain_num_patches(const te_domain* d) { return d ? d->desc.num_patches : -1; }

int te_level_alloc(const te_domain* d, int ncomp, int dtype, void** out) {
  if (!d || !out || dtype != TE_F64) return fail(TE_ERR_INVALID, "te_level_alloc: bad argument");
  *out = std::calloc((size_t)d->desc.num_patches * d->cs * ncomp, sizeof(double));
  return *out ? TE_OK : fail(TE_ERR_CUDA, "out of memory");
}
int te_level_free(void* p) {
  std::free(p);
  return TE_OK;
}
int te_device_alloc(size_t bytes, void** out) {
  *out = bytes ? std::malloc(bytes) : nullptr;
  return TE_OK;
}
int te_device_free(void* p) {
  std::free(p);
  return TE_OK;
}
int te_copy(void* dst, const void* src, size_t bytes) {
  if (bytes) std::memcpy(dst, src, bytes);
  return TE_OK;
}

int te_ghost_filler_create(const te_domain* d, int scheme, int fill_type, te_ghost_filler** out) {
  *out = new te_ghost_filler{d, scheme, fill_type};
  return TE_OK;
}
int te_ghost_filler_destroy(te_ghost_filler* g) {
  delete g;
  return TE_OK;
}
int te_ghost_fill(const te_ghost_filler* g, int ncomp, int dtype, void* u) {
  if (dtype != TE_F64) return fail(TE_ERR_UNSUPPORTED, "FP64 only");
  return wrap_rc(teo_ghost_fill(&g->d->desc, g->scheme, g->fill_type, ncomp, (double*)u));
}

int te_poisson_operator_create(const te_domain* d, const te_ghost_filler* g, int neumann, te_operator** out) {
  *out = new te_operator{d, g, 0, neumann};
  return TE_OK;
}
int te_varpoisson_operator_create(const te_domain*, const te_ghost_filler*, const void*, te_operator**) {
  return fail(TE_ERR_UNSUPPORTED, "the CPU stand-in has no VarPoisson operator");
}
int te_operator_destroy(te_operator* op) {
  delete op;
  return TE_OK;
}
int te_operator_apply(const te_operator* op, int ncomp, int dtype, void* u, void* f) {
  if (dtype != TE_F64) return fail(TE_ERR_UNSUPPORTED, "FP64 only");
  return wrap_rc(teo_operator_apply(&op->d->desc, op->g->scheme, op->g->fill_type, op->kind, op->neumann, nullptr,
                                    ncomp, (double*)u, (double*)f));
}
int te_operator_modify_rhs(const te_operator* op, int ncomp, int dtype, const void* u, void* f) {
  if (dtype != TE_F64) return fail(TE_ERR_UNSUPPORTED, "FP64 only");
  return wrap_rc(teo_modify_rhs(&op->d->desc, op->g->scheme, op->g->fill_type, op->kind, nullptr, ncomp,
                                (const double*)u, (double*)f));
}

int te_dft_patch_solver_create_tc(const te_operator* op, int neumann_mask, int, te_patch_solver** out) {
  *out = new te_patch_solver{op, 0, neumann_mask, 0.0, 0, 0};
  return TE_OK;
}
int te_dft_patch_solver_create(const te_operator* op, int neumann_mask, te_patch_solver** out) {
  return te_dft_patch_solver_create_tc(op, neumann_mask, TE_TC_TF32X3, out);
}
int te_bicgstab_patch_solver_create(const te_operator* op, double tol, int max_iterations, int cont,
                                    te_patch_solver** out) {
  *out = new te_patch_solver{op, 1, 0, tol, max_iterations, cont};
  return TE_OK;
}
int te_patch_solver_destroy(te_patch_solver* s) {
  delete s;
  return TE_OK;
}
static int patch_solve(const te_patch_solver* s, int ncomp, int dtype, const void* f, void* u, int mode) {
  if (dtype != TE_F64) return fail(TE_ERR_UNSUPPORTED, "FP64 only");
  long long its = 0;
  const te_operator* op = s->op;
  return wrap_rc(teo_patch_solver(&op->d->desc, op->g->scheme, op->g->fill_type, op->kind, nullptr, s->kind,
                                  s->neumann_mask, s->tol, s->max_it, s->cont, mode, ncomp, (const double*)f,
                                  (double*)u, &its));
}
int te_patch_solver_smooth(const te_patch_solver* s, int ncomp, int dtype, const void* f, void* u) {
  return patch_solve(s, ncomp, dtype, f, u, 0);
}
int te_patch_solver_apply(const te_patch_solver* s, int ncomp, int dtype, const void* f, void* u) {
  return patch_solve(s, ncomp, dtype, f, u, 1);
}

int te_linear_restrictor_create(const te_domain* fine, const te_domain* coarse, int extrapolate,
                                te_restrictor** out) {
  *out = new te_restrictor{fine, coarse, extrapolate};
  return TE_OK;
}
int te_restrictor_destroy(te_restrictor* r) {
  delete r;
  return TE_OK;
}
int te_restrict(const te_restrictor* r, int ncomp, int dtype, const void* fine, void* coarse_out) {
  if (dtype != TE_F64) return fail(TE_ERR_UNSUPPORTED, "FP64 only");
  return wrap_rc(teo_restrict(&r->fine->desc, &r->coarse->desc, r->extrapolate, ncomp, (const double*)fine,
                              (double*)coarse_out));
}
int te_direct_interpolator_create(const te_domain* coarse, const te_domain* fine, te_interpolator** out) {
  *out = new te_interpolator{coarse, fine};
  return TE_OK;
}
int te_interpolator_destroy(te_interpolator* i) {
  delete i;
  return TE_OK;
}
int te_interpolate(const te_interpolator* i, int ncomp, int dtype, const void* coarse, void* fine) {
  if (dtype != TE_F64) return fail(TE_ERR_UNSUPPORTED, "FP64 only");
  return wrap_rc(teo_interpolate(&i->coarse->desc, &i->fine->desc, ncomp, (const double*)coarse, (double*)fine));
}

// the cycle as the oracle's GMG configuration of its level chain (every level shares the finest
// level's ghost scheme, operator kind and smoother, as the oracle's hierarchies do)
int te_cycle_create(const te_cycle_level* levels, int num_levels, te_cycle_opts opts, int cycle_type, int,
                    te_cycle** out) {
  if (!levels || num_levels < 1 || !out) return fail(TE_ERR_INVALID, "null argument");
  auto c = std::make_unique<te_cycle>();
  for (int k = 0; k < num_levels; k++) c->descs.push_back(levels[k].op->d->desc);
  const te_operator* op = levels[0].op;
  const te_patch_solver* sm = levels[0].smoother;
  c->finest_op = op;
  teo_gmg_config& g = c->cfg;
  g.scheme = op->g->scheme;
  g.fill_type = op->g->fill_type;
  g.op_kind = op->kind;
  g.neumann = op->neumann;
  g.smoother = sm->kind;
  g.dft_neumann_mask = sm->neumann_mask;
  g.inner_tol = sm->kind ? sm->tol : 1e-12;
  g.inner_max_it = sm->kind ? sm->max_it : 1000;
  g.inner_continue_on_breakdown = sm->cont;
  g.pre_sweeps = opts.pre_sweeps;
  g.post_sweeps = opts.post_sweeps;
  g.mid_sweeps = opts.mid_sweeps;
  g.coarse_sweeps = opts.coarse_sweeps;
  g.extrapolate_boundary_ghosts = num_levels > 1 && levels[0].restrictor ? levels[0].restrictor->extrapolate : 0;
  g.cycle_type = cycle_type;
  g.use_precond = 1;
  *out = c.release();
  return TE_OK;
}
int te_cycle_destroy(te_cycle* c) {
  delete c;
  return TE_OK;
}
int te_cycle_apply(const te_cycle* c, int ncomp, const void* f, void* u) {
  return wrap_rc(teo_vcycle_apply(c->descs.data(), (int)c->descs.size(), &c->cfg, nullptr, ncomp, (const double*)f,
                                  (double*)u));
}

static int krylov(const te_operator* A, int ncomp, void* x, const void* b, const te_cycle* M, double tol, int max_it,
                  int flags, int kind, int* iterations, double* final_residual) {
  teo_gmg_config cfg{};
  std::vector<te_level_desc> one;
  const te_level_desc* levels;
  int n;
  if (M) {
    if (M->finest_op->d != A->d) return fail(TE_ERR_INVALID, "the cycle's finest level is not A's domain");
    cfg = M->cfg;
    levels = M->descs.data();
    n = (int)M->descs.size();
  } else {
    cfg.scheme = A->g->scheme;
    cfg.fill_type = A->g->fill_type;
    cfg.op_kind = A->kind;
    cfg.neumann = A->neumann;
    cfg.use_precond = 0;
    one.push_back(A->d->desc);
    levels = one.data();
    n = 1;
  }
  cfg.tol = tol;
  cfg.max_it = max_it;
  cfg.krylov = kind;
  cfg.precond_exit = flags & TE_BICGSTAB_PRECONDITIONED_EXIT;
  double res = 0;
  int its = 0;
  const int rc = teo_gmg_solve(levels, n, &cfg, nullptr, ncomp, (double*)x, (const double*)b, &its, &res);
  if (iterations) *iterations = its;
  if (final_residual) *final_residual = res;
  return wrap_rc(rc);
}
int te_bicgstab_solve(const te_operator* A, int ncomp, void* x, const void* b, const te_cycle* M, double tol,
                      int max_iterations, int flags, int* iterations, double* final_residual) {
  return krylov(A, ncomp, x, b, M, tol, max_iterations, flags, 0, iterations, final_residual);
}
int te_cg_solve(const te_operator* A, int ncomp, void* x, const void* b, const te_cycle* M, double tol,
                int max_iterations, int* iterations, double* final_residual) {
  return krylov(A, ncomp, x, b, M, tol, max_iterations, 0, 1, iterations, final_residual);
}
int te_ir_solve(const te_operator*, int, void*, const void*, const te_cycle*, double, int, int*, double*) {
  return fail(TE_ERR_UNSUPPORTED, "the CPU stand-in has no iterative refinement");
}
int te_bicgstab_batch_create(const te_operator*, int, void*, const void*, const te_cycle*, double, int, int, int,
                             const int*, te_bicgstab_batch**) {
  return fail(TE_ERR_UNSUPPORTED, "the CPU stand-in has no resumable batches");
}
int te_bicgstab_batch_step(te_bicgstab_batch*, int, int*) { return fail(TE_ERR_UNSUPPORTED, "no batches"); }
int te_bicgstab_batch_state(const te_bicgstab_batch*, int*, double*, int*, int*) {
  return fail(TE_ERR_UNSUPPORTED, "no batches");
}
int te_bicgstab_batch_destroy(te_bicgstab_batch*) { return TE_OK; }

long long te_domain_face_stride(const te_domain* d) {
  const int* n = d->desc.ns;
  if (d->desc.dim == 2) return n[0] > n[1] ? n[0] : n[1];
  long long a = (long long)n[1] * n[2], b = (long long)n[0] * n[2], c = (long long)n[0] * n[1];
  long long m = a > b ? a : b;
  return m > c ? m : c;
}
int te_domain_boundary_points(const te_domain*, double*) {
  return fail(TE_ERR_UNSUPPORTED, "the CPU stand-in has no boundary helpers");
}
int te_operator_add_dirichlet_bc_to_rhs(const te_operator*, int, void*, const double*, const double*) {
  return fail(TE_ERR_UNSUPPORTED, "the CPU stand-in has no boundary helpers");
}
int te_operator_add_neumann_bc_to_rhs(const te_operator*, int, void*, const double*) {
  return fail(TE_ERR_UNSUPPORTED, "the CPU stand-in has no boundary helpers");
}

}  // extern "C"
