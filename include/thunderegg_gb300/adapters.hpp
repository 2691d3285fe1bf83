// thunderegg_gb300/adapters.hpp -- ThunderEgg's extension interfaces implemented
// over the te_gpu C ABI, so that GPU objects drop into an existing ThunderEgg
// solver setup (GMG::CycleBuilder, Iterative::BiCGStab) in place of the CPU
// classes.  Header-only; include after ThunderEgg's headers are on the path
// and link libte_gpu.so.
//
//   flatten(domain)            Domain<D> -> te_level_desc tables
//   GpuDomain<D>               device-side Domain (te_domain) + device-backed Vectors
//   GpuGhostFiller<D>          GhostFiller<D>                 (GhostFiller.h:46-53)
//   GpuStarPatchOperator<D>    PatchOperator<D>, Poisson or VarPoisson (PatchOperator.h:61-151)
//   GpuDFTPatchSolver<D>       PatchSolver<D> (= GMG::Smoother<D>) (PatchSolver.h:98-170)
//   GpuBiCGStabPatchSolver<D>  PatchSolver<D>: Iterative::PatchSolver with an inner BiCGStab
//                              (Iterative/PatchSolver.h:53-175)
//   GpuLinearRestrictor<D>     GMG::Restrictor<D>             (GMG/Restrictor.h:48-54)
//   GpuDirectInterpolator<D>   GMG::Interpolator<D>           (GMG/Interpolator.h:47-54)
//   GpuCycle<D>                GMG::Cycle<D> (GMG/Cycle.h:39-105) over a GMG::Level<D> chain of
//                              GPU parts, e.g. CycleBuilder::getCycle()->getFinestLevel()
//   GpuCycleBuilder<D>         GMG::CycleBuilder<D>'s interface (GMG/CycleBuilder.h:97-192),
//                              getCycle() returning a GpuCycle
//   GpuVCycle<D>               Operator<D> applying a whole cycle built from raw handles
//   GpuBiCGStab<D>             Iterative::Solver<D>           (Iterative/Solver.h:47-69)
//   GpuCG<D>                   Iterative::Solver<D>, Iterative::CG's right-preconditioned form (CG.h:126-194)
//   GpuIterativeRefinement<D>  Iterative::Solver<D>: FP64 iterative refinement around a cycle (no
//                              reference counterpart)
//
// Vectors: ThunderEgg's Vector<D> is concrete; a device-backed one is made
// with its unmanaged constructor (Vector.h:199-215) over a GpuDomain's level
// buffer, patches contiguous.  The adapters pass such Vectors' device
// pointers straight to the ABI; a Vector whose patches are not contiguous is
// rejected.  On GB300 the Grace CPU reaches HBM coherently, so ThunderEgg CPU
// code may still read these Vectors (slowly).  The per-patch virtuals
// (applySinglePatch, solveSinglePatch, ...) have no per-patch device entry
// point and throw; the level-wide apply/smooth/restrict/interpolate run on the
// GPU.  ABI failures throw ThunderEgg::RuntimeError, a Krylov breakdown throws
// ThunderEgg::Iterative::BreakdownError.
#pragma once

#include <ThunderEgg/Domain.h>
#include <ThunderEgg/GMG/Cycle.h>
#include <ThunderEgg/GMG/CycleOpts.h>
#include <ThunderEgg/GMG/Level.h>
#include <ThunderEgg/GMG/Interpolator.h>
#include <ThunderEgg/GMG/Restrictor.h>
#include <ThunderEgg/GhostFiller.h>
#include <ThunderEgg/Iterative/BreakdownError.h>
#include <ThunderEgg/Iterative/Solver.h>
#include <ThunderEgg/Operator.h>
#include <ThunderEgg/PatchOperator.h>
#include <ThunderEgg/PatchSolver.h>
#include <ThunderEgg/RuntimeError.h>
#include <ThunderEgg/Vector.h>

#include <array>
#include <cstdio>
#include <functional>
#include <memory>
#include <string>
#include <vector>

#include "../te_gpu.h"

namespace thunderegg_gb300 {

inline void check(int rc) {
  if (rc == TE_OK) return;
  const char* m = te_last_error_message();
  std::string msg = std::string("te_gpu: ") + (m ? m : "");
  if (rc == TE_ERR_BREAKDOWN) throw ThunderEgg::Iterative::BreakdownError(msg);
  throw ThunderEgg::RuntimeError(msg);
}

// ---------------------------------------------------------------------------
// Domain<D> -> flat level tables (local index = position in the PatchInfo vector)
// ---------------------------------------------------------------------------
template <int D>
struct LevelTables {
  std::array<int, 3> ns{{1, 1, 1}};
  int num_ghost = 1, P = 0;
  std::vector<int> id, refine_level, parent_id, orth_on_parent, child_ids, nbr_type, nbr_ids, nbr_orth;
  std::vector<double> starts, spacings;
  te_level_desc desc() const {
    te_level_desc d;
    d.dim = D;
    for (int a = 0; a < 3; a++) d.ns[a] = ns[a];
    d.num_ghost = num_ghost;
    d.num_patches = P;
    d.id = id.data();
    d.refine_level = refine_level.data();
    d.parent_id = parent_id.data();
    d.orth_on_parent = orth_on_parent.data();
    d.child_ids = child_ids.data();
    d.starts = starts.data();
    d.spacings = spacings.data();
    d.nbr_type = nbr_type.data();
    d.nbr_ids = nbr_ids.data();
    d.nbr_orth = nbr_orth.data();
    return d;
  }
};

constexpr int face_slots(int D) { return D == 2 ? 8 : 26; }

// neighbours of one face dimension M: slot = Face<D,M>::sum_of_faces + face index (PatchInfo.h:233-290)
template <int D, int M>
void flatten_faces(const ThunderEgg::PatchInfo<D>& pi, int p, LevelTables<D>& t) {
  using namespace ThunderEgg;
  for (Face<D, M> f : Face<D, M>::getValues()) {
    const size_t k = (size_t)p * face_slots(D) + Face<D, M>::sum_of_faces + f.getIndex();
    if (!pi.hasNbr(f)) continue;
    switch (pi.getNbrType(f)) {
      case NbrType::Normal:
        t.nbr_type[k] = TE_NBR_NORMAL;
        t.nbr_ids[k * 4] = pi.getNormalNbrInfo(f).id;
        break;
      case NbrType::Coarse: {
        const auto& ci = pi.getCoarseNbrInfo(f);
        t.nbr_type[k] = TE_NBR_COARSE;
        t.nbr_ids[k * 4] = ci.id;
        t.nbr_orth[k] = (int)ci.orth_on_coarse.getIndex();
        break;
      }
      case NbrType::Fine: {
        const auto& fi = pi.getFineNbrInfo(f);
        t.nbr_type[k] = TE_NBR_FINE;
        for (size_t o = 0; o < fi.ids.size(); o++) t.nbr_ids[k * 4 + o] = fi.ids[o];
        break;
      }
      default:
        throw ThunderEgg::RuntimeError("unknown neighbour type");
    }
  }
}

template <int D>
LevelTables<D> flatten(const ThunderEgg::Domain<D>& dom) {
  using namespace ThunderEgg;
  LevelTables<D> t;
  const auto& pinfos = dom.getPatchInfoVector();
  const int P = (int)pinfos.size(), F = face_slots(D), C = 1 << D;
  t.P = P;
  for (int a = 0; a < D; a++) t.ns[a] = dom.getNs()[a];
  t.num_ghost = dom.getNumGhostCells();
  t.id.assign(P, 0);
  t.refine_level.assign(P, -1);
  t.parent_id.assign(P, -1);
  t.orth_on_parent.assign(P, -1);
  t.child_ids.assign((size_t)P * C, -1);
  t.starts.assign((size_t)P * D, 0.0);
  t.spacings.assign((size_t)P * D, 1.0);
  t.nbr_type.assign((size_t)P * F, TE_NBR_NONE);
  t.nbr_ids.assign((size_t)P * F * 4, -1);
  t.nbr_orth.assign((size_t)P * F, -1);
  for (int p = 0; p < P; p++) {
    const PatchInfo<D>& pi = pinfos[p];
    t.id[p] = pi.id;
    t.refine_level[p] = pi.refine_level;
    t.parent_id[p] = pi.parent_id;
    t.orth_on_parent[p] = pi.orth_on_parent == Orthant<D>::null() ? -1 : (int)pi.orth_on_parent.getIndex();
    for (int c = 0; c < C; c++) t.child_ids[(size_t)p * C + c] = pi.child_ids[c];
    for (int a = 0; a < D; a++) {
      t.starts[(size_t)p * D + a] = pi.starts[a];
      t.spacings[(size_t)p * D + a] = pi.spacings[a];
    }
    if constexpr (D == 2) {
      flatten_faces<2, 0>(pi, p, t);
      flatten_faces<2, 1>(pi, p, t);
    } else {
      flatten_faces<3, 0>(pi, p, t);
      flatten_faces<3, 1>(pi, p, t);
      flatten_faces<3, 2>(pi, p, t);
    }
  }
  return t;
}

// ---------------------------------------------------------------------------
// device level and device-backed Vectors
// ---------------------------------------------------------------------------
template <int D>
class GpuDomain {
 public:
  explicit GpuDomain(const ThunderEgg::Domain<D>& dom) : dom_(dom) {
    LevelTables<D> t = flatten(dom);
    te_level_desc d = t.desc();
    te_domain* h = nullptr;
    check(te_domain_create(&d, &h));
    h_ = std::shared_ptr<te_domain>(h, [](te_domain* x) { te_domain_destroy(x); });
  }
  te_domain* handle() const { return h_.get(); }
  const ThunderEgg::Domain<D>& domain() const { return dom_; }
  // doubles of one patch with ncomp components, ghosts included
  long long patchStride(int ncomp) const { return te_domain_patch_stride(h_.get(), ncomp); }

  // A zero-filled device level buffer and a Vector<D> over it.  The Vector does not own the
  // memory: keep the returned object alive as long as the Vector is used.
  struct DeviceVector {
    std::shared_ptr<double> mem;
    ThunderEgg::Vector<D> vec;
  };
  DeviceVector makeVector(int ncomp = 1) const {
    const long long stride = patchStride(ncomp);
    const int P = dom_.getNumLocalPatches();
    void* raw = nullptr;
    check(te_level_alloc(h_.get(), ncomp, TE_F64, &raw));
    double* p = static_cast<double*>(raw);
    std::shared_ptr<double> mem(p, [](double* x) { te_level_free(x); });
    std::vector<double*> starts(P);
    for (int i = 0; i < P; i++) starts[i] = p + (size_t)i * stride;
    std::array<int, D + 1> strides, lengths;
    const int g = dom_.getNumGhostCells();
    int s = 1;
    for (int a = 0; a < D; a++) {
      strides[a] = s;
      lengths[a] = dom_.getNs()[a];
      s *= dom_.getNs()[a] + 2 * g;
    }
    strides[D] = s;
    lengths[D] = ncomp;
    return DeviceVector{mem, ThunderEgg::Vector<D>(dom_.getCommunicator(), starts, strides, lengths, g)};
  }

 private:
  ThunderEgg::Domain<D> dom_;
  std::shared_ptr<te_domain> h_;
};

// device pointer of a Vector's level buffer; its patches must be contiguous
template <int D>
void* levelPointer(const ThunderEgg::Vector<D>& v, const GpuDomain<D>& gd) {
  const int P = v.getNumLocalPatches();
  if (P == 0) throw ThunderEgg::RuntimeError("empty vector");
  auto first = [&](int i) {
    auto view = v.getPatchView(i);
    return &view[view.getGhostStart()];
  };
  const double* base = first(0);
  const long long stride = gd.patchStride(v.getNumComponents());
  for (int i = 1; i < P; i++)
    if (first(i) != base + (size_t)i * stride)
      throw ThunderEgg::RuntimeError("GPU adapters need a device-backed Vector with contiguous patches");
  return const_cast<double*>(base);
}

// ---------------------------------------------------------------------------
// GhostFiller<D>
// ---------------------------------------------------------------------------
template <int D>
class GpuGhostFiller : public ThunderEgg::GhostFiller<D> {
 public:
  // scheme: TE_GHOST_BILINEAR / BIQUADRATIC / TRILINEAR; fill_type: TE_FILL_*
  GpuGhostFiller(std::shared_ptr<GpuDomain<D>> gd, int scheme, int fill_type = TE_FILL_FACES) : gd_(gd) {
    te_ghost_filler* h = nullptr;
    check(te_ghost_filler_create(gd->handle(), scheme, fill_type, &h));
    h_ = std::shared_ptr<te_ghost_filler>(h, [](te_ghost_filler* x) { te_ghost_filler_destroy(x); });
  }
  GpuGhostFiller* clone() const override { return new GpuGhostFiller(*this); }
  void fillGhost(const ThunderEgg::Vector<D>& u) const override {
    check(te_ghost_fill(h_.get(), u.getNumComponents(), TE_F64, levelPointer(u, *gd_)));
  }
  te_ghost_filler* handle() const { return h_.get(); }
  const std::shared_ptr<GpuDomain<D>>& gpuDomain() const { return gd_; }

 private:
  std::shared_ptr<GpuDomain<D>> gd_;
  std::shared_ptr<te_ghost_filler> h_;
};

// ---------------------------------------------------------------------------
// PatchOperator<D>: Poisson::StarPatchOperator or VarPoisson::StarPatchOperator
// ---------------------------------------------------------------------------
template <int D>
class GpuStarPatchOperator : public ThunderEgg::PatchOperator<D> {
 public:
  // Poisson (coeffs == nullptr) or VarPoisson with a device coefficient Vector
  GpuStarPatchOperator(const GpuGhostFiller<D>& gf, bool neumann = false,
                       const ThunderEgg::Vector<D>* coeffs = nullptr)
      : ThunderEgg::PatchOperator<D>(gf.gpuDomain()->domain(), gf), gd_(gf.gpuDomain()) {
    te_operator* h = nullptr;
    if (coeffs)
      check(te_varpoisson_operator_create(gd_->handle(), gf.handle(), levelPointer(*coeffs, *gd_), &h));
    else
      check(te_poisson_operator_create(gd_->handle(), gf.handle(), neumann ? 1 : 0, &h));
    h_ = std::shared_ptr<te_operator>(h, [](te_operator* x) { te_operator_destroy(x); });
  }
  GpuStarPatchOperator* clone() const override { return new GpuStarPatchOperator(*this); }
  // the whole level on the GPU (PatchOperator::apply, PatchOperator.h:126-143)
  void apply(const ThunderEgg::Vector<D>& u, ThunderEgg::Vector<D>& f) const override {
    check(te_operator_apply(h_.get(), u.getNumComponents(), TE_F64, levelPointer(u, *gd_), levelPointer(f, *gd_)));
  }
  void modifyRHSForInternalBoundaryConditions(const ThunderEgg::Vector<D>& u, ThunderEgg::Vector<D>& f) const {
    check(te_operator_modify_rhs(h_.get(), u.getNumComponents(), TE_F64, levelPointer(u, *gd_),
                                 levelPointer(f, *gd_)));
  }
  void applySinglePatch(const ThunderEgg::PatchInfo<D>&, const ThunderEgg::PatchView<const double, D>&,
                        const ThunderEgg::PatchView<double, D>&) const override {
    throw ThunderEgg::RuntimeError("GpuStarPatchOperator runs whole levels; use apply()");
  }
  void modifyRHSForInternalBoundaryConditions(const ThunderEgg::PatchInfo<D>&,
                                              const ThunderEgg::PatchView<const double, D>&,
                                              const ThunderEgg::PatchView<double, D>&) const override {
    throw ThunderEgg::RuntimeError("GpuStarPatchOperator runs whole levels");
  }
  void applySinglePatchWithInternalBoundaryConditions(const ThunderEgg::PatchInfo<D>&,
                                                      const ThunderEgg::PatchView<const double, D>&,
                                                      const ThunderEgg::PatchView<double, D>&) const override {
    throw ThunderEgg::RuntimeError("GpuStarPatchOperator runs whole levels");
  }
  te_operator* handle() const { return h_.get(); }
  const std::shared_ptr<GpuDomain<D>>& gpuDomain() const { return gd_; }

  using PointFn = std::function<double(const std::array<double, D>&)>;
  // Poisson/StarPatchOperator.h:187-204 (Poisson) and VarPoisson/StarPatchOperator.h:194-219
  // (VarPoisson: hfunc is the coefficient): the functions are evaluated on the host at the
  // boundary points, the terms are added on the device
  void addDrichletBCToRHS(ThunderEgg::Vector<D>& f, PointFn gfunc, PointFn hfunc = nullptr) const {
    std::vector<std::vector<double>> vals = boundaryValues({gfunc, hfunc ? hfunc : gfunc});
    DeviceData g(vals[0]), c(vals[1]);
    check(te_operator_add_dirichlet_bc_to_rhs(h_.get(), TE_F64, levelPointer(f, *gd_), g.p,
                                              hfunc ? c.p : nullptr));
  }
  // Poisson/StarPatchOperator.h:212-242: gfunc_grad[axis] is the derivative along that axis
  void addNeumannBCToRHS(ThunderEgg::Vector<D>& f, PointFn /*gfunc*/, std::array<PointFn, D> gfunc_grad) const {
    std::vector<PointFn> fns(gfunc_grad.begin(), gfunc_grad.end());
    std::vector<std::vector<double>> vals = boundaryValues(fns);
    const long long fs = te_domain_face_stride(gd_->handle());
    std::vector<double> sel(vals[0].size());
    for (size_t i = 0; i < sel.size(); i++) sel[i] = vals[(i / fs % (2 * D)) >> 1][i];
    DeviceData g(sel);
    check(te_operator_add_neumann_bc_to_rhs(h_.get(), TE_F64, levelPointer(f, *gd_), g.p));
  }

 private:
  // FP64 device copy of a host array
  struct DeviceData {
    double* p = nullptr;
    explicit DeviceData(const std::vector<double>& v) {
      void* raw = nullptr;
      check(te_device_alloc(v.size() * sizeof(double), &raw));
      p = static_cast<double*>(raw);
      check(te_copy(p, v.data(), v.size() * sizeof(double)));
    }
    ~DeviceData() { te_device_free(p); }
    DeviceData(const DeviceData&) = delete;
    DeviceData& operator=(const DeviceData&) = delete;
  };
  // each function at the boundary points of te_domain_boundary_points, [P][2D][face stride]
  std::vector<std::vector<double>> boundaryValues(const std::vector<PointFn>& fns) const {
    const long long fs = te_domain_face_stride(gd_->handle());
    const size_t npts = (size_t)gd_->domain().getNumLocalPatches() * 2 * D * fs;
    std::vector<double> pts(npts * D);
    {
      DeviceData dev(pts);
      check(te_domain_boundary_points(gd_->handle(), dev.p));
      check(te_copy(pts.data(), dev.p, pts.size() * sizeof(double)));
    }
    std::vector<std::vector<double>> out(fns.size(), std::vector<double>(npts, 0.0));
    std::array<double, D> x;
    for (size_t i = 0; i < npts; i++) {
      for (int a = 0; a < D; a++) x[a] = pts[i * D + a];
      for (size_t k = 0; k < fns.size(); k++) out[k][i] = fns[k](x);
    }
    return out;
  }
  std::shared_ptr<GpuDomain<D>> gd_;
  std::shared_ptr<te_operator> h_;
};

// ---------------------------------------------------------------------------
// PatchSolver<D> (also a GMG::Smoother<D>): the DFT patch solver
// ---------------------------------------------------------------------------
// the level-wide apply/smooth of any GPU patch solver
template <int D>
class GpuPatchSolver : public ThunderEgg::PatchSolver<D> {
 public:
  void apply(const ThunderEgg::Vector<D>& f, ThunderEgg::Vector<D>& u) const override {
    check(te_patch_solver_apply(h_.get(), u.getNumComponents(), TE_F64, levelPointer(f, *gd_),
                                levelPointer(u, *gd_)));
  }
  void smooth(const ThunderEgg::Vector<D>& f, ThunderEgg::Vector<D>& u) const override {
    check(te_patch_solver_smooth(h_.get(), u.getNumComponents(), TE_F64, levelPointer(f, *gd_),
                                 levelPointer(u, *gd_)));
  }
  void solveSinglePatch(const ThunderEgg::PatchInfo<D>&, const ThunderEgg::PatchView<const double, D>&,
                        const ThunderEgg::PatchView<double, D>&) const override {
    throw ThunderEgg::RuntimeError("GPU patch solvers run whole levels; use apply() or smooth()");
  }
  te_patch_solver* handle() const { return h_.get(); }

 protected:
  explicit GpuPatchSolver(const GpuStarPatchOperator<D>& op)
      : ThunderEgg::PatchSolver<D>(op.gpuDomain()->domain(), op.getGhostFiller()), gd_(op.gpuDomain()) {}
  void own(te_patch_solver* h) {
    h_ = std::shared_ptr<te_patch_solver>(h, [](te_patch_solver* x) { te_patch_solver_destroy(x); });
  }
  std::shared_ptr<GpuDomain<D>> gd_;
  std::shared_ptr<te_patch_solver> h_;
};

template <int D>
class GpuDFTPatchSolver : public GpuPatchSolver<D> {
 public:
  // tc_precision (no reference counterpart): TE_TC_TF32X3 or TE_TC_BF16 for the FP32 tensor-core transforms
  explicit GpuDFTPatchSolver(const GpuStarPatchOperator<D>& op, int neumann_mask = 0,
                             int tc_precision = TE_TC_TF32X3)
      : GpuPatchSolver<D>(op) {
    te_patch_solver* h = nullptr;
    check(te_dft_patch_solver_create_tc(op.handle(), neumann_mask, tc_precision, &h));
    this->own(h);
  }
  GpuDFTPatchSolver* clone() const override { return new GpuDFTPatchSolver(*this); }
};

// Iterative::PatchSolver<D> (Iterative/PatchSolver.h:121-175) with an inner BiCGStab: every patch
// solved by its own BiCGStab with internal Dirichlet conditions, one CTA per patch
template <int D>
class GpuBiCGStabPatchSolver : public GpuPatchSolver<D> {
 public:
  GpuBiCGStabPatchSolver(const GpuStarPatchOperator<D>& op, double tolerance = 1e-12, int max_iterations = 1000,
                         bool continue_on_breakdown = false)
      : GpuPatchSolver<D>(op) {
    te_patch_solver* h = nullptr;
    check(te_bicgstab_patch_solver_create(op.handle(), tolerance, max_iterations, continue_on_breakdown ? 1 : 0,
                                          &h));
    this->own(h);
  }
  // the reference's form: PatchSolver(const Iterative::Solver<D>& solver, const PatchOperator<D>& op,
  // bool continue_on_breakdown) with the inner solver's tolerance and iteration limit
  template <class InnerSolver>
  GpuBiCGStabPatchSolver(const InnerSolver& solver, const GpuStarPatchOperator<D>& op,
                         bool continue_on_breakdown = false)
      : GpuBiCGStabPatchSolver(op, solver.getTolerance(), solver.getMaxIterations(), continue_on_breakdown) {}
  GpuBiCGStabPatchSolver* clone() const override { return new GpuBiCGStabPatchSolver(*this); }
};

// Poisson::FFTWPatchSolver<D> (Poisson/FFTWPatchSolver.h:189-308) computes the
// same solve as DFTPatchSolver (the same transform families, eigenvalues, zero
// mode and normalisation, with the transforms as FFTs); the GPU runs both as
// dense contractions.
template <int D>
using GpuFFTWPatchSolver = GpuDFTPatchSolver<D>;

// ---------------------------------------------------------------------------
// GMG::Restrictor<D> and GMG::Interpolator<D>
// ---------------------------------------------------------------------------
template <int D>
class GpuLinearRestrictor : public ThunderEgg::GMG::Restrictor<D> {
 public:
  GpuLinearRestrictor(std::shared_ptr<GpuDomain<D>> fine, std::shared_ptr<GpuDomain<D>> coarse,
                      bool extrapolate_boundary_ghosts = false)
      : fine_(fine), coarse_(coarse) {
    te_restrictor* h = nullptr;
    check(te_linear_restrictor_create(fine->handle(), coarse->handle(), extrapolate_boundary_ghosts ? 1 : 0, &h));
    h_ = std::shared_ptr<te_restrictor>(h, [](te_restrictor* x) { te_restrictor_destroy(x); });
  }
  GpuLinearRestrictor* clone() const override { return new GpuLinearRestrictor(*this); }
  // Restrictor::restrict returns a new Vector (Restrictor.h:54): a device-backed coarse Vector whose
  // memory is kept alive by this restrictor (the most recent results are retained)
  ThunderEgg::Vector<D> restrict(const ThunderEgg::Vector<D>& fine) const override {
    auto out = coarse_->makeVector(fine.getNumComponents());
    check(te_restrict(h_.get(), fine.getNumComponents(), TE_F64, levelPointer(fine, *fine_),
                      levelPointer(out.vec, *coarse_)));
    keep_.push_back(out.mem);
    if (keep_.size() > 4) keep_.erase(keep_.begin());
    return out.vec;
  }
  te_restrictor* handle() const { return h_.get(); }

 private:
  std::shared_ptr<GpuDomain<D>> fine_, coarse_;
  std::shared_ptr<te_restrictor> h_;
  mutable std::vector<std::shared_ptr<double>> keep_;
};

template <int D>
class GpuDirectInterpolator : public ThunderEgg::GMG::Interpolator<D> {
 public:
  GpuDirectInterpolator(std::shared_ptr<GpuDomain<D>> coarse, std::shared_ptr<GpuDomain<D>> fine)
      : coarse_(coarse), fine_(fine) {
    te_interpolator* h = nullptr;
    check(te_direct_interpolator_create(coarse->handle(), fine->handle(), &h));
    h_ = std::shared_ptr<te_interpolator>(h, [](te_interpolator* x) { te_interpolator_destroy(x); });
  }
  GpuDirectInterpolator* clone() const override { return new GpuDirectInterpolator(*this); }
  void interpolate(const ThunderEgg::Vector<D>& coarse, ThunderEgg::Vector<D>& fine) const override {
    check(te_interpolate(h_.get(), fine.getNumComponents(), TE_F64, levelPointer(coarse, *coarse_),
                         levelPointer(fine, *fine_)));
  }
  te_interpolator* handle() const { return h_.get(); }

 private:
  std::shared_ptr<GpuDomain<D>> coarse_, fine_;
  std::shared_ptr<te_interpolator> h_;
};

// ---------------------------------------------------------------------------
// The multigrid cycle as the right preconditioner Mr (Cycle::apply,
// GMG/Cycle.h:94-98): a V-cycle by default, or the W / FMG cycle that
// CycleBuilder::getCycle (GMG/CycleBuilder.h:176-191) makes for cycle_type
// "W" / "F"
// ---------------------------------------------------------------------------
// what the GPU Krylov adapters need from a cycle used as Mr
class GpuCycleHandle {
 public:
  virtual ~GpuCycleHandle() = default;
  virtual te_cycle* handle() const = 0;
};

template <int D>
class GpuVCycle : public ThunderEgg::Operator<D>, public GpuCycleHandle {
 public:
  struct LevelParts {
    const GpuStarPatchOperator<D>* op;
    const GpuPatchSolver<D>* smoother;
    te_restrictor* restrictor;      // null on the coarsest level
    te_interpolator* interpolator;  // null on the finest level
  };
  // dtype TE_F32: the mixed-precision cycle (FP32 on every level, FP64 in and out)
  GpuVCycle(std::shared_ptr<GpuDomain<D>> finest, const std::vector<LevelParts>& parts, te_cycle_opts opts,
            int dtype = TE_F32, int cycle_type = TE_CYCLE_V)
      : finest_(finest) {
    std::vector<te_cycle_level> lv(parts.size());
    for (size_t k = 0; k < parts.size(); k++) {
      lv[k].op = parts[k].op->handle();
      lv[k].smoother = parts[k].smoother->handle();
      lv[k].restrictor = parts[k].restrictor;
      lv[k].interpolator = parts[k].interpolator;
    }
    te_cycle* h = nullptr;
    check(te_cycle_create(lv.data(), (int)lv.size(), opts, cycle_type, dtype, &h));
    h_ = std::shared_ptr<te_cycle>(h, [](te_cycle* x) { te_cycle_destroy(x); });
  }
  // the reference's CycleOpts, cycle_type included
  GpuVCycle(std::shared_ptr<GpuDomain<D>> finest, const std::vector<LevelParts>& parts,
            const ThunderEgg::GMG::CycleOpts& o, int dtype = TE_F32)
      : GpuVCycle(finest, parts, te_cycle_opts{o.pre_sweeps, o.post_sweeps, o.mid_sweeps, o.coarse_sweeps}, dtype,
                  cycle_type_of(o.cycle_type)) {}
  static int cycle_type_of(const std::string& t) {
    if (t == "V") return TE_CYCLE_V;
    if (t == "W") return TE_CYCLE_W;
    if (t == "F") return TE_CYCLE_FMG;
    throw ThunderEgg::RuntimeError("Unsupported Cycle type: " + t);
  }
  GpuVCycle* clone() const override { return new GpuVCycle(*this); }
  void apply(const ThunderEgg::Vector<D>& f, ThunderEgg::Vector<D>& u) const override {
    check(te_cycle_apply(h_.get(), u.getNumComponents(), levelPointer(f, *finest_), levelPointer(u, *finest_)));
  }
  te_cycle* handle() const override { return h_.get(); }

 private:
  std::shared_ptr<GpuDomain<D>> finest_;
  std::shared_ptr<te_cycle> h_;
};

// ---------------------------------------------------------------------------
// GMG::Cycle<D> on the GPU.  Built from a GMG::Level<D> chain whose parts are GPU
// adapters -- the chain a GMG::CycleBuilder<D> makes when it is handed GPU parts
// (CycleBuilder::getCycle()->getFinestLevel()), or the one GpuCycleBuilder<D> makes.
// apply runs the whole cycle on the device (Cycle::apply, GMG/Cycle.h:94-98: u is
// cleared, then the levels are visited); cycle_type "V", "W" or "F" as CycleOpts.
// ---------------------------------------------------------------------------
template <int D>
class GpuCycle : public ThunderEgg::GMG::Cycle<D>, public GpuCycleHandle {
 public:
  // dtype TE_F32: the mixed-precision cycle (FP32 on every level, FP64 in and out)
  GpuCycle(const ThunderEgg::GMG::Level<D>& finest, const ThunderEgg::GMG::CycleOpts& opts, int dtype = TE_F32)
      : ThunderEgg::GMG::Cycle<D>(finest) {
    std::vector<te_cycle_level> lv;
    const ThunderEgg::GMG::Level<D>* level = &finest;
    while (true) {
      te_cycle_level t{};
      const auto* op = dynamic_cast<const GpuStarPatchOperator<D>*>(&level->getOperator());
      const auto* sm = dynamic_cast<const GpuPatchSolver<D>*>(&level->getSmoother());
      if (!op || !sm) throw ThunderEgg::RuntimeError("GpuCycle needs GPU operators and patch solvers on every level");
      t.op = op->handle();
      t.smoother = sm->handle();
      if (!level->finest()) {
        const auto* in = dynamic_cast<const GpuDirectInterpolator<D>*>(&level->getInterpolator());
        if (!in) throw ThunderEgg::RuntimeError("GpuCycle needs GpuDirectInterpolators");
        t.interpolator = in->handle();
      }
      if (!level->coarsest()) {
        const auto* rs = dynamic_cast<const GpuLinearRestrictor<D>*>(&level->getRestrictor());
        if (!rs) throw ThunderEgg::RuntimeError("GpuCycle needs GpuLinearRestrictors");
        t.restrictor = rs->handle();
      }
      if (lv.empty()) finest_ = op->gpuDomain();
      lv.push_back(t);
      if (level->coarsest()) break;
      level = &level->getCoarser();
    }
    te_cycle* h = nullptr;
    check(te_cycle_create(lv.data(), (int)lv.size(),
                          te_cycle_opts{opts.pre_sweeps, opts.post_sweeps, opts.mid_sweeps, opts.coarse_sweeps},
                          GpuVCycle<D>::cycle_type_of(opts.cycle_type), dtype, &h));
    h_ = std::shared_ptr<te_cycle>(h, [](te_cycle* x) { te_cycle_destroy(x); });
  }
  GpuCycle* clone() const override { return new GpuCycle(*this); }
  void apply(const ThunderEgg::Vector<D>& f, ThunderEgg::Vector<D>& u) const override {
    check(te_cycle_apply(h_.get(), u.getNumComponents(), levelPointer(f, *finest_), levelPointer(u, *finest_)));
  }
  te_cycle* handle() const override { return h_.get(); }

 protected:
  void visit(const ThunderEgg::GMG::Level<D>&, const ThunderEgg::Vector<D>&, ThunderEgg::Vector<D>&) const override {
    throw ThunderEgg::RuntimeError("GpuCycle visits its levels on the device; use apply()");
  }

 private:
  std::shared_ptr<GpuDomain<D>> finest_;
  std::shared_ptr<te_cycle> h_;
};

// GMG::CycleBuilder<D>'s interface and ordering rules (GMG/CycleBuilder.h:97-192) for GPU parts;
// getCycle() returns a GpuCycle
template <int D>
class GpuCycleBuilder {
 public:
  explicit GpuCycleBuilder(const ThunderEgg::GMG::CycleOpts& opts, int dtype = TE_F32) : opts_(opts), dtype_(dtype) {}
  void addFinestLevel(const ThunderEgg::Operator<D>& op, const ThunderEgg::GMG::Smoother<D>& smoother,
                      const ThunderEgg::GMG::Restrictor<D>& restrictor) {
    if (finest_) throw ThunderEgg::RuntimeError("addFinestLevel has already been called");
    finest_ = std::make_shared<ThunderEgg::GMG::Level<D>>();
    finest_->setOperator(op);
    finest_->setSmoother(smoother);
    finest_->setRestrictor(restrictor);
    chain_.push_back(finest_);
  }
  void addIntermediateLevel(const ThunderEgg::Operator<D>& op, const ThunderEgg::GMG::Smoother<D>& smoother,
                            const ThunderEgg::GMG::Restrictor<D>& restrictor,
                            const ThunderEgg::GMG::Interpolator<D>& interpolator) {
    if (!finest_) throw ThunderEgg::RuntimeError("addFinestLevel has not been called yet");
    if (done_) throw ThunderEgg::RuntimeError("addCoarsestLevel has already been called");
    auto lv = std::make_shared<ThunderEgg::GMG::Level<D>>();
    lv->setOperator(op);
    lv->setSmoother(smoother);
    lv->setRestrictor(restrictor);
    lv->setInterpolator(interpolator);
    chain_.push_back(lv);
  }
  void addCoarsestLevel(const ThunderEgg::Operator<D>& op, const ThunderEgg::GMG::Smoother<D>& smoother,
                        const ThunderEgg::GMG::Interpolator<D>& interpolator) {
    if (!finest_) throw ThunderEgg::RuntimeError("addFinestLevel has not been called yet");
    if (done_) throw ThunderEgg::RuntimeError("addCoarsestLevel has already been called");
    auto lv = std::make_shared<ThunderEgg::GMG::Level<D>>();
    lv->setOperator(op);
    lv->setSmoother(smoother);
    lv->setInterpolator(interpolator);
    chain_.push_back(lv);
    done_ = true;
  }
  std::shared_ptr<ThunderEgg::GMG::Cycle<D>> getCycle() const {
    if (!done_) throw ThunderEgg::RuntimeError("Cycle is not finalized: addCoarsestLevel has not been called");
    // each level points to the next coarser one (Level::setCoarser, as CycleBuilder does)
    for (size_t k = chain_.size() - 1; k > 0; k--) chain_[k - 1]->setCoarser(chain_[k]);
    return std::make_shared<GpuCycle<D>>(*finest_, opts_, dtype_);
  }

 private:
  ThunderEgg::GMG::CycleOpts opts_;
  int dtype_;
  std::shared_ptr<ThunderEgg::GMG::Level<D>> finest_;
  std::vector<std::shared_ptr<ThunderEgg::GMG::Level<D>>> chain_;
  bool done_ = false;
};

// ---------------------------------------------------------------------------
// Iterative::Solver<D>: BiCGStab on the GPU (Iterative/BiCGStab.h:111-203)
// ---------------------------------------------------------------------------
template <int D>
class GpuBiCGStab : public ThunderEgg::Iterative::Solver<D> {
 public:
  double tolerance = 1e-12;
  int max_iterations = 1000;
  int flags = TE_BICGSTAB_PRECONDITIONED_EXIT;
  GpuBiCGStab* clone() const override { return new GpuBiCGStab(*this); }
  int solve(const ThunderEgg::Operator<D>& A, ThunderEgg::Vector<D>& x, const ThunderEgg::Vector<D>& b,
            const ThunderEgg::Operator<D>* Mr = nullptr, bool output = false,
            std::ostream& os = std::cout) const override {
    const auto* op = dynamic_cast<const GpuStarPatchOperator<D>*>(&A);
    if (!op) throw ThunderEgg::RuntimeError("GpuBiCGStab needs a GpuStarPatchOperator");
    const auto* cyc = Mr ? dynamic_cast<const GpuCycleHandle*>(Mr) : nullptr;
    if (Mr && !cyc) throw ThunderEgg::RuntimeError("GpuBiCGStab needs a GPU cycle (or no) preconditioner");
    if (output) return solvePrinting(*op, x, b, cyc, os);
    int its = 0;
    double res = 0;
    check(te_bicgstab_solve(op->handle(), x.getNumComponents(), levelPointer(x, *op->gpuDomain()),
                            levelPointer(b, *op->gpuDomain()), cyc ? cyc->handle() : nullptr, tolerance,
                            max_iterations, flags, &its, &res));
    return its;
  }

 private:
  // output = true: the reference's progress lines ("%5d %16.8e", BiCGStab.h:134-139,193-197),
  // before the first iteration and after each, from a resumable batch of one solve
  // advanced one iteration at a time
  int solvePrinting(const GpuStarPatchOperator<D>& op, ThunderEgg::Vector<D>& x, const ThunderEgg::Vector<D>& b,
                    const GpuCycleHandle* cyc, std::ostream& os) const {
    const int offs[2] = {0, op.gpuDomain()->domain().getNumLocalPatches()};
    te_bicgstab_batch* h = nullptr;
    check(te_bicgstab_batch_create(op.handle(), x.getNumComponents(), levelPointer(x, *op.gpuDomain()),
                                   levelPointer(b, *op.gpuDomain()), cyc ? cyc->handle() : nullptr, tolerance,
                                   max_iterations, flags, 1, offs, &h));
    std::unique_ptr<te_bicgstab_batch, int (*)(te_bicgstab_batch*)> guard(h, te_bicgstab_batch_destroy);
    int its = 0, status = TE_OK, running = 0, n = 1;
    double res = 0;
    auto line = [&] {
      char buf[64];
      std::snprintf(buf, sizeof buf, "%5d %16.8e\n", its, res);
      os << buf;
    };
    check(te_bicgstab_batch_state(h, &its, &res, &status, &running));
    line();
    int shown = its;
    while (n) {
      check(te_bicgstab_batch_step(h, 1, &n));
      check(te_bicgstab_batch_state(h, &its, &res, &status, &running));
      if (its != shown) {
        line();
        shown = its;
      }
    }
    if (status == TE_ERR_BREAKDOWN)
      throw ThunderEgg::Iterative::BreakdownError("te_gpu: BiCGStab broke down on iteration " + std::to_string(its));
    check(status);
    return its;
  }
};

// Iterative::CG on the GPU (te_cg_solve): the reference's right-preconditioned
// form, FP64 vectors, any GpuVCycle (or none) as Mr.  With output = true it
// prints one "%5d %16.8e" line, for the final iteration count and residual
// (the per-iteration lines of CG.h:151-156,179-183 need a per-iteration hook
// that the ABI does not have).
template <int D>
class GpuCG : public ThunderEgg::Iterative::Solver<D> {
 public:
  double tolerance = 1e-12;
  int max_iterations = 1000;
  GpuCG* clone() const override { return new GpuCG(*this); }
  int solve(const ThunderEgg::Operator<D>& A, ThunderEgg::Vector<D>& x, const ThunderEgg::Vector<D>& b,
            const ThunderEgg::Operator<D>* Mr = nullptr, bool output = false,
            std::ostream& os = std::cout) const override {
    const auto* op = dynamic_cast<const GpuStarPatchOperator<D>*>(&A);
    if (!op) throw ThunderEgg::RuntimeError("GpuCG needs a GpuStarPatchOperator");
    const auto* cyc = Mr ? dynamic_cast<const GpuCycleHandle*>(Mr) : nullptr;
    if (Mr && !cyc) throw ThunderEgg::RuntimeError("GpuCG needs a GPU cycle (or no) preconditioner");
    int its = 0;
    double res = 0;
    check(te_cg_solve(op->handle(), x.getNumComponents(), levelPointer(x, *op->gpuDomain()),
                      levelPointer(b, *op->gpuDomain()), cyc ? cyc->handle() : nullptr, tolerance, max_iterations,
                      &its, &res));
    if (output) {
      char buf[64];
      std::snprintf(buf, sizeof buf, "%5d %16.8e\n", its, res);
      os << buf;
    }
    return its;
  }
};

// FP64 iterative refinement around a GPU cycle (te_ir_solve; no reference counterpart):
// x += Mr (b - A x) until the true FP64 residual ||b - A x|| / ||b|| <= tolerance
template <int D>
class GpuIterativeRefinement : public ThunderEgg::Iterative::Solver<D> {
 public:
  double tolerance = 1e-10;
  int max_iterations = 200;
  GpuIterativeRefinement* clone() const override { return new GpuIterativeRefinement(*this); }
  int solve(const ThunderEgg::Operator<D>& A, ThunderEgg::Vector<D>& x, const ThunderEgg::Vector<D>& b,
            const ThunderEgg::Operator<D>* Mr = nullptr, bool output = false,
            std::ostream& os = std::cout) const override {
    const auto* op = dynamic_cast<const GpuStarPatchOperator<D>*>(&A);
    if (!op) throw ThunderEgg::RuntimeError("GpuIterativeRefinement needs a GpuStarPatchOperator");
    const auto* cyc = Mr ? dynamic_cast<const GpuCycleHandle*>(Mr) : nullptr;
    if (!cyc) throw ThunderEgg::RuntimeError("GpuIterativeRefinement needs a GPU cycle as Mr");
    int its = 0;
    double res = 0;
    check(te_ir_solve(op->handle(), x.getNumComponents(), levelPointer(x, *op->gpuDomain()),
                      levelPointer(b, *op->gpuDomain()), cyc->handle(), tolerance, max_iterations, &its, &res));
    if (output) {
      char buf[64];
      std::snprintf(buf, sizeof buf, "%5d %16.8e\n", its, res);
      os << buf;
    }
    return its;
  }
};

}  // namespace thunderegg_gb300
