// teref.cpp -- TEST INFRASTRUCTURE ONLY.
//
// Runs ThunderEgg's own classes (compiled from the reference sources by
// oracle/Makefile into oracle/_ref/libteref.so) on the flat mesh tables of
// include/te_gpu.h.  It exposes the same C functions as the oracle
// restatement (te_oracle.cpp) under a teref_ prefix, so tests can run both on
// identical inputs and pin the restatement to the reference, and so
// tests/golden/make_golden.py can write fixtures from the reference itself.

#include "te_gpu.h"
#include "te_oracle.h"

#include <ThunderEgg/BiLinearGhostFiller.h>
#include <ThunderEgg/BiQuadraticGhostFiller.h>
#include <ThunderEgg/Domain.h>
#include <ThunderEgg/GMG/CycleBuilder.h>
#include <ThunderEgg/GMG/DirectInterpolator.h>
#include <ThunderEgg/GMG/LinearRestrictor.h>
#include <ThunderEgg/Iterative/BiCGStab.h>
#include <ThunderEgg/Iterative/CG.h>
#include <ThunderEgg/Iterative/PatchSolver.h>
#include <ThunderEgg/Poisson/DFTPatchSolver.h>
#include <ThunderEgg/Poisson/StarPatchOperator.h>
#include <ThunderEgg/TriLinearGhostFiller.h>
#include <ThunderEgg/VarPoisson/StarPatchOperator.h>
#include <ThunderEgg/tpl/json.hpp>

#include <array>
#include <cstring>
#include <functional>
#include <memory>
#include <stdexcept>
#include <type_traits>
#include <string>
#include <vector>

#include "thunderegg_gb300/adapters.hpp"
#include "teref_domain.hpp"

using namespace ThunderEgg;

namespace {
std::string g_err;

using teref_tables::make_domain;
using teref_tables::set_face_nbrs;
using teref_tables::slots;
using teref_tables::wrap;
template <int D>
void copy_out(const Vector<D>& v, double* out) {
  // copy every cell (ghosts included) of a managed vector into a flat buffer
  long ps = 1;
  {
    auto view = v.getPatchView(0);
    for (int a = 0; a <= D; a++) ps *= view.getGhostEnd()[a] - view.getGhostStart()[a] + 1;
  }
  for (int p = 0; p < v.getNumLocalPatches(); p++) {
    auto view = v.getPatchView(p);
    const double* src = &view[view.getGhostStart()];
    std::memcpy(out + p * ps, src, sizeof(double) * ps);
  }
}

GhostFillingType gft(int t) {
  return t == TE_FILL_FACES ? GhostFillingType::Faces
                            : (t == TE_FILL_EDGES ? GhostFillingType::Edges : GhostFillingType::Corners);
}

template <int D>
std::unique_ptr<GhostFiller<D>> make_filler(const Domain<D>& dom, int scheme, int fill_type) {
  if constexpr (D == 2) {
    if (scheme == TE_GHOST_BILINEAR) return std::make_unique<BiLinearGhostFiller>(dom, gft(fill_type));
    return std::make_unique<BiQuadraticGhostFiller>(dom, gft(fill_type));
  } else {
    return std::make_unique<TriLinearGhostFiller>(dom, gft(fill_type));
  }
}

template <int D>
std::unique_ptr<PatchOperator<D>> make_op(const Domain<D>& dom, const GhostFiller<D>& gf, int kind,
                                          int neumann, const double* coeffs) {
  if (kind == 0) return std::make_unique<Poisson::StarPatchOperator<D>>(dom, gf, neumann != 0);
  std::vector<double> cbuf(coeffs, coeffs + (size_t)dom.getNumLocalPatches() *
                                               [&] {
                                                 long s = 1;
                                                 for (int a = 0; a < D; a++)
                                                   s *= dom.getNs()[a] + 2 * dom.getNumGhostCells();
                                                 return s;
                                               }());
  Vector<D> c = wrap<D>(dom, 1, cbuf.data());
  Vector<D> cm(c);  // managed copy (the operator keeps its own)
  return std::make_unique<VarPoisson::StarPatchOperator<D>>(cm, dom, gf);
}

// records MPIGhostFiller's neighbour calls in processLocalFills order
template <int D>
struct RecordingFiller : public MPIGhostFiller<D> {
  mutable std::vector<std::array<int, 6>> rows;
  const double* base = nullptr;
  long ps = 1;
  RecordingFiller(const Domain<D>& d, GhostFillingType t) : MPIGhostFiller<D>(d, t) {}
  RecordingFiller* clone() const override { return new RecordingFiller(*this); }
  int idx(const PatchView<const double, D>& v) const {
    return (int)((&v[v.getGhostStart()] - base) / ps);
  }
  void fillGhostCellsForNbrPatch(const PatchInfo<D>& pinfo, const PatchView<const double, D>&,
                                 const PatchView<const double, D>& nbr, Side<D> s, NbrType t,
                                 Orthant<D - 1> o) const override {
    rows.push_back({pinfo.local_index, idx(nbr), D - 1, (int)s.getIndex(), (int)t == (int)NbrType::Normal ? 0 : ((int)t == (int)NbrType::Coarse ? 1 : 2),
                    t == NbrType::Normal ? -1 : (int)o.getIndex()});
  }
  void fillGhostCellsForEdgeNbrPatch(const PatchInfo<D>& pinfo, const PatchView<const double, D>&,
                                     const PatchView<const double, D>& nbr, Edge e, NbrType t,
                                     Orthant<1> o) const override {
    rows.push_back({pinfo.local_index, idx(nbr), 1, (int)e.getIndex(), t == NbrType::Normal ? 0 : (t == NbrType::Coarse ? 1 : 2),
                    t == NbrType::Normal ? -1 : (int)o.getIndex()});
  }
  void fillGhostCellsForCornerNbrPatch(const PatchInfo<D>& pinfo, const PatchView<const double, D>&,
                                       const PatchView<const double, D>& nbr, Corner<D> c,
                                       NbrType t) const override {
    rows.push_back({pinfo.local_index, idx(nbr), 0, (int)c.getIndex(), t == NbrType::Normal ? 0 : (t == NbrType::Coarse ? 1 : 2),
                    t == NbrType::Normal ? -1 : 0});
  }
  void fillGhostCellsForLocalPatch(const PatchInfo<D>&, const PatchView<const double, D>&) const override {}
};

template <class Fn>
int guard(Fn fn) {
  try {
    fn();
    return TE_OK;
  } catch (const std::exception& e) {
    g_err = e.what();
    return TE_ERR_INVALID;
  } catch (...) {
    g_err = "unknown exception";
    return TE_ERR_INVALID;
  }
}

template <int D>
struct Stack {
  std::vector<Domain<D>> doms;
  std::vector<std::unique_ptr<GhostFiller<D>>> gfs;
  std::vector<std::unique_ptr<PatchOperator<D>>> ops;
};
}  // namespace

template <int D>
static int gmg(const te_level_desc* levels, int nlevels, const teo_gmg_config* cfg, const double* const* coeffs,
               int nc, double* u, const double* f, int* iterations, double* final_residual, bool solve) {
  std::vector<Domain<D>> doms;
  for (int k = 0; k < nlevels; k++) doms.push_back(make_domain<D>(&levels[k], k));
  std::vector<std::unique_ptr<GhostFiller<D>>> gfs;
  std::vector<std::unique_ptr<PatchOperator<D>>> ops;
  std::vector<std::unique_ptr<PatchSolver<D>>> sms;
  Iterative::BiCGStab<D> inner;
  inner.setTolerance(cfg->inner_tol);
  inner.setMaxIterations(cfg->inner_max_it);
  for (int k = 0; k < nlevels; k++) {
    gfs.push_back(make_filler<D>(doms[k], cfg->scheme, cfg->fill_type));
    ops.push_back(make_op<D>(doms[k], *gfs[k], cfg->op_kind, cfg->neumann, cfg->op_kind == 1 ? coeffs[k] : nullptr));
    if (cfg->smoother == 0) {
      if constexpr (D == 2)
        sms.push_back(std::make_unique<Poisson::DFTPatchSolver<D>>(*ops[k], std::bitset<4>(cfg->dft_neumann_mask)));
      else
        sms.push_back(std::make_unique<Poisson::DFTPatchSolver<D>>(*ops[k], std::bitset<6>(cfg->dft_neumann_mask)));
    } else {
      sms.push_back(std::make_unique<Iterative::PatchSolver<D>>(inner, *ops[k], cfg->inner_continue_on_breakdown != 0));
    }
  }
  GMG::CycleOpts opts;
  opts.pre_sweeps = cfg->pre_sweeps;
  opts.post_sweeps = cfg->post_sweeps;
  opts.coarse_sweeps = cfg->coarse_sweeps;
  opts.mid_sweeps = cfg->mid_sweeps;
  opts.cycle_type = cfg->cycle_type == 1 ? "W" : (cfg->cycle_type == 2 ? "F" : "V");
  GMG::CycleBuilder<D> b(opts);
  bool ex = cfg->extrapolate_boundary_ghosts != 0;
  for (int k = 0; k < nlevels; k++) {
    if (k == 0)
      b.addFinestLevel(*ops[k], *sms[k], GMG::LinearRestrictor<D>(doms[k], doms[k + 1], ex));
    else if (k + 1 < nlevels)
      b.addIntermediateLevel(*ops[k], *sms[k], GMG::LinearRestrictor<D>(doms[k], doms[k + 1], ex),
                             GMG::DirectInterpolator<D>(doms[k], doms[k - 1]));
    else
      b.addCoarsestLevel(*ops[k], *sms[k], GMG::DirectInterpolator<D>(doms[k], doms[k - 1]));
  }
  auto M = b.getCycle();
  Vector<D> uv = wrap<D>(doms[0], nc, u);
  Vector<D> fv = wrap<D>(doms[0], nc, const_cast<double*>(f));
  if (!solve) {
    M->apply(fv, uv);
    return TE_OK;
  }
  try {
    if (cfg->krylov == 1) {
      Iterative::CG<D> outer;
      outer.setTolerance(cfg->tol);
      outer.setMaxIterations(cfg->max_it);
      *iterations = outer.solve(*ops[0], uv, fv, cfg->use_precond ? M.get() : nullptr);
    } else {
      Iterative::BiCGStab<D> outer;
      outer.setTolerance(cfg->tol);
      outer.setMaxIterations(cfg->max_it);
      *iterations = outer.solve(*ops[0], uv, fv, cfg->use_precond ? M.get() : nullptr);
    }
  } catch (const Iterative::BreakdownError&) {
    return TE_ERR_BREAKDOWN;
  }
  // final relative residual ||b - A x|| / ||b||, as BiCGStab measures it
  Vector<D> r = fv.getZeroClone();
  ops[0]->apply(uv, r);
  r.scaleThenAdd(-1, fv);
  double bn = fv.twoNorm();
  *final_residual = bn == 0 ? 0 : r.twoNorm() / bn;
  return TE_OK;
}

extern "C" const char* teref_last_error(void) { return g_err.c_str(); }
extern "C" {

int teref_ghost_fill(const te_level_desc* d, int scheme, int fill_type, int nc, double* u) {
  return guard([&] {
    if (d->dim == 2) {
      auto dom = make_domain<2>(d);
      auto gf = make_filler<2>(dom, scheme, fill_type);
      gf->fillGhost(wrap<2>(dom, nc, u));
    } else {
      auto dom = make_domain<3>(d);
      auto gf = make_filler<3>(dom, scheme, fill_type);
      gf->fillGhost(wrap<3>(dom, nc, u));
    }
  });
}

static std::vector<std::array<int, 6>> g_calls;
int teref_ghost_num_calls(const te_level_desc* d, int fill_type) {
  g_calls.clear();
  guard([&] {
    std::vector<double> u;
    auto run = [&](auto dom, auto tag) {
      constexpr int D = decltype(tag)::value;
      long ps = 1;
      for (int a = 0; a < D; a++) ps *= dom.getNs()[a] + 2 * dom.getNumGhostCells();
      u.assign((size_t)ps * dom.getNumLocalPatches(), 0.0);
      RecordingFiller<D> f(dom, gft(fill_type));
      f.base = u.data();
      f.ps = ps;
      f.fillGhost(wrap<D>(dom, 1, u.data()));
      g_calls = f.rows;
    };
    if (d->dim == 2)
      run(make_domain<2>(d), std::integral_constant<int, 2>());
    else
      run(make_domain<3>(d), std::integral_constant<int, 3>());
  });
  return (int)g_calls.size();
}
int teref_ghost_calls(const te_level_desc* d, int fill_type, int* rows6) {
  teref_ghost_num_calls(d, fill_type);
  for (size_t k = 0; k < g_calls.size(); k++) std::memcpy(rows6 + 6 * k, g_calls[k].data(), 6 * sizeof(int));
  return TE_OK;
}

int teref_operator_apply(const te_level_desc* d, int scheme, int fill_type, int kind, int neumann,
                         const double* coeffs, int nc, double* u, double* f) {
  return guard([&] {
    auto run = [&](auto dom, auto tag) {
      constexpr int D = decltype(tag)::value;
      auto gf = make_filler<D>(dom, scheme, fill_type);
      auto op = make_op<D>(dom, *gf, kind, neumann, coeffs);
      Vector<D> fv = wrap<D>(dom, nc, f);
      op->apply(wrap<D>(dom, nc, u), fv);
    };
    if (d->dim == 2)
      run(make_domain<2>(d), std::integral_constant<int, 2>());
    else
      run(make_domain<3>(d), std::integral_constant<int, 3>());
  });
}

int teref_modify_rhs(const te_level_desc* d, int scheme, int fill_type, int kind, const double* coeffs,
                     int nc, const double* u, double* f) {
  return guard([&] {
    auto run = [&](auto dom, auto tag) {
      constexpr int D = decltype(tag)::value;
      auto gf = make_filler<D>(dom, scheme, fill_type);
      auto op = make_op<D>(dom, *gf, kind, 0, coeffs);
      Vector<D> uv = wrap<D>(dom, nc, const_cast<double*>(u));
      Vector<D> fv = wrap<D>(dom, nc, f);
      for (const PatchInfo<D>& pi : dom.getPatchInfoVector())
        op->modifyRHSForInternalBoundaryConditions(pi, uv.getPatchView(pi.local_index),
                                                   fv.getPatchView(pi.local_index));
    };
    if (d->dim == 2)
      run(make_domain<2>(d), std::integral_constant<int, 2>());
    else
      run(make_domain<3>(d), std::integral_constant<int, 3>());
  });
}

int teref_patch_solver(const te_level_desc* d, int scheme, int fill_type, int kind, const double* coeffs,
                       int smoother, int dft_neumann_mask, double tol, int max_it, int cont, int mode, int nc,
                       const double* f, double* u, long long* inner_its) {
  if (inner_its) *inner_its = -1;
  return guard([&] {
    auto run = [&](auto dom, auto tag) {
      constexpr int D = decltype(tag)::value;
      auto gf = make_filler<D>(dom, scheme, fill_type);
      auto op = make_op<D>(dom, *gf, kind, 0, coeffs);
      std::unique_ptr<PatchSolver<D>> ps;
      Iterative::BiCGStab<D> inner;
      inner.setTolerance(tol);
      inner.setMaxIterations(max_it);
      if (smoother == 0) {
        if constexpr (D == 2)
          ps = std::make_unique<Poisson::DFTPatchSolver<D>>(*op, std::bitset<4>(dft_neumann_mask));
        else
          ps = std::make_unique<Poisson::DFTPatchSolver<D>>(*op, std::bitset<6>(dft_neumann_mask));
      } else {
        ps = std::make_unique<Iterative::PatchSolver<D>>(inner, *op, cont != 0);
      }
      Vector<D> fv = wrap<D>(dom, nc, const_cast<double*>(f));
      Vector<D> uv = wrap<D>(dom, nc, u);
      if (mode == 0)
        ps->smooth(fv, uv);
      else
        ps->apply(fv, uv);
    };
    if (d->dim == 2)
      run(make_domain<2>(d), std::integral_constant<int, 2>());
    else
      run(make_domain<3>(d), std::integral_constant<int, 3>());
  });
}

int teref_restrict(const te_level_desc* fine, const te_level_desc* coarse, int extrapolate, int nc,
                   const double* f, double* c) {
  return guard([&] {
    auto run = [&](auto fd, auto cd, auto tag) {
      constexpr int D = decltype(tag)::value;
      GMG::LinearRestrictor<D> r(fd, cd, extrapolate != 0);
      Vector<D> out = r.restrict(wrap<D>(fd, nc, const_cast<double*>(f)));
      copy_out<D>(out, c);
    };
    if (fine->dim == 2)
      run(make_domain<2>(fine, 0), make_domain<2>(coarse, 1), std::integral_constant<int, 2>());
    else
      run(make_domain<3>(fine, 0), make_domain<3>(coarse, 1), std::integral_constant<int, 3>());
  });
}

int teref_interpolate(const te_level_desc* coarse, const te_level_desc* fine, int nc, const double* c,
                      double* f) {
  return guard([&] {
    auto run = [&](auto cd, auto fd, auto tag) {
      constexpr int D = decltype(tag)::value;
      GMG::DirectInterpolator<D> in(cd, fd);
      Vector<D> fv = wrap<D>(fd, nc, f);
      in.interpolate(wrap<D>(cd, nc, const_cast<double*>(c)), fv);
    };
    if (fine->dim == 2)
      run(make_domain<2>(coarse, 1), make_domain<2>(fine, 0), std::integral_constant<int, 2>());
    else
      run(make_domain<3>(coarse, 1), make_domain<3>(fine, 0), std::integral_constant<int, 3>());
  });
}

int teref_vcycle_apply(const te_level_desc* levels, int nlevels, const teo_gmg_config* cfg,
                       const double* const* coeffs, int nc, const double* f, double* u) {
  int rc = TE_OK;
  int g = guard([&] {
    if (levels[0].dim == 2)
      rc = gmg<2>(levels, nlevels, cfg, coeffs, nc, u, f, nullptr, nullptr, false);
    else
      rc = gmg<3>(levels, nlevels, cfg, coeffs, nc, u, f, nullptr, nullptr, false);
  });
  return g != TE_OK ? g : rc;
}

int teref_gmg_solve(const te_level_desc* levels, int nlevels, const teo_gmg_config* cfg,
                    const double* const* coeffs, int nc, double* u, const double* f, int* iterations,
                    double* final_residual) {
  int rc = TE_OK;
  int g = guard([&] {
    if (levels[0].dim == 2)
      rc = gmg<2>(levels, nlevels, cfg, coeffs, nc, u, f, iterations, final_residual, true);
    else
      rc = gmg<3>(levels, nlevels, cfg, coeffs, nc, u, f, iterations, final_residual, true);
  });
  return g != TE_OK ? g : rc;
}

// Domain<D> built by ThunderEgg from the tables, flattened again by the C++
// adapters' thunderegg_gb300::flatten (include/thunderegg_gb300/adapters.hpp):
// the round trip the adapters rely on.  Output arrays have the input's sizes.
// the reference's own right-hand-side boundary helpers (Poisson/StarPatchOperator.h:187-242,
// VarPoisson/StarPatchOperator.h:194-219) with C callbacks as the boundary data
int teref_add_bc_to_rhs(const te_level_desc* d, int kind, int neumann, teo_point_fn gfun, teo_point_fn hfun,
                        const teo_point_fn* grad, double* f) {
  return guard([&] {
    auto run = [&](auto dom, auto tag) {
      constexpr int D = decltype(tag)::value;
      auto wrapfn = [](teo_point_fn fn) {
        return std::function<double(const std::array<double, D>&)>(
            [fn](const std::array<double, D>& x) { return fn(x.data()); });
      };
      auto gf = make_filler<D>(dom, TE_GHOST_BILINEAR + (D == 3 ? 2 : 0), TE_FILL_FACES);
      Vector<D> fv = wrap<D>(dom, 1, f);
      if (kind == 0) {
        Poisson::StarPatchOperator<D> op(dom, *gf);
        if (neumann) {
          std::array<std::function<double(const std::array<double, D>&)>, D> g;
          for (int a = 0; a < D; a++) g[a] = wrapfn(grad[a]);
          op.addNeumannBCToRHS(fv, wrapfn(gfun), g);
        } else {
          op.addDrichletBCToRHS(fv, wrapfn(gfun));
        }
      } else {
        std::vector<double> ones((size_t)dom.getNumLocalPatches() * [&] {
          long s = 1;
          for (int a = 0; a < D; a++) s *= dom.getNs()[a] + 2 * dom.getNumGhostCells();
          return s;
        }(), 1.0);
        Vector<D> c = wrap<D>(dom, 1, ones.data());
        VarPoisson::StarPatchOperator<D> op(c, dom, *gf);
        op.addDrichletBCToRHS(fv, wrapfn(gfun), wrapfn(hfun));
      }
    };
    if (d->dim == 2)
      run(make_domain<2>(d), std::integral_constant<int, 2>());
    else
      run(make_domain<3>(d), std::integral_constant<int, 3>());
  });
}

int teref_flatten_roundtrip(const te_level_desc* in, int* id, int* refine_level, int* parent_id,
                            int* orth_on_parent, int* child_ids, double* starts, double* spacings, int* nbr_type,
                            int* nbr_ids, int* nbr_orth) {
  return guard([&] {
    auto out = [&](auto t) {
      std::copy(t.id.begin(), t.id.end(), id);
      std::copy(t.refine_level.begin(), t.refine_level.end(), refine_level);
      std::copy(t.parent_id.begin(), t.parent_id.end(), parent_id);
      std::copy(t.orth_on_parent.begin(), t.orth_on_parent.end(), orth_on_parent);
      std::copy(t.child_ids.begin(), t.child_ids.end(), child_ids);
      std::copy(t.starts.begin(), t.starts.end(), starts);
      std::copy(t.spacings.begin(), t.spacings.end(), spacings);
      std::copy(t.nbr_type.begin(), t.nbr_type.end(), nbr_type);
      std::copy(t.nbr_ids.begin(), t.nbr_ids.end(), nbr_ids);
      std::copy(t.nbr_orth.begin(), t.nbr_orth.end(), nbr_orth);
    };
    if (in->dim == 2)
      out(thunderegg_gb300::flatten<2>(make_domain<2>(in)));
    else
      out(thunderegg_gb300::flatten<3>(make_domain<3>(in)));
  });
}

// One level of a mesh JSON file (a PatchInfo array, json.cpp:240-300) read by
// ThunderEgg's own from_json into a Domain<D>, then flattened like
// teref_flatten_roundtrip: checks that files written by this repository's
// mesh.save_json_hierarchy are read by the reference as intended.
int teref_json_level(const char* text, int dim, int n, int num_ghost, int num_patches, int* id, int* refine_level,
                     int* parent_id, int* orth_on_parent, int* child_ids, double* starts, double* spacings,
                     int* nbr_type, int* nbr_ids, int* nbr_orth) {
  return guard([&] {
    auto out = [&](auto t) {
      if ((int)t.id.size() != num_patches) throw std::runtime_error("patch count differs");
      std::copy(t.id.begin(), t.id.end(), id);
      std::copy(t.refine_level.begin(), t.refine_level.end(), refine_level);
      std::copy(t.parent_id.begin(), t.parent_id.end(), parent_id);
      std::copy(t.orth_on_parent.begin(), t.orth_on_parent.end(), orth_on_parent);
      std::copy(t.child_ids.begin(), t.child_ids.end(), child_ids);
      std::copy(t.starts.begin(), t.starts.end(), starts);
      std::copy(t.spacings.begin(), t.spacings.end(), spacings);
      std::copy(t.nbr_type.begin(), t.nbr_type.end(), nbr_type);
      std::copy(t.nbr_ids.begin(), t.nbr_ids.end(), nbr_ids);
      std::copy(t.nbr_orth.begin(), t.nbr_orth.end(), nbr_orth);
    };
    auto read = [&](auto dimc) {
      constexpr int D = decltype(dimc)::value;
      std::vector<PatchInfo<D>> pinfos = tpl::nlohmann::json::parse(text).get<std::vector<PatchInfo<D>>>();
      std::array<int, D> ns;
      ns.fill(n);
      for (PatchInfo<D>& pi : pinfos) {
        pi.ns = ns;
        pi.num_ghost_cells = num_ghost;
        for (int a = 0; a < D; a++) pi.spacings[a] /= n;  // the file holds lengths
      }
      out(thunderegg_gb300::flatten<D>(
          Domain<D>(Communicator(MPI_COMM_WORLD), 0, ns, num_ghost, pinfos.begin(), pinfos.end())));
    };
    if (dim == 2)
      read(std::integral_constant<int, 2>());
    else
      read(std::integral_constant<int, 3>());
  });
}

}  // extern "C"
