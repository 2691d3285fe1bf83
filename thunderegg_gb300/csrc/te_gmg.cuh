// te_gmg.cuh -- transfer and cycle handles (internal).
#pragma once
#include <map>
#include <set>
#include <string>
#include <utility>

#include "te_ops.cuh"

struct te_restrictor {
  const te_domain* fine = nullptr;
  const te_domain* coarse = nullptr;
  int extrapolate = 0;
  // children of each coarse patch, in fine-patch order
  te::DevBuf<int> child_start;  // [Pc+1]
  te::DevBuf<int> child;        // fine local index
  te::DevBuf<int> child_orth;   // orth_on_parent (-1 = copied patch)
  te::DevBuf<int8_t> child_corner_nbr;  // fine patch has a neighbour at Corner(orth)
  // even patch sizes: child by orthant per coarse patch, or the copied fine patch
  bool even = false;
  te::DevBuf<int> by_orth;   // [Pc * 2^D]
  te::DevBuf<int> copy_of;   // [Pc]
  // every coarse patch is a copy or has all 2^D children: each fine patch
  // writes its quadrant of the parent (fine-patch-centric kernels)
  bool complete = false;
  te::DevBuf<int> fine_parent;  // [Pf] coarse local index
  te::DevBuf<int> fine_orth;    // [Pf] orth_on_parent, -1 for a copied patch
};

struct te_interpolator {
  const te_domain* coarse = nullptr;
  const te_domain* fine = nullptr;
  te::DevBuf<int> parent;  // coarse local index of each fine patch
  te::DevBuf<int> orth;    // orth_on_parent of each fine patch
};

namespace te {
void restrict_level(const te_restrictor* r, int nc, int dtype, const void* fine, void* coarse, cudaStream_t s);
void interpolate_level(const te_interpolator* in, int nc, int dtype, const void* coarse, void* fine,
                       cudaStream_t s);
void residual_restrict(const te_restrictor* r, const te_operator* op, int nc, int dtype, const void* f,
                       const void* u, void* coarse, cudaStream_t s);
void residual(const te_domain* d, int nc, int dtype, const void* f, void* r, cudaStream_t s);
// fused per-level kernels of the DFT-smoother V-cycle (te_fused.cu)
template <class T, class TF>
void vc_pre(const te_patch_solver* ps, const TF* f, T* out, cudaStream_t s);
template <class T, class TF>
void vc_restrict(const te_restrictor* r, const te_operator* op, const T* u, const TF* f, T* coarse,
                 cudaStream_t s);
template <class T, class TF, class TO>
void vc_post(const te_patch_solver* ps, const te_interpolator* in, const T* A, const T* uc, const TF* f, TO* out,
             cudaStream_t s);
// boundary corrections of the post-smooth right-hand side (FP32), [P][2D][face cells]
void vc_corr(const te_patch_solver* ps, const te_interpolator* in, const float* A, const float* uc, float* corr,
             cudaStream_t s);
int corr_stride(const Layout& L);
// fine-patch-centric residual + restriction (te_restrict.cu); false when the hierarchy does not qualify
template <class T, class TF>
bool vc_restrict_fine(const te_restrictor* r, const te_operator* op, const T* u, const TF* f, T* coarse,
                      cudaStream_t s);
}  // namespace te

// ---------------------------------------------------------------------------
// V-cycle
// ---------------------------------------------------------------------------
// The launch sequence of one cycle application is fixed, so it is captured
// once per (f, u) buffer pair into a CUDA graph on a private stream and
// replayed; the caller's stream is ordered around it with events.
// Set TE_NO_GRAPH=1 in the environment to launch eagerly instead.
struct te_cycle {
  std::vector<te_cycle_level> levels;
  te_cycle_opts opts{1, 1, 1, 1};
  int type = TE_CYCLE_V;  // CycleOpts::cycle_type "V", "W" or "F"
  int dtype = TE_F64;
  int nc = 1;
  cudaStream_t stream = nullptr;  // caller's stream (that of the level handles)
  cudaStream_t cap = nullptr;     // private capture stream
  cudaEvent_t ev_in = nullptr, ev_out = nullptr;
  bool use_graph = true;
  unsigned long long serial = 0;      // unique per cycle object
  unsigned long long generation = 0;  // bumped whenever the work buffers are reallocated
  struct G {
    cudaGraph_t g = nullptr;
    cudaGraphExec_t x = nullptr;
    long long launches = 0;
  };
  std::map<std::pair<const void*, void*>, G> graphs;
  std::set<std::pair<const void*, void*>> warmed;  // keys whose first application ran eagerly
  // per-level work buffers in the cycle's precision
  std::vector<te::DevBuf<char>> f, u, r;
  std::vector<te::DevBuf<char>> corr;  // tensor-core post-smooth: right-hand-side corrections per level
  // optional per-kernel timing of one eager application (te_cycle_timings)
  struct Mark {
    std::string name;
    cudaEvent_t ev;
  };
  mutable std::vector<Mark>* marks = nullptr;
  void mark(const std::string& name, cudaStream_t s) const {
    if (!marks) return;
    cudaEvent_t e;
    TE_CUDA(cudaEventCreate(&e));
    TE_CUDA(cudaEventRecord(e, s));
    marks->push_back({name, e});
  }
  // fused path: every level smooths with the DFT solver, one pre/post sweep,
  // even patch sizes, no ghost extrapolation, one component
  bool fusable = false;
  bool fused() const { return fusable && nc == 1 && type == TE_CYCLE_V; }
  // the W and FMG cycles run fused when every level takes the tensor-core path
  bool fused_wf() const {
    if (!fusable || nc != 1 || type == TE_CYCLE_V || dtype != TE_F32) return false;
    for (size_t k = 0; k < levels.size(); k++)
      if (!use_tc((int)k)) return false;
    return true;
  }
  // the FP32 fused cycle runs the DFT solves of level k on the tensor cores
  bool tc_enabled = true;
  bool use_tc(int k) const { return tc_enabled && dtype == TE_F32 && levels[k].smoother->tc_ok; }
  ~te_cycle() {
    clear_graphs();
    if (ev_in) cudaEventDestroy(ev_in);
    if (ev_out) cudaEventDestroy(ev_out);
    if (cap) cudaStreamDestroy(cap);
  }
  void clear_graphs() {
    for (auto& kv : graphs) {
      if (kv.second.x) cudaGraphExecDestroy(kv.second.x);
      if (kv.second.g) cudaGraphDestroy(kv.second.g);
    }
    graphs.clear();
  }
  size_t esize() const { return dtype == TE_F64 ? 8 : 4; }
  const te_domain* dom(int k) const { return levels[k].op->dom; }
  size_t bytes(int k) const { return (size_t)dom(k)->lay.P * dom(k)->lay.pstride(nc) * esize(); }
  void ensure(int nc_in) {
    if (nc_in == nc && !f.empty()) return;
    clear_graphs();
    generation++;
    nc = nc_in;
    size_t L = levels.size();
    f.clear();
    u.clear();
    r.clear();
    corr.clear();
    f.resize(L);
    u.resize(L);
    r.resize(L);
    corr.resize(L);
    for (size_t k = 0; k < L; k++) {
      r[k].alloc(bytes(k));
      u[k].alloc(bytes(k));
      if (k > 0 || dtype != TE_F64) f[k].alloc(bytes(k));
      if (use_tc((int)k)) {
        const te::Layout& Lk = dom(k)->lay;
        corr[k].alloc((size_t)Lk.P * 2 * Lk.D * te::corr_stride(Lk) * sizeof(float));
      }
    }
  }
  // Fused V-cycle: A = u[k] holds the pre-smoothed iterate, r[k] the post-smoothed
  // one (the level's result); returns the buffer holding the level's result.
  template <class T, class TF, class TO>
  const T* vfused(int k, const TF* fk, TO* out, cudaStream_t s) const {
    int last = (int)levels.size() - 1;
    T* A = (T*)u[k].p;
    const te_patch_solver* ps = levels[k].smoother;
    const bool tc = use_tc(k);
    if (tc)
      te::dft_tc<TF, T>(ps, fk, A, s);
    else
      te::vc_pre<T, TF>(ps, fk, A, s);
    mark("L" + std::to_string(k) + " pre-smooth", s);
    if (k == last) return A;
    T* fc = (T*)f[k + 1].p;
    te::vc_restrict<T, TF>(levels[k].restrictor, levels[k].op, A, fk, fc, s);
    mark("L" + std::to_string(k) + " residual+restrict", s);
    const T* uc = vfused<T, T, T>(k + 1, fc, (T*)r[k + 1].p, s);
    if (tc) {
      // boundary corrections of the corrected iterate (never stored), then the solve from f
      float* cr = (float*)corr[k].p;
      te::vc_corr(ps, levels[k + 1].interpolator, (const float*)A, (const float*)uc, cr, s);
      mark("L" + std::to_string(k) + " interpolate+post-corrections", s);
      te::dft_tc<TF, TO>(ps, fk, out, s, cr);
      mark("L" + std::to_string(k) + " post-smooth", s);
    } else {
      te::vc_post<T, TF, TO>(ps, levels[k + 1].interpolator, A, uc, fk, out, s);
      mark("L" + std::to_string(k) + " interpolate+post-smooth", s);
    }
    return (const T*)out;
  }
  // ---- the W and FMG cycles on the tensor-core path (FP32 in and out, one sweep each)
  // PatchSolver::smooth of level k from the iterate uin (nullptr: zero) into out: the
  // tensor-core solve of f minus the boundary corrections of uin
  void smooth_tc(int k, const float* fk, const float* uin, float* out, cudaStream_t s) const {
    const te_patch_solver* ps = levels[k].smoother;
    if (!uin) {
      te::dft_tc<float, float>(ps, fk, out, s);
      return;
    }
    float* cr = (float*)corr[k].p;
    te::vc_corr(ps, nullptr, uin, nullptr, cr, s);
    te::dft_tc<float, float>(ps, fk, out, s, cr);
  }
  // interpolate the coarse correction uc into A and smooth, into out: the corrections of
  // A + P uc (never stored), then the solve (out may be A: A is read only by the corrections)
  void corr_smooth_tc(int k, const float* fk, const float* A, const float* uc, float* out, cudaStream_t s) const {
    float* cr = (float*)corr[k].p;
    te::vc_corr(levels[k].smoother, levels[k + 1].interpolator, A, uc, cr, s);
    te::dft_tc<float, float>(levels[k].smoother, fk, out, s, cr);
  }
  // WCycle::visit (GMG/WCycle.h:50-84) and FMGCycle::visit (GMG/FMGCycle.h:68-104); uin: the
  // level's iterate on entry (nullptr: zero).  u[k] holds the pre- and mid-smoothed iterate,
  // r[k + 1] the coarse result, which the second coarse visit starts from (as in the reference)
  void wf_visit(int k, const float* fk, float* out, const float* uin, cudaStream_t s) const {
    const int last = (int)levels.size() - 1;
    if (k == last) {
      smooth_tc(k, fk, uin, out, s);
      return;
    }
    float* A = (float*)u[k].p;
    float* fc = (float*)f[k + 1].p;
    float* uc = (float*)r[k + 1].p;
    smooth_tc(k, fk, uin, A, s);
    te::vc_restrict<float, float>(levels[k].restrictor, levels[k].op, A, fk, fc, s);
    wf_visit(k + 1, fc, uc, nullptr, s);
    corr_smooth_tc(k, fk, A, uc, A, s);  // mid smooth
    te::vc_restrict<float, float>(levels[k].restrictor, levels[k].op, A, fk, fc, s);
    if (type == TE_CYCLE_W)
      wf_visit(k + 1, fc, uc, uc, s);
    else
      fmg_v_visit(k + 1, fc, uc, uc, s);
    corr_smooth_tc(k, fk, A, uc, out, s);
  }
  // FMGCycle::v_visit (GMG/FMGCycle.h:43-66) from the iterate uin; its coarser visit is wf_visit
  void fmg_v_visit(int k, const float* fk, float* out, const float* uin, cudaStream_t s) const {
    const int last = (int)levels.size() - 1;
    if (k == last) {
      smooth_tc(k, fk, uin, out, s);
      return;
    }
    float* A = (float*)u[k].p;
    float* fc = (float*)f[k + 1].p;
    float* uc = (float*)r[k + 1].p;
    smooth_tc(k, fk, uin, A, s);
    te::vc_restrict<float, float>(levels[k].restrictor, levels[k].op, A, fk, fc, s);
    wf_visit(k + 1, fc, uc, nullptr, s);
    corr_smooth_tc(k, fk, A, uc, out, s);
  }

  // `fresh`: u is known to be zero (ghosts included) before the first sweep
  void smooth(int k, const void* fk, void* uk, int times, bool fresh, cudaStream_t s) const {
    for (int i = 0; i < times; i++) te::patch_smooth(levels[k].smoother, nc, dtype, fk, uk, fresh && i == 0, s);
  }
  // Cycle::restrict (GMG/Cycle.h:57-65) into f[k + 1]; `fresh`: u is still zero
  void restrict_residual(int k, const void* fk, void* uk, bool fresh, cudaStream_t s) const {
    void* fc = f[k + 1].p;
    const te_restrictor* R = levels[k].restrictor;
    if (!R->extrapolate && !fresh) {
      // fused: fill ghosts, then r = f - A u restricted
      te::ghost_fill(levels[k].op->gf, nc, dtype, uk, s);
      te::residual_restrict(R, levels[k].op, nc, dtype, fk, uk, fc, s);
    } else {
      void* rk = r[k].p;
      te::operator_apply(levels[k].op, nc, dtype, uk, rk, s);
      te::residual(dom(k), nc, dtype, fk, rk, s);
      te::restrict_level(R, nc, dtype, rk, fc, s);
    }
  }
  // the coarse iterate u[k + 1] starts at zero (getZeroClone); a first sweep
  // from a fresh iterate writes every cell, otherwise it is cleared here
  void zero_coarse(int k, cudaStream_t s) const {
    const int last = (int)levels.size() - 1;
    const int first = k + 1 == last ? opts.coarse_sweeps : opts.pre_sweeps;
    if (first == 0) TE_CUDA(cudaMemsetAsync(u[k + 1].p, 0, bytes(k + 1), s));
  }
  // VCycle::visit (GMG/VCycle.h:46-70), WCycle::visit (GMG/WCycle.h:50-84),
  // FMGCycle::visit (GMG/FMGCycle.h:68-104).  `fresh`: u is zero on entry.
  // The W and FMG cycles smooth mid_sweeps times after the first coarse
  // correction, restrict the new residual and visit the coarser level again
  // from its first result (u[k + 1] is not cleared in between, as in the
  // reference); the FMG cycle's second visit is its v_visit.
  void visit(int k, const void* fk, void* uk, bool fresh, cudaStream_t s) const {
    const int last = (int)levels.size() - 1;
    if (k == last) {
      smooth(k, fk, uk, opts.coarse_sweeps, fresh, s);
      return;
    }
    smooth(k, fk, uk, opts.pre_sweeps, fresh, s);
    restrict_residual(k, fk, uk, fresh && opts.pre_sweeps == 0, s);
    void* fc = f[k + 1].p;
    void* uc = u[k + 1].p;
    zero_coarse(k, s);
    visit(k + 1, fc, uc, true, s);
    te::interpolate_level(levels[k + 1].interpolator, nc, dtype, uc, uk, s);
    if (type != TE_CYCLE_V) {
      smooth(k, fk, uk, opts.mid_sweeps, false, s);
      restrict_residual(k, fk, uk, false, s);
      if (type == TE_CYCLE_W)
        visit(k + 1, fc, uc, false, s);
      else
        v_visit(k + 1, fc, uc, s);
      te::interpolate_level(levels[k + 1].interpolator, nc, dtype, uc, uk, s);
    }
    smooth(k, fk, uk, opts.post_sweeps, false, s);
  }
  // FMGCycle::v_visit (GMG/FMGCycle.h:43-66): u enters with the level's previous
  // result; one pre/post-smoothed pass whose coarser visit is visit()
  void v_visit(int k, const void* fk, void* uk, cudaStream_t s) const {
    const int last = (int)levels.size() - 1;
    if (k == last) {
      smooth(k, fk, uk, opts.coarse_sweeps, false, s);
      return;
    }
    smooth(k, fk, uk, opts.pre_sweeps, false, s);
    restrict_residual(k, fk, uk, false, s);
    zero_coarse(k, s);
    visit(k + 1, f[k + 1].p, u[k + 1].p, true, s);
    te::interpolate_level(levels[k + 1].interpolator, nc, dtype, u[k + 1].p, uk, s);
    smooth(k, fk, uk, opts.post_sweeps, false, s);
  }
  // sweeps of the finest level's first smooth; a single-level cycle clears u first
  int first_sweeps() const { return levels.size() == 1 ? 0 : opts.pre_sweeps; }
  void body(const void* f64, void* u64, cudaStream_t s) const {
    // Cycle::apply (GMG/Cycle.h:94-98): u.setWithGhost(0); visit(finest, f, u)
    if (fused()) {
      if (dtype == TE_F64)
        vfused<double, double, double>(0, (const double*)f64, (double*)u64, s);
      else
        vfused<float, double, double>(0, (const double*)f64, (double*)u64, s);
      return;
    }
    if (dtype == TE_F64) {
      if (first_sweeps() == 0) TE_CUDA(cudaMemsetAsync(u64, 0, bytes(0), s));
      visit(0, f64, u64, true, s);
    } else if (fused_wf()) {
      te::convert_level(dom(0), nc, dtype, f[0].p, TE_F64, f64, s);
      wf_visit(0, (const float*)f[0].p, (float*)r[0].p, nullptr, s);
      te::convert_level(dom(0), nc, TE_F64, u64, dtype, r[0].p, s);
    } else {
      te::convert_level(dom(0), nc, dtype, f[0].p, TE_F64, f64, s);
      if (first_sweeps() == 0) TE_CUDA(cudaMemsetAsync(u[0].p, 0, bytes(0), s));
      visit(0, f[0].p, u[0].p, true, s);
      te::convert_level(dom(0), nc, TE_F64, u64, dtype, u[0].p, s);
    }
  }
  // FP32 in and out (dtype TE_F32): the float-float outer Krylov loop passes the
  // hi half of its vectors and takes an FP32 result
  void body_f32(const float* f32, float* u32, cudaStream_t s) const {
    if (fused()) {
      vfused<float, float, float>(0, f32, u32, s);
      return;
    }
    if (fused_wf()) {
      wf_visit(0, f32, u32, nullptr, s);
      return;
    }
    if (first_sweeps() == 0) TE_CUDA(cudaMemsetAsync(u32, 0, bytes(0), s));
    visit(0, f32, u32, true, s);
  }
  // run on stream s (which may itself be capturing)
  void apply_on(const void* f64, void* u64, cudaStream_t s) {
    if (!use_graph) {
      body(f64, u64, s);
      return;
    }
    auto key = std::make_pair(f64, u64);
    auto it = graphs.find(key);
    if (it == graphs.end() && !warmed.count(key)) {
      cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
      TE_CUDA(cudaStreamIsCapturing(s, &cs));
      if (cs == cudaStreamCaptureStatusNone) {
        // the first application runs eagerly: the autotuner times the launch shapes it has not
        // met (a capture cannot be timed); the graph is captured on the next application
        warmed.insert(key);
        body(f64, u64, s);
        return;
      }
    }
    if (it == graphs.end()) {
      G g;
      long long l0 = te::g_launches.load();
      TE_CUDA(cudaStreamBeginCapture(cap, cudaStreamCaptureModeThreadLocal));
      try {
        body(f64, u64, cap);
      } catch (...) {
        cudaGraph_t junk;
        cudaStreamEndCapture(cap, &junk);
        if (junk) cudaGraphDestroy(junk);
        throw;
      }
      TE_CUDA(cudaStreamEndCapture(cap, &g.g));
      TE_CUDA(cudaGraphInstantiate(&g.x, g.g, 0));
      g.launches = te::g_launches.load() - l0;
      te::g_launches.fetch_sub(g.launches);
      it = graphs.emplace(key, g).first;
    }
    TE_CUDA(cudaEventRecord(ev_in, s));
    TE_CUDA(cudaStreamWaitEvent(cap, ev_in, 0));
    TE_CUDA(cudaGraphLaunch(it->second.x, cap));
    te::count_launch((int)it->second.launches);
    TE_CUDA(cudaEventRecord(ev_out, cap));
    TE_CUDA(cudaStreamWaitEvent(s, ev_out, 0));
  }
};

