// te_gmg.cu -- GMG transfers, the V-cycle and the outer BiCGStab.
//
//   GMG::LinearRestrictor (GMG/LinearRestrictor.h:49-191) through
//     MPIRestrictor::restrict (GMG/MPIRestrictor.h:55-83): gathered per coarse
//     cell from the children in fine-patch order (InterLevelComm parent map,
//     GMG/InterLevelComm.h:125-160), so each coarse patch is written by one CTA.
//   GMG::DirectInterpolator (GMG/DirectInterpolator.h:60-91): fine += coarse.
//   GMG::VCycle::visit (GMG/VCycle.h:46-70), Cycle::restrict/apply (GMG/Cycle.h:57-98).
//   Iterative::BiCGStab::solve (Iterative/BiCGStab.h:111-203).

#include <cmath>
#include <cstring>

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
};

struct te_interpolator {
  const te_domain* coarse = nullptr;
  const te_domain* fine = nullptr;
  te::DevBuf<int> parent;  // coarse local index of each fine patch
  te::DevBuf<int> orth;    // orth_on_parent of each fine patch
};

namespace te {

static std::vector<int> parent_map(const te_domain* fine, const te_domain* coarse) {
  std::vector<int> m(fine->lay.P);
  for (int p = 0; p < fine->lay.P; p++) {
    auto it = coarse->id2l.find(fine->parent_id[p]);
    require(it != coarse->id2l.end(), "parent patch not on the coarser level");
    m[p] = it->second;
  }
  return m;
}

// ---------------------------------------------------------------------------
// restriction: one CTA per coarse patch, one thread per coarse cell
// ---------------------------------------------------------------------------
template <class T>
__global__ void restrict_kernel(Layout F, Layout C, int nc, const int* __restrict__ cstart,
                                const int* __restrict__ child, const int* __restrict__ corth,
                                const int8_t* __restrict__ corner_nbr, int extrapolate, const T* __restrict__ fine,
                                T* __restrict__ coarse) {
  int cp = blockIdx.x;
  long long fps = F.pstride(nc), cps = C.pstride(nc);
  int k0 = cstart[cp], k1 = cstart[cp + 1];
  int D = C.D;
  T wD = T(1.0 / (1 << D));
  int py = C.n1 + 2 * C.g;
  for (long long e = threadIdx.x; e < cps; e += blockDim.x) {
    int c = (int)(e / C.cs), k = (int)(e % C.cs);
    int cc[3];
    cc[0] = k % C.sy - C.g;
    cc[1] = (k / C.sy) % py - C.g;
    cc[2] = D == 3 ? k / C.sz - C.g : 0;
    bool in_c[3];
    int nout = 0;
    for (int a = 0; a < 3; a++) {
      in_c[a] = cc[a] >= 0 && cc[a] < C.n(a);
      nout += !in_c[a];
    }
    T v = T(0);
    for (int q = k0; q < k1; q++) {
      int fp = child[q], o = corth[q];
      const T* fv = fine + fp * fps + (long long)c * F.cs;
      if (o < 0) {  // copyToParent (:129-147)
        if (nout == 0 || extrapolate) v += fv[k];
        continue;
      }
      int st[3] = {0, 0, 0};
      for (int a = 0; a < D; a++) st[a] = ((o >> a) & 1) ? C.n(a) : 0;
      if (nout == 0) {  // restrictToCoarserParent (:101-128): fine loop order z, y, x
        int lo[3], hi[3];
        for (int a = 0; a < 3; a++) {
          if (a < D) {
            lo[a] = max(2 * cc[a] - st[a], 0);
            hi[a] = min(2 * cc[a] + 1 - st[a], F.n(a) - 1);
          } else {
            lo[a] = hi[a] = 0;
          }
        }
        for (int z = lo[2]; z <= hi[2]; z++)
          for (int y = lo[1]; y <= hi[1]; y++)
            for (int x = lo[0]; x <= hi[0]; x++) v += fv[F.at(x, y, z)] * wD;
        continue;
      }
      if (!extrapolate) continue;
      // extrapolateBoundaries (:49-100)
      if (nout == 1) {
        int a = !in_c[0] ? 0 : (!in_c[1] ? 1 : 2);
        int side_up = cc[a] >= C.n(a);
        if (((o >> a) & 1) != side_up) continue;  // not an exterior side of this orthant
        int lo[3], hi[3];
        for (int b = 0; b < 3; b++) {
          if (b == a || b >= D) {
            lo[b] = hi[b] = 0;
          } else {
            lo[b] = max(2 * cc[b] - st[b], 0);
            hi[b] = min(2 * cc[b] + 1 - st[b], F.n(b) - 1);
          }
        }
        int fin = side_up ? F.n(a) - 1 : 0, fgh = side_up ? F.n(a) : -1;
        for (int z = lo[2]; z <= hi[2]; z++)
          for (int y = lo[1]; y <= hi[1]; y++)
            for (int x = lo[0]; x <= hi[0]; x++) {
              int ci[3] = {x, y, z}, cg[3] = {x, y, z};
              ci[a] = fin;
              cg[a] = fgh;
              v += (T(3) * fv[F.at(cg[0], cg[1], cg[2])] - fv[F.at(ci[0], ci[1], ci[2])]) * wD;
            }
      } else if (nout == D) {  // corner ghost: Corner(orth) without neighbour
        bool match = true;
        for (int a = 0; a < D; a++) match &= (cc[a] >= C.n(a)) == (((o >> a) & 1) != 0);
        for (int a = 0; a < D; a++) match &= (cc[a] == -1 || cc[a] == C.n(a));
        if (!match || corner_nbr[q]) continue;
        int ci[3] = {0, 0, 0}, cg[3] = {0, 0, 0};
        for (int a = 0; a < D; a++) {
          bool up = (o >> a) & 1;
          ci[a] = up ? F.n(a) - 1 : 0;
          cg[a] = up ? F.n(a) : -1;
        }
        v += T(3) * fv[F.at(cg[0], cg[1], cg[2])] - fv[F.at(ci[0], ci[1], ci[2])];
      }
    }
    coarse[cp * cps + e] = v;
  }
}

template <class T>
__global__ void interpolate_kernel(Layout F, Layout C, int nc, const int* __restrict__ parent,
                                   const int* __restrict__ orth, const T* __restrict__ coarse, T* fine) {
  int fp = blockIdx.x;
  long long fps = F.pstride(nc), cps = C.pstride(nc);
  int o = orth[fp];
  const T* cv = coarse + (long long)parent[fp] * cps;
  T* fv = fine + fp * fps;
  int N = F.interior();
  int st[3] = {0, 0, 0};
  if (o >= 0)
    for (int a = 0; a < F.D; a++) st[a] = ((o >> a) & 1) ? C.n(a) : 0;
  for (int e = threadIdx.x; e < N * nc; e += blockDim.x) {
    int c = e / N, r = e % N;
    int x = r % F.n0, y = (r / F.n0) % F.n1, z = r / (F.n0 * F.n1);
    int k = F.at(x, y, z);
    T add;
    if (o >= 0)
      add = cv[(long long)c * C.cs + C.at((x + st[0]) / 2, F.D > 1 ? (y + st[1]) / 2 : 0, F.D > 2 ? (z + st[2]) / 2 : 0)];
    else
      add = cv[(long long)c * C.cs + k];
    fv[(long long)c * F.cs + k] += add;
  }
}

void restrict_level(const te_restrictor* r, int nc, int dtype, const void* fine, void* coarse, cudaStream_t s) {
  const Layout &F = r->fine->lay, &C = r->coarse->lay;
  if (dtype == TE_F64)
    restrict_kernel<double><<<C.P, 256, 0, s>>>(F, C, nc, r->child_start.p, r->child.p, r->child_orth.p,
                                                r->child_corner_nbr.p, r->extrapolate, (const double*)fine,
                                                (double*)coarse);
  else
    restrict_kernel<float><<<C.P, 256, 0, s>>>(F, C, nc, r->child_start.p, r->child.p, r->child_orth.p,
                                               r->child_corner_nbr.p, r->extrapolate, (const float*)fine,
                                               (float*)coarse);
  count_launch();
  TE_LAUNCH_CHECK();
}

void interpolate_level(const te_interpolator* in, int nc, int dtype, const void* coarse, void* fine,
                       cudaStream_t s) {
  const Layout &F = in->fine->lay, &C = in->coarse->lay;
  if (dtype == TE_F64)
    interpolate_kernel<double><<<F.P, 256, 0, s>>>(F, C, nc, in->parent.p, in->orth.p, (const double*)coarse,
                                                   (double*)fine);
  else
    interpolate_kernel<float><<<F.P, 256, 0, s>>>(F, C, nc, in->parent.p, in->orth.p, (const float*)coarse,
                                                  (float*)fine);
  count_launch();
  TE_LAUNCH_CHECK();
}

// r = f - r over interior cells (Cycle::restrict: r.scaleThenAdd(-1, f))
template <class T>
__global__ void residual_kernel(Layout L, int nc, long long n, const T* __restrict__ f, T* r) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    int x = (int)(i % L.n0);
    long long q = i / L.n0;
    int y = (int)(q % L.n1);
    q /= L.n1;
    int z = (int)(q % L.n2);
    q /= L.n2;
    long long k = q * L.cs + L.at(x, y, z);
    r[k] = r[k] * T(-1) + f[k];
  }
}

static void residual(const te_domain* d, int nc, int dtype, const void* f, void* r, cudaStream_t s) {
  long long n = (long long)d->lay.P * nc * d->lay.interior();
  int grid = (int)std::min<long long>((n + 255) / 256, 152 * 16);
  if (dtype == TE_F64)
    residual_kernel<double><<<grid, 256, 0, s>>>(d->lay, nc, n, (const double*)f, (double*)r);
  else
    residual_kernel<float><<<grid, 256, 0, s>>>(d->lay, nc, n, (const float*)f, (float*)r);
  count_launch();
  TE_LAUNCH_CHECK();
}

}  // namespace te

// ---------------------------------------------------------------------------
// V-cycle
// ---------------------------------------------------------------------------
struct te_cycle {
  std::vector<te_cycle_level> levels;
  te_cycle_opts opts{1, 1, 1, 1};
  int dtype = TE_F64;
  int nc = 1;
  cudaStream_t stream = nullptr;
  // per-level work buffers in the cycle's precision
  std::vector<te::DevBuf<char>> f, u, r;
  size_t esize() const { return dtype == TE_F64 ? 8 : 4; }
  const te_domain* dom(int k) const { return levels[k].op->dom; }
  size_t bytes(int k) const { return (size_t)dom(k)->lay.P * dom(k)->lay.pstride(nc) * esize(); }
  void ensure(int nc_in) {
    if (nc_in == nc && !f.empty()) return;
    nc = nc_in;
    size_t L = levels.size();
    f.clear();
    u.clear();
    r.clear();
    f.resize(L);
    u.resize(L);
    r.resize(L);
    for (size_t k = 0; k < L; k++) {
      r[k].alloc(bytes(k));
      if (k > 0 || dtype != TE_F64) {
        f[k].alloc(bytes(k));
        u[k].alloc(bytes(k));
      }
    }
  }
  void smooth(int k, const void* fk, void* uk, int times) const {
    for (int i = 0; i < times; i++) te::patch_smooth(levels[k].smoother, nc, dtype, fk, uk, false, stream);
  }
  // VCycle::visit (GMG/VCycle.h:46-70)
  void visit(int k, const void* fk, void* uk) const {
    int last = (int)levels.size() - 1;
    if (k == last) {
      smooth(k, fk, uk, opts.coarse_sweeps);
      return;
    }
    smooth(k, fk, uk, opts.pre_sweeps);
    // Cycle::restrict (GMG/Cycle.h:57-65): r = f - A u, then restrict(r)
    void* rk = r[k].p;
    te::operator_apply(levels[k].op, nc, dtype, uk, rk, stream);
    te::residual(dom(k), nc, dtype, fk, rk, stream);
    void* fc = f[k + 1].p;
    void* uc = u[k + 1].p;
    te::restrict_level(levels[k].restrictor, nc, dtype, rk, fc, stream);
    TE_CUDA(cudaMemsetAsync(uc, 0, bytes(k + 1), stream));
    visit(k + 1, fc, uc);
    te::interpolate_level(levels[k + 1].interpolator, nc, dtype, uc, uk, stream);
    smooth(k, fk, uk, opts.post_sweeps);
  }
  // Cycle::apply (GMG/Cycle.h:94-98); f and u are FP64 finest-level buffers
  void apply(const void* f64, void* u64) const {
    if (dtype == TE_F64) {
      TE_CUDA(cudaMemsetAsync(u64, 0, bytes(0), stream));
      visit(0, f64, u64);
    } else {
      te::convert_level(dom(0), nc, dtype, f[0].p, TE_F64, f64, stream);
      TE_CUDA(cudaMemsetAsync(u[0].p, 0, bytes(0), stream));
      visit(0, f[0].p, u[0].p);
      te::convert_level(dom(0), nc, TE_F64, u64, dtype, u[0].p, stream);
    }
  }
};

// ---------------------------------------------------------------------------
// outer BiCGStab, FP64, device vectors, host scalars (as the reference)
// ---------------------------------------------------------------------------
namespace te {

struct Krylov {
  const te_domain* d;
  int nc;
  cudaStream_t s;
  DevBuf<double> res;
  double* h = nullptr;
  Krylov(const te_domain* d, int nc) : d(d), nc(nc), s(d->stream), res(8) {
    TE_CUDA(cudaMallocHost(&h, 8 * sizeof(double)));
  }
  ~Krylov() {
    if (h) cudaFreeHost(h);
  }
  // launch up to 8 dot products, read them back with one synchronisation
  void dots(int n, const void* const* a, const void* const* b, double* out) {
    for (int i = 0; i < n; i++) reduce_dot(d, nc, TE_F64, a[i], b[i], res.p + i, s);
    TE_CUDA(cudaMemcpyAsync(h, res.p, n * sizeof(double), cudaMemcpyDeviceToHost, s));
    TE_CUDA(cudaStreamSynchronize(s));
    for (int i = 0; i < n; i++) out[i] = h[i];
  }
  double dot(const void* a, const void* b) {
    double o;
    dots(1, &a, &b, &o);
    return o;
  }
};

}  // namespace te

using namespace te;

extern "C" {

int te_linear_restrictor_create(const te_domain* fine, const te_domain* coarse, int extrapolate, te_restrictor** out) {
  return guard([&] {
    require(fine && coarse && out, "null argument");
    require(fine->lay.D == coarse->lay.D && fine->lay.n0 == coarse->lay.n0 && fine->lay.n1 == coarse->lay.n1 &&
                fine->lay.n2 == coarse->lay.n2 && fine->lay.g == coarse->lay.g,
            "levels must share patch shape");
    auto r = std::make_unique<te_restrictor>();
    r->fine = fine;
    r->coarse = coarse;
    r->extrapolate = extrapolate;
    auto pm = parent_map(fine, coarse);
    int Pc = coarse->lay.P;
    std::vector<std::vector<int>> kids(Pc);
    for (int p = 0; p < fine->lay.P; p++) kids[pm[p]].push_back(p);
    std::vector<int> start(Pc + 1, 0), child, orth;
    std::vector<int8_t> cnbr;
    for (int c = 0; c < Pc; c++) {
      start[c] = (int)child.size();
      for (int p : kids[c]) {
        child.push_back(p);
        int o = fine->orth_on_parent[p];
        orth.push_back(o);
        cnbr.push_back(o >= 0 && fine->nbr_type[(size_t)p * fine->F + o] >= 0 ? 1 : 0);
      }
    }
    start[Pc] = (int)child.size();
    cudaStream_t s = fine->stream;
    r->child_start.upload(start, s);
    r->child.upload(child, s);
    r->child_orth.upload(orth, s);
    r->child_corner_nbr.upload(cnbr, s);
    TE_CUDA(cudaStreamSynchronize(s));
    *out = r.release();
  });
}

int te_restrictor_destroy(te_restrictor* r) {
  delete r;
  return TE_OK;
}

int te_restrict(const te_restrictor* r, int nc, int dtype, const void* fine, void* coarse_out) {
  return guard([&] {
    require(r && fine && coarse_out, "null argument");
    restrict_level(r, nc, dtype, fine, coarse_out, r->fine->stream);
  });
}

int te_direct_interpolator_create(const te_domain* coarse, const te_domain* fine, te_interpolator** out) {
  return guard([&] {
    require(coarse && fine && out, "null argument");
    auto in = std::make_unique<te_interpolator>();
    in->coarse = coarse;
    in->fine = fine;
    cudaStream_t s = fine->stream;
    in->parent.upload(parent_map(fine, coarse), s);
    in->orth.upload(fine->orth_on_parent, s);
    TE_CUDA(cudaStreamSynchronize(s));
    *out = in.release();
  });
}

int te_interpolator_destroy(te_interpolator* i) {
  delete i;
  return TE_OK;
}

int te_interpolate(const te_interpolator* i, int nc, int dtype, const void* coarse, void* fine) {
  return guard([&] {
    require(i && coarse && fine, "null argument");
    interpolate_level(i, nc, dtype, coarse, fine, i->fine->stream);
  });
}

int te_vcycle_create(const te_cycle_level* levels, int num_levels, te_cycle_opts opts, int dtype, te_cycle** out) {
  return guard([&] {
    require(levels && out && num_levels >= 1, "bad arguments");
    require(dtype == TE_F64 || dtype == TE_F32, "bad dtype");
    auto c = std::make_unique<te_cycle>();
    c->levels.assign(levels, levels + num_levels);
    c->opts = opts;
    c->dtype = dtype;
    for (int k = 0; k < num_levels; k++) {
      require(levels[k].op && levels[k].smoother, "every level needs an operator and a smoother");
      if (k + 1 < num_levels) require(levels[k].restrictor != nullptr, "missing restrictor");
      if (k > 0) require(levels[k].interpolator != nullptr, "missing interpolator");
    }
    c->stream = levels[0].op->dom->stream;
    c->ensure(1);
    *out = c.release();
  });
}

int te_cycle_destroy(te_cycle* c) {
  delete c;
  return TE_OK;
}

int te_cycle_apply(const te_cycle* c, int nc, const void* f, void* u) {
  return guard([&] {
    require(c && f && u, "null argument");
    const_cast<te_cycle*>(c)->ensure(nc);
    c->apply(f, u);
  });
}

int te_bicgstab_solve(const te_operator* A, int nc, void* x, const void* b, const te_cycle* M, double tol,
                      int max_iterations, int flags, int* iterations, double* final_residual) {
  int status = TE_OK;
  int rc = guard([&] {
    require(A && x && b, "null argument");
    const te_domain* d = A->dom;
    cudaStream_t s = d->stream;
    size_t bytes = (size_t)d->lay.P * d->lay.pstride(nc) * sizeof(double);
    auto zero = [&]() {
      DevBuf<double> v(bytes / sizeof(double));
      TE_CUDA(cudaMemsetAsync(v.p, 0, bytes, s));
      return v;
    };
    Krylov K(d, nc);
    if (M) const_cast<te_cycle*>(M)->ensure(nc);
    DevBuf<double> resid = zero(), ms, mp;
    if (M) {
      ms = zero();
      mp = zero();
    }
    operator_apply(A, nc, TE_F64, x, resid.p, s);
    vec_dispatch(d, nc, TE_F64, OP_SCALE_THEN_ADD, resid.p, b, nullptr, -1, 0, 0);
    double r0 = std::sqrt(K.dot(b, b));
    DevBuf<double> rhat(bytes / 8), p(bytes / 8), ap = zero(), as = zero(), sv = zero();
    TE_CUDA(cudaMemcpyAsync(rhat.p, resid.p, bytes, cudaMemcpyDeviceToDevice, s));
    TE_CUDA(cudaMemcpyAsync(p.p, resid.p, bytes, cudaMemcpyDeviceToDevice, s));
    double rho = K.dot(rhat.p, resid.p);
    int its = 0;
    double residual = std::sqrt(K.dot(resid.p, resid.p)) / r0;
    if (final_residual) *final_residual = residual;
    if (r0 == 0) {
      *iterations = 0;
      return;
    }
    while (residual > tol && its < max_iterations) {
      if (rho == 0) {
        status = TE_ERR_BREAKDOWN;
        set_error("BiCGStab broke down, rho was 0 on iteration " + std::to_string(its));
        break;
      }
      if (M) {
        M->apply(p.p, mp.p);
        operator_apply(A, nc, TE_F64, mp.p, ap.p, s);
      } else {
        operator_apply(A, nc, TE_F64, p.p, ap.p, s);
      }
      double alpha = rho / K.dot(rhat.p, ap.p);
      vec_dispatch(d, nc, TE_F64, OP_COPY, sv.p, resid.p, nullptr, 0, 0, 0);
      vec_dispatch(d, nc, TE_F64, OP_ADD_SCALED, sv.p, ap.p, nullptr, -alpha, 0, 0);
      double snorm = std::sqrt(K.dot(sv.p, sv.p)) / r0;
      if (snorm <= tol) {
        // the reference adds alpha * p even when preconditioned (BiCGStab.h:163);
        // flag bit 0 selects the preconditioned update alpha * M p instead
        const void* dir = (M && (flags & 1)) ? (const void*)mp.p : (const void*)p.p;
        vec_dispatch(d, nc, TE_F64, OP_ADD_SCALED, x, dir, nullptr, alpha, 0, 0);
        if (final_residual) *final_residual = snorm;
        break;
      }
      if (M) {
        M->apply(sv.p, ms.p);
        operator_apply(A, nc, TE_F64, ms.p, as.p, s);
      } else {
        operator_apply(A, nc, TE_F64, sv.p, as.p, s);
      }
      const void* da[2] = {as.p, as.p};
      const void* db[2] = {sv.p, as.p};
      double w[2];
      K.dots(2, da, db, w);
      double omega = w[0] / w[1];
      if (M)
        vec_dispatch(d, nc, TE_F64, OP_ADD_SCALED2, x, mp.p, ms.p, alpha, omega, 0);
      else
        vec_dispatch(d, nc, TE_F64, OP_ADD_SCALED2, x, p.p, sv.p, alpha, omega, 0);
      vec_dispatch(d, nc, TE_F64, OP_ADD_SCALED2, resid.p, ap.p, as.p, -alpha, -omega, 0);
      const void* ra[2] = {resid.p, resid.p};
      const void* rb[2] = {rhat.p, resid.p};
      double rr[2];
      K.dots(2, ra, rb, rr);
      double rho_new = rr[0];
      double beta = rho_new * alpha / (rho * omega);
      vec_dispatch(d, nc, TE_F64, OP_ADD_SCALED, p.p, ap.p, nullptr, -omega, 0, 0);
      vec_dispatch(d, nc, TE_F64, OP_SCALE_THEN_ADD, p.p, resid.p, nullptr, beta, 0, 0);
      its++;
      rho = rho_new;
      residual = std::sqrt(rr[1]) / r0;
      if (final_residual) *final_residual = residual;
    }
    *iterations = its;
  });
  return rc != TE_OK ? rc : status;
}

}  // extern "C"
