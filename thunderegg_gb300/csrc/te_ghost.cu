// te_ghost.cu -- coarse-fine ghost filling on the GPU.
//
// ThunderEgg's MPIGhostFiller (MPIGhostFiller.h:821-1092) fills ghosts by
// scatter: zero every ghost face that has a neighbour, add each patch's own
// (local) terms, then let every patch write into its neighbours' ghosts
// ("fillGhostCellsFor*NbrPatch" calls, enumerated once in the constructor).
// Here the same call list is built on the host and transposed: each ghost
// slab knows the calls that target it, in the reference's order, and one
// thread per ghost cell gathers: v = 0; v = own terms; v = calls in order.
// No atomics, no cross-CTA writes; results are deterministic.
//
// The per-cell formulas are the gather form of
//   BiLinearGhostFiller.cpp:40-264,   BiQuadraticGhostFiller.cpp:34-334,
//   TriLinearGhostFiller.cpp:28-370.

#include <algorithm>
#include <array>
#include <cstring>

#include "te_ghost_dev.cuh"

namespace te {

int slot_of(int D, int M, int face) { return sum_of_faces(D, M) + face; }
int face_opposite(int D, int M, int v) { return v ^ ((1 << (D - M)) - 1); }

// Face::getSides (Face.h:497-526)
static void face_sides(int D, int M, int v, int* axis, int* upper) {
  if (M == D - 1) {
    axis[0] = v >> 1;
    upper[0] = v & 1;
  } else if (M == 0) {
    for (int i = 0; i < D; i++) {
      axis[i] = i;
      upper[i] = (v >> i) & 1;
    }
  } else {
    int not_axis = v >> 2, k = 0;
    for (int i = 0; i < 3; i++)
      if (i != not_axis) {
        axis[k] = i;
        upper[k] = (v >> k) & 1;
        k++;
      }
  }
}

FaceTable make_face_table(const Layout& L) {
  FaceTable t;
  std::memset(&t, 0, sizeof t);
  int D = L.D;
  for (int M = 0; M < D; M++)
    for (int f = 0; f < num_faces(D, M); f++) {
      FaceGeom& g = t.f[slot_of(D, M, f)];
      int ax[3], up[3];
      face_sides(D, M, f, ax, up);
      int ic[3] = {0, 0, 0}, gc[3] = {0, 0, 0};
      bool on[3] = {false, false, false};
      for (int i = 0; i < D - M; i++) {
        int a = ax[i];
        on[a] = true;
        ic[a] = up[i] ? L.n(a) - 1 : 0;
        gc[a] = up[i] ? L.n(a) : -1;
        g.inward[i] = up[i] ? -L.stride(a) : L.stride(a);
      }
      g.nsides = D - M;
      int k = 0;
      g.nt[0] = g.nt[1] = 1;
      g.tstride[0] = g.tstride[1] = 0;
      for (int a = 0; a < D; a++)
        if (!on[a]) {
          g.tstride[k] = L.stride(a);
          g.nt[k] = L.n(a);
          k++;
        }
      g.ibase = L.at(ic[0], ic[1], ic[2]);
      g.gbase = L.at(gc[0], gc[1], gc[2]);
    }
  return t;
}

constexpr int GHOST_THREADS = 128;

template <class T, int SCHEME>
__global__ void __launch_bounds__(GHOST_THREADS)
    ghost_fill_kernel(Layout L, int nc, FaceTable ft, const GSlab* __restrict__ slabs,
                      const GCall* __restrict__ calls, const int* __restrict__ slab_start, T* u) {
  int p = blockIdx.x;
  long long ps = L.pstride(nc);
  int s0 = slab_start[p], s1 = slab_start[p + 1];
  int D = L.D;
  for (int s = s0; s < s1; s++) {
    GSlab sl = slabs[s];
    const FaceGeom& g = ft.f[sl.M == D - 1 ? (D == 2 ? 4 : 20) + sl.face : (sl.M == 0 ? sl.face : 8 + sl.face)];
    int ni = g.nt[0], nj = g.nt[1];
    int per_c = ni * nj;
    int cnt = per_c * nc;
    // deeper ghost layers of faces with a neighbour are zeroed (zeroGhostCellsOnAllFaces)
    if (sl.zero && L.g > 1) {
      int layers = 1;
      for (int k = 0; k < g.nsides; k++) layers *= L.g;
      for (int e = threadIdx.x; e < cnt * layers; e += blockDim.x) {
        int lay = e / cnt, r = e % cnt;
        if (lay == 0) continue;
        int c = r / per_c, t = r % per_c, i = t % ni, j = t / ni;
        int idx = g.gbase + i * g.tstride[0] + j * g.tstride[1];
        int rem = lay;
        for (int k = 0; k < g.nsides; k++) {
          idx -= (rem % L.g) * g.inward[k];
          rem /= L.g;
        }
        u[p * ps + (long long)c * L.cs + idx] = T(0);
      }
    }
    for (int e = threadIdx.x; e < cnt; e += blockDim.x) {
      int c = e / per_c, t = e % per_c, i = t % ni, j = t / ni;
      T* gp = u + p * ps + (long long)c * L.cs + g.gbase + i * g.tstride[0] + j * g.tstride[1];
      PlainAcc<T> acc{u, ps, (long long)c * L.cs};
      *gp = gather_ghost<T, SCHEME>(acc, p, sl, g, ft, calls, D, i, j, sl.zero ? T(0) : *gp);
    }
  }
}

// ghost_fill_kernel for one ghost layer with the work of a patch spread over
// the whole CTA: every thread takes whole ghost values of any side of NP
// patches (the sides in side_code), then the remaining slabs (edges,
// corners) follow slab by slab when `other` is set.  Slabs write disjoint
// ghost cells and read only interior cells, so they need no order.
template <class T, int SCHEME>
__global__ void __launch_bounds__(GHOST_THREADS, 12)
    ghost_fill_sides_kernel(Layout L, int nc, FaceTable ft, const GSlab* __restrict__ slabs,
                            const GCall* __restrict__ calls, const int* __restrict__ slab_start,
                            const int* __restrict__ side_code, int NP, int gmax, int other, T* u) {
  const int D = L.D;
  const int side0 = D == 2 ? 4 : 20;
  const int p0 = blockIdx.x * NP;
  const long long ps = L.pstride(nc);
  const int per_side = nc * gmax, per_patch = 2 * D * per_side;
  for (int e = threadIdx.x; e < NP * per_patch; e += blockDim.x) {
    const int q = e / per_patch, rem = e - q * per_patch, sd = rem / per_side, r2 = rem - sd * per_side;
    const int c = r2 / gmax, r = r2 - c * gmax;
    const int p = p0 + q;
    if (p >= L.P) break;
    const FaceGeom& g = ft.f[side0 + sd];
    if (r >= g.nt[0] * g.nt[1]) continue;
    const int code = side_code[p * 2 * D + sd];
    if (code == -1) continue;
    const int i = r % g.nt[0], j = r / g.nt[0];
    PlainAcc<T> acc{u, ps, (long long)c * L.cs};
    u[p * ps + (long long)c * L.cs + g.gbase + i * g.tstride[0] + j * g.tstride[1]] =
        side_ghost<T, SCHEME>(acc, p, sd, code, slabs, calls, ft, D, i, j);
  }
  if (!other) return;
  for (int q = 0; q < NP; q++) {
    const int p = p0 + q;
    if (p >= L.P) return;
    for (int s = slab_start[p]; s < slab_start[p + 1]; s++) {
      const GSlab sl = slabs[s];
      if (sl.M == D - 1 && sl.zero) continue;  // filled above
      const FaceGeom& g = ft.f[sl.M == D - 1 ? side0 + sl.face : (sl.M == 0 ? sl.face : 8 + sl.face)];
      const int ni = g.nt[0], per_c = ni * g.nt[1];
      for (int e = threadIdx.x; e < per_c * nc; e += blockDim.x) {
        const int c = e / per_c, t = e - c * per_c, i = t % ni, j = t / ni;
        T* gp = u + p * ps + (long long)c * L.cs + g.gbase + i * g.tstride[0] + j * g.tstride[1];
        PlainAcc<T> acc{u, ps, (long long)c * L.cs};
        *gp = gather_ghost<T, SCHEME>(acc, p, sl, g, ft, calls, D, i, j, sl.zero ? T(0) : *gp);
      }
    }
  }
}

template <class T, int SCHEME>
static void launch_fill_sides(const te_ghost_filler* gf, int nc, T* u, cudaStream_t s) {
  const Layout& L = gf->dom->lay;
  int gmax = 1;
  for (int a = 0; a < L.D; a++) gmax = std::max(gmax, L.interior() / L.n(a));
  const int per_patch = 2 * L.D * nc * gmax;
  const int NP = std::max(1, GHOST_THREADS / per_patch);
  ghost_fill_sides_kernel<T, SCHEME><<<(L.P + NP - 1) / NP, GHOST_THREADS, 0, s>>>(
      L, nc, gf->faces, gf->d_slabs.p, gf->d_calls.p, gf->d_slab_start.p, gf->d_side_code.p, NP, gmax,
      gf->other_slabs ? 1 : 0, u);
}

template <class T>
static void launch_fill(const te_ghost_filler* gf, int nc, T* u, cudaStream_t s) {
  const Layout& L = gf->dom->lay;
  if (L.g == 1 && !generic_level_kernels()) {
    switch (gf->scheme) {
      case TE_GHOST_BILINEAR: launch_fill_sides<T, TE_GHOST_BILINEAR>(gf, nc, u, s); break;
      case TE_GHOST_BIQUADRATIC: launch_fill_sides<T, TE_GHOST_BIQUADRATIC>(gf, nc, u, s); break;
      default: launch_fill_sides<T, TE_GHOST_TRILINEAR>(gf, nc, u, s);
    }
    count_launch();
    TE_LAUNCH_CHECK();
    return;
  }
  dim3 grid(L.P), block(GHOST_THREADS);
  switch (gf->scheme) {
    case TE_GHOST_BILINEAR:
      ghost_fill_kernel<T, TE_GHOST_BILINEAR><<<grid, block, 0, s>>>(L, nc, gf->faces, gf->d_slabs.p,
                                                                     gf->d_calls.p, gf->d_slab_start.p, u);
      break;
    case TE_GHOST_BIQUADRATIC:
      ghost_fill_kernel<T, TE_GHOST_BIQUADRATIC><<<grid, block, 0, s>>>(L, nc, gf->faces, gf->d_slabs.p,
                                                                        gf->d_calls.p, gf->d_slab_start.p, u);
      break;
    default:
      ghost_fill_kernel<T, TE_GHOST_TRILINEAR><<<grid, block, 0, s>>>(L, nc, gf->faces, gf->d_slabs.p,
                                                                      gf->d_calls.p, gf->d_slab_start.p, u);
  }
  count_launch();
  TE_LAUNCH_CHECK();
}

void ghost_fill(const te_ghost_filler* g, int nc, int dtype, void* u, cudaStream_t s) {
  require(g && u, "null argument");
  if (g->h_slabs.empty()) return;
  if (dtype == TE_F64)
    launch_fill<double>(g, nc, (double*)u, s);
  else
    launch_fill<float>(g, nc, (float*)u, s);
}

}  // namespace te

using namespace te;

extern "C" {

int te_ghost_filler_create(const te_domain* d, int scheme, int fill_type, te_ghost_filler** out) {
  return guard([&] {
    require(d && out, "null argument");
    int D = d->lay.D;
    require(fill_type >= TE_FILL_FACES && fill_type <= TE_FILL_CORNERS, "bad fill type");
    if (D == 2)
      require(scheme == TE_GHOST_BILINEAR || scheme == TE_GHOST_BIQUADRATIC, "2D needs BiLinear or BiQuadratic");
    else
      require(scheme == TE_GHOST_TRILINEAR, "3D needs TriLinear");
    const Layout& L = d->lay;
    if (scheme == TE_GHOST_TRILINEAR)  // TriLinearGhostFiller.cpp:576-584
      require(L.n0 % 2 == 0 && L.n1 % 2 == 0 && L.n2 % 2 == 0,
              "TriLinearGhostFiller only supports even number patch sizes", TE_ERR_UNSUPPORTED);
    if (scheme == TE_GHOST_BIQUADRATIC) require(L.n0 >= 3 && L.n1 >= 3, "BiQuadratic needs n >= 3");
    auto g = std::make_unique<te_ghost_filler>();
    g->dom = d;
    g->scheme = scheme;
    g->fill_type = fill_type;
    g->faces = make_face_table(L);
    int F = d->F, P = L.P;
    // dimensionalities filled, in processLocalFills order (MPIGhostFiller.h:705-717, 956-985)
    std::vector<int> ms = {D - 1};
    if (D == 3 && fill_type >= TE_FILL_EDGES) ms.push_back(1);
    if (fill_type == TE_FILL_CORNERS) ms.push_back(0);
    // MPIGhostFiller::enumerateCalls (:779-836)
    for (int M : ms)
      for (int p = 0; p < P; p++)
        for (int f = 0; f < num_faces(D, M); f++) {
          int slot = slot_of(D, M, f);
          int t = d->nbr_type[(size_t)p * F + slot];
          if (t < 0) continue;
          const int* loc = &d->nbr_local[((size_t)p * F + slot) * 4];
          if (t == TE_NBR_NORMAL)
            g->calls.push_back({p, loc[0], M, f, t, -1});
          else if (t == TE_NBR_FINE)
            for (int i = 0; i < (1 << M); i++) g->calls.push_back({p, loc[i], M, f, t, i});
          else
            g->calls.push_back({p, loc[0], M, f, t, d->nbr_orth[(size_t)p * F + slot]});
        }
    // odd n with BiLinear coarse neighbours writes into corner ghosts
    // (BiLinearGhostFiller.cpp:118-134); that spill is not reproduced here.
    if (scheme == TE_GHOST_BILINEAR && (L.n0 % 2 || L.n1 % 2))
      for (auto& c : g->calls)
        require(c[4] == TE_NBR_NORMAL, "BiLinear with odd patch size across a coarse-fine face",
                TE_ERR_UNSUPPORTED);
    // transpose: incoming calls per (patch, slot), kept in call order (CSR: in_start, in_call)
    std::vector<int> in_start((size_t)P * F + 1, 0), in_slot(g->calls.size());
    for (size_t k = 0; k < g->calls.size(); k++) {
      auto& c = g->calls[k];
      int tgt = c[1], M = c[2], opp = face_opposite(D, M, c[3]);
      in_slot[k] = (int)((size_t)tgt * F + slot_of(D, M, opp));
      in_start[(size_t)in_slot[k] + 1]++;
    }
    for (size_t q = 0; q < (size_t)P * F; q++) in_start[q + 1] += in_start[q];
    std::vector<int> in_call(g->calls.size()), fill_pos(in_start.begin(), in_start.end() - 1);
    for (size_t k = 0; k < g->calls.size(); k++) in_call[(size_t)fill_pos[(size_t)in_slot[k]]++] = (int)k;
    struct Incoming {
      const int* b;
      const int* e;
      bool empty() const { return b == e; }
      size_t size() const { return (size_t)(e - b); }
      const int* begin() const { return b; }
      const int* end() const { return e; }
    };
    auto incoming_of = [&](size_t q) { return Incoming{in_call.data() + in_start[q], in_call.data() + in_start[q + 1]}; };
    std::vector<GCall> hc;
    g->h_slab_start.assign(P + 1, 0);
    for (int p = 0; p < P; p++) {
      g->h_slab_start[p] = (int)g->h_slabs.size();
      for (int M : ms)
        for (int f = 0; f < num_faces(D, M); f++) {
          int slot = slot_of(D, M, f);
          int t = d->nbr_type[(size_t)p * F + slot];
          const Incoming inc = incoming_of((size_t)p * F + slot);
          if (t < 0 && inc.empty()) continue;
          GSlab s;
          std::memset(&s, 0, sizeof s);
          s.patch = p;
          s.M = (int8_t)M;
          s.face = (int8_t)f;
          s.own_type = (int8_t)t;
          s.own_orth = (int8_t)(t == TE_NBR_COARSE ? d->nbr_orth[(size_t)p * F + slot] : -1);
          s.zero = t >= 0;
          require(inc.size() < 127, "too many calls into one ghost face");
          s.ncalls = (int8_t)inc.size();
          s.call0 = (int)hc.size();
          for (int k : inc) {
            auto& c = g->calls[k];
            GCall gc;
            gc.src = c[0];
            gc.type = (int8_t)c[4];
            gc.orth = (int8_t)c[5];
            gc.src_face = (int8_t)c[3];
            gc.pad = 0;
            hc.push_back(gc);
          }
          g->h_slabs.push_back(s);
        }
    }
    g->h_slab_start[P] = (int)g->h_slabs.size();
    std::vector<int> side_code((size_t)P * 2 * D, -1);
    for (size_t k = 0; k < g->h_slabs.size(); k++) {
      const GSlab& s = g->h_slabs[k];
      if (!(s.M == D - 1 && s.zero)) {
        g->other_slabs = true;
        continue;
      }
      int code = -2 - (int)k;
      if (s.own_type == TE_NBR_NORMAL && s.ncalls == 1) {
        const GCall& c = hc[s.call0];
        if (c.type == TE_NBR_NORMAL && c.src_face == (s.face ^ 1)) code = c.src;
      }
      side_code[(size_t)s.patch * 2 * D + s.face] = code;
    }
    std::vector<SideRec> side_rec((size_t)P * 2 * D);
    for (size_t k = 0; k < side_rec.size(); k++) {
      SideRec r;
      std::memset(&r, 0, sizeof r);
      r.code = side_code[k];
      r.own_type = -1;
      r.own_orth = -1;
      if (r.code <= -2) {
        const GSlab& s = g->h_slabs[(size_t)(-2 - r.code)];
        r.own_type = s.own_type;
        r.own_orth = s.own_orth;
        r.zero = s.zero;
        if (s.ncalls <= kSideRecCalls) {
          r.ncalls = s.ncalls;
          for (int c = 0; c < s.ncalls; c++) r.calls[c] = hc[(size_t)s.call0 + c];
        } else {
          r.ncalls = -1;
        }
      }
      side_rec[k] = r;
    }
    cudaStream_t st = d->stream;
    g->d_side_code.upload(side_code, st);
    g->d_side_rec.upload(side_rec, st);
    g->d_slabs.upload(g->h_slabs, st);
    g->d_calls.upload(hc, st);
    g->d_slab_start.upload(g->h_slab_start, st);
    TE_CUDA(cudaStreamSynchronize(st));
    *out = g.release();
  });
}

int te_ghost_filler_destroy(te_ghost_filler* g) {
  delete g;
  return TE_OK;
}

int te_ghost_fill(const te_ghost_filler* g, int nc, int dtype, void* u) {
  return guard([&] {
    require(g != nullptr, "null filler");
    ghost_fill(g, nc, dtype, u, g->dom->stream);
  });
}

int te_ghost_filler_num_calls(const te_ghost_filler* g) { return g ? (int)g->calls.size() : -1; }

int te_ghost_filler_calls(const te_ghost_filler* g, int* rows6) {
  return guard([&] {
    require(g && rows6, "null argument");
    for (size_t k = 0; k < g->calls.size(); k++) std::memcpy(rows6 + 6 * k, g->calls[k].data(), 6 * sizeof(int));
  });
}

}  // extern "C"
