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

#include <array>
#include <cstring>

#include "te_ghost.cuh"

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

// ---------------------------------------------------------------------------
// device: gather formulas
// ---------------------------------------------------------------------------
template <class T>
struct K {
  static constexpr T third = T(1.0 / 3.0);
  static constexpr T two3 = T(2.0 / 3.0);
  static constexpr T four3 = T(4.0 / 3.0);
};

// value of the interior slice (depth `dep` along every side of the face) of a patch
template <class T>
__device__ __forceinline__ T sv(const T* p, const FaceGeom& g, int dep, int i, int j) {
  int idx = g.ibase + i * g.tstride[0] + j * g.tstride[1];
  for (int k = 0; k < g.nsides; k++) idx += dep * g.inward[k];
  return p[idx];
}

// ---- BiLinear / TriLinear edges: own Coarse term on a 1-D ghost line
// (BiLinearGhostFiller.cpp:118-134, TriLinearGhostFiller.cpp:172-195)
template <class T>
__device__ __forceinline__ T lin_own_coarse_1d(T v, const T* p, const FaceGeom& g, int j, int n, int off) {
  if (j - 1 >= 0 && ((j - 1 + off) % 2 == 0)) v += -K<T>::third * sv(p, g, 0, j - 1, 0);
  v += K<T>::two3 * sv(p, g, 0, j, 0);
  if (j + 1 < n && ((j + 1 + off) % 2 != 0)) v += -K<T>::third * sv(p, g, 0, j + 1, 0);
  return v;
}

template <class T, int SCHEME>
__device__ T own_term(T v, const T* p, const FaceGeom& g, int M, int D, int type, int orth, int i, int j) {
  if (type == TE_NBR_NORMAL || type < 0) return v;
  const T third = K<T>::third;
  if (M == 0) {  // corners
    if (SCHEME == TE_GHOST_BIQUADRATIC) {
      // BiQuadraticGhostFiller.cpp:176-204
      if (type == TE_NBR_COARSE) return v + (T(2) * sv(p, g, 0, 0, 0) * third - sv(p, g, 1, 0, 0) * T(0.2));
      return v + (-sv(p, g, 0, 0, 0) * T(1.0 / 15.0));
    }
    // BiLinear :207-264, TriLinear :349-364
    if (type == TE_NBR_COARSE) return v + sv(p, g, 0, 0, 0) * third;
    return v + (-sv(p, g, 0, 0, 0) * third);
  }
  if (M == 1 && D == 3) {  // TriLinear edges
    int n = g.nt[0];
    if (type == TE_NBR_COARSE) return lin_own_coarse_1d(v, p, g, i, n, orth == 1 ? n : 0);
    return v + (-third * sv(p, g, 0, i, 0));
  }
  if (D == 2) {  // sides, 2D
    int n = g.nt[0];
    if (SCHEME == TE_GHOST_BILINEAR) {
      if (type == TE_NBR_COARSE) return lin_own_coarse_1d(v, p, g, i, n, orth == 1 ? n : 0);
      return v + (-third * sv(p, g, 0, i, 0));
    }
    // BiQuadratic: FillGhostForLocalWithCoarseNbr / WithFineNbr (:34-58)
    if (type == TE_NBR_COARSE) return v + (T(2) * sv(p, g, 0, i, 0) * third - sv(p, g, 1, i, 0) * T(0.2));
    const T c10 = T(0.1), c15 = T(1.0 / 15.0), c30 = T(1.0 / 30.0);
    if (i == 0) return v + (-sv(p, g, 0, 0, 0) * c10 + sv(p, g, 0, 1, 0) * c15 - sv(p, g, 0, 2, 0) * c30);
    if (i == n - 1)
      return v + (-sv(p, g, 0, n - 1, 0) * c10 + sv(p, g, 0, n - 2, 0) * c15 - sv(p, g, 0, n - 3, 0) * c30);
    return v + (-sv(p, g, 0, i - 1, 0) * c30 - sv(p, g, 0, i + 1, 0) * c30);
  }
  // TriLinear sides (:100-122, :74-82)
  if (type == TE_NBR_COARSE) {
    int si = (orth & 1) ? g.nt[0] : 0, sj = (orth & 2) ? g.nt[1] : 0;
    int oi = (i + si) % 2 == 0 ? i + 1 : i - 1;
    int oj = (j + sj) % 2 == 0 ? j + 1 : j - 1;
    const T sixth = T(1.0 / 6.0);
    v += T(5.0 / 6.0) * sv(p, g, 0, i, j);
    v -= sixth * sv(p, g, 0, oi, j);
    v -= sixth * sv(p, g, 0, i, oj);
    v -= sixth * sv(p, g, 0, oi, oj);
    return v;
  }
  return v - third * sv(p, g, 0, i, j);
}

// contribution of one incoming call (caller patch q, caller face geometry gq)
template <class T, int SCHEME>
__device__ T call_term(T v, const T* q, const FaceGeom& gq, int M, int D, int type, int orth, int i, int j) {
  if (type == TE_NBR_NORMAL) return sv(q, gq, 0, i, j);  // plain copy, an assignment
  const T third = K<T>::third;
  if (M == 0) {
    if (SCHEME == TE_GHOST_BIQUADRATIC) {  // :150-175
      if (type == TE_NBR_COARSE)
        return v + (T(2) * sv(q, gq, 0, 0, 0) * third + T(2) * sv(q, gq, 1, 0, 0) * T(0.2));
      return v + T(8) * sv(q, gq, 0, 0, 0) * T(1.0 / 15.0);
    }
    if (type == TE_NBR_COARSE) return v + T(4) * sv(q, gq, 0, 0, 0) * third;
    return v + T(2) * sv(q, gq, 0, 0, 0) * third;
  }
  if (M == 1) {  // 2D sides (BiLinear/BiQuadratic) or 3D edges (TriLinear)
    int n = gq.nt[0];
    int off = orth == 1 ? n : 0;
    if (SCHEME == TE_GHOST_BIQUADRATIC && D == 2) {
      if (type == TE_NBR_COARSE) {  // caller finer: CoarseNbrLower/Upper (:81-105)
        for (int idx = 2 * i - off; idx <= 2 * i + 1 - off; idx++)
          if (idx >= 0 && idx < n) v += sv(q, gq, 0, idx, 0) * third + sv(q, gq, 1, idx, 0) * T(0.2);
        return v;
      }
      // caller coarser: FineNbrLower/Upper (:106-148)
      const T c12 = T(1.0 / 12.0), c20 = T(0.05), c30 = T(1.0 / 30.0);
      if (orth == 0) {
        if (i == 0)
          return v + (T(0.75) * sv(q, gq, 0, 0, 0) - T(0.3) * sv(q, gq, 0, 1, 0) + sv(q, gq, 0, 2, 0) * c12);
        if (i == 1)
          return v + (T(0.35) * sv(q, gq, 0, 0, 0) + T(7) * sv(q, gq, 0, 1, 0) * c30 - sv(q, gq, 0, 2, 0) * c20);
        int k = i / 2;
        if (i % 2 == 0)
          return v + (sv(q, gq, 0, k - 1, 0) * c12 + sv(q, gq, 0, k, 0) * T(0.5) - sv(q, gq, 0, k + 1, 0) * c20);
        return v + (-sv(q, gq, 0, k - 1, 0) * c20 + sv(q, gq, 0, k, 0) * T(0.5) + sv(q, gq, 0, k + 1, 0) * c12);
      }
      if (i < n - 2) {
        int k = (i + n) / 2;
        if ((i + n) % 2 == 0)
          return v + (sv(q, gq, 0, k - 1, 0) * c12 + sv(q, gq, 0, k, 0) * T(0.5) - sv(q, gq, 0, k + 1, 0) * c20);
        return v + (-sv(q, gq, 0, k - 1, 0) * c20 + sv(q, gq, 0, k, 0) * T(0.5) + sv(q, gq, 0, k + 1, 0) * c12);
      }
      if (i == n - 2)
        return v + (T(0.35) * sv(q, gq, 0, n - 1, 0) + T(7) * sv(q, gq, 0, n - 2, 0) * c30 -
                    sv(q, gq, 0, n - 3, 0) * c20);
      return v + (T(0.75) * sv(q, gq, 0, n - 1, 0) - T(0.3) * sv(q, gq, 0, n - 2, 0) + sv(q, gq, 0, n - 3, 0) * c12);
    }
    // BiLinear sides (:61-105) and TriLinear edges (:140-171)
    if (type == TE_NBR_COARSE) {
      for (int idx = 2 * i - off; idx <= 2 * i + 1 - off; idx++)
        if (idx >= 0 && idx < n) v += K<T>::two3 * sv(q, gq, 0, idx, 0);
      return v;
    }
    return v + K<T>::two3 * sv(q, gq, 0, (i + off) / 2, 0);
  }
  // TriLinear sides (:58-99); offsets from getOffset (:28-44)
  int oi = (orth & 1) ? gq.nt[0] : 0, oj = (orth & 2) ? gq.nt[1] : 0;
  if (type == TE_NBR_COARSE) {
    for (int jj = 2 * j - oj; jj <= 2 * j + 1 - oj; jj++)
      for (int ii = 2 * i - oi; ii <= 2 * i + 1 - oi; ii++)
        if (ii >= 0 && ii < gq.nt[0] && jj >= 0 && jj < gq.nt[1]) v += third * sv(q, gq, 0, ii, jj);
    return v;
  }
  return v + K<T>::two3 * sv(q, gq, 0, (i + oi) / 2, (j + oj) / 2);
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
      const T* pu = u + p * ps + (long long)c * L.cs;
      T* gp = u + p * ps + (long long)c * L.cs + g.gbase + i * g.tstride[0] + j * g.tstride[1];
      T v = sl.zero ? T(0) : *gp;
      v = own_term<T, SCHEME>(v, pu, g, sl.M, D, sl.own_type, sl.own_orth, i, j);
      for (int k = 0; k < sl.ncalls; k++) {
        GCall cl = calls[sl.call0 + k];
        const FaceGeom& gq =
            ft.f[sl.M == D - 1 ? (D == 2 ? 4 : 20) + cl.src_face : (sl.M == 0 ? cl.src_face : 8 + cl.src_face)];
        const T* q = u + cl.src * ps + (long long)c * L.cs;
        v = call_term<T, SCHEME>(v, q, gq, sl.M, D, cl.type, cl.orth, i, j);
      }
      *gp = v;
    }
  }
}

template <class T>
static void launch_fill(const te_ghost_filler* gf, int nc, T* u, cudaStream_t s) {
  const Layout& L = gf->dom->lay;
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
    // transpose: incoming calls per (patch, slot), kept in call order
    std::vector<std::vector<int>> incoming((size_t)P * F);
    for (size_t k = 0; k < g->calls.size(); k++) {
      auto& c = g->calls[k];
      int tgt = c[1], M = c[2], opp = face_opposite(D, M, c[3]);
      incoming[(size_t)tgt * F + slot_of(D, M, opp)].push_back((int)k);
    }
    std::vector<GCall> hc;
    g->h_slab_start.assign(P + 1, 0);
    for (int p = 0; p < P; p++) {
      g->h_slab_start[p] = (int)g->h_slabs.size();
      for (int M : ms)
        for (int f = 0; f < num_faces(D, M); f++) {
          int slot = slot_of(D, M, f);
          int t = d->nbr_type[(size_t)p * F + slot];
          auto& inc = incoming[(size_t)p * F + slot];
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
    cudaStream_t st = d->stream;
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
