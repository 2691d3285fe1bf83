// te_ghost_dev.cuh -- device-side gather formulas of the three ghost schemes.
// Included by the ghost-fill kernel and by fused kernels that gather ghosts
// on the fly.
#pragma once
#include "te_ghost.cuh"

namespace te {

// ---------------------------------------------------------------------------
// device: gather formulas
// ---------------------------------------------------------------------------
template <class T>
struct K {
  static constexpr T third = T(1.0 / 3.0);
  static constexpr T two3 = T(2.0 / 3.0);
  static constexpr T four3 = T(4.0 / 3.0);
};

// Accessors return the value of cell `idx` (index within one padded
// component) of patch q.  PlainAcc reads a level buffer; other accessors
// (e.g. "u + interpolated coarse correction") let fused kernels gather
// ghosts of values that are never stored.
template <class T>
struct PlainAcc {
  const T* u;
  long long ps;  // patch stride
  long long co;  // component offset
  __device__ __forceinline__ T operator()(int q, int idx) const { return u[q * ps + co + idx]; }
};

// value of the interior slice (depth `dep` along every side of the face) of patch q
template <class T, class Acc>
__device__ __forceinline__ T sv(const Acc& acc, int q, const FaceGeom& g, int dep, int i, int j) {
  int idx = g.ibase + i * g.tstride[0] + j * g.tstride[1];
  for (int k = 0; k < g.nsides; k++) idx += dep * g.inward[k];
  return acc(q, idx);
}

// ---- BiLinear / TriLinear edges: own Coarse term on a 1-D ghost line
// (BiLinearGhostFiller.cpp:118-134, TriLinearGhostFiller.cpp:172-195)
template <class T, class Acc>
__device__ __forceinline__ T lin_own_coarse_1d(T v, const Acc& p, int pq, const FaceGeom& g, int j, int n, int off) {
  if (j - 1 >= 0 && ((j - 1 + off) % 2 == 0)) v += -K<T>::third * sv<T>(p, pq, g, 0, j - 1, 0);
  v += K<T>::two3 * sv<T>(p, pq, g, 0, j, 0);
  if (j + 1 < n && ((j + 1 + off) % 2 != 0)) v += -K<T>::third * sv<T>(p, pq, g, 0, j + 1, 0);
  return v;
}

template <class T, int SCHEME, class Acc>
__device__ T own_term(T v, const Acc& p, int pq, const FaceGeom& g, int M, int D, int type, int orth, int i, int j) {
  if (type == TE_NBR_NORMAL || type < 0) return v;
  const T third = K<T>::third;
  if (M == 0) {  // corners
    if (SCHEME == TE_GHOST_BIQUADRATIC) {
      // BiQuadraticGhostFiller.cpp:176-204
      if (type == TE_NBR_COARSE) return v + (T(2) * sv<T>(p, pq, g, 0, 0, 0) * third - sv<T>(p, pq, g, 1, 0, 0) * T(0.2));
      return v + (-sv<T>(p, pq, g, 0, 0, 0) * T(1.0 / 15.0));
    }
    // BiLinear :207-264, TriLinear :349-364
    if (type == TE_NBR_COARSE) return v + sv<T>(p, pq, g, 0, 0, 0) * third;
    return v + (-sv<T>(p, pq, g, 0, 0, 0) * third);
  }
  if (M == 1 && D == 3) {  // TriLinear edges
    int n = g.nt[0];
    if (type == TE_NBR_COARSE) return lin_own_coarse_1d<T>(v, p, pq, g, i, n, orth == 1 ? n : 0);
    return v + (-third * sv<T>(p, pq, g, 0, i, 0));
  }
  if (D == 2) {  // sides, 2D
    int n = g.nt[0];
    if (SCHEME == TE_GHOST_BILINEAR) {
      if (type == TE_NBR_COARSE) return lin_own_coarse_1d<T>(v, p, pq, g, i, n, orth == 1 ? n : 0);
      return v + (-third * sv<T>(p, pq, g, 0, i, 0));
    }
    // BiQuadratic: FillGhostForLocalWithCoarseNbr / WithFineNbr (:34-58)
    if (type == TE_NBR_COARSE) return v + (T(2) * sv<T>(p, pq, g, 0, i, 0) * third - sv<T>(p, pq, g, 1, i, 0) * T(0.2));
    const T c10 = T(0.1), c15 = T(1.0 / 15.0), c30 = T(1.0 / 30.0);
    if (i == 0) return v + (-sv<T>(p, pq, g, 0, 0, 0) * c10 + sv<T>(p, pq, g, 0, 1, 0) * c15 - sv<T>(p, pq, g, 0, 2, 0) * c30);
    if (i == n - 1)
      return v + (-sv<T>(p, pq, g, 0, n - 1, 0) * c10 + sv<T>(p, pq, g, 0, n - 2, 0) * c15 - sv<T>(p, pq, g, 0, n - 3, 0) * c30);
    return v + (-sv<T>(p, pq, g, 0, i - 1, 0) * c30 - sv<T>(p, pq, g, 0, i + 1, 0) * c30);
  }
  // TriLinear sides (:100-122, :74-82)
  if (type == TE_NBR_COARSE) {
    int si = (orth & 1) ? g.nt[0] : 0, sj = (orth & 2) ? g.nt[1] : 0;
    int oi = (i + si) % 2 == 0 ? i + 1 : i - 1;
    int oj = (j + sj) % 2 == 0 ? j + 1 : j - 1;
    const T sixth = T(1.0 / 6.0);
    v += T(5.0 / 6.0) * sv<T>(p, pq, g, 0, i, j);
    v -= sixth * sv<T>(p, pq, g, 0, oi, j);
    v -= sixth * sv<T>(p, pq, g, 0, i, oj);
    v -= sixth * sv<T>(p, pq, g, 0, oi, oj);
    return v;
  }
  return v - third * sv<T>(p, pq, g, 0, i, j);
}

// contribution of one incoming call (caller patch q, caller face geometry gq)
template <class T, int SCHEME, class Acc>
__device__ T call_term(T v, const Acc& q, int qq, const FaceGeom& gq, int M, int D, int type, int orth, int i, int j) {
  if (type == TE_NBR_NORMAL) return sv<T>(q, qq, gq, 0, i, j);  // plain copy, an assignment
  const T third = K<T>::third;
  if (M == 0) {
    if (SCHEME == TE_GHOST_BIQUADRATIC) {  // :150-175
      if (type == TE_NBR_COARSE)
        return v + (T(2) * sv<T>(q, qq, gq, 0, 0, 0) * third + T(2) * sv<T>(q, qq, gq, 1, 0, 0) * T(0.2));
      return v + T(8) * sv<T>(q, qq, gq, 0, 0, 0) * T(1.0 / 15.0);
    }
    if (type == TE_NBR_COARSE) return v + T(4) * sv<T>(q, qq, gq, 0, 0, 0) * third;
    return v + T(2) * sv<T>(q, qq, gq, 0, 0, 0) * third;
  }
  if (M == 1) {  // 2D sides (BiLinear/BiQuadratic) or 3D edges (TriLinear)
    int n = gq.nt[0];
    int off = orth == 1 ? n : 0;
    if (SCHEME == TE_GHOST_BIQUADRATIC && D == 2) {
      if (type == TE_NBR_COARSE) {  // caller finer: CoarseNbrLower/Upper (:81-105)
        for (int idx = 2 * i - off; idx <= 2 * i + 1 - off; idx++)
          if (idx >= 0 && idx < n) v += sv<T>(q, qq, gq, 0, idx, 0) * third + sv<T>(q, qq, gq, 1, idx, 0) * T(0.2);
        return v;
      }
      // caller coarser: FineNbrLower/Upper (:106-148)
      const T c12 = T(1.0 / 12.0), c20 = T(0.05), c30 = T(1.0 / 30.0);
      if (orth == 0) {
        if (i == 0)
          return v + (T(0.75) * sv<T>(q, qq, gq, 0, 0, 0) - T(0.3) * sv<T>(q, qq, gq, 0, 1, 0) + sv<T>(q, qq, gq, 0, 2, 0) * c12);
        if (i == 1)
          return v + (T(0.35) * sv<T>(q, qq, gq, 0, 0, 0) + T(7) * sv<T>(q, qq, gq, 0, 1, 0) * c30 - sv<T>(q, qq, gq, 0, 2, 0) * c20);
        int k = i / 2;
        if (i % 2 == 0)
          return v + (sv<T>(q, qq, gq, 0, k - 1, 0) * c12 + sv<T>(q, qq, gq, 0, k, 0) * T(0.5) - sv<T>(q, qq, gq, 0, k + 1, 0) * c20);
        return v + (-sv<T>(q, qq, gq, 0, k - 1, 0) * c20 + sv<T>(q, qq, gq, 0, k, 0) * T(0.5) + sv<T>(q, qq, gq, 0, k + 1, 0) * c12);
      }
      if (i < n - 2) {
        int k = (i + n) / 2;
        if ((i + n) % 2 == 0)
          return v + (sv<T>(q, qq, gq, 0, k - 1, 0) * c12 + sv<T>(q, qq, gq, 0, k, 0) * T(0.5) - sv<T>(q, qq, gq, 0, k + 1, 0) * c20);
        return v + (-sv<T>(q, qq, gq, 0, k - 1, 0) * c20 + sv<T>(q, qq, gq, 0, k, 0) * T(0.5) + sv<T>(q, qq, gq, 0, k + 1, 0) * c12);
      }
      if (i == n - 2)
        return v + (T(0.35) * sv<T>(q, qq, gq, 0, n - 1, 0) + T(7) * sv<T>(q, qq, gq, 0, n - 2, 0) * c30 -
                    sv<T>(q, qq, gq, 0, n - 3, 0) * c20);
      return v + (T(0.75) * sv<T>(q, qq, gq, 0, n - 1, 0) - T(0.3) * sv<T>(q, qq, gq, 0, n - 2, 0) + sv<T>(q, qq, gq, 0, n - 3, 0) * c12);
    }
    // BiLinear sides (:61-105) and TriLinear edges (:140-171)
    if (type == TE_NBR_COARSE) {
      for (int idx = 2 * i - off; idx <= 2 * i + 1 - off; idx++)
        if (idx >= 0 && idx < n) v += K<T>::two3 * sv<T>(q, qq, gq, 0, idx, 0);
      return v;
    }
    return v + K<T>::two3 * sv<T>(q, qq, gq, 0, (i + off) / 2, 0);
  }
  // TriLinear sides (:58-99); offsets from getOffset (:28-44)
  int oi = (orth & 1) ? gq.nt[0] : 0, oj = (orth & 2) ? gq.nt[1] : 0;
  if (type == TE_NBR_COARSE) {
    for (int jj = 2 * j - oj; jj <= 2 * j + 1 - oj; jj++)
      for (int ii = 2 * i - oi; ii <= 2 * i + 1 - oi; ii++)
        if (ii >= 0 && ii < gq.nt[0] && jj >= 0 && jj < gq.nt[1]) v += third * sv<T>(q, qq, gq, 0, ii, jj);
    return v;
  }
  return v + K<T>::two3 * sv<T>(q, qq, gq, 0, (i + oi) / 2, (j + oj) / 2);
}


// Value of ghost cell (i, j) of slab `sl` of patch p: zero (or the current
// value), the patch's own terms, then the incoming calls in reference order.
template <class T, int SCHEME, class Acc>
__device__ __forceinline__ T gather_ghost(const Acc& acc, int p, const GSlab& sl, const FaceGeom& g,
                                          const FaceTable& ft, const GCall* __restrict__ calls, int D, int i, int j,
                                          T start) {
  T v = sl.zero ? T(0) : start;
  v = own_term<T, SCHEME>(v, acc, p, g, sl.M, D, sl.own_type, sl.own_orth, i, j);
  for (int k = 0; k < sl.ncalls; k++) {
    GCall cl = calls[sl.call0 + k];
    const FaceGeom& gq =
        ft.f[sl.M == D - 1 ? (D == 2 ? 4 : 20) + cl.src_face : (sl.M == 0 ? cl.src_face : 8 + cl.src_face)];
    v = call_term<T, SCHEME>(v, acc, cl.src, gq, sl.M, D, cl.type, cl.orth, i, j);
  }
  return v;
}

// Side ghost (i, j) of patch p on side s, from the side's code (te_ghost_filler::
// d_side_code, not -1): a plain copy of the neighbour's face cells, or the
// side's slab.  The copy is the value gather_ghost gives for a slab whose one
// call is a Normal neighbour's and that has no own term.
template <class T, int SCHEME, class Acc>
__device__ __forceinline__ T side_ghost(const Acc& acc, int p, int s, int code, const GSlab* __restrict__ slabs,
                                        const GCall* __restrict__ calls, const FaceTable& ft, int D, int i,
                                        int j) {
  const int side0 = D == 2 ? 4 : 20;
  if (code >= 0) return sv<T>(acc, code, ft.f[side0 + (s ^ 1)], 0, i, j);
  const GSlab sl = slabs[-2 - code];
  return gather_ghost<T, SCHEME>(acc, p, sl, ft.f[side0 + s], ft, calls, D, i, j, T(0));
}

// side_ghost from the side's record (te_ghost_filler::d_side_rec, code not -1):
// the same terms in the same order, with the slab's own term and calls read
// from the record.  A side has one incoming call per neighbour: at most 2 in
// 2D and 4 in 3D; a record with more (ncalls -1 or above that) reads its slab.
// IN_SMEM: the record is in shared memory, so the calls are read one at a time in a
// loop (one copy of the call's code); otherwise the loop is unrolled, so that a record
// held in registers is indexed with constants.
template <class T, int SCHEME, int D, bool IN_SMEM = false, class Acc>
__device__ __forceinline__ T side_ghost_rec(const Acc& acc, int p, int s, const SideRec& r,
                                            const GSlab* __restrict__ slabs, const GCall* __restrict__ calls,
                                            const FaceTable& ft, int i, int j) {
  constexpr int side0 = D == 2 ? 4 : 20;
  constexpr int MAXC = D == 2 ? 2 : kSideRecCalls;
  if (r.code >= 0) return sv<T>(acc, r.code, ft.f[side0 + (s ^ 1)], 0, i, j);
  if (r.ncalls < 0 || r.ncalls > MAXC) return side_ghost<T, SCHEME>(acc, p, s, r.code, slabs, calls, ft, D, i, j);
  T v = T(0);
  v = own_term<T, SCHEME>(v, acc, p, ft.f[side0 + s], D - 1, D, r.own_type, r.own_orth, i, j);
  if constexpr (IN_SMEM) {
#pragma unroll 1
    for (int k = 0; k < r.ncalls; k++) {
      const GCall cl = r.calls[k];
      v = call_term<T, SCHEME>(v, acc, cl.src, ft.f[side0 + cl.src_face], D - 1, D, cl.type, cl.orth, i, j);
    }
  } else {
#pragma unroll
    for (int k = 0; k < MAXC; k++) {
      if (k >= r.ncalls) break;
      const GCall cl = r.calls[k];
      v = call_term<T, SCHEME>(v, acc, cl.src, ft.f[side0 + cl.src_face], D - 1, D, cl.type, cl.orth, i, j);
    }
  }
  return v;
}

// Face (side) ghosts of up to NP patches into shared memory,
// G[(q * 2D + side) * gstride + j*nt0 + i] for patch slot q, for every side
// with a neighbour; side_code[p * 2D + side] is that side's code (-1: none,
// the entry is left alone).  Every thread takes whole ghost values; there is
// no barrier inside: the caller synchronises before reading G.
template <class T, int SCHEME, class Acc>
__device__ __forceinline__ void side_ghosts_table(const Acc& acc, const int* pq, int NP,
                                                  const GSlab* __restrict__ slabs, const GCall* __restrict__ calls,
                                                  const int* __restrict__ side_code, const FaceTable& ft, int D,
                                                  T* G, int gstride) {
  const int side0 = D == 2 ? 4 : 20;
  const int per = 2 * D * gstride;
  for (int e = threadIdx.x; e < NP * per; e += blockDim.x) {
    const int q = e / per, rem = e - q * per, s = rem / gstride, r = rem - s * gstride;
    const int p = pq[q];
    if (p < 0) continue;
    const FaceGeom& g = ft.f[side0 + s];
    if (r >= g.nt[0] * g.nt[1]) continue;
    const int code = side_code[p * 2 * D + s];
    if (code == -1) continue;
    G[e] = side_ghost<T, SCHEME>(acc, p, s, code, slabs, calls, ft, D, r % g.nt[0], r / g.nt[0]);
  }
}

}  // namespace te
