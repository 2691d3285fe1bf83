// te_fused.cu -- the V-cycle's fused per-level kernels (DFT smoother path).
//
// One level of VCycle::visit (GMG/VCycle.h:46-70) with one pre- and one
// post-sweep of the DFT patch smoother is three kernels here instead of six:
//
//   vc_pre_kernel      the pre-smooth starts from u = 0, so its ghost fill and
//                      internal-boundary RHS terms vanish: A = DFT(f)
//   vc_restrict_kernel Cycle::restrict (GMG/Cycle.h:57-65): each coarse patch's
//                      CTA gathers the side ghosts of its children from A
//                      (MPIGhostFiller scheme formulas), forms r = f - A u in
//                      registers and averages it into the coarse cell
//   vc_post_kernel     DirectInterpolator (u = A + P u_coarse), ghost fill and
//                      the post-smooth (PatchSolver::smooth, PatchSolver.h:142-170)
//                      in one pass: the corrected iterate is never stored; the
//                      ghosts a patch needs are gathered from its neighbours'
//                      corrected values; the solve is written to a second
//                      buffer so no CTA overwrites values another one reads.
//
// The finest level reads f in FP64 and writes u in FP64 even when the cycle
// computes in FP32, so no conversion passes are needed.

#include <cstdlib>
#include <type_traits>

#include "te_dft.cuh"
#include "te_ghost_dev.cuh"
#include "te_gmg.cuh"

namespace te {

// u + interpolated coarse correction, evaluated on the fly (DirectInterpolator.h:60-91);
// uc == nullptr: u alone
template <class T>
struct InterpAcc {
  const T* A;
  const T* uc;
  const int* parent;
  const int* orth;
  Layout F, C;
  __device__ __forceinline__ T operator()(int q, int idx) const {
    if (!uc) return A[(long long)q * F.cs + idx];
    int x = idx % F.sy - F.g;
    int r = idx / F.sy;
    const int py = F.n1 + 2 * F.g;
    int y = r % py - F.g;
    int z = r / py - (F.D == 3 ? F.g : 0);
    int o = orth[q];
    int cidx;
    if (o >= 0) {
      int cx = (x + ((o & 1) ? C.n0 : 0)) / 2;
      int cy = F.D > 1 ? (y + ((o & 2) ? C.n1 : 0)) / 2 : 0;
      int cz = F.D > 2 ? (z + ((o & 4) ? C.n2 : 0)) / 2 : 0;
      cidx = C.at(cx, cy, cz);
    } else {
      cidx = idx;
    }
    return A[(long long)q * F.cs + idx] + uc[(long long)parent[q] * C.cs + cidx];
  }
};

// InterpAcc for cubic patches of NN cells with one ghost layer: the same
// values, with the padded-index decode done by constant divisors
template <class T, int DIM, int NN>
struct InterpAccN {
  const T* A;
  const T* uc;
  const int* parent;
  const int* orth;
  static constexpr int SY = NN + 2, SZ = DIM == 3 ? SY * SY : 0, CS = DIM == 3 ? SY * SY * SY : SY * SY;
  __device__ __forceinline__ T operator()(int q, int idx) const {
    if (!uc) return A[(long long)q * CS + idx];
    const int x = idx % SY - 1, r = idx / SY;
    const int y = r % SY - 1, z = DIM == 3 ? r / SY - 1 : 0;
    const int o = __ldg(orth + q);
    int cidx = idx;
    if (o >= 0) {
      const int cx = (x + ((o & 1) ? NN : 0)) >> 1;
      const int cy = (y + ((o & 2) ? NN : 0)) >> 1;
      const int cz = DIM == 3 ? (z + ((o & 4) ? NN : 0)) >> 1 : 0;
      cidx = (cx + 1) + (cy + 1) * SY + (DIM == 3 ? (cz + 1) * SZ : 0);
    }
    return A[(long long)q * CS + idx] + uc[(long long)__ldg(parent + q) * CS + cidx];
  }
};

__device__ __forceinline__ int side_tangential_index(const Layout& L, int a, int x, int y, int z) {
  if (a == 0) return y + z * L.n1;
  if (a == 1) return x + z * L.n0;
  return x + y * L.n0;
}

// ---------------------------------------------------------------------------
template <class T, class TF>
__global__ void __launch_bounds__(1024) vc_pre_kernel(Layout L, int ti_max, const int* __restrict__ plan_of_patch, const int* __restrict__ plan_mats,
                              const T* __restrict__ mats, const int* __restrict__ mat_off,
                              const T* __restrict__ inv_eig, const int* __restrict__ zero_mode, T scale,
                              const TF* __restrict__ f, T* __restrict__ out) {
  extern __shared__ __align__(16) unsigned char smraw[];
  T* sm = reinterpret_cast<T*>(smraw);
  const SmemLay S = smem_lay(L);
  const int p = blockIdx.x, N = L.interior();
  T* A = sm;
  T* B = A + S.size;
  const int plan = plan_of_patch[p];
  const T* MT[6];
  dft_mat_ptrs<T>(L, plan, plan_mats, mats, mat_off, MT);
  const TF* fp = f + (long long)p * L.cs;
#pragma unroll 4
  for (int e = threadIdx.x; e < N; e += blockDim.x) {
    int x = e % L.n0, r = e / L.n0, y = r % L.n1, z = r / L.n1;
    A[x + y * S.sy + z * S.sz] = (T)fp[L.at(x, y, z)];
  }
  __syncthreads();
  T* cur = dft_solve_smem<T>(L, S, MT, inv_eig + (long long)plan * N, zero_mode[p] != 0, A, B, ti_max);
  T* op = out + (long long)p * L.cs;
  const int py = L.n1 + 2 * L.g;
  for (int k = threadIdx.x; k < L.cs; k += blockDim.x) {
    int x = k % L.sy - L.g, q = k / L.sy, y = q % py - L.g, z = q / py - (L.D == 3 ? L.g : 0);
    bool in = x >= 0 && x < L.n0 && y >= 0 && y < L.n1 && z >= 0 && z < L.n2;
    op[k] = in ? cur[x + y * S.sy + z * S.sz] * scale : T(0);
  }
}

// ---------------------------------------------------------------------------
template <class T, class TF, int KIND, int SCHEME, int DIM>
__global__ void __launch_bounds__(1024)
    vc_restrict_kernel(Layout F, Layout C, const int* __restrict__ by_orth, const int* __restrict__ copy_of,
                       const int8_t* __restrict__ fntype, int FS, const T* __restrict__ finv, int neumann,
                       const T* __restrict__ coeff, FaceTable ft, const GSlab* __restrict__ slabs,
                       const GCall* __restrict__ calls, const int* __restrict__ side_code, int gstride,
                       const T* __restrict__ u, const TF* __restrict__ f, T* __restrict__ coarse) {
  extern __shared__ __align__(16) unsigned char smraw[];
  T* G = reinterpret_cast<T*>(smraw);  // [2^D][2D][gstride]
  const int cp = blockIdx.x;
  const int D = DIM;
  const int NCH = 1 << D;
  __shared__ int s_fp[8];
  __shared__ int s_has[8];
  __shared__ T s_inv[8][3];
  const int copy = copy_of[cp];
  if (threadIdx.x < NCH) {
    int q = threadIdx.x;
    int fp = copy >= 0 ? (q == 0 ? copy : -1) : by_orth[cp * NCH + q];
    s_fp[q] = fp;
    int m = 0;
    if (fp >= 0) {
      const int side0 = D == 2 ? 4 : 20;
      for (int sd = 0; sd < 2 * D; sd++) m |= (fntype[(size_t)fp * FS + side0 + sd] >= 0) << sd;
      for (int a2 = 0; a2 < 3; a2++) s_inv[q][a2] = finv[(size_t)fp * 6 + (KIND ? 3 : 0) + a2];
    }
    s_has[q] = m;
  }
  __syncthreads();
  PlainAcc<T> acc{u, (long long)F.cs, 0};
  side_ghosts_table<T, SCHEME>(acc, s_fp, NCH, slabs, calls, side_code, ft, D, G, gstride);
  __syncthreads();
  const T wD = T(1.0 / (1 << D));
  const int py = C.n1 + 2 * C.g;
  for (int e = threadIdx.x; e < C.cs; e += blockDim.x) {
    int cc[3];
    cc[0] = e % C.sy - C.g;
    int q = e / C.sy;
    cc[1] = q % py - C.g;
    cc[2] = q / py - (D == 3 ? C.g : 0);
    bool interior = cc[0] >= 0 && cc[0] < C.n0 && cc[1] >= 0 && cc[1] < C.n1 && cc[2] >= 0 && cc[2] < C.n2;
    T v = T(0);
    if (interior) {
      int o = 0, lo[3] = {0, 0, 0}, hi[3] = {0, 0, 0};
      if (copy >= 0) {
        for (int a2 = 0; a2 < D; a2++) lo[a2] = hi[a2] = cc[a2];
      } else {
        for (int a2 = 0; a2 < D; a2++) {
          int up = 2 * cc[a2] >= C.n(a2);
          o |= up << a2;
          lo[a2] = 2 * cc[a2] - (up ? C.n(a2) : 0);
          hi[a2] = lo[a2] + 1;
        }
      }
      const int fp = s_fp[o];
      if (fp >= 0) {
        const int hasn = s_has[o];
        const T* up_ = u + (long long)fp * F.cs;
        const TF* fv = f + (long long)fp * F.cs;
        const T* cf = KIND ? coeff + (long long)fp * F.cs : nullptr;
        const T* Gq = G + o * 2 * DIM * gstride;
        // r = f - A u at fine cell (x, y, z) (StarPatchOperator::applySinglePatch + scaleThenAdd)
        auto resid = [&](int x, int y, int z) -> T {
          int fk = F.at(x, y, z);
          int fc[3] = {x, y, z};
          T mid = up_[fk];
          T au = T(0);
#pragma unroll
          for (int a2 = 0; a2 < DIM; a2++) {
            int st = F.stride(a2);
            T lov, hiv;
            if (fc[a2] == 0)
              lov = ((hasn >> (2 * a2)) & 1) ? Gq[(2 * a2) * gstride + side_tangential_index(F, a2, x, y, z)]
                                             : (neumann ? mid : -mid);
            else
              lov = up_[fk - st];
            if (fc[a2] == F.n(a2) - 1)
              hiv = ((hasn >> (2 * a2 + 1)) & 1) ? Gq[(2 * a2 + 1) * gstride + side_tangential_index(F, a2, x, y, z)]
                                                 : (neumann ? mid : -mid);
            else
              hiv = up_[fk + st];
            if (KIND == 0) {
              au += ((hiv - T(2) * mid) + lov) * s_inv[o][a2];
            } else {
              T cl = cf[fk - st], cm = cf[fk], cu = cf[fk + st];
              au += ((cu + cm) * (hiv - mid) - (cl + cm) * (mid - lov)) * s_inv[o][a2];
            }
          }
          return au * T(-1) + (T)fv[fk];
        };
        if (copy >= 0) {
          v = resid(lo[0], lo[1], lo[2]);
        } else {
          // fine loop order z, y, x as restrictToCoarserParent (LinearRestrictor.h:115-127)
#pragma unroll
          for (int dz = 0; dz < (DIM == 3 ? 2 : 1); dz++)
#pragma unroll
            for (int dy = 0; dy < 2; dy++)
#pragma unroll
              for (int dx = 0; dx < 2; dx++) v += resid(lo[0] + dx, lo[1] + dy, lo[2] + dz) * wD;
        }
      }
    }
    coarse[(long long)cp * C.cs + e] = v;
  }
}

// ---------------------------------------------------------------------------
template <class T, class TF, class TO, int KIND, int SCHEME>
__global__ void __launch_bounds__(1024) vc_post_kernel(Layout F, Layout C, int ti_max, const int* __restrict__ parent, const int* __restrict__ porth,
                               const int8_t* __restrict__ ntype, int FS, const T* __restrict__ inv_tab,
                               const T* __restrict__ coeff, FaceTable ft, const GSlab* __restrict__ slabs,
                               const GCall* __restrict__ calls, const int* __restrict__ side_code, int gstride,
                               const int* __restrict__ plan_of_patch, const int* __restrict__ plan_mats,
                               const T* __restrict__ mats, const int* __restrict__ mat_off,
                               const T* __restrict__ inv_eig, const int* __restrict__ zero_mode, T scale,
                               const T* __restrict__ A, const T* __restrict__ uc, const TF* __restrict__ f,
                               TO* __restrict__ out) {
  extern __shared__ __align__(16) unsigned char smraw[];
  const SmemLay S = smem_lay(F);
  const int p = blockIdx.x, N = F.interior(), D = F.D;
  T* Ab = reinterpret_cast<T*>(smraw);
  T* Bb = Ab + S.size;
  T* G = Ab + S.mats;  // [2D][gstride]
  const int plan = plan_of_patch[p];
  const T* MT[6];
  dft_mat_ptrs<T>(F, plan, plan_mats, mats, mat_off, MT);
  InterpAcc<T> acc{A, uc, parent, porth, F, C};
  int pself[1] = {p};
  side_ghosts_table<T, SCHEME>(acc, pself, 1, slabs, calls, side_code, ft, D, G, gstride);
  __syncthreads();
  // f_copy with modifyRHSForInternalBoundaryConditions, sides in Side order
  const int side0 = D == 2 ? 4 : 20;
  T inv[3];
  for (int a = 0; a < 3; a++) inv[a] = inv_tab[(size_t)p * 6 + (KIND ? 3 : 0) + a];
  const TF* fp = f + (long long)p * F.cs;
  const T* cp = KIND ? coeff + (long long)p * F.cs : nullptr;
#pragma unroll 2
  for (int e = threadIdx.x; e < N; e += blockDim.x) {
    int x = e % F.n0, r = e / F.n0, y = r % F.n1, z = r / F.n1;
    int k = F.at(x, y, z);
    T v = (T)fp[k];
    int cc[3] = {x, y, z};
    for (int side = 0; side < 2 * D; side++) {
      int a = side >> 1, upr = side & 1;
      if (cc[a] != (upr ? F.n(a) - 1 : 0)) continue;
      if (ntype[(size_t)p * FS + side0 + side] < 0) continue;
      T gv = G[side * gstride + side_tangential_index(F, a, x, y, z)];
      T uv = acc(p, k);
      if (KIND == 0) {
        v -= (gv + uv) * inv[a];
      } else {
        int gk = k + (upr ? F.stride(a) : -F.stride(a));
        v -= (gv + uv) * (cp[k] + cp[gk]) * inv[a];
      }
    }
    Ab[x + y * S.sy + z * S.sz] = v;
  }
  __syncthreads();
  T* cur = dft_solve_smem<T>(F, S, MT, inv_eig + (long long)plan * N, zero_mode[p] != 0, Ab, Bb, ti_max);
  TO* op = out + (long long)p * F.cs;
  const int py = F.n1 + 2 * F.g;
  for (int k = threadIdx.x; k < F.cs; k += blockDim.x) {
    int x = k % F.sy - F.g, q = k / F.sy, y = q % py - F.g, z = q / py - (D == 3 ? F.g : 0);
    bool in = x >= 0 && x < F.n0 && y >= 0 && y < F.n1 && z >= 0 && z < F.n2;
    op[k] = in ? (TO)(cur[x + y * S.sy + z * S.sz] * scale) : TO(0);
  }
}

// ---------------------------------------------------------------------------
// Boundary corrections of the post-smooth right-hand side
// (modifyRHSForInternalBoundaryConditions, Poisson/StarPatchOperator.h:145-180,
// VarPoisson/StarPatchOperator.h:150-186) for the corrected iterate
// u = A + P u_coarse, which is never stored: one thread per cell of a side
// face that has a neighbour computes the ghost value (the filler's gather on
// the fly) and the correction c = (ghost + u_boundary) / h^2 (Poisson) or
// (ghost + u_boundary) (c_in + c_ghost) / (2 h^2) (VarPoisson).  The solve
// then subtracts the corrections of a cell's sides in side order:
// f_copy = f - c_side0 - c_side1 ...  Faces without a neighbour get 0.
// corr is [P][2D][gs], gs = the largest face size.
template <int KIND, int SCHEME, int DIM>
__global__ void __launch_bounds__(256)
    vc_corr_kernel(Layout F, Layout C, const int* __restrict__ parent, const int* __restrict__ porth,
                   const float* __restrict__ inv_tab, const float* __restrict__ coeff, FaceTable ft,
                   const GSlab* __restrict__ slabs, const GCall* __restrict__ calls,
                   const int* __restrict__ side_code, int gs, const float* __restrict__ A,
                   const float* __restrict__ uc, float* __restrict__ corr) {
  const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const long long total = (long long)F.P * 2 * DIM * gs;
  if (e >= total) return;
  const int r = (int)(e % gs);
  const int s = (int)((e / gs) % (2 * DIM));
  const int p = (int)(e / ((long long)gs * 2 * DIM));
  const int a = s >> 1, upr = s & 1;
  const int side0 = DIM == 2 ? 4 : 20;
  const FaceGeom& g = ft.f[side0 + s];
  if (r >= g.nt[0] * g.nt[1]) return;
  const int code = side_code[p * 2 * DIM + s];
  float c = 0.f;
  if (code != -1) {
    InterpAcc<float> acc{A, uc, parent, porth, F, C};
    const int i = r % g.nt[0], j = r / g.nt[0];
    const float gv = side_ghost<float, SCHEME>(acc, p, s, code, slabs, calls, ft, DIM, i, j);
    const int coord = upr ? F.n(a) - 1 : 0;
    int x, y, z;
    if (a == 0) {
      x = coord; y = i; z = j;
    } else if (a == 1) {
      x = i; y = coord; z = j;
    } else {
      x = i; y = j; z = coord;
    }
    const int k = F.at(x, y, z);
    const float uv = acc(p, k);
    const float inv = inv_tab[(size_t)p * 6 + (KIND ? 3 : 0) + a];
    if (KIND == 0) {
      c = (gv + uv) * inv;
    } else {
      const float* cp = coeff + (long long)p * F.cs;
      const int gk = k + (upr ? F.stride(a) : -F.stride(a));
      c = (gv + uv) * (cp[k] + cp[gk]) * inv;
    }
  }
  corr[e] = c;
}

// vc_corr_kernel for cubic patches of NN cells and one ghost layer (constant index arithmetic)
template <int KIND, int SCHEME, int DIM, int NN>
__global__ void __launch_bounds__(256)
    vc_corr_kernel_n(int P, const int* __restrict__ parent, const int* __restrict__ porth,
                     const float* __restrict__ inv_tab, const float* __restrict__ coeff, FaceTable ft,
                     const GSlab* __restrict__ slabs, const GCall* __restrict__ calls,
                     const int* __restrict__ side_code, const float* __restrict__ A, const float* __restrict__ uc,
                     float* __restrict__ corr) {
  constexpr int NF = DIM == 3 ? NN * NN : NN;
  constexpr int SY = NN + 2, SZ = DIM == 3 ? SY * SY : 0, CS = DIM == 3 ? SY * SY * SY : SY * SY;
  const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= (long long)P * 2 * DIM * NF) return;
  const int r = (int)(e % NF);
  const int s = (int)((e / NF) % (2 * DIM));
  const int p = (int)(e / (NF * 2 * DIM));
  const int code = side_code[p * 2 * DIM + s];
  float c = 0.f;
  if (code != -1) {
    const int a = s >> 1, upr = s & 1;
    const InterpAccN<float, DIM, NN> acc{A, uc, parent, porth};
    const int i = r % NN, j = r / NN;
    const float gv = side_ghost<float, SCHEME>(acc, p, s, code, slabs, calls, ft, DIM, i, j);
    const int edge = upr ? NN - 1 : 0;
    int x, y, z;
    if (a == 0) {
      x = edge; y = i; z = j;
    } else if (a == 1) {
      x = i; y = edge; z = j;
    } else {
      x = i; y = j; z = edge;
    }
    const int k = (x + 1) + (y + 1) * SY + (DIM == 3 ? (z + 1) * SZ : 0);
    const float uv = acc(p, k);
    const float inv = inv_tab[(size_t)p * 6 + (KIND ? 3 : 0) + a];
    if (KIND == 0) {
      c = (gv + uv) * inv;
    } else {
      const float* cp = coeff + (long long)p * CS;
      const int st = a == 0 ? 1 : (a == 1 ? SY : SZ);
      const int gk = k + (upr ? st : -st);
      c = (gv + uv) * (cp[k] + cp[gk]) * inv;
    }
  }
  corr[e] = c;
}

// ---------------------------------------------------------------------------
// host launchers
// ---------------------------------------------------------------------------
static size_t dft_bytes(const Layout& L, int tsize) {
  SmemLay S = smem_lay(L);
  return ((size_t)S.mats + smem_mat_elems(L)) * tsize;
}
static int gstride_of(const Layout& L) {
  int m = 1;
  for (int a = 0; a < L.D; a++) {
    int t = 1;
    for (int b = 0; b < L.D; b++)
      if (b != a) t *= L.n(b);
    m = std::max(m, t);
  }
  return m;
}
template <class K>
static void raise_smem(K kern, size_t bytes) {
  if (bytes > 40 * 1024)  // leave room for the static shared memory
    allow_max_dynamic_smem((const void*)kern);
}

static double dft_scale(const Layout& L) {
  double s = 1.0;
  for (int a = 0; a < L.D; a++) s *= 2.0 / L.n(a);
  return s;
}

template <class T>
static const T* mats_of(const te_patch_solver* ps);
template <>
const double* mats_of<double>(const te_patch_solver* ps) { return ps->mats.p; }
template <>
const float* mats_of<float>(const te_patch_solver* ps) { return ps->mats_f.p; }
template <class T>
static const T* ie_of(const te_patch_solver* ps);
template <>
const double* ie_of<double>(const te_patch_solver* ps) { return ps->inv_eig.p; }
template <>
const float* ie_of<float>(const te_patch_solver* ps) { return ps->inv_eig_f.p; }
template <class T>
static const T* coeff_of(const te_operator* op);
template <>
const double* coeff_of<double>(const te_operator* op) { return op->coeffs.p; }
template <>
const float* coeff_of<float>(const te_operator* op) { return op->coeffs_f.p; }

template <class T, class TF>
void vc_pre(const te_patch_solver* ps, const TF* f, T* out, cudaStream_t s) {
  const Layout& L = ps->op->dom->lay;
  size_t smem = dft_bytes(L, sizeof(T));
  auto kern = vc_pre_kernel<T, TF>;
  raise_smem(kern, smem);
  int ti_max, threads;
  dft_launch_shape(L, ti_max, threads);
  kern<<<L.P, threads, smem, s>>>(L, ti_max, ps->plan_of_patch.p, ps->plan_mats.p, mats_of<T>(ps), ps->mat_off.p,
                                          ie_of<T>(ps), ps->zero_mode.p, (T)dft_scale(L), f, out);
  count_launch();
  TE_LAUNCH_CHECK();
}

template <class T, class TF, int KIND, int SCHEME>
static void vc_restrict_t(const te_restrictor* r, const te_operator* op, const T* u, const TF* f, T* coarse,
                          cudaStream_t s) {
  const te_domain* fd = r->fine;
  const Layout &F = fd->lay, &C = r->coarse->lay;
  const te_ghost_filler* g = op->gf;
  int gs = gstride_of(F);
  size_t smem = (size_t)(1 << F.D) * 2 * F.D * gs * sizeof(T);
  auto kern = F.D == 2 ? vc_restrict_kernel<T, TF, KIND, SCHEME, 2> : vc_restrict_kernel<T, TF, KIND, SCHEME, 3>;
  raise_smem(kern, smem);
  int threads = C.P >= 2 * 152 ? 256 : 1024;
  kern<<<C.P, threads, smem, s>>>(F, C, r->by_orth.p, r->copy_of.p, fd->d_nbr_type.p, fd->F, fd->template inv<T>(),
                               op->neumann, coeff_of<T>(op), g->faces, g->d_slabs.p, g->d_calls.p,
                               g->d_side_code.p, gs, u, f, coarse);
  count_launch();
  TE_LAUNCH_CHECK();
}

template <class T, class TF>
void vc_restrict(const te_restrictor* r, const te_operator* op, const T* u, const TF* f, T* coarse,
                 cudaStream_t s) {
  if constexpr (std::is_same<T, float>::value) {
    static const bool off = [] {
      const char* e = getenv("TE_NO_FINE_RESTRICT");
      return e && e[0] == '1';
    }();
    if (!off && vc_restrict_fine<T, TF>(r, op, u, f, coarse, s)) return;
  }
  int sc = op->gf->scheme;
#define TE_VR(K, S) vc_restrict_t<T, TF, K, S>(r, op, u, f, coarse, s)
  if (op->kind == 0) {
    if (sc == TE_GHOST_BILINEAR) TE_VR(0, TE_GHOST_BILINEAR);
    else if (sc == TE_GHOST_BIQUADRATIC) TE_VR(0, TE_GHOST_BIQUADRATIC);
    else TE_VR(0, TE_GHOST_TRILINEAR);
  } else {
    if (sc == TE_GHOST_BILINEAR) TE_VR(1, TE_GHOST_BILINEAR);
    else if (sc == TE_GHOST_BIQUADRATIC) TE_VR(1, TE_GHOST_BIQUADRATIC);
    else TE_VR(1, TE_GHOST_TRILINEAR);
  }
#undef TE_VR
}

template <class T, class TF, class TO, int KIND, int SCHEME>
static void vc_post_t(const te_patch_solver* ps, const te_interpolator* in, const T* A, const T* uc, const TF* f,
                      TO* out, cudaStream_t s) {
  const te_operator* op = ps->op;
  const te_domain* d = op->dom;
  const Layout &F = d->lay, &C = in->coarse->lay;
  const te_ghost_filler* g = op->gf;
  int gs = gstride_of(F);
  size_t smem = dft_bytes(F, sizeof(T)) + (size_t)2 * F.D * gs * sizeof(T);
  auto kern = vc_post_kernel<T, TF, TO, KIND, SCHEME>;
  raise_smem(kern, smem);
  int ti_max, threads;
  dft_launch_shape(F, ti_max, threads);
  kern<<<F.P, threads, smem, s>>>(F, C, ti_max, in->parent.p, in->orth.p, d->d_nbr_type.p, d->F,
                                          d->template inv<T>(), coeff_of<T>(op), g->faces, g->d_slabs.p,
                                          g->d_calls.p, g->d_side_code.p, gs, ps->plan_of_patch.p,
                                          ps->plan_mats.p, mats_of<T>(ps), ps->mat_off.p, ie_of<T>(ps),
                                          ps->zero_mode.p, (T)dft_scale(F), A, uc, f, out);
  count_launch();
  TE_LAUNCH_CHECK();
}

template <class T, class TF, class TO>
void vc_post(const te_patch_solver* ps, const te_interpolator* in, const T* A, const T* uc, const TF* f, TO* out,
             cudaStream_t s) {
  const te_operator* op = ps->op;
  int sc = op->gf->scheme;
#define TE_VP(K, S) vc_post_t<T, TF, TO, K, S>(ps, in, A, uc, f, out, s)
  if (op->kind == 0) {
    if (sc == TE_GHOST_BILINEAR) TE_VP(0, TE_GHOST_BILINEAR);
    else if (sc == TE_GHOST_BIQUADRATIC) TE_VP(0, TE_GHOST_BIQUADRATIC);
    else TE_VP(0, TE_GHOST_TRILINEAR);
  } else {
    if (sc == TE_GHOST_BILINEAR) TE_VP(1, TE_GHOST_BILINEAR);
    else if (sc == TE_GHOST_BIQUADRATIC) TE_VP(1, TE_GHOST_BIQUADRATIC);
    else TE_VP(1, TE_GHOST_TRILINEAR);
  }
#undef TE_VP
}

int corr_stride(const Layout& L) { return gstride_of(L); }

template <int KIND, int SCHEME>
static void vc_corr_t(const te_patch_solver* ps, const te_interpolator* in, const float* A, const float* uc,
                      float* corr, cudaStream_t s) {
  const te_operator* op = ps->op;
  const te_domain* d = op->dom;
  // in == nullptr (with uc == nullptr): the corrections of A alone, e.g. on the coarsest level
  const Layout &F = d->lay, &C = in ? in->coarse->lay : d->lay;
  const int* parent = in ? in->parent.p : nullptr;
  const int* orth = in ? in->orth.p : nullptr;
  require(in || !uc, "vc_corr: a coarse correction needs its interpolator");
  const te_ghost_filler* g = op->gf;
  const int gs = gstride_of(F);
  const long long total = (long long)F.P * 2 * F.D * gs;
  const int threads = 256;
  const unsigned blocks = (unsigned)((total + threads - 1) / threads);
  const bool cube = F.g == 1 && F.n1 == F.n0 && (F.D == 2 || F.n2 == F.n0);
  auto fixed = [&](auto kn) {
    kn<<<blocks, threads, 0, s>>>(F.P, parent, orth, d->template inv<float>(), op->coeffs_f.p, g->faces,
                                  g->d_slabs.p, g->d_calls.p, g->d_side_code.p, A, uc, corr);
  };
  bool done = false;
  if (cube && F.D == 2 && SCHEME != TE_GHOST_TRILINEAR) {
    done = true;
    if (F.n0 == 16) fixed(vc_corr_kernel_n<KIND, SCHEME, 2, 16>);
    else if (F.n0 == 32) fixed(vc_corr_kernel_n<KIND, SCHEME, 2, 32>);
    else if (F.n0 == 64) fixed(vc_corr_kernel_n<KIND, SCHEME, 2, 64>);
    else done = false;
  } else if (cube && F.D == 3 && SCHEME == TE_GHOST_TRILINEAR) {
    done = true;
    if (F.n0 == 8) fixed(vc_corr_kernel_n<KIND, SCHEME, 3, 8>);
    else if (F.n0 == 16) fixed(vc_corr_kernel_n<KIND, SCHEME, 3, 16>);
    else done = false;
  }
  if (!done) {
    auto kern = F.D == 2 ? vc_corr_kernel<KIND, SCHEME, 2> : vc_corr_kernel<KIND, SCHEME, 3>;
    kern<<<blocks, threads, 0, s>>>(F, C, parent, orth, d->template inv<float>(), op->coeffs_f.p,
                                    g->faces, g->d_slabs.p, g->d_calls.p, g->d_side_code.p, gs, A, uc, corr);
  }
  count_launch();
  TE_LAUNCH_CHECK();
}

void vc_corr(const te_patch_solver* ps, const te_interpolator* in, const float* A, const float* uc, float* corr,
             cudaStream_t s) {
  const te_operator* op = ps->op;
  int sc = op->gf->scheme;
#define TE_VC(K, S) vc_corr_t<K, S>(ps, in, A, uc, corr, s)
  if (op->kind == 0) {
    if (sc == TE_GHOST_BILINEAR) TE_VC(0, TE_GHOST_BILINEAR);
    else if (sc == TE_GHOST_BIQUADRATIC) TE_VC(0, TE_GHOST_BIQUADRATIC);
    else TE_VC(0, TE_GHOST_TRILINEAR);
  } else {
    if (sc == TE_GHOST_BILINEAR) TE_VC(1, TE_GHOST_BILINEAR);
    else if (sc == TE_GHOST_BIQUADRATIC) TE_VC(1, TE_GHOST_BIQUADRATIC);
    else TE_VC(1, TE_GHOST_TRILINEAR);
  }
#undef TE_VC
}

template void vc_pre<double, double>(const te_patch_solver*, const double*, double*, cudaStream_t);
template void vc_pre<float, double>(const te_patch_solver*, const double*, float*, cudaStream_t);
template void vc_pre<float, float>(const te_patch_solver*, const float*, float*, cudaStream_t);
template void vc_restrict<double, double>(const te_restrictor*, const te_operator*, const double*, const double*,
                                          double*, cudaStream_t);
template void vc_restrict<float, double>(const te_restrictor*, const te_operator*, const float*, const double*,
                                         float*, cudaStream_t);
template void vc_restrict<float, float>(const te_restrictor*, const te_operator*, const float*, const float*,
                                        float*, cudaStream_t);
template void vc_post<double, double, double>(const te_patch_solver*, const te_interpolator*, const double*,
                                              const double*, const double*, double*, cudaStream_t);
template void vc_post<float, double, double>(const te_patch_solver*, const te_interpolator*, const float*,
                                             const float*, const double*, double*, cudaStream_t);
template void vc_post<float, float, float>(const te_patch_solver*, const te_interpolator*, const float*,
                                           const float*, const float*, float*, cudaStream_t);

}  // namespace te
