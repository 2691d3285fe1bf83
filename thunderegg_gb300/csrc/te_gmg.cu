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
#include <cstdio>
#include <cstdlib>
#include <cstring>

#include "te_gmg.cuh"
#include "te_tune.cuh"

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

// interpolate_kernel for cubic patches of NN cells with one ghost layer:
// fine += the parent's coarse cell (DirectInterpolator, GMG/DirectInterpolator.h:
// 40-91) with constant index arithmetic.  A CTA takes PPC fine patches (two
// for FP32, so each thread keeps as many bytes in flight as for FP64) and a
// thread loads all of its cells (fine and coarse) before it stores.
template <class T, int DIM, int NN, int PPC>
__global__ void __launch_bounds__(256)
    interpolate_n_kernel(int P, int nc, const int* __restrict__ parent, const int* __restrict__ orth,
                         const T* __restrict__ coarse, T* __restrict__ fine) {
  constexpr int SY = NN + 2, SZ = DIM == 3 ? SY * SY : 0, CS = DIM == 3 ? SY * SY * SY : SY * SY;
  constexpr int NI = DIM == 3 ? NN * NN * NN : NN * NN;
  constexpr int PER = (NI + 255) / 256;
  int fp[PPC], o[PPC];
  const T* cv[PPC];
  T* fv[PPC];
#pragma unroll
  for (int q = 0; q < PPC; q++) {
    fp[q] = blockIdx.x * PPC + q;
    const int pp = fp[q] < P ? fp[q] : blockIdx.x * PPC;  // a valid patch for the table loads
    o[q] = orth[pp];
    cv[q] = coarse + (long long)parent[pp] * CS * nc;
    fv[q] = fine + (long long)pp * CS * nc;
  }
  for (int c = 0; c < nc; c++) {
    T a[PPC][PER], b[PPC][PER];
#pragma unroll
    for (int q = 0; q < PPC; q++) {
      const int ox = (o[q] >= 0 && (o[q] & 1)) ? NN : 0, oy = (o[q] >= 0 && (o[q] & 2)) ? NN : 0,
                oz = (o[q] >= 0 && (o[q] & 4)) ? NN : 0;
#pragma unroll
      for (int r = 0; r < PER; r++) {
        const int e = threadIdx.x + r * 256;
        if ((NI % 256 == 0 || e < NI) && fp[q] < P) {
          const int x = e % NN, y = (e / NN) % NN, z = DIM == 3 ? e / (NN * NN) : 0;
          const int k = (x + 1) + (y + 1) * SY + (DIM == 3 ? (z + 1) * SZ : 0);
          const int kc = o[q] < 0 ? k
                                  : ((x + ox) >> 1) + 1 + (((y + oy) >> 1) + 1) * SY +
                                        (DIM == 3 ? (((z + oz) >> 1) + 1) * SZ : 0);
          a[q][r] = fv[q][(long long)c * CS + k];
          b[q][r] = cv[q][(long long)c * CS + kc];
        }
      }
    }
#pragma unroll
    for (int q = 0; q < PPC; q++) {
#pragma unroll
      for (int r = 0; r < PER; r++) {
        const int e = threadIdx.x + r * 256;
        if ((NI % 256 == 0 || e < NI) && fp[q] < P) {
          const int x = e % NN, y = (e / NN) % NN, z = DIM == 3 ? e / (NN * NN) : 0;
          const int k = (x + 1) + (y + 1) * SY + (DIM == 3 ? (z + 1) * SZ : 0);
          fv[q][(long long)c * CS + k] = a[q][r] + b[q][r];
        }
      }
    }
  }
}

// restrict_kernel turned around for complete levels of cubic NN patches
// without ghost extrapolation: one CTA per FINE patch writes its orthant of
// the parent (restrictToCoarserParent, GMG/LinearRestrictor.h:101-128: the
// average of the 2^D fine cells, summed in the reference's z, y, x order) or,
// for a patch that is its own parent, copies its interior (copyToParent,
// :129-147).  The coarse ghost ring is zero: the orthant-0 child (or the
// copied patch) writes it.
// NTR threads per CTA: 256, or 128 (two coarse cells per thread at twice the resident CTAs;
// the autotuner picks, both give the same bits)
template <class T, int DIM, int NN, int NTR = 256>
__global__ void __launch_bounds__(NTR, 2048 / NTR)
    restrict_n_kernel(int nc, const int* __restrict__ fparent, const int* __restrict__ forth,
                      const T* __restrict__ fine, T* __restrict__ coarse) {
  constexpr int SY = NN + 2, SZ = DIM == 3 ? SY * SY : 0, CS = DIM == 3 ? SY * SY * SY : SY * SY;
  constexpr int H = NN / 2;
  constexpr int NQ = DIM == 3 ? H * H * H : H * H;  // coarse cells of one orthant
  constexpr int NI = DIM == 3 ? NN * NN * NN : NN * NN;
  constexpr int RING = CS - NI;
  const int fp = blockIdx.x;
  const int o = forth[fp];
  const T* fv = fine + (long long)fp * CS * nc;
  T* cv = coarse + (long long)fparent[fp] * CS * nc;
  const T wD = T(1.0 / (1 << DIM));
  for (int c = 0; c < nc; c++) {
    const T* fc = fv + (long long)c * CS;
    T* cc = cv + (long long)c * CS;
    if (o < 0) {
      constexpr int PER = (NI + NTR - 1) / NTR;
      T v[PER];
#pragma unroll
      for (int r = 0; r < PER; r++) {
        const int e = threadIdx.x + r * NTR;
        if (NI % NTR == 0 || e < NI) {
          const int x = e % NN, y = (e / NN) % NN, z = DIM == 3 ? e / (NN * NN) : 0;
          v[r] = fc[(x + 1) + (y + 1) * SY + (DIM == 3 ? (z + 1) * SZ : 0)];
        }
      }
#pragma unroll
      for (int r = 0; r < PER; r++) {
        const int e = threadIdx.x + r * NTR;
        if (NI % NTR == 0 || e < NI) {
          const int x = e % NN, y = (e / NN) % NN, z = DIM == 3 ? e / (NN * NN) : 0;
          cc[(x + 1) + (y + 1) * SY + (DIM == 3 ? (z + 1) * SZ : 0)] = v[r];
        }
      }
    } else {
      const int ox = (o & 1) ? H : 0, oy = (o & 2) ? H : 0, oz = (o & 4) ? H : 0;
      constexpr int PER = (NQ + NTR - 1) / NTR;
      T v[PER];
#pragma unroll
      for (int r = 0; r < PER; r++) {
        const int e = threadIdx.x + r * NTR;
        if (NQ % NTR == 0 || e < NQ) {
          const int x = e % H, y = (e / H) % H, z = DIM == 3 ? e / (H * H) : 0;
          const int k = (2 * x + 1) + (2 * y + 1) * SY + (DIM == 3 ? (2 * z + 1) * SZ : 0);
          T s = T(0);
#pragma unroll
          for (int dz = 0; dz < (DIM == 3 ? 2 : 1); dz++)
#pragma unroll
            for (int dy = 0; dy < 2; dy++)
#pragma unroll
              for (int dx = 0; dx < 2; dx++) s += fc[k + dx + dy * SY + dz * SZ] * wD;
          v[r] = s;
        }
      }
#pragma unroll
      for (int r = 0; r < PER; r++) {
        const int e = threadIdx.x + r * NTR;
        if (NQ % NTR == 0 || e < NQ) {
          const int x = e % H, y = (e / H) % H, z = DIM == 3 ? e / (H * H) : 0;
          cc[(x + ox + 1) + (y + oy + 1) * SY + (DIM == 3 ? (z + oz + 1) * SZ : 0)] = v[r];
        }
      }
    }
    if (o <= 0) {
      // ghost ring: 2D rows 0 and SY-1, then the end cells of rows 1..NN; 3D planes
      // 0 and SY-1, then the 2D ring of planes 1..NN
      for (int e = threadIdx.x; e < RING; e += NTR) {
        int k;
        if (DIM == 2) {
          if (e < 2 * SY) {
            k = e < SY ? e : (SY - 1) * SY + (e - SY);
          } else {
            const int r2 = e - 2 * SY;
            k = (1 + (r2 >> 1)) * SY + ((r2 & 1) ? SY - 1 : 0);
          }
        } else {
          constexpr int PL = SY * SY, R2 = 2 * SY + 2 * NN;
          if (e < 2 * PL) {
            k = e < PL ? e : (SY - 1) * PL + (e - PL);
          } else {
            const int q = e - 2 * PL, z = 1 + q / R2, r = q % R2;
            int k2;
            if (r < 2 * SY) {
              k2 = r < SY ? r : (SY - 1) * SY + (r - SY);
            } else {
              const int r2 = r - 2 * SY;
              k2 = (1 + (r2 >> 1)) * SY + ((r2 & 1) ? SY - 1 : 0);
            }
            k = z * PL + k2;
          }
        }
        cc[k] = T(0);
      }
    }
  }
}

// Cycle::restrict fused: r = f - A u on the fine level (Poisson or VarPoisson
// star stencil, boundary ghosts -u / +u as enforceBoundaryConditions) is
// formed in registers and averaged straight into the coarse cell
// (restrictToCoarserParent / copyToParent).  u's ghosts across faces with a
// neighbour must already be filled.  Used when ghost extrapolation is off.
template <class T, int KIND>
__global__ void residual_restrict_kernel(Layout F, Layout C, int nc, const int* __restrict__ cstart,
                                         const int* __restrict__ child, const int* __restrict__ corth,
                                         const int8_t* __restrict__ fntype, int FS, const T* __restrict__ fsp,
                                         int neumann, const T* __restrict__ coeff, const T* __restrict__ fu,
                                         const T* __restrict__ ff, T* __restrict__ coarse) {
  const int cp = blockIdx.x;
  const int D = C.D;
  const T wD = T(1.0 / (1 << D));
  const int k0 = cstart[cp], k1 = cstart[cp + 1];
  const int py = C.n1 + 2 * C.g;
  const int side0 = D == 2 ? 4 : 20;
  const long long fps = F.pstride(nc), cps = C.pstride(nc);
  const int tot = C.cs * nc;
  for (int e = threadIdx.x; e < tot; e += blockDim.x) {
    int c = e / C.cs, k = e - c * C.cs;
    int cc[3];
    cc[0] = k % C.sy - C.g;
    int q = k / C.sy;
    cc[1] = q % py - C.g;
    cc[2] = q / py - (D == 3 ? C.g : 0);
    bool interior = cc[0] >= 0 && cc[0] < C.n0 && cc[1] >= 0 && cc[1] < C.n1 && cc[2] >= 0 && cc[2] < C.n2;
    T v = T(0);
    if (interior) {
      for (int qq = k0; qq < k1; qq++) {
        const int fp = child[qq], o = corth[qq];
        const T* u = fu + fp * fps + (long long)c * F.cs;
        const T* f = ff + fp * fps + (long long)c * F.cs;
        const T* cf = KIND ? coeff + (long long)fp * F.cs : nullptr;
        T inv[3];
        int hasn[6];
        for (int a = 0; a < 3; a++) inv[a] = fsp[(size_t)fp * 6 + (KIND ? 3 : 0) + a];
        for (int sd = 0; sd < 2 * D; sd++) hasn[sd] = fntype[(size_t)fp * FS + side0 + sd] >= 0;
        int lo[3], hi[3];
        for (int a = 0; a < 3; a++) {
          if (a >= D) {
            lo[a] = hi[a] = 0;
          } else if (o < 0) {
            lo[a] = hi[a] = cc[a];
          } else {
            int st = ((o >> a) & 1) ? C.n(a) : 0;
            lo[a] = max(2 * cc[a] - st, 0);
            hi[a] = min(2 * cc[a] + 1 - st, F.n(a) - 1);
          }
        }
        for (int z = lo[2]; z <= hi[2]; z++)
          for (int y = lo[1]; y <= hi[1]; y++)
            for (int x = lo[0]; x <= hi[0]; x++) {
              int fk = F.at(x, y, z);
              int fc[3] = {x, y, z};
              T mid = u[fk];
              T au = T(0);
              for (int a = 0; a < D; a++) {
                int st = F.stride(a);
                T lov, hiv;
                if (fc[a] == 0 && !hasn[2 * a])
                  lov = neumann ? mid : -mid;
                else
                  lov = u[fk - st];
                if (fc[a] == F.n(a) - 1 && !hasn[2 * a + 1])
                  hiv = neumann ? mid : -mid;
                else
                  hiv = u[fk + st];
                if (KIND == 0) {
                  au += ((hiv - T(2) * mid) + lov) * inv[a];
                } else {
                  T cl = cf[fk - st], cm = cf[fk], cu = cf[fk + st];
                  au += ((cu + cm) * (hiv - mid) - (cl + cm) * (mid - lov)) * inv[a];
                }
              }
              T r = au * T(-1) + f[fk];
              if (o < 0)
                v += r;
              else
                v += r * wD;
            }
      }
    }
    coarse[cp * cps + e] = v;
  }
}

// Even patch sizes: every coarse cell has exactly one contributing child (or
// is a copy), so the children's metadata is staged in shared memory once and
// each thread does one coarse cell without searching.
template <class T, int KIND>
__global__ void __launch_bounds__(256)
    residual_restrict_even_kernel(Layout F, Layout C, int nc, const int* __restrict__ by_orth,
                                  const int* __restrict__ copy_of, const int8_t* __restrict__ fntype, int FS,
                                  const T* __restrict__ finv, int neumann, const T* __restrict__ coeff,
                                  const T* __restrict__ fu, const T* __restrict__ ff, T* __restrict__ coarse) {
  const int cp = blockIdx.x;
  const int D = C.D;
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
  const T wD = T(1.0 / (1 << D));
  const int py = C.n1 + 2 * C.g;
  const long long fps = F.pstride(nc), cps = C.pstride(nc);
  const int tot = C.cs * nc;
  for (int e = threadIdx.x; e < tot; e += blockDim.x) {
    int c = e / C.cs, k = e - c * C.cs;
    int cc[3];
    cc[0] = k % C.sy - C.g;
    int q = k / C.sy;
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
        const T* u = fu + fp * fps + (long long)c * F.cs;
        const T* f = ff + fp * fps + (long long)c * F.cs;
        const T* cf = KIND ? coeff + (long long)fp * F.cs : nullptr;
        for (int z = lo[2]; z <= hi[2]; z++)
          for (int y = lo[1]; y <= hi[1]; y++)
            for (int x = lo[0]; x <= hi[0]; x++) {
              int fk = F.at(x, y, z);
              int fc[3] = {x, y, z};
              T mid = u[fk];
              T au = T(0);
              for (int a2 = 0; a2 < D; a2++) {
                int st = F.stride(a2);
                T lov = (fc[a2] == 0 && !((hasn >> (2 * a2)) & 1)) ? (neumann ? mid : -mid) : u[fk - st];
                T hiv = (fc[a2] == F.n(a2) - 1 && !((hasn >> (2 * a2 + 1)) & 1)) ? (neumann ? mid : -mid)
                                                                               : u[fk + st];
                if (KIND == 0) {
                  au += ((hiv - T(2) * mid) + lov) * s_inv[o][a2];
                } else {
                  T cl = cf[fk - st], cm = cf[fk], cu = cf[fk + st];
                  au += ((cu + cm) * (hiv - mid) - (cl + cm) * (mid - lov)) * s_inv[o][a2];
                }
              }
              T r = au * T(-1) + f[fk];
              v += copy >= 0 ? r : r * wD;
            }
      }
    }
    coarse[cp * cps + e] = v;
  }
}

void residual_restrict(const te_restrictor* r, const te_operator* op, int nc, int dtype, const void* f,
                       const void* u, void* coarse, cudaStream_t s) {
  const te_domain* fd = r->fine;
  const Layout &F = fd->lay, &C = r->coarse->lay;
  int threads = C.cs * nc >= 256 ? 256 : 128;
  if (r->even) {
#define TE_RRE(T, K, INV, CO)                                                                                  \
  residual_restrict_even_kernel<T, K><<<C.P, 256, 0, s>>>(F, C, nc, r->by_orth.p, r->copy_of.p, fd->d_nbr_type.p, \
                                                           fd->F, INV, op->neumann, CO, (const T*)u, (const T*)f,  \
                                                           (T*)coarse)
    if (dtype == TE_F64) {
      if (op->kind == 0)
        TE_RRE(double, 0, fd->d_inv.p, nullptr);
      else
        TE_RRE(double, 1, fd->d_inv.p, op->coeffs.p);
    } else {
      if (op->kind == 0)
        TE_RRE(float, 0, fd->d_inv_f.p, nullptr);
      else
        TE_RRE(float, 1, fd->d_inv_f.p, op->coeffs_f.p);
    }
#undef TE_RRE
    count_launch();
    TE_LAUNCH_CHECK();
    return;
  }
  if (dtype == TE_F64) {
    if (op->kind == 0)
      residual_restrict_kernel<double, 0><<<C.P, threads, 0, s>>>(
          F, C, nc, r->child_start.p, r->child.p, r->child_orth.p, fd->d_nbr_type.p, fd->F, fd->d_inv.p,
          op->neumann, nullptr, (const double*)u, (const double*)f, (double*)coarse);
    else
      residual_restrict_kernel<double, 1><<<C.P, threads, 0, s>>>(
          F, C, nc, r->child_start.p, r->child.p, r->child_orth.p, fd->d_nbr_type.p, fd->F, fd->d_inv.p, 0,
          op->coeffs.p, (const double*)u, (const double*)f, (double*)coarse);
  } else {
    if (op->kind == 0)
      residual_restrict_kernel<float, 0><<<C.P, threads, 0, s>>>(
          F, C, nc, r->child_start.p, r->child.p, r->child_orth.p, fd->d_nbr_type.p, fd->F, fd->d_inv_f.p,
          op->neumann, nullptr, (const float*)u, (const float*)f, (float*)coarse);
    else
      residual_restrict_kernel<float, 1><<<C.P, threads, 0, s>>>(
          F, C, nc, r->child_start.p, r->child.p, r->child_orth.p, fd->d_nbr_type.p, fd->F, fd->d_inv_f.p, 0,
          op->coeffs_f.p, (const float*)u, (const float*)f, (float*)coarse);
  }
  count_launch();
  TE_LAUNCH_CHECK();
}

void restrict_level(const te_restrictor* r, int nc, int dtype, const void* fine, void* coarse, cudaStream_t s) {
  const Layout &F = r->fine->lay, &C = r->coarse->lay;
  if (r->complete && !r->extrapolate && F.n0 == C.n0 && F.n1 == C.n1 && F.n2 == C.n2 && F.P > 0) {
    const bool fixed = with_cubic_size(F, [&](auto dim, auto nn) {
      constexpr int DIM = decltype(dim)::value, NN = decltype(nn)::value;
      auto run = [&](auto ntr) {
        constexpr int NTR = decltype(ntr)::value;
        if (dtype == TE_F64)
          restrict_n_kernel<double, DIM, NN, NTR><<<F.P, NTR, 0, s>>>(nc, r->fine_parent.p, r->fine_orth.p,
                                                                     (const double*)fine, (double*)coarse);
        else
          restrict_n_kernel<float, DIM, NN, NTR><<<F.P, NTR, 0, s>>>(nc, r->fine_parent.p, r->fine_orth.p,
                                                                    (const float*)fine, (float*)coarse);
        count_launch();
      };
      // a candidate rewrites the same coarse values, so it can run again for timing
      std::vector<TuneCandidate> cands = {{"threads=256", [&] { run(IntC<256>()); }},
                                          {"threads=128", [&] { run(IntC<128>()); }}};
      char key[96];
      std::snprintf(key, sizeof key, "D=%d n=%d P~2^%d %s nc=%d", DIM, NN, tune_bucket(F.P),
                    dtype == TE_F64 ? "f64" : "f32", nc);
      cands[tune_select("restrict_n", key, cands, s)].run();
    });
    if (fixed) {
      TE_LAUNCH_CHECK();
      return;
    }
  }
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
  if (F.n0 == C.n0 && F.n1 == C.n1 && F.n2 == C.n2 && F.P > 0) {
    const bool fixed = with_cubic_size(F, [&](auto dim, auto nn) {
      constexpr int DIM = decltype(dim)::value, NN = decltype(nn)::value;
      if (dtype == TE_F64)
        interpolate_n_kernel<double, DIM, NN, 1><<<F.P, 256, 0, s>>>(F.P, nc, in->parent.p, in->orth.p,
                                                                    (const double*)coarse, (double*)fine);
      else
        interpolate_n_kernel<float, DIM, NN, 2><<<(F.P + 1) / 2, 256, 0, s>>>(
            F.P, nc, in->parent.p, in->orth.p, (const float*)coarse, (float*)fine);
    });
    if (fixed) {
      count_launch();
      TE_LAUNCH_CHECK();
      return;
    }
  }
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

void residual(const te_domain* d, int nc, int dtype, const void* f, void* r, cudaStream_t s) {
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
    // even patch sizes: one child per coarse cell (by orthant) or a copied patch
    const Layout& FL = fine->lay;
    bool even = FL.n0 % 2 == 0 && FL.n1 % 2 == 0 && FL.n2 % 2 == 0 || (FL.D == 2 && FL.n0 % 2 == 0 && FL.n1 % 2 == 0);
    int NCH = 1 << FL.D;
    std::vector<int> by_orth((size_t)Pc * NCH, -1), copy_of(Pc, -1);
    for (int c = 0; c < Pc && even; c++) {
      auto& ks = kids[c];
      if (ks.size() == 1 && fine->orth_on_parent[ks[0]] < 0) {
        copy_of[c] = ks[0];
        continue;
      }
      for (int p : ks) {
        int o = fine->orth_on_parent[p];
        if (o < 0 || by_orth[(size_t)c * NCH + o] >= 0) even = false;
        else by_orth[(size_t)c * NCH + o] = p;
      }
    }
    r->even = even;
    bool complete = even;
    for (int c = 0; c < Pc && complete; c++)
      if (copy_of[c] < 0)
        for (int o = 0; o < NCH; o++) complete = complete && by_orth[(size_t)c * NCH + o] >= 0;
    r->complete = complete;
    std::vector<int> fpar(fine->lay.P), forth(fine->lay.P);
    for (int p = 0; p < fine->lay.P; p++) {
      fpar[p] = pm[p];
      forth[p] = fine->orth_on_parent[p];
    }
    cudaStream_t s = fine->stream;
    r->fine_parent.upload(fpar, s);
    r->fine_orth.upload(forth, s);
    r->by_orth.upload(by_orth, s);
    r->copy_of.upload(copy_of, s);
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
  return te_cycle_create(levels, num_levels, opts, TE_CYCLE_V, dtype, out);
}

int te_cycle_create(const te_cycle_level* levels, int num_levels, te_cycle_opts opts, int cycle_type, int dtype,
                    te_cycle** out) {
  return guard([&] {
    require(levels && out && num_levels >= 1, "bad arguments");
    require(dtype == TE_F64 || dtype == TE_F32, "bad dtype");
    require(cycle_type == TE_CYCLE_V || cycle_type == TE_CYCLE_W || cycle_type == TE_CYCLE_FMG,
            "Unsupported Cycle type", TE_ERR_UNSUPPORTED);
    require(opts.pre_sweeps >= 0 && opts.post_sweeps >= 0 && opts.mid_sweeps >= 0 && opts.coarse_sweeps >= 0,
            "sweep counts must be >= 0");
    auto c = std::make_unique<te_cycle>();
    c->levels.assign(levels, levels + num_levels);
    c->opts = opts;
    c->type = cycle_type;
    c->dtype = dtype;
    for (int k = 0; k < num_levels; k++) {
      require(levels[k].op && levels[k].smoother, "every level needs an operator and a smoother");
      if (k + 1 < num_levels) require(levels[k].restrictor != nullptr, "missing restrictor");
      if (k > 0) require(levels[k].interpolator != nullptr, "missing interpolator");
    }
    c->stream = levels[0].op->dom->stream;
    static std::atomic<unsigned long long> serials{1};
    c->serial = serials.fetch_add(1);
    const char* ng = getenv("TE_NO_GRAPH");
    c->use_graph = !(ng && ng[0] == '1');
    bool fz = num_levels >= 2 && opts.pre_sweeps == 1 && opts.post_sweeps == 1 && opts.coarse_sweeps == 1 &&
              (cycle_type == TE_CYCLE_V || opts.mid_sweeps == 1);
    const char* nf = getenv("TE_NO_FUSION");
    if (nf && nf[0] == '1') fz = false;
    for (int k = 0; k < num_levels && fz; k++) {
      fz &= levels[k].smoother->kind == 0;
      if (k + 1 < num_levels) fz &= levels[k].restrictor->even && !levels[k].restrictor->extrapolate;
    }
    c->fusable = fz;
    TE_CUDA(cudaStreamCreateWithFlags(&c->cap, cudaStreamNonBlocking));
    TE_CUDA(cudaEventCreateWithFlags(&c->ev_in, cudaEventDisableTiming));
    TE_CUDA(cudaEventCreateWithFlags(&c->ev_out, cudaEventDisableTiming));
    c->ensure(1);
    *out = c.release();
  });
}

int te_cycle_timings(const te_cycle* c, int nc, const void* f, void* u, int max_entries, char* names,
                     double* ms, int* count) {
  return guard([&] {
    require(c && f && u && names && ms && count, "null argument");
    te_cycle* m = const_cast<te_cycle*>(c);
    m->ensure(nc);
    std::vector<te_cycle::Mark> marks;
    cudaStream_t s = m->stream;
    TE_CUDA(cudaStreamSynchronize(s));
    // an FP32 fused cycle is timed the way the mixed-precision solve runs it: FP32 in and out
    const bool f32 = m->dtype == TE_F32 && m->fused();
    if (f32) convert_level(m->dom(0), nc, TE_F32, m->f[0].p, TE_F64, f, s);
    m->marks = &marks;
    try {
      m->mark("start", s);
      if (f32)
        m->body_f32((const float*)m->f[0].p, (float*)m->r[0].p, s);
      else
        m->body(f, u, s);
      m->mark("end", s);
    } catch (...) {
      m->marks = nullptr;
      for (auto& mk : marks) cudaEventDestroy(mk.ev);
      throw;
    }
    m->marks = nullptr;
    if (f32) convert_level(m->dom(0), nc, TE_F64, u, TE_F32, m->r[0].p, s);
    TE_CUDA(cudaStreamSynchronize(s));
    int n = 0;
    for (size_t i = 1; i + 1 < marks.size() && n < max_entries; i++, n++) {
      float t = 0;
      TE_CUDA(cudaEventElapsedTime(&t, marks[i - 1].ev, marks[i].ev));
      ms[n] = t;
      std::strncpy(names + 32 * n, marks[i].name.c_str(), 31);
      names[32 * n + 31] = 0;
    }
    for (auto& mk : marks) cudaEventDestroy(mk.ev);
    *count = n;
  });
}

int te_cycle_destroy(te_cycle* c) {
  delete c;
  return TE_OK;
}

int te_cycle_apply(const te_cycle* c, int nc, const void* f, void* u) {
  return guard([&] {
    require(c && f && u, "null argument");
    te_cycle* m = const_cast<te_cycle*>(c);
    m->ensure(nc);
    m->apply_on(f, u, m->stream);
  });
}

}  // extern "C"
