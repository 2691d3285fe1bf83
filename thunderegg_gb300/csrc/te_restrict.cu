// te_restrict.cu -- the fused residual + restriction of the FP32 V-cycle,
// fine-patch-centric (Cycle::restrict, GMG/Cycle.h:57-65: r = f - A u, then
// LinearRestrictor::restrictToCoarserParent, GMG/LinearRestrictor.h:115-127).
//
// One CTA per fine patch and one thread per 2x2(x2) block of fine cells,
// i.e. per cell of the patch's quadrant in its parent.  The padded patch is
// staged into shared memory with 16-byte loads while the right-hand-side
// values and the neighbour-side ghosts are fetched; its side ghost ring is
// replaced by the ghost filler's values gathered from the neighbours
// (te_ghost_dev.cuh) or, on the physical boundary, by -u (Dirichlet) / +u
// (Neumann).  Each thread then evaluates the star-stencil residual of its
// fine cells from shared memory, in the reference's operation order, sums
// them in z, y, x order with weight 2^-D and writes one coarse cell.  A
// copied patch (its own parent) writes its residual cell by cell.  The
// orthant-0 child (or the copy) zeroes the parent's ghost cells.
//
// Used when every coarse patch is a copy or has all 2^D children, the
// patches are cubic with n = 16, 32 or 64 (2D) or 8 or 16 (3D) and one ghost
// layer; other hierarchies use the coarse-patch-centric kernel in te_fused.cu.

#include <cstdio>
#include <string>
#include <vector>

#include "te_ghost_dev.cuh"
#include "te_gmg.cuh"
#include "te_tune.cuh"

namespace te {

template <int DIM, int NN>
struct RShape {
  static constexpr int SY = NN + 2;
  static constexpr int SZ = DIM == 3 ? SY * SY : 0;
  static constexpr int CS = DIM == 3 ? SY * SY * SY : SY * SY;
  static constexpr int H = NN / 2;
  static constexpr int NT = DIM == 3 ? H * H * H : H * H;  // threads: coarse cells of one quadrant
  static constexpr int NF = DIM == 3 ? NN * NN : NN;       // cells of one side face
};

// CPS: resident CTAs per SM the registers are budgeted for (0: as many as the threads allow);
// BPT: coarse cells (2^D-cell blocks of fine cells) per thread, 1 or 2 (half the threads, twice
// the patches resident per SM); the autotuner picks both, every choice computes the same bits
template <class T, class TF, int KIND, int SCHEME, int DIM, int NN, int CPS = 0, int BPT = 1>
__global__ void __launch_bounds__(RShape<DIM, NN>::NT / BPT, CPS ? CPS : 2048 * BPT / RShape<DIM, NN>::NT)
    vc_restrict_fine_kernel(const int* __restrict__ fparent, const int* __restrict__ forth,
                            const int8_t* __restrict__ fntype, int FS, const T* __restrict__ finv, int neumann,
                            const T* __restrict__ coeff, FaceTable ft, const GSlab* __restrict__ slabs,
                            const GCall* __restrict__ calls, const int* __restrict__ side_code,
                            const SideRec* __restrict__ recs, const T* __restrict__ u,
                            const TF* __restrict__ f, T* __restrict__ coarse) {
  using S = RShape<DIM, NN>;
  constexpr int NB = DIM == 3 ? 8 : 4;  // fine cells per coarse cell
  constexpr int NTB = S::NT / BPT;      // threads
  static_assert(S::NT % BPT == 0, "coarse cells must split evenly over the threads");
  __shared__ __align__(16) T tile[S::CS];
  __shared__ T gbuf[2 * DIM * S::NF];
  const int p = blockIdx.x, t = threadIdx.x;
  const int side0 = DIM == 2 ? 4 : 20;
  const T* up = u + (long long)p * S::CS;
  // this thread's coarse cells t + b NTB: their fine-cell block coordinates
  int bx[BPT], by[BPT], bz[BPT];
#pragma unroll
  for (int b = 0; b < BPT; b++) {
    const int c = t + b * NTB;
    bx[b] = c % S::H;
    by[b] = (c / S::H) % S::H;
    bz[b] = DIM == 3 ? c / (S::H * S::H) : 0;
  }
  // this thread's right-hand-side values, in flight while the patch is staged
  const TF* ff = f + (long long)p * S::CS;
  TF fv[BPT][NB];
#pragma unroll
  for (int b = 0; b < BPT; b++)
#pragma unroll
    for (int q = 0; q < NB; q++) {
      const int x = 2 * bx[b] + (q & 1), y = 2 * by[b] + ((q >> 1) & 1), z = 2 * bz[b] + (q >> 2);
      fv[b][q] = __ldg(ff + (x + 1) + (y + 1) * S::SY + (DIM == 3 ? (z + 1) * S::SZ : 0));
    }
  const int8_t* nt = fntype + (size_t)p * FS + side0;
  // every load is issued before the first shared-memory store: this thread's
  // side codes, its 16-byte pieces of the padded patch, then the neighbour-side
  // ghosts (gathered from the neighbours' values, not this tile)
  constexpr int NG = 2 * DIM * S::NF;
  constexpr int GPT = (NG + NTB - 1) / NTB;
  // 2D (one ghost per thread, a warp's threads on one or two sides): each warp copies the
  // records of its sides (te_ghost_filler::d_side_rec) into shared memory, so a coarse-fine
  // side's values are one dependent load away and no record is held in registers
  constexpr bool REC = DIM == 2 && GPT == 1 && NG % 32 == 0;
  constexpr int SPW = S::NF >= 32 ? 1 : 32 / S::NF;  // sides per gathering warp
  __shared__ SideRec srec[REC ? (NG / 32) * SPW : 1];
  int code[GPT];
  int my_rec = 0;
  if constexpr (REC) {
    code[0] = -1;
    if (t < NG) {
      const int w = t >> 5, l = t & 31, s0 = (w * 32) / S::NF;
      constexpr int WORDS = sizeof(SideRec) / sizeof(int);
      if (l < WORDS * SPW)
        reinterpret_cast<int*>(srec + w * SPW)[l] = reinterpret_cast<const int*>(recs + p * 2 * DIM + s0)[l];
      __syncwarp();
      my_rec = w * SPW + t / S::NF - s0;
      code[0] = srec[my_rec].code;
    }
  } else {
#pragma unroll
    for (int i = 0; i < GPT; i++) {
      const int e = t + i * NTB;
      code[i] = (NG % NTB == 0 || e < NG) ? side_code[p * 2 * DIM + e / S::NF] : -1;
    }
  }
  constexpr bool VEC = (S::CS * sizeof(T)) % 16 == 0;
  constexpr int V = 16 / sizeof(T);
  constexpr int TPT = VEC ? (S::CS / V + NTB - 1) / NTB : 1;
  float4 tv[TPT];
  if (VEC) {
    const float4* src = reinterpret_cast<const float4*>(up);
#pragma unroll
    for (int i = 0; i < TPT; i++) {
      const int e = t + i * NTB;
      if ((S::CS / V) % NTB == 0 || e < S::CS / V) tv[i] = __ldg(src + e);
    }
  }
  const PlainAcc<T> acc{u, (long long)S::CS, 0};
  T gv[GPT];
#pragma unroll
  for (int i = 0; i < GPT; i++) {
    const int e = t + i * NTB;
    if (code[i] != -1) {
      const int s = e / S::NF, r = e % S::NF;
      if constexpr (REC)
        gv[i] = side_ghost_rec<T, SCHEME, DIM, true>(acc, p, s, srec[my_rec], slabs, calls, ft, r % NN, r / NN);
      else
        gv[i] = side_ghost<T, SCHEME>(acc, p, s, code[i], slabs, calls, ft, DIM, r % NN, r / NN);
    }
  }
  // 1. the padded patch (its ghosts are replaced below) and the gathered ghosts
  if (VEC) {
    float4* dst = reinterpret_cast<float4*>(tile);
#pragma unroll
    for (int i = 0; i < TPT; i++) {
      const int e = t + i * NTB;
      if ((S::CS / V) % NTB == 0 || e < S::CS / V) dst[e] = tv[i];
    }
  } else {
    for (int e = t; e < S::CS; e += NTB) tile[e] = up[e];
  }
#pragma unroll
  for (int i = 0; i < GPT; i++)
    if (code[i] != -1) gbuf[t + i * NTB] = gv[i];
  const T i0 = finv[(size_t)p * 6 + (KIND ? 3 : 0)], i1 = finv[(size_t)p * 6 + (KIND ? 3 : 0) + 1];
  const T i2 = DIM == 3 ? finv[(size_t)p * 6 + (KIND ? 3 : 0) + 2] : T(0);
  __syncthreads();
  // 2. the side ghost ring: gathered values, or the boundary condition
  for (int e = t; e < 2 * DIM * S::NF; e += NTB) {
    const int s = e / S::NF, r = e % S::NF;
    const int a = s >> 1, upr = s & 1;
    const int i = r % NN, j = r / NN;
    const int edge = upr ? NN - 1 : 0;
    int x, y, z;
    if (a == 0) {
      x = edge; y = i; z = j;
    } else if (a == 1) {
      x = i; y = edge; z = j;
    } else {
      x = i; y = j; z = edge;
    }
    const int in = (x + 1) + (y + 1) * S::SY + (DIM == 3 ? (z + 1) * S::SZ : 0);
    const int st = a == 0 ? 1 : (a == 1 ? S::SY : S::SZ);
    tile[in + (upr ? st : -st)] = nt[s] >= 0 ? gbuf[e] : (neumann ? tile[in] : -tile[in]);
  }
  __syncthreads();
  // 3. residuals of this thread's fine cells, restricted
  const T* cf = KIND ? coeff + (long long)p * S::CS : nullptr;
  auto resid = [&](int x, int y, int z, TF fval) -> T {
    const int k = (x + 1) + (y + 1) * S::SY + (DIM == 3 ? (z + 1) * S::SZ : 0);
    const T mid = tile[k];
    T au = T(0);
#pragma unroll
    for (int a = 0; a < DIM; a++) {
      const int st = a == 0 ? 1 : (a == 1 ? S::SY : S::SZ);
      const T inv = a == 0 ? i0 : (a == 1 ? i1 : i2);
      const T lov = tile[k - st], hiv = tile[k + st];
      if (KIND == 0) {
        au += ((hiv - T(2) * mid) + lov) * inv;
      } else {
        const T cl = cf[k - st], cm = cf[k], cu = cf[k + st];
        au += ((cu + cm) * (hiv - mid) - (cl + cm) * (mid - lov)) * inv;
      }
    }
    return au * T(-1) + (T)fval;
  };
  const int o = forth[p];
  T* cp = coarse + (long long)fparent[p] * S::CS;
#pragma unroll
  for (int b = 0; b < BPT; b++) {
    if (o >= 0) {
      const T wD = T(1.0 / (1 << DIM));
      T v = T(0);
#pragma unroll
      for (int dz = 0; dz < (DIM == 3 ? 2 : 1); dz++)
#pragma unroll
        for (int dy = 0; dy < 2; dy++)
#pragma unroll
          for (int dx = 0; dx < 2; dx++)
            v += resid(2 * bx[b] + dx, 2 * by[b] + dy, 2 * bz[b] + dz, fv[b][dz * 4 + dy * 2 + dx]) * wD;
      const int cx = bx[b] + ((o & 1) ? S::H : 0), cy = by[b] + ((o & 2) ? S::H : 0);
      const int cz = bz[b] + ((o & 4) ? S::H : 0);
      cp[(cx + 1) + (cy + 1) * S::SY + (DIM == 3 ? (cz + 1) * S::SZ : 0)] = v;
    } else {
#pragma unroll
      for (int dz = 0; dz < (DIM == 3 ? 2 : 1); dz++)
#pragma unroll
        for (int dy = 0; dy < 2; dy++)
#pragma unroll
          for (int dx = 0; dx < 2; dx++) {
            const int x = 2 * bx[b] + dx, y = 2 * by[b] + dy, z = 2 * bz[b] + dz;
            cp[(x + 1) + (y + 1) * S::SY + (DIM == 3 ? (z + 1) * S::SZ : 0)] =
                resid(x, y, z, fv[b][dz * 4 + dy * 2 + dx]);
          }
    }
  }
  if (o <= 0) {
    for (int e = t; e < S::CS; e += NTB) {
      const int x = e % S::SY - 1, r2 = e / S::SY;
      const int y = r2 % S::SY - 1, z = DIM == 3 ? r2 / S::SY - 1 : 0;
      const bool inner = x >= 0 && x < NN && y >= 0 && y < NN && z >= 0 && z < NN;
      if (!inner) cp[e] = T(0);
    }
  }
}

template <class T, class TF, int KIND, int SCHEME, int DIM, int NN>
static void launch_fine(const te_restrictor* r, const te_operator* op, const T* u, const TF* f, T* coarse,
                        cudaStream_t s) {
  using S = RShape<DIM, NN>;
  const te_domain* fd = r->fine;
  const te_ghost_filler* g = op->gf;
  const T* coeff = KIND ? (const T*)op->coeff_ptr(sizeof(T) == 8 ? TE_F64 : TE_F32) : nullptr;
  // candidates: the register budget of as many resident CTAs as the threads allow (the
  // default), of three quarters of them and of half of them (more registers, no spills);
  // and, with two coarse cells per thread, half the threads per CTA at twice the CTAs
  constexpr int C0 = 2048 / S::NT, C1 = C0 * 3 / 4 > 0 ? C0 * 3 / 4 : 1, C2 = C0 / 2 > 0 ? C0 / 2 : 1;
  auto run2 = [&](auto cps, auto bpt) {
    constexpr int BPT = decltype(bpt)::value;
    vc_restrict_fine_kernel<T, TF, KIND, SCHEME, DIM, NN, decltype(cps)::value, BPT>
        <<<fd->lay.P, S::NT / BPT, 0, s>>>(r->fine_parent.p, r->fine_orth.p, fd->d_nbr_type.p, fd->F,
                                          fd->template inv<T>(), op->neumann, coeff, g->faces, g->d_slabs.p,
                                          g->d_calls.p, g->d_side_code.p, g->d_side_rec.p, u, f, coarse);
    count_launch();
  };
  auto run = [&](auto cps) { run2(cps, IntC<1>()); };
  // the kernel writes disjoint parts of the coarse level and reads only u and f, so a
  // candidate can run again for timing
  constexpr int D0 = 2 * C0, D1 = 2 * C1;
  std::vector<TuneCandidate> cands = {{"ctas=" + std::to_string(C0), [&] { run(IntC<C0>()); }},
                                      {"ctas=" + std::to_string(C1), [&] { run(IntC<C1>()); }},
                                      {"ctas=" + std::to_string(C2), [&] { run(IntC<C2>()); }},
                                      {"2 cells/thread ctas=" + std::to_string(D0), [&] { run2(IntC<D0>(), IntC<2>()); }},
                                      {"2 cells/thread ctas=" + std::to_string(D1), [&] { run2(IntC<D1>(), IntC<2>()); }}};
  char key[128];
  std::snprintf(key, sizeof key, "D=%d n=%d P~2^%d %s/%s kind=%d scheme=%d", DIM, NN, tune_bucket(fd->lay.P),
                sizeof(T) == 8 ? "f64" : "f32", sizeof(TF) == 8 ? "f64" : "f32", KIND, SCHEME);
  cands[tune_select("restrict_fine", key, cands, s)].run();
  TE_LAUNCH_CHECK();
}

template <class T, class TF, int KIND, int SCHEME>
static bool try_fine_k(const te_restrictor* r, const te_operator* op, const T* u, const TF* f, T* coarse,
                       cudaStream_t s) {
  const Layout& L = r->fine->lay;
  if (L.D == 2) {
    if constexpr (SCHEME == TE_GHOST_TRILINEAR) {
      return false;
    } else {
      if (L.n0 == 16) launch_fine<T, TF, KIND, SCHEME, 2, 16>(r, op, u, f, coarse, s);
      else if (L.n0 == 32) launch_fine<T, TF, KIND, SCHEME, 2, 32>(r, op, u, f, coarse, s);
      else if (L.n0 == 64) launch_fine<T, TF, KIND, SCHEME, 2, 64>(r, op, u, f, coarse, s);
      else return false;
      return true;
    }
  }
  if constexpr (SCHEME != TE_GHOST_TRILINEAR) {
    return false;
  } else {
    if (L.n0 == 8) launch_fine<T, TF, KIND, SCHEME, 3, 8>(r, op, u, f, coarse, s);
    else if (L.n0 == 16) launch_fine<T, TF, KIND, SCHEME, 3, 16>(r, op, u, f, coarse, s);
    else return false;
    return true;
  }
}

template <class T, class TF>
bool vc_restrict_fine(const te_restrictor* r, const te_operator* op, const T* u, const TF* f, T* coarse,
                      cudaStream_t s) {
  const Layout& L = r->fine->lay;
  if (!r->complete || L.g != 1 || L.n1 != L.n0 || (L.D == 3 && L.n2 != L.n0)) return false;
  const int sc = op->gf->scheme;
  if (op->kind == 0) {
    if (sc == TE_GHOST_BILINEAR) return try_fine_k<T, TF, 0, TE_GHOST_BILINEAR>(r, op, u, f, coarse, s);
    if (sc == TE_GHOST_BIQUADRATIC) return try_fine_k<T, TF, 0, TE_GHOST_BIQUADRATIC>(r, op, u, f, coarse, s);
    return try_fine_k<T, TF, 0, TE_GHOST_TRILINEAR>(r, op, u, f, coarse, s);
  }
  if (sc == TE_GHOST_BILINEAR) return try_fine_k<T, TF, 1, TE_GHOST_BILINEAR>(r, op, u, f, coarse, s);
  if (sc == TE_GHOST_BIQUADRATIC) return try_fine_k<T, TF, 1, TE_GHOST_BIQUADRATIC>(r, op, u, f, coarse, s);
  return try_fine_k<T, TF, 1, TE_GHOST_TRILINEAR>(r, op, u, f, coarse, s);
}

template bool vc_restrict_fine<float, float>(const te_restrictor*, const te_operator*, const float*, const float*,
                                             float*, cudaStream_t);
template bool vc_restrict_fine<float, double>(const te_restrictor*, const te_operator*, const float*,
                                              const double*, float*, cudaStream_t);

}  // namespace te
