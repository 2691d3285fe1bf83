// te_apply.cu -- the star-operator apply with its ghost fill fused into one
// kernel, for cubic patches with one ghost layer whose filler fills faces only
// (PatchOperator::apply, PatchOperator.h:126-143: f.setWithGhost(0),
// fillGhost(u), then per patch enforceBoundaryConditions and applySinglePatch,
// Poisson/StarPatchOperator.h:75-144; VarPoisson/StarPatchOperator.h:75-149).
//
// One CTA per patch.  The padded patch is staged into shared memory with
// 16-byte loads while the side ghosts are gathered from the neighbours with
// the filler's formulas (te_ghost_dev.cuh); the ghost ring -- gathered values,
// or -u / +u on the physical boundary -- goes into the tile and into u itself,
// the side effect the reference's apply has on u's ghost cells.  Every thread
// then evaluates the stencil of its cells from shared memory with the same
// arithmetic as the two-kernel path (stencil_n) and writes f over the whole
// padded patch (0 in the ghost cells).  With rhs the result is rhs - A u on the
// interior (the residual form of operator_residual).  The values, and so the
// bits, are those of ghost_fill followed by apply_n_kernel; only the second
// pass over u and the launch between them are gone.

#include <cstdio>
#include <cstdlib>
#include <string>
#include <vector>

#include "te_ghost_dev.cuh"
#include "te_ops.cuh"
#include "te_tune.cuh"

namespace te {

template <int DIM, int NN>
struct AShape {
  static constexpr int SY = NN + 2;
  static constexpr int SZ = DIM == 3 ? SY * SY : 0;
  static constexpr int CS = DIM == 3 ? SY * SY * SY : SY * SY;
  static constexpr int NF = DIM == 3 ? NN * NN : NN;  // cells of one side face
  static constexpr int NG = 2 * DIM * NF;             // side ghosts of a patch
};

// NT threads per CTA (one patch): 256, or 128 with twice the cells per thread and twice the
// patches resident per SM; the autotuner picks, both compute the same bits
template <class T, int KIND, int SCHEME, int DIM, int NN, int NT>
__global__ void __launch_bounds__(NT, 1536 / NT)
    apply_fused_kernel(const int8_t* __restrict__ ntype, int FS, const T* __restrict__ sp, int neumann,
                       const T* __restrict__ coeff, FaceTable ft, const GSlab* __restrict__ slabs,
                       const GCall* __restrict__ calls, const int* __restrict__ side_code,
                       const SideRec* __restrict__ recs, T* __restrict__ u, T* __restrict__ f,
                       const T* __restrict__ rhs) {
  using S = AShape<DIM, NN>;
  constexpr int NG = S::NG, NF = S::NF;
  constexpr int GPT = (NG + NT - 1) / NT;
  __shared__ __align__(16) T tile[S::CS];
  __shared__ T gbuf[NG];
  const int p = blockIdx.x, t = threadIdx.x;
  constexpr int side0 = DIM == 2 ? 4 : 20;
  T* up = u + (long long)p * S::CS;
  // one ghost per thread (2D n <= 64): each gathering warp copies its sides' records into
  // shared memory; otherwise every ghost's side code is read directly
  constexpr bool REC = DIM == 2 && GPT == 1 && NG % 32 == 0;
  constexpr int SPW = NF >= 32 ? 1 : 32 / NF;
  __shared__ SideRec srec[REC ? (NG / 32) * SPW : 1];
  int code[GPT];
  int my_rec = 0;
  if constexpr (REC) {
    code[0] = -1;
    if (t < NG) {
      const int w = t >> 5, l = t & 31, s0 = (w * 32) / NF;
      constexpr int WORDS = sizeof(SideRec) / sizeof(int);
      if (l < WORDS * SPW)
        reinterpret_cast<int*>(srec + w * SPW)[l] = reinterpret_cast<const int*>(recs + p * 2 * DIM + s0)[l];
      __syncwarp();
      my_rec = w * SPW + t / NF - s0;
      code[0] = srec[my_rec].code;
    }
  } else {
#pragma unroll
    for (int i = 0; i < GPT; i++) {
      const int e = t + i * NT;
      code[i] = (NG % NT == 0 || e < NG) ? side_code[p * 2 * DIM + e / NF] : -1;
    }
  }
  // the padded patch in 16-byte pieces, in flight while the ghosts are gathered
  constexpr bool VEC = (S::CS * sizeof(T)) % 16 == 0;
  constexpr int V = 16 / sizeof(T);
  constexpr int TPT = VEC ? (S::CS / V + NT - 1) / NT : 1;
  float4 tv[TPT];
  if (VEC) {
    const float4* src = reinterpret_cast<const float4*>(up);
#pragma unroll
    for (int i = 0; i < TPT; i++) {
      const int e = t + i * NT;
      if ((S::CS / V) % NT == 0 || e < S::CS / V) tv[i] = __ldg(src + e);
    }
  }
  const PlainAcc<T> acc{u, (long long)S::CS, 0};
  T gv[GPT];
#pragma unroll
  for (int i = 0; i < GPT; i++) {
    const int e = t + i * NT;
    if (code[i] != -1) {
      const int s = e / NF, r = e % NF;
      if constexpr (REC)
        gv[i] = side_ghost_rec<T, SCHEME, DIM, true>(acc, p, s, srec[my_rec], slabs, calls, ft, r % NN, r / NN);
      else
        gv[i] = side_ghost<T, SCHEME>(acc, p, s, code[i], slabs, calls, ft, DIM, r % NN, r / NN);
    }
  }
  if (VEC) {
    float4* dst = reinterpret_cast<float4*>(tile);
#pragma unroll
    for (int i = 0; i < TPT; i++) {
      const int e = t + i * NT;
      if ((S::CS / V) % NT == 0 || e < S::CS / V) dst[e] = tv[i];
    }
  } else {
    for (int e = t; e < S::CS; e += NT) tile[e] = up[e];
  }
#pragma unroll
  for (int i = 0; i < GPT; i++)
    if (code[i] != -1) gbuf[t + i * NT] = gv[i];
  T inv[3];
#pragma unroll
  for (int a = 0; a < 3; a++) inv[a] = a < DIM ? sp[(size_t)p * 6 + (KIND ? 3 : 0) + a] : T(0);
  __syncthreads();
  // the side ghost ring: gathered values (a side with a neighbour), or the boundary condition;
  // into the tile and into u
  const int8_t* nt = ntype + (size_t)p * FS + side0;
  for (int e = t; e < NG; e += NT) {
    const int s = e / NF, r = e % NF;
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
    const T g = nt[s] >= 0 ? gbuf[e] : (neumann ? tile[in] : -tile[in]);
    tile[in + (upr ? st : -st)] = g;
    up[in + (upr ? st : -st)] = g;
  }
  __syncthreads();
  // f over the whole padded patch: the stencil on the interior, 0 in the ghost cells
  const T* cp = KIND ? coeff + (long long)p * S::CS : nullptr;
  T* fp = f + (long long)p * S::CS;
  const T* rp = rhs ? rhs + (long long)p * S::CS : nullptr;
  constexpr int PER = (S::CS + NT - 1) / NT;
#pragma unroll
  for (int q = 0; q < PER; q++) {
    const int k = t + q * NT;
    if (k >= S::CS) break;
    const int x = k % S::SY, y = (k / S::SY) % S::SY, z = DIM == 3 ? k / S::SZ : 1;
    T v = T(0);
    if (x >= 1 && x <= NN && y >= 1 && y <= NN && z >= 1 && z <= NN) {
      v = stencil_n<T, KIND, DIM, S::SY, S::SZ>(tile, cp, k, inv);
      if (rp) v = rp[k] - v;
    }
    fp[k] = v;
  }
}

template <class T, int KIND, int SCHEME>
static bool fused_t(const te_operator* op, T* u, T* f, const T* rhs, cudaStream_t s) {
  const te_domain* d = op->dom;
  const te_ghost_filler* g = op->gf;
  const Layout& L = d->lay;
  const T* coeff = KIND ? (const T*)op->coeff_ptr(sizeof(T) == 8 ? TE_F64 : TE_F32) : nullptr;
  const T* inv = d->template inv<T>();
  const int neumann = KIND ? 0 : op->neumann;
  bool done = false;
  auto run = [&](auto dim, auto nn) {
    constexpr int DIM = decltype(dim)::value, NN = decltype(nn)::value;
    auto launch = [&](auto nt) {
      constexpr int NT = decltype(nt)::value;
      apply_fused_kernel<T, KIND, SCHEME, DIM, NN, NT><<<L.P, NT, 0, s>>>(
          d->d_nbr_type.p, d->F, inv, neumann, coeff, g->faces, g->d_slabs.p, g->d_calls.p, g->d_side_code.p,
          g->d_side_rec.p, u, f, rhs);
      count_launch();
    };
    // re-running a candidate for timing writes the same f and the same ghosts of u
    std::vector<TuneCandidate> cands = {{"threads=256", [&] { launch(IntC<256>()); }},
                                        {"threads=128", [&] { launch(IntC<128>()); }}};
    char key[128];
    std::snprintf(key, sizeof key, "D=%d n=%d P~2^%d %s kind=%d scheme=%d rhs=%d", DIM, NN, tune_bucket(L.P),
                  sizeof(T) == 8 ? "f64" : "f32", KIND, SCHEME, rhs ? 1 : 0);
    cands[tune_select("apply_fused", key, cands, s)].run();
    done = true;
  };
  if (L.D == 2 && SCHEME != TE_GHOST_TRILINEAR) {
    if (L.n0 == 16) run(IntC<2>(), IntC<16>());
    else if (L.n0 == 32) run(IntC<2>(), IntC<32>());
    else if (L.n0 == 64) run(IntC<2>(), IntC<64>());
  } else if (L.D == 3 && SCHEME == TE_GHOST_TRILINEAR) {
    if (L.n0 == 8) run(IntC<3>(), IntC<8>());
    else if (L.n0 == 16) run(IntC<3>(), IntC<16>());
  }
  if (done) TE_LAUNCH_CHECK();
  return done;
}

// f = A u (rhs null) or f = rhs - A u, with u's side ghosts filled as a side effect, in one
// kernel; false (nothing ran) where the level does not qualify: one component, cubic patches of
// n = 16, 32, 64 (2D) or 8, 16 (3D) with one ghost layer, a filler of faces only
template <class T>
bool operator_apply_fused(const te_operator* op, int nc, T* u, T* f, const T* rhs, cudaStream_t s) {
  const Layout& L = op->dom->lay;
  const te_ghost_filler* g = op->gf;
  if (nc != 1 || L.g != 1 || L.n1 != L.n0 || (L.D == 3 && L.n2 != L.n0) || g->fill_type != TE_FILL_FACES ||
      g->other_slabs || generic_level_kernels())
    return false;
  const char* e = std::getenv("TE_NO_FUSED_APPLY");
  if (e && e[0] == '1') return false;
  if (op->kind == 0) {
    if (g->scheme == TE_GHOST_BILINEAR) return fused_t<T, 0, TE_GHOST_BILINEAR>(op, u, f, rhs, s);
    if (g->scheme == TE_GHOST_BIQUADRATIC) return fused_t<T, 0, TE_GHOST_BIQUADRATIC>(op, u, f, rhs, s);
    return fused_t<T, 0, TE_GHOST_TRILINEAR>(op, u, f, rhs, s);
  }
  if (g->scheme == TE_GHOST_BILINEAR) return fused_t<T, 1, TE_GHOST_BILINEAR>(op, u, f, rhs, s);
  if (g->scheme == TE_GHOST_BIQUADRATIC) return fused_t<T, 1, TE_GHOST_BIQUADRATIC>(op, u, f, rhs, s);
  return fused_t<T, 1, TE_GHOST_TRILINEAR>(op, u, f, rhs, s);
}

template bool operator_apply_fused<double>(const te_operator*, int, double*, double*, const double*, cudaStream_t);
template bool operator_apply_fused<float>(const te_operator*, int, float*, float*, const float*, cudaStream_t);

}  // namespace te
