// te_krylov.cu -- the outer Iterative::BiCGStab (Iterative/BiCGStab.h:111-203) in FP64,
// for one solve or a batch of independent solves sharing one level buffer.
//
// The reference keeps alpha, omega, rho and beta on the host and reduces with
// MPI_Allreduce after every dot product.  Here every solve's scalars live in
// device memory: each vector update is fused with the dot products that
// follow it, and the last block of each solve's reduction finalises that
// solve's scalars.  The host reads all scalars back once per iteration to test
// convergence and breakdown per solve; converged solves are masked out of the
// updates.  One iteration (two preconditioner applications, two operator
// applications, five fused kernels) is captured into a CUDA graph and replayed.
//
// A batch is a union of solves whose finest-level patches are contiguous
// ranges [offs[b], offs[b+1]).  A solve's reductions are split into a fixed
// number of chunks that depends only on its own patch count, and summed in a
// fixed order, so a solve gives bit-identical results alone or in any batch.
//
// Arithmetic per element follows the reference's operation order:
//   s = r + ap*(-alpha); x += mp*alpha + ms*omega; r += ap*(-alpha) + as*(-omega);
//   p += ap*(-omega); p = p*beta + r.

#include <cmath>
#include <cstdlib>
#include <cstring>
#include <set>
#include <string>
#include <algorithm>
#include <tuple>

#include "te_df64.cuh"
#include "te_ghost_dev.cuh"
#include "te_gmg.cuh"

namespace te {

enum Slot {
  S_RHO = 0,
  S_R0,
  S_RHAT_AP,
  S_ALPHA,
  S_SS,
  S_AS_S,
  S_AS_AS,
  S_OMEGA,
  S_RR,
  S_R_RHAT,
  S_BETA,
  S_DONE,
  S_BB,
  S_XNZ = 14,   // the solve's x has a nonzero value on entry
  S_TRUE = 15,  // float-float loop: ||b - A x||^2 in FP64 after convergence
  S_NSLOTS = 16
};

constexpr int KT = 256;
// At most 256 blocks per solve: a 1,444-patch solve then gives each block about 5.6 patches (22
// cells a thread), so the block's reduction tail is spread over more cells; a served batch of
// 16 such solves ran 16.20 ms with 1,024 blocks per solve, 15.95 ms with 256 and 16.15 ms with 128.
constexpr int MAX_CHUNKS = 256;

// chunks of one solve's reductions: a function of its own patch count only
inline int chunks_for(int patches) { return patches < MAX_CHUNKS ? patches : MAX_CHUNKS; }

struct Batch {
  int B;              // solves
  const int* offs;    // [B+1] patch ranges
  const int* nch;     // [B] chunks of each solve
  const int* active;  // [B] 1 while the solve iterates
};

// Interior cells threadIdx.x, + blockDim.x, ... of a patch (x fastest) walked
// without divisions: the start and the stride are decomposed once into cell
// coordinates, and each step adds them with at most one carry per axis (the
// stride's coordinate on each axis is below that axis' size).
struct InteriorWalk {
  int x0, y0, z0, dx, dy, dz;
  __device__ __forceinline__ explicit InteriorWalk(const Layout& L) {
    x0 = threadIdx.x % L.n0;
    y0 = (threadIdx.x / L.n0) % L.n1;
    z0 = threadIdx.x / (L.n0 * L.n1);
    dx = blockDim.x % L.n0;
    dy = (blockDim.x / L.n0) % L.n1;
    dz = blockDim.x / (L.n0 * L.n1);
  }
};

// iterate the interior cells of chunk `ch` of solve `b`
#define TE_CHUNK_LOOP(BT, L, nc, b, ch, k, body)                                       \
  {                                                                                    \
    const int _N = (L).interior();                                                     \
    const long long _ps = (L).pstride(nc);                                             \
    const InteriorWalk _w(L);                                                          \
    for (int _p = (BT).offs[b] + (ch); _p < (BT).offs[(b) + 1]; _p += (BT).nch[b])     \
      for (int _c = 0; _c < (nc); _c++) {                                              \
        const long long _base = _p * _ps + (long long)_c * (L).cs;                     \
        int _x = _w.x0, _y = _w.y0, _z = _w.z0;                                        \
        _Pragma("unroll 4") for (int _e = threadIdx.x; _e < _N; _e += blockDim.x) {    \
          const long long k = _base + (L).at(_x, _y, _z);                              \
          body;                                                                        \
          _x += _w.dx;                                                                 \
          _y += _w.dy;                                                                 \
          _z += _w.dz;                                                                 \
          if (_x >= (L).n0) {                                                          \
            _x -= (L).n0;                                                              \
            _y++;                                                                      \
          }                                                                            \
          if (_y >= (L).n1) {                                                          \
            _y -= (L).n1;                                                              \
            _z++;                                                                      \
          }                                                                            \
        }                                                                              \
      }                                                                                \
  }

// Per-block sums -> part; the last block of solve b sums its chunks in a
// fixed order into S[b][slot0 ...] and finalises scalars.
// finalize_kind: 1 alpha, 2 omega, 3 beta + rho commit, 4 initial r0, 5 early-exit test
// blk: this block's sums, valid on thread 0
template <int NV>
__device__ void k_reduce_blk(const double (&blk)[NV], const Batch& bt, int b, int ch, double* part,
                             unsigned int* counter, double* S, int slot0, int finalize_kind, double tol) {
  __shared__ double fin[NV][KT];
  __shared__ bool last;
  const int CH = bt.nch[b];
  if (threadIdx.x == 0) {
    for (int i = 0; i < NV; i++) part[((size_t)i * bt.B + b) * MAX_CHUNKS + ch] = blk[i];
    __threadfence();
    unsigned int done = atomicAdd(&counter[b], 1u);
    last = done == (unsigned)(CH - 1);
  }
  __syncthreads();
  if (!last) return;
  __threadfence();
  for (int i = 0; i < NV; i++) {
    double s = 0;
    for (int c = threadIdx.x; c < CH; c += blockDim.x) s += __ldcg(&part[((size_t)i * bt.B + b) * MAX_CHUNKS + c]);
    fin[i][threadIdx.x] = s;
  }
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if ((int)threadIdx.x < w)
      for (int i = 0; i < NV; i++) fin[i][threadIdx.x] += fin[i][threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    double* Sb = S + (size_t)b * S_NSLOTS;
    double tot[NV];
    for (int i = 0; i < NV; i++) {
      tot[i] = fin[i][0];
      Sb[slot0 + i] = tot[i];
    }
    if (finalize_kind == 1) {  // alpha = rho / (rhat . ap)
      Sb[S_ALPHA] = Sb[S_RHO] / tot[0];
    } else if (finalize_kind == 2) {  // omega = (as . s) / (as . as)
      Sb[S_OMEGA] = tot[0] / tot[1];
    } else if (finalize_kind == 3) {  // beta = rho_new * alpha / (rho * omega); rho = rho_new
      if (Sb[S_DONE] == 0.0) {
        Sb[S_BETA] = Sb[S_R_RHAT] * Sb[S_ALPHA] / (Sb[S_RHO] * Sb[S_OMEGA]);
        Sb[S_RHO] = Sb[S_R_RHAT];
      }
    } else if (finalize_kind == 5) {  // ||s|| / ||b|| <= tol (BiCGStab.h:162)
      Sb[S_DONE] = sqrt(tot[0]) / Sb[S_R0] <= tol ? 1.0 : 0.0;
    }
    counter[b] = 0u;
  }
}

// Per-patch partial sums (one block per patch p of solve b): the last block of
// the solve sums its patches' partials in patch order and finalises.  The
// order depends only on the solve's own patches, not on the batch.
template <int NV>
__device__ void kp_reduce(const double (&blk)[NV], int B, int b, int first, int count, int p, double* part,
                          int P, unsigned int* counter, double* S, int slot0, int finalize_kind) {
  __shared__ double fin[NV][KT];
  __shared__ bool last;
  if (threadIdx.x == 0) {
    for (int i = 0; i < NV; i++) part[(size_t)i * P + p] = blk[i];
    __threadfence();
    unsigned int done = atomicAdd(&counter[b], 1u);
    last = done == (unsigned)(count - 1);
  }
  __syncthreads();
  if (!last) return;
  __threadfence();
  for (int i = 0; i < NV; i++) {
    double s = 0;
    for (int c = threadIdx.x; c < count; c += blockDim.x) s += __ldcg(&part[(size_t)i * P + first + c]);
    fin[i][threadIdx.x] = s;
  }
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if ((int)threadIdx.x < w)
      for (int i = 0; i < NV; i++) fin[i][threadIdx.x] += fin[i][threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    double* Sb = S + (size_t)b * S_NSLOTS;
    double tot[NV];
    for (int i = 0; i < NV; i++) {
      tot[i] = fin[i][0];
      Sb[slot0 + i] = tot[i];
    }
    if (finalize_kind == 1) Sb[S_ALPHA] = Sb[S_RHO] / tot[0];  // alpha = rho / (rhat . ap)
    else if (finalize_kind == 2) Sb[S_OMEGA] = tot[0] / tot[1];  // omega = (as . s) / (as . as)
    counter[b] = 0u;
  }
}

template <int NV>
__device__ void k_reduce(double (&v)[NV], const Batch& bt, int b, int ch, double* part, unsigned int* counter,
                         double* S, int slot0, int finalize_kind, double tol) {
  __shared__ double red[NV][KT / 32];
#pragma unroll
  for (int i = 0; i < NV; i++) {
    double x = v[i];
    for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
    if ((threadIdx.x & 31) == 0) red[i][threadIdx.x >> 5] = x;
  }
  __syncthreads();
  double blk[NV];
  if (threadIdx.x == 0)
    for (int i = 0; i < NV; i++) {
      double s = 0;
      for (int w = 0; w < (int)(blockDim.x >> 5); w++) s += red[i][w];
      blk[i] = s;
    }
  k_reduce_blk<NV>(blk, bt, b, ch, part, counter, S, slot0, finalize_kind, tol);
}

#define TE_BLOCK_SOLVE(bt)                  \
  const int b = blockIdx.x / MAX_CHUNKS;    \
  const int ch = blockIdx.x % MAX_CHUNKS;   \
  if (ch >= (bt).nch[b] || !(bt).active[b]) return;

// dots of up to three pairs into S[b][slot0 ...], walking the cells with a Cells
// walker (ChunkCells, or CubeCells for cubic patches) four at a time, their loads
// issued before their products are summed in visit order
template <int NV, class Cells>
__global__ void __launch_bounds__(KT) k_dots_c(Layout L, int nc, Batch bt, const double* a0, const double* b0,
                                               const double* a1, const double* b1, const double* a2,
                                               const double* b2, double* part, unsigned int* counter, double* S,
                                               int slot0, int fin) {
  TE_BLOCK_SOLVE(bt);
  double v[NV];
  for (int i = 0; i < NV; i++) v[i] = 0;
  const double* as[3] = {a0, a1, a2};
  const double* bs[3] = {b0, b1, b2};
  Cells cells(bt, L, nc, b, ch);
  long long k[4];
  while (cells.next(k)) {
    double x[NV][4], y[NV][4];
#pragma unroll
    for (int u = 0; u < 4; u++)
      if (k[u] >= 0)
#pragma unroll
        for (int i = 0; i < NV; i++) {
          x[i][u] = __ldg(as[i] + k[u]);
          y[i][u] = __ldg(bs[i] + k[u]);
        }
#pragma unroll
    for (int u = 0; u < 4; u++)
      if (k[u] >= 0)
#pragma unroll
        for (int i = 0; i < NV; i++) v[i] += x[i][u] * y[i][u];
  }
  k_reduce<NV>(v, bt, b, ch, part, counter, S, slot0, fin, 0);
}

// s = r + ap * (-alpha);  S_SS = s . s; S_DONE = (||s|| / ||b|| <= tol)
__global__ void __launch_bounds__(KT) k_s(Layout L, int nc, Batch bt, double tol, const double* r, const double* ap,
                                          double* s, double* part, unsigned int* counter, double* S) {
  TE_BLOCK_SOLVE(bt);
  const double alpha = S[(size_t)b * S_NSLOTS + S_ALPHA];
  double v[1] = {0};
  TE_CHUNK_LOOP(bt, L, nc, b, ch, k, {
    double sv = r[k];
    sv += ap[k] * -alpha;
    s[k] = sv;
    v[0] += sv * sv;
  });
  k_reduce<1>(v, bt, b, ch, part, counter, S, S_SS, 5, tol);
}

// early exit when ||s|| / ||b|| <= tol: x += dir * alpha (reference: dir = p);
// otherwise x += mp*alpha + ms*omega, r += ap*(-alpha) + as*(-omega) and the
// dots r.r, r.rhat; the last block forms beta and commits rho.
__global__ void __launch_bounds__(KT) k_xr(Layout L, int nc, Batch bt, double* x, double* r, const double* mp,
                                           const double* ms, const double* ap, const double* as, const double* rhat,
                                           const double* dir, double* part, unsigned int* counter, double* S) {
  TE_BLOCK_SOLVE(bt);
  const double* Sb = S + (size_t)b * S_NSLOTS;
  const double alpha = Sb[S_ALPHA], omega = Sb[S_OMEGA];
  const bool done = Sb[S_DONE] != 0.0;
  double v[2] = {0, 0};
  TE_CHUNK_LOOP(bt, L, nc, b, ch, k, {
    if (done) {
      x[k] += dir[k] * alpha;
    } else {
      x[k] += mp[k] * alpha + ms[k] * omega;
      double rv = r[k];
      rv += ap[k] * -alpha + as[k] * -omega;
      r[k] = rv;
      v[0] += rv * rv;
      v[1] += rv * rhat[k];
    }
  });
  k_reduce<2>(v, bt, b, ch, part, counter, S, S_RR, 3, 0);
}

// p += ap*(-omega); p = p*beta + r
__global__ void __launch_bounds__(KT) k_p(Layout L, int nc, Batch bt, double* p, const double* ap, const double* r,
                                          const double* S) {
  TE_BLOCK_SOLVE(bt);
  const double* Sb = S + (size_t)b * S_NSLOTS;
  if (Sb[S_DONE] != 0.0) return;
  const double omega = Sb[S_OMEGA], beta = Sb[S_BETA];
  TE_CHUNK_LOOP(bt, L, nc, b, ch, k, {
    double pv = p[k];
    pv += ap[k] * -omega;
    p[k] = pv * beta + r[k];
  });
}

// ---------------------------------------------------------------------------
// Float-float outer loop (mixed precision: FP32 V-cycle preconditioner).
// The same recurrences and operation order as the FP64 kernels above, with
// every Krylov vector a float-float pair stored as hi and lo FP32 arrays and
// the preconditioner results mp, ms plain FP32 (they are FP32 values).  The
// iterate is split: x stays FP64 and the loop accumulates a float-float
// correction dx, folded into x (x += dx, dx = 0, in FP64) at every true-
// residual check.  A float-float x re-rounded to 48 bits at each restart
// stalls the true residual near 1e-10 on meshes of 2048^2 cells; after the
// first check dx only carries the small correction, so 48 bits suffice, and
// the loop itself needs no FP64 arithmetic.
// ---------------------------------------------------------------------------
struct DV {
  float* hi;
  float* lo;
};
struct CV {
  const float* hi;
  const float* lo;  // null: the vector is FP32 (lo = 0)
};
__host__ __device__ __forceinline__ CV as_cv(const DV& v) { return CV{v.hi, v.lo}; }
__device__ __forceinline__ df64 ldv(const CV& v, long long k) { return df64(v.hi[k], v.lo ? v.lo[k] : 0.f); }
__device__ __forceinline__ void stv(const DV& v, long long k, df64 x) {
  v.hi[k] = x.hi;
  v.lo[k] = x.lo;
}

// The interior cells of chunk `ch` of solve `b` (the cells TE_CHUNK_LOOP
// visits, in the same order per thread), U at a time: next() fills k[0..U-1]
// with padded offsets (-1 past the end), so a kernel can load the operands of
// U cells before it computes and stores any of them.
template <int U>
struct ChunkCells {
  const Layout& L;
  const int nc, N, pend, pstep;
  const long long ps;
  const InteriorWalk w;
  int p, c, e, x, y, z;
  long long base;
  __device__ __forceinline__ ChunkCells(const Batch& bt, const Layout& L_, int nc_, int b, int ch)
      : L(L_), nc(nc_), N(L_.interior()), pend(bt.offs[b + 1]), pstep(bt.nch[b]), ps(L_.pstride(nc_)), w(L_) {
    p = bt.offs[b] + ch;
    c = 0;
    restart();
  }
  __device__ __forceinline__ void restart() {
    e = threadIdx.x;
    x = w.x0;
    y = w.y0;
    z = w.z0;
    base = (long long)p * ps + (long long)c * L.cs;
  }
  __device__ __forceinline__ bool next(long long (&k)[U]) {
#pragma unroll
    for (int r = 0; r < U; r++) {
      while (p < pend && e >= N) {  // this patch-component is done: the next one
        if (++c == nc) {
          c = 0;
          p += pstep;
        }
        restart();
      }
      if (p >= pend) {
        k[r] = -1;
        continue;
      }
      k[r] = base + L.at(x, y, z);
      e += blockDim.x;
      x += w.dx;
      y += w.dy;
      z += w.dz;
      if (x >= L.n0) {
        x -= L.n0;
        y++;
      }
      if (y >= L.n1) {
        y -= L.n1;
        z++;
      }
    }
    return k[0] >= 0;
  }
};

// ChunkCells for cubic patches of NN cells with one ghost layer whose interior is a
// multiple of KT cells (2D n = 16, 32, 64; 3D n = 8, 16), launched with KT threads:
// the same cells in the same order per thread, each at its thread's offset in the
// patch plus a compile-time step (thread t's j-th cell of a patch is e = t + KT j).
template <int DIM, int NN, int U>
struct CubeCells {
  static constexpr int SY = NN + 2, SZ = DIM == 3 ? SY * SY : 0;
  static constexpr int N = DIM == 3 ? NN * NN * NN : NN * NN;
  static constexpr int CPT = N / KT;
  static constexpr int STEP = DIM == 2 ? (KT / NN) * SY : (KT / (NN * NN)) * SZ;
  static_assert(N % KT == 0 && KT % NN == 0 && (DIM == 2 || KT % (NN * NN) == 0), "cells must tile the threads");
  const int nc, pend, pstep, cs;
  const long long ps;
  const int toff;
  int p, c, j;
  long long base;
  __device__ __forceinline__ CubeCells(const Batch& bt, const Layout& L, int nc_, int b, int ch)
      : nc(nc_), pend(bt.offs[b + 1]), pstep(bt.nch[b]), cs(L.cs), ps(L.pstride(nc_)),
        toff((int)(threadIdx.x % NN + 1) + (int)((threadIdx.x / NN) % NN + 1) * SY +
             (DIM == 3 ? (int)(threadIdx.x / (NN * NN) + 1) * SZ : 0)) {
    p = bt.offs[b] + ch;
    c = 0;
    j = 0;
    base = (long long)p * ps + toff;
  }
  __device__ __forceinline__ bool next(long long (&k)[U]) {
#pragma unroll
    for (int r = 0; r < U; r++) {
      if (j == CPT) {
        j = 0;
        if (++c == nc) {
          c = 0;
          p += pstep;
        }
        base = (long long)p * ps + (long long)c * cs + toff;
      }
      k[r] = p < pend ? base + (long long)j * STEP : -1;
      j++;
    }
    return k[0] >= 0;
  }
};

// calls fn(CubeCells<...>) for the layouts CubeCells covers, else fn(ChunkCells)
template <int U, class Fn>
void with_cells(const Layout& L, Fn&& fn) {
  bool done = false;
  with_cubic_size(L, [&](auto dim, auto nn) {
    constexpr int DIM = decltype(dim)::value, NN = decltype(nn)::value;
    constexpr int N = DIM == 3 ? NN * NN * NN : NN * NN;
    if constexpr (N % KT == 0 && KT % NN == 0 && (DIM == 2 || KT % (NN * NN) == 0)) {
      fn((CubeCells<DIM, NN, U>*)nullptr);
      done = true;
    }
  });
  if (!done) fn((ChunkCells<U>*)nullptr);
}

// block sums of float-float accumulators (the FP64 pipe stays idle until the last block)
template <int NV>
__device__ void kd_reduce(df64 (&v)[NV], const Batch& bt, int b, int ch, double* part, unsigned int* counter,
                          double* S, int slot0, int finalize_kind, double tol) {
  __shared__ df64 red[NV][KT / 32];
#pragma unroll
  for (int i = 0; i < NV; i++) {
    df64 x = v[i];
    for (int o = 16; o > 0; o >>= 1) x += df_shfl_down(x, o);
    if ((threadIdx.x & 31) == 0) red[i][threadIdx.x >> 5] = x;
  }
  __syncthreads();
  double blk[NV];
  if (threadIdx.x == 0)
    for (int i = 0; i < NV; i++) {
      df64 t = red[i][0];
      for (int w = 1; w < (int)(blockDim.x >> 5); w++) t += red[i][w];
      blk[i] = df_to_double(t);
    }
  k_reduce_blk<NV>(blk, bt, b, ch, part, counter, S, slot0, finalize_kind, tol);
}

// the solve's scalars as float-float numbers, split once per block
__device__ __forceinline__ void kd_scalars(const double* Sb, df64* sc, int n, int s0, int s1) {
  if (threadIdx.x < n) sc[threadIdx.x] = df64(Sb[threadIdx.x == 0 ? s0 : s1]);
  __syncthreads();
}

template <int NV>
__global__ void __launch_bounds__(KT) kd_dots(Layout L, int nc, Batch bt, CV a0, CV b0, CV a1, CV b1, CV a2, CV b2,
                                              double* part, unsigned int* counter, double* S, int slot0, int fin) {
  TE_BLOCK_SOLVE(bt);
  dot2 d[NV];
  TE_CHUNK_LOOP(bt, L, nc, b, ch, k, {
    d[0].add(ldv(a0, k), ldv(b0, k));
    if (NV > 1) d[1].add(ldv(a1, k), ldv(b1, k));
    if (NV > 2) d[2].add(ldv(a2, k), ldv(b2, k));
  });
  df64 v[NV];
  for (int i = 0; i < NV; i++) v[i] = d[i].value();
  kd_reduce<NV>(v, bt, b, ch, part, counter, S, slot0, fin, 0);
}

template <class Cells>
__global__ void __launch_bounds__(KT, 8) kd_s(Layout L, int nc, Batch bt, double tol, CV r, CV ap, DV s, double* part,
                                           unsigned int* counter, double* S) {
  TE_BLOCK_SOLVE(bt);
  __shared__ df64 sc[1];
  kd_scalars(S + (size_t)b * S_NSLOTS, sc, 1, S_ALPHA, S_ALPHA);
  const df64 nalpha = -sc[0];
  dot2 d;
  Cells cells(bt, L, nc, b, ch);
  long long k[2];
  while (cells.next(k)) {
    df64 rv[2], av[2];
#pragma unroll
    for (int u = 0; u < 2; u++)
      if (k[u] >= 0) {
        rv[u] = ldv(r, k[u]);
        av[u] = ldv(ap, k[u]);
      }
#pragma unroll
    for (int u = 0; u < 2; u++)
      if (k[u] >= 0) {
        const df64 sv = rv[u] + av[u] * nalpha;
        stv(s, k[u], sv);
        d.add(sv, sv);
      }
  }
  df64 v[1] = {d.value()};
  kd_reduce<1>(v, bt, b, ch, part, counter, S, S_SS, 5, tol);
}

template <class Cells>
__global__ void __launch_bounds__(KT, 4) kd_xr(Layout L, int nc, Batch bt, DV dx, DV r, const float* mp,
                                            const float* ms,
                                            CV ap, CV as, CV rhat, CV dir, double* part, unsigned int* counter,
                                            double* S) {
  TE_BLOCK_SOLVE(bt);
  const double* Sb = S + (size_t)b * S_NSLOTS;
  __shared__ df64 sc[2];
  kd_scalars(Sb, sc, 2, S_ALPHA, S_OMEGA);
  const df64 alpha = sc[0], omega = sc[1];
  const df64 nalpha = -alpha, nomega = -omega;
  const bool done = Sb[S_DONE] != 0.0;
  dot2 d0, d1;
  const CV xc = as_cv(dx), rc = as_cv(r);
  if (done) {
    TE_CHUNK_LOOP(bt, L, nc, b, ch, k, { stv(dx, k, ldv(xc, k) + ldv(dir, k) * alpha); });
  } else {
    Cells cells(bt, L, nc, b, ch);
    long long k[2];
    while (cells.next(k)) {
      df64 xv[2], rv[2], av[2], sv[2], hv[2];
      float mv[2], nv[2];
#pragma unroll
      for (int u = 0; u < 2; u++)
        if (k[u] >= 0) {
          xv[u] = ldv(xc, k[u]);
          mv[u] = mp[k[u]];
          nv[u] = ms[k[u]];
          rv[u] = ldv(rc, k[u]);
          av[u] = ldv(ap, k[u]);
          sv[u] = ldv(as, k[u]);
          hv[u] = ldv(rhat, k[u]);
        }
#pragma unroll
      for (int u = 0; u < 2; u++)
        if (k[u] >= 0) {
          stv(dx, k[u], xv[u] + df_sum2(alpha, mv[u], omega, nv[u]));
          const df64 rn = rv[u] + df_sum2(av[u], nalpha, sv[u], nomega);
          stv(r, k[u], rn);
          d0.add(rn, rn);
          d1.add(rn, hv[u]);
        }
    }
  }
  df64 v[2] = {d0.value(), d1.value()};
  kd_reduce<2>(v, bt, b, ch, part, counter, S, S_RR, 3, 0);
}

template <class Cells>
__global__ void __launch_bounds__(KT) kd_p(Layout L, int nc, Batch bt, DV p, CV ap, CV r, const double* S) {
  TE_BLOCK_SOLVE(bt);
  const double* Sb = S + (size_t)b * S_NSLOTS;
  if (Sb[S_DONE] != 0.0) return;
  __shared__ df64 sc[2];
  kd_scalars(Sb, sc, 2, S_OMEGA, S_BETA);
  const df64 nomega = -sc[0], beta = sc[1];
  const CV pc = as_cv(p);
  Cells cells(bt, L, nc, b, ch);
  long long k[2];
  while (cells.next(k)) {
    df64 pv[2], av[2], rv[2];
#pragma unroll
    for (int u = 0; u < 2; u++)
      if (k[u] >= 0) {
        pv[u] = ldv(pc, k[u]);
        av[u] = ldv(ap, k[u]);
        rv[u] = ldv(r, k[u]);
      }
#pragma unroll
    for (int u = 0; u < 2; u++)
      if (k[u] >= 0) stv(p, k[u], (pv[u] + av[u] * nomega) * beta + rv[u]);
  }
}

// Whole-vector conversions: each thread takes CONV_U elements per round and
// loads them all before converting and storing any.
constexpr int CONV_U = 4;
// one split into three vectors (resid, rhat and p start equal)
__global__ void kd_split3(const double* __restrict__ src, DV d0, DV d1, DV d2, long long n) {
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long i0 = blockIdx.x * (long long)blockDim.x + threadIdx.x; i0 < n; i0 += CONV_U * stride) {
    double v[CONV_U];
#pragma unroll
    for (int u = 0; u < CONV_U; u++) v[u] = i0 + u * stride < n ? src[i0 + u * stride] : 0.0;
#pragma unroll
    for (int u = 0; u < CONV_U; u++) {
      const long long i = i0 + u * stride;
      if (i >= n) continue;
      const df64 s = df_split_bits(v[u]);
      stv(d0, i, s);
      stv(d1, i, s);
      stv(d2, i, s);
    }
  }
}

// x += dx in FP64, then dx = 0: the loop's float-float correction folded into the FP64 iterate
// (dx's parts widened by integer operations: two FP64 additions per element, no conversions)
__global__ void kd_fold(DV dx, double* __restrict__ x, long long n) {
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long i0 = blockIdx.x * (long long)blockDim.x + threadIdx.x; i0 < n; i0 += CONV_U * stride) {
    df64 d[CONV_U];
    double v[CONV_U];
#pragma unroll
    for (int u = 0; u < CONV_U; u++) {
      const long long i = i0 + u * stride;
      d[u] = i < n ? ldv(as_cv(dx), i) : df64(0.f, 0.f);
      v[u] = i < n ? x[i] : 0.0;
    }
#pragma unroll
    for (int u = 0; u < CONV_U; u++) {
      const long long i = i0 + u * stride;
      if (i >= n) continue;
      x[i] = v[u] + df_to_double_bits(d[u]);
      stv(dx, i, df64(0.f, 0.f));
    }
  }
}

// FP32 values of a level buffer, read as float-float numbers
struct F32Acc {
  const float* u;
  long long ps;
  __device__ __forceinline__ df64 operator()(int q, int idx) const { return df64(u[q * ps + idx], 0.f); }
};

// exact (hi - 2 mid) + lo of three FP32 values, rounded once to float-float
__device__ __forceinline__ df64 df_second_difference(float hi, float mid, float lo) {
  const df64 a = two_sum(hi, -2.f * mid);
  const df64 b = two_sum(a.hi, lo);
  return fast_two_sum(b.hi, __fadd_rn(a.lo, b.lo));
}

// f = A u for an FP32 level buffer u (ghosts not filled), in float-float:
// the side ghosts of every face with a neighbour are gathered with the ghost
// filler's formulas (te_ghost_dev.cuh) into shared memory, physical-boundary
// ghosts are -u (Dirichlet) or +u (Neumann) (enforceBoundaryConditions), and
// the star stencil runs in the reference's operation order.  u is not
// modified.  One CTA per patch; f's ghost cells are set to 0.  Cells away from
// the patch boundary need no ghost and are computed while the gather runs;
// the boundary cells follow the barrier.  NN > 0: cubic patches of NN cells
// and one ghost layer, with the index arithmetic known at compile time.
template <int KIND, int SCHEME, int DIM, int NN>
__global__ void __launch_bounds__(256)
    apply_df_kernel(Layout L, const int8_t* __restrict__ ntype, int FS, const float2* __restrict__ inv_df,
                    int neumann, CV coeff, FaceTable ft, const GSlab* __restrict__ slabs,
                    const GCall* __restrict__ calls, const int* __restrict__ side_code, int gs,
                    const float* __restrict__ u, DV f) {
  extern __shared__ df64 G[];  // [2D][gs]
  __shared__ int has[6];
  const int p = blockIdx.x;
  const int side0 = DIM == 2 ? 4 : 20;
  df64 inv[3];
#pragma unroll
  for (int a = 0; a < 3; a++) {
    const float2 v = __ldg(inv_df + (size_t)p * 6 + (KIND ? 3 : 0) + a);
    inv[a] = df64(v.x, v.y);
  }
  const int n0 = NN ? NN : L.n0, n1 = NN ? NN : L.n1, n2 = DIM == 3 ? (NN ? NN : L.n2) : 1;
  const int sy = NN ? NN + 2 : L.sy, py = NN ? NN + 2 : L.n1 + 2 * L.g;
  const int sz = DIM == 3 ? sy * py : 0, g = NN ? 1 : L.g;
  const int cs = NN ? (DIM == 3 ? sy * sy * sy : sy * sy) : L.cs;
  const F32Acc acc{u, (long long)cs};
  for (int e = threadIdx.x; e < 2 * DIM * gs; e += blockDim.x) {
    const int s = e / gs, r = e % gs;
    const FaceGeom& gf = ft.f[side0 + s];
    if (r >= gf.nt[0] * gf.nt[1]) continue;
    const int code = side_code[p * 2 * DIM + s];
    if (code == -1) continue;
    G[e] = side_ghost<df64, SCHEME>(acc, p, s, code, slabs, calls, ft, DIM, r % gf.nt[0], r / gf.nt[0]);
  }
  if (threadIdx.x < 2 * DIM) has[threadIdx.x] = ntype[(size_t)p * FS + side0 + threadIdx.x] >= 0;
  const float* up = u + (long long)p * cs;
  const long long base = (long long)p * cs;
  const int nn[3] = {n0, n1, n2};
  const int str[3] = {1, sy, sz};
  // pass 0: cells away from the boundary (and the ghost cells of f); pass 1: boundary cells
  for (int pass = 0; pass < 2; pass++) {
    if (pass == 1) __syncthreads();
    for (int e = threadIdx.x; e < cs; e += blockDim.x) {
      const int c0 = e % sy - g, q = e / sy;
      const int c1 = q % py - g, c2 = DIM == 3 ? q / py - g : 0;
      const bool interior = c0 >= 0 && c0 < n0 && c1 >= 0 && c1 < n1 && c2 >= 0 && c2 < n2;
      const bool edge = interior && (c0 == 0 || c0 == n0 - 1 || c1 == 0 || c1 == n1 - 1 ||
                                     (DIM == 3 && (c2 == 0 || c2 == n2 - 1)));
      if (edge != (pass == 1)) continue;
      df64 res(0.f, 0.f);
      if (interior && KIND == 0 && !edge) {
        const float mid = up[e];
        res = df_second_difference(up[e + 1], mid, up[e - 1]) * inv[0];
        res += df_second_difference(up[e + sy], mid, up[e - sy]) * inv[1];
        if (DIM == 3) res += df_second_difference(up[e + sz], mid, up[e - sz]) * inv[2];
      } else if (interior) {
        const int cc[3] = {c0, c1, c2};
        const df64 mid(up[e], 0.f);
#pragma unroll
        for (int a = 0; a < DIM; a++) {
          const int st = str[a];
          const int tan = a == 0 ? c1 + c2 * n1 : (a == 1 ? c0 + c2 * n0 : c0 + c1 * n0);
          df64 lo, hi;
          if (cc[a] == 0)
            lo = has[2 * a] ? G[(2 * a) * gs + tan] : (neumann ? mid : -mid);
          else
            lo = df64(up[e - st], 0.f);
          if (cc[a] == nn[a] - 1)
            hi = has[2 * a + 1] ? G[(2 * a + 1) * gs + tan] : (neumann ? mid : -mid);
          else
            hi = df64(up[e + st], 0.f);
          if (KIND == 0) {
            res += ((hi - df64(2.0) * mid) + lo) * inv[a];
          } else {
            const df64 cl = ldv(coeff, base + e - st), cm = ldv(coeff, base + e), cu = ldv(coeff, base + e + st);
            res += ((cu + cm) * (hi - mid) - (cl + cm) * (mid - lo)) * inv[a];
          }
        }
      }
      stv(f, base + e, res);
    }
  }
}

// f = A u (as apply_df_kernel) fused with the dot products that follow it in
// the iteration: NV = 1: rhat . f (-> alpha); NV = 2: f . w and f . f (-> omega).
// Cubic patches of NN cells with one ghost layer; patches of solves that have
// stopped are skipped.  Cells are enumerated explicitly: the (NN-2)^D cells
// away from the patch boundary before the barrier that publishes the gathered
// ghosts, the boundary shell after it.  f's ghost cells are not written (the
// outer loop never reads them).
template <int KIND, int SCHEME, int DIM, int NN, int NV, int NT>
__global__ void __launch_bounds__(NT, 2048 / NT)
    apply_dots_kernel(Layout L, const int8_t* __restrict__ ntype, int FS, const float2* __restrict__ inv_df,
                      int neumann, CV coeff, FaceTable ft, const GSlab* __restrict__ slabs,
                      const GCall* __restrict__ calls, const int* __restrict__ side_code,
                      const SideRec* __restrict__ recs, int gs,
                      const float* __restrict__ u, DV f, CV w, Batch bt, const int* __restrict__ patch_solve,
                      double* part, unsigned int* counter, double* S, int slot0, int finalize_kind) {
  extern __shared__ df64 G[];  // [2D][gs]
  __shared__ int has[6];
  const int p = blockIdx.x;
  const int b = patch_solve[p];
  if (!bt.active[b]) return;
  constexpr int SY = NN + 2, SZ = DIM == 3 ? SY * SY : 0, CS = DIM == 3 ? SY * SY * SY : SY * SY;
  constexpr int NF = DIM == 3 ? NN * NN : NN;
  constexpr int NIN = DIM == 3 ? (NN - 2) * (NN - 2) * (NN - 2) : (NN - 2) * (NN - 2);
  constexpr int NSH = (DIM == 3 ? NN * NN * NN : NN * NN) - NIN;
  const int side0 = DIM == 2 ? 4 : 20;
  df64 inv[3];
#pragma unroll
  for (int a = 0; a < 3; a++) {
    const float2 v = __ldg(inv_df + (size_t)p * 6 + (KIND ? 3 : 0) + a);
    inv[a] = df64(v.x, v.y);
  }
  const F32Acc acc{u, (long long)CS};
  // side ghosts gathered into registers first; they are written to shared
  // memory after the interior cells, so the gather's dependent loads overlap
  // the interior work instead of delaying the barrier
  constexpr int NG = 2 * DIM * NF;
  constexpr int GPT = (NG + NT - 1) / NT;
  df64 gv[GPT];
#pragma unroll
  for (int i = 0; i < GPT; i++) {
    const int e = threadIdx.x + i * NT;
    gv[i] = df64(0.f, 0.f);
    if (NG % NT == 0 || e < NG) {
      const int s = e / NF, r = e % NF;
      if constexpr (GPT == 1) {
        // the side's record: a coarse-fine side's values are one dependent load away
        const SideRec rec = recs[p * 2 * DIM + s];
        if (rec.code != -1) gv[i] = side_ghost_rec<df64, SCHEME, DIM>(acc, p, s, rec, slabs, calls, ft, r % NN, r / NN);
      } else {
        const int code = side_code[p * 2 * DIM + s];
        if (code != -1) gv[i] = side_ghost<df64, SCHEME>(acc, p, s, code, slabs, calls, ft, DIM, r % NN, r / NN);
      }
    }
  }
  if (threadIdx.x < 2 * DIM) has[threadIdx.x] = ntype[(size_t)p * FS + side0 + threadIdx.x] >= 0;
  const float* up = u + (long long)p * CS;
  const long long base = (long long)p * CS;
  dot2 v[NV];
  auto emitw = [&](int k, df64 res, df64 wv) {
    stv(f, base + k, res);
    if (NV == 1) {
      v[0].add(wv, res);
    } else {
      v[0].add(res, wv);
      v[1].add(res, res);
    }
  };
  auto emit = [&](int k, df64 res) { emitw(k, res, ldv(w, base + k)); };
  auto interior_k = [&](int e) {
    const int x = e % (NN - 2) + 1, r = e / (NN - 2);
    const int y = r % (NN - 2) + 1, z = DIM == 3 ? r / (NN - 2) + 1 : 0;
    return (x + 1) + (y + 1) * SY + (DIM == 3 ? (z + 1) * SZ : 0);
  };
  // cells away from the boundary: every neighbour is an interior FP32 value
  if (KIND == 0) {
    // two cells per round, all their loads issued before either is computed
    for (int e0 = threadIdx.x; e0 < NIN; e0 += 2 * NT) {
      int kk[2];
      bool ok[2];
      float m[2], xp[2], xm[2], yp[2], ym[2], zp[2], zm[2];
      df64 wv[2];
#pragma unroll
      for (int q = 0; q < 2; q++) {
        ok[q] = e0 + q * NT < NIN;
        const int k = interior_k(ok[q] ? e0 + q * NT : e0);
        kk[q] = k;
        m[q] = up[k];
        xp[q] = up[k + 1];
        xm[q] = up[k - 1];
        yp[q] = up[k + SY];
        ym[q] = up[k - SY];
        zp[q] = DIM == 3 ? up[k + SZ] : 0.f;
        zm[q] = DIM == 3 ? up[k - SZ] : 0.f;
        wv[q] = ldv(w, base + k);
      }
#pragma unroll
      for (int q = 0; q < 2; q++) {
        if (!ok[q]) continue;
        df64 res = df_second_difference(xp[q], m[q], xm[q]) * inv[0];
        res += df_second_difference(yp[q], m[q], ym[q]) * inv[1];
        if (DIM == 3) res += df_second_difference(zp[q], m[q], zm[q]) * inv[2];
        emitw(kk[q], res, wv[q]);
      }
    }
  } else {
    for (int e = threadIdx.x; e < NIN; e += blockDim.x) {
      const int k = interior_k(e);
      const df64 mid(up[k], 0.f);
      df64 res(0.f, 0.f);
#pragma unroll
      for (int a = 0; a < DIM; a++) {
        const int st = a == 0 ? 1 : (a == 1 ? SY : SZ);
        const df64 lo(up[k - st], 0.f), hi(up[k + st], 0.f);
        const df64 cl = ldv(coeff, base + k - st), cm = ldv(coeff, base + k), cu = ldv(coeff, base + k + st);
        res += ((cu + cm) * (hi - mid) - (cl + cm) * (mid - lo)) * inv[a];
      }
      emit(k, res);
    }
  }
#pragma unroll
  for (int i = 0; i < GPT; i++) {
    const int e = threadIdx.x + i * NT;
    if (NG % NT == 0 || e < NG) G[(e / NF) * gs + e % NF] = gv[i];
  }
  __syncthreads();
  // the boundary shell: 2D: the ring; 3D: the z = 0 and z = NN-1 planes, then the ring of every inner slice
  for (int e = threadIdx.x; e < NSH; e += blockDim.x) {
    int x, y, z = 0;
    int q = e;
    if (DIM == 3) {
      if (q < 2 * NN * NN) {
        z = q < NN * NN ? 0 : NN - 1;
        q %= NN * NN;
        x = q % NN;
        y = q / NN;
      } else {
        q -= 2 * NN * NN;
        z = q / (4 * NN - 4) + 1;
        q %= 4 * NN - 4;
        if (q < NN) { x = q; y = 0; }
        else if (q < 2 * NN) { x = q - NN; y = NN - 1; }
        else if (q < 3 * NN - 2) { x = 0; y = q - 2 * NN + 1; }
        else { x = NN - 1; y = q - 3 * NN + 3; }
      }
    } else {
      if (q < NN) { x = q; y = 0; }
      else if (q < 2 * NN) { x = q - NN; y = NN - 1; }
      else if (q < 3 * NN - 2) { x = 0; y = q - 2 * NN + 1; }
      else { x = NN - 1; y = q - 3 * NN + 3; }
    }
    const int k = (x + 1) + (y + 1) * SY + (DIM == 3 ? (z + 1) * SZ : 0);
    const int cc[3] = {x, y, z};
    const df64 mid(up[k], 0.f);
    df64 res(0.f, 0.f);
#pragma unroll
    for (int a = 0; a < DIM; a++) {
      const int st = a == 0 ? 1 : (a == 1 ? SY : SZ);
      const int tan = a == 0 ? y + z * NN : (a == 1 ? x + z * NN : x + y * NN);
      df64 lo, hi;
      if (cc[a] == 0)
        lo = has[2 * a] ? G[(2 * a) * gs + tan] : (neumann ? mid : -mid);
      else
        lo = df64(up[k - st], 0.f);
      if (cc[a] == NN - 1)
        hi = has[2 * a + 1] ? G[(2 * a + 1) * gs + tan] : (neumann ? mid : -mid);
      else
        hi = df64(up[k + st], 0.f);
      if (KIND == 0) {
        res += ((hi - df64(2.0) * mid) + lo) * inv[a];
      } else {
        const df64 cl = ldv(coeff, base + k - st), cm = ldv(coeff, base + k), cu = ldv(coeff, base + k + st);
        res += ((cu + cm) * (hi - mid) - (cl + cm) * (mid - lo)) * inv[a];
      }
    }
    emit(k, res);
  }
  // block sums of the threads' compensated pairs (s, c), then this solve's patch partials in
  // patch order: every pair into shared memory; the 32 threads of warp 0 merge NT / 32 pairs
  // each (thread l: l, l + 32, ...), then across the warp -- a merge adds the s parts exactly
  // (TwoSum) and carries its error with the c parts, as Dot2 accumulates one pair
  __shared__ float2 red[NV][NT];
#pragma unroll
  for (int i = 0; i < NV; i++) red[i][threadIdx.x] = make_float2(v[i].s, v[i].c);
  __syncthreads();
  double blk[NV];
  if (threadIdx.x < 32) {
    const int l = threadIdx.x;
#pragma unroll
    for (int i = 0; i < NV; i++) {
      float sm = red[i][l].x, cm = red[i][l].y;
#pragma unroll
      for (int q = 1; q < NT / 32; q++) {
        const float2 o = red[i][l + 32 * q];
        const df64 t2 = two_sum(sm, o.x);
        sm = t2.hi;
        cm = __fadd_rn(cm, __fadd_rn(o.y, t2.lo));
      }
#pragma unroll
      for (int off = 16; off > 0; off >>= 1) {
        const float so = __shfl_down_sync(0xffffffffu, sm, off), co = __shfl_down_sync(0xffffffffu, cm, off);
        const df64 t2 = two_sum(sm, so);
        sm = t2.hi;
        cm = __fadd_rn(cm, __fadd_rn(co, t2.lo));
      }
      blk[i] = df_to_double(two_sum(sm, cm));
    }
  }
  const int first = bt.offs[b];
  kp_reduce<NV>(blk, bt.B, b, first, bt.offs[b + 1] - first, p, part, L.P, counter, S, slot0, finalize_kind);
}

template <int KIND, int SCHEME, int DIM, int NN>
static void apply_df_launch(const te_operator* A, const float* u, DV f, cudaStream_t st) {
  const te_domain* d = A->dom;
  const Layout& L = d->lay;
  const te_ghost_filler* g = A->gf;
  const int gs = corr_stride(L);
  const size_t smem = (size_t)2 * L.D * gs * sizeof(df64);
  const long long n = (long long)L.P * L.cs;
  CV coeff{KIND ? A->coeffs_df.p : nullptr, KIND ? A->coeffs_df.p + n : nullptr};
  auto kern = apply_df_kernel<KIND, SCHEME, DIM, NN>;
  if (smem > 40 * 1024)
    allow_max_dynamic_smem((const void*)kern);
  kern<<<L.P, 256, smem, st>>>(L, d->d_nbr_type.p, d->F, (const float2*)d->d_inv_df.p, A->neumann, coeff,
                               g->faces, g->d_slabs.p, g->d_calls.p, g->d_side_code.p, gs, u, f);
  count_launch();
  TE_LAUNCH_CHECK();
}

// the general apply (any patch shape); cubic levels with the usual sizes take apply_dots
template <int KIND, int SCHEME>
static void apply_df_t(const te_operator* A, const float* u, DV f, cudaStream_t st) {
  if (A->dom->lay.D == 2)
    apply_df_launch<KIND, SCHEME, 2, 0>(A, u, f, st);
  else
    apply_df_launch<KIND, SCHEME, 3, 0>(A, u, f, st);
}

static void apply_df(const te_operator* A, const float* u, DV f, cudaStream_t st) {
  const int sc = A->gf->scheme;
#define TE_AD(K, S) apply_df_t<K, S>(A, u, f, st)
  if (A->kind == 0) {
    if (sc == TE_GHOST_BILINEAR) TE_AD(0, TE_GHOST_BILINEAR);
    else if (sc == TE_GHOST_BIQUADRATIC) TE_AD(0, TE_GHOST_BIQUADRATIC);
    else TE_AD(0, TE_GHOST_TRILINEAR);
  } else {
    if (sc == TE_GHOST_BILINEAR) TE_AD(1, TE_GHOST_BILINEAR);
    else if (sc == TE_GHOST_BIQUADRATIC) TE_AD(1, TE_GHOST_BIQUADRATIC);
    else TE_AD(1, TE_GHOST_TRILINEAR);
  }
#undef TE_AD
}

// S[solve][S_XNZ] = 1 for every solve whose x (its patch range, ghosts included) has a nonzero
// value; every writer stores the same value
__global__ void x_nonzero(const double* __restrict__ x, long long n, long long pstride,
                          const int* __restrict__ patch_solve, double* __restrict__ S) {
  // x != 0.0 tested on the bits (every value but +0 and -0 has a nonzero bit below the sign),
  // so the FP64 pipe stays idle
  const long long* xb = reinterpret_cast<const long long*>(x);
  const long long step = (long long)gridDim.x * blockDim.x;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += 4 * step) {
    unsigned long long v[4];
#pragma unroll
    for (int k = 0; k < 4; k++) v[k] = i + k * step < n ? (unsigned long long)__ldg(xb + i + k * step) : 0ull;
#pragma unroll
    for (int k = 0; k < 4; k++)
      if ((v[k] << 1) != 0ull) S[(size_t)patch_solve[(i + k * step) / pstride] * S_NSLOTS + S_XNZ] = 1.0;
  }
}

// scalar exchange between a Krylov run's device state and mapped host memory (KrylovWork)
__global__ void scalars_to_host(double* __restrict__ dst, const double* __restrict__ src, int n) {
  for (int i = threadIdx.x; i < n; i += blockDim.x) dst[i] = src[i];
}
__global__ void scalars_from_host(double* __restrict__ dst, const double* __restrict__ src, int n) {
  for (int i = threadIdx.x; i < n; i += blockDim.x) dst[i] = src[i];
}
struct FlagChunk {
  static constexpr int N = 256;
  int v[N];
};
__global__ void set_flags(int* __restrict__ dst, FlagChunk c, int n) {
  if ((int)threadIdx.x < n) dst[threadIdx.x] = c.v[threadIdx.x];
}
struct ErrFlags {
  static constexpr int N = 32;
  int* p[N];
  int n;
};
// or of the flags (each cleared) into *out
__global__ void take_flags(ErrFlags f, int* out) {
  int v = 0;
  if ((int)threadIdx.x < f.n) {
    v = f.p[threadIdx.x][0];
    f.p[threadIdx.x][0] = 0;
  }
  v = __any_sync(0xffffffffu, v != 0);
  if (threadIdx.x == 0) *(volatile int*)out = v;
}

struct KrylovWork {
  const te_domain* d;
  int nc;
  int B;
  size_t n;
  std::vector<int> h_offs, h_nch;
  DevBuf<double> resid, rhat, p, ap, as, s, ms, mp, S, part;
  DevBuf<unsigned int> counter;
  DevBuf<int> offs, nch, active;
  DevBuf<int> patch_solve;  // [P] solve of each finest patch
  DevBuf<double> part_p;    // [2][P] per-patch dot partials of the fused apply
  DevBuf<double> dx;        // float-float loop: correction to x since the last fold (allocated on first use)
  double* h = nullptr;       // per-solve scalars on the host (pinned, mapped)
  double* h_dev = nullptr;   // the same memory as the device sees it
  int* h_active = nullptr;
  int* h_tcerr = nullptr;    // tensor-core smoother error flags gathered for the host (pinned, mapped)
  int* h_tcerr_dev = nullptr;
  cudaStream_t cap = nullptr;
  cudaEvent_t ev_in = nullptr, ev_out = nullptr;
  struct G {
    cudaGraph_t g = nullptr;
    cudaGraphExec_t x = nullptr;
    long long launches = 0;
  };
  // keyed by x, b, the cycle's serial number and buffer generation, tol, flags
  std::map<std::tuple<void*, const void*, unsigned long long, unsigned long long, double, int>, G> graphs;
  // keys whose first iteration ran eagerly (the autotuner times launch shapes it has not met then)
  std::set<std::tuple<void*, const void*, unsigned long long, unsigned long long, double, int>> warmed;
  KrylovWork(const te_domain* d, int nc, const std::vector<int>& offsets) : d(d), nc(nc) {
    B = (int)offsets.size() - 1;
    h_offs = offsets;
    for (int b = 0; b < B; b++) h_nch.push_back(chunks_for(offsets[b + 1] - offsets[b]));
    n = (size_t)d->lay.P * d->lay.pstride(nc);
    for (auto* buf : {&resid, &rhat, &p, &ap, &as, &s, &ms, &mp}) {
      buf->alloc(n);
      TE_CUDA(cudaMemsetAsync(buf->p, 0, n * sizeof(double), d->stream));
    }
    S.alloc((size_t)B * S_NSLOTS);
    part.alloc((size_t)3 * B * MAX_CHUNKS);
    counter.alloc(B);
    TE_CUDA(cudaMemsetAsync(counter.p, 0, B * sizeof(unsigned int), d->stream));
    offs.upload(h_offs, d->stream);
    {
      std::vector<int> ps(d->lay.P, 0);
      for (int b2 = 0; b2 < B; b2++)
        for (int q = offsets[b2]; q < offsets[b2 + 1]; q++) ps[q] = b2;
      patch_solve.upload(ps, d->stream);
      part_p.alloc((size_t)2 * d->lay.P);
    }
    nch.upload(h_nch, d->stream);
    active.alloc(B);
    TE_CUDA(cudaHostAlloc(&h, (size_t)B * S_NSLOTS * sizeof(double), cudaHostAllocMapped));
    TE_CUDA(cudaHostGetDevicePointer((void**)&h_dev, h, 0));
    TE_CUDA(cudaMallocHost(&h_active, (size_t)B * sizeof(int)));
    TE_CUDA(cudaHostAlloc(&h_tcerr, sizeof(int), cudaHostAllocMapped));
    TE_CUDA(cudaHostGetDevicePointer((void**)&h_tcerr_dev, h_tcerr, 0));
    TE_CUDA(cudaStreamCreateWithFlags(&cap, cudaStreamNonBlocking));
    TE_CUDA(cudaEventCreateWithFlags(&ev_in, cudaEventDisableTiming));
    TE_CUDA(cudaEventCreateWithFlags(&ev_out, cudaEventDisableTiming));
  }
  ~KrylovWork() {
    for (auto& kv : graphs) {
      if (kv.second.x) cudaGraphExecDestroy(kv.second.x);
      if (kv.second.g) cudaGraphDestroy(kv.second.g);
    }
    if (h) cudaFreeHost(h);
    if (h_active) cudaFreeHost(h_active);
    if (h_tcerr) cudaFreeHost(h_tcerr);
    if (ev_in) cudaEventDestroy(ev_in);
    if (ev_out) cudaEventDestroy(ev_out);
    if (cap) cudaStreamDestroy(cap);
  }
  Batch batch() const { return Batch{B, offs.p, nch.p, active.p}; }
  // float-float views of the work buffers: hi in the first n floats, lo in the next n
  DV dv(DevBuf<double>& v) const { return DV{(float*)v.p, (float*)v.p + n}; }
  CV cv(const DevBuf<double>& v) const { return CV{(const float*)v.p, (const float*)v.p + n}; }
  float* f32(DevBuf<double>& v) const { return (float*)v.p; }
  int grid() const { return B * MAX_CHUNKS; }
  // The per-iteration scalar exchange uses no copy engine: a kernel writes the scalars into
  // mapped host memory (and reads them from there), and the active flags travel as kernel
  // arguments.  Copies of other streams (a serving loop's uploads and downloads of whole
  // right-hand sides and solutions) then cannot hold up an iteration's convergence test.
  void read_scalars(cudaStream_t st) {
    scalars_to_host<<<1, 256, 0, st>>>(h_dev, S.p, B * S_NSLOTS);
    count_launch();
    TE_LAUNCH_CHECK();
    TE_CUDA(cudaStreamSynchronize(st));
  }
  // the host's scalars of solves [i0, i1) into the device copy
  void push_scalars(cudaStream_t st, int i0 = 0, int i1 = -1) {
    if (i1 < 0) i1 = B;
    scalars_from_host<<<1, 256, 0, st>>>(S.p + (size_t)i0 * S_NSLOTS, h_dev + (size_t)i0 * S_NSLOTS,
                                         (i1 - i0) * S_NSLOTS);
    count_launch();
    TE_LAUNCH_CHECK();
  }
  void push_active(cudaStream_t st) {
    for (int i0 = 0; i0 < B; i0 += FlagChunk::N) {
      FlagChunk c;
      const int m = std::min(FlagChunk::N, B - i0);
      for (int k = 0; k < m; k++) c.v[k] = h_active[i0 + k];
      set_flags<<<1, FlagChunk::N, 0, st>>>(active.p + i0, c, m);
      count_launch();
      TE_LAUNCH_CHECK();
    }
  }
};

static void launch_dots(KrylovWork& W, int nv, const double* a0, const double* b0, const double* a1, const double* b1,
                        const double* a2, const double* b2, int slot0, int fin, cudaStream_t st) {
  const Layout& L = W.d->lay;
  Batch bt = W.batch();
  with_cells<4>(L, [&](auto* cells) {
    using C = std::remove_pointer_t<decltype(cells)>;
    if (nv == 1)
      k_dots_c<1, C><<<W.grid(), KT, 0, st>>>(L, W.nc, bt, a0, b0, a1, b1, a2, b2, W.part.p, W.counter.p, W.S.p,
                                              slot0, fin);
    else if (nv == 2)
      k_dots_c<2, C><<<W.grid(), KT, 0, st>>>(L, W.nc, bt, a0, b0, a1, b1, a2, b2, W.part.p, W.counter.p, W.S.p,
                                              slot0, fin);
    else
      k_dots_c<3, C><<<W.grid(), KT, 0, st>>>(L, W.nc, bt, a0, b0, a1, b1, a2, b2, W.part.p, W.counter.p, W.S.p,
                                              slot0, fin);
  });
  count_launch();
  TE_LAUNCH_CHECK();
}

// one BiCGStab iteration (everything between two convergence tests)
static void iteration(KrylovWork& W, const te_operator* A, te_cycle* M, double* x, double tol, int flags,
                      cudaStream_t st) {
  const Layout& L = W.d->lay;
  int nc = W.nc;
  Batch bt = W.batch();
  double* mp = M ? W.mp.p : W.p.p;
  double* ms = M ? W.ms.p : W.s.p;
  if (M) M->body(W.p.p, W.mp.p, st);
  operator_apply(A, nc, TE_F64, mp, W.ap.p, st);
  launch_dots(W, 1, W.rhat.p, W.ap.p, nullptr, nullptr, nullptr, nullptr, S_RHAT_AP, 1, st);
  k_s<<<W.grid(), KT, 0, st>>>(L, nc, bt, tol, W.resid.p, W.ap.p, W.s.p, W.part.p, W.counter.p, W.S.p);
  count_launch();
  TE_LAUNCH_CHECK();
  if (M) M->body(W.s.p, W.ms.p, st);
  operator_apply(A, nc, TE_F64, ms, W.as.p, st);
  launch_dots(W, 2, W.as.p, W.s.p, W.as.p, W.as.p, nullptr, nullptr, S_AS_S, 2, st);
  const double* dir = (M && (flags & TE_BICGSTAB_PRECONDITIONED_EXIT)) ? W.mp.p : W.p.p;
  k_xr<<<W.grid(), KT, 0, st>>>(L, nc, bt, x, W.resid.p, mp, ms, W.ap.p, W.as.p, W.rhat.p, dir, W.part.p,
                                W.counter.p, W.S.p);
  count_launch();
  TE_LAUNCH_CHECK();
  k_p<<<W.grid(), KT, 0, st>>>(L, nc, bt, W.p.p, W.ap.p, W.resid.p, W.S.p);
  count_launch();
  TE_LAUNCH_CHECK();
}

template <int KIND, int SCHEME, int DIM, int NN, int NV>
static void apply_dots_launch(const te_operator* A, KrylovWork& W, const float* u, DV f, CV w, int slot0, int fin,
                              cudaStream_t st) {
  const te_domain* d = A->dom;
  const Layout& L = d->lay;
  const te_ghost_filler* g = A->gf;
  const int gs = corr_stride(L);
  const size_t smem = (size_t)2 * L.D * gs * sizeof(df64);
  const long long n = (long long)L.P * L.cs;
  CV coeff{KIND ? A->coeffs_df.p : nullptr, KIND ? A->coeffs_df.p + n : nullptr};
  // 2D patches up to 32^2: 128 threads per patch, twice the patches resident of 256 (the gather of
  // a 32^2 patch's 128 side ghosts is one per thread); larger patches keep 256
  constexpr int NT = DIM == 2 && NN <= 32 ? 128 : 256;
  auto kern = apply_dots_kernel<KIND, SCHEME, DIM, NN, NV, NT>;
  if (smem > 40 * 1024)
    allow_max_dynamic_smem((const void*)kern);
  kern<<<L.P, NT, smem, st>>>(L, d->d_nbr_type.p, d->F, (const float2*)d->d_inv_df.p, A->neumann, coeff, g->faces,
                               g->d_slabs.p, g->d_calls.p, g->d_side_code.p, g->d_side_rec.p, gs, u, f, w, W.batch(),
                               W.patch_solve.p, W.part_p.p, W.counter.p, W.S.p, slot0, fin);
  count_launch();
  TE_LAUNCH_CHECK();
}

template <int NV, int KIND, int SCHEME>
static bool apply_dots_t(const te_operator* A, KrylovWork& W, const float* u, DV f, CV w, int slot0, int fin,
                         cudaStream_t st) {
  const Layout& L = A->dom->lay;
  if (!(L.g == 1 && L.n1 == L.n0 && (L.D == 2 || L.n2 == L.n0))) return false;
  if (L.D == 2) {
    if constexpr (SCHEME == TE_GHOST_TRILINEAR) {
      return false;
    } else {
      if (L.n0 == 16) apply_dots_launch<KIND, SCHEME, 2, 16, NV>(A, W, u, f, w, slot0, fin, st);
      else if (L.n0 == 32) apply_dots_launch<KIND, SCHEME, 2, 32, NV>(A, W, u, f, w, slot0, fin, st);
      else if (L.n0 == 64) apply_dots_launch<KIND, SCHEME, 2, 64, NV>(A, W, u, f, w, slot0, fin, st);
      else return false;
      return true;
    }
  }
  if constexpr (SCHEME != TE_GHOST_TRILINEAR) {
    return false;
  } else {
    if (L.n0 == 8) apply_dots_launch<KIND, SCHEME, 3, 8, NV>(A, W, u, f, w, slot0, fin, st);
    else if (L.n0 == 16) apply_dots_launch<KIND, SCHEME, 3, 16, NV>(A, W, u, f, w, slot0, fin, st);
    else return false;
    return true;
  }
}

// f = A u with the dots that follow it; false when the level does not qualify (the caller then
// runs apply_df and the separate dot kernel)
template <int NV>
static bool apply_dots(const te_operator* A, KrylovWork& W, const float* u, DV f, CV w, int slot0, int fin,
                       cudaStream_t st) {
  if (W.nc != 1) return false;
  static const bool off = [] {
    const char* e = getenv("TE_NO_FUSED_DOTS");
    return e && e[0] == '1';
  }();
  if (off) return false;
  const int sc = A->gf->scheme;
  if (A->kind == 0) {
    if (sc == TE_GHOST_BILINEAR) return apply_dots_t<NV, 0, TE_GHOST_BILINEAR>(A, W, u, f, w, slot0, fin, st);
    if (sc == TE_GHOST_BIQUADRATIC) return apply_dots_t<NV, 0, TE_GHOST_BIQUADRATIC>(A, W, u, f, w, slot0, fin, st);
    return apply_dots_t<NV, 0, TE_GHOST_TRILINEAR>(A, W, u, f, w, slot0, fin, st);
  }
  if (sc == TE_GHOST_BILINEAR) return apply_dots_t<NV, 1, TE_GHOST_BILINEAR>(A, W, u, f, w, slot0, fin, st);
  if (sc == TE_GHOST_BIQUADRATIC) return apply_dots_t<NV, 1, TE_GHOST_BIQUADRATIC>(A, W, u, f, w, slot0, fin, st);
  return apply_dots_t<NV, 1, TE_GHOST_TRILINEAR>(A, W, u, f, w, slot0, fin, st);
}

// one float-float iteration; M is an FP32 cycle
static void iteration_df(KrylovWork& W, const te_operator* A, te_cycle* M, double tol, int flags, cudaStream_t st) {
  const Layout& L = W.d->lay;
  const int nc = W.nc;
  Batch bt = W.batch();
  const CV none{nullptr, nullptr};
  M->body_f32(W.f32(W.p), W.f32(W.mp), st);
  if (!apply_dots<1>(A, W, W.f32(W.mp), W.dv(W.ap), W.cv(W.rhat), S_RHAT_AP, 1, st)) {
    apply_df(A, W.f32(W.mp), W.dv(W.ap), st);
    kd_dots<1><<<W.grid(), KT, 0, st>>>(L, nc, bt, W.cv(W.rhat), W.cv(W.ap), none, none, none, none, W.part.p,
                                        W.counter.p, W.S.p, S_RHAT_AP, 1);
    count_launch();
    TE_LAUNCH_CHECK();
  }
  with_cells<2>(L, [&](auto* cells) {
    kd_s<std::remove_pointer_t<decltype(cells)>><<<W.grid(), KT, 0, st>>>(
        L, nc, bt, tol, W.cv(W.resid), W.cv(W.ap), W.dv(W.s), W.part.p, W.counter.p, W.S.p);
  });
  count_launch();
  TE_LAUNCH_CHECK();
  M->body_f32(W.f32(W.s), W.f32(W.ms), st);
  if (!apply_dots<2>(A, W, W.f32(W.ms), W.dv(W.as), W.cv(W.s), S_AS_S, 2, st)) {
    apply_df(A, W.f32(W.ms), W.dv(W.as), st);
    kd_dots<2><<<W.grid(), KT, 0, st>>>(L, nc, bt, W.cv(W.as), W.cv(W.s), W.cv(W.as), W.cv(W.as), none, none,
                                        W.part.p, W.counter.p, W.S.p, S_AS_S, 2);
    count_launch();
    TE_LAUNCH_CHECK();
  }
  const CV dir = (flags & TE_BICGSTAB_PRECONDITIONED_EXIT) ? CV{W.f32(W.mp), nullptr} : W.cv(W.p);
  with_cells<2>(L, [&](auto* cells) {
    kd_xr<std::remove_pointer_t<decltype(cells)>><<<W.grid(), KT, 0, st>>>(
        L, nc, bt, W.dv(W.dx), W.dv(W.resid), W.f32(W.mp), W.f32(W.ms), W.cv(W.ap), W.cv(W.as), W.cv(W.rhat), dir,
        W.part.p, W.counter.p, W.S.p);
  });
  count_launch();
  TE_LAUNCH_CHECK();
  with_cells<2>(L, [&](auto* cells) {
    kd_p<std::remove_pointer_t<decltype(cells)>><<<W.grid(), KT, 0, st>>>(L, nc, bt, W.dv(W.p), W.cv(W.ap),
                                                                          W.cv(W.resid), W.S.p);
  });
  count_launch();
  TE_LAUNCH_CHECK();
}

// the float-float outer loop runs when the preconditioner is an FP32 cycle
static bool use_df(const te_operator* A, int nc, const te_cycle* M, int flags) {
  if (!M || M->dtype != TE_F32 || nc != 1 || (flags & TE_BICGSTAB_FP64_OUTER)) return false;
  if (A->kind == 1 && !A->coeffs_df.p) return false;
  const char* e = getenv("TE_KRYLOV_FP64");
  return !(e && e[0] == '1');
}

// One batched BiCGStab run as a resumable object: start() forms the initial
// residuals, step(k) advances up to k iterations (replaying the iteration's
// CUDA graph and testing convergence on the host after each), and the
// float-float loop's residual-replacement check runs when every solve has
// stopped.  solve_batched runs it to the end in one call; the serving loop
// (te_bicgstab_batch_*) steps it a few iterations at a time.
struct BatchRun {
  const te_operator* A;
  int nc;
  const te_domain* d;
  cudaStream_t st;
  int B;
  KrylovWork* Wp;
  te_cycle* M;
  double* x;
  const double* b;
  size_t bytes;
  bool df;
  long long nvals;
  double tol;
  int max_iterations, flags;
  std::vector<double> rho, r0, residual, finals;
  std::vector<int> its, statuses;
  int nactive = 0, restart = 0;
  bool done = false, use_graph = true;
  bool zero_x = false;  // float-float start: every solve's x was zero
  // slot mode (TE_BICGSTAB_SLOTS): solves are reset and finished one at a time while the
  // others iterate; step() only iterates
  bool slot_mode = false;
  std::vector<int> offs, restarts;
  std::tuple<void*, const void*, unsigned long long, unsigned long long, double, int> gkey;

  BatchRun(const te_operator* A_, int nc_, void* xv, const void* bv, const te_cycle* Mc, double tol_, int max_it,
           int flags_, const std::vector<int>& offsets)
      : A(A_), nc(nc_), d(A_->dom), st(A_->dom->stream), B((int)offsets.size() - 1), x((double*)xv),
        b((const double*)bv), tol(tol_), max_iterations(max_it), flags(flags_) {
    offs = offsets;
    restarts.assign(B, 0);
    slot_mode = (flags & TE_BICGSTAB_SLOTS) != 0;
    // the solver's work vectors live with the operator (freed with it), per component count and batch layout
    auto& slot = A->krylov[std::make_pair(nc, offsets)];
    if (!slot) slot = std::make_shared<KrylovWork>(d, nc, offsets);
    Wp = std::static_pointer_cast<KrylovWork>(slot).get();
    M = const_cast<te_cycle*>(Mc);
    if (M) M->ensure(nc);
    bytes = Wp->n * sizeof(double);
    df = use_df(A, nc, M, flags);
    nvals = (long long)Wp->n;
    rho.assign(B, 0.0);
    r0.assign(B, 0.0);
    residual.assign(B, 0.0);
    finals.assign(B, 0.0);
    its.assign(B, 0);
    statuses.assign(B, TE_OK);
    const char* ng = getenv("TE_NO_GRAPH");
    use_graph = !(ng && ng[0] == '1');
    gkey = std::make_tuple((void*)x, (const void*)b, M ? M->serial : 0ull, M ? M->generation : 0ull, tol,
                           flags | (df ? 1 << 30 : 0));
  }

  void start() {
    KrylovWork& W = *Wp;
    TE_CUDA(cudaMemsetAsync(W.S.p, 0, (size_t)B * S_NSLOTS * sizeof(double), st));
    for (int i = 0; i < B; i++) W.h_active[i] = 1;
    W.push_active(st);
    if (df) {
      // resid = b - A x in FP64, then split into float-float; rhat = p = resid (BiCGStab.h:113-131);
      // the correction dx starts at 0
      if (!W.dx.p) W.dx.alloc(W.n);
      TE_CUDA(cudaMemsetAsync(W.dx.p, 0, (size_t)W.n * sizeof(double), st));
      folded = true;
      // when every solve starts from x = 0 (a served request's first batch), b - A x is b itself,
      // bit for bit (A 0 = 0), and the FP64 operator pass is skipped
      x_nonzero<<<1216, 256, 0, st>>>(x, nvals, d->lay.pstride(nc), W.patch_solve.p, W.S.p);
      count_launch();
      TE_LAUNCH_CHECK();
      launch_dots(W, 1, b, b, nullptr, nullptr, nullptr, nullptr, S_BB, 0, st);
      W.read_scalars(st);
      zero_x = true;
      for (int i = 0; i < B; i++) zero_x = zero_x && W.h[(size_t)i * S_NSLOTS + S_XNZ] == 0.0;
      const double* r_in = b;
      if (!zero_x) {
        operator_residual(A, nc, x, b, W.ap.p, st);
        r_in = W.ap.p;
        // rhat = resid here, so rhat . resid and resid . resid are one sum (the same bits)
        launch_dots(W, 2, b, b, W.ap.p, W.ap.p, nullptr, nullptr, S_BB, 0, st);
      }
      kd_split3<<<1216, 256, 0, st>>>(r_in, W.dv(W.resid), W.dv(W.rhat), W.dv(W.p), nvals);
      count_launch();
      TE_LAUNCH_CHECK();
      if (!zero_x) W.read_scalars(st);
    } else {
      // resid = b - A x; rhat = p = resid (BiCGStab.h:113-131)
      operator_residual(A, nc, x, b, W.resid.p, st);
      TE_CUDA(cudaMemcpyAsync(W.rhat.p, W.resid.p, bytes, cudaMemcpyDeviceToDevice, st));
      TE_CUDA(cudaMemcpyAsync(W.p.p, W.resid.p, bytes, cudaMemcpyDeviceToDevice, st));
      launch_dots(W, 2, b, b, W.resid.p, W.resid.p, nullptr, nullptr, S_BB, 0, st);
      W.read_scalars(st);
    }
    nactive = 0;
    for (int i = 0; i < B; i++) {
      double* h = W.h + (size_t)i * S_NSLOTS;
      double bb = h[S_BB], rr = df && zero_x ? bb : h[S_BB + 1], rh = rr;
      r0[i] = std::sqrt(bb);
      rho[i] = rh;
      residual[i] = r0[i] != 0 ? std::sqrt(rr) / r0[i] : 0.0;
      statuses[i] = TE_OK;
      for (int k = 0; k < S_NSLOTS; k++) h[k] = 0.0;
      h[S_RHO] = rho[i];
      h[S_R0] = r0[i];
      finals[i] = residual[i];
      // zero right-hand side or already converged: no iterations (BiCGStab.h:140-144); a
      // non-finite right-hand side or initial residual is a breakdown (the reference would
      // return at once, its comparisons with NaN being false)
      const bool finite = std::isfinite(bb) && std::isfinite(rr);
      if (!finite) statuses[i] = TE_ERR_BREAKDOWN;
      W.h_active[i] = (finite && r0[i] != 0 && residual[i] > tol && max_iterations > 0) ? 1 : 0;
      if (W.h_active[i] && rho[i] == 0) {  // BiCGStab.h:149-151
        statuses[i] = TE_ERR_BREAKDOWN;
        W.h_active[i] = 0;
      }
      nactive += W.h_active[i];
    }
    W.push_scalars(st);
    W.push_active(st);
  }

  void iterate_once() {
    KrylovWork& W = *Wp;
    folded = false;
    bool eager = !use_graph;
    if (use_graph && !W.graphs.count(gkey) && !W.warmed.count(gkey)) {
      // the first iteration of a new graph key runs eagerly: launches of shapes the autotuner
      // has not met yet are timed there (a capture cannot be), and later captures reuse the choices
      W.warmed.insert(gkey);
      eager = true;
    }
    if (!eager) {
      auto it = W.graphs.find(gkey);
      if (it == W.graphs.end()) {
        KrylovWork::G g;
        long long l0 = g_launches.load();
        TE_CUDA(cudaStreamBeginCapture(W.cap, cudaStreamCaptureModeThreadLocal));
        try {
          if (df)
            iteration_df(W, A, M, tol, flags, W.cap);
          else
            iteration(W, A, M, x, tol, flags, W.cap);
        } catch (...) {
          cudaGraph_t junk = nullptr;
          cudaStreamEndCapture(W.cap, &junk);
          if (junk) cudaGraphDestroy(junk);
          throw;
        }
        TE_CUDA(cudaStreamEndCapture(W.cap, &g.g));
        TE_CUDA(cudaGraphInstantiate(&g.x, g.g, 0));
        g.launches = g_launches.load() - l0;
        g_launches.fetch_sub(g.launches);
        it = W.graphs.emplace(gkey, g).first;
      }
      TE_CUDA(cudaEventRecord(W.ev_in, st));
      TE_CUDA(cudaStreamWaitEvent(W.cap, W.ev_in, 0));
      TE_CUDA(cudaGraphLaunch(it->second.x, W.cap));
      count_launch((int)it->second.launches);
      TE_CUDA(cudaEventRecord(W.ev_out, W.cap));
      TE_CUDA(cudaStreamWaitEvent(st, W.ev_out, 0));
    } else if (df) {
      iteration_df(W, A, M, tol, flags, st);
    } else {
      iteration(W, A, M, x, tol, flags, st);
    }
    W.read_scalars(st);
    bool changed = false;
    for (int i = 0; i < B; i++) {
      if (!W.h_active[i]) continue;
      const double* h = W.h + (size_t)i * S_NSLOTS;
      if (h[S_DONE] != 0.0) {  // ||s|| / ||b|| <= tol: x updated, stop (BiCGStab.h:162-168)
        finals[i] = std::sqrt(h[S_SS]) / r0[i];
        W.h_active[i] = 0;
        changed = true;
        continue;
      }
      its[i]++;
      rho[i] = h[S_RHO];
      residual[i] = std::sqrt(h[S_RR]) / r0[i];
      finals[i] = residual[i];
      if (!std::isfinite(residual[i]) || !std::isfinite(rho[i])) {
        // non-finite scalars (a singular operator or preconditioner): stop this solve
        // instead of iterating to the limit on NaN
        statuses[i] = TE_ERR_BREAKDOWN;
        W.h_active[i] = 0;
        changed = true;
      } else if (residual[i] <= tol || its[i] >= max_iterations) {
        W.h_active[i] = 0;
        changed = true;
      } else if (rho[i] == 0) {  // BiCGStab.h:149-151
        statuses[i] = TE_ERR_BREAKDOWN;
        W.h_active[i] = 0;
        changed = true;
      }
    }
    if (changed) {
      nactive = 0;
      for (int i = 0; i < B; i++) nactive += W.h_active[i];
      W.push_active(st);
    }
  }

  // x += dx, dx = 0 over every solve (a solve still iterating keeps x + dx)
  bool folded = true;
  void fold() {
    if (!df || folded) return;
    kd_fold<<<1216, 256, 0, st>>>(Wp->dv(Wp->dx), x, nvals);
    count_launch();
    TE_LAUNCH_CHECK();
    folded = true;
  }

  // Residual replacement: the float-float recurrence keeps ~1e-14 of the
  // initial residual, so check every solve's true residual b - A x in FP64
  // (the residual each solve reports) and, while restarts are allowed,
  // restart the ones above tol from it.  True when some solve restarted.
  bool replacement_check(bool allow_restart) {
    KrylovWork& W = *Wp;
    fold();
    for (int i = 0; i < B; i++) W.h_active[i] = statuses[i] == TE_OK ? 1 : 0;
    W.push_active(st);
    operator_residual(A, nc, x, b, W.ap.p, st);
    launch_dots(W, 1, W.ap.p, W.ap.p, nullptr, nullptr, nullptr, nullptr, S_TRUE, 0, st);
    W.read_scalars(st);
    nactive = 0;
    for (int i = 0; i < B; i++) {
      double* h = W.h + (size_t)i * S_NSLOTS;
      const bool ok = statuses[i] == TE_OK && r0[i] != 0;
      const double tr = ok ? std::sqrt(h[S_TRUE]) / r0[i] : 0.0;
      if (ok) finals[i] = tr;
      W.h_active[i] = (allow_restart && ok && tr > tol && its[i] < max_iterations) ? 1 : 0;
      const double rr = h[S_TRUE];
      for (int k = 0; k < S_NSLOTS; k++) h[k] = 0.0;
      h[S_RHO] = rr;  // rhat = r
      h[S_R0] = r0[i];
      rho[i] = rr;
      nactive += W.h_active[i];
    }
    W.push_active(st);
    if (nactive == 0) return false;
    kd_split3<<<1216, 256, 0, st>>>(W.ap.p, W.dv(W.resid), W.dv(W.rhat), W.dv(W.p), nvals);
    count_launch();
    TE_LAUNCH_CHECK();
    W.push_scalars(st);
    return true;
  }

  void finish() {
    fold();
    TE_CUDA(cudaStreamSynchronize(st));
    done = true;
    check_tc();
  }

  // a tensor-core DFT smoother whose MMA completion wait timed out flags it; the results are invalid
  void check_tc() {
    if (!M) return;
    ErrFlags ef;
    ef.n = 0;
    for (const te_cycle_level& lv : M->levels)
      if (lv.smoother && lv.smoother->tc_ok && ef.n < ErrFlags::N) ef.p[ef.n++] = lv.smoother->tc_err.p;
    if (ef.n == 0) return;
    // every level's flag, read and cleared on the device, or-ed into mapped host memory
    take_flags<<<1, 32, 0, st>>>(ef, Wp->h_tcerr_dev);
    count_launch();
    TE_LAUNCH_CHECK();
    TE_CUDA(cudaStreamSynchronize(st));
    if (*(volatile int*)Wp->h_tcerr)
      throw Error(TE_ERR_TIMEOUT, "tensor-core DFT: an MMA completion wait timed out; results are invalid");
  }

  // ---- slot mode: one solve reset or finished while the others keep their state
  long long slot_begin(int i) const { return (long long)offs[i] * d->lay.pstride(nc); }
  long long slot_len(int i) const { return (long long)(offs[i + 1] - offs[i]) * d->lay.pstride(nc); }
  // only solve i active on the device (for its reductions); returns the flags to restore
  std::vector<int> only(int i) {
    KrylovWork& W = *Wp;
    std::vector<int> saved(W.h_active, W.h_active + B);
    for (int j = 0; j < B; j++) W.h_active[j] = j == i ? 1 : 0;
    W.push_active(st);
    return saved;
  }
  void restore(const std::vector<int>& saved) {
    KrylovWork& W = *Wp;
    nactive = 0;
    for (int j = 0; j < B; j++) {
      W.h_active[j] = saved[j];
      nactive += saved[j];
    }
    W.push_active(st);
  }
  // solve i's Krylov vectors from the FP64 residual in ap: resid = rhat = p = ap on its
  // patch range only
  void split_slot(int i) {
    KrylovWork& W = *Wp;
    const long long o = slot_begin(i), n = slot_len(i);
    if (df) {
      auto at = [&](DevBuf<double>& v) {
        DV w = W.dv(v);
        return DV{w.hi + o, w.lo + o};
      };
      kd_split3<<<1216, 256, 0, st>>>(W.ap.p + o, at(W.resid), at(W.rhat), at(W.p), n);
      count_launch();
      TE_LAUNCH_CHECK();
    } else {
      for (DevBuf<double>* v : {&W.resid, &W.rhat, &W.p})
        TE_CUDA(cudaMemcpyAsync(v->p + o, W.ap.p + o, n * sizeof(double), cudaMemcpyDeviceToDevice, st));
    }
  }
  // solve i's scalars restart with rho = rr (rhat = r) and its reference norm r0
  void restart_row(int i, double rr) {
    KrylovWork& W = *Wp;
    double* h = W.h + (size_t)i * S_NSLOTS;
    for (int k = 0; k < S_NSLOTS; k++) h[k] = 0.0;
    h[S_RHO] = rr;
    h[S_R0] = r0[i];
    rho[i] = rr;
    W.push_scalars(st, i, i + 1);
  }
  // a new system in solve i: its b and x have been written into its patch range
  void reset_slot(int i) {
    KrylovWork& W = *Wp;
    std::vector<int> saved = only(i);
    if (df) {  // the new system's correction starts at 0
      const long long o = slot_begin(i), n = slot_len(i);
      DV w = W.dv(W.dx);
      TE_CUDA(cudaMemsetAsync(w.hi + o, 0, (size_t)n * sizeof(float), st));
      TE_CUDA(cudaMemsetAsync(w.lo + o, 0, (size_t)n * sizeof(float), st));
    }
    operator_residual(A, nc, x, b, W.ap.p, st);
    launch_dots(W, 2, b, b, W.ap.p, W.ap.p, nullptr, nullptr, S_BB, 0, st);
    W.read_scalars(st);
    const double* h = W.h + (size_t)i * S_NSLOTS;
    const double bb = h[S_BB], rr = h[S_BB + 1];
    r0[i] = std::sqrt(bb);
    residual[i] = r0[i] != 0 ? std::sqrt(rr) / r0[i] : 0.0;
    finals[i] = residual[i];
    its[i] = 0;
    restarts[i] = 0;
    statuses[i] = TE_OK;
    restart_row(i, rr);
    split_slot(i);
    const bool finite = std::isfinite(bb) && std::isfinite(rr);
    if (!finite) statuses[i] = TE_ERR_BREAKDOWN;
    bool run = finite && r0[i] != 0 && residual[i] > tol && max_iterations > 0;  // BiCGStab.h:140-144
    if (run && rr == 0) {
      statuses[i] = TE_ERR_BREAKDOWN;
      run = false;
    }
    saved[i] = run ? 1 : 0;
    restore(saved);
    done = false;
  }
  // the listed solves stopped on their recurrences: one FP64 residual b - A x and one
  // masked reduction give their true residuals, which decide per solve between finished
  // (x holds its result) and a restart from that residual (at most 8 per solve)
  void finish_slots(const std::vector<int>& sl, int* finished) {
    KrylovWork& W = *Wp;
    std::vector<char> seen(B, 0);
    for (int i : sl) {
      require(i >= 0 && i < B, "slot out of range");
      require(!seen[i], "slot listed twice");
      require(!W.h_active[i], "solve is still iterating");
      seen[i] = 1;
    }
    fold();
    std::vector<int> saved(W.h_active, W.h_active + B);
    for (int j = 0; j < B; j++) W.h_active[j] = seen[j];
    W.push_active(st);
    operator_residual(A, nc, x, b, W.ap.p, st);
    launch_dots(W, 1, W.ap.p, W.ap.p, nullptr, nullptr, nullptr, nullptr, S_TRUE, 0, st);
    W.read_scalars(st);
    for (size_t k = 0; k < sl.size(); k++) {
      const int i = sl[k];
      const double rr = W.h[(size_t)i * S_NSLOTS + S_TRUE];
      const bool ok = statuses[i] == TE_OK && r0[i] != 0;
      const double tr = ok ? std::sqrt(rr) / r0[i] : 0.0;
      if (ok) finals[i] = tr;
      const bool again = ok && tr > tol && its[i] < max_iterations && restarts[i] < 8;
      if (again) {
        restarts[i]++;
        restart_row(i, rr);
        split_slot(i);
      }
      saved[i] = again ? 1 : 0;
      finished[k] = again ? 0 : 1;
    }
    restore(saved);
    TE_CUDA(cudaStreamSynchronize(st));
    check_tc();
  }

  // up to k iterations; returns the number of solves still iterating (0: finished, x holds the results)
  int step(long long k) {
    if (slot_mode) {  // only iterate: resets and finishes are per solve
      long long n = 0;
      while (nactive > 0 && n < k) {
        iterate_once();
        n++;
      }
      return nactive;
    }
    long long n = 0;
    while (!done) {
      if (nactive > 0) {
        if (n >= k) break;
        iterate_once();
        n++;
        continue;
      }
      if (df && replacement_check(restart < 8)) {
        restart++;
        continue;
      }
      finish();
    }
    return done ? 0 : nactive;
  }

  int worst() const {
    int w = TE_OK;
    for (int i = 0; i < B; i++)
      if (statuses[i] != TE_OK) w = statuses[i];
    return w;
  }
};

static int solve_batched(const te_operator* A, int nc, void* xv, const void* bv, const te_cycle* Mc, double tol,
                         int max_iterations, int flags, const std::vector<int>& offsets, int* iterations,
                         double* final_residuals, int* statuses) {
  BatchRun r(A, nc, xv, bv, Mc, tol, max_iterations, flags, offsets);
  r.start();
  r.step(1ll << 60);
  const int B = (int)offsets.size() - 1;
  for (int i = 0; i < B; i++) {
    iterations[i] = r.its[i];
    statuses[i] = r.statuses[i];
    if (final_residuals) final_residuals[i] = r.finals[i];
  }
  return r.worst();
}

}  // namespace te

using namespace te;

extern "C" {

int te_bicgstab_solve(const te_operator* A, int nc, void* xv, const void* bv, const te_cycle* Mc, double tol,
                      int max_iterations, int flags, int* iterations, double* final_residual) {
  int status = TE_OK;
  int rc = guard([&] {
    require(A && xv && bv && iterations, "null argument");
    std::vector<int> offs = {0, A->dom->lay.P};
    int st = TE_OK;
    status = solve_batched(A, nc, xv, bv, Mc, tol, max_iterations, flags, offs, iterations, final_residual, &st);
    if (status == TE_ERR_BREAKDOWN)
      set_error("BiCGStab broke down on iteration " + std::to_string(*iterations) +
                " (rho was 0, or a residual or scalar was not finite)");
  });
  return rc != TE_OK ? rc : status;
}

int te_bicgstab_solve_batched(const te_operator* A, int nc, void* xv, const void* bv, const te_cycle* Mc, double tol,
                              int max_iterations, int flags, int num_solves, const int* patch_offsets,
                              int* iterations, double* final_residuals, int* statuses) {
  int status = TE_OK;
  int rc = guard([&] {
    require(A && xv && bv && patch_offsets && iterations && statuses, "null argument");
    require(num_solves >= 1, "num_solves must be >= 1");
    std::vector<int> offs(patch_offsets, patch_offsets + num_solves + 1);
    require(offs[0] == 0 && offs[num_solves] == A->dom->lay.P, "patch_offsets must span the finest level");
    for (int i = 0; i < num_solves; i++) require(offs[i + 1] > offs[i], "every solve needs at least one patch");
    status = solve_batched(A, nc, xv, bv, Mc, tol, max_iterations, flags, offs, iterations, final_residuals, statuses);
    if (status == TE_ERR_BREAKDOWN)
      set_error("BiCGStab broke down in at least one solve of the batch (rho was 0, or a residual or scalar was "
                "not finite)");
  });
  return rc != TE_OK ? rc : status;
}

int te_bicgstab_batch_create(const te_operator* A, int nc, void* xv, const void* bv, const te_cycle* Mc, double tol,
                             int max_iterations, int flags, int num_solves, const int* patch_offsets,
                             te_bicgstab_batch** out) {
  return guard([&] {
    require(A && xv && bv && patch_offsets && out, "null argument");
    require(num_solves >= 1, "num_solves must be >= 1");
    std::vector<int> offs(patch_offsets, patch_offsets + num_solves + 1);
    require(offs[0] == 0 && offs[num_solves] == A->dom->lay.P, "patch_offsets must span the finest level");
    for (int i = 0; i < num_solves; i++) require(offs[i + 1] > offs[i], "every solve needs at least one patch");
    auto r = std::make_unique<BatchRun>(A, nc, xv, bv, Mc, tol, max_iterations, flags, offs);
    r->start();
    *out = reinterpret_cast<te_bicgstab_batch*>(r.release());
  });
}

int te_bicgstab_batch_step(te_bicgstab_batch* h, int max_iterations, int* num_running) {
  return guard([&] {
    require(h && num_running, "null argument");
    require(max_iterations >= 0, "max_iterations must be >= 0");
    *num_running = reinterpret_cast<BatchRun*>(h)->step(max_iterations);
  });
}

int te_bicgstab_batch_state(const te_bicgstab_batch* h, int* iterations, double* residuals, int* statuses,
                            int* running) {
  return guard([&] {
    require(h, "null argument");
    const BatchRun* r = reinterpret_cast<const BatchRun*>(h);
    for (int i = 0; i < r->B; i++) {
      if (iterations) iterations[i] = r->its[i];
      if (residuals) residuals[i] = r->finals[i];
      if (statuses) statuses[i] = r->statuses[i];
      if (running) running[i] = (!r->done && r->Wp->h_active[i]) ? 1 : 0;
    }
  });
}

int te_bicgstab_batch_reset(te_bicgstab_batch* h, int slot) {
  return guard([&] {
    require(h, "null argument");
    BatchRun* r = reinterpret_cast<BatchRun*>(h);
    require(r->slot_mode, "the batch was not created with TE_BICGSTAB_SLOTS");
    require(slot >= 0 && slot < r->B, "slot out of range");
    require(!r->Wp->h_active[slot], "slot is still iterating");
    r->reset_slot(slot);
  });
}

int te_bicgstab_batch_finish_slots(te_bicgstab_batch* h, int num_slots, const int* slots, int* finished) {
  return guard([&] {
    require(h && (num_slots == 0 || (slots && finished)), "null argument");
    require(num_slots >= 0, "num_slots must be >= 0");
    BatchRun* r = reinterpret_cast<BatchRun*>(h);
    require(r->slot_mode, "the batch was not created with TE_BICGSTAB_SLOTS");
    if (num_slots == 0) return;
    r->finish_slots(std::vector<int>(slots, slots + num_slots), finished);
  });
}

int te_bicgstab_batch_sync_x(te_bicgstab_batch* h) {
  return guard([&] {
    require(h, "null argument");
    BatchRun* r = reinterpret_cast<BatchRun*>(h);
    r->fold();
    TE_CUDA(cudaStreamSynchronize(r->st));
  });
}

int te_bicgstab_batch_destroy(te_bicgstab_batch* h) {
  delete reinterpret_cast<BatchRun*>(h);
  return TE_OK;
}

}  // extern "C"
