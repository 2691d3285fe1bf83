// te_dft.cuh -- shared-memory transform passes of the DFT patch solver.
#pragma once
#include "te_internal.cuh"

namespace te {

// Shared-memory layout of one patch (no ghosts): x stride 1, y stride n0+1,
// z stride (n0+1)*n1.  The odd row pitch keeps the lanes of a warp, which
// walk 32 different lines, on different banks.
struct SmemLay {
  int sy, sz, size;
  int mats;  // element offset of the matrices after the two data buffers (16-byte aligned)
};
__host__ __device__ inline SmemLay smem_lay(const Layout& L) {
  SmemLay s;
  s.sy = L.n0 + 1;
  s.sz = s.sy * L.n1;
  s.size = s.sz * L.n2;
  s.mats = (2 * s.size + 3) / 4 * 4;
  return s;
}
__host__ __device__ inline int smem_mat_elems(const Layout&) { return 0; }

// TI consecutive matrix values; 16-byte vector loads when TI and n allow.
// The matrices are read straight from global memory: every lane of a warp
// reads the same address, and the few KB of transform matrices stay in L1.
template <class T, int TI>
__device__ __forceinline__ void load_row(const T* m, T (&v)[TI], bool vec) {
  if (TI == 8 && vec && sizeof(T) == 4) {
    float4 a = __ldg(reinterpret_cast<const float4*>(m)), b = __ldg(reinterpret_cast<const float4*>(m) + 1);
    v[0] = a.x; v[1] = a.y; v[2] = a.z; v[3] = a.w; v[4] = b.x; v[5] = b.y; v[6] = b.z; v[7] = b.w;
  } else if (TI == 8 && vec && sizeof(T) == 8) {
    const double2* q = reinterpret_cast<const double2*>(m);
    double2 a = __ldg(q), b = __ldg(q + 1), c = __ldg(q + 2), d = __ldg(q + 3);
    v[0] = a.x; v[1] = a.y; v[2] = b.x; v[3] = b.y; v[4] = c.x; v[5] = c.y; v[6] = d.x; v[7] = d.y;
  } else {
#pragma unroll
    for (int t = 0; t < TI; t++) v[t] = __ldg(m + t);
  }
}

// One transform pass along axis a: out[line][i] = sum_j M[i][j] in[line][j].
// A task is (line, tile of TI consecutive outputs); tasks are line-fastest so
// the lanes of a warp share the matrix values (broadcast) and read 32
// different lines.  MT holds M transposed: MT[j*n + i].
template <class T, int TI>
__device__ __forceinline__ void dft_pass(const Layout& L, const SmemLay& S, int a, const T* MT, const T* in,
                                         T* out) {
  const int n = L.n(a);
  const int lines = L.interior() / n;
  const int tiles = n / TI;
  const int st = a == 0 ? 1 : (a == 1 ? S.sy : S.sz);
  for (int task = threadIdx.x; task < lines * tiles; task += blockDim.x) {
    int l = task % lines, i0 = (task / lines) * TI;
    int base;
    if (a == 0) {
      int y = l % L.n1, z = l / L.n1;
      base = y * S.sy + z * S.sz;
    } else if (a == 1) {
      int x = l % L.n0, z = l / L.n0;
      base = x + z * S.sz;
    } else {
      int x = l % L.n0, y = l / L.n0;
      base = x + y * S.sy;
    }
    T acc[TI];
#pragma unroll
    for (int t = 0; t < TI; t++) acc[t] = T(0);
    const T* src = in + base;
    const T* m = MT + i0;
    const bool vec = (n % 4) == 0;
#pragma unroll 4
    for (int j = 0; j < n; j++) {
      T v = src[j * st];
      T mv[TI];
      load_row<T, TI>(m + j * n, mv, vec);
#pragma unroll
      for (int t = 0; t < TI; t++) acc[t] += mv[t] * v;
    }
#pragma unroll
    for (int t = 0; t < TI; t++) out[base + (i0 + t) * st] = acc[t];
  }
}

// ti_max caps the outputs per thread: 8 for throughput on large levels,
// 1 to spread a patch over many threads on small (latency-bound) levels
template <class T>
__device__ __forceinline__ void dft_pass_any(const Layout& L, const SmemLay& S, int a, const T* MT, const T* in,
                                             T* out, int ti_max) {
  int n = L.n(a);
  if (n % 8 == 0 && ti_max >= 8)
    dft_pass<T, 8>(L, S, a, MT, in, out);
  else if (n % 4 == 0 && ti_max >= 4)
    dft_pass<T, 4>(L, S, a, MT, in, out);
  else if (n % 2 == 0 && ti_max >= 2)
    dft_pass<T, 2>(L, S, a, MT, in, out);
  else
    dft_pass<T, 1>(L, S, a, MT, in, out);
}

// outputs per thread and threads per CTA for a level of P patches
inline void dft_launch_shape(const Layout& L, int& ti_max, int& threads) {
  const bool big = L.P >= 2 * 152;
  ti_max = big ? 8 : 1;
  int best = 32;
  for (int a = 0; a < L.D; a++) {
    int n = L.n(a);
    int ti = (n % 8 == 0 && ti_max >= 8) ? 8 : (n % 4 == 0 && ti_max >= 4) ? 4 : (n % 2 == 0 && ti_max >= 2) ? 2 : 1;
    best = best > (L.interior() / n) * (n / ti) ? best : (L.interior() / n) * (n / ti);
  }
  best = (best + 31) / 32 * 32;
  int cap = big ? 256 : 1024;
  threads = best < cap ? best : cap;
}


// The whole solve of one patch held in shared memory `cur` (scratch `nxt`):
// forward transforms, multiply by 1/eigenvalue, inverse transforms.
// Returns the buffer that holds the result.  MTs: 2*D transposed matrices
// (forward axes then inverse axes) at offsets moff.
// MT[q] (q < 2D): global pointers to the transposed matrices, forward axes then inverse axes
template <class T>
__device__ T* dft_solve_smem(const Layout& L, const SmemLay& S, const T* const* MT, const T* ie, bool zero_mode,
                             T* cur, T* nxt, int ti_max) {
  const int D = L.D, N = L.interior();
  for (int a = 0; a < D; a++) {
    dft_pass_any<T>(L, S, a, MT[a], cur, nxt, ti_max);
    __syncthreads();
    T* t = cur;
    cur = nxt;
    nxt = t;
  }
  for (int e = threadIdx.x; e < N; e += blockDim.x) {
    int x = e % L.n0, r = e / L.n0, y = r % L.n1, z = r / L.n1;
    cur[x + y * S.sy + z * S.sz] *= ie[e];
  }
  __syncthreads();
  if (zero_mode && threadIdx.x == 0) cur[0] = T(0);
  __syncthreads();
  for (int a = 0; a < D; a++) {
    dft_pass_any<T>(L, S, a, MT[D + a], cur, nxt, ti_max);
    __syncthreads();
    T* t = cur;
    cur = nxt;
    nxt = t;
  }
  return cur;
}

// global pointers of the 2*D transform matrices of `plan`
template <class T>
__device__ __forceinline__ void dft_mat_ptrs(const Layout& L, int plan, const int* __restrict__ plan_mats,
                                             const T* __restrict__ mats, const int* __restrict__ mat_off,
                                             const T** MT) {
  for (int q = 0; q < 2 * L.D; q++) MT[q] = mats + mat_off[plan_mats[plan * 6 + (q / L.D) * 3 + q % L.D]];
}

}  // namespace te
