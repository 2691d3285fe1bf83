// te_runtime.cu -- library state, Domain upload and Vector<D> algebra.
//
// Vector algebra follows ThunderEgg's Vector<D> (Vector.h:391-611): every
// operation touches interior cells only (ghosts preserved) unless it is one
// of the *WithGhost variants.  Reductions accumulate in FP64 in a fixed order
// (per-block tree, then the block partials in index order), so repeated runs
// are bit-identical.

#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <algorithm>
#include <mutex>
#include <set>
#include <type_traits>

#include "te_df64.cuh"
#include "te_internal.cuh"

namespace te {

static thread_local std::string t_err;
// per thread: a worker thread can create handles bound to its own stream while other threads
// launch on theirs
static thread_local cudaStream_t g_stream = nullptr;
std::atomic<long long> g_launches{0};

void set_error(const std::string& msg) { t_err = msg; }

int guard_impl(void (*fn)(void*), void* ctx) {
  try {
    fn(ctx);
    return TE_OK;
  } catch (const Error& e) {
    t_err = e.what();
    return e.code;
  } catch (const std::exception& e) {
    t_err = e.what();
    return TE_ERR_INVALID;
  }
}

void cuda_check(cudaError_t e, const char* what) {
  if (e != cudaSuccess) throw Error(TE_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

cudaStream_t current_stream() { return g_stream; }

void allow_max_dynamic_smem(const void* kern) {
  static std::mutex mu;
  static std::set<std::pair<int, const void*>> done;
  int dev = 0;
  TE_CUDA(cudaGetDevice(&dev));
  std::lock_guard<std::mutex> lock(mu);
  if (done.count({dev, kern})) return;
  int optin = 0;
  TE_CUDA(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
  cudaFuncAttributes fa;
  TE_CUDA(cudaFuncGetAttributes(&fa, kern));
  TE_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, optin - (int)fa.sharedSizeBytes));
  done.insert({dev, kern});
}

// ---------------------------------------------------------------------------
// element access in either precision
// ---------------------------------------------------------------------------
template <class T>
struct Elem;

// Interior cells are visited one padded (patch, component) block at a time:
// block b handles blocks pc = b, b + gridDim.x, ...; threads walk its interior
// cells with 32-bit index arithmetic.
__device__ __forceinline__ int interior_offset(const Layout& L, int e) {
  int x = e % L.n0;
  int r = e / L.n0;
  int y = r % L.n1;
  int z = r / L.n1;
  return L.at(x, y, z);
}

// offset of interior cell e of a cubic patch with one ghost layer (NN cells a side), or of any
// patch through the layout (NN = 0)
template <int DIM, int NN>
__device__ __forceinline__ int cell_offset(const Layout& L, int e) {
  if constexpr (NN > 0) {
    constexpr int SY = NN + 2, SZ = DIM == 3 ? SY * SY : 0;
    const int x = e % NN, r = e / NN;
    return (x + 1) + (r % NN + 1) * SY + (DIM == 3 ? (r / NN + 1) * SZ : 0);
  } else {
    return interior_offset(L, e);
  }
}

template <class T, int OP>
__device__ __forceinline__ T vec_op(T xv, T av, T bv, double alpha, double beta, double gamma) {
  if (OP == OP_SET) xv = (T)alpha;
  if (OP == OP_SCALE) xv *= (T)alpha;
  if (OP == OP_SHIFT) xv += (T)alpha;
  if (OP == OP_COPY) xv = av;
  if (OP == OP_ADD) xv += av;
  // reference: view += b_view * alpha  (Vector.h:495)
  if (OP == OP_ADD_SCALED) xv += av * (T)alpha;
  // view += a * alpha + b * beta  (Vector.h:507-511)
  if (OP == OP_ADD_SCALED2) xv += av * (T)alpha + bv * (T)beta;
  // view = view * alpha + b  (Vector.h:523)
  if (OP == OP_SCALE_THEN_ADD) xv = xv * (T)alpha + av;
  if (OP == OP_SCALE_THEN_ADD_SCALED) xv = xv * (T)alpha + av * (T)beta;
  if (OP == OP_SCALE_THEN_ADD_SCALED2) xv = xv * (T)alpha + av * (T)beta + bv * (T)gamma;
  return xv;
}

// Each thread takes VEC_UNROLL cells of a patch-component per round and
// loads all of their operands before it computes, so several loads per thread
// are in flight; x is read only by the operations that use it.
constexpr int VEC_UNROLL = 4;
template <class T, int OP, int DIM = 0, int NN = 0>
__global__ void vec_kernel(Layout L, int npc, T* x, const T* a, const T* b, double alpha, double beta,
                           double gamma) {
  constexpr bool RX = OP != OP_SET && OP != OP_COPY;
  constexpr bool RA = OP != OP_SET && OP != OP_SCALE && OP != OP_SHIFT;
  constexpr bool RB = OP == OP_ADD_SCALED2 || OP == OP_SCALE_THEN_ADD_SCALED2;
  const int N = NN > 0 ? (DIM == 3 ? NN * NN * NN : NN * NN) : L.interior();
  const int CS = NN > 0 ? (DIM == 3 ? (NN + 2) * (NN + 2) * (NN + 2) : (NN + 2) * (NN + 2)) : L.cs;
  for (int pc = blockIdx.x; pc < npc; pc += gridDim.x) {
    const long long base = (long long)pc * CS;
    for (int e0 = threadIdx.x; e0 < N; e0 += VEC_UNROLL * blockDim.x) {
      long long kk[VEC_UNROLL];
      T xs[VEC_UNROLL], as[VEC_UNROLL], bs[VEC_UNROLL];
#pragma unroll
      for (int r = 0; r < VEC_UNROLL; r++) {
        const int e = e0 + r * blockDim.x;
        kk[r] = e < N ? base + cell_offset<DIM, NN>(L, e) : -1;
        xs[r] = RX && kk[r] >= 0 ? x[kk[r]] : T(0);
        as[r] = RA && kk[r] >= 0 ? a[kk[r]] : T(0);
        bs[r] = RB && kk[r] >= 0 ? b[kk[r]] : T(0);
      }
#pragma unroll
      for (int r = 0; r < VEC_UNROLL; r++)
        if (kk[r] >= 0) x[kk[r]] = vec_op<T, OP>(xs[r], as[r], bs[r], alpha, beta, gamma);
    }
  }
}

template <class T>
__global__ void fill_all_kernel(T* x, long long n, T v) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x)
    x[i] = v;
}

template <class TD, class TS>
__global__ void convert_kernel(TD* dst, const TS* src, long long n) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x)
    dst[i] = (TD)src[i];
}

static int grid_for(long long n, int block = 256) {
  long long g = (n + block - 1) / block;
  int cap = 152 * 16;
  return (int)(g < 1 ? 1 : (g > cap ? cap : g));
}

template <class T>
static void launch_vec(const te_domain* d, int nc, int op, T* x, const T* a, const T* b, double al,
                       double be, double ga, cudaStream_t s) {
  int npc = d->lay.P * nc;
  if (npc == 0) return;
  int grid = npc < 152 * 8 ? npc : 152 * 8;
  // cubic patches with one ghost layer: constant index arithmetic (nc == 1)
  auto run = [&](auto opc) {
    constexpr int OPV = decltype(opc)::value;
    const bool cubic = nc == 1 && with_cubic_size(d->lay, [&](auto dim, auto nn) {
                         vec_kernel<T, OPV, decltype(dim)::value, decltype(nn)::value>
                             <<<grid, 256, 0, s>>>(d->lay, npc, x, a, b, al, be, ga);
                       });
    if (!cubic) vec_kernel<T, OPV><<<grid, 256, 0, s>>>(d->lay, npc, x, a, b, al, be, ga);
  };
#define TE_VEC_CASE(OPV)  \
  case OPV:               \
    run(IntC<OPV>());     \
    break;
  switch (op) {
    TE_VEC_CASE(OP_SET)
    TE_VEC_CASE(OP_SCALE)
    TE_VEC_CASE(OP_SHIFT)
    TE_VEC_CASE(OP_COPY)
    TE_VEC_CASE(OP_ADD)
    TE_VEC_CASE(OP_ADD_SCALED)
    TE_VEC_CASE(OP_ADD_SCALED2)
    TE_VEC_CASE(OP_SCALE_THEN_ADD)
    TE_VEC_CASE(OP_SCALE_THEN_ADD_SCALED)
    TE_VEC_CASE(OP_SCALE_THEN_ADD_SCALED2)
  }
#undef TE_VEC_CASE
  count_launch();
  TE_LAUNCH_CHECK();
}

void vec_dispatch(const te_domain* d, int nc, int dtype, int op, void* x, const void* a,
                         const void* b, double al, double be, double ga) {
  require(d != nullptr && x != nullptr, "null domain or vector");
  require(nc >= 1, "ncomp must be >= 1");
  cudaStream_t s = d->stream;
  if (dtype == TE_F64)
    launch_vec<double>(d, nc, op, (double*)x, (const double*)a, (const double*)b, al, be, ga, s);
  else if (dtype == TE_F32)
    launch_vec<float>(d, nc, op, (float*)x, (const float*)a, (const float*)b, al, be, ga, s);
  else
    throw Error(TE_ERR_INVALID, "bad dtype");
}

// ---------------------------------------------------------------------------
// deterministic reductions: block tree + last-block-done final pass
// ---------------------------------------------------------------------------
constexpr int RED_THREADS = 256;

__device__ __forceinline__ double warp_sum(double v) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  return v;
}
__device__ __forceinline__ double warp_max(double v) {
  for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_down_sync(0xffffffffu, v, o));
  return v;
}

template <bool MAX>
__device__ double block_reduce(double v) {
  __shared__ double sm[RED_THREADS / 32];
  v = MAX ? warp_max(v) : warp_sum(v);
  int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  if (l == 0) sm[w] = v;
  __syncthreads();
  if (w == 0) {
    v = l < RED_THREADS / 32 ? sm[l] : (MAX ? 0.0 : 0.0);
    v = MAX ? warp_max(v) : warp_sum(v);
  }
  return v;
}

// The end of a reduction launch: the block's sum (or maximum) of t goes to partials[block];
// the last block to finish combines the partials in block order into *out.
template <int MODE>
__device__ void reduce_finish(double t, double* partials, unsigned int* counter, double* out) {
  double b = block_reduce<MODE == 1>(t);
  __shared__ bool last;
  if (threadIdx.x == 0) {
    partials[blockIdx.x] = b;
    __threadfence();
    unsigned int done = atomicAdd(counter, 1u);
    last = (done == gridDim.x - 1);
  }
  __syncthreads();
  if (last) {
    __threadfence();
    double v = 0.0;
    for (int i = threadIdx.x; i < (int)gridDim.x; i += blockDim.x) {
      double pv = ((volatile double*)partials)[i];
      v = MODE == 0 ? v + pv : fmax(v, pv);
    }
    v = block_reduce<MODE == 1>(v);
    if (threadIdx.x == 0) {
      *out = v;
      *counter = 0u;
    }
  }
}

// MODE 0: dot(x, y); MODE 1: max(x) with 0 floor (Vector::infNorm, Vector.h:568-578).
// DIM, NN > 0: cubic patches of NN cells with one ghost layer, constant index arithmetic
template <class T, int MODE, int DIM = 0, int NN = 0>
__global__ void reduce_kernel(Layout L, int npc, const T* x, const T* y, double* partials,
                              unsigned int* counter, double* out) {
  // VEC_UNROLL independent partial sums per thread (loads of a round issued
  // together), combined in a fixed order: the result depends only on the
  // level's layout and the launch shape
  // FP64 data accumulate in FP64.  FP32 data stay on the FP32 pipes (GB300's FP64 rate is
  // 1/64 of its FP32 rate): dot products accumulate in float-float with Ogita-Rump-Oishi
  // Dot2 (exact FP32 products, compensated sums; about twice FP32's precision), the
  // maximum in FP32 (exact); each thread's partials become FP64 once, at the end
  constexpr bool F32 = sizeof(T) == 4;
  double acc[VEC_UNROLL];
  dot2 acc2[VEC_UNROLL];
  float accm[VEC_UNROLL];
#pragma unroll
  for (int r = 0; r < VEC_UNROLL; r++) {
    acc[r] = 0.0;
    accm[r] = 0.f;
  }
  const int N = NN > 0 ? (DIM == 3 ? NN * NN * NN : NN * NN) : L.interior();
  const int CS = NN > 0 ? (DIM == 3 ? (NN + 2) * (NN + 2) * (NN + 2) : (NN + 2) * (NN + 2)) : L.cs;
  // the rounds (patch-component pc, first cell e0) of this thread, in order; the next round's
  // loads are issued before the current round is summed
  auto load = [&](int pc_, int e0_, T (&xs)[VEC_UNROLL], T (&ys)[VEC_UNROLL]) {
    const long long base = (long long)pc_ * CS;
#pragma unroll
    for (int r = 0; r < VEC_UNROLL; r++) {
      const int e = e0_ + r * blockDim.x;
      const long long k = pc_ < npc && e < N ? base + cell_offset<DIM, NN>(L, e) : -1;
      xs[r] = k >= 0 ? x[k] : T(0);
      ys[r] = MODE == 0 && k >= 0 ? y[k] : T(0);
    }
  };
  int pc = blockIdx.x, e0 = threadIdx.x;
  if (e0 >= N) {  // more threads than cells: this thread's first round is the next patch's
    e0 = N;
  }
  T xs[VEC_UNROLL], ys[VEC_UNROLL];
  load(pc, e0, xs, ys);
  while (pc < npc) {
    int pc1 = pc, e1 = e0 + VEC_UNROLL * blockDim.x;
    if (e1 >= N) {
      pc1 += gridDim.x;
      e1 = threadIdx.x;
    }
    T xn[VEC_UNROLL], yn[VEC_UNROLL];
    load(pc1, e1, xn, yn);
    {
#pragma unroll
      for (int r = 0; r < VEC_UNROLL; r++) {
        if (F32) {
          if (MODE == 0)
            acc2[r].add(df64((float)xs[r], 0.f), df64((float)ys[r], 0.f));
          else
            accm[r] = fmaxf((float)xs[r], accm[r]);
        } else {
          if (MODE == 0)
            acc[r] += (double)xs[r] * (double)ys[r];
          else
            acc[r] = fmax((double)xs[r], acc[r]);
        }
      }
    }
#pragma unroll
    for (int r = 0; r < VEC_UNROLL; r++) {
      xs[r] = xn[r];
      ys[r] = yn[r];
    }
    pc = pc1;
    e0 = e1;
  }
  if (F32) {
#pragma unroll
    for (int r = 0; r < VEC_UNROLL; r++) acc[r] = MODE == 0 ? df_to_double(acc2[r].value()) : (double)accm[r];
  }
  static_assert(VEC_UNROLL == 4, "the partial sums are combined as four");
  double t = MODE == 0 ? (acc[0] + acc[1]) + (acc[2] + acc[3]) : fmax(fmax(acc[0], acc[1]), fmax(acc[2], acc[3]));
  reduce_finish<MODE>(t, partials, counter, out);
}

// Dot products of cubic levels with one ghost layer, read as aligned pairs of the padded
// component: a padded row has NN + 2 cells, an even number, so a pair (2j, 2j + 1) never
// straddles two rows, and one 8-byte (FP32) or 16-byte (FP64) load brings two cells (the
// launcher uses it for FP32).  The
// ghost cells of a pair are masked to 0 (their contents are never used).  Each thread issues
// the loads of PU pairs (128 bytes of x and y) before it sums any of them: the kernel is held
// by the bytes it has in flight, and reduce_kernel keeps half as many.  FP32 products are
// summed with Dot2 as in reduce_kernel, into four partial sums per thread; the order of the
// sums depends only on the level's size and the launch shape.
template <class T, int DIM, int NN>
__global__ void __launch_bounds__(RED_THREADS, 4) dot_pairs_kernel(int npairs, const T* __restrict__ x,
                                                                  const T* __restrict__ y, double* partials,
                                                                  unsigned int* counter, double* out) {
  using V2 = typename std::conditional<sizeof(T) == 4, float2, double2>::type;
  constexpr bool F32 = sizeof(T) == 4;
  constexpr int SY = NN + 2;
  static_assert(SY % 2 == 0, "a padded row holds whole pairs");
  constexpr int CP = (DIM == 3 ? SY * SY * SY : SY * SY) / 2;  // pairs per padded component
  constexpr int PU = F32 ? 8 : 4;
  const V2* xp = reinterpret_cast<const V2*>(x);
  const V2* yp = reinterpret_cast<const V2*>(y);
  const int stride = gridDim.x * blockDim.x;
  dot2 a2[4];
  double ad[4];
#pragma unroll
  for (int r = 0; r < 4; r++) ad[r] = 0.0;
#pragma unroll 1
  for (int q0 = blockIdx.x * blockDim.x + threadIdx.x; q0 < npairs; q0 += PU * stride) {
    V2 xs[PU], ys[PU];
#pragma unroll
    for (int r = 0; r < PU; r++) {
      const int q = q0 + r * stride;
      if (q < npairs) {
        xs[r] = __ldg(xp + q);
        ys[r] = __ldg(yp + q);
      } else {
        xs[r] = V2{T(0), T(0)};
        ys[r] = V2{T(0), T(0)};
      }
    }
#pragma unroll
    for (int r = 0; r < PU; r++) {
      const int q = q0 + r * stride;
      if (q >= npairs) continue;
      const int c = 2 * (q % CP);  // first cell of the pair within its padded component
      const int cx = c % SY, rest = c / SY;
      const int cy = DIM == 3 ? rest % SY : rest, cz = DIM == 3 ? rest / SY : 1;
      const bool row = cy >= 1 && cy <= NN && cz >= 1 && cz <= NN;
      const bool in0 = row && cx >= 1, in1 = row && cx + 1 <= NN;
      const T x0 = in0 ? xs[r].x : T(0), y0 = in0 ? ys[r].x : T(0);
      const T x1 = in1 ? xs[r].y : T(0), y1 = in1 ? ys[r].y : T(0);
      if constexpr (F32) {
        a2[r % 4].add(df64(x0, 0.f), df64(y0, 0.f));
        a2[r % 4].add(df64(x1, 0.f), df64(y1, 0.f));
      } else {
        ad[r % 4] += x0 * y0;
        ad[r % 4] += x1 * y1;
      }
    }
  }
  if constexpr (F32) {
#pragma unroll
    for (int r = 0; r < 4; r++) ad[r] = df_to_double(a2[r].value());
  }
  reduce_finish<0>((ad[0] + ad[1]) + (ad[2] + ad[3]), partials, counter, out);
}

// blocks of a reduction launch: as many as are resident at once (one wave, no tail), at most
// the partials the domain holds and one per patch-component
static int red_grid(const void* kern, const te_domain* d, int npc) {
  static std::mutex mu;
  static std::map<const void*, int> occ;
  static int sms = 0;
  std::lock_guard<std::mutex> lock(mu);
  if (!sms) TE_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, 0));
  auto it = occ.find(kern);
  if (it == occ.end()) {
    int o = 0;
    TE_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&o, kern, RED_THREADS, 0));
    it = occ.emplace(kern, std::max(1, o)).first;
  }
  return std::max(1, std::min({sms * it->second, d->red_blocks, npc}));
}

static void reduce_launch(const te_domain* d, int nc, int dtype, const void* x, const void* y, int mode,
                          double* d_out, cudaStream_t s) {
  const int npc = d->lay.P * nc;
  auto run = [&](auto kern, auto* xp, auto* yp) {
    kern<<<red_grid((const void*)kern, d, npc), RED_THREADS, 0, s>>>(d->lay, npc, xp, yp, d->d_partials.p,
                                                                     d->d_counter.p, d_out);
  };
  const double *xd = (const double*)x, *yd = (const double*)y;
  const float *xf = (const float*)x, *yf = (const float*)y;
  // an FP32 dot product of buffers aligned for paired loads (device allocations are); FP64 dot
  // products keep reduce_kernel, which measured faster for them (107 vs 133 us on 23,104
  // patches of 32^2: its next round's loads are in flight while it sums the current one)
  const bool paired = mode == 0 && dtype == TE_F32 && y && ((uintptr_t)x % 8 == 0) && ((uintptr_t)y % 8 == 0) &&
                      (long long)npc * d->lay.cs < (1ll << 31) - (1ll << 24);  // pair indices (and a round past them) fit an int
  // cubic patches with one ghost layer: constant index arithmetic
  const bool cubic = with_cubic_size(d->lay, [&](auto dim, auto nn) {
    constexpr int DIM = decltype(dim)::value, NN = decltype(nn)::value;
    if (paired) {
      const int npairs = npc * ((DIM == 3 ? (NN + 2) * (NN + 2) * (NN + 2) : (NN + 2) * (NN + 2)) / 2);
      auto pr = [&](auto kern, auto* xp, auto* yp) {
        kern<<<red_grid((const void*)kern, d, npc), RED_THREADS, 0, s>>>(npairs, xp, yp, d->d_partials.p,
                                                                         d->d_counter.p, d_out);
      };
      pr(dot_pairs_kernel<float, DIM, NN>, xf, yf);
      return;
    }
    if (dtype == TE_F64) {
      if (mode == 0) run(reduce_kernel<double, 0, DIM, NN>, xd, yd);
      else run(reduce_kernel<double, 1, DIM, NN>, xd, (const double*)nullptr);
    } else {
      if (mode == 0) run(reduce_kernel<float, 0, DIM, NN>, xf, yf);
      else run(reduce_kernel<float, 1, DIM, NN>, xf, (const float*)nullptr);
    }
  });
  if (!cubic) {
    if (dtype == TE_F64) {
      if (mode == 0) run(reduce_kernel<double, 0>, xd, yd);
      else run(reduce_kernel<double, 1>, xd, (const double*)nullptr);
    } else {
      if (mode == 0) run(reduce_kernel<float, 0>, xf, yf);
      else run(reduce_kernel<float, 1>, xf, (const float*)nullptr);
    }
  }
  count_launch();
  TE_LAUNCH_CHECK();
}

void reduce_dot(const te_domain* d, int nc, int dtype, const void* x, const void* y, double* d_out,
                cudaStream_t s) {
  reduce_launch(d, nc, dtype, x, y, 0, d_out, s);
}
void reduce_max(const te_domain* d, int nc, int dtype, const void* x, double* d_out, cudaStream_t s) {
  reduce_launch(d, nc, dtype, x, nullptr, 1, d_out, s);
}

static double reduce_host(const te_domain* d, int nc, int dtype, const void* x, const void* y, int mode) {
  require(d && x, "null domain or vector");
  reduce_launch(d, nc, dtype, x, y, mode, d->d_result.p, d->stream);
  TE_CUDA(cudaMemcpyAsync(d->h_result, d->d_result.p, sizeof(double), cudaMemcpyDeviceToHost, d->stream));
  TE_CUDA(cudaStreamSynchronize(d->stream));
  return *d->h_result;
}

void convert_level(const te_domain* d, int nc, int dst_dtype, void* dst, int src_dtype, const void* src,
                   cudaStream_t s) {
  long long n = (long long)d->lay.P * d->lay.pstride(nc);
  int grid = grid_for(n);
  if (dst_dtype == TE_F32 && src_dtype == TE_F64)
    convert_kernel<float, double><<<grid, 256, 0, s>>>((float*)dst, (const double*)src, n);
  else if (dst_dtype == TE_F64 && src_dtype == TE_F32)
    convert_kernel<double, float><<<grid, 256, 0, s>>>((double*)dst, (const float*)src, n);
  else if (dst_dtype == src_dtype) {
    TE_CUDA(cudaMemcpyAsync(dst, src, n * (dst_dtype == TE_F64 ? 8 : 4), cudaMemcpyDeviceToDevice, s));
    return;
  } else
    throw Error(TE_ERR_INVALID, "bad dtype");
  count_launch();
  TE_LAUNCH_CHECK();
}

}  // namespace te

te_domain::~te_domain() {
  if (h_result) cudaFreeHost(h_result);
}

using namespace te;

// ===========================================================================
// C ABI
// ===========================================================================
extern "C" {

const char* te_last_error_message(void) { return t_err.c_str(); }

int te_set_stream(void* s) {
  g_stream = (cudaStream_t)s;
  return TE_OK;
}

int te_synchronize(void) {
  return guard([&] { TE_CUDA(cudaStreamSynchronize(g_stream)); });
}

long long te_kernel_launch_count(void) { return g_launches.load(); }

int te_domain_create(const te_level_desc* desc, te_domain** out) {
  return guard([&] {
    require(desc && out, "null argument");
    require(desc->dim == 2 || desc->dim == 3, "dim must be 2 or 3");
    require(desc->num_ghost >= 1, "num_ghost must be >= 1");
    require(desc->num_patches >= 1, "num_patches must be >= 1");
    auto d = std::make_unique<te_domain>();
    int D = desc->dim, P = desc->num_patches;
    d->stream = g_stream;
    Layout& L = d->lay;
    L.D = D;
    L.n0 = desc->ns[0];
    L.n1 = D > 1 ? desc->ns[1] : 1;
    L.n2 = D > 2 ? desc->ns[2] : 1;
    for (int a = 0; a < D; a++) require(desc->ns[a] >= 1, "ns must be >= 1");
    L.g = desc->num_ghost;
    L.P = P;
    int g = L.g;
    L.sy = L.n0 + 2 * g;
    L.sz = D > 2 ? L.sy * (L.n1 + 2 * g) : 0;
    L.cs = D > 2 ? L.sz * (L.n2 + 2 * g) : L.sy * (L.n1 + 2 * g);
    if (D == 2) L.sz = 0;
    int F = num_slots(D), C = 1 << D;
    d->F = F;
    d->id.assign(desc->id, desc->id + P);
    d->refine_level.assign(desc->refine_level, desc->refine_level + P);
    d->parent_id.assign(desc->parent_id, desc->parent_id + P);
    d->orth_on_parent.assign(desc->orth_on_parent, desc->orth_on_parent + P);
    d->child_ids.assign(desc->child_ids, desc->child_ids + (size_t)P * C);
    d->starts.assign(desc->starts, desc->starts + (size_t)P * D);
    d->spacings.assign(desc->spacings, desc->spacings + (size_t)P * D);
    d->nbr_type.assign(desc->nbr_type, desc->nbr_type + (size_t)P * F);
    d->nbr_ids.assign(desc->nbr_ids, desc->nbr_ids + (size_t)P * F * 4);
    d->nbr_orth.assign(desc->nbr_orth, desc->nbr_orth + (size_t)P * F);
    // Domain::indexPatchesLocal (Domain.h:94-110): local index = position
    d->id2l.reserve((size_t)P * 2);
    for (int p = 0; p < P; p++) {
      require(d->id2l.count(d->id[p]) == 0, "duplicate patch id");
      d->id2l[d->id[p]] = p;
    }
    d->nbr_local.assign((size_t)P * F * 4, -1);
    for (int p = 0; p < P; p++)
      for (int s = 0; s < F; s++) {
        int t = d->nbr_type[(size_t)p * F + s];
        if (t < 0) continue;
        require(t <= 2, "bad neighbour type");
        int nn = 1;
        if (t == TE_NBR_FINE) {
          int M = (D == 2) ? (s < 4 ? 0 : 1) : (s < 8 ? 0 : (s < 20 ? 1 : 2));
          nn = 1 << M;
        }
        for (int i = 0; i < nn; i++) {
          auto it = d->id2l.find(d->nbr_ids[((size_t)p * F + s) * 4 + i]);
          require(it != d->id2l.end(), "neighbour id not on this level (multi-rank meshes are not supported)");
          d->nbr_local[((size_t)p * F + s) * 4 + i] = it->second;
        }
      }
    cudaStream_t st = d->stream;
    std::vector<int8_t> t8(d->nbr_type.begin(), d->nbr_type.end()), o8(d->nbr_orth.begin(), d->nbr_orth.end());
    d->d_nbr_type.upload(t8, st);
    d->d_nbr_orth.upload(o8, st);
    d->d_nbr_local.upload(d->nbr_local, st);
    d->d_spacings.upload(d->spacings, st);
    std::vector<float> spf(d->spacings.begin(), d->spacings.end());
    d->d_spacings_f.upload(spf, st);
    std::vector<double> inv((size_t)P * 6, 1.0);
    for (int p = 0; p < P; p++)
      for (int a = 0; a < D; a++) {
        double h = d->spacings[(size_t)p * D + a];
        inv[(size_t)p * 6 + a] = 1.0 / (h * h);
        inv[(size_t)p * 6 + 3 + a] = 1.0 / (2.0 * h * h);
      }
    d->d_inv.upload(inv, st);
    d->d_inv_f.upload(std::vector<float>(inv.begin(), inv.end()), st);
    std::vector<float> inv_df(2 * inv.size());
    for (size_t i = 0; i < inv.size(); i++) {
      float h = (float)inv[i];
      inv_df[2 * i] = h;
      inv_df[2 * i + 1] = (float)(inv[i] - (double)h);
    }
    d->d_inv_df.upload(inv_df, st);
    d->red_blocks = 152 * 8;
    d->d_partials.alloc(d->red_blocks);
    d->d_counter.alloc(1);
    TE_CUDA(cudaMemsetAsync(d->d_counter.p, 0, sizeof(unsigned int), st));
    d->d_result.alloc(1);
    TE_CUDA(cudaMallocHost(&d->h_result, sizeof(double)));
    TE_CUDA(cudaStreamSynchronize(st));
    *out = d.release();
  });
}

int te_domain_destroy(te_domain* d) {
  delete d;
  return TE_OK;
}

long long te_domain_patch_stride(const te_domain* d, int ncomp) { return d ? d->lay.pstride(ncomp) : -1; }
int te_domain_num_patches(const te_domain* d) { return d ? d->lay.P : -1; }

int te_level_alloc(const te_domain* d, int nc, int dt, void** out) {
  return guard([&] {
    require(d && out, "null argument");
    require(nc >= 1, "ncomp must be >= 1");
    require(dt == TE_F64 || dt == TE_F32, "bad dtype");
    const size_t bytes = (size_t)d->lay.P * d->lay.pstride(nc) * (dt == TE_F64 ? 8 : 4);
    void* p = nullptr;
    cuda_check(cudaMalloc(&p, bytes), "cudaMalloc (level buffer)");
    const cudaError_t e = cudaMemsetAsync(p, 0, bytes, d->stream);
    if (e == cudaSuccess) {
      const cudaError_t e2 = cudaStreamSynchronize(d->stream);
      if (e2 != cudaSuccess) {
        cudaFree(p);
        cuda_check(e2, "cudaStreamSynchronize (level buffer)");
      }
    } else {
      cudaFree(p);
      cuda_check(e, "cudaMemsetAsync (level buffer)");
    }
    *out = p;
  });
}

int te_device_alloc(size_t bytes, void** out) {
  return guard([&] {
    require(out, "null argument");
    void* p = nullptr;
    if (bytes) cuda_check(cudaMalloc(&p, bytes), "cudaMalloc");
    *out = p;
  });
}

int te_device_free(void* p) {
  return guard([&] {
    if (p) cuda_check(cudaFree(p), "cudaFree");
  });
}

int te_copy(void* dst, const void* src, size_t bytes) {
  return guard([&] {
    require((dst && src) || !bytes, "null argument");
    if (bytes) cuda_check(cudaMemcpy(dst, src, bytes, cudaMemcpyDefault), "cudaMemcpy");
  });
}

int te_level_free(void* p) {
  return guard([&] {
    if (p) cuda_check(cudaFree(p), "cudaFree (level buffer)");
  });
}

int te_vec_set(const te_domain* d, int nc, int dt, void* x, double alpha, int with_ghost) {
  return guard([&] {
    require(d && x, "null argument");
    if (with_ghost) {  // Vector::setWithGhost (Vector.h:404-412)
      long long n = (long long)d->lay.P * d->lay.pstride(nc);
      if (dt == TE_F64)
        fill_all_kernel<double><<<grid_for(n), 256, 0, d->stream>>>((double*)x, n, alpha);
      else
        fill_all_kernel<float><<<grid_for(n), 256, 0, d->stream>>>((float*)x, n, (float)alpha);
      count_launch();
      TE_LAUNCH_CHECK();
    } else {
      vec_dispatch(d, nc, dt, OP_SET, x, nullptr, nullptr, alpha, 0, 0);
    }
  });
}
int te_vec_scale(const te_domain* d, int nc, int dt, void* x, double alpha) {
  return guard([&] { vec_dispatch(d, nc, dt, OP_SCALE, x, nullptr, nullptr, alpha, 0, 0); });
}
int te_vec_shift(const te_domain* d, int nc, int dt, void* x, double delta) {
  return guard([&] { vec_dispatch(d, nc, dt, OP_SHIFT, x, nullptr, nullptr, delta, 0, 0); });
}
int te_vec_copy(const te_domain* d, int nc, int dt, void* x, const void* b, int with_ghost) {
  return guard([&] {
    require(d && x && b, "null argument");
    if (with_ghost) {  // Vector::copyWithGhost (Vector.h:455-463)
      long long n = (long long)d->lay.P * d->lay.pstride(nc);
      TE_CUDA(cudaMemcpyAsync(x, b, n * (dt == TE_F64 ? 8 : 4), cudaMemcpyDeviceToDevice, d->stream));
    } else {
      vec_dispatch(d, nc, dt, OP_COPY, x, b, nullptr, 0, 0, 0);
    }
  });
}
int te_vec_add(const te_domain* d, int nc, int dt, void* x, const void* b) {
  return guard([&] { vec_dispatch(d, nc, dt, OP_ADD, x, b, nullptr, 0, 0, 0); });
}
int te_vec_add_scaled(const te_domain* d, int nc, int dt, void* x, double alpha, const void* a) {
  return guard([&] { vec_dispatch(d, nc, dt, OP_ADD_SCALED, x, a, nullptr, alpha, 0, 0); });
}
int te_vec_add_scaled2(const te_domain* d, int nc, int dt, void* x, double alpha, const void* a, double beta,
                       const void* b) {
  return guard([&] { vec_dispatch(d, nc, dt, OP_ADD_SCALED2, x, a, b, alpha, beta, 0); });
}
int te_vec_scale_then_add(const te_domain* d, int nc, int dt, void* x, double alpha, const void* b) {
  return guard([&] { vec_dispatch(d, nc, dt, OP_SCALE_THEN_ADD, x, b, nullptr, alpha, 0, 0); });
}
int te_vec_scale_then_add_scaled(const te_domain* d, int nc, int dt, void* x, double alpha, double beta,
                                 const void* b) {
  return guard([&] { vec_dispatch(d, nc, dt, OP_SCALE_THEN_ADD_SCALED, x, b, nullptr, alpha, beta, 0); });
}
int te_vec_scale_then_add_scaled2(const te_domain* d, int nc, int dt, void* x, double alpha, double beta,
                                  const void* b, double gamma, const void* c) {
  return guard([&] { vec_dispatch(d, nc, dt, OP_SCALE_THEN_ADD_SCALED2, x, b, c, alpha, beta, gamma); });
}
int te_vec_two_norm(const te_domain* d, int nc, int dt, const void* x, double* out) {
  return guard([&] {
    require(out != nullptr, "null output");
    *out = std::sqrt(reduce_host(d, nc, dt, x, x, 0));
  });
}
int te_vec_inf_norm(const te_domain* d, int nc, int dt, const void* x, double* out) {
  return guard([&] {
    require(out != nullptr, "null output");
    *out = reduce_host(d, nc, dt, x, nullptr, 1);
  });
}
int te_vec_dot(const te_domain* d, int nc, int dt, const void* x, const void* b, double* out) {
  return guard([&] {
    require(out != nullptr && b != nullptr, "null argument");
    *out = reduce_host(d, nc, dt, x, b, 0);
  });
}
int te_vec_convert(const te_domain* d, int nc, int dst_dtype, void* dst, int src_dtype, const void* src) {
  return guard([&] {
    require(d && dst && src, "null argument");
    convert_level(d, nc, dst_dtype, dst, src_dtype, src, d->stream);
  });
}

}  // extern "C"
