// te_noalloc.cu -- a dot product of two level buffers that allocates nothing.
//
// Some callers cannot call cudaMalloc at the point where they need a
// reduction: hosts whose device memory is owned by another allocator (a pool
// that reserved the GPU's memory at start-up and forbids raw cudaMalloc after
// it), or callers that must not pay the device-wide synchronisation that
// cudaMalloc/cudaFree can cause while other streams are running.  For them,
// te_level_dot_noalloc takes only the level layout and two device buffers and
// keeps its scratch in a fixed, file-scope device array.
//
// The scratch is TE_NOALLOC_MAX_PARTIALS + 1 doubles (512 KiB + 8 bytes): one
// partial sum per (patch, component) plus the result.  Every GPU that loads
// this library holds that array until the process exits.  Calls share it, so
// calls whose work overlaps on the GPU (different streams, or threads) race;
// serialise them.  Nothing in it has to start at zero: each call writes every
// slot it later reads.  The device address of the array is looked up once per
// device, on the first call made with that device current; make that first
// call before starting any stream capture.  The call ends by copying the
// result to the host and synchronising the caller's stream.

#include <cuda_runtime.h>

#include <mutex>

#include "te_internal.cuh"

namespace {

__device__ __align__(256) double g_noalloc_scratch[TE_NOALLOC_MAX_PARTIALS + 1];

constexpr int kMaxDevices = 64;
double* g_scratch_ptr[kMaxDevices] = {nullptr};
std::mutex g_scratch_mu;

// device address of the scratch array for the current device (set up once)
double* scratch_for_current_device() {
  int dev = 0;
  te::cuda_check(cudaGetDevice(&dev), "cudaGetDevice");
  te::require(dev >= 0 && dev < kMaxDevices, "device index out of range for the no-allocation scratch table");
  std::lock_guard<std::mutex> lock(g_scratch_mu);
  if (!g_scratch_ptr[dev]) {
    void* p = nullptr;
    te::cuda_check(cudaGetSymbolAddress(&p, g_noalloc_scratch), "cudaGetSymbolAddress(g_noalloc_scratch)");
    g_scratch_ptr[dev] = static_cast<double*>(p);
  }
  return g_scratch_ptr[dev];
}

constexpr int kThreads = 256;

__device__ __forceinline__ double block_sum(double v) {
  __shared__ double red[kThreads / 32];
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
  __syncthreads();
  double s = 0;
  if (threadIdx.x == 0)
    for (int w = 0; w < kThreads / 32; w++) s += red[w];
  return s;
}

// one block per (patch, component): its interior dot product into scratch[pc]
template <class T>
__global__ void __launch_bounds__(kThreads) dot_partials(te::Layout L, const T* x, const T* y, double* scratch) {
  const int pc = blockIdx.x;
  const long long base = (long long)pc * L.cs;
  double acc = 0;
  for (int e = threadIdx.x; e < L.interior(); e += blockDim.x) {
    int xx = e % L.n0, r = e / L.n0, yy = r % L.n1, zz = r / L.n1;
    long long k = base + L.at(xx, yy, zz);
    acc += (double)x[k] * (double)y[k];
  }
  double s = block_sum(acc);
  if (threadIdx.x == 0) scratch[pc] = s;
}

// fixed-order sum of the partials into scratch[TE_NOALLOC_MAX_PARTIALS]
__global__ void __launch_bounds__(kThreads) dot_final(int npc, double* scratch) {
  __shared__ double fin[kThreads];
  double s = 0;
  for (int i = threadIdx.x; i < npc; i += blockDim.x) s += scratch[i];
  fin[threadIdx.x] = s;
  __syncthreads();
  for (int w = kThreads / 2; w > 0; w >>= 1) {
    if ((int)threadIdx.x < w) fin[threadIdx.x] += fin[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) scratch[TE_NOALLOC_MAX_PARTIALS] = fin[0];
}

}  // namespace

extern "C" int te_level_dot_noalloc(int dim, const int* ns, int num_ghost, int num_patches, int ncomp, int dtype,
                                    const void* x, const void* y, double* out, void* cuda_stream) {
  return te::guard([&] {
    te::require(ns && x && y && out, "null argument");
    te::require(dim == 2 || dim == 3, "dim must be 2 or 3");
    te::require(num_ghost >= 1 && num_patches >= 1 && ncomp >= 1, "num_ghost, num_patches and ncomp must be >= 1");
    te::require(dtype == TE_F64 || dtype == TE_F32, "bad dtype");
    long long npc = (long long)num_patches * ncomp;
    te::require(npc <= TE_NOALLOC_MAX_PARTIALS,
                "te_level_dot_noalloc: num_patches * ncomp = " + std::to_string(npc) + " exceeds the limit of " +
                    std::to_string(TE_NOALLOC_MAX_PARTIALS) + " (its fixed scratch array)",
                TE_ERR_UNSUPPORTED);
    te::Layout L;
    L.D = dim;
    L.n0 = ns[0];
    L.n1 = dim > 1 ? ns[1] : 1;
    L.n2 = dim > 2 ? ns[2] : 1;
    te::require(L.n0 >= 1 && L.n1 >= 1 && L.n2 >= 1, "ns must be >= 1");
    L.g = num_ghost;
    L.P = num_patches;
    L.sy = L.n0 + 2 * L.g;
    L.sz = dim > 2 ? L.sy * (L.n1 + 2 * L.g) : 0;
    L.cs = dim > 2 ? L.sz * (L.n2 + 2 * L.g) : L.sy * (L.n1 + 2 * L.g);
    double* scratch = scratch_for_current_device();
    cudaStream_t s = static_cast<cudaStream_t>(cuda_stream);
    if (dtype == TE_F64)
      dot_partials<double><<<(int)npc, kThreads, 0, s>>>(L, (const double*)x, (const double*)y, scratch);
    else
      dot_partials<float><<<(int)npc, kThreads, 0, s>>>(L, (const float*)x, (const float*)y, scratch);
    te::cuda_check(cudaGetLastError(), "dot_partials launch");
    dot_final<<<1, kThreads, 0, s>>>((int)npc, scratch);
    te::cuda_check(cudaGetLastError(), "dot_final launch");
    te::count_launch(2);
    te::cuda_check(cudaMemcpyAsync(out, scratch + TE_NOALLOC_MAX_PARTIALS, sizeof(double), cudaMemcpyDeviceToHost, s),
                   "copy result");
    te::cuda_check(cudaStreamSynchronize(s), "cudaStreamSynchronize");
  });
}
