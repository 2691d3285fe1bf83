// te_internal.cuh -- shared internals of the te_gpu library (not part of the ABI).
#pragma once

#include <cuda_runtime.h>

#include <atomic>
#include <cstdint>
#include <cstdlib>
#include <map>
#include <memory>
#include <stdexcept>
#include <string>
#include <type_traits>
#include <unordered_map>
#include <vector>

#include "te_gpu.h"

namespace te {

// ---------------------------------------------------------------------------
// errors: every ABI entry point runs its body through guard(); failures are
// thrown as te::Error and turned into a status code + message.
// ---------------------------------------------------------------------------
struct Error : std::runtime_error {
  int code;
  Error(int code, const std::string& msg) : std::runtime_error(msg), code(code) {}
};
void set_error(const std::string& msg);
int guard_impl(void (*fn)(void*), void* ctx);
template <class F>
int guard(F&& f) {
  return guard_impl([](void* c) { (*static_cast<F*>(c))(); }, &f);
}
void cuda_check(cudaError_t e, const char* what);
#define TE_CUDA(call) ::te::cuda_check((call), #call)
inline void require(bool ok, const std::string& msg, int code = TE_ERR_INVALID) {
  if (!ok) throw Error(code, msg);
}

// current stream for newly created handles; launch accounting
cudaStream_t current_stream();
// Raise a kernel's dynamic shared-memory limit, once, to the device's opt-in maximum.  The
// limit belongs to the function, not to a launch: setting it per launch to that launch's size
// would let a later, smaller setting invalidate a launch recorded earlier in a CUDA graph.
// The shared memory each launch requests still sets its occupancy.
void allow_max_dynamic_smem(const void* kern);
extern std::atomic<long long> g_launches;
inline void count_launch(int n = 1) { g_launches.fetch_add(n, std::memory_order_relaxed); }
#define TE_LAUNCH_CHECK() ::te::cuda_check(cudaGetLastError(), "kernel launch")

// ---------------------------------------------------------------------------
// device buffers
// ---------------------------------------------------------------------------
template <class T>
struct DevBuf {
  T* p = nullptr;
  size_t n = 0;
  DevBuf() = default;
  explicit DevBuf(size_t count) { alloc(count); }
  DevBuf(const DevBuf&) = delete;
  DevBuf& operator=(const DevBuf&) = delete;
  DevBuf(DevBuf&& o) noexcept : p(o.p), n(o.n) { o.p = nullptr; o.n = 0; }
  DevBuf& operator=(DevBuf&& o) noexcept {
    if (this != &o) {
      release();
      p = o.p;
      n = o.n;
      o.p = nullptr;
      o.n = 0;
    }
    return *this;
  }
  ~DevBuf() { release(); }
  void alloc(size_t count) {
    release();
    n = count;
    if (count) TE_CUDA(cudaMalloc(&p, count * sizeof(T)));
  }
  void release() {
    if (p) cudaFree(p);
    p = nullptr;
    n = 0;
  }
  void upload(const std::vector<T>& h, cudaStream_t s) {
    if (h.size() != n) alloc(h.size());
    if (n) TE_CUDA(cudaMemcpyAsync(p, h.data(), n * sizeof(T), cudaMemcpyHostToDevice, s));
  }
};

// ---------------------------------------------------------------------------
// level layout (ThunderEgg Vector<D>, Vector.h:133-153), passed by value to kernels
// ---------------------------------------------------------------------------
struct Layout {
  int D;
  int n0, n1, n2;  // cells per axis (n1 = n2 = 1 beyond D)
  int g;           // ghost layers
  int P;           // patches
  int sy, sz;      // strides of axis 1 and 2 (axis 0 stride is 1)
  int cs;          // cells of one padded component
  __host__ __device__ long long pstride(int nc) const { return (long long)cs * nc; }
  __host__ __device__ int at(int x, int y, int z) const {
    return (x + g) + (y + g) * sy + (z + g) * sz;
  }
  __host__ __device__ int interior() const { return n0 * n1 * n2; }
  __host__ __device__ int n(int a) const { return a == 0 ? n0 : (a == 1 ? n1 : n2); }
  __host__ __device__ int stride(int a) const { return a == 0 ? 1 : (a == 1 ? sy : sz); }
};

// Level kernels with constant index arithmetic exist for cubic patches with
// one ghost layer of 8, 16, 32 or 64 cells (2D) and 8 or 16 cells (3D).
// with_cubic_size calls fn(IntC<DIM>(), IntC<NN>()) for such a level and
// returns true; otherwise it returns false and the caller launches the
// general kernel.  TE_GENERIC_LEVEL_KERNELS=1 keeps the general kernels.
template <int V>
using IntC = std::integral_constant<int, V>;
inline bool generic_level_kernels() {
  static const bool on = [] {
    const char* e = getenv("TE_GENERIC_LEVEL_KERNELS");
    return e && e[0] == '1';
  }();
  return on;
}
template <class Fn>
bool with_cubic_size(const Layout& L, Fn&& fn) {
  if (generic_level_kernels() || L.g != 1 || L.n0 != L.n1 || (L.D == 3 && L.n1 != L.n2)) return false;
  if (L.D == 2) {
    switch (L.n0) {
      case 8: fn(IntC<2>(), IntC<8>()); return true;
      case 16: fn(IntC<2>(), IntC<16>()); return true;
      case 32: fn(IntC<2>(), IntC<32>()); return true;
      case 64: fn(IntC<2>(), IntC<64>()); return true;
    }
  } else if (L.D == 3) {
    switch (L.n0) {
      case 8: fn(IntC<3>(), IntC<8>()); return true;
      case 16: fn(IntC<3>(), IntC<16>()); return true;
    }
  }
  return false;
}

inline int num_slots(int D) { return D == 2 ? 8 : 26; }
inline int sum_of_faces(int D, int M) {
  if (D == 2) return M == 0 ? 0 : 4;
  return M == 0 ? 0 : (M == 1 ? 8 : 20);
}
inline int num_faces(int D, int M) {
  if (D == 2) return 4;
  return M == 0 ? 8 : (M == 1 ? 12 : 6);
}

}  // namespace te

// ---------------------------------------------------------------------------
// handles
// ---------------------------------------------------------------------------
struct te_domain {
  te::Layout lay;
  int F = 8;
  cudaStream_t stream = nullptr;
  // host copies of the level tables
  std::vector<int> id, refine_level, parent_id, orth_on_parent, child_ids, nbr_type, nbr_ids, nbr_orth,
      nbr_local;
  std::vector<double> starts, spacings;
  std::unordered_map<int, int> id2l;
  // device copies
  te::DevBuf<int8_t> d_nbr_type;   // [P*F]
  te::DevBuf<int8_t> d_nbr_orth;   // [P*F]
  te::DevBuf<int> d_nbr_local;     // [P*F*4]
  te::DevBuf<double> d_spacings;   // [P*D]
  te::DevBuf<float> d_spacings_f;  // [P*D]
  // per patch and axis: 1/h^2 (Poisson) and 1/(2 h^2) (VarPoisson), [P*6], in both precisions
  te::DevBuf<double> d_inv;
  te::DevBuf<float> d_inv_f;
  te::DevBuf<float> d_inv_df;  // [P*6][2]: float-float split (hi, lo) of d_inv
  template <class T>
  const T* inv() const;
  // reduction scratch: per-block partials + completion counter + result
  te::DevBuf<double> d_partials;
  te::DevBuf<unsigned int> d_counter;
  te::DevBuf<double> d_result;
  double* h_result = nullptr;  // pinned
  int red_blocks = 0;
  bool has_nbr_slot(int p, int slot) const { return nbr_type[(size_t)p * F + slot] >= 0; }
  ~te_domain();
};

template <>
inline const double* te_domain::inv<double>() const { return d_inv.p; }
template <>
inline const float* te_domain::inv<float>() const { return d_inv_f.p; }

namespace te {
enum VecOp {
  OP_SET,
  OP_SCALE,
  OP_SHIFT,
  OP_COPY,
  OP_ADD,
  OP_ADD_SCALED,
  OP_ADD_SCALED2,
  OP_SCALE_THEN_ADD,
  OP_SCALE_THEN_ADD_SCALED,
  OP_SCALE_THEN_ADD_SCALED2
};
// Vector<D> algebra on interior cells (Vector.h:391-611)
void vec_dispatch(const te_domain* d, int nc, int dtype, int op, void* x, const void* a, const void* b,
                  double al, double be, double ga);
// reductions used by the vector ABI and the Krylov solver
void reduce_dot(const te_domain* d, int nc, int dtype, const void* x, const void* y, double* d_out,
                cudaStream_t s);
void reduce_max(const te_domain* d, int nc, int dtype, const void* x, double* d_out, cudaStream_t s);
// level buffer conversion
void convert_level(const te_domain* d, int nc, int dst_dtype, void* dst, int src_dtype, const void* src,
                   cudaStream_t s);
}  // namespace te
