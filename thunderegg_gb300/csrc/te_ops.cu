// te_ops.cu -- star operators, DFT patch solver and BiCGStab patch solver.
//
// Operators (one CTA per patch):
//   Poisson::StarPatchOperator::applySinglePatch (Poisson/StarPatchOperator.h:75-144)
//   VarPoisson::StarPatchOperator::applySinglePatch (VarPoisson/StarPatchOperator.h:78-133)
//   modifyRHSForInternalBoundaryConditions (Poisson :165-180, VarPoisson :134-153)
// Patch solvers (one CTA per patch, block Jacobi over the level):
//   Poisson::DFTPatchSolver::solveSinglePatch (Poisson/DFTPatchSolver.h:420-450): the
//     n x n sine/cosine transform matrices are applied along each axis from
//     shared memory (the reference calls dgemv_ per line)
//   Iterative::PatchSolver::solveSinglePatch (Iterative/PatchSolver.h:134-175) with the
//     inner BiCGStab (Iterative/BiCGStab.h:111-203): the whole Krylov state of one
//     patch lives in shared memory; reductions are block-level, FP64, fixed order.

#include <cmath>
#include <cstring>
#include <map>
#include <tuple>

#include "te_dft.cuh"
#include "te_ops.cuh"
#include "te_tune.cuh"

namespace te {

__device__ __forceinline__ void decompose(const Layout& L, int e, int& x, int& y, int& z) {
  x = e % L.n0;
  int r = e / L.n0;
  y = r % L.n1;
  z = r / L.n1;
}

// ghost value for a side that has no neighbour: -interior (Dirichlet) or
// +interior (Neumann) (enforceBoundaryConditions); sides with a neighbour get
// -interior only when `internal` (enforceInternalBoundaryConditions)
template <class T>
__device__ void enforce_bc(const Layout& L, const int8_t* ntype, int F, int p, int nc, bool neumann,
                           bool internal, T* u) {
  int D = L.D;
  int side_slot0 = D == 2 ? 4 : 20;
  for (int side = 0; side < 2 * D; side++) {
    bool has = ntype[(size_t)p * F + side_slot0 + side] >= 0;
    if (has && !internal) continue;
    bool copy = !has && neumann;
    int axis = side >> 1, up = side & 1;
    int t0 = axis == 0 ? 1 : 0, t1 = axis == 2 ? 1 : 2;
    int n0 = L.n(t0), n1 = D == 3 ? L.n(t1) : 1;
    int cnt = n0 * n1 * nc;
    for (int e = threadIdx.x; e < cnt; e += blockDim.x) {
      int c = e / (n0 * n1), r = e % (n0 * n1), i = r % n0, j = r / n0;
      int cc[3];
      cc[t0] = i;
      if (D == 3) cc[t1] = j;
      if (D == 2) cc[2] = 0;
      cc[axis] = up ? L.n(axis) - 1 : 0;
      int in = L.at(cc[0], cc[1], cc[2]);
      cc[axis] = up ? L.n(axis) : -1;
      int gh = L.at(cc[0], cc[1], cc[2]);
      T v = u[(long long)c * L.cs + in];
      u[(long long)c * L.cs + gh] = copy ? v : -v;
    }
  }
}

// one interior cell of the star stencil; f = sum over axes, axis 0 first
template <class T, int KIND>
__device__ __forceinline__ T stencil(const Layout& L, const T* u, const T* c, int k, const T* inv) {
  T r = T(0);
#pragma unroll
  for (int a = 0; a < 3; a++) {
    if (a >= L.D) break;
    int st = L.stride(a);
    T lo = u[k - st], mid = u[k], hi = u[k + st];
    if (KIND == 0) {
      r += ((hi - T(2) * mid) + lo) * inv[a];
    } else {
      T cl = c[k - st], cm = c[k], cu = c[k + st];
      r += ((cu + cm) * (hi - mid) - (cl + cm) * (mid - lo)) * inv[a];
    }
  }
  return r;
}

template <class T, int KIND>
__global__ void __launch_bounds__(256)
    apply_kernel(Layout L, int nc, const int8_t* __restrict__ ntype, int F, const T* __restrict__ sp,
                 int neumann, const T* __restrict__ coeff, T* u, T* __restrict__ f) {
  int p = blockIdx.x;
  long long ps = L.pstride(nc);
  T* up = u + p * ps;
  T* fp = f + p * ps;
  const T* cp = KIND ? coeff + (long long)p * L.cs : nullptr;
  enforce_bc<T>(L, ntype, F, p, nc, neumann != 0, false, up);
  __syncthreads();
  T inv[3];
  for (int a = 0; a < 3; a++) inv[a] = sp[(size_t)p * 6 + (KIND ? 3 : 0) + a];
  const int py = L.n1 + 2 * L.g;
  const int tot = L.cs * nc;
  for (int e = threadIdx.x; e < tot; e += blockDim.x) {
    int c = e / L.cs, k = e - c * L.cs;
    int x = k % L.sy - L.g;
    int q = k / L.sy;
    int y = q % py - L.g;
    int z = q / py - (L.D == 3 ? L.g : 0);
    bool interior = x >= 0 && x < L.n0 && y >= 0 && y < L.n1 && z >= 0 && z < L.n2;
    T v = T(0);
    if (interior) v = stencil<T, KIND>(L, up + c * L.cs, cp, k, inv);
    fp[e] = v;
  }
}

// modifyRHSForInternalBoundaryConditions for one interior cell: sides in Side order
template <class T, int KIND>
__device__ __forceinline__ T modify_cell(const Layout& L, const int8_t* ntype, int F, int p, const T* u,
                                         const T* c, int x, int y, int z, int k, T fv, const T* inv) {
  int D = L.D;
  int side_slot0 = D == 2 ? 4 : 20;
  int cc[3] = {x, y, z};
  for (int side = 0; side < 2 * D; side++) {
    int axis = side >> 1, upr = side & 1;
    if (cc[axis] != (upr ? L.n(axis) - 1 : 0)) continue;
    if (ntype[(size_t)p * F + side_slot0 + side] < 0) continue;
    int gk = k + (upr ? L.stride(axis) : -L.stride(axis));
    if (KIND == 0)
      fv -= (u[gk] + u[k]) * inv[axis];
    else
      fv -= (u[gk] + u[k]) * (c[k] + c[gk]) * inv[axis];
  }
  return fv;
}

template <class T, int KIND>
__global__ void modify_rhs_kernel(Layout L, int nc, const int8_t* __restrict__ ntype, int F,
                                  const T* __restrict__ sp, const T* __restrict__ coeff, const T* u, T* f) {
  int p = blockIdx.x;
  long long ps = L.pstride(nc);
  T inv[3];
  for (int a = 0; a < 3; a++) inv[a] = sp[(size_t)p * 6 + (KIND ? 3 : 0) + a];
  int N = L.interior();
  const T* cp = KIND ? coeff + (long long)p * L.cs : nullptr;
  for (int e = threadIdx.x; e < N * nc; e += blockDim.x) {
    int c = e / N, x, y, z;
    decompose(L, e % N, x, y, z);
    int k = L.at(x, y, z);
    const T* uc = u + p * ps + (long long)c * L.cs;
    T* fc = f + p * ps + (long long)c * L.cs;
    fc[k] = modify_cell<T, KIND>(L, ntype, F, p, uc, cp, x, y, z, k, fc[k], inv);
  }
}

// apply_kernel for cubic patches of NN cells with one ghost layer: the same
// per-cell arithmetic with constant strides (stencil_n, te_ops.cuh); a thread
// loads all of its cells' stencils before it stores, so each thread keeps
// several loads in flight.
template <class T, int KIND, int DIM, int NN>
__global__ void __launch_bounds__(256)
    apply_n_kernel(Layout L, int nc, const int8_t* __restrict__ ntype, int F, const T* __restrict__ sp,
                   int neumann, const T* __restrict__ coeff, T* u, T* __restrict__ f,
                   const T* __restrict__ rhs) {
  constexpr int SY = NN + 2, SZ = DIM == 3 ? SY * SY : 0, CS = DIM == 3 ? SY * SY * SY : SY * SY;
  constexpr int PER = (CS + 255) / 256;
  const int p = blockIdx.x;
  T* up = u + (long long)p * CS * nc;
  T* fp = f + (long long)p * CS * nc;
  const T* cp = KIND ? coeff + (long long)p * CS : nullptr;
  enforce_bc<T>(L, ntype, F, p, nc, neumann != 0, false, up);
  __syncthreads();
  T inv[DIM];
#pragma unroll
  for (int a = 0; a < DIM; a++) inv[a] = sp[(size_t)p * 6 + (KIND ? 3 : 0) + a];
  for (int c = 0; c < nc; c++) {
    const T* uc = up + (long long)c * CS;
    T v[PER];
#pragma unroll
    for (int r = 0; r < PER; r++) {
      const int k = threadIdx.x + r * 256;
      v[r] = T(0);
      if (k < CS) {
        const int x = k % SY, y = (k / SY) % SY, z = DIM == 3 ? k / SZ : 1;
        if (x >= 1 && x <= NN && y >= 1 && y <= NN && z >= 1 && z <= NN) {
          v[r] = stencil_n<T, KIND, DIM, SY, SZ>(uc, cp, k, inv);
          // residual form: rhs - A u, the value of (A u) * -1 + rhs (Vector::scaleThenAdd)
          if (rhs) v[r] = rhs[(long long)p * CS * nc + (long long)c * CS + k] - v[r];
        }
      }
    }
#pragma unroll
    for (int r = 0; r < PER; r++) {
      const int k = threadIdx.x + r * 256;
      if (k < CS) fp[(long long)c * CS + k] = v[r];
    }
  }
}
// rhs != nullptr: f = rhs - A u on interior cells (constant-size kernels only;
// returns false when the level has none and nothing ran)
template <class T, int KIND>
static bool launch_apply(const te_operator* op, int nc, const T* inv, const T* coeff, int neumann, T* u, T* f,
                         cudaStream_t s, const T* rhs = nullptr) {
  const te_domain* d = op->dom;
  const Layout& L = d->lay;
  const bool fixed = with_cubic_size(L, [&](auto dim, auto nn) {
    apply_n_kernel<T, KIND, decltype(dim)::value, decltype(nn)::value>
        <<<L.P, 256, 0, s>>>(L, nc, d->d_nbr_type.p, d->F, inv, neumann, coeff, u, f, rhs);
  });
  if (!fixed) {
    if (rhs) return false;
    apply_kernel<T, KIND><<<L.P, 256, 0, s>>>(L, nc, d->d_nbr_type.p, d->F, inv, neumann, coeff, u, f);
  }
  count_launch();
  TE_LAUNCH_CHECK();
  return true;
}

void operator_residual(const te_operator* op, int nc, void* u, const void* b, void* r, cudaStream_t s) {
  const te_domain* d = op->dom;
  if (operator_apply_fused<double>(op, nc, (double*)u, (double*)r, (const double*)b, s)) return;
  ghost_fill(op->gf, nc, TE_F64, u, s);
  const bool fused =
      op->kind == 0
          ? launch_apply<double, 0>(op, nc, d->d_inv.p, nullptr, op->neumann, (double*)u, (double*)r, s,
                                    (const double*)b)
          : launch_apply<double, 1>(op, nc, d->d_inv.p, op->coeffs.p, 0, (double*)u, (double*)r, s,
                                    (const double*)b);
  if (fused) return;
  // Cycle::restrict's form (GMG/Cycle.h:59-61): r = A u, then r = r * -1 + b
  if (op->kind == 0)
    launch_apply<double, 0>(op, nc, d->d_inv.p, nullptr, op->neumann, (double*)u, (double*)r, s);
  else
    launch_apply<double, 1>(op, nc, d->d_inv.p, op->coeffs.p, 0, (double*)u, (double*)r, s);
  vec_dispatch(d, nc, TE_F64, OP_SCALE_THEN_ADD, r, b, nullptr, -1.0, 0.0, 0.0);
}

void operator_apply(const te_operator* op, int nc, int dtype, void* u, void* f, cudaStream_t s) {
  const te_domain* d = op->dom;
  if (dtype == TE_F64 ? operator_apply_fused<double>(op, nc, (double*)u, (double*)f, nullptr, s)
                      : operator_apply_fused<float>(op, nc, (float*)u, (float*)f, nullptr, s))
    return;
  ghost_fill(op->gf, nc, dtype, u, s);
  if (dtype == TE_F64) {
    if (op->kind == 0)
      launch_apply<double, 0>(op, nc, d->d_inv.p, nullptr, op->neumann, (double*)u, (double*)f, s);
    else
      launch_apply<double, 1>(op, nc, d->d_inv.p, op->coeffs.p, 0, (double*)u, (double*)f, s);
  } else {
    if (op->kind == 0)
      launch_apply<float, 0>(op, nc, d->d_inv_f.p, nullptr, op->neumann, (float*)u, (float*)f, s);
    else
      launch_apply<float, 1>(op, nc, d->d_inv_f.p, op->coeffs_f.p, 0, (float*)u, (float*)f, s);
  }
}

// ---------------------------------------------------------------------------
// DFT patch solver
// ---------------------------------------------------------------------------
enum DftType { DCT_II, DCT_III, DCT_IV, DST_II, DST_III, DST_IV };

// getTransformArray (Poisson/DFTPatchSolver.h:131-196): matrix[i*n + j]
static std::vector<double> transform_matrix(int type, int n) {
  std::vector<double> m((size_t)n * n, 0.0);
  switch (type) {
    case DCT_II:
      for (int j = 0; j < n; j++)
        for (int i = 0; i < n; i++) m[i * n + j] = std::cos(M_PI / n * (i * (j + 0.5)));
      break;
    case DCT_III:
      for (int i = 0; i < n; i++) m[i * n] = 0.5;
      for (int j = 1; j < n; j++)
        for (int i = 0; i < n; i++) m[i * n + j] = std::cos(M_PI / n * ((i + 0.5) * j));
      break;
    case DCT_IV:
      for (int j = 0; j < n; j++)
        for (int i = 0; i < n; i++) m[i * n + j] = std::cos(M_PI / n * ((i + 0.5) * (j + 0.5)));
      break;
    case DST_II:
      for (int i = 0; i < n; i++)
        for (int j = 0; j < n; j++) m[i * n + j] = std::sin(M_PI / n * ((i + 1) * (j + 0.5)));
      break;
    case DST_III:
      for (int i = 0; i < n; i += 2) m[i * n + n - 1] = 0.5;
      for (int i = 1; i < n; i += 2) m[i * n + n - 1] = -0.5;
      for (int i = 0; i < n; i++)
        for (int j = 0; j < n - 1; j++) m[i * n + j] = std::sin(M_PI / n * ((i + 0.5) * (j + 1)));
      break;
    case DST_IV:
      for (int j = 0; j < n; j++)
        for (int i = 0; i < n; i++) m[i * n + j] = std::sin(M_PI / n * ((i + 0.5) * (j + 0.5)));
      break;
  }
  return m;
}

// DFTPatchSolver::solveSinglePatch for one patch per CTA.  UZERO: the
// iterate is known to be zero (first sweep after u.setWithGhost(0)), so the
// internal-boundary RHS terms vanish and u is not read; u's ghosts are zeroed.
template <class T, int KIND, bool UZERO>
__global__ void __launch_bounds__(1024) dft_kernel(Layout L, int ti_max, const int8_t* __restrict__ ntype, int F, const T* __restrict__ sp, T scale,
                           const T* __restrict__ coeff, const int* __restrict__ plan_of_patch,
                           const int* __restrict__ plan_mats, const T* __restrict__ mats,
                           const int* __restrict__ mat_off, const T* __restrict__ inv_eig,
                           const int* __restrict__ zero_mode, const T* __restrict__ f, T* u) {
  extern __shared__ __align__(16) unsigned char smraw[];
  T* sm = reinterpret_cast<T*>(smraw);
  const SmemLay S = smem_lay(L);
  const int p = blockIdx.x;
  const int N = L.interior();
  T* A = sm;
  T* B = A + S.size;
  const long long ps = L.pstride(1);
  const T* fp = f + p * ps;
  T* up = u + p * ps;
  const T* cp = KIND ? coeff + (long long)p * L.cs : nullptr;
  const int plan = plan_of_patch[p];
  const T* MT[6];
  dft_mat_ptrs<T>(L, plan, plan_mats, mats, mat_off, MT);
  T inv[3];
  for (int a = 0; a < 3; a++) inv[a] = sp[(size_t)p * 6 + (KIND ? 3 : 0) + a];
  // f_copy with the internal boundary conditions folded in (modifyRHS)
#pragma unroll 2
  for (int e = threadIdx.x; e < N; e += blockDim.x) {
    int x = e % L.n0, r = e / L.n0, y = r % L.n1, z = r / L.n1;
    int k = L.at(x, y, z);
    T v = fp[k];
    if (!UZERO) v = modify_cell<T, KIND>(L, ntype, F, p, up, cp, x, y, z, k, v, inv);
    A[x + y * S.sy + z * S.sz] = v;
  }
  __syncthreads();
  T* cur = dft_solve_smem<T>(L, S, MT, inv_eig + (long long)plan * N, zero_mode[p] != 0, A, B, ti_max);
  if (UZERO) {
    for (int k = threadIdx.x; k < L.cs; k += blockDim.x) up[k] = T(0);
    __syncthreads();
  }
  for (int e = threadIdx.x; e < N; e += blockDim.x) {
    int x = e % L.n0, r = e / L.n0, y = r % L.n1, z = r / L.n1;
    up[L.at(x, y, z)] = cur[x + y * S.sy + z * S.sz] * scale;
  }
}

// ---------------------------------------------------------------------------
// BiCGStab patch solver
// ---------------------------------------------------------------------------
// threads per patch of the BiCGStab patch solver: tuned among 64, 128, 256 and 512

__device__ __forceinline__ double bsum(double v, double* red) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  __syncthreads();
  if (l == 0) red[w] = v;
  __syncthreads();
  double s = 0;
  for (int i = 0; i < (int)(blockDim.x >> 5); i++) s += red[i];
  return s;
}

template <class T>
__device__ double dotp(const Layout& L, const T* a, const T* b, double* red) {
  int N = L.interior();
  double acc = 0;
  for (int e = threadIdx.x; e < N; e += blockDim.x) {
    int x, y, z;
    decompose(L, e, x, y, z);
    int k = L.at(x, y, z);
    acc += (double)a[k] * (double)b[k];
  }
  return bsum(acc, red);
}

// y = A_internal x on one patch (applySinglePatchWithInternalBoundaryConditions)
template <class T, int KIND>
__device__ void patch_apply(const Layout& L, const int8_t* ntype, int F, int p, bool neumann, T* x, T* y,
                            const T* c, const T* inv) {
  enforce_bc<T>(L, ntype, F, p, 1, neumann, true, x);
  enforce_bc<T>(L, ntype, F, p, 1, neumann, false, x);
  __syncthreads();
  int N = L.interior();
  for (int e = threadIdx.x; e < N; e += blockDim.x) {
    int xx, yy, zz;
    decompose(L, e, xx, yy, zz);
    int k = L.at(xx, yy, zz);
    y[k] = stencil<T, KIND>(L, x, c, k, inv);
  }
  __syncthreads();
}

// vector update over interior cells
#define TE_FOR_INTERIOR(L, k, body)                          \
  for (int _e = threadIdx.x; _e < (L).interior(); _e += blockDim.x) { \
    int _x, _y, _z;                                          \
    decompose((L), _e, _x, _y, _z);                          \
    int k = (L).at(_x, _y, _z);                              \
    body;                                                    \
  }

template <class T, int KIND, int NT>
__global__ void __launch_bounds__(NT)
    bicgstab_patch_kernel(Layout L, const int8_t* __restrict__ ntype, int F, const T* __restrict__ sp,
                          int neumann, const T* __restrict__ coeff, const T* __restrict__ f, T* u, double tol,
                          int max_it, int cont, bool use_smem, T* gscratch, unsigned long long* its_out,
                          int* status) {
  extern __shared__ unsigned char smraw[];
  __shared__ double red[NT / 32];
  int p = blockIdx.x;
  int cs = L.cs;
  T* base = use_smem ? reinterpret_cast<T*>(smraw) : gscratch + (long long)p * 8 * cs;
  T *x = base, *b = x + cs, *r = b + cs, *rh = r + cs, *pv = rh + cs, *ap = pv + cs, *as = ap + cs, *s = as + cs;
  const T* fp = f + (long long)p * cs;
  T* up = u + (long long)p * cs;
  const T* cp = KIND ? coeff + (long long)p * cs : nullptr;
  T inv[3];
  for (int a = 0; a < 3; a++) inv[a] = sp[(size_t)p * 6 + (KIND ? 3 : 0) + a];
  // x = u (all cells); b = f_copy (zero ghosts, modifyRHS applied); others zero
  for (int e = threadIdx.x; e < cs; e += blockDim.x) {
    x[e] = up[e];
    b[e] = T(0);
    r[e] = T(0);
    ap[e] = T(0);
    as[e] = T(0);
    s[e] = T(0);
  }
  __syncthreads();
  for (int e = threadIdx.x; e < L.interior(); e += blockDim.x) {
    int xx, yy, zz;
    decompose(L, e, xx, yy, zz);
    int k = L.at(xx, yy, zz);
    b[k] = modify_cell<T, KIND>(L, ntype, F, p, up, cp, xx, yy, zz, k, fp[k], inv);
  }
  __syncthreads();
  bool nm = neumann != 0;
  // BiCGStab::solve (Iterative/BiCGStab.h:111-203), no preconditioner
  patch_apply<T, KIND>(L, ntype, F, p, nm, x, r, cp, inv);
  TE_FOR_INTERIOR(L, k, r[k] = r[k] * T(-1) + b[k]);
  __syncthreads();
  double r0 = sqrt(dotp(L, b, b, red));
  for (int e = threadIdx.x; e < cs; e += blockDim.x) {
    rh[e] = r[e];
    pv[e] = r[e];
  }
  __syncthreads();
  double rho = dotp(L, rh, r, red);
  int it = 0;
  double residual = sqrt(dotp(L, r, r, red)) / r0;
  if (r0 != 0) {
    while (residual > tol && it < max_it) {
      if (rho == 0) {
        if (!cont && threadIdx.x == 0) *status = 1;
        break;
      }
      patch_apply<T, KIND>(L, ntype, F, p, nm, pv, ap, cp, inv);
      double alpha = rho / dotp(L, rh, ap, red);
      TE_FOR_INTERIOR(L, k, s[k] = r[k]);
      TE_FOR_INTERIOR(L, k, s[k] += ap[k] * (T)(-alpha));
      __syncthreads();
      if (sqrt(dotp(L, s, s, red)) / r0 <= tol) {
        TE_FOR_INTERIOR(L, k, x[k] += pv[k] * (T)alpha);
        __syncthreads();
        break;
      }
      patch_apply<T, KIND>(L, ntype, F, p, nm, s, as, cp, inv);
      double omega = dotp(L, as, s, red) / dotp(L, as, as, red);
      TE_FOR_INTERIOR(L, k, x[k] += pv[k] * (T)alpha + s[k] * (T)omega);
      TE_FOR_INTERIOR(L, k, r[k] += ap[k] * (T)(-alpha) + as[k] * (T)(-omega));
      __syncthreads();
      double rho_new = dotp(L, r, rh, red);
      double beta = rho_new * alpha / (rho * omega);
      TE_FOR_INTERIOR(L, k, pv[k] += ap[k] * (T)(-omega));
      TE_FOR_INTERIOR(L, k, pv[k] = pv[k] * (T)beta + r[k]);
      __syncthreads();
      it++;
      rho = rho_new;
      residual = sqrt(dotp(L, r, r, red)) / r0;
    }
  }
  __syncthreads();
  for (int e = threadIdx.x; e < cs; e += blockDim.x) up[e] = x[e];
  if (threadIdx.x == 0) atomicAdd(its_out, (unsigned long long)it);
}

// Right-hand-side boundary helpers (Poisson/StarPatchOperator.h:187-242,
// VarPoisson/StarPatchOperator.h:194-219): one CTA per patch walks its sides in
// side order (a barrier between sides), so an edge or corner cell receives its
// terms in the reference's order; each term is formed in the reference's
// operation order with FP64 arithmetic that is not contracted into FMAs, so
// FP64 results match it bit for bit.  mode 0: Poisson Dirichlet, f += -2 g / h^2;
// mode 1: VarPoisson Dirichlet, f -= 2 g c / h^2; mode 2: Neumann, f += dg / h on
// lower sides and f -= dg / h on upper sides.  Boundary data: [P][2D][fs].
__host__ __device__ inline long long face_stride(const Layout& L) {
  long long a = (long long)L.n1 * L.n2, b = (long long)L.n0 * L.n2, c = (long long)L.n0 * L.n1;
  long long m = a > b ? a : b;
  return L.D == 3 ? (m > c ? m : c) : (L.n0 > L.n1 ? L.n0 : L.n1);
}

template <class T>
__global__ void __launch_bounds__(256)
    bc_rhs_kernel(Layout L, const int8_t* __restrict__ ntype, int F, const double* __restrict__ sp, int mode,
                  long long fs, const double* __restrict__ gv, const double* __restrict__ cv, T* f) {
  const int p = blockIdx.x, D = L.D;
  const int side0 = D == 2 ? 4 : 20;
  T* fp = f + (long long)p * L.cs;
  for (int side = 0; side < 2 * D; side++) {
    if (ntype[(size_t)p * F + side0 + side] < 0) {
      const int axis = side >> 1, upper = side & 1;
      const int t0 = axis == 0 ? 1 : 0, t1 = axis == 2 ? 1 : 2;
      const int m0 = L.n(t0), m1 = D == 3 ? L.n(t1) : 1;
      const double h = sp[(size_t)p * D + axis];
      const double h2 = __dmul_rn(h, h);
      const long long base = ((long long)p * 2 * D + side) * fs;
      for (int e = threadIdx.x; e < m0 * m1; e += blockDim.x) {
        int c[3] = {0, 0, 0};
        c[t0] = e % m0;
        if (D == 3) c[t1] = e / m0;
        c[axis] = upper ? L.n(axis) - 1 : 0;
        const int k = L.at(c[0], c[1], c[2]);
        const double g = gv[base + e];
        double v;
        if (mode == 0)
          v = __ddiv_rn(__dmul_rn(-2.0, g), h2);
        else if (mode == 1)
          v = -__ddiv_rn(__dmul_rn(__dmul_rn(2.0, g), cv[base + e]), h2);
        else
          v = upper ? -__ddiv_rn(g, h) : __ddiv_rn(g, h);
        if (sizeof(T) == 8)
          fp[k] = (T)__dadd_rn((double)fp[k], v);
        else
          fp[k] = fp[k] + (T)v;
      }
    }
    __syncthreads();
  }
}

static size_t dft_smem(const Layout& L, int tsize) {
  SmemLay S = smem_lay(L);
  return ((size_t)S.mats + smem_mat_elems(L)) * tsize;
}

template <class T>
static void launch_dft(const te_patch_solver* ps, const T* f, T* u, const T* coeff, const T* mats,
                       const T* ie, bool uzero, cudaStream_t s) {
  const te_domain* d = ps->op->dom;
  size_t smem = dft_smem(d->lay, sizeof(T));
  int ti_max, threads;
  dft_launch_shape(d->lay, ti_max, threads);
  auto kern = ps->op->kind == 0 ? (uzero ? dft_kernel<T, 0, true> : dft_kernel<T, 0, false>)
                                : (uzero ? dft_kernel<T, 1, true> : dft_kernel<T, 1, false>);
  double scale = 1.0;
  for (int a = 0; a < d->lay.D; a++) scale *= 2.0 / d->lay.n(a);
  kern<<<d->lay.P, threads, smem, s>>>(d->lay, ti_max, d->d_nbr_type.p, d->F, d->template inv<T>(), (T)scale, coeff,
                                        ps->plan_of_patch.p, ps->plan_mats.p, mats, ps->mat_off.p, ie,
                                        ps->zero_mode.p, f, u);
  count_launch();
  TE_LAUNCH_CHECK();
}

// raise the dynamic shared-memory limit of every DFT kernel instance once
static void dft_set_smem_limits(size_t smem64, size_t smem32) {
  auto set = [](const void* k, size_t sm) {
    if (sm > 40 * 1024) allow_max_dynamic_smem(k);
  };
  set((const void*)dft_kernel<double, 0, true>, smem64);
  set((const void*)dft_kernel<double, 0, false>, smem64);
  set((const void*)dft_kernel<double, 1, true>, smem64);
  set((const void*)dft_kernel<double, 1, false>, smem64);
  set((const void*)dft_kernel<float, 0, true>, smem32);
  set((const void*)dft_kernel<float, 0, false>, smem32);
  set((const void*)dft_kernel<float, 1, true>, smem32);
  set((const void*)dft_kernel<float, 1, false>, smem32);
}

template <class T, int KIND, int NT>
static void launch_bcg_nt(const te_patch_solver* ps, const T* f, T* u, const T* coeff, cudaStream_t s) {
  const te_domain* d = ps->op->dom;
  const Layout& L = d->lay;
  size_t need = (size_t)8 * L.cs * sizeof(T);
  bool use_smem = need <= 200 * 1024;
  T* scratch = use_smem ? nullptr : reinterpret_cast<T*>(ps->scratch.p);
  size_t smem = use_smem ? need : 0;
  bicgstab_patch_kernel<T, KIND, NT><<<L.P, NT, smem, s>>>(L, d->d_nbr_type.p, d->F, d->template inv<T>(),
                                                          ps->op->neumann, coeff, f, u, ps->tol, ps->max_it, ps->cont,
                                                          use_smem, scratch, ps->its.p, ps->status.p);
  count_launch();
  TE_LAUNCH_CHECK();
}

// The thread count is tuned per (dimension, patch shape, precision, operator), not per patch
// count, so that a solve alone and the same solve in a batch use the same kernel (the count
// sets the order of the block reductions).  Tuning runs on scratch copies of u, since a
// candidate overwrites it.
template <class T>
static void launch_bcg(const te_patch_solver* ps, const T* f, T* u, const T* coeff, cudaStream_t s) {
  const Layout& L = ps->op->dom->lay;
  const int kind = ps->op->kind;
  auto run = [&](int nt, T* out) {
    if (kind == 0) {
      if (nt == 64) launch_bcg_nt<T, 0, 64>(ps, f, out, coeff, s);
      else if (nt == 128) launch_bcg_nt<T, 0, 128>(ps, f, out, coeff, s);
      else if (nt == 256) launch_bcg_nt<T, 0, 256>(ps, f, out, coeff, s);
      else launch_bcg_nt<T, 0, 512>(ps, f, out, coeff, s);
    } else {
      if (nt == 64) launch_bcg_nt<T, 1, 64>(ps, f, out, coeff, s);
      else if (nt == 128) launch_bcg_nt<T, 1, 128>(ps, f, out, coeff, s);
      else if (nt == 256) launch_bcg_nt<T, 1, 256>(ps, f, out, coeff, s);
      else launch_bcg_nt<T, 1, 512>(ps, f, out, coeff, s);
    }
  };
  static const int nts[4] = {256, 128, 64, 512};  // 256 (the default) first
  char key[128];
  std::snprintf(key, sizeof key, "D=%d n=%dx%dx%d %s kind=%d", L.D, L.n0, L.n1, L.n2, sizeof(T) == 8 ? "f64" : "f32",
                kind);
  cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
  TE_CUDA(cudaStreamIsCapturing(s, &cap));
  std::vector<TuneCandidate> cands;
  DevBuf<T> tmp;
  if (cap == cudaStreamCaptureStatusNone && !tune_settled("bcg_patch", key)) {
    const size_t n = (size_t)L.P * L.cs;
    tmp.alloc(n);
    for (int i = 0; i < 4; i++)
      cands.push_back({"threads=" + std::to_string(nts[i]), [&, i, n] {
                         TE_CUDA(cudaMemcpyAsync(tmp.p, u, n * sizeof(T), cudaMemcpyDeviceToDevice, s));
                         run(nts[i], tmp.p);
                       }});
  } else {
    for (int i = 0; i < 4; i++) cands.push_back({"threads=" + std::to_string(nts[i]), [] {}});
  }
  const int pick = tune_select("bcg_patch", key, cands, s, 3);
  run(nts[pick], u);
}

// shared-memory limits and global scratch are set up when the solver is
// created, so that launches can be captured into CUDA graphs
static void bcg_prepare(te_patch_solver* ps) {
  const Layout& L = ps->op->dom->lay;
  auto setup = [&](auto tag, std::initializer_list<const void*> ks) {
    using T = decltype(tag);
    size_t need = (size_t)8 * L.cs * sizeof(T);
    if (need <= 200 * 1024) {
      if (need > 40 * 1024)
        for (const void* k : ks) allow_max_dynamic_smem(k);
    } else {
      size_t bytes = (size_t)L.P * need;
      if (ps->scratch.n < bytes) ps->scratch.alloc(bytes);
    }
  };
  setup(double(0), {(const void*)bicgstab_patch_kernel<double, 0, 64>, (const void*)bicgstab_patch_kernel<double, 1, 64>,
                    (const void*)bicgstab_patch_kernel<double, 0, 128>, (const void*)bicgstab_patch_kernel<double, 1, 128>,
                    (const void*)bicgstab_patch_kernel<double, 0, 256>, (const void*)bicgstab_patch_kernel<double, 1, 256>,
                    (const void*)bicgstab_patch_kernel<double, 0, 512>, (const void*)bicgstab_patch_kernel<double, 1, 512>});
  setup(float(0), {(const void*)bicgstab_patch_kernel<float, 0, 64>, (const void*)bicgstab_patch_kernel<float, 1, 64>,
                   (const void*)bicgstab_patch_kernel<float, 0, 128>, (const void*)bicgstab_patch_kernel<float, 1, 128>,
                   (const void*)bicgstab_patch_kernel<float, 0, 256>, (const void*)bicgstab_patch_kernel<float, 1, 256>,
                   (const void*)bicgstab_patch_kernel<float, 0, 512>, (const void*)bicgstab_patch_kernel<float, 1, 512>});
}

void patch_smooth(const te_patch_solver* ps, int nc, int dtype, const void* f, void* u, bool zero_first,
                  cudaStream_t s) {
  const te_operator* op = ps->op;
  const te_domain* d = op->dom;
  require(nc == 1, "patch solvers support one component", TE_ERR_UNSUPPORTED);
  if (ps->kind == 0 && zero_first) {
    // PatchSolver::apply / a first sweep on u.setWithGhost(0): with u == 0 the
    // ghost fill and the RHS modification contribute exactly zero
    if (dtype == TE_F64)
      launch_dft<double>(ps, (const double*)f, (double*)u, op->coeffs.p, ps->mats.p, ps->inv_eig.p, true, s);
    else if (ps->tc_ok)
      dft_tc<float, float>(ps, (const float*)f, (float*)u, s, nullptr, true);
    else
      launch_dft<float>(ps, (const float*)f, (float*)u, op->coeffs_f.p, ps->mats_f.p, ps->inv_eig_f.p, true, s);
    return;
  }
  if (zero_first) {
    // PatchSolver::apply: u.setWithGhost(0) (PatchSolver.h:118)
    TE_CUDA(cudaMemsetAsync(u, 0, (size_t)d->lay.P * d->lay.pstride(nc) * (dtype == TE_F64 ? 8 : 4), s));
  } else {
    ghost_fill(op->gf, nc, dtype, u, s);  // PatchSolver::smooth (PatchSolver.h:152)
  }
  if (ps->kind == 0) {
    if (dtype == TE_F64)
      launch_dft<double>(ps, (const double*)f, (double*)u, op->coeffs.p, ps->mats.p, ps->inv_eig.p, false, s);
    else
      launch_dft<float>(ps, (const float*)f, (float*)u, op->coeffs_f.p, ps->mats_f.p, ps->inv_eig_f.p, false, s);
  } else {
    if (dtype == TE_F64)
      launch_bcg<double>(ps, (const double*)f, (double*)u, op->coeffs.p, s);
    else
      launch_bcg<float>(ps, (const float*)f, (float*)u, op->coeffs_f.p, s);
  }
}

template <class T>
__global__ void cast_kernel(T* dst, const double* src, long long n) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    dst[i] = (T)src[i];
}

// nearest float-float split: hi = fl32(v), lo = fl32(v - hi)
__global__ void split_df_kernel(float* hi, float* lo, const double* src, long long n) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    double v = src[i];
    float h = (float)v;
    hi[i] = h;
    lo[i] = (float)(v - (double)h);
  }
}

}  // namespace te

using namespace te;

extern "C" {

static int make_operator(const te_domain* d, const te_ghost_filler* g, int kind, int neumann, const void* coeffs,
                         te_operator** out) {
  return guard([&] {
    require(d && g && out, "null argument");
    require(g->dom == d, "ghost filler belongs to another domain");
    auto op = std::make_unique<te_operator>();
    op->dom = d;
    op->gf = g;
    op->kind = kind;
    op->neumann = neumann;
    op->faces = make_face_table(d->lay);
    if (kind == 1) {
      require(coeffs != nullptr, "null coefficients");
      long long n = (long long)d->lay.P * d->lay.pstride(1);
      op->coeffs.alloc(n);
      TE_CUDA(cudaMemcpyAsync(op->coeffs.p, coeffs, n * sizeof(double), cudaMemcpyDeviceToDevice, d->stream));
      ghost_fill(g, 1, TE_F64, op->coeffs.p, d->stream);  // VarPoisson ctor (:70)
      op->coeffs_f.alloc(n);
      cast_kernel<float><<<304, 256, 0, d->stream>>>(op->coeffs_f.p, op->coeffs.p, n);
      count_launch();
      TE_LAUNCH_CHECK();
      op->coeffs_df.alloc(2 * n);
      split_df_kernel<<<304, 256, 0, d->stream>>>(op->coeffs_df.p, op->coeffs_df.p + n, op->coeffs.p, n);
      count_launch();
      TE_LAUNCH_CHECK();
      TE_CUDA(cudaStreamSynchronize(d->stream));
    }
    *out = op.release();
  });
}

int te_poisson_operator_create(const te_domain* d, const te_ghost_filler* g, int neumann, te_operator** out) {
  return make_operator(d, g, 0, neumann, nullptr, out);
}

int te_varpoisson_operator_create(const te_domain* d, const te_ghost_filler* g, const void* coeffs,
                                  te_operator** out) {
  return make_operator(d, g, 1, 0, coeffs, out);
}

int te_operator_destroy(te_operator* op) {
  delete op;
  return TE_OK;
}

int te_operator_apply(const te_operator* op, int nc, int dtype, void* u, void* f) {
  return guard([&] {
    require(op && u && f, "null argument");
    operator_apply(op, nc, dtype, u, f, op->dom->stream);
  });
}

int te_operator_modify_rhs(const te_operator* op, int nc, int dtype, const void* u, void* f) {
  return guard([&] {
    require(op && u && f, "null argument");
    const te_domain* d = op->dom;
    cudaStream_t s = d->stream;
    if (dtype == TE_F64) {
      if (op->kind == 0)
        modify_rhs_kernel<double, 0><<<d->lay.P, 256, 0, s>>>(d->lay, nc, d->d_nbr_type.p, d->F, d->d_inv.p,
                                                              nullptr, (const double*)u, (double*)f);
      else
        modify_rhs_kernel<double, 1><<<d->lay.P, 256, 0, s>>>(d->lay, nc, d->d_nbr_type.p, d->F, d->d_inv.p,
                                                              op->coeffs.p, (const double*)u, (double*)f);
    } else {
      if (op->kind == 0)
        modify_rhs_kernel<float, 0><<<d->lay.P, 256, 0, s>>>(d->lay, nc, d->d_nbr_type.p, d->F, d->d_inv_f.p,
                                                             nullptr, (const float*)u, (float*)f);
      else
        modify_rhs_kernel<float, 1><<<d->lay.P, 256, 0, s>>>(d->lay, nc, d->d_nbr_type.p, d->F, d->d_inv_f.p,
                                                             op->coeffs_f.p, (const float*)u, (float*)f);
    }
    count_launch();
    TE_LAUNCH_CHECK();
  });
}

int te_dft_patch_solver_create(const te_operator* op, int neumann_mask, te_patch_solver** out) {
  return guard([&] {
    require(op && out, "null argument");
    const te_domain* d = op->dom;
    const Layout& L = d->lay;
    int D = L.D, P = L.P, N = L.interior();
    size_t smem = dft_smem(L, sizeof(double));
    require(smem <= 220 * 1024, "patch too large for the DFT patch solver", TE_ERR_UNSUPPORTED);
    dft_set_smem_limits(smem, dft_smem(L, sizeof(float)));
    auto ps = std::make_unique<te_patch_solver>();
    ps->op = op;
    ps->kind = 0;
    ps->neumann_mask = neumann_mask;
    int side_slot0 = D == 2 ? 4 : 20;
    auto neu = [&](int p, int side) {
      return d->nbr_type[(size_t)p * d->F + side_slot0 + side] < 0 && ((neumann_mask >> side) & 1);
    };
    // plan cache keyed like the reference: (neumann bitset, spacings[0]) (:385-413)
    std::map<std::pair<unsigned long, double>, int> plan_id;
    std::map<std::pair<int, int>, int> mat_id;
    std::vector<std::vector<double>> mats;
    std::vector<int> plan_mats, plan_of(P), zero(P, 0);
    std::vector<double> eig_inv;
    auto get_mat = [&](int type, int n) {
      auto k = std::make_pair(type, n);
      auto it = mat_id.find(k);
      if (it != mat_id.end()) return it->second;
      auto m = transform_matrix(type, n);
      std::vector<double> mt(m.size());
      for (int i = 0; i < n; i++)
        for (int j = 0; j < n; j++) mt[(size_t)j * n + i] = m[(size_t)i * n + j];
      mats.push_back(mt);
      return mat_id[k] = (int)mats.size() - 1;
    };
    bool all_neumann = neumann_mask == (1 << (2 * D)) - 1;
    for (int p = 0; p < P; p++) {
      unsigned long mask = 0;
      for (int s = 0; s < 2 * D; s++)
        if (neu(p, s)) mask |= 1ul << s;
      auto key = std::make_pair(mask, d->spacings[(size_t)p * D]);
      bool any_nbr = false;
      for (int s = 0; s < d->F; s++) any_nbr |= d->nbr_type[(size_t)p * d->F + s] >= 0;
      zero[p] = all_neumann && !any_nbr;
      auto it = plan_id.find(key);
      if (it != plan_id.end()) {
        plan_of[p] = it->second;
        continue;
      }
      int id = (int)plan_id.size();
      plan_id[key] = id;
      plan_of[p] = id;
      int fwd[3] = {0, 0, 0}, inv[3] = {0, 0, 0};
      for (int a = 0; a < D; a++) {  // getTransformsForPatch / getInverseTransformsForPatch (:272-313)
        bool lo = neu(p, 2 * a), hi = neu(p, 2 * a + 1);
        int tf = (lo && hi) ? DCT_II : lo ? DCT_IV : hi ? DST_IV : DST_II;
        int ti = (lo && hi) ? DCT_III : lo ? DCT_IV : hi ? DST_IV : DST_III;
        fwd[a] = get_mat(tf, L.n(a));
        inv[a] = get_mat(ti, L.n(a));
      }
      for (int a = 0; a < 3; a++) plan_mats.push_back(fwd[a]);
      for (int a = 0; a < 3; a++) plan_mats.push_back(inv[a]);
      // getEigenValues (:320-361): e = ((0 - v0) - v1) - v2, then 1/e
      std::vector<double> e(N, 0.0);
      for (int a = 0; a < D; a++) {
        int n = L.n(a);
        double h = d->spacings[(size_t)p * D + a];
        bool lo = neu(p, 2 * a), hi = neu(p, 2 * a + 1);
        for (int idx = 0; idx < N; idx++) {
          int c3[3] = {idx % L.n0, (idx / L.n0) % L.n1, idx / (L.n0 * L.n1)};
          int xi = c3[a];
          double val;
          if (lo && hi)
            val = 4 / (h * h) * std::pow(std::sin(xi * M_PI / (2 * n)), 2);
          else if (lo || hi)
            val = 4 / (h * h) * std::pow(std::sin((xi + 0.5) * M_PI / (2 * n)), 2);
          else
            val = 4 / (h * h) * std::pow(std::sin((xi + 1) * M_PI / (2 * n)), 2);
          e[idx] -= val;
        }
      }
      for (int idx = 0; idx < N; idx++) eig_inv.push_back(e[idx] == 0 ? 0.0 : 1.0 / e[idx]);
    }
    ps->nplans = (int)plan_id.size();
    std::vector<int> off;
    std::vector<double> flat;
    for (auto& m : mats) {
      off.push_back((int)flat.size());
      flat.insert(flat.end(), m.begin(), m.end());
    }
    cudaStream_t st = d->stream;
    ps->plan_of_patch.upload(plan_of, st);
    ps->plan_mats.upload(plan_mats, st);
    ps->mats.upload(flat, st);
    ps->mats_f.upload(std::vector<float>(flat.begin(), flat.end()), st);
    ps->mat_off.upload(off, st);
    ps->inv_eig.upload(eig_inv, st);
    ps->inv_eig_f.upload(std::vector<float>(eig_inv.begin(), eig_inv.end()), st);
    ps->zero_mode.upload(zero, st);
    dft_tc_prepare(ps.get(), mats, plan_mats, st);
    TE_CUDA(cudaStreamSynchronize(st));
    *out = ps.release();
  });
}

int te_bicgstab_patch_solver_create(const te_operator* op, double tol, int max_iterations, int cont,
                                    te_patch_solver** out) {
  return guard([&] {
    require(op && out, "null argument");
    require(max_iterations >= 0, "max_iterations must be >= 0");
    auto ps = std::make_unique<te_patch_solver>();
    ps->op = op;
    ps->kind = 1;
    ps->tol = tol;
    ps->max_it = max_iterations;
    ps->cont = cont;
    ps->its.alloc(1);
    ps->status.alloc(1);
    bcg_prepare(ps.get());
    TE_CUDA(cudaMemsetAsync(ps->its.p, 0, sizeof(unsigned long long), op->dom->stream));
    TE_CUDA(cudaMemsetAsync(ps->status.p, 0, sizeof(int), op->dom->stream));
    TE_CUDA(cudaStreamSynchronize(op->dom->stream));
    *out = ps.release();
  });
}

int te_patch_solver_destroy(te_patch_solver* s) {
  delete s;
  return TE_OK;
}

static int solver_call(const te_patch_solver* ps, int nc, int dtype, const void* f, void* u, bool zero_first) {
  return guard([&] {
    require(ps && f && u, "null argument");
    cudaStream_t s = ps->op->dom->stream;
    patch_smooth(ps, nc, dtype, f, u, zero_first, s);
    if (ps->kind == 1 && !ps->cont) {  // breakdown is reported, as BreakdownError is thrown
      int st = 0;
      TE_CUDA(cudaMemcpyAsync(&st, ps->status.p, sizeof(int), cudaMemcpyDeviceToHost, s));
      TE_CUDA(cudaStreamSynchronize(s));
      if (st) {
        TE_CUDA(cudaMemsetAsync(ps->status.p, 0, sizeof(int), s));
        throw Error(TE_ERR_BREAKDOWN, "BiCGStab broke down in a patch solve");
      }
    }
  });
}

int te_patch_solver_smooth(const te_patch_solver* s, int nc, int dtype, const void* f, void* u) {
  return solver_call(s, nc, dtype, f, u, false);
}
int te_patch_solver_apply(const te_patch_solver* s, int nc, int dtype, const void* f, void* u) {
  return solver_call(s, nc, dtype, f, u, true);
}
long long te_domain_face_stride(const te_domain* d) { return d ? face_stride(d->lay) : -1; }

int te_domain_boundary_points(const te_domain* d, double* coords) {
  return guard([&] {
    require(d && coords, "null argument");
    const Layout& L = d->lay;
    const int D = L.D;
    const long long fs = face_stride(L);
    std::vector<double> h((size_t)L.P * 2 * D * fs * D, 0.0);
    for (int p = 0; p < L.P; p++)
      for (int side = 0; side < 2 * D; side++) {
        const int axis = side >> 1, upper = side & 1;
        const int t0 = axis == 0 ? 1 : 0, t1 = axis == 2 ? 1 : 2;
        const int m0 = L.n(t0), m1 = D == 3 ? L.n(t1) : 1;
        for (int e = 0; e < m0 * m1; e++) {
          double* x = &h[(((size_t)p * 2 * D + side) * fs + e) * D];
          const int k[3] = {e % m0, e / m0, 0};
          for (int a = 0; a < D; a++) {
            const double st = d->starts[(size_t)p * D + a], sp = d->spacings[(size_t)p * D + a];
            // DomainTools::GetRealCoordBound (DomainTools.h:179-210)
            if (a == axis)
              x[a] = upper ? st + sp * L.n(a) : st;
            else
              x[a] = st + sp / 2.0 + sp * k[a == t0 ? 0 : 1];
          }
        }
      }
    TE_CUDA(cudaMemcpyAsync(coords, h.data(), h.size() * sizeof(double), cudaMemcpyHostToDevice, d->stream));
    TE_CUDA(cudaStreamSynchronize(d->stream));
  });
}

static int add_bc_rhs(const te_operator* op, int dtype, void* f, int mode, const double* g, const double* c) {
  return guard([&] {
    require(op && f && g, "null argument");
    require(dtype == TE_F64 || dtype == TE_F32, "bad dtype");
    const te_domain* d = op->dom;
    const long long fs = face_stride(d->lay);
    if (dtype == TE_F64)
      bc_rhs_kernel<double><<<d->lay.P, 256, 0, d->stream>>>(d->lay, d->d_nbr_type.p, d->F, d->d_spacings.p, mode,
                                                            fs, g, c, (double*)f);
    else
      bc_rhs_kernel<float><<<d->lay.P, 256, 0, d->stream>>>(d->lay, d->d_nbr_type.p, d->F, d->d_spacings.p, mode,
                                                           fs, g, c, (float*)f);
    count_launch();
    TE_LAUNCH_CHECK();
  });
}

int te_operator_add_dirichlet_bc_to_rhs(const te_operator* op, int dtype, void* f, const double* gvals,
                                        const double* cvals) {
  if (op && op->kind == 1 && !cvals) {
    return guard([&] { require(false, "VarPoisson's addDrichletBCToRHS needs the coefficient at the boundary points"); });
  }
  return add_bc_rhs(op, dtype, f, op && op->kind == 1 ? 1 : 0, gvals, cvals);
}

int te_operator_add_neumann_bc_to_rhs(const te_operator* op, int dtype, void* f, const double* dgvals) {
  if (op && op->kind != 0) {
    return guard([&] {
      require(false, "addNeumannBCToRHS exists for the Poisson operator only (as in the reference)",
              TE_ERR_UNSUPPORTED);
    });
  }
  return add_bc_rhs(op, dtype, f, 2, dgvals, nullptr);
}

int te_patch_solver_uses_tensor_cores(const te_patch_solver* s, int* out) {
  return guard([&] {
    require(s && out, "null argument");
    *out = s->tc_ok ? 1 : 0;
  });
}

int te_dft_patch_solver_create_tc(const te_operator* op, int neumann_mask, int tc_precision, te_patch_solver** out) {
  int rc = te_dft_patch_solver_create(op, neumann_mask, out);
  if (rc != TE_OK) return rc;
  return guard([&] {
    te_patch_solver* ps = *out;
    if (tc_precision != TE_TC_TF32X3 && tc_precision != TE_TC_BF16) {
      te_patch_solver_destroy(ps);
      *out = nullptr;
      require(false, "tc_precision must be TE_TC_TF32X3 or TE_TC_BF16");
    }
    if (tc_precision == TE_TC_BF16 && !(ps->tc_ok && ps->tc_operands != 1)) {
      te_patch_solver_destroy(ps);
      *out = nullptr;
      require(false, "BF16 transforms need the tensor-core path (cubic patches n = 16, 32, 64 in 2D or 16 in 3D, "
                     "one set of transform matrices per level)", TE_ERR_UNSUPPORTED);
    }
    ps->tc_prec = tc_precision;
  });
}

}  // extern "C"
