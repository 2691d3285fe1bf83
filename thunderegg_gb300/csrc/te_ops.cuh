// te_ops.cuh -- operator and patch-solver handles (internal).
#pragma once
#include <map>
#include <memory>
#include <vector>

#include "te_ghost.cuh"

struct te_operator {
  const te_domain* dom = nullptr;
  const te_ghost_filler* gf = nullptr;
  int kind = 0;  // 0 Poisson::StarPatchOperator, 1 VarPoisson::StarPatchOperator
  int neumann = 0;
  te::DevBuf<double> coeffs;    // VarPoisson: ghost-filled coefficient level buffer (1 component)
  te::DevBuf<float> coeffs_f;   // FP32 copy for the mixed-precision cycle
  te::DevBuf<float> coeffs_df;  // float-float split [2 * size]: hi, then lo (mixed-precision outer Krylov)
  te::FaceTable faces;
  // work vectors of te_bicgstab_solve(_batched) with this operator, per
  // component count and batch layout (patch offsets of the solves)
  mutable std::map<std::pair<int, std::vector<int>>, std::shared_ptr<void>> krylov;
  const void* coeff_ptr(int dtype) const {
    return kind == 0 ? nullptr : (dtype == TE_F64 ? (const void*)coeffs.p : (const void*)coeffs_f.p);
  }
};

struct te_patch_solver {
  const te_operator* op = nullptr;
  int kind = 0;  // 0 DFT, 1 BiCGStab patch solver
  // DFT plans (Poisson/DFTPatchSolver.h:385-413)
  int neumann_mask = 0;
  int nplans = 0;
  te::DevBuf<int> plan_of_patch;       // [P]
  te::DevBuf<int> plan_mats;           // [nplans * 6]: fwd matrix id per axis, inv matrix id per axis
  te::DevBuf<double> mats;             // transposed matrices, n*n each, concatenated
  te::DevBuf<float> mats_f;
  te::DevBuf<int> mat_off;             // offset of each matrix
  te::DevBuf<double> inv_eig;          // [nplans * n0*n1*n2]  1 / eigenvalue
  te::DevBuf<float> inv_eig_f;
  te::DevBuf<int> zero_mode;           // [P] pure-Neumann patch without neighbours
  // BiCGStab patch solver (Iterative/PatchSolver.h:121-175)
  double tol = 1e-12;
  int max_it = 1000;
  int cont = 1;
  te::DevBuf<unsigned long long> its;  // total inner iterations (statistics)
  te::DevBuf<int> status;              // breakdown flag
  mutable te::DevBuf<char> scratch;    // global-memory fallback for large patches
  // tensor-core DFT (te_dft_tc.cu): usable when every patch shares the transform matrices
  bool tc_ok = false;
  int tc_pass_mat[6] = {0, 0, 0, 0, 0, 0};
  int tc_nmat = 0;
  float tc_scale = 1.f;  // prod 2/n
  int tc_operands = 0;    // kernel variants the autotuner may pick: 0 both, 1 operands in shared memory
                          // only, 2 operands in tensor memory only (TE_TC_OPERANDS=smem / tmem)
  int tc_prec = 0;        // transforms: 0 = 3xTF32, 1 = BF16 operands with per-patch scaling
  te::DevBuf<uint16_t> tc_bmat16;  // [tc_nmat][n*n] BF16 bits, row-major
  te::DevBuf<float> tc_bmat;  // [tc_nmat][2][n*n] TF32 hi/lo parts, row-major
  te::DevBuf<int> tc_err;     // set when an MMA wait timed out
};

namespace te {
// one interior cell k of the star stencil of a cubic patch (constant strides SY, SZ), axis 0
// first, in the reference's operation order (Poisson/StarPatchOperator.h:96-110,
// VarPoisson/StarPatchOperator.h:93-113); u and c may point to global or shared memory
template <class T, int KIND, int DIM, int SY, int SZ>
__device__ __forceinline__ T stencil_n(const T* u, const T* c, int k, const T* inv) {
  T r = T(0);
#pragma unroll
  for (int a = 0; a < DIM; a++) {
    const int st = a == 0 ? 1 : (a == 1 ? SY : SZ);
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
// f = A u (rhs null) or rhs - A u with u's side ghosts filled, in one kernel where the level
// qualifies (te_apply.cu); false when nothing ran
template <class T>
bool operator_apply_fused(const te_operator* op, int nc, T* u, T* f, const T* rhs, cudaStream_t s);
void operator_apply(const te_operator* op, int nc, int dtype, void* u, void* f, cudaStream_t s);
// r = b - A u (FP64; u's ghosts are filled as by operator_apply); one pass on cubic levels
void operator_residual(const te_operator* op, int nc, void* u, const void* b, void* r, cudaStream_t s);
void patch_smooth(const te_patch_solver* ps, int nc, int dtype, const void* f, void* u, bool zero_first,
                  cudaStream_t s);
// tensor-core DFT solve of every patch: out = DFT-solve(in) (in == out allowed)
void dft_tc_prepare(te_patch_solver* ps, const std::vector<std::vector<double>>& mats_t,
                    const std::vector<int>& plan_mats, cudaStream_t st);
// corr (optional, FP32 [P][2D][n^(D-1)]): per-side right-hand-side corrections subtracted while staging
// zero_ghosts: also write 0 into out's ghost cells (PatchSolver::apply's u.setWithGhost(0)); the fused
// cycle never reads the ghosts of the solve's output and skips it
template <class TI, class TO>
void dft_tc(const te_patch_solver* ps, const TI* in, TO* out, cudaStream_t s, const float* corr = nullptr,
            bool zero_ghosts = false);
int dft_tc_error(const te_patch_solver* ps, cudaStream_t s);
}  // namespace te
