// te_dft_tc.cu -- the DFT patch solve (Poisson/DFTPatchSolver.h:226-269,
// solveSinglePatch: forward transform per axis, divide by the eigenvalues,
// inverse transform per axis, scale by prod 2/n) on the tcgen05 tensor cores.
//
// Every pass of the separable transform applies one n x n matrix along one
// axis to all lines of all patches: a batched dense contraction
//   D[line][i] = sum_j A[line][j] M[i][j]
// with the lines of G patches stacked as the M = 128-row operand A (K = n) and
// the transform matrix as operand B (N = n).  The data are FP32; each product
// runs as 3xTF32 (A_hi B_hi + A_hi B_lo + A_lo B_hi, FP32 accumulation in
// TMEM), which keeps about 22 significant bits, close to FP32.
//
// One CTA holds G patches: ROWS = 128 (2D) or 256 (3D, n = 16) lines, each
// taken by SPLIT threads (SPLIT * ROWS threads; thread t has line t % ROWS and
// the n / SPLIT columns of part t / ROWS, so the warps of a part cover the four
// TMEM lane quarters).  After each pass every thread reads its columns back
// from TMEM (tcgen05.ld), splits them into TF32 hi/lo parts and writes them
// into the operand tile of the next pass; when the next pass runs along
// another axis the write is a transpose (each thread writes one element into
// n / SPLIT different lines).  The
// forward passes run x, y(, z); the inverse passes z(, y), x, so the pass after
// the eigenvalue divide needs no transpose.  CTAs loop over patch groups.
//
// Each CTA loads the next group's right-hand sides into registers while the
// current group's passes run, and writes whole padded patches (zero ghosts)
// through a shared-memory transpose so the stores are coalesced.
//
// Requirements (checked when the solver is created): cubic patches with
// n = 16, 32 or 64 (2D) or n = 16 (3D), one ghost layer, and one set of
// transform matrices for all patches of the level (the eigenvalues may differ
// per patch).

#include <cstdio>
#include <cstdlib>
#include <cstring>

#include "te_ops.cuh"
#include "te_tc.cuh"

namespace te {

struct DftTcArgs {
  Layout L;
  int ngroups;
  int pass_mat[6];           // matrix slot (hi and lo tiles) of each pass
  int nmat;                  // distinct matrices
  const float* bmat;         // [nmat][2][n*n]: hi then lo, row-major M[i][j]
  const int* plan_of_patch;  // [P]
  const float* inv_eig;      // [nplans][n^D]
  const int* zero_mode;      // [P]
  const float* corr;         // optional [P][2D][n^(D-1)]: right-hand-side corrections per side face
  float scale;               // prod 2/n, applied to the last pass's result
  int zero_ghosts;           // also write 0 into the output's ghost cells (PatchSolver::apply)
  int* err;
};

template <int DIM, int NN>
struct TcShape {
  static constexpr int SPLIT = 2;                               // threads per line
  static constexpr int RPP = DIM == 2 ? NN : NN * NN;          // lines per patch
  static constexpr int NCELL = RPP * NN;                        // cells per patch
  static constexpr int ROWS = RPP > 128 ? RPP : 128;            // lines per CTA
  static constexpr int THREADS = ROWS * SPLIT;                  // threads per CTA
  static constexpr int JN = NN / SPLIT;                         // columns per thread
  static constexpr int G = ROWS / RPP;                          // patches per CTA
  static constexpr int R = ROWS / 128;                          // 128-row blocks
  static constexpr int PITCH = NN >= 32 ? 128 : 4 * NN;         // bytes per tile row within a K atom
  static constexpr int ATILE = ROWS * NN * 4;                   // bytes of one operand-A tile
  static constexpr int BTILE = NN * NN * 4;                     // bytes of one operand-B tile
  static constexpr int COLS_USED = R * NN;
  static constexpr int NCOLS = COLS_USED <= 32 ? 32 : (COLS_USED <= 64 ? 64 : (COLS_USED <= 128 ? 128 : 256));
  // resident CTAs per SM the registers are sized for (shared memory allows four for 2D n <= 32;
  // four lines per thread group and three CTAs measured slower than two and four)
  static constexpr int MIN_CTAS = NN == 64 ? 1 : 512 / ROWS;
};

__device__ __forceinline__ void line_coords(int a, int line, int j, int n, int& cx, int& cy, int& cz) {
  if (a == 0) {
    cx = j;
    cy = line % n;
    cz = line / n;
  } else if (a == 1) {
    cy = j;
    cx = line % n;
    cz = line / n;
  } else {
    cz = j;
    cx = line % n;
    cy = line / n;
  }
}

constexpr long long kWaitLimit = 2000000000ll;  // clock cycles (about one second)

// Global offset of interior cell c (x fastest) of a patch, one ghost layer
template <int DIM, int NN>
__device__ __forceinline__ int interior_offset(int c) {
  constexpr int SY = NN + 2, SZ = DIM == 3 ? SY * SY : 0;
  const int x = c % NN, r = c / NN;
  return (x + 1) + (r % NN + 1) * SY + (DIM == 3 ? (r / NN + 1) * SZ : 0);
}

template <class TI, class TO, int DIM, int NN>
__global__ void __launch_bounds__(TcShape<DIM, NN>::THREADS, TcShape<DIM, NN>::MIN_CTAS)
    dft_tc_kernel(DftTcArgs a, const TI* in, TO* out) {
  using S = TcShape<DIM, NN>;
  constexpr int SY = NN + 2;
  constexpr int CS = DIM == 3 ? SY * SY * SY : SY * SY;  // padded cells per patch
  constexpr int NT = S::THREADS;
  constexpr int JN = S::JN;
  constexpr int PER = S::G * S::NCELL / NT;                // interior cells per thread per group
  constexpr int OP = NN + 1;                               // row pitch (floats) of the output staging
  constexpr int NF = S::RPP;                               // cells of one side face
  constexpr int CPER = S::G * 2 * DIM * NF / NT;           // corrections per thread per group
  static_assert(S::G * S::NCELL % NT == 0, "cells must split evenly over the threads");
  static_assert(S::G * 2 * DIM * NF % NT == 0, "corrections must split evenly over the threads");
  static_assert(JN % 8 == 0, "TMEM is read in blocks of 8 columns");
  static_assert(NT % NN == 0, "every thread's cells share one x");
  extern __shared__ uint8_t dsm[];
  __shared__ uint64_t bar;
  __shared__ uint32_t tmem_base;
  const int t = threadIdx.x, warp = t >> 5;
  const int P = a.L.P;
  const uint32_t raw = tc::smem_addr(dsm);
  uint8_t* sm = dsm + ((1024 - (raw & 1023)) & 1023);
  uint8_t* Ahi = sm;
  uint8_t* Alo = sm + S::ATILE;
  uint8_t* Bm = sm + 2 * S::ATILE;
  float* stage = reinterpret_cast<float*>(sm);  // output staging over both A tiles: [ROWS][OP]
  float* cbuf = reinterpret_cast<float*>(Bm + a.nmat * 2 * S::BTILE);  // [G][2D][NF] corrections
  const bool has_corr = a.corr != nullptr;

  // the first group's right-hand sides, in flight while the CTA sets up
  TI pf[PER];
  float cpf[CPER];
  auto prefetch = [&](int grp) {
    const int p0 = grp * S::G;
#pragma unroll
    for (int k = 0; k < PER; k++) {
      int e = t + k * NT;
      int i = e / S::NCELL, c = e % S::NCELL;
      int p = p0 + i;
      pf[k] = p < P ? __ldg(in + (long long)p * CS + interior_offset<DIM, NN>(c)) : TI(0);
    }
    if (has_corr) {
#pragma unroll
      for (int k = 0; k < CPER; k++) {
        int e = t + k * NT;
        int p = p0 + e / (2 * DIM * NF);
        cpf[k] = p < P ? __ldg(a.corr + (long long)p0 * 2 * DIM * NF + e) : 0.f;
      }
    }
  };
  prefetch(blockIdx.x);

  // transform matrices into their swizzled tiles
  for (int e = t; e < a.nmat * 2 * NN * NN; e += NT) {
    int m = e / (NN * NN), r = e % (NN * NN);
    *reinterpret_cast<float*>(Bm + m * S::BTILE + tc::tile_offset(r / NN, r % NN, NN, NN)) = a.bmat[e];
  }
  // the first group's corrections; later groups' are written before the barrier that ends the previous group
  if (has_corr) {
#pragma unroll
    for (int k = 0; k < CPER; k++) cbuf[t + k * NT] = cpf[k];
  }
  if (t == 0) tc::mbar_init(&bar, 1);
  if (warp == 0) tc::tmem_alloc(&tmem_base, S::NCOLS);
  tc::fence_async_smem();
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tmem = tmem_base;
  // this thread's line and columns: TMEM lane line % 128 (a warp reads the 32 lanes of its quarter),
  // column block line / 128, columns j0 .. j0 + JN - 1 of the line
  const int line = t % S::ROWS, j0 = (t / S::ROWS) * JN;
  const uint32_t my_row = tmem + ((uint32_t)((line & 127) & ~31) << 16) + (uint32_t)(line >> 7) * NN + j0;
  constexpr uint32_t idesc = tc::idesc_tf32(128, NN);
  const uint32_t a_hi = tc::smem_addr(Ahi), a_lo = tc::smem_addr(Alo), b0 = tc::smem_addr(Bm);
  const int my_i = line / S::RPP, my_line = line % S::RPP;
  uint32_t phase = 0;
  bool abort = false;

  for (int grp = blockIdx.x; grp < a.ngroups && !abort; grp += gridDim.x) {
    const int p0 = grp * S::G;
    // f_copy = f - corrections of the cell's sides, in side order (x, then y, then z
    // sides): each thread's cells share one x (NT is a multiple of n), so the x
    // sides concern two threads in n and the y and z sides whole rows (an FP64
    // right-hand side takes its corrections in FP64)
    if (has_corr) {
      const int xt = t % NN;
      if (xt == 0 || xt == NN - 1) {
        const int side = xt == 0 ? 0 : 1;
#pragma unroll
        for (int k = 0; k < PER; k++) {
          const int e = t + k * NT, i = e / S::NCELL, c = e % S::NCELL;
          pf[k] -= (TI)cbuf[i * 2 * DIM * NF + side * NF + c / NN];
        }
      }
#pragma unroll
      for (int k = 0; k < PER; k++) {
        const int e = t + k * NT, i = e / S::NCELL, c = e % S::NCELL;
        const int y = (c / NN) % NN, z = DIM == 3 ? c / (NN * NN) : 0;
        if (y == 0 || y == NN - 1) pf[k] -= (TI)cbuf[i * 2 * DIM * NF + (y == 0 ? 2 : 3) * NF + xt + NN * z];
      }
      if (DIM == 3) {
#pragma unroll
        for (int k = 0; k < PER; k++) {
          const int e = t + k * NT, i = e / S::NCELL, c = e % S::NCELL;
          const int y = (c / NN) % NN, z = c / (NN * NN);
          if (z == 0 || z == NN - 1) pf[k] -= (TI)cbuf[i * 2 * DIM * NF + (z == 0 ? 4 : 5) * NF + xt + NN * y];
        }
      }
    }
    // right-hand sides into the operand tiles of the x pass: line (i, y[, z]), k = x
#pragma unroll
    for (int k = 0; k < PER; k++) {
      int e = t + k * NT;
      int i = e / S::NCELL, c = e % S::NCELL;
      float v = (float)pf[k];
      float hi = tc::to_tf32(v), lo = v - hi;
      uint32_t off = tc::tile_offset(i * S::RPP + c / NN, c % NN, S::ROWS, NN);
      *reinterpret_cast<float*>(Ahi + off) = hi;
      *reinterpret_cast<float*>(Alo + off) = lo;
    }
    // the next group's loads overlap this group's transforms
    if (grp + (int)gridDim.x < a.ngroups) prefetch(grp + gridDim.x);
    const int my_p = p0 + my_i;
    const bool my_valid = my_p < P;
    const int my_plan = my_valid ? __ldg(a.plan_of_patch + my_p) : 0;
    const bool my_zero = my_valid && __ldg(a.zero_mode + my_p) != 0;
#pragma unroll
    for (int q = 0; q < 2 * DIM; q++) {
      tc::fence_async_smem();
      tc::fence_before_sync();
      __syncthreads();
      if (t == 0) {
        tc::fence_after_sync();
        const uint32_t bh = b0 + a.pass_mat[q] * 2 * S::BTILE, bl = bh + S::BTILE;
#pragma unroll
        for (int r = 0; r < S::R; r++) {
#pragma unroll
          for (int ks = 0; ks < NN / 8; ks++) {
            uint32_t ao = (ks >> 2) * S::ROWS * S::PITCH + r * 128 * S::PITCH + (ks & 3) * 32;
            uint32_t bo = (ks >> 2) * NN * S::PITCH + (ks & 3) * 32;
            uint32_t d = tmem + r * NN;
            uint64_t dah = tc::smem_desc(a_hi + ao, NN), dal = tc::smem_desc(a_lo + ao, NN);
            uint64_t dbh = tc::smem_desc(bh + bo, NN), dbl = tc::smem_desc(bl + bo, NN);
            tc::mma_tf32(d, dah, dbh, idesc, ks > 0);
            tc::mma_tf32(d, dah, dbl, idesc, 1);
            tc::mma_tf32(d, dal, dbh, idesc, 1);
          }
        }
        tc::commit(&bar);
      }
      // one thread waits for the MMAs (bounded) and tells the others at the barrier
      int late = 0;
      if (t == 0) late = !tc::mbar_wait(&bar, phase, kWaitLimit);
      if (__syncthreads_or(late)) {
        abort = true;
        break;
      }
      phase ^= 1;
      tc::fence_after_sync();
      float v[JN];  // columns j0 .. j0 + JN - 1 of this thread's line
      if (JN % 16 == 0) {
#pragma unroll
        for (int c = 0; c < JN; c += 16) tc::tmem_ld16(my_row + c, *reinterpret_cast<float(*)[16]>(&v[c]));
      } else {
#pragma unroll
        for (int c = 0; c < JN; c += 8) tc::tmem_ld8(my_row + c, *reinterpret_cast<float(*)[8]>(&v[c]));
      }
      tc::tmem_ld_wait();
      const int ax = q < DIM ? q : 2 * DIM - 1 - q;  // axis of this pass
      if (q == DIM - 1 && my_valid) {
        // eigenvalue divide; the cell of (line, j) on the last axis is line + RPP * j
        const float* ie = a.inv_eig + (long long)my_plan * S::NCELL + my_line;
#pragma unroll
        for (int j = 0; j < JN; j++) v[j] *= __ldg(ie + S::RPP * (j0 + j));
        if (my_zero && my_line == 0 && j0 == 0) v[0] = 0.f;
      }
      if (q == 2 * DIM - 1) {
        // line (i, y[, z]) with x = j: into the staging rows, then whole padded patches out
#pragma unroll
        for (int j = 0; j < JN; j++) stage[line * OP + j0 + j] = v[j] * a.scale;
        __syncthreads();
        // interior rows, coalesced: thread t writes cells t, t + ROWS, ... of the group
#pragma unroll
        for (int k = 0; k < PER; k++) {
          const int e = t + k * NT;
          const int i = e / S::NCELL, c = e % S::NCELL;
          const int p = p0 + i;
          if (p < P) out[(long long)p * CS + interior_offset<DIM, NN>(c)] = (TO)stage[(i * S::RPP + c / NN) * OP + c % NN];
        }
        if (a.zero_ghosts) {
          for (int e = t; e < S::G * CS; e += NT) {
            const int i = e / CS, k = e % CS;
            const int p = p0 + i;
            if (p >= P) break;
            const int x = k % SY - 1, r2 = k / SY;
            const int y = r2 % SY - 1, z = DIM == 3 ? r2 / SY - 1 : 0;
            const bool inner = x >= 0 && x < NN && y >= 0 && y < NN && z >= 0 && z < NN;
            if (!inner) out[(long long)p * CS + k] = TO(0);
          }
        }
        continue;
      }
      const int nx = q + 1 < DIM ? q + 1 : 2 * DIM - 2 - q;  // axis of the next pass
      if (nx == ax) {
        // own line, 16-byte chunks: the 8 lanes of a store phase hit 8 different chunk positions
#pragma unroll
        for (int j = 0; j < JN; j += 4) {
          float4 hi, lo;
          hi.x = tc::to_tf32(v[j]);
          hi.y = tc::to_tf32(v[j + 1]);
          hi.z = tc::to_tf32(v[j + 2]);
          hi.w = tc::to_tf32(v[j + 3]);
          lo.x = v[j] - hi.x;
          lo.y = v[j + 1] - hi.y;
          lo.z = v[j + 2] - hi.z;
          lo.w = v[j + 3] - hi.w;
          uint32_t off = tc::tile_offset(line, j0 + j, S::ROWS, NN);
          *reinterpret_cast<float4*>(Ahi + off) = hi;
          *reinterpret_cast<float4*>(Alo + off) = lo;
        }
      } else {
#pragma unroll
        for (int j = 0; j < JN; j++) {
          int cx, cy, cz;
          line_coords(ax, my_line, j0 + j, NN, cx, cy, cz);
          const int nline = nx == 0 ? cy + NN * cz : (nx == 1 ? cx + NN * cz : cx + NN * cy);
          const int k = nx == 0 ? cx : (nx == 1 ? cy : cz);
          float hi = tc::to_tf32(v[j]), lo = v[j] - hi;
          uint32_t off = tc::tile_offset(my_i * S::RPP + nline, k, S::ROWS, NN);
          *reinterpret_cast<float*>(Ahi + off) = hi;
          *reinterpret_cast<float*>(Alo + off) = lo;
        }
      }
    }
    // the next group's corrections (prefetched above; this group no longer reads cbuf)
    if (has_corr) {
#pragma unroll
      for (int k = 0; k < CPER; k++) cbuf[t + k * NT] = cpf[k];
    }
    // the staging rows overlap the operand tiles the next group writes
    __syncthreads();
  }
  if (abort) {
    // the MMA that did not finish in time: wait for it once more before freeing TMEM
    if (t == 0) tc::mbar_wait(&bar, phase, kWaitLimit);
    if (t == 0) atomicExch(a.err, 1);
  }
  tc::fence_before_sync();
  __syncthreads();
  if (warp == 0) {
    tc::fence_after_sync();
    tc::tmem_dealloc(tmem, S::NCOLS);
  }
}

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
namespace {

float tf32_round_host(float x) {
  uint32_t b;
  std::memcpy(&b, &x, 4);
  if ((b & 0x7f800000u) != 0x7f800000u) {
    b += 0x1000u;  // nearest, ties away from zero
    b &= 0xffffe000u;
  }
  float r;
  std::memcpy(&r, &b, 4);
  return r;
}

template <int DIM, int NN>
size_t tc_smem_bytes(int nmat) {
  using S = TcShape<DIM, NN>;
  return 1024 + 2 * (size_t)S::ATILE + (size_t)nmat * 2 * S::BTILE + (size_t)S::G * 2 * DIM * S::RPP * 4;
}

}  // namespace

void dft_tc_prepare(te_patch_solver* ps, const std::vector<std::vector<double>>& mats_t,
                    const std::vector<int>& plan_mats, cudaStream_t st) {
  ps->tc_ok = false;
  const char* env = std::getenv("TE_NO_TC");
  if (env && env[0] == '1') return;
  const Layout& L = ps->op->dom->lay;
  const int D = L.D, n = L.n0;
  if (L.n1 != n || (D == 3 && L.n2 != n) || L.g != 1) return;
  if (!((D == 2 && (n == 16 || n == 32 || n == 64)) || (D == 3 && n == 16))) return;
  const int nplans = (int)plan_mats.size() / 6;
  if (nplans < 1) return;
  for (int pl = 1; pl < nplans; pl++)
    for (int a = 0; a < D; a++)
      if (plan_mats[pl * 6 + a] != plan_mats[a] || plan_mats[pl * 6 + 3 + a] != plan_mats[3 + a]) return;
  // passes: forward x, y(, z), inverse (z,) y, x; each distinct matrix is stored once (a cube with one
  // boundary type per axis needs two), which keeps four CTAs' shared memory on an SM
  double scale = 1.0;
  for (int ax = 0; ax < D; ax++) scale *= 2.0 / n;
  ps->tc_scale = (float)scale;
  std::vector<int> ids;
  for (int q = 0; q < 2 * D; q++) {
    int ax = q < D ? q : 2 * D - 1 - q;
    int key = plan_mats[(q < D ? 0 : 3) + ax];
    int slot = -1;
    for (size_t u = 0; u < ids.size(); u++)
      if (ids[u] == key) slot = (int)u;
    if (slot < 0) {
      ids.push_back(key);
      slot = (int)ids.size() - 1;
    }
    ps->tc_pass_mat[q] = slot;
  }
  ps->tc_nmat = (int)ids.size();
  std::vector<float> b((size_t)ps->tc_nmat * 2 * n * n);
  for (int u = 0; u < ps->tc_nmat; u++) {
    const std::vector<double>& mt = mats_t[ids[u]];  // transposed: mt[j*n + i] = M[i][j]
    float* hi = &b[(size_t)u * 2 * n * n];
    float* lo = hi + n * n;
    for (int i = 0; i < n; i++)
      for (int j = 0; j < n; j++) {
        double m = mt[(size_t)j * n + i];
        float h = tf32_round_host((float)m);
        hi[i * n + j] = h;
        lo[i * n + j] = tf32_round_host((float)(m - (double)h));
      }
  }
  ps->tc_bmat.upload(b, st);
  ps->tc_err.alloc(1);
  TE_CUDA(cudaMemsetAsync(ps->tc_err.p, 0, sizeof(int), st));
  ps->tc_ok = true;
}

template <class TI, class TO, int DIM, int NN>
static void dft_tc_t(const te_patch_solver* ps, const TI* in, TO* out, cudaStream_t s, const float* corr,
                     bool zero_ghosts) {
  using S = TcShape<DIM, NN>;
  const Layout& L = ps->op->dom->lay;
  DftTcArgs a;
  a.L = L;
  a.ngroups = (L.P + S::G - 1) / S::G;
  for (int q = 0; q < 6; q++) a.pass_mat[q] = ps->tc_pass_mat[q];
  a.nmat = ps->tc_nmat;
  a.bmat = ps->tc_bmat.p;
  a.plan_of_patch = ps->plan_of_patch.p;
  a.inv_eig = ps->inv_eig_f.p;
  a.zero_mode = ps->zero_mode.p;
  a.corr = corr;
  a.scale = ps->tc_scale;
  a.zero_ghosts = zero_ghosts ? 1 : 0;
  a.err = ps->tc_err.p;
  auto kern = dft_tc_kernel<TI, TO, DIM, NN>;
  size_t smem = tc_smem_bytes<DIM, NN>(a.nmat);
  // at most 512 / NCOLS resident CTAs per SM, so every TMEM allocation succeeds at once
  static int sm_count = 0;
  if (!sm_count) TE_CUDA(cudaDeviceGetAttribute(&sm_count, cudaDevAttrMultiProcessorCount, 0));
  const int tmem_cap = 512 / S::NCOLS;
  const size_t per_sm = 227 * 1024;
  if (smem * tmem_cap < per_sm) smem = per_sm / tmem_cap + 1;
  TE_CUDA(cudaFuncSetAttribute((const void*)kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  TE_CUDA(cudaFuncSetAttribute((const void*)kern, cudaFuncAttributePreferredSharedMemoryCarveout, 100));
  // resident CTAs per SM from the shared-memory, register, thread and TMEM limits
  static int smem_sm = 0, reserved = 0, regs_sm = 0, threads_sm = 0;
  if (!smem_sm) {
    TE_CUDA(cudaDeviceGetAttribute(&smem_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, 0));
    TE_CUDA(cudaDeviceGetAttribute(&reserved, cudaDevAttrReservedSharedMemoryPerBlock, 0));
    TE_CUDA(cudaDeviceGetAttribute(&regs_sm, cudaDevAttrMaxRegistersPerMultiprocessor, 0));
    TE_CUDA(cudaDeviceGetAttribute(&threads_sm, cudaDevAttrMaxThreadsPerMultiProcessor, 0));
  }
  cudaFuncAttributes fa;
  TE_CUDA(cudaFuncGetAttributes(&fa, (const void*)kern));
  int occ = (int)(smem_sm / (smem + fa.sharedSizeBytes + reserved));
  occ = std::min(occ, threads_sm / S::THREADS);
  occ = std::min(occ, regs_sm / std::max(1, fa.numRegs * S::THREADS));
  occ = std::min(occ, tmem_cap);
  require(occ >= 1, "tensor-core DFT: kernel does not fit on an SM", TE_ERR_UNSUPPORTED);
  int grid = std::min(a.ngroups, occ * sm_count);
  kern<<<grid, S::THREADS, smem, s>>>(a, in, out);
  count_launch();
  TE_LAUNCH_CHECK();
}

template <class TI, class TO>
void dft_tc(const te_patch_solver* ps, const TI* in, TO* out, cudaStream_t s, const float* corr,
            bool zero_ghosts) {
  const Layout& L = ps->op->dom->lay;
  require(ps->tc_ok, "tensor-core DFT not prepared for this solver", TE_ERR_UNSUPPORTED);
  if (L.D == 2 && L.n0 == 16)
    dft_tc_t<TI, TO, 2, 16>(ps, in, out, s, corr, zero_ghosts);
  else if (L.D == 2 && L.n0 == 32)
    dft_tc_t<TI, TO, 2, 32>(ps, in, out, s, corr, zero_ghosts);
  else if (L.D == 2 && L.n0 == 64)
    dft_tc_t<TI, TO, 2, 64>(ps, in, out, s, corr, zero_ghosts);
  else
    dft_tc_t<TI, TO, 3, 16>(ps, in, out, s, corr, zero_ghosts);
}

int dft_tc_error(const te_patch_solver* ps, cudaStream_t s) {
  if (!ps->tc_ok) return 0;
  int e = 0;
  TE_CUDA(cudaMemcpyAsync(&e, ps->tc_err.p, sizeof(int), cudaMemcpyDeviceToHost, s));
  TE_CUDA(cudaStreamSynchronize(s));
  return e;
}

template void dft_tc<double, float>(const te_patch_solver*, const double*, float*, cudaStream_t, const float*, bool);
template void dft_tc<float, float>(const te_patch_solver*, const float*, float*, cudaStream_t, const float*, bool);
template void dft_tc<double, double>(const te_patch_solver*, const double*, double*, cudaStream_t, const float*, bool);

}  // namespace te
