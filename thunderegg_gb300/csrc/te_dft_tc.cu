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

#include <cuda_bf16.h>

#include "te_ops.cuh"
#include "te_tc.cuh"
#include "te_tune.cuh"

namespace te {

struct DftTcArgs {
  Layout L;
  int ngroups;
  int pass_mat[6];           // matrix slot (hi and lo tiles) of each pass
  int nmat;                  // distinct matrices
  const float* bmat;         // [nmat][2][n*n]: hi then lo, row-major M[i][j]
  const uint16_t* bmat16;    // [nmat][n*n]: BF16 bits, row-major M[i][j] (BF16 transforms)
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
  // TMEM-operand kernel: accumulator, A hi and A lo of every row block (3xTF32) or the
  // accumulator and one A of packed BF16 pairs (BF16)
  static constexpr int cols_t(int opk) { return opk ? R * NN + R * NN / 2 : 3 * R * NN; }
  static constexpr int ncols_t(int opk) {
    return cols_t(opk) <= 32 ? 32 : (cols_t(opk) <= 64 ? 64 : (cols_t(opk) <= 128 ? 128 : 256));
  }
  static constexpr int MIN_CTAS_T = NN == 64 ? 2 : 512 / ROWS;
  static constexpr int PITCH16 = 2 * NN >= 128 ? 128 : 2 * NN;  // bytes per BF16 tile row within a K atom
  static constexpr int BTILE16 = (NN * NN * 2 + 1023) / 1024 * 1024;  // BF16 tile, 1024-byte aligned
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
// The same solve with both A operands (TF32 hi and lo parts) in tensor memory.
//
// The accumulator of a pass and the two A operands of the next pass share the
// TMEM lanes of the lines: lane = line % 128, column block = line / 128.  After
// a pass every thread reads its line's columns back (tcgen05.ld).  When the
// next pass runs along the same axis it splits them into TF32 hi/lo and stores
// them straight into the A columns (tcgen05.st); when it runs along another
// axis the FP32 values go through a shared-memory exchange buffer, transposed,
// and each thread reads its new line back with 16-byte loads before the split.
// The tensor cores then read A from TMEM and only the n x n transform matrices
// from shared memory, so shared-memory traffic per cell and pass is one FP32
// write and one read instead of two TF32 writes and three operand reads.
// ---------------------------------------------------------------------------

// Exchange buffer: [ROWS][NN] floats, row = a line of the current orientation,
// k = its K index.  16-byte chunks are XOR-swizzled by the row (and for n = 16
// rows of odd 16-line groups swap parity) so that a warp's scalar transposed
// writes and a quarter warp's 16-byte row reads hit distinct banks; only the 3D
// passes between y and z keep a two-way conflict.
template <int NN>
__device__ __forceinline__ int xbuf_index(int row, int k) {
  const int pr = NN == 16 ? (row ^ ((row >> 4) & 1)) : row;
  const int sw = NN == 16 ? ((pr >> 1) & 3) : (pr & 7);
  return pr * NN + (((k >> 2) ^ sw) << 2) + (k & 3);
}

// 2D exchange buffer: rows of NN + 4 floats (a patch's rows contiguous; 16 floats between
// the patches of n = 16).  Row (i, r), element k sits at i * XPS + r * XP + k, so a warp's
// transposed scalar writes (32 lines of one patch, or 16 of two), its 16-byte row reads
// (a quarter warp: eight consecutive rows) and its cell-order accesses (consecutive x) hit
// distinct banks, and every index a thread touches is its own base plus a compile-time
// offset.
template <int NN>
struct Xb2 {
  static constexpr int XP = NN + 4;
  static constexpr int XPS = NN * XP + (NN == 16 ? 16 : 0);
};

// floats of the exchange buffer
template <int DIM, int NN>
constexpr int xbuf_floats() {
  return DIM == 2 ? TcShape<DIM, NN>::G * Xb2<NN>::XPS : TcShape<DIM, NN>::ROWS * NN;
}

// OPK = 0: 3xTF32 products (A hi and lo in TMEM, FP32 accumulation); OPK = 1: BF16 operands
// (one product per K step, FP32 accumulation), each patch's right-hand side scaled by a power
// of two that brings its largest magnitude into [1, 2) and the result scaled back
template <class TI, class TO, int DIM, int NN, int OPK>
__global__ void __launch_bounds__(TcShape<DIM, NN>::THREADS, TcShape<DIM, NN>::MIN_CTAS_T)
    dft_tct_kernel(DftTcArgs a, const TI* in, TO* out) {
  using S = TcShape<DIM, NN>;
  constexpr int SY = NN + 2;
  constexpr int CS = DIM == 3 ? SY * SY * SY : SY * SY;  // padded cells per patch
  constexpr int NT = S::THREADS;
  constexpr int JN = S::JN;
  constexpr int PER = S::G * S::NCELL / NT;                // interior cells per thread per group
  constexpr int NF = S::RPP;                               // cells of one side face
  constexpr int CPER = S::G * 2 * DIM * NF / NT;           // corrections per thread per group
  constexpr int RN = S::R * NN;                            // TMEM columns of one FP32 operand
  constexpr int NCOLS = S::ncols_t(OPK);
  constexpr int BT = OPK ? S::BTILE16 : 2 * S::BTILE;      // shared-memory bytes per matrix
  static_assert(S::G * S::NCELL % NT == 0, "cells must split evenly over the threads");
  static_assert(S::NCELL % NT == 0, "a thread's k-th cell lies in patch k / (NCELL / NT)");
  static_assert(S::G * 2 * DIM * NF % NT == 0, "corrections must split evenly over the threads");
  static_assert(JN % 8 == 0, "TMEM is accessed in blocks of 8 columns");
  static_assert(NT % NN == 0, "every thread's cells share one x");
  extern __shared__ uint8_t dsm[];
  __shared__ uint64_t bar;
  __shared__ uint32_t tmem_base;
  const int t = threadIdx.x, warp = t >> 5;
  const int P = a.L.P;
  const uint32_t raw = tc::smem_addr(dsm);
  uint8_t* sm = dsm + ((1024 - (raw & 1023)) & 1023);
  uint8_t* Bm = sm;                                                   // matrices: 1024-byte aligned tiles
  float* xb = reinterpret_cast<float*>(Bm + a.nmat * BT);             // exchange buffer
  float* cbuf = xb + xbuf_floats<DIM, NN>();                          // [G][2D][NF] corrections
  __shared__ uint32_t pmax[2][S::G];                                  // BF16: |f| maximum per patch (bits)
  const bool has_corr = a.corr != nullptr;
  // a thread's k-th cell of a group (e = t + k * NT) lies in patch k / KPP; in 2D its x is
  // tx and its y is ty + YS * (k % KPP)
  constexpr int KPP = S::NCELL / NT;
  constexpr int YS = NT / NN;
  constexpr int XP = Xb2<NN>::XP, XPS = Xb2<NN>::XPS;
  const int tx = t % NN, ty = t / NN;
  const int gbase = (tx + 1) + (ty + 1) * SY;  // 2D: offset of the thread's first cell in a padded patch
  const int xbase = ty * XP + tx;              // 2D: its exchange-buffer index

  TI pf[PER];
  float cpf[CPER];
  auto prefetch = [&](int grp) {
    const int p0 = grp * S::G;
    if constexpr (DIM == 2) {
      const TI* src = in + (long long)p0 * CS + gbase;
#pragma unroll
      for (int k = 0; k < PER; k++)
        pf[k] = p0 + k / KPP < P ? __ldg(src + (k / KPP) * CS + YS * (k % KPP) * SY) : TI(0);
    } else {
#pragma unroll
      for (int k = 0; k < PER; k++) {
        int e = t + k * NT;
        int i = e / S::NCELL, c = e % S::NCELL;
        int p = p0 + i;
        pf[k] = p < P ? __ldg(in + (long long)p * CS + interior_offset<DIM, NN>(c)) : TI(0);
      }
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

  if (OPK == 0) {
    for (int e = t; e < a.nmat * 2 * NN * NN; e += NT) {
      int m = e / (NN * NN), r = e % (NN * NN);
      *reinterpret_cast<float*>(Bm + m * S::BTILE + tc::tile_offset(r / NN, r % NN, NN, NN)) = a.bmat[e];
    }
  } else {
    for (int e = t; e < a.nmat * NN * NN; e += NT) {
      int m = e / (NN * NN), r = e % (NN * NN);
      *reinterpret_cast<uint16_t*>(Bm + m * BT + tc::tile_offset16(r / NN, r % NN, NN, NN)) = a.bmat16[e];
    }
    if (t < 2 * S::G) pmax[t / S::G][t % S::G] = 0u;
  }
  if (has_corr) {
#pragma unroll
    for (int k = 0; k < CPER; k++) cbuf[t + k * NT] = cpf[k];
  }
  if (t == 0) tc::mbar_init(&bar, 1);
  if (warp == 0) tc::tmem_alloc(&tmem_base, NCOLS);
  tc::fence_async_smem();
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tmem = tmem_base;
  // this thread's line (TMEM lane line % 128, read by the warp of that lane quarter) and columns
  const int line = t % S::ROWS, j0 = (t / S::ROWS) * JN;
  const uint32_t lane = tmem + ((uint32_t)((line & 127) & ~31) << 16) + (uint32_t)(line >> 7) * NN + j0;
  const uint32_t my_d = lane, my_ah = lane + RN, my_al = lane + 2 * RN;
  // BF16: packed pairs, NN / 2 columns per row block
  const uint32_t my_a16 = tmem + ((uint32_t)((line & 127) & ~31) << 16) + RN + (uint32_t)(line >> 7) * (NN / 2) + j0 / 2;
  constexpr uint32_t idesc = OPK ? tc::idesc_bf16(128, NN) : tc::idesc_tf32(128, NN);
  const uint32_t b0 = tc::smem_addr(Bm);
  const int my_i = line / S::RPP, my_line = line % S::RPP;
  uint32_t phase = 0;
  bool abort = false;
  int late = 0;  // this warp's last MMA wait ran out
  // A transpose between 2D passes moves values only among the lines of one patch, which the
  // warps {w, w + 4} (n <= 32) or {w, w + 1, w + 4, w + 5} (n = 64) hold: a named barrier of
  // those warps suffices.  In 3D a patch spans the whole CTA.
  auto xchg_sync = [&] {
    if constexpr (DIM == 2 && NN <= 32) {
      asm volatile("bar.sync %0, 64;" ::"r"(1 + (warp & 3)) : "memory");
    } else if constexpr (DIM == 2) {
      asm volatile("bar.sync %0, 128;" ::"r"(1 + ((warp & 3) >> 1)) : "memory");
    } else {
      __syncthreads();
    }
  };

  // 2D: this thread's row of the exchange buffer (its line, from column j0)
  const int rbase = my_i * XPS + my_line * XP + j0;
  // this thread's line from the exchange buffer
  auto read_row = [&](float (&v)[JN]) {
#pragma unroll
    for (int c = 0; c < JN; c += 4) {
      const float4 q = *reinterpret_cast<const float4*>(xb + (DIM == 2 ? rbase + c : xbuf_index<NN>(line, j0 + c)));
      v[c] = q.x;
      v[c + 1] = q.y;
      v[c + 2] = q.z;
      v[c + 3] = q.w;
    }
  };
  // 3xTF32: split into TF32 hi / lo and store into this thread's A columns;
  // BF16: round to BF16 pairs (even k in the low half) into its packed A columns
  auto store_a = [&](const float (&v)[JN]) {
#pragma unroll
    for (int c = 0; c < JN; c += 8) {
      if (OPK == 0) {
        float hi[8], lo[8];
#pragma unroll
        for (int j = 0; j < 8; j++) {
          hi[j] = tc::to_tf32(v[c + j]);
          lo[j] = v[c + j] - hi[j];
        }
        tc::tmem_st8(my_ah + c, hi);
        tc::tmem_st8(my_al + c, lo);
      } else {
        uint32_t w[4];
#pragma unroll
        for (int j = 0; j < 4; j++) {
          const __nv_bfloat162 b2 = __floats2bfloat162_rn(v[c + 2 * j], v[c + 2 * j + 1]);
          w[j] = *reinterpret_cast<const uint32_t*>(&b2);
        }
        tc::tmem_st4u(my_a16 + c / 2, w);
      }
    }
  };

  for (int grp = blockIdx.x; grp < a.ngroups && !abort; grp += gridDim.x) {
    const int p0 = grp * S::G;
    if (DIM == 2 && has_corr) {
      // f - corrections, x side first, then y side (the order of the general form below)
      if (tx == 0 || tx == NN - 1) {
        const float* cs = cbuf + (tx == 0 ? 0 : NF) + ty;
#pragma unroll
        for (int k = 0; k < PER; k++) pf[k] -= (TI)cs[(k / KPP) * 4 * NF + YS * (k % KPP)];
      }
#pragma unroll
      for (int k = 0; k < PER; k++) {
        const int y = ty + YS * (k % KPP);
        if (y == 0 || y == NN - 1) pf[k] -= (TI)cbuf[(k / KPP) * 4 * NF + (y == 0 ? 2 : 3) * NF + tx];
      }
    } else if (has_corr) {
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
    // right-hand sides into the exchange buffer in x-pass orientation: line (i, y[, z]), k = x
    float pm[S::G];
#pragma unroll
    for (int i = 0; i < S::G; i++) pm[i] = 0.f;
#pragma unroll
    for (int k = 0; k < PER; k++) {
      const float v = (float)pf[k];
      if constexpr (DIM == 2) {
        xb[(k / KPP) * XPS + xbase + YS * (k % KPP) * XP] = v;
      } else {
        const int e = t + k * NT;
        const int i = e / S::NCELL, c = e % S::NCELL;
        xb[xbuf_index<NN>(i * S::RPP + c / NN, c % NN)] = v;
      }
      if (OPK) pm[k / KPP] = fmaxf(pm[k / KPP], fabsf(v));
    }
    const int pbuf = ((grp - (int)blockIdx.x) / (int)gridDim.x) & 1;
    if (OPK) {
#pragma unroll
      for (int i = 0; i < S::G; i++) {
        const uint32_t m = __reduce_max_sync(0xffffffffu, __float_as_uint(pm[i]));
        if ((t & 31) == 0 && m) atomicMax(&pmax[pbuf][i], m);
      }
    }
    if (grp + (int)gridDim.x < a.ngroups) prefetch(grp + gridDim.x);
    const int my_p = p0 + my_i;
    const bool my_valid = my_p < P;
    const int my_plan = my_valid ? __ldg(a.plan_of_patch + my_p) : 0;
    const bool my_zero = my_valid && __ldg(a.zero_mode + my_p) != 0;
    __syncthreads();
    // BF16: the power of two 2^-e with 2^e <= max |f| < 2^(e+1), and its inverse for the result
    float psc = 1.f, pinv = 1.f;
    if (OPK) {
      const uint32_t ex = (pmax[pbuf][my_i] >> 23) & 0xffu;
      if (ex >= 1u && ex <= 253u) {
        psc = __uint_as_float((254u - ex) << 23);
        pinv = __uint_as_float(ex << 23);
      }
      if (t < S::G) pmax[pbuf ^ 1][t] = 0u;  // the next group's maxima (its atomics follow the group's last barrier)
    }
    {
      float v[JN];
      read_row(v);
      if (OPK) {
#pragma unroll
        for (int j = 0; j < JN; j++) v[j] *= psc;
      }
      store_a(v);
    }
#pragma unroll
    for (int q = 0; q < 2 * DIM; q++) {
      tc::tmem_st_wait();
      tc::fence_before_sync();
      // the A operands of every line are in place; a warp whose last wait timed out ends the group
      if (__syncthreads_or(late)) {
        abort = true;
        break;
      }
      if (t == 0) {
        tc::fence_after_sync();
        if (OPK == 0) {
          const uint32_t bh = b0 + a.pass_mat[q] * 2 * S::BTILE, bl = bh + S::BTILE;
#pragma unroll
          for (int r = 0; r < S::R; r++) {
#pragma unroll
            for (int ks = 0; ks < NN / 8; ks++) {
              const uint32_t bo = (ks >> 2) * NN * S::PITCH + (ks & 3) * 32;
              const uint32_t d = tmem + r * NN;
              const uint32_t ah = tmem + RN + r * NN + ks * 8, al = tmem + 2 * RN + r * NN + ks * 8;
              const uint64_t dbh = tc::smem_desc(bh + bo, NN), dbl = tc::smem_desc(bl + bo, NN);
              tc::mma_tf32_ta(d, ah, dbh, idesc, ks > 0);
              tc::mma_tf32_ta(d, ah, dbl, idesc, 1);
              tc::mma_tf32_ta(d, al, dbh, idesc, 1);
            }
          }
        } else {
          // K = 16 per step: 32 bytes of a tile row; a K atom of PITCH16 bytes holds PITCH16 / 32 steps
          constexpr int SPA = S::PITCH16 / 32;
          const uint32_t bb = b0 + a.pass_mat[q] * BT;
#pragma unroll
          for (int r = 0; r < S::R; r++) {
#pragma unroll
            for (int ks = 0; ks < NN / 16; ks++) {
              const uint32_t bo = (ks / SPA) * NN * S::PITCH16 + (ks % SPA) * 32;
              const uint32_t d = tmem + r * NN;
              const uint32_t aa = tmem + RN + r * (NN / 2) + ks * 8;
              tc::mma_bf16_ta(d, aa, tc::smem_desc_pitch(bb + bo, S::PITCH16), idesc, ks > 0);
            }
          }
        }
        tc::commit(&bar);
      }
      // each warp waits for the MMAs itself (lane 0 polls, bounded) and starts its epilogue at
      // once; a timeout is carried to the next CTA barrier, where every warp leaves together
      int ok = 1;
      if ((t & 31) == 0) ok = tc::mbar_wait(&bar, phase, kWaitLimit) ? 1 : 0;
      if (!__shfl_sync(0xffffffffu, ok, 0)) late = 1;
      phase ^= 1;
      tc::fence_after_sync();
      float v[JN];
      if (JN % 16 == 0) {
#pragma unroll
        for (int c = 0; c < JN; c += 16) tc::tmem_ld16(my_d + c, *reinterpret_cast<float(*)[16]>(&v[c]));
      } else {
#pragma unroll
        for (int c = 0; c < JN; c += 8) tc::tmem_ld8(my_d + c, *reinterpret_cast<float(*)[8]>(&v[c]));
      }
      tc::tmem_ld_wait();
      const int ax = q < DIM ? q : 2 * DIM - 1 - q;
      if (q == DIM - 1 && my_valid) {
        const float* ie = a.inv_eig + (long long)my_plan * S::NCELL + my_line;
#pragma unroll
        for (int j = 0; j < JN; j++) v[j] *= __ldg(ie + S::RPP * (j0 + j));
        if (my_zero && my_line == 0 && j0 == 0) v[0] = 0.f;
      }
      if (q == 2 * DIM - 1) {
        // line (i, y[, z]) with x = j: own row of the exchange buffer, then coalesced stores
#pragma unroll
        for (int c = 0; c < JN; c += 4) {
          float4 w;
          const float sc = a.scale * pinv;
          w.x = v[c] * sc;
          w.y = v[c + 1] * sc;
          w.z = v[c + 2] * sc;
          w.w = v[c + 3] * sc;
          *reinterpret_cast<float4*>(xb + (DIM == 2 ? rbase + c : xbuf_index<NN>(line, j0 + c))) = w;
        }
        __syncthreads();
        if constexpr (DIM == 2) {
          TO* dst = out + (long long)p0 * CS + gbase;
#pragma unroll
          for (int k = 0; k < PER; k++)
            if (p0 + k / KPP < P)
              dst[(k / KPP) * CS + YS * (k % KPP) * SY] = (TO)xb[(k / KPP) * XPS + xbase + YS * (k % KPP) * XP];
        } else {
#pragma unroll
          for (int k = 0; k < PER; k++) {
            const int e = t + k * NT;
            const int i = e / S::NCELL, c = e % S::NCELL;
            const int p = p0 + i;
            if (p < P) out[(long long)p * CS + interior_offset<DIM, NN>(c)] = (TO)xb[xbuf_index<NN>(i * S::RPP + c / NN, c % NN)];
          }
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
        store_a(v);
      } else {
        if constexpr (DIM == 2) {
          // line (i, a), column b becomes line (i, b), column a
          float* tb = xb + my_i * XPS + j0 * XP + my_line;
#pragma unroll
          for (int j = 0; j < JN; j++) tb[j * XP] = v[j];
        } else {
#pragma unroll
          for (int j = 0; j < JN; j++) {
            int cx, cy, cz;
            line_coords(ax, my_line, j0 + j, NN, cx, cy, cz);
            const int nline = nx == 0 ? cy + NN * cz : (nx == 1 ? cx + NN * cz : cx + NN * cy);
            const int k = nx == 0 ? cx : (nx == 1 ? cy : cz);
            xb[xbuf_index<NN>(my_i * S::RPP + nline, k)] = v[j];
          }
        }
        xchg_sync();
        read_row(v);
        store_a(v);
      }
    }
    if (has_corr) {
#pragma unroll
      for (int k = 0; k < CPER; k++) cbuf[t + k * NT] = cpf[k];
    }
    // the output rows in the exchange buffer are read before the next group writes it
    if (__syncthreads_or(late)) abort = true;
  }
  if (abort) {
    // the MMAs last issued (every warp toggled its phase after its wait): wait for them once more
    // before TMEM is freed
    if (t == 0) tc::mbar_wait(&bar, phase ^ 1, kWaitLimit);
    if (t == 0) atomicExch(a.err, 1);
  }
  tc::fence_before_sync();
  __syncthreads();
  if (warp == 0) {
    tc::fence_after_sync();
    tc::tmem_dealloc(tmem, NCOLS);
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

// TMEM-operand kernel: matrices, exchange buffer, corrections
template <int DIM, int NN>
size_t tct_smem_bytes(int nmat, int opk) {
  using S = TcShape<DIM, NN>;
  const size_t bt = opk ? (size_t)S::BTILE16 : 2 * (size_t)S::BTILE;
  return 1024 + (size_t)nmat * bt + (size_t)xbuf_floats<DIM, NN>() * 4 + (size_t)S::G * 2 * DIM * S::RPP * 4;
}

uint16_t bf16_round_host(float x) {
  uint32_t b;
  std::memcpy(&b, &x, 4);
  if ((b & 0x7f800000u) != 0x7f800000u) b += 0x7fffu + ((b >> 16) & 1u);  // nearest, ties to even
  return (uint16_t)(b >> 16);
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
  // BF16 copies of the same matrices (te_patch_solver_set_tc_precision)
  std::vector<uint16_t> b16((size_t)ps->tc_nmat * n * n);
  for (int u = 0; u < ps->tc_nmat; u++) {
    const std::vector<double>& mt = mats_t[ids[u]];
    for (int i = 0; i < n; i++)
      for (int j = 0; j < n; j++) b16[(size_t)u * n * n + i * n + j] = bf16_round_host((float)mt[(size_t)j * n + i]);
  }
  ps->tc_bmat16.upload(b16, st);
  const char* ops = std::getenv("TE_TC_OPERANDS");
  ps->tc_operands = ops ? (std::strcmp(ops, "smem") == 0 ? 1 : (std::strcmp(ops, "tmem") == 0 ? 2 : 0)) : 0;
  ps->tc_err.alloc(1);
  TE_CUDA(cudaMemsetAsync(ps->tc_err.p, 0, sizeof(int), st));
  ps->tc_ok = true;
}

// One launch shape of the solve: the kernel variant (operands in shared memory, or in
// tensor memory) and the resident CTAs per SM it is held to (shared memory is padded so
// that no more fit; the TMEM columns always fit).
struct TcLaunch {
  const void* kern;
  size_t smem;
  int ctas;
  int grid;
  bool ok;
};

template <class TI, class TO, int DIM, int NN>
static TcLaunch tc_launch_shape(const void* kern, size_t smem_need, int ncols, int ngroups, int want_ctas) {
  using S = TcShape<DIM, NN>;
  static int sm_count = 0, smem_sm = 0, reserved = 0, regs_sm = 0, threads_sm = 0;
  if (!sm_count) {
    TE_CUDA(cudaDeviceGetAttribute(&sm_count, cudaDevAttrMultiProcessorCount, 0));
    TE_CUDA(cudaDeviceGetAttribute(&smem_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, 0));
    TE_CUDA(cudaDeviceGetAttribute(&reserved, cudaDevAttrReservedSharedMemoryPerBlock, 0));
    TE_CUDA(cudaDeviceGetAttribute(&regs_sm, cudaDevAttrMaxRegistersPerMultiprocessor, 0));
    TE_CUDA(cudaDeviceGetAttribute(&threads_sm, cudaDevAttrMaxThreadsPerMultiProcessor, 0));
  }
  cudaFuncAttributes fa;
  TE_CUDA(cudaFuncGetAttributes(&fa, kern));
  // the most CTAs per SM the threads, registers, shared memory and TMEM columns allow
  int occ = threads_sm / S::THREADS;
  occ = std::min(occ, regs_sm / std::max(1, fa.numRegs * S::THREADS));
  occ = std::min(occ, 512 / ncols);
  occ = std::min(occ, (int)(smem_sm / (smem_need + fa.sharedSizeBytes + reserved)));
  TcLaunch l{kern, smem_need, 0, 0, false};
  if (occ < 1) return l;
  l.ctas = want_ctas > 0 ? std::min(want_ctas, occ) : occ;
  // pad shared memory so that at most l.ctas CTAs are resident on an SM
  const size_t cap = (size_t)smem_sm / l.ctas - fa.sharedSizeBytes - reserved;
  l.smem = std::max(smem_need, std::min(cap, (size_t)227 * 1024));
  l.grid = std::min(ngroups, l.ctas * sm_count);
  l.ok = true;
  return l;
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
  a.bmat16 = ps->tc_bmat16.p;
  a.plan_of_patch = ps->plan_of_patch.p;
  a.inv_eig = ps->inv_eig_f.p;
  a.zero_mode = ps->zero_mode.p;
  a.corr = corr;
  a.scale = ps->tc_scale;
  a.zero_ghosts = zero_ghosts ? 1 : 0;
  a.err = ps->tc_err.p;
  const int opk = ps->tc_prec;
  // candidates: 3xTF32 runs either kernel (operands in shared memory -- the default -- or in
  // tensor memory; both give the same bits), BF16 the tensor-memory kernel; each at every
  // resident-CTA count from the most that fit down to one
  struct Variant {
    const char* name;
    const void* kern;
    size_t smem;
    int ncols;
  };
  std::vector<Variant> vars;
  const int force = ps->tc_operands;  // 0 either, 1 shared memory only, 2 tensor memory only
  if (opk == 0 && force != 2)
    vars.push_back({"smem", (const void*)dft_tc_kernel<TI, TO, DIM, NN>, tc_smem_bytes<DIM, NN>(a.nmat), S::NCOLS});
  if (opk == 1 || force != 1)
    vars.push_back({"tmem", opk ? (const void*)dft_tct_kernel<TI, TO, DIM, NN, 1>
                                : (const void*)dft_tct_kernel<TI, TO, DIM, NN, 0>,
                    tct_smem_bytes<DIM, NN>(a.nmat, opk), S::ncols_t(opk)});
  std::vector<TcLaunch> shapes;
  std::vector<TuneCandidate> cands;
  for (const Variant& v : vars) {
    const TcLaunch full = tc_launch_shape<TI, TO, DIM, NN>(v.kern, v.smem, v.ncols, a.ngroups, 0);
    if (!full.ok) continue;
    for (int c = full.ctas; c >= 1; c--) {
      const TcLaunch l = c == full.ctas ? full : tc_launch_shape<TI, TO, DIM, NN>(v.kern, v.smem, v.ncols, a.ngroups, c);
      if (!l.ok) continue;
      shapes.push_back(l);
      const size_t idx = shapes.size() - 1;
      cands.push_back({std::string(v.name) + " ctas=" + std::to_string(l.ctas), [&, idx] {
                         const TcLaunch& sh = shapes[idx];
                         allow_max_dynamic_smem(sh.kern);
                         TE_CUDA(cudaFuncSetAttribute(sh.kern, cudaFuncAttributePreferredSharedMemoryCarveout, 100));
                         void* args[] = {(void*)&a, (void*)&in, (void*)&out};
                         TE_CUDA(cudaLaunchKernel(sh.kern, dim3(sh.grid), dim3(S::THREADS), args, sh.smem, s));
                         count_launch();
                       }});
    }
  }
  require(!cands.empty(), "tensor-core DFT: kernel does not fit on an SM", TE_ERR_UNSUPPORTED);
  char key[160];
  std::snprintf(key, sizeof key, "D=%d n=%d P~2^%d in=%s out=%s corr=%d ghosts=%d prec=%s", DIM, NN,
                tune_bucket(L.P), sizeof(TI) == 8 ? "f64" : "f32", sizeof(TO) == 8 ? "f64" : "f32", corr ? 1 : 0,
                zero_ghosts ? 1 : 0, opk ? "bf16" : "tf32x3");
  // a solve in place cannot be repeated for timing: it uses the choice made for its shape, or the default
  const int pick = (const void*)in == (const void*)out ? (tune_settled("dft_tc", key) ? tune_select("dft_tc", key, cands, s) : 0)
                                                       : tune_select("dft_tc", key, cands, s);
  cands[pick].run();
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
