// te_tc.cuh -- inline-PTX wrappers for the 5th-generation tensor cores
// (tcgen05: TMEM allocation, MMA from shared-memory descriptors, commit to an
// mbarrier, TMEM loads) used by the tensor-core DFT patch solver.
//
// Shared-memory operand layout (K-major, swizzled): an operand tile of R rows
// and K = n 32-bit elements is stored as ceil(4n/128) column blocks ("K atoms")
// of `pitch` = min(4n, 128) bytes per row.  Inside a block, row m starts at
// m * pitch and its 16-byte chunks are permuted by the swizzle that matches the
// pitch (bits [4, 4+b) of the byte offset XOR bits [7, 7+b), b = log2(pitch/16)),
// which is the canonical 128/64/32-byte swizzled K-major layout of the MMA
// descriptors: 8-row groups `8 * pitch` bytes apart.  Tiles start on 1024-byte
// boundaries so the swizzle phase is that of the absolute address.
#pragma once
#include <cstdint>

namespace te {
namespace tc {

__device__ __forceinline__ uint32_t smem_addr(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

// byte offset of element (m, k) of a tile with `rows` rows, K = n, 4-byte elements
__host__ __device__ __forceinline__ uint32_t tile_offset(int m, int k, int rows, int n) {
  const int pitch = n >= 32 ? 128 : 4 * n;
  const int ka = k >> 5, kk = k & 31;
  uint32_t o = (uint32_t)m * pitch + (uint32_t)kk * 4;
  const uint32_t mask = pitch / 16 - 1;
  o ^= ((o >> 7) & mask) << 4;
  return (uint32_t)ka * rows * pitch + o;
}

// the same layout for 2-byte elements (BF16 operand tiles): pitch = min(2n, 128)
// bytes, so a K atom holds pitch / 2 elements
__host__ __device__ __forceinline__ uint32_t tile_offset16(int m, int k, int rows, int n) {
  const int pitch = 2 * n >= 128 ? 128 : 2 * n;
  const int per = pitch / 2;
  const int ka = k / per, kk = k % per;
  uint32_t o = (uint32_t)m * pitch + (uint32_t)kk * 2;
  const uint32_t mask = pitch / 16 - 1;
  o ^= ((o >> 7) & mask) << 4;
  return (uint32_t)ka * rows * pitch + o;
}

// shared-memory matrix descriptor of a K-major swizzled tile with rows of
// `pitch` bytes (128, 64 or 32), starting at the byte address `addr`
__device__ __forceinline__ uint64_t smem_desc_pitch(uint32_t addr, int pitch) {
  const uint64_t layout = pitch == 128 ? 2 : (pitch == 64 ? 4 : 6);  // 128B / 64B / 32B swizzle
  uint64_t d = 0;
  d |= (uint64_t)((addr & 0x3FFFF) >> 4);
  d |= (uint64_t)1 << 16;
  d |= (uint64_t)((8 * pitch) >> 4) << 32;
  d |= (uint64_t)1 << 46;
  d |= layout << 61;
  return d;
}

// shared-memory matrix descriptor of a K-major swizzled tile (starting at the
// byte address `addr`, already offset to the row block and K step)
__device__ __forceinline__ uint64_t smem_desc(uint32_t addr, int n) {
  const int pitch = n >= 32 ? 128 : 4 * n;
  const uint64_t layout = pitch == 128 ? 2 : (pitch == 64 ? 4 : 6);  // 128B / 64B / 32B swizzle
  uint64_t d = 0;
  d |= (uint64_t)((addr & 0x3FFFF) >> 4);         // start address
  d |= (uint64_t)1 << 16;                          // leading byte offset (unused when K stays in one atom)
  d |= (uint64_t)((8 * pitch) >> 4) << 32;         // stride byte offset: 8-row groups
  d |= (uint64_t)1 << 46;                          // descriptor version
  d |= layout << 61;
  return d;
}

// instruction descriptor: kind::tf32, FP32 accumulate, both operands K-major
__host__ __device__ constexpr uint32_t idesc_tf32(int M, int N) {
  return (1u << 4)                    // D format F32
         | (2u << 7)                  // A format TF32
         | (2u << 10)                 // B format TF32
         | ((uint32_t)(N >> 3) << 17)  // N / 8
         | ((uint32_t)(M >> 4) << 24); // M / 16
}

// instruction descriptor: kind::f16 with BF16 operands, FP32 accumulate, both K-major
__host__ __device__ constexpr uint32_t idesc_bf16(int M, int N) {
  return (1u << 4)                    // D format F32
         | (1u << 7)                  // A format BF16
         | (1u << 10)                 // B format BF16
         | ((uint32_t)(N >> 3) << 17)
         | ((uint32_t)(M >> 4) << 24);
}

// kind::f16 MMA (BF16 operands, K = 16 per instruction) with A in tensor memory: the
// 16 elements of a row's K step packed in pairs into 8 consecutive 32-bit columns
__device__ __forceinline__ void mma_bf16_ta(uint32_t d_tmem, uint32_t a_tmem, uint64_t b, uint32_t idesc,
                                            int accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], [%1], %2, %3, p;\n\t}\n" ::"r"(d_tmem),
      "r"(a_tmem), "l"(b), "r"(idesc), "r"(accumulate));
}

__device__ __forceinline__ void mma_tf32(uint32_t d_tmem, uint64_t a, uint64_t b, uint32_t idesc, int accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(d_tmem),
      "l"(a), "l"(b), "r"(idesc), "r"(accumulate));
}

// the same MMA with operand A in tensor memory: M = 128 rows in the 128 TMEM lanes, the
// K = 8 TF32 elements of a step in 8 consecutive 32-bit columns starting at `a_tmem`
__device__ __forceinline__ void mma_tf32_ta(uint32_t d_tmem, uint32_t a_tmem, uint64_t b, uint32_t idesc,
                                            int accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::tf32 [%0], [%1], %2, %3, p;\n\t}\n" ::"r"(d_tmem),
      "r"(a_tmem), "l"(b), "r"(idesc), "r"(accumulate));
}

// arrive on `bar` when every MMA this thread issued so far has completed
__device__ __forceinline__ void commit(uint64_t* bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_addr(bar))
               : "memory");
}

__device__ __forceinline__ void fence_before_sync() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_after_sync() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
// make this thread's generic-proxy shared-memory writes visible to the tensor cores
__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

// TMEM allocation: one full warp executes these
__device__ __forceinline__ void tmem_alloc(uint32_t* dst_smem, uint32_t ncols) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_addr(dst_smem)),
               "r"(ncols)
               : "memory");
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}

// 16 consecutive 32-bit columns of this thread's TMEM lane
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float (&v)[16]) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
      "%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
        "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
#pragma unroll
  for (int i = 0; i < 16; i++) v[i] = __uint_as_float(r[i]);
}
// 8 consecutive 32-bit columns of this thread's TMEM lane
__device__ __forceinline__ void tmem_ld8(uint32_t taddr, float (&v)[8]) {
  uint32_t r[8];
  asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7])
               : "r"(taddr));
#pragma unroll
  for (int i = 0; i < 8; i++) v[i] = __uint_as_float(r[i]);
}
__device__ __forceinline__ void tmem_ld_wait() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }

// store 16 / 8 consecutive 32-bit columns of this thread's TMEM lane
__device__ __forceinline__ void tmem_st16(uint32_t taddr, const float (&v)[16]) {
  asm volatile(
      "tcgen05.st.sync.aligned.32x32b.x16.b32 [%0], {%1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
      "%15, %16};" ::"r"(taddr),
      "r"(__float_as_uint(v[0])), "r"(__float_as_uint(v[1])), "r"(__float_as_uint(v[2])), "r"(__float_as_uint(v[3])),
      "r"(__float_as_uint(v[4])), "r"(__float_as_uint(v[5])), "r"(__float_as_uint(v[6])), "r"(__float_as_uint(v[7])),
      "r"(__float_as_uint(v[8])), "r"(__float_as_uint(v[9])), "r"(__float_as_uint(v[10])), "r"(__float_as_uint(v[11])),
      "r"(__float_as_uint(v[12])), "r"(__float_as_uint(v[13])), "r"(__float_as_uint(v[14])),
      "r"(__float_as_uint(v[15]))
      : "memory");
}
__device__ __forceinline__ void tmem_st8(uint32_t taddr, const float (&v)[8]) {
  asm volatile("tcgen05.st.sync.aligned.32x32b.x8.b32 [%0], {%1, %2, %3, %4, %5, %6, %7, %8};" ::"r"(taddr),
               "r"(__float_as_uint(v[0])), "r"(__float_as_uint(v[1])), "r"(__float_as_uint(v[2])),
               "r"(__float_as_uint(v[3])), "r"(__float_as_uint(v[4])), "r"(__float_as_uint(v[5])),
               "r"(__float_as_uint(v[6])), "r"(__float_as_uint(v[7]))
               : "memory");
}
__device__ __forceinline__ void tmem_st4u(uint32_t taddr, const uint32_t (&v)[4]) {
  asm volatile("tcgen05.st.sync.aligned.32x32b.x4.b32 [%0], {%1, %2, %3, %4};" ::"r"(taddr), "r"(v[0]), "r"(v[1]),
               "r"(v[2]), "r"(v[3])
               : "memory");
}
__device__ __forceinline__ void tmem_st_wait() { asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory"); }

// mbarrier with a single expected arrival per phase
__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
// test the phase; while it is incomplete the thread is suspended in hardware (issuing
// nothing) until it completes or about `suspend_ns` nanoseconds have passed
__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity, uint32_t suspend_ns = 1000000u) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n\tselp.u32 %0, 1, 0, p;\n\t}\n"
      : "=r"(ok)
      : "r"(smem_addr(bar)), "r"(parity), "r"(suspend_ns)
      : "memory");
  return ok != 0;
}
// wait for the phase with the given parity to complete; false after ~`limit` clock cycles
// (each try suspends for at most about a millisecond, so the limit is checked regularly)
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, long long limit) {
  long long t0 = clock64();
  while (!mbar_try_wait(bar, parity))
    if (clock64() - t0 > limit) return false;
  return true;
}

// round to TF32 (10 explicit mantissa bits), nearest, ties away from zero
__device__ __forceinline__ float to_tf32(float x) {
  uint32_t r;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
  return __uint_as_float(r);
}

}  // namespace tc
}  // namespace te
