// Fifth-generation tensor cores (tcgen05, sm_100 family; sm_103a here) in inline PTX: tensor-memory
// (TMEM) allocation, shared-memory matrix descriptors, the TF32 matrix multiply-accumulate issued by
// one thread, its completion on an mbarrier, and TMEM loads into registers.
//
// Operands live in shared memory in the canonical K-major layout without swizzling: 8-row x 16-byte
// core matrices (8 rows of 4 TF32 values), rows of a core matrix 16 bytes apart; LBO is the byte
// distance between core matrices along K, SBO between core matrices along M (or N). The contraction
// operands here have K = 8 (two K-chunks of 4): element (r, k) of an operand sits at byte
//   (r / 8) * SBO + (k / 4) * LBO + (r % 8) * 16 + (k % 4) * 4,   LBO = 128, SBO = 256.
// The accumulator D (M = 128 rows, N columns, FP32) occupies TMEM lanes 0..127 (row r in lane r)
// and N consecutive columns from its base address; warp w of a warpgroup reads lanes 32(w%4)..+31.
//
// FP32-accurate products from TF32 inputs: x = hi + lo with hi = tf32(x) (round to nearest) and
// lo = x - hi (exact in FP32); a*b ~ a_hi b_hi + a_hi b_lo + a_lo b_hi, each a tensor-core MMA with
// FP32 accumulation (the a_lo b_lo term and lo's own TF32 rounding are below 2^-20 relative).
#pragma once
#include <cstdint>

#include "dg_tma.cuh"

namespace dg {
namespace tc {

constexpr uint32_t kLBO = 128, kSBO = 256;

// Byte offset of element (r, k) of a K = 8 operand in the canonical layout.
__host__ __device__ constexpr uint32_t operand_offset(int r, int k) {
    return (r >> 3) * kSBO + (k >> 2) * kLBO + (r & 7) * 16 + (k & 3) * 4;
}
// Bytes of an operand of `rows` rows (a multiple of 8), K = 8.
__host__ __device__ constexpr uint32_t operand_bytes(int rows) { return (rows >> 3) * kSBO; }

// Shared-memory matrix descriptor (tcgen05): start address, LBO, SBO (all >> 4), the fixed
// version bits 46-48 = 0b001, base offset 0, no swizzling.
__device__ __forceinline__ uint64_t smem_desc(const void* p) {
    const uint64_t addr = smem_u32(p);
    return ((addr & 0x3FFFFull) >> 4) | (static_cast<uint64_t>(kLBO >> 4) << 16) |
           (static_cast<uint64_t>(kSBO >> 4) << 32) | (1ull << 46);
}

// Instruction descriptor of kind::tf32: D in FP32, A and B TF32, both K-major, M x N.
__host__ __device__ constexpr uint32_t idesc_tf32(int M, int N) {
    return (1u << 4) | (2u << 7) | (2u << 10) | (static_cast<uint32_t>(N >> 3) << 17) |
           (static_cast<uint32_t>(M >> 4) << 24);
}

// Round-to-nearest TF32 part of x (an FP32 bit pattern with the low 13 mantissa bits zero).
__device__ __forceinline__ float tf32_hi(float x) {
    uint32_t r;
    asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
    return __uint_as_float(r);
}

// Allocates ncols (a power of two, >= 32) TMEM columns for this CTA; the address is written to
// *slot (shared memory). Executed by one whole warp. The warp then gives up the right to allocate
// again, so that other CTAs on the SM are not kept waiting.
__device__ __forceinline__ void tmem_alloc(uint32_t* slot, uint32_t ncols) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(slot)), "r"(ncols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
// Frees the CTA's TMEM; the same warp that allocated, after every MMA and TMEM load completed.
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}

__device__ __forceinline__ void fence_before_sync() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_after_sync() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// D[taddr] (+)= A * B^T, issued by a single thread; accumulate = false overwrites D.
__device__ __forceinline__ void mma_tf32(uint32_t taddr, uint64_t adesc, uint64_t bdesc, uint32_t idesc, bool accumulate) {
    const uint32_t acc = accumulate ? 1u : 0u;
    asm volatile(
        "{\n"
        "  .reg .pred p;\n"
        "  setp.ne.u32 p, %4, 0;\n"
        "  tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n"
        "}\n" ::"r"(taddr),
        "l"(adesc), "l"(bdesc), "r"(idesc), "r"(acc)
        : "memory");
}

// The mbarrier arrives once every MMA this thread issued before has completed.
__device__ __forceinline__ void commit(uint64_t* bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
                 : "memory");
}

// 16 consecutive FP32 columns of one TMEM lane per thread (lane = lane base of taddr + lane id of
// the thread within its warp). The load and its wait are one asm statement, so no use of the
// registers can be scheduled before the data has arrived.
__device__ __forceinline__ void ld_32x32b_x16(uint32_t taddr, float* v) {
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15}, "
        "[%16];\n"
        "tcgen05.wait::ld.sync.aligned;"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
          "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr)
        : "memory");
#pragma unroll
    for (int q = 0; q < 16; ++q) v[q] = __uint_as_float(r[q]);
}

}  // namespace tc
}  // namespace dg
