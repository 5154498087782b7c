// Helpers shared by the tcgen05 kernels (tc_m2l.cu, tc_rcr3.cu): the no-swizzle K-major
// core-matrix layout of shared-memory operands, shared-memory matrix descriptors, TF32 hi/lo
// splitting, and mbarrier waits with a time limit.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace fmm {

// byte offset of element (row r, k) in a no-swizzle K-major tile of KC columns: 8-row x 16-byte
// core matrices, K-adjacent cores 128 B apart (leading byte offset), 8-row groups 32 KC apart
// (stride byte offset)
__host__ __device__ __forceinline__ uint32_t core_off(int r, int k, int KC)
{
    return (uint32_t)((r >> 3) * 32 * KC + (k >> 2) * 128 + (r & 7) * 16 + (k & 3) * 4);
}

// x rounded to the nearest TF32 value (10 explicit mantissa bits; halves away from zero) by
// adding half a TF32 unit to the magnitude bits and clearing the 13 low bits.  As the hi part of
// a split, x = hi + lo with lo = tf32_round(x - hi) keeps about 24 bits, against about 20 for
// truncated halves.
__host__ __device__ __forceinline__ uint32_t tf32_round_bits(uint32_t u) { return (u + 0x1000u) & 0xffffe000u; }
__device__ __forceinline__ float tf32_round(float x) { return __uint_as_float(tf32_round_bits(__float_as_uint(x))); }

__device__ __forceinline__ uint32_t smem_u32(const void *ptr) { return (uint32_t)__cvta_generic_to_shared(ptr); }

// shared-memory matrix descriptor (no swizzle): start, leading and stride byte offsets (>> 4),
// descriptor version 1 at bits 46-47
__device__ __forceinline__ uint64_t smem_desc(uint32_t addr, uint32_t lbo, uint32_t sbo)
{
    return (uint64_t)((addr >> 4) & 0x3FFF) | ((uint64_t)((lbo >> 4) & 0x3FFF) << 16) |
           ((uint64_t)((sbo >> 4) & 0x3FFF) << 32) | ((uint64_t)1 << 46);
}

// wait for the phase of the given parity of an mbarrier, at most `limit` SM clock cycles;
// false when the wait gave up
__device__ __forceinline__ bool mbar_wait_limit(uint32_t bar, uint32_t parity, long long limit)
{
    long long t0 = clock64();
    for (int tries = 0;; tries++) {
        uint32_t done;
        asm volatile("{\n\t.reg .pred q;\n\tmbarrier.try_wait.parity.shared::cta.b64 q, [%1], %2;\n\tselp.u32 %0, 1, 0, q;\n\t}"
                     : "=r"(done) : "r"(bar), "r"(parity) : "memory");
        if (done) return true;
        if (clock64() - t0 > limit) return false;
        // a waiting warp leaves its issue slots to the warps that work
        if (tries >= 4) __nanosleep(64);
    }
}

// the kernel's waits: at most ~1 s of SM clock
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity) { return mbar_wait_limit(bar, parity, 2000000000LL); }

__device__ __forceinline__ void mbar_arrive(uint32_t bar)
{
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(bar) : "memory");
}


} // namespace fmm
