// Warp-MMA building blocks of the d = 32 chunk kernel (mgb_mma32.cu): scaled
// FP16 piece tiles in shared memory, ldmatrix fragment loads, mma.sync
// m16n8k16 (FP16 in, FP32 accumulate), the exact two-piece split, the
// per-matrix power-of-two scale, and the bulk copy (cp.async.bulk) of a
// contiguous range into shared memory on an mbarrier.
//
// Pieces: an FP32 matrix X with max |x| in [2^e, 2^(e+1)) is scaled by
// 2^k, k = 14 - e (exact), so that max |x 2^k| < 2^15 < 65504, and split as
// x 2^k = x0 + x1 + r with x0 = fp16(x 2^k), x1 = fp16(x 2^k - x0) (the
// difference is exact in FP32): |r| <= 2^-22 |x 2^k| for normal x1, and
// below 2^-25 absolute where x1 is subnormal, i.e. 2^-39 of the largest
// element.  A product is X0 Y0 + X0 Y1 + X1 Y0 (X1 Y1 <= 2^-22 relative is
// dropped), rescaled by 2^-(kx + ky) in FP32: 7e-8 relative per 32^3
// product on random data, against 1.0e-7 for FP32 FMA and 2.7e-8 for a
// six-product three-piece BF16 split at twice the tensor work.
//
// A piece tile holds one 32 x 32 operand piece as 64-byte rows, the 16-byte
// chunk c of row r stored at c ^ ((r >> 1) & 3): ldmatrix of 8 consecutive
// rows and the row stores of two consecutive rows are free of bank conflicts.
#pragma once

#include <cstdint>
#include <cuda_fp16.h>

#include "mgb_tc.cuh"

namespace mgb {
namespace wm {

constexpr uint32_t PT = 32 * 64;  // bytes per piece tile (32 rows x 64 B)
constexpr int NPC = 2;            // pieces per operand

// byte offset of (row, col) in a piece tile; col a multiple of 8 for ldmatrix rows
__device__ __forceinline__ uint32_t toff(int r, int c) {
    return (uint32_t)r * 64u + ((uint32_t)((c >> 3) ^ ((r >> 1) & 3)) << 4) + (uint32_t)(c & 7) * 2u;
}

__device__ __forceinline__ void ldsm4(uint32_t a, uint32_t (&r)[4]) {
    asm volatile("ldmatrix.sync.aligned.m8n8.x4.shared.b16 {%0,%1,%2,%3}, [%4];"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
                 : "r"(a));
}
__device__ __forceinline__ void ldsm4t(uint32_t a, uint32_t (&r)[4]) {
    asm volatile("ldmatrix.sync.aligned.m8n8.x4.trans.shared.b16 {%0,%1,%2,%3}, [%4];"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
                 : "r"(a));
}
__device__ __forceinline__ void mma16816(float (&c)[4], const uint32_t (&a)[4], uint32_t b0, uint32_t b1) {
    asm("mma.sync.aligned.m16n8k16.row.col.f32.f16.f16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, {%0,%1,%2,%3};"
        : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}
// d = a b (the accumulator starts from zero; no register to clear first)
__device__ __forceinline__ void mma16816_first(float (&d)[4], const uint32_t (&a)[4], uint32_t b0, uint32_t b1) {
    asm("mma.sync.aligned.m16n8k16.row.col.f32.f16.f16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, {%10,%10,%10,%10};"
        : "=f"(d[0]), "=f"(d[1]), "=f"(d[2]), "=f"(d[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1), "f"(0.f));
}

// |x| as ordered integer bits (non-negative floats order like their bits)
__device__ __forceinline__ uint32_t absbits(float x) { return __float_as_uint(x) & 0x7fffffffu; }
// the scale exponent k for a matrix whose max |x| has the bits u
__device__ __forceinline__ int scale_exp(uint32_t u) {
    const int e = (int)(u >> 23) - 127;
    return min(126, max(-126, 14 - e));
}
// 2^k for |k| <= 126 (a normal float)
__device__ __forceinline__ float pow2f(int k) { return __int_as_float((127 + k) << 23); }
// warp-wide max of u into *slot (shared memory), one atomic per warp; every
// lane of the warp must call it
__device__ __forceinline__ void max_into(uint32_t* slot, uint32_t u) {
    const uint32_t w = __reduce_max_sync(0xffffffffu, u);
    if ((threadIdx.x & 31) == 0) atomicMax(slot, w);
}

// Exact two-piece FP16 split of (x, y) 2^k (sc = 2^k), packed per piece (low
// half = the first value).
__device__ __forceinline__ void split2(float x, float y, float sc, uint32_t& p0, uint32_t& p1) {
    const float xs = x * sc, ys = y * sc;
    const __half2 h0 = __floats2half2_rn(xs, ys);
    const float2 f0 = __half22float2(h0);
    const __half2 h1 = __floats2half2_rn(xs - f0.x, ys - f0.y);
    p0 = *reinterpret_cast<const uint32_t*>(&h0);
    p1 = *reinterpret_cast<const uint32_t*>(&h1);
}

// Store a pair (row r, columns c, c+1) of FP32 values as pieces of tile set t.
__device__ __forceinline__ void put_pair(uint8_t* t, int r, int c, float x, float y, float sc) {
    uint32_t p0, p1;
    split2(x, y, sc, p0, p1);
    const uint32_t o = toff(r, c);
    *reinterpret_cast<uint32_t*>(t + o) = p0;
    *reinterpret_cast<uint32_t*>(t + PT + o) = p1;
}

// Store four consecutive FP32 values (row r, columns c..c+3, c % 4 == 0).
__device__ __forceinline__ void put_quad(uint8_t* t, int r, int c, float4 v, float sc) {
    uint32_t a0, a1, b0, b1;
    split2(v.x, v.y, sc, a0, a1);
    split2(v.z, v.w, sc, b0, b1);
    const uint32_t o = toff(r, c);
    *reinterpret_cast<uint2*>(t + o) = make_uint2(a0, b0);
    *reinterpret_cast<uint2*>(t + PT + o) = make_uint2(a1, b1);
}

__device__ __forceinline__ uint32_t max4(float4 v) {
    return max(max(absbits(v.x), absbits(v.y)), max(absbits(v.z), absbits(v.w)));
}

// Bulk copy of `bytes` (a multiple of 16) from global to shared memory,
// completing on the mbarrier.
__device__ __forceinline__ void bulk_load(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
    const uint32_t b = tc::su32(bar);
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(b), "r"(bytes) : "memory");
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(tc::su32(dst)),
        "l"(src), "r"(bytes), "r"(b)
        : "memory");
}

}  // namespace wm
}  // namespace mgb
