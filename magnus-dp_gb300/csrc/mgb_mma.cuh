// Warp-MMA building blocks of the d = 32 chunk kernels (mgb_mma32.cu,
// mgb_mma32t.cu): BF16 piece tiles in shared memory, ldmatrix fragment loads,
// mma.sync m16n8k16, the exact three-piece BF16 split, and the bulk copy
// (cp.async.bulk) of a contiguous range into shared memory on an mbarrier.
//
// A piece tile holds one 32 x 32 operand piece as 64-byte rows, the 16-byte
// chunk c of row r stored at c ^ ((r >> 1) & 3): ldmatrix of 8 consecutive
// rows and the row stores of two consecutive rows are free of bank conflicts.
#pragma once

#include <cstdint>
#include <cuda_bf16.h>

#include "mgb_tc.cuh"

namespace mgb {
namespace wm {

constexpr uint32_t PT = 32 * 64;  // bytes per piece tile (32 rows x 64 B)

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
    asm("mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, {%0,%1,%2,%3};"
        : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

// Exact three-piece BF16 split of two values, packed per piece (low half =
// the first value).
__device__ __forceinline__ void split2(float x, float y, uint32_t& p0, uint32_t& p1, uint32_t& p2) {
    const __nv_bfloat162 b0 = __floats2bfloat162_rn(x, y);
    const float2 f0 = __bfloat1622float2(b0);
    const float rx = x - f0.x, ry = y - f0.y;
    const __nv_bfloat162 b1 = __floats2bfloat162_rn(rx, ry);
    const float2 f1 = __bfloat1622float2(b1);
    const __nv_bfloat162 b2 = __floats2bfloat162_rn(rx - f1.x, ry - f1.y);
    p0 = *reinterpret_cast<const uint32_t*>(&b0);
    p1 = *reinterpret_cast<const uint32_t*>(&b1);
    p2 = *reinterpret_cast<const uint32_t*>(&b2);
}

// Store a pair (row r, columns c, c+1) of FP32 values as pieces of tile set t.
__device__ __forceinline__ void put_pair(uint8_t* t, int r, int c, float x, float y) {
    uint32_t p0, p1, p2;
    split2(x, y, p0, p1, p2);
    const uint32_t o = toff(r, c);
    *reinterpret_cast<uint32_t*>(t + o) = p0;
    *reinterpret_cast<uint32_t*>(t + PT + o) = p1;
    *reinterpret_cast<uint32_t*>(t + 2 * PT + o) = p2;
}

// Store four consecutive FP32 values (row r, columns c..c+3, c % 4 == 0).
__device__ __forceinline__ void put_quad(uint8_t* t, int r, int c, float4 v) {
    uint32_t a0, a1, a2, b0, b1, b2;
    split2(v.x, v.y, a0, a1, a2);
    split2(v.z, v.w, b0, b1, b2);
    const uint32_t o = toff(r, c);
    *reinterpret_cast<uint2*>(t + o) = make_uint2(a0, b0);
    *reinterpret_cast<uint2*>(t + PT + o) = make_uint2(a1, b1);
    *reinterpret_cast<uint2*>(t + 2 * PT + o) = make_uint2(a2, b2);
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
