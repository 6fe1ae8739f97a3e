// blocks.cuh -- 2x2 block arithmetic and warp reductions shared by the CUDA units.
#pragma once
#include <cuda_runtime.h>

// 2x2 block [a b; c d], row-major, 32-byte aligned (one 256-bit access per block)
using blk4 = double4_32a;
__host__ __device__ __forceinline__ blk4 mk4(double a, double b, double c, double e) {
    blk4 r;
    r.x = a; r.y = b; r.z = c; r.w = e;
    return r;
}

// Correctly rounded reciprocal of a pivot block's determinant: the same value
// as 1 / det (one real number, one rounding), by the reciprocal intrinsic
// rather than a general division.
__device__ __forceinline__ float rcp_rn(float x) { return __frcp_rn(x); }
__device__ __forceinline__ double rcp_rn(double x) { return __drcp_rn(x); }

// ------------------------------------------------------------------ helpers
__device__ __forceinline__ blk4 mm(blk4 a, blk4 b) {  // 2x2 row-major product
    return mk4(a.x * b.x + a.y * b.z, a.x * b.y + a.y * b.w,
                        a.z * b.x + a.w * b.z, a.z * b.y + a.w * b.w);
}
__device__ __forceinline__ blk4 sub4(blk4 a, blk4 b) {
    return mk4(a.x - b.x, a.y - b.y, a.z - b.z, a.w - b.w);
}
__device__ __forceinline__ blk4 add4(blk4 a, blk4 b) {
    return mk4(a.x + b.x, a.y + b.y, a.z + b.z, a.w + b.w);
}
__device__ __forceinline__ double2 mv(blk4 a, double2 v) {
    return make_double2(a.x * v.x + a.y * v.y, a.z * v.x + a.w * v.y);
}
__device__ __forceinline__ blk4 shfl4(blk4 v, int src) {
    return mk4(__shfl_sync(0xffffffffu, v.x, src), __shfl_sync(0xffffffffu, v.y, src),
                        __shfl_sync(0xffffffffu, v.z, src), __shfl_sync(0xffffffffu, v.w, src));
}
__device__ __forceinline__ blk4 warp_sum4(blk4 v) {
    for (int o = 16; o > 0; o >>= 1) {
        v.x += __shfl_xor_sync(0xffffffffu, v.x, o);
        v.y += __shfl_xor_sync(0xffffffffu, v.y, o);
        v.z += __shfl_xor_sync(0xffffffffu, v.z, o);
        v.w += __shfl_xor_sync(0xffffffffu, v.w, o);
    }
    return v;
}
__device__ __forceinline__ double2 warp_sum2(double2 v) {
    for (int o = 16; o > 0; o >>= 1) {
        v.x += __shfl_xor_sync(0xffffffffu, v.x, o);
        v.y += __shfl_xor_sync(0xffffffffu, v.y, o);
    }
    return v;
}
__device__ __forceinline__ void atomic_max_nonneg(unsigned long long *a, double v) {
    atomicMax(a, (unsigned long long)__double_as_longlong(v));
}
// Smith's complex division (a+ib)/(c+id).
__device__ __forceinline__ double2 cdiv(double a, double b, double c, double d) {
    if (fabs(c) >= fabs(d)) {
        const double r = d / c, den = c + d * r;
        return make_double2((a + b * r) / den, (b - a * r) / den);
    }
    const double r = c / d, den = c * r + d;
    return make_double2((a * r + b) / den, (b * r - a) / den);
}

