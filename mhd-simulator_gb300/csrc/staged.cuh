// staged.cuh -- shared-memory plane staging helpers of the stencil kernels:
// zero-filling cp.async copies, the coefficient record types of the level
// precisions, and wrapped coordinates.
#pragma once
#include "common.cuh"

namespace mhdproj {
namespace staged {

// cp.async with zero fill: `valid` false copies nothing and writes zeros,
// which is the value of a cell outside a closed boundary.
__device__ __forceinline__ void cp_async4(void* smem, const void* gmem, bool valid) {
    const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
    const int n = valid ? 4 : 0;
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4, %2;\n" ::"r"(s), "l"(gmem), "r"(n) : "memory");
}
__device__ __forceinline__ void cp_async8(void* smem, const void* gmem, bool valid) {
    const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
    const int n = valid ? 8 : 0;
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8, %2;\n" ::"r"(s), "l"(gmem), "r"(n) : "memory");
}
__device__ __forceinline__ void cp_async16(void* smem, const void* gmem, bool valid) {
    const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
    const int n = valid ? 16 : 0;
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(s), "l"(gmem), "r"(n) : "memory");
}
// Copy of two consecutive cells of a vector field (8 bytes FP32, 4 bytes
// FP16/BF16).
template <class VT>
__device__ __forceinline__ void cp_async_pair(void* smem, const VT* gmem, bool valid) {
    if (sizeof(VT) == 4) cp_async8(smem, gmem, valid);
    else cp_async4(smem, gmem, valid);
}
__device__ __forceinline__ void cp_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_wait() { asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory"); }

// Coefficient records: FP32 float4 (beta_x, beta_y, beta_z, reaction) or four
// FP16/BF16 values packed in 8 bytes.
template <int CK> struct CoefStore { using T = uint2; };
template <> struct CoefStore<0> { using T = float4; };

template <int CK> __device__ __forceinline__ float4 unpack(const typename CoefStore<CK>::T& v);
template <> __device__ __forceinline__ float4 unpack<0>(const float4& v) { return v; }
template <> __device__ __forceinline__ float4 unpack<1>(const uint2& u) {
    const __half2 a = *reinterpret_cast<const __half2*>(&u.x), b = *reinterpret_cast<const __half2*>(&u.y);
    const float2 fa = __half22float2(a), fb = __half22float2(b);
    return make_float4(fa.x, fa.y, fb.x, fb.y);
}
template <> __device__ __forceinline__ float4 unpack<2>(const uint2& u) {
    const __nv_bfloat162 a = *reinterpret_cast<const __nv_bfloat162*>(&u.x);
    const __nv_bfloat162 b = *reinterpret_cast<const __nv_bfloat162*>(&u.y);
    const float2 fa = __bfloat1622float2(a), fb = __bfloat1622float2(b);
    return make_float4(fa.x, fa.y, fb.x, fb.y);
}

// Wrapped or absent coordinate along one axis.
__device__ __forceinline__ int axis_src(int c, int n, bool periodic, bool* ok) {
    if (c < 0) {
        *ok = periodic;
        return periodic ? c + n : 0;
    }
    if (c >= n) {
        *ok = periodic;
        return periodic ? c - n : n - 1;
    }
    *ok = true;
    return c;
}

// Rotating slot indices of the plane rings: index of plane zA + k.
struct Slots {
    int j3, j4, j5;
    __device__ __forceinline__ Slots() : j3(0), j4(0), j5(0) {}
    __device__ __forceinline__ void next() {
        j3 = j3 == 2 ? 0 : j3 + 1;
        j4 = (j4 + 1) & 3;
        j5 = j5 == 4 ? 0 : j5 + 1;
    }
    __device__ __forceinline__ int s3(int k) const {  // k in -2 .. 2
        int v = j3 + k;
        v = v < 0 ? v + 3 : v;
        return v >= 3 ? v - 3 : v;
    }
    __device__ __forceinline__ int s4(int k) const { return (j4 + k) & 3; }
    __device__ __forceinline__ int s5(int k) const {  // k in -4 .. 4
        int v = j5 + k;
        v = v < 0 ? v + 5 : v;
        return v >= 5 ? v - 5 : v;
    }
};

}  // namespace staged
}  // namespace mhdproj
