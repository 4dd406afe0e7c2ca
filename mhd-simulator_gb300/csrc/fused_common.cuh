// fused_common.cuh -- helpers shared by the fused smoothing passes: the
// tile geometry, quad loads and stores of the level vectors, the split-row
// smoother records and the Gauss-Seidel neighbour sum.
#pragma once
#include <type_traits>

#include "staged.cuh"

namespace mhdproj {
namespace fused {
using namespace staged;

constexpr int PX = 64;           // cells per tile row
constexpr int QX = PX / 4;       // 16 threads per tile row, one quad each
constexpr int XO = 4;            // staged rows start at x0 - XO
constexpr int RW = PX + 2 * XO;  // 72 staged columns: x0-4 .. x0+67
constexpr int HW = RW / 2;       // 36 columns per half row (even x, then odd x)
constexpr int NQ = RW / 4;       // 18 quads per staged row

// Quads of a vector field as loaded (16 bytes FP32, 8 bytes FP16/BF16),
// kept in the load type until the stage that uses them: a conversion right
// after the load would wait for the load.
template <class VT> struct Raw4 { using T = float4; };
template <> struct Raw4<__half> { using T = uint2; };
template <> struct Raw4<__nv_bfloat16> { using T = uint2; };
template <class VT>
__device__ __forceinline__ typename Raw4<VT>::T ldg_quad(const VT* p, bool ok) {
    using R = typename Raw4<VT>::T;
    R v;
    if (ok) v = __ldg(reinterpret_cast<const R*>(p));
    else v = R{};  // float4 / uint2: zeros
    return v;
}
template <class VT> __device__ __forceinline__ float4 cvt4r(const typename Raw4<VT>::T& v);
template <> __device__ __forceinline__ float4 cvt4r<float>(const float4& v) { return v; }
template <> __device__ __forceinline__ float4 cvt4r<__half>(const uint2& u) {
    const float2 a = __half22float2(*reinterpret_cast<const __half2*>(&u.x));
    const float2 b = __half22float2(*reinterpret_cast<const __half2*>(&u.y));
    return make_float4(a.x, a.y, b.x, b.y);
}
template <> __device__ __forceinline__ float4 cvt4r<__nv_bfloat16>(const uint2& u) {
    const float2 a = __bfloat1622float2(*reinterpret_cast<const __nv_bfloat162*>(&u.x));
    const float2 b = __bfloat1622float2(*reinterpret_cast<const __nv_bfloat162*>(&u.y));
    return make_float4(a.x, a.y, b.x, b.y);
}
template <class VT> __device__ __forceinline__ void st4(VT* p, float4 v);
template <> __device__ __forceinline__ void st4<float>(float* p, float4 v) { *reinterpret_cast<float4*>(p) = v; }
template <> __device__ __forceinline__ void st4<__half>(__half* p, float4 v) {
    const __half2 a = __floats2half2_rn(v.x, v.y), b = __floats2half2_rn(v.z, v.w);
    *reinterpret_cast<uint2*>(p) = make_uint2(*reinterpret_cast<const unsigned*>(&a), *reinterpret_cast<const unsigned*>(&b));
}
template <> __device__ __forceinline__ void st4<__nv_bfloat16>(__nv_bfloat16* p, float4 v) {
    const __nv_bfloat162 a = __floats2bfloat162_rn(v.x, v.y), b = __floats2bfloat162_rn(v.z, v.w);
    *reinterpret_cast<uint2*>(p) = make_uint2(*reinterpret_cast<const unsigned*>(&a), *reinterpret_cast<const unsigned*>(&b));
}
// Two consecutive coarse cells (a quad's parents).
template <class VT> struct Raw2 { using T = float2; };
template <> struct Raw2<__half> { using T = __half2; };
template <> struct Raw2<__nv_bfloat16> { using T = __nv_bfloat162; };
__device__ __forceinline__ void zero2(float2& v) { v = make_float2(0.f, 0.f); }
__device__ __forceinline__ void zero2(__half2& v) { v = __float2half2_rn(0.f); }
__device__ __forceinline__ void zero2(__nv_bfloat162& v) { v = __float2bfloat162_rn(0.f); }
template <class VT>
__device__ __forceinline__ typename Raw2<VT>::T ldg_pair(const VT* p, bool ok) {
    using R = typename Raw2<VT>::T;
    R v;
    if (ok) v = __ldg(reinterpret_cast<const R*>(p));
    else zero2(v);
    return v;
}
__device__ __forceinline__ float2 cvt2(const float2& v) { return v; }
__device__ __forceinline__ float2 cvt2(const __half2& v) { return __half22float2(v); }
__device__ __forceinline__ float2 cvt2(const __nv_bfloat162& v) { return __bfloat1622float2(v); }
template <class VT> __device__ __forceinline__ void st2(VT* p, float2 v);
template <> __device__ __forceinline__ void st2<float>(float* p, float2 v) { *reinterpret_cast<float2*>(p) = v; }
template <> __device__ __forceinline__ void st2<__half>(__half* p, float2 v) {
    *reinterpret_cast<__half2*>(p) = __floats2half2_rn(v.x, v.y);
}
template <> __device__ __forceinline__ void st2<__nv_bfloat16>(__nv_bfloat16* p, float2 v) {
    *reinterpret_cast<__nv_bfloat162*>(p) = __floats2bfloat162_rn(v.x, v.y);
}

// The smoother records in HBM are split along whole grid rows: row (y, z)
// holds its nx/2 even-x records, then its nx/2 odd-x records.  Position of
// column x in its row:
__device__ __forceinline__ int split_x(int x, int nx) { return (x & 1) * (nx >> 1) + (x >> 1); }

// Two adjacent records of one half row (offsets o, o+1; o even).
template <int CK, class CT>
__device__ __forceinline__ void rec2(const CT* p, float4* a, float4* b) {
    if constexpr (CK == 0) {
        *a = unpack<0>(reinterpret_cast<const float4*>(p)[0]);
        *b = unpack<0>(reinterpret_cast<const float4*>(p)[1]);
    } else {
        const uint4 u = *reinterpret_cast<const uint4*>(p);
        *a = unpack<CK>(make_uint2(u.x, u.y));
        *b = unpack<CK>(make_uint2(u.z, u.w));
    }
}

// Sums of beta * e over the six neighbours, added to acc, for the two cells
// of one colour of a quad: half h, offsets o and o+1 of the split planes
// (o = row * RW + h * HW + 2q); *d their diagonals.  c/cn: record planes z,
// z+1; e/em/ep: correction planes z, z-1, z+1.  The x neighbours lie in the
// other half: for h = 0 (even x) at other[2q-1 .. 2q+1], for h = 1 at
// other[2q .. 2q+2].
template <int CK, class CT>
__device__ __forceinline__ float2 gs_sum2(const CT* c, const CT* cn, const float* e, const float* em,
                                          const float* ep, int o, int h, float2 acc, float2* d) {
    const int ot = h ? o - HW : o + HW;  // the other half, same index
    const float2 f = *reinterpret_cast<const float2*>(e + ot);
    const float s = e[h ? ot + 2 : ot - 1];
    const float xm0 = h ? f.x : s, xp0 = h ? f.y : f.x;
    const float xm1 = h ? f.y : f.x, xp1 = h ? s : f.y;
    float4 own0, own1, yh0, yh1, zh0, zh1;
    rec2<CK>(c + o, &own0, &own1);
    rec2<CK>(c + o + RW, &yh0, &yh1);
    rec2<CK>(cn + o, &zh0, &zh1);
    const float bxh0 = unpack<CK>(c[ot + h]).x, bxh1 = unpack<CK>(c[ot + h + 1]).x;
    const float2 ym = *reinterpret_cast<const float2*>(e + o - RW);
    const float2 yp = *reinterpret_cast<const float2*>(e + o + RW);
    const float2 zm = *reinterpret_cast<const float2*>(em + o);
    const float2 zp = *reinterpret_cast<const float2*>(ep + o);
    float a0 = acc.x, a1 = acc.y;
    a0 = fmaf(own0.x, xm0, a0);
    a1 = fmaf(own1.x, xm1, a1);
    a0 = fmaf(bxh0, xp0, a0);
    a1 = fmaf(bxh1, xp1, a1);
    a0 = fmaf(own0.y, ym.x, a0);
    a1 = fmaf(own1.y, ym.y, a1);
    a0 = fmaf(yh0.y, yp.x, a0);
    a1 = fmaf(yh1.y, yp.y, a1);
    a0 = fmaf(own0.z, zm.x, a0);
    a1 = fmaf(own1.z, zm.y, a1);
    a0 = fmaf(zh0.z, zp.x, a0);
    a1 = fmaf(zh1.z, zp.y, a1);
    *d = make_float2(own0.w, own1.w);
    return make_float2(a0, a1);
}

__device__ __forceinline__ float2 divide2(float2 s, float2 d) {
    return make_float2(d.x > 0.f ? __fdividef(s.x, d.x) : 0.f, d.y > 0.f ? __fdividef(s.y, d.y) : 0.f);
}

// Red half (x parity of the red cells) of row y at plane z; x0-4 is even.
__device__ __forceinline__ int red_half(int y, int z) { return (y + z) & 1; }

template <int N>
using Phase = std::integral_constant<int, N>;

}  // namespace fused
}  // namespace mhdproj
