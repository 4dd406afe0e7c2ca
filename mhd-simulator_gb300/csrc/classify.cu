// classify.cu -- fluid mobility and cell phase lanes from the material ids,
// the thermal phase and the moving-interface field: the `phase` and
// `surface` passes of the reference (src/fluid/phase.wgsl:10-31) as driven
// by FluidState::update_cells (src/fluid/mod.rs:713-852).
//
// phase   (no interface): the liquid fraction of the fluid's material is the
//         thermal solver's state.y; a cell is mobile when it exceeds 1e-6.
//         Writes FluidCell.reserved.y (lane 13).
// surface (interface field present): the interface fraction a must lie in
//         [-eps, 1+eps] (eps = 1e-5, src/surface.rs:12) and be finite, else
//         flag bit 1; f = thermal state.y where a > 0 (1 without a thermal
//         phase); walls are cells of another non-air material; a cell is
//         mobile unless it is a wall or frozen liquid (a > 0 and f <= 1e-6).
//         Writes FluidCell.reserved = (1, f, a, interface.y) (lanes 12-15).
// Both set flag bit 0 when a cell's mobility changed; the mask holds 0/1.
//
// The inputs keep the reference's records through strides: the thermal
// packet is 16 floats per cell with state.y at float 1; the interface field
// is a vec4 per cell with (a, y) at floats 0 and 1.
#include <cuda_runtime.h>

#include <cstdint>
#include <cstdio>
#include <string>

#include "mhdproj.h"

namespace {

constexpr float kFractionTolerance = 1e-5f;

__global__ void k_classify(uint32_t n, const uint32_t* __restrict__ materials, uint32_t liquid,
                           const float* __restrict__ thermal, uint32_t thermal_stride,
                           const float* __restrict__ interface, uint32_t interface_stride, uint32_t* mask,
                           float* cells, uint32_t* flags) {
    uint32_t changed = 0;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        bool mobile;
        if (!interface) {  // phase (phase.wgsl:10-17)
            float fraction = 0.0f;
            if (materials[i] == liquid) fraction = thermal[(size_t)i * thermal_stride];
            mobile = fraction > 1e-6f;
            cells[(size_t)i * 16 + 13] = fraction;
        } else {  // surface (phase.wgsl:20-31)
            const float a = interface[(size_t)i * interface_stride];
            const float eps = kFractionTolerance;
            if (!(a >= -eps && a <= 1.0f + eps)) {
                changed |= 2u;
                continue;
            }
            float f = 1.0f;
            if (thermal && a > 0.0f) f = thermal[(size_t)i * thermal_stride];
            const uint32_t m = materials[i];
            const bool wall = m != 0u && m != liquid;
            mobile = !wall && !(a > 0.0f && f <= 1e-6f);
            float* r = cells + (size_t)i * 16 + 12;
            r[0] = 1.0f;
            r[1] = f;
            r[2] = a;
            r[3] = interface[(size_t)i * interface_stride + 1];
        }
        const bool old = mask[i] != 0u;
        if (mobile != old) {
            mask[i] = mobile ? 1u : 0u;
            changed |= 1u;
        }
    }
    // one atomic per warp
    changed = __reduce_or_sync(0xffffffffu, changed);
    if ((threadIdx.x & 31) == 0 && changed) atomicOr(flags, changed);
}

thread_local std::string g_classify_error;

int classify_fail(int code, const char* msg) {
    g_classify_error = msg;
    return code;
}

}  // namespace

extern "C" const char* mhdproj_classify_last_error(void) { return g_classify_error.c_str(); }

// Reads the changed flags back (one u32).  flags_device is caller scratch
// (one u32 on the device); the call allocates nothing.
extern "C" int mhdproj_classify_cells(const mhdproj_grid* grid, const uint32_t* materials, uint32_t liquid_material,
                                      const float* thermal, uint32_t thermal_stride, const float* interface,
                                      uint32_t interface_stride, uint32_t* mask, float* cells,
                                      uint32_t* flags_device, uint32_t* changed, void* stream) {
    g_classify_error.clear();
    if (!grid || !materials || !mask || !cells || !flags_device || !changed)
        return classify_fail(MHDPROJ_ERR_INVALID, "null argument");
    if (!interface && !thermal)
        return classify_fail(MHDPROJ_ERR_INVALID, "the phase pass needs the thermal phase field");
    if ((thermal && thermal_stride == 0) || (interface && interface_stride < 2))
        return classify_fail(MHDPROJ_ERR_INVALID, "thermal stride must be >= 1 and interface stride >= 2");
    const uint64_t n64 = (uint64_t)grid->nx * grid->ny * grid->nz;
    if (n64 == 0 || n64 > 0xFFFFFFFFull) return classify_fail(MHDPROJ_ERR_INVALID, "grid size out of range");
    const uint32_t n = (uint32_t)n64;
    cudaStream_t s = (cudaStream_t)stream;
    cudaError_t e = cudaMemsetAsync(flags_device, 0, 4, s);
    int sms = 152;
    int dev = 0;
    if (e == cudaSuccess) e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e == cudaSuccess) {
        const uint32_t want = (n + 255) / 256;
        const uint32_t cap = (uint32_t)sms * 8;
        k_classify<<<want < cap ? want : cap, 256, 0, s>>>(n, materials, liquid_material, thermal, thermal_stride,
                                                          interface, interface_stride, mask, cells, flags_device);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(changed, flags_device, 4, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) {
        char buf[256];
        snprintf(buf, sizeof buf, "classify: %s", cudaGetErrorString(e));
        return classify_fail(MHDPROJ_ERR_CUDA, buf);
    }
    if (*changed & 2u)  // src/fluid/mod.rs:838-840
        return classify_fail(MHDPROJ_ERR_INVALID,
                             "Fluid interface fractions must be finite and within the accepted [0,1] roundoff "
                             "tolerance");
    return 0;
}
