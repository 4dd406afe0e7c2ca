// noalloc.cu -- divergence statistics of a face-velocity field that allocate
// nothing: the reduction scratch is a fixed array in the library's device
// image instead of memory obtained from cudaMalloc.
//
// Who needs it: code that must not allocate device memory once it is running
// -- a time loop that reserved its whole memory budget at start-up, or a
// diagnostics hook called from another library's stream without a projection
// context -- and still wants to check how divergence-free a field is.
//
// Limits: the scratch holds one partial pair per block for at most
// NOALLOC_MAX_BLOCKS blocks of 32x8 (x, y) cells, so a plane may have at most
// 4096 such tiles (nx*ny up to about one million cells); larger planes are
// rejected.  The array is shared by every call on a device and keeps the
// previous call's contents; each call clears the completion counter first.
// Calls that overlap on the GPU (two streams at once) race on the array.
// The first call on a device looks up the array's device address.  Every call
// waits for its result on the host, so none may be made on a stream that is
// being captured into a CUDA graph.
#include <cuda_runtime.h>

#include <algorithm>
#include <climits>
#include <cmath>
#include <mutex>
#include <string>

#include "../../include/mhdproj.h"
#include "common.cuh"

namespace mhdproj {
void set_global_error(const std::string& msg);
}

namespace {
using namespace mhdproj;

constexpr int NOALLOC_MAX_BLOCKS = 4096;
// [0, MAXB): per-block max |div|; [MAXB, 2 MAXB): per-block sum div^2;
// [2 MAXB, 3 MAXB): per-block fluid-cell count; [3 MAXB]: max; [3 MAXB + 1]:
// sum; [3 MAXB + 2]: count; [3 MAXB + 3]: completion counter (u32).
// 12,296 doubles = 96 KiB per device.
constexpr int NOALLOC_SLOTS = 3 * NOALLOC_MAX_BLOCKS + 8;
constexpr int RES = 3 * NOALLOC_MAX_BLOCKS;
static __device__ __align__(256) double g_noalloc_scratch[NOALLOC_SLOTS];

constexpr int MAX_DEVICES = 64;
std::mutex g_mutex;
double* g_scratch_addr[MAX_DEVICES] = {};

__global__ void __launch_bounds__(TILE_THREADS) k_divergence_static(Grid3 g, float h, const uint8_t* __restrict__ solid,
                                                                    const float* __restrict__ u,
                                                                    const float* __restrict__ v,
                                                                    const float* __restrict__ w, double* scratch,
                                                                    int nblocks) {
    __shared__ double sh[8 * 2];
    __shared__ double shm[8];
    __shared__ bool last;
    const int nx = g.nx, ny = g.ny, nz = g.nz;
    const float inv_h = 1.0f / h;
    const int x = blockIdx.x * TX + threadIdx.x;
    const int y = blockIdx.y * TY + threadIdx.y;
    const int z0 = blockIdx.z * g.zper, z1 = min(g.nz, z0 + g.zper);
    float mx = 0.0f;
    Acc acc;
    double cnt = 0.0;
    if (x < nx && y < ny) {
        for (int z = z0; z < z1; z++) {
            const int i = x + nx * (y + ny * z);
            if (solid[i]) continue;
            cnt += 1.0;
            // on a periodic axis the high face of the last cell is face 0
            const int xh = (x + 1 == nx && (g.periodic & 1u)) ? 0 : x + 1;
            const int yh = (y + 1 == ny && (g.periodic & 2u)) ? 0 : y + 1;
            const int zh = (z + 1 == nz && (g.periodic & 4u)) ? 0 : z + 1;
            df d = two_sum(u[xh + (nx + 1) * (y + ny * z)], -u[x + (nx + 1) * (y + ny * z)]);
            d = df_add(d, two_sum(v[x + nx * (yh + (ny + 1) * z)], -v[x + nx * (y + (ny + 1) * z)]));
            d = df_add(d, two_sum(w[x + nx * (y + ny * zh)], -w[x + nx * (y + ny * z)]));
            const float dv = df_to_f(d) * inv_h;
            mx = fmaxf(mx, fabsf(dv));
            acc.add_prod(dv, dv);
        }
    }
    const int t = threadIdx.x + blockDim.x * threadIdx.y;
    const double m = warp_max((double)mx);
    if ((t & 31) == 0) shm[t >> 5] = m;
    double s1[2] = {acc.total(), cnt};
    block_sum<2>(s1, sh);
    const int b = blockIdx.x + gridDim.x * (blockIdx.y + gridDim.y * blockIdx.z);
    unsigned int* counter = reinterpret_cast<unsigned int*>(scratch + RES + 3);
    if (t == 0) {
        double mm = 0.0;
        for (int k = 0; k < 8; k++) mm = fmax(mm, shm[k]);
        scratch[b] = mm;
        scratch[NOALLOC_MAX_BLOCKS + b] = s1[0];
        scratch[2 * NOALLOC_MAX_BLOCKS + b] = s1[1];
        __threadfence();
        last = atomicAdd(counter, 1u) == (unsigned)(nblocks - 1);
    }
    __syncthreads();
    if (!last) return;
    __threadfence();
    double mb = 0.0, sb = 0.0, cb = 0.0;
    for (int k = t; k < nblocks; k += TILE_THREADS) {
        mb = fmax(mb, ((volatile double*)scratch)[k]);
        sb += ((volatile double*)scratch)[NOALLOC_MAX_BLOCKS + k];
        cb += ((volatile double*)scratch)[2 * NOALLOC_MAX_BLOCKS + k];
    }
    mb = warp_max(mb);
    __syncthreads();
    if ((t & 31) == 0) shm[t >> 5] = mb;
    double s2[2] = {sb, cb};
    block_sum<2>(s2, sh);
    if (t == 0) {
        double mm = 0.0;
        for (int k = 0; k < 8; k++) mm = fmax(mm, shm[k]);
        scratch[RES] = mm;
        scratch[RES + 1] = s2[0];
        scratch[RES + 2] = s2[1];
        *counter = 0u;
    }
}

// Set-up, once per device with that device current: the host-side symbol is
// not a device address, so ask the runtime for the array's address.
cudaError_t scratch_address(double** out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= MAX_DEVICES) return cudaErrorInvalidDevice;
    std::lock_guard<std::mutex> lock(g_mutex);
    if (!g_scratch_addr[dev]) {
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess) return e;
        g_scratch_addr[dev] = static_cast<double*>(p);
    }
    *out = g_scratch_addr[dev];
    return cudaSuccess;
}
}  // namespace

extern "C" int mhdproj_divergence_noalloc(const mhdproj_grid* grid, const uint8_t* solid, const float* u,
                                          const float* v, const float* w, double* out, void* stream) {
    if (!grid || !solid || !u || !v || !w || !out) {
        set_global_error("mhdproj_divergence_noalloc: grid, solid, u, v, w and out must not be NULL");
        return MHDPROJ_ERR_INVALID;
    }
    if (grid->nx == 0 || grid->ny == 0 || grid->nz == 0 || !(grid->h > 0.0f)) {
        set_global_error("mhdproj_divergence_noalloc: invalid grid");
        return MHDPROJ_ERR_INVALID;
    }
    // every index is a 32-bit int in the kernel: each array must stay below 2^31 elements
    const long long nx = grid->nx, ny = grid->ny, nz = grid->nz;
    const long long largest = std::max(std::max((nx + 1) * ny * nz, nx * (ny + 1) * nz), nx * ny * (nz + 1));
    if (nx > INT_MAX || ny > INT_MAX || nz > INT_MAX || largest >= (1ll << 31)) {
        set_global_error("mhdproj_divergence_noalloc: a face array of 2^31 or more elements is not supported");
        return MHDPROJ_ERR_INVALID;
    }
    const long long tiles = ((nx + TX - 1) / TX) * ((ny + TY - 1) / TY);
    if (tiles > NOALLOC_MAX_BLOCKS) {
        set_global_error("mhdproj_divergence_noalloc: an x-y plane of more than 4096 tiles of 32x8 cells "
                         "exceeds the fixed scratch (nx*ny up to about 1M cells)");
        return MHDPROJ_ERR_INVALID;
    }
    double* scratch = nullptr;
    cudaError_t e = scratch_address(&scratch);
    if (e != cudaSuccess) {
        set_global_error(std::string("mhdproj_divergence_noalloc: cudaGetSymbolAddress: ") + cudaGetErrorString(e));
        return MHDPROJ_ERR_CUDA;
    }
    cudaStream_t s = (cudaStream_t)stream;
    int zc = (int)(NOALLOC_MAX_BLOCKS / tiles);
    if (zc > (int)grid->nz) zc = (int)grid->nz;
    if (zc > 8) zc = 8;
    if (zc < 1) zc = 1;
    Grid3 g;
    g.nx = grid->nx;
    g.ny = grid->ny;
    g.nz = grid->nz;
    g.periodic = grid->periodic;
    g.zper = (g.nz + zc - 1) / zc;
    zc = (g.nz + g.zper - 1) / g.zper;
    const dim3 gridDim((grid->nx + TX - 1) / TX, (grid->ny + TY - 1) / TY, zc);
    const int nblocks = (int)(gridDim.x * gridDim.y * gridDim.z);
    // the completion counter must start at zero
    e = cudaMemsetAsync(scratch + RES + 3, 0, sizeof(double), s);
    if (e == cudaSuccess) {
        k_divergence_static<<<gridDim, dim3(TX, TY, 1), 0, s>>>(g, grid->h, solid, u, v, w, scratch, nblocks);
        e = cudaGetLastError();
    }
    double res[3] = {0.0, 0.0, 0.0};
    if (e == cudaSuccess) e = cudaMemcpyAsync(res, scratch + RES, 3 * sizeof(double), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) {
        set_global_error(std::string("mhdproj_divergence_noalloc: ") + cudaGetErrorString(e));
        return MHDPROJ_ERR_CUDA;
    }
    out[0] = res[0];
    out[1] = res[2] > 0.0 ? std::sqrt(res[1] / res[2]) : 0.0;
    return 0;
}
