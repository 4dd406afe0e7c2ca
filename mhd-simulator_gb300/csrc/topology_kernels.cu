// topology_kernels.cu -- connected components of the non-solid cells on the
// GPU: the gauge cells of the projection without a host round trip.
//
// The reference labels components on the host: it reads the whole mask back,
// runs a breadth-first search from every unvisited fluid cell in x-fastest
// order and writes class | root << 2 back (anchors(), src/fluid/mod.rs:
// 1447-1493, called from update_cells, :854-870).  A component's root is the
// first cell the scan meets, i.e. its smallest flat index.  Here the same
// labels come from a lock-free union-find whose links always point from a
// larger index to a smaller one, so every tree's root is the smallest index
// of its component and the encoded mask is identical to the search's.
//
//   k_cc_rows      one warp per grid row: every fluid cell points at the first
//                  cell of its x-run (the run start is the run's smallest
//                  index), from warp ballots over 32-cell chunks;
//   k_cc_link      per fluid cell, the -y and -z links (and the periodic x
//                  wrap), skipped where the cell before it in x already made
//                  the same link (its run and the neighbour's run are joined
//                  once per overlap, not once per cell);
//   k_cc_resolve   every label replaced by its root; roots and fluid cells
//                  counted; components that reach an open top face marked;
//   k_cc_classify  the GB300 solver's classes (0 solid, 1 active, 2 pinned
//                  gauge cell) and counts.
//
// Loops that follow or swing labels are bounded: a label only ever decreases,
// so a root walk ends within n steps, and a link retry makes one label
// smaller; on a bound the kernels record an error and stop.
#include <cuda_runtime.h>
#include <stdint.h>

#include "kernels.h"

namespace mhdproj {

namespace {
constexpr uint32_t kSolid = 0xFFFFFFFFu;

__device__ __forceinline__ uint32_t load_label(const uint32_t* L, uint64_t i) {
    // labels change under other threads' atomicMin: read through L2
    return __ldcg(L + i);
}

// Root of x's tree (the label that points at itself), or kSolid after
// `bound` steps.
__device__ __forceinline__ uint32_t find_root(const uint32_t* L, uint32_t x, uint64_t bound) {
    for (uint64_t s = 0; s <= bound; s++) {
        const uint32_t y = load_label(L, x);
        if (y == x) return x;
        x = y;
    }
    return kSolid;
}

// Join the trees of a and b: the larger root is linked under the smaller one.
// When the atomicMin meets a label that is no longer a root, it has still
// lowered that label to the other root (which joins the two trees at that
// cell), and the loop goes on with the label it replaced.  Returns false on
// the bound.
__device__ bool unite(uint32_t* L, uint32_t a, uint32_t b, uint64_t bound) {
    for (uint64_t s = 0; s <= bound; s++) {
        a = find_root(L, a, bound);
        b = find_root(L, b, bound);
        if (a == kSolid || b == kSolid) return false;
        if (a == b) return true;
        if (a < b) {
            const uint32_t old = atomicMin(L + b, a);
            if (old == b) return true;
            b = old;
        } else {
            const uint32_t old = atomicMin(L + a, b);
            if (old == a) return true;
            a = old;
        }
    }
    return false;
}

__device__ __forceinline__ bool fluid(const uint8_t* solid, uint64_t i) { return solid[i] == 0; }

__global__ void k_cc_rows(const uint8_t* __restrict__ solid, uint32_t* __restrict__ L, int nx, long long rows) {
    const long long row = (long long)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    if (row >= rows) return;  // whole warps leave together
    const int lane = threadIdx.x & 31;
    const uint64_t base = (uint64_t)row * nx;
    uint32_t carry_fluid = 0, carry_start = 0;
    for (int x0 = 0; x0 < nx; x0 += 32) {
        const int x = x0 + lane;
        const bool f = x < nx && fluid(solid, base + x);
        const uint32_t fl = __ballot_sync(0xFFFFFFFFu, f);
        // a run starts where a fluid cell follows a solid one (or the row start)
        const uint32_t starts = fl & ~((fl << 1) | carry_fluid);
        const uint32_t upto = starts & (0xFFFFFFFFu >> (31 - lane));
        const uint32_t start = upto ? (uint32_t)(base + x0 + (31 - __clz(upto))) : carry_start;
        if (x < nx) L[base + x] = f ? start : kSolid;
        carry_fluid = fl >> 31;
        carry_start = __shfl_sync(0xFFFFFFFFu, start, 31);
    }
}

__global__ void k_cc_link(const uint8_t* __restrict__ solid, uint32_t* L, int nx, int ny, int nz, int periodic,
                          int* error) {
    const uint64_t n = (uint64_t)nx * ny * nz, sxy = (uint64_t)nx * ny;
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    bool ok = true;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        if (!fluid(solid, i)) continue;
        const int x = (int)(i % nx);
        const int y = (int)((i / nx) % ny);
        const int z = (int)(i / sxy);
        const bool left = x > 0 && fluid(solid, i - 1);
        // -y neighbour (periodic wrap to the last row)
        long long jy = -1;
        if (y > 0) jy = (long long)(i - nx);
        else if ((periodic & 2) && ny > 1) jy = (long long)(i + (uint64_t)nx * (ny - 1));
        if (jy >= 0 && fluid(solid, jy) && !(left && fluid(solid, jy - 1)))
            ok &= unite(L, (uint32_t)i, (uint32_t)jy, n);
        // -z neighbour
        long long jz = -1;
        if (z > 0) jz = (long long)(i - sxy);
        else if ((periodic & 4) && nz > 1) jz = (long long)(i + sxy * (nz - 1));
        if (jz >= 0 && fluid(solid, jz) && !(left && fluid(solid, jz - 1)))
            ok &= unite(L, (uint32_t)i, (uint32_t)jz, n);
        // periodic x: the first cell of a row meets the last one
        if ((periodic & 1) && x == 0 && nx > 1 && fluid(solid, i + nx - 1))
            ok &= unite(L, (uint32_t)i, (uint32_t)(i + nx - 1), n);
    }
    if (!ok) atomicExch(error, 1);
}

__device__ __forceinline__ void block_add(unsigned long long* out, unsigned long long v) {
    v += __shfl_down_sync(0xFFFFFFFFu, v, 16);
    v += __shfl_down_sync(0xFFFFFFFFu, v, 8);
    v += __shfl_down_sync(0xFFFFFFFFu, v, 4);
    v += __shfl_down_sync(0xFFFFFFFFu, v, 2);
    v += __shfl_down_sync(0xFFFFFFFFu, v, 1);
    if ((threadIdx.x & 31) == 0 && v) atomicAdd(out, v);
}

// Labels to roots.  mask (optional): the reference's encoding, 0 for solid
// cells, 1 | root << 2 for members, 2 | root << 2 for roots.  topflag
// (optional): 1 at the root of every component with a cell in the top
// z-layer.
__global__ void k_cc_resolve(const uint8_t* __restrict__ solid, uint32_t* L, uint32_t* __restrict__ mask,
                             uint8_t* __restrict__ topflag, int nx, int ny, int nz, TopoCounts* counts) {
    const uint64_t n = (uint64_t)nx * ny * nz, top0 = (uint64_t)nx * ny * (nz - 1);
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    const uint64_t n_pad = (n + stride - 1) / stride * stride;  // every lane runs every round
    unsigned long long roots = 0, fl = 0;
    bool ok = true;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n_pad; i += stride) {
        if (i >= n || !fluid(solid, i)) {
            if (i < n && mask) mask[i] = 0u;
            continue;
        }
        const uint32_t r = find_root(L, (uint32_t)i, n);
        if (r == kSolid) {
            ok = false;
            continue;
        }
        L[i] = r;
        fl++;
        roots += r == (uint32_t)i;
        if (mask) mask[i] = (r == (uint32_t)i ? 2u : 1u) | (r << 2);
        if (topflag && i >= top0) topflag[r] = 1;
    }
    block_add(&counts->components, roots);
    block_add(&counts->fluid, fl);
    if (!ok) atomicExch(&counts->error, 1);
}

__global__ void k_cc_classify(const uint8_t* __restrict__ solid, const uint32_t* __restrict__ L,
                              const uint8_t* __restrict__ topflag, uint8_t* __restrict__ cls, uint64_t n,
                              TopoCounts* counts) {
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    const uint64_t n_pad = (n + stride - 1) / stride * stride;
    unsigned long long pinned = 0, active = 0;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n_pad; i += stride) {
        if (i >= n) continue;
        uint8_t c = 0;
        if (fluid(solid, i)) {
            const bool pin = L[i] == (uint32_t)i && !(topflag && topflag[i]);
            c = pin ? 2 : 1;
            pinned += pin;
            active += !pin;
        }
        cls[i] = c;
    }
    block_add(&counts->pinned, pinned);
    block_add(&counts->active, active);
}
}  // namespace

int launch_topology(const uint8_t* solid, int nx, int ny, int nz, int periodic, int outlet, uint32_t* labels,
                    uint8_t* topflag, uint32_t* mask_out, uint8_t* cls_out, TopoCounts* counts, cudaStream_t s) {
    const uint64_t n = (uint64_t)nx * ny * nz;
    const long long rows = (long long)ny * nz;
    const bool top_open = cls_out && outlet && !(periodic & 4);
    cudaMemsetAsync(counts, 0, sizeof(TopoCounts), s);
    if (top_open) cudaMemsetAsync(topflag, 0, n, s);
    k_cc_rows<<<(unsigned)((rows + 7) / 8), 256, 0, s>>>(solid, labels, nx, rows);
    const uint64_t want = (n + 255) / 256;
    const unsigned blocks = (unsigned)(want < 152ull * 16 ? (want ? want : 1) : 152ull * 16);
    k_cc_link<<<blocks, 256, 0, s>>>(solid, labels, nx, ny, nz, periodic, &counts->error);
    k_cc_resolve<<<blocks, 256, 0, s>>>(solid, labels, mask_out, top_open ? topflag : nullptr, nx, ny, nz, counts);
    if (cls_out) k_cc_classify<<<blocks, 256, 0, s>>>(solid, labels, top_open ? topflag : nullptr, cls_out, n, counts);
    return cls_out ? 4 : 3;
}

}  // namespace mhdproj
