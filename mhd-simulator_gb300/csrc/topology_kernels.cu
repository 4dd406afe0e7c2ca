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
//   k_cc_link      one warp per row: the -y and -z links (and the periodic x
//                  wrap), skipped where the cell before it in x already made
//                  the same link (its run and the neighbour's run are joined
//                  once per overlap, not once per cell);
//   k_cc_resolve   one warp per row: one root walk per run, the reference's
//                  encoded mask or the classes, the roots listed and counted,
//                  components that reach an open top face marked;
//   k_cc_gauges    the GB300 solver's gauge cells (class 2) from the root
//                  list.
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
// `bound` steps.  Path halving: every visited cell is pointed at its
// grandparent (an atomicMin, so a label still only decreases and still names
// a cell of the same component), which keeps the trees the links build
// shallow for the walks that follow.
__device__ __forceinline__ uint32_t find_root(uint32_t* L, uint32_t x, uint64_t bound) {
    for (uint64_t s = 0; s <= bound; s++) {
        const uint32_t y = load_label(L, x);
        if (y == x) return x;
        const uint32_t z = load_label(L, y);
        if (z == y) return y;
        atomicMin(L + x, z);
        x = z;
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

// Bits of the 32-cell chunk at x0 of the row at `base` that are fluid.
__device__ __forceinline__ uint32_t chunk_fluid(const uint8_t* solid, uint64_t base, int x0, int nx, bool have) {
    const int x = x0 + (threadIdx.x & 31);
    return __ballot_sync(0xFFFFFFFFu, have && x < nx && fluid(solid, base + x));
}

// One warp per grid row.  The row's cell x links to the cell below it in y
// (and in z) when both are fluid, unless cell x-1 and the cell below it are
// fluid too: then the two x-runs are joined already through x-1.
__global__ void k_cc_link(const uint8_t* __restrict__ solid, uint32_t* L, int nx, int ny, int nz, int periodic,
                          int* error) {
    const long long rows = (long long)ny * nz;
    const long long row = (long long)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    if (row >= rows) return;  // whole warps leave together
    const int lane = threadIdx.x & 31;
    const uint64_t n = (uint64_t)nx * ny * nz, sxy = (uint64_t)nx * ny;
    const int y = (int)(row % ny), z = (int)(row / ny);
    const uint64_t base = (uint64_t)row * nx;
    const bool hy = y > 0 || ((periodic & 2) && ny > 1);
    const bool hz = z > 0 || ((periodic & 4) && nz > 1);
    const uint64_t ybase = y > 0 ? base - nx : base + (uint64_t)nx * (ny - 1);
    const uint64_t zbase = z > 0 ? base - sxy : base + sxy * (nz - 1);
    bool ok = true;
    uint32_t carry = 0;  // bit 0: x0-1 fluid and its y neighbour fluid; bit 1: the same for z
    for (int x0 = 0; x0 < nx; x0 += 32) {
        const uint32_t f = chunk_fluid(solid, base, x0, nx, true);
        const uint32_t both_y = f & chunk_fluid(solid, ybase, x0, nx, hy);
        const uint32_t both_z = f & chunk_fluid(solid, zbase, x0, nx, hz);
        const uint32_t need_y = both_y & ~((both_y << 1) | (carry & 1));
        const uint32_t need_z = both_z & ~((both_z << 1) | (carry >> 1));
        const uint64_t i = base + x0 + lane;
        if ((need_y >> lane) & 1) ok &= unite(L, (uint32_t)i, (uint32_t)(ybase + x0 + lane), n);
        if ((need_z >> lane) & 1) ok &= unite(L, (uint32_t)i, (uint32_t)(zbase + x0 + lane), n);
        carry = (both_y >> 31) | ((both_z >> 31) << 1);
    }
    // periodic x: the first cell of the row meets the last one
    if (lane == 0 && (periodic & 1) && nx > 1 && fluid(solid, base) && fluid(solid, base + nx - 1))
        ok &= unite(L, (uint32_t)base, (uint32_t)(base + nx - 1), n);
    if (!ok) atomicExch(error, 1);
}

__device__ __forceinline__ void warp_add(unsigned long long* out, unsigned long long v) {
    v += __shfl_down_sync(0xFFFFFFFFu, v, 16);
    v += __shfl_down_sync(0xFFFFFFFFu, v, 8);
    v += __shfl_down_sync(0xFFFFFFFFu, v, 4);
    v += __shfl_down_sync(0xFFFFFFFFu, v, 2);
    v += __shfl_down_sync(0xFFFFFFFFu, v, 1);
    if ((threadIdx.x & 31) == 0 && v) atomicAdd(out, v);
}

// Labels to roots, one warp per grid row.  After the links only run starts
// have changed labels (a link moves roots, and every root is a run start), so
// every cell of a run has its run start's root: one root walk per run, handed
// to the run's cells by shuffles.  Outputs, each optional:
//   mask     the reference's encoding: 0 for solid cells, 1 | root << 2 for
//            members, 2 | root << 2 for roots;
//   cls      0 for solid cells, 1 for fluid ones (gauge cells are set by
//            k_cc_gauges from the root list);
//   roots    the component roots, appended (counts->components is the
//            length); without a list the roots are only counted;
//   topflag  1 at the root of every component with a cell in the top z-layer.
__global__ void k_cc_resolve(const uint8_t* __restrict__ solid, uint32_t* L, uint32_t* __restrict__ mask,
                             uint8_t* __restrict__ cls, uint32_t* __restrict__ roots, uint8_t* __restrict__ topflag,
                             int nx, int ny, int nz, TopoCounts* counts) {
    const long long rows = (long long)ny * nz;
    const long long row = (long long)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    if (row >= rows) return;
    const int lane = threadIdx.x & 31;
    const uint64_t n = (uint64_t)nx * ny * nz;
    const uint64_t base = (uint64_t)row * nx;
    const bool top = topflag && row / ny == nz - 1;
    unsigned long long root_count = 0, fl_count = 0;
    bool ok = true;
    uint32_t carry_fluid = 0, carry_root = 0;
    for (int x0 = 0; x0 < nx; x0 += 32) {
        const int x = x0 + lane;
        const uint64_t i = base + x;
        const uint32_t f = chunk_fluid(solid, base, x0, nx, true);
        const uint32_t starts = f & ~((f << 1) | carry_fluid);
        uint32_t r = 0;
        if ((starts >> lane) & 1) {
            r = find_root(L, (uint32_t)i, n);
            if (r == kSolid) ok = false;
        }
        const uint32_t upto = starts & (0xFFFFFFFFu >> (31 - lane));
        const uint32_t from = __shfl_sync(0xFFFFFFFFu, r, upto ? 31 - __clz(upto) : 0);
        const uint32_t root = upto ? from : carry_root;
        const bool fl = (f >> lane) & 1;
        const bool is_root = fl && root == (uint32_t)i;
        if (x < nx) {
            if (mask) mask[i] = fl ? ((is_root ? 2u : 1u) | (root << 2)) : 0u;
            if (cls) cls[i] = fl ? 1 : 0;
            if (fl && top) topflag[root] = 1;
        }
        const uint32_t rb = __ballot_sync(0xFFFFFFFFu, is_root);
        if (roots && rb) {
            unsigned long long at = 0;
            if (lane == 0) at = atomicAdd(&counts->components, (unsigned long long)__popc(rb));
            at = __shfl_sync(0xFFFFFFFFu, at, 0);
            if (is_root) roots[at + __popc(rb & ((1u << lane) - 1))] = (uint32_t)i;
        } else if (!roots) {
            root_count += (lane == 0) ? __popc(rb) : 0;
        }
        fl_count += (lane == 0) ? __popc(f) : 0;
        carry_fluid = f >> 31;
        carry_root = __shfl_sync(0xFFFFFFFFu, root, 31);
    }
    warp_add(&counts->components, root_count);
    warp_add(&counts->fluid, fl_count);
    if (!ok) atomicExch(&counts->error, 1);
}

// Gauge cells: the root of every component that does not reach an open top
// face (topflag null: every root) becomes class 2.
__global__ void k_cc_gauges(const uint32_t* __restrict__ roots, const uint8_t* __restrict__ topflag,
                            uint8_t* __restrict__ cls, TopoCounts* counts) {
    const unsigned long long m = counts->components;
    unsigned long long pinned = 0;
    const unsigned long long stride = (unsigned long long)gridDim.x * blockDim.x;
    const unsigned long long m_pad = (m + stride - 1) / stride * stride;
    for (unsigned long long k = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x; k < m_pad; k += stride) {
        if (k >= m) continue;
        const uint32_t r = roots[k];
        if (!(topflag && topflag[r])) {
            cls[r] = 2;
            pinned++;
        }
    }
    warp_add(&counts->pinned, pinned);
}
}  // namespace

int launch_topology(const uint8_t* solid, int nx, int ny, int nz, int periodic, int outlet, uint32_t* labels,
                    uint32_t* roots, uint8_t* topflag, uint32_t* mask_out, uint8_t* cls_out, TopoCounts* counts,
                    cudaStream_t s) {
    const uint64_t n = (uint64_t)nx * ny * nz;
    const long long rows = (long long)ny * nz;
    const bool top_open = cls_out && outlet && !(periodic & 4);
    cudaMemsetAsync(counts, 0, sizeof(TopoCounts), s);
    if (top_open) cudaMemsetAsync(topflag, 0, n, s);
    const unsigned row_blocks = (unsigned)((rows + 7) / 8);  // 8 rows (warps) per block
    k_cc_rows<<<row_blocks, 256, 0, s>>>(solid, labels, nx, rows);
    k_cc_link<<<row_blocks, 256, 0, s>>>(solid, labels, nx, ny, nz, periodic, &counts->error);
    k_cc_resolve<<<row_blocks, 256, 0, s>>>(solid, labels, mask_out, cls_out, cls_out ? roots : nullptr,
                                            top_open ? topflag : nullptr, nx, ny, nz, counts);
    if (!cls_out) return 3;
    k_cc_gauges<<<152 * 2, 256, 0, s>>>(roots, top_open ? topflag : nullptr, cls_out, counts);
    return 4;
}

}  // namespace mhdproj
