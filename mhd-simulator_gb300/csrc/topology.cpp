// topology.cpp -- connected components, gauge cells and the aggregation
// hierarchy sizes, on the host (they change only with the solid topology).
#include "topology.h"

#include <vector>

namespace mhdproj {

namespace {
struct Walker {
    uint32_t nx, ny, nz, periodic;
    // neighbour of cell i along axis a in direction dir, or -1
    long long step(uint64_t i, int a, int dir) const {
        const uint64_t x = i % nx, y = (i / nx) % ny, z = i / ((uint64_t)nx * ny);
        long long c[3] = {(long long)x, (long long)y, (long long)z};
        const long long d[3] = {nx, ny, nz};
        c[a] += dir;
        if (c[a] < 0 || c[a] >= d[a]) {
            if (!(periodic & (1u << a))) return -1;
            c[a] = (c[a] + d[a]) % d[a];
        }
        return c[0] + d[0] * (c[1] + d[1] * c[2]);
    }
};
}  // namespace

uint32_t host_classify(const uint8_t* solid, const uint32_t dims[3], uint32_t periodic, int outlet, uint8_t* cls,
                       uint32_t* components) {
    const Walker W{dims[0], dims[1], dims[2], periodic};
    const uint64_t n = (uint64_t)dims[0] * dims[1] * dims[2];
    const bool top_open = outlet && !(periodic & 4u);
    std::vector<uint32_t> queue(n ? n : 1);
    std::vector<uint8_t> seen(n ? n : 1, 0);
    uint32_t pinned = 0, comps = 0;
    for (uint64_t i = 0; i < n; i++) cls[i] = solid[i] ? 0 : 1;
    for (uint64_t root = 0; root < n; root++) {
        if (cls[root] == 0 || seen[root]) continue;
        comps++;
        uint64_t head = 0, tail = 0;
        bool touches = false;
        seen[root] = 1;
        queue[tail++] = (uint32_t)root;
        while (head < tail) {
            const uint32_t i = queue[head++];
            if (top_open && i / ((uint64_t)dims[0] * dims[1]) == dims[2] - 1) touches = true;
            for (int a = 0; a < 3; a++)
                for (int dir = -1; dir <= 1; dir += 2) {
                    const long long j = W.step(i, a, dir);
                    if (j < 0 || cls[j] == 0 || seen[j]) continue;
                    seen[j] = 1;
                    queue[tail++] = (uint32_t)j;
                }
        }
        if (!touches) {
            cls[root] = 2;
            pinned++;
        }
    }
    if (components) *components = comps;
    return pinned;
}

uint32_t host_anchors(uint32_t* mask, const uint32_t dims[3], uint32_t periodic) {
    const Walker W{dims[0], dims[1], dims[2], periodic};
    const uint64_t n = (uint64_t)dims[0] * dims[1] * dims[2];
    std::vector<uint32_t> roots(n ? n : 1, 0), queue(n ? n : 1);
    uint32_t components = 0;
    // Breadth-first labelling: 4 marks a root, 3 a visited member.
    for (uint64_t root = 0; root < n; root++) {
        if (mask[root] != 1u) continue;
        components++;
        mask[root] = 4u;
        roots[root] = (uint32_t)root;
        uint64_t head = 0, tail = 0;
        queue[tail++] = (uint32_t)root;
        while (head < tail) {
            const uint32_t i = queue[head++];
            for (int a = 0; a < 3; a++)
                for (int dir = -1; dir <= 1; dir += 2) {
                    const long long j = W.step(i, a, dir);
                    if (j < 0 || mask[j] != 1u) continue;
                    mask[j] = 3u;
                    roots[j] = (uint32_t)root;
                    queue[tail++] = (uint32_t)j;
                }
        }
    }
    for (uint64_t i = 0; i < n; i++) {
        if (mask[i] == 3u) mask[i] = 1u | (roots[i] << 2);
        else if (mask[i] == 4u) mask[i] = 2u | (roots[i] << 2);
    }
    return components;
}

int host_hierarchy(const uint32_t dims[4], uint32_t* levels, uint64_t* coarse_cells) {
    unsigned __int128 count = 1;
    for (int a = 0; a < 3; a++) count *= dims[a];
    if (count > (unsigned __int128)UINT64_MAX) return 1;  // grid count overflow
    for (int a = 0; a < 3; a++)
        if (dims[a] > 0x7FFFFFFFu) return 2;  // beyond signed shader coordinates
    if (dims[0] == 0 || dims[1] == 0 || dims[2] == 0 || (uint64_t)count != (uint64_t)dims[3]) return 3;
    uint64_t d[3] = {dims[0], dims[1], dims[2]}, offset = 0;
    uint32_t nl = 1;
    while (d[0] > 4 || d[1] > 4 || d[2] > 4) {
        for (int a = 0; a < 3; a++) d[a] = (d[a] + 1) / 2;
        if (offset > 0xFFFFFFFFull) return 4;
        offset += d[0] * d[1] * d[2];
        nl++;
        if (offset > 0xFFFFFFFFull) return 4;  // coarse indices beyond u32
    }
    if (levels) *levels = nl;
    if (coarse_cells) *coarse_cells = offset;
    return 0;
}
}  // namespace mhdproj
