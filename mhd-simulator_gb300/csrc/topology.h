// topology.h -- host-side graph utilities of the projection.
#pragma once
#include <stdint.h>

namespace mhdproj {
// Connected components of the non-solid cells (6-neighbour, periodic wrap).
// cls: 0 solid, 1 active, 2 pinned gauge cell.  A component that reaches the
// top z-layer while `outlet` is set needs no gauge; every other component is
// pinned at its first cell in x-fastest order.  Returns the pinned count and
// the component count in *components.
uint32_t host_classify(const uint8_t* solid, const uint32_t dims[3], uint32_t periodic, int outlet, uint8_t* cls,
                       uint32_t* components);
// anchors() of src/fluid/mod.rs:1447-1493: mask in 0/1, out class | root << 2.
uint32_t host_anchors(uint32_t* mask, const uint32_t dims[3], uint32_t periodic);
// hierarchy() of src/fluid/multigrid.rs:25-65.  0 on success.
int host_hierarchy(const uint32_t dims[4], uint32_t* levels, uint64_t* coarse_cells);
}  // namespace mhdproj
