// The occluder BVH built on the device (dl_bvh.cu): the host builder's tree (build_bvh in
// dl_host.cpp, the same rules from dl_bvh_rules.hpp) from the occluder triangles already resident
// in device memory, in the layout the traversal reads.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <functional>

#include "dl_host.hpp"

namespace dl {

struct DeviceBvhInput {
    const float *positions;           // flattened mesh vertices, 3 floats each
    const uint32_t *indices;          // flattened mesh indices (mesh-local vertex numbers)
    const uint32_t *mesh_vertex_base;  // per mesh: first vertex in `positions`
    const uint32_t *mesh_index_base;   // per mesh: first index in `indices`
    const uint32_t *occ_mesh, *occ_tri;  // per occluder: mesh and triangle
    uint32_t occluders;
    uint64_t *held = nullptr;  // device bytes the caller holds; the build's scratch counts here
    uint64_t cap = 0;          // ... and may not take it past this (0: no cap)
};

struct DeviceBvh {
    BvhNode *nodes = nullptr;  // depth-first, the root first, each left subtree before its right one
    float4 *tris = nullptr;    // leaf order, 3 per triangle: v0 (w: occluder bits), e1, e2
    uint32_t *occ_leaf = nullptr;  // occluder -> its slot in leaf order
    uint32_t node_count = 0;
    uint32_t depth = 0;        // the deepest node's level, the root being 1
    bool too_deep = false;     // a subtree outgrew the builder's stack (the tree is unusable)
};

struct DeviceBvhError {
    cudaError_t code;
    const char *what;
};

// Builds the BVH on `stream` and waits for it. Output arrays come from `alloc(bytes)` (device
// memory the caller owns); scratch memory is the builder's own and freed before it returns.
// Throws DeviceBvhError on a CUDA failure.
void build_bvh_device(const DeviceBvhInput &in, const std::function<void *(size_t)> &alloc, cudaStream_t stream,
                      DeviceBvh &out);

}  // namespace dl
