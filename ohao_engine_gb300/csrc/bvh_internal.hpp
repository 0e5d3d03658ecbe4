// bvh_internal.hpp -- declarations shared by the host context (abi.cpp) and
// the CUDA translation units. Not part of the public ABI.
#pragma once
#include <cstddef>
#include <cstdint>
#include <string>

#include <cuda_runtime.h>

#include "../../include/ohao_pt.h"

namespace ohao {

struct BvhBuildInfo {
    uint32_t nnodes;
    uint32_t height;
};

// Device scratch needed to build a BVH over n primitive boxes.
size_t bvh_build_scratch_bytes(uint32_t n);

// Builds the 8-wide BVH over n boxes (6 floats lo.xyz, hi.xyz per primitive,
// device). d_nodes must hold n (>= the wide node count) x 80 bytes,
// d_prim_order n uint32 (leaf slot -> box index), d_root_box 6 floats.
// Synchronises `st` (the node count is needed by the caller).
ohao_status bvh_build(const float* d_boxes, uint32_t n, void* d_scratch, size_t scratch_bytes, uint4* d_nodes,
                      uint32_t* d_prim_order, float* d_root_box, BvhBuildInfo* info, cudaStream_t st,
                      std::string& err);

// Triangle gather kernels (scene_kernels.cu).
// Flat: world-space triangles of all visible instances, instance-major.
// *out = max(*out, max of a[0..n)); the caller zeroes *out first.
void launch_max_u32(const uint32_t* a, size_t n, uint32_t* out, cudaStream_t st);
void launch_flat_triangles(const float* pos, const uint32_t* indices, const uint32_t* inst_first_index,
                           const uint32_t* inst_tri_offset, const float* inst_o2w, uint32_t n_inst, uint32_t total,
                           float* tri_verts /*9 per tri*/, uint32_t* tri_inst, uint32_t* tri_prim, float* boxes,
                           cudaStream_t st);
// One BLAS: object-space triangles of indices [first_index, first_index + 3*ntris).
void launch_blas_triangles(const float* pos, const uint32_t* indices, uint32_t first_index, uint32_t ntris,
                           float* tri_verts, uint32_t* tri_inst, uint32_t* tri_prim, float* boxes, cudaStream_t st);
// Record gather: recs[j] = (v0, prim; v1, inst; v2, ref = order[j]).
// World boxes of n instances from their object-to-world transforms (12
// floats each) and the (first record, count) span of their BLAS's triangle
// records (48 B each, object space).
void launch_instance_boxes(const float* o2w, const uint32_t* span, const float4* recs, uint32_t n, float* boxes,
                           cudaStream_t st);
void launch_gather_records(const float* tri_verts, const uint32_t* tri_inst, const uint32_t* tri_prim,
                           const uint32_t* order, uint32_t n, float4* recs, cudaStream_t st);

}  // namespace ohao
