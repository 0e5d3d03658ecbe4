// scene_kernels.cu -- triangle preparation for the BVH builds.
//
// Flat mode transforms every visible instance's triangles to world space
// (x' = ((m0*x + m1*y) + m2*z) + m3 per row, the instance transform of
// buildTLAS, rt_acceleration_structure.cpp:437-445); BLAS mode reads the
// object-space triangles of one createBLAS index range
// (rt_acceleration_structure.cpp:205-300). Boxes are per-triangle min/max.
#include "bvh_internal.hpp"

#include <algorithm>

namespace ohao {

namespace {

__device__ __forceinline__ void tri_box(const float v[9], float* box) {
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        box[a] = fminf(fminf(v[a], v[3 + a]), v[6 + a]);
        box[3 + a] = fmaxf(fmaxf(v[a], v[3 + a]), v[6 + a]);
    }
}

__global__ void k_flat_tris(const float* __restrict__ pos, const uint32_t* __restrict__ indices,
                            const uint32_t* __restrict__ inst_first_index, const uint32_t* __restrict__ inst_tri_offset,
                            const float* __restrict__ o2w, uint32_t n_inst, uint32_t total, float* __restrict__ tv,
                            uint32_t* __restrict__ tinst, uint32_t* __restrict__ tprim, float* __restrict__ boxes) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= total) return;
    // last instance whose offset <= i
    uint32_t lo = 0, hi = n_inst - 1;
    while (lo < hi) {
        const uint32_t mid = (lo + hi + 1) / 2;
        if (inst_tri_offset[mid] <= i) lo = mid;
        else hi = mid - 1;
    }
    const uint32_t ii = lo;
    const uint32_t p = i - inst_tri_offset[ii];
    const float* m = o2w + ii * 12;
    float v[9];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        const uint32_t vi = indices[inst_first_index[ii] + 3 * p + k];
        const float x = pos[3 * vi], y = pos[3 * vi + 1], z = pos[3 * vi + 2];
        v[3 * k + 0] = ((m[0] * x + m[1] * y) + m[2] * z) + m[3];
        v[3 * k + 1] = ((m[4] * x + m[5] * y) + m[6] * z) + m[7];
        v[3 * k + 2] = ((m[8] * x + m[9] * y) + m[10] * z) + m[11];
    }
#pragma unroll
    for (int k = 0; k < 9; ++k) tv[static_cast<size_t>(i) * 9 + k] = v[k];
    tinst[i] = ii;
    tprim[i] = p;
    tri_box(v, boxes + static_cast<size_t>(i) * 6);
}

__global__ void k_blas_tris(const float* __restrict__ pos, const uint32_t* __restrict__ indices, uint32_t first_index,
                            uint32_t ntris, float* __restrict__ tv, uint32_t* __restrict__ tinst,
                            uint32_t* __restrict__ tprim, float* __restrict__ boxes) {
    const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= ntris) return;
    float v[9];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        const uint32_t vi = indices[first_index + 3 * p + k];
        v[3 * k + 0] = pos[3 * vi];
        v[3 * k + 1] = pos[3 * vi + 1];
        v[3 * k + 2] = pos[3 * vi + 2];
    }
#pragma unroll
    for (int k = 0; k < 9; ++k) tv[static_cast<size_t>(p) * 9 + k] = v[k];
    tinst[p] = 0xFFFFFFFFu;
    tprim[p] = p;
    tri_box(v, boxes + static_cast<size_t>(p) * 6);
}

__global__ void k_gather(const float* __restrict__ tv, const uint32_t* __restrict__ tinst,
                         const uint32_t* __restrict__ tprim, const uint32_t* __restrict__ order, uint32_t n,
                         float4* __restrict__ recs) {
    const uint32_t j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= n) return;
    const uint32_t b = order[j];
    const float* v = tv + static_cast<size_t>(b) * 9;
    recs[static_cast<size_t>(j) * 3 + 0] = make_float4(v[0], v[1], v[2], __uint_as_float(tprim[b]));
    recs[static_cast<size_t>(j) * 3 + 1] = make_float4(v[3], v[4], v[5], __uint_as_float(tinst[b]));
    recs[static_cast<size_t>(j) * 3 + 2] = make_float4(v[6], v[7], v[8], __uint_as_float(b));
}

// World box of instance i: min/max of its object-to-world transform applied
// to every vertex of every triangle record of its BLAS (the same rounding as
// the host: x' = ((m0*x + m1*y) + m2*z) + m3 per row), padded by 2^-20 of the
// coordinate magnitude. Exact for the instance's geometry, where the 8
// transformed corners of the BLAS box overestimate a rotated instance by up
// to sqrt(3) per axis. One block per instance.
__global__ void k_instance_boxes(const float* __restrict__ o2w, const uint2* __restrict__ span,
                                 const float4* __restrict__ recs, uint32_t n, float* __restrict__ boxes) {
    __shared__ float red[6][32];
    for (uint32_t i = blockIdx.x; i < n; i += gridDim.x) {
        float m[12];
#pragma unroll
        for (int k = 0; k < 12; ++k) m[k] = o2w[static_cast<size_t>(i) * 12 + k];
        float v[6] = {INFINITY, INFINITY, INFINITY, -INFINITY, -INFINITY, -INFINITY};
        const uint2 sp = span[i];
        for (uint32_t t = threadIdx.x; t < sp.y; t += blockDim.x) {
            const float4* r = recs + (static_cast<size_t>(sp.x) + t) * 3;
#pragma unroll
            for (int q = 0; q < 3; ++q) {
                const float4 p = r[q];
#pragma unroll
                for (int a = 0; a < 3; ++a) {
                    const float w = ((m[a * 4] * p.x + m[a * 4 + 1] * p.y) + m[a * 4 + 2] * p.z) + m[a * 4 + 3];
                    v[a] = fminf(v[a], w);
                    v[3 + a] = fmaxf(v[3 + a], w);
                }
            }
        }
#pragma unroll
        for (int k = 0; k < 6; ++k)
            for (int off = 16; off > 0; off >>= 1) {
                const float o = __shfl_down_sync(0xFFFFFFFFu, v[k], off);
                v[k] = k < 3 ? fminf(v[k], o) : fmaxf(v[k], o);
            }
        const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
        if (lane == 0)
            for (int k = 0; k < 6; ++k) red[k][warp] = v[k];
        __syncthreads();
        if (threadIdx.x == 0) {
            const int nw = static_cast<int>(blockDim.x >> 5);
            for (int w = 1; w < nw; ++w)
                for (int k = 0; k < 6; ++k) v[k] = k < 3 ? fminf(v[k], red[k][w]) : fmaxf(v[k], red[k][w]);
            for (int a = 0; a < 3; ++a) {
                const float pad = (fabsf(v[a]) + fabsf(v[3 + a])) * 0x1p-20f;
                boxes[static_cast<size_t>(i) * 6 + a] = v[a] - pad;
                boxes[static_cast<size_t>(i) * 6 + 3 + a] = v[3 + a] + pad;
            }
        }
        __syncthreads();
    }
}

// Largest value of a uint32 array (atomicMax into *out, which the caller
// zeroes): the index and material-id range checks of a device-side
// geometry upload.
__global__ void k_max_u32(const uint32_t* __restrict__ a, size_t n, uint32_t* __restrict__ out) {
    uint32_t m = 0;
    for (size_t i = blockIdx.x * static_cast<size_t>(blockDim.x) + threadIdx.x; i < n;
         i += static_cast<size_t>(gridDim.x) * blockDim.x)
        m = a[i] > m ? a[i] : m;
    for (int off = 16; off > 0; off >>= 1) {
        const uint32_t o = __shfl_down_sync(0xFFFFFFFFu, m, off);
        m = o > m ? o : m;
    }
    if ((threadIdx.x & 31) == 0 && m) atomicMax(out, m);
}

}  // namespace

void launch_max_u32(const uint32_t* a, size_t n, uint32_t* out, cudaStream_t st) {
    if (n == 0) return;
    const size_t want = (n + 255) / 256;
    k_max_u32<<<static_cast<unsigned>(std::min<size_t>(want, 152 * 8)), 256, 0, st>>>(a, n, out);
}

void launch_instance_boxes(const float* o2w, const uint32_t* span, const float4* recs, uint32_t n, float* boxes,
                           cudaStream_t st) {
    if (n == 0) return;
    k_instance_boxes<<<std::min<uint32_t>(n, 65535u), 256, 0, st>>>(o2w, reinterpret_cast<const uint2*>(span), recs,
                                                                    n, boxes);
}

void launch_flat_triangles(const float* pos, const uint32_t* indices, const uint32_t* inst_first_index,
                           const uint32_t* inst_tri_offset, const float* inst_o2w, uint32_t n_inst, uint32_t total,
                           float* tri_verts, uint32_t* tri_inst, uint32_t* tri_prim, float* boxes, cudaStream_t st) {
    if (total == 0) return;
    k_flat_tris<<<(total + 255) / 256, 256, 0, st>>>(pos, indices, inst_first_index, inst_tri_offset, inst_o2w, n_inst,
                                                     total, tri_verts, tri_inst, tri_prim, boxes);
}

void launch_blas_triangles(const float* pos, const uint32_t* indices, uint32_t first_index, uint32_t ntris,
                           float* tri_verts, uint32_t* tri_inst, uint32_t* tri_prim, float* boxes, cudaStream_t st) {
    if (ntris == 0) return;
    k_blas_tris<<<(ntris + 255) / 256, 256, 0, st>>>(pos, indices, first_index, ntris, tri_verts, tri_inst, tri_prim,
                                                     boxes);
}

void launch_gather_records(const float* tri_verts, const uint32_t* tri_inst, const uint32_t* tri_prim,
                           const uint32_t* order, uint32_t n, float4* recs, cudaStream_t st) {
    if (n == 0) return;
    k_gather<<<(n + 255) / 256, 256, 0, st>>>(tri_verts, tri_inst, tri_prim, order, n, recs);
}

}  // namespace ohao
