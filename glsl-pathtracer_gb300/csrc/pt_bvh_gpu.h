// pt_bvh_gpu.h - the acceleration structure built on the GPU (pt_bvh_gpu.cu).
#pragma once

#include <cuda_runtime.h>

#include <string>

#include "bvh8.h"

namespace ptgb {

// Meshes as the reference's Scene holds them: triangles of mesh m are
// [mesh_tri_offset[m], mesh_tri_offset[m+1]) of vert_indices; instances
// give a mesh, a material and a transform (16 floats, row-vector Mat4).
struct GpuBuildInput {
    const float4* verts = nullptr;  // device: verticesUVX
    const int* vidx = nullptr;      // device: vert_indices
    const int* mesh_tri_offset = nullptr;  // host
    int num_meshes = 0;
    const float* transforms = nullptr;     // host
    const int* inst_mesh = nullptr;        // host
    const int* inst_material = nullptr;    // host
    int num_instances = 0;
};

// Device arrays in the layout of bvh8.h (owned; release() frees them).
struct GpuBvh {
    WideNode* nodes = nullptr;
    WideTri* tris = nullptr;
    InstRef* insts = nullptr;
    int num_nodes = 0, num_tris = 0, num_insts = 0;
    int tlas_root = 0, tlas_first_node = 0, blas_depth = 0, tlas_depth = 0;
    void release();
};

cudaError_t gpu_build_bvh(const GpuBuildInput& in, GpuBvh& out, cudaStream_t s, std::string& err);

}  // namespace ptgb
