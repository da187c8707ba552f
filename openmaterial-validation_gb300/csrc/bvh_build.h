// GPU build of the two-level 8-wide BVH (see bvh_build.cu).
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <vector>

#include "omv_types.h"

namespace omv {

struct MeshGeom {
    bool valid = false;
    int num_faces = 0;
    const float* d_pos = nullptr;       // device, 3 floats per vertex
    const uint32_t* d_faces = nullptr;  // device, 3 indices per face
    const float* h_pos = nullptr;       // the same positions and faces on the host
    const uint32_t* h_faces = nullptr;
    float lo[3] = {0, 0, 0};            // exact bounds of the referenced vertices
    float hi[3] = {0, 0, 0};
};

struct InstanceGeom {
    bool valid = false;
    int mesh = -1;
    int part = 0;  // scene of a group (one top-level tree per scene)
    float xf[3][4] = {};
};

struct AccelResult {
    Bvh8Node* nodes = nullptr;       // device; owned by the caller after the build
    float4* tris = nullptr;          // device
    uint32_t* tlas_items = nullptr;  // device
    uint32_t num_nodes = 0;
    size_t num_tris = 0;
    std::vector<uint32_t> blas_root;  // per mesh, 0xFFFFFFFF when the mesh is invalid
    uint32_t tlas_root = 0xFFFFFFFFu;    // scene 0's
    std::vector<uint32_t> tlas_roots;    // per scene of a group
    uint32_t num_valid_instances = 0;
};

enum class BvhBuilder { Sah = 0, Ploc = 1, Lbvh = 2, HostSah = 3 };  // OMV_BVH_SAH / _PLOC / _LBVH / _HOST_SAH

// Builds every BLAS and the TLAS; throws std::runtime_error on CUDA errors.
void build_accel(const std::vector<MeshGeom>& meshes, const std::vector<InstanceGeom>& insts, BvhBuilder builder,
                 AccelResult& out, cudaStream_t stream, int nparts = 1);

}  // namespace omv
