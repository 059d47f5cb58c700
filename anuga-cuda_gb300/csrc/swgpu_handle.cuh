// swgpu_handle.cuh -- the state behind one swgpu handle (one mesh on one
// device): device arrays, parameters, control block, the captured step
// graph and host copies of the geometry that the mixed path derives from.
#pragma once

#include <string>
#include <vector>

#include "swgpu_internal.cuh"

namespace swgpu {

constexpr int kStepsPerGraph = 16;  // default steps captured in one graph

struct Handle {
    int device = 0;
    int precision = SWGPU_FP64;
    int timestepping_method = SWGPU_EULER;
    cudaStream_t stream = nullptr;
    DevMesh M{};
    DevState S{};
    DevMixed X{};
    DevParams P{};
    BcTag *d_tags = nullptr;
    int ntags = 0;
    int steps_per_graph = kStepsPerGraph;
    float *trk_hmax = nullptr, *trk_tarr = nullptr;  // tracking buffers (S.hmax/S.tarr when on)
    int nscen = 1;               // scenarios (Ctrl blocks); > 1 for an ensemble
    std::vector<int64_t> scen_offsets;  // ensemble: first triangle of each scenario, + N
    int *d_blk_scen = nullptr;   // ensemble: scenario of each 256-triangle block
    Ctrl *d_ctrl = nullptr;      // [nscen]
    Ctrl *h_ctrl = nullptr;      // pinned mirror [nscen]
    RunSummary *d_summary = nullptr;
    RunSummary *h_summary = nullptr;  // pinned
    unsigned int *d_halt_bits = nullptr;  // one bit per scenario
    unsigned int *h_halt_bits = nullptr;  // pinned copy
    double *d_scalar = nullptr;  // mass / misc
    double *h_scalar = nullptr;  // pinned
    std::vector<void *> allocs;
    cudaGraphExec_t graph = nullptr;  // steps_per_graph fused steps
    bool resume_after_yield = false;
    bool vertices_stale = true;
    bool mixed_from_stage = true;  // mixed: FP64 stage upload not yet converted to depth
    bool elevation_set = false;
    bool unusable = false;  // a kernel reported SWGPU_ETIMEOUT: only destroy is allowed
    std::string err;
    // host copies needed to rebuild mixed geometry
    std::vector<double> h_vxy, h_cxy, h_normals, h_len, h_areas, h_radii;
    std::vector<int> h_nbr, h_surr;
    std::vector<uint8_t> h_nb;
};

// Derives the FP32 geometry of the mixed path from the host geometry and the
// current bed and friction (swgpu_mixed.cu).
int build_mixed_geometry(Handle *h);

}  // namespace swgpu
