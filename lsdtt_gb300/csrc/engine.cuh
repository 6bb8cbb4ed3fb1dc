// engine.cuh -- the D8 engine's device state and the stage entry points each
// .cu file implements. One engine per grid shape; every array is allocated
// once at create() and reused by every build().
#pragma once

#include <cstdint>
#include <string>
#include <cuda_runtime.h>

#include "common.cuh"
#include "prims.cuh"

struct lsdtt_gpu_flow
{
    lsdtt_gb300::Grid g{};
    // Per-cell outputs (the lsdtt_flowinfo state).
    std::int64_t* receiver = nullptr;   // [n]
    std::uint8_t* dir = nullptr;        // [n]
    std::uint8_t* donors = nullptr;     // [n]
    std::uint8_t* mask = nullptr;       // [n] private copy of the validity mask
    std::int64_t* outlets = nullptr;    // [n]
    std::int64_t* topo = nullptr;       // [n]
    std::int64_t* svec = nullptr;       // [n]
    std::int64_t* sv_start = nullptr;   // [n]
    std::uint64_t* sv_size = nullptr;   // [n]
    std::int32_t* depth = nullptr;      // [n] distance to the outlet, in cells
    std::int32_t* height = nullptr;     // [n] longest path from a headwater
    std::uint32_t* topo_pos = nullptr;  // [n] position in the topological order
    // Device scalars: [0] n_valid, [1] n_outlets, [2] max height, [3] spare.
    std::int64_t* dscal = nullptr;
    unsigned long long* derr = nullptr;  // [0] error word, [1] first unresolved flat
    std::int64_t* hscal = nullptr;       // pinned host mirror of dscal
    unsigned long long* herr = nullptr;  // pinned host mirror of derr
    // Workspace for the list ranking, RMQ and sort.
    lsdtt_gb300::Scratch ws{};
    std::size_t ws_bytes = 0;

    // Host-visible state after build.
    std::int64_t n_valid = 0;
    std::int64_t n_outlets = 0;
    std::int64_t max_height = 0;
    bool built = false;
    bool has_topo = false;
    bool has_sv = false;
    bool acyclic = false;
    bool interior_nodata_is_outlet = true;
};

namespace lsdtt_gb300
{

// Thread-local error message shared by every entry point.
void set_error(const std::string& msg);
int fail(int status, const std::string& msg);
int cuda_fail(cudaError_t e, const char* where);

// d8.cu
cudaError_t launch_receivers(lsdtt_gpu_flow* f, const float* z, const std::uint8_t* mask,
                             const std::uint8_t* forced_plane, int interior_nodata_is_outlet,
                             int allow_pits_as_outlets, cudaStream_t st);
cudaError_t launch_donors_outlets(lsdtt_gpu_flow* f, cudaStream_t st);

// stack.cu: Euler tour of the receiver forest, list ranking, s-vector,
// contributing counts, depths, heights and the Kahn topological order.
cudaError_t build_stack(lsdtt_gpu_flow* f, bool want_topo, cudaStream_t st);
cudaError_t accumulate(lsdtt_gpu_flow* f, const double* w, double* out, cudaStream_t st, bool* exact_path);

// unet.cu: the learned preconditioner's forward pass for the hillslope
// solver. unet_forward_dev enqueues y = net(r) on st; *y_dev points at the
// handle's output image, valid until the next call on the handle.
int unet_check_shape(const lsdtt_gpu_unet* U, int H, int W);
cudaError_t unet_forward_dev(lsdtt_gpu_unet* U, const float* r_dev, int H, int W, cudaStream_t st,
                             const float** y_dev);

}  // namespace lsdtt_gb300
