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
    unsigned* dundec = nullptr;          // receivers tile pass left undecided cells
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

// ---- packed ensembles ------------------------------------------------------
// Ensemble members are stored back to back in one flat buffer: member k owns
// cells [base, base + nr*nc) in its own row-major order, and every base is a
// multiple of kPackAlign so that a 256-thread block never straddles two
// members. Receivers, outlets and the stack use packed (global) indices.
constexpr std::int64_t kPackAlign = 256;

struct PackedMember
{
    std::int64_t base;
    std::int32_t nr, nc;
    double cell;
    double nodata;
    char bc[4];
    std::int32_t tile_base;  // first fill tile (kT x kT) of this member
    std::int32_t ntx, nty;   // fill tiles across, down
    std::int32_t rtile_base;  // first 128 x 32 receiver tile of this member
    std::int32_t nrx, nry;    // receiver tiles across, down
    std::int64_t perim_base;  // first perimeter cell of this member in the fixup numbering
};

struct Packed
{
    const PackedMember* m;            // [n_members] (device)
    const std::uint16_t* blk_member;  // [n / kPackAlign]: member of each aligned block
    std::int64_t n;                   // packed length (multiple of kPackAlign)
    std::int32_t n_members;
};

__host__ __device__ inline Grid member_grid(const PackedMember& M)
{
    Grid g{};
    g.nr = M.nr;
    g.nc = M.nc;
    g.cell = M.cell;
    g.nodata = M.nodata;
    g.bc[0] = M.bc[0];
    g.bc[1] = M.bc[1];
    g.bc[2] = M.bc[2];
    g.bc[3] = M.bc[3];
    g.n = static_cast<std::int64_t>(M.nr) * M.nc;
    return g;
}

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
// With `packed`, f holds a packed ensemble (f->g.n = packed length, global
// receivers) and the tour links are found member by member.
cudaError_t build_stack(lsdtt_gpu_flow* f, bool want_topo, cudaStream_t st, const Packed* packed = nullptr);
cudaError_t accumulate(lsdtt_gpu_flow* f, const double* w, double* out, cudaStream_t st, bool* exact_path);

// unet.cu: the learned preconditioner's forward pass for the hillslope
// solver. unet_forward_dev enqueues y = net(r) on st; *y_dev points at the
// handle's output image, valid until the next call on the handle.
int unet_check_shape(const lsdtt_gpu_unet* U, int H, int W);
cudaError_t unet_forward_dev(lsdtt_gpu_unet* U, const float* r_dev, int H, int W, cudaStream_t st,
                             const float** y_dev);

}  // namespace lsdtt_gb300
