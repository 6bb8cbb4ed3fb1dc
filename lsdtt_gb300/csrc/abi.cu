// abi.cu -- the C-ABI entry points declared in include/lsdtt_gb300.h: argument
// checks with the reference's messages, engine lifetime, and the mapping of
// device error words to status codes.

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "engine.cuh"

namespace lsdtt_gb300
{

namespace
{
thread_local std::string g_last_error;
}

void set_error(const std::string& msg) { g_last_error = msg; }

int fail(int status, const std::string& msg)
{
    g_last_error = msg;
    return status;
}

int cuda_fail(cudaError_t e, const char* where)
{
    if (e == cudaErrorMemoryAllocation)
        return fail(LSDTT_GPU_ENOMEM, std::string(where) + ": out of device memory");
    return fail(LSDTT_GPU_ECUDA, std::string(where) + ": " + cudaGetErrorString(e));
}

int check_grid(const lsdtt_gpu_grid* grid, const char* who, bool flow_rules, Grid* out)
{
    if (!grid) return fail(LSDTT_GPU_EINVAL, std::string(who) + ": grid is null");
    if (!(grid->n_rows > 0 && grid->n_cols > 0 && grid->cell_size > 0.0))
        return fail(LSDTT_GPU_EINVAL, std::string(who) + ": raster metadata is invalid");
    const std::int64_t n = static_cast<std::int64_t>(grid->n_rows) * grid->n_cols;
    if (n >= (std::int64_t(1) << 31))
        return fail(LSDTT_GPU_EINVAL, std::string(who) + ": grids of 2^31 cells or more are not supported");
    Grid g{};
    g.nr = grid->n_rows;
    g.nc = grid->n_cols;
    g.cell = grid->cell_size;
    g.nodata = grid->no_data_value;
    g.n = n;
    for (int i = 0; i < 4; ++i)
    {
        char c = grid->boundary_conditions[i];
        if (c >= 'A' && c <= 'Z') c = static_cast<char>(c - 'A' + 'a');
        if (flow_rules && c != 'o' && c != 'n' && c != 'p' && c != 'b')
            return fail(LSDTT_GPU_EINVAL,
                        std::string("lsdtt_flowinfo: invalid boundary code '") + grid->boundary_conditions[i] + "'");
        g.bc[i] = c;
    }
    if (flow_rules)
    {
        // parse_boundary_conditions (src/cpu/lsdtt_flowinfo_cpu.cpp:845-884)
        if ((g.bc[0] == 'p') != (g.bc[2] == 'p'))
            return fail(LSDTT_GPU_EINVAL, "lsdtt_flowinfo: north and south periodic boundary flags must match");
        if ((g.bc[1] == 'p') != (g.bc[3] == 'p'))
            return fail(LSDTT_GPU_EINVAL, "lsdtt_flowinfo: east and west periodic boundary flags must match");
    }
    *out = g;
    return LSDTT_GPU_OK;
}

bool device_ok()
{
    int n = 0;
    return cudaGetDeviceCount(&n) == cudaSuccess && n > 0;
}

namespace
{

__global__ void check_valid_z(const float* __restrict__ z, const std::uint8_t* __restrict__ mask, std::int64_t n,
                              float ndv, unsigned long long* __restrict__ first_bad)
{
    LSDTT_COUNT();
    const std::int64_t i = static_cast<std::int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n || !mask[i]) return;
    const float v = z[i];
    if (!isfinite(v) || v == ndv) atomicMin(first_bad, static_cast<unsigned long long>(i));
}

__global__ void check_finite_w(const double* __restrict__ w, const std::uint8_t* __restrict__ mask, std::int64_t n,
                               unsigned long long* __restrict__ first_bad)
{
    LSDTT_COUNT();
    const std::int64_t i = static_cast<std::int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n || !mask[i]) return;
    if (!isfinite(w[i])) atomicMin(first_bad, static_cast<unsigned long long>(i));
}

__global__ void copy_mask(const std::uint8_t* __restrict__ in, std::int64_t n, std::uint8_t* __restrict__ out)
{
    LSDTT_COUNT();
    const std::int64_t i = static_cast<std::int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i < n) out[i] = in[i] ? 1 : 0;
}

__global__ void stamp_forced(const std::int64_t* __restrict__ forced, std::int64_t nf, std::int64_t n,
                             const std::uint8_t* __restrict__ mask, std::uint8_t* __restrict__ plane,
                             unsigned long long* __restrict__ bad)
{
    LSDTT_COUNT();
    const std::int64_t i = static_cast<std::int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= nf) return;
    const std::int64_t f = forced[i];
    if (f < 0 || f >= n || !mask[f])
    {
        atomicMin(bad, static_cast<unsigned long long>(i));
        return;
    }
    plane[f] = 1;
}

}  // namespace
}  // namespace lsdtt_gb300

namespace lsdtt_gb300
{

unsigned long long launches_abi();
unsigned long long launches_d8();
unsigned long long launches_fill();
unsigned long long launches_hillslope();
unsigned long long launches_lem();
unsigned long long launches_stack();
unsigned long long launches_stream_power();
unsigned long long launches_unet();
unsigned long long launches_ensemble();
unsigned long long launches_queries();
unsigned long long launches_dinf();

namespace
{
struct ProfRec
{
    std::string name;
    double bytes;
    cudaEvent_t b, e;
};
std::mutex g_prof_mu;
bool g_prof_on = false;
std::vector<ProfRec> g_prof;
}  // namespace

bool profiling_enabled() { return g_prof_on; }

void profile_begin(const char* kernel, double bytes, cudaStream_t, cudaEvent_t* b, cudaEvent_t* e)
{
    std::lock_guard<std::mutex> lk(g_prof_mu);
    ProfRec r{kernel, bytes, nullptr, nullptr};
    if (cudaEventCreate(&r.b) != cudaSuccess || cudaEventCreate(&r.e) != cudaSuccess) return;
    *b = r.b;
    *e = r.e;
    g_prof.push_back(r);
}

}  // namespace lsdtt_gb300

using namespace lsdtt_gb300;

extern "C" {

unsigned long long lsdtt_gpu_launch_count(void)
{
    return launches_abi() + launches_d8() + launches_fill() + launches_hillslope() + launches_lem() +
           launches_stack() + launches_stream_power() + launches_unet() +
           launches_ensemble() + launches_queries() + launches_dinf();
}

int lsdtt_gpu_profile_enable(int32_t on)
{
    std::lock_guard<std::mutex> lk(g_prof_mu);
    for (auto& r : g_prof)
    {
        cudaEventDestroy(r.b);
        cudaEventDestroy(r.e);
    }
    g_prof.clear();
    g_prof_on = on != 0;
    return LSDTT_GPU_OK;
}

int lsdtt_gpu_profile_read(const char* kernel, double* total_ms, int64_t* launches, double* bytes)
{
    if (!kernel || !total_ms || !launches || !bytes) return fail(LSDTT_GPU_EINVAL, "lsdtt_gpu_profile_read: null");
    std::lock_guard<std::mutex> lk(g_prof_mu);
    double t = 0.0, by = 0.0;
    std::int64_t k = 0;
    for (auto& r : g_prof)
    {
        if (r.name != kernel) continue;
        float ms = 0.0f;
        cudaError_t e = cudaEventSynchronize(r.e);
        if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, r.b, r.e);
        if (e != cudaSuccess) return cuda_fail(e, "lsdtt_gpu_profile_read");
        t += ms;
        by += r.bytes;
        ++k;
    }
    *total_ms = t;
    *launches = k;
    *bytes = by;
    return LSDTT_GPU_OK;
}

int lsdtt_gpu_profile_names(char* buf, int64_t buflen, int64_t* needed)
{
    if (!needed) return fail(LSDTT_GPU_EINVAL, "lsdtt_gpu_profile_names: null");
    std::lock_guard<std::mutex> lk(g_prof_mu);
    std::string all;
    std::vector<std::string> seen;
    for (const auto& r : g_prof)
    {
        if (std::find(seen.begin(), seen.end(), r.name) != seen.end()) continue;
        seen.push_back(r.name);
        all += r.name;
        all += '\n';
    }
    *needed = static_cast<int64_t>(all.size()) + 1;
    if (buf && buflen > 0)
    {
        const std::size_t k = std::min<std::size_t>(all.size(), static_cast<std::size_t>(buflen - 1));
        std::memcpy(buf, all.data(), k);
        buf[k] = '\0';
    }
    return LSDTT_GPU_OK;
}

const char* lsdtt_gpu_last_error(void) { return g_last_error.c_str(); }

const char* lsdtt_gpu_version(void) { return "lsdtt_gb300 0.1 (sm_103a)"; }

int lsdtt_gpu_device_available(void) { return device_ok() ? 1 : 0; }

int lsdtt_gpu_flow_create(const lsdtt_gpu_grid* grid, lsdtt_gpu_flow** out)
{
    if (!out) return fail(LSDTT_GPU_EINVAL, "lsdtt_gpu_flow_create: out is null");
    *out = nullptr;
    if (!device_ok()) return fail(LSDTT_GPU_ENODEV, "lsdtt_gpu_flow_create: no CUDA device");
    Grid g{};
    if (int s = check_grid(grid, "lsdtt_flowinfo", true, &g)) return s;
    auto* f = new lsdtt_gpu_flow();
    f->g = g;
    const std::size_t n = static_cast<std::size_t>(g.n);
    cudaError_t e = cudaSuccess;
    auto alloc = [&](auto** p, std::size_t count) {
        if (e == cudaSuccess) e = cudaMalloc(reinterpret_cast<void**>(p), sizeof(**p) * (count ? count : 1));
    };
    alloc(&f->receiver, n);
    alloc(&f->dir, n);
    alloc(&f->donors, n);
    alloc(&f->mask, n);
    alloc(&f->outlets, n);
    alloc(&f->topo, n);
    alloc(&f->svec, n);
    alloc(&f->sv_start, n);
    alloc(&f->sv_size, n);
    alloc(&f->depth, n);
    alloc(&f->height, n);
    alloc(&f->topo_pos, n);
    alloc(&f->dscal, 4);
    alloc(&f->derr, 4);
    alloc(&f->dundec, 1);
    // Workspace: the Euler-tour ranking peaks at ~60 B per cell (tour links
    // 16 B, level-0 ruler records 32 B, the ruler lists and the upper
    // levels; prefix arrays only for tours short enough for the serial
    // ranking); the range-max structure and the sort need ~58 B per cell
    // after the tour is released.
    f->ws_bytes = n * 84 + (std::size_t(64) << 20);
    if (e == cudaSuccess) e = cudaMalloc(reinterpret_cast<void**>(&f->ws.base), f->ws_bytes);
    f->ws.cap = f->ws_bytes;
    if (e == cudaSuccess) e = cudaMallocHost(reinterpret_cast<void**>(&f->hscal), sizeof(std::int64_t) * 4);
    if (e == cudaSuccess) e = cudaMallocHost(reinterpret_cast<void**>(&f->herr), sizeof(unsigned long long) * 4);
    if (e != cudaSuccess)
    {
        lsdtt_gpu_flow_destroy(f);
        return cuda_fail(e, "lsdtt_gpu_flow_create");
    }
    *out = f;
    return LSDTT_GPU_OK;
}

int lsdtt_gpu_flow_destroy(lsdtt_gpu_flow* f)
{
    if (!f) return LSDTT_GPU_OK;
    cudaFree(f->receiver);
    cudaFree(f->dir);
    cudaFree(f->donors);
    cudaFree(f->mask);
    cudaFree(f->outlets);
    cudaFree(f->topo);
    cudaFree(f->svec);
    cudaFree(f->sv_start);
    cudaFree(f->sv_size);
    cudaFree(f->depth);
    cudaFree(f->height);
    cudaFree(f->topo_pos);
    cudaFree(f->dscal);
    cudaFree(f->derr);
    cudaFree(f->dundec);
    cudaFree(f->ws.base);
    cudaFreeHost(f->hscal);
    cudaFreeHost(f->herr);
    delete f;
    return LSDTT_GPU_OK;
}

int lsdtt_gpu_flow_build(lsdtt_gpu_flow* f, const float* z_dev, const std::uint8_t* mask_dev,
                         const lsdtt_gpu_flow_options* options, const std::int64_t* forced_dev, std::int64_t n_forced,
                         void* stream)
{
    if (!f) return fail(LSDTT_GPU_EINVAL, "lsdtt_gpu_flow_build: flow is null");
    if (!z_dev || !mask_dev) return fail(LSDTT_GPU_EINVAL, "lsdtt_gpu_flow_build: z or mask is null");
    lsdtt_gpu_flow_options o{1, 1, 1, 1, 0};
    if (options) o = *options;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const Grid& g = f->g;
    const std::int64_t n = g.n;
    f->built = false;
    f->has_topo = false;
    f->has_sv = false;
    f->ws.used = 0;
    const unsigned nb = grid_blocks(n, 256);

    // validate_inputs (src/cpu/lsdtt_flowinfo_cpu.cpp:887-966): every valid
    // cell needs a finite, non-nodata elevation. derr[1] = first bad cell,
    // derr[3] = first bad forced-outlet entry.
    unsigned long long init[4] = {0ull, ~0ull, 0ull, ~0ull};
    cudaMemcpyAsync(f->derr, init, sizeof(init), cudaMemcpyHostToDevice, st);
    copy_mask<<<nb, 256, 0, st>>>(mask_dev, n, f->mask);
    check_valid_z<<<nb, 256, 0, st>>>(z_dev, f->mask, n, static_cast<float>(g.nodata), f->derr + 1);
    std::uint8_t* plane = nullptr;
    if (n_forced > 0 && forced_dev)
    {
        plane = f->ws.take<std::uint8_t>(static_cast<std::size_t>(n));
        cudaMemsetAsync(plane, 0, static_cast<std::size_t>(n), st);
        stamp_forced<<<grid_blocks(n_forced, 256), 256, 0, st>>>(forced_dev, n_forced, n, f->mask, plane,
                                                                f->derr + 3);
    }
    cudaMemcpyAsync(f->herr, f->derr, sizeof(init), cudaMemcpyDeviceToHost, st);
    cudaError_t e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return cuda_fail(e, "lsdtt_gpu_flow_build");
    if (f->herr[1] != ~0ull)
    {
        const std::int64_t b = static_cast<std::int64_t>(f->herr[1]);
        return fail(LSDTT_GPU_EINVAL, "lsdtt_flowinfo: valid mask cell has nodata or non-finite DEM value at row " +
                                          std::to_string(b / g.nc) + ", col " + std::to_string(b % g.nc));
    }
    if (f->herr[3] != ~0ull)
    {
        // validate_forced_outlet_flats (flowinfo_cpu.cpp:969-1008): the
        // first failing entry, with the reference's two messages.
        const std::uint64_t i = f->herr[3];
        std::int64_t fl = -1;
        e = cudaMemcpy(&fl, forced_dev + i, sizeof(fl), cudaMemcpyDeviceToHost);
        if (e != cudaSuccess) return cuda_fail(e, "lsdtt_gpu_flow_build");
        if (fl < 0 || fl >= n)
            return fail(LSDTT_GPU_EINVAL, "lsdtt_flowinfo: forced outlet flat index " + std::to_string(fl) +
                                              " (entry " + std::to_string(i) + ") is outside the raster, which has " +
                                              std::to_string(n) + " cells");
        return fail(LSDTT_GPU_EINVAL, "lsdtt_flowinfo: forced outlet flat index " + std::to_string(fl) + " (entry " +
                                          std::to_string(i) + ", row " + std::to_string(fl / g.nc) + ", col " +
                                          std::to_string(fl % g.nc) +
                                          ") lands on a nodata or masked cell, so it cannot act as a flow termination");
    }
    cudaMemcpyAsync(f->derr, init, sizeof(init), cudaMemcpyHostToDevice, st);

    e = launch_receivers(f, z_dev, f->mask, plane, o.interior_nodata_is_outlet, o.allow_pits_as_outlets, st);
    if (e == cudaSuccess) e = launch_donors_outlets(f, st);
    if (e != cudaSuccess) return cuda_fail(e, "lsdtt_gpu_flow_build");
    cudaMemcpyAsync(f->hscal, f->dscal, sizeof(std::int64_t) * 2, cudaMemcpyDeviceToHost, st);
    cudaMemcpyAsync(f->herr, f->derr, sizeof(unsigned long long) * 2, cudaMemcpyDeviceToHost, st);
    e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return cuda_fail(e, "lsdtt_gpu_flow_build");
    if ((f->herr[0] & 0xffffffffull) == 4)
    {
        const std::int64_t b = static_cast<std::int64_t>(f->herr[1]);
        return fail(LSDTT_GPU_EUNRESOLVED, "lsdtt_flowinfo: could not assign a receiver at row " +
                                               std::to_string(b / g.nc) + ", col " + std::to_string(b % g.nc) +
                                               ". The DEM likely contains an unresolved sink or flat.");
    }
    f->n_valid = f->hscal[0];
    f->n_outlets = f->hscal[1];
    f->interior_nodata_is_outlet = o.interior_nodata_is_outlet != 0;
    f->acyclic = true;  // strictly downhill receivers cannot close a cycle

    const bool need_topo = o.build_topological_order || o.build_s_vector || o.require_acyclic_graph;
    if (need_topo || o.build_s_vector)
    {
        if (o.build_s_vector && f->n_valid > 0 && f->n_outlets == 0)
            return fail(LSDTT_GPU_ESTATE, "lsdtt_flowinfo: cannot build s_vector because no outlets were found");
        e = build_stack(f, need_topo, st);
        if (e != cudaSuccess) return cuda_fail(e, "lsdtt_gpu_flow_build");
        cudaMemcpyAsync(f->herr, f->derr, sizeof(unsigned long long), cudaMemcpyDeviceToHost, st);
        e = cudaStreamSynchronize(st);
        if (e != cudaSuccess) return cuda_fail(e, "lsdtt_gpu_flow_build");
        const unsigned code = static_cast<unsigned>(f->herr[0] & 0xffffffffull);
        if (code == 5)
        {
            f->acyclic = false;
            if (o.require_acyclic_graph)
                return fail(LSDTT_GPU_ECYCLIC,
                            "lsdtt_flowinfo: routing graph is cyclic or incomplete. This usually means the DEM still "
                            "contains unresolved flats, pits, or incompatible periodic routing.");
        }
        else if (code != 0)
            return fail(LSDTT_GPU_EOVERFLOW, "lsdtt_gpu_flow_build: device work list overflow (code " +
                                                 std::to_string(code) + ")");
        f->has_topo = o.build_topological_order != 0;
        f->has_sv = o.build_s_vector != 0;
    }
    f->built = true;
    return LSDTT_GPU_OK;
}

int lsdtt_gpu_flow_get_view(const lsdtt_gpu_flow* f, lsdtt_gpu_flow_view* v)
{
    if (!f || !v) return fail(LSDTT_GPU_EINVAL, "lsdtt_gpu_flow_get_view: null argument");
    if (!f->built) return fail(LSDTT_GPU_ESTATE, "lsdtt_gpu_flow_get_view: engine has not been built");
    std::memset(v, 0, sizeof(*v));
    v->receiver = f->receiver;
    v->direction = f->dir;
    v->donor_count = f->donors;
    v->outlets = f->outlets;
    v->topological_order = f->has_topo ? f->topo : nullptr;
    v->s_vector = f->has_sv ? f->svec : nullptr;
    v->s_vector_start = f->has_sv ? f->sv_start : nullptr;
    v->s_vector_size = f->has_sv ? f->sv_size : nullptr;
    v->n_cells = f->g.n;
    v->n_valid_cells = f->n_valid;
    v->n_outlets = f->n_outlets;
    v->is_acyclic = f->acyclic ? 1 : 0;
    v->has_topological_order = f->has_topo ? 1 : 0;
    v->has_s_vector = f->has_sv ? 1 : 0;
    return LSDTT_GPU_OK;
}

int lsdtt_gpu_flow_accumulate(lsdtt_gpu_flow* f, const double* w_dev, double* out_dev, void* stream)
{
    if (!f || !out_dev) return fail(LSDTT_GPU_EINVAL, "lsdtt_gpu_flow_accumulate: null argument");
    if (!f->built || !f->has_topo)
        return fail(LSDTT_GPU_ESTATE, "lsdtt_flowinfo::accumulate: topological_order not built - set "
                                      "build_topological_order = true in lsdtt_flowinfo_options");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    if (w_dev)
    {
        // cell_weights must be finite on every valid cell (:2001-2015).
        unsigned long long init = ~0ull;
        cudaMemcpyAsync(f->derr + 1, &init, sizeof(init), cudaMemcpyHostToDevice, st);
        check_finite_w<<<grid_blocks(f->g.n, 256), 256, 0, st>>>(w_dev, f->mask, f->g.n, f->derr + 1);
        cudaMemcpyAsync(f->herr + 1, f->derr + 1, sizeof(init), cudaMemcpyDeviceToHost, st);
        cudaError_t e0 = cudaStreamSynchronize(st);
        if (e0 != cudaSuccess) return cuda_fail(e0, "lsdtt_gpu_flow_accumulate");
        if (f->herr[1] != ~0ull)
            return fail(LSDTT_GPU_EINVAL,
                        "lsdtt_flowinfo::accumulate: cell_weights must be finite for all valid cells");
    }
    bool exact = false;
    f->ws.used = 0;
    cudaError_t e = accumulate(f, w_dev, out_dev, st, &exact);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return cuda_fail(e, "lsdtt_gpu_flow_accumulate");
    return LSDTT_GPU_OK;
}

}  // extern "C"

namespace lsdtt_gb300
{
LSDTT_DEFINE_LAUNCH_READER(abi)
}  // namespace lsdtt_gb300
