// pending.cu -- entry points whose kernels land in later files. Each fails
// loudly with LSDTT_GPU_ESTATE until then; none computes anything on the CPU.
#include "engine.cuh"

using namespace lsdtt_gb300;

extern "C" {

int lsdtt_gpu_fill_pits(const lsdtt_gpu_grid*, const float*, const std::uint8_t*, float, float*, void*)
{
    return fail(LSDTT_GPU_ESTATE, "lsdtt_gpu_fill_pits: not available in this build");
}

int lsdtt_gpu_stream_power_d8(lsdtt_gpu_flow*, const float*, const float*, float, float, float, float, float,
                              std::int32_t, float, float*, void*)
{
    return fail(LSDTT_GPU_ESTATE, "lsdtt_gpu_stream_power_d8: not available in this build");
}

int lsdtt_gpu_route_host(const lsdtt_gpu_grid*, const float*, const std::uint8_t*, float, const lsdtt_gpu_flow_options*,
                         float*, std::int64_t*, std::int64_t*, std::uint64_t*, void*)
{
    return fail(LSDTT_GPU_ESTATE, "lsdtt_gpu_route_host: not available in this build");
}

}  // extern "C"
