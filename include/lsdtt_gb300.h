/*
 * lsdtt_gb300.h -- C ABI of the GB300 (sm_103a) backend for the lsdtt3
 * landscape-evolution timestep hot path.
 *
 * Every entry point takes plain pointers and sizes, returns an int status
 * (LSDTT_GPU_OK == 0) and never throws. Pointers named *_dev are device
 * pointers (cudaMalloc'd or from any allocator on the current device);
 * pointers named *_host are host pointers. `stream` is a cudaStream_t passed
 * as void* (NULL = the legacy default stream). Calls on one handle are not
 * thread safe; distinct handles may be used from distinct threads.
 *
 * The message of the last failing call on the calling thread is returned by
 * lsdtt_gpu_last_error(); it is the reference's exception text where the
 * reference throws (e.g. "lsdtt_flowinfo: could not assign a receiver at row
 * R, col C. The DEM likely contains an unresolved sink or flat.").
 *
 * There is no CPU fallback: with no usable device every call returns
 * LSDTT_GPU_ENODEV.
 *
 * Reference paths are relative to the lsdtt3 checkout.
 */
#ifndef LSDTT_GB300_H
#define LSDTT_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes -------------------------------------------------------- */
enum lsdtt_gpu_status
{
    LSDTT_GPU_OK = 0,
    LSDTT_GPU_ENODEV = 1,      /* no CUDA device / driver                      */
    LSDTT_GPU_ENOMEM = 2,      /* device allocation failed                     */
    LSDTT_GPU_EINVAL = 3,      /* bad argument (message names it)              */
    LSDTT_GPU_EUNRESOLVED = 4, /* unresolved sink: message carries (row, col)  */
    LSDTT_GPU_ECYCLIC = 5,     /* routing graph cyclic or incomplete           */
    LSDTT_GPU_ENOCONV = 6,     /* iterative solve did not converge             */
    LSDTT_GPU_ETIMEOUT = 7,    /* a bounded device wait gave up                */
    LSDTT_GPU_ECUDA = 8,       /* CUDA runtime error (message has the text)    */
    LSDTT_GPU_EOVERFLOW = 9,   /* a device work list exceeded its capacity     */
    LSDTT_GPU_ESTATE = 10      /* handle not built / component not available   */
};

/* ---- grid ---------------------------------------------------------------- */
/* lsdtt_raster_meta (src/core/lsdtt_raster_meta.hpp) reduced to what the path
 * reads, plus the NESW boundary string ('o' open, 'n' no-flux, 'p' periodic,
 * 'b' base level). */
typedef struct lsdtt_gpu_grid
{
    int32_t n_rows;
    int32_t n_cols;
    double cell_size;
    double no_data_value;
    char boundary_conditions[4];
} lsdtt_gpu_grid;

int lsdtt_gpu_device_available(void);
const char* lsdtt_gpu_last_error(void);
const char* lsdtt_gpu_version(void);

/* ---- instrumentation (no reference counterpart; tracing for the backend) --
 * launch_count: kernels of this library executed since load (each kernel's
 * first block bumps a device counter; reading it synchronises the device).
 * profile_enable(1) starts recording a CUDA event pair around each kernel
 * launch of the ensemble step (and the hot launches of the single-grid
 * path), on the launch's own stream; profile_read sums, for one
 * kernel name, the elapsed time, the number of launches and the algorithmic
 * bytes those launches move (the per-cell byte counts of the backend's
 * design notes times the cells each launch covers). profile_enable(0) stops
 * recording and drops the records. */
unsigned long long lsdtt_gpu_launch_count(void);
int lsdtt_gpu_profile_enable(int32_t on);
int lsdtt_gpu_profile_read(const char* kernel, double* total_ms, int64_t* launches, double* bytes);
/* The names of every kernel (or stage) with profile records, one per line
 * in first-launch order; *needed receives the buffer size the list takes
 * (with its terminating NUL), buf (may be NULL) the list, truncated to
 * buflen. */
int lsdtt_gpu_profile_names(char* buf, int64_t buflen, int64_t* needed);

/* ---- failure-detection self-tests (no reference counterpart) --------------
 * Every wait inside this library's kernels is bounded: a wait that runs out
 * raises an abort flag, the kernel returns, and the call reports
 * LSDTT_GPU_ETIMEOUT while the context stays usable. These two entry points
 * run the library's own wait routines against a condition that nothing ever
 * satisfies, with the given poll limit: the grid barrier of the cooperative
 * stream-power sweep (one block at a barrier that expects two) and the
 * mbarrier wait of the warp-specialised tensor-core convolutions (a phase
 * nobody completes). Both return LSDTT_GPU_ETIMEOUT when the wait gave up
 * as designed; LSDTT_GPU_OK would mean it was released, a fault. */
int lsdtt_gpu_selftest_grid_barrier(int32_t spin_limit);
int lsdtt_gpu_selftest_mbarrier_wait(int32_t tries);

/* ---- fill ----------------------------------------------------------------
 * Replaces fill_pits(const lsdtt_raster_cpu&, float min_slope,
 * const std::string& bc, int n_threads, priority_flood_queue_backend)
 * (src/cpu/lsdtt_raster_flow_preprocessing_cpu.hpp:191-199,
 *  .cpp:727-782). Output cells that are masked or nodata hold no_data_value.
 * The result is the reference's priority flood in its own order (each raised
 * cell takes its value from its first-popped neighbour, the FIFO front taken
 * when it is at most the heap top), bit for bit, except that heap entries of
 * equal value are taken in (row, col) order where the reference's heap
 * layout decides. Errors: LSDTT_GPU_EINVAL (arguments), LSDTT_GPU_ETIMEOUT
 * (the relaxation did not converge), LSDTT_GPU_EOVERFLOW (a window replay
 * outgrew its arrays). */
int lsdtt_gpu_fill_pits(const lsdtt_gpu_grid* grid, const float* z_dev, const uint8_t* mask_dev,
                        float min_slope, float* filled_dev, void* stream);

/* Allocation-free variant of lsdtt_gpu_fill_pits (no counterpart in the
 * reference). For callers that must not have a library allocate device
 * memory -- a host framework that has reserved the device's memory for its
 * own allocator, or a latency-critical loop where a growing or failing
 * stream-ordered allocation is unacceptable. Its working memory is one
 * fixed array inside the library (64 MiB + 64 KiB, held on every device
 * that loads the library), so grids are limited to about 8192 x 8192 cells
 * at min_slope <= 0 and, because the raised cells' reference order needs
 * about 240 bytes a cell of replay buffers, about 520 x 520 cells at
 * min_slope > 0; larger grids return LSDTT_GPU_EINVAL. Same results as
 * lsdtt_gpu_fill_pits. It is never capturable: every call reads flags back
 * to the host between passes, and a call on a stream that is capturing
 * returns LSDTT_GPU_EINVAL before it enqueues anything. All calls share the
 * array, so calls that overlap on the GPU race; order them on one stream. */
int lsdtt_gpu_fill_pits_noalloc(const lsdtt_gpu_grid* grid, const float* z_dev, const uint8_t* mask_dev,
                                float min_slope, float* filled_dev, void* stream);

/* ---- D8 engine (lsdtt_flowinfo) ------------------------------------------
 * Replaces lsdtt_flowinfo(dem, mask, meta, options) and the lsdtt_flow_base
 * queries built on it (src/core/lsdtt_flow_base.hpp:126-491,
 * src/cpu/lsdtt_flowinfo_cpu.cpp:197-253). The engine owns its device arrays;
 * build() may be called again with new elevations of the same grid. */
typedef struct lsdtt_gpu_flow_options
{
    int32_t interior_nodata_is_outlet; /* default 1 */
    int32_t require_acyclic_graph;     /* default 1 */
    int32_t build_topological_order;   /* default 1 */
    int32_t build_s_vector;            /* default 1 */
    int32_t allow_pits_as_outlets;     /* default 0 */
} lsdtt_gpu_flow_options;

typedef struct lsdtt_gpu_flow lsdtt_gpu_flow;

typedef struct lsdtt_gpu_flow_view
{
    const int64_t* receiver;          /* [n]  -1 nodata, -2 outlet              */
    const uint8_t* direction;         /* [n]  0..7, 255 none                     */
    const uint8_t* donor_count;       /* [n]                                     */
    const int64_t* outlets;           /* [n_outlets] row-major                   */
    const int64_t* topological_order; /* [n_valid] or NULL when not kept         */
    const int64_t* s_vector;          /* [n_valid] or NULL when not built        */
    const int64_t* s_vector_start;    /* [n] (-1 for nodata) or NULL             */
    const uint64_t* s_vector_size;    /* [n] contributing-cell counts or NULL    */
    int64_t n_cells;
    int64_t n_valid_cells;
    int64_t n_outlets;
    int32_t is_acyclic;
    int32_t has_topological_order;
    int32_t has_s_vector;
    int32_t reserved;
} lsdtt_gpu_flow_view;

int lsdtt_gpu_flow_create(const lsdtt_gpu_grid* grid, lsdtt_gpu_flow** out);
int lsdtt_gpu_flow_destroy(lsdtt_gpu_flow* flow);
int lsdtt_gpu_flow_build(lsdtt_gpu_flow* flow, const float* z_dev, const uint8_t* mask_dev,
                         const lsdtt_gpu_flow_options* options, const int64_t* forced_outlets_dev,
                         int64_t n_forced, void* stream);
int lsdtt_gpu_flow_get_view(const lsdtt_gpu_flow* flow, lsdtt_gpu_flow_view* view);

/* lsdtt_flowinfo::accumulate(cell_weights) (src/cpu/lsdtt_flowinfo_cpu.cpp:
 * 1979-2046): weights_dev NULL = cell_size^2 on every valid cell. Bitwise the
 * reference's forward push in topological order. */
int lsdtt_gpu_flow_accumulate(lsdtt_gpu_flow* flow, const double* weights_dev, double* out_dev,
                              void* stream);

/* ---- query rasters on the D8 engine ---------------------------------------
 * The lsdtt_flow_base rasters built on the s-vector
 * (src/core/lsdtt_flow_base.hpp:126-491; src/cpu/lsdtt_flowinfo_cpu.cpp:
 * 2255-2965), on a built engine with its s-vector. `kind` selects:
 *   0 get_distance_from_outlet_raster()                           (:2255-2302)
 *   1 get_height_above_channel_raster(values, vmask, threshold)   (:2309-2382)
 *   2 get_height_above_channel_mask_donor_raster(values, vmask, channel_mask)
 *                                          (:2407-2474; donor_dev = donor_flat)
 *   3 get_distance_to_channel_raster(threshold)                   (:2482-2553)
 *   4 get_height_to_farthest_ridge_raster(values, vmask)          (:2571-2649)
 *   5 get_distance_to_farthest_ridge_raster()                     (:2651-2713)
 *   6 get_downstream_path_sum_raster(values, vmask, channel_mask = sink_mask)
 *                                                                 (:2721-2791)
 *   7 get_upslope_sum_raster(values, vmask, include_self)         (:2800-2868)
 *   8 get_upslope_mean_raster(values, vmask, include_self)        (:2876-2960)
 * Device arrays of n_rows * n_cols: values (float, the elev or values
 * argument), value_mask_dev (u8) and channel_mask_dev (u8) where the query
 * takes them (NULL otherwise); out_dev / out_mask_dev receive the raster's
 * data and mask (no_data_value where the mask is 0); donor_dev (int64, may
 * be NULL) the nearest channel cell of kind 2 (-1 where none). Same bits as
 * the reference. The engine's workspace holds the passes' arrays. */
int lsdtt_gpu_flow_query(lsdtt_gpu_flow* flow, int32_t kind, const float* values_dev, const uint8_t* value_mask_dev,
                         const uint8_t* channel_mask_dev, int32_t threshold, int32_t include_self, float* out_dev,
                         uint8_t* out_mask_dev, int64_t* donor_dev, void* stream);

/* ---- D-infinity flow graph ------------------------------------------------
 * Replaces lsdtt_flowgraph_cpu(dem, mask, meta, options) with
 * options.method = d_infinity (src/cpu/lsdtt_flowgraph_cpu.hpp:149-160;
 * .cpp:87-178, 423-662 Tarboton's facets, 874-985 donor counts and Kahn's
 * topological order, 988-1039 accumulate) and
 * compute_dinf_stream_power_incision (src/cpu/lsdtt_stream_power_cpu.hpp:
 * 113-129, .cpp:329-602; area smoothing kernel 1, no width factor). The
 * handle owns its device arrays; build() may be called again with new
 * elevations of the same grid. The receiver graph and the topological
 * order are the reference's; weights and facet slopes follow its float
 * arithmetic with the in-facet angle as the double atan2 rounded to float. */
typedef struct lsdtt_gpu_dinf lsdtt_gpu_dinf;
typedef struct lsdtt_gpu_dinf_view
{
    const int64_t* receivers;         /* [2n] per cell: receiver 0, receiver 1 (-1 none) */
    const float* weights;             /* [2n] their flow fractions               */
    const uint8_t* n_receivers;       /* [n]  0 (outlet, sink or invalid), 1, 2  */
    const float* slope;               /* [n]  steepest facet slope (nodata: none) */
    const float* bearing;             /* [n]  compass bearing, degrees (nodata: none) */
    const uint8_t* donor_count;       /* [n]  unique donors, capped at 255        */
    const int64_t* topological_order; /* [n_valid_cells]                          */
    int64_t n_cells;
    int64_t n_valid_cells;
    int64_t n_levels;                 /* heights in the topological order         */
} lsdtt_gpu_dinf_view;

int lsdtt_gpu_dinf_create(const lsdtt_gpu_grid* grid, lsdtt_gpu_dinf** out);
int lsdtt_gpu_dinf_destroy(lsdtt_gpu_dinf* dinf);
int lsdtt_gpu_dinf_build(lsdtt_gpu_dinf* dinf, const float* z_dev, const uint8_t* mask_dev,
                         int32_t interior_nodata_is_outlet, void* stream);
int lsdtt_gpu_dinf_get_view(const lsdtt_gpu_dinf* dinf, lsdtt_gpu_dinf_view* view);
/* accumulate(cell_weights): weights_dev NULL = cell_size^2 per valid cell. */
int lsdtt_gpu_dinf_accumulate(lsdtt_gpu_dinf* dinf, const double* weights_dev, double* out_dev, void* stream);
/* One implicit D-infinity stream-power step of z_dev (the surface the graph
 * was built on) into z_out_dev. */
int lsdtt_gpu_dinf_stream_power(lsdtt_gpu_dinf* dinf, const float* z_dev, float K, float m, float n, float dt,
                                float incision_threshold_area, int32_t divide_area_by_dx, float slope_clamp,
                                float* z_out_dev, void* stream);

/* ---- stream power ---------------------------------------------------------
 * compute_d8_stream_power_incision (src/cpu/lsdtt_stream_power_cpu.hpp:74-89,
 * .cpp:159-326) on a built engine, moving-average kernel 1 and no width
 * correction. k_field_dev may be NULL (scalar K). */
int lsdtt_gpu_stream_power_d8(lsdtt_gpu_flow* flow, const float* z_dev, const float* k_field_dev,
                              float K, float m, float n, float dt, float incision_threshold_area,
                              int32_t divide_area_by_dx, float slope_clamp, float* z_out_dev,
                              void* stream);

/* ---- implicit hillslope diffusion ------------------------------------------
 * One backward-Euler step of linear hillslope diffusion over dt: the Newton
 * step of compute_hillslope_newton (src/cpu/lsdtt_hillslope_newton_cpu.cpp:
 * 196-675; operator src/cpu/lsdtt_hillslope_operator_cpu.hpp:83-322) with
 * alpha = 1, solved matrix-free by Jacobi-PCG to ||r||_2 <= rel_tol*||b||_2.
 * is_channel_dev may be NULL (no channel cells). Returns LSDTT_GPU_ENOCONV
 * (with z_out still written) when max_iter is reached first. */
typedef struct lsdtt_gpu_solve_report
{
    int32_t iterations;
    int32_t converged;
    double relative_residual;
    double initial_residual_inf; /* ||F||_inf before the step (m/yr) */
    /* Filled by every hillslope solve; the learned fields stay 0 without a
     * network. explicit_relative_residual is the largest, over the linear
     * solves, of ||b - A x||_2 / ||b||_2 recomputed in FP64 from the final
     * FP32 iterate (the recurrence residual above is what the 1e-8 test
     * reads); -1 from lsdtt_gpu_hillslope_linear_implicit, which does not
     * compute it. */
    int32_t linear_solves;
    int32_t network_applications;
    int32_t rejected_solves;      /* learned solves the Jacobi acceptance check rejected */
    int32_t fallback_iterations;  /* Jacobi-PCG iterations run after a rejection */
    double explicit_relative_residual;
} lsdtt_gpu_solve_report;

int lsdtt_gpu_hillslope_linear_implicit(const lsdtt_gpu_grid* grid, const float* z_dev, const uint8_t* mask_dev,
                                        const uint8_t* is_channel_dev, float D, float dt, double rel_tol,
                                        int32_t max_iter, float* z_out_dev, lsdtt_gpu_solve_report* report,
                                        void* stream);

/* Backward-Euler hillslope diffusion over dt_total, linear or nonlinear
 * (Roering critical-slope flux): compute_hillslope_newton_transient
 * (src/cpu/lsdtt_hillslope_newton_cpu.hpp:305-310, .cpp:690-788) with the
 * reference's sub-step controller, feasibility line search and convergence
 * test ||F||_inf <= residual_tol (<= 0: 1e-12 m/yr). The inner linear solves
 * are Jacobi-PCG on the lagged-coefficient operator to rel_tol. report->
 * iterations is the total number of PCG iterations. */
int lsdtt_gpu_hillslope_implicit(const lsdtt_gpu_grid* grid, const float* z_dev, const uint8_t* mask_dev,
                                 const uint8_t* is_channel_dev, float D, float Sc, int32_t nonlinear, float dt_total,
                                 double rel_tol, int32_t max_pcg_iter, double residual_tol, int32_t max_outer,
                                 float* z_out_dev, lsdtt_gpu_solve_report* report, void* stream);

/* ---- learned preconditioner -----------------------------------------------
 * No reference counterpart: the reference solves its implicit hillslope steps
 * with Eigen (src/cpu/lsdtt_hillslope_newton_cpu.cpp:196-675). A 4-level
 * U-Net with additive skips maps a residual r to a correction e ~ A^-1 r:
 *   x0 = bf16(r/rms r); e0 = relu(conv 1->16); e1 = relu(conv(pool e0) 16->32)
 *   e2 = relu(conv(pool e1) 32->64); e3 = relu(conv(pool e2) 64->64)
 *   d2 = relu(conv(up e3) 64->64) + e2; d1 = relu(conv(up d2) 64->32) + e1
 *   d0 = relu(conv(up d1) 32->16) + e0; y = rms(r) * conv(d0) 16->1
 * 3x3 convolutions with zero padding, 2x2 mean pooling, nearest upsampling,
 * BF16 weights and activations, FP32 accumulation. The parameter vector
 * (FP32 master copy) holds the weights of the eight convolutions in that
 * order, each [Cout][3][3][Cin], then their biases. Images are n_rows x
 * n_cols with both sides multiples of 8, within the capacity given at
 * creation. */
typedef struct lsdtt_gpu_unet lsdtt_gpu_unet;

int lsdtt_gpu_unet_create(int32_t max_rows, int32_t max_cols, uint64_t seed, lsdtt_gpu_unet** out);
int lsdtt_gpu_unet_destroy(lsdtt_gpu_unet* net);
int64_t lsdtt_gpu_unet_num_params(const lsdtt_gpu_unet* net);
int lsdtt_gpu_unet_get_params(const lsdtt_gpu_unet* net, float* params_host, int64_t count);
int lsdtt_gpu_unet_set_params(lsdtt_gpu_unet* net, const float* params_host, int64_t count);
/* Convolution kernels of the 16-64-channel layers: 0 = mma.sync (m16n8k16
 * BF16), 1 = tcgen05 (UMMA M=128, FP32 accumulator in tensor memory, one
 * 3-row halo per 128-pixel tile), 2 = tcgen05 over rolling input rows (each
 * CTA walks down a 128-pixel band, one new input row per tile), 3 = the
 * rolling-row form with producer, MMA and epilogue warps meeting at
 * mbarriers (the default). Kinds 1-3 also run the 16 -> 1 output layer on
 * the tensor cores and give identical bits. */
int lsdtt_gpu_unet_set_conv_kernel(lsdtt_gpu_unet* net, int32_t kind);
/* LSDTT_GPU_ETIMEOUT when a tcgen05 convolution gave up waiting for its
 * MMAs since the handle was created (the outputs of that call are invalid). */
int lsdtt_gpu_unet_status(const lsdtt_gpu_unet* net);
/* y = net(r), device FP32 images */
int lsdtt_gpu_unet_apply(lsdtt_gpu_unet* net, const float* r_dev, int32_t n_rows, int32_t n_cols, float* y_dev,
                         void* stream);
/* loss = sum (net(r) - e)^2 / sum e^2 and its gradient (grad_host may be
 * NULL) without changing the weights. */
int lsdtt_gpu_unet_loss_grad(lsdtt_gpu_unet* net, const float* r_dev, const float* e_dev, int32_t n_rows,
                             int32_t n_cols, double* loss, float* grad_host, void* stream);
/* One optimiser step on the pair (r, e); *loss is the loss before it.
 * optimizer: 0 = SGD with momentum 0.9, 1 = Adam (0.9, 0.999, 1e-8). */
int lsdtt_gpu_unet_train_step(lsdtt_gpu_unet* net, const float* r_dev, const float* e_dev, int32_t n_rows,
                              int32_t n_cols, int32_t optimizer, float lr, double* loss, void* stream);

/* Residual/correction pairs from the plain solver: the first linear system
 * of lsdtt_gpu_hillslope_implicit's step of length dt (the lagged-coefficient
 * operator at z for nonlinear = 1) is solved by Jacobi-PCG, and at n_pairs
 * iterations k spread evenly over the solve the residual r_k and the
 * remaining correction x_final - x_k are written: r_out_dev[j*N + i] =
 * r_k[i] / A_ii (the Jacobi-scaled residual, metres, the network's input),
 * e_out_dev[j*N + i] = x_final[i] - x_k[i]. *n_written is the number of
 * pairs written (fewer when the solve is shorter). */
int lsdtt_gpu_hillslope_capture_pairs(const lsdtt_gpu_grid* grid, const float* z_dev, const uint8_t* mask_dev,
                                      const uint8_t* is_channel_dev, float D, float Sc, int32_t nonlinear, float dt,
                                      double rel_tol, int32_t max_iter, int32_t n_pairs, float* r_out_dev,
                                      float* e_out_dev, int32_t* n_written, void* stream);

/* lsdtt_gpu_hillslope_implicit with the network as the preconditioner: each
 * linear system is solved by flexible (Polak-Ribiere) PCG with
 *   M^-1 r = y + D^-1 (r - A y),  y = net(D^-1 r)  (D = diag A),
 * to the same relative residual rel_tol. Plain Jacobi-PCG is the acceptance check and
 * the fallback: the FP64 explicit residual of the learned iterate must be
 * within max(rel_tol, 4x the FP32 representation floor of the iterate) of
 * ||b||, else Jacobi-PCG restarts from that iterate (or from zero when it is
 * not finite) and finishes the solve. A learned solve whose residual does
 * not halve within 16 iterations is handed to Jacobi-PCG the same way, and
 * after two rejections in one call the network is not used again in that
 * call. The grid sides must be multiples of 8 within the network's
 * capacity. */
int lsdtt_gpu_hillslope_implicit_learned(const lsdtt_gpu_grid* grid, const float* z_dev, const uint8_t* mask_dev,
                                         const uint8_t* is_channel_dev, float D, float Sc, int32_t nonlinear,
                                         float dt_total, double rel_tol, int32_t max_pcg_iter, double residual_tol,
                                         int32_t max_outer, lsdtt_gpu_unet* net, float* z_out_dev,
                                         lsdtt_gpu_solve_report* report, void* stream);

/* ---- LEM timestep ----------------------------------------------------------
 * run_lem_step (src/cpu/lsdtt_lem_cpu.cpp:285-732) for the D8 coupled
 * regime with the "roering_implicit" linear hillslope model, optionally
 * preceded by fill_pits(z, fill_min_slope, bc) as the benchmark
 * configurations ask: fill -> D8 engine -> stream power -> hillslope ->
 * uplift on valid cells -> boundary flats restored to their pre-step value
 * minus base-level fall -> statistics. The LEM handle owns every buffer. */
typedef struct lsdtt_gpu_lem_options
{
    float timestep;
    float erodibility;
    float m_exponent;
    float n_exponent;
    float uplift_rate;
    float hillslope_diffusivity;
    float slope_clamp;            /* reference default 1e-5 */
    float baselevel_fall_rate;
    float fill_min_slope;         /* <= 0: no per-step fill */
    int32_t enable_hillslope;     /* linear implicit hillslope step */
    int32_t divide_area_by_dx;    /* reference default 1 */
    double hillslope_rel_tol;     /* PCG relative residual, e.g. 1e-8 */
    int32_t hillslope_max_iter;
    int32_t hillslope_nonlinear;  /* 1: Roering critical-slope law (enable_nonlinear_hillslopes) */
    float critical_slope;         /* Sc of the Roering law */
} lsdtt_gpu_lem_options;

/* lsdtt_lem_step_stats (src/cpu/lsdtt_lem_cpu.hpp:185-211) */
typedef struct lsdtt_gpu_lem_stats
{
    float delta_max_elevation;
    float delta_mean_elevation;
    float max_local_elevation_change;
    float p999_local_elevation_change;
    float mean_erosion_rate;
    float max_erosion_rate;
    int32_t hillslope_iterations;
    int32_t reserved;
} lsdtt_gpu_lem_stats;

typedef struct lsdtt_gpu_lem lsdtt_gpu_lem;

/* mask_dev is copied; boundary flats (build_boundary_flats,
 * src/cpu/lsdtt_lem_cpu.cpp:735-808) are derived from it and the grid's
 * boundary string. */
int lsdtt_gpu_lem_create(const lsdtt_gpu_grid* grid, const uint8_t* mask_dev, const lsdtt_gpu_lem_options* options,
                         lsdtt_gpu_lem** out, void* stream);
int lsdtt_gpu_lem_destroy(lsdtt_gpu_lem* lem);
/* Advances z_dev (in place) by one timestep. stats may be NULL. With the
 * Roering law (or a preconditioner attached) the hillslope stage is
 * lsdtt_gpu_hillslope_implicit over the timestep (the reference's
 * compute_hillslope_newton_transient); otherwise one linear
 * backward-Euler step. */
int lsdtt_gpu_lem_step(lsdtt_gpu_lem* lem, float* z_dev, lsdtt_gpu_lem_stats* stats, void* stream);
/* Attach a trained network (NULL detaches): the hillslope solves of later
 * steps use lsdtt_gpu_hillslope_implicit_learned. The network must fit the
 * grid (sides multiples of 8 within its capacity) and outlive its use. */
int lsdtt_gpu_lem_set_preconditioner(lsdtt_gpu_lem* lem, lsdtt_gpu_unet* net);

/* ---- batched ensembles -----------------------------------------------------
 * Parameter-sweep ensembles of independent LEM runs on grids of different
 * shapes. Each member advances exactly as lsdtt_gpu_lem_step would advance
 * it alone (same fill, D8 receivers, contributing counts, stream power,
 * linear implicit hillslope solved to the member's own relative residual,
 * uplift and boundary restore); the reference runs one grid per lsdtt-lem
 * process (src/cpu/lsdtt_lem_cpu.cpp:285-732), so this has no counterpart
 * beyond that loop. The members' cells are packed back to back in one
 * device buffer and every stage is one launch over all members; a step is
 * replayed as one captured CUDA graph whose fill-pass, stream-power level
 * and PCG iteration schedule is taken from an eager step and autotuned. A
 * step that outgrows the captured schedule is detected on the device,
 * undone and rerun eagerly, and the graph is captured again. */
typedef struct lsdtt_gpu_member
{
    lsdtt_gpu_grid grid;
    lsdtt_gpu_lem_options options;
} lsdtt_gpu_member;

typedef struct lsdtt_gpu_ensemble lsdtt_gpu_ensemble;

/* use_graph = 0 runs every step eagerly (host-driven loops). */
int lsdtt_gpu_ensemble_create(const lsdtt_gpu_member* members, int32_t n_members, int32_t use_graph,
                              lsdtt_gpu_ensemble** out, void* stream);
int lsdtt_gpu_ensemble_destroy(lsdtt_gpu_ensemble* ens);
/* Packed layout: member k's cells are [offsets[k], offsets[k] + n_rows*n_cols)
 * of the packed buffers; offsets has n_members + 1 entries (the last is the
 * packed length). */
int lsdtt_gpu_ensemble_offsets(const lsdtt_gpu_ensemble* ens, int64_t* offsets_host);
/* Member k's surface and validity mask (device arrays of its grid). The
 * mask also fixes the member's boundary flats. */
int lsdtt_gpu_ensemble_set_member(lsdtt_gpu_ensemble* ens, int32_t k, const float* z_dev, const uint8_t* mask_dev,
                                  void* stream);
/* Member k's surface only (same grid, mask unchanged), ordered on `stream`:
 * a caller that edits members between steps keeps the captured step graph,
 * which set_member (a mask change) has to rebuild. */
int lsdtt_gpu_ensemble_set_surface(lsdtt_gpu_ensemble* ens, int32_t k, const float* z_dev, void* stream);
int lsdtt_gpu_ensemble_get_member(const lsdtt_gpu_ensemble* ens, int32_t k, float* z_dev, void* stream);
/* All members' surfaces at once, in the packed layout (offsets above; the
 * padding between members is ignored), between host memory and the
 * ensemble, ordered on `stream`. This is the host-buffer path of a caller
 * that keeps its ensemble state on the host. */
int lsdtt_gpu_ensemble_upload(lsdtt_gpu_ensemble* ens, const float* z_host, void* stream);
int lsdtt_gpu_ensemble_download(const lsdtt_gpu_ensemble* ens, float* z_host, void* stream);
/* Advances every member by n_steps steps. stats (n_members entries, may be
 * NULL) receive the last step's statistics; p999_local_elevation_change is
 * not computed in an ensemble and is 0. */
int lsdtt_gpu_ensemble_step(lsdtt_gpu_ensemble* ens, int32_t n_steps, lsdtt_gpu_lem_stats* stats, void* stream);

typedef struct lsdtt_gpu_ensemble_info
{
    int64_t packed_cells;         /* packed buffer length */
    int64_t member_cells;         /* sum of the members' n_rows * n_cols */
    int32_t graph_enabled;
    int32_t graph_captures;
    int32_t graph_replays;
    int32_t eager_steps;
    int32_t fill_pass_cap;        /* captured schedule */
    int32_t depth_cap;
    int32_t sweep_split_level;    /* levels from here on run in one block */
    int32_t sweep_block;          /* threads per block of the level launches */
    int32_t hillslope_iteration_cap;
    int32_t last_fill_passes;     /* of the last eager step */
    int32_t last_max_depth;
    int32_t last_hillslope_iterations;
    double tuned_sweep_ms;        /* autotuner: best stream-power sweep time */
    double untuned_sweep_ms;      /* ... and one launch per level */
    int32_t sweep_dataflow;       /* sweep in use: 0 level launches, 1 in-order dataflow, 2 cooperative levels,
                                     3 member clusters */
    int32_t deep_members;         /* captured steps: members in the deep group, whose sweep runs beside the
                                     other members' sweep and hillslope solve (0: one group) */
    double dataflow_sweep_ms;     /* autotuner: the dataflow sweep's time */
    double coop_sweep_ms;         /* autotuner: the cooperative level sweep's best time */
    double cluster_sweep_ms;      /* autotuner: the member-cluster sweep's time */
} lsdtt_gpu_ensemble_info;

int lsdtt_gpu_ensemble_get_info(const lsdtt_gpu_ensemble* ens, lsdtt_gpu_ensemble_info* info);
/* The next captured step uses these fill-pass and PCG-iteration counts (0:
 * the recorded count plus margin) instead of the tuned ones, once; a
 * replay that outgrows them is undone and rerun like any other.
 * sweep_mode fixes the stream-power sweep from now on (0: one launch per
 * depth level plus the small-level tail, 1: the in-order dataflow sweep,
 * 2: one cooperative launch with a grid barrier per level plus the tail,
 * 3: one cluster of CTAs per member walking its own levels; -1: leave it to
 * the autotuner). */
int lsdtt_gpu_ensemble_override_schedule(lsdtt_gpu_ensemble* ens, int32_t fill_pass_cap,
                                         int32_t hillslope_iteration_cap, int32_t sweep_mode);
/* Member groups of captured steps (off by default): with the member-cluster
 * sweep, the members deeper than 3/4 of the deepest sweep on a second,
 * high-priority stream while the others sweep and solve their hillslope,
 * and their own solve follows. The results are the same either way. On the
 * 256-member benchmark ensemble it was slower (the others' PCG traffic
 * slows the latency-bound deep sweep, and depths cluster near the
 * deepest), so it is an option for ensembles with a few much deeper
 * members. 1 turns it on, 0 off (the next step captures again). */
int lsdtt_gpu_ensemble_set_member_groups(lsdtt_gpu_ensemble* ens, int32_t enabled);

/* ---- whole routing pass with host buffers ---------------------------------
 * fill_pits(z, min_slope, bc) then lsdtt_flowinfo on the filled surface, then
 * the results copied back: filled elevations, int64 receivers, topological
 * order and contributing-cell counts (s_vector_size). Any output pointer may
 * be NULL to skip that copy. This is the call a host-side caller (CLI,
 * Python binding) makes; it keeps one engine per grid shape internally. */
int lsdtt_gpu_route_host(const lsdtt_gpu_grid* grid, const float* z_host, const uint8_t* mask_host,
                         float min_slope, const lsdtt_gpu_flow_options* options, float* filled_host,
                         int64_t* receiver_host, int64_t* topo_host, uint64_t* counts_host,
                         void* stream);

#ifdef __cplusplus
}
#endif

#endif /* LSDTT_GB300_H */
