/*
 * plbm_c.h — C ABI of portlbm_gb300, the GB300 (sm_103a) implementation of PortLBM's
 * per-timestep D2Q9 BGK update.
 *
 * Each entry point replaces one member of the reference's public API
 * (SC-SGS/PortLBM, paths relative to that project):
 *   lbm::create_handler(const core::Properties&)      include/lbm/portlbm_factory.hpp:59
 *   lbm::create_handler(const std::string& settings)  include/lbm/portlbm_factory.hpp:73
 *   execution::AlgorithmHandler virtual API           include/lbm/execution/algorithm_handler.hpp:40-156
 * The C++ wrapper in portlbm_gb300.hpp maps these calls back to that class API and the
 * status codes back to the reference's exception types.
 *
 * All functions return PLBM_OK (0) or a negative status; plbm_last_error() then holds
 * the message.  Handles are not thread-safe except as documented for start/pause.
 * Plain pointers and sizes only: no C++ or torch types cross this boundary.
 */
#ifndef PLBM_C_H
#define PLBM_C_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Status codes.  PROPERTY  <-> lbm::exceptions::json::PropertyArgumentException
 *                UNKNOWN   <-> lbm::exceptions::Exception ("Unknown algorithm/data layout")
 *                WAIT      <-> lbm::exceptions::algorithm::WaitException
 *                IO/PARSE  <-> nlohmann::json parse or missing-key errors of json_to_properties */
enum {
    PLBM_OK = 0,
    PLBM_ERR_PROPERTY = -1,
    PLBM_ERR_UNKNOWN = -2,
    PLBM_ERR_WAIT = -3,
    PLBM_ERR_CUDA = -4,
    PLBM_ERR_IO = -5,
    PLBM_ERR_PARSE = -6,
    PLBM_ERR_ARGUMENT = -7,
    PLBM_ERR_NUMERIC = -8,
    PLBM_ERR_NO_DEVICE = -9
};

/* Which result array plbm_get_results() returns (core::Results, include/lbm/core/simulation.hpp:144-216). */
enum { PLBM_DENSITY = 0, PLBM_X_VELOCITY = 1, PLBM_Y_VELOCITY = 2, PLBM_ABS_VELOCITY = 3 };

/* Arithmetic form of the step.  F64_STRICT is the drop-in: IEEE double in the reference's
 * operation order, no fused multiply-add, identical results.  F64_FAST reassociates the BGK
 * update into fewer FP64 instructions (FMA) and agrees to <= 1e-12.  F32_REF restates the
 * reference's USE_FLOAT build (include/lbm/core/constants.hpp:17-21).  F32, F16S and BF16S
 * store populations in float / half / bfloat16 (the latter two shifted by w_i * rho0) and
 * collide in FP32.  F64_Q60 keeps FP64 accuracy (populations as 64-bit fixed point,
 * round(f * 2^60), finer than an FP64 ulp for |f| >= 2^-7) and collides on the integer pipe,
 * which GB300 issues ~38x faster than FP64; agrees with F64_STRICT to <= 1e-12 and fails with
 * PLBM_ERR_NUMERIC if a population leaves [-4, 4).  F16C stores the same shifted deviations as
 * F16S in a 16-bit float of 1 sign, 4 exponent and 11 significand bits (the FP16C format of Lehmann
 * et al., Phys. Rev. E 106, 015308, 2022; half the rounding error of IEEE half) for |f - w rho0|
 * < 0.5, and fails with PLBM_ERR_NUMERIC when a deviation leaves that range. */
enum { PLBM_F64_STRICT = 0, PLBM_F64_FAST = 1, PLBM_F32_REF = 2, PLBM_F32 = 3, PLBM_F16S = 4, PLBM_BF16S = 5,
       PLBM_F64_Q60 = 6, PLBM_F16C = 7 };

typedef struct plbm_handler plbm_handler;

/* POD mirror of core::Properties (include/lbm/core/properties.hpp:30-166) as passed to its
 * constructor (src/lbm/core/simulation.cpp:21-58): vertical/horizontal_nodes are INNER
 * extents; the library adds the two ghost layers.  Strings are NUL-terminated and copied. */
typedef struct {
    const char *algorithm;      /* "nptl" | "lptl" | "npol" | "nsol" */
    const char *data_layout;    /* "collision" | "stream" | "bundle" */
    int debug_mode;
    unsigned work_group_size;
    unsigned time_steps;
    unsigned frame_update_interval;
    const char *scenario;       /* the reference's eight scenarios */
    unsigned vertical_nodes;
    unsigned horizontal_nodes;
    double inlet_velocity_x, inlet_velocity_y, inlet_density;
    double outlet_velocity_x, outlet_velocity_y, outlet_density;
    double relaxation_time;
} plbm_properties;

/* Options with no counterpart in the reference; plbm_default_options() gives the drop-in. */
typedef struct {
    int precision;          /* PLBM_F64_STRICT ... PLBM_F16C */
    int nan_protection;     /* WITH_NAN_PROTECTION (CMakeLists.txt:28, default ON) */
    int use_graph;          /* capture chunks of steps in a CUDA graph */
    int device;             /* CUDA device ordinal */
    const int8_t *mask;     /* optional geometry: inner W*H flags (0 fluid, 1 solid), row-major
                               from (x=1, y=1); replaces walls + scenario stencil. Copied. */
    int gather;             /* PLBM_GATHER_*: how nptl/lptl gather the nodes next to obstacles in
                               the f32/f16s/bf16s forms (same results either way) */
} plbm_options;

/* PLBM_GATHER_OPEN: branch to the per-direction gather (and, for f16s/bf16s nptl/stream, the
 * vectorised rows), fastest when obstacles are rare; PLBM_GATHER_POROUS: one selected load per
 * direction for every interior node, fastest when most warps hold an obstacle; PLBM_GATHER_AUTO:
 * porous when more than PLBM_GATHER_POROUS_FRACTION of the 32-node row segments holding fluid
 * mix interior nodes next to a solid with nodes that are not. */
enum { PLBM_GATHER_AUTO = 0, PLBM_GATHER_OPEN = 1, PLBM_GATHER_POROUS = 2 };
#define PLBM_GATHER_POROUS_FRACTION 0.04

void plbm_default_options(plbm_options *opt);
/* The gather the handler runs (PLBM_GATHER_OPEN or PLBM_GATHER_POROUS, AUTO resolved). */
int plbm_gather_form(plbm_handler *h, int *form);

/* Validates like core::Properties::validate() (src/lbm/core/simulation.cpp:60-125) without
 * touching a GPU. */
int plbm_validate(const plbm_properties *props);

/* lbm::create_handler(props) — builds the simulation and initialises the domain on the GPU. */
int plbm_create(const plbm_properties *props, const plbm_options *opt, plbm_handler **out);
/* lbm::create_handler(settings_path) — reads settings.json (README.md:99-121 schema); an
 * optional "gb300" object may carry {"precision": "f64_fast", "nanProtection": true}. */
int plbm_create_from_json(const char *settings_path, const plbm_options *opt, plbm_handler **out);
void plbm_destroy(plbm_handler *h);

/* AlgorithmHandler::initialize()  :55-60  — rebuild; re-reads settings.json when created from one. */
int plbm_initialize(plbm_handler *h);
/* AlgorithmHandler::start()  — runs the remaining steps on a worker thread and returns. */
int plbm_start(plbm_handler *h);
/* AlgorithmHandler::pause()  — the step in flight completes, then the loop stops. */
int plbm_pause(plbm_handler *h);
/* AlgorithmHandler::block_until_finished()  — joins; PLBM_ERR_WAIT if never started. */
int plbm_block_until_finished(plbm_handler *h);
int plbm_is_finished(plbm_handler *h, int *finished);

/* AlgorithmHandler::get_densities() / get_x_velocities() / get_y_velocities() /
 * get_absolute_velocities(): host arrays of (W*H) doubles, row-major over the inner domain,
 * owned by the handle and valid until initialize()/destroy.  Updated on frame steps
 * (iteration % frame_update_interval == interval - 1) and when the run finishes. */
int plbm_get_results(plbm_handler *h, int which, const double **data, size_t *count);

/* get_horizontal_nodes()/get_vertical_nodes() return stored extents (inner + 2), as the
 * reference's do; the Domain fields are core::Domain's (include/lbm/core/domain.hpp:29-85). */
int plbm_get_extents(plbm_handler *h, unsigned *horizontal_nodes, unsigned *vertical_nodes);
int plbm_get_domain(plbm_handler *h, unsigned out7[7]);
int plbm_get_progress(plbm_handler *h, double *progress);
int plbm_get_last_frametime(plbm_handler *h, double *ms);
int plbm_get_current_iteration(plbm_handler *h, unsigned *iteration);
int plbm_get_properties(plbm_handler *h, plbm_properties *out); /* strings owned by the handle */

/* Writes settings.json like file_interaction::properties_to_json (file_interaction.cpp:11-37). */
int plbm_properties_to_json(const plbm_properties *props, const char *path);
/* Reads settings.json like file_interaction::json_to_properties (file_interaction.cpp:39-69);
 * strings are copied into thread-local storage valid until the next call on this thread. */
int plbm_json_to_properties(const char *path, int offset, plbm_properties *out);

/* core::Domain(Properties&) (src/lbm/core/simulation.cpp:194-382) for these properties, without a
 * GPU: out7 = {total_node_count, horizontal_nodes, vertical_nodes, subdomain_vertical_nodes,
 * subdomain_horizontal_nodes, subdomain_count_vertical, subdomain_count_horizontal}.
 * PLBM_ERR_PROPERTY when nsol's work-group size is below 6. */
int plbm_compute_domain(const plbm_properties *props, unsigned out7[7]);
/* The phase flags setup_domain (include/lbm/core/domain_initialization.hpp:453-518) gives the inner
 * W*H nodes (row-major from (x=1, y=1); 0 fluid, 1 solid), without a GPU.  The porous scenario
 * draws from the process-wide rand() sequence, as the reference does. */
int plbm_make_flags(const plbm_properties *props, int8_t *out);

/* ---- measurement hooks (no counterpart in the reference) ------------------------------ */

/* Runs n steps synchronously on the calling thread with device-resident data; writes the
 * average device time per step (CUDA events) to *ms_per_step when non-NULL. */
int plbm_run_steps(plbm_handler *h, unsigned n, double *ms_per_step);
/* Copies the device results to the host arrays now (as a frame step would). */
int plbm_sync_results(plbm_handler *h);

/* ---- headless frame export (replaces the reference's GUI frames, include/lbm/gui/lbm_gui.hpp:
 * 825-870; no counterpart API) ----------------------------------------------------------------
 * plbm_set_frame_export: from the next plbm_start on, every frame step (frameUpdateInterval) and
 * the last step write the selected results (bit i of `fields` = PLBM_DENSITY + i) as
 * <directory>/frame_<iteration, 9 digits>_<rho|jx|jy|jabs>.npy, float64, shape (H, W), row-major
 * over the inner domain.  NULL/empty directory or fields = 0 turns it off.  The directory is
 * created.  plbm_write_npy writes any rows x cols double array in the same format. */
int plbm_set_frame_export(plbm_handler *h, const char *directory, unsigned fields);
int plbm_write_npy(const char *path, const double *data, unsigned rows, unsigned cols);

/* ---- benchmark driver (src/lbm/benchmark/benchmark.cpp:30-383, main_gpu.cpp:160-174) --------
 * plbm_benchmark_run runs the reference's benchmark phases on libplbm handlers: phase 0 sweeps
 * algorithms x dataLayouts x work-group sizes (plus lptl with "auto") for 10 steps, phase 1 the
 * same for timeSteps and keeps each algorithm's fastest layout and work-group size (mean
 * initialisation + run time), phase 2 runs that setup on every phaseTwoScenarios entry.  Settings
 * come from settings_path read with node-count offset -2 (as the reference does), the sweep from
 * benchmark_path (NULL: <root>/settings/benchmark.json, root = the settings file's grandparent
 * directory).  Results go to <output_root or root>/benchmarks/phase<N>/ with the reference's file
 * names and JSON shape; every entry also lists "mlups" per run and, if hbm_gbs > 0,
 * "hbmFraction" (algorithmic bytes / run time / hbm_gbs).  phases: bit N runs phase N (0: all).
 * Unlike the reference it does not rewrite settings.json for each configuration.
 * plbm_benchmark_work_group_sizes: the work-group sizes the sweep tests for a device maximum
 * (Benchmark::get_work_group_sizes, benchmark.cpp:30-62). */
int plbm_benchmark_run(const char *settings_path, const char *benchmark_path, const char *output_root,
                       const plbm_options *opts, unsigned phases, double hbm_gbs);
int plbm_benchmark_work_group_sizes(unsigned max_work_group_size, unsigned *out, unsigned capacity, unsigned *count);
/* Kernel launches issued per step (for launch accounting). */
int plbm_launches_per_step(plbm_handler *h, unsigned *n);
/* Algorithmic HBM bytes per node update of the hot kernel (9 loads + 9 stores). */
int plbm_bytes_per_node(plbm_handler *h, double *bytes);
/* Reads back the total fluid mass and momentum (FP64 reductions on the GPU). */
int plbm_mass_momentum(plbm_handler *h, double out3[3]);

/* ---- no-allocation entry point (no counterpart in the reference) ----------------------------
 * plbm_nptl_steps_noalloc runs `steps` timesteps of the nptl step kernel (FP64 drop-in form,
 * stream layout) on buffers the caller owns, and allocates no device memory: it is for callers
 * that own all device memory through their own allocator or arena, or that cannot afford the
 * device synchronisation cudaMalloc/cudaFree may cause.  The outlet's previous-step jy column,
 * the step's only other state, lives in a fixed 1 MiB __device__ array (2 x 65536 doubles) that
 * every GPU loading the library holds until exit, so inner_h is limited to PLBM_NOALLOC_MAX_ROWS
 * and larger domains are rejected with PLBM_ERR_ARGUMENT.
 *   lattice0/1  device, 9 * P * inner_h doubles each, P = inner_w rounded up to a multiple of 32
 *   flags       device, inner_w * inner_h int8, row-major from (x=1, y=1): 0 fluid, 1 solid.  Values
 *               are not checked (that would need a synchronising read-back): any value other than 0
 *               acts as solid, both for the node and as a bounce-back source of its neighbours
 *   results     device, 4 * inner_w * inner_h doubles: rho | jx | jy | |j|, written on the last
 *               step of the call
 * first_step == 0 starts a run: it fills both lattices with the rest state, the results with
 * rho = -1 / j = 0 and clears the jy column.  Step t reads lattice[t & 1] and writes
 * lattice[(t + 1) & 1]; continue a run by passing first_step = the number of steps done.
 * All calls share the jy array and it keeps the last call's contents: calls that overlap on the
 * GPU (other streams or threads, or two runs interleaved) race on it.  The first call on each
 * device fetches the array's device address (with that device current); make that first call
 * before any stream capture.  Work is queued on `stream` (a cudaStream_t; NULL = legacy default
 * stream) and not synchronised.  inner_w is limited to 2^30.  A CUDA error already pending on the
 * calling thread when the call starts is returned as PLBM_ERR_CUDA, named in the message and left
 * pending (not cleared). */
#define PLBM_NOALLOC_MAX_ROWS 65536
typedef struct {
    void *lattice0, *lattice1;
    const int8_t *flags;
    double *results;
    unsigned inner_w, inner_h;
    double relaxation_time;
    double inlet_density, inlet_velocity_x, inlet_velocity_y;
    double outlet_density, outlet_velocity_x, outlet_velocity_y;
    unsigned first_step, steps;
    int nan_protection;
    void *stream;
} plbm_noalloc_args;

int plbm_nptl_steps_noalloc(const plbm_noalloc_args *args);
/* Message of the last failed plbm_nptl_steps_noalloc call on this thread. */
const char *plbm_noalloc_last_error(void);

/* ---- steady state and synthetic geometry (no counterpart in the reference) -------------- */

/* Runs the loop in chunks of K steps until the residual
 *   r = ||j^n - j^(n-K)||_2 / (K ||j^n||_2)   over fluid nodes (FP64 reductions on the GPU)
 * falls below `target` or `max_steps` is reached; writes the steps taken and the last residual
 * (INFINITY when no window had a snapshot from exactly K steps before it: the snapshot carries
 * over from the previous call and is dropped by plbm_set_equilibrium and re-initialisation).
 * Results on the host are those of the last step. */
int plbm_run_to_residual(plbm_handler *h, double target, unsigned K, unsigned max_steps, unsigned *steps,
                         double *residual);
/* Re-encodes the state of a handler that is not stepping into another shifted storage form
 * (PLBM_F32, PLBM_F16S, PLBM_BF16S, PLBM_F16C) and continues in it: every shifted form stores the
 * deviation from the same reference state, so each lattice (and halo) value is decoded, rescaled
 * exactly and rounded once.  Used to finish a 16-bit run in FP32 once the 16-bit form has reached
 * its rounding floor.  PLBM_ERR_NUMERIC, handler unchanged, when the state does not fit F16C. */
int plbm_set_precision(plbm_handler *h, int precision);
/* Porous channel geometry: solid walls on the first and last inner rows plus non-overlapping disks
 * (radius uniform in [rmin, rmax]) placed at seeded random positions until the fluid fraction of
 * the interior drops to `porosity`.  out: W*H int8 (0 fluid, 1 solid).  Returns the disk count
 * (>= 0) or a negative status. */
int plbm_porous_disks(unsigned inner_w, unsigned inner_h, uint64_t seed, double porosity, double rmin, double rmax,
                      int8_t *out);

/* ---- batches of independent domains (no counterpart in the reference) ------------------
 * Many channels of different sizes, relaxation times and inlet densities advanced together:
 * PLBM_BATCH_PERSISTENT runs one persistent launch per step whose blocks take tiles of every
 * domain from a shared work queue; PLBM_BATCH_PERSISTENT_GRAPH replays runs of those steps from a
 * captured CUDA graph; PLBM_BATCH_PER_DOMAIN launches one kernel per domain per step (the
 * comparison).  Each domain is a channel with its own W x H mask (0 fluid, 1 solid; copied),
 * zero inlet/outlet velocity; nptl update, stream layout.  Precisions: PLBM_F32, PLBM_F16S,
 * PLBM_BF16S, PLBM_F16C, PLBM_F64_Q60. */
typedef struct plbm_batch plbm_batch;
typedef struct {
    unsigned inner_w, inner_h;
    double relaxation_time, inlet_density, outlet_density;
    const int8_t *mask;
} plbm_batch_domain;
enum { PLBM_BATCH_PERSISTENT = 0, PLBM_BATCH_PERSISTENT_GRAPH = 1, PLBM_BATCH_PER_DOMAIN = 2 };

int plbm_batch_create(unsigned n, const plbm_batch_domain *domains, int precision, plbm_batch **out);
void plbm_batch_destroy(plbm_batch *b);
/* Tile shape and resident blocks per SM of the persistent launch: a block of tile_w x (tile_h & 255)
 * threads, each sweeping rows = ((tile_h >> 8) & 255) rows (at least 1), so a tile covers
 * tile_w x ((tile_h & 255) * rows) nodes.  PLBM_BATCH_TILE_VEC in tile_h selects vectorised rows
 * for PLBM_F16S / PLBM_BF16S / PLBM_F16C batches (8 nodes per thread, one warp per 256-node row segment):
 * tile_w must then be 32 and (tile_h & 255) at most 8, and a tile covers
 * 256 x ((tile_h & 255) * rows) nodes. */
#define PLBM_BATCH_TILE_VEC 0x10000
int plbm_batch_set_tile(plbm_batch *b, int tile_w, int tile_h, int blocks_per_sm);
/* Times `steps` persistent steps for each candidate tile shape and occupancy, keeps the fastest
 * (the timed steps advance the batch). */
int plbm_batch_autotune(plbm_batch *b, unsigned steps, int *tile_w, int *tile_h, int *blocks_per_sm);
/* Advances every domain by `steps`; results are written on the last one.  Device ms per step. */
int plbm_batch_run(plbm_batch *b, unsigned steps, int mode, double *ms_per_step);
int plbm_batch_results(plbm_batch *b, unsigned domain, int which, double *out);
int plbm_batch_info(plbm_batch *b, unsigned long long *nodes, unsigned *tiles);
const char *plbm_batch_last_error(void);

/* ---- learned warm start (no counterpart in the reference) -----------------------------------
 * plbm_set_equilibrium: replaces the state of an nptl/lptl handler that has not stepped (or has
 * stepped an even number of times) by the equilibrium populations of the given inner fields
 * rho, jx, jy (W*H host doubles each; solid entries ignored).
 * plbm_nn_*: the convolutional neural operator's kernels.  Activations NHWC bfloat16 on the
 * device; weights W[co][(ky*3+kx)*Cin+ci] bfloat16; 3x3 convolutions with zero padding run as
 * implicit GEMMs on the BF16 tensor cores with FP32 accumulation; gw/gb accumulate (FP32). */
int plbm_set_equilibrium(plbm_handler *h, const double *rho, const double *jx, const double *jy);
int plbm_nn_conv_fwd(const void *x, const void *w, const float *bias, void *y, int N, int H, int W, int Cin, int Cout,
                     int relu, void *stream);
int plbm_nn_conv_dgrad(const void *g, const void *w, void *gx, int N, int H, int W, int Cin, int Cout, void *stream);
/* The input gradient of plbm_nn_conv_dgrad with the weights also given re-laid out,
 * wt[ci][8 - tap][co] = w[co][tap][ci] (the tensor-core kernels read wt; other shapes read w). */
int plbm_nn_conv_dgrad_pre(const void *g, const void *w, const void *wt, void *gx, int N, int H, int W, int Cin,
                           int Cout, void *stream);
/* wt = the layout above for `layers` layers in one launch: segs (device, 3 ints per layer) holds
 * each layer's element offset in the flat w / wt buffers, Cin and Cout; max_elems bounds 9 Cin Cout. */
int plbm_nn_flip_layers(const void *w, void *wt, const int *segs, int layers, int max_elems, void *stream);
int plbm_nn_conv_wgrad(const void *x, const void *g, float *gw, float *gb, int N, int H, int W, int Cin, int Cout,
                       void *stream);
int plbm_nn_relu_bwd(const void *y, void *g, long long n, void *stream);
/* The ReLU backward of g ([P, C] bfloat16, in place: g = g where y > 0, else 0) together with the
 * bias gradient gb[c] += sum over the P pixels of the masked g[p][c] (FP32), in one pass over g. */
int plbm_nn_relu_bwd_bias(const void *y, void *g, float *gb, long long P, int C, void *stream);
int plbm_nn_pool2(const void *x, void *y, int N, int H, int W, int C, void *stream);
int plbm_nn_pool2_bwd(const void *gy, void *gx, int N, int H, int W, int C, void *stream);
int plbm_nn_up2(const void *x, void *y, int N, int H, int W, int C, void *stream);
int plbm_nn_up2_bwd(const void *gy, void *gx, int N, int H, int W, int C, void *stream);
int plbm_nn_add(const void *a, const void *b, void *y, long long n, void *stream);
int plbm_nn_mse(const void *pred, const float *target, const int8_t *mask, void *grad, float *loss, long long P, int C,
                float inv_count, void *stream);
int plbm_nn_adam(float *w, const float *g, float *m, float *v, void *w_bf16, long long n, float lr, float b1, float b2,
                 float eps, int t, void *stream);
/* Adam as plbm_nn_adam with the learning rate read from *lr (device) and the step count kept in
 * state[0..1] (two device ints, zeroed before the first update): the update uses step state[0] + 1
 * and stores it, so a launch captured in a CUDA graph advances its own count on every replay. */
int plbm_nn_adam_dev(float *w, const float *g, float *m, float *v, void *w_bf16, long long n, const float *lr, float b1,
                     float b2, float eps, int *state, void *stream);
/* Network input [N,H,W,C] (C >= 4): channel 0 the int8 solid mask, channels 1..3 the per-sample
 * scalars features[3n..3n+2] as constant planes, further channels zero. */
/* 1 when plbm_nn_conv_fwd runs the shape (input channels Cin, output channels Cout) on tcgen05:
 * W a multiple of 128 or a power of two below 128 with H a multiple of 128 / W, and either Cin a
 * multiple of 32 with Cout <= 128 (TMA-fed kernel) or 9 * Cin <= 64 with Cout <= 64 (kernel whose
 * threads write the im2col tile).  plbm_nn_conv_dgrad uses it with the two channel counts
 * exchanged.  Other shapes run the mma.sync kernel. */
int plbm_nn_conv_on_tensor_cores(int H, int W, int Cin, int Cout);
/* 1 when plbm_nn_conv_wgrad runs the shape on tcgen05: the image tiling above, Cout <= 128, and
 * either Cin a multiple of 32 up to 128 (TMA-fed input tiles) or Cin <= 32 (im2col tiles written by
 * the CTA's threads). */
int plbm_nn_wgrad_on_tensor_cores(int H, int W, int Cin, int Cout);
/* Synchronises the device and reports whether a tensor-core convolution gave up on a wait (its
 * output is then invalid); clears the flag. */
int plbm_nn_status(int *failed);
int plbm_nn_assemble(const int8_t *mask, const float *features, void *y, int N, int H, int W, int C, void *stream);

/* Last error message for h (or of the last failed create when h is NULL). */
const char *plbm_last_error(const plbm_handler *h);
const char *plbm_version(void);

#ifdef __cplusplus
}
#endif
#endif
