/*
 * nsdg.h — C ABI of the GB300 (sm_103a) sea-ice dynamics kernel.
 *
 * This is the drop-in boundary for neXtSIM_DG's dynamics hot path: the DG
 * transport of ice thickness / concentration / damage, the mEVP or BBM stress
 * update and the CG2 momentum sub-cycle.  Every entry point takes plain
 * pointers and sizes, returns an int status (NSDG_OK == 0) and never aborts.
 * All arrays are FP64 in the reference's ModelArray layout:
 *   - H / DG / DGSTRESS fields: element-major, component fastest,
 *     element index = i + nx*j  (ModelArray.hpp:358-361 in the reference);
 *   - coordinates: VERTEX type, (nx+1)*(ny+1) nodes, 2 components (x, y).
 *
 * Entry point  ->  reference interface it replaces
 *   nsdg_kernel_create      MEVPDynamicsKernel(const DynamicsParameters&)
 *                           (dynamics/src/include/MEVPDynamicsKernel.hpp:25-28),
 *                           BBMDynamicsKernel (BBMDynamicsKernel.hpp:20-24)
 *   nsdg_kernel_initialise  DynamicsKernel::initialise / CGDynamicsKernel::initialise
 *                           (DynamicsKernel.hpp:44-75; CGDynamicsKernel.cpp:24-51)
 *   nsdg_kernel_set_data    DynamicsKernel::setData / CGDynamicsKernel::setData
 *                           (DynamicsKernel.hpp:93-110; CGDynamicsKernel.cpp:54-90;
 *                           BrittleCGDynamicsKernel.hpp:138-145)
 *   nsdg_kernel_get_dg0     DynamicsKernel::getDG0Data / CGDynamicsKernel::getDG0Data
 *                           (DynamicsKernel.hpp:119-130; CGDynamicsKernel.cpp:93-118)
 *   nsdg_kernel_get_dg      DynamicsKernel::getDGData (DynamicsKernel.hpp:138-156)
 *   nsdg_kernel_update      VPCGDynamicsKernel::update (VPCGDynamicsKernel.hpp:63-94),
 *                           BrittleCGDynamicsKernel::update (BrittleCGDynamicsKernel.hpp:91-136)
 *   nsdg_transport_*        DGTransport<DG> (dynamics/src/include/DGTransport.hpp:27-152),
 *                           dgLimit.hpp:16-85 and Tools::MeanValue (Tools.hpp:24-50)
 *   nsdg_restart_*          ParaGridIO::getModelState / readForcingTimeStatic /
 *                           dumpModelState (core/src/ParaGridIO.cpp:87-348)
 *   nsdg_diagnostic_writer_* ParaGridIO::writeDiagnosticTime (ParaGridIO.cpp:350-500)
 */
#ifndef NSDG_H
#define NSDG_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------ */
#define NSDG_OK 0
#define NSDG_ERR_BAD_ARG 1          /* invalid argument / call order             */
#define NSDG_ERR_UNKNOWN_FIELD 2    /* reference: std::out_of_range from .at()   */
#define NSDG_ERR_SIZE_MISMATCH 3    /* array size does not match the mesh        */
#define NSDG_ERR_CUDA 4             /* CUDA runtime error (message in last_error)*/
#define NSDG_ERR_NUMERIC 5          /* non-finite velocity or stress detected    */
#define NSDG_ERR_UNSUPPORTED 6      /* e.g. spherical coordinates                */
#define NSDG_ERR_LOGIC 7            /* reference: std::logic_error               */
#define NSDG_ERR_NO_DEVICE 8        /* no CUDA device is visible                 */

/* ---- rheologies and precision modes ------------------------------------ */
#define NSDG_RHEOLOGY_MEVP 0        /* MEVPDynamicsKernel                        */
#define NSDG_RHEOLOGY_BBM 1         /* BBMDynamicsKernel                         */

#define NSDG_PRECISION_FP64 0       /* every operation in FP64                   */
#define NSDG_PRECISION_MIXED 1      /* FP32 bulk; FP64 conservation sums, inverse
                                       mass matrices, Delta and viscosity        */

/*
 * Physical and numerical parameters.  Defaults (nsdg_default_params) are the
 * reference's: DynamicsParameters.hpp:22-40, VPParameters.hpp:20-25,
 * MEBParameters.hpp:40-65; alpha = beta = 1500 (VPCGDynamicsKernel.hpp:125-126);
 * n_steps = 100 (DynamicsKernel.hpp:187).
 */
typedef struct nsdg_params {
    /* DynamicsParameters */
    double rho_ice, rho_atm, rho_ocean;
    double C_atm, C_ocean;
    double F_atm, F_ocean;
    double fc;
    double ocean_turning_angle; /* degrees */
    double gravity;
    /* VPParameters */
    double Pstar, DeltaMin;
    /* mEVP relaxation constants */
    double alpha, beta;
    /* MEBParameters (BBM) */
    double compaction_param, nu0, young, P0;
    double undamaged_time_relaxation_sigma, exponent_relaxation_sigma;
    double exponent_compression_factor, tan_phi, compr_strength, C_lab;
    /* sub-cycle count (mEVP iterations or BBM sub-steps) */
    int n_steps;
    /* NSDG_PRECISION_* */
    int precision;
} nsdg_params;

/* Fills *p with the reference defaults. */
void nsdg_default_params(nsdg_params* p);

/* Human-readable name of a status code (static storage). */
const char* nsdg_status_string(int status);

/* Library version string, e.g. "nsdg-gb300 0.1 sm_103a". */
const char* nsdg_version(void);

/* ======================================================================== */
/* Dynamics kernel (the DynamicsKernel drop-in)                             */
/* ======================================================================== */
typedef struct nsdg_kernel nsdg_kernel;

/* dg_comp: DG components of the advected fields (1, 3 or 6; DGCOMP in the
 * reference).  Velocity is CG2 and stress DG 8 (CGDEGREE 2, DGSTRESSCOMP 8).
 * No device work happens here. */
int nsdg_kernel_create(int rheology, int dg_comp, const nsdg_params* params,
    nsdg_kernel** out);
int nsdg_kernel_destroy(nsdg_kernel* k);

/* Message of the last failing call on this handle ("" if none). */
const char* nsdg_kernel_last_error(const nsdg_kernel* k);

/* Builds the mesh (landmask, Dirichlet lists from the mask and the four
 * domain edges), the FP64 per-element operators, and uploads them.
 * coords: (nx+1)*(ny+1)*2 doubles; mask: nx*ny doubles (1.0 = ice).
 * is_spherical != 0: coords are (lon, lat) in radians; the mesh is rotated
 * so that its poles lie in Greenland / Antarctica and the operators carry the
 * spherical metric terms (DynamicsKernel.hpp:44-58, ParametricMap.cpp:298-353,
 * CGDynamicsKernel.cpp:331-351).  nx and ny must be at least 2
 * (NSDG_ERR_BAD_ARG otherwise: the kernels are not written for a single row
 * or column of cells, which the reference's mesh allows). */
int nsdg_kernel_initialise(nsdg_kernel* k, size_t nx, size_t ny,
    const double* coords, int is_spherical, const double* mask);

/* setData semantics of the reference: hice/cice/ssh/damage and unknown names
 * follow DGModelArray::ma2dg (zero, then all components if n_comp equals the
 * DG count, else component 0 only); u, v, uwind, vwind, uocean, vocean are
 * DG->CG2 interpolated.  data: n_elements*n_comp doubles from host memory,
 * which the caller may reuse when the call returns (the copy has landed; the
 * conversion on the device runs on behind the return, ahead of any later
 * work on the handle).  Pinned host memory makes the copy faster. */
int nsdg_kernel_set_data(nsdg_kernel* k, const char* name, const double* data,
    size_t n_elements, size_t n_comp);

/* The benchmark forcing computed on the device.  In the reference the
 * atmosphere and ocean boundary modules update their fields right before the
 * dynamics (core/src/PrognosticData.cpp:87-95) and the dynamics module passes
 * them to its kernel with setData.  For the benchmark case they are closed-
 * form fields on the cell centres x = i dx, y = j dy, dx = length_x / nx
 * (physics/src/BenchmarkCoordinates.cpp:21-40):
 *   ocean  u = ocean_vmax (2 y / length_y - 1), v = ocean_vmax (1 - 2 x / length_x)
 *          (physics/src/modules/OceanBoundaryModule/BenchmarkOcean.cpp:15-39);
 *   wind   a cyclone centred at (centre_x + centre_vx t, centre_y + centre_vy t),
 *          t the seconds since the first update: x' = x - x0, y' = y - y0,
 *          scale = wind_A exp(-wind_k hypot(x', y')),
 *          u = -scale wind_vmax (cos a x' + sin a y'),
 *          v = -scale wind_vmax (-sin a x' + cos a y'), a = wind_angle_deg
 *          (physics/src/modules/AtmosphereBoundaryModule/BenchmarkAtmosphere.cpp:29-77).
 * nsdg_kernel_benchmark_ocean / _atmosphere compute these on the device and
 * feed them to the handle exactly as set_data of the H fields uocean/vocean
 * or uwind/vwind would (DG0 -> CG2 interpolation), with no host copy.
 * nsdg_benchmark_forcing_defaults fills the reference's constants for a box
 * of length_x x length_y: wind_A 1e-5, wind_vmax 30 m/s, wind_k 1e-5 1/m,
 * 72 degrees, the centre starting mid-box and reaching the far corner
 * after 5 days, ocean_vmax 0.01 m/s. */
typedef struct nsdg_benchmark_forcing {
    double length_x, length_y;
    double wind_A, wind_vmax, wind_k, wind_angle_deg;
    double centre_x, centre_y, centre_vx, centre_vy;
    double ocean_vmax;
} nsdg_benchmark_forcing;
void nsdg_benchmark_forcing_defaults(nsdg_benchmark_forcing* f, double length_x, double length_y);
int nsdg_kernel_benchmark_ocean(nsdg_kernel* k, const nsdg_benchmark_forcing* f);
int nsdg_kernel_benchmark_atmosphere(nsdg_kernel* k, const nsdg_benchmark_forcing* f, double seconds);

/* getDG0Data: component 0 (cell average) of hice, cice, damage, u, v,
 * uiostress, viostress or a stored field.  out: n_elements doubles. */
int nsdg_kernel_get_dg0(nsdg_kernel* k, const char* name, double* out, size_t n_elements);

/* getDGData: all components (n_comp must be the stored DG count, or 1). */
int nsdg_kernel_get_dg(nsdg_kernel* k, const char* name, double* out,
    size_t n_elements, size_t n_comp);

/* One module step in one call, as MEVPDynamics::update / BBMDynamics::update
 * (MEVPDynamics.cpp:59-87, BBMDynamics.cpp:63-104) make it with separate
 * calls: the inputs as nsdg_kernel_set_data takes them, in order, then
 * nsdg_kernel_update(t_start, dt), then the cell averages of the outputs as
 * nsdg_kernel_get_dg0 returns them.  Every host buffer has n_elements
 * (x n_comp) doubles.  The host copies of all inputs are issued at once and
 * the call waits once, at the end; the results are those of the separate
 * calls.  Errors as those calls report them; an unknown output name is
 * NSDG_ERR_UNKNOWN_FIELD before anything is copied.  No reference
 * counterpart (the reference makes the separate calls). */
typedef struct nsdg_field_in {
    const char* name;
    const double* data;
    size_t n_comp;
} nsdg_field_in;
typedef struct nsdg_field_out {
    const char* name;
    double* data;
} nsdg_field_out;
int nsdg_kernel_module_step(nsdg_kernel* k, const nsdg_field_in* in, size_t n_in, double t_start, double dt,
    const nsdg_field_out* out, size_t n_out);

/* One model step of length dt seconds (TimestepTime::step).  The step is
 * enqueued on the handle's CUDA stream (as one CUDA graph) and the call
 * returns without waiting; every get / snapshot / mean-value call waits for
 * it and reports NSDG_ERR_NUMERIC if the step produced non-finite values. */
int nsdg_kernel_update(nsdg_kernel* k, double t_start, double dt);

/* Waits for the enqueued work and reports device-side numeric faults. */
int nsdg_kernel_synchronize(nsdg_kernel* k);

/* Device-side state snapshot (checkpoint/resume).  nsdg_kernel_snapshot_size
 * returns the byte count; save writes it to a host buffer, load restores it. */
int nsdg_kernel_snapshot_size(nsdg_kernel* k, size_t* bytes);
int nsdg_kernel_snapshot_save(nsdg_kernel* k, void* buffer, size_t bytes);
int nsdg_kernel_snapshot_load(nsdg_kernel* k, const void* buffer, size_t bytes);

/* FP64 integral of a DG field over the mesh (Tools::MeanValue), computed on
 * the GPU with a deterministic warp-shuffle + block reduction. */
int nsdg_kernel_mean_value(nsdg_kernel* k, const char* name, double* out);

/* Measurement hooks (used by bench.py).  Times `steps` updates on the
 * handle's stream with CUDA events; *ms is the total device time. */
int nsdg_kernel_time_updates(nsdg_kernel* k, double dt, int steps, float* ms);
/* Times `reps` launches of one kernel of the step in isolation on the handle's
 * stream and returns the mean duration.  kernel_id: 0 = element stress kernel,
 * 1 = node momentum kernel, 2 = the transport stage the updates use, 13 = the
 * per-element transport kernel (kTransportStage); for mixed-precision mEVP
 * also 3 = stress kernel with operators by global loads, 4 = with operator
 * tiles by TMA, and on parallelogram meshes 5, 6, 7 = the coefficient kernel
 * with FP64 viscosity form 0, 1, 2 (see nsdg_selftest_viscosity), 8 = with
 * the float-pair form 3 (nsdg_selftest_viscosity_ff), 12 = with the checked
 * form 4 (nsdg_selftest_viscosity_checked); for FP64 mEVP 9, 10, 11 = the
 * stress kernel with FP64 FMAs, with float pairs, with float pairs staged by
 * TMA.  *name gets its name. */
int nsdg_kernel_time_kernel(nsdg_kernel* k, int kernel_id, int reps, float* mean_ms,
    const char** name);
/* Which mixed-precision mEVP stress kernel the updates use: *kind 0 =
 * operators by global loads, 1 = operator tiles by TMA, 2 = parallelogram
 * coefficients (chosen by timing at initialise; NSDG_STRESS_KERNEL =
 * global|tma|affine fixes it); for a mixed-precision BBM handle 2 = the
 * parallelogram BBM stress kernel, 0 = per-element operators
 * (NSDG_BBM_STRESS_KERNEL=general); *mismatch = the largest relative
 * difference, in FP64, between the exact operators and those rebuilt from
 * parallelogram coefficients (-1 when not evaluated, e.g. spherical or FP64
 * handles). */
int nsdg_kernel_stress_variant(nsdg_kernel* k, int* kind, double* mismatch);
/* Which transport stage the updates use: *tiled 1 = the parallelogram-mesh
 * kernel (mixed-precision mEVP on a Cartesian parallelogram mesh without
 * periodic edges: tiles of 32 x 8 elements, each interior edge flux evaluated
 * once into shared memory, the cell term from the Jacobian coefficients,
 * diagonal M^{-1}), 0 = the per-element kernel (NSDG_TRANSPORT_KERNEL=element
 * before initialise fixes it); *cell_mismatch = the largest relative
 * difference, in FP64, between the exact cell operators and those rebuilt
 * from the coefficients, *offdiag = the largest off-diagonal entry of an
 * element's M^{-1} relative to its diagonal (-1 when not evaluated). */
int nsdg_kernel_transport_variant(nsdg_kernel* k, int* tiled, double* cell_mismatch, double* offdiag);
/* Whether host arrays that are not page-locked move by a kernel that reads
 * or writes them directly (*direct = 1: the GPU accesses pageable host
 * memory, as on Grace, at the CPU-GPU link's rate; a copy from pageable
 * memory is staged through a driver buffer and runs at about half of it).
 * set_data, get_dg0 and module_step use it for such arrays; page-locked
 * arrays keep the copy engine.  NSDG_HOST_DIRECT=0 before initialise turns
 * it off.  No reference counterpart. */
int nsdg_kernel_host_direct(nsdg_kernel* k, int* direct);
/* The evaluation of P/(8 alpha Delta) in the parallelogram stress kernel:
 * 0 CUDA's rsqrt(double), 1 and 2 one FP64 Newton step from an FP32 seed
 * (2, the default: conversions on the integer pipe), 3 the same step in
 * float pairs, 4 form 3 checked against form 2's rounding, with form 2 where
 * the check fails: bitwise form 2.  NSDG_VISC_FORM=0..4 in the environment
 * before initialise selects one.  No reference counterpart. */
int nsdg_kernel_viscosity_form(nsdg_kernel* k, int* form);
/* Kernel launches issued by one update (for gpu_launches accounting). */
int nsdg_kernel_launches_per_update(nsdg_kernel* k, int* launches);

/* ======================================================================== */
/* Batched ensembles                                                         */
/* ======================================================================== */
/* Several independent dynamics kernels (ensemble members, uneven grids) stepped
 * together: one CUDA graph per step runs each member's transport and
 * preparation and then the mEVP sub-cycle of all members as one element launch
 * and one node launch per iteration.  No reference counterpart: the reference
 * runs one model (one kernel) per process.  Members must be initialised
 * Cartesian mEVP kernels in NSDG_PRECISION_MIXED with the same parameters; they keep
 * their own setData / getDG0Data, which are ordered after the ensemble's
 * update.  The element tile shape of every grid size is chosen at creation by
 * timing the candidates on the GPU; then the whole element phase is timed with
 * those tiles and with the TMA-staged kernel (32 consecutive elements per
 * block, 32 x 1) and the faster is kept (nsdg_ensemble_tile reports the
 * choice; NSDG_STRESS_KERNEL=tma|global in the environment fixes it). */
typedef struct nsdg_ensemble nsdg_ensemble;
int nsdg_ensemble_create(nsdg_kernel* const* members, int n_members, nsdg_ensemble** out);
int nsdg_ensemble_destroy(nsdg_ensemble* ens);
const char* nsdg_ensemble_last_error(const nsdg_ensemble* ens);
int nsdg_ensemble_update(nsdg_ensemble* ens, double t_start, double dt);
int nsdg_ensemble_synchronize(nsdg_ensemble* ens);
int nsdg_ensemble_time_updates(nsdg_ensemble* ens, double dt, int steps, float* ms);
int nsdg_ensemble_tile(nsdg_ensemble* ens, int member, int* tile_w, int* tile_h);
int nsdg_ensemble_launches_per_update(nsdg_ensemble* ens, int* launches);
/* on != 0: run the mEVP sub-cycle of all members as one persistent
 * cooperative launch per update (the iterations' element and node phases as
 * grid-stride loops separated by grid barriers whose waits are bounded: a wait
 * that runs out reports NSDG_ERR_CUDA through the next read) instead of one
 * element and one node launch per iteration.  Bitwise the same results.
 * Every member must be a parallelogram mesh (NSDG_ERR_UNSUPPORTED otherwise).
 * No reference counterpart. */
int nsdg_ensemble_set_persistent(nsdg_ensemble* ens, int on);

/* ======================================================================== */
/* Stand-alone DG transport (the DGTransport<DG> class of the reference)    */
/* ======================================================================== */
typedef struct nsdg_transport nsdg_transport;

/* Mesh given explicitly, as the reference tests build ParametricMesh by hand:
 * vertices (nx+1)*(ny+1)*2; landmask nx*ny (nonzero = ice, NULL = all ice);
 * dirichlet lists per edge (0 bottom, 1 right, 2 top, 3 left) of element ids;
 * periodic entries as 4 size_t each {edge type (0 X-edge, 1 Y-edge), cell 1,
 * cell 2, edge id}, segment by segment in the reference order.
 * dg: 1, 3, 6 or 8; scheme: 1, 2 or 3 (rk1/rk2/rk3). */
int nsdg_transport_create(int dg, size_t nx, size_t ny, const double* vertices,
    const unsigned char* landmask, const size_t* const dirichlet[4],
    const size_t n_dirichlet[4], const size_t* periodic, size_t n_periodic,
    int scheme, nsdg_transport** out);
int nsdg_transport_destroy(nsdg_transport* t);
const char* nsdg_transport_last_error(const nsdg_transport* t);
/* DG velocity components (n_elements*dg each, element-major). */
int nsdg_transport_set_velocity(nsdg_transport* t, const double* vx, const double* vy);
/* DGTransport::reinitnormalvelocity (DGTransport.cpp:158-252). */
int nsdg_transport_reinit_normal_velocity(nsdg_transport* t);
/* DGTransport::step on a host field (n_elements*dg), in place, `nsteps` times.
 * limit_max / limit_min != 0 apply LimitMax(phi, max) / LimitMin(phi, min)
 * after every step (dgLimit.hpp), as the periodic reference test does. */
int nsdg_transport_step(nsdg_transport* t, double dt, double* phi, int nsteps,
    int limit_max, double max_value, int limit_min, double min_value);
/* Tools::MeanValue of a host DG field (computed on the GPU, FP64). */
int nsdg_transport_mean_value(nsdg_transport* t, const double* phi, double* out);

/* ======================================================================== */
/* Warm-start network (no counterpart in the reference)                      */
/* ======================================================================== */
/* A stack of 3x3 convolutions (ReLU between layers) on the cell grid, trained
 * and evaluated on the GPU with BF16 tensor-core kernels accumulating in FP32.
 * channels: n_layers+1 counts, each 16, 32, 48 or 64; the first `used_outputs`
 * output channels enter the masked mean-squared-error loss.  Parameters are
 * one FP32 vector: per layer the weights W[co][3*dy+dx][ci] then the biases. */
typedef struct nsdg_net nsdg_net;
int nsdg_net_create(int n_layers, const int* channels, int height, int width, int max_batch,
    int used_outputs, unsigned long long seed, nsdg_net** out);
int nsdg_net_destroy(nsdg_net* net);
const char* nsdg_net_last_error(const nsdg_net* net);
int nsdg_net_param_count(nsdg_net* net, size_t* n);
int nsdg_net_get_params(nsdg_net* net, float* host, size_t n);
int nsdg_net_set_params(nsdg_net* net, const float* host, size_t n);
int nsdg_net_get_grads(nsdg_net* net, float* host, size_t n);
/* host input [batch][h][w][ch0] (rounded to BF16), target [batch][h][w][chL],
 * mask [batch][h][w]; target and mask may be NULL */
int nsdg_net_set_batch(nsdg_net* net, int batch, const float* input, const float* target,
    const float* mask);
int nsdg_net_forward(nsdg_net* net, int batch, float* out_host);
/* The forward pass `reps` times on the network's stream, without copies:
 * *ms = milliseconds per pass by CUDA events.  No reference counterpart. */
int nsdg_net_time_forward(nsdg_net* net, int batch, int reps, float* ms);
/* loss and gradients of the last forward pass (gradients stay on the device) */
int nsdg_net_loss_backward(nsdg_net* net, int batch, float* loss);
int nsdg_net_adam_step(nsdg_net* net, float lr, float beta1, float beta2, float eps);

/* ---- learned warm start of the mEVP sub-cycle ----------------------------
 * No counterpart in the reference, which always runs the fixed mEVP count
 * (VPCGDynamicsKernel.hpp:76, DynamicsKernel.hpp:187: nSteps = 100).  The
 * network maps, per cell, NSDG_WARM_FEATURES features of the state at the
 * start of the sub-cycle (h, A, sea mask, u and v at the four CG2 nodes the
 * cell owns, wind and ocean velocity, the 18 stress-divergence entries
 * carried from the last sub-cycle, and the change of those u, v and
 * divergence values since the start of the previous sub-cycle) to the
 * increments of u, v and divergence that the plain sub-cycle reaches after
 * n_steps - K iterations; the warm sub-cycle adds them and runs K iterations.
 * Such a network has NSDG_WARM_FEATURES input channels, NSDG_WARM_TARGETS
 * output channels and NSDG_WARM_USED used outputs; its height/width are the
 * grid's ny/nx. */
#define NSDG_WARM_FEATURES 64
#define NSDG_WARM_TARGETS 32
#define NSDG_WARM_USED 26
#define NSDG_NET_NORM_FLOATS 192 /* feature mean[64], 1/std[64], target mean[32], std[32] */
/* Device dataset of `capacity` samples (features, targets, mask per cell). */
int nsdg_net_dataset_reserve(nsdg_net* net, int capacity);
/* Per-channel mean/std of the first `count` samples over sea cells; the
 * network normalises its inputs and outputs with them. */
int nsdg_net_dataset_normalise(nsdg_net* net, int count);
/* `iterations` Adam steps on random batches drawn (seeded) from the first
 * `count` samples; *loss = mean loss of the last 20 steps. */
int nsdg_net_train(nsdg_net* net, int count, int iterations, int batch, float lr,
    unsigned long long seed, float* loss);
int nsdg_net_get_normalisation(nsdg_net* net, float* host, size_t n);
int nsdg_net_set_normalisation(nsdg_net* net, const float* host, size_t n);
/* One plain model step, as nsdg_kernel_update (mEVP, mixed precision), that
 * also writes dataset sample `slot` (slot < 0: none): the features at the
 * start of the sub-cycle and the increments after n_steps - k_iters
 * iterations.  *plain_ratio = |u^n - u^(n-1)| / |u^n - u^0| of the plain
 * sub-cycle's last iteration (RMS over CG2 nodes: the warm-start residual). */
int nsdg_kernel_warm_sample(nsdg_kernel* k, double t_start, double dt, int k_iters,
    nsdg_net* net, int slot, double* plain_ratio);
/* Attaches (net != NULL) or detaches the warm start.  Each later update runs
 * network + k_iters iterations and accepts the result when the warm start is
 * enabled, the attempt produced only finite values and its residual (as
 * above) is at most `kappa`; otherwise it restores the state at the start of
 * the sub-cycle and runs the plain n_steps iterations.  With audit_every > 0,
 * the first update and every audit_every-th after it are audited: the warm
 * attempt and the plain sub-cycle both run from the same start, the plain
 * result is kept, and the warm start stays enabled until the next audit
 * only if |warm - plain| / |plain - start| (RMS over CG2 nodes) <= audit_tol.
 * All decisions are taken on the device, inside the update's CUDA graphs.
 * The net must stay alive while attached.  mEVP in mixed precision only
 * (NSDG_ERR_UNSUPPORTED otherwise). */
int nsdg_kernel_set_warm_start(nsdg_kernel* k, nsdg_net* net, int k_iters, double kappa,
    int audit_every, double audit_tol);
typedef struct nsdg_warm_stats {
    long long accepted, fallbacks;       /* warm updates accepted / fallen back   */
    long long audited, audit_rejected;    /* audited updates / audits that disabled it */
    double last_ratio, last_audit_error;
    int enabled;                         /* current audit                     */
    int launches_warm, launches_audited, launches_fallback; /* kernels per graph    */
} nsdg_warm_stats;
int nsdg_kernel_warm_stats(nsdg_kernel* k, nsdg_warm_stats* out);

/* ======================================================================== */
/* Failure-detection self-test                                               */
/* ======================================================================== */
/* No counterpart in the reference.  The only waits in the library's kernels
 * (the TMA stress kernel's mbarrier waits) are bounded in time; this runs one
 * such wait on an mbarrier that nothing completes, with a limit of
 * limit_seconds (0 < limit <= 2), and reports *timed_out = 1 when the wait ran
 * out and the kernel returned as it must.  The GPU context stays usable. */
/* Host only (no GPU): the largest relative FP64 difference between the exact
 * mEVP stress operators of a Cartesian mesh (coords as for
 * nsdg_kernel_initialise) and those rebuilt from parallelogram coefficients.
 * Mixed-precision handles use the parallelogram stress kernel when it is at
 * most 1e-9. */
int nsdg_mesh_parallelogram_mismatch(size_t nx, size_t ny, const double* coords, int dg_comp, double* mismatch);
/* Host only (no GPU): every check that admits the parallelogram kernels, as
 * out[4]: 0 the mEVP stress operators' mismatch (as above), 1 the transport
 * cell operators rebuilt from the coefficients, 2 the largest off-diagonal of
 * an element's M^{-1} relative to its diagonal, 3 the BBM projection and
 * divergence operators rebuilt from the unit square's; FP64, relative.
 * Mixed-precision handles take the tiled transport when 1 <= 1e-9 and
 * 2 <= 1e-12, the parallelogram BBM kernel when 0 and 3 <= 1e-9. */
int nsdg_mesh_parallelogram_checks(size_t nx, size_t ny, const double* coords, int dg_comp, double* out);

/* The closed (Dirichlet) element sides a handle derives from its mask at
 * initialise (ParametricMesh::landmaskFromModelArray, dirichletFromMask,
 * dirichletFromEdge and sortDirichlet, ParametricMesh.cpp:217-272): counts[s]
 * ascending element ids i + nx*j for side s (0 bottom, 1 right, 2 top,
 * 3 left), written to ids side after side.  mask: nx*ny doubles, 1.0 = ice.
 * NSDG_ERR_SIZE_MISMATCH (counts still set) when capacity < their sum.
 * Host only. */
int nsdg_mesh_dirichlet(size_t nx, size_t ny, const double* mask, size_t* counts, size_t* ids,
    size_t capacity);
/* P / (8 alpha Delta), Delta = sqrt(inv + delta_min^2), for n host values by
 * the three FP64 forms of the mixed-precision stress kernels: out[k n + i]
 * for form k = 0 (CUDA's rsqrt(double)), 1 (one Newton-Raphson step in FP64
 * from an FP32 rsqrtf seed), 2 (the same with float/double conversions on
 * the integer pipe).  Inputs: inv >= 0, Pa >= 0. */
int nsdg_selftest_viscosity(size_t n, const float* inv, const double* Pa, double delta_min, float* out);
/* The same quantity by form 3: the Newton step of form 2 from the same seed
 * with float pairs on the FP32 pipe (one FP64 subtraction per value).  out[n].
 * The stress kernel with this form runs only through
 * nsdg_kernel_time_kernel(kernel_id = 8). */
int nsdg_selftest_viscosity_ff(size_t n, const float* inv, const double* Pa, double delta_min, float* out);
/* The kernels' form 4 (the float-pair form checked against form 2's rounding,
 * form 2 where the check fails) at each (inv, Pa): out[n], bitwise equal to
 * form 2 (out[2 n + i] of nsdg_selftest_viscosity).  No reference counterpart. */
int nsdg_selftest_viscosity_checked(size_t n, const float* inv, const double* Pa, double delta_min, float* out);
/* The float-pair arithmetic of the FP64 path's stress kernel
 * (kMevpStressPairs) on n value pairs (a[i], x[i]), returned in FP64:
 * out[4 i + 0] = split(a) - a (the representation error of the pair),
 * out[4 i + 1] = RN_float(x) widened back to double by its bit pattern,
 * out[4 i + 2] = a x in float pairs,
 * out[4 i + 3] = sum_k a[j_k] x[j_k] over j_k = (i + 7 k) mod n, k < 9, in
 *                float pairs (the kernel's dot-product accumulation).
 * Inputs must be finite and, where non-zero, between 2^-74 and 2^127 in
 * magnitude.  No reference counterpart: a check of this library's arithmetic. */
int nsdg_selftest_pairs(size_t n, const double* a, const double* x, double* out);
int nsdg_selftest_bounded_wait(double limit_seconds, int* timed_out);

/* ======================================================================== */
/* Allocation-free entry point                                               */
/* ======================================================================== */
/* No counterpart in the reference.  Tools::MeanValue (the FP64 mesh integral
 * of a DG field) for callers that cannot allocate device memory: a host model
 * whose pool allocator owns the GPU memory, or a time-critical loop that may
 * not pay cudaMalloc's implicit synchronisation.  phi: device array
 * double[dg][n_elements] (component-major); jw: device array
 * double[9][n_elements], Jacobian times Gauss weight at the 3x3 Gauss points,
 * point q = ix + 3 iy at local coordinates (g[ix], g[iy]) of the unit square,
 * g = (1/2 - sqrt(3/20), 1/2, 1/2 + sqrt(3/20)), x fastest (for a field that
 * is not symmetric the other order gives a wrong integral);
 * out: one device double; stream: a cudaStream_t (NULL = legacy default).
 * The reduction's scratch is a fixed array inside the library, held on every
 * GPU that loads it until the process exits; n_elements above
 * NSDG_NOALLOC_MAX_ELEMENTS returns NSDG_ERR_SIZE_MISMATCH.  The first call on
 * a device looks up that array's address with the device current (make it
 * before any stream capture that would record a later call), and keeps it
 * for the life of the process: after cudaDeviceReset (or anything else that
 * re-creates the device's primary context) that address is stale, so do not
 * call this entry point on a device after resetting it.  Calls share the
 * array: calls that overlap on the GPU race.  Nothing is allocated. */
#define NSDG_NOALLOC_MAX_ELEMENTS (1u << 24)
int nsdg_mean_value_noalloc(int dg, size_t n_elements, const double* phi, const double* jw,
    double* out, void* stream);

/* ======================================================================== */
/* Restart and forcing files: ParaGridIO's NetCDF-4 layout (reading)         */
/* ======================================================================== */
/* Replaces the netCDF-C reads of ParaGridIO::getModelState
 * (core/src/ParaGridIO.cpp:87-208) and ParaGridIO::readForcingTimeStatic
 * (core/src/ParaGridIO.cpp:210-270) with a self-contained host reader of the
 * HDF5 subset netCDF-4 files use (no netCDF or HDF5 library needed).  A file
 * holds the groups "structure" (attribute "type"), "metadata" and "data";
 * the model fields are the variables of "data".  Host code only: no GPU is
 * touched; the values go to a kernel handle through nsdg_kernel_set_data. */
typedef struct nsdg_restart nsdg_restart;

/* ModelArray::Type (core/src/discontinuousgalerkin/include/ModelArrayDetails.hpp:19-28) */
#define NSDG_MA_H 0
#define NSDG_MA_VERTEX 1
#define NSDG_MA_U 2
#define NSDG_MA_V 3
#define NSDG_MA_Z 4
#define NSDG_MA_DG 5
#define NSDG_MA_DGSTRESS 6
#define NSDG_MA_CG 7
#define NSDG_MA_NONE (-1) /* no ModelArray type for the variable's dimensions */

/* Opens and maps a file; NSDG_ERR_BAD_ARG when it cannot be opened,
 * NSDG_ERR_UNSUPPORTED for HDF5 features outside the subset (compression,
 * old-style groups), NSDG_ERR_LOGIC for a damaged file (message in
 * nsdg_restart_last_error of the returned handle, or of NULL). */
int nsdg_restart_open(const char* path, nsdg_restart** out);
int nsdg_restart_close(nsdg_restart* r);
const char* nsdg_restart_last_error(const nsdg_restart* r);
/* Number of netCDF variables in a group ("data", "metadata/time"; "" is the
 * root group), in creation order; NSDG_ERR_UNKNOWN_FIELD for no such group. */
int nsdg_restart_num_vars(nsdg_restart* r, const char* group, size_t* n);
/* Variable `index` of `group`: its name (NUL-terminated, at most name_cap
 * bytes), the ModelArray type its dimension names give (the dimension keys
 * of ParaGridIO.cpp:34-47, accepting the time record dimension of forcing
 * files in front), the component count (DG, DGSTRESS, VERTEX: the last
 * dimension; otherwise 1), the number of time records (1 for variables
 * without the unlimited "time" dimension) and the values per record.  Any
 * output pointer may be NULL. */
int nsdg_restart_var_info(nsdg_restart* r, const char* group, size_t index, char* name, size_t name_cap,
    int* model_type, size_t* n_components, size_t* n_records, size_t* n_values);
/* The variable's dimension names, comma-separated in netCDF order ("time,y,x"). */
int nsdg_restart_dim_names(nsdg_restart* r, const char* path, char* out, size_t cap);
/* Record `record` of the variable at `path` ("data/hice") as double, in
 * ModelArray order (index = component + n_components (i + nx j), the order
 * the file stores); n must equal the values per record. */
int nsdg_restart_read(nsdg_restart* r, const char* path, size_t record, double* out, size_t n);
/* A text attribute of the object at `path` (attribute non-NULL: "structure"
 * and "type"), or the first string of a string variable (attribute NULL:
 * "metadata/time/formatted").  NSDG_ERR_SIZE_MISMATCH when cap is too small. */
int nsdg_restart_text(nsdg_restart* r, const char* path, const char* attribute, char* out, size_t cap);

/* Writing: ParaGridIO::dumpModelState (core/src/ParaGridIO.cpp:272-348)
 * with CommonRestartMetadata's "structure" and "metadata" groups
 * (core/src/CommonRestartMetadata.cpp:18-72).  create() lays out the groups,
 * the metadata time (seconds since 1970 and its formatted string) and every
 * dimension of the data group (xdim, ydim, zdim, xvertex, yvertex, x_cg,
 * y_cg, dg_comp, dgstress_comp, ncoords); add() copies one field in
 * ModelArray order with the dimensions of its type and a missing_value
 * attribute; save() writes the file (NetCDF-4 layout, contiguous doubles).
 * The writer is host memory only. */
typedef struct nsdg_restart_writer nsdg_restart_writer;
int nsdg_restart_writer_create(size_t nx, size_t ny, size_t nz, int dg_comp, int dgstress_comp, int cg_degree,
    const char* structure_type, long long time_seconds, const char* time_formatted, nsdg_restart_writer** out);
int nsdg_restart_writer_add(nsdg_restart_writer* w, const char* name, int model_type, const double* data, size_t n);
int nsdg_restart_writer_save(nsdg_restart_writer* w, const char* path);
int nsdg_restart_writer_destroy(nsdg_restart_writer* w);
const char* nsdg_restart_writer_last_error(const nsdg_restart_writer* w);
/* Diagnostic files: ParaGridIO::writeDiagnosticTime
 * (core/src/ParaGridIO.cpp:350-500).  The same groups, with an unlimited
 * "time" axis in the data group; each record() call is one
 * writeDiagnosticTime call: it appends the time (seconds since 1970) and one
 * record of every field (n_fields names, NSDG_MA_* types, data in ModelArray
 * order, value counts).  The first call defines the variables; "mask" and
 * VERTEX fields are written once, without the time axis, the mask with the
 * dimensions (xdim, ydim) in the order the reference lists them; a later
 * record naming a field the first did not gives NSDG_ERR_UNKNOWN_FIELD, and
 * a field it leaves out holds the fill value there.  Records stay in host
 * memory until nsdg_restart_writer_save writes the file (the reference
 * writes them when its open file is closed). */
int nsdg_diagnostic_writer_create(size_t nx, size_t ny, size_t nz, int dg_comp, int dgstress_comp, int cg_degree,
    const char* structure_type, long long time_seconds, const char* time_formatted, nsdg_restart_writer** out);
int nsdg_diagnostic_writer_record(nsdg_restart_writer* w, double time_seconds, size_t n_fields,
    const char* const* names, const int* model_types, const double* const* data, const size_t* n);

/* ======================================================================== */
/* Column thermodynamics: ice growth (the step before the dynamics)          */
/* ======================================================================== */
/* IceGrowth::update (physics/src/IceGrowth.cpp:148-171) on the GPU with the
 * modules it drives: ThermoIce0 (zero-layer vertical growth, the default,
 * physics/src/modules/IceThermodynamicsModule/ThermoIce0.cpp:85-172) or
 * ThermoWinton (three-layer, .../ThermoWinton.cpp:102-342),
 * HiblerSpread (lateral growth and melt, .../HiblerSpread.cpp:53-66),
 * ConstantHealing (damage healing, .../ConstantHealing.cpp:53-73) and
 * IceMinima, or their Dummy / NoHealing alternatives.  Per element, in the
 * reference's order: true thicknesses from the cell averages, the minimum
 * limits, vertical growth, new ice over open water, lateral spread, the
 * limits again, healing.  All arithmetic is FP64, element-local, in the
 * reference's operation order (bit-identical to the CPU oracle).  Fields are
 * one double per element (H-type ModelArrays, index i + nx j); the update
 * runs over the ocean elements of the mask (ModelComponent::overElements). */
typedef struct nsdg_ice_growth nsdg_ice_growth;

typedef struct nsdg_ice_growth_params {
    double ks;           /* snow conductivity, W K^-1 m^-1 (nextsim_thermo.ks: 0.3096) */
    double h_min;        /* minimum ice thickness, m (nextsim_thermo.min_thick: 0.01) */
    double c_min;        /* minimum concentration (nextsim_thermo.min_conc: 1e-12) */
    double h0;           /* thickness of newly frozen ice, m (Hibler.h0: 0.25) */
    double phi_m;        /* melt exponent (Hibler.phiM: 0.5) */
    double healing_time; /* healing time scale, s (ConstantHealing.td: 15 days) */
    int use_thermo;      /* nextsim_thermo.use_thermo_forcing (1) */
    int thermo_model;    /* 0 ThermoIce0, 1 DummyIceThermodynamics, 2 ThermoWinton (three
                            temperature levels: "tice", "tice_1", "tice_2") */
    int lateral_model;   /* 0 HiblerSpread, 1 DummyIceSpread */
    int healing_model;   /* 0 ConstantHealing, 1 NoHealing */
    int flooding;        /* ThermoIce0 snow-to-ice conversion (1) */
} nsdg_ice_growth_params;

/* Field slots (the names nsdg_ice_growth_set_field / get_field take).
 * Inputs: the prognostic cell averages and the forcing the other modules
 * provide; outputs: IceGrowth's and ThermoIce0's arrays after an update.
 * qow, qio and damage are read and written.  Outputs that an update leaves
 * untouched keep their previous values (as the reference's member arrays
 * do); every slot starts at zero. */
enum {
    NSDG_IG_HICE_CELL = 0, /* "hice": cell-averaged ice thickness, m (Protected::H_ICE) */
    NSDG_IG_CICE0,         /* "cice": ice concentration (Protected::C_ICE) */
    NSDG_IG_HSNOW_CELL,    /* "hsnow": cell-averaged snow thickness, m */
    NSDG_IG_TICE0,         /* "tice": ice surface temperature, C (Protected::T_ICE) */
    NSDG_IG_QIA,           /* "qia": ice-atmosphere heat flux, W m^-2 */
    NSDG_IG_DQIA_DT,       /* "dqia_dt": its temperature derivative, W m^-2 K^-1 */
    NSDG_IG_QOW,           /* "qow": open-water heat flux, W m^-2 (read, written) */
    NSDG_IG_QIO,           /* "qio": ice-ocean heat flux, W m^-2 (read, written) */
    NSDG_IG_SUBLIM,        /* "sublim": sublimation rate, kg m^-2 s^-1 */
    NSDG_IG_SNOWFALL,      /* "snowfall": snowfall rate, kg m^-2 s^-1 */
    NSDG_IG_PENSW,         /* "penSW": penetrating short wave, W m^-2 */
    NSDG_IG_SST,           /* "sst": sea surface temperature, C */
    NSDG_IG_TF,            /* "tf": sea water freezing point, C */
    NSDG_IG_MLBHC,         /* "mlbhc": mixed layer bulk heat capacity, J K^-1 m^-2 */
    NSDG_IG_DAMAGE,        /* "damage" (read, written) */
    NSDG_IG_HICE,          /* "hice_updated": true ice thickness after the update, m */
    NSDG_IG_CICE,          /* "cice_updated" */
    NSDG_IG_HSNOW,         /* "hsnow_updated": true snow thickness, m */
    NSDG_IG_HICE0,         /* "hice_initial": true ice thickness at the start, m */
    NSDG_IG_HSNOW0,        /* "hsnow_initial" */
    NSDG_IG_NEWICE,        /* "newice": new ice over open water, m */
    NSDG_IG_DELTA_CICE,    /* "delta_cice" */
    NSDG_IG_DELTA_HICE,    /* "delta_hice": vertical thickness change, m */
    NSDG_IG_TICE,          /* "tice_updated": updated ice temperature, C */
    NSDG_IG_QIC,           /* "qic": conductive heat flux in the ice, W m^-2 */
    NSDG_IG_SNOW_TO_ICE,   /* "snow_to_ice": flooded snow converted to ice, m */
    NSDG_IG_TOP_MELT,      /* "top_melt", m */
    NSDG_IG_BOT_MELT,      /* "bottom_melt", m */
    NSDG_IG_SNOW_MELT,     /* "snow_melt", m */
    NSDG_IG_DELTA_CFREEZE, /* "delta_cfreeze" */
    NSDG_IG_DELTA_CMELT,   /* "delta_cmelt" */
    NSDG_IG_TICE0_1,       /* "tice_1": ice temperature, upper layer, C (ThermoWinton) */
    NSDG_IG_TICE0_2,       /* "tice_2": ice temperature, lower layer, C (ThermoWinton) */
    NSDG_IG_TICE_1,        /* "tice_updated_1" */
    NSDG_IG_TICE_2,        /* "tice_updated_2" */
    NSDG_IG_NFIELDS
};

void nsdg_ice_growth_default_params(nsdg_ice_growth_params* p);
/* mask: n_elements doubles, > 0 for ocean (NULL: all ocean). */
int nsdg_ice_growth_create(size_t n_elements, const double* mask, const nsdg_ice_growth_params* p,
    nsdg_ice_growth** out);
int nsdg_ice_growth_destroy(nsdg_ice_growth* g);
const char* nsdg_ice_growth_last_error(nsdg_ice_growth* g);
int nsdg_ice_growth_set_field(nsdg_ice_growth* g, const char* name, const double* data, size_t n);
int nsdg_ice_growth_get_field(nsdg_ice_growth* g, const char* name, double* out, size_t n);
/* One IceGrowth::update of dt seconds. */
int nsdg_ice_growth_update(nsdg_ice_growth* g, double dt);
/* Device time of `reps` updates (the fields evolve), for the benchmark. */
int nsdg_ice_growth_time_updates(nsdg_ice_growth* g, double dt, int reps, float* ms);
/* Device-side coupling with a dynamics handle on the same mesh, replacing
 * the host round trip of PrognosticData::update / updatePrognosticFields
 * (core/src/PrognosticData.cpp:83-118):
 *   direction 0: the dynamics' DG0 thickness, concentration and damage
 *                become the growth inputs "hice", "cice", "damage";
 *   direction 1: hice_updated x cice_updated, cice_updated and damage
 *                become the dynamics' "hice", "cice", "damage" as H-type
 *                inputs (component 0 set, higher components zeroed, as
 *                setData does with a one-component array).
 * Ordered after both handles' queued work; no host copies. */
int nsdg_ice_growth_exchange(nsdg_ice_growth* g, nsdg_kernel* k, int direction);

#ifdef __cplusplus
}
#endif

#endif /* NSDG_H */
