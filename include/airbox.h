/* airbox.h - C ABI of libairbox.so, the GB300 (sm_103a) compute core of the
 * airbox-flow tool.
 *
 * Every entry point replaces one function of the reference's engine surface,
 * src/engine.js (module.exports at src/engine.js:803), and is named after it.
 * Plain pointers and sizes only; all host buffers are caller-owned, all device
 * memory is owned by the opaque handles.  Every call returns an abx_status;
 * on failure abx_last_error() holds the reference's message text for that
 * condition (German, as thrown by engine.js) or a CUDA error string.
 *
 * Threading: a handle may be used from one thread at a time.  Each simulation
 * handle owns one CUDA stream; calls block until their GPU work is done.
 * There is no CPU fallback: without a usable sm_103a GPU every compute call
 * fails with ABX_ERR_CUDA.
 */
#ifndef AIRBOX_H
#define AIRBOX_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Version of the structures and entry points below; a host compares it with abx_abi_version() before use.
 * 2: prepare timings in abx_geom_info, coordinate channels in abx_net_params, batch groups.
 * 3: abx_run_params.flags (bfloat16 storage only on request), vectorised-kernel fields in abx_sim_info,
 *    stop rules in abx_converge_params, tensor-core convolutions of the warm-start network. */
#define ABX_ABI_VERSION 3

/* Status codes.  The first group mirrors the errors engine.js throws. */
typedef enum {
  ABX_OK = 0,
  ABX_ERR_NO_TRIANGLES = 1,      /* src/engine.js:26  "STL enthält keine Dreiecke." */
  ABX_ERR_SAME_AXIS = 2,         /* src/engine.js:33  seal and inlet on the same axis */
  ABX_ERR_GRID_TOO_LARGE = 3,    /* src/engine.js:124 grid above the cell cap */
  ABX_ERR_NO_OPENING = 4,        /* src/engine.js:156 no inlet opening found */
  ABX_ERR_OPENING_TOO_SMALL = 5, /* src/engine.js:171 opening below 8 cells */
  ABX_ERR_SEAL_OUTSIDE = 6,      /* src/engine.js:180 seal plane outside the model */
  ABX_ERR_LEAK = 7,              /* src/engine.js:195 air leaks through a thin wall */
  ABX_ERR_LID_TOO_LOW = 8,       /* src/engine.js:200 outlet lid lower than a cell */
  ABX_ERR_BAD_OUTLET = 9,        /* src/engine.js:210 outlet not above the filter */
  ABX_ERR_UNSTABLE = 10,         /* src/engine.js:335 non-finite flux at a progress check */
  ABX_ERR_NOT_PREPARED = 11,     /* src/engine.js:796 run without a prepared geometry */
  ABX_ERR_CANCELLED = 12,        /* progress callback asked to stop (the UI's cancel, src/ui.html:508) */
  ABX_ERR_INVALID_ARGUMENT = 20, /* bad pointer, size or parameter (no reference counterpart) */
  ABX_ERR_CUDA = 21,             /* CUDA runtime error; no GPU fallback exists */
  ABX_ERR_OUT_OF_MEMORY = 22
} abx_status;

/* Population storage of a simulation. */
typedef enum {
  ABX_STORE_F32 = 0,        /* float32 populations, float32 collision (the WGSL lbm_step contract, src/engine.js:378-450) */
  ABX_STORE_F32_EXACT = 1,  /* float32 populations, float64 collision in cpuStep's exact operation order (src/engine.js:266-321) */
  ABX_STORE_F16 = 2,        /* binary16 shifted deviations f - w_i, float32 collision */
  ABX_STORE_BF16 = 3,       /* bfloat16 shifted deviations f - w_i, float32 collision; only with
                               ABX_RUN_ALLOW_BF16: its 8 significant bits do not resolve the density
                               differences behind zeta on large, fine grids (6.5 % off the float64 run
                               on a 512x256x384-cell airbox, where float16 stays within 0.5 %) */
  ABX_STORE_F64 = 4         /* float64 populations and collision (an FP64 run on the GPU) */
} abx_storage;

/* Message of the last failed call on this thread ("" if none). */
const char *abx_last_error(void);
int abx_abi_version(void);
/* Number of CUDA devices visible (0 without a GPU); never fails. */
int abx_device_count(void);

/* parseSTL (src/engine.js:15-28).  Binary if 84 + 50 n == len, else ASCII
 * "vertex x y z" records.  Call with out == NULL to get *nfloats (9 per
 * triangle), then again with cap >= *nfloats. */
int abx_parse_stl(const void *buf, size_t len, float *out, size_t cap, size_t *nfloats);

/* prepare(p) parameters (src/engine.js:111, fields of src/ui.html:477-479). */
typedef struct {
  double dx;                     /* cell size h, mm */
  int seal_axis;                 /* p.sealAxis 0..2 */
  double seal_sign;              /* p.sealSign +-1 */
  double seal;                   /* p.seal, model coordinate of the seal plane */
  int inlet_axis;                /* p.inletAxis 0..2 */
  double inlet_sign;             /* p.inletSign +-1 */
  double inlet_yaw;              /* p.inletYaw, degrees */
  double pleat;                  /* p.pleat, mm */
  int has_click; double click[3];            /* p.click (model coordinates) or none */
  int has_outlet; double outlet_center[3];   /* p.outlet.enabled / .center */
  double outlet_diameter, outlet_height;     /* p.outlet.diameter / .height */
  double max_cells;              /* cell cap; the reference's is 4.5e6 (src/engine.js:124) */
  int device;                    /* CUDA device ordinal */
} abx_prepare_params;

typedef struct abx_geom abx_geom;

/* prepare(p) (src/engine.js:111-234): frame transform, grid sizing, GPU parity
 * voxelizer at 3x oversampling with the 27->1 downsample, opening detection,
 * inlet duct, flood fill, leak check, outlet plane/plenum.  `tris` holds
 * nfloats model-space floats (9 per triangle) in host memory. */
int abx_prepare(const float *tris, size_t nfloats, const abx_prepare_params *p, abx_geom **out);
void abx_geom_free(abx_geom *g);

/* The prepare() return object's scalars and its `summary` (src/engine.js:226-233). */
typedef struct {
  int nx, ny, nz; int64_t N;
  int nf;                 /* fluid cells (g.nf) */
  int top, jm, kw0, kf;
  int n_holes, n_open, af, n_out, leak_cells, pleat_ok;
  double h, origin[3], mn[3], mx[3], pleat;
  double volume_l, inlet_cm2, filter_cm2, outlet_cm2, outlet_cm2_real;
  double frame_cy, frame_sy;  /* cos/sin of the yaw used by the frame */
  int64_t kernel_launches;    /* kernels prepare() launched */
  int64_t h2d_bytes, d2h_bytes;  /* bytes prepare() copied host->device / device->host */
  double ms_voxelize, ms_masks, ms_device;  /* wall time: GPU voxelizer (incl. read-back), opening/duct/flood/
                                               leak/outlet, classes/segments/device arrays */
} abx_geom_info;
int abx_geom_get_info(const abx_geom *g, abx_geom_info *out);
/* Host copies of g.solid / g.fluid / g.outlet (N bytes each, index (i*ny+j)*nz+k),
 * g.opening (nx*ny) and g.xc/g.dc/g.zc (float).  Any pointer may be NULL. */
int abx_geom_get_masks(const abx_geom *g, uint8_t *solid, uint8_t *fluid, uint8_t *opening, uint8_t *outlet,
                       float *xc, float *dc, float *zc);
/* The fine (3x) voxel grid of voxelize() (src/engine.js:45-93), nxf*nyf*nzf bytes,
 * recomputed on the GPU on demand.  For grids up to 2^31 fine voxels. */
int abx_geom_get_fine(const abx_geom *g, uint8_t *fine, size_t cap);

/* abx_run_params.flags */
#define ABX_RUN_ALLOW_BF16 1u    /* accept ABX_STORE_BF16 (rejected otherwise: its KPIs can miss 0.5 %) */

/* simulate() parameters (src/engine.js:237, fields of src/ui.html:502-504). */
typedef struct {
  double K, aniso, u, tau;       /* filter resistance, cross-pleat factor, inlet speed, relaxation time */
  int steps, avg, every;         /* time steps, averaged tail, progress interval */
  int storage;                   /* abx_storage */
  unsigned flags;                /* ABX_RUN_* bits; 0 for the reference's behaviour */
} abx_run_params;

typedef struct abx_sim abx_sim;

/* setupSim(g, p) (src/engine.js:239-264) plus device state: populations set
 * to w_i, averages cleared.  `ns` is the optional partial bounce-back field
 * (src/engine.js:238, 313-317): NF floats in fluid-cell order, or NULL. */
int abx_sim_create(abx_geom *g, const abx_run_params *p, const float *ns, abx_sim **out);
void abx_sim_free(abx_sim *s);

typedef struct {
  int NF, Ain, Af, Lp, n_layer_m, n_layer_t;
  double u0, tau0, sig, aniso, cs2s, uface;
  int step, nacc;               /* steps done, steps accumulated */
  int64_t Np;                   /* padded cells held on the device */
  int64_t state_bytes;          /* device bytes of populations + averages */
  int tma_pipeline;             /* 1 when the step kernel is fed by TMA tensor copies */
  int vec_width;                /* cells per thread of the vectorised step kernel (0: one cell per lane) */
  int64_t vec_interior_cells;   /* fluid cells it moves as vectors (known after the first step; the rest
                                   run one per lane) */
} abx_sim_info;
int abx_sim_get_info(const abx_sim *s, abx_sim_info *out);

/* Back to the initial state (f = w_i, averages and history cleared). */
int abx_sim_reset(abx_sim *s);

/* n calls of cpuStep (src/engine.js:266-321) / lbm_step (:378-450), adding to
 * the averages when `accumulate` is nonzero. */
int abx_sim_step(abx_sim *s, int n, int accumulate);

/* Progress report of simulate()'s onProgress (src/engine.js:330-339,351-354). */
typedef struct {
  int step, steps;
  double gamma, mass_ratio, elapsed_s, eta_s, mlups;
} abx_progress;
/* Return nonzero to cancel the run (ABX_ERR_CANCELLED). */
typedef int (*abx_progress_fn)(const abx_progress *info, void *user);

/* The simulate() step loop (src/engine.js:341-358, simulateGPU :613-630):
 * steps with the averaging window, a probe every `every` steps, and the
 * instability check of progressInfo (:335).  With cb == NULL the host does
 * not wait for the GPU until the end. */
int abx_sim_run(abx_sim *s, abx_progress_fn cb, void *user);

/* Post-collision populations f (19*NF floats, f[i*NF + a]) in the reference's
 * layout, and the way back (for self-tests and warm starts). */
int abx_sim_get_f(abx_sim *s, float *f);
int abx_sim_set_f(abx_sim *s, const float *f);
/* Clears the time averages (sums and step count) and keeps the populations:
 * the next accumulating steps start a new averaging window.  No counterpart
 * in the reference (its averaging window is fixed by steps/avg); used by the
 * windowed convergence run. */
int abx_sim_clear_acc(abx_sim *s);
/* Time-averaged fields acc[comp*NF + a], comp = ux, uy, uz, rho, divided by
 * the accumulated step count as simulate() does (src/engine.js:356). */
int abx_sim_get_acc(abx_sim *s, float *acc);

/* evaluate() metrics (src/engine.js:681-685). */
typedef struct {
  double gamma, gammaCore, lowCore, highCore, reverse, maxToMean, zeta, inlet_cm2, filter_cm2;
  double wm, cm; int n, cn, pinN, pbN, jb;
} abx_metrics;
/* field3d (src/engine.js:698-719) on the device: on every cell of the grid
 * (index (i*ny + j)*nz + k; NaN where there is no air or k < kB) the speed
 * |u|/u0, the static pressure relative to the space under the filter and
 * the total-pressure loss since the inlet, both over q = u0^2/2.  Any of the
 * three outputs may be NULL. */
typedef struct {
  int nx, ny, nz, kB, jm, top;
  double h, x0, d0, z0, zIn, pleat;
  double pin, rho_ref;        /* reference total pressure at the inlet, mean density on layer jb */
} abx_field3d_info;
int abx_sim_field3d(abx_sim *s, float *spd, float *pst, float *loss, abx_field3d_info *info);

/* The cut planes of evaluate (src/engine.js:662-680): out holds planInlet
 * (speed, ua = ux/u0, ub = uz/u0; nx*nz floats each, index i*nz + k), planLow
 * (same layout) and lon (speed, ua = uz/u0, ub = uy/u0; nz*ny floats each,
 * index k*ny + j): 6*nx*nz + 3*nz*ny floats. */
typedef struct {
  int ic, jc, jlow, n1, n2, lon_n1, lon_n2;
  double depth_inlet, depth_low, x_lon;
} abx_planes_info;
int abx_sim_planes(abx_sim *s, float *out, abx_planes_info *info);

/* streamlines (src/engine.js:721-758) traced on the device, one warp per
 * seed: pts (3 floats per point, model coordinates), spd (|u|/u0 per point),
 * off (n_lines + 1 prefix counts).  With capacities too small (e.g. 0) the
 * counts are still reported and ABX_ERR_INVALID_ARGUMENT is returned.  A line
 * keeps at most ABX_MAX_LINE_POINTS points and at most max_seeds + 1 seeds are
 * traced, so cap_points = (max_seeds + 1) * ABX_MAX_LINE_POINTS and
 * cap_lines = max_seeds + 2 always suffice (one call, one trace). */
#define ABX_MAX_LINE_POINTS 2001
typedef struct {
  int seeds_opening, seeds_traced, n_lines, n_points;
} abx_lines_info;
int abx_sim_streamlines(abx_sim *s, int max_seeds, float *pts, float *spd, uint32_t *off, size_t cap_points,
                        size_t cap_lines, abx_lines_info *info);

/* evaluate() (src/engine.js:632-691) on the device: filter map at layer jm,
 * gamma, gamma core, lowCore, highCore, reverse, maxToMean and zeta, with
 * float64 sums.  fmap (nx*nz floats, w/mean or NaN) and hist (3 doubles
 * [step, gamma, massRatio] per progress check, hist_cap rows) may be NULL. */
int abx_sim_evaluate(abx_sim *s, abx_metrics *m, float *fmap, double *hist, int hist_cap, int *nhist);

/* simulate(g, p, onProgress, ns) in one call (src/engine.js:341-358):
 * setupSim, the step loop and evaluate. */
int abx_simulate(abx_geom *g, const abx_run_params *p, const float *ns, abx_progress_fn cb, void *user,
                 abx_metrics *m, float *fmap, double *hist, int hist_cap, int *nhist);

/* Accounting of a simulation handle since its last reset (no reference
 * counterpart; used for roofline and end-to-end figures).  Device times are
 * measured with CUDA events on the handle's stream while timing is enabled;
 * counters are kept always. */
typedef struct {
  double step_ms;                 /* device time of all step-kernel launches */
  int64_t step_launches;
  double step_ms_plain;           /* ... of the launches that do not accumulate averages */
  int64_t step_launches_plain;
  double run_ms;                  /* device time of abx_sim_run calls */
  double eval_ms;                 /* device time of abx_sim_evaluate calls */
  int64_t cell_updates;           /* fluid-cell updates done (NF per step) */
  int64_t kernel_launches;        /* kernels launched by this handle */
  int64_t h2d_bytes, d2h_bytes;   /* bytes copied host->device / device->host by this handle */
} abx_sim_timing;
int abx_sim_set_timing(abx_sim *s, int enabled);
int abx_sim_get_timing(const abx_sim *s, abx_sim_timing *out);

/* voxelize() without any device allocation.  No counterpart in the reference.
 *
 * For callers that cannot allocate GPU memory themselves: a host application
 * whose memory pool owns every device byte (a framework allocator, a fixed
 * budget, a process that must not call cudaMalloc while other work is in
 * flight).  They pass their own device buffers for the input and the output,
 * and the call uses no cudaMalloc, cudaFree or other allocating routine.
 *
 * The parity voxelizer of src/engine.js:45-93 on the grid nx x ny x nz with
 * cell size h and the given origin: d_tris holds nfloats floats of
 * local-frame triangles (9 per triangle) in device memory, d_vox receives
 * nx*ny*nz bytes (index (i*ny + j)*nz + k, 1 = inside) in device memory.
 * The result is bit-identical to the voxel grid abx_prepare builds (the fine
 * grid of abx_geom_get_fine when called with 3*nx, 3*ny, 3*nz and h/3).
 *
 * Its scratch is a fixed 32 MiB array inside the library, held by every GPU
 * that loads it until the process exits.  Grids and meshes needing more
 * scratch are rejected with ABX_ERR_INVALID_ARGUMENT and a message giving the
 * size.  The first call on a device looks up that array's device address
 * (cudaGetSymbolAddress, with the device current); make that first call
 * before any stream capture.  The address is looked up again when the
 * device's context has changed since (after a cudaDeviceReset the library
 * is loaded anew at another address) and after a call that failed with a
 * CUDA error; such a call, too, should come before any stream capture.
 * The call makes the current device's primary context current (cudaSetDevice).
 * All calls share the one array and it keeps the
 * previous call's contents, so calls that overlap on the GPU (other streams,
 * other threads) race: issue them one after another.  stream may be NULL. */
int abx_voxelize_static(const float *d_tris, size_t nfloats, const double origin[3], double h, int nx, int ny, int nz,
                        uint8_t *d_vox, void *stream);

/* ======================================================================
 * Learned warm start and windowed convergence.  No counterpart in the
 * reference: engine.js always starts from f = w_i (src/engine.js:261) and
 * runs the fixed steps/avg schedule.
 *
 * The network is a 3-D convolutional encoder-decoder on an R^3 resampling
 * of the grid (levels L, channels base << l).  Input: fluid / inlet /
 * outlet / filter fraction of each voxel's footprint, wall distance, K,
 * the grid extent (and optionally the voxel's coordinates); output: the time-averaged u / u0 and (rho - 1)/(5 u0^2).
 * Training, inference, the resampling and the equilibrium initialisation
 * all run in the library's CUDA kernels on the network's device.
 * ====================================================================== */
typedef struct abx_net abx_net;

typedef struct {
  int res;                  /* R, a power of two >= 8, divisible by 2^(levels-1) */
  int base;                 /* channels of level 0 (a multiple of 8) */
  int levels;               /* encoder levels, 1..6 */
  int device;
  unsigned long long seed;  /* weight initialisation */
  int coords;               /* nonzero: three more input channels, the voxel's coordinates / R */
} abx_net_params;

typedef struct {
  int res, base, levels, in_channels, out_channels, n_samples;
  long long n_params;
  int tensor_cores;         /* 1: convolutions of up to 128 channels run on the tensor cores (tcgen05, bf16
                               operands, float32 accumulation); 0: all on the float32 kernels */
} abx_net_info;

int abx_net_create(const abx_net_params *p, abx_net **out);
/* Convolutions on the tensor cores (on; where the GPU has tcgen05 tensor cores) or all on the
 * float32 kernels (off).  A new network starts on the tensor cores where the GPU has them, unless
 * the environment sets ABX_NN_TC=0.  No counterpart in the reference. */
int abx_net_set_tensor_cores(abx_net *n, int on);
void abx_net_free(abx_net *n);
int abx_net_get_info(const abx_net *n, abx_net_info *out);
/* All weights and biases, n_params floats (layer by layer, weights
 * [cout][cin][3][3][3] then biases). */
int abx_net_get_weights(abx_net *n, float *w);
int abx_net_set_weights(abx_net *n, const float *w);

/* Training set, kept on the device: adds the features of s's geometry and K
 * and, as the target, s's current time averages (after abx_sim_run). */
int abx_net_add_sample(abx_net *n, abx_sim *s);
int abx_net_clear_samples(abx_net *n);
/* Read back stored sample i: x (in_channels*R^3), t (4*R^3), m (R^3); any may be NULL. */
int abx_net_get_sample(abx_net *n, int i, float *x, float *t, float *m);

typedef struct {
  int first, count;         /* samples [first, first+count) */
  int epochs, batch;
  double lr, lr_min;        /* Adam; rate decays from lr to lr_min (cosine) over the call, with a linear
                               warm-up over the network's first 100 updates */
  unsigned long long seed;  /* shuffling and mirror augmentation */
  int flip;                 /* nonzero: mirror half the samples along x */
} abx_train_params;
/* epoch_loss: `epochs` doubles (mean weighted MSE per epoch), may be NULL. */
int abx_net_train(abx_net *n, const abx_train_params *p, double *epoch_loss);
int abx_net_eval_loss(abx_net *n, int first, int count, double *loss);

/* One forward (and backward) pass on caller device buffers, for checks:
 * d_x (B*in_channels*R^3), d_t (B*4*R^3), d_m (B*R^3); writes the prediction
 * to d_pred (B*4*R^3) and, when d_grad is not NULL, the gradient of
 * loss = scale * sum m (pred - t)^2 w.r.t. the parameters to d_grad. */
int abx_net_forward_backward(abx_net *n, const float *d_x, const float *d_t, const float *d_m, int B, double scale,
                             float *d_pred, float *d_grad, double *loss);

/* Network input for s's geometry (in_channels*R^3 floats, host) and the
 * prediction (4*R^3, host); either may be NULL. */
int abx_net_predict(abx_net *n, abx_sim *s, float *features, float *pred);

/* Warm start: f = feq(rho, u) of the prediction, interpolated to every fluid
 * cell (weighted by voxel fluid fraction, |u| <= 0.2, 0.9 <= rho <= 1.1);
 * averages and step count cleared. */
int abx_sim_warm_start(abx_sim *s, abx_net *n);

/* Stop rules of the convergence run. */
#define ABX_RULE_CHANGE 0   /* the running average's gamma core and zeta moved less than tol over the last window */
#define ABX_RULE_STDERR 1   /* batch means: the standard error of gamma core and zeta, estimated from the
                               scatter of the windows' own averages (at least min_windows of them), is at most
                               tol / 2 of the running average's value */

typedef struct {
  int settle;               /* steps before averaging starts */
  int window;               /* steps between checks of the running average */
  int min_avg;              /* averaged steps before the stop rule may fire */
  int max_steps;            /* give up after this many steps (settle included) */
  double tol;               /* relative tolerance of the stop rule */
  int rule;                 /* ABX_RULE_CHANGE or ABX_RULE_STDERR */
  int min_windows;          /* ABX_RULE_STDERR: windows before the standard error counts (>= 2) */
} abx_converge_params;

typedef struct {
  abx_metrics metrics;      /* evaluate() of the running average at the stop */
  int steps, windows, converged;
  double change;            /* ABX_RULE_CHANGE: last window's relative change of the running average's KPIs;
                               ABX_RULE_STDERR: the larger relative standard error of gamma core and zeta */
} abx_converge_result;

/* Convergence run from the current state: `settle` steps, then steps added to
 * a running average, evaluated every `window` steps, until the stop rule
 * (`rule`, see ABX_RULE_*) fires or max_steps.  Non-finite KPIs end the run
 * with ABX_ERR_UNSTABLE.  The standard-error rule keeps a copy of the running
 * sums (4 values per padded cell) on the device from its first call on. */
int abx_sim_converge(abx_sim *s, const abx_converge_params *p, abx_converge_result *r);

typedef struct {
  abx_converge_result run;  /* the windowed run (or the plain run after a fallback) */
  int fell_back;            /* 1: the warm-started run did not converge; re-run from f = w_i on the full schedule */
  int warm_steps;           /* steps of the warm-started attempt */
  double infer_ms;          /* features + network + equilibrium initialisation */
  double total_ms;          /* wall time of the whole call */
} abx_warm_result;

/* Warm start, windowed run, and the fallback: when the warm-started run does
 * not converge within max_steps (or goes unstable) the simulation is reset to
 * f = w_i and runs the reference's steps/avg schedule (abx_sim_run). */
int abx_sim_solve_warm(abx_sim *s, abx_net *n, const abx_converge_params *p, abx_warm_result *r);

/* ======================================================================
 * Batched variants: many simulations of different airboxes (uneven sizes,
 * their own K / aniso / u / tau) advanced together, one kernel launch per
 * LBM step over a tile list covering every variant, the steps captured in
 * CUDA graphs.  The reference batches only variants sharing one geometry
 * (GpuSim, src/engine.js:495-545, one lbm_step dispatch over B copies);
 * here the geometries differ too.  Storage: float32, float16 or bfloat16;
 * all variants share steps / avg / every and the storage.
 * ====================================================================== */
typedef struct abx_batch abx_batch;

int abx_batch_create(abx_geom *const *geoms, const abx_run_params *params, int n, abx_batch **out);
void abx_batch_free(abx_batch *b);

/* Variant i as a simulation handle owned by the batch (do not free it):
 * abx_sim_evaluate / abx_sim_get_acc / abx_sim_get_f read its state. */
int abx_batch_sim(abx_batch *b, int i, abx_sim **out);

/* Block shape of the batched step kernel: shape 0..2 (segments per warp 1/1/2,
 * registers sized for 4/3/2 resident blocks per SM) and the grid (>= the
 * number of tiles: one tile per block; fewer: blocks loop over the tiles). */
typedef struct {
  int shape, spw, min_blocks;
  unsigned grid, ntiles;
  double ms_per_step;            /* of the chosen candidate, from the tuning run */
  double group_bytes;            /* chosen group budget (0: no limit) */
  int n_groups;
  int n_candidates;
  int cand_shape[48];
  unsigned cand_grid[48];
  double cand_group_bytes[48];
  int cand_groups[48];
  double cand_ms[48];            /* time per LBM step of every candidate tried */
} abx_batch_tuning;

/* Variants run in groups of consecutive variants whose state fits
 * group_bytes (at most 96 per group; 0: no byte limit).  A chunk of steps
 * runs group by group, each group for the whole chunk, so that a group that
 * fits in L2 stays there across its steps. */
int abx_batch_set_grouping(abx_batch *b, double group_bytes);

/* Autotuner: times a few steps of every candidate group budget x shape x
 * grid on this batch's own domains, keeps the fastest, and resets every
 * variant to f = w_i (the timed steps are discarded). */
int abx_batch_tune(abx_batch *b, abx_batch_tuning *out);
int abx_batch_set_shape(abx_batch *b, int shape, unsigned grid);

/* Every variant back to f = w_i (averages and history cleared). */
int abx_batch_reset(abx_batch *b);

/* simulate()'s step loop (src/engine.js:341-358) for all variants at once:
 * averaging window, a progress probe of every variant at each multiple of
 * `every`.  A variant that goes unstable stops stepping (its evaluate then
 * reports nothing new); the others go on.  status (n ints, may be NULL)
 * receives 0 or the step where variant i went unstable. */
int abx_batch_run(abx_batch *b, int *status);

typedef struct {
  int n;                          /* variants */
  long long cells;                /* fluid cells over all variants */
  long long state_bytes;
  unsigned ntiles1, ntiles2;      /* tiles of 8 and 16 segments */
  int shape;
  unsigned grid;
  double run_ms;                  /* device time of the last abx_batch_run */
  long long kernel_launches;      /* of the last abx_batch_run */
  int n_groups;
  double group_bytes;
} abx_batch_info;
int abx_batch_get_info(const abx_batch *b, abx_batch_info *out);

#ifdef __cplusplus
}
#endif
#endif /* AIRBOX_H */
