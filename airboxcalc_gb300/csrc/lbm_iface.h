// lbm_iface.h - argument blocks and launchers shared by the host code
// (api.cpp) and the kernel translation units.  Plain C++, no CUDA headers
// beyond the runtime's stream type.
#pragma once
#include <cuda_runtime_api.h>
#include <cuda_bf16.h>
#include <vector_types.h>
#include <stdint.h>

#include "airbox.h"

namespace abx {

struct StepArgs {
  void *f;                 // populations A[19][Np], storage type of the run
  const uint32_t *mask;    // Np cell mask words
  const uint2 *seg;        // fluid segments: {base index, bit l set if cell base + l is fluid}
  uint32_t nseg;
  int64_t Np;
  void *acc;               // averages [4][Np] (float, or double for the float64 run)
  const float *ns;         // partial bounce-back per padded cell, or null
  const int *status;       // nonzero once the run went unstable: steps become no-ops
  unsigned long long *diag;  // 8 words: where a pipeline wait gave up (TMA kernel), or null
  long long off[19];       // pull offset of direction q in the padded layout
  double u0, tau0, sig, aniso, cs2s;
  // the same five rounded to float32 on the host: the float32 collision reads them straight from the
  // parameter bank instead of converting the doubles in every warp (a slow pipe on this GPU)
  float u0f, tau0f, sigf, anisof, cs2sf;
};

struct StateArgs {
  void *f;
  const uint32_t *mask;
  int64_t Np;
  void *acc;
  const int64_t *cells;    // padded index of fluid cell a (the reference's compact order)
  int64_t ncells;
  int *status;
  int form;                // 0: "out" form (even steps done), 1: "in" form
  long long off[19];
};

struct ProbeArgs {
  const int64_t *plist;    // padded indices: layer jm cells, then layer top+1 cells
  int nM, nT;
  int step, slot;
  double Ain, u0;
  double *hist;            // 4 doubles per slot: step, gamma, massRatio, outflow
  float *vy;               // nM + nT floats: the probed -u_y values of one check
  double *part;            // 2 doubles per block of the first pass
  int nblocks;             // blocks of the first pass
};
constexpr int kProbeThreads = 256;

struct EvalArgs {
  int nx, ny, nz;
  int64_t nzp, kpad;
  int jm, jb, nacc;
  double u0;
  const uint8_t *opening;  // nx*ny
  const float *ns;         // padded, or null
  float *fmap;             // nx*nz, or null
  double *out;             // 13 doubles
  const void *base;        // null, or running sums to subtract (same type as acc): the averages of the steps since
  int base_nacc;           // that snapshot, which held base_nacc steps
};

// TMA descriptors of one simulation: five CUtensorMap (made by make_tma,
// passed to the kernels by value) and the persistent grid size.
struct alignas(64) TmaBlob {
  unsigned char maps[5 * 128];
  uint32_t ntiles = 0, grid = 0;
  bool ready = false;
};
// Encode the tensor maps of a simulation's arrays and size the persistent
// grid; returns cudaErrorNotSupported when TMA cannot be used for `storage`.
// free_tma marks the descriptors unused.
cudaError_t make_tma(int storage, const StepArgs &a, TmaBlob *out);
void free_tma(TmaBlob *b);

// Work lists of the vectorised step kernel (lbm_vec.cuh), built per geometry and block width V (cells per
// thread, consecutive along k): interior blocks - V fluid cells whose 18 pull neighbours are all fluid, all of
// class bulk or all of class filter - and every other fluid cell in a dense list (one per lane).
struct VecArgs {
  const uint32_t *blk;     // padded index of the first cell of every interior block: bulk blocks, then filter blocks
  uint32_t n_bulk, n_filter;
  const uint32_t *bcell;   // padded index of every fluid cell outside the interior blocks, rising
  uint32_t nbcell;
};
// The lists of a geometry for block width V (2, 4 or 8): call with blk == bcell == nullptr to get the three
// counts (counts[0..2] = bulk blocks, filter blocks, boundary cells), then with arrays of those sizes.
// block_counts / offsets: scratch of prep_compact_blocks(nseg * 32) and + 1 entries.
cudaError_t prep_vec_lists(const uint2 *seg, uint32_t nseg, const uint32_t *mask, int V, uint32_t *blk,
                           uint32_t *bcell, uint32_t *block_counts, unsigned long long *offsets,
                           unsigned long long *counts, cudaStream_t st);
// Shared-memory limits of the vectorised kernels for a storage and V (call once, outside stream capture).
cudaError_t prepare_step_vec(int storage, int V);
// One step through the vectorised kernel (lbm_fast.cu; float32, float16 and bfloat16 with V = 2 or 4; no partial
// bounce-back field).
cudaError_t launch_step_vec(int storage, int V, bool odd, bool acc, const StepArgs &a, const VecArgs &v,
                            cudaStream_t st);

// Launchers (defined in lbm_fast.cu / lbm_exact.cu).  storage: abx_storage
// value; tma (may be null) selects the TMA-pipelined kernel.
cudaError_t launch_step(int storage, bool odd, bool acc, bool has_ns, const StepArgs &a, const TmaBlob *tma,
                        cudaStream_t st);
cudaError_t launch_init(int storage, const StateArgs &a, cudaStream_t st);
cudaError_t launch_get_f(int storage, const StateArgs &a, float *out, cudaStream_t st);
cudaError_t launch_set_f(int storage, const StateArgs &a, const float *in, cudaStream_t st);
cudaError_t launch_get_acc(int storage, const StateArgs &a, float *out, int nacc, cudaStream_t st);
cudaError_t launch_probe(int storage, const StateArgs &a, const ProbeArgs &p, cudaStream_t st);
cudaError_t launch_evaluate(int storage, const StateArgs &a, const EvalArgs &e, cudaStream_t st);
// step kernels of the float32-collision storages (lbm_fast.cu)
cudaError_t launch_step_fast(int storage, bool odd, bool acc, bool has_ns, const StepArgs &a, const TmaBlob *tma,
                             cudaStream_t st);

// One step of many domains in one launch (lbm_fast.cu; float32, float16, bfloat16 storage).  Up to
// kBatchChunk variants per launch, their StepArgs passed by value (kernel parameter); tiles[t] = {variant,
// first segment} of 8*spw segments, variants vbase.. of the chunk in tiles [t0, t1); grid blocks loop over
// the tiles (grid >= t1 - t0: one tile per block).  shape (0..kBatchShapes-1) selects segments per warp
// (spw) and the resident blocks per SM the kernel's registers are sized for.
constexpr int kBatchChunk = 96;
struct BatchParams {
  StepArgs v[kBatchChunk];
  uint32_t vbase;
};
static_assert(sizeof(BatchParams) <= 32764, "kernel parameter limit");
constexpr int kBatchShapes = 3;
int batch_shape_spw(int shape);
int batch_shape_minblocks(int shape);
cudaError_t launch_step_batch(int storage, bool odd, bool acc, int shape, const BatchParams &P, const uint2 *tiles,
                              uint32_t t0, uint32_t t1, uint32_t grid, cudaStream_t st);

// Mask construction (lbm_exact.cu): class bytes (0 not fluid, 1 bulk, 2 inlet,
// 3 outlet, 4 filter; index (i*ny+j)*nz+k) -> padded mask words, cell (i,j,k)
// at padded index (i*ny+j)*nzp + k + kpad.
cudaError_t launch_build_mask(const uint8_t *cls, int nx, int ny, int nz, int64_t nzp, int64_t kpad, uint32_t *mask,
                              cudaStream_t st);
// Scatter compact-order values (ns) to the padded layout.
cudaError_t launch_scatter_f32(const float *src, const int64_t *cells, int64_t n, float *dst, cudaStream_t st);

// Voxelizer (voxelize.cu), bit-exact with src/engine.js:45-93 and the
// 27->1 downsample of :127-135.
struct VoxJob {
  const float *tris;       // device, local-frame triangles, 9 floats each
  int64_t ntri;
  double origin[3];
  double hf;               // fine cell size h/3
  int nx, ny, nz;          // coarse grid
  int kf;                  // fine slice index for the opening search
};
struct VoxOut {
  uint8_t *solid;          // device, nx*ny*nz
  uint8_t *slice;          // device, nxf*nyf: 1 where fine voxel (i,j,kf) is set
  uint8_t *fine;           // device, nxf*nyf*nzf or null (tests)
  int64_t launches = 0;    // kernels launched (filled in)
  int64_t d2h_bytes = 0;   // bytes read back to the host (filled in)
};
// Runs the whole voxelizer; scratch is allocated and freed inside.
cudaError_t run_voxelizer(const VoxJob &job, VoxOut &out, cudaStream_t st);
// The voxelizer on a caller-given grid (nx, ny, nz at cell size h, i.e. the
// reference's voxelize(T, origin, nx, ny, nz, h)) writing the voxel grid to
// d_vox, with its scratch in a fixed device array instead of allocations.
// Returns an abx_status value; msg receives the text of a failure.
int voxelize_static(const float *d_tris, size_t nfloats, const double origin[3], double h, int nx, int ny, int nz,
                    uint8_t *d_vox, cudaStream_t st, char *msg, size_t msg_len);

// ---------------------------------------------------------------- prepare stages (prepare.cu)
struct MaskArgs {
  int nx, ny, nz;
  int64_t N;
  uint8_t *solid, *fluid, *outlet;   // N bytes each, index (i*ny + j)*nz + k
  const uint8_t *opening;            // nx*ny
  const uint8_t *close_row;          // ny: rows made solid (beyond the model's depth)
  int kw0, top;
};
// duct and closing rows into solid, fluid/outlet cleared, the opening's k = 0 cells seeded
cudaError_t prep_duct(const MaskArgs &a, cudaStream_t st);
// one round of line sweeps along k, j, i; *changed |= 1 when a cell joined the air
cudaError_t prep_flood_round(const MaskArgs &a, int *changed, cudaStream_t st);
cudaError_t prep_leak(const MaskArgs &a, int *leak, cudaStream_t st);
// jpt >= 0: lid plenum from row jpt (counts[0] += cells added) with a round outlet of radius^2 r2 around
// (cx, cz) at row jpt; jpt < 0: row `top` is the outlet.  counts[1] += outlet cells
cudaError_t prep_outlet(const MaskArgs &a, int jpt, const float *xc, const float *zc, double cx, double cz, double r2,
                        unsigned long long *counts, cudaStream_t st);
// counts[0..2] += air cells, air on layer jm, air on row top
cudaError_t prep_counts(const MaskArgs &a, int jm, unsigned long long *counts, cudaStream_t st);
// setupSim classes (0 no air, 1 bulk, 2 inlet, 3 outlet, 4 filter) into cls; *ain += inlet cells
cudaError_t prep_classes(const MaskArgs &a, const uint8_t *filt_row, uint8_t *cls, unsigned long long *ain,
                         cudaStream_t st);
// air bits per column (W words each) into bits; count[t] += 32-cell runs holding air at column shift t
cudaError_t prep_kpad_counts(const MaskArgs &a, int W, uint32_t *bits, unsigned long long *count, cudaStream_t st);
// ordered compactions: the padded index of every air cell, and the {base, lanes} of every 32-cell run
// holding air (out may be null: offsets[blocks] then receives the count only); block_counts and offsets
// hold prep_compact_blocks(items) and prep_compact_blocks(items) + 1 entries
int64_t prep_compact_blocks(int64_t n);
cudaError_t prep_cells(const MaskArgs &a, int64_t nzp, int64_t kpad, int64_t *cells, uint32_t *block_counts,
                       unsigned long long *offsets, cudaStream_t st);
cudaError_t prep_segments(const MaskArgs &a, int W, const uint32_t *bits, int64_t nzp, int64_t kpad, uint2 *seg,
                          uint32_t *block_counts, unsigned long long *offsets, cudaStream_t st);
// set the interior flag (kSegInterior) of the segments whose fluid cells all carry the mask word kMaskInterior
cudaError_t prep_seg_interior(uint2 *seg, uint32_t nseg, const uint32_t *mask, cudaStream_t st);

// Opening search on the fine slice kf (src/engine.js:141-171), prepare.cu.  Cell c = i*nyf + j.
struct OpenArgs {
  const uint8_t *slice;    // nxf*nyf: 1 where the fine voxel (i, j, kf) is material
  int nxf, nyf;
  uint8_t *outside;        // empty cells 4-connected to the slice's border
  int32_t *label;          // hole cells: the lowest index of their component (its root); -1 elsewhere
  uint32_t *size;          // at a root: the cells of its component
  uint32_t *claim;         // breadth-first search of the click case
  double origin0, origin1, hf;
};
struct OpenOut {
  unsigned long long best;   // (size << 32) | (0xFFFFFFFF - root) of the largest kept component (first of equals)
  uint32_t n_kept;           // components above 25 mm^2
  uint32_t n_open;           // coarse opening cells
};
// outside seeded on the border, labels and sizes cleared, claims freed
cudaError_t open_init(const OpenArgs &a, cudaStream_t st);
// one round of line sweeps along j and i; *changed |= 1 when a cell joined the outside
cudaError_t open_outside_round(const OpenArgs &a, int *changed, cudaStream_t st);
// holes (empty, not outside, cell centre below the seal) labelled with their own index
cudaError_t open_holes(const OpenArgs &a, cudaStream_t st);
// one round of line sweeps carrying the lowest label along runs of hole cells
cudaError_t open_label_round(const OpenArgs &a, int *changed, cudaStream_t st);
// component sizes, then the kept components ({root, size} into kept, at most cap) and out->best / n_kept
cudaError_t open_components(const OpenArgs &a, OpenOut *out, uint2 *kept, uint32_t cap, cudaStream_t st);
// click: for each of the n kept components, the reference's breadth-first order of its cells (into order at
// offs[b]) and the smallest squared distance to (cx, cy) over every third cell of that order (bits of the
// double, into dmin[b])
cudaError_t open_bfs_click(const OpenArgs &a, const uint2 *kept, const int64_t *offs, int n, int32_t *order,
                           double cx, double cy, unsigned long long *dmin, cudaStream_t st);
// the coarse opening: cells (nx*ny) holding at least 5 of their 9 fine cells in the component of `root`;
// sel (nx*ny counters) must be zero; out->n_open += opening cells
cudaError_t open_select(const OpenArgs &a, uint32_t root, int nx, int ny, uint32_t *sel, uint8_t *opening,
                        OpenOut *out, cudaStream_t st);

// ---------------------------------------------------------------- post-processing (postproc.cu)
struct PostArgs {
  int nx, ny, nz;
  int64_t nzp, kpad, Np;
  const uint32_t *mask;      // padded; nonzero: fluid
  const float *ns;           // padded partial bounce-back, or null (cells with ns > 0.5 count as no air)
  const uint8_t *opening;    // nx*ny
  const void *acc;           // running sums [4][Np]
  int acc_double;            // sums in float64 (the float64 run)
  double dn;                 // averaged steps (>= 1)
  double u0;
  const float *avg;          // [4][Np] averages as float32 (post_average), read by the kernels below
};
constexpr int kMaxLinePoints = ABX_MAX_LINE_POINTS;   // points one streamline can keep (6000 steps, every 3rd, plus the last)
// the float32 averages sum / nacc of every padded cell into avg (4 * Np floats)
cudaError_t post_average(const PostArgs &a, float *avg, cudaStream_t st);
// field3d: d_scal receives pin and rhoRef; spd/pst/loss (nx*ny*nz floats, may be null)
cudaError_t post_field3d(const PostArgs &a, int kB, int jb, double *d_scal, float *spd, float *pst, float *loss,
                         cudaStream_t st);
// cut planes: out = planInlet (speed, ua, ub; nx*nz each), planLow (same), lon (speed, ua, ub; nz*ny each)
cudaError_t post_planes(const PostArgs &a, int ic, int jc, int jlow, float *out, cudaStream_t st);
// streamlines: seeds (3 doubles each, grid-cell coordinates) -> pts (4 doubles per point, kMaxLinePoints
// per seed) and count (points per seed)
cudaError_t post_streamlines(const PostArgs &a, const double *seeds, int nseeds, int top, double *pts, int *count,
                             cudaStream_t st);

// ---------------------------------------------------------------- warm start
// The padded grid as the resampling kernels see it (warmstart.cu).
struct GridDesc {
  int nx, ny, nz;
  int64_t nzp, kpad, Np;
  const uint32_t *mask;    // nonzero: fluid cell; class in bits 19..20
};
// Network input (9 x R^3 floats), with two R^3 int scratch arrays for the jump flood.
cudaError_t ws_features(const GridDesc &g, int R, float K, float *out, int *seed_a, int *seed_b, cudaStream_t st);
// Voxel coordinates (3 x R^3: (a + 0.5) / R along x, y, z).
cudaError_t ws_coords(int R, float *out, cudaStream_t st);
// Training target (4 x R^3) and loss weight (R^3) from a run's averages.
cudaError_t ws_targets(const GridDesc &g, int storage, const void *acc, int nacc, double u0, int R, float *t, float *m,
                       cudaStream_t st);
// Equilibrium populations of the predicted field (4 x R^3) on every fluid cell, "out" form.
cudaError_t ws_apply(int storage, const StateArgs &a, const GridDesc &g, const float *pred, const float *fluid, int R,
                     double u0, cudaStream_t st);
// Mirror one sample's C x R^3 block along x, negating channel neg (< 0: none).
cudaError_t ws_flip_x(float *t, int C, int R, int neg, cudaStream_t st);

// Layer kernels of the network (nn.cu), float32 [B][C][D][H][W].
cudaError_t nn_conv3d(const float *x, const float *w, const float *b, float *y, int B, int Cin, int Cout, int D,
                      int H, int W, int s, int relu, int accum, cudaStream_t st);
// ReLU adjoint applied to dy in place (relu != 0), then dx (+)= data gradient (dx may be null), dw, db;
// part: scratch of at least nn_wgrad_scratch_floats(Cin, Cout, output voxels) floats.
cudaError_t nn_conv3d_backward(const float *x, const float *w, const float *y, float *dy, float *dx, float *dw,
                               float *db, float *part, int64_t part_floats, int B, int Cin, int Cout, int D, int H,
                               int W, int s, int relu, int accum_dx, cudaStream_t st);
int64_t nn_wgrad_scratch_floats(int Cin, int Cout, int Vo);
// The same convolutions on the tensor cores (nn_tc.cu; tcgen05, bf16 operands, float32 accumulation and float32
// tensors in and out).  Scratch: a channels-last bf16 copy of a layer's input, its bf16 weight slices, three
// shifted channels-first copies of the input and a channels-first copy of the output gradient (weight gradient),
// and the weight-gradient partial sums; err receives 1 if a kernel gave up waiting.
struct TcScratch {
  __nv_bfloat16 *cl = nullptr, *w = nullptr, *xs = nullptr, *dyc = nullptr;
  float *part = nullptr;
  int64_t cl_elems = 0, w_elems = 0, xs_elems = 0, dyc_elems = 0, part_floats = 0;
  int *err = nullptr;
};
struct TcNeed {
  int64_t cl_elems = 0, w_elems = 0, xs_elems = 0, dyc_elems = 0, part_floats = 0;
};
// true on a GPU whose tensor cores these kernels drive (compute capability 10.x)
bool nn_tc_available();
// grow `n` to what one layer (B samples, Cin -> Cout, D^3 input, stride s) needs
void nn_tc_need(int B, int Cin, int Cout, int D, int s, TcNeed *n);
int tc_wgrad_splits();
cudaError_t nn_tc_conv3d(const float *x, const float *w, const float *b, float *y, int B, int Cin, int Cout, int D, int H,
                         int W, int s, int relu, int accum, const TcScratch &sc, cudaStream_t st);
// as nn_conv3d_backward; part / part_floats: the float32 weight-gradient scratch for the layers whose weight
// gradient runs on the float32 kernels (output planes of fewer than 64 voxels)
cudaError_t nn_tc_conv3d_backward(const float *x, const float *w, const float *y, float *dy, float *dx, float *dw,
                                  float *db, float *part, int64_t part_floats, int B, int Cin, int Cout, int D, int H,
                                  int W, int s, int relu, int accum_dx, const TcScratch &sc, cudaStream_t st);
cudaError_t nn_upsample2(const float *x, float *y, int64_t BC, int D, int H, int W, cudaStream_t st);
cudaError_t nn_upsample2_backward(const float *dy, float *dx, int64_t BC, int D, int H, int W, int accum,
                                  cudaStream_t st);
cudaError_t nn_axpy(float *y, const float *x, float a, int64_t n, cudaStream_t st);
cudaError_t nn_mse(const float *pred, const float *target, const float *mask, float *grad, double *part, int nparts,
                   int B, int C, int64_t V, double scale, cudaStream_t st);
cudaError_t nn_adam(float *p, const float *g, float *m, float *v, int64_t n, float lr, float b1, float b2, float eps,
                    int t, cudaStream_t st);

}  // namespace abx
