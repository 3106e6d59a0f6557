// lbm_kernels.cuh - step, probe, state and evaluate kernels, templated on the
// population storage.  Included by lbm_fast.cu (float32 / float16 / bfloat16
// storage, float32 collision) and lbm_exact.cu (compiled with -fmad=false:
// float32 storage with cpuStep's float64 collision, and a float64 run).
//
// Memory layout in HBM (one simulation):
//   populations  A[q][p], q = 0..18, p = (i*ny + j)*nzp + k + kpad; kpad in [0,32) is
//                chosen per geometry so that the columns' fluid runs fill whole
//                32-cell segments, nzp = nz + kpad rounded up to 32
//                one array only: A-A streaming updates it in place
//   mask         uint32 per padded cell (see d3q19.cuh)
//   averages     acc[c][p], c = ux, uy, uz, rho (float32; float64 for the float64 run)
//   segments     {base, lane mask} of every 32-cell run along k holding a fluid cell
//
// A-A streaming.  The reference pulls f_q(x) = f*_q(x - c_q) from a second
// array (src/engine.js:272-276, bounce-back from the cell's own opposite
// population when the neighbour is not fluid).  Here one array holds the
// state in one of two forms:
//   "out" form (after an even number of steps): A[opp q][x] = f*_q(x)
//   "in"  form (after an odd  number of steps): A[q][x + c_q] = f*_q(x) when
//          x + c_q is fluid, else A[opp q][x] = f*_q(x) (already bounced back)
// An odd step reads out-form neighbours and writes in-form; an even step reads
// and writes only its own cell.  Every location a thread reads is written by
// that same thread only, so no step needs a second array.
#pragma once
#include <math.h>
#include <stdint.h>

#include "d3q19.cuh"
#include "lbm_iface.h"

namespace abx {

template <class L> __device__ __forceinline__ CollideParams<L> make_params(const StepArgs &a) {
  CollideParams<L> P;
  if constexpr (sizeof(L) == 4) {
    P.u0 = a.u0f; P.tau0 = a.tau0f; P.sig = a.sigf; P.aniso = a.anisof; P.cs2s = a.cs2sf;
  } else {
    P.u0 = (L)a.u0; P.tau0 = (L)a.tau0; P.sig = (L)a.sig; P.aniso = (L)a.aniso; P.cs2s = (L)a.cs2s;
  }
  return P;
}

// Tuning knobs (compile-time): minimum resident blocks per SM of the step
// kernel (0 = let the compiler choose the register count).
#ifndef ABX_STEP_MINBLOCKS
#define ABX_STEP_MINBLOCKS 4
#endif

// Segments per warp: with 2, a warp issues the loads of both of its segments
// before computing either (more bytes in flight per warp).
#ifndef ABX_STEP_SPW
#define ABX_STEP_SPW 1
#endif
constexpr int kStepSpw = ABX_STEP_SPW;

// One warp's share of a step: the fluid cells (lane masks) of SPW segments {base | flag, lane mask}.
template <int K, bool ODD, bool ACC, bool HAS_NS, int SPW, class Args>
__device__ __forceinline__ void step_cells(const Args &a, const uint2 (&sg)[SPW], const uint32_t lane) {
  using S = Store<K>;
  using T = typename S::T;
  using L = typename S::L;
  using Acc = typename S::Acc;
  T *f = (T *)a.f;
  const uint32_t Np = (uint32_t)a.Np;
  bool act[SPW];
  uint32_t p[SPW], m[SPW];
  L fi[SPW][19];
  Acc av[SPW][4];
#pragma unroll
  for (int j = 0; j < SPW; j++) {
    act[j] = (sg[j].y >> lane) & 1u;
    // 32-bit element indices: the host guarantees 19 * Np < 2^32
    p[j] = seg_base(sg[j]) + lane;
    // in flight together with the population loads below; known without a load in the interior segments of
    // an odd step, and of an even step for the float32 storage (the 16-bit even steps keep the plain load: they
    // have no register to spare for the branch)
    m[j] = act[j] ? (((ODD || K == kStoreF32) && (sg[j].x & kSegInterior)) ? kMaskInterior : a.mask[p[j]]) : 0u;
    if (!act[j]) continue;
    if (ODD) {
      // Pull from the neighbours first.  For a fluid cell x every x - c_q lies
      // inside the padded array (fluid never touches the grid faces), so the
      // loads are in bounds even where the neighbour is solid; those
      // directions are then bounced back from the cell's own slot.
#pragma unroll
      for (int q = 0; q < 19; q++)
        fi[j][q] = toc<K>(S::ldr(f + ((uint32_t)opp(q) * Np + p[j] - (uint32_t)a.off[q])), q);
    } else {
#pragma unroll
      for (int q = 0; q < 19; q++) fi[j][q] = toc<K>(S::ldr(f + ((uint32_t)q * Np + p[j])), q);
    }
    // running sums of the averages: loaded now, in flight with the populations
    if (ACC) {
      const Acc *acc = (const Acc *)a.acc;
      av[j][0] = acc[p[j]]; av[j][1] = acc[Np + p[j]]; av[j][2] = acc[2u * Np + p[j]]; av[j][3] = acc[3u * Np + p[j]];
    }
  }
#pragma unroll
  for (int j = 0; j < SPW; j++) {
    if (!act[j]) continue;
    if (ODD && m[j] != kMaskInterior) {
#pragma unroll
      for (int q = 1; q < 19; q++)
        if (!((m[j] >> q) & 1u)) fi[j][q] = toc<K>(S::ldr(f + ((uint32_t)q * Np + p[j])), q);
    }
    const uint32_t cls = (m[j] >> kClassShift) & 3u;
    L nsv = (L)0;
    if (HAS_NS) nsv = (L)a.ns[p[j]];
    L fo[19], ux, uy, uz, rho;
    if constexpr (sizeof(L) == 4)
      collide_fast<HAS_NS, S::kCollideShifted, S::kFastMath>(fi[j], cls, nsv, make_params<L>(a), fo, ux, uy, uz, rho);
    else collide<L, HAS_NS>(fi[j], cls, nsv, make_params<L>(a), fo, ux, uy, uz, rho);
    if (ODD && (sg[j].x & kSegInterior)) {
      // every neighbour is fluid: each population goes to the neighbour's slot (warp-uniform branch)
#pragma unroll
      for (int q = 0; q < 19; q++) S::str(f + ((uint32_t)q * Np + p[j] + (uint32_t)a.off[q]), fromc<K>(fo[q], q));
    } else {
#pragma unroll
      for (int q = 0; q < 19; q++) {
        uint32_t idx;
        if (ODD)
          idx = ((m[j] >> opp(q)) & 1u) ? (uint32_t)q * Np + p[j] + (uint32_t)a.off[q] : (uint32_t)opp(q) * Np + p[j];
        else idx = (uint32_t)opp(q) * Np + p[j];
        S::str(f + idx, fromc<K>(fo[q], q));
      }
    }
    if (ACC) {
      Acc *acc = (Acc *)a.acc;
      acc[p[j]] = (Acc)((L)av[j][0] + ux);
      acc[Np + p[j]] = (Acc)((L)av[j][1] + uy);
      acc[2u * Np + p[j]] = (Acc)((L)av[j][2] + uz);
      acc[3u * Np + p[j]] = (Acc)((L)av[j][3] + rho);
    }
  }
}

// One warp's share of a step: SPW segments starting at s0 of the domain described by `a`.
template <int K, bool ODD, bool ACC, bool HAS_NS, int SPW, class Args>
__device__ __forceinline__ void step_warp(const Args &a, const uint32_t s0, const uint32_t lane) {
  if (s0 >= a.nseg) return;
  // the run-state word changes only between launches: a plain load issued together with the segment's
  const int halted = a.status ? *a.status : 0;
  uint2 sg[SPW];
#pragma unroll
  for (int j = 0; j < SPW; j++) sg[j] = (s0 + j < a.nseg) ? a.seg[s0 + j] : make_uint2(0, 0);
  if (halted) return;
  step_cells<K, ODD, ACC, HAS_NS, SPW>(a, sg, lane);
}

// Traversal order: blocks run in rising index order, so a step ends with the last segments' lines in
// L2.  Odd steps walk the segments backwards: each step starts where the previous one ended and reads
// what is still in L2 (state up to about the L2's 129 MB stays on chip across steps).
#ifndef ABX_STEP_ALTERNATE
#define ABX_STEP_ALTERNATE 1
#endif

// Persistent form (default): a grid of resident blocks (SMs x ABX_STEP_MINBLOCKS) whose warps loop over the
// segments, so no warp slot idles between blocks (config3 float32: 1102 -> 1043 us per step); 0 launches one
// block per 8 segments.
#ifndef ABX_STEP_PERSIST
#define ABX_STEP_PERSIST 1
#endif

// Programmatic dependent launch between consecutive steps: a step kernel waits until the previous kernel of its
// stream has completed and its writes are visible before it touches memory, then lets the next kernel be
// launched as soon as all of its own blocks are running, so one step's launch overlaps the previous step's tail.
// Both are no-ops for a kernel launched without the programmatic-serialization attribute.
__device__ __forceinline__ void step_dependency_wait() {
  asm volatile("griddepcontrol.wait;" ::: "memory");
  asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}

template <int K, bool ODD, bool ACC, bool HAS_NS>
__global__ void __launch_bounds__(256, ABX_STEP_MINBLOCKS) aa_step_kernel(const StepArgs a) {
  step_dependency_wait();
#if ABX_STEP_PERSIST
  const uint32_t nw = gridDim.x * 8u;
  for (uint32_t s = blockIdx.x * 8u + (threadIdx.x >> 5); s < a.nseg; s += nw)
    step_warp<K, ODD, ACC, HAS_NS, 1>(a, (ABX_STEP_ALTERNATE && ODD) ? a.nseg - 1u - s : s, threadIdx.x & 31);
#else
  const uint32_t blk = (ABX_STEP_ALTERNATE && ODD) ? gridDim.x - 1u - blockIdx.x : blockIdx.x;
  step_warp<K, ODD, ACC, HAS_NS, kStepSpw>(a, (blk * 8u + (threadIdx.x >> 5)) * kStepSpw, threadIdx.x & 31);
#endif
}

// Blocks of the step kernel for nseg segments: one per 8*SPW segments, or (persistent form) the resident
// blocks of the device.
inline unsigned step_grid(uint32_t nseg) {
  const unsigned need = (nseg + 8u * kStepSpw - 1) / (8u * kStepSpw);
#if ABX_STEP_PERSIST
  static int nsm = 0;
  if (!nsm) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    if (nsm <= 0) nsm = 1;
  }
  const unsigned res = (unsigned)nsm * ABX_STEP_MINBLOCKS;
  return need < res ? need : res;
#else
  return need;
#endif
}

// One step of many domains in one launch.  tiles[t] = {variant, first segment}: a block takes 8*SPW
// consecutive segments of one variant; the blocks loop over tiles [t0, t1) (persistent when the grid is
// smaller).  The variants' arguments travel as one kernel parameter (constant bank, read with the tile's
// variant index), so the per-cell code is the single-domain kernel's.  SPW (segments per warp) and MINB
// (resident blocks per SM the registers are sized for) are the autotuner's knobs.
template <int K, bool ODD, bool ACC, int SPW, int MINB>
__global__ void __launch_bounds__(256, MINB)
    aa_step_batch_kernel(const __grid_constant__ BatchParams P, const uint2 *__restrict__ tiles, uint32_t t0,
                         uint32_t t1) {
  step_dependency_wait();
  const uint32_t n = t1 - t0;
  for (uint32_t i = blockIdx.x; i < n; i += gridDim.x) {
    const uint2 tile = tiles[t0 + ((ABX_STEP_ALTERNATE && ODD) ? n - 1u - i : i)];
    step_warp<K, ODD, ACC, false, SPW>(P.v[tile.x - P.vbase], tile.y + (threadIdx.x >> 5) * SPW, threadIdx.x & 31);
  }
}

// Post-collision populations f*_q(x) of the current state (either form).
template <int K>
__device__ __forceinline__ void read_post_all(const StateArgs &a, int64_t x, double (&f)[19]) {
  using T = typename Store<K>::T;
  const T *A = (const T *)a.f;
  const uint32_t m = a.mask[x];
#pragma unroll
  for (int q = 0; q < 19; q++) {
    const int o = opp(q);
    int64_t idx = (int64_t)o * a.Np + x;
    if (a.form && ((m >> o) & 1u)) idx = (int64_t)q * a.Np + x + a.off[q];
    f[q] = (double)Store<K>::ld(A + idx, weight<typename Store<K>::L>(q));
  }
}

// Set every fluid cell to w_q (valid in both forms) and clear the averages.
template <int K>
__global__ void init_state_kernel(const StateArgs a) {
  using S = Store<K>;
  using T = typename S::T;
  using L = typename S::L;
  using Acc = typename S::Acc;
  T *f = (T *)a.f;
  for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < a.Np; p += (int64_t)gridDim.x * blockDim.x) {
#pragma unroll
    for (int q = 0; q < 19; q++) S::st(f + (int64_t)q * a.Np + p, weight<L>(q), weight<L>(q));
    if (a.acc) {
      Acc *acc = (Acc *)a.acc;
      for (int c = 0; c < 4; c++) acc[(int64_t)c * a.Np + p] = (Acc)0;
    }
  }
}

// f in the reference's compact layout f[q*NF + a] from the device state.
template <int K>
__global__ void get_f_kernel(const StateArgs a, float *out) {
  for (int64_t n = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; n < a.ncells; n += (int64_t)gridDim.x * blockDim.x) {
    double f[19];
    read_post_all<K>(a, a.cells[n], f);
    for (int q = 0; q < 19; q++) out[(int64_t)q * a.ncells + n] = (float)f[q];
  }
}

// Device state in "out" form from f[q*NF + a].
template <int K>
__global__ void set_f_kernel(const StateArgs a, const float *in) {
  using S = Store<K>;
  using T = typename S::T;
  using L = typename S::L;
  T *f = (T *)a.f;
  for (int64_t n = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; n < a.ncells; n += (int64_t)gridDim.x * blockDim.x) {
    const int64_t x = a.cells[n];
#pragma unroll
    for (int q = 0; q < 19; q++) S::st(f + (int64_t)opp(q) * a.Np + x, (L)in[(int64_t)q * a.ncells + n], weight<L>(q));
  }
}

// Averages acc[c*NF + a] / nacc, rounded to float32 like the reference's
// Float32Array division (src/engine.js:356).
template <int K>
__global__ void get_acc_kernel(const StateArgs a, float *out, int nacc) {
  using Acc = typename Store<K>::Acc;
  const Acc *acc = (const Acc *)a.acc;
  const double dn = nacc > 1 ? (double)nacc : 1.0;
  for (int64_t n = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; n < a.ncells; n += (int64_t)gridDim.x * blockDim.x) {
    const int64_t x = a.cells[n];
    for (int c = 0; c < 4; c++) out[(int64_t)c * a.ncells + n] = (float)((double)acc[(int64_t)c * a.Np + x] / dn);
  }
}

// ---------------------------------------------------------------- block reductions (1024 threads)
__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}
__device__ __forceinline__ double nan_max(double a, double b) {
  if (isnan(a) || isnan(b)) return NAN;
  return a > b ? a : b;
}
__device__ __forceinline__ double warp_max(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = nan_max(v, __shfl_xor_sync(0xffffffffu, v, o));
  return v;
}
// Sum of NV doubles over the block, fixed order (deterministic); result in every thread.
template <int NV>
__device__ __forceinline__ void block_sum(double (&v)[NV], double *sh) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
  for (int i = 0; i < NV; i++) v[i] = warp_sum(v[i]);
  __syncthreads();
  if (lane == 0)
    for (int i = 0; i < NV; i++) sh[i * 32 + w] = v[i];
  __syncthreads();
  if (w == 0) {
    for (int i = 0; i < NV; i++) {
      double t = lane < nw ? sh[i * 32 + lane] : 0.0;
      t = warp_sum(t);
      if (lane == 0) sh[i * 32] = t;
    }
  }
  __syncthreads();
  for (int i = 0; i < NV; i++) v[i] = sh[i * 32];
  __syncthreads();
}
__device__ __forceinline__ double block_max(double v, double *sh) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
  v = warp_max(v);
  __syncthreads();
  if (lane == 0) sh[w] = v;
  __syncthreads();
  if (w == 0) {
    double t = lane < nw ? sh[lane] : -INFINITY;
    t = warp_max(t);
    if (lane == 0) sh[0] = t;
  }
  __syncthreads();
  v = sh[0];
  __syncthreads();
  return v;
}

// probeCPU + progressInfo (src/engine.js:324-339) for one progress check, in
// two launches.  First pass (many blocks): vy = my/r of the post-collision
// populations of every probe cell (layer jm, then layer top+1), stored as
// float32 like the reference's Float32Array, and per-block sums of -vy over
// each layer.  Second pass (one block): the fixed-order total, the mean of
// layer jm, the absolute deviations, gamma, the mass ratio and the
// instability flag (first non-finite outflow).  Deterministic for a given
// grid size.
template <int K>
__global__ void __launch_bounds__(kProbeThreads) probe_pass1_kernel(const StateArgs a, ProbeArgs pr) {
  __shared__ double sh[2 * 32];
  const int np = pr.nM + pr.nT;
  double v[2] = {0.0, 0.0};  // sw, qo of this block
  for (int n = blockIdx.x * blockDim.x + threadIdx.x; n < np; n += gridDim.x * blockDim.x) {
    double f[19];
    read_post_all<K>(a, pr.plist[n], f);
    double r = 0, my = 0;
#pragma unroll
    for (int q = 0; q < 19; q++) { r += f[q]; my += (double)cy(q) * f[q]; }
    const float vy = (float)(my / r);
    pr.vy[n] = vy;
    if (n < pr.nM) v[0] += -(double)vy; else v[1] += -(double)vy;
  }
  block_sum<2>(v, sh);
  if (threadIdx.x == 0) { pr.part[2 * blockIdx.x] = v[0]; pr.part[2 * blockIdx.x + 1] = v[1]; }
}

static __global__ void __launch_bounds__(1024) probe_pass2_kernel(ProbeArgs pr, int *status) {
  __shared__ double sh[2 * 32];
  double v[2] = {0.0, 0.0};
  for (int b = threadIdx.x; b < pr.nblocks; b += blockDim.x) { v[0] += pr.part[2 * b]; v[1] += pr.part[2 * b + 1]; }
  block_sum<2>(v, sh);
  const double wm = v[0] / pr.nM, qo = v[1];
  double d[1] = {0.0};
  for (int n = threadIdx.x; n < pr.nM; n += blockDim.x) d[0] += fabs(-(double)pr.vy[n] - wm);
  block_sum<1>(d, sh);
  if (threadIdx.x == 0) {
    double *h = pr.hist + 4 * (int64_t)pr.slot;
    h[0] = pr.step;
    h[1] = 1 - d[0] / (2 * pr.nM * wm);
    h[2] = qo / (pr.Ain * pr.u0);
    h[3] = qo;
    if (!isfinite(qo) && status && *status == 0) *status = pr.step;
  }
}

// evaluate() metrics (src/engine.js:632-660, 681-685) in one block of 1024
// threads with float64 sums.  Pass 1: filter-map mean, core mean, inlet and
// sub-pleat density sums; pass 2: deviations, shares, peak ratio, fmap.
template <int K>
__global__ void __launch_bounds__(1024) evaluate_kernel(const StateArgs a, EvalArgs e) {
  using Acc = typename Store<K>::Acc;
  __shared__ double sh[6 * 32];
  const Acc *acc = (const Acc *)a.acc;
  const int nx = e.nx, ny = e.ny, nz = e.nz;
  const int64_t nzp = e.nzp, kpad = e.kpad;
  const Acc *base = (const Acc *)e.base;
  const int nacc = base ? e.nacc - e.base_nacc : e.nacc;
  const double dn = nacc > 1 ? (double)nacc : 1.0;
  auto P = [&](int i, int j, int k) -> int64_t { return ((int64_t)i * ny + j) * nzp + k + kpad; };
  auto fluid = [&](int64_t p) -> bool {
    if (!(a.mask[p] & kFluidBit)) return false;
    return !(e.ns && e.ns[p] > 0.5f);
  };
  // mean field as the reference holds it: float32(acc / nacc); the float64 run keeps float64
  auto mean = [&](int c, int64_t p) -> double {
    const int64_t i = (int64_t)c * a.Np + p;
    const double m = (base ? (double)acc[i] - (double)base[i] : (double)acc[i]) / dn;
    if constexpr (sizeof(Acc) == 8) return m;
    else return (double)(float)m;
  };
  auto core = [&](int i, int k) -> bool {
    if (i < 1 || i > nx - 2 || k < 1 || k > nz - 2) return false;
    return fluid(P(i, e.jm, k)) && fluid(P(i - 1, e.jm, k)) && fluid(P(i + 1, e.jm, k)) && fluid(P(i, e.jm, k - 1)) &&
           fluid(P(i, e.jm, k + 1));
  };
  const int64_t nxz = (int64_t)nx * nz;
  // pass 1: sw, n, csum, cn, pin, pinN, pb, pbN
  double v[6] = {0, 0, 0, 0, 0, 0};
  double cnt[4] = {0, 0, 0, 0};
  for (int64_t x = threadIdx.x; x < nxz; x += blockDim.x) {
    const int i = (int)(x / nz), k = (int)(x % nz);
    const int64_t p = P(i, e.jm, k);
    if (fluid(p)) {
      const double w = -mean(1, p);
      v[0] += w; cnt[0] += 1;
      if (core(i, k)) { v[1] += w; cnt[1] += 1; }
    }
    const int64_t pb = P(i, e.jb, k);
    if (fluid(pb)) { v[3] += mean(3, pb); cnt[3] += 1; }
  }
  for (int64_t x = threadIdx.x; x < (int64_t)nx * ny; x += blockDim.x) {
    if (!e.opening[x]) continue;
    const int i = (int)(x / ny), j = (int)(x % ny);
    const int64_t p = P(i, j, 1);
    if (fluid(p)) { v[2] += mean(3, p); cnt[2] += 1; }
  }
  double r1[8] = {v[0], v[1], v[2], v[3], cnt[0], cnt[1], cnt[2], cnt[3]};
  {
    double t[6];
    for (int i = 0; i < 6; i++) t[i] = r1[i];
    block_sum<6>(t, sh);
    for (int i = 0; i < 6; i++) r1[i] = t[i];
    double u[2] = {r1[6], r1[7]};
    block_sum<2>(u, sh);
    r1[6] = u[0]; r1[7] = u[1];
  }
  const double sw = r1[0], csum = r1[1], pin = r1[2], pb = r1[3];
  const double n = r1[4], cn = r1[5], pinN = r1[6], pbN = r1[7];
  const double wm = sw / n, cm = csum / cn;
  // pass 2: dev, cdev, rev, low, high, max
  double d[5] = {0, 0, 0, 0, 0};
  double mxr = 0.0;
  for (int64_t x = threadIdx.x; x < nxz; x += blockDim.x) {
    const int i = (int)(x / nz), k = (int)(x % nz);
    const int64_t p = P(i, e.jm, k);
    if (!fluid(p)) { if (e.fmap) e.fmap[x] = NAN; continue; }
    const double w = -mean(1, p);
    d[0] += fabs(w - wm);
    if (w < 0) d[2] += 1;
    mxr = nan_max(mxr, w / wm);
    if (core(i, k)) {
      d[1] += fabs(w - cm);
      if (w < 0.5 * cm) d[3] += 1;
      if (w > 1.5 * cm) d[4] += 1;
    }
    if (e.fmap) e.fmap[x] = (float)(w / wm);
  }
  block_sum<5>(d, sh);
  mxr = block_max(mxr, sh);
  if (threadIdx.x == 0) {
    double *o = e.out;
    o[0] = 1 - d[0] / (2 * n * wm);            // gamma
    o[1] = 1 - d[1] / (2 * cn * cm);           // gammaCore
    o[2] = d[3] / cn;                          // lowCore
    o[3] = d[4] / cn;                          // highCore
    o[4] = d[2] / n;                           // reverse
    o[5] = mxr;                                // maxToMean
    o[6] = ((pin / pinN - pb / pbN) / 3) / (0.5 * e.u0 * e.u0);  // zeta
    o[7] = wm; o[8] = cm; o[9] = n; o[10] = cn; o[11] = pinN; o[12] = pbN;
  }
}

}  // namespace abx
