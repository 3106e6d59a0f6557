// prepare.cu - the mask stages of prepare() and the device geometry of
// setupSim on the GPU.
//
//   opening          src/engine.js:141-171 on the fine slice kf: empty cells
//                    4-connected to the slice border (line sweeps to a fixed
//                    point), holes below the seal, their 4-connected components
//                    (label = lowest index, i.e. the reference's scan-order
//                    numbering), sizes, the components above 25 mm^2, the
//                    largest (first of equals) or, with a click, the one whose
//                    every-third cell in the reference's breadth-first order
//                    comes closest, and the coarse cells holding 5 of 9
//   duct / closing   src/engine.js:174-178: cells before the inlet wall are
//                    solid except under the opening; rows beyond the model's
//                    depth are solid
//   flood            :181-189: the air is every cell 6-connected to the
//                    opening's k = 0 cells through non-solid cells with j >= top.
//                    Computed as the fixed point of line sweeps (forward and
//                    backward along k, j and i in turn, until a round adds no
//                    cell): the same set as the reference's breadth-first search
//   leak             :191-195: air on a side face or the far face
//   outlet           :197-213: row `top`, or the lid plenum with a round outlet
//   classes          setupSim :248-255: bulk, inlet, outlet, filter
//   kpad / segments  the padded layout: the shift of every column that
//                    minimises the 32-cell runs holding air, the list of those
//                    runs with their lane masks, and the compact cell list
//                    (cells in (i, j, k) order, the reference's compact order)
//
// Integer work (and float64 with explicitly rounded operations where the
// reference compares coordinates); every result is independent of scheduling.
#include <stdint.h>

#include "d3q19.cuh"
#include "lbm_iface.h"

namespace abx {

static unsigned grid_of(int64_t n, int per_thread = 1) {
  int64_t b = (n / per_thread + 255) / 256;
  if (b > 152 * 16) b = 152 * 16;
  return (unsigned)(b < 1 ? 1 : b);
}

__global__ void duct_kernel(const MaskArgs a) {
  for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < a.N; c += (int64_t)gridDim.x * blockDim.x) {
    const int k = (int)(c % a.nz);
    const int64_t ij = c / a.nz;
    const int j = (int)(ij % a.ny);
    uint8_t s = a.solid[c];
    if (k < a.kw0) s = a.opening[ij] ? 0 : 1;
    if (a.close_row[j]) s = 1;
    a.solid[c] = s;
    a.fluid[c] = 0;
    a.outlet[c] = 0;
  }
}

__global__ void seed_kernel(const MaskArgs a) {
  const int64_t n = (int64_t)a.nx * a.ny;
  for (int64_t ij = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; ij < n; ij += (int64_t)gridDim.x * blockDim.x) {
    const int64_t c = ij * a.nz;
    if (a.opening[ij] && (int)(ij % a.ny) >= a.top && !a.solid[c]) a.fluid[c] = 1;
  }
}

// Lines are walked in chunks of kWalk cells whose loads are issued together before the chunk is processed in
// order (a line's cells ahead of the walk are written only by the walking thread itself): along j and i the
// steps are nz and ny*nz cells apart, and one dependent load per step would wait on the memory latency.
constexpr int kWalk = 16;

// One sweep along AXIS (2: k, 1: j, 0: i), one thread per grid line, forward then backward: a cell joins
// the air when its predecessor on the line is air and it is open (not solid, j >= top).
template <int AXIS>
__global__ void sweep_kernel(const MaskArgs a, int *changed) {
  int64_t lines, stride;
  int len;
  if (AXIS == 2) { lines = (int64_t)a.nx * a.ny; stride = 1; len = a.nz; }
  else if (AXIS == 1) { lines = (int64_t)a.nx * a.nz; stride = a.nz; len = a.ny; }
  else { lines = (int64_t)a.ny * a.nz; stride = (int64_t)a.ny * a.nz; len = a.nx; }
  bool any = false;
  for (int64_t l = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; l < lines; l += (int64_t)gridDim.x * blockDim.x) {
    int64_t base;
    int jfix = -1;
    if (AXIS == 2) { base = l * a.nz; jfix = (int)(l % a.ny); }
    else if (AXIS == 1) { base = (l / a.nz) * a.ny * a.nz + l % a.nz; }
    else { base = l; jfix = (int)(l / a.nz); }
    if (jfix >= 0 && jfix < a.top) continue;   // the whole line is closed
    for (int dir = 0; dir < 2; dir++) {
      // forward: t = 1 .. len-1 after t = 0; backward: t = len-2 .. 0 after t = len-1
      uint8_t prev = a.fluid[base + (dir ? (int64_t)(len - 1) * stride : 0)];
      for (int s0 = 1; s0 < len; s0 += kWalk) {
        uint8_t f[kWalk], sol[kWalk];
#pragma unroll
        for (int u = 0; u < kWalk; u++) {
          const int s = s0 + u, t = dir ? len - 1 - s : s;
          if (s < len) { f[u] = a.fluid[base + t * stride]; sol[u] = a.solid[base + t * stride]; }
        }
#pragma unroll
        for (int u = 0; u < kWalk; u++) {
          const int s = s0 + u, t = dir ? len - 1 - s : s;
          if (s < len) {
            const bool open = !sol[u] && (AXIS == 1 ? t >= a.top : true);
            if (!f[u] && prev && open) { a.fluid[base + t * stride] = 1; f[u] = 1; any = true; }
            prev = f[u];
          }
        }
      }
    }
  }
  if (__syncthreads_or(any) && threadIdx.x == 0) atomicOr(changed, 1);
}

__global__ void leak_kernel(const MaskArgs a, int *leak) {
  bool any = false;
  for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < a.N; c += (int64_t)gridDim.x * blockDim.x) {
    const int k = (int)(c % a.nz);
    const int64_t ij = c / a.nz;
    const int j = (int)(ij % a.ny), i = (int)(ij / a.ny);
    if (j >= a.top && k >= a.kw0 && (i == 0 || i == a.nx - 1 || k == a.nz - 1) && a.fluid[c]) any = true;
  }
  if (__syncthreads_or(any) && threadIdx.x == 0) atomicOr(leak, 1);
}

// Outlet: the lid plenum (jpt >= 0) or row `top`.  counts[0] += cells added above top, counts[1] += outlet cells.
__global__ void outlet_kernel(const MaskArgs a, int jpt, const float *xc, const float *zc, double cx, double cz,
                              double r2, unsigned long long *counts) {
  const int64_t n = (int64_t)a.nx * a.nz;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n; t += (int64_t)gridDim.x * blockDim.x) {
    const int i = (int)(t / a.nz), k = (int)(t % a.nz);
    const int64_t ctop = ((int64_t)i * a.ny + a.top) * a.nz + k;
    if (!a.fluid[ctop]) continue;
    if (jpt < 0) {
      a.outlet[ctop] = 1;
      atomicAdd(counts + 1, 1ull);
      continue;
    }
    for (int j = jpt; j < a.top; j++) {
      const int64_t c = ((int64_t)i * a.ny + j) * a.nz + k;
      a.fluid[c] = 1;
      a.solid[c] = 0;
    }
    atomicAdd(counts, (unsigned long long)(a.top - jpt));
    const double ddx = (double)xc[i] - cx, ddz = (double)zc[k] - cz;
    if (ddx * ddx + ddz * ddz <= r2) {
      a.outlet[((int64_t)i * a.ny + jpt) * a.nz + k] = 1;
      atomicAdd(counts + 1, 1ull);
    }
  }
}

// counts[0] air cells, [1] air on layer jm, [2] air on row top
__global__ void count_kernel(const MaskArgs a, int jm, unsigned long long *counts) {
  unsigned long long nf = 0, af = 0, lk = 0;
  for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < a.N; c += (int64_t)gridDim.x * blockDim.x) {
    if (!a.fluid[c]) continue;
    const int j = (int)((c / a.nz) % a.ny);
    nf++;
    af += j == jm;
    lk += j == a.top;
  }
  for (int o = 16; o > 0; o >>= 1) {
    nf += __shfl_xor_sync(0xffffffffu, nf, o);
    af += __shfl_xor_sync(0xffffffffu, af, o);
    lk += __shfl_xor_sync(0xffffffffu, lk, o);
  }
  if ((threadIdx.x & 31) == 0) {
    if (nf) atomicAdd(counts, nf);
    if (af) atomicAdd(counts + 1, af);
    if (lk) atomicAdd(counts + 2, lk);
  }
}

// setupSim's classes (src/engine.js:252-254): 0 no air, 1 bulk, 2 inlet, 3 outlet, 4 filter; ain += inlet cells.
__global__ void class_kernel(const MaskArgs a, const uint8_t *filt_row, uint8_t *cls, unsigned long long *ain) {
  unsigned long long n_in = 0;
  for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < a.N; c += (int64_t)gridDim.x * blockDim.x) {
    uint8_t cl = 0;
    if (a.fluid[c]) {
      const int k = (int)(c % a.nz);
      const int64_t ij = c / a.nz;
      cl = 1;
      if (k == 0 && a.opening[ij]) { cl = 2; n_in++; }
      else if (a.outlet[c]) cl = 3;
      else if (filt_row[ij % a.ny]) cl = 4;
    }
    cls[c] = cl;
  }
  for (int o = 16; o > 0; o >>= 1) n_in += __shfl_xor_sync(0xffffffffu, n_in, o);
  if ((threadIdx.x & 31) == 0 && n_in) atomicAdd(ain, n_in);
}

// Air bits of every column, W words per column (bit k of the column at word k/32), the last word zero.
__global__ void colbits_kernel(const MaskArgs a, int W, uint32_t *bits) {
  const int64_t cols = (int64_t)a.nx * a.ny, n = cols * W;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n; t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t ij = t / W;
    const int w = (int)(t % W);
    uint32_t v = 0;
    for (int b = 0; b < 32; b++) {
      const int k = w * 32 + b;
      if (k < a.nz && a.fluid[ij * a.nz + k]) v |= 1u << b;
    }
    bits[t] = v;
  }
}

// The 32 bits of a column starting at bit `b` (bits before 0 read as 0).
__device__ __forceinline__ uint32_t bits32(const uint32_t *col, int b) {
  if (b < 0) return col[0] << (-b);
  const int w = b >> 5, o = b & 31;
  return o ? (col[w] >> o) | (col[w + 1] << (32 - o)) : col[w];
}

// count[t] += 32-cell runs holding air over all columns when every column is shifted by t (t = 0..31)
__global__ void kpad_count_kernel(int64_t cols, int nz, int W, const uint32_t *bits, unsigned long long *count) {
  unsigned long long c[32];
#pragma unroll
  for (int t = 0; t < 32; t++) c[t] = 0;
  for (int64_t ij = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; ij < cols; ij += (int64_t)gridDim.x * blockDim.x) {
    const uint32_t *col = bits + ij * W;
#pragma unroll
    for (int t = 0; t < 32; t++)
      for (int s = 0; 32 * s - t < nz; s++) c[t] += bits32(col, 32 * s - t) != 0u;
  }
#pragma unroll
  for (int t = 0; t < 32; t++) {
    unsigned long long v = c[t];
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if ((threadIdx.x & 31) == 0 && v) atomicAdd(count + t, v);
  }
}

// Ordered compaction in three passes over items [0, n): blocks of kItems items count their hits, one block
// turns the counts into offsets, the blocks write their hits in order.
constexpr int kPerThread = 16, kItems = 256 * kPerThread;

struct CellItems {   // dense cell c -> its padded index, if air
  const uint8_t *fluid;
  int nz;
  int64_t nzp, kpad;
  __device__ bool hit(int64_t c) const { return fluid[c] != 0; }
  __device__ int64_t value(int64_t c) const { return (c / nz) * nzp + c % nz + kpad; }
};
struct SegItems {    // run slot r = column * S + s -> {padded base, lane mask}, if the run holds air
  const uint32_t *bits;
  int W, S;
  int64_t nzp, kpad;
  __device__ uint32_t lanes(int64_t r) const {
    return bits32(bits + (r / S) * W, (int)(32 * (r % S) - kpad));
  }
  __device__ bool hit(int64_t r) const { return lanes(r) != 0u; }
  __device__ uint2 value(int64_t r) const {
    return make_uint2((uint32_t)((r / S) * nzp + 32 * (r % S)), lanes(r));
  }
};

template <class Items>
__global__ void compact_count_kernel(const Items it, int64_t n, uint32_t *block_counts) {
  __shared__ uint32_t red[8];
  const int64_t b0 = (int64_t)blockIdx.x * kItems + (int64_t)threadIdx.x * kPerThread;
  uint32_t cnt = 0;
  for (int e = 0; e < kPerThread; e++) cnt += (b0 + e < n) && it.hit(b0 + e);
  for (int o = 16; o > 0; o >>= 1) cnt += __shfl_xor_sync(0xffffffffu, cnt, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = cnt;
  __syncthreads();
  if (threadIdx.x == 0) {
    uint32_t t = 0;
    for (int w = 0; w < 8; w++) t += red[w];
    block_counts[blockIdx.x] = t;
  }
}

// exclusive scan of nb block counts into offsets (one block of 1024 threads, chunked), total at offsets[nb]
__global__ void compact_scan_kernel(const uint32_t *counts, int64_t nb, unsigned long long *offsets) {
  __shared__ unsigned long long sh[1024];
  unsigned long long carry = 0;
  for (int64_t base = 0; base < nb; base += 1024) {
    const int64_t i = base + threadIdx.x;
    const unsigned long long v = i < nb ? counts[i] : 0ull;
    sh[threadIdx.x] = v;
    __syncthreads();
    for (int o = 1; o < 1024; o <<= 1) {
      const unsigned long long x = threadIdx.x >= (unsigned)o ? sh[threadIdx.x - o] : 0ull;
      __syncthreads();
      sh[threadIdx.x] += x;
      __syncthreads();
    }
    if (i < nb) offsets[i] = carry + sh[threadIdx.x] - v;
    const unsigned long long total = sh[1023];
    __syncthreads();
    carry += total;
  }
  if (threadIdx.x == 0) offsets[nb] = carry;
}

template <class Items, class T>
__global__ void compact_write_kernel(const Items it, int64_t n, const unsigned long long *offsets, T *out) {
  __shared__ uint32_t sh[256];
  const int64_t b0 = (int64_t)blockIdx.x * kItems + (int64_t)threadIdx.x * kPerThread;
  uint32_t cnt = 0;
  for (int e = 0; e < kPerThread; e++) cnt += (b0 + e < n) && it.hit(b0 + e);
  sh[threadIdx.x] = cnt;
  __syncthreads();
  for (int o = 1; o < 256; o <<= 1) {
    const uint32_t x = threadIdx.x >= (unsigned)o ? sh[threadIdx.x - o] : 0u;
    __syncthreads();
    sh[threadIdx.x] += x;
    __syncthreads();
  }
  unsigned long long pos = offsets[blockIdx.x] + sh[threadIdx.x] - cnt;
  for (int e = 0; e < kPerThread; e++)
    if (b0 + e < n && it.hit(b0 + e)) out[pos++] = it.value(b0 + e);
}

template <class Items, class T>
static cudaError_t compact(const Items &it, int64_t n, T *out, uint32_t *block_counts, unsigned long long *offsets,
                           cudaStream_t st) {
  const int64_t nb = (n + kItems - 1) / kItems;
  if (nb == 0) return cudaMemsetAsync(offsets, 0, sizeof(unsigned long long), st);
  compact_count_kernel<Items><<<(unsigned)nb, 256, 0, st>>>(it, n, block_counts);
  compact_scan_kernel<<<1, 1024, 0, st>>>(block_counts, nb, offsets);
  if (out) compact_write_kernel<Items, T><<<(unsigned)nb, 256, 0, st>>>(it, n, offsets, out);
  return cudaGetLastError();
}

int64_t prep_compact_blocks(int64_t n) { return (n + kItems - 1) / kItems; }

cudaError_t prep_duct(const MaskArgs &a, cudaStream_t st) {
  duct_kernel<<<grid_of(a.N), 256, 0, st>>>(a);
  seed_kernel<<<grid_of((int64_t)a.nx * a.ny), 256, 0, st>>>(a);
  return cudaGetLastError();
}

cudaError_t prep_flood_round(const MaskArgs &a, int *changed, cudaStream_t st) {
  sweep_kernel<2><<<grid_of((int64_t)a.nx * a.ny), 256, 0, st>>>(a, changed);
  sweep_kernel<1><<<grid_of((int64_t)a.nx * a.nz), 256, 0, st>>>(a, changed);
  sweep_kernel<0><<<grid_of((int64_t)a.ny * a.nz), 256, 0, st>>>(a, changed);
  return cudaGetLastError();
}

cudaError_t prep_leak(const MaskArgs &a, int *leak, cudaStream_t st) {
  leak_kernel<<<grid_of(a.N), 256, 0, st>>>(a, leak);
  return cudaGetLastError();
}

cudaError_t prep_outlet(const MaskArgs &a, int jpt, const float *xc, const float *zc, double cx, double cz, double r2,
                        unsigned long long *counts, cudaStream_t st) {
  outlet_kernel<<<grid_of((int64_t)a.nx * a.nz), 256, 0, st>>>(a, jpt, xc, zc, cx, cz, r2, counts);
  return cudaGetLastError();
}

cudaError_t prep_counts(const MaskArgs &a, int jm, unsigned long long *counts, cudaStream_t st) {
  count_kernel<<<grid_of(a.N), 256, 0, st>>>(a, jm, counts);
  return cudaGetLastError();
}

cudaError_t prep_classes(const MaskArgs &a, const uint8_t *filt_row, uint8_t *cls, unsigned long long *ain,
                         cudaStream_t st) {
  class_kernel<<<grid_of(a.N), 256, 0, st>>>(a, filt_row, cls, ain);
  return cudaGetLastError();
}

cudaError_t prep_kpad_counts(const MaskArgs &a, int W, uint32_t *bits, unsigned long long *count, cudaStream_t st) {
  const int64_t cols = (int64_t)a.nx * a.ny;
  colbits_kernel<<<grid_of(cols * W), 256, 0, st>>>(a, W, bits);
  kpad_count_kernel<<<grid_of(cols), 256, 0, st>>>(cols, a.nz, W, bits, count);
  return cudaGetLastError();
}

cudaError_t prep_cells(const MaskArgs &a, int64_t nzp, int64_t kpad, int64_t *cells, uint32_t *block_counts,
                       unsigned long long *offsets, cudaStream_t st) {
  const CellItems it{a.fluid, a.nz, nzp, kpad};
  return compact(it, a.N, cells, block_counts, offsets, st);
}

// One warp per segment: flag the segment interior when every fluid lane's mask word is kMaskInterior.
__global__ void seg_interior_kernel(uint2 *seg, uint32_t nseg, const uint32_t *__restrict__ mask) {
  const uint32_t s = blockIdx.x * 8u + (threadIdx.x >> 5), lane = threadIdx.x & 31u;
  if (s >= nseg) return;   // uniform per warp
  const uint2 g = seg[s];
  const bool edge = ((g.y >> lane) & 1u) && mask[seg_base(g) + lane] != kMaskInterior;
  const unsigned any = __ballot_sync(0xffffffffu, edge);
  if (lane == 0 && !any) seg[s].x = seg_base(g) | kSegInterior;
}

// ABX_SEG_INTERIOR=0 leaves every segment unflagged (every step loads every mask word)
#ifndef ABX_SEG_INTERIOR
#define ABX_SEG_INTERIOR 1
#endif
cudaError_t prep_seg_interior(uint2 *seg, uint32_t nseg, const uint32_t *mask, cudaStream_t st) {
  if (nseg == 0 || !ABX_SEG_INTERIOR) return cudaSuccess;
  seg_interior_kernel<<<(nseg + 7u) / 8u, 256, 0, st>>>(seg, nseg, mask);
  return cudaGetLastError();
}

cudaError_t prep_segments(const MaskArgs &a, int W, const uint32_t *bits, int64_t nzp, int64_t kpad, uint2 *seg,
                          uint32_t *block_counts, unsigned long long *offsets, cudaStream_t st) {
  const int S = (int)(nzp / 32);
  const SegItems it{bits, W, S, nzp, kpad};
  return compact(it, (int64_t)a.nx * a.ny * S, seg, block_counts, offsets, st);
}

// ------------------------------------------------------------------ work lists of the vectorised step kernel
// Item i of the block lists is block i % nb of segment i / nb (nb = 32 / V blocks per segment).  A block is
// interior of class cls when its V cells are all fluid and every one's mask word is kMaskInterior with that
// class in the class bits: all 18 pull neighbours fluid, no bounce-back, one collision branch.
__device__ __forceinline__ bool vec_block_is(const uint2 s, const uint32_t *__restrict__ mask, int V, int blk,
                                             uint32_t want) {
  const uint32_t vm = (V >= 32) ? 0xffffffffu : ((1u << V) - 1u);
  if (((s.y >> (blk * V)) & vm) != vm) return false;
  const uint32_t base = seg_base(s) + (uint32_t)(blk * V);
  for (int c = 0; c < V; c++)
    if (mask[base + c] != want) return false;
  return true;
}
constexpr uint32_t kMaskInteriorFilter = kMaskInterior | (kClsFilter << kClassShift);

struct VecBlockItems {
  const uint2 *seg;
  const uint32_t *mask;
  int V, nb;
  uint32_t want;
  __device__ bool hit(int64_t i) const { return vec_block_is(seg[i / nb], mask, V, (int)(i % nb), want); }
  __device__ uint32_t value(int64_t i) const { return seg_base(seg[i / nb]) + (uint32_t)((i % nb) * V); }
};
struct VecBoundaryCells {   // cell i % 32 of segment i / 32 -> its padded index, if fluid and not in an interior block
  const uint2 *seg;
  const uint32_t *mask;
  int V;
  __device__ bool hit(int64_t i) const {
    const uint2 s = seg[i / 32];
    const int lane = (int)(i % 32), b = lane / V;
    if (!((s.y >> lane) & 1u)) return false;
    return !vec_block_is(s, mask, V, b, kMaskInterior) && !vec_block_is(s, mask, V, b, kMaskInteriorFilter);
  }
  __device__ uint32_t value(int64_t i) const { return seg_base(seg[i / 32]) + (uint32_t)(i % 32); }
};

cudaError_t prep_vec_lists(const uint2 *seg, uint32_t nseg, const uint32_t *mask, int V, uint32_t *blk,
                           uint32_t *bcell, uint32_t *block_counts, unsigned long long *offsets,
                           unsigned long long *counts, cudaStream_t st) {
  if (V != 2 && V != 4 && V != 8) return cudaErrorInvalidValue;
  const int nb = 32 / V;
  const int64_t nitems = (int64_t)nseg * nb, ncells = (int64_t)nseg * 32;
  cudaError_t e;
  // bulk blocks, then filter blocks behind them, then the boundary cells; counts[] receive the three totals
  const VecBlockItems bulk{seg, mask, V, nb, kMaskInterior};
  if ((e = compact(bulk, nitems, (uint32_t *)nullptr, block_counts, offsets, st)) != cudaSuccess) return e;
  if ((e = cudaMemcpyAsync(counts + 0, offsets + prep_compact_blocks(nitems), sizeof(unsigned long long),
                           cudaMemcpyDeviceToDevice, st)) != cudaSuccess) return e;
  const VecBlockItems filt{seg, mask, V, nb, kMaskInteriorFilter};
  if ((e = compact(filt, nitems, (uint32_t *)nullptr, block_counts, offsets, st)) != cudaSuccess) return e;
  if ((e = cudaMemcpyAsync(counts + 1, offsets + prep_compact_blocks(nitems), sizeof(unsigned long long),
                           cudaMemcpyDeviceToDevice, st)) != cudaSuccess) return e;
  const VecBoundaryCells bnd{seg, mask, V};
  if ((e = compact(bnd, ncells, (uint32_t *)nullptr, block_counts, offsets, st)) != cudaSuccess) return e;
  if ((e = cudaMemcpyAsync(counts + 2, offsets + prep_compact_blocks(ncells), sizeof(unsigned long long),
                           cudaMemcpyDeviceToDevice, st)) != cudaSuccess) return e;
  if (!blk && !bcell) return cudaSuccess;
  // the lists: the filter blocks are written behind the bulk blocks (their count is known on the host by now)
  unsigned long long c[3];
  if ((e = cudaMemcpyAsync(c, counts, sizeof c, cudaMemcpyDeviceToHost, st)) != cudaSuccess) return e;
  if ((e = cudaStreamSynchronize(st)) != cudaSuccess) return e;
  if ((e = compact(bulk, nitems, blk, block_counts, offsets, st)) != cudaSuccess) return e;
  if ((e = compact(filt, nitems, blk + c[0], block_counts, offsets, st)) != cudaSuccess) return e;
  return compact(bnd, ncells, bcell, block_counts, offsets, st);
}

// ------------------------------------------------------------------ opening search (src/engine.js:141-171)
constexpr uint32_t kClaimFree = 0xFFFFFFFFu, kClaimDone = 0xFFFFFFFEu;

__global__ void open_init_kernel(const OpenArgs a) {
  const int64_t n = (int64_t)a.nxf * a.nyf;
  for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < n; c += (int64_t)gridDim.x * blockDim.x) {
    const int i = (int)(c / a.nyf), j = (int)(c % a.nyf);
    const bool border = i == 0 || i == a.nxf - 1 || j == 0 || j == a.nyf - 1;
    a.outside[c] = (border && !a.slice[c]) ? 1 : 0;
    a.label[c] = -1;
    a.size[c] = 0;
    a.claim[c] = kClaimFree;
  }
}

// ROWS: one thread per row i, along j; else one thread per column j, along i (a row apart per step), walked
// in chunks of kWalk cells.  Forward then backward: an empty cell joins the outside when its predecessor on
// the line is outside.
template <bool ROWS>
__global__ void open_outside_kernel(const OpenArgs a, int *changed) {
  const int lines = ROWS ? a.nxf : a.nyf, len = ROWS ? a.nyf : a.nxf;
  const int64_t stride = ROWS ? 1 : a.nyf;
  bool any = false;
  for (int l = blockIdx.x * blockDim.x + threadIdx.x; l < lines; l += gridDim.x * blockDim.x) {
    const int64_t base = ROWS ? (int64_t)l * a.nyf : (int64_t)l;
    for (int dir = 0; dir < 2; dir++) {
      // forward: t = 1 .. len-1 after t = 0; backward: t = len-2 .. 0 after t = len-1
      uint8_t prev = a.outside[base + (dir ? (int64_t)(len - 1) * stride : 0)];
      for (int s0 = 1; s0 < len; s0 += kWalk) {
        uint8_t o[kWalk], m[kWalk];
#pragma unroll
        for (int u = 0; u < kWalk; u++) {
          const int s = s0 + u, t = dir ? len - 1 - s : s;
          if (s < len) { o[u] = a.outside[base + t * stride]; m[u] = a.slice[base + t * stride]; }
        }
#pragma unroll
        for (int u = 0; u < kWalk; u++) {
          const int s = s0 + u, t = dir ? len - 1 - s : s;
          if (s < len) {
            if (!o[u] && prev && !m[u]) { a.outside[base + t * stride] = 1; o[u] = 1; any = true; }
            prev = o[u];
          }
        }
      }
    }
  }
  if (__syncthreads_or(any) && threadIdx.x == 0) atomicOr(changed, 1);
}

// holes (:153): empty, not outside, fine-cell centre below the seal (origin_1 + (j + 0.5) hf > 0)
__global__ void open_holes_kernel(const OpenArgs a) {
  const int64_t n = (int64_t)a.nxf * a.nyf;
  for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < n; c += (int64_t)gridDim.x * blockDim.x) {
    const int j = (int)(c % a.nyf);
    const double y = __dadd_rn(a.origin1, __dmul_rn((double)j + 0.5, a.hf));
    a.label[c] = (!a.slice[c] && !a.outside[c] && y > 0.0) ? (int32_t)c : -1;
  }
}

// the lower label moves along runs of hole cells, forward then backward (walked in chunks like the outside);
// at the fixed point every cell of a component carries the component's lowest index
template <bool ROWS>
__global__ void open_label_kernel(const OpenArgs a, int *changed) {
  const int lines = ROWS ? a.nxf : a.nyf, len = ROWS ? a.nyf : a.nxf;
  const int64_t stride = ROWS ? 1 : a.nyf;
  bool any = false;
  for (int l = blockIdx.x * blockDim.x + threadIdx.x; l < lines; l += gridDim.x * blockDim.x) {
    const int64_t base = ROWS ? (int64_t)l * a.nyf : (int64_t)l;
    for (int dir = 0; dir < 2; dir++) {
      int32_t prev = a.label[base + (dir ? (int64_t)(len - 1) * stride : 0)];
      for (int s0 = 1; s0 < len; s0 += kWalk) {
        int32_t v[kWalk];
#pragma unroll
        for (int u = 0; u < kWalk; u++) {
          const int s = s0 + u, t = dir ? len - 1 - s : s;
          if (s < len) v[u] = a.label[base + t * stride];
        }
#pragma unroll
        for (int u = 0; u < kWalk; u++) {
          const int s = s0 + u, t = dir ? len - 1 - s : s;
          if (s < len) {
            if (v[u] >= 0 && prev >= 0 && prev < v[u]) { a.label[base + t * stride] = prev; v[u] = prev; any = true; }
            prev = v[u];
          }
        }
      }
    }
  }
  if (__syncthreads_or(any) && threadIdx.x == 0) atomicOr(changed, 1);
}

__global__ void open_size_kernel(const OpenArgs a) {
  const int64_t n = (int64_t)a.nxf * a.nyf;
  for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < n; c += (int64_t)gridDim.x * blockDim.x) {
    const int32_t l = a.label[c];
    if (l >= 0) atomicAdd(a.size + l, 1u);
  }
}

// kept components (:155): cells * hf * hf > 25, in the reference's left-to-right float64 order
__global__ void open_roots_kernel(const OpenArgs a, OpenOut *out, uint2 *kept, uint32_t cap) {
  const int64_t n = (int64_t)a.nxf * a.nyf;
  for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < n; c += (int64_t)gridDim.x * blockDim.x) {
    if (a.label[c] != (int32_t)c) continue;
    const uint32_t s = a.size[c];
    if (!(__dmul_rn(__dmul_rn((double)s, a.hf), a.hf) > 25.0)) continue;
    const uint32_t k = atomicAdd(&out->n_kept, 1u);
    if (k < cap) kept[k] = make_uint2((uint32_t)c, s);
    atomicMax(&out->best, ((unsigned long long)s << 32) | (0xFFFFFFFFull - (unsigned long long)c));
  }
}

// neighbour `slot` of cell c in components2d's order (:102): i-1, i+1, j-1, j+1; -1 outside the slice
__device__ __forceinline__ int32_t open_nb(const OpenArgs &a, int32_t c, int slot) {
  const int i = c / a.nyf, j = c % a.nyf;
  switch (slot) {
    case 0: return i > 0 ? c - a.nyf : -1;
    case 1: return i < a.nxf - 1 ? c + a.nyf : -1;
    case 2: return j > 0 ? c - 1 : -1;
    default: return j < a.nyf - 1 ? c + 1 : -1;
  }
}

// squared distance of fine cell c's centre to the click, as in :160-161 (rounded operations, no fusion), as
// the bits of the (non-negative) double: ordered like the values
__device__ __forceinline__ unsigned long long open_dist_bits(const OpenArgs &a, int32_t c, double cx, double cy) {
  const double x = __dadd_rn(a.origin0, __dmul_rn((double)(c / a.nyf) + 0.5, a.hf));
  const double y = __dadd_rn(a.origin1, __dmul_rn((double)(c % a.nyf) + 0.5, a.hf));
  const double dx = __dsub_rn(x, cx), dy = __dsub_rn(y, cy);
  return (unsigned long long)__double_as_longlong(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)));
}

// One block per kept component: its breadth-first order, level by level.  The queue of components2d
// (:99-104) appends, for each cell in queue order, its unvisited neighbours in slot order; so a cell of the
// next level is appended by the first cell of the current level (in queue order) that has it as a
// neighbour, and its place in the next level is the rank of (parent's place * 4 + slot) among all such
// claims.  Pass 1 takes the smallest claim per cell (atomicMin), pass 2 ranks the winning claims with a
// block-wide scan in claim order.
constexpr int kBfsThreads = 1024;
__global__ void __launch_bounds__(kBfsThreads) open_bfs_kernel(const OpenArgs a, const uint2 *kept,
                                                               const int64_t *offs, int32_t *order, double cx,
                                                               double cy, unsigned long long *dmin) {
  __shared__ uint32_t warp_tot[kBfsThreads / 32];
  __shared__ uint32_t chunk_tot;
  __shared__ unsigned long long best;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int32_t root = (int32_t)kept[blockIdx.x].x;
  const int64_t ncell = kept[blockIdx.x].y;
  int32_t *ord = order + offs[blockIdx.x];
  if (tid == 0) {
    ord[0] = root;
    a.claim[root] = kClaimDone;
    best = open_dist_bits(a, root, cx, cy);   // place 0 is sampled
  }
  __syncthreads();
  int64_t lo = 0, hi = 1;   // the current level is ord[lo, hi)
  while (lo < hi) {
    // pass 1: every unvisited hole neighbour of the level keeps its smallest claim
    for (int64_t p0 = lo; p0 < hi; p0 += kBfsThreads / 4) {
      const int64_t t = p0 + (tid >> 2);
      if (t < hi) {
        const int32_t d = open_nb(a, ord[t], tid & 3);
        if (d >= 0 && a.label[d] == root && __ldcg(a.claim + d) != kClaimDone)
          atomicMin(a.claim + d, (uint32_t)((t - lo) * 4 + (tid & 3)));
      }
    }
    __syncthreads();
    // pass 2: the winning claims, ranked in claim order, form the next level
    int64_t next = hi;
    for (int64_t p0 = lo; p0 < hi; p0 += kBfsThreads / 4) {
      const int64_t t = p0 + (tid >> 2);
      int32_t d = -1;
      uint32_t flag = 0;
      if (t < hi) {
        d = open_nb(a, ord[t], tid & 3);
        if (d >= 0 && a.label[d] == root && __ldcg(a.claim + d) == (uint32_t)((t - lo) * 4 + (tid & 3))) flag = 1;
      }
      // block-wide exclusive scan of flag in thread order (= claim order)
      uint32_t inc = flag;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const uint32_t v = __shfl_up_sync(0xffffffffu, inc, o);
        if (lane >= o) inc += v;
      }
      if (lane == 31) warp_tot[warp] = inc;
      __syncthreads();
      if (warp == 0) {
        uint32_t w = warp_tot[lane], wi = w;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
          const uint32_t v = __shfl_up_sync(0xffffffffu, wi, o);
          if (lane >= o) wi += v;
        }
        warp_tot[lane] = wi - w;          // exclusive prefix of the warp totals
        if (lane == 31) chunk_tot = wi;
      }
      __syncthreads();
      if (flag) {
        const int64_t pos = next + warp_tot[warp] + inc - 1;
        if (pos < ncell) {
          ord[pos] = d;
          a.claim[d] = kClaimDone;
          if (pos % 3 == 0) atomicMin(&best, open_dist_bits(a, d, cx, cy));
        }
      }
      next += chunk_tot;
      __syncthreads();   // warp_tot and chunk_tot are reused by the next chunk
    }
    lo = hi;
    hi = next < ncell ? next : ncell;
  }
  if (tid == 0) dmin[blockIdx.x] = best;
}

// fine cells of the chosen component per coarse cell (:164), then the cells holding at least 5 (:166)
__global__ void open_sel_kernel(const OpenArgs a, int32_t root, int ny, uint32_t *sel) {
  const int64_t n = (int64_t)a.nxf * a.nyf;
  for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < n; c += (int64_t)gridDim.x * blockDim.x) {
    if (a.label[c] != root) continue;
    const int i = (int)(c / a.nyf), j = (int)(c % a.nyf);
    atomicAdd(sel + (int64_t)(i / 3) * ny + j / 3, 1u);
  }
}

__global__ void open_mark_kernel(const uint32_t *sel, int64_t n, uint8_t *opening, OpenOut *out) {
  uint32_t cnt = 0;
  for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < n; c += (int64_t)gridDim.x * blockDim.x) {
    const uint8_t o = sel[c] >= 5 ? 1 : 0;
    opening[c] = o;
    cnt += o;
  }
  for (int o = 16; o > 0; o >>= 1) cnt += __shfl_xor_sync(0xffffffffu, cnt, o);
  if ((threadIdx.x & 31) == 0 && cnt) atomicAdd(&out->n_open, cnt);
}

cudaError_t open_init(const OpenArgs &a, cudaStream_t st) {
  open_init_kernel<<<grid_of((int64_t)a.nxf * a.nyf), 256, 0, st>>>(a);
  return cudaGetLastError();
}

cudaError_t open_outside_round(const OpenArgs &a, int *changed, cudaStream_t st) {
  open_outside_kernel<true><<<grid_of(a.nxf), 256, 0, st>>>(a, changed);
  open_outside_kernel<false><<<grid_of(a.nyf), 256, 0, st>>>(a, changed);
  return cudaGetLastError();
}

cudaError_t open_holes(const OpenArgs &a, cudaStream_t st) {
  open_holes_kernel<<<grid_of((int64_t)a.nxf * a.nyf), 256, 0, st>>>(a);
  return cudaGetLastError();
}

cudaError_t open_label_round(const OpenArgs &a, int *changed, cudaStream_t st) {
  open_label_kernel<true><<<grid_of(a.nxf), 256, 0, st>>>(a, changed);
  open_label_kernel<false><<<grid_of(a.nyf), 256, 0, st>>>(a, changed);
  return cudaGetLastError();
}

cudaError_t open_components(const OpenArgs &a, OpenOut *out, uint2 *kept, uint32_t cap, cudaStream_t st) {
  const int64_t n = (int64_t)a.nxf * a.nyf;
  open_size_kernel<<<grid_of(n), 256, 0, st>>>(a);
  open_roots_kernel<<<grid_of(n), 256, 0, st>>>(a, out, kept, cap);
  return cudaGetLastError();
}

cudaError_t open_bfs_click(const OpenArgs &a, const uint2 *kept, const int64_t *offs, int n, int32_t *order,
                           double cx, double cy, unsigned long long *dmin, cudaStream_t st) {
  if (n <= 0) return cudaSuccess;
  open_bfs_kernel<<<n, kBfsThreads, 0, st>>>(a, kept, offs, order, cx, cy, dmin);
  return cudaGetLastError();
}

cudaError_t open_select(const OpenArgs &a, uint32_t root, int nx, int ny, uint32_t *sel, uint8_t *opening,
                        OpenOut *out, cudaStream_t st) {
  open_sel_kernel<<<grid_of((int64_t)a.nxf * a.nyf), 256, 0, st>>>(a, (int32_t)root, ny, sel);
  open_mark_kernel<<<grid_of((int64_t)nx * ny), 256, 0, st>>>(sel, (int64_t)nx * ny, opening, out);
  return cudaGetLastError();
}

}  // namespace abx
