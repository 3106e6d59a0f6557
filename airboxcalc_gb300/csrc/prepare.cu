// prepare.cu - the mask stages of prepare() and the device geometry of
// setupSim on the GPU.
//
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
// Integer work only; every result is independent of scheduling.
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
    uint8_t prev = a.fluid[base];
    for (int t = 1; t < len; t++) {
      const int64_t c = base + t * stride;
      uint8_t f = a.fluid[c];
      const bool open = !a.solid[c] && (AXIS == 1 ? t >= a.top : true);
      if (!f && prev && open) { a.fluid[c] = 1; f = 1; any = true; }
      prev = f;
    }
    prev = a.fluid[base + (int64_t)(len - 1) * stride];
    for (int t = len - 2; t >= 0; t--) {
      const int64_t c = base + t * stride;
      uint8_t f = a.fluid[c];
      const bool open = !a.solid[c] && (AXIS == 1 ? t >= a.top : true);
      if (!f && prev && open) { a.fluid[c] = 1; f = 1; any = true; }
      prev = f;
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

}  // namespace abx
