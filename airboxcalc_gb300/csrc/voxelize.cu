// voxelize.cu - the parity voxelizer of src/engine.js:45-93 fused with the
// 27->1 downsample of src/engine.js:127-135, bit-exact with the reference.
// Compiled with -fmad=false: every double operation rounds on its own, as in
// the JavaScript (numbers are IEEE doubles; hits are stored as float32, :78).
//
// Pipeline on the fine grid (3x per axis, cell size hf = h/3):
//   1 tri_setup     one thread per triangle: jittered coordinates, den, the
//                   covered column box [i0,i1]x[j0,j1] (:53-59), its size
//   2 scan          exclusive prefix of the box sizes = flat (triangle, column) work list
//   3 count         one thread per work item: barycentric test at the column
//                   centre (:60-69), count hits per column (pass 0 of :71)
//   4 scan          column offsets into the hit array (:77-78)
//   5 scatter       same test, write float32 hit depth (pass 1 of :72)
//   6 columns       one thread per column: sort its hits (:85), turn pairs into
//                   fine-k intervals [ceil(z0/hf-.5), ceil(z1/hf-.5)-1] (:86-90)
//                   and record the opening-search slice voxel at kf (:144)
//   7 downsample    one thread per coarse cell: count fine voxels of its 3x3x3
//                   block from the intervals of its 9 columns; solid if >= 7
// The fine grid itself is never stored (1.36 GB for a 512x256x384 grid); a
// separate kernel writes it for tests.
#include <math.h>
#include <stdint.h>
#include <stdio.h>

#include <cuda.h>

#include <mutex>

#include "lbm_iface.h"

namespace abx {

struct TriRec {
  double ax, ay, az, bx, by, bz, cx, cy, cz, den;
  int i0, i1, j0, j1;
};

// Math.max/Math.min of src/engine.js:58-59 for finite values.
__device__ __forceinline__ double dmin3(double a, double b, double c) { double m = a < b ? a : b; return m < c ? m : c; }
__device__ __forceinline__ double dmax3(double a, double b, double c) { double m = a > b ? a : b; return m > c ? m : c; }

__global__ void tri_setup_kernel(const float *T, int64_t ntri, double o0, double o1, double o2, double h, int nx,
                                 int ny, TriRec *rec, int64_t *work) {
  const double jx = 1.37e-4, jy = 2.71e-4;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < ntri; t += (int64_t)gridDim.x * blockDim.x) {
    const float *v = T + t * 9;
    TriRec r;
    r.ax = (double)v[0] - o0 - jx; r.ay = (double)v[1] - o1 - jy; r.az = (double)v[2] - o2;
    r.bx = (double)v[3] - o0 - jx; r.by = (double)v[4] - o1 - jy; r.bz = (double)v[5] - o2;
    r.cx = (double)v[6] - o0 - jx; r.cy = (double)v[7] - o1 - jy; r.cz = (double)v[8] - o2;
    r.den = (r.by - r.cy) * (r.ax - r.cx) + (r.cx - r.bx) * (r.ay - r.cy);
    int64_t n = 0;
    r.i0 = 0; r.i1 = -1; r.j0 = 0; r.j1 = -1;
    if (!(fabs(r.den) < 1e-12)) {
      double i0 = floor(dmin3(r.ax, r.bx, r.cx) / h - 0.5), i1 = ceil(dmax3(r.ax, r.bx, r.cx) / h - 0.5);
      double j0 = floor(dmin3(r.ay, r.by, r.cy) / h - 0.5), j1 = ceil(dmax3(r.ay, r.by, r.cy) / h - 0.5);
      i0 = i0 > 0 ? i0 : 0; j0 = j0 > 0 ? j0 : 0;
      i1 = i1 < nx - 1 ? i1 : nx - 1; j1 = j1 < ny - 1 ? j1 : ny - 1;
      if (i1 >= i0 && j1 >= j0) {
        r.i0 = (int)i0; r.i1 = (int)i1; r.j0 = (int)j0; r.j1 = (int)j1;
        n = (int64_t)(r.i1 - r.i0 + 1) * (r.j1 - r.j0 + 1);
      }
    }
    rec[t] = r;
    work[t] = n;
  }
}

// ------------------------------------------------------------------ exclusive scan (int64)
// Three phases: per-block scan with block totals, a one-block scan of the
// totals, and the add-back.  Each block covers 1024 threads x 4 items.
constexpr int kScanThreads = 1024, kScanItems = 4, kScanTile = kScanThreads * kScanItems;

template <class In>
__global__ void scan_tiles_kernel(const In *in, int64_t n, int64_t *out, int64_t *tile_sums) {
  __shared__ int64_t sh[kScanThreads / 32];
  const int64_t base = (int64_t)blockIdx.x * kScanTile + (int64_t)threadIdx.x * kScanItems;
  int64_t v[kScanItems], s = 0;
#pragma unroll
  for (int i = 0; i < kScanItems; i++) { v[i] = base + i < n ? (int64_t)in[base + i] : 0; s += v[i]; }
  // inclusive scan of the thread sums across the block
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  int64_t x = s;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) { const int64_t y = __shfl_up_sync(0xffffffffu, x, o); if (lane >= o) x += y; }
  if (lane == 31) sh[w] = x;
  __syncthreads();
  if (w == 0) {
    int64_t t = sh[lane];
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) { const int64_t y = __shfl_up_sync(0xffffffffu, t, o); if (lane >= o) t += y; }
    sh[lane] = t;
  }
  __syncthreads();
  int64_t run = x - s + (w > 0 ? sh[w - 1] : 0);
#pragma unroll
  for (int i = 0; i < kScanItems; i++) { if (base + i < n) out[base + i] = run; run += v[i]; }
  if (threadIdx.x == kScanThreads - 1) tile_sums[blockIdx.x] = run;
}

__global__ void scan_sums_kernel(int64_t *sums, int64_t n, int64_t *total) {
  // one block, sequential over chunks of 1024
  __shared__ int64_t sh[kScanThreads / 32];
  __shared__ int64_t carry;
  if (threadIdx.x == 0) carry = 0;
  __syncthreads();
  for (int64_t c0 = 0; c0 < n; c0 += kScanThreads) {
    const int64_t i = c0 + threadIdx.x;
    const int64_t s = i < n ? sums[i] : 0;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    int64_t x = s;
    for (int o = 1; o < 32; o <<= 1) { const int64_t y = __shfl_up_sync(0xffffffffu, x, o); if (lane >= o) x += y; }
    if (lane == 31) sh[w] = x;
    __syncthreads();
    if (w == 0) {
      int64_t t = sh[lane];
      for (int o = 1; o < 32; o <<= 1) { const int64_t y = __shfl_up_sync(0xffffffffu, t, o); if (lane >= o) t += y; }
      sh[lane] = t;
    }
    __syncthreads();
    const int64_t excl = carry + x - s + (w > 0 ? sh[w - 1] : 0);
    if (i < n) sums[i] = excl;
    __syncthreads();
    if (threadIdx.x == kScanThreads - 1) carry = excl + s;
    __syncthreads();
  }
  if (threadIdx.x == 0) *total = carry;
}

__global__ void scan_add_kernel(int64_t *out, int64_t n, const int64_t *tile_offsets) {
  const int64_t base = (int64_t)blockIdx.x * kScanTile;
  const int64_t add = tile_offsets[blockIdx.x];
  for (int i = threadIdx.x; i < kScanTile; i += blockDim.x)
    if (base + i < n) out[base + i] += add;
}

// out[0..n) = exclusive prefix of in; out[n] = total.  tmp: ceil(n/tile) + 1 int64.
template <class In>
static cudaError_t scan_exclusive(const In *in, int64_t n, int64_t *out, int64_t *tmp, cudaStream_t st) {
  const int64_t tiles = (n + kScanTile - 1) / kScanTile;
  if (tiles == 0) return cudaMemsetAsync(out, 0, sizeof(int64_t), st);
  scan_tiles_kernel<In><<<(unsigned)tiles, kScanThreads, 0, st>>>(in, n, out, tmp);
  scan_sums_kernel<<<1, kScanThreads, 0, st>>>(tmp, tiles, out + n);
  scan_add_kernel<<<(unsigned)tiles, 256, 0, st>>>(out, n, tmp);
  return cudaGetLastError();
}

// ------------------------------------------------------------------ work items
__device__ __forceinline__ int64_t find_tri(const int64_t *pre, int64_t ntri, int64_t w) {
  // last t with pre[t] <= w (pre is non-decreasing, pre[0] = 0)
  int64_t lo = 0, hi = ntri - 1;
  while (lo < hi) {
    const int64_t mid = (lo + hi + 1) >> 1;
    if (pre[mid] <= w) lo = mid; else hi = mid - 1;
  }
  return lo;
}

// Barycentric test of src/engine.js:61-69; returns true and the float32 hit depth.
__device__ __forceinline__ bool column_hit(const TriRec &r, int i, int j, double h, float *z) {
  const double px = ((double)i + 0.5) * h, py = ((double)j + 0.5) * h;
  const double l1 = ((r.by - r.cy) * (px - r.cx) + (r.cx - r.bx) * (py - r.cy)) / r.den;
  if (l1 < 0) return false;
  const double l2 = ((r.cy - r.ay) * (px - r.cx) + (r.ax - r.cx) * (py - r.cy)) / r.den;
  if (l2 < 0) return false;
  const double l3 = 1 - l1 - l2;
  if (l3 < 0) return false;
  *z = (float)(l1 * r.az + l2 * r.bz + l3 * r.cz);
  return true;
}

template <bool SCATTER>
__global__ void hits_kernel(const TriRec *rec, const int64_t *pre, int64_t ntri, int64_t W, double h, int nyf,
                            uint32_t *cnt, const int64_t *off, uint32_t *cursor, float *hits) {
  for (int64_t w = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; w < W; w += (int64_t)gridDim.x * blockDim.x) {
    const int64_t t = find_tri(pre, ntri, w);
    const TriRec r = rec[t];
    const int64_t rel = w - pre[t];
    const int nj = r.j1 - r.j0 + 1;
    const int i = r.i0 + (int)(rel / nj), j = r.j0 + (int)(rel % nj);
    float z;
    if (!column_hit(r, i, j, h, &z)) continue;
    const int64_t col = (int64_t)i * nyf + j;
    if (!SCATTER) atomicAdd(&cnt[col], 1u);
    else hits[off[col] + atomicAdd(&cursor[col], 1u)] = z;
  }
}

// ------------------------------------------------------------------ columns
constexpr int kLocalSort = 64;

// Sort the column's hits (:85), convert each pair to a fine-k interval
// (:86-90) written back in place as int pairs, record the interval count and
// whether the opening-search slice kf is set.
__global__ void columns_kernel(const int64_t *off, int64_t ncol, float *hits, double h, int nzf, int kf,
                               int *nivl, uint8_t *slice) {
  for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < ncol; c += (int64_t)gridDim.x * blockDim.x) {
    const int64_t a = off[c];
    const int n = (int)(off[c + 1] - a);
    float *z = hits + a;
    int *iv = (int *)z;
    int ni = 0;
    bool at_kf = false;
    if (n >= 2) {
      float loc[kLocalSort];
      const bool local = n <= kLocalSort;
      float *zs = local ? loc : z;
      if (local)
        for (int i = 0; i < n; i++) loc[i] = z[i];
      for (int i = 1; i < n; i++) {  // insertion sort, ascending
        const float v = zs[i];
        int k = i - 1;
        while (k >= 0 && zs[k] > v) { zs[k + 1] = zs[k]; k--; }
        zs[k + 1] = v;
      }
      const int m = n - (n % 2);
      for (int k = 0; k < m; k += 2) {
        const double z0 = (double)zs[k], z1 = (double)zs[k + 1];
        double k0 = ceil(z0 / h - 0.5), k1 = ceil(z1 / h - 0.5) - 1;
        k0 = k0 > 0 ? k0 : 0;
        k1 = k1 < nzf - 1 ? k1 : nzf - 1;
        if (k0 > k1) continue;
        const int i0 = (int)k0, i1 = (int)k1;
        if (kf >= i0 && kf <= i1) at_kf = true;
        iv[2 * ni] = i0; iv[2 * ni + 1] = i1;  // 2*ni <= k: no unread hit is overwritten
        ni++;
      }
    }
    nivl[c] = ni;
    slice[c] = at_kf ? 1 : 0;
  }
}

// Coarse solid = at least 7 of the 27 fine voxels set (src/engine.js:128-135).
__global__ void downsample_kernel(const int64_t *off, const float *hits, const int *nivl, int nx, int ny, int nz,
                                  uint8_t *solid) {
  const int nyf = 3 * ny;
  const int64_t N = (int64_t)nx * ny * nz;
  for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < N; c += (int64_t)gridDim.x * blockDim.x) {
    const int k = (int)(c % nz);
    const int64_t ij = c / nz;
    const int j = (int)(ij % ny), i = (int)(ij / ny);
    const int lo = 3 * k, hi = 3 * k + 2;
    int s = 0;
    for (int a = 0; a < 3; a++)
      for (int b = 0; b < 3; b++) {
        const int64_t col = (int64_t)(3 * i + a) * nyf + (3 * j + b);
        const int *iv = (const int *)(hits + off[col]);
        const int ni = nivl[col];
        for (int e = 0; e < ni; e++) {
          const int k0 = iv[2 * e] > lo ? iv[2 * e] : lo, k1 = iv[2 * e + 1] < hi ? iv[2 * e + 1] : hi;
          if (k1 >= k0) s += k1 - k0 + 1;
        }
      }
    solid[c] = s >= 7 ? 1 : 0;
  }
}

__global__ void fine_kernel(const int64_t *off, const float *hits, const int *nivl, int64_t ncol, int nzf,
                            uint8_t *fine) {
  const int64_t total = ncol * nzf;
  for (int64_t x = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; x < total; x += (int64_t)gridDim.x * blockDim.x) {
    const int64_t col = x / nzf;
    const int k = (int)(x % nzf);
    const int *iv = (const int *)(hits + off[col]);
    uint8_t v = 0;
    for (int e = 0; e < nivl[col]; e++)
      if (k >= iv[2 * e] && k <= iv[2 * e + 1]) { v = 1; break; }
    fine[x] = v;
  }
}

static unsigned grid_for(int64_t n, int64_t cap = 152 * 32) {
  int64_t b = (n + 255) / 256;
  if (b > cap) b = cap;
  return (unsigned)(b < 1 ? 1 : b);
}

#define ABX_CK(x) do { cudaError_t e_ = (x); if (e_ != cudaSuccess) { rc = e_; goto done; } } while (0)

cudaError_t run_voxelizer(const VoxJob &job, VoxOut &out, cudaStream_t st) {
  cudaError_t rc = cudaSuccess;
  const int nxf = 3 * job.nx, nyf = 3 * job.ny, nzf = 3 * job.nz;
  const int64_t ncol = (int64_t)nxf * nyf, ntri = job.ntri;
  TriRec *rec = nullptr;
  int64_t *pre = nullptr, *off = nullptr, *tmp = nullptr;
  uint32_t *cnt = nullptr, *cursor = nullptr;
  float *hits = nullptr;
  int *nivl = nullptr;
  int64_t W = 0, H = 0;
  const int64_t tmp_n = (ncol > ntri ? ncol : ntri) / kScanTile + 2;
  ABX_CK(cudaMallocAsync((void **)&rec, sizeof(TriRec) * (ntri > 0 ? ntri : 1), st));
  ABX_CK(cudaMallocAsync((void **)&pre, sizeof(int64_t) * (ntri + 1), st));
  ABX_CK(cudaMallocAsync((void **)&tmp, sizeof(int64_t) * tmp_n, st));
  ABX_CK(cudaMallocAsync((void **)&cnt, sizeof(uint32_t) * ncol, st));
  ABX_CK(cudaMallocAsync((void **)&cursor, sizeof(uint32_t) * ncol, st));
  ABX_CK(cudaMallocAsync((void **)&off, sizeof(int64_t) * (ncol + 1), st));
  ABX_CK(cudaMallocAsync((void **)&nivl, sizeof(int) * ncol, st));
  ABX_CK(cudaMemsetAsync(cnt, 0, sizeof(uint32_t) * ncol, st));
  ABX_CK(cudaMemsetAsync(cursor, 0, sizeof(uint32_t) * ncol, st));
  if (ntri > 0) {
    tri_setup_kernel<<<grid_for(ntri), 256, 0, st>>>(job.tris, ntri, job.origin[0], job.origin[1], job.origin[2],
                                                      job.hf, nxf, nyf, rec, pre);
    ABX_CK(cudaGetLastError());
    // in-place exclusive scan of the per-triangle counts
    ABX_CK(scan_exclusive<int64_t>(pre, ntri, pre, tmp, st));
    ABX_CK(cudaMemcpyAsync(&W, pre + ntri, sizeof(int64_t), cudaMemcpyDeviceToHost, st));
    ABX_CK(cudaStreamSynchronize(st));
    if (W > 0) {
      hits_kernel<false><<<grid_for(W), 256, 0, st>>>(rec, pre, ntri, W, job.hf, nyf, cnt, nullptr, nullptr, nullptr);
      ABX_CK(cudaGetLastError());
    }
  }
  ABX_CK(scan_exclusive<uint32_t>(cnt, ncol, off, tmp, st));
  ABX_CK(cudaMemcpyAsync(&H, off + ncol, sizeof(int64_t), cudaMemcpyDeviceToHost, st));
  ABX_CK(cudaStreamSynchronize(st));
  ABX_CK(cudaMallocAsync((void **)&hits, sizeof(float) * (H > 0 ? H : 1), st));
  if (W > 0) {
    hits_kernel<true><<<grid_for(W), 256, 0, st>>>(rec, pre, ntri, W, job.hf, nyf, cnt, off, cursor, hits);
    ABX_CK(cudaGetLastError());
  }
  columns_kernel<<<grid_for(ncol), 256, 0, st>>>(off, ncol, hits, job.hf, nzf, job.kf, nivl, out.slice);
  ABX_CK(cudaGetLastError());
  downsample_kernel<<<grid_for((int64_t)job.nx * job.ny * job.nz), 256, 0, st>>>(off, hits, nivl, job.nx, job.ny,
                                                                                   job.nz, out.solid);
  ABX_CK(cudaGetLastError());
  if (out.fine) {
    fine_kernel<<<grid_for(ncol * nzf), 256, 0, st>>>(off, hits, nivl, ncol, nzf, out.fine);
    ABX_CK(cudaGetLastError());
  }
  ABX_CK(cudaStreamSynchronize(st));
  // kernels: setup, 2 scans of 3, count, scatter, columns, downsample (+ fine)
  out.launches = 1 + 3 + (W > 0 ? 2 : 0) + 3 + 2 + (out.fine ? 1 : 0);
  out.d2h_bytes = 2 * sizeof(int64_t);
done:
  cudaFreeAsync(rec, st); cudaFreeAsync(pre, st); cudaFreeAsync(tmp, st); cudaFreeAsync(cnt, st);
  cudaFreeAsync(cursor, st); cudaFreeAsync(off, st); cudaFreeAsync(nivl, st); cudaFreeAsync(hits, st);
  return rc;
}

// ------------------------------------------------------------------ voxelizer without device allocation
// For callers that cannot allocate device memory themselves (see
// abx_voxelize_static in include/airbox.h).  Same kernels as run_voxelizer;
// the scratch lives in this fixed device array instead of cudaMallocAsync.
constexpr size_t kStaticScratchBytes = 32u << 20;   // 32 MiB, held by every GPU that loads the library
static __device__ __align__(256) unsigned char g_vox_scratch[kStaticScratchBytes];

static std::mutex g_scratch_mu;
// Device address of g_vox_scratch per device ordinal, and the id of the context it was resolved in.  A
// cudaDeviceReset (or any other end of the primary context) loads the module again at a new address, so the
// cached address is used only while the current context is the one it came from; otherwise, and after any
// failed call, it is resolved again.
struct ScratchSlot {
  void *addr = nullptr;
  unsigned long long ctx = 0;
};
static ScratchSlot g_scratch_slot[256];

// Unique id of the calling thread's current context (0 when it cannot be read): cuCtxGetCurrent and
// cuCtxGetId through the runtime's driver entry points (no link against libcuda).
static unsigned long long current_context_id() {
  using GetCurrent = CUresult (*)(CUcontext *);
  using GetId = CUresult (*)(CUcontext, unsigned long long *);
  static GetCurrent get_current = nullptr;
  static GetId get_id = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void *p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &p, 4000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      get_current = (GetCurrent)p;
    p = nullptr;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      get_id = (GetId)p;
  });
  if (!get_current || !get_id) return 0;
  CUcontext c = nullptr;
  unsigned long long id = 0;
  if (get_current(&c) != CUDA_SUCCESS || !c || get_id(c, &id) != CUDA_SUCCESS) return 0;
  return id;
}

static size_t align256(size_t v) { return (v + 255) / 256 * 256; }

int voxelize_static(const float *d_tris, size_t nfloats, const double origin[3], double h, int nx, int ny, int nz,
                    uint8_t *d_vox, cudaStream_t st, char *msg, size_t msg_len) {
  auto err = [&](int code, const char *fmt, long long a, long long b) {
    snprintf(msg, msg_len, fmt, a, b);
    return code;
  };
  if ((!d_tris && nfloats) || !d_vox || !origin || nx <= 0 || ny <= 0 || nz <= 0 || !(h > 0))
    return err(20, "voxelize_static: bad argument (%lld, %lld)", (long long)nfloats, (long long)nx);
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess || dev < 0 || dev >= 256) return err(21, "voxelize_static: no current CUDA device (%lld, %lld)", e, dev);
  // cudaSetDevice makes the device's primary context current (initialising it if needed), so that its id
  // can be read; no allocation is involved
  e = cudaSetDevice(dev);
  if (e != cudaSuccess) return err(21, "voxelize_static: cudaSetDevice failed (error %lld, device %lld)", e, dev);
  const unsigned long long ctx = current_context_id();
  void *base = nullptr;
  {
    std::lock_guard<std::mutex> lock(g_scratch_mu);
    ScratchSlot &slot = g_scratch_slot[dev];
    if (!slot.addr || ctx == 0 || slot.ctx != ctx) {
      // the symbol's name is only a host-side stand-in: resolve its device address with the device current,
      // once per device and context
      slot.addr = nullptr;
      e = cudaGetSymbolAddress(&slot.addr, g_vox_scratch);
      if (e != cudaSuccess) {
        slot.addr = nullptr;
        return err(21, "voxelize_static: cudaGetSymbolAddress failed (error %lld, device %lld)", e, dev);
      }
      slot.ctx = ctx;
    }
    base = slot.addr;
  }
  // any failure below drops the cached address, so that the next call resolves it again
  auto drop = [&](int rc) {
    if (rc) {
      std::lock_guard<std::mutex> lock(g_scratch_mu);
      g_scratch_slot[dev].addr = nullptr;
    }
    return rc;
  };
  const int64_t ncol = (int64_t)nx * ny, ntri = (int64_t)(nfloats / 9);
  const int64_t tmp_n = (ncol > ntri ? ncol : ntri) / kScanTile + 2;
  // fixed part of the scratch: triangle records, prefix sums, column counters and offsets
  size_t o = 0;
  const size_t o_rec = o;    o += align256(sizeof(TriRec) * (size_t)(ntri > 0 ? ntri : 1));
  const size_t o_pre = o;    o += align256(sizeof(int64_t) * (size_t)(ntri + 1));
  const size_t o_tmp = o;    o += align256(sizeof(int64_t) * (size_t)tmp_n);
  const size_t o_cnt = o;    o += align256(sizeof(uint32_t) * (size_t)ncol);
  const size_t o_cur = o;    o += align256(sizeof(uint32_t) * (size_t)ncol);
  const size_t o_off = o;    o += align256(sizeof(int64_t) * (size_t)(ncol + 1));
  const size_t o_niv = o;    o += align256(sizeof(int) * (size_t)ncol);
  const size_t o_sli = o;    o += align256((size_t)ncol);
  const size_t o_hit = o;
  if (o_hit > kStaticScratchBytes)
    return err(20, "voxelize_static: this grid and mesh need %lld bytes of scratch before the hits; the library holds %lld",
               (long long)o_hit, (long long)kStaticScratchBytes);
  unsigned char *S = (unsigned char *)base;
  TriRec *rec = (TriRec *)(S + o_rec);
  int64_t *pre = (int64_t *)(S + o_pre), *tmp = (int64_t *)(S + o_tmp), *off = (int64_t *)(S + o_off);
  uint32_t *cnt = (uint32_t *)(S + o_cnt), *cursor = (uint32_t *)(S + o_cur);
  int *nivl = (int *)(S + o_niv);
  uint8_t *slice = (uint8_t *)(S + o_sli);
  float *hits = (float *)(S + o_hit);
  int64_t W = 0, H = 0;
#define ABX_SC(x) do { cudaError_t e_ = (x); if (e_ != cudaSuccess) return drop(err(21, "voxelize_static: CUDA error %lld at step %lld", e_, __LINE__)); } while (0)
  // the scratch keeps the previous call's contents: zero what the passes accumulate into
  ABX_SC(cudaMemsetAsync(cnt, 0, sizeof(uint32_t) * (size_t)ncol, st));
  ABX_SC(cudaMemsetAsync(cursor, 0, sizeof(uint32_t) * (size_t)ncol, st));
  if (ntri > 0) {
    tri_setup_kernel<<<grid_for(ntri), 256, 0, st>>>(d_tris, ntri, origin[0], origin[1], origin[2], h, nx, ny, rec, pre);
    ABX_SC(cudaGetLastError());
    ABX_SC(scan_exclusive<int64_t>(pre, ntri, pre, tmp, st));
    ABX_SC(cudaMemcpyAsync(&W, pre + ntri, sizeof(int64_t), cudaMemcpyDeviceToHost, st));
    ABX_SC(cudaStreamSynchronize(st));
    if (W > 0) {
      hits_kernel<false><<<grid_for(W), 256, 0, st>>>(rec, pre, ntri, W, h, ny, cnt, nullptr, nullptr, nullptr);
      ABX_SC(cudaGetLastError());
    }
  }
  ABX_SC(scan_exclusive<uint32_t>(cnt, ncol, off, tmp, st));
  ABX_SC(cudaMemcpyAsync(&H, off + ncol, sizeof(int64_t), cudaMemcpyDeviceToHost, st));
  ABX_SC(cudaStreamSynchronize(st));
  if (o_hit + sizeof(float) * (size_t)H > kStaticScratchBytes)
    return err(20, "voxelize_static: %lld surface hits need more scratch than the library holds (%lld bytes)", (long long)H,
               (long long)kStaticScratchBytes);
  if (W > 0) {
    hits_kernel<true><<<grid_for(W), 256, 0, st>>>(rec, pre, ntri, W, h, ny, cnt, off, cursor, hits);
    ABX_SC(cudaGetLastError());
  }
  columns_kernel<<<grid_for(ncol), 256, 0, st>>>(off, ncol, hits, h, nz, 0, nivl, slice);
  ABX_SC(cudaGetLastError());
  fine_kernel<<<grid_for(ncol * nz), 256, 0, st>>>(off, hits, nivl, ncol, nz, d_vox);
  ABX_SC(cudaGetLastError());
  ABX_SC(cudaStreamSynchronize(st));
#undef ABX_SC
  return 0;
}

}  // namespace abx
