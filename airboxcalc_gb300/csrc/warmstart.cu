// warmstart.cu - resampling between a simulation's padded grid and the R^3
// grid of the warm-start network, on the device:
//
//   ws_features  network input per voxel: fluid / inlet / outlet / filter
//                fraction of the voxel's footprint, distance to the nearest
//                solid voxel (jump flooding, in grid cells), the filter's K
//                and the grid's extent
//   ws_targets   training target per voxel: the time-averaged u / u0 and
//                (rho - 1) / (5 u0^2) over the footprint's fluid cells, and
//                the fluid fraction as the loss weight
//   ws_apply     warm start: the predicted field, trilinearly interpolated
//                to every fluid cell (weighted by voxel fluid fraction), as
//                equilibrium populations in the run's storage format
//
// Voxel v = (a*R + b)*R + c covers the cells whose centres lie in
// [a, a+1) * nx/R along x (b, c: y, z); an empty footprint takes the nearest
// cell.  The equilibrium is the one of cpuStep (src/engine.js:288-291).
#include <math.h>
#include <stdint.h>

#include "d3q19.cuh"
#include "lbm_iface.h"

namespace abx {

__device__ __forceinline__ void footprint(int a, int n, int R, int &i0, int &i1) {
  const double s = (double)n / R;
  i0 = (int)ceil(a * s - 0.5);
  i1 = (int)ceil((a + 1) * s - 0.5);
  if (i1 <= i0) {
    i0 = min((int)floor((a + 0.5) * s), n - 1);
    i1 = i0 + 1;
  }
  i0 = max(i0, 0);
  i1 = min(i1, n);
}

__device__ __forceinline__ uint32_t cell_mask(const GridDesc &g, int i, int j, int k) {
  return g.mask[((int64_t)i * g.ny + j) * g.nzp + k + g.kpad];
}

__global__ void features_kernel(const GridDesc g, int R, float K, float *__restrict__ out, int *__restrict__ seed) {
  const int V = R * R * R;
  for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < V; v += gridDim.x * blockDim.x) {
    const int c = v % R, b = (v / R) % R, a = v / (R * R);
    int i0, i1, j0, j1, k0, k1;
    footprint(a, g.nx, R, i0, i1);
    footprint(b, g.ny, R, j0, j1);
    footprint(c, g.nz, R, k0, k1);
    int n = 0, nf = 0, nin = 0, nout = 0, nfil = 0;
    for (int i = i0; i < i1; i++)
      for (int j = j0; j < j1; j++)
        for (int k = k0; k < k1; k++) {
          const uint32_t m = cell_mask(g, i, j, k);
          n++;
          if (!m) continue;
          nf++;
          const uint32_t cls = (m >> kClassShift) & 3u;
          nin += cls == kClsInlet;
          nout += cls == kClsOutlet;
          nfil += cls == kClsFilter;
        }
    const float inv = 1.0f / (float)n;
    out[0 * V + v] = nf * inv;
    out[1 * V + v] = nin * inv;
    out[2 * V + v] = nout * inv;
    out[3 * V + v] = nfil * inv;
    out[4 * V + v] = 0.0f;  // wall distance, filled by the jump flood
    out[5 * V + v] = K / 3.0f;
    out[6 * V + v] = g.nx / 128.0f;
    out[7 * V + v] = g.ny / 64.0f;
    out[8 * V + v] = g.nz / 128.0f;
    seed[v] = nf * 2 < n ? v : -1;  // solid voxel: its own nearest solid voxel
  }
}

__device__ __forceinline__ float vox_dist2(int v, int w, int R, float sx, float sy, float sz) {
  const float da = (float)(v / (R * R) - w / (R * R)) * sx;
  const float db = (float)((v / R) % R - (w / R) % R) * sy;
  const float dc = (float)(v % R - w % R) * sz;
  return da * da + db * db + dc * dc;
}

// One jump-flooding pass: each voxel takes the nearest of the seeds known to it and to the 26 voxels
// `step` away (ties: the smaller voxel index, so the result does not depend on scheduling).
__global__ void jfa_kernel(const int *__restrict__ in, int *__restrict__ out, int R, int step, float sx, float sy,
                           float sz) {
  const int V = R * R * R;
  for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < V; v += gridDim.x * blockDim.x) {
    const int c = v % R, b = (v / R) % R, a = v / (R * R);
    int best = in[v];
    float bd = best >= 0 ? vox_dist2(v, best, R, sx, sy, sz) : INFINITY;
    for (int da = -1; da <= 1; da++)
      for (int db = -1; db <= 1; db++)
        for (int dc = -1; dc <= 1; dc++) {
          const int aa = a + da * step, bb = b + db * step, cc = c + dc * step;
          if (aa < 0 || aa >= R || bb < 0 || bb >= R || cc < 0 || cc >= R) continue;
          const int s = in[(aa * R + bb) * R + cc];
          if (s < 0) continue;
          const float d = vox_dist2(v, s, R, sx, sy, sz);
          if (d < bd || (d == bd && s < best)) { bd = d; best = s; }
        }
    out[v] = best;
  }
}

__global__ void jfa_dist_kernel(const int *__restrict__ seed, int R, float sx, float sy, float sz,
                                float *__restrict__ dist) {
  const int V = R * R * R;
  for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < V; v += gridDim.x * blockDim.x) {
    const int s = seed[v];
    const float d = s >= 0 ? sqrtf(vox_dist2(v, s, R, sx, sy, sz)) : 40.0f;
    dist[v] = fminf(d / 20.0f, 2.0f);
  }
}

template <typename Acc>
__global__ void targets_kernel(const GridDesc g, const Acc *__restrict__ acc, double inv_n, double u0, int R,
                               float *__restrict__ t, float *__restrict__ m) {
  const int V = R * R * R;
  const double su = 1.0 / u0, sr = 1.0 / (5.0 * u0 * u0);
  for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < V; v += gridDim.x * blockDim.x) {
    const int c = v % R, b = (v / R) % R, a = v / (R * R);
    int i0, i1, j0, j1, k0, k1;
    footprint(a, g.nx, R, i0, i1);
    footprint(b, g.ny, R, j0, j1);
    footprint(c, g.nz, R, k0, k1);
    int n = 0, nf = 0;
    double s[4] = {0, 0, 0, 0};
    for (int i = i0; i < i1; i++)
      for (int j = j0; j < j1; j++)
        for (int k = k0; k < k1; k++) {
          n++;
          const int64_t p = ((int64_t)i * g.ny + j) * g.nzp + k + g.kpad;
          if (!g.mask[p]) continue;
          nf++;
          for (int q = 0; q < 4; q++) s[q] += (double)acc[(int64_t)q * g.Np + p];
        }
    if (nf) {
      const double w = inv_n / nf;
      t[0 * V + v] = (float)(s[0] * w * su);
      t[1 * V + v] = (float)(s[1] * w * su);
      t[2 * V + v] = (float)(s[2] * w * su);
      t[3 * V + v] = (float)((s[3] * w - 1.0) * sr);
    } else {
      for (int q = 0; q < 4; q++) t[q * V + v] = 0.0f;
    }
    m[v] = (float)nf / (float)n;
  }
}

// Warm start: equilibrium of the interpolated prediction on every fluid cell, in "out" form (the
// state after an even number of steps: the post-collision value of direction q at A[opp q][x]).
template <int K>
__global__ void apply_kernel(const StateArgs a, const GridDesc g, const float *__restrict__ pred,
                             const float *__restrict__ fluid, int R, double u0) {
  using S = Store<K>;
  using T = typename S::T;
  using L = typename S::L;
  T *f = (T *)a.f;
  const int V = R * R * R;
  for (int64_t n = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; n < a.ncells; n += (int64_t)gridDim.x * blockDim.x) {
    const int64_t x = a.cells[n];
    const int k = (int)(x % g.nzp - g.kpad);
    const int64_t ij = x / g.nzp;
    const int j = (int)(ij % g.ny), i = (int)(ij / g.ny);
    // voxel-space coordinates of the cell centre
    const float fa = (i + 0.5f) * R / g.nx - 0.5f, fb = (j + 0.5f) * R / g.ny - 0.5f, fc = (k + 0.5f) * R / g.nz - 0.5f;
    const int a0 = min(max((int)floorf(fa), 0), R - 2), b0 = min(max((int)floorf(fb), 0), R - 2),
              c0 = min(max((int)floorf(fc), 0), R - 2);
    const float wa = fminf(fmaxf(fa - a0, 0.0f), 1.0f), wb = fminf(fmaxf(fb - b0, 0.0f), 1.0f),
                wc = fminf(fmaxf(fc - c0, 0.0f), 1.0f);
    float p[4] = {0, 0, 0, 0}, wsum = 0.0f;
    for (int corner = 0; corner < 8; corner++) {
      const int da = corner >> 2, db = (corner >> 1) & 1, dc = corner & 1;
      const int v = ((a0 + da) * R + b0 + db) * R + c0 + dc;
      const float w = (da ? wa : 1.0f - wa) * (db ? wb : 1.0f - wb) * (dc ? wc : 1.0f - wc) * fluid[v];
      wsum += w;
      for (int q = 0; q < 4; q++) p[q] += w * pred[q * V + v];
    }
    if (wsum > 1e-6f) {
      for (int q = 0; q < 4; q++) p[q] /= wsum;
    } else {  // no fluid voxel around: the nearest voxel's prediction
      const int v = ((min(max((int)rintf(fa), 0), R - 1)) * R + min(max((int)rintf(fb), 0), R - 1)) * R +
                    min(max((int)rintf(fc), 0), R - 1);
      for (int q = 0; q < 4; q++) p[q] = pred[q * V + v];
    }
    L ux = (L)(p[0] * u0), uy = (L)(p[1] * u0), uz = (L)(p[2] * u0);
    L rho = (L)(1.0 + 5.0 * u0 * u0 * p[3]);
    // keep the start inside the lattice's stable range
    const L sp = sqrt(ux * ux + uy * uy + uz * uz), cap = (L)0.2;
    if (!(sp <= cap)) {
      const L r = sp > cap ? cap / sp : (L)0;
      ux *= r; uy *= r; uz *= r;
    }
    if (!(rho >= (L)0.9)) rho = (L)0.9;
    if (rho > (L)1.1) rho = (L)1.1;
    const L u2 = ux * ux + uy * uy + uz * uz;
#pragma unroll
    for (int q = 0; q < 19; q++) {
      const L cu = (L)cx(q) * ux + (L)cy(q) * uy + (L)cz(q) * uz;
      const L w = weight<L>(q);
      const L fe = w * rho * ((L)1 + (L)3 * cu + (L)4.5 * cu * cu - (L)1.5 * u2);
      S::st(f + (int64_t)opp(q) * a.Np + x, fe, w);
    }
  }
}

static unsigned grid_for(int64_t n) {
  int64_t b = (n + 255) / 256;
  if (b > 152 * 8) b = 152 * 8;
  return (unsigned)(b < 1 ? 1 : b);
}

cudaError_t ws_features(const GridDesc &g, int R, float K, float *out, int *seed_a, int *seed_b, cudaStream_t st) {
  const int V = R * R * R;
  features_kernel<<<grid_for(V), 256, 0, st>>>(g, R, K, out, seed_a);
  const float sx = (float)g.nx / R, sy = (float)g.ny / R, sz = (float)g.nz / R;
  int *in = seed_a, *out_s = seed_b;
  // steps R/2, R/4, ..., 1, then 1 once more
  for (int step = R / 2;; step = step > 1 ? step / 2 : 0) {
    const int s = step > 0 ? step : 1;
    jfa_kernel<<<grid_for(V), 256, 0, st>>>(in, out_s, R, s, sx, sy, sz);
    int *t = in; in = out_s; out_s = t;
    if (step == 0) break;
  }
  jfa_dist_kernel<<<grid_for(V), 256, 0, st>>>(in, R, sx, sy, sz, out + 4 * V);
  return cudaGetLastError();
}

__global__ void coords_kernel(int R, float *__restrict__ out) {
  const int V = R * R * R;
  for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < V; v += gridDim.x * blockDim.x) {
    const int c = v % R, b = (v / R) % R, a = v / (R * R);
    out[v] = (a + 0.5f) / R;
    out[V + v] = (b + 0.5f) / R;
    out[2 * V + v] = (c + 0.5f) / R;
  }
}

cudaError_t ws_coords(int R, float *out, cudaStream_t st) {
  coords_kernel<<<grid_for((int64_t)R * R * R), 256, 0, st>>>(R, out);
  return cudaGetLastError();
}

cudaError_t ws_targets(const GridDesc &g, int storage, const void *acc, int nacc, double u0, int R, float *t, float *m,
                       cudaStream_t st) {
  const double inv_n = 1.0 / (nacc > 1 ? nacc : 1);
  const int V = R * R * R;
  if (storage == kStoreF64) targets_kernel<double><<<grid_for(V), 256, 0, st>>>(g, (const double *)acc, inv_n, u0, R, t, m);
  else targets_kernel<float><<<grid_for(V), 256, 0, st>>>(g, (const float *)acc, inv_n, u0, R, t, m);
  return cudaGetLastError();
}

cudaError_t ws_apply(int storage, const StateArgs &a, const GridDesc &g, const float *pred, const float *fluid, int R,
                     double u0, cudaStream_t st) {
  const unsigned grid = grid_for(a.ncells);
  switch (storage) {
    case kStoreF32: apply_kernel<kStoreF32><<<grid, 256, 0, st>>>(a, g, pred, fluid, R, u0); break;
    case kStoreF32Exact: apply_kernel<kStoreF32Exact><<<grid, 256, 0, st>>>(a, g, pred, fluid, R, u0); break;
    case kStoreF16: apply_kernel<kStoreF16><<<grid, 256, 0, st>>>(a, g, pred, fluid, R, u0); break;
    case kStoreBF16: apply_kernel<kStoreBF16><<<grid, 256, 0, st>>>(a, g, pred, fluid, R, u0); break;
    case kStoreF64: apply_kernel<kStoreF64><<<grid, 256, 0, st>>>(a, g, pred, fluid, R, u0); break;
    default: return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

// Mirror a batch slot along x (the first spatial axis) in place, negating channel `neg` (or none when
// neg < 0): the mirrored airbox's flow.
__global__ void flip_x_kernel(float *__restrict__ t, int C, int R, int neg) {
  const int half = R / 2, plane = R * R;
  const int64_t n = (int64_t)C * half * plane;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const int ch = (int)(i / ((int64_t)half * plane));
    const int r = (int)(i % ((int64_t)half * plane));
    const int a = r / plane, bc = r % plane;
    float *base = t + (int64_t)ch * R * plane;
    const int64_t p = (int64_t)a * plane + bc, q = (int64_t)(R - 1 - a) * plane + bc;
    float u = base[p], w = base[q];
    if (ch == neg) { u = -u; w = -w; }
    base[p] = w;
    base[q] = u;
  }
}

cudaError_t ws_flip_x(float *t, int C, int R, int neg, cudaStream_t st) {
  flip_x_kernel<<<grid_for((int64_t)C * (R / 2) * R * R), 256, 0, st>>>(t, C, R, neg);
  return cudaGetLastError();
}

}  // namespace abx
