// nn.cu - layer kernels of the warm-start network (a small 3-D convolutional
// encoder-decoder), forward and backward, float32, tensors [B][C][D][H][W]
// with W fastest (D, H, W run along the grid's x, y, z).
//
//   conv3d       3x3x3, padding 1, stride 1 or 2, bias, optional ReLU; with
//                TRANS the same kernel computes the data gradient of a
//                stride-1 convolution (flipped, transposed weights)
//   conv3d_bwd   ReLU mask, data gradient of a stride-2 convolution (gather
//                form), weight and bias gradients (voxel range split over
//                blocks, partial sums reduced in a fixed order)
//   upsample2    nearest-neighbour x2 and its adjoint
//   axpy         skip connections
//   mse          weighted mean squared error and its gradient
//   adam         parameter update
//
// Every reduction runs in a fixed order: the results do not depend on
// scheduling.  No counterpart in the reference (it has no learned part).
#include <math.h>
#include <stdint.h>

#include <algorithm>

#include "lbm_iface.h"

namespace abx {

constexpr int kCo = 8;           // output channels per thread
constexpr int kCiChunk = 32;     // input channels staged in shared memory at a time
constexpr int kConvThreads = 128;

// y[b][co][o] (+)= bias[co] + sum_{ci,k} w[co][ci][k] * x[b][ci][o*s + k - 1], ReLU optional.
// TRANS (stride 1 only): y[b][c][p] (+)= sum_{c',k} w[c'][c][26-k] * x[b][c'][p + k - 1], i.e. the data
// gradient of the convolution whose weights are w (Cin/Cout here are that convolution's Cout/Cin).
// One thread: one output voxel x kCo output channels; the weights of kCiChunk input channels for the
// block's channel group sit in shared memory as [ci][k][kCo] (two 128-bit loads per tap).
template <bool TRANS>
__global__ void __launch_bounds__(kConvThreads) conv3d_kernel(const float *__restrict__ x, const float *__restrict__ w,
                                                              const float *__restrict__ bias, float *__restrict__ y,
                                                              int Cin, int Cout, int D, int H, int W, int s, int relu,
                                                              int accum) {
  __shared__ __align__(16) float ws[kCiChunk * 27 * kCo];
  const int Do = (D - 1) / s + 1, Ho = (H - 1) / s + 1, Wo = (W - 1) / s + 1;
  const int Vo = Do * Ho * Wo, Vi = D * H * W;
  const int b = blockIdx.z, co0 = blockIdx.y * kCo;
  const int nco = min(kCo, Cout - co0);
  const int v = blockIdx.x * blockDim.x + threadIdx.x;
  const bool live = v < Vo;
  int ox = 0, oy = 0, oz = 0;
  if (live) { ox = v % Wo; oy = (v / Wo) % Ho; oz = v / (Wo * Ho); }
  // taps inside the volume (bit k) and the input index of the centre tap
  uint32_t valid = 0;
#pragma unroll
  for (int k = 0; k < 27; k++) {
    const int iz = oz * s + k / 9 - 1, iy = oy * s + (k / 3) % 3 - 1, ix = ox * s + k % 3 - 1;
    if (iz >= 0 && iz < D && iy >= 0 && iy < H && ix >= 0 && ix < W) valid |= 1u << k;
  }
  const int centre = ((oz * s) * H + oy * s) * W + ox * s;
  float acc[kCo];
#pragma unroll
  for (int c = 0; c < kCo; c++) acc[c] = 0.0f;
  const float *xb = x + (int64_t)b * Cin * Vi;
  for (int ci0 = 0; ci0 < Cin; ci0 += kCiChunk) {
    const int nci = min(kCiChunk, Cin - ci0);
    __syncthreads();
    for (int i = threadIdx.x; i < nci * 27 * kCo; i += blockDim.x) {
      const int c = i % kCo, k = (i / kCo) % 27, ci = ci0 + i / (kCo * 27);
      float wv = 0.0f;
      if (c < nco) {
        if (TRANS) wv = w[((int64_t)ci * Cout + co0 + c) * 27 + 26 - k];
        else wv = w[((int64_t)(co0 + c) * Cin + ci) * 27 + k];
      }
      ws[i] = wv;
    }
    __syncthreads();
    if (!live) continue;
    for (int cc = 0; cc < nci; cc++) {
      const float *xc = xb + (int64_t)(ci0 + cc) * Vi + centre;
      const float4 *wc = reinterpret_cast<const float4 *>(ws + cc * 27 * kCo);
#pragma unroll
      for (int k = 0; k < 27; k++) {
        if (!(valid >> k & 1u)) continue;
        const float xv = __ldg(xc + ((k / 9 - 1) * H + ((k / 3) % 3 - 1)) * W + (k % 3 - 1));
        const float4 w0 = wc[2 * k], w1 = wc[2 * k + 1];
        acc[0] = fmaf(w0.x, xv, acc[0]); acc[1] = fmaf(w0.y, xv, acc[1]);
        acc[2] = fmaf(w0.z, xv, acc[2]); acc[3] = fmaf(w0.w, xv, acc[3]);
        acc[4] = fmaf(w1.x, xv, acc[4]); acc[5] = fmaf(w1.y, xv, acc[5]);
        acc[6] = fmaf(w1.z, xv, acc[6]); acc[7] = fmaf(w1.w, xv, acc[7]);
      }
    }
  }
  if (!live) return;
  float *yb = y + (int64_t)b * Cout * Vo + v;
#pragma unroll
  for (int c = 0; c < kCo; c++) {
    if (c >= nco) break;
    float r = acc[c] + (bias ? bias[co0 + c] : 0.0f);
    if (relu && r < 0.0f) r = 0.0f;
    float *o = yb + (int64_t)(co0 + c) * Vo;
    *o = accum ? *o + r : r;
  }
}

// dy <- dy * (y > 0) in place (ReLU adjoint)
__global__ void relu_bwd_kernel(const float *__restrict__ y, float *__restrict__ dy, int64_t n) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    if (!(y[i] > 0.0f)) dy[i] = 0.0f;
}

// Data gradient of a strided convolution, gather form:
// dx[b][ci][p] (+)= sum_{co,k} w[co][ci][k] * dy[b][co][(p + 1 - k)/s] over the k where that output exists.
// One thread: one input voxel x kCo input channels.
__global__ void __launch_bounds__(kConvThreads) conv3d_bwd_data_kernel(const float *__restrict__ dy,
                                                                       const float *__restrict__ w,
                                                                       float *__restrict__ dx, int Cin, int Cout, int D,
                                                                       int H, int W, int s, int accum) {
  const int Do = (D - 1) / s + 1, Ho = (H - 1) / s + 1, Wo = (W - 1) / s + 1;
  const int Vo = Do * Ho * Wo, Vi = D * H * W;
  const int b = blockIdx.z, ci0 = blockIdx.y * kCo;
  const int nci = min(kCo, Cin - ci0);
  const int v = blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= Vi) return;
  const int ix = v % W, iy = (v / W) % H, iz = v / (W * H);
  const float *dyb = dy + (int64_t)b * Cout * Vo;
  float acc[kCo];
#pragma unroll
  for (int c = 0; c < kCo; c++) acc[c] = 0.0f;
  for (int k = 0; k < 27; k++) {
    const int tz = iz + 1 - k / 9, ty = iy + 1 - (k / 3) % 3, tx = ix + 1 - k % 3;
    if (tz < 0 || ty < 0 || tx < 0 || tz % s || ty % s || tx % s) continue;
    const int oz = tz / s, oy = ty / s, ox = tx / s;
    if (oz >= Do || oy >= Ho || ox >= Wo) continue;
    const int o = (oz * Ho + oy) * Wo + ox;
    for (int co = 0; co < Cout; co++) {
      const float g = dyb[(int64_t)co * Vo + o];
      const float *wk = w + ((int64_t)co * Cin + ci0) * 27 + k;
#pragma unroll
      for (int c = 0; c < kCo; c++)
        if (c < nci) acc[c] = fmaf(wk[c * 27], g, acc[c]);
    }
  }
#pragma unroll
  for (int c = 0; c < kCo; c++) {
    if (c >= nci) break;
    float *o = dx + ((int64_t)b * Cin + ci0 + c) * Vi + v;
    *o = accum ? *o + acc[c] : acc[c];
  }
}

// Weight and bias gradients, partial sums over a slice of the output voxels:
// part[split][co][ci][0..26] = sum_{b, o in slice} dy[b][co][o] * x[b][ci][o*s + k - 1],
// part[split][co][ci][27]    = sum dy[b][co][o] (the bias gradient; used from ci = 0).
// Grid (Cin, Cout, splits); the block reduction runs in a fixed order.
__global__ void __launch_bounds__(256) conv3d_wgrad_kernel(const float *__restrict__ x, const float *__restrict__ dy,
                                                           float *__restrict__ part, int B, int Cin, int Cout, int D,
                                                           int H, int W, int s) {
  __shared__ float red[28][8];
  const int ci = blockIdx.x, co = blockIdx.y, split = blockIdx.z, nsplit = gridDim.z;
  const int Do = (D - 1) / s + 1, Ho = (H - 1) / s + 1, Wo = (W - 1) / s + 1;
  const int Vo = Do * Ho * Wo, Vi = D * H * W;
  const int lo = (int)((int64_t)Vo * split / nsplit), hi = (int)((int64_t)Vo * (split + 1) / nsplit);
  float acc[28];
#pragma unroll
  for (int k = 0; k < 28; k++) acc[k] = 0.0f;
  for (int b = 0; b < B; b++) {
    const float *dyc = dy + ((int64_t)b * Cout + co) * Vo;
    const float *xc = x + ((int64_t)b * Cin + ci) * Vi;
    for (int o = lo + threadIdx.x; o < hi; o += blockDim.x) {
      const float g = dyc[o];
      if (g == 0.0f) continue;
      acc[27] += g;
      const int ox = o % Wo, oy = (o / Wo) % Ho, oz = o / (Wo * Ho);
      const int cz = oz * s, cy = oy * s, cx = ox * s;
      const float *xp = xc + (cz * H + cy) * W + cx;
#pragma unroll
      for (int k = 0; k < 27; k++) {
        const int dz = k / 9 - 1, dyy = (k / 3) % 3 - 1, dxx = k % 3 - 1;
        if (cz + dz < 0 || cz + dz >= D || cy + dyy < 0 || cy + dyy >= H || cx + dxx < 0 || cx + dxx >= W) continue;
        acc[k] = fmaf(g, __ldg(xp + (dz * H + dyy) * W + dxx), acc[k]);
      }
    }
  }
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
  for (int k = 0; k < 28; k++) {
    float v = acc[k];
    for (int off = 16; off > 0; off >>= 1) v += __shfl_xor_sync(0xffffffffu, v, off);
    if (lane == 0) red[k][wid] = v;
  }
  __syncthreads();
  if (threadIdx.x < 28) {
    float t = 0.0f;
    for (int i = 0; i < nw; i++) t += red[threadIdx.x][i];
    part[(((int64_t)split * Cout + co) * Cin + ci) * 28 + threadIdx.x] = t;
  }
}

// dw[co][ci][k] = sum over splits; db[co] = sum over splits of the ci = 0 entry 27.
__global__ void wgrad_reduce_kernel(const float *__restrict__ part, float *__restrict__ dw, float *__restrict__ db,
                                    int Cin, int Cout, int nsplit) {
  const int n = Cout * Cin * 28;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const int k = i % 28, ci = (i / 28) % Cin, co = i / (28 * Cin);
    float t = 0.0f;
    for (int sp = 0; sp < nsplit; sp++) t += part[(int64_t)sp * n + i];
    if (k < 27) dw[((int64_t)co * Cin + ci) * 27 + k] = t;
    else if (ci == 0) db[co] = t;
  }
}

// y[bc][z][y][x] = x[bc][z/2][y/2][x/2]  (D, H, W: output size, even)
__global__ void upsample2_kernel(const float *__restrict__ x, float *__restrict__ y, int64_t BC, int D, int H, int W) {
  const int64_t V = (int64_t)D * H * W, n = BC * V;
  const int h = H / 2, w2 = W / 2;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t bc = i / V;
    const int v = (int)(i % V);
    const int xx = v % W, yy = (v / W) % H, zz = v / (W * H);
    y[i] = x[bc * (V / 8) + ((zz >> 1) * h + (yy >> 1)) * w2 + (xx >> 1)];
  }
}
// dx (+)= sum over each 2x2x2 block of dy (D, H, W: size of x)
__global__ void upsample2_bwd_kernel(const float *__restrict__ dy, float *__restrict__ dx, int64_t BC, int D, int H,
                                     int W, int accum) {
  const int64_t V = (int64_t)D * H * W, n = BC * V;
  const int H2 = 2 * H, W2 = 2 * W;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t bc = i / V;
    const int v = (int)(i % V);
    const int xx = v % W, yy = (v / W) % H, zz = v / (W * H);
    const float *d = dy + bc * V * 8;
    float t = 0.0f;
    for (int a = 0; a < 2; a++)
      for (int bb = 0; bb < 2; bb++)
        for (int c = 0; c < 2; c++) t += d[((2 * zz + a) * H2 + (2 * yy + bb)) * W2 + (2 * xx + c)];
    dx[i] = accum ? dx[i] + t : t;
  }
}

__global__ void axpy_kernel(float *__restrict__ y, const float *__restrict__ x, float a, int64_t n) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    y[i] += a * x[i];
}

// Weighted squared error: part[block] = scale * sum m[b][v] (pred - target)^2 over the block's share;
// grad = 2 scale m (pred - target) (optional).  The caller sums part[] in order.
__global__ void mse_kernel(const float *__restrict__ pred, const float *__restrict__ target,
                           const float *__restrict__ mask, float *__restrict__ grad, double *__restrict__ part, int C,
                           int64_t V, int64_t n, double scale) {
  __shared__ double sh[32];
  double local = 0.0;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t b = i / (C * V), v = i % V;
    const float m = mask[b * V + v];
    const float d = pred[i] - target[i];
    local += (double)m * d * d;
    if (grad) grad[i] = (float)(2.0 * scale * m * d);
  }
  for (int off = 16; off > 0; off >>= 1) local += __shfl_xor_sync(0xffffffffu, local, off);
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = local;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int i = 0; i < (int)(blockDim.x >> 5); i++) t += sh[i];
    part[blockIdx.x] = t * scale;
  }
}

__global__ void adam_kernel(float *__restrict__ p, const float *__restrict__ g, float *__restrict__ m,
                            float *__restrict__ v, int64_t n, float lr, float b1, float b2, float eps, float c1,
                            float c2) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const float gi = g[i];
    const float mi = b1 * m[i] + (1.0f - b1) * gi, vi = b2 * v[i] + (1.0f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    p[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
  }
}

static unsigned blocks_for(int64_t n) {
  int64_t b = (n + 255) / 256;
  if (b > 152 * 16) b = 152 * 16;
  return (unsigned)(b < 1 ? 1 : b);
}

static bool dims_ok(int64_t a, int64_t b, int64_t c) { return a > 0 && b > 0 && c > 0 && a * b * c < (1ll << 31); }

cudaError_t nn_conv3d(const float *x, const float *w, const float *b, float *y, int B, int Cin, int Cout, int D,
                      int H, int W, int s, int relu, int accum, cudaStream_t st) {
  if (!dims_ok(D, H, W) || B <= 0 || B > 65535 || Cin <= 0 || Cout <= 0 || (s != 1 && s != 2))
    return cudaErrorInvalidValue;
  const int Do = (D - 1) / s + 1, Ho = (H - 1) / s + 1, Wo = (W - 1) / s + 1;
  const int Vo = Do * Ho * Wo;
  const dim3 grid((Vo + kConvThreads - 1) / kConvThreads, (Cout + kCo - 1) / kCo, B);
  conv3d_kernel<false><<<grid, kConvThreads, 0, st>>>(x, w, b, y, Cin, Cout, D, H, W, s, relu, accum);
  return cudaGetLastError();
}

int64_t nn_wgrad_scratch_floats(int Cin, int Cout, int Vo) {
  int64_t nsplit = (152 * 4 + (int64_t)Cin * Cout - 1) / ((int64_t)Cin * Cout);
  nsplit = std::min<int64_t>(std::max<int64_t>(nsplit, 1), std::max(1, Vo / 1024));
  return nsplit * Cin * Cout * 28;
}

cudaError_t nn_conv3d_backward(const float *x, const float *w, const float *y, float *dy, float *dx, float *dw,
                               float *db, float *part, int64_t part_floats, int B, int Cin, int Cout, int D, int H,
                               int W, int s, int relu, int accum_dx, cudaStream_t st) {
  if (!dims_ok(D, H, W) || B <= 0 || B > 65535 || Cin <= 0 || Cout <= 0 || (s != 1 && s != 2))
    return cudaErrorInvalidValue;
  const int Do = (D - 1) / s + 1, Ho = (H - 1) / s + 1, Wo = (W - 1) / s + 1;
  const int Vo = Do * Ho * Wo, Vi = D * H * W;
  if (relu) relu_bwd_kernel<<<blocks_for((int64_t)B * Cout * Vo), 256, 0, st>>>(y, dy, (int64_t)B * Cout * Vo);
  if (dx) {
    const dim3 grid((Vi + kConvThreads - 1) / kConvThreads, (Cin + kCo - 1) / kCo, B);
    if (s == 1) conv3d_kernel<true><<<grid, kConvThreads, 0, st>>>(dy, w, nullptr, dx, Cout, Cin, D, H, W, 1, 0, accum_dx);
    else conv3d_bwd_data_kernel<<<grid, kConvThreads, 0, st>>>(dy, w, dx, Cin, Cout, D, H, W, s, accum_dx);
  }
  // enough blocks to fill the GPU: the voxel range is split when (Cin, Cout) pairs are few
  const int64_t want = nn_wgrad_scratch_floats(Cin, Cout, Vo) / ((int64_t)Cin * Cout * 28);
  const int64_t nsplit = std::min<int64_t>(want, part_floats / ((int64_t)Cin * Cout * 28));
  if (nsplit < 1) return cudaErrorInvalidValue;
  conv3d_wgrad_kernel<<<dim3(Cin, Cout, (unsigned)nsplit), 256, 0, st>>>(x, dy, part, B, Cin, Cout, D, H, W, s);
  wgrad_reduce_kernel<<<blocks_for((int64_t)Cin * Cout * 28), 256, 0, st>>>(part, dw, db, Cin, Cout, (int)nsplit);
  return cudaGetLastError();
}

cudaError_t nn_upsample2(const float *x, float *y, int64_t BC, int D, int H, int W, cudaStream_t st) {
  upsample2_kernel<<<blocks_for(BC * D * H * W), 256, 0, st>>>(x, y, BC, D, H, W);
  return cudaGetLastError();
}
cudaError_t nn_upsample2_backward(const float *dy, float *dx, int64_t BC, int D, int H, int W, int accum,
                                  cudaStream_t st) {
  upsample2_bwd_kernel<<<blocks_for(BC * D * H * W), 256, 0, st>>>(dy, dx, BC, D, H, W, accum);
  return cudaGetLastError();
}

cudaError_t nn_axpy(float *y, const float *x, float a, int64_t n, cudaStream_t st) {
  axpy_kernel<<<blocks_for(n), 256, 0, st>>>(y, x, a, n);
  return cudaGetLastError();
}

cudaError_t nn_mse(const float *pred, const float *target, const float *mask, float *grad, double *part, int nparts,
                   int B, int C, int64_t V, double scale, cudaStream_t st) {
  mse_kernel<<<nparts, 256, 0, st>>>(pred, target, mask, grad, part, C, V, (int64_t)B * C * V, scale);
  return cudaGetLastError();
}

cudaError_t nn_adam(float *p, const float *g, float *m, float *v, int64_t n, float lr, float b1, float b2, float eps,
                    int t, cudaStream_t st) {
  const float c1 = 1.0f - powf(b1, (float)t), c2 = 1.0f - powf(b2, (float)t);
  adam_kernel<<<blocks_for(n), 256, 0, st>>>(p, g, m, v, n, lr, b1, b2, eps, c1, c2);
  return cudaGetLastError();
}

}  // namespace abx
