// net.h - the warm-start network on the host side: a 3-D convolutional
// encoder-decoder on an R^3 resampling of the grid, its device-resident
// training set, the training loop (Adam) and inference.  All arithmetic runs
// in the kernels of nn.cu / warmstart.cu.
//
// Architecture (levels L, channels c_l = base << l):
//   encoder  level 0: conv(9 -> c0), conv(c0 -> c0)
//            level l: conv stride 2 (c_{l-1} -> c_l), conv(c_l -> c_l)
//   decoder  level l = L-2 .. 0: upsample x2, conv(c_{l+1} -> c_l),
//            + encoder level l output (skip), conv(c_l -> c_l)
//   head     conv(c0 -> 4), no activation
// Every conv is 3x3x3 with padding 1 and a ReLU except the head.
// Input channels: fluid, inlet, outlet, filter fraction, wall distance, K,
// grid extent (3), optionally the voxel's coordinates (3); output: u / u0 (3) and (rho - 1) / (5 u0^2).
#pragma once
#include <cuda_runtime_api.h>
#include <stdint.h>

#include <string>
#include <vector>

#include "lbm_iface.h"

namespace abx {

class WarmNet {
 public:
  static constexpr int kGeomIn = 9, kOut = 4;   // geometry channels, output channels

  struct Conv { int cin, cout, stride, relu; int64_t w_off, b_off; };
  struct Tensor { int C, D; int64_t off; };           // C x D^3 floats per sample, at cap_B * off
  struct Node { int kind, in, in2, out, conv; };      // kind: 0 conv, 1 upsample, 2 add
  struct Sample { float *buf = nullptr; double msum = 0; };   // [n_in V | 4 V | V]

  int R = 0, base = 0, levels = 0, device = 0;
  int n_in = kGeomIn;                                 // + 3 voxel-coordinate channels when enabled
  cudaStream_t st = nullptr;
  std::vector<Conv> convs;
  std::vector<Tensor> tensors;
  std::vector<Node> nodes;
  int64_t n_params = 0, per_sample = 0;
  float *d_p = nullptr, *d_g = nullptr, *d_m = nullptr, *d_v = nullptr;
  int adam_t = 0;
  int cap_B = 0;
  float *d_act = nullptr, *d_grad = nullptr, *d_bt = nullptr, *d_bm = nullptr, *d_part = nullptr;
  int64_t part_floats = 0;
  double *d_mse = nullptr;
  int mse_parts = 0;
  int *d_seed = nullptr;                              // 2 x R^3 jump-flood scratch
  std::vector<Sample> samples;
  std::string err;
  // convolutions on the tensor cores (nn_tc.cu) where a layer's channels allow (<= 128 in and out), else the
  // float32 kernels of nn.cu; tcs is sized for tcs_B samples
  bool use_tc = false;
  TcScratch tcs;
  int tcs_B = 0;
  bool tc_layer(const Conv &c) const { return use_tc && c.cin <= 128 && c.cout <= 128; }
  cudaError_t tc_alloc(int B);
  void tc_free();

  ~WarmNet();
  // Builds the layer list, allocates the parameters and initialises them from `seed`.
  cudaError_t init(int R, int base, int levels, int device, uint64_t seed, bool coords = false);
  int64_t voxels() const { return (int64_t)R * R * R; }
  float *tensor(int t, int b = 0) const { return d_act + tensors[t].off * cap_B + (int64_t)b * tensors[t].C * tensors[t].D * tensors[t].D * tensors[t].D; }
  float *grad(int t, int b = 0) const { return d_grad + tensors[t].off * cap_B + (int64_t)b * tensors[t].C * tensors[t].D * tensors[t].D * tensors[t].D; }
  float *input(int b = 0) const { return tensor(0, b); }
  float *output(int b = 0) const { return tensor((int)tensors.size() - 1, b); }

  cudaError_t ensure_batch(int B);
  cudaError_t forward(int B);
  // loss = scale * sum m (pred - t)^2 (summed on the host in a fixed order); with `backward` the
  // parameter gradient lands in d_g.
  cudaError_t loss(int B, const float *t, const float *m, double scale, bool backward, double *out);
  cudaError_t features(const GridDesc &g, float K, float *dst);
  cudaError_t add_sample(const GridDesc &g, float K, int storage, const void *acc, int nacc, double u0);
  // Stage sample `idx` into batch slot b (mirrored along x when flip).
  cudaError_t stage(int idx, int b, bool flip);
  cudaError_t train(int first, int count, int epochs, int batch, double lr, double lr_min, uint64_t seed, bool flip,
                    double *epoch_loss);
  cudaError_t eval_loss(int first, int count, double *out);
  void clear_samples();
};

}  // namespace abx
