// net.cpp - host side of the warm-start network (see net.h).
#include "net.h"

#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>

namespace abx {

#define NCK(x)                          \
  do {                                  \
    cudaError_t e_ = (x);               \
    if (e_ != cudaSuccess) return e_;   \
  } while (0)

// splitmix64: a small portable generator (weights, shuffles, augmentation draws)
static uint64_t splitmix(uint64_t &s) {
  uint64_t z = (s += 0x9E3779B97F4A7C15ull);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}
static double uniform01(uint64_t &s) { return (double)(splitmix(s) >> 11) * (1.0 / 9007199254740992.0); }

WarmNet::~WarmNet() {
  cudaSetDevice(device);
  tc_free();
  cudaFree(d_p); cudaFree(d_g); cudaFree(d_m); cudaFree(d_v);
  cudaFree(d_act); cudaFree(d_grad); cudaFree(d_bt); cudaFree(d_bm); cudaFree(d_part);
  cudaFree(d_mse); cudaFree(d_seed);
  clear_samples();
  if (st) cudaStreamDestroy(st);
}

void WarmNet::clear_samples() {
  cudaSetDevice(device);
  for (auto &s : samples) cudaFree(s.buf);
  samples.clear();
}

cudaError_t WarmNet::init(int R_, int base_, int levels_, int device_, uint64_t seed, bool coords) {
  R = R_; base = base_; levels = levels_; device = device_;
  n_in = kGeomIn + (coords ? 3 : 0);
  NCK(cudaSetDevice(device));
  NCK(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
  auto add_tensor = [&](int C, int D) {
    int64_t off = tensors.empty() ? 0 : tensors.back().off + (int64_t)tensors.back().C * tensors.back().D *
                                                                 tensors.back().D * tensors.back().D;
    tensors.push_back({C, D, off});
    return (int)tensors.size() - 1;
  };
  auto add_conv = [&](int in, int cout, int stride, int relu) {
    const int cin = tensors[in].C;
    Conv c{cin, cout, stride, relu, n_params, n_params + (int64_t)cout * cin * 27};
    n_params += (int64_t)cout * cin * 27 + cout;
    convs.push_back(c);
    const int out = add_tensor(cout, (tensors[in].D - 1) / stride + 1);
    nodes.push_back({0, in, -1, out, (int)convs.size() - 1});
    return out;
  };
  auto ch = [&](int l) { return base << l; };
  int t = add_tensor(n_in, R);
  std::vector<int> skip(levels);
  for (int l = 0; l < levels; l++) {
    t = add_conv(t, ch(l), l == 0 ? 1 : 2, 1);
    t = add_conv(t, ch(l), 1, 1);
    skip[l] = t;
  }
  for (int l = levels - 2; l >= 0; l--) {
    const int u = add_tensor(tensors[t].C, tensors[t].D * 2);
    nodes.push_back({1, t, -1, u, -1});
    const int a = add_conv(u, ch(l), 1, 1);
    const int s = add_tensor(ch(l), tensors[a].D);
    nodes.push_back({2, a, skip[l], s, -1});
    t = add_conv(s, ch(l), 1, 1);
  }
  add_conv(t, kOut, 1, 0);
  per_sample = tensors.back().off + (int64_t)tensors.back().C * R * R * R;
  for (auto &T : tensors)
    if (T.D * (R / T.D) != R) return cudaErrorInvalidValue;
  // parameters: He-uniform weights (head scaled by 0.1), zero biases
  std::vector<float> h(n_params, 0.0f);
  uint64_t s = seed;
  for (size_t i = 0; i < convs.size(); i++) {
    const Conv &c = convs[i];
    double bound = std::sqrt(6.0 / (c.cin * 27.0));
    if (i + 1 == convs.size()) bound *= 0.1;
    for (int64_t k = 0; k < (int64_t)c.cout * c.cin * 27; k++) h[c.w_off + k] = (float)((2 * uniform01(s) - 1) * bound);
  }
  NCK(cudaMalloc(&d_p, sizeof(float) * n_params));
  NCK(cudaMalloc(&d_g, sizeof(float) * n_params));
  NCK(cudaMalloc(&d_m, sizeof(float) * n_params));
  NCK(cudaMalloc(&d_v, sizeof(float) * n_params));
  NCK(cudaMemcpyAsync(d_p, h.data(), sizeof(float) * n_params, cudaMemcpyHostToDevice, st));
  NCK(cudaMemsetAsync(d_m, 0, sizeof(float) * n_params, st));
  NCK(cudaMemsetAsync(d_v, 0, sizeof(float) * n_params, st));
  for (auto &n : nodes)
    if (n.kind == 0) {
      const Conv &c = convs[n.conv];
      const int Do = tensors[n.out].D;
      part_floats = std::max(part_floats, nn_wgrad_scratch_floats(c.cin, c.cout, Do * Do * Do));
    }
  NCK(cudaMalloc(&d_part, sizeof(float) * part_floats));
  mse_parts = 152 * 2;
  NCK(cudaMalloc(&d_mse, sizeof(double) * mse_parts));
  NCK(cudaMalloc(&d_seed, sizeof(int) * 2 * voxels()));
  NCK(cudaStreamSynchronize(st));
  return cudaSuccess;
}

void WarmNet::tc_free() {
  cudaFree(tcs.cl); cudaFree(tcs.w); cudaFree(tcs.xs); cudaFree(tcs.dyc); cudaFree(tcs.part); cudaFree(tcs.err);
  tcs = TcScratch{};
  tcs_B = 0;
}

cudaError_t WarmNet::tc_alloc(int B) {
  if (tcs_B >= B) return cudaSuccess;
  tc_free();
  TcNeed need;
  for (const Node &n : nodes)
    if (n.kind == 0 && tc_layer(convs[n.conv])) {
      const Conv &c = convs[n.conv];
      nn_tc_need(B, c.cin, c.cout, tensors[n.in].D, c.stride, &need);
    }
  NCK(cudaMalloc((void **)&tcs.cl, 2 * std::max<int64_t>(need.cl_elems, 8)));
  NCK(cudaMalloc((void **)&tcs.w, 2 * std::max<int64_t>(need.w_elems, 8)));
  NCK(cudaMalloc((void **)&tcs.xs, 2 * std::max<int64_t>(need.xs_elems, 8)));
  NCK(cudaMalloc((void **)&tcs.dyc, 2 * std::max<int64_t>(need.dyc_elems, 8)));
  NCK(cudaMalloc((void **)&tcs.part, 4 * std::max<int64_t>(need.part_floats, 8)));
  NCK(cudaMalloc((void **)&tcs.err, sizeof(int)));
  NCK(cudaMemsetAsync(tcs.err, 0, sizeof(int), st));
  tcs.cl_elems = need.cl_elems; tcs.w_elems = need.w_elems; tcs.xs_elems = need.xs_elems;
  tcs.dyc_elems = need.dyc_elems; tcs.part_floats = need.part_floats;
  tcs_B = B;
  return cudaSuccess;
}

cudaError_t WarmNet::ensure_batch(int B) {
  if (B <= cap_B) return cudaSuccess;
  NCK(cudaSetDevice(device));
  NCK(cudaStreamSynchronize(st));
  cudaFree(d_act); cudaFree(d_grad); cudaFree(d_bt); cudaFree(d_bm);
  d_act = d_grad = d_bt = d_bm = nullptr;
  cap_B = 0;
  NCK(cudaMalloc(&d_act, sizeof(float) * per_sample * B));
  NCK(cudaMalloc(&d_grad, sizeof(float) * per_sample * B));
  NCK(cudaMalloc(&d_bt, sizeof(float) * kOut * voxels() * B));
  NCK(cudaMalloc(&d_bm, sizeof(float) * voxels() * B));
  cap_B = B;
  return cudaSuccess;
}

cudaError_t WarmNet::forward(int B) {
  if (use_tc) NCK(tc_alloc(cap_B));
  for (const Node &n : nodes) {
    const Tensor &ti = tensors[n.in];
    if (n.kind == 0) {
      const Conv &c = convs[n.conv];
      if (tc_layer(c))
        NCK(nn_tc_conv3d(tensor(n.in), d_p + c.w_off, d_p + c.b_off, tensor(n.out), B, c.cin, c.cout, ti.D, ti.D, ti.D,
                         c.stride, c.relu, 0, tcs, st));
      else
        NCK(nn_conv3d(tensor(n.in), d_p + c.w_off, d_p + c.b_off, tensor(n.out), B, c.cin, c.cout, ti.D, ti.D, ti.D,
                      c.stride, c.relu, 0, st));
    } else if (n.kind == 1) {
      const int D = tensors[n.out].D;
      NCK(nn_upsample2(tensor(n.in), tensor(n.out), (int64_t)B * ti.C, D, D, D, st));
    } else {
      const int64_t cnt = (int64_t)B * ti.C * ti.D * ti.D * ti.D;
      NCK(cudaMemcpyAsync(tensor(n.out), tensor(n.in), sizeof(float) * cnt, cudaMemcpyDeviceToDevice, st));
      NCK(nn_axpy(tensor(n.out), tensor(n.in2), 1.0f, cnt, st));
    }
  }
  return cudaSuccess;
}

cudaError_t WarmNet::loss(int B, const float *t, const float *m, double scale, bool backward, double *out) {
  const int last = (int)tensors.size() - 1;
  if (backward) NCK(cudaMemsetAsync(d_grad, 0, sizeof(float) * per_sample * cap_B, st));
  NCK(nn_mse(output(), t, m, backward ? grad(last) : nullptr, d_mse, mse_parts, B, kOut, voxels(), scale, st));
  std::vector<double> part(mse_parts);
  NCK(cudaMemcpyAsync(part.data(), d_mse, sizeof(double) * mse_parts, cudaMemcpyDeviceToHost, st));
  if (backward) {
    for (int i = (int)nodes.size() - 1; i >= 0; i--) {
      const Node &n = nodes[i];
      const Tensor &ti = tensors[n.in];
      if (n.kind == 0) {
        const Conv &c = convs[n.conv];
        if (tc_layer(c))
          NCK(nn_tc_conv3d_backward(tensor(n.in), d_p + c.w_off, tensor(n.out), grad(n.out),
                                    n.in == 0 ? nullptr : grad(n.in), d_g + c.w_off, d_g + c.b_off, d_part, part_floats,
                                    B, c.cin, c.cout, ti.D, ti.D, ti.D, c.stride, c.relu, 1, tcs, st));
        else
          NCK(nn_conv3d_backward(tensor(n.in), d_p + c.w_off, tensor(n.out), grad(n.out), n.in == 0 ? nullptr : grad(n.in),
                                 d_g + c.w_off, d_g + c.b_off, d_part, part_floats, B, c.cin, c.cout, ti.D, ti.D, ti.D,
                                 c.stride, c.relu, 1, st));
      } else if (n.kind == 1) {
        NCK(nn_upsample2_backward(grad(n.out), grad(n.in), (int64_t)B * ti.C, ti.D, ti.D, ti.D, 1, st));
      } else {
        const int64_t cnt = (int64_t)B * ti.C * ti.D * ti.D * ti.D;
        NCK(nn_axpy(grad(n.in), grad(n.out), 1.0f, cnt, st));
        NCK(nn_axpy(grad(n.in2), grad(n.out), 1.0f, cnt, st));
      }
    }
  }
  NCK(cudaStreamSynchronize(st));
  if (use_tc && tcs.err) {
    int e = 0;
    NCK(cudaMemcpy(&e, tcs.err, sizeof e, cudaMemcpyDeviceToHost));
    if (e) return cudaErrorLaunchTimeout;   // a tensor-core kernel gave up waiting for its copies
  }
  double sum = 0;
  for (double v : part) sum += v;
  *out = sum;
  return cudaSuccess;
}

cudaError_t WarmNet::features(const GridDesc &g, float K, float *dst) {
  NCK(ws_features(g, R, K, dst, d_seed, d_seed + voxels(), st));
  if (n_in > kGeomIn) NCK(ws_coords(R, dst + (int64_t)kGeomIn * voxels(), st));
  return cudaSuccess;
}

cudaError_t WarmNet::add_sample(const GridDesc &g, float K, int storage, const void *acc, int nacc, double u0) {
  NCK(cudaSetDevice(device));
  const int64_t V = voxels();
  Sample s;
  NCK(cudaMalloc(&s.buf, sizeof(float) * (n_in + kOut + 1) * V));
  cudaError_t e = features(g, K, s.buf);
  if (e == cudaSuccess) e = ws_targets(g, storage, acc, nacc, u0, R, s.buf + (int64_t)n_in * V, s.buf + (int64_t)(n_in + kOut) * V, st);
  std::vector<float> m(V);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(m.data(), s.buf + (int64_t)(n_in + kOut) * V, sizeof(float) * V, cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) { cudaFree(s.buf); return e; }
  for (float v : m) s.msum += v;
  samples.push_back(s);
  return cudaSuccess;
}

cudaError_t WarmNet::stage(int idx, int b, bool flip) {
  const int64_t V = voxels();
  const Sample &s = samples[idx];
  NCK(cudaMemcpyAsync(input(b), s.buf, sizeof(float) * n_in * V, cudaMemcpyDeviceToDevice, st));
  NCK(cudaMemcpyAsync(d_bt + (int64_t)b * kOut * V, s.buf + (int64_t)n_in * V, sizeof(float) * kOut * V,
                      cudaMemcpyDeviceToDevice, st));
  NCK(cudaMemcpyAsync(d_bm + (int64_t)b * V, s.buf + (int64_t)(n_in + kOut) * V, sizeof(float) * V, cudaMemcpyDeviceToDevice,
                      st));
  if (flip) {
    NCK(ws_flip_x(input(b), kGeomIn, R, -1, st));   // the coordinate channels stay: the mirrored box's own
    NCK(ws_flip_x(d_bt + (int64_t)b * kOut * V, kOut, R, 0, st));
    NCK(ws_flip_x(d_bm + (int64_t)b * V, 1, R, -1, st));
  }
  return cudaSuccess;
}

cudaError_t WarmNet::train(int first, int count, int epochs, int batch, double lr, double lr_min, uint64_t seed,
                           bool flip, double *epoch_loss) {
  NCK(cudaSetDevice(device));
  NCK(ensure_batch(batch));
  std::vector<int> order(count);
  uint64_t rs = seed;
  const int per_epoch = (count + batch - 1) / batch;
  const int64_t total = (int64_t)per_epoch * epochs;
  int64_t it = 0;
  for (int ep = 0; ep < epochs; ep++) {
    for (int i = 0; i < count; i++) order[i] = first + i;
    for (int i = count - 1; i > 0; i--) std::swap(order[i], order[(int)(splitmix(rs) % (uint64_t)(i + 1))]);
    double sum = 0, wsum = 0;
    for (int b0 = 0; b0 < count; b0 += batch) {
      const int B = std::min(batch, count - b0);
      double msum = 0;
      for (int b = 0; b < B; b++) {
        NCK(stage(order[b0 + b], b, flip && (splitmix(rs) & 1)));
        msum += samples[order[b0 + b]].msum;
      }
      NCK(forward(B));
      double L = 0;
      NCK(loss(B, d_bt, d_bm, 1.0 / (kOut * std::max(msum, 1.0)), true, &L));
      // cosine decay from lr to lr_min over this call, scaled by a linear warm-up over the network's
      // first kWarmup updates
      constexpr int kWarmup = 100;
      double rate = lr_min + 0.5 * (lr - lr_min) * (1 + std::cos(M_PI * (double)it / (double)std::max<int64_t>(1, total)));
      if (adam_t < kWarmup) rate *= (double)(adam_t + 1) / kWarmup;
      adam_t++;
      NCK(nn_adam(d_p, d_g, d_m, d_v, n_params, (float)rate, 0.9f, 0.999f, 1e-8f, adam_t, st));
      it++;
      sum += L * B;
      wsum += B;
    }
    if (epoch_loss) epoch_loss[ep] = sum / std::max(wsum, 1.0);
  }
  return cudaStreamSynchronize(st);
}

cudaError_t WarmNet::eval_loss(int first, int count, double *out) {
  NCK(cudaSetDevice(device));
  const int batch = std::max(1, std::min(cap_B > 0 ? cap_B : 4, count));
  NCK(ensure_batch(batch));
  double sum = 0;
  for (int b0 = 0; b0 < count; b0 += batch) {
    const int B = std::min(batch, count - b0);
    double msum = 0;
    for (int b = 0; b < B; b++) {
      NCK(stage(first + b0 + b, b, false));
      msum += samples[first + b0 + b].msum;
    }
    NCK(forward(B));
    double L = 0;
    NCK(loss(B, d_bt, d_bm, 1.0 / (kOut * std::max(msum, 1.0)), false, &L));
    sum += L * B;
  }
  *out = sum / std::max(count, 1);
  return cudaSuccess;
}

}  // namespace abx
