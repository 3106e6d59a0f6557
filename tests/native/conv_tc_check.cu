// Native check of the tensor-core convolutions (nn_tc.cu) against the float32 convolutions (nn.cu), layer by layer.
//
// Every operand (input, weights, output gradient) is a bfloat16 value held in float32, so the tensor-core path,
// which rounds its operands to bfloat16, multiplies exactly the numbers the float32 path multiplies; both sum the
// products in float32, in different orders.  Forward output, data gradient (accumulated onto a non-zero buffer),
// weight gradient and bias gradient must then agree to float32 summation error: relative L2 below 1e-5.
//
// Shapes: every convolution of the warm-start network at 8^3 .. 64^3 (bases 8 and 16, strides 1 and 2, 9 and 12
// input channels, the 4-channel linear head) and wide layers (64, 128 channels).  The weight gradient of layers
// whose output planes hold fewer than 64 voxels runs on the float32 kernels by design and is compared all the same.
//
// Then the failure path: with the forward kernel's test hook set, the copies of the first K-step are never issued,
// so the MMA thread's bounded wait runs out; the launch must end by itself within seconds with the error flag set,
// and the next (normal) launch must give the right result on the same context.
//
// Prints one line per layer and "all match" at the end; exit status 0 when every comparison passed.
#include "nn.cu"
#include "nn_tc.cu"

#include <chrono>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <vector>

using namespace abx;

#define CK(x)                                                                              \
  do {                                                                                     \
    cudaError_t e_ = (x);                                                                  \
    if (e_ != cudaSuccess) {                                                               \
      printf("CUDA error %s at line %d\n", cudaGetErrorString(e_), __LINE__);              \
      return 1;                                                                            \
    }                                                                                      \
  } while (0)

static uint64_t rng_state = 0x2545F4914F6CDD1Dull;
static float uniform_pm1() {   // xorshift64*, uniform in [-1, 1)
  rng_state ^= rng_state >> 12; rng_state ^= rng_state << 25; rng_state ^= rng_state >> 27;
  const uint64_t r = rng_state * 0x2545F4914F6CDD1Dull;
  return (float)((r >> 40) * (1.0 / 16777216.0)) * 2.0f - 1.0f;
}
// nearest bfloat16 (ties to even), returned as float32; inputs are finite
static float to_bf16(float f) {
  uint32_t u;
  memcpy(&u, &f, 4);
  u += 0x7FFFu + ((u >> 16) & 1u);
  u &= 0xFFFF0000u;
  memcpy(&f, &u, 4);
  return f;
}
static std::vector<float> draw(int64_t n, float scale) {
  std::vector<float> v(n);
  for (auto &x : v) x = to_bf16(uniform_pm1() * scale);
  return v;
}

static double worst = 0.0;
static bool compare(const char *what, const std::vector<float> &got, const std::vector<float> &ref) {
  double num = 0, den = 0;
  for (size_t i = 0; i < got.size(); i++) {
    const double d = (double)got[i] - ref[i];
    num += d * d;
    den += (double)ref[i] * ref[i];
  }
  const double r = std::sqrt(num / (den > 0 ? den : 1e-300));
  worst = r > worst ? r : worst;
  const bool ok = r < 1e-5;   // NaN fails
  printf("  %-3s rel_l2 %.2e%s", what, r, ok ? "" : " MISMATCH");
  return ok;
}

static std::vector<float> fetch(const float *d, int64_t n) {
  std::vector<float> h(n);
  cudaMemcpy(h.data(), d, n * sizeof(float), cudaMemcpyDeviceToHost);
  return h;
}

struct Layer { int Cin, Cout, D, s, relu; };

int main() {
  if (!nn_tc_available()) {
    printf("tensor cores unavailable\n");
    return 4;
  }
  const Layer layers[] = {
      {9, 8, 8, 1, 1},    {12, 8, 8, 1, 1},   {8, 8, 8, 1, 1},    {8, 16, 8, 2, 1},   {16, 16, 4, 1, 1},
      {16, 8, 8, 1, 1},   {8, 4, 8, 1, 0},    {9, 8, 16, 1, 1},   {8, 16, 16, 2, 1},  {16, 32, 8, 2, 1},
      {32, 32, 4, 1, 1},  {32, 16, 8, 1, 1},  {9, 16, 32, 1, 1},  {16, 16, 32, 1, 1}, {16, 32, 32, 2, 1},
      {32, 16, 16, 1, 1}, {16, 4, 32, 1, 0},  {9, 8, 64, 1, 1},   {8, 8, 64, 1, 1},   {8, 16, 64, 2, 1},
      {16, 8, 64, 1, 1},  {32, 64, 32, 2, 1}, {64, 64, 16, 1, 1}, {128, 64, 16, 1, 1}, {64, 128, 16, 2, 1},
      {128, 128, 8, 1, 1},
  };
  const int B = 2;
  TcNeed need;
  for (const Layer &l : layers) nn_tc_need(B, l.Cin, l.Cout, l.D, l.s, &need);
  TcScratch sc;
  CK(cudaMalloc((void **)&sc.cl, need.cl_elems * 2));
  CK(cudaMalloc((void **)&sc.w, need.w_elems * 2));
  CK(cudaMalloc((void **)&sc.xs, need.xs_elems * 2));
  CK(cudaMalloc((void **)&sc.dyc, need.dyc_elems * 2));
  CK(cudaMalloc((void **)&sc.part, need.part_floats * 4));
  CK(cudaMalloc((void **)&sc.err, sizeof(int)));
  CK(cudaMemset(sc.err, 0, sizeof(int)));
  sc.cl_elems = need.cl_elems; sc.w_elems = need.w_elems; sc.xs_elems = need.xs_elems;
  sc.dyc_elems = need.dyc_elems; sc.part_floats = need.part_floats;

  bool all = true;
  for (const Layer &l : layers) {
    const int D = l.D, Do = (D - 1) / l.s + 1;
    const int64_t nx = (int64_t)B * l.Cin * D * D * D, ny = (int64_t)B * l.Cout * Do * Do * Do;
    const int64_t nw = (int64_t)l.Cout * l.Cin * 27;
    const std::vector<float> hx = draw(nx, 1.0f), hw = draw(nw, 0.25f), hb = draw(l.Cout, 0.1f);
    const std::vector<float> hdy = draw(ny, 1.0f), hdx0 = draw(nx, 0.5f);
    const int64_t pf = nn_wgrad_scratch_floats(l.Cin, l.Cout, Do * Do * Do);
    float *x, *w, *b, *y[2], *dy[2], *dx[2], *dw[2], *db[2], *part;
    CK(cudaMalloc(&x, nx * 4)); CK(cudaMalloc(&w, nw * 4)); CK(cudaMalloc(&b, l.Cout * 4));
    CK(cudaMalloc(&part, pf * 4));
    for (int k = 0; k < 2; k++) {
      CK(cudaMalloc(&y[k], ny * 4)); CK(cudaMalloc(&dy[k], ny * 4)); CK(cudaMalloc(&dx[k], nx * 4));
      CK(cudaMalloc(&dw[k], nw * 4)); CK(cudaMalloc(&db[k], l.Cout * 4));
      CK(cudaMemcpy(dy[k], hdy.data(), ny * 4, cudaMemcpyHostToDevice));
      CK(cudaMemcpy(dx[k], hdx0.data(), nx * 4, cudaMemcpyHostToDevice));
    }
    CK(cudaMemcpy(x, hx.data(), nx * 4, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(w, hw.data(), nw * 4, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(b, hb.data(), l.Cout * 4, cudaMemcpyHostToDevice));
    // [0]: float32 kernels, [1]: tensor cores; both backward passes mask with the float32 forward's output
    CK(nn_conv3d(x, w, b, y[0], B, l.Cin, l.Cout, D, D, D, l.s, l.relu, 0, 0));
    CK(nn_tc_conv3d(x, w, b, y[1], B, l.Cin, l.Cout, D, D, D, l.s, l.relu, 0, sc, 0));
    CK(nn_conv3d_backward(x, w, y[0], dy[0], dx[0], dw[0], db[0], part, pf, B, l.Cin, l.Cout, D, D, D, l.s, l.relu, 1, 0));
    CK(nn_tc_conv3d_backward(x, w, y[0], dy[1], dx[1], dw[1], db[1], part, pf, B, l.Cin, l.Cout, D, D, D, l.s, l.relu, 1,
                             sc, 0));
    CK(cudaDeviceSynchronize());
    int err = 0;
    CK(cudaMemcpy(&err, sc.err, sizeof err, cudaMemcpyDeviceToHost));
    printf("Cin %3d Cout %3d D %2d s %d relu %d:", l.Cin, l.Cout, D, l.s, l.relu);
    bool ok = err == 0;
    ok &= compare("y", fetch(y[1], ny), fetch(y[0], ny));
    ok &= compare("dx", fetch(dx[1], nx), fetch(dx[0], nx));
    ok &= compare("dw", fetch(dw[1], nw), fetch(dw[0], nw));
    ok &= compare("db", fetch(db[1], l.Cout), fetch(db[0], l.Cout));
    printf("%s\n", err ? "  (a kernel gave up waiting)" : "");
    all &= ok;
    cudaFree(x); cudaFree(w); cudaFree(b); cudaFree(part);
    for (int k = 0; k < 2; k++) { cudaFree(y[k]); cudaFree(dy[k]); cudaFree(dx[k]); cudaFree(dw[k]); cudaFree(db[k]); }
    if (err) break;
  }
  // failure path (one small layer, four CTAs)
  if (all) {
    const Layer l{16, 16, 8, 1, 1};
    const int D = l.D, Bf = 1;
    const int64_t nx = (int64_t)Bf * l.Cin * D * D * D, ny = (int64_t)Bf * l.Cout * D * D * D, nw = (int64_t)l.Cout * l.Cin * 27;
    const std::vector<float> hx = draw(nx, 1.0f), hw = draw(nw, 0.25f), hb = draw(l.Cout, 0.1f);
    float *x, *w, *b, *y[2];
    CK(cudaMalloc(&x, nx * 4)); CK(cudaMalloc(&w, nw * 4)); CK(cudaMalloc(&b, l.Cout * 4));
    CK(cudaMalloc(&y[0], ny * 4)); CK(cudaMalloc(&y[1], ny * 4));
    CK(cudaMemcpy(x, hx.data(), nx * 4, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(w, hw.data(), nw * 4, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(b, hb.data(), l.Cout * 4, cudaMemcpyHostToDevice));
    CK(cudaMemset(sc.err, 0, sizeof(int)));
    tc::g_test_drop_kstep = 0;
    const auto t0 = std::chrono::steady_clock::now();
    CK(nn_tc_conv3d(x, w, b, y[1], Bf, l.Cin, l.Cout, D, D, D, l.s, l.relu, 0, sc, 0));
    CK(cudaDeviceSynchronize());
    const double sec = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    tc::g_test_drop_kstep = -1;
    int err = 0;
    CK(cudaMemcpy(&err, sc.err, sizeof err, cudaMemcpyDeviceToHost));
    printf("failure path: missing copies -> error flag %d after %.2f s\n", err, sec);
    bool ok = err == 1;
    CK(cudaMemset(sc.err, 0, sizeof(int)));
    CK(nn_conv3d(x, w, b, y[0], Bf, l.Cin, l.Cout, D, D, D, l.s, l.relu, 0, 0));
    CK(nn_tc_conv3d(x, w, b, y[1], Bf, l.Cin, l.Cout, D, D, D, l.s, l.relu, 0, sc, 0));
    CK(cudaDeviceSynchronize());
    CK(cudaMemcpy(&err, sc.err, sizeof err, cudaMemcpyDeviceToHost));
    printf("failure path: next launch, error flag %d:", err);
    ok &= err == 0;
    ok &= compare("y", fetch(y[1], ny), fetch(y[0], ny));
    printf("\n");
    all &= ok;
    cudaFree(x); cudaFree(w); cudaFree(b); cudaFree(y[0]); cudaFree(y[1]);
  }
  printf("worst rel_l2 %.2e\n%s\n", worst, all ? "all match" : "MISMATCH");
  return all ? 0 : 3;
}
