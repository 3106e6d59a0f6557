// api.cpp - the C ABI of libairbox.so (include/airbox.h): geometry
// preparation around the GPU voxelizer, simulation handles, the step loop
// with CUDA graphs, probes and evaluation.
//
// Compiled with -ffp-contract=off: the frame transform, grid sizing and the
// setupSim coefficients must round exactly as the reference's JavaScript
// doubles do (src/engine.js:31-43, 111-125, 259).
#include "../../include/airbox.h"

#include <cuda_runtime_api.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <memory>
#include <string>
#include <tuple>
#include <vector>

#include "lbm_iface.h"
#include "net.h"

using namespace abx;

// ------------------------------------------------------------------ errors
static thread_local std::string g_err;

static int fail(int code, const char *fmt, ...) {
  char buf[1024];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  g_err = buf;
  return code;
}
static int cuda_fail(cudaError_t e, const char *what) {
  if (e == cudaErrorMemoryAllocation) return fail(ABX_ERR_OUT_OF_MEMORY, "CUDA out of memory in %s", what);
  return fail(ABX_ERR_CUDA, "CUDA error in %s: %s", what, cudaGetErrorString(e));
}
#define CK(x, what)                               \
  do {                                            \
    cudaError_t e_ = (x);                         \
    if (e_ != cudaSuccess) return cuda_fail(e_, what); \
  } while (0)

extern "C" const char *abx_last_error(void) { return g_err.c_str(); }

// A pending error of an earlier, unrelated CUDA call in this process (another
// library, a destructor) must not be reported as this call's failure.
static void clear_stale_error() { (void)cudaGetLastError(); }
extern "C" int abx_abi_version(void) { return ABX_ABI_VERSION; }
extern "C" int abx_device_count(void) {
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess) { cudaGetLastError(); return 0; }
  return n;
}

// ------------------------------------------------------------------ parseSTL (src/engine.js:15-28)
static bool stl_num_char(unsigned char c) {
  return (c >= '0' && c <= '9') || c == '-' || c == '+' || c == '.' || c == 'e' || c == 'E';
}
static bool stl_space(unsigned char c) { return c == ' ' || c == '\t' || c == '\n' || c == '\r' || c == '\v' || c == '\f'; }

// Number() of a token of [-+0-9.eE]: the whole token must be a decimal literal, else NaN.
static double token_number(const unsigned char *s, size_t n) {
  std::string t(reinterpret_cast<const char *>(s), n);
  char *end = nullptr;
  const double v = std::strtod(t.c_str(), &end);
  return (end == t.c_str() + n) ? v : std::nan("");
}

extern "C" int abx_parse_stl(const void *buf_, size_t len, float *out, size_t cap, size_t *nfloats) {
  if (!buf_ && len) return fail(ABX_ERR_INVALID_ARGUMENT, "parse_stl: null buffer");
  if (!nfloats) return fail(ABX_ERR_INVALID_ARGUMENT, "parse_stl: null size pointer");
  const unsigned char *buf = static_cast<const unsigned char *>(buf_);
  uint32_t n = 0;
  if (len >= 84) std::memcpy(&n, buf + 80, 4);  // little-endian hosts only (x86-64, aarch64)
  if (n > 0 && 84ull + 50ull * n == (unsigned long long)len) {
    *nfloats = (size_t)n * 9;
    if (out) {
      if (cap < *nfloats) return fail(ABX_ERR_INVALID_ARGUMENT, "parse_stl: output too small");
      for (uint32_t t = 0; t < n; t++) std::memcpy(out + (size_t)t * 9, buf + 84 + (size_t)t * 50 + 12, 36);
    }
    return ABX_OK;
  }
  // ASCII: every "vertex" followed by whitespace-separated number tokens, three of them
  size_t cnt = 0;
  for (size_t p = 0; p + 6 <= len;) {
    if (std::memcmp(buf + p, "vertex", 6) != 0) { p++; continue; }
    size_t q = p + 6;
    double v[3];
    bool ok = true;
    for (int c = 0; c < 3; c++) {
      const size_t q0 = q;
      while (q < len && stl_space(buf[q])) q++;
      if (q == q0) { ok = false; break; }
      const size_t t0 = q;
      while (q < len && stl_num_char(buf[q])) q++;
      if (q == t0) { ok = false; break; }
      v[c] = token_number(buf + t0, q - t0);
    }
    if (!ok) { p++; continue; }
    if (out) {
      if (cap < cnt + 3) return fail(ABX_ERR_INVALID_ARGUMENT, "parse_stl: output too small");
      for (int c = 0; c < 3; c++) out[cnt + c] = (float)v[c];
    }
    cnt += 3;
    p = q;
  }
  if (cnt < 9) return fail(ABX_ERR_NO_TRIANGLES, "STL enthält keine Dreiecke.");
  *nfloats = cnt;
  return ABX_OK;
}

// ------------------------------------------------------------------ geometry
struct Frame {
  int dAx, iAx, oAx;
  double sd, si, seal, cy, sy;
  void local(const double q[3], double L[3]) const {  // makeFrame.toLocal (src/engine.js:39)
    const double a = q[oAx], b = -si * q[iAx];
    L[0] = cy * a + sy * b;
    L[1] = -sd * (q[dAx] - seal);
    L[2] = -sy * a + cy * b;
  }
  void model(double X, double D, double Z, double q[3]) const {  // makeFrame.toModel (src/engine.js:40)
    q[oAx] = cy * X - sy * Z;
    q[dAx] = seal - sd * D;
    q[iAx] = -si * (sy * X + cy * Z);
  }
};

struct abx_geom {
  int device = 0;
  Frame fr{};
  int nx = 0, ny = 0, nz = 0, nxf = 0, nyf = 0, nzf = 0, kf = 0, kw0 = -1, top = -1, jm = 0, jpt = -1;
  int nf = 0, nOpen = 0, nHoles = 0, Af = 0, nOut = 0, leak = 0;
  int64_t N = 0, nzp = 0, Np = 0;
  double h = 0, hf = 0, origin[3] = {0, 0, 0}, mn[3] = {0, 0, 0}, mx[3] = {0, 0, 0}, pleat = 0;
  bool has_outlet = false;
  std::vector<float> tris_local, xc, dc, zc;
  std::vector<uint8_t> opening;      // nx*ny, host copy of d_opening
  // device-side, shared by the simulations of this geometry
  uint8_t *d_solid = nullptr, *d_fluid = nullptr, *d_outlet = nullptr;   // N bytes each
  uint32_t *d_mask = nullptr;
  uint2 *d_seg = nullptr;
  uint32_t nseg = 0;
  int64_t kpad = 0;
  uint8_t *d_opening = nullptr;
  int64_t *d_cells = nullptr;       // padded index of each fluid cell, compact (c) order
  std::vector<int64_t> layer_m, layer_t;   // padded indices of the air on layers jm and top+1, compact order
  int Ain = 0, Lp = 0;
  int64_t launches = 0, h2d = 0, d2h = 0;
  double ms_vox = 0, ms_masks = 0, ms_device = 0;
  // work lists of the vectorised step kernel, per block width V = 2, 4, 8 (built on first use)
  struct VecLists {
    bool ready = false;
    uint32_t *d_blk = nullptr;
    uint32_t *d_bcell = nullptr;
    uint32_t n_bulk = 0, n_filter = 0, nbcell = 0;
  } vec[3];
  ~abx_geom() {
    cudaSetDevice(device);
    cudaFree(d_solid); cudaFree(d_fluid); cudaFree(d_outlet);
    cudaFree(d_mask); cudaFree(d_seg); cudaFree(d_opening); cudaFree(d_cells);
    for (auto &v : vec) { cudaFree(v.d_blk); cudaFree(v.d_bcell); }
  }
};

static int first_ge(const std::vector<float> &a, double v) {  // firstGE, src/engine.js:13
  for (size_t i = 0; i < a.size(); i++) if ((double)a[i] >= v) return (int)i;
  return (int)a.size() - 1;
}

static void fmt_number(char *out, size_t n, double v) {  // shortest round-trip, like Number#toString
  for (int prec = 1; prec <= 17; prec++) {
    std::snprintf(out, n, "%.*g", prec, v);
    if (std::strtod(out, nullptr) == v) return;
  }
}

namespace {
struct DevBuf {  // scoped device allocation
  void *p = nullptr;
  ~DevBuf() { if (p) cudaFree(p); }
};
struct AsyncBuf {  // scoped stream-ordered allocation (cudaMallocAsync), freed on its stream
  void *p = nullptr;
  cudaStream_t st = nullptr;
  ~AsyncBuf() { if (p) cudaFreeAsync(p, st); }
};
struct StreamHolder {
  cudaStream_t s = nullptr;
  ~StreamHolder() { if (s) cudaStreamDestroy(s); }
};
}  // namespace

// Opening search on the fine slice (src/engine.js:141-171), on the GPU: g.d_opening (device), g.opening (host
// copy), g.nHoles, g.nOpen; the reference's errors when no hole is large enough or the opening is too small.
static int find_opening(abx_geom &g, const abx_prepare_params *p, const uint8_t *d_slice, cudaStream_t st) {
  const int nx = g.nx, ny = g.ny, nxf = g.nxf, nyf = g.nyf;
  const int64_t nfs = (int64_t)nxf * nyf;
  // a kept component has more than 25 / hf^2 cells
  const double kcap = std::floor((double)nfs * g.hf * g.hf / 25.0) + 2;
  const uint32_t cap = (uint32_t)std::min<double>(kcap, (double)nfs + 1);
  // one stream-ordered scratch block: outside, labels, sizes, claims, result, flag, kept list, coarse counters
  auto al = [](size_t v) { return (v + 255) / 256 * 256; };
  size_t nb = 0;
  const size_t o_out = nb;  nb += al(sizeof(OpenOut));
  const size_t o_flag = nb; nb += al(sizeof(int));
  const size_t o_lab = nb;  nb += al(sizeof(int32_t) * (size_t)nfs);
  const size_t o_size = nb; nb += al(sizeof(uint32_t) * (size_t)nfs);
  const size_t o_clm = nb;  nb += al(sizeof(uint32_t) * (size_t)nfs);
  const size_t o_kept = nb; nb += al(sizeof(uint2) * cap);
  const size_t o_sel = nb;  nb += al(sizeof(uint32_t) * (size_t)nx * ny);
  const size_t o_outs = nb; nb += al((size_t)nfs);
  AsyncBuf scratch{nullptr, st};
  CK(cudaMallocAsync(&scratch.p, nb, st), "prepare: opening");
  unsigned char *S = (unsigned char *)scratch.p;
  OpenArgs a{d_slice, nxf, nyf, S + o_outs, (int32_t *)(S + o_lab), (uint32_t *)(S + o_size),
             (uint32_t *)(S + o_clm), g.origin[0], g.origin[1], g.hf};
  OpenOut *out = (OpenOut *)(S + o_out);
  int *changed = (int *)(S + o_flag);
  uint2 *kept = (uint2 *)(S + o_kept);
  CK(cudaMemsetAsync(out, 0, sizeof(OpenOut), st), "prepare: opening");
  CK(open_init(a, st), "prepare: opening");
  g.launches += 1;
  // empty cells reachable from the border (:144-151), then the holes' components (:153-155, components2d
  // :95-108): rounds of line sweeps until a round changes nothing (each round changes a cell otherwise)
  for (int pass = 0; pass < 2; pass++) {
    if (pass == 1) {
      CK(open_holes(a, st), "prepare: opening");
      g.launches += 1;
    }
    for (int64_t round = 0;; round++) {
      if (round > nfs) return fail(ABX_ERR_CUDA, "prepare: opening search did not settle");
      CK(cudaMemsetAsync(changed, 0, sizeof(int), st), "prepare: opening");
      CK(pass == 0 ? open_outside_round(a, changed, st) : open_label_round(a, changed, st), "prepare: opening");
      int c = 0;
      CK(cudaMemcpyAsync(&c, changed, sizeof(int), cudaMemcpyDeviceToHost, st), "prepare: opening");
      CK(cudaStreamSynchronize(st), "prepare: opening");
      g.launches += 3;
      g.d2h += sizeof(int);
      if (!c) break;
    }
  }
  CK(open_components(a, out, kept, cap, st), "prepare: opening");
  OpenOut o{};
  CK(cudaMemcpyAsync(&o, out, sizeof o, cudaMemcpyDeviceToHost, st), "prepare: opening");
  CK(cudaStreamSynchronize(st), "prepare: opening");
  g.launches += 2;
  g.d2h += sizeof o;
  if (o.n_kept > cap) return fail(ABX_ERR_CUDA, "prepare: more openings than the search holds");
  g.nHoles = (int)o.n_kept;
  if (!o.n_kept) return fail(ABX_ERR_NO_OPENING, "Auf der gewählten Einlassseite wurde keine Öffnung gefunden.");
  uint32_t root = 0xFFFFFFFFu - (uint32_t)(o.best & 0xFFFFFFFFull);   // the largest, first of equals (:168)
  if (p->has_click) {
    // the component holding the sampled cell nearest to the click, first of equals in component order (:158-163)
    const int n = (int)o.n_kept;
    std::vector<uint2> kv(n);
    CK(cudaMemcpyAsync(kv.data(), kept, sizeof(uint2) * n, cudaMemcpyDeviceToHost, st), "prepare: opening");
    CK(cudaStreamSynchronize(st), "prepare: opening");
    std::vector<int64_t> offs(n);
    int64_t tot = 0;
    for (int b = 0; b < n; b++) { offs[b] = tot; tot += kv[b].y; }
    // per component: its cells in breadth-first order, its offset in that array, its smallest distance
    const size_t b_off = al(sizeof(int32_t) * (size_t)std::max<int64_t>(tot, 1)), b_min = b_off + al(sizeof(int64_t) * n);
    AsyncBuf bfs{nullptr, st};
    CK(cudaMallocAsync(&bfs.p, b_min + sizeof(unsigned long long) * n, st), "prepare: opening");
    unsigned char *B = (unsigned char *)bfs.p;
    CK(cudaMemcpyAsync(B + b_off, offs.data(), sizeof(int64_t) * n, cudaMemcpyHostToDevice, st), "prepare: opening");
    double L[3];
    g.fr.local(p->click, L);
    CK(open_bfs_click(a, kept, (const int64_t *)(B + b_off), n, (int32_t *)B, L[0], L[1],
                      (unsigned long long *)(B + b_min), st), "prepare: opening");
    std::vector<unsigned long long> dm(n);
    CK(cudaMemcpyAsync(dm.data(), B + b_min, sizeof(unsigned long long) * n, cudaMemcpyDeviceToHost, st),
       "prepare: opening");
    CK(cudaStreamSynchronize(st), "prepare: opening");
    g.launches += 1;
    g.h2d += (int64_t)(sizeof(int64_t) * n);
    g.d2h += (int64_t)((sizeof(uint2) + sizeof(unsigned long long)) * n);
    std::vector<int> idx(n);
    for (int b = 0; b < n; b++) idx[b] = b;
    std::sort(idx.begin(), idx.end(), [&](int x, int y) { return kv[x].x < kv[y].x; });
    root = kv[idx[0]].x;   // comps[0] stays chosen when no distance is below Infinity (a non-finite click)
    double bd = INFINITY;
    for (int b : idx) {
      double d;
      std::memcpy(&d, &dm[b], sizeof d);
      if (d < bd) { bd = d; root = kv[b].x; }
    }
  }
  // coarse opening: cells holding at least 5 of their 9 fine cells in the chosen component (:164-166)
  uint32_t *sel = (uint32_t *)(S + o_sel);
  CK(cudaMemsetAsync(sel, 0, sizeof(uint32_t) * (size_t)nx * ny, st), "prepare: opening");
  CK(cudaMalloc((void **)&g.d_opening, std::max<size_t>((size_t)nx * ny, 1)), "prepare: opening");
  CK(open_select(a, root, nx, ny, sel, g.d_opening, out, st), "prepare: opening");
  g.opening.assign((size_t)nx * ny, 0);
  CK(cudaMemcpyAsync(g.opening.data(), g.d_opening, g.opening.size(), cudaMemcpyDeviceToHost, st), "prepare: opening");
  CK(cudaMemcpyAsync(&o, out, sizeof o, cudaMemcpyDeviceToHost, st), "prepare: opening");
  CK(cudaStreamSynchronize(st), "prepare: opening");
  g.launches += 2;
  g.d2h += (int64_t)(g.opening.size() + sizeof o);
  g.nOpen = (int)o.n_open;
  if (g.nOpen < 8) return fail(ABX_ERR_OPENING_TOO_SMALL, "Einlassöffnung ist zu klein für die gewählte Zellgröße.");
  return ABX_OK;
}

// Opening search (GPU), then duct, closing, flood, leak check and outlet (src/engine.js:141-216).
static int finish_geometry(abx_geom &g, const abx_prepare_params *p, const uint8_t *d_slice, cudaStream_t st) {
  const int nx = g.nx, ny = g.ny, nz = g.nz;
  const double h = g.h;
  int rc = find_opening(g, p, d_slice, st);
  if (rc) return rc;

  // device: inlet duct, closed bottom, flood, leak, outlet (:174-216)
  g.kw0 = -1;
  for (int k = 0; k < nz; k++) if ((double)g.zc[k] >= g.mn[2]) { g.kw0 = k; break; }
  std::vector<uint8_t> close_row(ny, 0);
  for (int j = 0; j < ny; j++) close_row[j] = (double)g.dc[j] > g.mx[1] - 0.5 * h ? 1 : 0;
  g.top = -1;
  for (int j = 0; j < ny; j++) if ((double)g.dc[j] >= 0) { g.top = j; break; }
  if (g.top < 0) return fail(ABX_ERR_SEAL_OUTSIDE, "Dichtebene liegt außerhalb des Modells.");
  const int top = g.top;
  DevBuf dclose, dflag, dcount;
  CK(cudaMalloc(&dclose.p, ny), "prepare: rows");
  CK(cudaMemcpyAsync(dclose.p, close_row.data(), ny, cudaMemcpyHostToDevice, st), "prepare: rows");
  CK(cudaMalloc((void **)&g.d_fluid, (size_t)g.N), "prepare: fluid");
  CK(cudaMalloc((void **)&g.d_outlet, (size_t)g.N), "prepare: outlet");
  CK(cudaMalloc(&dflag.p, 2 * sizeof(int)), "prepare: flags");
  CK(cudaMalloc(&dcount.p, 5 * sizeof(unsigned long long)), "prepare: counts");
  MaskArgs a{nx, ny, nz, g.N, g.d_solid, g.d_fluid, g.d_outlet, g.d_opening, (const uint8_t *)dclose.p, g.kw0, top};
  CK(prep_duct(a, st), "prepare: duct");
  g.launches += 2;
  g.h2d += (int64_t)ny;
  // flood: rounds of line sweeps until a round adds no cell (each round at least one cell otherwise)
  int *changed = (int *)dflag.p;
  for (int64_t round = 0;; round++) {
    if (round > g.N) return fail(ABX_ERR_CUDA, "prepare: flood fill did not settle");
    CK(cudaMemsetAsync(changed, 0, sizeof(int), st), "prepare: flood");
    CK(prep_flood_round(a, changed, st), "prepare: flood");
    int c = 0;
    CK(cudaMemcpyAsync(&c, changed, sizeof(int), cudaMemcpyDeviceToHost, st), "prepare: flood");
    CK(cudaStreamSynchronize(st), "prepare: flood");
    g.launches += 3;
    g.d2h += sizeof(int);
    if (!c) break;
  }
  // leak: fluid on the side faces or the far face (:191-195)
  int *leak = (int *)dflag.p + 1;
  CK(cudaMemsetAsync(leak, 0, sizeof(int), st), "prepare: leak");
  CK(prep_leak(a, leak, st), "prepare: leak");
  int leaked = 0;
  CK(cudaMemcpyAsync(&leaked, leak, sizeof(int), cudaMemcpyDeviceToHost, st), "prepare: leak");
  CK(cudaStreamSynchronize(st), "prepare: leak");
  g.launches += 1;
  g.d2h += sizeof(int);
  if (leaked) {
    char hs[40];
    fmt_number(hs, sizeof hs, h);
    return fail(ABX_ERR_LEAK,
                "Bei %s mm Zellgröße läuft die Luft durch eine zu dünne Wand nach außen (Wände sollten mindestens so "
                "dick wie eine Zelle sein). Bitte eine kleinere Zellgröße wählen.",
                hs);
  }
  // outlet: lid plenum with a round outlet, or the whole row `top` (:197-213)
  unsigned long long *cnt = (unsigned long long *)dcount.p;
  CK(cudaMemsetAsync(cnt, 0, 5 * sizeof(unsigned long long), st), "prepare: outlet");
  int jpt = -1;
  double L[3] = {0, 0, 0}, r2 = 0;
  if (g.has_outlet) {
    g.jpt = first_ge(g.dc, -p->outlet_height);
    if (g.jpt >= top) return fail(ABX_ERR_LID_TOO_LOW, "Deckelhöhe ist kleiner als eine Zelle.");
    jpt = g.jpt;
    g.fr.local(p->outlet_center, L);
    r2 = (p->outlet_diameter / 2) * (p->outlet_diameter / 2);
  }
  DevBuf dxc, dzc;
  CK(cudaMalloc(&dxc.p, sizeof(float) * nx), "prepare: outlet");
  CK(cudaMalloc(&dzc.p, sizeof(float) * nz), "prepare: outlet");
  CK(cudaMemcpyAsync(dxc.p, g.xc.data(), sizeof(float) * nx, cudaMemcpyHostToDevice, st), "prepare: outlet");
  CK(cudaMemcpyAsync(dzc.p, g.zc.data(), sizeof(float) * nz, cudaMemcpyHostToDevice, st), "prepare: outlet");
  CK(prep_outlet(a, jpt, (const float *)dxc.p, (const float *)dzc.p, L[0], L[2], r2, cnt, st), "prepare: outlet");
  // counts after the plenum (:214-216): cells, filter-layer cells, cells on the outlet row
  g.jm = first_ge(g.dc, g.pleat / 2);
  CK(prep_counts(a, g.jm, cnt + 2, st), "prepare: counts");
  unsigned long long hc[5];
  CK(cudaMemcpyAsync(hc, cnt, sizeof hc, cudaMemcpyDeviceToHost, st), "prepare: counts");
  CK(cudaStreamSynchronize(st), "prepare: counts");
  g.launches += 2;
  g.h2d += (int64_t)(sizeof(float) * (nx + nz));
  g.d2h += sizeof hc;
  g.nOut = (int)hc[1];
  if (g.has_outlet && g.nOut < 4)
    return fail(ABX_ERR_BAD_OUTLET, "Der Auslass liegt nicht über der Filterfläche oder ist zu klein.");
  g.nf = (int)hc[2];
  g.Af = (int)hc[3];
  g.leak = (int)hc[4];
  return ABX_OK;
}

// Cell classes of setupSim (src/engine.js:248-255), device mask, fluid
// segments and the compact cell list.
static uint2 seg2(uint32_t base, uint32_t lanes) {
  uint2 v;
  v.x = base;
  v.y = lanes;
  return v;
}

// The k offset in [0,32) that packs the columns' fluid cells into the fewest
// 32-cell segments (whole warps of fluid cells in the step kernels).
static int build_device_geometry(abx_geom &g, cudaStream_t st) {
  const int nx = g.nx, ny = g.ny, nz = g.nz;
  MaskArgs a{nx, ny, nz, g.N, g.d_solid, g.d_fluid, g.d_outlet, g.d_opening, nullptr, g.kw0, g.top};
  // kpad: the column shift with the fewest 32-cell runs holding air (first of equals)
  const int W = (nz + 31) / 32 + 1;
  DevBuf dbits, dkc;
  CK(cudaMalloc(&dbits.p, sizeof(uint32_t) * (size_t)nx * ny * W), "prepare: column bits");
  CK(cudaMalloc(&dkc.p, 32 * sizeof(unsigned long long)), "prepare: kpad");
  CK(cudaMemsetAsync(dkc.p, 0, 32 * sizeof(unsigned long long), st), "prepare: kpad");
  CK(prep_kpad_counts(a, W, (uint32_t *)dbits.p, (unsigned long long *)dkc.p, st), "prepare: kpad");
  unsigned long long kc[32];
  CK(cudaMemcpyAsync(kc, dkc.p, sizeof kc, cudaMemcpyDeviceToHost, st), "prepare: kpad");
  CK(cudaStreamSynchronize(st), "prepare: kpad");
  int best = 0;
  for (int t = 1; t < 32; t++) if (kc[t] < kc[best]) best = t;
  g.kpad = best;
  g.nzp = (g.nz + g.kpad + 31) / 32 * 32;
  g.Np = (int64_t)g.nx * g.ny * g.nzp;
  if (19 * g.Np >= (1ll << 32)) return fail(ABX_ERR_INVALID_ARGUMENT, "prepare: grid above 2^32 / 19 padded cells");
  // classes (setupSim :248-255) and the cell mask words
  const double dtop = g.dc[g.top];
  std::vector<uint8_t> filt(ny, 0);
  g.Lp = 0;
  for (int j = 0; j < ny; j++)
    if ((double)g.dc[j] > dtop && (double)g.dc[j] <= g.pleat) { filt[j] = 1; g.Lp++; }
  DevBuf dfilt, dcls, dain;
  CK(cudaMalloc(&dfilt.p, ny), "prepare: classes");
  CK(cudaMemcpyAsync(dfilt.p, filt.data(), ny, cudaMemcpyHostToDevice, st), "prepare: classes");
  CK(cudaMalloc(&dcls.p, (size_t)g.N), "prepare: class array");
  CK(cudaMalloc(&dain.p, sizeof(unsigned long long)), "prepare: classes");
  CK(cudaMemsetAsync(dain.p, 0, sizeof(unsigned long long), st), "prepare: classes");
  CK(prep_classes(a, (const uint8_t *)dfilt.p, (uint8_t *)dcls.p, (unsigned long long *)dain.p, st), "prepare: classes");
  CK(cudaMalloc((void **)&g.d_mask, sizeof(uint32_t) * (size_t)g.Np), "prepare: mask");
  CK(launch_build_mask((const uint8_t *)dcls.p, nx, ny, nz, g.nzp, g.kpad, g.d_mask, st), "prepare: build mask");
  // compact cell list, in (i, j, k) order
  const int64_t nb = prep_compact_blocks(g.N);
  DevBuf dbc, doff;
  CK(cudaMalloc(&dbc.p, sizeof(uint32_t) * std::max<int64_t>(nb, 1)), "prepare: compaction");
  CK(cudaMalloc(&doff.p, sizeof(unsigned long long) * (nb + 1)), "prepare: compaction");
  CK(cudaMalloc((void **)&g.d_cells, sizeof(int64_t) * std::max(g.nf, 1)), "prepare: cells");
  CK(prep_cells(a, g.nzp, g.kpad, g.d_cells, (uint32_t *)dbc.p, (unsigned long long *)doff.p, st), "prepare: cells");
  unsigned long long ncells = 0;
  CK(cudaMemcpyAsync(&ncells, (unsigned long long *)doff.p + nb, sizeof ncells, cudaMemcpyDeviceToHost, st), "prepare: cells");
  // fluid segments: 32-cell runs along k holding air, with their lane masks
  const int64_t S = g.nzp / 32, nslot = (int64_t)nx * ny * S, nb2 = prep_compact_blocks(nslot);
  DevBuf dbc2, doff2;
  CK(cudaMalloc(&dbc2.p, sizeof(uint32_t) * std::max<int64_t>(nb2, 1)), "prepare: segments");
  CK(cudaMalloc(&doff2.p, sizeof(unsigned long long) * (nb2 + 1)), "prepare: segments");
  CK(prep_segments(a, W, (const uint32_t *)dbits.p, g.nzp, g.kpad, nullptr, (uint32_t *)dbc2.p,
                   (unsigned long long *)doff2.p, st), "prepare: segments");
  unsigned long long nseg = 0, ain = 0;
  CK(cudaMemcpyAsync(&nseg, (unsigned long long *)doff2.p + nb2, sizeof nseg, cudaMemcpyDeviceToHost, st), "prepare: segments");
  CK(cudaMemcpyAsync(&ain, dain.p, sizeof ain, cudaMemcpyDeviceToHost, st), "prepare: classes");
  CK(cudaStreamSynchronize(st), "prepare: segments");
  if ((int64_t)ncells != g.nf) return fail(ABX_ERR_CUDA, "prepare: cell list has %llu cells, expected %d", ncells, g.nf);
  g.Ain = (int)ain;
  g.nseg = (uint32_t)nseg;
  CK(cudaMalloc((void **)&g.d_seg, sizeof(uint2) * std::max<unsigned long long>(nseg, 1)), "prepare: segments");
  CK(prep_segments(a, W, (const uint32_t *)dbits.p, g.nzp, g.kpad, g.d_seg, (uint32_t *)dbc2.p,
                   (unsigned long long *)doff2.p, st), "prepare: segments");
  CK(prep_seg_interior(g.d_seg, g.nseg, g.d_mask, st), "prepare: segments");
  // the air of layers jm and top+1 in compact order (the progress probe's cells, :327-333)
  auto layer = [&](int j, std::vector<int64_t> &out) -> int {
    out.clear();
    if (j < 0 || j >= ny) return ABX_OK;
    std::vector<uint8_t> lay((size_t)nx * nz);
    CK(cudaMemcpy2DAsync(lay.data(), nz, g.d_fluid + (size_t)j * nz, (size_t)ny * nz, nz, nx, cudaMemcpyDeviceToHost, st),
       "prepare: layers");
    CK(cudaStreamSynchronize(st), "prepare: layers");
    g.d2h += (int64_t)lay.size();
    for (int i = 0; i < nx; i++)
      for (int k = 0; k < nz; k++)
        if (lay[(size_t)i * nz + k]) out.push_back(((int64_t)i * ny + j) * g.nzp + k + g.kpad);
    return ABX_OK;
  };
  if (int rc = layer(g.jm, g.layer_m)) return rc;
  if (int rc = layer(g.top + 1, g.layer_t)) return rc;
  g.launches += 10;
  g.h2d += ny;
  g.d2h += (int64_t)(sizeof kc + 3 * sizeof(unsigned long long));
  return ABX_OK;
}

extern "C" int abx_prepare(const float *tris, size_t nfloats, const abx_prepare_params *p, abx_geom **out) {
  clear_stale_error();
  if (!p || !out || (!tris && nfloats)) return fail(ABX_ERR_INVALID_ARGUMENT, "prepare: null argument");
  *out = nullptr;
  if (p->seal_axis < 0 || p->seal_axis > 2 || p->inlet_axis < 0 || p->inlet_axis > 2)
    return fail(ABX_ERR_INVALID_ARGUMENT, "prepare: axis out of range");
  if (p->seal_axis == p->inlet_axis)
    return fail(ABX_ERR_SAME_AXIS, "Einlassseite und Filterebene liegen auf derselben Achse.");
  if (!(p->dx > 0) || !std::isfinite(p->dx)) return fail(ABX_ERR_INVALID_ARGUMENT, "prepare: dx must be positive");
  for (size_t i = 0; i < nfloats; i++)
    if (!std::isfinite(tris[i])) return fail(ABX_ERR_INVALID_ARGUMENT, "STL enthält ungültige Koordinaten (NaN/Inf).");
  std::unique_ptr<abx_geom> G(new abx_geom());
  abx_geom &g = *G;
  g.device = p->device;
  g.has_outlet = p->has_outlet != 0;
  g.pleat = p->pleat;
  // makeFrame (:31-43)
  g.fr.dAx = p->seal_axis; g.fr.iAx = p->inlet_axis; g.fr.oAx = 3 - p->seal_axis - p->inlet_axis;
  g.fr.sd = p->seal_sign; g.fr.si = p->inlet_sign; g.fr.seal = p->seal;
  const double yaw = p->inlet_yaw * M_PI / 180;
  g.fr.cy = std::cos(yaw); g.fr.sy = std::sin(yaw);
  // local triangles stored as float32, bounding box from the doubles (:112-118)
  const size_t nverts = nfloats / 3;
  g.tris_local.assign(nfloats, 0.0f);
  for (int a = 0; a < 3; a++) { g.mn[a] = INFINITY; g.mx[a] = -INFINITY; }
  for (size_t v = 0; v < nverts; v++) {
    const double q[3] = {tris[v * 3], tris[v * 3 + 1], tris[v * 3 + 2]};
    double L[3];
    g.fr.local(q, L);
    for (int a = 0; a < 3; a++) {
      g.tris_local[v * 3 + a] = (float)L[a];
      if (L[a] < g.mn[a]) g.mn[a] = L[a];
      if (L[a] > g.mx[a]) g.mx[a] = L[a];
    }
  }
  if (nverts == 0) for (int a = 0; a < 3; a++) { g.mn[a] = 0; g.mx[a] = 0; }
  // grid (:119-125)
  const double h = p->dx, hf = h / 3;
  g.h = h; g.hf = hf;
  g.origin[0] = g.mn[0] - h;
  g.origin[1] = (g.has_outlet ? std::min(g.mn[1], -p->outlet_height) : g.mn[1]) - h;
  g.origin[2] = g.mn[2] - 10 * h;
  const double fx = std::ceil((g.mx[0] - g.origin[0] + h) / h), fy = std::ceil((g.mx[1] - g.origin[1] + h) / h),
               fz = std::ceil((g.mx[2] - g.origin[2] + h) / h);
  const double Nd = fx * fy * fz;
  if (Nd > p->max_cells) return fail(ABX_ERR_GRID_TOO_LARGE, "Gitter zu groß (%.1f Mio. Zellen) – Zellgröße erhöhen.", Nd / 1e6);
  if (fx * 3 > 2e9 || fy * 3 > 2e9 || fz * 3 > 2e9 || fx * fy * 9 > 2e9)
    return fail(ABX_ERR_INVALID_ARGUMENT, "prepare: fine grid too large for this library");
  g.nx = (int)fx; g.ny = (int)fy; g.nz = (int)fz;
  g.N = (int64_t)g.nx * g.ny * g.nz;
  g.nxf = 3 * g.nx; g.nyf = 3 * g.ny; g.nzf = 3 * g.nz;
  g.nzp = (g.nz + 31) / 32 * 32;
  g.Np = (int64_t)g.nx * g.ny * g.nzp;
  // the step kernels index populations with 32-bit element offsets
  if (19 * g.Np >= (1ll << 32)) return fail(ABX_ERR_INVALID_ARGUMENT, "prepare: grid above 2^32 / 19 padded cells");
  g.kf = (int)std::floor((g.mn[2] + 1.5 - g.origin[2]) / hf);
  if (g.kf < 0 || g.kf >= g.nzf) return fail(ABX_ERR_INVALID_ARGUMENT, "prepare: opening slice outside the grid");
  g.xc.resize(g.nx); g.dc.resize(g.ny); g.zc.resize(g.nz);
  for (int i = 0; i < g.nx; i++) g.xc[i] = (float)(g.origin[0] + (i + 0.5) * h);
  for (int j = 0; j < g.ny; j++) g.dc[j] = (float)(g.origin[1] + (j + 0.5) * h);
  for (int k = 0; k < g.nz; k++) g.zc[k] = (float)(g.origin[2] + (k + 0.5) * h);

  // GPU: voxelize at 3x oversampling and downsample (:125-135)
  using clk = std::chrono::steady_clock;
  const auto t0 = clk::now();
  CK(cudaSetDevice(g.device), "prepare: set device");
  StreamHolder sh;
  CK(cudaStreamCreateWithFlags(&sh.s, cudaStreamNonBlocking), "prepare: stream");
  DevBuf dtris, dsolid, dslice;
  const int64_t ntri = (int64_t)(nfloats / 9);
  CK(cudaMalloc(&dtris.p, sizeof(float) * std::max<size_t>(nfloats, 1)), "prepare: triangles");
  if (nfloats)
    CK(cudaMemcpyAsync(dtris.p, g.tris_local.data(), sizeof(float) * nfloats, cudaMemcpyHostToDevice, sh.s), "prepare: upload");
  CK(cudaMalloc(&dsolid.p, (size_t)g.N), "prepare: solid");
  CK(cudaMalloc(&dslice.p, (size_t)g.nxf * g.nyf), "prepare: slice");
  VoxJob job{(const float *)dtris.p, ntri, {g.origin[0], g.origin[1], g.origin[2]}, hf, g.nx, g.ny, g.nz, g.kf};
  VoxOut vo{(uint8_t *)dsolid.p, (uint8_t *)dslice.p, nullptr};
  CK(run_voxelizer(job, vo, sh.s), "prepare: voxelize");
  CK(cudaStreamSynchronize(sh.s), "prepare: sync");
  g.d_solid = (uint8_t *)dsolid.p;   // the geometry keeps the solid mask on the device
  dsolid.p = nullptr;
  g.launches += vo.launches;
  g.h2d += (int64_t)(sizeof(float) * nfloats);
  g.d2h += vo.d2h_bytes;
  const auto t1 = clk::now();
  int rc = finish_geometry(g, p, (const uint8_t *)dslice.p, sh.s);
  if (rc) return rc;
  const auto t2 = clk::now();
  rc = build_device_geometry(g, sh.s);
  if (rc) return rc;
  const auto t3 = clk::now();
  g.ms_vox = std::chrono::duration<double, std::milli>(t1 - t0).count();
  g.ms_masks = std::chrono::duration<double, std::milli>(t2 - t1).count();
  g.ms_device = std::chrono::duration<double, std::milli>(t3 - t2).count();
  *out = G.release();
  return ABX_OK;
}

extern "C" void abx_geom_free(abx_geom *g) { delete g; }

extern "C" int abx_geom_get_info(const abx_geom *g, abx_geom_info *o) {
  if (!g || !o) return fail(ABX_ERR_INVALID_ARGUMENT, "geom_get_info: null argument");
  std::memset(o, 0, sizeof *o);
  o->nx = g->nx; o->ny = g->ny; o->nz = g->nz; o->N = g->N; o->nf = g->nf;
  o->top = g->top; o->jm = g->jm; o->kw0 = g->kw0; o->kf = g->kf;
  o->n_holes = g->nHoles; o->n_open = g->nOpen; o->af = g->Af; o->n_out = g->nOut; o->leak_cells = g->leak;
  o->pleat_ok = g->jm > g->top;
  o->h = g->h; o->pleat = g->pleat;
  for (int a = 0; a < 3; a++) { o->origin[a] = g->origin[a]; o->mn[a] = g->mn[a]; o->mx[a] = g->mx[a]; }
  const double h = g->h;
  o->volume_l = g->nf * std::pow(h, 3) / 1e6;   // summary (:229-230)
  o->inlet_cm2 = g->nOpen * h * h / 100;
  o->filter_cm2 = g->Af * h * h / 100;
  o->outlet_cm2 = g->leak * h * h / 100;
  o->outlet_cm2_real = g->has_outlet ? g->nOut * h * h / 100 : 0;
  o->frame_cy = g->fr.cy; o->frame_sy = g->fr.sy;
  o->kernel_launches = g->launches; o->h2d_bytes = g->h2d; o->d2h_bytes = g->d2h;
  o->ms_voxelize = g->ms_vox; o->ms_masks = g->ms_masks; o->ms_device = g->ms_device;
  return ABX_OK;
}

extern "C" int abx_geom_get_masks(const abx_geom *g, uint8_t *solid, uint8_t *fluid, uint8_t *opening,
                                  uint8_t *outlet, float *xc, float *dc, float *zc) {
  clear_stale_error();
  if (!g) return fail(ABX_ERR_INVALID_ARGUMENT, "geom_get_masks: null geometry");
  if (solid || fluid || outlet) CK(cudaSetDevice(g->device), "geom_get_masks");
  if (solid) CK(cudaMemcpy(solid, g->d_solid, (size_t)g->N, cudaMemcpyDeviceToHost), "geom_get_masks");
  if (fluid) CK(cudaMemcpy(fluid, g->d_fluid, (size_t)g->N, cudaMemcpyDeviceToHost), "geom_get_masks");
  if (outlet) CK(cudaMemcpy(outlet, g->d_outlet, (size_t)g->N, cudaMemcpyDeviceToHost), "geom_get_masks");
  if (opening) std::memcpy(opening, g->opening.data(), g->opening.size());
  if (xc) std::memcpy(xc, g->xc.data(), sizeof(float) * g->xc.size());
  if (dc) std::memcpy(dc, g->dc.data(), sizeof(float) * g->dc.size());
  if (zc) std::memcpy(zc, g->zc.data(), sizeof(float) * g->zc.size());
  return ABX_OK;
}

extern "C" int abx_geom_get_fine(const abx_geom *g, uint8_t *fine, size_t cap) {
  clear_stale_error();
  if (!g || !fine) return fail(ABX_ERR_INVALID_ARGUMENT, "geom_get_fine: null argument");
  const int64_t nfine = (int64_t)g->nxf * g->nyf * g->nzf;
  if ((int64_t)cap < nfine) return fail(ABX_ERR_INVALID_ARGUMENT, "geom_get_fine: buffer smaller than nxf*nyf*nzf");
  if (nfine >= (1ll << 31)) return fail(ABX_ERR_INVALID_ARGUMENT, "geom_get_fine: fine grid above 2^31 voxels");
  CK(cudaSetDevice(g->device), "geom_get_fine: set device");
  StreamHolder sh;
  CK(cudaStreamCreateWithFlags(&sh.s, cudaStreamNonBlocking), "geom_get_fine: stream");
  DevBuf dtris, dsolid, dslice, dfine;
  const size_t nfl = g->tris_local.size();
  CK(cudaMalloc(&dtris.p, sizeof(float) * std::max<size_t>(nfl, 1)), "geom_get_fine");
  if (nfl) CK(cudaMemcpyAsync(dtris.p, g->tris_local.data(), sizeof(float) * nfl, cudaMemcpyHostToDevice, sh.s), "geom_get_fine");
  CK(cudaMalloc(&dsolid.p, (size_t)g->N), "geom_get_fine");
  CK(cudaMalloc(&dslice.p, (size_t)g->nxf * g->nyf), "geom_get_fine");
  CK(cudaMalloc(&dfine.p, (size_t)nfine), "geom_get_fine");
  VoxJob job{(const float *)dtris.p, (int64_t)(nfl / 9), {g->origin[0], g->origin[1], g->origin[2]}, g->hf, g->nx, g->ny, g->nz, g->kf};
  VoxOut vo{(uint8_t *)dsolid.p, (uint8_t *)dslice.p, (uint8_t *)dfine.p};
  CK(run_voxelizer(job, vo, sh.s), "geom_get_fine: voxelize");
  CK(cudaMemcpyAsync(fine, dfine.p, (size_t)nfine, cudaMemcpyDeviceToHost, sh.s), "geom_get_fine: download");
  CK(cudaStreamSynchronize(sh.s), "geom_get_fine: sync");
  return ABX_OK;
}

// ------------------------------------------------------------------ simulation
static size_t store_bytes(int s) {
  switch (s) {
    case ABX_STORE_F32: case ABX_STORE_F32_EXACT: return 4;
    case ABX_STORE_F16: case ABX_STORE_BF16: return 2;
    case ABX_STORE_F64: return 8;
  }
  return 0;
}
static size_t acc_bytes(int s) { return s == ABX_STORE_F64 ? 8 : 4; }

struct abx_sim {
  abx_geom *g = nullptr;     // must outlive the run calls; the destructor does not touch it
  int device = 0;
  abx_run_params p{};
  cudaStream_t st = nullptr;
  void *d_f = nullptr, *d_acc = nullptr;
  float *d_ns = nullptr;
  int *d_status = nullptr;
  unsigned long long *d_diag = nullptr;
  double *d_hist = nullptr, *d_eval = nullptr;
  void *d_acc_snap = nullptr;      // running sums at the start of the convergence run's current window
  float *d_fmap = nullptr;
  int64_t *d_plist = nullptr;
  float *d_probe_vy = nullptr;     // probe scratch: -u_y of every probe cell
  double *d_probe_part = nullptr;  // probe scratch: per-block partial sums
  int probe_blocks = 1;
  int hist_cap = 0, nhist = 0;
  int step = 0, nacc = 0, form = 0;
  int Ain = 0, Af = 0, Lp = 0, nM = 0, nT = 0;
  double u0 = 0, tau0 = 0, sig = 0, aniso = 0, cs2s = 0, uface = 0;
  bool has_ns = false;
  TmaBlob tma;               // tensor maps of the TMA-pipelined step kernel (tma.ready when in use)
  int vec_V = 0;             // block width of the vectorised step kernel (0: the one-cell-per-lane kernel)
  bool va_ready = false;
  VecArgs va{};              // its work lists (the geometry's)
  bool use_graphs = true;    // ABX_NO_GRAPH=1 launches the step kernels one by one
  std::map<std::tuple<int, int, int>, cudaGraphExec_t> graphs;
  bool timing = false;
  std::vector<cudaEvent_t> ev_pool;
  size_t ev_used = 0;
  double step_ms = 0, step_ms_plain = 0, run_ms = 0, eval_ms = 0;
  int64_t step_launches = 0, step_launches_plain = 0, cell_updates = 0, launches = 0, h2d = 0, d2h = 0;
  std::vector<int> ev_kind;   // per event pair: 0 plain steps, 1 accumulating steps, 2 run, 3 evaluate
  std::vector<int> ev_nsteps;
  ~abx_sim() {
    cudaSetDevice(device);
    for (auto &kv : graphs) cudaGraphExecDestroy(kv.second);
    free_tma(&tma);
    for (auto e : ev_pool) cudaEventDestroy(e);
    cudaFree(d_f); cudaFree(d_acc); cudaFree(d_ns); cudaFree(d_status); cudaFree(d_diag); cudaFree(d_hist);
    cudaFree(d_eval); cudaFree(d_acc_snap);
    cudaFree(d_fmap); cudaFree(d_plist); cudaFree(d_probe_vy); cudaFree(d_probe_part);
    if (st) cudaStreamDestroy(st);
  }
};

static void offsets(const abx_geom &g, long long off[19]) {
  static const int CXv[19] = {0, 1, -1, 0, 0, 0, 0, 1, -1, 1, -1, 1, -1, 1, -1, 0, 0, 0, 0};
  static const int CYv[19] = {0, 0, 0, 1, -1, 0, 0, 1, -1, -1, 1, 0, 0, 0, 0, 1, -1, 1, -1};
  static const int CZv[19] = {0, 0, 0, 0, 0, 1, -1, 0, 0, 0, 0, 1, -1, -1, 1, 1, -1, -1, 1};
  for (int q = 0; q < 19; q++) off[q] = ((long long)CXv[q] * g.ny + CYv[q]) * g.nzp + CZv[q];
}

static StepArgs step_args(const abx_sim &s) {
  StepArgs a{};
  a.f = s.d_f; a.mask = s.g->d_mask; a.seg = s.g->d_seg; a.nseg = s.g->nseg; a.Np = s.g->Np;
  a.acc = s.d_acc; a.ns = s.has_ns ? s.d_ns : nullptr; a.status = s.d_status; a.diag = s.d_diag;
  offsets(*s.g, a.off);
  a.u0 = s.u0; a.tau0 = s.tau0; a.sig = s.sig; a.aniso = s.aniso; a.cs2s = s.cs2s;
  a.u0f = (float)s.u0; a.tau0f = (float)s.tau0; a.sigf = (float)s.sig; a.anisof = (float)s.aniso;
  a.cs2sf = (float)s.cs2s;
  return a;
}
static StateArgs state_args(const abx_sim &s) {
  StateArgs a{};
  a.f = s.d_f; a.mask = s.g->d_mask; a.Np = s.g->Np; a.acc = s.d_acc; a.cells = s.g->d_cells;
  a.ncells = s.g->nf; a.status = s.d_status; a.form = s.form;
  offsets(*s.g, a.off);
  return a;
}

static int sim_reset(abx_sim *s) {
  CK(cudaSetDevice(s->g->device), "sim: set device");
  CK(launch_init(s->p.storage, state_args(*s), s->st), "sim: init");
  CK(cudaMemsetAsync(s->d_status, 0, sizeof(int), s->st), "sim: init");
  CK(cudaMemsetAsync(s->d_diag, 0, 8 * sizeof(unsigned long long), s->st), "sim: init");
  CK(cudaStreamSynchronize(s->st), "sim: init");
  s->step = 0; s->nacc = 0; s->form = 0; s->nhist = 0;
  s->step_ms = 0; s->step_ms_plain = 0; s->run_ms = 0; s->eval_ms = 0;
  s->step_launches = 0; s->step_launches_plain = 0; s->cell_updates = 0;
  s->launches = 1; s->h2d = 0; s->d2h = 0;
  s->ev_used = 0; s->ev_kind.clear(); s->ev_nsteps.clear();
  return ABX_OK;
}

static int vec_index(int V) { return V == 2 ? 0 : V == 4 ? 1 : V == 8 ? 2 : -1; }

// The geometry's interior-block and boundary-segment lists for block width V (built once, kept on the device).
static int geom_vec_lists(abx_geom &g, int V, cudaStream_t st) {
  const int vi = vec_index(V);
  if (vi < 0) return fail(ABX_ERR_INVALID_ARGUMENT, "vector lists: block width %d", V);
  abx_geom::VecLists &L = g.vec[vi];
  if (L.ready) return ABX_OK;
  CK(cudaSetDevice(g.device), "vector lists: set device");
  const int64_t items = (int64_t)g.nseg * 32;
  const int64_t nb = prep_compact_blocks(std::max<int64_t>(items, 1));
  DevBuf dbc, doff, dcnt;
  CK(cudaMalloc(&dbc.p, sizeof(uint32_t) * std::max<int64_t>(nb, 1)), "vector lists");
  CK(cudaMalloc(&doff.p, sizeof(unsigned long long) * (nb + 1)), "vector lists");
  CK(cudaMalloc(&dcnt.p, 3 * sizeof(unsigned long long)), "vector lists");
  CK(prep_vec_lists(g.d_seg, g.nseg, g.d_mask, V, nullptr, nullptr, (uint32_t *)dbc.p, (unsigned long long *)doff.p,
                    (unsigned long long *)dcnt.p, st), "vector lists: count");
  unsigned long long c[3];
  CK(cudaMemcpyAsync(c, dcnt.p, sizeof c, cudaMemcpyDeviceToHost, st), "vector lists");
  CK(cudaStreamSynchronize(st), "vector lists");
  CK(cudaMalloc((void **)&L.d_blk, sizeof(uint32_t) * std::max<unsigned long long>(c[0] + c[1], 1)), "vector lists");
  CK(cudaMalloc((void **)&L.d_bcell, sizeof(uint32_t) * std::max<unsigned long long>(c[2], 1)), "vector lists");
  CK(prep_vec_lists(g.d_seg, g.nseg, g.d_mask, V, L.d_blk, L.d_bcell, (uint32_t *)dbc.p, (unsigned long long *)doff.p,
                    (unsigned long long *)dcnt.p, st), "vector lists: write");
  CK(cudaStreamSynchronize(st), "vector lists");
  L.n_bulk = (uint32_t)c[0]; L.n_filter = (uint32_t)c[1]; L.nbcell = (uint32_t)c[2];
  L.ready = true;
  return ABX_OK;
}

// Block width of the vectorised step kernel for a storage; opt-in with ABX_VEC=1 (ABX_VEC_V=n: that width where the
// storage has it).  The one-cell-per-lane kernel is the default: it is the faster of the two on GB300.
static int vec_width(int storage) {
  const char *on = std::getenv("ABX_VEC");
  if (!on || on[0] != '1') return 0;
  int want = 0;
  if (const char *e = std::getenv("ABX_VEC_V")) want = std::atoi(e);
  switch (storage) {
    case ABX_STORE_F32: return (want == 2 || want == 4) ? want : 2;
    case ABX_STORE_F16: case ABX_STORE_BF16: return (want == 2 || want == 4) ? want : 4;
  }
  return 0;
}

extern "C" int abx_sim_create(abx_geom *g, const abx_run_params *p, const float *ns, abx_sim **out) {
  clear_stale_error();
  if (!out) return fail(ABX_ERR_INVALID_ARGUMENT, "sim_create: null output");
  *out = nullptr;
  if (!g) return fail(ABX_ERR_NOT_PREPARED, "Bitte zuerst die Geometrie prüfen.");
  if (!p) return fail(ABX_ERR_INVALID_ARGUMENT, "sim_create: null parameters");
  if (p->storage < ABX_STORE_F32 || p->storage > ABX_STORE_F64) return fail(ABX_ERR_INVALID_ARGUMENT, "sim_create: unknown storage");
  if (p->steps < 0 || p->every <= 0) return fail(ABX_ERR_INVALID_ARGUMENT, "sim_create: steps >= 0 and every > 0 required");
  if (p->storage == ABX_STORE_BF16 && !(p->flags & ABX_RUN_ALLOW_BF16))
    return fail(ABX_ERR_INVALID_ARGUMENT,
                "sim_create: bfloat16 storage keeps 8 significant bits of f - w_i, too few for the density "
                "differences behind zeta (6.5 %% off the float64 run on a 512x256x384-cell airbox, where float16 "
                "stays within 0.5 %%); use float16, or set ABX_RUN_ALLOW_BF16 to run it anyway");
  if (g->nf <= 0) return fail(ABX_ERR_INVALID_ARGUMENT, "sim_create: geometry has no fluid cells");
  std::unique_ptr<abx_sim> S(new abx_sim());
  abx_sim &s = *S;
  s.g = g; s.p = *p; s.device = g->device;
  // setupSim scalars (src/engine.js:246-263)
  s.Ain = g->Ain; s.Lp = g->Lp;
  std::vector<int64_t> plist(g->layer_m);
  s.nM = (int)plist.size();
  plist.insert(plist.end(), g->layer_t.begin(), g->layer_t.end());
  s.nT = (int)plist.size() - s.nM;
  s.Af = s.nM;
  s.u0 = p->u; s.tau0 = p->tau; s.aniso = p->aniso;
  s.uface = s.u0 * s.Ain / s.Af;
  s.sig = p->K * 0.5 * s.u0 * s.u0 / (s.uface * std::max(s.Lp, 1));
  s.cs2s = 18 * M_SQRT2 * 0.17 * 0.17;
  CK(cudaSetDevice(g->device), "sim_create: set device");
  CK(cudaStreamCreateWithFlags(&s.st, cudaStreamNonBlocking), "sim_create: stream");
  int64_t create_h2d = (int64_t)(sizeof(int64_t) * plist.size()) + (ns ? (int64_t)sizeof(float) * g->nf : 0);
  CK(cudaMalloc(&s.d_f, store_bytes(p->storage) * 19 * (size_t)g->Np), "sim_create: populations");
  CK(cudaMalloc(&s.d_acc, acc_bytes(p->storage) * 4 * (size_t)g->Np), "sim_create: averages");
  CK(cudaMalloc((void **)&s.d_status, sizeof(int)), "sim_create: status");
  CK(cudaMalloc((void **)&s.d_diag, 8 * sizeof(unsigned long long)), "sim_create: diagnostics");
  s.hist_cap = p->steps / p->every + 2;
  CK(cudaMalloc((void **)&s.d_hist, sizeof(double) * 4 * s.hist_cap), "sim_create: history");
  CK(cudaMalloc((void **)&s.d_eval, sizeof(double) * 16), "sim_create: metrics");
  CK(cudaMalloc((void **)&s.d_fmap, sizeof(float) * (size_t)g->nx * g->nz), "sim_create: fmap");
  CK(cudaMalloc((void **)&s.d_plist, sizeof(int64_t) * std::max<size_t>(plist.size(), 1)), "sim_create: probe list");
  if (!plist.empty())
    CK(cudaMemcpyAsync(s.d_plist, plist.data(), sizeof(int64_t) * plist.size(), cudaMemcpyHostToDevice, s.st), "sim_create");
  s.probe_blocks = (int)std::min<size_t>(std::max<size_t>((plist.size() + kProbeThreads - 1) / kProbeThreads, 1), 152 * 4);
  CK(cudaMalloc((void **)&s.d_probe_vy, sizeof(float) * std::max<size_t>(plist.size(), 1)), "sim_create: probe scratch");
  CK(cudaMalloc((void **)&s.d_probe_part, sizeof(double) * 2 * s.probe_blocks), "sim_create: probe scratch");
  if (ns) {
    s.has_ns = true;
    CK(cudaMalloc((void **)&s.d_ns, sizeof(float) * (size_t)g->Np), "sim_create: ns");
    CK(cudaMemsetAsync(s.d_ns, 0, sizeof(float) * (size_t)g->Np, s.st), "sim_create: ns");
    DevBuf tmp;
    CK(cudaMalloc(&tmp.p, sizeof(float) * (size_t)g->nf), "sim_create: ns");
    CK(cudaMemcpyAsync(tmp.p, ns, sizeof(float) * (size_t)g->nf, cudaMemcpyHostToDevice, s.st), "sim_create: ns");
    CK(launch_scatter_f32((const float *)tmp.p, g->d_cells, g->nf, s.d_ns, s.st), "sim_create: ns");
    CK(cudaStreamSynchronize(s.st), "sim_create: ns");
  }
  if (const char *ng = std::getenv("ABX_NO_GRAPH")) s.use_graphs = ng[0] != '1';
  // TMA-pipelined step kernel for the float32-collision storages, opt-in with ABX_TMA=1 (the direct-load
  // kernel is the default: it is the faster of the two on GB300)
  const char *use_tma = std::getenv("ABX_TMA");
  if ((p->storage == ABX_STORE_F32 || p->storage == ABX_STORE_F16 || p->storage == ABX_STORE_BF16) &&
      use_tma && use_tma[0] == '1') {
    cudaError_t te = make_tma(p->storage, step_args(s), &s.tma);
    if (te != cudaSuccess && te != cudaErrorNotSupported) return cuda_fail(te, "sim_create: tensor maps");
    cudaGetLastError();
  }
  // the vectorised step kernel (not with a partial bounce-back field, nor next to the opt-in TMA kernel); its
  // work lists are built before the first step
  if (!ns && !s.tma.ready) s.vec_V = vec_width(p->storage);
  if (s.vec_V) CK(prepare_step_vec(p->storage, s.vec_V), "sim_create: vector kernel");
  int rc = sim_reset(&s);
  if (rc) return rc;
  s.h2d = create_h2d;
  if (ns) s.launches += 1;
  *out = S.release();
  return ABX_OK;
}

extern "C" void abx_sim_free(abx_sim *s) { delete s; }

extern "C" int abx_sim_get_info(const abx_sim *s, abx_sim_info *o) {
  if (!s || !o) return fail(ABX_ERR_INVALID_ARGUMENT, "sim_get_info: null argument");
  std::memset(o, 0, sizeof *o);
  o->NF = s->g->nf; o->Ain = s->Ain; o->Af = s->Af; o->Lp = s->Lp; o->n_layer_m = s->nM; o->n_layer_t = s->nT;
  o->u0 = s->u0; o->tau0 = s->tau0; o->sig = s->sig; o->aniso = s->aniso; o->cs2s = s->cs2s; o->uface = s->uface;
  o->step = s->step; o->nacc = s->nacc; o->Np = s->g->Np;
  o->state_bytes = (int64_t)(store_bytes(s->p.storage) * 19 + acc_bytes(s->p.storage) * 4) * s->g->Np;
  o->tma_pipeline = s->tma.ready ? 1 : 0;
  o->vec_width = s->vec_V;
  o->vec_interior_cells = s->va_ready ? (int64_t)(s->va.n_bulk + s->va.n_filter) * s->vec_V : 0;
  return ABX_OK;
}

extern "C" int abx_sim_reset(abx_sim *s) {
  clear_stale_error();
  if (!s) return fail(ABX_ERR_INVALID_ARGUMENT, "sim_reset: null simulation");
  return sim_reset(s);
}

static cudaEvent_t next_event(abx_sim *s) {
  if (s->ev_used == s->ev_pool.size()) {
    cudaEvent_t e;
    if (cudaEventCreate(&e) != cudaSuccess) return nullptr;
    s->ev_pool.push_back(e);
  }
  return s->ev_pool[s->ev_used++];
}

// Launch n steps starting at the current step (odd kernel when the state is
// in "out" form), as one CUDA graph per (n, form, accumulate).
static int run_steps(abx_sim *s, int n, bool acc) {
  if (n <= 0) return ABX_OK;
  if (s->vec_V && !s->va_ready) {
    if (int rc = geom_vec_lists(*s->g, s->vec_V, s->st)) return rc;
    const abx_geom::VecLists &L = s->g->vec[vec_index(s->vec_V)];
    s->va.blk = L.d_blk; s->va.n_bulk = L.n_bulk; s->va.n_filter = L.n_filter;
    s->va.bcell = L.d_bcell; s->va.nbcell = L.nbcell;
    s->va_ready = true;
  }
  if (!s->use_graphs) {
    const StepArgs a = step_args(*s);
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    if (s->timing) {
      e0 = next_event(s); e1 = next_event(s);
      if (e0 && e1) { cudaEventRecord(e0, s->st); s->ev_kind.push_back(acc ? 1 : 0); s->ev_nsteps.push_back(n); }
    }
    for (int i = 0; i < n; i++) {
      CK(s->vec_V ? launch_step_vec(s->p.storage, s->vec_V, s->form == 0, acc, a, s->va, s->st)
                  : launch_step(s->p.storage, s->form == 0, acc, s->has_ns, a, s->tma.ready ? &s->tma : nullptr, s->st),
         "run: step");
      s->form ^= 1;
    }
    if (e0 && e1) cudaEventRecord(e1, s->st);
    s->step += n;
    if (acc) s->nacc += n;
    s->step_launches += n;
    if (!acc) s->step_launches_plain += n;
    s->launches += n;
    s->cell_updates += (int64_t)n * s->g->nf;
    return ABX_OK;
  }
  const auto key = std::make_tuple(n, s->form, acc ? 1 : 0);
  auto it = s->graphs.find(key);
  if (it == s->graphs.end()) {
    const StepArgs a = step_args(*s);
    cudaGraph_t graph;
    CK(cudaStreamBeginCapture(s->st, cudaStreamCaptureModeThreadLocal), "run: capture");
    cudaError_t le = cudaSuccess;
    int form = s->form;
    for (int i = 0; i < n && le == cudaSuccess; i++) {
      le = s->vec_V ? launch_step_vec(s->p.storage, s->vec_V, form == 0, acc, a, s->va, s->st)
                    : launch_step(s->p.storage, form == 0, acc, s->has_ns, a, s->tma.ready ? &s->tma : nullptr, s->st);
      form ^= 1;
    }
    cudaError_t ce = cudaStreamEndCapture(s->st, &graph);
    if (le != cudaSuccess) { if (ce == cudaSuccess) cudaGraphDestroy(graph); return cuda_fail(le, "run: step launch"); }
    CK(ce, "run: capture");
    cudaGraphExec_t exec;
    cudaError_t ie = cudaGraphInstantiate(&exec, graph, 0);
    cudaGraphDestroy(graph);
    CK(ie, "run: graph instantiate");
    it = s->graphs.emplace(key, exec).first;
  }
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  if (s->timing) {
    e0 = next_event(s); e1 = next_event(s);
    if (e0 && e1) { cudaEventRecord(e0, s->st); s->ev_kind.push_back(acc ? 1 : 0); s->ev_nsteps.push_back(n); }
  }
  CK(cudaGraphLaunch(it->second, s->st), "run: graph launch");
  if (e0 && e1) cudaEventRecord(e1, s->st);
  s->form ^= (n & 1);
  s->step += n;
  if (acc) s->nacc += n;
  s->step_launches += n;
  if (!acc) s->step_launches_plain += n;
  s->launches += n;
  s->cell_updates += (int64_t)n * s->g->nf;
  return ABX_OK;
}

static int collect_timing(abx_sim *s) {
  if (!s->timing) return ABX_OK;
  CK(cudaStreamSynchronize(s->st), "timing: sync");
  for (size_t i = 0; i + 1 < s->ev_used; i += 2) {
    float ms = 0;
    CK(cudaEventElapsedTime(&ms, s->ev_pool[i], s->ev_pool[i + 1]), "timing: elapsed");
    const int kind = s->ev_kind[i / 2];
    if (kind <= 1) s->step_ms += ms;
    if (kind == 0) s->step_ms_plain += ms;
    if (kind == 2) s->run_ms += ms;
    if (kind == 3) s->eval_ms += ms;
  }
  s->ev_used = 0;
  s->ev_kind.clear();
  s->ev_nsteps.clear();
  return ABX_OK;
}

static int pipeline_timeout(abx_sim *s) {
  unsigned long long d[8] = {0, 0, 0, 0, 0, 0, 0, 0};
  cudaMemcpy(d, s->d_diag, sizeof d, cudaMemcpyDeviceToHost);
  return fail(ABX_ERR_CUDA,
              "step kernel: a shared-memory pipeline wait timed out (run halted; block %llu, barrier word %016llx, "
              "tiles %llu, grid %llu, iteration %llu, tile %llu, armed bytes %llu, smem %llu odd %llu acc %llu, "
              "segments %llu)",
              d[1], d[2], d[3] & 0xffffffffull, d[3] >> 32, d[4] & 0xffffffffull, d[4] >> 32, d[5],
              d[6] & 0xffffffffull, (d[6] >> 32) & 1, (d[6] >> 33) & 1, d[7]);
}

extern "C" int abx_sim_step(abx_sim *s, int n, int accumulate) {
  clear_stale_error();
  if (!s || n < 0) return fail(ABX_ERR_INVALID_ARGUMENT, "sim_step: bad argument");
  CK(cudaSetDevice(s->g->device), "sim_step: set device");
  int rc = run_steps(s, n, accumulate != 0);
  if (rc) return rc;
  rc = collect_timing(s);
  if (rc) return rc;
  CK(cudaStreamSynchronize(s->st), "sim_step: sync");
  int st = 0;
  CK(cudaMemcpy(&st, s->d_status, sizeof(int), cudaMemcpyDeviceToHost), "sim_step: status");
  if (st == -2) return fail(ABX_ERR_CUDA, "step kernel: a TMA copy failed its alignment check (run halted)");
  if (st < 0) return pipeline_timeout(s);
  return ABX_OK;
}

static int check_unstable(abx_sim *s) {
  int st = 0;
  CK(cudaMemcpyAsync(&st, s->d_status, sizeof(int), cudaMemcpyDeviceToHost, s->st), "run: status");
  CK(cudaStreamSynchronize(s->st), "run: status");
  if (st == -2) return fail(ABX_ERR_CUDA, "step kernel: a TMA copy failed its alignment check (run halted)");
  if (st < 0) return pipeline_timeout(s);
  if (st)
    return fail(ABX_ERR_UNSTABLE,
                "Rechnung instabil bei Schritt %d. Zellgröße vergrößern oder Viskosität (tau) erhöhen.", st);
  return ABX_OK;
}

// The step loop of simulate (src/engine.js:346-355): averaging for steps past
// steps - avg, a progress check at every multiple of `every` and at the end.
extern "C" int abx_sim_run(abx_sim *s, abx_progress_fn cb, void *user) {
  clear_stale_error();
  if (!s) return fail(ABX_ERR_INVALID_ARGUMENT, "sim_run: null simulation");
  CK(cudaSetDevice(s->g->device), "sim_run: set device");
  const int steps = s->p.steps, avg = s->p.avg, every = s->p.every;
  const int start_acc = steps - avg;
  const auto t0 = std::chrono::steady_clock::now();
  StateArgs sa = state_args(*s);
  cudaEvent_t r0 = nullptr, r1 = nullptr;
  if (s->timing) { r0 = next_event(s); r1 = next_event(s); if (r0 && r1) { cudaEventRecord(r0, s->st); s->ev_kind.push_back(2); s->ev_nsteps.push_back(0); } }
  // r0/r1 occupy one event pair slot; the step chunks use the following slots
  while (s->step < steps) {
    int stop = (s->step / every + 1) * every;
    if (stop > steps) stop = steps;
    if (s->step < start_acc && stop > start_acc) stop = start_acc;
    const bool acc = s->step >= start_acc;
    int rc = run_steps(s, stop - s->step, acc);
    if (rc) return rc;
    if (s->step % every == 0 || s->step == steps) {
      if (s->nhist >= s->hist_cap) return fail(ABX_ERR_INVALID_ARGUMENT, "sim_run: history full (reset the simulation)");
      ProbeArgs pr{};
      pr.plist = s->d_plist; pr.nM = s->nM; pr.nT = s->nT; pr.step = s->step; pr.slot = s->nhist;
      pr.Ain = s->Ain; pr.u0 = s->u0; pr.hist = s->d_hist;
      pr.vy = s->d_probe_vy; pr.part = s->d_probe_part; pr.nblocks = s->probe_blocks;
      sa.form = s->form;
      CK(launch_probe(s->p.storage, sa, pr, s->st), "sim_run: probe");
      s->nhist++;
      s->launches += 2;
      if (cb) {
        double h[4];
        CK(cudaMemcpyAsync(h, s->d_hist + 4 * (s->nhist - 1), sizeof h, cudaMemcpyDeviceToHost, s->st), "sim_run: probe");
        s->d2h += sizeof h;
        CK(cudaStreamSynchronize(s->st), "sim_run: probe");
        if (!std::isfinite(h[3]))
          return fail(ABX_ERR_UNSTABLE,
                      "Rechnung instabil bei Schritt %d. Zellgröße vergrößern oder Viskosität (tau) erhöhen.", s->step);
        const double el = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
        abx_progress info{s->step, steps, h[1], h[2], el, el / s->step * (steps - s->step),
                          (double)s->g->nf * s->step / el / 1e6};
        if (cb(&info, user)) return fail(ABX_ERR_CANCELLED, "Rechnung abgebrochen.");
      }
    }
  }
  if (r0 && r1) cudaEventRecord(r1, s->st);
  int rc = collect_timing(s);
  if (rc) return rc;
  s->d2h += sizeof(int);
  return check_unstable(s);
}

extern "C" int abx_sim_get_f(abx_sim *s, float *f) {
  clear_stale_error();
  if (!s || !f) return fail(ABX_ERR_INVALID_ARGUMENT, "sim_get_f: null argument");
  CK(cudaSetDevice(s->g->device), "sim_get_f");
  DevBuf tmp;
  const size_t n = (size_t)19 * s->g->nf;
  CK(cudaMalloc(&tmp.p, sizeof(float) * n), "sim_get_f");
  CK(launch_get_f(s->p.storage, state_args(*s), (float *)tmp.p, s->st), "sim_get_f");
  s->launches++; s->d2h += (int64_t)(sizeof(float) * n);
  CK(cudaMemcpyAsync(f, tmp.p, sizeof(float) * n, cudaMemcpyDeviceToHost, s->st), "sim_get_f");
  CK(cudaStreamSynchronize(s->st), "sim_get_f");
  return ABX_OK;
}

extern "C" int abx_sim_set_f(abx_sim *s, const float *f) {
  clear_stale_error();
  if (!s || !f) return fail(ABX_ERR_INVALID_ARGUMENT, "sim_set_f: null argument");
  CK(cudaSetDevice(s->g->device), "sim_set_f");
  DevBuf tmp;
  const size_t n = (size_t)19 * s->g->nf;
  CK(cudaMalloc(&tmp.p, sizeof(float) * n), "sim_set_f");
  CK(cudaMemcpyAsync(tmp.p, f, sizeof(float) * n, cudaMemcpyHostToDevice, s->st), "sim_set_f");
  CK(launch_set_f(s->p.storage, state_args(*s), (const float *)tmp.p, s->st), "sim_set_f");
  s->launches++; s->h2d += (int64_t)(sizeof(float) * n);
  CK(cudaStreamSynchronize(s->st), "sim_set_f");
  s->form = 0;
  return ABX_OK;
}

extern "C" int abx_sim_clear_acc(abx_sim *s) {
  clear_stale_error();
  if (!s) return fail(ABX_ERR_INVALID_ARGUMENT, "sim_clear_acc: null simulation");
  CK(cudaSetDevice(s->g->device), "sim_clear_acc");
  CK(cudaMemsetAsync(s->d_acc, 0, acc_bytes(s->p.storage) * 4 * (size_t)s->g->Np, s->st), "sim_clear_acc");
  s->nacc = 0;
  return ABX_OK;
}

extern "C" int abx_sim_get_acc(abx_sim *s, float *acc) {
  clear_stale_error();
  if (!s || !acc) return fail(ABX_ERR_INVALID_ARGUMENT, "sim_get_acc: null argument");
  CK(cudaSetDevice(s->g->device), "sim_get_acc");
  DevBuf tmp;
  const size_t n = (size_t)4 * s->g->nf;
  CK(cudaMalloc(&tmp.p, sizeof(float) * n), "sim_get_acc");
  CK(launch_get_acc(s->p.storage, state_args(*s), (float *)tmp.p, s->nacc, s->st), "sim_get_acc");
  s->launches++; s->d2h += (int64_t)(sizeof(float) * n);
  CK(cudaMemcpyAsync(acc, tmp.p, sizeof(float) * n, cudaMemcpyDeviceToHost, s->st), "sim_get_acc");
  CK(cudaStreamSynchronize(s->st), "sim_get_acc");
  return ABX_OK;
}

static int sim_evaluate(abx_sim *s, abx_metrics *m, float *fmap, double *hist, int hist_cap, int *nhist,
                        const void *base, int base_nacc);

extern "C" int abx_sim_evaluate(abx_sim *s, abx_metrics *m, float *fmap, double *hist, int hist_cap, int *nhist) {
  clear_stale_error();
  if (!s || !m) return fail(ABX_ERR_INVALID_ARGUMENT, "sim_evaluate: null argument");
  return sim_evaluate(s, m, fmap, hist, hist_cap, nhist, nullptr, 0);
}

// evaluate() of the running averages, or (base != null) of the averages of the steps since the snapshot base
static int sim_evaluate(abx_sim *s, abx_metrics *m, float *fmap, double *hist, int hist_cap, int *nhist,
                        const void *base, int base_nacc) {
  CK(cudaSetDevice(s->g->device), "sim_evaluate");
  const abx_geom &g = *s->g;
  EvalArgs e{};
  e.nx = g.nx; e.ny = g.ny; e.nz = g.nz; e.nzp = g.nzp; e.kpad = g.kpad; e.jm = g.jm;
  e.jb = first_ge(g.dc, g.pleat + 2 * g.h);
  e.nacc = s->nacc; e.u0 = s->u0; e.opening = g.d_opening; e.ns = s->has_ns ? s->d_ns : nullptr;
  e.fmap = s->d_fmap; e.out = s->d_eval;
  e.base = base; e.base_nacc = base_nacc;
  cudaEvent_t v0 = nullptr, v1 = nullptr;
  if (s->timing) { v0 = next_event(s); v1 = next_event(s); if (v0 && v1) { cudaEventRecord(v0, s->st); s->ev_kind.push_back(3); s->ev_nsteps.push_back(0); } }
  CK(launch_evaluate(s->p.storage, state_args(*s), e, s->st), "sim_evaluate");
  s->launches++;
  double o[13];
  CK(cudaMemcpyAsync(o, s->d_eval, sizeof o, cudaMemcpyDeviceToHost, s->st), "sim_evaluate");
  if (fmap)
    CK(cudaMemcpyAsync(fmap, s->d_fmap, sizeof(float) * (size_t)g.nx * g.nz, cudaMemcpyDeviceToHost, s->st), "sim_evaluate");
  std::vector<double> hh((size_t)4 * std::max(s->nhist, 1));
  if (s->nhist) CK(cudaMemcpyAsync(hh.data(), s->d_hist, sizeof(double) * 4 * s->nhist, cudaMemcpyDeviceToHost, s->st), "sim_evaluate");
  if (v0 && v1) cudaEventRecord(v1, s->st);
  s->d2h += (int64_t)(sizeof o + (fmap ? sizeof(float) * (size_t)g.nx * g.nz : 0) + sizeof(double) * 4 * s->nhist);
  CK(cudaStreamSynchronize(s->st), "sim_evaluate");
  { int trc = collect_timing(s); if (trc) return trc; }
  std::memset(m, 0, sizeof *m);
  m->gamma = o[0]; m->gammaCore = o[1]; m->lowCore = o[2]; m->highCore = o[3]; m->reverse = o[4];
  m->maxToMean = o[5]; m->zeta = o[6];
  m->inlet_cm2 = s->Ain * g.h * g.h / 100; m->filter_cm2 = s->Af * g.h * g.h / 100;
  m->wm = o[7]; m->cm = o[8]; m->n = (int)o[9]; m->cn = (int)o[10]; m->pinN = (int)o[11]; m->pbN = (int)o[12];
  m->jb = e.jb;
  if (hist || nhist) {
    int k = 0;
    for (int i = 0; i < s->nhist; i++) {
      if (!std::isfinite(hh[4 * i + 3])) break;  // the reference throws before recording that entry
      if (hist && k < hist_cap) { hist[3 * k] = hh[4 * i]; hist[3 * k + 1] = hh[4 * i + 1]; hist[3 * k + 2] = hh[4 * i + 2]; }
      k++;
    }
    if (nhist) *nhist = k;
  }
  return ABX_OK;
}

extern "C" int abx_simulate(abx_geom *g, const abx_run_params *p, const float *ns, abx_progress_fn cb, void *user,
                            abx_metrics *m, float *fmap, double *hist, int hist_cap, int *nhist) {
  abx_sim *s = nullptr;
  int rc = abx_sim_create(g, p, ns, &s);
  if (rc) return rc;
  rc = abx_sim_run(s, cb, user);
  if (!rc) rc = abx_sim_evaluate(s, m, fmap, hist, hist_cap, nhist);
  std::string keep = g_err;
  abx_sim_free(s);
  g_err = keep;
  return rc;
}

extern "C" int abx_voxelize_static(const float *d_tris, size_t nfloats, const double origin[3], double h, int nx,
                                   int ny, int nz, uint8_t *d_vox, void *stream) {
  char msg[512] = {0};
  const int rc = voxelize_static(d_tris, nfloats, origin, h, nx, ny, nz, d_vox, (cudaStream_t)stream, msg, sizeof msg);
  if (rc) return fail(rc, "%s", msg);
  return ABX_OK;
}

extern "C" int abx_sim_set_timing(abx_sim *s, int enabled) {
  if (!s) return fail(ABX_ERR_INVALID_ARGUMENT, "sim_set_timing: null simulation");
  s->timing = enabled != 0;
  return ABX_OK;
}

extern "C" int abx_sim_get_timing(const abx_sim *s, abx_sim_timing *o) {
  if (!s || !o) return fail(ABX_ERR_INVALID_ARGUMENT, "sim_get_timing: null argument");
  std::memset(o, 0, sizeof *o);
  o->step_ms = s->step_ms; o->step_launches = s->step_launches;
  o->step_ms_plain = s->step_ms_plain; o->step_launches_plain = s->step_launches_plain;
  o->run_ms = s->run_ms; o->eval_ms = s->eval_ms; o->cell_updates = s->cell_updates;
  o->kernel_launches = s->launches; o->h2d_bytes = s->h2d; o->d2h_bytes = s->d2h;
  return ABX_OK;
}

// ------------------------------------------------------------------ learned warm start
struct abx_net {
  WarmNet net;
};

static GridDesc grid_desc(const abx_geom &g) {
  GridDesc d{};
  d.nx = g.nx; d.ny = g.ny; d.nz = g.nz; d.nzp = g.nzp; d.kpad = g.kpad; d.Np = g.Np; d.mask = g.d_mask;
  return d;
}

extern "C" int abx_net_create(const abx_net_params *p, abx_net **out) {
  clear_stale_error();
  if (!p || !out) return fail(ABX_ERR_INVALID_ARGUMENT, "net_create: null argument");
  *out = nullptr;
  const int R = p->res, L = p->levels;
  if (R < 8 || R > 256 || (R & (R - 1))) return fail(ABX_ERR_INVALID_ARGUMENT, "net_create: res must be a power of two in [8, 256]");
  if (L < 1 || L > 6 || (R >> (L - 1)) < 2) return fail(ABX_ERR_INVALID_ARGUMENT, "net_create: levels must be 1..6 with res / 2^(levels-1) >= 2");
  if (p->base <= 0 || p->base % 8 || (p->base << (L - 1)) > 512) return fail(ABX_ERR_INVALID_ARGUMENT, "net_create: base must be a positive multiple of 8 with base * 2^(levels-1) <= 512");
  int nd = 0;
  CK(cudaGetDeviceCount(&nd), "net_create: device count");
  if (p->device < 0 || p->device >= nd) return fail(ABX_ERR_INVALID_ARGUMENT, "net_create: no device %d", p->device);
  std::unique_ptr<abx_net> n(new abx_net());
  n->net.device = p->device;
  cudaError_t e = n->net.init(R, p->base, L, p->device, p->seed, p->coords != 0);
  if (e != cudaSuccess) return cuda_fail(e, "net_create");
  // convolutions on the tensor cores where the GPU has them, unless ABX_NN_TC=0
  const char *tc = std::getenv("ABX_NN_TC");
  n->net.use_tc = nn_tc_available() && !(tc && tc[0] == '0');
  *out = n.release();
  return ABX_OK;
}

extern "C" int abx_net_set_tensor_cores(abx_net *n, int on) {
  clear_stale_error();
  if (!n) return fail(ABX_ERR_INVALID_ARGUMENT, "net_set_tensor_cores: null network");
  CK(cudaSetDevice(n->net.device), "net_set_tensor_cores");
  if (on && !nn_tc_available()) return fail(ABX_ERR_INVALID_ARGUMENT, "net_set_tensor_cores: this GPU has no tcgen05 tensor cores");
  CK(cudaStreamSynchronize(n->net.st), "net_set_tensor_cores");
  n->net.use_tc = on != 0;
  if (!on) n->net.tc_free();
  return ABX_OK;
}

extern "C" void abx_net_free(abx_net *n) { delete n; }

extern "C" int abx_net_get_info(const abx_net *n, abx_net_info *o) {
  if (!n || !o) return fail(ABX_ERR_INVALID_ARGUMENT, "net_get_info: null argument");
  std::memset(o, 0, sizeof *o);
  o->res = n->net.R; o->base = n->net.base; o->levels = n->net.levels;
  o->in_channels = n->net.n_in; o->out_channels = WarmNet::kOut;
  o->n_samples = (int)n->net.samples.size(); o->n_params = n->net.n_params;
  o->tensor_cores = n->net.use_tc ? 1 : 0;
  return ABX_OK;
}

extern "C" int abx_net_get_weights(abx_net *n, float *w) {
  clear_stale_error();
  if (!n || !w) return fail(ABX_ERR_INVALID_ARGUMENT, "net_get_weights: null argument");
  CK(cudaSetDevice(n->net.device), "net_get_weights");
  CK(cudaMemcpyAsync(w, n->net.d_p, sizeof(float) * n->net.n_params, cudaMemcpyDeviceToHost, n->net.st), "net_get_weights");
  CK(cudaStreamSynchronize(n->net.st), "net_get_weights");
  return ABX_OK;
}

extern "C" int abx_net_set_weights(abx_net *n, const float *w) {
  clear_stale_error();
  if (!n || !w) return fail(ABX_ERR_INVALID_ARGUMENT, "net_set_weights: null argument");
  for (int64_t i = 0; i < n->net.n_params; i++)
    if (!std::isfinite(w[i])) return fail(ABX_ERR_INVALID_ARGUMENT, "net_set_weights: weight %lld is not finite", (long long)i);
  CK(cudaSetDevice(n->net.device), "net_set_weights");
  CK(cudaMemcpyAsync(n->net.d_p, w, sizeof(float) * n->net.n_params, cudaMemcpyHostToDevice, n->net.st), "net_set_weights");
  CK(cudaMemsetAsync(n->net.d_m, 0, sizeof(float) * n->net.n_params, n->net.st), "net_set_weights");
  CK(cudaMemsetAsync(n->net.d_v, 0, sizeof(float) * n->net.n_params, n->net.st), "net_set_weights");
  n->net.adam_t = 0;
  CK(cudaStreamSynchronize(n->net.st), "net_set_weights");
  return ABX_OK;
}

static int net_sim_check(abx_net *n, abx_sim *s, const char *what) {
  if (!n || !s) return fail(ABX_ERR_INVALID_ARGUMENT, "%s: null argument", what);
  if (s->g->device != n->net.device)
    return fail(ABX_ERR_INVALID_ARGUMENT, "%s: the network lives on device %d, the simulation on device %d", what,
                n->net.device, s->g->device);
  return ABX_OK;
}

extern "C" int abx_net_add_sample(abx_net *n, abx_sim *s) {
  clear_stale_error();
  if (int rc = net_sim_check(n, s, "net_add_sample")) return rc;
  if (s->nacc <= 0) return fail(ABX_ERR_INVALID_ARGUMENT, "net_add_sample: the simulation has no time averages (run it first)");
  CK(cudaSetDevice(s->g->device), "net_add_sample");
  CK(cudaStreamSynchronize(s->st), "net_add_sample");
  cudaError_t e = n->net.add_sample(grid_desc(*s->g), (float)s->p.K, s->p.storage, s->d_acc, s->nacc, s->u0);
  if (e != cudaSuccess) return cuda_fail(e, "net_add_sample");
  return ABX_OK;
}

extern "C" int abx_net_clear_samples(abx_net *n) {
  if (!n) return fail(ABX_ERR_INVALID_ARGUMENT, "net_clear_samples: null network");
  n->net.clear_samples();
  return ABX_OK;
}

extern "C" int abx_net_get_sample(abx_net *n, int i, float *x, float *t, float *m) {
  clear_stale_error();
  if (!n) return fail(ABX_ERR_INVALID_ARGUMENT, "net_get_sample: null network");
  if (i < 0 || i >= (int)n->net.samples.size()) return fail(ABX_ERR_INVALID_ARGUMENT, "net_get_sample: no sample %d", i);
  const int64_t V = n->net.voxels();
  const float *b = n->net.samples[i].buf;
  CK(cudaSetDevice(n->net.device), "net_get_sample");
  if (x) CK(cudaMemcpyAsync(x, b, sizeof(float) * n->net.n_in * V, cudaMemcpyDeviceToHost, n->net.st), "net_get_sample");
  if (t) CK(cudaMemcpyAsync(t, b + (int64_t)n->net.n_in * V, sizeof(float) * WarmNet::kOut * V, cudaMemcpyDeviceToHost, n->net.st), "net_get_sample");
  if (m) CK(cudaMemcpyAsync(m, b + (int64_t)(n->net.n_in + WarmNet::kOut) * V, sizeof(float) * V, cudaMemcpyDeviceToHost, n->net.st), "net_get_sample");
  CK(cudaStreamSynchronize(n->net.st), "net_get_sample");
  return ABX_OK;
}

extern "C" int abx_net_train(abx_net *n, const abx_train_params *p, double *epoch_loss) {
  clear_stale_error();
  if (!n || !p) return fail(ABX_ERR_INVALID_ARGUMENT, "net_train: null argument");
  const int ns = (int)n->net.samples.size();
  if (p->first < 0 || p->count <= 0 || p->first + p->count > ns)
    return fail(ABX_ERR_INVALID_ARGUMENT, "net_train: samples [%d, %d) outside the %d stored", p->first, p->first + p->count, ns);
  if (p->epochs <= 0 || p->batch <= 0 || p->batch > 1024 || !(p->lr > 0) || !(p->lr_min >= 0))
    return fail(ABX_ERR_INVALID_ARGUMENT, "net_train: epochs > 0, 0 < batch <= 1024, lr > 0 and lr_min >= 0 required");
  cudaError_t e = n->net.train(p->first, p->count, p->epochs, p->batch, p->lr, p->lr_min, p->seed, p->flip != 0, epoch_loss);
  if (e != cudaSuccess) return cuda_fail(e, "net_train");
  return ABX_OK;
}

extern "C" int abx_net_eval_loss(abx_net *n, int first, int count, double *loss) {
  clear_stale_error();
  if (!n || !loss) return fail(ABX_ERR_INVALID_ARGUMENT, "net_eval_loss: null argument");
  const int ns = (int)n->net.samples.size();
  if (first < 0 || count <= 0 || first + count > ns)
    return fail(ABX_ERR_INVALID_ARGUMENT, "net_eval_loss: samples [%d, %d) outside the %d stored", first, first + count, ns);
  cudaError_t e = n->net.eval_loss(first, count, loss);
  if (e != cudaSuccess) return cuda_fail(e, "net_eval_loss");
  return ABX_OK;
}

extern "C" int abx_net_forward_backward(abx_net *n, const float *d_x, const float *d_t, const float *d_m, int B,
                                        double scale, float *d_pred, float *d_grad, double *loss) {
  clear_stale_error();
  if (!n || !d_x || !d_t || !d_m || !d_pred || !loss || B <= 0 || B > 1024)
    return fail(ABX_ERR_INVALID_ARGUMENT, "net_forward_backward: bad argument");
  WarmNet &w = n->net;
  CK(cudaSetDevice(w.device), "net_forward_backward");
  CK(w.ensure_batch(B), "net_forward_backward");
  const int64_t V = w.voxels();
  CK(cudaMemcpyAsync(w.input(), d_x, sizeof(float) * B * w.n_in * V, cudaMemcpyDeviceToDevice, w.st), "net_forward_backward");
  CK(w.forward(B), "net_forward_backward");
  CK(w.loss(B, d_t, d_m, scale, d_grad != nullptr, loss), "net_forward_backward");
  CK(cudaMemcpyAsync(d_pred, w.output(), sizeof(float) * B * WarmNet::kOut * V, cudaMemcpyDeviceToDevice, w.st), "net_forward_backward");
  if (d_grad) CK(cudaMemcpyAsync(d_grad, w.d_g, sizeof(float) * w.n_params, cudaMemcpyDeviceToDevice, w.st), "net_forward_backward");
  CK(cudaStreamSynchronize(w.st), "net_forward_backward");
  return ABX_OK;
}

// features of s's geometry into the network's input slot 0 and one forward pass
static int net_infer(abx_net *n, abx_sim *s) {
  WarmNet &w = n->net;
  CK(cudaSetDevice(w.device), "net: set device");
  CK(w.ensure_batch(1), "net: buffers");
  CK(w.features(grid_desc(*s->g), (float)s->p.K, w.input()), "net: features");
  CK(w.forward(1), "net: forward");
  return ABX_OK;
}

extern "C" int abx_net_predict(abx_net *n, abx_sim *s, float *features, float *pred) {
  clear_stale_error();
  if (int rc = net_sim_check(n, s, "net_predict")) return rc;
  if (int rc = net_infer(n, s)) return rc;
  WarmNet &w = n->net;
  const int64_t V = w.voxels();
  if (features) CK(cudaMemcpyAsync(features, w.input(), sizeof(float) * w.n_in * V, cudaMemcpyDeviceToHost, w.st), "net_predict");
  if (pred) CK(cudaMemcpyAsync(pred, w.output(), sizeof(float) * WarmNet::kOut * V, cudaMemcpyDeviceToHost, w.st), "net_predict");
  CK(cudaStreamSynchronize(w.st), "net_predict");
  return ABX_OK;
}

extern "C" int abx_sim_warm_start(abx_sim *s, abx_net *n) {
  clear_stale_error();
  if (int rc = net_sim_check(n, s, "sim_warm_start")) return rc;
  if (int rc = net_infer(n, s)) return rc;
  WarmNet &w = n->net;
  CK(cudaStreamSynchronize(w.st), "sim_warm_start");
  if (int rc = sim_reset(s)) return rc;
  CK(ws_apply(s->p.storage, state_args(*s), grid_desc(*s->g), w.output(), w.input(), w.R, s->u0, s->st), "sim_warm_start: apply");
  CK(cudaStreamSynchronize(s->st), "sim_warm_start");
  s->launches += 1;
  return ABX_OK;
}

extern "C" int abx_sim_converge(abx_sim *s, const abx_converge_params *p, abx_converge_result *r) {
  clear_stale_error();
  if (!s || !p || !r) return fail(ABX_ERR_INVALID_ARGUMENT, "sim_converge: null argument");
  if (p->settle < 0 || p->window <= 0 || p->min_avg < p->window || p->max_steps < p->settle + p->window || !(p->tol > 0))
    return fail(ABX_ERR_INVALID_ARGUMENT,
                "sim_converge: settle >= 0, window > 0, min_avg >= window, max_steps >= settle + window and tol > 0 required");
  if (p->rule != ABX_RULE_CHANGE && p->rule != ABX_RULE_STDERR)
    return fail(ABX_ERR_INVALID_ARGUMENT, "sim_converge: unknown stop rule %d", p->rule);
  if (p->rule == ABX_RULE_STDERR && p->min_windows < 2)
    return fail(ABX_ERR_INVALID_ARGUMENT, "sim_converge: the standard-error rule needs min_windows >= 2");
  CK(cudaSetDevice(s->g->device), "sim_converge");
  std::memset(r, 0, sizeof *r);
  r->change = INFINITY;
  const size_t acc_sz = acc_bytes(s->p.storage) * 4 * (size_t)s->g->Np;
  if (p->rule == ABX_RULE_STDERR && !s->d_acc_snap) CK(cudaMalloc(&s->d_acc_snap, acc_sz), "sim_converge: snapshot");
  if (p->settle > 0) {
    if (int rc = run_steps(s, p->settle, false)) return rc;
    r->steps = p->settle;
  }
  CK(cudaMemsetAsync(s->d_acc, 0, acc_sz, s->st), "sim_converge");
  s->nacc = 0;
  double pg = NAN, pz = NAN;
  std::vector<double> wg, wz;   // the windows' own gamma core and zeta (standard-error rule)
  while (r->steps + p->window <= p->max_steps) {
    const int snap_nacc = s->nacc;
    if (p->rule == ABX_RULE_STDERR)
      CK(cudaMemcpyAsync(s->d_acc_snap, s->d_acc, acc_sz, cudaMemcpyDeviceToDevice, s->st), "sim_converge: snapshot");
    if (int rc = run_steps(s, p->window, true)) return rc;
    abx_metrics m;
    if (int rc = sim_evaluate(s, &m, nullptr, nullptr, 0, nullptr, nullptr, 0)) return rc;
    r->steps += p->window;
    r->windows++;
    r->metrics = m;
    if (!std::isfinite(m.gammaCore) || !std::isfinite(m.zeta))
      return fail(ABX_ERR_UNSTABLE, "Rechnung instabil bei Schritt %d. Zellgröße vergrößern oder Viskosität (tau) erhöhen.", s->step);
    if (p->rule == ABX_RULE_CHANGE) {
      if (r->windows >= 2)
        r->change = std::max(std::fabs(m.gammaCore - pg) / std::fabs(m.gammaCore), std::fabs(m.zeta - pz) / std::fabs(m.zeta));
      if (s->nacc >= p->min_avg && r->change < p->tol) {
        r->converged = 1;
        break;
      }
      pg = m.gammaCore;
      pz = m.zeta;
    } else {
      abx_metrics mw;
      if (int rc = sim_evaluate(s, &mw, nullptr, nullptr, 0, nullptr, s->d_acc_snap, snap_nacc)) return rc;
      wg.push_back(mw.gammaCore);
      wz.push_back(mw.zeta);
      const size_t n = wg.size();
      if (n >= 2) {
        // batch means: standard error of the mean of the n window averages, relative to the running average
        auto rel_se = [n](const std::vector<double> &v, double ref) {
          double mean = 0;
          for (double x : v) mean += x;
          mean /= (double)n;
          double ss = 0;
          for (double x : v) ss += (x - mean) * (x - mean);
          return std::sqrt(ss / (double)(n - 1) / (double)n) / std::fabs(ref);
        };
        r->change = std::max(rel_se(wg, m.gammaCore), rel_se(wz, m.zeta));
      }
      if ((int)n >= p->min_windows && s->nacc >= p->min_avg && r->change <= 0.5 * p->tol) {
        r->converged = 1;
        break;
      }
    }
  }
  return ABX_OK;
}

extern "C" int abx_sim_solve_warm(abx_sim *s, abx_net *n, const abx_converge_params *p, abx_warm_result *r) {
  clear_stale_error();
  if (!s || !n || !p || !r) return fail(ABX_ERR_INVALID_ARGUMENT, "sim_solve_warm: null argument");
  std::memset(r, 0, sizeof *r);
  const auto t0 = std::chrono::steady_clock::now();
  if (int rc = abx_sim_warm_start(s, n)) return rc;
  r->infer_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
  int rc = abx_sim_converge(s, p, &r->run);
  r->warm_steps = r->run.steps;
  if (rc == ABX_ERR_UNSTABLE || (rc == ABX_OK && !r->run.converged)) {
    // residuals did not fall: the reference's start and schedule
    r->fell_back = 1;
    if ((rc = sim_reset(s))) return rc;
    if ((rc = abx_sim_run(s, nullptr, nullptr))) return rc;
    abx_metrics m;
    if ((rc = abx_sim_evaluate(s, &m, nullptr, nullptr, 0, nullptr))) return rc;
    r->run.metrics = m;
    r->run.steps = s->p.steps;
    r->run.windows = 1;
    r->run.converged = 0;
  } else if (rc) {
    return rc;
  }
  r->total_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
  return ABX_OK;
}

// ------------------------------------------------------------------ batched variants
struct abx_batch {
  int device = 0, n = 0;
  std::vector<abx_sim *> sims;       // owned
  int storage = 0, steps = 0, avg = 0, every = 1;
  cudaStream_t st = nullptr;
  // Variants run in groups: consecutive variants whose state fits `group_bytes` (and at most kBatchChunk
  // of them).  A chunk of steps runs group by group, each group for the whole chunk, so a group's state
  // can stay in L2 across its steps; one launch per step and group, arguments by value.
  double group_bytes = 0;                    // 0: one group of up to kBatchChunk variants after another
  std::vector<BatchParams> chunks;           // one per group
  std::vector<uint32_t> cstart[2];           // per spw: first tile of group c (and the end as last entry)
  std::vector<uint2> tiles[2];               // host copy (variant-major)
  uint2 *d_tiles[2] = {nullptr, nullptr};   // tiles of 8 (spw 1) and 16 (spw 2) segments
  uint32_t ntiles[2] = {0, 0};
  int shape = 0;
  uint32_t grid = 0;
  int step = 0, form = 0, nacc = 0;
  std::map<std::tuple<int, int, int, int, uint32_t>, cudaGraphExec_t> graphs;  // (n, form, acc, shape, grid)
  cudaEvent_t ev[2] = {nullptr, nullptr};
  double run_ms = 0;
  int64_t launches = 0;
  ~abx_batch() {
    cudaSetDevice(device);
    if (st) cudaStreamSynchronize(st);
    drop_graphs();
    for (auto e : ev) if (e) cudaEventDestroy(e);
    cudaFree(d_tiles[0]); cudaFree(d_tiles[1]);
    for (auto *s : sims) delete s;
    if (st) cudaStreamDestroy(st);
  }
  void drop_graphs() {
    for (auto &kv : graphs) cudaGraphExecDestroy(kv.second);
    graphs.clear();
  }
  static double state_bytes(const abx_sim *s) {
    return (double)s->g->Np * (store_bytes(s->p.storage) * 19 + 4 + acc_bytes(s->p.storage) * 4);
  }
  // Split the variants into groups of at most `bytes` of state (bytes <= 0: no limit)
  void regroup(double bytes) {
    group_bytes = bytes;
    chunks.clear();
    cstart[0].clear(); cstart[1].clear();
    std::vector<uint32_t> first_tile[2];
    for (int k = 0; k < 2; k++) { first_tile[k].assign(n + 1, 0); }
    for (int k = 0; k < 2; k++) {
      uint32_t v = 0;
      for (uint32_t t = 0; t <= tiles[k].size(); t++) {
        const uint32_t tv = t < tiles[k].size() ? tiles[k][t].x : (uint32_t)n;
        while (v <= tv && v <= (uint32_t)n) first_tile[k][v++] = t;
      }
    }
    double acc_bytes_ = 0;
    for (int i = 0; i < n; i++) {
      const double sb = state_bytes(sims[i]);
      const bool start = chunks.empty() || (int)(i - chunks.back().vbase) >= kBatchChunk ||
                         (bytes > 0 && acc_bytes_ + sb > bytes);
      if (start) {
        chunks.emplace_back();
        BatchParams &P = chunks.back();
        std::memset(&P, 0, sizeof P);
        P.vbase = (uint32_t)i;
        acc_bytes_ = 0;
        for (int k = 0; k < 2; k++) cstart[k].push_back(first_tile[k][i]);
      }
      chunks.back().v[i - chunks.back().vbase] = step_args(*sims[i]);
      acc_bytes_ += sb;
    }
    for (int k = 0; k < 2; k++) cstart[k].push_back((uint32_t)tiles[k].size());
    drop_graphs();
  }
  uint32_t tiles_of(int sh) const { return ntiles[batch_shape_spw(sh) - 1]; }
  const uint2 *tile_ptr(int sh) const { return d_tiles[batch_shape_spw(sh) - 1]; }
  // nsteps steps of every group, group by group, starting in form `form0`
  cudaError_t launch(int nsteps, int form0, bool acc, int sh, uint32_t grid_) const {
    const std::vector<uint32_t> &cs = cstart[batch_shape_spw(sh) - 1];
    for (size_t c = 0; c < chunks.size(); c++) {
      const uint32_t t0 = cs[c], t1 = cs[c + 1];
      if (t1 <= t0) continue;
      int form = form0;
      for (int i = 0; i < nsteps; i++, form ^= 1) {
        cudaError_t e = launch_step_batch(storage, form == 0, acc, sh, chunks[c], tile_ptr(sh), t0, t1,
                                          std::min(grid_, t1 - t0), st);
        if (e != cudaSuccess) return e;
      }
    }
    return cudaSuccess;
  }
};

extern "C" int abx_batch_create(abx_geom *const *geoms, const abx_run_params *params, int n, abx_batch **out) {
  clear_stale_error();
  if (!geoms || !params || !out || n <= 0) return fail(ABX_ERR_INVALID_ARGUMENT, "batch_create: bad argument");
  *out = nullptr;
  const abx_run_params &p0 = params[0];
  if (p0.storage != ABX_STORE_F32 && p0.storage != ABX_STORE_F16 && p0.storage != ABX_STORE_BF16)
    return fail(ABX_ERR_INVALID_ARGUMENT, "batch_create: batches run float32, float16 or bfloat16 storage");
  for (int i = 0; i < n; i++) {
    if (!geoms[i]) return fail(ABX_ERR_NOT_PREPARED, "batch_create: variant %d has no geometry", i);
    if (geoms[i]->device != geoms[0]->device) return fail(ABX_ERR_INVALID_ARGUMENT, "batch_create: variants on different devices");
    const abx_run_params &p = params[i];
    if (p.storage != p0.storage || p.steps != p0.steps || p.avg != p0.avg || p.every != p0.every)
      return fail(ABX_ERR_INVALID_ARGUMENT, "batch_create: variant %d differs in storage, steps, avg or every", i);
  }
  std::unique_ptr<abx_batch> B(new abx_batch());
  abx_batch &b = *B;
  b.device = geoms[0]->device; b.n = n;
  b.storage = p0.storage; b.steps = p0.steps; b.avg = p0.avg; b.every = p0.every;
  b.sims.reserve(n);
  for (int i = 0; i < n; i++) {
    abx_sim *s = nullptr;
    if (int rc = abx_sim_create(geoms[i], &params[i], nullptr, &s)) return rc;
    free_tma(&s->tma);  // batched steps use the tile-list kernel
    b.sims.push_back(s);
  }
  CK(cudaSetDevice(b.device), "batch_create");
  CK(cudaStreamCreateWithFlags(&b.st, cudaStreamNonBlocking), "batch_create: stream");
  CK(cudaEventCreate(&b.ev[0]), "batch_create: events");
  CK(cudaEventCreate(&b.ev[1]), "batch_create: events");
  std::vector<uint2> (&tiles)[2] = b.tiles;
  for (int i = 0; i < n; i++) {
    const uint32_t nseg = b.sims[i]->g->nseg;
    for (int k = 0; k < 2; k++)
      for (uint32_t s0 = 0; s0 < nseg; s0 += 8u * (k + 1)) tiles[k].push_back(seg2((unsigned)i, s0));
  }
  b.regroup(0);
  for (int k = 0; k < 2; k++) {
    b.ntiles[k] = (uint32_t)tiles[k].size();
    CK(cudaMalloc((void **)&b.d_tiles[k], sizeof(uint2) * std::max<size_t>(tiles[k].size(), 1)), "batch_create: tiles");
    if (!tiles[k].empty())
      CK(cudaMemcpyAsync(b.d_tiles[k], tiles[k].data(), sizeof(uint2) * tiles[k].size(), cudaMemcpyHostToDevice, b.st), "batch_create");
  }
  CK(cudaStreamSynchronize(b.st), "batch_create");
  b.shape = 0;
  b.grid = std::max<uint32_t>(b.tiles_of(0), 1);
  *out = B.release();
  return ABX_OK;
}

extern "C" void abx_batch_free(abx_batch *b) { delete b; }

extern "C" int abx_batch_sim(abx_batch *b, int i, abx_sim **out) {
  if (!b || !out || i < 0 || i >= b->n) return fail(ABX_ERR_INVALID_ARGUMENT, "batch_sim: no variant %d", i);
  *out = b->sims[i];
  return ABX_OK;
}

static int batch_sync_state(abx_batch *b) {
  for (auto *s : b->sims) { s->step = b->step; s->form = b->form; s->nacc = b->nacc; }
  return ABX_OK;
}

extern "C" int abx_batch_reset(abx_batch *b) {
  clear_stale_error();
  if (!b) return fail(ABX_ERR_INVALID_ARGUMENT, "batch_reset: null batch");
  CK(cudaSetDevice(b->device), "batch_reset");
  CK(cudaStreamSynchronize(b->st), "batch_reset");
  for (auto *s : b->sims)
    if (int rc = sim_reset(s)) return rc;
  b->step = 0; b->form = 0; b->nacc = 0;
  return ABX_OK;
}

// n batched steps from the current form, one CUDA graph per (n, form, acc, shape, grid)
static int batch_steps(abx_batch *b, int n, bool acc) {
  if (n <= 0) return ABX_OK;
  const auto key = std::make_tuple(n, b->form, acc ? 1 : 0, b->shape, b->grid);
  auto it = b->graphs.find(key);
  if (it == b->graphs.end()) {
    cudaGraph_t graph;
    CK(cudaStreamBeginCapture(b->st, cudaStreamCaptureModeThreadLocal), "batch: capture");
    const cudaError_t le = b->launch(n, b->form, acc, b->shape, b->grid);
    cudaError_t ce = cudaStreamEndCapture(b->st, &graph);
    if (le != cudaSuccess) { if (ce == cudaSuccess) cudaGraphDestroy(graph); return cuda_fail(le, "batch: step launch"); }
    CK(ce, "batch: capture");
    cudaGraphExec_t exec;
    cudaError_t ie = cudaGraphInstantiate(&exec, graph, 0);
    cudaGraphDestroy(graph);
    CK(ie, "batch: graph instantiate");
    it = b->graphs.emplace(key, exec).first;
  }
  CK(cudaGraphLaunch(it->second, b->st), "batch: graph launch");
  b->form ^= (n & 1);
  b->step += n;
  if (acc) b->nacc += n;
  b->launches += (int64_t)n * (int64_t)b->chunks.size();
  return ABX_OK;
}

extern "C" int abx_batch_set_shape(abx_batch *b, int shape, unsigned grid) {
  if (!b || shape < 0 || shape >= kBatchShapes || grid == 0)
    return fail(ABX_ERR_INVALID_ARGUMENT, "batch_set_shape: shape 0..%d and grid > 0 required", kBatchShapes - 1);
  b->shape = shape;
  b->grid = std::min<uint32_t>(grid, std::max<uint32_t>(b->tiles_of(shape), 1));
  return ABX_OK;
}

extern "C" int abx_batch_set_grouping(abx_batch *b, double group_bytes) {
  if (!b || !(group_bytes >= 0)) return fail(ABX_ERR_INVALID_ARGUMENT, "batch_set_grouping: group_bytes >= 0 required");
  CK(cudaSetDevice(b->device), "batch_set_grouping");
  CK(cudaStreamSynchronize(b->st), "batch_set_grouping");
  b->regroup(group_bytes);
  return ABX_OK;
}

extern "C" int abx_batch_tune(abx_batch *b, abx_batch_tuning *out) {
  clear_stale_error();
  if (!b || !out) return fail(ABX_ERR_INVALID_ARGUMENT, "batch_tune: null argument");
  CK(cudaSetDevice(b->device), "batch_tune");
  std::memset(out, 0, sizeof *out);
  if (int rc = abx_batch_reset(b)) return rc;
  int nsm = 0, l2 = 0;
  CK(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, b->device), "batch_tune");
  CK(cudaDeviceGetAttribute(&l2, cudaDevAttrL2CacheSize, b->device), "batch_tune");
  // candidates: group budgets (none, and fractions of the L2) x block shapes x grids; each candidate times a
  // sequence of steps per group, so that L2 reuse across a group's steps shows
  constexpr int kSteps = 8;
  const double budgets[4] = {0.0, 0.75 * l2, 0.5 * l2, 0.25 * l2};
  double best = INFINITY;
  int best_shape = 0;
  uint32_t best_grid = 1;
  double best_budget = 0;
  for (int bi = 0; bi < 4; bi++) {
    b->regroup(budgets[bi]);
    for (int sh = 0; sh < kBatchShapes; sh++) {
      const uint32_t nt = b->tiles_of(sh);
      if (nt == 0) continue;
      const uint32_t mb = (uint32_t)batch_shape_minblocks(sh);
      const uint32_t grids[3] = {(uint32_t)nsm * mb, (uint32_t)nsm * mb * 2, nt};
      for (int gi = 0; gi < 3; gi++) {
        const uint32_t grid = std::min(grids[gi], nt);
        bool dup = false;
        for (int c = 0; c < out->n_candidates; c++)
          dup |= out->cand_shape[c] == sh && out->cand_grid[c] == grid && out->cand_group_bytes[c] == budgets[bi];
        if (dup || out->n_candidates >= 48) continue;
        CK(b->launch(2, 0, false, sh, grid), "batch_tune");
        CK(cudaEventRecord(b->ev[0], b->st), "batch_tune");
        CK(b->launch(kSteps, 0, false, sh, grid), "batch_tune");
        CK(cudaEventRecord(b->ev[1], b->st), "batch_tune");
        CK(cudaEventSynchronize(b->ev[1]), "batch_tune");
        float ms = 0;
        CK(cudaEventElapsedTime(&ms, b->ev[0], b->ev[1]), "batch_tune");
        const double per = ms / kSteps;
        const int c = out->n_candidates++;
        out->cand_shape[c] = sh; out->cand_grid[c] = grid; out->cand_ms[c] = per;
        out->cand_group_bytes[c] = budgets[bi]; out->cand_groups[c] = (int)b->chunks.size();
        if (per < best) { best = per; best_shape = sh; best_grid = grid; best_budget = budgets[bi]; }
      }
    }
  }
  b->regroup(best_budget);
  b->shape = best_shape;
  b->grid = best_grid;
  out->shape = best_shape; out->spw = batch_shape_spw(best_shape); out->min_blocks = batch_shape_minblocks(best_shape);
  out->grid = best_grid; out->ntiles = b->tiles_of(best_shape); out->ms_per_step = best;
  out->group_bytes = best_budget; out->n_groups = (int)b->chunks.size();
  return abx_batch_reset(b);   // the tuning steps advanced the state: start over from f = w_i
}

extern "C" int abx_batch_run(abx_batch *b, int *status) {
  clear_stale_error();
  if (!b) return fail(ABX_ERR_INVALID_ARGUMENT, "batch_run: null batch");
  CK(cudaSetDevice(b->device), "batch_run");
  const int start_acc = b->steps - b->avg;
  b->launches = 0;
  CK(cudaEventRecord(b->ev[0], b->st), "batch_run");
  while (b->step < b->steps) {
    int stop = (b->step / b->every + 1) * b->every;
    if (stop > b->steps) stop = b->steps;
    if (b->step < start_acc && stop > start_acc) stop = start_acc;
    const bool acc = b->step >= start_acc;
    if (int rc = batch_steps(b, stop - b->step, acc)) return rc;
    if (b->step % b->every == 0 || b->step == b->steps) {
      batch_sync_state(b);
      for (auto *s : b->sims) {
        if (s->nhist >= s->hist_cap) return fail(ABX_ERR_INVALID_ARGUMENT, "batch_run: history full (reset the batch)");
        ProbeArgs pr{};
        pr.plist = s->d_plist; pr.nM = s->nM; pr.nT = s->nT; pr.step = s->step; pr.slot = s->nhist;
        pr.Ain = s->Ain; pr.u0 = s->u0; pr.hist = s->d_hist;
        pr.vy = s->d_probe_vy; pr.part = s->d_probe_part; pr.nblocks = s->probe_blocks;
        CK(launch_probe(s->p.storage, state_args(*s), pr, b->st), "batch_run: probe");
        s->nhist++;
        b->launches += 2;
      }
    }
  }
  CK(cudaEventRecord(b->ev[1], b->st), "batch_run");
  CK(cudaEventSynchronize(b->ev[1]), "batch_run");
  float ms = 0;
  CK(cudaEventElapsedTime(&ms, b->ev[0], b->ev[1]), "batch_run");
  b->run_ms = ms;
  batch_sync_state(b);
  for (int i = 0; i < b->n; i++) {
    abx_sim *s = b->sims[i];
    s->cell_updates += (int64_t)s->step * s->g->nf;
    if (status) {
      int v = 0;
      CK(cudaMemcpy(&v, s->d_status, sizeof(int), cudaMemcpyDeviceToHost), "batch_run: status");
      status[i] = v > 0 ? v : 0;
      if (v < 0) return fail(ABX_ERR_CUDA, "batch_run: variant %d: step kernel halted (%d)", i, v);
    }
  }
  return ABX_OK;
}

extern "C" int abx_batch_get_info(const abx_batch *b, abx_batch_info *o) {
  if (!b || !o) return fail(ABX_ERR_INVALID_ARGUMENT, "batch_get_info: null argument");
  std::memset(o, 0, sizeof *o);
  o->n = b->n;
  for (auto *s : b->sims) {
    o->cells += s->g->nf;
    o->state_bytes += (long long)(store_bytes(s->p.storage) * 19 + acc_bytes(s->p.storage) * 4) * s->g->Np;
  }
  o->ntiles1 = b->ntiles[0]; o->ntiles2 = b->ntiles[1];
  o->shape = b->shape; o->grid = b->grid; o->run_ms = b->run_ms; o->kernel_launches = b->launches;
  o->n_groups = (int)b->chunks.size(); o->group_bytes = b->group_bytes;
  return ABX_OK;
}

// ------------------------------------------------------------------ post-processing
// Arguments of the post-processing kernels, with the float32 averages made into `avg` (4 * Np floats).
static int post_args(abx_sim &s, DevBuf &avg, PostArgs *out, const char *what) {
  const abx_geom &g = *s.g;
  PostArgs a{};
  a.nx = g.nx; a.ny = g.ny; a.nz = g.nz; a.nzp = g.nzp; a.kpad = g.kpad; a.Np = g.Np;
  a.mask = g.d_mask; a.ns = s.has_ns ? s.d_ns : nullptr; a.opening = g.d_opening;
  a.acc = s.d_acc; a.acc_double = s.p.storage == ABX_STORE_F64; a.dn = s.nacc > 1 ? s.nacc : 1; a.u0 = s.u0;
  CK(cudaMalloc(&avg.p, sizeof(float) * 4 * (size_t)g.Np), what);
  a.avg = (const float *)avg.p;
  CK(post_average(a, (float *)avg.p, s.st), what);
  s.launches++;
  *out = a;
  return ABX_OK;
}

static int find_index_ge(const std::vector<float> &a, double v) {  // Array#findIndex(z => z >= v)
  for (size_t i = 0; i < a.size(); i++) if ((double)a[i] >= v) return (int)i;
  return -1;
}

static double js_round(double x) { const double r = std::floor(x); return (x - r >= 0.5) ? r + 1 : r; }

extern "C" int abx_sim_field3d(abx_sim *s, float *spd, float *pst, float *loss, abx_field3d_info *info) {
  clear_stale_error();
  if (!s) return fail(ABX_ERR_INVALID_ARGUMENT, "sim_field3d: null simulation");
  const abx_geom &g = *s->g;
  CK(cudaSetDevice(g.device), "sim_field3d");
  const int kB = std::max(2, find_index_ge(g.zc, g.mn[2]) - 2);
  const int jb = first_ge(g.dc, g.pleat + 2 * g.h);
  const size_t N = (size_t)g.N;
  DevBuf scal, out;
  CK(cudaMalloc(&scal.p, 2 * sizeof(double)), "sim_field3d");
  float *o[3] = {nullptr, nullptr, nullptr};
  float *host[3] = {spd, pst, loss};
  int nout = 0;
  for (int i = 0; i < 3; i++) nout += host[i] != nullptr;
  if (nout) {
    CK(cudaMalloc(&out.p, sizeof(float) * N * nout), "sim_field3d");
    int k = 0;
    for (int i = 0; i < 3; i++) if (host[i]) o[i] = (float *)out.p + N * k++;
  }
  DevBuf avg;
  PostArgs pa;
  if (int rc = post_args(*s, avg, &pa, "sim_field3d")) return rc;
  CK(post_field3d(pa, kB, jb, (double *)scal.p, o[0], o[1], o[2], s->st), "sim_field3d");
  s->launches += 2;
  double sc[2];
  CK(cudaMemcpyAsync(sc, scal.p, sizeof sc, cudaMemcpyDeviceToHost, s->st), "sim_field3d");
  for (int i = 0; i < 3; i++)
    if (host[i]) CK(cudaMemcpyAsync(host[i], o[i], sizeof(float) * N, cudaMemcpyDeviceToHost, s->st), "sim_field3d");
  CK(cudaStreamSynchronize(s->st), "sim_field3d");
  s->d2h += (int64_t)(sizeof sc + sizeof(float) * N * nout);
  if (info) {
    std::memset(info, 0, sizeof *info);
    info->nx = g.nx; info->ny = g.ny; info->nz = g.nz; info->kB = kB; info->jm = g.jm; info->top = g.top;
    info->h = g.h; info->x0 = g.xc[0]; info->d0 = g.dc[0]; info->z0 = g.zc[0]; info->zIn = g.mn[2];
    info->pleat = g.pleat; info->pin = sc[0]; info->rho_ref = sc[1];
  }
  return ABX_OK;
}

extern "C" int abx_sim_planes(abx_sim *s, float *out, abx_planes_info *info) {
  clear_stale_error();
  if (!s) return fail(ABX_ERR_INVALID_ARGUMENT, "sim_planes: null simulation");
  const abx_geom &g = *s->g;
  CK(cudaSetDevice(g.device), "sim_planes");
  double si = 0, sj = 0;
  int so = 0;
  for (int i = 0; i < g.nx; i++)
    for (int j = 0; j < g.ny; j++)
      if (g.opening[(size_t)i * g.ny + j]) { si += i; sj += j; so++; }
  const int ic = (int)js_round(si / so), jc = (int)js_round(sj / so);
  const int jlow = first_ge(g.dc, g.pleat + 12);
  const size_t n = 6 * (size_t)g.nx * g.nz + 3 * (size_t)g.nz * g.ny;
  if (out) {
    DevBuf d;
    CK(cudaMalloc(&d.p, sizeof(float) * n), "sim_planes");
    DevBuf avg;
    PostArgs pa;
    if (int rc = post_args(*s, avg, &pa, "sim_planes")) return rc;
    CK(post_planes(pa, ic, jc, jlow, (float *)d.p, s->st), "sim_planes");
    s->launches++;
    CK(cudaMemcpyAsync(out, d.p, sizeof(float) * n, cudaMemcpyDeviceToHost, s->st), "sim_planes");
    CK(cudaStreamSynchronize(s->st), "sim_planes");
    s->d2h += (int64_t)(sizeof(float) * n);
  }
  if (info) {
    std::memset(info, 0, sizeof *info);
    info->ic = ic; info->jc = jc; info->jlow = jlow; info->n1 = g.nx; info->n2 = g.nz;
    info->lon_n1 = g.nz; info->lon_n2 = g.ny;
    info->depth_inlet = g.dc[jc]; info->depth_low = g.dc[jlow]; info->x_lon = g.xc[ic];
  }
  return ABX_OK;
}

extern "C" int abx_sim_streamlines(abx_sim *s, int max_seeds, float *pts, float *spd, uint32_t *off, size_t cap_points,
                                   size_t cap_lines, abx_lines_info *info) {
  clear_stale_error();
  if (!s || max_seeds <= 0) return fail(ABX_ERR_INVALID_ARGUMENT, "sim_streamlines: bad argument");
  const abx_geom &g = *s->g;
  CK(cudaSetDevice(g.device), "sim_streamlines");
  // seeds: four per opening cell, kS cells before the box, thinned to about max_seeds (:736-739)
  const int kS = std::max(2, find_index_ge(g.zc, g.mn[2]) - 3);
  static const double D[4][2] = {{-0.25, -0.25}, {0.25, -0.25}, {-0.25, 0.25}, {0.25, 0.25}};
  std::vector<double> all;
  for (int i = 0; i < g.nx; i++)
    for (int j = 0; j < g.ny; j++)
      if (g.opening[(size_t)i * g.ny + j])
        for (int d = 0; d < 4; d++) { all.push_back(i + D[d][0]); all.push_back(j + D[d][1]); all.push_back(kS); }
  const int nall = (int)(all.size() / 3);
  const double stride = std::max(1.0, (double)nall / max_seeds);
  std::vector<double> sel;
  for (double x = 0; x < nall; x += stride) {
    const size_t k = (size_t)std::floor(x);
    sel.insert(sel.end(), all.begin() + 3 * k, all.begin() + 3 * k + 3);
  }
  const int nsel = (int)(sel.size() / 3);
  std::vector<int> cnt(std::max(nsel, 1));
  std::vector<double> P((size_t)std::max(nsel, 1) * 4 * kMaxLinePoints);
  if (nsel) {
    DevBuf dseeds, dpts, dcnt;
    CK(cudaMalloc(&dseeds.p, sizeof(double) * sel.size()), "sim_streamlines");
    CK(cudaMalloc(&dpts.p, sizeof(double) * P.size()), "sim_streamlines");
    CK(cudaMalloc(&dcnt.p, sizeof(int) * nsel), "sim_streamlines");
    CK(cudaMemcpyAsync(dseeds.p, sel.data(), sizeof(double) * sel.size(), cudaMemcpyHostToDevice, s->st), "sim_streamlines");
    DevBuf avg;
    PostArgs pa;
    if (int rc = post_args(*s, avg, &pa, "sim_streamlines")) return rc;
    CK(post_streamlines(pa, (const double *)dseeds.p, nsel, g.top, (double *)dpts.p, (int *)dcnt.p, s->st),
       "sim_streamlines");
    s->launches++;
    CK(cudaMemcpyAsync(cnt.data(), dcnt.p, sizeof(int) * nsel, cudaMemcpyDeviceToHost, s->st), "sim_streamlines");
    CK(cudaMemcpyAsync(P.data(), dpts.p, sizeof(double) * P.size(), cudaMemcpyDeviceToHost, s->st), "sim_streamlines");
    CK(cudaStreamSynchronize(s->st), "sim_streamlines");
    s->h2d += (int64_t)(sizeof(double) * sel.size());
    s->d2h += (int64_t)(sizeof(int) * nsel + sizeof(double) * P.size());
  }
  // lines of at least two points, in model coordinates (:752-756)
  size_t np = 0, nl = 0;
  bool fits = true;
  if (off && cap_lines >= 1) off[0] = 0; else fits = false;
  for (int sd = 0; sd < nsel; sd++) {
    const int m = cnt[sd];
    if (m < 2) continue;
    const double *Q = P.data() + (size_t)sd * 4 * kMaxLinePoints;
    for (int q = 0; q < m; q++) {
      if (np + q < cap_points && pts && spd) {
        double mm[3];
        g.fr.model((double)g.xc[0] + Q[4 * q] * g.h, (double)g.dc[0] + Q[4 * q + 1] * g.h,
                   (double)g.zc[0] + Q[4 * q + 2] * g.h, mm);
        pts[3 * (np + q)] = (float)mm[0]; pts[3 * (np + q) + 1] = (float)mm[1]; pts[3 * (np + q) + 2] = (float)mm[2];
        spd[np + q] = (float)Q[4 * q + 3];
      } else {
        fits = false;
      }
    }
    np += m;
    nl++;
    if (off && nl < cap_lines) off[nl] = (uint32_t)np; else fits = false;
  }
  if (info) { info->seeds_opening = nall; info->seeds_traced = nsel; info->n_lines = (int)nl; info->n_points = (int)np; }
  if (!fits)
    return fail(ABX_ERR_INVALID_ARGUMENT, "sim_streamlines: %zu points / %zu lines need larger buffers", np, nl + 1);
  return ABX_OK;
}
