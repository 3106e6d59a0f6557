// postproc.cu - post-processing of the time-averaged fields on the device
// (compiled with -fmad=false: float64 arithmetic in the reference's order).
//
//   field3d      src/engine.js:698-719: |u|/u0, static pressure and total-pressure
//                loss on the whole grid (NaN where there is no air)
//   planes       src/engine.js:662-680: the cut planes planInlet, planLow, lon
//   streamlines  src/engine.js:721-758: RK2 traces of the averaged velocity from
//                the inlet opening, one warp per seed
//
// The averages are read as the reference holds them: the Float32Array of
// simulate() (sum / nacc rounded to float32, :356), made once per call.  Sums the reference takes
// in one loop (the inlet's mass-weighted total pressure, the reference
// density under the filter) run in one thread, in its order.  Math.hypot
// follows V8's published algorithm (scale by the largest magnitude,
// Kahan-compensated sum of squares).
#include <math.h>
#include <stdint.h>

#include "lbm_iface.h"

namespace abx {

// The averages as the reference holds them, sum / nacc rounded to float32 (a Float32Array, :356),
// computed once per call into a float array that the kernels below read.
template <typename Acc>
__global__ void average_kernel(const Acc *__restrict__ acc, int64_t n, double dn, float *__restrict__ out) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    out[i] = (float)((double)acc[i] / dn);
}

struct AvgView {
  const float *avg;
  int64_t Np;
  __device__ __forceinline__ double operator()(int comp, int64_t p) const { return (double)avg[comp * Np + p]; }
};

__device__ __forceinline__ double js_hypot3(double x, double y, double z) {
  const double a[3] = {fabs(x), fabs(y), fabs(z)};
  // ECMAScript Math.hypot: an infinite argument gives +Infinity even next to a NaN
  for (int i = 0; i < 3; i++) if (isinf(a[i])) return INFINITY;
  double mx = 0;
  for (int i = 0; i < 3; i++) {
    if (isnan(a[i])) return NAN;
    if (a[i] > mx) mx = a[i];
  }
  if (mx == 0) return 0;
  double sum = 0, comp = 0;
  for (int i = 0; i < 3; i++) {
    const double n = a[i] / mx;
    const double summand = n * n - comp;
    const double pre = sum + summand;
    comp = (pre - sum) - summand;
    sum = pre;
  }
  return sqrt(sum) * mx;
}

__device__ __forceinline__ double js_round(double x) {
  const double r = floor(x);
  return (x - r >= 0.5) ? r + 1 : r;
}

__device__ __forceinline__ bool air(const PostArgs &a, int64_t p) {
  return a.mask[p] != 0u && !(a.ns && a.ns[p] > 0.5f);
}
__device__ __forceinline__ int64_t padded(const PostArgs &a, int i, int j, int k) {
  return ((int64_t)i * a.ny + j) * a.nzp + k + a.kpad;
}

// out[0] = pin (mass-flow-weighted total pressure at k = kB over the opening, :705-711),
// out[1] = rhoRef (mean density on layer jb, :658-659)
__global__ void post_scalars_kernel(const PostArgs a, int kB, int jb, double *out) {
  const AvgView U{a.avg, a.Np};
  // loads issued unconditionally (every index is inside the arrays) so that the loop pipelines; the sums
  // still take the cells in the reference's order
  double pb = 0;
  int pbN = 0;
  for (int i = 0; i < a.nx; i++)
#pragma unroll 8
    for (int k = 0; k < a.nz; k++) {
      const int64_t p = padded(a, i, jb, k);
      const bool f = air(a, p);
      const double v = U(3, p);
      if (f) { pb += v; pbN++; }
    }
  double pin = 0, win = 0;
  for (int i = 0; i < a.nx; i++)
#pragma unroll 4
    for (int j = 0; j < a.ny; j++) {
      const int64_t p = padded(a, i, j, kB);
      const bool use = a.opening[(int64_t)i * a.ny + j] && air(a, p);
      const double ux = U(0, p), uy = U(1, p), uz = U(2, p), r = U(3, p);
      if (!use) continue;
      const double w = uz > 0 ? uz : 0;
      pin += w * (r / 3 + 0.5 * (ux * ux + uy * uy + uz * uz));
      win += w;
    }
  out[0] = pin / (win > 1e-12 ? win : 1e-12);
  out[1] = pb / pbN;
}

__global__ void field3d_kernel(const PostArgs a, int kB, const double *scal, float *spd, float *pst, float *loss) {
  const AvgView U{a.avg, a.Np};
  const int64_t N = (int64_t)a.nx * a.ny * a.nz;
  const double q = 0.5 * a.u0 * a.u0, pin = scal[0], rhoRef = scal[1];
  for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < N; c += (int64_t)gridDim.x * blockDim.x) {
    const int k = (int)(c % a.nz);
    const int64_t ij = c / a.nz;
    const int64_t p = ij * a.nzp + k + a.kpad;
    float s = NAN, ps = NAN, l = NAN;
    if (air(a, p) && k >= kB) {
      const double ux = U(0, p), uy = U(1, p), uz = U(2, p), rho = U(3, p);
      s = (float)(js_hypot3(ux, uy, uz) / a.u0);
      ps = (float)((rho - rhoRef) / 3 / q);
      l = (float)((pin - (rho / 3 + 0.5 * (ux * ux + uy * uy + uz * uz))) / q);
    }
    if (spd) spd[c] = s;
    if (pst) pst[c] = ps;
    if (loss) loss[c] = l;
  }
}

// planInlet (j = jc), planLow (j = jlow): speed, ua = ux/u0, ub = uz/u0 over (i, k);
// lon (i = ic): speed, ua = uz/u0, ub = uy/u0 over (k, j).
__global__ void planes_kernel(const PostArgs a, int ic, int jc, int jlow, float *out) {
  const AvgView U{a.avg, a.Np};
  const int64_t P = (int64_t)a.nx * a.nz, Q = (int64_t)a.nz * a.ny, n = 2 * P + Q;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n; t += (int64_t)gridDim.x * blockDim.x) {
    float *s, *ua, *ub;
    int64_t p;
    bool lon = t >= 2 * P;
    if (!lon) {
      const int pl = (int)(t / P);
      const int64_t x = t % P;
      s = out + pl * 3 * P + x; ua = s + P; ub = ua + P;
      p = padded(a, (int)(x / a.nz), pl == 0 ? jc : jlow, (int)(x % a.nz));
    } else {
      const int64_t x = t - 2 * P;
      s = out + 6 * P + x; ua = s + Q; ub = ua + Q;
      p = padded(a, ic, (int)(x % a.ny), (int)(x / a.ny));
    }
    if (!air(a, p)) { *s = NAN; *ua = 0.0f; *ub = 0.0f; continue; }
    const double ux = U(0, p) / a.u0, uy = U(1, p) / a.u0, uz = U(2, p) / a.u0;
    *s = (float)js_hypot3(ux, uy, uz);
    *ua = (float)(lon ? uz : ux);
    *ub = (float)(lon ? uy : uz);
  }
}

// The streamline trace on the GB300's float64 units: their throughput is a small fraction of float32's, and
// one thread per seed makes each RK2 step a long chain of dependent float64 instructions.  Here one warp traces
// one seed and the independent parts of each step run on separate lanes: the eight trilinear corners (lanes
// 0..7), the four running sums over the corners (lanes 0..3: x, y, z velocity and the weights, each added in
// the reference's corner order), and the per-axis divisions (lanes 0..2).  Every lane holds the same position,
// so the trace's branches are warp-uniform; every value is the reference's float64 operation sequence.
struct TraceWarp {
  double (*cor)[4];   // [8][4] this warp's corner products (w u_x, w u_y, w u_z, w), shared memory
  double *bc;         // [4] broadcast slots, shared memory
  int lane;
};

// Sum of w * u over the air corners of (x, y, z) (the trilinear loop of :741-747) into v[0..2], the weight sum
// returned.
__device__ double trace_vel_warp(const PostArgs &a, const AvgView &U, const TraceWarp &t, double x, double y, double z,
                                 double v[3]) {
  const double fi0 = floor(x), fj0 = floor(y), fk0 = floor(z);
  const double fx = x - fi0, fy = y - fj0, fz = z - fk0;
  const int i0 = (int)fi0, j0 = (int)fj0, k0 = (int)fk0;
  bool valid = false;
  if (t.lane < 8) {
    // corner lane = da * 4 + db * 2 + dc: the reference loop's nesting order
    const int da = (t.lane >> 2) & 1, db = (t.lane >> 1) & 1, dc = t.lane & 1;
    const int i = i0 + da, j = j0 + db, k = k0 + dc;
    if (!(i < 0 || j < 0 || k < 0 || i >= a.nx || j >= a.ny || k >= a.nz)) {
      const int64_t p = padded(a, i, j, k);
      if (air(a, p)) {
        const double w = (da ? fx : 1 - fx) * (db ? fy : 1 - fy) * (dc ? fz : 1 - fz);
        t.cor[t.lane][0] = w * U(0, p);
        t.cor[t.lane][1] = w * U(1, p);
        t.cor[t.lane][2] = w * U(2, p);
        t.cor[t.lane][3] = w;
        valid = true;
      }
    }
  }
  const unsigned vm = __ballot_sync(0xffffffffu, valid);
  __syncwarp();
  if (t.lane < 4) {
    double s = 0;
    for (int l = 0; l < 8; l++)
      if ((vm >> l) & 1u) s += t.cor[l][t.lane];
    t.bc[t.lane] = s;
  }
  __syncwarp();
  v[0] = t.bc[0]; v[1] = t.bc[1]; v[2] = t.bc[2];
  const double wsum = t.bc[3];
  __syncwarp();   // the slots are rewritten by the next call
  return wsum;
}

// Math.hypot (V8: scale by the largest magnitude, Kahan-compensated sum of squares), the three scalings on
// lanes 0..2
__device__ double js_hypot3_warp(const TraceWarp &t, double x, double y, double z) {
  const double a[3] = {fabs(x), fabs(y), fabs(z)};
  for (int i = 0; i < 3; i++) if (isinf(a[i])) return INFINITY;
  double mx = 0;
  for (int i = 0; i < 3; i++) {
    if (isnan(a[i])) return NAN;
    if (a[i] > mx) mx = a[i];
  }
  if (mx == 0) return 0;
  if (t.lane < 3) t.bc[t.lane] = (t.lane == 0 ? a[0] : t.lane == 1 ? a[1] : a[2]) / mx;
  __syncwarp();
  const double n3[3] = {t.bc[0], t.bc[1], t.bc[2]};
  __syncwarp();
  double sum = 0, comp = 0;
  for (int i = 0; i < 3; i++) {
    const double summand = n3[i] * n3[i] - comp;
    const double pre = sum + summand;
    comp = (pre - sum) - summand;
    sum = pre;
  }
  return sqrt(sum) * mx;
}

// base[c] + (f * v[c]) / m for c = 0, 1, 2 (lane c), left to right as the reference writes it
__device__ void trace_step_warp(const TraceWarp &t, const double base[3], double f, const double v[3], double m,
                                double out[3]) {
  if (t.lane < 3) {
    const double b = t.lane == 0 ? base[0] : t.lane == 1 ? base[1] : base[2];
    const double c = t.lane == 0 ? v[0] : t.lane == 1 ? v[1] : v[2];
    t.bc[t.lane] = b + f * c / m;
  }
  __syncwarp();
  out[0] = t.bc[0]; out[1] = t.bc[1]; out[2] = t.bc[2];
  __syncwarp();
}

__device__ __forceinline__ bool trace_inside(const PostArgs &a, double x, double y, double z) {
  const double ri = js_round(x), rj = js_round(y), rk = js_round(z);
  if (ri < 0 || rj < 0 || rk < 0 || ri >= a.nx || rj >= a.ny || rk >= a.nz) return false;
  return air(a, padded(a, (int)ri, (int)rj, (int)rk));
}

constexpr int kTraceWarps = 4;   // seeds per block

// One warp per seed: the trace of :739-751, up to kMaxLinePoints points (x, y, z, |u|/u0) in grid-cell
// coordinates into the seed's slot; count[s] = points kept.
__global__ void __launch_bounds__(32 * kTraceWarps) streamline_kernel(const PostArgs a, const double *seeds, int nseeds,
                                                                      int top, double *pts, int *count) {
  __shared__ double cor[kTraceWarps][8][4];
  __shared__ double bc[kTraceWarps][4];
  const int wib = threadIdx.x >> 5;
  const int s = blockIdx.x * kTraceWarps + wib;
  if (s >= nseeds) return;   // whole warps leave together
  const TraceWarp t{cor[wib], bc[wib], (int)(threadIdx.x & 31)};
  const AvgView U{a.avg, a.Np};
  double pos[3] = {seeds[3 * s], seeds[3 * s + 1], seeds[3 * s + 2]}, mid[3], v1[3], v2[3];
  double *P = pts + (int64_t)s * 4 * kMaxLinePoints;
  const double ds = 0.35;
  int m = 0;
  for (int st = 0; st < 6000; st++) {
    if (!trace_inside(a, pos[0], pos[1], pos[2]) || trace_vel_warp(a, U, t, pos[0], pos[1], pos[2], v1) < 0.3) break;
    const double m1 = js_hypot3_warp(t, v1[0], v1[1], v1[2]);
    if (m1 < 0.01 * a.u0) break;
    if (st % 3 == 0) {
      if (t.lane == 0) { P[4 * m] = pos[0]; P[4 * m + 1] = pos[1]; P[4 * m + 2] = pos[2]; P[4 * m + 3] = m1 / a.u0; }
      m++;
    }
    trace_step_warp(t, pos, 0.5 * ds, v1, m1, mid);
    if (trace_vel_warp(a, U, t, mid[0], mid[1], mid[2], v2) < 0.3) break;
    const double m2 = js_hypot3_warp(t, v2[0], v2[1], v2[2]);
    if (m2 < 0.01 * a.u0) break;
    trace_step_warp(t, pos, ds, v2, m2, pos);
    if (pos[1] < top + 0.5) {
      if (t.lane == 0) { P[4 * m] = pos[0]; P[4 * m + 1] = pos[1]; P[4 * m + 2] = pos[2]; P[4 * m + 3] = m2 / a.u0; }
      m++;
      break;
    }
  }
  if (t.lane == 0) count[s] = m;
}

static unsigned grid_of(int64_t n) {
  int64_t b = (n + 255) / 256;
  if (b > 152 * 8) b = 152 * 8;
  return (unsigned)(b < 1 ? 1 : b);
}

cudaError_t post_average(const PostArgs &a, float *avg, cudaStream_t st) {
  const int64_t n = 4 * a.Np;
  if (a.acc_double) average_kernel<double><<<grid_of(n), 256, 0, st>>>((const double *)a.acc, n, a.dn, avg);
  else average_kernel<float><<<grid_of(n), 256, 0, st>>>((const float *)a.acc, n, a.dn, avg);
  return cudaGetLastError();
}

cudaError_t post_field3d(const PostArgs &a, int kB, int jb, double *d_scal, float *spd, float *pst, float *loss,
                         cudaStream_t st) {
  const int64_t N = (int64_t)a.nx * a.ny * a.nz;
  post_scalars_kernel<<<1, 1, 0, st>>>(a, kB, jb, d_scal);
  field3d_kernel<<<grid_of(N), 256, 0, st>>>(a, kB, d_scal, spd, pst, loss);
  return cudaGetLastError();
}

cudaError_t post_planes(const PostArgs &a, int ic, int jc, int jlow, float *out, cudaStream_t st) {
  const int64_t n = 2 * (int64_t)a.nx * a.nz + (int64_t)a.nz * a.ny;
  planes_kernel<<<grid_of(n), 256, 0, st>>>(a, ic, jc, jlow, out);
  return cudaGetLastError();
}

cudaError_t post_streamlines(const PostArgs &a, const double *seeds, int nseeds, int top, double *pts, int *count,
                             cudaStream_t st) {
  if (nseeds <= 0) return cudaSuccess;
  const unsigned blocks = (unsigned)((nseeds + kTraceWarps - 1) / kTraceWarps);
  streamline_kernel<<<blocks, 32 * kTraceWarps, 0, st>>>(a, seeds, nseeds, top, pts, count);
  return cudaGetLastError();
}

}  // namespace abx
