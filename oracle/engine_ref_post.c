/* engine_ref_post.c - ORACLE ONLY (test infrastructure, never linked into the
 * product): plain-C restatement of the reference's post-processing of the
 * time-averaged fields, the checker of the GPU versions.
 *
 *   ora_field3d      field3d (src/engine.js:698-719): speed, static pressure and
 *                    total-pressure loss on the whole grid
 *   ora_planes       the cut planes of evaluate (:662-680): planInlet, planLow, lon
 *   ora_streamlines  streamlines (:721-758): RK2 traces from the inlet opening
 *
 * JavaScript numbers are float64; the averages are the Float32Array of
 * simulate() (acc /= nacc, :356); outputs are Float32Array.  Math.hypot is
 * restated after V8's published algorithm (scale by the largest magnitude,
 * Kahan-compensated sum of squares, sqrt times the scale); with no JavaScript
 * runtime here that choice is unpinned against V8 itself.  Parity unpinned:
 * the reference ships no fixture for these functions.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include "engine_ref.h"

double ora_js_hypot3(double x, double y, double z) {
  const double a[3] = {fabs(x), fabs(y), fabs(z)};
  /* ECMAScript Math.hypot: an infinite argument gives +Infinity even next to a NaN */
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

double ora_js_round(double x) {  /* Math.round: nearest, ties toward +infinity */
  const double r = floor(x);
  return (x - r >= 0.5) ? r + 1 : r;
}

static int find_index_ge(const float *a, int n, double v) { /* Array#findIndex(z => z >= v) */
  for (int i = 0; i < n; i++) if ((double)a[i] >= v) return i;
  return -1;
}

static int first_ge_post(const float *arr, int n, double v) {  /* firstGE, src/engine.js:13 */
  for (int i = 0; i < n; i++) if ((double)arr[i] >= v) return i;
  return n - 1;
}

static uint8_t *fluid_mask(const ora_geom *g, const ora_sim *S, const float *ns) {
  uint8_t *fl = (uint8_t *)malloc((size_t)g->N);
  for (int64_t c = 0; c < g->N; c++) {
    const int32_t a = S->cid[c];
    fl[c] = g->fluid[c] && !(ns && a >= 0 && ns[a] > 0.5f) ? 1 : 0;
  }
  return fl;
}

/* field3d (:698-719); rhoRef = pb / pbN of evaluate (:658-659), recomputed here in the same order. */
void ora_field3d(const ora_geom *g, const ora_sim *S, double u0, const float *acc, const float *ns, float *spd,
                 float *pst, float *loss, int *kB_out, double *pin_out, double *rho_ref_out) {
  const int nx = g->nx, ny = g->ny, nz = g->nz, NF = S->NF;
  const int64_t N = g->N;
  const double q = 0.5 * u0 * u0;
  uint8_t *fl = fluid_mask(g, S, ns);
  double pb = 0; int pbN = 0;
  const int jb = first_ge_post(g->dc, ny, g->pleat + 2 * g->h);
  for (int i = 0; i < nx; i++) for (int k = 0; k < nz; k++) {
    const int64_t c = ((int64_t)i * ny + jb) * nz + k;
    if (fl[c]) { pb += (double)acc[3 * (int64_t)NF + S->cid[c]]; pbN++; }
  }
  const double rhoRef = pb / pbN;
  const int fi = find_index_ge(g->zc, nz, g->mn[2]);
  const int kB = (fi - 2) > 2 ? fi - 2 : 2;
#define PTOT(a) ((double)acc[3 * (int64_t)NF + (a)] / 3 + 0.5 * ((double)acc[(a)] * (double)acc[(a)] + \
                 (double)acc[(int64_t)NF + (a)] * (double)acc[(int64_t)NF + (a)] +                  \
                 (double)acc[2 * (int64_t)NF + (a)] * (double)acc[2 * (int64_t)NF + (a)]))
  double pin = 0, win = 0;
  for (int i = 0; i < nx; i++) for (int j = 0; j < ny; j++) if (g->opening[(int64_t)i * ny + j]) {
    const int64_t c = ((int64_t)i * ny + j) * nz + kB;
    const int32_t a = S->cid[c];
    if (a < 0 || !fl[c]) continue;
    const double uz = (double)acc[2 * (int64_t)NF + a];
    const double w = uz > 0 ? uz : 0;  /* Math.max(uz, 0) */
    pin += w * PTOT(a);
    win += w;
  }
  pin /= (win > 1e-12 ? win : 1e-12);
  for (int64_t c = 0; c < N; c++) {
    spd[c] = pst[c] = loss[c] = NAN;
    const int32_t a = S->cid[c];
    if (a < 0 || !fl[c] || c % nz < kB) continue;
    const double ux = acc[a], uy = acc[(int64_t)NF + a], uz = acc[2 * (int64_t)NF + a];
    spd[c] = (float)(ora_js_hypot3(ux, uy, uz) / u0);
    pst[c] = (float)(((double)acc[3 * (int64_t)NF + a] - rhoRef) / 3 / q);
    loss[c] = (float)((pin - PTOT(a)) / q);
  }
#undef PTOT
  *kB_out = kB; *pin_out = pin; *rho_ref_out = rhoRef;
  free(fl);
}

/* The cut planes of evaluate (:662-680).  out: planInlet speed, ua, ub (nx*nz each), planLow speed, ua,
 * ub, lon speed, ua, ub (nz*ny each).  meta: ic, jc, jlow. */
void ora_planes(const ora_geom *g, const ora_sim *S, double u0, const float *acc, const float *ns, float *out,
                int meta[3]) {
  const int nx = g->nx, ny = g->ny, nz = g->nz, NF = S->NF;
  uint8_t *fl = fluid_mask(g, S, ns);
  double si = 0, sj = 0; int so = 0;
  for (int i = 0; i < nx; i++) for (int j = 0; j < ny; j++) if (g->opening[(int64_t)i * ny + j]) { si += i; sj += j; so++; }
  const int ic = (int)ora_js_round(si / so), jc = (int)ora_js_round(sj / so);
  const int jlow = first_ge_post(g->dc, ny, g->pleat + 12);
  const int64_t P = (int64_t)nx * nz, Q = (int64_t)nz * ny;
  for (int pl = 0; pl < 2; pl++) {
    const int j = pl == 0 ? jc : jlow;
    float *s = out + pl * 3 * P, *a = s + P, *b = a + P;
    for (int64_t x = 0; x < P; x++) { s[x] = NAN; a[x] = 0; b[x] = 0; }
    for (int i = 0; i < nx; i++) for (int k = 0; k < nz; k++) {
      const int64_t c = ((int64_t)i * ny + j) * nz + k;
      if (!fl[c]) continue;
      const int32_t q = S->cid[c];
      const double ux = (double)acc[q] / u0, uy = (double)acc[(int64_t)NF + q] / u0, uz = (double)acc[2 * (int64_t)NF + q] / u0;
      s[(int64_t)i * nz + k] = (float)ora_js_hypot3(ux, uy, uz);
      a[(int64_t)i * nz + k] = (float)ux;
      b[(int64_t)i * nz + k] = (float)uz;
    }
  }
  float *s = out + 6 * P, *a = s + Q, *b = a + Q;
  for (int64_t x = 0; x < Q; x++) { s[x] = NAN; a[x] = 0; b[x] = 0; }
  for (int k = 0; k < nz; k++) for (int j = 0; j < ny; j++) {
    const int64_t c = ((int64_t)ic * ny + j) * nz + k;
    if (!fl[c]) continue;
    const int32_t q = S->cid[c];
    const double ux = (double)acc[q] / u0, uy = (double)acc[(int64_t)NF + q] / u0, uz = (double)acc[2 * (int64_t)NF + q] / u0;
    s[(int64_t)k * ny + j] = (float)ora_js_hypot3(ux, uy, uz);
    a[(int64_t)k * ny + j] = (float)uz;
    b[(int64_t)k * ny + j] = (float)uy;
  }
  meta[0] = ic; meta[1] = jc; meta[2] = jlow;
  free(fl);
}

/* Trilinear velocity with wall cells weighted zero (:724-734); returns the weight of the fluid corners. */
static double vel(const ora_geom *g, const ora_sim *S, const uint8_t *fl, const float *acc, double x, double y,
                  double z, double out[3]) {
  const int nx = g->nx, ny = g->ny, nz = g->nz, NF = S->NF;
  const double fi0 = floor(x), fj0 = floor(y), fk0 = floor(z);
  const int i0 = (int)fi0, j0 = (int)fj0, k0 = (int)fk0;
  const double fx = x - fi0, fy = y - fj0, fz = z - fk0;
  out[0] = out[1] = out[2] = 0;
  double wsum = 0;
  for (int a = 0; a < 2; a++) for (int b = 0; b < 2; b++) for (int c = 0; c < 2; c++) {
    const int i = i0 + a, j = j0 + b, k = k0 + c;
    if (i < 0 || j < 0 || k < 0 || i >= nx || j >= ny || k >= nz) continue;
    const double w = (a ? fx : 1 - fx) * (b ? fy : 1 - fy) * (c ? fz : 1 - fz);
    const int64_t cc = ((int64_t)i * ny + j) * nz + k;
    const int32_t q = S->cid[cc];
    if (q < 0 || !fl[cc]) continue;
    out[0] += w * (double)acc[q]; out[1] += w * (double)acc[(int64_t)NF + q]; out[2] += w * (double)acc[2 * (int64_t)NF + q];
    wsum += w;
  }
  return wsum;
}

static int inside(const ora_geom *g, const uint8_t *fl, double x, double y, double z) {
  const double ri = ora_js_round(x), rj = ora_js_round(y), rk = ora_js_round(z);
  if (ri < 0 || rj < 0 || rk < 0 || ri >= g->nx || rj >= g->ny || rk >= g->nz) return 0;
  return fl[((int64_t)ri * g->ny + (int64_t)rj) * g->nz + (int64_t)rk] != 0;
}

/* streamlines (:721-758).  pts: 3 floats per point in model coordinates, spd: |u|/u0 per point, off:
 * nlines+1 prefix counts.  Returns 0, or -1 when a capacity is too small (counts still reported). */
int ora_streamlines(const ora_geom *g, const ora_sim *S, double u0, const float *acc, const float *ns, int max_seeds,
                    float *pts, float *spd, uint32_t *off, int cap_pts, int cap_lines, int *nlines_out,
                    int *npts_out) {
  const int nx = g->nx, ny = g->ny, nz = g->nz;
  uint8_t *fl = fluid_mask(g, S, ns);
  const int fi = find_index_ge(g->zc, nz, g->mn[2]);
  const int kS = (fi - 3) > 2 ? fi - 3 : 2;
  static const double D[4][2] = {{-0.25, -0.25}, {0.25, -0.25}, {-0.25, 0.25}, {0.25, 0.25}};
  int nseed = 0;
  for (int i = 0; i < nx; i++) for (int j = 0; j < ny; j++) if (g->opening[(int64_t)i * ny + j]) nseed += 4;
  double (*seeds)[3] = (double (*)[3])malloc(sizeof(double) * 3 * (size_t)(nseed > 0 ? nseed : 1));
  int n = 0;
  for (int i = 0; i < nx; i++) for (int j = 0; j < ny; j++) if (g->opening[(int64_t)i * ny + j])
    for (int d = 0; d < 4; d++) { seeds[n][0] = i + D[d][0]; seeds[n][1] = j + D[d][1]; seeds[n][2] = kS; n++; }
  const double stride = (double)nseed / max_seeds > 1 ? (double)nseed / max_seeds : 1;
  const double ds = 0.35;
  double *P = (double *)malloc(sizeof(double) * 3 * 2100);
  double *V = (double *)malloc(sizeof(double) * 2100);
  int nl = 0, np = 0, ok = 1;
  if (off && cap_lines >= 1) off[0] = 0;
  for (double s = 0; s < nseed; s += stride) {
    const double *sd = seeds[(int)floor(s)];
    double x = sd[0], y = sd[1], z = sd[2], v1[3], v2[3];
    int m = 0;
    for (int st = 0; st < 6000; st++) {
      if (!inside(g, fl, x, y, z) || vel(g, S, fl, acc, x, y, z, v1) < 0.3) break;
      const double m1 = ora_js_hypot3(v1[0], v1[1], v1[2]);
      if (m1 < 0.01 * u0) break;
      if (st % 3 == 0) { P[3 * m] = x; P[3 * m + 1] = y; P[3 * m + 2] = z; V[m] = m1 / u0; m++; }
      const double xm = x + 0.5 * ds * v1[0] / m1, ym = y + 0.5 * ds * v1[1] / m1, zm = z + 0.5 * ds * v1[2] / m1;
      if (vel(g, S, fl, acc, xm, ym, zm, v2) < 0.3) break;
      const double m2 = ora_js_hypot3(v2[0], v2[1], v2[2]);
      if (m2 < 0.01 * u0) break;
      x += ds * v2[0] / m2; y += ds * v2[1] / m2; z += ds * v2[2] / m2;
      if (y < g->top + 0.5) { P[3 * m] = x; P[3 * m + 1] = y; P[3 * m + 2] = z; V[m] = m2 / u0; m++; break; }
    }
    if (m < 2) continue;
    for (int q = 0; q < m; q++) {
      double mm[3];
      ora_to_model(&g->fr, (double)g->xc[0] + P[3 * q] * g->h, (double)g->dc[0] + P[3 * q + 1] * g->h,
                   (double)g->zc[0] + P[3 * q + 2] * g->h, mm);
      if (np + q < cap_pts && pts && spd) {
        pts[3 * (np + q)] = (float)mm[0]; pts[3 * (np + q) + 1] = (float)mm[1]; pts[3 * (np + q) + 2] = (float)mm[2];
        spd[np + q] = (float)V[q];
      } else ok = 0;
    }
    np += m;
    nl++;
    if (off && nl < cap_lines) off[nl] = (uint32_t)np; else ok = 0;
  }
  *nlines_out = nl; *npts_out = np;
  free(P); free(V); free(seeds); free(fl);
  return ok ? 0 : -1;
}
