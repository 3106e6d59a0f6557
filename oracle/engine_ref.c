/* engine_ref.c - ORACLE ONLY: test infrastructure, never linked into the product.
 *
 * A plain-C restatement of the reference compute core, src/engine.js (Awsmqt/AirboxCalc):
 *   constants          src/engine.js:4-13
 *   parseSTL           src/engine.js:15-28
 *   makeFrame          src/engine.js:31-43
 *   voxelize           src/engine.js:45-93
 *   components2d       src/engine.js:95-108
 *   prepare            src/engine.js:111-234
 *   setupSim           src/engine.js:239-264
 *   cpuStep            src/engine.js:266-321   (engine_ref_step.inc)
 *   probeCPU/progress  src/engine.js:324-339
 *   simulate           src/engine.js:341-358
 *   evaluate (metrics) src/engine.js:632-660,681-685
 *
 * Arithmetic contract: JS numbers are IEEE doubles, so every local is a double,
 * and values are rounded to float32 exactly where the JS stores into a
 * Float32Array (local triangles :113-117, voxel hits :78/:72, xc/dc/zc :136-139,
 * f/f2/acc :343-344, probe output :325, acc averaging :356).  The file is
 * compiled with -O2 -ffp-contract=off and without fast-math, so the operation
 * order written here is the one executed.  Only tests/, __graft_entry__.smoke()
 * and bench.py's CPU-baseline leg load this code.
 *
 * Parity status: the reference ships no tests, fixtures or golden vectors, and
 * engine.js cannot run here (no JavaScript runtime).  STL parsing, the frame
 * transform, the parity voxelizer and the 27->1 downsample are pinned against
 * the reference's own Python CLI (airbox_cfd.py load_stl/to_local/voxelize),
 * imported and run to make tests/golden/, and so are the solid and fluid masks
 * after downsample, duct, closing and flood, and the KPI formulas of evaluate
 * (against the CLI's report() on its own averaged fields).  The LBM step and
 * the probe are NOT pinned by any reference output ("parity unpinned" for those
 * rows: the CLI's solver uses other boundary numerics); they are checked by
 * known-answer properties (rest state, mass conservation, mirror symmetry) and
 * by the reference's own GPU-vs-CPU self-test criterion (src/engine.js:597-611,
 * threshold :772).
 */
#include "engine_ref.h"

#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

static const int CX[19] = {0, 1, -1, 0, 0, 0, 0, 1, -1, 1, -1, 1, -1, 1, -1, 0, 0, 0, 0};
static const int CY[19] = {0, 0, 0, 1, -1, 0, 0, 1, -1, -1, 1, 0, 0, 0, 0, 1, -1, 1, -1};
static const int CZ[19] = {0, 0, 0, 0, 0, 1, -1, 0, 0, 0, 0, 1, -1, -1, 1, 1, -1, -1, 1};
static const int OPP[19] = {0, 2, 1, 4, 3, 6, 5, 8, 7, 10, 9, 12, 11, 14, 13, 16, 15, 18, 17};
static const double WT[19] = {1.0 / 3, 1.0 / 18, 1.0 / 18, 1.0 / 18, 1.0 / 18, 1.0 / 18, 1.0 / 18,
                              1.0 / 36, 1.0 / 36, 1.0 / 36, 1.0 / 36, 1.0 / 36, 1.0 / 36,
                              1.0 / 36, 1.0 / 36, 1.0 / 36, 1.0 / 36, 1.0 / 36, 1.0 / 36};

/* Math.min / Math.max: NaN in, NaN out. */
static double js_min(double a, double b) { if (isnan(a) || isnan(b)) return NAN; return a < b ? a : b; }
static double js_max(double a, double b) { if (isnan(a) || isnan(b)) return NAN; return a > b ? a : b; }
static float js_minf(float a, float b) { if (isnan(a) || isnan(b)) return NAN; return a < b ? a : b; }

/* firstGE (src/engine.js:13) over a Float32Array. */
static int first_ge(const float *arr, int n, double v) {
  for (int i = 0; i < n; i++) if ((double)arr[i] >= v) return i;
  return n - 1;
}

/* ------------------------------------------------------------------ parseSTL (:15-28) */
static int is_num_char(unsigned char c) {
  return (c >= '0' && c <= '9') || c == '-' || c == '+' || c == '.' || c == 'e' || c == 'E';
}
static int is_ws(unsigned char c) { return c == ' ' || c == '\t' || c == '\n' || c == '\r' || c == '\v' || c == '\f'; }

/* JS Number() of a token made only of [-+0-9.eE]: a complete decimal literal, else NaN. */
static double js_number(const char *s, size_t n) {
  char tmp[128];
  if (n == 0 || n >= sizeof tmp) return NAN;
  memcpy(tmp, s, n); tmp[n] = 0;
  /* strtod also takes hex and inf/nan, which the character class cannot spell. */
  char *end = NULL;
  double v = strtod(tmp, &end);
  if (end != tmp + n) return NAN;
  /* JS rejects a sign followed by nothing numeric, which strtod already fails on. */
  return v;
}

int ora_parse_stl(const uint8_t *buf, size_t len, float *out, size_t cap, size_t *nfloats, char *msg) {
  uint32_t n = 0;
  if (len >= 84) memcpy(&n, buf + 80, 4);
  if (n > 0 && 84ull + 50ull * n == (unsigned long long)len) {
    *nfloats = (size_t)n * 9;
    if (out) {
      if (cap < *nfloats) return ORA_NOMEM;
      for (uint32_t i = 0; i < n; i++)
        for (int k = 0; k < 9; k++) memcpy(&out[(size_t)i * 9 + k], buf + 84 + (size_t)i * 50 + 12 + k * 4, 4);
    }
    return ORA_OK;
  }
  /* ASCII: the regex vertex\s+(num)\s+(num)\s+(num), global, left to right. */
  size_t count = 0, p = 0;
  while (p + 6 <= len) {
    if (memcmp(buf + p, "vertex", 6) != 0) { p++; continue; }
    size_t q = p + 6;
    double v[3]; int ok = 1;
    for (int c = 0; c < 3 && ok; c++) {
      size_t ws = q;
      while (q < len && is_ws(buf[q])) q++;
      if (q == ws) { ok = 0; break; }
      size_t t0 = q;
      while (q < len && is_num_char(buf[q])) q++;
      if (q == t0) { ok = 0; break; }
      v[c] = js_number((const char *)buf + t0, q - t0);
    }
    if (!ok) { p++; continue; }
    if (out) {
      if (cap < count + 3) return ORA_NOMEM;
      out[count] = (float)v[0]; out[count + 1] = (float)v[1]; out[count + 2] = (float)v[2];
    }
    count += 3;
    p = q;
  }
  if (count < 9) {
    if (msg) snprintf(msg, 512, "STL enthält keine Dreiecke.");
    return ORA_NO_TRIANGLES;
  }
  *nfloats = count;
  return ORA_OK;
}

/* ------------------------------------------------------------------ makeFrame (:31-43) */
void ora_make_frame(const ora_prep_params *p, ora_frame *fr) {
  fr->dAx = p->sealAxis; fr->iAx = p->inletAxis; fr->oAx = 3 - p->sealAxis - p->inletAxis;
  fr->sd = p->sealSign; fr->si = p->inletSign; fr->seal = p->seal;
  fr->yaw_deg = p->inletYaw;
  const double yaw = p->inletYaw * M_PI / 180;
  fr->cy = cos(yaw); fr->sy = sin(yaw);
}

void ora_to_local(const ora_frame *fr, const double q[3], double out[3]) {
  const double a = q[fr->oAx], b = -fr->si * q[fr->iAx];
  out[0] = fr->cy * a + fr->sy * b;
  out[1] = -fr->sd * (q[fr->dAx] - fr->seal);
  out[2] = -fr->sy * a + fr->cy * b;
}

void ora_to_model(const ora_frame *fr, double X, double D, double Z, double out[3]) {
  out[fr->oAx] = fr->cy * X - fr->sy * Z;
  out[fr->dAx] = fr->seal - fr->sd * D;
  out[fr->iAx] = -fr->si * (fr->sy * X + fr->cy * Z);
}

/* ------------------------------------------------------------------ voxelize (:45-93) */
static int cmp_float(const void *a, const void *b) {
  const double x = *(const float *)a, y = *(const float *)b;
  return x < y ? -1 : x > y ? 1 : 0;
}

void ora_voxelize(const float *T, size_t nfloats, const double origin[3], int nx, int ny, int nz,
                  double h, uint8_t *vox) {
  const int64_t ncol = (int64_t)nx * ny;
  const int64_t ntri = (int64_t)(nfloats / 9);
  const double jx = 1.37e-4, jy = 2.71e-4;
  int32_t *cnt = (int32_t *)calloc((size_t)ncol + 1, sizeof(int32_t));
  float *hits = NULL; int32_t *pos = NULL;
  for (int pass = 0; pass < 2; pass++) {
    for (int64_t t = 0; t < ntri; t++) {
      const int64_t o = t * 9;
      const double ax = (double)T[o] - origin[0] - jx, ay = (double)T[o + 1] - origin[1] - jy, az = (double)T[o + 2] - origin[2];
      const double bx = (double)T[o + 3] - origin[0] - jx, by = (double)T[o + 4] - origin[1] - jy, bz = (double)T[o + 5] - origin[2];
      const double cx = (double)T[o + 6] - origin[0] - jx, cy = (double)T[o + 7] - origin[1] - jy, cz = (double)T[o + 8] - origin[2];
      const double den = (by - cy) * (ax - cx) + (cx - bx) * (ay - cy);
      if (fabs(den) < 1e-12) continue;
      const double i0 = js_max(0, floor(js_min(js_min(ax, bx), cx) / h - 0.5));
      const double i1 = js_min(nx - 1, ceil(js_max(js_max(ax, bx), cx) / h - 0.5));
      const double j0 = js_max(0, floor(js_min(js_min(ay, by), cy) / h - 0.5));
      const double j1 = js_min(ny - 1, ceil(js_max(js_max(ay, by), cy) / h - 0.5));
      for (double i = i0; i <= i1; i++) {
        const double px = (i + 0.5) * h;
        for (double j = j0; j <= j1; j++) {
          const double py = (j + 0.5) * h;
          const double l1 = ((by - cy) * (px - cx) + (cx - bx) * (py - cy)) / den;
          if (l1 < 0) continue;
          const double l2 = ((cy - ay) * (px - cx) + (ax - cx) * (py - cy)) / den;
          if (l2 < 0) continue;
          const double l3 = 1 - l1 - l2;
          if (l3 < 0) continue;
          const int64_t col = (int64_t)i * ny + (int64_t)j;
          if (pass == 0) cnt[col + 1]++;
          else hits[pos[col]++] = (float)(l1 * az + l2 * bz + l3 * cz);
        }
      }
    }
    if (pass == 0) {
      for (int64_t c = 0; c < ncol; c++) cnt[c + 1] += cnt[c];
      hits = (float *)malloc(sizeof(float) * (size_t)(cnt[ncol] > 0 ? cnt[ncol] : 1));
      pos = (int32_t *)malloc(sizeof(int32_t) * (size_t)(ncol > 0 ? ncol : 1));
      memcpy(pos, cnt, sizeof(int32_t) * (size_t)ncol);
    }
  }
  memset(vox, 0, (size_t)((int64_t)nx * ny * nz));
  for (int64_t c = 0; c < ncol; c++) {
    const int32_t a = cnt[c], b = cnt[c + 1];
    if (b - a < 2) continue;
    float *zs = hits + a;
    qsort(zs, (size_t)(b - a), sizeof(float), cmp_float);
    const int len = b - a, m = len - (len % 2);
    const int64_t base = c * nz;
    for (int k = 0; k < m; k += 2) {
      const double k0 = js_max(0, ceil((double)zs[k] / h - 0.5));
      const double k1 = js_min(nz - 1, ceil((double)zs[k + 1] / h - 0.5) - 1);
      for (double kk = k0; kk <= k1; kk++) vox[base + (int64_t)kk] = 1;
    }
  }
  free(cnt); free(hits); free(pos);
}

/* ------------------------------------------------------------------ prepare (:111-234) */
#define FAIL(code, ...) do { g->err = (code); snprintf(g->msg, sizeof g->msg, __VA_ARGS__); goto fail; } while (0)

static void js_fmt_number(char *out, size_t n, double v) {
  /* Shortest round-trip decimal, like JS Number#toString for the cell sizes used here. */
  for (int prec = 1; prec <= 17; prec++) {
    snprintf(out, n, "%.*g", prec, v);
    if (strtod(out, NULL) == v) return;
  }
}

int ora_prepare(const float *T0, size_t nfloats, const ora_prep_params *p, ora_geom *g) {
  memset(g, 0, sizeof *g);
  uint8_t *fine = NULL, *empty = NULL, *outside = NULL, *holes = NULL, *sel = NULL;
  int32_t *q = NULL, *lab = NULL, *comp_start = NULL, *comp_len = NULL, *comp_cells = NULL, *Q = NULL;
  float *T = NULL;
  if (p->sealAxis == p->inletAxis) {
    g->err = ORA_SAME_AXIS;
    snprintf(g->msg, sizeof g->msg, "Einlassseite und Filterebene liegen auf derselben Achse.");
    return g->err;
  }
  ora_make_frame(p, &g->fr);
  const size_t nverts = nfloats / 3;
  T = (float *)calloc(nfloats ? nfloats : 1, sizeof(float));
  double mn[3] = {INFINITY, INFINITY, INFINITY}, mx[3] = {-INFINITY, -INFINITY, -INFINITY};
  for (size_t v = 0; v < nverts; v++) {
    const double qq[3] = {T0[v * 3], T0[v * 3 + 1], T0[v * 3 + 2]};
    double L[3];
    ora_to_local(&g->fr, qq, L);
    for (int a = 0; a < 3; a++) {
      T[v * 3 + a] = (float)L[a];
      if (L[a] < mn[a]) mn[a] = L[a];
      if (L[a] > mx[a]) mx[a] = L[a];
    }
  }
  const double h = p->dx, hf = h / 3;
  const int sub = 3, duct = 10;
  double origin[3] = {mn[0] - h, (p->has_outlet ? js_min(mn[1], -p->out_height) : mn[1]) - h, mn[2] - duct * h};
  const int nx = (int)ceil((mx[0] - origin[0] + h) / h), ny = (int)ceil((mx[1] - origin[1] + h) / h),
            nz = (int)ceil((mx[2] - origin[2] + h) / h);
  const int64_t N = (int64_t)nx * ny * nz;
  g->nx = nx; g->ny = ny; g->nz = nz; g->N = N; g->h = h; g->hf = hf; g->pleat = p->pleat;
  memcpy(g->origin, origin, sizeof origin); memcpy(g->mn, mn, sizeof mn); memcpy(g->mx, mx, sizeof mx);
  if ((double)N > p->max_cells) FAIL(ORA_GRID_TOO_LARGE, "Gitter zu groß (%.1f Mio. Zellen) – Zellgröße erhöhen.", (double)N / 1e6);
  const int nxf = nx * sub, nyf = ny * sub, nzf = nz * sub;
  g->nxf = nxf; g->nyf = nyf; g->nzf = nzf;
  fine = (uint8_t *)malloc((size_t)((int64_t)nxf * nyf * nzf));
  if (!fine) FAIL(ORA_NOMEM, "out of memory");
  ora_voxelize(T, nfloats, origin, nxf, nyf, nzf, hf, fine);
  g->solid = (uint8_t *)calloc((size_t)N, 1);
  for (int i = 0; i < nx; i++) for (int j = 0; j < ny; j++) for (int k = 0; k < nz; k++) {
    int s = 0;
    for (int a = 0; a < 3; a++) for (int b = 0; b < 3; b++) {
      const int64_t base = ((int64_t)(i * 3 + a) * nyf + (j * 3 + b)) * nzf + k * 3;
      s += fine[base] + fine[base + 1] + fine[base + 2];
    }
    if (s >= 7) g->solid[((int64_t)i * ny + j) * nz + k] = 1;
  }
  g->xc = (float *)malloc(sizeof(float) * nx); g->dc = (float *)malloc(sizeof(float) * ny);
  g->zc = (float *)malloc(sizeof(float) * nz);
  for (int i = 0; i < nx; i++) g->xc[i] = (float)(origin[0] + (i + 0.5) * h);
  for (int j = 0; j < ny; j++) g->dc[j] = (float)(origin[1] + (j + 0.5) * h);
  for (int k = 0; k < nz; k++) g->zc[k] = (float)(origin[2] + (k + 0.5) * h);

  /* openings: holes in the frontmost material layer (:141-171) */
  const int kf = (int)floor((mn[2] + 1.5 - origin[2]) / hf);
  g->kf = kf;
  const int64_t nfs = (int64_t)nxf * nyf;
  empty = (uint8_t *)malloc((size_t)nfs); outside = (uint8_t *)calloc((size_t)nfs, 1);
  q = (int32_t *)malloc(sizeof(int32_t) * (size_t)nfs);
  for (int i = 0; i < nxf; i++) for (int j = 0; j < nyf; j++)
    empty[(int64_t)i * nyf + j] = fine[((int64_t)i * nyf + j) * nzf + kf] ? 0 : 1;
  int64_t qh = 0, qt = 0;
#define PUSH(c) do { int64_t c_ = (c); if (empty[c_] && !outside[c_]) { outside[c_] = 1; q[qt++] = (int32_t)c_; } } while (0)
  for (int i = 0; i < nxf; i++) { PUSH((int64_t)i * nyf); PUSH((int64_t)i * nyf + nyf - 1); }
  for (int j = 0; j < nyf; j++) { PUSH(j); PUSH((int64_t)(nxf - 1) * nyf + j); }
  while (qh < qt) {
    const int64_t c = q[qh++]; const int i = (int)(c / nyf), j = (int)(c % nyf);
    if (i > 0) PUSH(c - nyf);
    if (i < nxf - 1) PUSH(c + nyf);
    if (j > 0) PUSH(c - 1);
    if (j < nyf - 1) PUSH(c + 1);
  }
#undef PUSH
  holes = (uint8_t *)malloc((size_t)nfs);
  for (int64_t c = 0; c < nfs; c++)
    holes[c] = empty[c] && !outside[c] && (origin[1] + ((double)(c % nyf) + 0.5) * hf > 0) ? 1 : 0;
  if (p->keep_fine) { g->holes_slice = holes; holes = NULL; }
  const uint8_t *hm = g->holes_slice ? g->holes_slice : holes;
  /* components2d (:95-108): labels in scan order, cells in BFS order */
  lab = (int32_t *)malloc(sizeof(int32_t) * (size_t)nfs);
  for (int64_t c = 0; c < nfs; c++) lab[c] = -1;
  comp_cells = (int32_t *)malloc(sizeof(int32_t) * (size_t)nfs);
  int ncomp = 0, cap = 64;
  comp_start = (int32_t *)malloc(sizeof(int32_t) * cap); comp_len = (int32_t *)malloc(sizeof(int32_t) * cap);
  int64_t ncells = 0;
  for (int64_t s = 0; s < nfs; s++) {
    if (!hm[s] || lab[s] >= 0) continue;
    const int id = ncomp;
    int64_t h0 = ncells, t0 = ncells;
    comp_cells[t0++] = (int32_t)s; lab[s] = id;
    while (h0 < t0) {
      const int64_t c = comp_cells[h0++]; const int i = (int)(c / nyf), j = (int)(c % nyf);
      const int64_t nbv[4] = {i > 0 ? c - nyf : -1, i < nxf - 1 ? c + nyf : -1, j > 0 ? c - 1 : -1, j < nyf - 1 ? c + 1 : -1};
      for (int d = 0; d < 4; d++) {
        const int64_t e = nbv[d];
        if (e >= 0 && hm[e] && lab[e] < 0) { lab[e] = id; comp_cells[t0++] = (int32_t)e; }
      }
    }
    if (ncomp == cap) { cap *= 2; comp_start = (int32_t *)realloc(comp_start, sizeof(int32_t) * cap); comp_len = (int32_t *)realloc(comp_len, sizeof(int32_t) * cap); }
    comp_start[ncomp] = (int32_t)ncells; comp_len[ncomp] = (int32_t)(t0 - ncells); ncomp++;
    ncells = t0;
  }
  /* filter: area > 25 mm^2 */
  int nkeep = 0;
  for (int c = 0; c < ncomp; c++) {
    if ((double)comp_len[c] * hf * hf > 25) { comp_start[nkeep] = comp_start[c]; comp_len[nkeep] = comp_len[c]; nkeep++; }
  }
  g->nHoles = nkeep;
  if (!nkeep) FAIL(ORA_NO_OPENING, "Auf der gewählten Einlassseite wurde keine Öffnung gefunden.");
  int best = 0;
  if (p->has_click) {
    double L[3]; ora_to_local(&g->fr, p->click, L);
    double bd = INFINITY;
    for (int c = 0; c < nkeep; c++) {
      for (int s = 0; s < comp_len[c]; s += 3) {
        const int32_t cc = comp_cells[comp_start[c] + s];
        const double x = origin[0] + ((double)(cc / nyf) + 0.5) * hf, y = origin[1] + ((double)(cc % nyf) + 0.5) * hf;
        const double d = (x - L[0]) * (x - L[0]) + (y - L[1]) * (y - L[1]);
        if (d < bd) { bd = d; best = c; }
      }
    }
  } else {
    for (int c = 1; c < nkeep; c++) if (comp_len[c] > comp_len[best]) best = c;
  }
  sel = (uint8_t *)calloc((size_t)nx * ny, 1);
  for (int s = 0; s < comp_len[best]; s++) {
    const int32_t c = comp_cells[comp_start[best] + s];
    sel[(int64_t)((c / nyf) / 3) * ny + ((c % nyf) / 3)]++;
  }
  g->opening = (uint8_t *)calloc((size_t)nx * ny, 1);
  int nOpen = 0;
  for (int64_t c = 0; c < (int64_t)nx * ny; c++) if (sel[c] >= 5) { g->opening[c] = 1; nOpen++; }
  g->nOpen = nOpen;
  if (nOpen < 8) FAIL(ORA_OPENING_TOO_SMALL, "Einlassöffnung ist zu klein für die gewählte Zellgröße.");

  /* inlet duct, closed bottom, outlet plane (:173-216) */
  int kw0 = -1;
  for (int k = 0; k < nz; k++) if ((double)g->zc[k] >= mn[2]) { kw0 = k; break; }
  g->kw0 = kw0;
  uint8_t *solid = g->solid;
  for (int i = 0; i < nx; i++) for (int j = 0; j < ny; j++) for (int k = 0; k < kw0; k++)
    solid[((int64_t)i * ny + j) * nz + k] = g->opening[(int64_t)i * ny + j] ? 0 : 1;
  for (int j = 0; j < ny; j++) if ((double)g->dc[j] > mx[1] - 0.5 * h)
    for (int i = 0; i < nx; i++) for (int k = 0; k < nz; k++) solid[((int64_t)i * ny + j) * nz + k] = 1;
  int top = -1;
  for (int j = 0; j < ny; j++) if ((double)g->dc[j] >= 0) { top = j; break; }
  g->top = top;
  if (top < 0) FAIL(ORA_SEAL_OUTSIDE, "Dichtebene liegt außerhalb des Modells.");
  g->fluid = (uint8_t *)calloc((size_t)N, 1);
  uint8_t *fluid = g->fluid;
  Q = (int32_t *)malloc(sizeof(int32_t) * (size_t)N);
  qh = 0; qt = 0;
#define VISIT(c_, j_) do { int64_t cc_ = (c_); if (!fluid[cc_] && !solid[cc_] && (j_) >= top) { fluid[cc_] = 1; Q[qt++] = (int32_t)cc_; } } while (0)
  for (int64_t c = 0; c < (int64_t)nx * ny; c++) if (g->opening[c]) VISIT(c * nz, (int)(c % ny));
  while (qh < qt) {
    const int64_t c = Q[qh++]; const int k = (int)(c % nz); const int64_t ij = c / nz;
    const int j = (int)(ij % ny), i = (int)(ij / ny);
    if (i > 0) VISIT(c - (int64_t)ny * nz, j);
    if (i < nx - 1) VISIT(c + (int64_t)ny * nz, j);
    if (j > 0) VISIT(c - nz, j - 1);
    if (j < ny - 1) VISIT(c + nz, j + 1);
    if (k > 0) VISIT(c - 1, j);
    if (k < nz - 1) VISIT(c + 1, j);
  }
#undef VISIT
  int leaked = 0;
  for (int i = 0; i < nx && !leaked; i++) for (int j = top; j < ny && !leaked; j++) for (int k = kw0; k < nz; k++) {
    if ((i == 0 || i == nx - 1 || k == nz - 1) && fluid[((int64_t)i * ny + j) * nz + k]) { leaked = 1; break; }
  }
  if (leaked) {
    char hs[32]; js_fmt_number(hs, sizeof hs, h);
    FAIL(ORA_LEAK, "Bei %s mm Zellgröße läuft die Luft durch eine zu dünne Wand nach außen (Wände sollten mindestens so dick wie eine Zelle sein). Bitte eine kleinere Zellgröße wählen.", hs);
  }
  g->outlet = (uint8_t *)calloc((size_t)N, 1);
  int nOut = 0;
  if (p->has_outlet) {
    const int jpt = first_ge(g->dc, ny, -p->out_height);
    g->jpt = jpt;
    if (jpt >= top) FAIL(ORA_LID_TOO_LOW, "Deckelhöhe ist kleiner als eine Zelle.");
    double L[3]; ora_to_local(&g->fr, p->out_center, L);
    const double r2 = (p->out_diameter / 2) * (p->out_diameter / 2);
    for (int i = 0; i < nx; i++) for (int k = 0; k < nz; k++) {
      if (!fluid[((int64_t)i * ny + top) * nz + k]) continue;
      for (int j = jpt; j < top; j++) { const int64_t c = ((int64_t)i * ny + j) * nz + k; fluid[c] = 1; solid[c] = 0; qt++; }
      const double ddx = (double)g->xc[i] - L[0], ddz = (double)g->zc[k] - L[2];
      if (ddx * ddx + ddz * ddz <= r2) { g->outlet[((int64_t)i * ny + jpt) * nz + k] = 1; nOut++; }
    }
    if (nOut < 4) FAIL(ORA_BAD_OUTLET, "Der Auslass liegt nicht über der Filterfläche oder ist zu klein.");
  } else {
    g->jpt = -1;
    for (int i = 0; i < nx; i++) for (int k = 0; k < nz; k++) {
      const int64_t c = ((int64_t)i * ny + top) * nz + k;
      if (fluid[c]) { g->outlet[c] = 1; nOut++; }
    }
  }
  g->nOut = nOut;
  g->nf = (int)qt;
  g->jm = first_ge(g->dc, ny, p->pleat / 2);
  int Af = 0;
  for (int i = 0; i < nx; i++) for (int k = 0; k < nz; k++) Af += fluid[((int64_t)i * ny + g->jm) * nz + k];
  g->Af = Af;
  int leak = 0;
  for (int i = 0; i < nx; i++) for (int k = 0; k < nz; k++) leak += fluid[((int64_t)i * ny + top) * nz + k];
  g->leak = leak;
  if (p->keep_fine) { g->fine = fine; fine = NULL; }
  free(fine); free(empty); free(outside); free(holes); free(sel); free(q); free(lab);
  free(comp_start); free(comp_len); free(comp_cells); free(Q); free(T);
  return ORA_OK;
fail:
  free(fine); free(empty); free(outside); free(holes); free(sel); free(q); free(lab);
  free(comp_start); free(comp_len); free(comp_cells); free(Q); free(T);
  return g->err;
}
#undef FAIL

void ora_geom_free(ora_geom *g) {
  free(g->xc); free(g->dc); free(g->zc); free(g->solid); free(g->fluid); free(g->opening);
  free(g->outlet); free(g->fine); free(g->holes_slice);
  memset(g, 0, sizeof *g);
}

/* ------------------------------------------------------------------ setupSim (:239-264) */
int ora_setup(const ora_geom *g, const ora_run_params *p, ora_sim *S) {
  memset(S, 0, sizeof *S);
  const int ny = g->ny, nz = g->nz; const int64_t N = g->N;
  const int NF = g->nf;
  S->NF = NF; S->N = N;
  S->cid = (int32_t *)malloc(sizeof(int32_t) * (size_t)N);
  S->cells = (int32_t *)malloc(sizeof(int32_t) * (size_t)(NF ? NF : 1));
  int m = 0;
  for (int64_t c = 0; c < N; c++) { if (g->fluid[c]) { S->cid[c] = m; S->cells[m++] = (int32_t)c; } else S->cid[c] = -1; }
  int64_t off[19];
  for (int i = 0; i < 19; i++) off[i] = ((int64_t)CX[i] * ny + CY[i]) * nz + CZ[i];
  S->nb = (int32_t *)malloc(sizeof(int32_t) * (size_t)NF * 19);
  S->flag = (uint32_t *)calloc((size_t)(NF ? NF : 1), sizeof(uint32_t));
  S->jsOf = (int32_t *)malloc(sizeof(int32_t) * (size_t)(NF ? NF : 1));
  int Ain = 0, Lp = 0;
  const double dtop = g->dc[g->top];
  for (int j = 0; j < ny; j++) if ((double)g->dc[j] > dtop && (double)g->dc[j] <= g->pleat) Lp++;
  for (int a = 0; a < NF; a++) {
    const int64_t c = S->cells[a]; const int k = (int)(c % nz); const int64_t ij = c / nz; const int j = (int)(ij % ny);
    S->jsOf[a] = j;
    for (int i = 0; i < 19; i++) { const int64_t s = c - off[i]; S->nb[(int64_t)a * 19 + i] = s >= 0 && s < N ? S->cid[s] : -1; }
    if (k == 0 && g->opening[ij]) { S->flag[a] = 1; Ain++; }
    else if (g->outlet[c]) S->flag[a] = 2;
    else if ((double)g->dc[j] > dtop && (double)g->dc[j] <= g->pleat) S->flag[a] = 3;
  }
  int nM = 0, nT = 0;
  for (int a = 0; a < NF; a++) { if (S->jsOf[a] == g->jm) nM++; if (S->jsOf[a] == g->top + 1) nT++; }
  S->layerM = (int32_t *)malloc(sizeof(int32_t) * (size_t)(nM ? nM : 1));
  S->layerT = (int32_t *)malloc(sizeof(int32_t) * (size_t)(nT ? nT : 1));
  nM = 0; nT = 0;
  for (int a = 0; a < NF; a++) { if (S->jsOf[a] == g->jm) S->layerM[nM++] = a; if (S->jsOf[a] == g->top + 1) S->layerT[nT++] = a; }
  S->nM = nM; S->nT = nT; S->Af = nM; S->Ain = Ain; S->Lp = Lp;
  const double u0 = p->u, uface = u0 * Ain / nM;
  S->u0 = u0; S->tau0 = p->tau; S->aniso = p->aniso;
  S->sig = p->K * 0.5 * u0 * u0 / (uface * (Lp > 1 ? Lp : 1));
  S->cs2s = 18 * M_SQRT2 * 0.17 * 0.17;
  return ORA_OK;
}

void ora_sim_free(ora_sim *S) {
  free(S->cid); free(S->cells); free(S->nb); free(S->flag); free(S->jsOf); free(S->layerM); free(S->layerT);
  memset(S, 0, sizeof *S);
}

void ora_init_f32(const ora_sim *S, float *f) {
  for (int i = 0; i < 19; i++) for (int a = 0; a < S->NF; a++) f[(int64_t)i * S->NF + a] = (float)WT[i];
}
void ora_init_f64(const ora_sim *S, double *f) {
  for (int i = 0; i < 19; i++) for (int a = 0; a < S->NF; a++) f[(int64_t)i * S->NF + a] = WT[i];
}

/* ------------------------------------------------------------------ cpuStep (:266-321) */
#define STEP_NAME step_f32
#define ST float
#define LT double
#define SQRT sqrt
#define MIN js_min
#include "engine_ref_step.inc"
#undef STEP_NAME
#undef ST
#undef LT
#undef SQRT
#undef MIN

#define STEP_NAME step_f64
#define ST double
#define LT double
#define SQRT sqrt
#define MIN js_min
#include "engine_ref_step.inc"
#undef STEP_NAME
#undef ST
#undef LT
#undef SQRT
#undef MIN

#define STEP_NAME step_f32l
#define ST float
#define LT float
#define SQRT sqrtf
#define MIN js_minf
#include "engine_ref_step.inc"
#undef STEP_NAME
#undef ST
#undef LT
#undef SQRT
#undef MIN

void ora_step_f32(const ora_sim *S, const float *f, float *f2, float *acc, const float *ns, int nthreads) { step_f32(S, f, f2, acc, ns, nthreads); }
void ora_step_f64(const ora_sim *S, const double *f, double *f2, double *acc, const float *ns, int nthreads) { step_f64(S, f, f2, acc, ns, nthreads); }
void ora_step_f32l(const ora_sim *S, const float *f, float *f2, float *acc, const float *ns, int nthreads) { step_f32l(S, f, f2, acc, ns, nthreads); }

/* ------------------------------------------------------------------ probe + progress (:324-339) */
#define PROBE_BODY(ST)                                                                          \
  const int NF = S->NF, nM = S->nM, np = S->nM + S->nT;                                         \
  double sw = 0, dev = 0, qo = 0;                                                               \
  float *vy = (float *)malloc(sizeof(float) * (size_t)(np ? np : 1));                           \
  for (int n = 0; n < np; n++) {                                                                \
    const int a = n < nM ? S->layerM[n] : S->layerT[n - nM];                                    \
    double r = 0, my = 0;                                                                       \
    for (int i = 0; i < 19; i++) { const double v = (double)f[(int64_t)i * NF + a]; r += v; my += CY[i] * v; } \
    vy[n] = (float)(my / r);                                                                    \
  }                                                                                             \
  for (int n = 0; n < nM; n++) sw += -(double)vy[n];                                            \
  const double wm = sw / nM;                                                                    \
  for (int n = 0; n < nM; n++) dev += fabs(-(double)vy[n] - wm);                                \
  for (int n = nM; n < np; n++) qo += -(double)vy[n];                                           \
  free(vy);                                                                                     \
  out[0] = 1 - dev / (2 * nM * wm); out[1] = qo / (S->Ain * S->u0); out[2] = qo;

static void probe_f32(const ora_sim *S, const float *f, double out[3]) { PROBE_BODY(float) }
static void probe_f64(const ora_sim *S, const double *f, double out[3]) { PROBE_BODY(double) }

/* ------------------------------------------------------------------ simulate (:341-358) */
#define SIMULATE_BODY(ST, STEP, PROBE, INIT)                                                    \
  const int NF = S->NF;                                                                         \
  ST *f = (ST *)malloc(sizeof(ST) * 19 * (size_t)NF), *f2 = (ST *)calloc(19 * (size_t)NF, sizeof(ST)); \
  ST *acc = (ST *)calloc(4 * (size_t)NF, sizeof(ST));                                          \
  INIT(S, f);                                                                                   \
  int nacc = 0, nh = 0, rc = ORA_OK;                                                            \
  for (int step = 1; step <= steps; step++) {                                                   \
    const int doAcc = step > steps - avg;                                                       \
    STEP(S, f, f2, doAcc ? acc : NULL, ns, nthreads);                                           \
    ST *tmp = f; f = f2; f2 = tmp;                                                              \
    if (doAcc) nacc++;                                                                          \
    if (step % every == 0 || step == steps) {                                                   \
      double pr[3]; PROBE(S, f, pr);                                                            \
      if (!isfinite(pr[2])) {                                                                   \
        if (msg) snprintf(msg, 512, "Rechnung instabil bei Schritt %d. Zellgröße vergrößern oder Viskosität (tau) erhöhen.", step); \
        rc = ORA_UNSTABLE; break;                                                               \
      }                                                                                         \
      if (hist) { hist[3 * nh] = step; hist[3 * nh + 1] = pr[0]; hist[3 * nh + 2] = pr[1]; }    \
      nh++;                                                                                     \
    }                                                                                           \
  }                                                                                             \
  const double dn = nacc > 1 ? nacc : 1;                                                        \
  for (int64_t x = 0; x < 4 * (int64_t)NF; x++) acc_out[x] = (ST)((double)acc[x] / dn);         \
  if (nhist) *nhist = nh;                                                                       \
  free(f); free(f2); free(acc);                                                                 \
  return rc;

int ora_simulate_f32(const ora_sim *S, int steps, int avg, int every, const float *ns, int nthreads,
                     float *acc_out, double *hist, int *nhist, char *msg) {
  SIMULATE_BODY(float, step_f32, probe_f32, ora_init_f32)
}
int ora_simulate_f64(const ora_sim *S, int steps, int avg, int every, const float *ns, int nthreads,
                     double *acc_out, double *hist, int *nhist, char *msg) {
  SIMULATE_BODY(double, step_f64, probe_f64, ora_init_f64)
}

/* ------------------------------------------------------------------ evaluate (:632-660, :681-685) */
#define EVAL_BODY(ST)                                                                           \
  const int nx = g->nx, ny = g->ny, nz = g->nz, NF = S->NF;                                     \
  const int64_t N = g->N, nxz = (int64_t)nx * nz;                                               \
  uint8_t *fl = (uint8_t *)malloc((size_t)N);                                                   \
  for (int64_t c = 0; c < N; c++) {                                                             \
    const int32_t a = S->cid[c];                                                                \
    fl[c] = g->fluid[c] && !(ns && a >= 0 && ns[a] > 0.5f) ? 1 : 0;                              \
  }                                                                                             \
  const int jm = g->jm;                                                                         \
  /* w = -mean(u_y) on layer jm; fmap holds it (NaN = no air), :638-640 */                      \
  double *wv = (double *)malloc(sizeof(double) * (size_t)nxz);                                  \
  double sw = 0; int n = 0;                                                                     \
  for (int i = 0; i < nx; i++) for (int k = 0; k < nz; k++) {                                  \
    const int64_t c = ((int64_t)i * ny + jm) * nz + k;                                          \
    wv[(int64_t)i * nz + k] = NAN;                                                              \
    if (fl[c]) { const int32_t a = S->cid[c]; const double w = -(double)acc[(int64_t)NF + a];    \
      wv[(int64_t)i * nz + k] = w; sw += w; n++; }                                              \
  }                                                                                             \
  const double wm = sw / n;                                                                     \
  double dev = 0, cdev = 0, csum = 0, mxr = 0; int cn = 0, low = 0, high = 0, rev = 0;          \
  uint8_t *core = (uint8_t *)calloc((size_t)nxz, 1);                                            \
  for (int i = 1; i < nx - 1; i++) for (int k = 1; k < nz - 1; k++) {                           \
    _Bool ok = fl[((int64_t)i * ny + jm) * nz + k] && fl[((int64_t)(i - 1) * ny + jm) * nz + k] && \
               fl[((int64_t)(i + 1) * ny + jm) * nz + k] && fl[((int64_t)i * ny + jm) * nz + k - 1] && \
               fl[((int64_t)i * ny + jm) * nz + k + 1];                                         \
    if (ok) core[(int64_t)i * nz + k] = 1;                                                      \
  }                                                                                             \
  for (int64_t x = 0; x < nxz; x++) if (core[x]) { csum += wv[x]; cn++; }                      \
  const double cm = csum / cn;                                                                  \
  for (int64_t x = 0; x < nxz; x++) {                                                           \
    const double w = wv[x]; fmap[x] = NAN; if (isnan(w)) continue;                              \
    dev += fabs(w - wm); if (w < 0) rev++; mxr = js_max(mxr, w / wm);                           \
    if (core[x]) { cdev += fabs(w - cm); if (w < 0.5 * cm) low++; if (w > 1.5 * cm) high++; }   \
    fmap[x] = (float)(w / wm);                                                                  \
  }                                                                                             \
  double pin = 0, pb = 0; int pinN = 0, pbN = 0;                                                \
  const int jb = first_ge(g->dc, ny, g->pleat + 2 * g->h);                                     \
  for (int i = 0; i < nx; i++) for (int j = 0; j < ny; j++) if (g->opening[(int64_t)i * ny + j]) { \
    const int64_t c = ((int64_t)i * ny + j) * nz + 1;                                           \
    if (fl[c]) { const int32_t a = S->cid[c]; pin += (a < 0 ? NAN : (double)acc[3 * (int64_t)NF + a]); pinN++; } \
  }                                                                                             \
  for (int i = 0; i < nx; i++) for (int k = 0; k < nz; k++) {                                   \
    const int64_t c = ((int64_t)i * ny + jb) * nz + k;                                          \
    if (fl[c]) { const int32_t a = S->cid[c]; pb += (a < 0 ? NAN : (double)acc[3 * (int64_t)NF + a]); pbN++; } \
  }                                                                                             \
  const double h = g->h;                                                                        \
  m->zeta = ((pin / pinN - pb / pbN) / 3) / (0.5 * u0 * u0);                                    \
  m->gamma = 1 - dev / (2 * n * wm); m->gammaCore = 1 - cdev / (2 * cn * cm);                   \
  m->lowCore = (double)low / cn; m->highCore = (double)high / cn; m->reverse = (double)rev / n; \
  m->maxToMean = mxr; m->inlet_cm2 = S->Ain * h * h / 100; m->filter_cm2 = S->Af * h * h / 100; \
  m->wm = wm; m->cm = cm; m->n = n; m->cn = cn; m->pinN = pinN; m->pbN = pbN; m->jb = jb;       \
  free(fl); free(core); free(wv);

void ora_evaluate_f32(const ora_geom *g, const ora_sim *S, double u0, const float *acc,
                      const float *ns, ora_metrics *m, float *fmap) { EVAL_BODY(float) }
void ora_evaluate_f64(const ora_geom *g, const ora_sim *S, double u0, const double *acc,
                      const float *ns, ora_metrics *m, float *fmap) { EVAL_BODY(double) }
