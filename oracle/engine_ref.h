/* engine_ref.h - ORACLE ONLY (test infrastructure, never linked into the product).
 *
 * Plain-C restatement of the reference compute core in src/engine.js, used by
 * tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg as the
 * checker.  See engine_ref.c for the per-function citations and the parity
 * status.
 */
#ifndef AIRBOX_ENGINE_REF_H
#define AIRBOX_ENGINE_REF_H
#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum {
  ORA_OK = 0, ORA_NO_TRIANGLES = 1, ORA_SAME_AXIS = 2, ORA_GRID_TOO_LARGE = 3,
  ORA_NO_OPENING = 4, ORA_OPENING_TOO_SMALL = 5, ORA_SEAL_OUTSIDE = 6, ORA_LEAK = 7,
  ORA_LID_TOO_LOW = 8, ORA_BAD_OUTLET = 9, ORA_UNSTABLE = 10, ORA_NOMEM = 11
};

typedef struct {
  int dAx, iAx, oAx;
  double sd, si, seal, yaw_deg, cy, sy;
} ora_frame;

typedef struct {
  double dx;
  int sealAxis; double sealSign, seal;
  int inletAxis; double inletSign, inletYaw;
  double pleat;
  int has_click; double click[3];
  int has_outlet; double out_center[3], out_diameter, out_height;
  double max_cells;          /* reference: 4.5e6 */
  int keep_fine;             /* keep the fine (3x) voxel grid for tests */
} ora_prep_params;

typedef struct {
  int nx, ny, nz; int64_t N;
  int nxf, nyf, nzf, kf, kw0;
  double h, hf, origin[3], mn[3], mx[3], pleat;
  int top, jm, nf, nOpen, Af, nHoles, nOut, leak, jpt;
  ora_frame fr;
  float *xc, *dc, *zc;
  uint8_t *solid, *fluid, *opening, *outlet, *fine, *holes_slice;
  int err; char msg[512];
} ora_geom;

typedef struct {
  double K, aniso, u, tau;
} ora_run_params;

typedef struct {
  int NF, Ain, Af, Lp, nM, nT;
  double u0, tau0, sig, aniso, cs2s;
  int32_t *cid, *cells, *nb, *jsOf, *layerM, *layerT;
  uint32_t *flag;
  int64_t N;
} ora_sim;

typedef struct {
  double gamma, gammaCore, lowCore, highCore, reverse, maxToMean, zeta, inlet_cm2, filter_cm2;
  double wm, cm; int n, cn, pinN, pbN, jb;
} ora_metrics;

int ora_parse_stl(const uint8_t *buf, size_t len, float *out, size_t cap, size_t *nfloats, char *msg);
void ora_make_frame(const ora_prep_params *p, ora_frame *fr);
void ora_to_local(const ora_frame *fr, const double q[3], double out[3]);
void ora_to_model(const ora_frame *fr, double X, double D, double Z, double out[3]);
int ora_prepare(const float *tris, size_t nfloats, const ora_prep_params *p, ora_geom *g);
void ora_geom_free(ora_geom *g);
void ora_voxelize(const float *T, size_t nfloats, const double origin[3], int nx, int ny, int nz,
                  double h, uint8_t *vox);
int ora_setup(const ora_geom *g, const ora_run_params *p, ora_sim *S);
void ora_sim_free(ora_sim *S);
void ora_init_f32(const ora_sim *S, float *f);
void ora_init_f64(const ora_sim *S, double *f);
void ora_step_f32(const ora_sim *S, const float *f, float *f2, float *acc, const float *ns, int nthreads);
void ora_step_f64(const ora_sim *S, const double *f, double *f2, double *acc, const float *ns, int nthreads);
void ora_step_f32l(const ora_sim *S, const float *f, float *f2, float *acc, const float *ns, int nthreads);
int ora_simulate_f32(const ora_sim *S, int steps, int avg, int every, const float *ns, int nthreads,
                     float *acc_out, double *hist, int *nhist, char *msg);
int ora_simulate_f64(const ora_sim *S, int steps, int avg, int every, const float *ns, int nthreads,
                     double *acc_out, double *hist, int *nhist, char *msg);
void ora_evaluate_f32(const ora_geom *g, const ora_sim *S, double u0, const float *acc,
                      const float *ns, ora_metrics *m, float *fmap);
void ora_evaluate_f64(const ora_geom *g, const ora_sim *S, double u0, const double *acc,
                      const float *ns, ora_metrics *m, float *fmap);

/* post-processing of the averages (engine_ref_post.c) */
double ora_js_hypot3(double x, double y, double z);
double ora_js_round(double x);
void ora_field3d(const ora_geom *g, const ora_sim *S, double u0, const float *acc, const float *ns, float *spd,
                 float *pst, float *loss, int *kB_out, double *pin_out, double *rho_ref_out);
void ora_planes(const ora_geom *g, const ora_sim *S, double u0, const float *acc, const float *ns, float *out,
                int meta[3]);
int ora_streamlines(const ora_geom *g, const ora_sim *S, double u0, const float *acc, const float *ns, int max_seeds,
                    float *pts, float *spd, uint32_t *off, int cap_pts, int cap_lines, int *nlines_out,
                    int *npts_out);

#ifdef __cplusplus
}
#endif
#endif
