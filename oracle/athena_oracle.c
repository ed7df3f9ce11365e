/* athena_oracle.c -- CPU restatement of the reference's finite-volume (M)HD stage.
 *
 * TEST INFRASTRUCTURE ONLY. This file is the oracle: the CUDA product path is checked
 * against it, and bench.py times it as the CPU baseline. Nothing in the product links
 * or calls it. It is pinned against the reference itself: tests/golden/ holds states
 * produced by the unmodified reference solver (built by oracle/build_ref.py), and the
 * tests check this restatement against them (bit-exact in FP64 on one block).
 *
 * Scope: uniform Cartesian mesh held as ONE block with NG ghost layers and periodic
 * boundaries (a same-level periodic mesh split into MeshBlocks gives the same result,
 * because ghost exchange is an exact copy). Adiabatic EOS, hydro or MHD.
 *
 * Each routine follows a reference routine (paths relative to the reference src/):
 *   coordinates        coordinates/coordinates.cpp:88-150, coordinates/cartesian.cpp:26-36,
 *                      mesh/mesh.hpp:389-405,467-488 (uniform generator)
 *   c2p                eos/adiabatic_mhd.cpp:41-90, eos/adiabatic_hydro.cpp:39-81,
 *                      field/field.cpp:112-180 (cell-centred B)
 *   donor cell         reconstruct/dc.cpp:24-110
 *   PLM (uniform)      reconstruct/plm.cpp:27-351
 *   PPM                reconstruct/ppm.cpp:44-923 (uniform Cartesian branch)
 *   HLLC               hydro/rsolvers/hydro/hllc.cpp:32-179
 *   HLLE (hydro)       hydro/rsolvers/hydro/hlle.cpp:38-162
 *   HLLE (MHD)         hydro/rsolvers/mhd/hlle_mhd.cpp:25-182
 *   HLLD               hydro/rsolvers/mhd/hlld.cpp:38-382
 *   CT weight          hydro/hydro.cpp:154-158
 *   flux sweeps        hydro/calculate_fluxes.cpp:36-320 (loop extents for MHD)
 *   corner EMF         field/calculate_corner_e.cpp:129-229
 *   flux divergence    hydro/add_flux_divergence.cpp:39-96
 *   CT update          field/ct.cpp:31-116
 *   register averaging mesh/weighted_ave.cpp:33-237 (cell), :238- (face)
 *   stage logic        task_list/time_integrator.cpp:1385-1653, 1965-2093
 *   stage weights      task_list/time_integrator.cpp:100-600
 *   block dt           hydro/new_blockdt.cpp:42-190, mesh/mesh.cpp:1078-1118
 *   periodic ghosts    bvals/fc/bvals_fc.cpp:344-397 (face ranges), bvals/cc/bvals_cc.cpp
 *
 * Arithmetic is kept operation-for-operation identical to the reference so that the
 * FP64 result is bitwise reproducible; build with -ffp-contract=off.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define NHYD 5
#define IDN 0
#define IVX 1
#define IVY 2
#define IVZ 3
#define IPR 4
#define IEN 4
#define IBY 5
#define IBZ 6
#define TINYN 1.0e-20
#define SMALLN 1.0e-8
#define SQ(x) ((x) * (x))

/* std::min / std::max semantics (first argument wins ties, incl. signed zeros) */
static inline double fmin_ref(double a, double b) { return (b < a) ? b : a; }
static inline double fmax_ref(double a, double b) { return (a < b) ? b : a; }

enum { ORC_HLLE = 0, ORC_HLLC = 1, ORC_HLLD = 2, ORC_LHLLC = 3, ORC_LHLLD = 4 };
enum { ORC_VL2 = 0, ORC_RK1 = 1, ORC_RK2 = 2, ORC_RK3 = 3 };

typedef struct {
  int nx1, nx2, nx3, ng;
  int mhd, rsolver, xorder, integrator;
  double gamma, dfloor, pfloor, cfl;
  double x1min, x1max, x2min, x2max, x3min, x3max;
} orc_params;

typedef struct {
  orc_params p;
  int n1, n2, n3, is, ie, js, je, ks, ke;
  size_t ncell;
  double *u, *u1, *w, *w1, *bcc;            /* cell arrays (5 or 3 vars) */
  double *b1, *b2, *b3, *r1, *r2, *r3;      /* face fields and their register */
  double *f1, *f2, *f3;                     /* fluxes (5 vars), face-array sized */
  double *e3x1, *e2x1, *wx1, *e1x2, *e3x2, *wx2, *e1x3, *e2x3, *wx3;
  double *e1, *e2, *e3, *cce;               /* edge EMFs, cell-centre E (3 vars) */
  double *x1f, *x2f, *x3f, *x1v, *x2v, *x3v;
  double dx1, dx2, dx3;
  double dt, time;
  int nstages;
  double delta[4], g1[4], g2[4], g3[4], beta[4];
  /* self-gravity (SELF_GRAVITY_ENABLED == 2): potential with one ghost layer, the
   * attached multigrid solver (mg_oracle.c) and 4 pi G */
  double *phi;
  struct orc_mg_s *mg;
  double four_pi_G;
} orc_sim;

/* mg_oracle.c */
struct orc_mg_s;
double *orc_mg_u(struct orc_mg_s *m);
double *orc_mg_src(struct orc_mg_s *m);
void orc_mg_solve(struct orc_mg_s *m);
int orc_mg_size(const struct orc_mg_s *m);

/* ---------------------------------------------------------------- indexing ---- */
#define C3(s, k, j, i) ((((size_t)(k)) * (s)->n2 + (size_t)(j)) * (s)->n1 + (size_t)(i))
#define F1I(s, k, j, i) ((((size_t)(k)) * (s)->n2 + (size_t)(j)) * ((s)->n1 + 1) + (size_t)(i))
#define F2I(s, k, j, i) ((((size_t)(k)) * ((s)->n2 + 1) + (size_t)(j)) * (s)->n1 + (size_t)(i))
#define F3I(s, k, j, i) C3(s, k, j, i)
/* edge arrays are allocated (n3+1)(n2+1)(n1+1) */
#define EI(s, k, j, i) ((((size_t)(k)) * ((s)->n2 + 1) + (size_t)(j)) * ((s)->n1 + 1) + (size_t)(i))

static size_t f1n(const orc_sim *s) { return (size_t)s->n3 * s->n2 * (s->n1 + 1); }
static size_t f2n(const orc_sim *s) { return (size_t)s->n3 * (s->n2 + 1) * s->n1; }
static size_t f3n(const orc_sim *s) { return (size_t)(s->n3 + 1) * s->n2 * s->n1; }
static size_t en(const orc_sim *s) { return (size_t)(s->n3 + 1) * (s->n2 + 1) * (s->n1 + 1); }

/* ------------------------------------------------------------- coordinates ---- */
/* mesh/mesh.hpp:389-405 (symmetric logical position) and :467-488 (generator) */
static double gen_rx(int64_t index, int64_t nrange) {
  int64_t noffset = index - nrange / 2;
  int64_t noffset_ceil = index - (nrange + 1) / 2;
  return (double)(noffset + noffset_ceil) / (2.0 * nrange);
}
static double gen_x(double rx, double xmin, double xmax) {
  return 0.5 * (xmin + xmax) + (rx * xmax - rx * xmin);
}
/* coordinates/coordinates.cpp:127-145 (uniform branch), cartesian.cpp:26-29 */
static void make_axis(int nx, int ng, double xmin, double xmax, double *xf, double *xv,
                      double *dx) {
  int il = ng, iu = ng + nx - 1;
  *dx = (xmax - xmin) / (iu - il + 1);
  for (int i = il - ng; i <= iu + ng + 1; ++i) {
    int64_t noff = (int64_t)(i - il);
    xf[i] = gen_x(gen_rx(noff, nx), xmin, xmax);
  }
  xf[il] = xmin;
  xf[iu + 1] = xmax;
  for (int i = il - ng; i <= iu + ng; ++i) xv[i] = 0.5 * (xf[i + 1] + xf[i]);
}

/* ------------------------------------------------------------------ setup ---- */
static void set_weights(orc_sim *s) {
  /* task_list/time_integrator.cpp:100-600 (no orbital advection) */
  int it = s->p.integrator;
  memset(s->delta, 0, sizeof(s->delta));
  if (it == ORC_VL2) {
    s->nstages = 2;
    s->beta[0] = 0.5; s->beta[1] = 1.0;
    s->delta[0] = 1.0; s->g1[0] = 0.0; s->g2[0] = 1.0; s->g3[0] = 0.0;
    s->delta[1] = 0.0; s->g1[1] = 0.0; s->g2[1] = 1.0; s->g3[1] = 0.0;
  } else if (it == ORC_RK1) {
    s->nstages = 1;
    s->beta[0] = 1.0;
    s->delta[0] = 1.0; s->g1[0] = 0.0; s->g2[0] = 1.0; s->g3[0] = 0.0;
  } else if (it == ORC_RK2) {
    s->nstages = 2;
    s->beta[0] = 1.0; s->beta[1] = 0.5;
    s->delta[0] = 1.0; s->g1[0] = 0.0; s->g2[0] = 1.0; s->g3[0] = 0.0;
    s->delta[1] = 0.0; s->g1[1] = 0.5; s->g2[1] = 0.5; s->g3[1] = 0.0;
  } else {
    s->nstages = 3;
    s->beta[0] = 1.0; s->beta[1] = 0.25; s->beta[2] = 0.66666666666666667;
    s->delta[0] = 1.0; s->g1[0] = 0.0; s->g2[0] = 1.0; s->g3[0] = 0.0;
    s->delta[1] = 0.0; s->g1[1] = 0.25; s->g2[1] = 0.75; s->g3[1] = 0.0;
    s->delta[2] = 0.0; s->g1[2] = 0.66666666666666667; s->g2[2] = 0.33333333333333333;
    s->g3[2] = 0.0;
  }
}

orc_sim *orc_create(const orc_params *p) {
  orc_sim *s = (orc_sim *)calloc(1, sizeof(orc_sim));
  s->p = *p;
  int g = p->ng;
  s->n1 = p->nx1 + 2 * g; s->n2 = p->nx2 + 2 * g; s->n3 = p->nx3 + 2 * g;
  s->is = g; s->ie = g + p->nx1 - 1;
  s->js = g; s->je = g + p->nx2 - 1;
  s->ks = g; s->ke = g + p->nx3 - 1;
  s->ncell = (size_t)s->n1 * s->n2 * s->n3;
  size_t nc = s->ncell;
  s->u = calloc(NHYD * nc, 8); s->u1 = calloc(NHYD * nc, 8);
  s->w = calloc(NHYD * nc, 8); s->w1 = calloc(NHYD * nc, 8);
  s->f1 = calloc(NHYD * f1n(s), 8); s->f2 = calloc(NHYD * f2n(s), 8);
  s->f3 = calloc(NHYD * f3n(s), 8);
  if (p->mhd) {
    s->bcc = calloc(3 * nc, 8);
    s->b1 = calloc(f1n(s), 8); s->b2 = calloc(f2n(s), 8); s->b3 = calloc(f3n(s), 8);
    s->r1 = calloc(f1n(s), 8); s->r2 = calloc(f2n(s), 8); s->r3 = calloc(f3n(s), 8);
    s->e3x1 = calloc(f1n(s), 8); s->e2x1 = calloc(f1n(s), 8); s->wx1 = calloc(f1n(s), 8);
    s->e1x2 = calloc(f2n(s), 8); s->e3x2 = calloc(f2n(s), 8); s->wx2 = calloc(f2n(s), 8);
    s->e1x3 = calloc(f3n(s), 8); s->e2x3 = calloc(f3n(s), 8); s->wx3 = calloc(f3n(s), 8);
    s->e1 = calloc(en(s), 8); s->e2 = calloc(en(s), 8); s->e3 = calloc(en(s), 8);
    s->cce = calloc(3 * nc, 8);
  }
  s->x1f = calloc(s->n1 + 1, 8); s->x1v = calloc(s->n1, 8);
  s->x2f = calloc(s->n2 + 1, 8); s->x2v = calloc(s->n2, 8);
  s->x3f = calloc(s->n3 + 1, 8); s->x3v = calloc(s->n3, 8);
  make_axis(p->nx1, g, p->x1min, p->x1max, s->x1f, s->x1v, &s->dx1);
  make_axis(p->nx2, g, p->x2min, p->x2max, s->x2f, s->x2v, &s->dx2);
  make_axis(p->nx3, g, p->x3min, p->x3max, s->x3f, s->x3v, &s->dx3);
  set_weights(s);
  s->dt = 1.79769313486231570815e308; /* mesh/mesh.cpp:91 */
  return s;
}

void orc_destroy(orc_sim *s) {
  if (!s) return;
  double *ptrs[] = {s->u, s->u1, s->w, s->w1, s->bcc, s->b1, s->b2, s->b3, s->r1, s->r2,
                    s->r3, s->f1, s->f2, s->f3, s->e3x1, s->e2x1, s->wx1, s->e1x2, s->e3x2,
                    s->wx2, s->e1x3, s->e2x3, s->wx3, s->e1, s->e2, s->e3, s->cce, s->x1f,
                    s->x2f, s->x3f, s->x1v, s->x2v, s->x3v, s->phi};
  for (size_t n = 0; n < sizeof(ptrs) / sizeof(ptrs[0]); ++n) free(ptrs[n]);
  free(s);
}

/* Sizes of the arrays the caller exchanges (full arrays including ghosts). */
void orc_dims(const orc_sim *s, int64_t *out) {
  out[0] = s->n1; out[1] = s->n2; out[2] = s->n3; out[3] = (int64_t)s->ncell;
}
double *orc_array(orc_sim *s, int which) {
  switch (which) {
    case 0: return s->u;
    case 1: return s->b1;
    case 2: return s->b2;
    case 3: return s->b3;
    case 4: return s->w;
    case 5: return s->bcc;
    case 6: return s->x1f;
    case 7: return s->x2f;
    case 8: return s->x3f;
    default: return NULL;
  }
}
double orc_get_dt(const orc_sim *s) { return s->dt; }
void orc_set_dt(orc_sim *s, double dt) { s->dt = dt; }
double orc_get_time(const orc_sim *s) { return s->time; }

/* --------------------------------------------------------- periodic ghosts ---- */
static inline int wrap_c(int i, int lo, int hi, int n) {
  if (i < lo) return i + n;
  if (i > hi) return i - n;
  return i;
}
/* A ghost location takes the value at its periodic image; for the face-normal index
 * the owned range is [s, e+1] (bvals/fc/bvals_fc.cpp:351-394, no exchange of the
 * shared face), for cell indices it is [s, e]. */
static void periodic_cc(orc_sim *s, double *a, int nvar) {
  int nx1 = s->p.nx1, nx2 = s->p.nx2, nx3 = s->p.nx3;
  for (int n = 0; n < nvar; ++n) {
    double *v = a + (size_t)n * s->ncell;
#pragma omp parallel for collapse(2)
    for (int k = 0; k < s->n3; ++k)
      for (int j = 0; j < s->n2; ++j)
        for (int i = 0; i < s->n1; ++i) {
          int kk = wrap_c(k, s->ks, s->ke, nx3), jj = wrap_c(j, s->js, s->je, nx2),
              ii = wrap_c(i, s->is, s->ie, nx1);
          if (kk != k || jj != j || ii != i) v[C3(s, k, j, i)] = v[C3(s, kk, jj, ii)];
        }
  }
}
static void periodic_fc(orc_sim *s, double *b1, double *b2, double *b3) {
  int nx1 = s->p.nx1, nx2 = s->p.nx2, nx3 = s->p.nx3;
#pragma omp parallel for collapse(2)
  for (int k = 0; k < s->n3; ++k)
    for (int j = 0; j < s->n2; ++j)
      for (int i = 0; i <= s->n1; ++i) {
        int kk = wrap_c(k, s->ks, s->ke, nx3), jj = wrap_c(j, s->js, s->je, nx2),
            ii = wrap_c(i, s->is, s->ie + 1, nx1);
        if (kk != k || jj != j || ii != i) b1[F1I(s, k, j, i)] = b1[F1I(s, kk, jj, ii)];
      }
#pragma omp parallel for collapse(2)
  for (int k = 0; k < s->n3; ++k)
    for (int j = 0; j <= s->n2; ++j)
      for (int i = 0; i < s->n1; ++i) {
        int kk = wrap_c(k, s->ks, s->ke, nx3), jj = wrap_c(j, s->js, s->je + 1, nx2),
            ii = wrap_c(i, s->is, s->ie, nx1);
        if (kk != k || jj != j || ii != i) b2[F2I(s, k, j, i)] = b2[F2I(s, kk, jj, ii)];
      }
#pragma omp parallel for collapse(2)
  for (int k = 0; k <= s->n3; ++k)
    for (int j = 0; j < s->n2; ++j)
      for (int i = 0; i < s->n1; ++i) {
        int kk = wrap_c(k, s->ks, s->ke + 1, nx3), jj = wrap_c(j, s->js, s->je, nx2),
            ii = wrap_c(i, s->is, s->ie, nx1);
        if (kk != k || jj != j || ii != i) b3[F3I(s, k, j, i)] = b3[F3I(s, kk, jj, ii)];
      }
}

/* --------------------------------------------------------------------- EOS ---- */
/* field/field.cpp:112-180 (uniform weights 0.5) and eos/adiabatic_mhd.cpp:41-90 */
static void c2p(orc_sim *s) {
  const double gm1 = s->p.gamma - 1.0;
  const double df = s->p.dfloor, pf = s->p.pfloor;
  const size_t nc = s->ncell;
#pragma omp parallel for collapse(2)
  for (int k = 0; k < s->n3; ++k)
    for (int j = 0; j < s->n2; ++j)
      for (int i = 0; i < s->n1; ++i) {
        size_t c = C3(s, k, j, i);
        double pb = 0.0;
        if (s->p.mhd) {
          double bc1 = 0.5 * s->b1[F1I(s, k, j, i)] + 0.5 * s->b1[F1I(s, k, j, i + 1)];
          double bc2 = 0.5 * s->b2[F2I(s, k, j, i)] + 0.5 * s->b2[F2I(s, k, j + 1, i)];
          double bc3 = 0.5 * s->b3[F3I(s, k, j, i)] + 0.5 * s->b3[F3I(s, k + 1, j, i)];
          s->bcc[c] = bc1; s->bcc[nc + c] = bc2; s->bcc[2 * nc + c] = bc3;
          pb = 0.5 * (SQ(bc1) + SQ(bc2) + SQ(bc3));
        }
        double *ud = &s->u[c], *ue = &s->u[4 * nc + c];
        double m1 = s->u[nc + c], m2 = s->u[2 * nc + c], m3 = s->u[3 * nc + c];
        *ud = (*ud > df) ? *ud : df;
        s->w1[c] = *ud;
        double di = 1.0 / *ud;
        s->w1[nc + c] = m1 * di;
        s->w1[2 * nc + c] = m2 * di;
        s->w1[3 * nc + c] = m3 * di;
        double e_k = 0.5 * di * (SQ(m1) + SQ(m2) + SQ(m3));
        double wp = s->p.mhd ? gm1 * (*ue - e_k - pb) : gm1 * (*ue - e_k);
        if (s->p.mhd)
          *ue = (wp > pf) ? *ue : ((pf / gm1) + e_k + pb);
        else
          *ue = (wp > pf) ? *ue : ((pf / gm1) + e_k);
        s->w1[4 * nc + c] = (wp > pf) ? wp : pf;
      }
  double *t = s->w; s->w = s->w1; s->w1 = t; /* time_integrator.cpp:2035 swap */
}

/* eos/adiabatic_mhd.cpp:149-156 */
static inline double fast_speed(const double *pr, double bx, double gamma) {
  double asq = gamma * pr[IPR];
  double vaxsq = bx * bx;
  double ct2 = (pr[IBY] * pr[IBY] + pr[IBZ] * pr[IBZ]);
  double qsq = vaxsq + ct2 + asq;
  double tmp = vaxsq + ct2 - asq;
  return sqrt(0.5 * (qsq + sqrt(tmp * tmp + 4.0 * asq * ct2)) / pr[IDN]);
}

/* hydro/hydro.cpp:154-158 */
static inline double ct_weight(double dflx, double rhol, double rhor, double dx, double dt) {
  double v_over_c = (1024.0) * dt * dflx / (dx * (rhol + rhor));
  double tmp_min = (0.5 < v_over_c) ? 0.5 : v_over_c;
  return 0.5 + ((-0.5 > tmp_min) ? -0.5 : tmp_min);
}

/* ----------------------------------------------------------- Riemann solvers ---- */
/* Inputs wl/wr in rotated order (IDN, vn, vt1, vt2, IPR[, IBY, IBZ]); outputs flux in the
 * same rotated order (7 entries for MHD). */
static void rs_hllc(const double *wli, const double *wri, double gamma, double *flxi) {
  /* hydro/rsolvers/hydro/hllc.cpp:54-168 */
  double gm1 = gamma - 1.0, igm1 = 1.0 / gm1;
  double cl = sqrt(gamma * wli[IPR] / wli[IDN]);
  double cr = sqrt(gamma * wri[IPR] / wri[IDN]);
  double el = wli[IPR] * igm1 + 0.5 * wli[IDN] * (SQ(wli[IVX]) + SQ(wli[IVY]) + SQ(wli[IVZ]));
  double er = wri[IPR] * igm1 + 0.5 * wri[IDN] * (SQ(wri[IVX]) + SQ(wri[IVY]) + SQ(wri[IVZ]));
  double rhoa = .5 * (wli[IDN] + wri[IDN]);
  double ca = .5 * (cl + cr);
  double pmid = .5 * (wli[IPR] + wri[IPR] + (wli[IVX] - wri[IVX]) * rhoa * ca);
  double umid = .5 * (wli[IVX] + wri[IVX] + (wli[IPR] - wri[IPR]) / (rhoa * ca));
  double rhol = wli[IDN] + (wli[IVX] - umid) * rhoa / ca;
  double rhor = wri[IDN] + (umid - wri[IVX]) * rhoa / ca;
  (void)rhol; (void)rhor;
  double ql = (pmid <= wli[IPR]) ? 1.0
              : sqrt(1.0 + (gamma + 1) / (2 * gamma) * (pmid / wli[IPR] - 1.0));
  double qr = (pmid <= wri[IPR]) ? 1.0
              : sqrt(1.0 + (gamma + 1) / (2 * gamma) * (pmid / wri[IPR] - 1.0));
  double al = wli[IVX] - cl * ql;
  double ar = wri[IVX] + cr * qr;
  double bp = ar > 0.0 ? ar : (TINYN);
  double bm = al < 0.0 ? al : -(TINYN);
  double vxl = wli[IVX] - al;
  double vxr = wri[IVX] - ar;
  double tl = wli[IPR] + vxl * wli[IDN] * wli[IVX];
  double tr = wri[IPR] + vxr * wri[IDN] * wri[IVX];
  double ml = wli[IDN] * vxl;
  double mr = -(wri[IDN] * vxr);
  double am = (tl - tr) / (ml + mr);
  double cp = (ml * tr + mr * tl) / (ml + mr);
  cp = cp > 0.0 ? cp : 0.0;
  vxl = wli[IVX] - bm;
  vxr = wri[IVX] - bp;
  double fl[5], fr[5];
  fl[IDN] = wli[IDN] * vxl;
  fr[IDN] = wri[IDN] * vxr;
  fl[IVX] = wli[IDN] * wli[IVX] * vxl + wli[IPR];
  fr[IVX] = wri[IDN] * wri[IVX] * vxr + wri[IPR];
  fl[IVY] = wli[IDN] * wli[IVY] * vxl;
  fr[IVY] = wri[IDN] * wri[IVY] * vxr;
  fl[IVZ] = wli[IDN] * wli[IVZ] * vxl;
  fr[IVZ] = wri[IDN] * wri[IVZ] * vxr;
  fl[IEN] = el * vxl + wli[IPR] * wli[IVX];
  fr[IEN] = er * vxr + wri[IPR] * wri[IVX];
  double sl, sr, sm;
  if (am >= 0.0) {
    sl = am / (am - bm); sr = 0.0; sm = -bm / (am - bm);
  } else {
    sl = 0.0; sr = -am / (bp - am); sm = bp / (bp - am);
  }
  flxi[IDN] = sl * fl[IDN] + sr * fr[IDN];
  flxi[IVX] = sl * fl[IVX] + sr * fr[IVX] + sm * cp;
  flxi[IVY] = sl * fl[IVY] + sr * fr[IVY];
  flxi[IVZ] = sl * fl[IVZ] + sr * fr[IVZ];
  flxi[IEN] = sl * fl[IEN] + sr * fr[IEN] + sm * cp * am;
}

static void rs_hlle_hydro(const double *wli, const double *wri, double gamma, double *flxi) {
  /* hydro/rsolvers/hydro/hlle.cpp:64-151 (adiabatic branch) */
  double gm1 = gamma - 1.0, igm1 = 1.0 / gm1;
  double sqrtdl = sqrt(wli[IDN]), sqrtdr = sqrt(wri[IDN]);
  double isdlpdr = 1.0 / (sqrtdl + sqrtdr);
  double wroe[5];
  wroe[IDN] = sqrtdl * sqrtdr;
  wroe[IVX] = (sqrtdl * wli[IVX] + sqrtdr * wri[IVX]) * isdlpdr;
  wroe[IVY] = (sqrtdl * wli[IVY] + sqrtdr * wri[IVY]) * isdlpdr;
  wroe[IVZ] = (sqrtdl * wli[IVZ] + sqrtdr * wri[IVZ]) * isdlpdr;
  double el = wli[IPR] * igm1 + 0.5 * wli[IDN] * (SQ(wli[IVX]) + SQ(wli[IVY]) + SQ(wli[IVZ]));
  double er = wri[IPR] * igm1 + 0.5 * wri[IDN] * (SQ(wri[IVX]) + SQ(wri[IVY]) + SQ(wri[IVZ]));
  double hroe = ((el + wli[IPR]) / sqrtdl + (er + wri[IPR]) / sqrtdr) * isdlpdr;
  double cl = sqrt(gamma * wli[IPR] / wli[IDN]);
  double cr = sqrt(gamma * wri[IPR] / wri[IDN]);
  double q = hroe - 0.5 * (SQ(wroe[IVX]) + SQ(wroe[IVY]) + SQ(wroe[IVZ]));
  double a = (q < 0.0) ? 0.0 : sqrt(gm1 * q);
  double al = fmin_ref(wroe[IVX] - a, wli[IVX] - cl);
  double ar = fmax_ref(wroe[IVX] + a, wri[IVX] + cr);
  double bp = ar > 0.0 ? ar : 0.0;
  double bm = al < 0.0 ? al : 0.0;
  double vxl = wli[IVX] - bm, vxr = wri[IVX] - bp;
  double fl[5], fr[5];
  fl[IDN] = wli[IDN] * vxl; fr[IDN] = wri[IDN] * vxr;
  fl[IVX] = wli[IDN] * wli[IVX] * vxl; fr[IVX] = wri[IDN] * wri[IVX] * vxr;
  fl[IVY] = wli[IDN] * wli[IVY] * vxl; fr[IVY] = wri[IDN] * wri[IVY] * vxr;
  fl[IVZ] = wli[IDN] * wli[IVZ] * vxl; fr[IVZ] = wri[IDN] * wri[IVZ] * vxr;
  fl[IVX] += wli[IPR]; fr[IVX] += wri[IPR];
  fl[IEN] = el * vxl + wli[IPR] * wli[IVX];
  fr[IEN] = er * vxr + wri[IPR] * wri[IVX];
  double tmp = 0.0;
  if (bp != bm) tmp = 0.5 * (bp + bm) / (bp - bm);
  for (int n = 0; n < 5; ++n) flxi[n] = 0.5 * (fl[n] + fr[n]) + (fl[n] - fr[n]) * tmp;
}

static void rs_hlle_mhd(const double *wli, const double *wri, double bxi, double gamma,
                        double *flxi) {
  /* hydro/rsolvers/mhd/hlle_mhd.cpp:60-163 (adiabatic branch) */
  double gm1 = gamma - 1.0;
  double sqrtdl = sqrt(wli[IDN]), sqrtdr = sqrt(wri[IDN]);
  double isdlpdr = 1.0 / (sqrtdl + sqrtdr);
  double wroe[7];
  wroe[IDN] = sqrtdl * sqrtdr;
  wroe[IVX] = (sqrtdl * wli[IVX] + sqrtdr * wri[IVX]) * isdlpdr;
  wroe[IVY] = (sqrtdl * wli[IVY] + sqrtdr * wri[IVY]) * isdlpdr;
  wroe[IVZ] = (sqrtdl * wli[IVZ] + sqrtdr * wri[IVZ]) * isdlpdr;
  wroe[IBY] = (sqrtdr * wli[IBY] + sqrtdl * wri[IBY]) * isdlpdr;
  wroe[IBZ] = (sqrtdr * wli[IBZ] + sqrtdl * wri[IBZ]) * isdlpdr;
  double x = 0.5 * (SQ(wli[IBY] - wri[IBY]) + SQ(wli[IBZ] - wri[IBZ])) / (SQ(sqrtdl + sqrtdr));
  double y = 0.5 * (wli[IDN] + wri[IDN]) / wroe[IDN];
  double pbl = 0.5 * (bxi * bxi + SQ(wli[IBY]) + SQ(wli[IBZ]));
  double pbr = 0.5 * (bxi * bxi + SQ(wri[IBY]) + SQ(wri[IBZ]));
  double el = wli[IPR] / gm1 + 0.5 * wli[IDN] * (SQ(wli[IVX]) + SQ(wli[IVY]) + SQ(wli[IVZ])) + pbl;
  double er = wri[IPR] / gm1 + 0.5 * wri[IDN] * (SQ(wri[IVX]) + SQ(wri[IVY]) + SQ(wri[IVZ])) + pbr;
  double hroe = ((el + wli[IPR] + pbl) / sqrtdl + (er + wri[IPR] + pbr) / sqrtdr) * isdlpdr;
  double cl = fast_speed(wli, bxi, gamma);
  double cr = fast_speed(wri, bxi, gamma);
  double btsq = SQ(wroe[IBY]) + SQ(wroe[IBZ]);
  double vaxsq = bxi * bxi / wroe[IDN];
  double bt_starsq = (gm1 - (gm1 - 1.0) * y) * btsq;
  double hp = hroe - (vaxsq + btsq / wroe[IDN]);
  double vsq = SQ(wroe[IVX]) + SQ(wroe[IVY]) + SQ(wroe[IVZ]);
  double twid_asq = fmax_ref((gm1 * (hp - 0.5 * vsq) - (gm1 - 1.0) * x), 0.0);
  double ct2 = bt_starsq / wroe[IDN];
  double tsum = vaxsq + ct2 + twid_asq;
  double tdif = vaxsq + ct2 - twid_asq;
  double cf2_cs2 = sqrt(tdif * tdif + 4.0 * twid_asq * ct2);
  double cfsq = 0.5 * (tsum + cf2_cs2);
  double a = sqrt(cfsq);
  double al = fmin_ref((wroe[IVX] - a), (wli[IVX] - cl));
  double ar = fmax_ref((wroe[IVX] + a), (wri[IVX] + cr));
  double bp = ar > 0.0 ? ar : 0.0;
  double bm = al < 0.0 ? al : 0.0;
  double vxl = wli[IVX] - bm, vxr = wri[IVX] - bp;
  double fl[7], fr[7];
  fl[IDN] = wli[IDN] * vxl; fr[IDN] = wri[IDN] * vxr;
  fl[IVX] = wli[IDN] * wli[IVX] * vxl + pbl - SQ(bxi);
  fr[IVX] = wri[IDN] * wri[IVX] * vxr + pbr - SQ(bxi);
  fl[IVY] = wli[IDN] * wli[IVY] * vxl - bxi * wli[IBY];
  fr[IVY] = wri[IDN] * wri[IVY] * vxr - bxi * wri[IBY];
  fl[IVZ] = wli[IDN] * wli[IVZ] * vxl - bxi * wli[IBZ];
  fr[IVZ] = wri[IDN] * wri[IVZ] * vxr - bxi * wri[IBZ];
  fl[IVX] += wli[IPR]; fr[IVX] += wri[IPR];
  fl[IEN] = el * vxl + wli[IVX] * (wli[IPR] + pbl - bxi * bxi);
  fr[IEN] = er * vxr + wri[IVX] * (wri[IPR] + pbr - bxi * bxi);
  fl[IEN] -= bxi * (wli[IBY] * wli[IVY] + wli[IBZ] * wli[IVZ]);
  fr[IEN] -= bxi * (wri[IBY] * wri[IVY] + wri[IBZ] * wri[IVZ]);
  fl[IBY] = wli[IBY] * vxl - bxi * wli[IVY];
  fr[IBY] = wri[IBY] * vxr - bxi * wri[IVY];
  fl[IBZ] = wli[IBZ] * vxl - bxi * wli[IVZ];
  fr[IBZ] = wri[IBZ] * vxr - bxi * wri[IVZ];
  double tmp = 0.0;
  if (bp != bm) tmp = 0.5 * (bp + bm) / (bp - bm);
  for (int n = 0; n < 7; ++n) flxi[n] = 0.5 * (fl[n] + fr[n]) + (fl[n] - fr[n]) * tmp;
}

typedef struct { double d, mx, my, mz, e, by, bz; } cons1d;

static void rs_hlld(const double *wli, const double *wri, double bxi, double gamma,
                    double *flxi) {
  /* hydro/rsolvers/mhd/hlld.cpp:56-371 */
  double igm1 = 1.0 / (gamma - 1.0);
  cons1d ul, ur, ulst, uldst, urdst, urst, fl, fr;
  double spd[5];
  double bxsq = bxi * bxi;
  double pbl = 0.5 * (bxsq + (SQ(wli[IBY]) + SQ(wli[IBZ])));
  double pbr = 0.5 * (bxsq + (SQ(wri[IBY]) + SQ(wri[IBZ])));
  double kel = 0.5 * wli[IDN] * (SQ(wli[IVX]) + (SQ(wli[IVY]) + SQ(wli[IVZ])));
  double ker = 0.5 * wri[IDN] * (SQ(wri[IVX]) + (SQ(wri[IVY]) + SQ(wri[IVZ])));
  ul.d = wli[IDN]; ul.mx = wli[IVX] * ul.d; ul.my = wli[IVY] * ul.d; ul.mz = wli[IVZ] * ul.d;
  ul.e = wli[IPR] * igm1 + kel + pbl; ul.by = wli[IBY]; ul.bz = wli[IBZ];
  ur.d = wri[IDN]; ur.mx = wri[IVX] * ur.d; ur.my = wri[IVY] * ur.d; ur.mz = wri[IVZ] * ur.d;
  ur.e = wri[IPR] * igm1 + ker + pbr; ur.by = wri[IBY]; ur.bz = wri[IBZ];
  double cfl = fast_speed(wli, bxi, gamma);
  double cfr = fast_speed(wri, bxi, gamma);
  spd[0] = fmin_ref(wli[IVX] - cfl, wri[IVX] - cfr);
  spd[4] = fmax_ref(wli[IVX] + cfl, wri[IVX] + cfr);
  double ptl = wli[IPR] + pbl, ptr = wri[IPR] + pbr;
  fl.d = ul.mx;
  fl.mx = ul.mx * wli[IVX] + ptl - bxsq;
  fl.my = ul.my * wli[IVX] - bxi * ul.by;
  fl.mz = ul.mz * wli[IVX] - bxi * ul.bz;
  fl.e = wli[IVX] * (ul.e + ptl - bxsq) - bxi * (wli[IVY] * ul.by + wli[IVZ] * ul.bz);
  fl.by = ul.by * wli[IVX] - bxi * wli[IVY];
  fl.bz = ul.bz * wli[IVX] - bxi * wli[IVZ];
  fr.d = ur.mx;
  fr.mx = ur.mx * wri[IVX] + ptr - bxsq;
  fr.my = ur.my * wri[IVX] - bxi * ur.by;
  fr.mz = ur.mz * wri[IVX] - bxi * ur.bz;
  fr.e = wri[IVX] * (ur.e + ptr - bxsq) - bxi * (wri[IVY] * ur.by + wri[IVZ] * ur.bz);
  fr.by = ur.by * wri[IVX] - bxi * wri[IVY];
  fr.bz = ur.bz * wri[IVX] - bxi * wri[IVZ];
  double sdl = spd[0] - wli[IVX], sdr = spd[4] - wri[IVX];
  spd[2] = (sdr * ur.mx - sdl * ul.mx + (ptl - ptr)) / (sdr * ur.d - sdl * ul.d);
  double sdml = spd[0] - spd[2], sdmr = spd[4] - spd[2];
  double sdml_inv = 1.0 / sdml, sdmr_inv = 1.0 / sdmr;
  ulst.d = ul.d * sdl * sdml_inv;
  urst.d = ur.d * sdr * sdmr_inv;
  double ulst_d_inv = 1.0 / ulst.d, urst_d_inv = 1.0 / urst.d;
  double sqrtdl = sqrt(ulst.d), sqrtdr = sqrt(urst.d);
  spd[1] = spd[2] - fabs(bxi) / sqrtdl;
  spd[3] = spd[2] + fabs(bxi) / sqrtdr;
  double ptstl = ptl + ul.d * sdl * (spd[2] - wli[IVX]);
  double ptstr = ptr + ur.d * sdr * (spd[2] - wri[IVX]);
  double ptst = 0.5 * (ptstr + ptstl);
  ulst.mx = ulst.d * spd[2];
  if (fabs(ul.d * sdl * sdml - bxsq) < (SMALLN) * ptst) {
    ulst.my = ulst.d * wli[IVY]; ulst.mz = ulst.d * wli[IVZ];
    ulst.by = ul.by; ulst.bz = ul.bz;
  } else {
    double tmp = bxi * (sdl - sdml) / (ul.d * sdl * sdml - bxsq);
    ulst.my = ulst.d * (wli[IVY] - ul.by * tmp);
    ulst.mz = ulst.d * (wli[IVZ] - ul.bz * tmp);
    tmp = (ul.d * SQ(sdl) - bxsq) / (ul.d * sdl * sdml - bxsq);
    ulst.by = ul.by * tmp; ulst.bz = ul.bz * tmp;
  }
  double vbstl = (ulst.mx * bxi + (ulst.my * ulst.by + ulst.mz * ulst.bz)) * ulst_d_inv;
  ulst.e = (sdl * ul.e - ptl * wli[IVX] + ptst * spd[2] +
            bxi * (wli[IVX] * bxi + (wli[IVY] * ul.by + wli[IVZ] * ul.bz) - vbstl)) * sdml_inv;
  urst.mx = urst.d * spd[2];
  if (fabs(ur.d * sdr * sdmr - bxsq) < (SMALLN) * ptst) {
    urst.my = urst.d * wri[IVY]; urst.mz = urst.d * wri[IVZ];
    urst.by = ur.by; urst.bz = ur.bz;
  } else {
    double tmp = bxi * (sdr - sdmr) / (ur.d * sdr * sdmr - bxsq);
    urst.my = urst.d * (wri[IVY] - ur.by * tmp);
    urst.mz = urst.d * (wri[IVZ] - ur.bz * tmp);
    tmp = (ur.d * SQ(sdr) - bxsq) / (ur.d * sdr * sdmr - bxsq);
    urst.by = ur.by * tmp; urst.bz = ur.bz * tmp;
  }
  double vbstr = (urst.mx * bxi + (urst.my * urst.by + urst.mz * urst.bz)) * urst_d_inv;
  urst.e = (sdr * ur.e - ptr * wri[IVX] + ptst * spd[2] +
            bxi * (wri[IVX] * bxi + (wri[IVY] * ur.by + wri[IVZ] * ur.bz) - vbstr)) * sdmr_inv;
  if (0.5 * bxsq < (SMALLN) * ptst) {
    uldst = ulst; urdst = urst;
  } else {
    double invsumd = 1.0 / (sqrtdl + sqrtdr);
    double bxsig = (bxi > 0.0 ? 1.0 : -1.0);
    uldst.d = ulst.d; urdst.d = urst.d;
    uldst.mx = ulst.mx; urdst.mx = urst.mx;
    double tmp = invsumd * (sqrtdl * (ulst.my * ulst_d_inv) + sqrtdr * (urst.my * urst_d_inv) +
                            bxsig * (urst.by - ulst.by));
    uldst.my = uldst.d * tmp; urdst.my = urdst.d * tmp;
    tmp = invsumd * (sqrtdl * (ulst.mz * ulst_d_inv) + sqrtdr * (urst.mz * urst_d_inv) +
                     bxsig * (urst.bz - ulst.bz));
    uldst.mz = uldst.d * tmp; urdst.mz = urdst.d * tmp;
    tmp = invsumd * (sqrtdl * urst.by + sqrtdr * ulst.by +
                     bxsig * sqrtdl * sqrtdr * ((urst.my * urst_d_inv) - (ulst.my * ulst_d_inv)));
    uldst.by = urdst.by = tmp;
    tmp = invsumd * (sqrtdl * urst.bz + sqrtdr * ulst.bz +
                     bxsig * sqrtdl * sqrtdr * ((urst.mz * urst_d_inv) - (ulst.mz * ulst_d_inv)));
    uldst.bz = urdst.bz = tmp;
    tmp = spd[2] * bxi + (uldst.my * uldst.by + uldst.mz * uldst.bz) / uldst.d;
    uldst.e = ulst.e - sqrtdl * bxsig * (vbstl - tmp);
    urdst.e = urst.e + sqrtdr * bxsig * (vbstr - tmp);
  }
#define DIFFW(dst, a, b, sp) \
  dst.d = sp * (a.d - b.d); dst.mx = sp * (a.mx - b.mx); dst.my = sp * (a.my - b.my); \
  dst.mz = sp * (a.mz - b.mz); dst.e = sp * (a.e - b.e); dst.by = sp * (a.by - b.by); \
  dst.bz = sp * (a.bz - b.bz);
  cons1d t1, t0, t3, t4;
  DIFFW(t1, uldst, ulst, spd[1]);
  DIFFW(t0, ulst, ul, spd[0]);
  DIFFW(t3, urdst, urst, spd[3]);
  DIFFW(t4, urst, ur, spd[4]);
#undef DIFFW
  if (spd[0] >= 0.0) {
    flxi[IDN] = fl.d; flxi[IVX] = fl.mx; flxi[IVY] = fl.my; flxi[IVZ] = fl.mz;
    flxi[IEN] = fl.e; flxi[IBY] = fl.by; flxi[IBZ] = fl.bz;
  } else if (spd[4] <= 0.0) {
    flxi[IDN] = fr.d; flxi[IVX] = fr.mx; flxi[IVY] = fr.my; flxi[IVZ] = fr.mz;
    flxi[IEN] = fr.e; flxi[IBY] = fr.by; flxi[IBZ] = fr.bz;
  } else if (spd[1] >= 0.0) {
    flxi[IDN] = fl.d + t0.d; flxi[IVX] = fl.mx + t0.mx; flxi[IVY] = fl.my + t0.my;
    flxi[IVZ] = fl.mz + t0.mz; flxi[IEN] = fl.e + t0.e; flxi[IBY] = fl.by + t0.by;
    flxi[IBZ] = fl.bz + t0.bz;
  } else if (spd[2] >= 0.0) {
    flxi[IDN] = fl.d + t0.d + t1.d; flxi[IVX] = fl.mx + t0.mx + t1.mx;
    flxi[IVY] = fl.my + t0.my + t1.my; flxi[IVZ] = fl.mz + t0.mz + t1.mz;
    flxi[IEN] = fl.e + t0.e + t1.e; flxi[IBY] = fl.by + t0.by + t1.by;
    flxi[IBZ] = fl.bz + t0.bz + t1.bz;
  } else if (spd[3] > 0.0) {
    flxi[IDN] = fr.d + t4.d + t3.d; flxi[IVX] = fr.mx + t4.mx + t3.mx;
    flxi[IVY] = fr.my + t4.my + t3.my; flxi[IVZ] = fr.mz + t4.mz + t3.mz;
    flxi[IEN] = fr.e + t4.e + t3.e; flxi[IBY] = fr.by + t4.by + t3.by;
    flxi[IBZ] = fr.bz + t4.bz + t3.bz;
  } else {
    flxi[IDN] = fr.d + t4.d; flxi[IVX] = fr.mx + t4.mx; flxi[IVY] = fr.my + t4.my;
    flxi[IVZ] = fr.mz + t4.mz; flxi[IEN] = fr.e + t4.e; flxi[IBY] = fr.by + t4.by;
    flxi[IBZ] = fr.bz + t4.bz;
  }
}

/* LHLLC, the fork's low-dissipation HLLC (hydro/rsolvers/hydro/lhllc.cpp:26-180): PVRS
 * wave speeds, a shock detector th = min(1, (cmax - min(dvn,0)) / (cmax - min(dvt,0)))^4
 * weighting the pressure jump in the contact speed, and a low-Mach factor phi on the
 * contact pressure */
static void rs_lhllc(const double *wli, const double *wri, double gamma, double dvn,
                     double dvt, double *flxi) {
  double gm1 = gamma - 1.0, igm1 = 1.0 / gm1;
  double fl[5], fr[5];
  double cl = sqrt(gamma * wli[IPR] / wli[IDN]);
  double cr = sqrt(gamma * wri[IPR] / wri[IDN]);
  double vsql = SQ(wli[IVX]) + SQ(wli[IVY]) + SQ(wli[IVZ]);
  double vsqr = SQ(wri[IVX]) + SQ(wri[IVY]) + SQ(wri[IVZ]);
  double el = wli[IPR] * igm1 + 0.5 * wli[IDN] * vsql;
  double er = wri[IPR] * igm1 + 0.5 * wri[IDN] * vsqr;
  double rhoa = .5 * (wli[IDN] + wri[IDN]);
  double ca = .5 * (cl + cr);
  double pmid = .5 * (wli[IPR] + wri[IPR] + (wli[IVX] - wri[IVX]) * rhoa * ca);
  double umid = .5 * (wli[IVX] + wri[IVX] + (wli[IPR] - wri[IPR]) / (rhoa * ca));
  double rhol = wli[IDN] + (wli[IVX] - umid) * rhoa / ca;
  double rhor = wri[IDN] + (umid - wri[IVX]) * rhoa / ca;
  (void)rhol; (void)rhor;
  double ql = (pmid <= wli[IPR]) ? 1.0
              : sqrt(1.0 + (gamma + 1) / (2 * gamma) * (pmid / wli[IPR] - 1.0));
  double qr = (pmid <= wri[IPR]) ? 1.0
              : sqrt(1.0 + (gamma + 1) / (2 * gamma) * (pmid / wri[IPR] - 1.0));
  double al = wli[IVX] - cl * ql;
  double ar = wri[IVX] + cr * qr;
  double bp = ar > 0.0 ? ar : (TINYN);
  double bm = al < 0.0 ? al : -(TINYN);
  double vxl = al - wli[IVX], vxr = ar - wri[IVX];
  double ml = wli[IDN] * vxl, mr = wri[IDN] * vxr;
  double cmax = fmax_ref(cl, cr);
  double th1 = fmin_ref(1.0, (cmax - fmin_ref(dvn, 0.0)) / (cmax - fmin_ref(dvt, 0.0)));
  double th = th1 * th1 * th1 * th1;
  double am = (mr * wri[IVX] - ml * wli[IVX] - th * (wri[IPR] - wli[IPR])) / (mr - ml);
  double chi = fmin_ref(1.0, sqrt(fmax_ref(vsql, vsqr)) / cmax);
  double phi = chi * (2.0 - chi);
  double cp = (mr * wli[IPR] - ml * wri[IPR] + phi * mr * ml * (wri[IVX] - wli[IVX])) / (mr - ml);
  cp = cp > 0.0 ? cp : 0.0;
  double uxl = wli[IVX] - bm, uxr = wri[IVX] - bp;
  fl[IDN] = wli[IDN] * uxl; fr[IDN] = wri[IDN] * uxr;
  fl[IVX] = wli[IDN] * wli[IVX] * uxl + wli[IPR]; fr[IVX] = wri[IDN] * wri[IVX] * uxr + wri[IPR];
  fl[IVY] = wli[IDN] * wli[IVY] * uxl; fr[IVY] = wri[IDN] * wri[IVY] * uxr;
  fl[IVZ] = wli[IDN] * wli[IVZ] * uxl; fr[IVZ] = wri[IDN] * wri[IVZ] * uxr;
  fl[IEN] = el * uxl + wli[IPR] * wli[IVX]; fr[IEN] = er * uxr + wri[IPR] * wri[IVX];
  double sl, sr, sm;
  if (am >= 0.0) { sl = am / (am - bm); sr = 0.0; sm = -bm / (am - bm); }
  else { sl = 0.0; sr = -am / (bp - am); sm = bp / (bp - am); }
  flxi[IDN] = sl * fl[IDN] + sr * fr[IDN];
  flxi[IVX] = sl * fl[IVX] + sr * fr[IVX] + sm * cp;
  flxi[IVY] = sl * fl[IVY] + sr * fr[IVY];
  flxi[IVZ] = sl * fl[IVZ] + sr * fr[IVZ];
  flxi[IEN] = sl * fl[IEN] + sr * fr[IEN] + sm * cp * am;
}

/* LHLLD, the fork's low-dissipation HLLD (hydro/rsolvers/mhd/lhlld.cpp:36-388): HLLD with
 * the shock detector on the pressure jump of S_M and the low-Mach factor phi in the
 * star-state total pressure */
static void rs_lhlld(const double *wli, const double *wri, double bxi, double gamma,
                     double dvn, double dvt, double *flxi) {
  double igm1 = 1.0 / (gamma - 1.0);
  cons1d ul, ur, ulst, uldst, urdst, urst, fl, fr;
  double spd[5];
  double bxsq = bxi * bxi;
  double pbl = 0.5 * (bxsq + (SQ(wli[IBY]) + SQ(wli[IBZ])));
  double pbr = 0.5 * (bxsq + (SQ(wri[IBY]) + SQ(wri[IBZ])));
  double kel = 0.5 * wli[IDN] * (SQ(wli[IVX]) + (SQ(wli[IVY]) + SQ(wli[IVZ])));
  double ker = 0.5 * wri[IDN] * (SQ(wri[IVX]) + (SQ(wri[IVY]) + SQ(wri[IVZ])));
  ul.d = wli[IDN]; ul.mx = wli[IVX] * ul.d; ul.my = wli[IVY] * ul.d; ul.mz = wli[IVZ] * ul.d;
  ul.e = wli[IPR] * igm1 + kel + pbl; ul.by = wli[IBY]; ul.bz = wli[IBZ];
  ur.d = wri[IDN]; ur.mx = wri[IVX] * ur.d; ur.my = wri[IVY] * ur.d; ur.mz = wri[IVZ] * ur.d;
  ur.e = wri[IPR] * igm1 + ker + pbr; ur.by = wri[IBY]; ur.bz = wri[IBZ];
  double cfl = fast_speed(wli, bxi, gamma);
  double cfr = fast_speed(wri, bxi, gamma);
  spd[0] = fmin_ref(wli[IVX] - cfl, wri[IVX] - cfr);
  spd[4] = fmax_ref(wli[IVX] + cfl, wri[IVX] + cfr);
  double cfmax = fmax_ref(cfl, cfr);
  double ptl = wli[IPR] + pbl, ptr = wri[IPR] + pbr;
  fl.d = ul.mx;
  fl.mx = ul.mx * wli[IVX] + ptl - bxsq;
  fl.my = ul.my * wli[IVX] - bxi * ul.by;
  fl.mz = ul.mz * wli[IVX] - bxi * ul.bz;
  fl.e = wli[IVX] * (ul.e + ptl - bxsq) - bxi * (wli[IVY] * ul.by + wli[IVZ] * ul.bz);
  fl.by = ul.by * wli[IVX] - bxi * wli[IVY];
  fl.bz = ul.bz * wli[IVX] - bxi * wli[IVZ];
  fr.d = ur.mx;
  fr.mx = ur.mx * wri[IVX] + ptr - bxsq;
  fr.my = ur.my * wri[IVX] - bxi * ur.by;
  fr.mz = ur.mz * wri[IVX] - bxi * ur.bz;
  fr.e = wri[IVX] * (ur.e + ptr - bxsq) - bxi * (wri[IVY] * ur.by + wri[IVZ] * ur.bz);
  fr.by = ur.by * wri[IVX] - bxi * wri[IVY];
  fr.bz = ur.bz * wri[IVX] - bxi * wri[IVZ];
  double sdl = spd[0] - wli[IVX], sdr = spd[4] - wri[IVX];
  double sdld = sdl * ul.d, sdrd = sdr * ur.d;
  double th1 = fmin_ref(1.0, (cfmax - fmin_ref(dvn, 0.0)) / (cfmax - fmin_ref(dvt, 0.0)));
  double th = th1 * th1 * th1 * th1;
  spd[2] = (sdr * ur.mx - sdl * ul.mx + th * (ptl - ptr)) / (sdrd - sdld);
  double sdml = spd[0] - spd[2], sdmr = spd[4] - spd[2];
  double sdml_inv = 1.0 / sdml, sdmr_inv = 1.0 / sdmr;
  ulst.d = sdld * sdml_inv;
  urst.d = sdrd * sdmr_inv;
  double ulst_d_inv = 1.0 / ulst.d, urst_d_inv = 1.0 / urst.d;
  double sqrtdl = sqrt(ulst.d), sqrtdr = sqrt(urst.d);
  spd[1] = spd[2] - fabs(bxi) / sqrtdl;
  spd[3] = spd[2] + fabs(bxi) / sqrtdr;
  double clsq = ((pbl + kel) + sqrt(SQ(pbl + kel) - 2.0 * kel * bxsq)) / ul.d;
  double crsq = ((pbr + ker) + sqrt(SQ(pbr + ker) - 2.0 * ker * bxsq)) / ur.d;
  double chi = fmin_ref(1.0, sqrt(fmax_ref(clsq, crsq)) / cfmax);
  double phi = chi * (2.0 - chi);
  double ptst = (sdrd * ptl - sdld * ptr + phi * sdrd * sdld * (wri[IVX] - wli[IVX])) /
                (sdrd - sdld);
  ulst.mx = ulst.d * spd[2];
  if (fabs(sdld * sdml - bxsq) < (SMALLN) * ptst) {
    ulst.my = ulst.d * wli[IVY]; ulst.mz = ulst.d * wli[IVZ];
    ulst.by = ul.by; ulst.bz = ul.bz;
  } else {
    double tmp = bxi * (sdl - sdml) / (sdld * sdml - bxsq);
    ulst.my = ulst.d * (wli[IVY] - ul.by * tmp);
    ulst.mz = ulst.d * (wli[IVZ] - ul.bz * tmp);
    tmp = (sdld * sdl - bxsq) / (sdld * sdml - bxsq);
    ulst.by = ul.by * tmp; ulst.bz = ul.bz * tmp;
  }
  double vbstl = (ulst.mx * bxi + (ulst.my * ulst.by + ulst.mz * ulst.bz)) * ulst_d_inv;
  ulst.e = (sdl * ul.e - ptl * wli[IVX] + ptst * spd[2] +
            bxi * (wli[IVX] * bxi + (wli[IVY] * ul.by + wli[IVZ] * ul.bz) - vbstl)) * sdml_inv;
  urst.mx = urst.d * spd[2];
  if (fabs(sdrd * sdmr - bxsq) < (SMALLN) * ptst) {
    urst.my = urst.d * wri[IVY]; urst.mz = urst.d * wri[IVZ];
    urst.by = ur.by; urst.bz = ur.bz;
  } else {
    double tmp = bxi * (sdr - sdmr) / (sdrd * sdmr - bxsq);
    urst.my = urst.d * (wri[IVY] - ur.by * tmp);
    urst.mz = urst.d * (wri[IVZ] - ur.bz * tmp);
    tmp = (sdrd * sdr - bxsq) / (sdrd * sdmr - bxsq);
    urst.by = ur.by * tmp; urst.bz = ur.bz * tmp;
  }
  double vbstr = (urst.mx * bxi + (urst.my * urst.by + urst.mz * urst.bz)) * urst_d_inv;
  urst.e = (sdr * ur.e - ptr * wri[IVX] + ptst * spd[2] +
            bxi * (wri[IVX] * bxi + (wri[IVY] * ur.by + wri[IVZ] * ur.bz) - vbstr)) * sdmr_inv;
  if (0.5 * bxsq < (SMALLN) * ptst) {
    uldst = ulst; urdst = urst;
  } else {
    double invsumd = 1.0 / (sqrtdl + sqrtdr);
    double bxsig = (bxi > 0.0 ? 1.0 : -1.0);
    uldst.d = ulst.d; urdst.d = urst.d;
    uldst.mx = ulst.mx; urdst.mx = urst.mx;
    double tmp = invsumd * (sqrtdl * (ulst.my * ulst_d_inv) + sqrtdr * (urst.my * urst_d_inv) +
                            bxsig * (urst.by - ulst.by));
    uldst.my = uldst.d * tmp; urdst.my = urdst.d * tmp;
    tmp = invsumd * (sqrtdl * (ulst.mz * ulst_d_inv) + sqrtdr * (urst.mz * urst_d_inv) +
                     bxsig * (urst.bz - ulst.bz));
    uldst.mz = uldst.d * tmp; urdst.mz = urdst.d * tmp;
    tmp = invsumd * (sqrtdl * urst.by + sqrtdr * ulst.by +
                     bxsig * sqrtdl * sqrtdr * ((urst.my * urst_d_inv) - (ulst.my * ulst_d_inv)));
    uldst.by = urdst.by = tmp;
    tmp = invsumd * (sqrtdl * urst.bz + sqrtdr * ulst.bz +
                     bxsig * sqrtdl * sqrtdr * ((urst.mz * urst_d_inv) - (ulst.mz * ulst_d_inv)));
    uldst.bz = urdst.bz = tmp;
    tmp = spd[2] * bxi + (uldst.my * uldst.by + uldst.mz * uldst.bz) / uldst.d;
    uldst.e = ulst.e - sqrtdl * bxsig * (vbstl - tmp);
    urdst.e = urst.e + sqrtdr * bxsig * (vbstr - tmp);
  }
#define DIFFW(dst, a, b, sp) \
  dst.d = sp * (a.d - b.d); dst.mx = sp * (a.mx - b.mx); dst.my = sp * (a.my - b.my); \
  dst.mz = sp * (a.mz - b.mz); dst.e = sp * (a.e - b.e); dst.by = sp * (a.by - b.by); \
  dst.bz = sp * (a.bz - b.bz);
  cons1d t1, t0, t3, t4;
  DIFFW(t1, uldst, ulst, spd[1]);
  DIFFW(t0, ulst, ul, spd[0]);
  DIFFW(t3, urdst, urst, spd[3]);
  DIFFW(t4, urst, ur, spd[4]);
#undef DIFFW
  if (spd[0] >= 0.0) {
    flxi[IDN] = fl.d; flxi[IVX] = fl.mx; flxi[IVY] = fl.my; flxi[IVZ] = fl.mz;
    flxi[IEN] = fl.e; flxi[IBY] = fl.by; flxi[IBZ] = fl.bz;
  } else if (spd[4] <= 0.0) {
    flxi[IDN] = fr.d; flxi[IVX] = fr.mx; flxi[IVY] = fr.my; flxi[IVZ] = fr.mz;
    flxi[IEN] = fr.e; flxi[IBY] = fr.by; flxi[IBZ] = fr.bz;
  } else if (spd[1] >= 0.0) {
    flxi[IDN] = fl.d + t0.d; flxi[IVX] = fl.mx + t0.mx; flxi[IVY] = fl.my + t0.my;
    flxi[IVZ] = fl.mz + t0.mz; flxi[IEN] = fl.e + t0.e; flxi[IBY] = fl.by + t0.by;
    flxi[IBZ] = fl.bz + t0.bz;
  } else if (spd[2] >= 0.0) {
    flxi[IDN] = fl.d + t0.d + t1.d; flxi[IVX] = fl.mx + t0.mx + t1.mx;
    flxi[IVY] = fl.my + t0.my + t1.my; flxi[IVZ] = fl.mz + t0.mz + t1.mz;
    flxi[IEN] = fl.e + t0.e + t1.e; flxi[IBY] = fl.by + t0.by + t1.by;
    flxi[IBZ] = fl.bz + t0.bz + t1.bz;
  } else if (spd[3] > 0.0) {
    flxi[IDN] = fr.d + t4.d + t3.d; flxi[IVX] = fr.mx + t4.mx + t3.mx;
    flxi[IVY] = fr.my + t4.my + t3.my; flxi[IVZ] = fr.mz + t4.mz + t3.mz;
    flxi[IEN] = fr.e + t4.e + t3.e; flxi[IBY] = fr.by + t4.by + t3.by;
    flxi[IBZ] = fr.bz + t4.bz + t3.bz;
  } else {
    flxi[IDN] = fr.d + t4.d; flxi[IVX] = fr.mx + t4.mx; flxi[IVY] = fr.my + t4.my;
    flxi[IVZ] = fr.mz + t4.mz; flxi[IEN] = fr.e + t4.e; flxi[IBY] = fr.by + t4.by;
    flxi[IBZ] = fr.bz + t4.bz;
  }
}

/* Hydro::CalculateVelocityDifferences (hydro/calculate_velocity_differences.cpp:20-52,
 * 3-D): normal velocity jump across the face and the smallest transverse velocity
 * difference around it (the LHLLC/LHLLD shock detector) */
static void velocity_differences(const orc_sim *s, int dir, int k, int j, int i, double *dvn,
                                 double *dvt) {
  const size_t nc = s->ncell;
  const double *vx = s->w + (size_t)IVX * nc, *vy = s->w + (size_t)IVY * nc,
               *vz = s->w + (size_t)IVZ * nc;
#define W(a, kk, jj, ii) (a)[C3(s, kk, jj, ii)]
  double dvl, dvr, dwl, dwr;
  if (dir == 0) {
    *dvn = W(vx, k, j, i) - W(vx, k, j, i - 1);
    dvl = fmin_ref(W(vy, k, j + 1, i - 1) - W(vy, k, j, i - 1), W(vy, k, j, i - 1) - W(vy, k, j - 1, i - 1));
    dvr = fmin_ref(W(vy, k, j + 1, i) - W(vy, k, j, i), W(vy, k, j, i) - W(vy, k, j - 1, i));
    dwl = fmin_ref(W(vz, k + 1, j, i - 1) - W(vz, k, j, i - 1), W(vz, k, j, i - 1) - W(vz, k - 1, j, i - 1));
    dwr = fmin_ref(W(vz, k + 1, j, i) - W(vz, k, j, i), W(vz, k, j, i) - W(vz, k - 1, j, i));
  } else if (dir == 1) {
    *dvn = W(vy, k, j, i) - W(vy, k, j - 1, i);
    dvl = fmin_ref(W(vz, k + 1, j - 1, i) - W(vz, k, j - 1, i), W(vz, k, j - 1, i) - W(vz, k - 1, j - 1, i));
    dvr = fmin_ref(W(vz, k + 1, j, i) - W(vz, k, j, i), W(vz, k, j, i) - W(vz, k - 1, j, i));
    dwl = fmin_ref(W(vx, k, j - 1, i + 1) - W(vx, k, j - 1, i), W(vx, k, j - 1, i) - W(vx, k, j - 1, i - 1));
    dwr = fmin_ref(W(vx, k, j, i + 1) - W(vx, k, j, i), W(vx, k, j, i) - W(vx, k, j, i - 1));
  } else {
    *dvn = W(vz, k, j, i) - W(vz, k - 1, j, i);
    dvl = fmin_ref(W(vx, k - 1, j, i + 1) - W(vx, k - 1, j, i), W(vx, k - 1, j, i) - W(vx, k - 1, j, i - 1));
    dvr = fmin_ref(W(vx, k, j, i + 1) - W(vx, k, j, i), W(vx, k, j, i) - W(vx, k, j, i - 1));
    dwl = fmin_ref(W(vy, k - 1, j + 1, i) - W(vy, k - 1, j, i), W(vy, k - 1, j, i) - W(vy, k - 1, j - 1, i));
    dwr = fmin_ref(W(vy, k, j + 1, i) - W(vy, k, j, i), W(vy, k, j, i) - W(vy, k, j - 1, i));
  }
#undef W
  *dvt = fmin_ref(fmin_ref(dvl, dvr), fmin_ref(dwl, dwr));
}

/* ----------------------------------------------------------- reconstruction ---- */
/* value of wave variable n of cell (k,j,i) for a sweep along dir; MHD transverse
 * components come from bcc in the cyclic order of reconstruct/plm.cpp:44-55,156-170,268-282 */
static inline double wave_var(const orc_sim *s, int dir, int n, int k, int j, int i) {
  size_t c = C3(s, k, j, i);
  if (n < NHYD) return s->w[(size_t)n * s->ncell + c];
  static const int by_of[3] = {1, 2, 0}, bz_of[3] = {2, 0, 1};
  int comp = (n == IBY) ? by_of[dir] : bz_of[dir];
  return s->bcc[(size_t)comp * s->ncell + c];
}

/* PPM of one cell on a uniform Cartesian axis (reconstruct/ppm.cpp:44-342 with the
 * uniform weights of reconstruct/reconstruction.cpp:420-431): from the five values
 * q[-2..2] returns qminus (state at the lower face) and qplus (upper face). */
static inline double sgn(double x) { return (x < 0.0) ? -1.0 : 1.0; }
static void ppm_cell(double q_im2, double q_im1, double q, double q_ip1, double q_ip2,
                     double *qminus_out, double *qplus_out) {
  const double C2 = 1.25;
  const double c1 = 0.5, c2 = 0.5, c3 = 0.5, c4 = 0.5, c5 = 1.0 / 6.0, c6 = -1.0 / 6.0;
  double qa = (q - q_im1);
  double qb = (q_ip1 - q);
  double dd_im1 = c1 * qa + c2 * (q_im1 - q_im2);
  double dd = c1 * qb + c2 * qa;
  double dd_ip1 = c1 * (q_ip2 - q_ip1) + c2 * qb;
  double dph = (c3 * q_im1 + c4 * q) + (c5 * dd_im1 + c6 * dd);
  double dph_ip1 = (c3 * q + c4 * q_ip1) + (c5 * dd + c6 * dd_ip1);
  double d2qc_im1 = q_im2 + q - 2.0 * q_im1;
  double d2qc = q_im1 + q_ip1 - 2.0 * q;
  double d2qc_ip1 = q + q_ip2 - 2.0 * q_ip1;
  {
    double qa_tmp = dph - q_im1, qb_tmp = q - dph;
    double a = 3.0 * (q_im1 + q - 2.0 * dph), b = d2qc_im1, c = d2qc;
    double qd = 0.0;
    if (sgn(a) == sgn(b) && sgn(a) == sgn(c))
      qd = sgn(a) * fmin_ref(C2 * fabs(b), fmin_ref(C2 * fabs(c), fabs(a)));
    double dph_tmp = 0.5 * (q_im1 + q) - qd / 6.0;
    if (qa_tmp * qb_tmp < 0.0) dph = dph_tmp;
  }
  {
    double qa_tmp = dph_ip1 - q, qb_tmp = q_ip1 - dph_ip1;
    double a = 3.0 * (q + q_ip1 - 2.0 * dph_ip1), b = d2qc, c = d2qc_ip1;
    double qd = 0.0;
    if (sgn(a) == sgn(b) && sgn(a) == sgn(c))
      qd = sgn(a) * fmin_ref(C2 * fabs(b), fmin_ref(C2 * fabs(c), fabs(a)));
    double dphip1_tmp = 0.5 * (q + q_ip1) - qd / 6.0;
    if (qa_tmp * qb_tmp < 0.0) dph_ip1 = dphip1_tmp;
  }
  double d2qf = 6.0 * (dph + dph_ip1 - 2.0 * q);
  double qminus = dph, qplus = dph_ip1;
  double dqf_minus = q - qminus, dqf_plus = qplus - q;
  double qa_tmp = dqf_minus * dqf_plus;
  double qb_tmp = (q_ip1 - q) * (q - q_im1);
  double a = d2qc_im1, b = d2qc, c = d2qc_ip1, d = d2qf, qe = 0.0;
  if (sgn(a) == sgn(b) && sgn(a) == sgn(c) && sgn(a) == sgn(d))
    qe = sgn(d) * fmin_ref(fmin_ref(C2 * fabs(a), C2 * fabs(b)), fmin_ref(C2 * fabs(c), fabs(d)));
  a = fmax_ref(fabs(q_im1), fabs(q_im2));
  b = fmax_ref(fmax_ref(fabs(q), fabs(q_ip1)), fabs(q_ip2));
  double rho = 0.0;
  if (fabs(d) > (1.0e-12) * fmax_ref(a, b)) rho = qe / d;
  double tmp_m = q - rho * dqf_minus, tmp_p = q + rho * dqf_plus;
  double tmp2_m = q - 2.0 * dqf_plus, tmp2_p = q + 2.0 * dqf_minus;
  if ((qa_tmp <= 0.0 || qb_tmp <= 0.0)) {
    if (rho <= (1.0 - (1.0e-12))) {
      qminus = tmp_m;
      qplus = tmp_p;
    }
  } else {
    if (fabs(dqf_minus) >= 2.0 * fabs(dqf_plus)) qminus = tmp2_m;
    if (fabs(dqf_plus) >= 2.0 * fabs(dqf_minus)) qplus = tmp2_p;
  }
  *qminus_out = qminus;
  *qplus_out = qplus;
}

/* left/right states at the face with face index (k,j,i) in direction dir
 * (face between the cell at index-1 and the cell at index along dir). */
static void recon_face(const orc_sim *s, int dir, int order, int k, int j, int i,
                       double *wl, double *wr) {
  int nw = s->p.mhd ? 7 : 5;
  int dk = dir == 2, dj = dir == 1, di = dir == 0;
  if (order == 1) {  /* reconstruct/dc.cpp:24-110 */
    for (int n = 0; n < nw; ++n) {
      wl[n] = wave_var(s, dir, n, k - dk, j - dj, i - di);
      wr[n] = wave_var(s, dir, n, k, j, i);
    }
    return;
  }
  if (order == 3) { /* PPM: wl from cell f-1 (qplus), wr from cell f (qminus), then floors */
    for (int n = 0; n < nw; ++n) {
      double v[6];
      for (int q = 0; q < 6; ++q)
        v[q] = wave_var(s, dir, n, k + (q - 3) * dk, j + (q - 3) * dj, i + (q - 3) * di);
      double qm, qp, dummy;
      ppm_cell(v[0], v[1], v[2], v[3], v[4], &dummy, &qp);
      ppm_cell(v[1], v[2], v[3], v[4], v[5], &qm, &dummy);
      wl[n] = qp;
      wr[n] = qm;
    }
    /* eos ApplyPrimitiveFloors (ppm.cpp:326-332) */
    wl[IDN] = (wl[IDN] > s->p.dfloor) ? wl[IDN] : s->p.dfloor;
    wl[IPR] = (wl[IPR] > s->p.pfloor) ? wl[IPR] : s->p.pfloor;
    wr[IDN] = (wr[IDN] > s->p.dfloor) ? wr[IDN] : s->p.dfloor;
    wr[IPR] = (wr[IPR] > s->p.pfloor) ? wr[IPR] : s->p.pfloor;
    return;
  }
  /* reconstruct/plm.cpp uniform VL branch: cell c gives wl(c+1) and wr(c) */
  const double *xf = dir == 0 ? s->x1f : (dir == 1 ? s->x2f : s->x3f);
  const double *xv = dir == 0 ? s->x1v : (dir == 1 ? s->x2v : s->x3v);
  double dxf = dir == 0 ? s->dx1 : (dir == 1 ? s->dx2 : s->dx3);
  int f = dir == 0 ? i : (dir == 1 ? j : k);
  int cL = f - 1, cR = f;
  double cpL = (xf[cL + 1] - xv[cL]) / dxf; /* coefficient of wl(cL+1) */
  double cmR = (xv[cR] - xf[cR]) / dxf;     /* coefficient of wr(cR) */
  for (int n = 0; n < nw; ++n) {
    double a0 = wave_var(s, dir, n, k - 2 * dk, j - 2 * dj, i - 2 * di);
    double a1 = wave_var(s, dir, n, k - dk, j - dj, i - di);
    double a2 = wave_var(s, dir, n, k, j, i);
    double a3 = wave_var(s, dir, n, k + dk, j + dj, i + di);
    /* left cell (index f-1): neighbours a0, a1, a2 */
    double dwl = (a1 - a0), dwr = (a2 - a1);
    double dw2 = dwl * dwr;
    double dwm = 2.0 * dw2 / (dwl + dwr);
    if (dw2 <= 0.0) dwm = 0.0;
    wl[n] = a1 + cpL * dwm;
    /* right cell (index f): neighbours a1, a2, a3 */
    dwl = (a2 - a1); dwr = (a3 - a2);
    dw2 = dwl * dwr;
    dwm = 2.0 * dw2 / (dwl + dwr);
    if (dw2 <= 0.0) dwm = 0.0;
    wr[n] = a2 - cmR * dwm;
  }
}

/* ------------------------------------------------------------ flux sweeps ---- */
static void sweep(orc_sim *s, int dir, int order) {
  const int mhd = s->p.mhd;
  int kl = s->ks, ku = s->ke, jl = s->js, ju = s->je, il = s->is, iu = s->ie;
  /* loop extents: hydro/calculate_fluxes.cpp:63-74, 164-172, 274-279 */
  if (dir == 0) {
    iu = s->ie + 1;
    if (mhd) { jl = s->js - 1; ju = s->je + 1; kl = s->ks - 1; ku = s->ke + 1; }
  } else if (dir == 1) {
    ju = s->je + 1; il = s->is - 1; iu = s->ie + 1;
    if (mhd) { kl = s->ks - 1; ku = s->ke + 1; }
  } else {
    ku = s->ke + 1;
    if (mhd) { il = s->is - 1; iu = s->ie + 1; jl = s->js - 1; ju = s->je + 1; }
  }
  const int ivx = IVX + dir, ivy = IVX + ((dir) + 1) % 3, ivz = IVX + ((dir) + 2) % 3;
  const double dxw = dir == 0 ? s->dx1 : (dir == 1 ? s->dx2 : s->dx3);
  double *flx = dir == 0 ? s->f1 : (dir == 1 ? s->f2 : s->f3);
  const size_t fn = dir == 0 ? f1n(s) : (dir == 1 ? f2n(s) : f3n(s));
  const double *bn = dir == 0 ? s->b1 : (dir == 1 ? s->b2 : s->b3);
  double *ey = dir == 0 ? s->e3x1 : (dir == 1 ? s->e1x2 : s->e2x3);
  double *ez = dir == 0 ? s->e2x1 : (dir == 1 ? s->e3x2 : s->e1x3);
  double *wct = dir == 0 ? s->wx1 : (dir == 1 ? s->wx2 : s->wx3);
#pragma omp parallel for collapse(2)
  for (int k = kl; k <= ku; ++k)
    for (int j = jl; j <= ju; ++j)
      for (int i = il; i <= iu; ++i) {
        double wl[7], wr[7], wli[7], wri[7], fx[7];
        recon_face(s, dir, order, k, j, i, wl, wr);
        wli[IDN] = wl[IDN]; wli[IVX] = wl[ivx]; wli[IVY] = wl[ivy]; wli[IVZ] = wl[ivz];
        wli[IPR] = wl[IPR];
        wri[IDN] = wr[IDN]; wri[IVX] = wr[ivx]; wri[IVY] = wr[ivy]; wri[IVZ] = wr[ivz];
        wri[IPR] = wr[IPR];
        size_t fi = dir == 0 ? F1I(s, k, j, i) : (dir == 1 ? F2I(s, k, j, i) : F3I(s, k, j, i));
        if (mhd) {
          wli[IBY] = wl[IBY]; wli[IBZ] = wl[IBZ];
          wri[IBY] = wr[IBY]; wri[IBZ] = wr[IBZ];
          double bx = bn[fi];
          if (s->p.rsolver == ORC_HLLD) {
            rs_hlld(wli, wri, bx, s->p.gamma, fx);
          } else if (s->p.rsolver == ORC_LHLLD) {
            double dvn, dvt;
            velocity_differences(s, dir, k, j, i, &dvn, &dvt);
            rs_lhlld(wli, wri, bx, s->p.gamma, dvn, dvt, fx);
          } else {
            rs_hlle_mhd(wli, wri, bx, s->p.gamma, fx);
          }
          ey[fi] = -fx[IBY];
          ez[fi] = fx[IBZ];
          wct[fi] = ct_weight(fx[IDN], wli[IDN], wri[IDN], dxw, s->dt);
        } else {
          if (s->p.rsolver == ORC_HLLC) {
            rs_hllc(wli, wri, s->p.gamma, fx);
          } else if (s->p.rsolver == ORC_LHLLC) {
            double dvn, dvt;
            velocity_differences(s, dir, k, j, i, &dvn, &dvt);
            rs_lhllc(wli, wri, s->p.gamma, dvn, dvt, fx);
          } else {
            rs_hlle_hydro(wli, wri, s->p.gamma, fx);
          }
        }
        flx[IDN * fn + fi] = fx[IDN];
        flx[ivx * fn + fi] = fx[IVX];
        flx[ivy * fn + fi] = fx[IVY];
        flx[ivz * fn + fi] = fx[IVZ];
        flx[IEN * fn + fi] = fx[IEN];
      }
}

/* ------------------------------------------------------------- corner EMF ---- */
static void corner_e(orc_sim *s) {
  /* field/calculate_corner_e.cpp:129-229 (3-D, Newtonian) */
  const size_t nc = s->ncell;
  const double *w = s->w, *bcc = s->bcc;
  double *cc = s->cce;
#pragma omp parallel for collapse(2)
  for (int k = s->ks - 1; k <= s->ke + 1; ++k)
    for (int j = s->js - 1; j <= s->je + 1; ++j)
      for (int i = s->is - 1; i <= s->ie + 1; ++i) {
        size_t c = C3(s, k, j, i);
        cc[c] = w[IVZ * nc + c] * bcc[nc + c] - w[IVY * nc + c] * bcc[2 * nc + c];
        cc[nc + c] = w[IVX * nc + c] * bcc[2 * nc + c] - w[IVZ * nc + c] * bcc[c];
        cc[2 * nc + c] = w[IVY * nc + c] * bcc[c] - w[IVX * nc + c] * bcc[nc + c];
      }
#define CC(n, k, j, i) cc[(size_t)(n) * nc + C3(s, k, j, i)]
#define WX1(k, j, i) s->wx1[F1I(s, k, j, i)]
#define WX2(k, j, i) s->wx2[F2I(s, k, j, i)]
#define WX3(k, j, i) s->wx3[F3I(s, k, j, i)]
#define E1X2(k, j, i) s->e1x2[F2I(s, k, j, i)]
#define E1X3(k, j, i) s->e1x3[F3I(s, k, j, i)]
#define E2X1(k, j, i) s->e2x1[F1I(s, k, j, i)]
#define E2X3(k, j, i) s->e2x3[F3I(s, k, j, i)]
#define E3X1(k, j, i) s->e3x1[F1I(s, k, j, i)]
#define E3X2(k, j, i) s->e3x2[F2I(s, k, j, i)]
#pragma omp parallel for collapse(2)
  for (int k = s->ks; k <= s->ke + 1; ++k)
    for (int j = s->js; j <= s->je + 1; ++j)
      for (int i = s->is; i <= s->ie + 1; ++i) {
        double de1_l3 = (1.0 - WX2(k - 1, j, i)) * (E1X3(k, j, i) - CC(0, k - 1, j, i)) +
                        (WX2(k - 1, j, i)) * (E1X3(k, j - 1, i) - CC(0, k - 1, j - 1, i));
        double de1_r3 = (1.0 - WX2(k, j, i)) * (E1X3(k, j, i) - CC(0, k, j, i)) +
                        (WX2(k, j, i)) * (E1X3(k, j - 1, i) - CC(0, k, j - 1, i));
        double de1_l2 = (1.0 - WX3(k, j - 1, i)) * (E1X2(k, j, i) - CC(0, k, j - 1, i)) +
                        (WX3(k, j - 1, i)) * (E1X2(k - 1, j, i) - CC(0, k - 1, j - 1, i));
        double de1_r2 = (1.0 - WX3(k, j, i)) * (E1X2(k, j, i) - CC(0, k, j, i)) +
                        (WX3(k, j, i)) * (E1X2(k - 1, j, i) - CC(0, k - 1, j, i));
        s->e1[EI(s, k, j, i)] = 0.25 * (de1_l3 + de1_r3 + de1_l2 + de1_r2 + E1X2(k - 1, j, i) +
                                        E1X2(k, j, i) + E1X3(k, j - 1, i) + E1X3(k, j, i));
        double de2_l3 = (1.0 - WX1(k - 1, j, i)) * (E2X3(k, j, i) - CC(1, k - 1, j, i)) +
                        (WX1(k - 1, j, i)) * (E2X3(k, j, i - 1) - CC(1, k - 1, j, i - 1));
        double de2_r3 = (1.0 - WX1(k, j, i)) * (E2X3(k, j, i) - CC(1, k, j, i)) +
                        (WX1(k, j, i)) * (E2X3(k, j, i - 1) - CC(1, k, j, i - 1));
        double de2_l1 = (1.0 - WX3(k, j, i - 1)) * (E2X1(k, j, i) - CC(1, k, j, i - 1)) +
                        (WX3(k, j, i - 1)) * (E2X1(k - 1, j, i) - CC(1, k - 1, j, i - 1));
        double de2_r1 = (1.0 - WX3(k, j, i)) * (E2X1(k, j, i) - CC(1, k, j, i)) +
                        (WX3(k, j, i)) * (E2X1(k - 1, j, i) - CC(1, k - 1, j, i));
        s->e2[EI(s, k, j, i)] = 0.25 * (de2_l3 + de2_r3 + de2_l1 + de2_r1 + E2X3(k, j, i - 1) +
                                        E2X3(k, j, i) + E2X1(k - 1, j, i) + E2X1(k, j, i));
        double de3_l2 = (1.0 - WX1(k, j - 1, i)) * (E3X2(k, j, i) - CC(2, k, j - 1, i)) +
                        (WX1(k, j - 1, i)) * (E3X2(k, j, i - 1) - CC(2, k, j - 1, i - 1));
        double de3_r2 = (1.0 - WX1(k, j, i)) * (E3X2(k, j, i) - CC(2, k, j, i)) +
                        (WX1(k, j, i)) * (E3X2(k, j, i - 1) - CC(2, k, j, i - 1));
        double de3_l1 = (1.0 - WX2(k, j, i - 1)) * (E3X1(k, j, i) - CC(2, k, j, i - 1)) +
                        (WX2(k, j, i - 1)) * (E3X1(k, j - 1, i) - CC(2, k, j - 1, i - 1));
        double de3_r1 = (1.0 - WX2(k, j, i)) * (E3X1(k, j, i) - CC(2, k, j, i)) +
                        (WX2(k, j, i)) * (E3X1(k, j - 1, i) - CC(2, k, j - 1, i));
        s->e3[EI(s, k, j, i)] = 0.25 * (de3_l1 + de3_r1 + de3_l2 + de3_r2 + E3X2(k, j, i - 1) +
                                        E3X2(k, j, i) + E3X1(k, j - 1, i) + E3X1(k, j, i));
      }
#undef CC
#undef WX1
#undef WX2
#undef WX3
#undef E1X2
#undef E1X3
#undef E2X1
#undef E2X3
#undef E3X1
#undef E3X2
}

/* ---------------------------------------------------------- conservative update ---- */
static void flux_divergence(orc_sim *s, double wght) {
  /* hydro/add_flux_divergence.cpp:53-92 with Cartesian areas/volume
   * (coordinates/coordinates.cpp:436-540) */
  const size_t nc = s->ncell, n1f = f1n(s), n2f = f2n(s), n3f = f3n(s);
  const double a1 = s->dx2 * s->dx3, a2 = s->dx1 * s->dx3, a3 = s->dx1 * s->dx2;
  const double vol = s->dx1 * s->dx2 * s->dx3;
#pragma omp parallel for collapse(2)
  for (int k = s->ks; k <= s->ke; ++k)
    for (int j = s->js; j <= s->je; ++j)
      for (int i = s->is; i <= s->ie; ++i)
        for (int n = 0; n < NHYD; ++n) {
          double d = (a1 * s->f1[n * n1f + F1I(s, k, j, i + 1)] - a1 * s->f1[n * n1f + F1I(s, k, j, i)]);
          d += (a2 * s->f2[n * n2f + F2I(s, k, j + 1, i)] - a2 * s->f2[n * n2f + F2I(s, k, j, i)]);
          d += (a3 * s->f3[n * n3f + F3I(s, k + 1, j, i)] - a3 * s->f3[n * n3f + F3I(s, k, j, i)]);
          s->u[n * nc + C3(s, k, j, i)] -= wght * d / vol;
        }
}

static void ct_update(orc_sim *s, double wght) {
  /* field/ct.cpp:38-113 with Cartesian edge lengths/areas */
  const double ar1 = s->dx2 * s->dx3, ar2 = s->dx1 * s->dx3, ar3 = s->dx1 * s->dx2;
  const double l1 = s->dx1, l2 = s->dx2, l3 = s->dx3;
#pragma omp parallel for collapse(2)
  for (int k = s->ks; k <= s->ke; ++k)
    for (int j = s->js; j <= s->je; ++j)
      for (int i = s->is; i <= s->ie + 1; ++i) {
        double *b = &s->b1[F1I(s, k, j, i)];
        *b -= (wght / ar1) * (l3 * s->e3[EI(s, k, j + 1, i)] - l3 * s->e3[EI(s, k, j, i)]);
        *b += (wght / ar1) * (l2 * s->e2[EI(s, k + 1, j, i)] - l2 * s->e2[EI(s, k, j, i)]);
      }
#pragma omp parallel for collapse(2)
  for (int k = s->ks; k <= s->ke; ++k)
    for (int j = s->js; j <= s->je + 1; ++j)
      for (int i = s->is; i <= s->ie; ++i) {
        double *b = &s->b2[F2I(s, k, j, i)];
        *b += (wght / ar2) * (l3 * s->e3[EI(s, k, j, i + 1)] - l3 * s->e3[EI(s, k, j, i)]);
        *b -= (wght / ar2) * (l1 * s->e1[EI(s, k + 1, j, i)] - l1 * s->e1[EI(s, k, j, i)]);
      }
#pragma omp parallel for collapse(2)
  for (int k = s->ks; k <= s->ke + 1; ++k)
    for (int j = s->js; j <= s->je; ++j)
      for (int i = s->is; i <= s->ie; ++i) {
        double *b = &s->b3[F3I(s, k, j, i)];
        *b -= (wght / ar3) * (l2 * s->e2[EI(s, k, j, i + 1)] - l2 * s->e2[EI(s, k, j, i)]);
        *b += (wght / ar3) * (l1 * s->e1[EI(s, k, j + 1, i)] - l1 * s->e1[EI(s, k, j, i)]);
      }
}

/* register averaging on the interior (cells) or the owned faces (fields):
 * mesh/weighted_ave.cpp:33-237 (out += w1*in for wght[0]==1; out = w0*out + w1*in) */
static void ave_cc(orc_sim *s, double *out, const double *in, double w0, double w1) {
  const size_t nc = s->ncell;
  for (int n = 0; n < NHYD; ++n)
#pragma omp parallel for collapse(2)
    for (int k = s->ks; k <= s->ke; ++k)
      for (int j = s->js; j <= s->je; ++j)
        for (int i = s->is; i <= s->ie; ++i) {
          size_t c = n * nc + C3(s, k, j, i);
          if (w0 == 1.0) out[c] += w1 * in[c];
          else out[c] = w0 * out[c] + w1 * in[c];
        }
}
static void ave_fc(orc_sim *s, double **out, double **in, double w0, double w1) {
  for (int d = 0; d < 3; ++d) {
    int iu = s->ie + (d == 0), ju = s->je + (d == 1), ku = s->ke + (d == 2);
#pragma omp parallel for collapse(2)
    for (int k = s->ks; k <= ku; ++k)
      for (int j = s->js; j <= ju; ++j)
        for (int i = s->is; i <= iu; ++i) {
          size_t c = d == 0 ? F1I(s, k, j, i) : (d == 1 ? F2I(s, k, j, i) : F3I(s, k, j, i));
          if (w0 == 1.0) out[d][c] += w1 * in[d][c];
          else out[d][c] = w0 * out[d][c] + w1 * in[d][c];
        }
  }
}

/* --------------------------------------------------------------- timestep ---- */
static double block_dt(orc_sim *s) {
  /* hydro/new_blockdt.cpp:58-158 */
  const size_t nc = s->ncell;
  double mindt = 1.79769313486231570815e308;
#pragma omp parallel for collapse(2) reduction(min : mindt)
  for (int k = s->ks; k <= s->ke; ++k)
    for (int j = s->js; j <= s->je; ++j)
      for (int i = s->is; i <= s->ie; ++i) {
        size_t c = C3(s, k, j, i);
        double wi[7];
        for (int n = 0; n < 5; ++n) wi[n] = s->w[n * nc + c];
        double dt1, dt2, dt3;
        if (s->p.mhd) {
          double bc1 = s->bcc[c], bc2 = s->bcc[nc + c], bc3 = s->bcc[2 * nc + c];
          double bx = bc1 + fabs(s->b1[F1I(s, k, j, i)] - bc1);
          wi[IBY] = bc2; wi[IBZ] = bc3;
          double cf = fast_speed(wi, bx, s->p.gamma);
          dt1 = s->dx1 / (fabs(wi[IVX]) + cf);
          wi[IBY] = bc3; wi[IBZ] = bc1;
          bx = bc2 + fabs(s->b2[F2I(s, k, j, i)] - bc2);
          cf = fast_speed(wi, bx, s->p.gamma);
          dt2 = s->dx2 / (fabs(wi[IVY]) + cf);
          wi[IBY] = bc1; wi[IBZ] = bc2;
          bx = bc3 + fabs(s->b3[F3I(s, k, j, i)] - bc3);
          cf = fast_speed(wi, bx, s->p.gamma);
          dt3 = s->dx3 / (fabs(wi[IVZ]) + cf);
        } else {
          double cs = sqrt(s->p.gamma * wi[IPR] / wi[IDN]);
          dt1 = s->dx1 / (fabs(wi[IVX]) + cs);
          dt2 = s->dx2 / (fabs(wi[IVY]) + cs);
          dt3 = s->dx3 / (fabs(wi[IVZ]) + cs);
        }
        mindt = fmin_ref(mindt, dt1);
        mindt = fmin_ref(mindt, dt2);
        mindt = fmin_ref(mindt, dt3);
      }
  return mindt * s->p.cfl;
}

static void new_time_step(orc_sim *s, double tlim) {
  /* mesh/mesh.cpp:1078-1118 */
  double bdt = block_dt(s);
  s->dt = 2.0 * s->dt;
  s->dt = fmin_ref(s->dt, bdt);
  if (s->time < tlim && (tlim - s->time) < s->dt) s->dt = tlim - s->time;
}

/* ------------------------------------------------------------------ driver ---- */
static void boundaries(orc_sim *s) {
  periodic_cc(s, s->u, NHYD);
  if (s->p.mhd) periodic_fc(s, s->b1, s->b2, s->b3);
}

/* Mesh::Initialize tail (mesh/mesh.cpp:1405-1649): ghosts, W(U), first dt. */
/* ---------------------------------------------------------- self-gravity ---- */
/* Couple a multigrid solver covering the same cubic mesh (one block). */
int orc_attach_gravity(orc_sim *s, struct orc_mg_s *mg, double four_pi_G) {
  const int n = orc_mg_size(mg);
  if (n != s->p.nx1 || n != s->p.nx2 || n != s->p.nx3) return -1;
  s->mg = mg;
  s->four_pi_G = four_pi_G;
  if (!s->phi) s->phi = calloc(s->ncell, 8);
  return 0;
}
double *orc_phi(orc_sim *s) { return s->phi; }

/* MGGravityDriver::Solve (gravity/mg_gravity.cpp:166-211): LoadSource of u(IDN) times
 * 4 pi G (multigrid/multigrid.cpp:194-233), the solve, and RetrieveResult with one ghost
 * layer (multigrid.cpp:269-286) */
static void gravity_solve(orc_sim *s) {
  const int n = s->p.nx1, nt = n + 2;
  double *src = orc_mg_src(s->mg);
  const double fac = s->four_pi_G;
  for (int k = 0; k < n; ++k)
    for (int j = 0; j < n; ++j)
      for (int i = 0; i < n; ++i) {
        double d = s->u[C3(s, k + s->ks, j + s->js, i + s->is)];
        src[((size_t)(k + 1) * nt + (j + 1)) * nt + (i + 1)] = (fac == 1.0) ? d : d * fac;
      }
  orc_mg_solve(s->mg);
  const double *u = orc_mg_u(s->mg);
  for (int k = -1; k <= n; ++k)
    for (int j = -1; j <= n; ++j)
      for (int i = -1; i <= n; ++i)
        s->phi[C3(s, k + s->ks, j + s->js, i + s->is)] =
            u[((size_t)(k + 1) * nt + (j + 1)) * nt + (i + 1)];
}

/* HydroSourceTerms::SelfGravity (hydro/srcterms/self_gravity.cpp:35-125): momentum from
 * the face potentials, energy from the mass fluxes; three passes in the reference's
 * order, each its own read-modify-write of U */
static void self_gravity(orc_sim *s, double dt) {
  const size_t nc = s->ncell, n1f = f1n(s), n2f = f2n(s), n3f = f3n(s);
  const double *phi = s->phi, *w = s->w;
  double *u = s->u;
  for (int dir = 0; dir < 3; ++dir) {
    const double dx = dir == 0 ? s->dx1 : (dir == 1 ? s->dx2 : s->dx3);
    const size_t st = dir == 0 ? 1 : (dir == 1 ? (size_t)s->n1 : (size_t)s->n1 * s->n2);
    const double *fl = dir == 0 ? s->f1 : (dir == 1 ? s->f2 : s->f3);
    (void)n1f; (void)n2f; (void)n3f;
#pragma omp parallel for collapse(2)
    for (int k = s->ks; k <= s->ke; ++k)
      for (int j = s->js; j <= s->je; ++j)
        for (int i = s->is; i <= s->ie; ++i) {
          const size_t c = C3(s, k, j, i);
          const double dtodx = dt / dx;
          const double phic = phi[c];
          const double phil = 0.5 * (phi[c - st] + phi[c]);
          const double phir = 0.5 * (phi[c] + phi[c + st]);
          u[(1 + dir) * nc + c] -= dtodx * w[c] * (phir - phil);
          size_t fl_l, fl_r;
          if (dir == 0) { fl_l = F1I(s, k, j, i); fl_r = F1I(s, k, j, i + 1); }
          else if (dir == 1) { fl_l = F2I(s, k, j, i); fl_r = F2I(s, k, j + 1, i); }
          else { fl_l = F3I(s, k, j, i); fl_r = F3I(s, k + 1, j, i); }
          u[4 * nc + c] -= dtodx * (fl[fl_l] * (phic - phil) + fl[fl_r] * (phir - phic));
        }
  }
}

void orc_initialize(orc_sim *s, double tlim) {
  if (s->mg) gravity_solve(s); /* mesh/mesh.cpp:1398-1402 */
  boundaries(s);
  c2p(s);
  s->time = 0.0;
  new_time_step(s, tlim);
}

static void swapp(double **a, double **b) { double *t = *a; *a = *b; *b = t; }

void orc_stage(orc_sim *s, int l) {
  const size_t nc = s->ncell;
  if (l == 0) { /* StartupTaskList: time_integrator.cpp:1386-1398 */
    memset(s->u1, 0, NHYD * nc * 8);
    if (s->p.mhd) {
      memset(s->r1, 0, f1n(s) * 8); memset(s->r2, 0, f2n(s) * 8); memset(s->r3, 0, f3n(s) * 8);
    }
  }
  int order = (s->p.integrator == ORC_VL2 && l == 0) ? 1 : s->p.xorder;
  sweep(s, 0, order);
  sweep(s, 1, order);
  sweep(s, 2, order);
  if (s->p.mhd) corner_e(s);
  /* IntegrateHydro (time_integrator.cpp:1563-1616) */
  if (s->delta[l] != 0.0) ave_cc(s, s->u1, s->u, 1.0, s->delta[l]);
  int do_swap = (s->g1[l] == 0.0 && s->g2[l] == 1.0 && s->g3[l] == 0.0);
  if (do_swap) swapp(&s->u, &s->u1);
  else ave_cc(s, s->u, s->u1, s->g1[l], s->g2[l]);
  flux_divergence(s, s->beta[l] * s->dt);
  /* AddSourceTerms (:1655-1676); every stage of these integrators is a main stage */
  if (s->mg) self_gravity(s, s->beta[l] * s->dt);
  if (s->p.mhd) { /* IntegrateField (:1618-1653) */
    double *bo[3] = {s->r1, s->r2, s->r3}, *bi[3] = {s->b1, s->b2, s->b3};
    if (s->delta[l] != 0.0) ave_fc(s, bo, bi, 1.0, s->delta[l]);
    if (do_swap) {
      swapp(&s->b1, &s->r1); swapp(&s->b2, &s->r2); swapp(&s->b3, &s->r3);
    } else {
      double *bo2[3] = {s->b1, s->b2, s->b3}, *bi2[3] = {s->r1, s->r2, s->r3};
      ave_fc(s, bo2, bi2, s->g1[l], s->g2[l]);
    }
    ct_update(s, s->beta[l] * s->dt);
  }
  boundaries(s);
  c2p(s);
  if (s->mg) gravity_solve(s); /* main.cpp:461-466 */
}

/* One cycle (main.cpp:459-485): all stages, time advance, new dt. */
void orc_cycle(orc_sim *s, int ncycles, double tlim) {
  for (int c = 0; c < ncycles; ++c) {
    for (int l = 0; l < s->nstages; ++l) orc_stage(s, l);
    s->time += s->dt;
    new_time_step(s, tlim);
  }
}

/* Runs whole cycles until time >= tlim (or nlim cycles, if nlim >= 0). */
int orc_run(orc_sim *s, double tlim, int nlim) {
  int n = 0;
  while (s->time < tlim && (nlim < 0 || n < nlim)) {
    orc_cycle(s, 1, tlim);
    ++n;
  }
  return n;
}

int orc_num_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}
