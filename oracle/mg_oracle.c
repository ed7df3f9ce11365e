/* mg_oracle.c -- CPU restatement of the reference's multigrid Poisson solver.
 *
 * TEST INFRASTRUCTURE ONLY (the oracle): the CUDA multigrid is checked against it and
 * bench.py times it as the CPU baseline. Pinned against the reference binary (poisson
 * and uniform-sphere runs) in tests/golden/.
 *
 * Scope: a uniform cubic mesh held as one grid per level (N = 2^L cells per side, one
 * ghost layer). On such a mesh the reference's hierarchy -- every MeshBlock coarsened
 * to one cell, then a root grid coarsened to one cell -- visits the same sequence of
 * uniform levels, with the same stencils, colour parity, boundary fills and coarsest
 * solve, so one grid per level reproduces it.
 *
 * Reference routines followed (paths relative to the reference src/):
 *   smoother        gravity/mg_gravity.cpp:220-273  (red-black GS, omega = 1.15)
 *   defect          gravity/mg_gravity.cpp:283-314
 *   restriction     multigrid/multigrid.cpp:684-725, RestrictBlock :331-358
 *   prolongation    multigrid/multigrid.cpp:733-832 (trilinear, 27/9/3/1 over 64)
 *   FMG prolong.    multigrid/multigrid.cpp:838-1048 (separable (5,30,-3)/32)
 *   V / FMG cycles  multigrid/multigrid_driver.cpp:553-762
 *   coarsest grid   multigrid/multigrid_driver.cpp:778-823
 *   defect norm     multigrid/multigrid.cpp:555-600, multigrid_driver.cpp:826-862
 *   average         multigrid/multigrid_driver.cpp:305-340, multigrid.cpp:624-641
 *   physical BCs    bvals/cc/mg/bvals_mg.cpp:321-368 (face order and extents),
 *                   multigrid/mgbval_zerograd.cpp, mgbval_zerofixed.cpp,
 *                   mgbval_multipole.cpp:28-426
 *   multipoles      multigrid/multigrid.cpp:1054-1300, multigrid_driver.cpp:1909-2018
 *   coordinates     multigrid/multigrid.cpp:1321-1346
 *   FAS             multigrid/multigrid_driver.cpp:292-295 (on with a multipole face),
 *                   task_list/mg_task_list.cpp:258-264, multigrid.cpp:331-388,648-653
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

enum { MG_PERIODIC = 0, MG_ZEROGRAD = 1, MG_ZEROFIXED = 2, MG_MULTIPOLE = 3 };

typedef struct {
  int lmax;                 /* finest level: N = 2^lmax */
  double xmin[3], xmax[3];
  int bc[6];                /* ix1, ox1, ix2, ox2, ix3, ox3 */
  int mporder;              /* 2 or 4 when a multipole boundary is used */
  int autompo, nodipole;
  double mporigin[3];
  int fmg;                  /* 1: FMG (mgmode=FMG), 0: iterate from the current u (MGI) */
  double eps;               /* <gravity> threshold (>= 0: iterate to it), < 0: niter cycles */
  int niter;
  double omega;
} orc_mg_params;

typedef struct orc_mg_s {
  orc_mg_params p;
  int nl;                   /* number of levels = lmax + 1 */
  double **u, **src, **def, **uold;
  int fas;                  /* full approximation scheme (multipole boundaries) */
  double **xf[3], **xv[3];  /* per-level coordinates incl. ghosts */
  double *dx;               /* per-level cell width (x1; the mesh is cubic) */
  double rdx;               /* finest width */
  int coffset;
  int periodic;             /* every face periodic: ghosts are a plain wrap */
  int subtract_average;     /* multigrid_driver.cpp:139-300: on unless a multipole face */
  double mpc[25], mpo[3];
  double last_ave;
  int iterations;
  double last_norm;
} orc_mg;

#define N_(L) (1 << (L))
#define NT_(L) (N_(L) + 2)
#define IX(L, k, j, i) ((((size_t)(k)) * NT_(L) + (size_t)(j)) * NT_(L) + (size_t)(i))

orc_mg *orc_mg_create(const orc_mg_params *p) {
  orc_mg *m = (orc_mg *)calloc(1, sizeof(orc_mg));
  m->p = *p;
  if (m->p.omega == 0.0) m->p.omega = 1.15;
  m->nl = p->lmax + 1;
  m->u = calloc(m->nl, sizeof(double *));
  m->src = calloc(m->nl, sizeof(double *));
  m->def = calloc(m->nl, sizeof(double *));
  m->uold = calloc(m->nl, sizeof(double *));
  m->dx = calloc(m->nl, sizeof(double));
  for (int d = 0; d < 3; ++d) {
    m->xf[d] = calloc(m->nl, sizeof(double *));
    m->xv[d] = calloc(m->nl, sizeof(double *));
  }
  for (int L = 0; L < m->nl; ++L) {
    size_t n = (size_t)NT_(L) * NT_(L) * NT_(L);
    m->u[L] = calloc(n, 8);
    m->src[L] = calloc(n, 8);
    m->def[L] = calloc(n, 8);
    m->uold[L] = calloc(n, 8);
    int nc = N_(L), ngh = 1;
    for (int d = 0; d < 3; ++d) {
      double *xf = calloc(nc + 3, 8), *xv = calloc(nc + 2, 8);
      double w = (p->xmax[d] - p->xmin[d]) / nc;
      for (int i = 0; i <= nc + 2 * ngh; ++i) xf[i] = p->xmin[d] + (i - ngh) * w;
      xf[ngh] = p->xmin[d];
      xf[nc + ngh] = p->xmax[d];
      for (int i = 0; i < nc + 2 * ngh; ++i) xv[i] = 0.5 * (xf[i] + xf[i + 1]);
      m->xf[d][L] = xf;
      m->xv[d][L] = xv;
    }
  }
  /* the finest width as the reference derives it (multigrid.cpp:60); coarser levels
   * scale it by powers of two (mg_gravity.cpp:223-224) */
  m->rdx = (p->xmax[0] - p->xmin[0]) / (double)N_(p->lmax);
  for (int L = 0; L < m->nl; ++L) m->dx[L] = m->rdx * (double)(1 << (p->lmax - L));
  m->periodic = 1;
  m->subtract_average = 1;
  for (int f = 0; f < 6; ++f) {
    if (p->bc[f] != MG_PERIODIC) m->periodic = 0;
    if (p->bc[f] == MG_MULTIPOLE) m->subtract_average = 0;
  }
  m->fas = !m->subtract_average;
  for (int d = 0; d < 3; ++d) m->mpo[d] = p->mporigin[d];
  return m;
}

void orc_mg_destroy(orc_mg *m) {
  if (!m) return;
  for (int L = 0; L < m->nl; ++L) {
    free(m->u[L]); free(m->src[L]); free(m->def[L]); free(m->uold[L]);
    for (int d = 0; d < 3; ++d) { free(m->xf[d][L]); free(m->xv[d][L]); }
  }
  free(m->u); free(m->src); free(m->def); free(m->uold); free(m->dx);
  for (int d = 0; d < 3; ++d) { free(m->xf[d]); free(m->xv[d]); }
  free(m);
}

double *orc_mg_u(orc_mg *m) { return m->u[m->nl - 1]; }
double *orc_mg_src(orc_mg *m) { return m->src[m->nl - 1]; }
int orc_mg_iterations(const orc_mg *m) { return m->iterations; }
int orc_mg_size(const orc_mg *m) { return 1 << m->p.lmax; }
double orc_mg_last_norm(const orc_mg *m) { return m->last_norm; }
int orc_mg_coffset(const orc_mg *m) { return m->coffset; }
void orc_mg_set_coffset(orc_mg *m, int c) { m->coffset = c; }
void orc_mg_mpcoeff(const orc_mg *m, double *out) {
  memcpy(out, m->mpc, sizeof(m->mpc));
  out[25] = m->mpo[0]; out[26] = m->mpo[1]; out[27] = m->mpo[2];
}

/* ------------------------------------------------------------------ multipole ---- */
static double mp_phi(const orc_mg *m, double x, double y, double z) {
  const double *c = m->mpc;
  double x2 = x * x, y2 = y * y, z2 = z * z, xy = x * y, yz = y * z, zx = z * x;
  double r2 = x2 + y2 + z2;
  double ir2 = 1.0 / r2, ir1 = sqrt(ir2);
  double ir3 = ir2 * ir1, ir5 = ir3 * ir2;
  if (m->p.mporder == 2)
    return ir1 * c[0] + ir3 * (c[1] * y + c[2] * z + c[3] * x) +
           ir5 * (c[4] * xy + c[5] * yz + (3.0 * z2 - r2) * c[6] + c[7] * zx +
                  c[8] * 0.5 * (x2 - y2));
  double ir7 = ir5 * ir2, ir9 = ir7 * ir2;
  double hx2my2 = 0.5 * (x2 - y2);
  double x2mty2 = x2 - 3.0 * y2;
  double tx2my2 = 3.0 * x2 - y2;
  return ir1 * c[0] + ir3 * (c[1] * y + c[2] * z + c[3] * x) +
         ir5 * (c[4] * xy + c[5] * yz + (3.0 * z2 - r2) * c[6] + c[7] * zx +
                c[8] * 0.5 * (x2 - y2)) +
         ir7 * (y * tx2my2 * c[9] + x * x2mty2 * c[15] + xy * z * c[10] + z * hx2my2 * c[14] +
                (5.0 * z2 - r2) * (y * c[11] + x * c[13]) + z * (z2 - 3.0 * r2) * c[12]) +
         ir9 * (xy * hx2my2 * c[16] + 0.125 * (x2 * x2mty2 - y2 * tx2my2) * c[24] +
                yz * tx2my2 * c[17] + zx * x2mty2 * c[23] +
                (7.0 * z2 - r2) * (xy * c[18] + hx2my2 * c[22]) +
                (7.0 * z2 - 3.0 * r2) * (yz * c[19] + zx * c[21]) +
                (35.0 * z2 * z2 - 30.0 * z2 * r2 + 3.0 * r2 * r2) * c[20]);
}

static void multipole_moments(orc_mg *m) {
  /* multigrid.cpp:1054-1265 and the scaling of multigrid_driver.cpp:1939-1988 */
  const int L = m->nl - 1, n = N_(L);
  const double *src = m->src[L];
  const double *x1f = m->xf[0][L], *x2f = m->xf[1][L], *x3f = m->xf[2][L];
  const double *x1v = m->xv[0][L], *x2v = m->xv[1][L], *x3v = m->xv[2][L];
  double vol = (x1f[2] - x1f[1]) * (x2f[2] - x2f[1]) * (x3f[2] - x3f[1]);
  if (m->p.autompo) { /* multigrid.cpp:1270-1297, multigrid_driver.cpp:1990-2018 */
    double m0 = 0, m1 = 0, m2 = 0, m3 = 0;
    for (int k = 1; k <= n; ++k)
      for (int j = 1; j <= n; ++j)
        for (int i = 1; i <= n; ++i) {
          double s = src[IX(L, k, j, i)] * vol;
          m0 += s; m1 += s * x2v[j]; m2 += s * x3v[k]; m3 += s * x1v[i];
        }
    double im = 1.0 / m0;
    m->mpo[0] = im * m3; m->mpo[1] = im * m1; m->mpo[2] = im * m2;
  }
  double mm[25];
  memset(mm, 0, sizeof(mm));
  for (int k = 1; k <= n; ++k) {
    double z = x3v[k] - m->mpo[2], z2 = z * z;
    for (int j = 1; j <= n; ++j) {
      double y = x2v[j] - m->mpo[1], y2 = y * y, yz = y * z;
      for (int i = 1; i <= n; ++i) {
        double x = x1v[i] - m->mpo[0];
        double x2 = x * x, xy = x * y, zx = z * x;
        double r2 = x2 + y2 + z2;
        double s = src[IX(L, k, j, i)] * vol;
        mm[0] += s;
        if (!m->p.nodipole) { mm[1] += s * y; mm[2] += s * z; mm[3] += s * x; }
        mm[4] += s * xy; mm[5] += s * yz; mm[6] += s * (3.0 * z2 - r2); mm[7] += s * zx;
        if (m->p.mporder == 4) {
          double hx2my2 = 0.5 * (x2 - y2), x2mty2 = x2 - 3.0 * y2, tx2my2 = 3.0 * x2 - y2;
          double fz2mr2 = 5.0 * z2 - r2, sz2mr2 = 7.0 * z2 - r2, sz2mtr2 = 7.0 * z2 - 3.0 * r2;
          mm[8] += s * hx2my2;
          mm[9] += s * y * tx2my2; mm[10] += s * xy * z; mm[11] += s * y * fz2mr2;
          mm[12] += s * z * (z2 - 3.0 * r2); mm[13] += s * x * fz2mr2;
          mm[14] += s * z * hx2my2; mm[15] += s * x * x2mty2;
          mm[16] += s * xy * hx2my2; mm[17] += s * yz * tx2my2; mm[18] += s * xy * sz2mr2;
          mm[19] += s * yz * sz2mtr2;
          mm[20] += s * (35.0 * z2 * z2 - 30.0 * z2 * r2 + 3.0 * r2 * r2);
          mm[21] += s * zx * sz2mtr2; mm[22] += s * hx2my2 * sz2mr2; mm[23] += s * zx * x2mty2;
          mm[24] += s * 0.125 * (x2 * x2mty2 - y2 * tx2my2);
        } else {
          mm[8] += s * 0.5 * (x2 - y2);
        }
      }
    }
  }
  const double PI = 3.1415926535897932;
  const double c0 = -0.25 / PI, c1 = -0.25 / PI, c2 = -0.0625 / PI, c2a = -0.75 / PI;
  const double c30 = -0.0625 / PI, c31 = -0.0625 * 1.5 / PI, c32 = -0.25 * 15.0 / PI,
               c33 = -0.0625 * 2.5 / PI;
  const double c40 = -0.0625 * 0.0625 / PI, c41 = -0.0625 * 2.5 / PI, c42 = -0.0625 * 5.0 / PI,
               c43 = -0.0625 * 17.5 / PI, c44 = -0.25 * 35.0 / PI;
  double sc[25] = {c0, c1, c1, c1, c2a, c2a, c2, c2a, c2a, c33, c32, c31, c30, c31, c32, c33,
                   c44, c43, c42, c41, c40, c41, c42, c43, c44};
  int nc = m->p.mporder == 4 ? 25 : 9;
  for (int q = 0; q < 25; ++q) m->mpc[q] = (q < nc) ? mm[q] * sc[q] : 0.0;
}

/* ------------------------------------------------------------------ boundaries ---- */
static void fill_periodic(orc_mg *m, double *a, int L) {
  int n = N_(L), nt = NT_(L);
  for (int k = 0; k < nt; ++k)
    for (int j = 0; j < nt; ++j)
      for (int i = 0; i < nt; ++i) {
        int kk = k == 0 ? n : (k == n + 1 ? 1 : k);
        int jj = j == 0 ? n : (j == n + 1 ? 1 : j);
        int ii = i == 0 ? n : (i == n + 1 ? 1 : i);
        if (kk != k || jj != j || ii != i) a[IX(L, k, j, i)] = a[IX(L, kk, jj, ii)];
      }
}

/* one face: dir 0..2, side 0 inner / 1 outer, over the given transverse extents */
static void face_bc(orc_mg *m, double *a, int L, int dir, int side, int lo1, int hi1, int lo2,
                    int hi2) {
  int n = N_(L);
  int bc = m->p.bc[2 * dir + side];
  int gi = side ? n + 1 : 0, ii = side ? n : 1;
  const double *xf = m->xf[dir][L];
  for (int b = lo2; b <= hi2; ++b)
    for (int a1 = lo1; a1 <= hi1; ++a1) {
      size_t g, s;
      double px = 0, py = 0, pz = 0;
      if (dir == 0) { /* a1 = j, b = k */
        g = IX(L, b, a1, gi); s = IX(L, b, a1, ii);
        px = xf[side ? n + 1 : 1]; py = m->xv[1][L][a1]; pz = m->xv[2][L][b];
      } else if (dir == 1) { /* a1 = i, b = k */
        g = IX(L, b, gi, a1); s = IX(L, b, ii, a1);
        px = m->xv[0][L][a1]; py = xf[side ? n + 1 : 1]; pz = m->xv[2][L][b];
      } else { /* a1 = i, b = j */
        g = IX(L, gi, b, a1); s = IX(L, ii, b, a1);
        px = m->xv[0][L][a1]; py = m->xv[1][L][b]; pz = xf[side ? n + 1 : 1];
      }
      if (bc == MG_ZEROGRAD) a[g] = a[s];
      else if (bc == MG_ZEROFIXED) a[g] = -a[s];
      else if (bc == MG_MULTIPOLE)
        a[g] = 2.0 * mp_phi(m, px - m->mpo[0], py - m->mpo[1], pz - m->mpo[2]) - a[s];
    }
}

static void apply_bc(orc_mg *m, double *a, int L) {
  if (m->periodic) { fill_periodic(m, a, L); return; }
  int n = N_(L);
  /* bvals_mg.cpp:339-366: x1 faces over interior j,k (extended where the neighbouring
   * face has no physical boundary), x2 faces over i incl. ghosts, x3 over i and j incl.
   * ghosts; periodic axes are wrapped first (inter-block exchange). */
  int px = m->p.bc[0] == MG_PERIODIC, py = m->p.bc[2] == MG_PERIODIC,
      pz = m->p.bc[4] == MG_PERIODIC;
  if (px || py || pz) {
    int nt = NT_(L);
    for (int k = 0; k < nt; ++k)
      for (int j = 0; j < nt; ++j)
        for (int i = 0; i < nt; ++i) {
          int kk = k, jj = j, ii = i;
          if (pz) kk = k == 0 ? n : (k == n + 1 ? 1 : k);
          if (py) jj = j == 0 ? n : (j == n + 1 ? 1 : j);
          if (px) ii = i == 0 ? n : (i == n + 1 ? 1 : i);
          if (kk != k || jj != j || ii != i) a[IX(L, k, j, i)] = a[IX(L, kk, jj, ii)];
        }
  }
  int bjs = py ? 0 : 1, bje = py ? n + 1 : n, bks = pz ? 0 : 1, bke = pz ? n + 1 : n;
  if (!px) { face_bc(m, a, L, 0, 0, bjs, bje, bks, bke); face_bc(m, a, L, 0, 1, bjs, bje, bks, bke); }
  if (!py) { face_bc(m, a, L, 1, 0, 0, n + 1, bks, bke); face_bc(m, a, L, 1, 1, 0, n + 1, bks, bke); }
  if (!pz) { face_bc(m, a, L, 2, 0, 0, n + 1, 0, n + 1); face_bc(m, a, L, 2, 1, 0, n + 1, 0, n + 1); }
}

/* -------------------------------------------------------------------- kernels ---- */
static void smooth(orc_mg *m, int L, int color) {
  double *u = m->u[L];
  const double *src = m->src[L];
  double dx = m->dx[L], dx2 = dx * dx, isix = m->p.omega / 6.0;
  int n = N_(L);
  color ^= m->coffset;
#pragma omp parallel for if (n >= 32)
  for (int k = 1; k <= n; ++k)
    for (int j = 1; j <= n; ++j) {
      int c = (color + k + j) & 1;
      for (int i = 1 + c; i <= n; i += 2) {
        size_t q = IX(L, k, j, i);
        size_t sk = (size_t)NT_(L) * NT_(L), sj = NT_(L);
        u[q] -= ((6.0 * u[q] - u[q + sk] - u[q + sj] - u[q + 1] - u[q - sk] - u[q - sj] -
                  u[q - 1]) + src[q] * dx2) * isix;
      }
    }
}

static void defect(orc_mg *m, int L) {
  double *def = m->def[L];
  const double *u = m->u[L], *src = m->src[L];
  double dx = m->dx[L], idx2 = 1.0 / (dx * dx);
  int n = N_(L);
  size_t sk = (size_t)NT_(L) * NT_(L), sj = NT_(L);
#pragma omp parallel for if (n >= 32)
  for (int k = 1; k <= n; ++k)
    for (int j = 1; j <= n; ++j)
      for (int i = 1; i <= n; ++i) {
        size_t q = IX(L, k, j, i);
        def[q] = (6.0 * u[q] - u[q + sk] - u[q + sj] - u[q + 1] - u[q - sk] - u[q - sj] -
                  u[q - 1]) * idx2 + src[q];
      }
}

/* FAS right-hand side: src -= L'(u) on the interior (mg_gravity.cpp:324-351) */
static void fas_rhs(orc_mg *m, int L) {
  double *src = m->src[L];
  const double *u = m->u[L];
  double dx = m->dx[L], idx2 = 1.0 / (dx * dx);
  int n = N_(L);
  size_t sk = (size_t)NT_(L) * NT_(L), sj = NT_(L);
  for (int k = 1; k <= n; ++k)
    for (int j = 1; j <= n; ++j)
      for (int i = 1; i <= n; ++i) {
        size_t q = IX(L, k, j, i);
        src[q] -= (6.0 * u[q] - u[q + sk] - u[q + sj] - u[q + 1] - u[q - sk] - u[q - sj] -
                   u[q - 1]) * idx2;
      }
}
static void store_old(orc_mg *m, int L) {
  memcpy(m->uold[L], m->u[L], sizeof(double) * (size_t)NT_(L) * NT_(L) * NT_(L));
}

static void restrict_to(orc_mg *m, double *dst, const double *s, int Lc) {
  int n = N_(Lc), Lf = Lc + 1;
#pragma omp parallel for if (n >= 32)
  for (int k = 1; k <= n; ++k) {
    int fk = 2 * k - 1;
    for (int j = 1; j <= n; ++j) {
      int fj = 2 * j - 1;
      for (int i = 1; i <= n; ++i) {
        int fi = 2 * i - 1;
        dst[IX(Lc, k, j, i)] =
            0.125 * (s[IX(Lf, fk, fj, fi)] + s[IX(Lf, fk, fj, fi + 1)] +
                     s[IX(Lf, fk, fj + 1, fi)] + s[IX(Lf, fk, fj + 1, fi + 1)] +
                     s[IX(Lf, fk + 1, fj, fi)] + s[IX(Lf, fk + 1, fj, fi + 1)] +
                     s[IX(Lf, fk + 1, fj + 1, fi)] + s[IX(Lf, fk + 1, fj + 1, fi + 1)]);
      }
    }
  }
}

static void prolongate_correct(orc_mg *m, int Lc) {
  const double *s = m->u[Lc];
  double *d = m->u[Lc + 1];
  int n = N_(Lc), Lf = Lc + 1;
#define S(kk, jj, ii) s[IX(Lc, kk, jj, ii)]
#pragma omp parallel for if (n >= 16)
  for (int k = 1; k <= n; ++k) {
    int fk = 2 * (k - 1) + 1;
    for (int j = 1; j <= n; ++j) {
      int fj = 2 * (j - 1) + 1;
      for (int i = 1; i <= n; ++i) {
        int fi = 2 * (i - 1) + 1;
        for (int oz = 0; oz < 2; ++oz)
          for (int oy = 0; oy < 2; ++oy)
            for (int ox = 0; ox < 2; ++ox) {
              int dz = oz ? 1 : -1, dy = oy ? 1 : -1, dxx = ox ? 1 : -1;
              d[IX(Lf, fk + oz, fj + oy, fi + ox)] +=
                  0.015625 * (27.0 * S(k, j, i) + S(k + dz, j + dy, i + dxx) +
                              9.0 * (S(k, j, i + dxx) + S(k, j + dy, i) + S(k + dz, j, i)) +
                              3.0 * (S(k + dz, j + dy, i) + S(k + dz, j, i + dxx) +
                                     S(k, j + dy, i + dxx)));
            }
      }
    }
  }
#undef S
}

static void fmg_prolongate(orc_mg *m, int Lc) {
  const double *s = m->u[Lc];
  double *d = m->u[Lc + 1];
  int n = N_(Lc), Lf = Lc + 1;
  static const double w0[3] = {5.0, 30.0, -3.0}, w1[3] = {-3.0, 30.0, 5.0};
#pragma omp parallel for if (n >= 16)
  for (int k = 1; k <= n; ++k) {
    int fk = 2 * (k - 1) + 1;
    for (int j = 1; j <= n; ++j) {
      int fj = 2 * (j - 1) + 1;
      for (int i = 1; i <= n; ++i) {
        int fi = 2 * (i - 1) + 1;
        for (int oz = 0; oz < 2; ++oz)
          for (int oy = 0; oy < 2; ++oy)
            for (int ox = 0; ox < 2; ++ox) {
              const double *wz = oz ? w1 : w0, *wy = oy ? w1 : w0, *wx = ox ? w1 : w0;
              double acc = 0.0;
              int first = 1;
              for (int a = 0; a < 3; ++a)
                for (int b = 0; b < 3; ++b)
                  for (int c = 0; c < 3; ++c) {
                    double t = (wz[a] * wy[b] * wx[c]) * s[IX(Lc, k - 1 + a, j - 1 + b, i - 1 + c)];
                    if (first) { acc = t; first = 0; }
                    else acc = acc + t;
                  }
              d[IX(Lf, fk + oz, fj + oy, fi + ox)] = acc / 32768.0;
            }
      }
    }
  }
}

/* ------------------------------------------------------------------ reductions ---- */
static double total(orc_mg *m, const double *a, int L) {
  int n = N_(L);
  double s = 0.0;
  for (int k = 1; k <= n; ++k)
    for (int j = 1; j <= n; ++j)
      for (int i = 1; i <= n; ++i) s += a[IX(L, k, j, i)];
  double dx = m->dx[L];
  return s * dx * dx * dx;
}
static void subtract(double *a, int L, double ave) {
  size_t nt = (size_t)NT_(L) * NT_(L) * NT_(L);
  for (size_t q = 0; q < nt; ++q) a[q] -= ave;
}
static double domain_volume(const orc_mg *m) {
  return (m->p.xmax[0] - m->p.xmin[0]) * (m->p.xmax[1] - m->p.xmin[1]) *
         (m->p.xmax[2] - m->p.xmin[2]);
}

double orc_mg_defect_norm(orc_mg *m) {
  const int L = m->nl - 1, n = N_(L);
  apply_bc(m, m->u[L], L);
  defect(m, L);
  double s = 0.0;
  for (int k = 1; k <= n; ++k)
    for (int j = 1; j <= n; ++j)
      for (int i = 1; i <= n; ++i) {
        double v = m->def[L][IX(L, k, j, i)];
        s += v * v;
      }
  double dx = m->dx[L];
  s = s * dx * dx * dx / domain_volume(m);
  return sqrt(s);
}

/* ---------------------------------------------------------------- cycles ---- */
static void coarsest(orc_mg *m) {
  /* multigrid_driver.cpp:778-823 with ni = 1 (cubic power-of-two root grid) */
  if (m->subtract_average) {
    if (m->fas) { apply_bc(m, m->u[0], 0); store_old(m, 0); }
    memset(m->u[0], 0, sizeof(double) * 27);
    return;
  }
  apply_bc(m, m->u[0], 0);
  if (m->fas) { store_old(m, 0); fas_rhs(m, 0); }
  smooth(m, 0, 0);
  apply_bc(m, m->u[0], 0);
  smooth(m, 0, 1);
  apply_bc(m, m->u[0], 0);
}

static void vcycle(orc_mg *m, int top) {
  /* SolveVCycle(1,1) from level `top` = the current FMG level (multigrid_driver.cpp:684-694;
   * OneStepToCoarser :629-682, OneStepToFiner :583-627) */
  m->coffset ^= 1;
  for (int L = top; L > 0; --L) {
    apply_bc(m, m->u[L], L);
    if (m->fas && L < top) { store_old(m, L); fas_rhs(m, L); }
    smooth(m, L, 0);
    apply_bc(m, m->u[L], L);
    smooth(m, L, 1);
    apply_bc(m, m->u[L], L);
    defect(m, L);
    restrict_to(m, m->src[L - 1], m->def[L], L - 1);
    if (m->fas) restrict_to(m, m->u[L - 1], m->u[L], L - 1);
    else memset(m->u[L - 1], 0, sizeof(double) * (size_t)NT_(L - 1) * NT_(L - 1) * NT_(L - 1));
  }
  coarsest(m);
  for (int L = 0; L < top; ++L) {
    apply_bc(m, m->u[L], L);
    if (m->fas) {
      size_t nt = (size_t)NT_(L) * NT_(L) * NT_(L);
      for (size_t q = 0; q < nt; ++q) m->u[L][q] -= m->uold[L][q];
    }
    prolongate_correct(m, L);
    apply_bc(m, m->u[L + 1], L + 1);
    smooth(m, L + 1, 0);
    apply_bc(m, m->u[L + 1], L + 1);
    smooth(m, L + 1, 1);
  }
  apply_bc(m, m->u[top], top);
}

void orc_mg_vcycles(orc_mg *m, int n) {
  for (int q = 0; q < n; ++q) vcycle(m, m->nl - 1);
}

/* MGGravityDriver::Solve after LoadSource (gravity/mg_gravity.cpp:166-211):
 * SetupMultigrid, then FMG+iterate or iterate, average subtraction when periodic. */
void orc_mg_solve(orc_mg *m) {
  const int top = m->nl - 1;
  m->iterations = 0;
  if (m->subtract_average) { /* SubtractAverage(src) */
    double tot = total(m, m->src[top], top);
    m->last_ave = tot / domain_volume(m);
    subtract(m->src[top], top, m->last_ave);
  }
  int needs_mp = 0;
  for (int f = 0; f < 6; ++f) needs_mp |= (m->p.bc[f] == MG_MULTIPOLE);
  if (needs_mp) multipole_moments(m);
  if (m->p.fmg) {
    /* RestrictFMGSource; the coarsest u keeps its content from the previous solve,
     * as the reference's root grid does */
    for (int L = top; L > 0; --L) restrict_to(m, m->src[L - 1], m->src[L], L - 1);
    for (int f = 0; f <= top; ++f) {
      vcycle(m, f);
      if (f != top) {
        apply_bc(m, m->u[f], f);
        fmg_prolongate(m, f);
      }
    }
    if (m->subtract_average) {
      double tot = total(m, m->u[top], top);
      subtract(m->u[top], top, tot / domain_volume(m));
    }
  }
  if (m->p.eps >= 0.0) { /* SolveIterative (:721-760) */
    double def = orc_mg_defect_norm(m);
    int n = 0;
    while (def > m->p.eps) {
      vcycle(m, top);
      m->iterations++;
      double old = def;
      def = orc_mg_defect_norm(m);
      if (def / old > 0.8 && m->p.eps == 0.0) break;
      if (n > 100) break;
      n++;
    }
    m->last_norm = def;
  } else {
    for (int q = 0; q < m->p.niter; ++q) { vcycle(m, top); m->iterations++; }
    m->last_norm = orc_mg_defect_norm(m);
  }
  if (m->subtract_average) {
    double tot = total(m, m->u[top], top);
    subtract(m->u[top], top, tot / domain_volume(m));
  }
  apply_bc(m, m->u[top], top);
}
