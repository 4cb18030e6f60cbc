/*
 * fest_oracle.c - CPU restatement (FP64) of FEST-3D's explicit
 * residual-and-update path.  TEST INFRASTRUCTURE ONLY (see fest_oracle.h).
 *
 * Conventions: arrays keep the reference's Fortran shapes and lower bounds
 * (column-major, i fastest, variables outermost).  Variable indices l are
 * 1-based as in the reference.  Each routine names the reference lines it
 * restates.  Compile the parity build with -ffp-contract=off.
 */
#include "fest_oracle.h"
#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* ---- SST constants (global/global_sst.f90:6-16) ------------------------ */
static const double sigma_k1 = 0.85, sigma_k2 = 1.0, sigma_w1 = 0.5,
                    sigma_w2 = 0.856, beta1 = 0.075, beta2 = 0.0828,
                    bstar = 0.09, kappa_sst = 0.41, a1_sst = 0.31;

/* ---- Spalart-Allmaras constants (global/global_sa.f90:6-22); the
 * parameter powers cv1**3 and cw3**6 are folded by the compiler to the
 * correctly rounded values pow gives */
static const double cb1 = 0.1355, cb2 = 0.6220, cw2 = 0.3, cw3 = 2.0, cv1 = 7.1,
                    sigma_sa = 2. / 3., kappa_sa = 0.41;
#define CW1_SA ((cb1 / (kappa_sa * kappa_sa)) + ((1 + cb2) / sigma_sa))
/* x**6 as gfortran expands an integer power: x2 = x*x, x4 = x2*x2, x4*x2 */
static inline double pow6(double x) {
  double x2 = x * x, x4 = x2 * x2;
  return x4 * x2;
}

/* ---- k-kL constants (global/global_kkl.f90); cmu**0.25 and cmu**0.75
 * are the correctly rounded powers a compiler folds them to */
static const double kkl_zeta1 = 1.2, kkl_zeta2 = 0.97, kkl_zeta3 = 0.13, kkl_sigma_k = 1.0,
                    kkl_sigma_phi = 1.0, kkl_cmu = 0.09, kkl_kappa = 0.41, kkl_c11 = 10.0, kkl_c12 = 1.3,
                    kkl_cd1 = 4.7;

struct fo_block {
  fest_extent d;
  fest_flow flow;
  fest_scheme sc;
  fest_bc bc;
  int n_grad;
  int ppm_flag;
  double c1, c2, c3;
  int *mF, *mG, *mH; /* make_{F,G,H}_flux_zero(1:imx) etc */
  double *a[FO_NARRAYS];
  long sz[FO_NARRAYS];
};

/* ---- generic strided views ---------------------------------------------- */
typedef struct {
  double *p;
  int lo0, lo1, lo2;
  int n0, n1, n2;
  size_t nn;
} V;

static inline double *at(V a, int i, int j, int k, int l) {
  return a.p + ((size_t)(k - a.lo2) * a.n1 + (size_t)(j - a.lo1)) * a.n0 +
         (size_t)(i - a.lo0) + a.nn * (size_t)(l - 1);
}
static V mkv(double *p, int lo0, int lo1, int lo2, int n0, int n1, int n2) {
  V v;
  v.p = p; v.lo0 = lo0; v.lo1 = lo1; v.lo2 = lo2;
  v.n0 = n0; v.n1 = n1; v.n2 = n2;
  v.nn = (size_t)n0 * n1 * n2;
  return v;
}
/* AoS view of 4-double records (faces {A,nx,ny,nz}, cells {vol,cx,cy,cz}) */
typedef struct {
  double *p;
  int n0, n1;
} R4;
static inline double *r4(R4 a, int i, int j, int k) {
  return a.p + 4 * (((size_t)(k + 2) * a.n1 + (size_t)(j + 2)) * a.n0 + (size_t)(i + 2));
}

#define IMX (b->d.imx)
#define JMX (b->d.jmx)
#define KMX (b->d.kmx)
#define NV (b->d.n_var)

static V vqp(fo_block *b) { return mkv(b->a[FO_QP], -2, -2, -2, IMX + 5, JMX + 5, KMX + 5); }
static V vpad(fo_block *b, int id) { return mkv(b->a[id], -2, -2, -2, IMX + 5, JMX + 5, KMX + 5); }
static R4 vcells(fo_block *b) { R4 r = {b->a[FO_CELLS], IMX + 5, JMX + 5}; return r; }
static R4 vfaces(fo_block *b, int dir) {
  R4 r;
  r.p = b->a[FO_IFACES + dir];
  r.n0 = IMX + 5 + (dir == 0);
  r.n1 = JMX + 5 + (dir == 1);
  return r;
}
/* face-state arrays of direction dir (face_interpolant.f90:43-54) */
static V vfs(fo_block *b, int id, int dir) {
  int f0 = dir == 0, f1 = dir == 1, f2 = dir == 2;
  return mkv(b->a[id], 1 - f0, 1 - f1, 1 - f2, IMX - 1 + 3 * f0, JMX - 1 + 3 * f1,
             KMX - 1 + 3 * f2);
}
/* flux arrays F/G/H (scheme.f90:52-60), lower bound 1 */
static V vflux(fo_block *b, int dir) {
  return mkv(b->a[FO_F + dir], 1, 1, 1, IMX - 1 + (dir == 0), JMX - 1 + (dir == 1),
             KMX - 1 + (dir == 2));
}
static V vres(fo_block *b) { return mkv(b->a[FO_RES], 1, 1, 1, IMX - 1, JMX - 1, KMX - 1); }
static V vgrad(fo_block *b, int c) { return mkv(b->a[FO_GX + c], 0, 0, 0, IMX + 1, JMX + 1, KMX + 1); }
static V vdt(fo_block *b) { return mkv(b->a[FO_DT], 1, 1, 1, IMX - 1, JMX - 1, KMX - 1); }

/* Fortran intrinsics with the reference's semantics */
static inline double fsign(double a, double bb) { return copysign(fabs(a), bb); }
static inline double fmax2(double a, double bb) { return a > bb ? a : bb; }
static inline double fmin2(double a, double bb) { return a < bb ? a : bb; }
/* max(0, 1-floor(|M|)) of ausm.f90:70 etc: 1 for |M|<1, else 0 */
static inline double subsonic(double M) {
  double f = floor(fabs(M));
  double v = 1.0 - f;
  return v > 0.0 ? v : 0.0;
}

static int g_threads = 1;
int fo_set_threads(int n) {
  int old = g_threads;
  g_threads = n < 1 ? 1 : n;
  return old;
}
#ifdef _OPENMP
#define OMP_FOR _Pragma("omp parallel for collapse(2) schedule(static) num_threads(g_threads)")
#else
#define OMP_FOR
#endif

/* ======================================================================== */
fo_block *fo_create(const fest_extent *d, const fest_flow *flow,
                    const fest_scheme *scheme, const fest_bc *bc) {
  fo_block *b = (fo_block *)calloc(1, sizeof(fo_block));
  b->d = *d;
  b->flow = *flow;
  b->sc = *scheme;
  b->bc = *bc;
  int imx = d->imx, jmx = d->jmx, kmx = d->kmx, n = d->n_var;
  long P = (long)(imx + 5) * (jmx + 5) * (kmx + 5);
  long N = (long)(imx - 1) * (jmx - 1) * (kmx - 1);
  long Ng = (long)(imx + 1) * (jmx + 1) * (kmx + 1);
  /* get_n_grad (gradients.f90:229-270): LCTM2015 adds the intermittency's */
  b->n_grad = scheme->turbulence == FEST_TURB_NONE ? 4 : scheme->turbulence == FEST_TURB_SA ? 5 : 6;
  if (scheme->transition == FEST_TRANSITION_LCTM2015) b->n_grad += 1;
  b->sz[FO_QP] = P * n;
  b->sz[FO_TEMP] = P;
  b->sz[FO_NODES] = (long)(imx + 6) * (jmx + 6) * (kmx + 6) * 3;
  b->sz[FO_CELLS] = P * 4;
  b->sz[FO_IFACES] = (long)(imx + 6) * (jmx + 5) * (kmx + 5) * 4;
  b->sz[FO_JFACES] = (long)(imx + 5) * (jmx + 6) * (kmx + 5) * 4;
  b->sz[FO_KFACES] = (long)(imx + 5) * (jmx + 5) * (kmx + 6) * 4;
  b->sz[FO_XL] = b->sz[FO_XR] = (long)(imx + 2) * (jmx - 1) * (kmx - 1) * n;
  b->sz[FO_YL] = b->sz[FO_YR] = (long)(imx - 1) * (jmx + 2) * (kmx - 1) * n;
  b->sz[FO_ZL] = b->sz[FO_ZR] = (long)(imx - 1) * (jmx - 1) * (kmx + 2) * n;
  b->sz[FO_PDIF] = Ng;
  b->sz[FO_F] = (long)imx * (jmx - 1) * (kmx - 1) * n;
  b->sz[FO_G] = (long)(imx - 1) * jmx * (kmx - 1) * n;
  b->sz[FO_H] = (long)(imx - 1) * (jmx - 1) * kmx * n;
  b->sz[FO_RES] = N * n;
  b->sz[FO_GX] = b->sz[FO_GY] = b->sz[FO_GZ] = Ng * b->n_grad;
  b->sz[FO_MU] = b->sz[FO_MUT] = b->sz[FO_F1] = b->sz[FO_DIST] = P;
  b->sz[FO_DT] = N;
  b->sz[FO_USTORE] = P * n;
  b->sz[FO_RSTORE] = N * n;
  for (int id = 0; id < FO_NARRAYS; ++id)
    b->a[id] = (double *)calloc((size_t)(b->sz[id] > 0 ? b->sz[id] : 1), sizeof(double));
  /* setup_viscosity: mu = mu_ref (viscosity.f90:565) */
  for (long p = 0; p < P; ++p) b->a[FO_MU][p] = flow->mu_ref;
  /* setup_bc: c1,c2,c3 and flux masks (bc.f90:48-66) */
  b->c2 = 1 + scheme->accur;
  b->c3 = 0.5 * scheme->accur;
  b->c1 = b->c2 - b->c3;
  b->mF = (int *)malloc(sizeof(int) * (imx + 1));
  b->mG = (int *)malloc(sizeof(int) * (jmx + 1));
  b->mH = (int *)malloc(sizeof(int) * (kmx + 1));
  for (int i = 0; i <= imx; ++i) b->mF[i] = 1;
  for (int j = 0; j <= jmx; ++j) b->mG[j] = 1;
  for (int k = 0; k <= kmx; ++k) b->mH[k] = 1;
#define WALLISH(id) ((id) == -5 || (id) == -6 || (id) == -7)
  if (WALLISH(bc->id[0])) b->mF[1] = 0;
  if (WALLISH(bc->id[2])) b->mG[1] = 0;
  if (WALLISH(bc->id[4])) b->mH[1] = 0;
  if (WALLISH(bc->id[1])) b->mF[imx] = 0;
  if (WALLISH(bc->id[3])) b->mG[jmx] = 0;
  if (WALLISH(bc->id[5])) b->mH[kmx] = 0;
  /* ppm_flag (boundary_state_reconstruction.f90:45-47) */
  b->ppm_flag = (scheme->interpolant == FEST_INTERP_PPM || scheme->interpolant == FEST_INTERP_WENO ||
                 scheme->interpolant == FEST_INTERP_WENO_NM);
  for (int f = 0; f < 6; ++f)
    if (bc->id[f] == -7) b->ppm_flag = 1;
  return b;
}

void fo_destroy(fo_block *b) {
  if (!b) return;
  for (int id = 0; id < FO_NARRAYS; ++id) free(b->a[id]);
  free(b->mF); free(b->mG); free(b->mH);
  free(b);
}
double *fo_ptr(fo_block *b, int id) { return (id >= 0 && id < FO_NARRAYS) ? b->a[id] : 0; }
long fo_size(const fo_block *b, int id) { return (id >= 0 && id < FO_NARRAYS) ? b->sz[id] : 0; }
int fo_n_grad(const fo_block *b) { return b->n_grad; }

/* ======================================================================== */
/* grid.f90:137-236 ghost_grid, then geometry.f90:548-580 setup_geometry     */
static double *node(fo_block *b, int i, int j, int k) {
  return b->a[FO_NODES] + 3 * (((size_t)(k + 2) * (JMX + 6) + (size_t)(j + 2)) * (IMX + 6) + (size_t)(i + 2));
}

static double vol_tet(const double *p1, const double *p2, const double *p3, const double *p4) {
  /* geometry.f90:341-362 */
  double v = (p4[0] - p1[0]) * ((p2[1] - p1[1]) * (p3[2] - p1[2]) - (p2[2] - p1[2]) * (p3[1] - p1[1])) +
             (p4[1] - p1[1]) * ((p2[2] - p1[2]) * (p3[0] - p1[0]) - (p2[0] - p1[0]) * (p3[2] - p1[2])) +
             (p4[2] - p1[2]) * ((p2[0] - p1[0]) * (p3[1] - p1[1]) - (p2[1] - p1[1]) * (p3[0] - p1[0]));
  return -v / 6.;
}
static double vol_hex(const double *p[8]) {
  /* geometry.f90:364-436: two 5-tetrahedra splits, the larger one */
  double v1 = 0.;
  v1 = v1 + vol_tet(p[0], p[4], p[7], p[5]);
  v1 = v1 + vol_tet(p[6], p[7], p[5], p[2]);
  v1 = v1 + vol_tet(p[7], p[3], p[0], p[2]);
  v1 = v1 + vol_tet(p[5], p[0], p[2], p[7]);
  v1 = v1 + vol_tet(p[0], p[1], p[5], p[2]);
  double v = 0.;
  v = v + vol_tet(p[1], p[5], p[4], p[6]);
  v = v + vol_tet(p[7], p[4], p[6], p[3]);
  v = v + vol_tet(p[4], p[0], p[1], p[3]);
  v = v + vol_tet(p[6], p[1], p[3], p[4]);
  v = v + vol_tet(p[1], p[2], p[6], p[3]);
  return fmax2(v, v1);
}

void fo_setup_geometry(fo_block *b) {
  int imx = IMX, jmx = JMX, kmx = KMX;
  /* ghost_grid: I, then J, then K, each over the full other ranges */
  for (int k = -2; k <= kmx + 3; ++k)
    for (int j = -2; j <= jmx + 3; ++j)
      for (int c = 0; c < 3; ++c) {
        node(b, 0, j, k)[c] = 2 * node(b, 1, j, k)[c] - node(b, 2, j, k)[c];
        node(b, -1, j, k)[c] = 2 * node(b, 0, j, k)[c] - node(b, 1, j, k)[c];
        node(b, -2, j, k)[c] = 2 * node(b, -1, j, k)[c] - node(b, 0, j, k)[c];
        node(b, imx + 1, j, k)[c] = 2 * node(b, imx, j, k)[c] - node(b, imx - 1, j, k)[c];
        node(b, imx + 2, j, k)[c] = 2 * node(b, imx + 1, j, k)[c] - node(b, imx, j, k)[c];
        node(b, imx + 3, j, k)[c] = 2 * node(b, imx + 2, j, k)[c] - node(b, imx + 1, j, k)[c];
      }
  for (int k = -2; k <= kmx + 3; ++k)
    for (int i = -2; i <= imx + 3; ++i)
      for (int c = 0; c < 3; ++c) {
        node(b, i, 0, k)[c] = 2 * node(b, i, 1, k)[c] - node(b, i, 2, k)[c];
        node(b, i, -1, k)[c] = 2 * node(b, i, 0, k)[c] - node(b, i, 1, k)[c];
        node(b, i, -2, k)[c] = 2 * node(b, i, -1, k)[c] - node(b, i, 0, k)[c];
        node(b, i, jmx + 1, k)[c] = 2 * node(b, i, jmx, k)[c] - node(b, i, jmx - 1, k)[c];
        node(b, i, jmx + 2, k)[c] = 2 * node(b, i, jmx + 1, k)[c] - node(b, i, jmx, k)[c];
        node(b, i, jmx + 3, k)[c] = 2 * node(b, i, jmx + 2, k)[c] - node(b, i, jmx + 1, k)[c];
      }
  for (int j = -2; j <= jmx + 3; ++j)
    for (int i = -2; i <= imx + 3; ++i)
      for (int c = 0; c < 3; ++c) {
        node(b, i, j, 0)[c] = 2 * node(b, i, j, 1)[c] - node(b, i, j, 2)[c];
        node(b, i, j, -1)[c] = 2 * node(b, i, j, 0)[c] - node(b, i, j, 1)[c];
        node(b, i, j, -2)[c] = 2 * node(b, i, j, -1)[c] - node(b, i, j, 0)[c];
        node(b, i, j, kmx + 1)[c] = 2 * node(b, i, j, kmx)[c] - node(b, i, j, kmx - 1)[c];
        node(b, i, j, kmx + 2)[c] = 2 * node(b, i, j, kmx + 1)[c] - node(b, i, j, kmx)[c];
        node(b, i, j, kmx + 3)[c] = 2 * node(b, i, j, kmx + 2)[c] - node(b, i, j, kmx + 1)[c];
      }
  /* compute_face_area_vectors (geometry.f90:236-314) */
  for (int dir = 0; dir < 3; ++dir) {
    R4 fa = vfaces(b, dir);
    int ie = imx + 2 + (dir == 0), je = jmx + 2 + (dir == 1), ke = kmx + 2 + (dir == 2);
    for (int k = -2; k <= ke; ++k)
      for (int j = -2; j <= je; ++j)
        for (int i = -2; i <= ie; ++i) {
          const double *a0, *a1, *b0, *b1;
          if (dir == 0) {
            a1 = node(b, i, j + 1, k + 1); a0 = node(b, i, j, k);
            b1 = node(b, i, j, k + 1); b0 = node(b, i, j + 1, k);
          } else if (dir == 1) {
            a1 = node(b, i + 1, j, k + 1); a0 = node(b, i, j, k);
            b1 = node(b, i + 1, j, k); b0 = node(b, i, j, k + 1);
          } else {
            a1 = node(b, i + 1, j + 1, k); a0 = node(b, i, j, k);
            b1 = node(b, i, j + 1, k); b0 = node(b, i + 1, j, k);
          }
          double d1x = a1[0] - a0[0], d1y = a1[1] - a0[1], d1z = a1[2] - a0[2];
          double d2x = b1[0] - b0[0], d2y = b1[1] - b0[1], d2z = b1[2] - b0[2];
          double *f = r4(fa, i, j, k);
          f[1] = 0.5 * (d1y * d2z - d1z * d2y);
          f[2] = 0.5 * (d1z * d2x - d1x * d2z);
          f[3] = 0.5 * (d1x * d2y - d1y * d2x);
          /* compute_face_areas (geometry.f90:200-216) */
          f[0] = sqrt(f[1] * f[1] + f[2] * f[2] + f[3] * f[3]);
        }
    /* pole faces: zero area (geometry.f90:211-216) */
    int idmin = b->bc.id[2 * dir], idmax = b->bc.id[2 * dir + 1];
    int nmax = (dir == 0 ? imx : dir == 1 ? jmx : kmx);
    for (int k = -2; k <= ke; ++k)
      for (int j = -2; j <= je; ++j)
        for (int i = -2; i <= ie; ++i) {
          int c = dir == 0 ? i : dir == 1 ? j : k;
          if ((idmin == -7 && c <= 1) || (idmax == -7 && c >= nmax)) r4(fa, i, j, k)[0] = 0.;
        }
    /* normalize_face_normals (geometry.f90:50-110) */
    for (int k = -2; k <= ke; ++k)
      for (int j = -2; j <= je; ++j)
        for (int i = -2; i <= ie; ++i) {
          double *f = r4(fa, i, j, k);
          if (f[0] != 0.) {
            f[1] = f[1] / f[0];
            f[2] = f[2] / f[0];
            f[3] = f[3] / f[0];
          }
        }
  }
  if (b->bc.id[0] == -7) { /* geometry.f90:96-106 */
    R4 fa = vfaces(b, 0);
    for (int k = -2; k <= kmx + 2; ++k)
      for (int j = -2; j <= jmx + 2; ++j)
        for (int i = -2; i <= 1; ++i) {
          r4(fa, i, j, k)[1] = r4(fa, 2, j, k)[1];
          r4(fa, i, j, k)[2] = r4(fa, 2, j, k)[2];
        }
  }
  /* compute_volumes (geometry.f90:441-487) */
  R4 cl = vcells(b);
  for (int k = -2; k <= kmx + 2; ++k)
    for (int j = -2; j <= jmx + 2; ++j)
      for (int i = -2; i <= imx + 2; ++i) r4(cl, i, j, k)[0] = 1.;
  for (int k = 0; k <= kmx; ++k)
    for (int j = 0; j <= jmx; ++j)
      for (int i = 0; i <= imx; ++i) {
        const double *p[8] = {node(b, i, j, k),         node(b, i + 1, j, k),
                              node(b, i + 1, j + 1, k), node(b, i, j + 1, k),
                              node(b, i, j, k + 1),     node(b, i + 1, j, k + 1),
                              node(b, i + 1, j + 1, k + 1), node(b, i, j + 1, k + 1)};
        r4(cl, i, j, k)[0] = vol_hex(p);
      }
  /* compute_ghost_cell_centroid (geometry.f90:491-545) */
  for (int k = -2; k <= kmx + 2; ++k)
    for (int j = -2; j <= jmx + 2; ++j)
      for (int i = -2; i <= imx + 2; ++i)
        for (int c = 0; c < 3; ++c) {
          double s = node(b, i, j, k)[c] + node(b, i + 1, j, k)[c] + node(b, i + 1, j + 1, k)[c] +
                     node(b, i + 1, j + 1, k + 1)[c] + node(b, i + 1, j, k + 1)[c] +
                     node(b, i, j + 1, k)[c] + node(b, i, j + 1, k + 1)[c] + node(b, i, j, k + 1)[c];
          r4(cl, i, j, k)[1 + c] = 0.125 * s;
        }
}

/* wall_dist.f90:84-131 */
void fo_find_wall_dist(fo_block *b, const double *w, int nw) {
  int imx = IMX, jmx = JMX, kmx = KMX;
  int n0 = imx + 6, n1 = jmx + 6, n2 = kmx + 6;
  double *nd = (double *)malloc(sizeof(double) * (size_t)n0 * n1 * n2);
#define ND(i, j, k) nd[((size_t)((k) + 2) * n1 + (size_t)((j) + 2)) * n0 + (size_t)((i) + 2)]
#ifdef _OPENMP
#pragma omp parallel for collapse(2) num_threads(g_threads)
#endif
  for (int k = -2; k <= kmx + 3; ++k)
    for (int j = -2; j <= jmx + 3; ++j)
      for (int i = -2; i <= imx + 3; ++i) {
        const double *p = node(b, i, j, k);
        double dmin = 1.e+20;
        for (int n = 0; n < nw; ++n) {
          double dx = w[3 * n] - p[0], dy = w[3 * n + 1] - p[1], dz = w[3 * n + 2] - p[2];
          double cur = sqrt(dx * dx + dy * dy + dz * dz);
          dmin = fmin2(dmin, cur);
        }
        ND(i, j, k) = dmin;
      }
  V dist = vpad(b, FO_DIST);
  for (int k = -2; k <= kmx + 2; ++k)
    for (int j = -2; j <= jmx + 2; ++j)
      for (int i = -2; i <= imx + 2; ++i)
        *at(dist, i, j, k, 1) =
            0.125 * (ND(i, j, k) + ND(i, j + 1, k) + ND(i, j + 1, k + 1) + ND(i, j, k + 1) +
                     ND(i + 1, j, k + 1) + ND(i + 1, j, k) + ND(i + 1, j + 1, k) +
                     ND(i + 1, j + 1, k + 1));
#undef ND
  free(nd);
}

/* ======================================================================== */
/* boundary conditions                                                       */
/* ghost / interior cell of face f, layer l (1..3), tangential (ta, tb)     */
static void ghost_ijk(const fo_block *b, int f, int l, int ta, int tb, int *i, int *j, int *k) {
  switch (f) {
  case 0: *i = 1 - l; *j = ta; *k = tb; break;
  case 1: *i = b->d.imx + l - 1; *j = ta; *k = tb; break;
  case 2: *i = ta; *j = 1 - l; *k = tb; break;
  case 3: *i = ta; *j = b->d.jmx + l - 1; *k = tb; break;
  case 4: *i = ta; *j = tb; *k = 1 - l; break;
  default: *i = ta; *j = tb; *k = b->d.kmx + l - 1; break;
  }
}
static void inner_ijk(const fo_block *b, int f, int m, int ta, int tb, int *i, int *j, int *k) {
  switch (f) {
  case 0: *i = m; *j = ta; *k = tb; break;
  case 1: *i = b->d.imx - m; *j = ta; *k = tb; break;
  case 2: *i = ta; *j = m; *k = tb; break;
  case 3: *i = ta; *j = b->d.jmx - m; *k = tb; break;
  case 4: *i = ta; *j = tb; *k = m; break;
  default: *i = ta; *j = tb; *k = b->d.kmx - m; break;
  }
}
static void tang_range(const fo_block *b, int f, int *na, int *nb) {
  int dir = f / 2;
  *na = (dir == 0 ? b->d.jmx : b->d.imx) - 1;
  *nb = (dir == 2 ? b->d.jmx : b->d.kmx) - 1;
}

static double *Qp(fo_block *b, int i, int j, int k, int l) { return at(vqp(b), i, j, k, l); }

enum { CP_ANTI, CP_FLAT, CP_SYMM };
/* copy_bc.f90:58-131 copy3 */
static void copy3(fo_block *b, int l, int type, int f) {
  double a1, a2, a3;
  int il[3];
  if (type == CP_ANTI) { a1 = 1.; a2 = -1.; a3 = 0.; il[0] = 1; il[1] = 2; il[2] = 3; }
  else if (type == CP_FLAT) { a1 = 1.; a2 = 1.; a3 = 0.; il[0] = 1; il[1] = 1; il[2] = 1; }
  else { a1 = b->c1; a2 = b->c2; a3 = b->c3; il[0] = 1; il[1] = 2; il[2] = 3; }
  int na, nb;
  tang_range(b, f, &na, &nb);
  for (int L = 1; L <= 3; ++L)
    for (int tb = 1; tb <= nb; ++tb)
      for (int ta = 1; ta <= na; ++ta) {
        int gi, gj, gk, ii, ij, ik, ji, jj, jk;
        ghost_ijk(b, f, L, ta, tb, &gi, &gj, &gk);
        inner_ijk(b, f, il[L - 1], ta, tb, &ii, &ij, &ik);
        inner_ijk(b, f, il[L - 1] + 1, ta, tb, &ji, &jj, &jk);
        *Qp(b, gi, gj, gk, l) = (a2 * *Qp(b, ii, ij, ik, l) - a3 * *Qp(b, ji, jj, jk, l)) / a1;
      }
}
/* bc_primitive.f90:484-525 fix */
static void fixv(fo_block *b, int l, double val, int f) {
  int na, nb;
  tang_range(b, f, &na, &nb);
  for (int L = 1; L <= 3; ++L)
    for (int tb = 1; tb <= nb; ++tb)
      for (int ta = 1; ta <= na; ++ta) {
        int gi, gj, gk;
        ghost_ijk(b, f, L, ta, tb, &gi, &gj, &gk);
        *Qp(b, gi, gj, gk, l) = val;
      }
}
static int is_sst(const fo_block *b) {
  return b->sc.turbulence == FEST_TURB_SST || b->sc.turbulence == FEST_TURB_SST2003;
}
static int is_sa(const fo_block *b) { return b->sc.turbulence == FEST_TURB_SA; }
static int is_kkl(const fo_block *b) { return b->sc.turbulence == FEST_TURB_KKL; }
static int is_turb(const fo_block *b) { return b->sc.turbulence != FEST_TURB_NONE; }
/* LCTM2015 (scheme%transition 'lctm2015' on SST): the eighth variable is
 * the intermittency */
static int is_lctm(const fo_block *b) { return b->sc.transition == FEST_TRANSITION_LCTM2015; }

/* bc_primitive.f90:1778-1945 temp_based_density */
static void temp_based_density(fo_block *b, int f) {
  double T = b->bc.fixed_wall_temperature[f], R = b->flow.R_gas, gm = b->flow.gm;
  if (T < 0.0 || T > 1.0) {
    int na, nb;
    tang_range(b, f, &na, &nb);
    for (int tb = 1; tb <= nb; ++tb)
      for (int ta = 1; ta <= na; ++ta) {
        int i1, j1, k1;
        inner_ijk(b, f, 1, ta, tb, &i1, &j1, &k1);
        if (T < 0.0) {
          double p = *Qp(b, i1, j1, k1, 5), rho = *Qp(b, i1, j1, k1, 1);
          double stag = (p / (R * rho)) * (1 + (0.5 * (gm - 1.) * gm * p / rho));
          for (int L = 1; L <= 3; ++L) {
            int gi, gj, gk;
            ghost_ijk(b, f, L, ta, tb, &gi, &gj, &gk);
            *Qp(b, gi, gj, gk, 1) = *Qp(b, gi, gj, gk, 5) / (R * stag);
          }
        } else {
          for (int L = 1; L <= 3; ++L) {
            int gi, gj, gk, ii, ij, ik;
            ghost_ijk(b, f, L, ta, tb, &gi, &gj, &gk);
            inner_ijk(b, f, L, ta, tb, &ii, &ij, &ik);
            double Ti = *Qp(b, ii, ij, ik, 5) / (R * *Qp(b, ii, ij, ik, 1));
            *Qp(b, gi, gj, gk, 1) = *Qp(b, gi, gj, gk, 5) / (R * (2 * T - Ti));
          }
        }
      }
  } else {
    copy3(b, 1, CP_SYMM, f);
  }
}

/* bc_primitive.f90:564-643 set_omega_at_wall */
static void set_omega_at_wall(fo_block *b, int f) {
  double R = b->flow.R_gas, mu_ref = b->flow.mu_ref, Tr = b->flow.T_ref, S = b->flow.Sutherland_temp;
  V dist = vpad(b, FO_DIST);
  int na, nb;
  tang_range(b, f, &na, &nb);
  for (int L = 1; L <= 3; ++L)
    for (int tb = 1; tb <= nb; ++tb)
      for (int ta = 1; ta <= na; ++ta) {
        int g0i, g0j, g0k, i1, j1, k1, gi, gj, gk, ii, ij, ik;
        ghost_ijk(b, f, 1, ta, tb, &g0i, &g0j, &g0k);
        inner_ijk(b, f, 1, ta, tb, &i1, &j1, &k1);
        ghost_ijk(b, f, L, ta, tb, &gi, &gj, &gk);
        inner_ijk(b, f, L, ta, tb, &ii, &ij, &ik);
        double Tf = 0.5 * ((*Qp(b, g0i, g0j, g0k, 5) / *Qp(b, g0i, g0j, g0k, 1)) +
                           (*Qp(b, i1, j1, k1, 5) / *Qp(b, i1, j1, k1, 1))) / R;
        double mu = mu_ref * pow(Tf / Tr, 1.5) * ((Tr + S) / (Tf + S));
        double rho = 0.5 * (*Qp(b, g0i, g0j, g0k, 1) + *Qp(b, i1, j1, k1, 1));
        double dd = 2 * *at(dist, i1, j1, k1, 1);
        *Qp(b, gi, gj, gk, 7) = 120 * mu / (rho * beta1 * (dd * dd)) - *Qp(b, ii, ij, ik, 7);
      }
}

/* FT_bc.f90:15-107 flow_tangency (j/k faces reflect with I-face normals) */
static void flow_tangency(fo_block *b, int f) {
  R4 If = vfaces(b, 0), own = vfaces(b, f / 2);
  int na, nb;
  tang_range(b, f, &na, &nb);
  for (int tb = 1; tb <= nb; ++tb)
    for (int ta = 1; ta <= na; ++ta) {
      int fi, fj, fk; /* boundary face index: 1 or imx on the normal axis */
      inner_ijk(b, f, 1, ta, tb, &fi, &fj, &fk);
      if (f == 1) fi = b->d.imx;
      if (f == 3) fj = b->d.jmx;
      if (f == 5) fk = b->d.kmx;
      if (f == 0) fi = 1;
      if (f == 2) fj = 1;
      if (f == 4) fk = 1;
      const double *fn = r4(own, fi, fj, fk);
      const double *fr = r4(If, fi, fj, fk);
      for (int L = 1; L <= 3; ++L) {
        int gi, gj, gk, ii, ij, ik;
        ghost_ijk(b, f, L, ta, tb, &gi, &gj, &gk);
        inner_ijk(b, f, L, ta, tb, &ii, &ij, &ik);
        double u = *Qp(b, ii, ij, ik, 2), v = *Qp(b, ii, ij, ik, 3), w = *Qp(b, ii, ij, ik, 4);
        double dot = u * fn[1] + v * fn[2] + w * fn[3];
        *Qp(b, gi, gj, gk, 2) = u - (2.0 * dot * fr[1]);
        *Qp(b, gi, gj, gk, 3) = v - (2.0 * dot * fr[2]);
        *Qp(b, gi, gj, gk, 4) = w - (2.0 * dot * fr[3]);
      }
    }
}

/* far_field (bc_primitive.f90:645-1234) and total_pressure (1237-1776):
 * Riemann invariants on layer 1, then layers 2,3 := layer 1 on the full
 * plane.  For SST the last (j,k) cell in loop order decides whether the
 * turbulence ghosts end flat-copied or fixed. */
static void riemann_face(fo_block *b, int f, int total_pressure) {
  double gm = b->flow.gm;
  R4 fa = vfaces(b, f / 2);
  int na, nb;
  tang_range(b, f, &na, &nb);
  int last_positive = 0;
  double sgn = (f % 2 == 0) ? -1.0 : 1.0;
  for (int tb = 1; tb <= nb; ++tb)
    for (int ta = 1; ta <= na; ++ta) {
      int ii, ij, ik, gi, gj, gk, fi, fj, fk;
      inner_ijk(b, f, 1, ta, tb, &ii, &ij, &ik);
      ghost_ijk(b, f, 1, ta, tb, &gi, &gj, &gk);
      fi = ii; fj = ij; fk = ik;
      if (f == 1) fi = b->d.imx;
      if (f == 3) fj = b->d.jmx;
      if (f == 5) fk = b->d.kmx;
      const double *fn = r4(fa, fi, fj, fk);
      double nx = sgn * fn[1], ny = sgn * fn[2], nz = sgn * fn[3];
      double u = *Qp(b, ii, ij, ik, 2), v = *Qp(b, ii, ij, ik, 3), w = *Qp(b, ii, ij, ik, 4);
      double uf = b->flow.x_speed_inf, vf = b->flow.y_speed_inf, wf = b->flow.z_speed_inf;
      double pI = *Qp(b, ii, ij, ik, 5), rI = *Qp(b, ii, ij, ik, 1);
      double cexp = sqrt(gm * pI / rI);
      double cinf = sqrt(gm * b->flow.pressure_inf / b->flow.density_inf);
      double Unexp = u * nx + v * ny + w * nz;
      double Uninf = uf * nx + vf * ny + wf * nz;
      double Rinf = Uninf - 2 * cinf / (gm - 1.);
      double Rexp = Unexp + 2 * cexp / (gm - 1.);
      double Unb = 0.5 * (Rexp + Rinf);
      double Cb = 0.25 * (gm - 1.) * (Rexp - Rinf);
      double s;
      if (Unb > 0.) {
        double vd = Unb - Unexp;
        *Qp(b, gi, gj, gk, 2) = u + vd * nx;
        *Qp(b, gi, gj, gk, 3) = v + vd * ny;
        *Qp(b, gi, gj, gk, 4) = w + vd * nz;
        if (!total_pressure) {
          s = pI / pow(rI, gm);
          double rg = pow(Cb * Cb / (gm * s), 1. / (gm - 1.));
          *Qp(b, gi, gj, gk, 1) = rg;
          *Qp(b, gi, gj, gk, 5) = (rg * Cb * Cb / gm);
        }
        last_positive = 1;
      } else {
        double vd = Unb - Uninf;
        *Qp(b, gi, gj, gk, 2) = uf + vd * nx;
        *Qp(b, gi, gj, gk, 3) = vf + vd * ny;
        *Qp(b, gi, gj, gk, 4) = wf + vd * nz;
        if (!total_pressure) {
          s = b->flow.pressure_inf / pow(b->flow.density_inf, gm);
          double rg = pow(Cb * Cb / (gm * s), 1. / (gm - 1.));
          *Qp(b, gi, gj, gk, 1) = rg;
          *Qp(b, gi, gj, gk, 5) = (rg * Cb * Cb / gm);
        }
        last_positive = 0;
      }
      if (total_pressure) {
        double ug = *Qp(b, gi, gj, gk, 2), vg = *Qp(b, gi, gj, gk, 3), wg = *Qp(b, gi, gj, gk, 4);
        double Mb = sqrt(ug * ug + vg * vg + wg * wg) / Cb;
        double pg = b->bc.fixed_Tpressure[f] / pow((1 + 0.5 * (gm - 1.) * Mb * Mb), gm / (gm - 1.));
        *Qp(b, gi, gj, gk, 5) = pg;
        *Qp(b, gi, gj, gk, 1) = gm * pg / (Cb * Cb);
      }
    }
  if (is_sst(b) && na > 0 && nb > 0) {
    if (last_positive) { copy3(b, 6, CP_FLAT, f); copy3(b, 7, CP_FLAT, f); }
    else { fixv(b, 6, b->bc.fixed_tk[f], f); fixv(b, 7, b->bc.fixed_tw[f], f); }
  }
  if (is_sa(b) && na > 0 && nb > 0) {
    if (last_positive) copy3(b, 6, CP_FLAT, f);
    else fixv(b, 6, b->bc.fixed_tv[f], f);
  }
  if (is_kkl(b) && na > 0 && nb > 0) {
    if (last_positive) { copy3(b, 6, CP_FLAT, f); copy3(b, 7, CP_FLAT, f); }
    else { fixv(b, 6, b->bc.fixed_tk[f], f); fixv(b, 7, b->bc.fixed_tkl[f], f); }
  }
  if (is_lctm(b) && na > 0 && nb > 0) {
    if (last_positive) copy3(b, 8, CP_FLAT, f);
    else fixv(b, 8, b->bc.fixed_tgm[f], f);
  }
  /* plane copy of layer 1 into layers 2 and 3, all tangential indices */
  int imx = IMX, jmx = JMX, kmx = KMX;
  for (int l = 1; l <= NV; ++l)
    for (int L = 2; L <= 3; ++L) {
      if (f / 2 == 0) {
        int g1 = (f == 0) ? 0 : imx, gL = (f == 0) ? 1 - L : imx + L - 1;
        for (int k = -2; k <= kmx + 2; ++k)
          for (int j = -2; j <= jmx + 2; ++j) *Qp(b, gL, j, k, l) = *Qp(b, g1, j, k, l);
      } else if (f / 2 == 1) {
        int g1 = (f == 2) ? 0 : jmx, gL = (f == 2) ? 1 - L : jmx + L - 1;
        for (int k = -2; k <= kmx + 2; ++k)
          for (int i = -2; i <= imx + 2; ++i) *Qp(b, i, gL, k, l) = *Qp(b, i, g1, k, l);
      } else {
        int g1 = (f == 4) ? 0 : kmx, gL = (f == 4) ? 1 - L : kmx + L - 1;
        for (int j = -2; j <= jmx + 2; ++j)
          for (int i = -2; i <= imx + 2; ++i) *Qp(b, i, j, gL, l) = *Qp(b, i, j, g1, l);
      }
    }
}

/* bc_primitive.f90:1948-1978 periodic_bc (single block, full planes) */
static void periodic_bc(fo_block *b, int f) {
  int imx = IMX, jmx = JMX, kmx = KMX;
  for (int l = 1; l <= NV; ++l)
    for (int L = 0; L < 3; ++L) {
      for (int k = -2; k <= kmx + 2; ++k)
        for (int j = -2; j <= jmx + 2; ++j)
          for (int i = -2; i <= imx + 2; ++i) {
            int src, dst;
            if (f == 0) { dst = -2 + L; src = imx - 3 + L; if (i != dst) continue; *Qp(b, i, j, k, l) = *Qp(b, src, j, k, l); }
            else if (f == 1) { dst = imx + L; src = 1 + L; if (i != dst) continue; *Qp(b, i, j, k, l) = *Qp(b, src, j, k, l); }
            else if (f == 2) { dst = -2 + L; src = jmx - 3 + L; if (j != dst) continue; *Qp(b, i, j, k, l) = *Qp(b, i, src, k, l); }
            else if (f == 3) { dst = jmx + L; src = 1 + L; if (j != dst) continue; *Qp(b, i, j, k, l) = *Qp(b, i, src, k, l); }
            else if (f == 4) { dst = -2 + L; src = kmx - 3 + L; if (k != dst) continue; *Qp(b, i, j, k, l) = *Qp(b, i, j, src, l); }
            else { dst = kmx + L; src = 1 + L; if (k != dst) continue; *Qp(b, i, j, k, l) = *Qp(b, i, j, src, l); }
          }
    }
}

/* the block a face's interface pairs with: itself when partner_block is the
 * block's own number (the reference's process_id), else the one block of
 * the list with that number (NULL if there is none or more than one) */
static fo_block *partner_of(fo_block **blocks, int nblocks, fo_block *b, int f) {
  const int pb = b->bc.partner_block[f];
  if (pb == b->bc.block_id) return b;
  fo_block *found = NULL;
  for (int m = 0; m < nblocks; ++m)
    if (blocks[m] != b && blocks[m]->bc.block_id == pb) {
      if (found) return NULL;
      found = blocks[m];
    }
  return found;
}
/* apply_interface's receive loops (interface1.f90:96-464): the sender packs
 * its layer l with j fastest over its own ranges; the receiver unpacks it
 * over the ranges of change_map_to_particular_range (mapping.f90:159-236),
 * each direction forwards or backwards, the two loops swapped by
 * dir_switch.  Returns the partner's position (pa, pb) of column (ta, tb). */
static void interface_pos(int orient, int na, int nb, int ta, int tb, int *pa, int *pb) {
  const int a = (orient & 1) ? na - ta : ta - 1;
  const int c = (orient & 2) ? nb - tb : tb - 1;
  if (orient & 4) { *pa = 1 + c; *pb = 1 + a; }
  else { *pa = 1 + a; *pb = 1 + c; }
}

/* interface1.f90:96-700 apply_interface / apply_periodic_bc: every
 * receiving face is packed from a snapshot of its partner's interior
 * layers 1..3 taken before any ghost is written. */
void fo_apply_interface(fo_block **blocks, int nblocks) {
  int cnt = 0;
  double **buf = (double **)calloc((size_t)nblocks * 6, sizeof(double *));
  for (int bi = 0; bi < nblocks; ++bi) {
    fo_block *b = blocks[bi];
    for (int f = 0; f < 6; ++f) {
      int id = b->bc.id[f];
      if (!(id == -10 || id >= 0)) continue;
      fo_block *p = partner_of(blocks, nblocks, b, f);
      if (!p) continue;
      int pf = b->bc.partner_face[f];
      int orient = b->bc.partner_orient[f];
      int na, nb, pa, pb;
      tang_range(b, f, &na, &nb);
      tang_range(p, pf, &pa, &pb);
      if (orient & 4) { int t = pa; pa = pb; pb = t; }
      if (na != pa || nb != pb) continue;
      double *s = (double *)malloc(sizeof(double) * (size_t)3 * (na > 0 ? na : 1) * (nb > 0 ? nb : 1) * b->d.n_var);
      size_t c = 0;
      for (int l = 1; l <= b->d.n_var; ++l)
        for (int L = 1; L <= 3; ++L)
          for (int tb = 1; tb <= nb; ++tb)
            for (int ta = 1; ta <= na; ++ta) {
              int ii, ij, ik, qa, qb;
              interface_pos(orient, na, nb, ta, tb, &qa, &qb);
              inner_ijk(p, pf, L, qa, qb, &ii, &ij, &ik);
              s[c++] = *Qp(p, ii, ij, ik, l);
            }
      buf[bi * 6 + f] = s;
      ++cnt;
    }
  }
  for (int bi = 0; bi < nblocks; ++bi) {
    fo_block *b = blocks[bi];
    for (int f = 0; f < 6; ++f) {
      double *s = buf[bi * 6 + f];
      if (!s) continue;
      int na, nb;
      tang_range(b, f, &na, &nb);
      size_t c = 0;
      for (int l = 1; l <= b->d.n_var; ++l)
        for (int L = 1; L <= 3; ++L)
          for (int tb = 1; tb <= nb; ++tb)
            for (int ta = 1; ta <= na; ++ta) {
              int gi, gj, gk;
              ghost_ijk(b, f, L, ta, tb, &gi, &gj, &gk);
              *Qp(b, gi, gj, gk, l) = s[c++];
            }
      free(s);
    }
  }
  free(buf);
  (void)cnt;
}

/* bc_primitive.f90:209-224 corner / edge averaging */
static void corners(fo_block *b) {
  int imx = IMX, jmx = JMX, kmx = KMX;
  for (int l = 1; l <= NV; ++l) {
#define Q(i, j, k) (*Qp(b, (i), (j), (k), l))
    for (int i = -2; i <= imx + 2; ++i) Q(i, 0, 0) = 0.33 * (Q(i, 1, 1) + Q(i, 0, 1) + Q(i, 1, 0));
    for (int i = -2; i <= imx + 2; ++i) Q(i, 0, kmx) = 0.33 * (Q(i, 1, kmx - 1) + Q(i, 0, kmx - 1) + Q(i, 1, kmx));
    for (int i = -2; i <= imx + 2; ++i) Q(i, jmx, 0) = 0.33 * (Q(i, jmx - 1, 1) + Q(i, jmx, 1) + Q(i, jmx - 1, 0));
    for (int i = -2; i <= imx + 2; ++i)
      Q(i, jmx, kmx) = 0.33 * (Q(i, jmx - 1, kmx - 1) + Q(i, jmx, kmx - 1) + Q(i, jmx - 1, kmx));
    for (int k = -2; k <= kmx + 2; ++k) Q(imx, 0, k) = 0.33 * (Q(imx - 1, 1, k) + Q(imx - 1, 0, k) + Q(imx, 1, k));
    for (int k = -2; k <= kmx + 2; ++k) Q(0, 0, k) = 0.33 * (Q(1, 1, k) + Q(1, 0, k) + Q(0, 1, k));
    for (int k = -2; k <= kmx + 2; ++k) Q(0, jmx, k) = 0.33 * (Q(1, jmx - 1, k) + Q(1, jmx, k) + Q(0, jmx - 1, k));
    for (int k = -2; k <= kmx + 2; ++k)
      Q(imx, jmx, k) = 0.33 * (Q(imx - 1, jmx - 1, k) + Q(imx - 1, jmx, k) + Q(imx, jmx - 1, k));
    Q(0, 0, 0) = 0.33 * (Q(1, 0, 0) + Q(0, 1, 0) + Q(0, 0, 1));
    Q(imx, 0, 0) = 0.33 * (Q(imx - 1, 0, 0) + Q(imx, 1, 0) + Q(imx, 0, 1));
    Q(0, jmx, 0) = 0.33 * (Q(1, jmx, 0) + Q(0, jmx - 1, 0) + Q(0, jmx, 1));
    Q(0, 0, kmx) = 0.33 * (Q(1, 0, kmx) + Q(0, 1, kmx) + Q(0, 0, kmx - 1));
    Q(imx, jmx, 0) = 0.33 * (Q(imx - 1, jmx, 0) + Q(imx, jmx - 1, 0) + Q(imx, jmx, 1));
    Q(imx, 0, kmx) = 0.33 * (Q(imx - 1, 0, kmx) + Q(imx, 1, kmx) + Q(imx, 0, kmx - 1));
    Q(0, jmx, kmx) = 0.33 * (Q(1, jmx, kmx) + Q(0, jmx - 1, kmx) + Q(0, jmx, kmx - 1));
    Q(imx, jmx, kmx) = 0.33 * (Q(imx - 1, jmx, kmx) + Q(imx, jmx - 1, kmx) + Q(imx, jmx, kmx - 1));
#undef Q
  }
}

/* bc_primitive.f90:55-226 populate_ghost_primitive */
int fo_populate_ghost_primitive(fo_block *b, int it) {
  int sst = is_sst(b), sa = is_sa(b), kkl = is_kkl(b), lctm = is_lctm(b);
  for (int f = 0; f < 6; ++f) {
    switch (b->bc.id[f]) {
    case -1: /* supersonic_inlet */
      if (it <= 2) {
        fixv(b, 1, b->bc.fixed_density[f], f);
        fixv(b, 2, b->bc.fixed_x_speed[f], f);
        fixv(b, 3, b->bc.fixed_y_speed[f], f);
        fixv(b, 4, b->bc.fixed_z_speed[f], f);
        fixv(b, 5, b->bc.fixed_pressure[f], f);
        if (sst) { fixv(b, 6, b->bc.fixed_tk[f], f); fixv(b, 7, b->bc.fixed_tw[f], f); }
        if (sa) fixv(b, 6, b->bc.fixed_tv[f], f);
        if (kkl) { fixv(b, 6, b->bc.fixed_tk[f], f); fixv(b, 7, b->bc.fixed_tkl[f], f); }
        if (lctm) fixv(b, 8, b->bc.fixed_tgm[f], f); /* bc_primitive.f90:258-264, 339-345 */
      }
      break;
    case -2: /* supersonic_outlet */
    case -7: /* pole */
      for (int l = 1; l <= NV; ++l) copy3(b, l, CP_FLAT, f);
      break;
    case -3: /* subsonic_inlet */
      if (it <= 2) {
        fixv(b, 1, b->bc.fixed_density[f], f);
        fixv(b, 2, b->bc.fixed_x_speed[f], f);
        fixv(b, 3, b->bc.fixed_y_speed[f], f);
        fixv(b, 4, b->bc.fixed_z_speed[f], f);
        if (sst) { fixv(b, 6, b->bc.fixed_tk[f], f); fixv(b, 7, b->bc.fixed_tw[f], f); }
        if (sa) fixv(b, 6, b->bc.fixed_tv[f], f);
        if (kkl) { fixv(b, 6, b->bc.fixed_tk[f], f); fixv(b, 7, b->bc.fixed_tkl[f], f); }
        if (lctm) fixv(b, 8, b->bc.fixed_tgm[f], f); /* bc_primitive.f90:258-264, 339-345 */
      }
      copy3(b, 5, CP_FLAT, f);
      break;
    case -4: /* subsonic_outlet */
      for (int l = 1; l <= 4; ++l) copy3(b, l, CP_FLAT, f);
      if (it <= 2) fixv(b, 5, b->bc.fixed_pressure[f], f);
      if (sst) { copy3(b, 6, CP_FLAT, f); copy3(b, 7, CP_FLAT, f); }
      if (sa) copy3(b, 6, CP_FLAT, f);
      if (kkl) { copy3(b, 6, CP_FLAT, f); copy3(b, 7, CP_FLAT, f); }
      if (lctm) copy3(b, 8, CP_FLAT, f); /* bc_primitive.f90:384-387 */
      break;
    case -5: /* wall: pressure symm, temp_based_density, no_slip */
      copy3(b, 5, CP_SYMM, f);
      temp_based_density(b, f);
      copy3(b, 2, CP_ANTI, f);
      copy3(b, 3, CP_ANTI, f);
      copy3(b, 4, CP_ANTI, f);
      if (sst) { copy3(b, 6, CP_ANTI, f); set_omega_at_wall(b, f); }
      if (sa) copy3(b, 6, CP_ANTI, f);
      if (kkl) { copy3(b, 6, CP_ANTI, f); copy3(b, 7, CP_ANTI, f); }
      if (lctm) copy3(b, 8, CP_FLAT, f); /* flat at the wall too (bc_primitive.f90:554-557) */
      break;
    case -6: /* slip_wall */
      copy3(b, 1, CP_SYMM, f);
      copy3(b, 5, CP_SYMM, f);
      if (sst) { copy3(b, 6, CP_SYMM, f); copy3(b, 7, CP_SYMM, f); }
      if (sa) copy3(b, 6, CP_SYMM, f);
      if (kkl) { copy3(b, 6, CP_SYMM, f); copy3(b, 7, CP_SYMM, f); }
      if (lctm) copy3(b, 8, CP_FLAT, f); /* flat, not symm (bc_primitive.f90:436-439) */
      flow_tangency(b, f);
      break;
    case -8: riemann_face(b, f, 0); break;
    case -9: periodic_bc(b, f); break;
    case -11: riemann_face(b, f, 1); break;
    default: break; /* -10 and >= 0: interface, handled by fo_apply_interface */
    }
  }
  corners(b);
  return FEST_OK;
}

void fo_compute_temperature(fo_block *b) {
  V q = vqp(b), T = vpad(b, FO_TEMP);
  for (int k = -2; k <= KMX + 2; ++k)
    for (int j = -2; j <= JMX + 2; ++j)
      for (int i = -2; i <= IMX + 2; ++i)
        *at(T, i, j, k, 1) = *at(q, i, j, k, 5) / (b->flow.R_gas * *at(q, i, j, k, 1));
}

/* ======================================================================== */
/* face reconstruction                                                       */
static inline double limiter(const fo_block *b, double r) {
  if (b->sc.limiter == FEST_LIMITER_VAN_ALBADA) return ((r * r) + r) / ((r * r) + 1.0);
  const double alpha = 2. / 3.;
  return fmax2(0., fmin2(fmin2(2 * r, alpha * (r - 1.0) + 1.0), 2.));
}

/* muscl.f90:115-200 compute_face_state */
static void muscl_dir(fo_block *b, int dir, int lam, int turb) {
  V q = vqp(b), L = vfs(b, FO_XL + 2 * dir, dir), R = vfs(b, FO_XR + 2 * dir, dir);
  int ii = dir == 0, jj = dir == 1, kk = dir == 2;
  const double phi = 1.0, kappa = 1. / 3., eps = 1e-14;
  for (int l = 1; l <= NV; ++l) {
    int sw = (l >= 6) ? turb : lam;
    OMP_FOR
    for (int k = 1 - kk; k <= KMX - 1 + kk; ++k)
      for (int j = 1 - jj; j <= JMX - 1 + jj; ++j)
        for (int i = 1 - ii; i <= IMX - 1 + ii; ++i) {
          double qc = *at(q, i, j, k, l);
          double fd = *at(q, i + ii, j + jj, k + kk, l) - qc;
          double bd = qc - *at(q, i - ii, j - jj, k - kk, l);
          double r = fd / (bd + fsign(eps, bd));
          double psi1 = limiter(b, r);
          r = bd / (fd + fsign(eps, fd));
          double psi2 = limiter(b, r);
          psi1 = (1 - (1 - psi1) * sw);
          psi2 = (1 - (1 - psi2) * sw);
          *at(L, i + ii, j + jj, k + kk, l) = qc + 0.25 * phi * (((1. - kappa) * psi1 * bd) + ((1. + kappa) * psi2 * fd));
          *at(R, i, j, k, l) = qc - 0.25 * phi * (((1. + kappa) * psi1 * bd) + ((1. - kappa) * psi2 * fd));
        }
  }
}

/* muscl.f90:37-112 / ppm.f90:109-186 pressure_based_switching */
static void pressure_switch(fo_block *b, int dir) {
  V q = vqp(b), L = vfs(b, FO_XL + 2 * dir, dir), R = vfs(b, FO_XR + 2 * dir, dir);
  V pd = mkv(b->a[FO_PDIF], 0, 0, 0, IMX + 1, JMX + 1, KMX + 1);
  int i_f = dir == 0, j_f = dir == 1, k_f = dir == 2;
  int imx = IMX, jmx = JMX, kmx = KMX;
  for (int k = 1; k <= kmx - 1; ++k)
    for (int j = 1; j <= jmx - 1; ++j)
      for (int i = 1; i <= imx - 1; ++i) {
        double pd2 = fabs(*at(q, i + i_f, j + j_f, k + k_f, 5) - *at(q, i - i_f, j - j_f, k - k_f, 5));
        *at(pd, i, j, k, 1) = 1 - (pd2 / (pd2 + b->flow.pressure_inf));
      }
  /* ghost copies: low side then high side of the switched direction */
  for (int k = 1; k <= kmx - 1; ++k)
    for (int j = 1; j <= jmx - 1; ++j)
      for (int i = 1; i <= imx - 1; ++i) {
        int c = dir == 0 ? i : dir == 1 ? j : k;
        if (c != 1) continue;
        *at(pd, i - i_f, j - j_f, k - k_f, 1) = *at(pd, i, j, k, 1);
      }
  for (int k = 1; k <= kmx - 1; ++k)
    for (int j = 1; j <= jmx - 1; ++j)
      for (int i = 1; i <= imx - 1; ++i) {
        int c = dir == 0 ? i : dir == 1 ? j : k, n = dir == 0 ? imx : dir == 1 ? jmx : kmx;
        if (c != n - 1) continue;
        *at(pd, i + i_f, j + j_f, k + k_f, 1) = *at(pd, i, j, k, 1);
      }
  for (int k = 1; k <= kmx - (1 - k_f); ++k)
    for (int j = 1; j <= jmx - (1 - j_f); ++j)
      for (int i = 1; i <= imx - (1 - i_f); ++i)
        for (int l = 1; l <= NV; ++l) {
          double qm = *at(q, i - i_f, j - j_f, k - k_f, l), qc = *at(q, i, j, k, l);
          *at(L, i, j, k, l) = qm + (*at(pd, i - i_f, j - j_f, k - k_f, 1) * (*at(L, i, j, k, l) - qm));
          *at(R, i, j, k, l) = qc - (*at(pd, i, j, k, 1) * (qc - *at(R, i, j, k, l)));
        }
}

/* weno.f90:24-93 and weno_NM.f90:21-120 compute_face_states */
static void weno_dir(fo_block *b, int dir, int nm) {
  V q = vqp(b), L = vfs(b, FO_XL + 2 * dir, dir), R = vfs(b, FO_XR + 2 * dir, dir);
  R4 cl = vcells(b);
  int i_f = dir == 0, j_f = dir == 1, k_f = dir == 2;
  const double eps = 1e-6;
  double g[3] = {1.0 / 10.0, 6.0 / 10.0, 3.0 / 10.0};
  for (int l = 1; l <= NV; ++l) {
    OMP_FOR
    for (int k = 1 - k_f; k <= KMX - 1 + k_f; ++k)
      for (int j = 1 - j_f; j <= JMX - 1 + j_f; ++j)
        for (int i = 1 - i_f; i <= IMX - 1 + i_f; ++i) {
          double U[5], P[3], B[3], w[3];
          for (int s = -2; s <= 2; ++s) U[s + 2] = *at(q, i + s * i_f, j + s * j_f, k + s * k_f, l);
#define u(s) U[(s) + 2]
          if (!nm) {
            P[0] = (2.0 * u(-2) - 7.0 * u(-1) + 11.0 * u(0)) / 6.0;
            P[1] = (-1.0 * u(-1) + 5.0 * u(0) + 2.0 * u(1)) / 6.0;
            P[2] = (2.0 * u(0) + 5.0 * u(1) - 1.0 * u(2)) / 6.0;
            double t1, t2;
            t1 = u(-2) - 2.0 * u(-1) + u(0); t2 = u(-2) - 4.0 * u(-1) + 3.0 * u(0);
            B[0] = (13.0 / 12.0) * (t1 * t1) + (1.0 / 4.0) * (t2 * t2);
            t1 = u(-1) - 2.0 * u(0) + u(1); t2 = u(-1) - u(1);
            B[1] = (13.0 / 12.0) * (t1 * t1) + (1.0 / 4.0) * (t2 * t2);
            t1 = u(0) - 2.0 * u(1) + u(2); t2 = 3.0 * u(0) - 4.0 * u(1) + u(2);
            B[2] = (13.0 / 12.0) * (t1 * t1) + (1.0 / 4.0) * (t2 * t2);
            for (int m = 0; m < 3; ++m) { double e = eps + B[m]; w[m] = g[m] / (e * e); }
            *at(L, i + i_f, j + j_f, k + k_f, l) =
                (0.0 + w[0] * P[0] + w[1] * P[1] + w[2] * P[2]) / (0.0 + w[0] + w[1] + w[2]);
            P[0] = (2.0 * u(2) - 7.0 * u(1) + 11.0 * u(0)) / 6.0;
            P[1] = (-1.0 * u(1) + 5.0 * u(0) + 2.0 * u(-1)) / 6.0;
            P[2] = (2.0 * u(0) + 5.0 * u(-1) - 1.0 * u(-2)) / 6.0;
            { double e; e = eps + B[2]; w[0] = g[0] / (e * e);
              e = eps + B[1]; w[1] = g[1] / (e * e);
              e = eps + B[0]; w[2] = g[2] / (e * e); }
            *at(R, i, j, k, l) = (0.0 + w[0] * P[0] + w[1] * P[1] + w[2] * P[2]) / (0.0 + w[0] + w[1] + w[2]);
          } else {
            double vol[5];
            for (int s = -2; s <= 2; ++s) vol[s + 2] = r4(cl, i + s * i_f, j + s * j_f, k + s * k_f)[0];
#define vv(s) vol[(s) + 2]
            double a12 = vv(2) / (vv(1) + vv(2)), a01 = vv(1) / (vv(0) + vv(1));
            double a10 = vv(0) / (vv(-1) + vv(0)), a21 = vv(-1) / (vv(-2) + vv(-1));
#undef vv
            double U01 = (1.0 - a01) * u(0) + a01 * u(1);
            double U12 = (1.0 - a12) * u(1) + a12 * u(2);
            double U10 = (1.0 - a10) * u(-1) + a10 * u(0);
            double U21 = (1.0 - a21) * u(-2) + a21 * u(-1);
            double U00 = u(-1) + (1.0 - a21) * (u(-1) - u(-2));
            double U11 = u(1) + a12 * (u(1) - u(2));
            double t1, t2;
            P[0] = (6.0 * u(0) - 1.0 * U10 - 2.0 * U00) / 3.0;
            P[1] = (-1.0 * U10 + 2.0 * u(0) + 2.0 * U01) / 3.0;
            P[2] = (2.0 * U01 + 2.0 * u(1) - 1.0 * U12) / 3.0;
            t1 = 2 * U10 - 2.0 * U00; t2 = 4 * u(0) - 2.0 * U10 - 2.0 * U00;
            B[0] = (13.0 / 12.0) * (t1 * t1) + (1.0 / 4.0) * (t2 * t2);
            t1 = 2 * U10 - 4.0 * u(0) + 2 * U01; t2 = -2 * U10 + 2.0 * U01;
            B[1] = (13.0 / 12.0) * (t1 * t1) + (1.0 / 4.0) * (t2 * t2);
            t1 = 2 * U01 - 4.0 * u(1) + 2 * U12; t2 = -6 * U01 + 8.0 * u(1) - 2.0 * U12;
            B[2] = (13.0 / 12.0) * (t1 * t1) + (1.0 / 4.0) * (t2 * t2);
            for (int m = 0; m < 3; ++m) { double e = eps + B[m]; w[m] = g[m] / (e * e); }
            *at(L, i + i_f, j + j_f, k + k_f, l) =
                (0.0 + w[0] * P[0] + w[1] * P[1] + w[2] * P[2]) / (0.0 + w[0] + w[1] + w[2]);
            P[0] = (6.0 * u(0) - 1.0 * U01 - 2.0 * U11) / 3.0;
            P[1] = (-1.0 * U01 + 2.0 * u(0) + 2.0 * U10) / 3.0;
            P[2] = (2.0 * U10 + 2.0 * u(-1) - 1.0 * U21) / 3.0;
            t1 = 2 * U01 - 2.0 * U11; t2 = 4 * u(0) - 2.0 * U01 - 2.0 * U11;
            B[0] = (13.0 / 12.0) * (t1 * t1) + (1.0 / 4.0) * (t2 * t2);
            t1 = 2 * U01 - 4.0 * u(0) + 2 * U10; t2 = -2 * U01 + 2.0 * U10;
            B[1] = (13.0 / 12.0) * (t1 * t1) + (1.0 / 4.0) * (t2 * t2);
            t1 = 2 * U10 - 4.0 * u(-1) + 2 * U21; t2 = -6 * U10 + 8.0 * u(-1) - 2.0 * U21;
            B[2] = (13.0 / 12.0) * (t1 * t1) + (1.0 / 4.0) * (t2 * t2);
            for (int m = 0; m < 3; ++m) { double e = eps + B[m]; w[m] = g[m] / (e * e); }
            *at(R, i, j, k, l) = (0.0 + w[0] * P[0] + w[1] * P[1] + w[2] * P[2]) / (0.0 + w[0] + w[1] + w[2]);
          }
#undef u
        }
  }
}

/* ppm.f90:21-107 compute_face_estimates + remove_extrema */
static void ppm_dir(fo_block *b, int dir, int lim) {
  V q = vqp(b), L = vfs(b, FO_XL + 2 * dir, dir), R = vfs(b, FO_XR + 2 * dir, dir);
  int i_f = dir == 0, j_f = dir == 1, k_f = dir == 2;
  for (int l = 1; l <= NV; ++l)
    for (int k = 1 - k_f; k <= KMX - 1 + 2 * k_f; ++k)
      for (int j = 1 - j_f; j <= JMX - 1 + 2 * j_f; ++j)
        for (int i = 1 - i_f; i <= IMX - 1 + 2 * i_f; ++i) {
          double e = (7. * (*at(q, i, j, k, l) + *at(q, i - i_f, j - j_f, k - k_f, l)) -
                      (*at(q, i + i_f, j + j_f, k + k_f, l) + *at(q, i - 2 * i_f, j - 2 * j_f, k - 2 * k_f, l))) / 12.;
          *at(L, i, j, k, l) = e;
          *at(R, i, j, k, l) = e;
        }
  if (!lim) return;
  for (int l = 1; l <= NV; ++l)
    for (int k = 1 - k_f; k <= KMX - 1 + k_f; ++k)
      for (int j = 1 - j_f; j <= JMX - 1 + j_f; ++j)
        for (int i = 1 - i_f; i <= IMX - 1 + i_f; ++i) {
          double qc = *at(q, i, j, k, l);
          double *lp = at(L, i + i_f, j + j_f, k + k_f, l), *rp = at(R, i, j, k, l);
          if ((*lp - qc) * (qc - *rp) <= 0) {
            *lp = qc;
            *rp = qc;
          } else {
            double dqrl = *lp - *rp;
            double dq6 = 6. * (qc - 0.5 * (*lp + *rp));
            if (dqrl * dq6 > dqrl * dqrl) *rp = 3. * qc - 2. * *lp;
            else if (-dqrl * dqrl > dqrl * dq6) *lp = 3. * qc - 2. * *rp;
          }
        }
}

/* face_interpolant.f90:61-76 first order */
static void first_order_dir(fo_block *b, int dir) {
  V q = vqp(b), L = vfs(b, FO_XL + 2 * dir, dir), R = vfs(b, FO_XR + 2 * dir, dir);
  int i_f = dir == 0, j_f = dir == 1, k_f = dir == 2;
  for (int l = 1; l <= NV; ++l)
    for (int k = 1 - k_f; k <= KMX - 1 + 2 * k_f; ++k)
      for (int j = 1 - j_f; j <= JMX - 1 + 2 * j_f; ++j)
        for (int i = 1 - i_f; i <= IMX - 1 + 2 * i_f; ++i) {
          *at(L, i, j, k, l) = *at(q, i - i_f, j - j_f, k - k_f, l);
          *at(R, i, j, k, l) = *at(q, i, j, k, l);
        }
}

int fo_compute_face_interpolant(fo_block *b) {
  const fest_scheme *s = &b->sc;
  int lam[3] = {s->ilimiter_switch, s->jlimiter_switch, s->klimiter_switch};
  int trb[3] = {s->itlimiter_switch, s->jtlimiter_switch, s->ktlimiter_switch};
  int pb[3] = {s->iPB_switch, s->jPB_switch, s->kPB_switch};
  for (int dir = 0; dir < 3; ++dir) {
    switch (s->interpolant) {
    case FEST_INTERP_NONE: first_order_dir(b, dir); break;
    case FEST_INTERP_MUSCL:
      muscl_dir(b, dir, lam[dir], trb[dir]);
      if (pb[dir] == 1) pressure_switch(b, dir);
      break;
    case FEST_INTERP_PPM:
      ppm_dir(b, dir, lam[dir] == 1);
      if (pb[dir] == 1) pressure_switch(b, dir);
      break;
    case FEST_INTERP_WENO: weno_dir(b, dir, 0); break;
    case FEST_INTERP_WENO_NM: weno_dir(b, dir, 1); break;
    default: return FEST_ERR_ARG;
    }
  }
  return FEST_OK;
}

/* boundary_state_reconstruction.f90:78-412 */
static void bnd_muscl(fo_block *b, int dir, int c, int lam, int turb) {
  V q = vqp(b), L = vfs(b, FO_XL + 2 * dir, dir), R = vfs(b, FO_XR + 2 * dir, dir);
  int ii = dir == 0, jj = dir == 1, kk = dir == 2;
  const double phi = 1.0, kappa = 1. / 3.;
  int na = (dir == 0 ? JMX : IMX) - 1, nb = (dir == 2 ? JMX : KMX) - 1;
  for (int l = 1; l <= NV; ++l) {
    int sw = (l >= 6) ? turb : lam;
    for (int tb = 1; tb <= nb; ++tb)
      for (int ta = 1; ta <= na; ++ta) {
        int i = dir == 0 ? c : ta, j = dir == 0 ? ta : dir == 1 ? c : tb, k = dir == 2 ? c : tb;
        if (dir == 2) { i = ta; j = tb; }
        double qc = *at(q, i, j, k, l);
        double fd = *at(q, i + ii, j + jj, k + kk, l) - qc;
        double bd = qc - *at(q, i - ii, j - jj, k - kk, l);
        double r = fd / bd;
        double psi1 = fmax2(0., fmin2(fmin2(2 * r, (2 + r) / 3.), 2.));
        psi1 = (1 - (1 - psi1) * sw);
        r = bd / fd;
        double psi2 = fmax2(0., fmin2(fmin2(2 * r, (2 + r) / 3.), 2.));
        psi2 = (1 - (1 - psi2) * sw);
        if (psi1 != psi1) psi1 = 2.;
        if (psi2 != psi2) psi2 = 2.;
        *at(L, i + ii, j + jj, k + kk, l) = qc + 0.25 * phi * (((1. - kappa) * psi1 * bd) + ((1. + kappa) * psi2 * fd));
        *at(R, i, j, k, l) = qc - 0.25 * phi * (((1. + kappa) * psi1 * bd) + ((1. - kappa) * psi2 * fd));
      }
  }
}

void fo_reconstruct_boundary_state(fo_block *b) {
  if (b->sc.interpolant == FEST_INTERP_NONE) return;
  const fest_scheme *s = &b->sc;
  int lam[3] = {s->ilimiter_switch, s->jlimiter_switch, s->klimiter_switch};
  int trb[3] = {s->itlimiter_switch, s->jtlimiter_switch, s->ktlimiter_switch};
  V q = vqp(b);
  for (int f = 0; f < 6; ++f) {
    int id = b->bc.id[f];
    if (!(id < 0 && id != -10)) continue;
    int dir = f / 2, hi = f % 2;
    int n = dir == 0 ? IMX : dir == 1 ? JMX : KMX;
    V L = vfs(b, FO_XL + 2 * dir, dir), R = vfs(b, FO_XR + 2 * dir, dir);
    if (b->ppm_flag) bnd_muscl(b, dir, hi ? n - 1 : 1, lam[dir], trb[dir]);
    int na = (dir == 0 ? JMX : IMX) - 1, nb = (dir == 2 ? JMX : KMX) - 1;
    for (int l = 1; l <= NV; ++l)
      for (int tb = 1; tb <= nb; ++tb)
        for (int ta = 1; ta <= na; ++ta) {
          int i, j, k, gi, gj, gk, ci, cj, ck;
          /* face index, cell outside (ghost 0 / n) and cell inside */
          int fc = hi ? n : 1, go = hi ? n : 0, in = hi ? n - 1 : 1;
          if (dir == 0) { i = fc; j = ta; k = tb; gi = go; gj = ta; gk = tb; ci = in; cj = ta; ck = tb; }
          else if (dir == 1) { i = ta; j = fc; k = tb; gi = ta; gj = go; gk = tb; ci = ta; cj = in; ck = tb; }
          else { i = ta; j = tb; k = fc; gi = ta; gj = tb; gk = go; ci = ta; cj = tb; ck = in; }
          double qg = *at(q, gi, gj, gk, l), qi = *at(q, ci, cj, ck, l);
          if (id == -8 || id == -9) {
            *at(L, i, j, k, l) = qg;
            *at(R, i, j, k, l) = qg;
          } else if (!hi) {
            *at(L, i, j, k, l) = 0.5 * (qg + qi);
          } else {
            *at(R, i, j, k, l) = 0.5 * (qi + qg);
          }
        }
  }
}

/* ======================================================================== */
/* convective fluxes                                                         */
static double wall_mask(const fo_block *b, int dir, int i, int j, int k) {
  return dir == 0 ? b->mF[i] : dir == 1 ? b->mG[j] : b->mH[k];
}

/* ausm.f90:16-157, van_leer.f90:17-149, ldfss0.f90:18-164 */
static void flux_ausm_family(const fo_block *b, int kind, const double *qL, const double *qR,
                             const double *fc, double mask, double *Fo) {
  double gm = b->flow.gm;
  int n = b->d.n_var;
  double Fp[8], Fm[8];
  double c = 0.5 * (sqrt(gm * qL[4] / qL[0]) + sqrt(gm * qR[4] / qR[0]));
  double vn = qL[1] * fc[1] + qL[2] * fc[2] + qL[3] * fc[3];
  double ML = vn / c;
  double ap = 0.5 * (1.0 + fsign(1.0, ML));
  double bL = -subsonic(ML);
  double t = 1. + ML;
  double Mp = 0.25 * (t * t);
  double Dp = 0.25 * (t * t) * (2. - ML);
  double cp = (ap * (1.0 + bL) * ML) - bL * Mp;
  double sDp = (ap * (1. + bL)) - (bL * Dp);
  vn = qR[1] * fc[1] + qR[2] * fc[2] + qR[3] * fc[3];
  double MR = vn / c;
  double am = 0.5 * (1.0 - fsign(1.0, MR));
  double bR = -subsonic(MR);
  t = 1. - MR;
  double Mm = -0.25 * (t * t);
  double Dm = 0.25 * (t * t) * (2. + MR);
  double cm = (am * (1.0 + bR) * MR) - bR * Mm;
  double sDm = (am * (1. + bR)) - (bR * Dm);
  if (kind == FEST_FLUX_AUSM) {
    double tc = cp + cm;
    cp = fmax2(0., tc);
    cm = fmin2(0., tc);
  } else if (kind == FEST_FLUX_LDFSS0) {
    double s = sqrt((ML * ML + MR * MR) * 0.5) - 1;
    double Ml = 0.25 * bL * bR * (s * s);
    double Mpl = Ml * (1 - (qL[4] - qR[4]) / (2 * qL[0] * (c * c)));
    double Mml = Ml * (1 - (qL[4] - qR[4]) / (2 * qR[0] * (c * c)));
    cp = cp - Mpl;
    cm = cm + Mml;
  }
  Fp[0] = qL[0] * c * cp;
  Fm[0] = qR[0] * c * cm;
  Fp[0] = Fp[0] * mask;
  Fm[0] = Fm[0] * mask;
  Fp[1] = (Fp[0] * qL[1]) + (sDp * qL[4] * fc[1]);
  Fp[2] = (Fp[0] * qL[2]) + (sDp * qL[4] * fc[2]);
  Fp[3] = (Fp[0] * qL[3]) + (sDp * qL[4] * fc[3]);
  Fp[4] = Fp[0] * ((0.5 * (qL[1] * qL[1] + qL[2] * qL[2] + qL[3] * qL[3])) + ((gm / (gm - 1.)) * qL[4] / qL[0]));
  Fm[1] = (Fm[0] * qR[1]) + (sDm * qR[4] * fc[1]);
  Fm[2] = (Fm[0] * qR[2]) + (sDm * qR[4] * fc[2]);
  Fm[3] = (Fm[0] * qR[3]) + (sDm * qR[4] * fc[3]);
  Fm[4] = Fm[0] * ((0.5 * (qR[1] * qR[1] + qR[2] * qR[2] + qR[3] * qR[3])) + ((gm / (gm - 1.)) * qR[4] / qR[0]));
  for (int l = 5; l < n; ++l) { Fp[l] = Fp[0] * qL[l]; Fm[l] = Fm[0] * qR[l]; }
  for (int l = 0; l < n; ++l) { Fp[l] = Fp[l] * fc[0]; Fm[l] = Fm[l] * fc[0]; Fo[l] = Fp[l] + Fm[l]; }
}

/* slau.f90:19-207, ausmP.f90:22-201, ausmUP.f90:19-219 */
static void flux_mass_family(const fo_block *b, int kind, const double *qL, const double *qR,
                             const double *fc, double mask, double *Fo) {
  double gm = b->flow.gm;
  int n = b->d.n_var;
  double rL = qL[0], uL = qL[1], vL = qL[2], wL = qL[3], pL = qL[4];
  double rR = qR[0], uR = qR[1], vR = qR[2], wR = qR[3], pR = qR[4];
  double HL = (0.5 * (uL * uL + vL * vL + wL * wL)) + ((gm / (gm - 1.)) * pL / rL);
  double HR = (0.5 * (uR * uR + vR * vR + wR * wR)) + ((gm / (gm - 1.)) * pR / rR);
  double nx = fc[1], ny = fc[2], nz = fc[3];
  double mass, pbar;
  if (kind == FEST_FLUX_SLAU) {
    double cL = sqrt(gm * pL / rL), cR = sqrt(gm * pR / rR);
    double C = 0.5 * (cL + cR);
    double delp = pR - pL;
    double VnL = uL * nx + vL * ny + wL * nz;
    double VnR = uR * nx + vR * ny + wR * nz;
    double ML = VnL / C, MR = VnR / C;
    double aL = fmax2(0.0, 1.0 - floor(fabs(ML)));
    double aR = fmax2(0.0, 1.0 - floor(fabs(MR)));
    double betaL = (1.0 - aL) * 0.5 * (1.0 + fsign(1.0, ML)) + (aL) * 0.25 * (2.0 - ML) * ((ML + 1.0) * (ML + 1.0));
    double betaR = (1.0 - aR) * 0.5 * (1.0 - fsign(1.0, MR)) + (aR) * 0.25 * (2.0 + MR) * ((MR - 1.0) * (MR - 1.0));
    double vt = sqrt(0.5 * ((uL * uL) + (vL * vL) + (wL * wL) + (uR * uR) + (vR * vR) + (wR * wR)));
    double Mcap = fmin2(1.0, vt / C);
    double Xi = (1.0 - Mcap) * (1.0 - Mcap);
    double Vnabs = (rL * fabs(VnL) + rR * fabs(VnR)) / (rL + rR);
    double fnG = -1.0 * fmax2(fmin2(ML, 0.0), -1.0) * fmin2(fmax2(MR, 0.0), 1.0);
    pbar = 0.5 * ((pL + pR) + (betaL - betaR) * (pL - pR) + (1.0 - Xi) * (betaL + betaR - 1.0) * (pL + pR));
    double VnabsL = (1.0 - fnG) * Vnabs + fnG * fabs(VnL);
    double VnabsR = (1.0 - fnG) * Vnabs + fnG * fabs(VnR);
    mass = 0.5 * ((rL * (VnL + VnabsL) + rR * (VnR - VnabsR)) - (Xi * delp / C));
  } else {
    double VnL = uL * nx + vL * ny + wL * nz;
    double VnR = uR * nx + vR * ny + wR * nz;
    double cs = sqrt(2.0 * (gm - 1.0) * (0.5 * (HL + HR)) / (gm + 1.0));
    double cL, cR;
    if (kind == FEST_FLUX_AUSMP) {
      cL = cs * cs / (fmax2(cs, fabs(VnL)));
      cR = cs * cs / (fmax2(cs, fabs(VnR)));
    } else {
      cL = cs * cs / (fmax2(cs, VnL));
      cR = cs * cs / (fmax2(cs, -VnR));
    }
    double C = fmin2(cL, cR);
    double ML = VnL / C, MR = VnR / C;
    double Mb = 0, fna = 0, alfa = 0.1875;
    if (kind == FEST_FLUX_AUSMUP) {
      Mb = sqrt(0.5 * ((VnL * VnL) + (VnR * VnR)) / (C * C));
      double Mo = sqrt(fmin2(1.0, fmax2(Mb * Mb, b->flow.MInf * b->flow.MInf)));
      fna = Mo * (2.0 - Mo);
      alfa = 3.0 * (-4.0 + (5.0 * fna * fna)) / 16.0;
    }
    double aL = subsonic(ML), aR = subsonic(MR);
    double t;
    t = 1.0 + ML;
    double FmL = (0.5 * (1.0 + fsign(1.0, ML)) * (1.0 - aL) * ML) + aL * 0.25 * (t * t);
    double betaL = (0.5 * (1.0 + fsign(1.0, ML)) * (1.0 - aL)) + aL * 0.25 * (t * t) * (2.0 - ML);
    t = 1.0 - MR;
    double FmR = (0.5 * (1.0 - fsign(1.0, MR)) * (1.0 - aR) * MR) - aR * 0.25 * (t * t);
    double betaR = (0.5 * (1.0 - fsign(1.0, MR)) * (1.0 - aR)) + aR * 0.25 * (t * t) * (2.0 + MR);
    t = ML * ML - 1.0;
    FmL = FmL + aL * 0.1250 * (t * t);
    betaL = betaL + aL * alfa * (t * t) * ML;
    t = MR * MR - 1.0;
    FmR = FmR - aR * 0.1250 * (t * t);
    betaR = betaR - aR * alfa * (t * t) * MR;
    double Mface = FmL + FmR;
    pbar = betaL * pL + betaR * pR;
    if (kind == FEST_FLUX_AUSMUP) {
      const double Kp = 0.25, Ku = 0.75, sigma = 1.0;
      double Pu = -Ku * betaL * betaR * (rL + rR) * fna * C * (VnR - VnL);
      double Mp = -2.0 * Kp * fmax2(1.0 - (sigma * Mb * Mb), 0.0) * (pR - pL) / (fna * (rL + rR) * C * C);
      Mface = FmL + FmR + Mp;
      pbar = betaL * pL + betaR * pR + Pu;
    }
    if (Mface > 0.0) mass = Mface * C * rL;
    else mass = Mface * C * rR;
  }
  mass = mass * mask;
  double Fp[8], Fm[8];
  Fp[0] = 0.5 * (mass + fabs(mass));
  Fp[1] = Fp[0] * uL; Fp[2] = Fp[0] * vL; Fp[3] = Fp[0] * wL; Fp[4] = Fp[0] * HL;
  Fm[0] = 0.5 * (mass - fabs(mass));
  Fm[1] = Fm[0] * uR; Fm[2] = Fm[0] * vR; Fm[3] = Fm[0] * wR; Fm[4] = Fm[0] * HR;
  for (int l = 5; l < n; ++l) { Fp[l] = Fp[0] * qL[l]; Fm[l] = Fm[0] * qR[l]; }
  for (int l = 0; l < n; ++l) Fo[l] = Fp[l] + Fm[l];
  Fo[1] = Fo[1] + (pbar * nx);
  Fo[2] = Fo[2] + (pbar * ny);
  Fo[3] = Fo[3] + (pbar * nz);
  for (int l = 0; l < n; ++l) Fo[l] = Fo[l] * fc[0];
}

int fo_compute_fluxes(fo_block *b) {
  int kind = b->sc.scheme_name;
  int n = NV, err = FEST_OK;
  for (int dir = 0; dir < 3; ++dir) {
    V Fl = vflux(b, dir), L = vfs(b, FO_XL + 2 * dir, dir), R = vfs(b, FO_XR + 2 * dir, dir);
    R4 fa = vfaces(b, dir);
    if (dir == 2 && KMX == 2) {
      memset(b->a[FO_H], 0, sizeof(double) * (size_t)b->sz[FO_H]);
      continue;
    }
    int i_f = dir == 0, j_f = dir == 1, k_f = dir == 2;
    OMP_FOR
    for (int k = 1; k <= KMX - 1 + k_f; ++k)
      for (int j = 1; j <= JMX - 1 + j_f; ++j)
        for (int i = 1; i <= IMX - 1 + i_f; ++i) {
          double qL[8], qR[8], Fo[8];
          for (int l = 1; l <= n; ++l) { qL[l - 1] = *at(L, i, j, k, l); qR[l - 1] = *at(R, i, j, k, l); }
          const double *fc = r4(fa, i, j, k);
          double m = wall_mask(b, dir, i, j, k);
          if (kind == FEST_FLUX_AUSM || kind == FEST_FLUX_VAN_LEER || kind == FEST_FLUX_LDFSS0)
            flux_ausm_family(b, kind, qL, qR, fc, m, Fo);
          else
            flux_mass_family(b, kind, qL, qR, fc, m, Fo);
          for (int l = 1; l <= n; ++l) *at(Fl, i, j, k, l) = Fo[l - 1];
        }
    for (long p = 0; p < b->sz[FO_F + dir]; ++p)
      if (b->a[FO_F + dir][p] != b->a[FO_F + dir][p]) err = FEST_ERR_NAN;
  }
  return err;
}

/* scheme.f90:111-141 */
void fo_compute_residue(fo_block *b) {
  V r = vres(b), F = vflux(b, 0), G = vflux(b, 1), H = vflux(b, 2);
  for (int l = 1; l <= NV; ++l) {
    OMP_FOR
    for (int k = 1; k <= KMX - 1; ++k)
      for (int j = 1; j <= JMX - 1; ++j)
        for (int i = 1; i <= IMX - 1; ++i)
          *at(r, i, j, k, l) = (*at(F, i + 1, j, k, l) - *at(F, i, j, k, l)) +
                               (*at(G, i, j + 1, k, l) - *at(G, i, j, k, l)) +
                               (*at(H, i, j, k + 1, l) - *at(H, i, j, k, l));
  }
}

/* ======================================================================== */
/* gradients (gradients.f90:276-482) */
static void gradient_G(fo_block *b, V grad, int lg, V var, int lv, int c) {
  R4 If = vfaces(b, 0), Jf = vfaces(b, 1), Kf = vfaces(b, 2), cl = vcells(b);
  OMP_FOR
  for (int k = 0; k <= KMX; ++k)
    for (int j = 0; j <= JMX; ++j)
      for (int i = 0; i <= IMX; ++i) {
        double v0 = *at(var, i, j, k, lv);
        const double *fi0 = r4(If, i, j, k), *fj0 = r4(Jf, i, j, k), *fk0 = r4(Kf, i, j, k);
        const double *fi1 = r4(If, i + 1, j, k), *fj1 = r4(Jf, i, j + 1, k), *fk1 = r4(Kf, i, j, k + 1);
        double s = -((*at(var, i - 1, j, k, lv) + v0) * fi0[1 + c] * fi0[0]);
        s = s - (*at(var, i, j - 1, k, lv) + v0) * fj0[1 + c] * fj0[0];
        s = s - (*at(var, i, j, k - 1, lv) + v0) * fk0[1 + c] * fk0[0];
        s = s + (*at(var, i + 1, j, k, lv) + v0) * fi1[1 + c] * fi1[0];
        s = s + (*at(var, i, j + 1, k, lv) + v0) * fj1[1 + c] * fj1[0];
        s = s + (*at(var, i, j, k + 1, lv) + v0) * fk1[1 + c] * fk1[0];
        *at(grad, i, j, k, lg) = s / (2 * r4(cl, i, j, k)[0]);
      }
}

/* gradients.f90:486-676 apply_gradient_bc */
static void gradient_bc(fo_block *b) {
  V q = vqp(b), T = vpad(b, FO_TEMP);
  V g[3] = {vgrad(b, 0), vgrad(b, 1), vgrad(b, 2)};
  R4 cl = vcells(b);
  int ng = b->n_grad;
  for (int f = 0; f < 6; ++f) {
    if (!(b->bc.id[f] < 0)) continue;
    int dir = f / 2, hi = f % 2;
    R4 fa = vfaces(b, dir);
    int n = dir == 0 ? IMX : dir == 1 ? JMX : KMX;
    double sig = hi ? -1 : 1;
    double Tw = b->bc.fixed_wall_temperature[f];
    int na = (dir == 0 ? JMX : IMX) - 1, nb = (dir == 2 ? JMX : KMX) - 1;
    for (int tb = 1; tb <= nb; ++tb)
      for (int ta = 1; ta <= na; ++ta) {
        int fcx = hi ? n : 1;
        int i, j, k;
        if (dir == 0) { i = fcx; j = ta; k = tb; }
        else if (dir == 1) { i = ta; j = fcx; k = tb; }
        else { i = ta; j = tb; k = fcx; }
        /* ghost G = face - il, interior I = face - iu */
        int il = hi ? 0 : 1, iu = hi ? 1 : 0;
        int Gi = i - (dir == 0) * il, Gj = j - (dir == 1) * il, Gk = k - (dir == 2) * il;
        int Ii = i - (dir == 0) * iu, Ij = j - (dir == 1) * iu, Ik = k - (dir == 2) * iu;
        const double *fc = r4(fa, i, j, k);
        double nx = fc[1], ny = fc[2], nz = fc[3];
        double vI = r4(cl, Ii, Ij, Ik)[0];
        double cc[3] = {fc[0] * nx / vI, fc[0] * ny / vI, fc[0] * nz / vI};
        double TI = *at(T, Ii, Ij, Ik, 1), TG = *at(T, Gi, Gj, Gk, 1);
        for (int l = 1; l <= ng; ++l) {
          double qI = *at(q, Ii, Ij, Ik, l + 1), qG = *at(q, Gi, Gj, Gk, l + 1);
          for (int c = 0; c < 3; ++c) *at(g[c], Gi, Gj, Gk, l) = sig * (qI - qG) * cc[c];
        }
        for (int c = 0; c < 3; ++c) *at(g[c], Gi, Gj, Gk, 4) = sig * (TI - TG) * cc[c];
        if (b->bc.id[f] == -5 && (Tw < 1. && Tw >= 0.))
          for (int c = 0; c < 3; ++c) *at(g[c], Gi, Gj, Gk, 4) = -*at(g[c], Ii, Ij, Ik, 4);
        for (int l = 1; l <= ng; ++l) {
          double gx = *at(g[0], Ii, Ij, Ik, l), gy = *at(g[1], Ii, Ij, Ik, l), gz = *at(g[2], Ii, Ij, Ik, l);
          double dot = (gx * nx) + (gy * ny) + (gz * nz);
          *at(g[0], Gi, Gj, Gk, l) = *at(g[0], Gi, Gj, Gk, l) + (gx - dot * nx);
          *at(g[1], Gi, Gj, Gk, l) = *at(g[1], Gi, Gj, Gk, l) + (gy - dot * ny);
          *at(g[2], Gi, Gj, Gk, l) = *at(g[2], Gi, Gj, Gk, l) + (gz - dot * nz);
        }
      }
  }
}

int fo_evaluate_all_gradients(fo_block *b) {
  V q = vqp(b), T = vpad(b, FO_TEMP);
  V g[3] = {vgrad(b, 0), vgrad(b, 1), vgrad(b, 2)};
  int ncomp = (KMX > 2) ? 3 : 2;
  for (int c = 0; c < ncomp; ++c) {
    gradient_G(b, g[c], 1, q, 2, c);
    gradient_G(b, g[c], 2, q, 3, c);
    gradient_G(b, g[c], 3, q, 4, c);
    gradient_G(b, g[c], 4, T, 1, c);
  }
  if (KMX <= 2) memset(b->a[FO_GZ], 0, sizeof(double) * (size_t)b->sz[FO_GZ]);
  if (is_sst(b) || is_kkl(b))  /* gradtk, gradtw / gradtkl (gradients.f90:171-200) */
    for (int c = 0; c < ncomp; ++c) {
      gradient_G(b, g[c], 5, q, 6, c);
      gradient_G(b, g[c], 6, q, 7, c);
    }
  if (is_sa(b))  /* gradtv (gradients.f90:165-169) */
    for (int c = 0; c < ncomp; ++c) gradient_G(b, g[c], 5, q, 6, c);
  if (is_lctm(b))  /* gradtgm (gradients.f90:382-388) */
    for (int c = 0; c < ncomp; ++c) gradient_G(b, g[c], 7, q, 8, c);
  int err = FEST_OK;
  for (int c = 0; c < 3; ++c)
    for (long p = 0; p < b->sz[FO_GX + c]; ++p)
      if (b->a[FO_GX + c][p] != b->a[FO_GX + c][p]) err = FEST_ERR_NAN;
  gradient_bc(b);
  return err;
}

/* ======================================================================== */
/* viscosity (viscosity.f90:52-546) */
int fo_calculate_viscosity(fo_block *b) {
  V q = vqp(b), mu = vpad(b, FO_MU), mut = vpad(b, FO_MUT), F1 = vpad(b, FO_F1), dist = vpad(b, FO_DIST);
  V g[3] = {vgrad(b, 0), vgrad(b, 1), vgrad(b, 2)};
  const fest_flow *fl = &b->flow;
  if (fl->mu_ref != 0. && fl->mu_variation == FEST_MU_SUTHERLAND) {
    OMP_FOR
    for (int k = 0; k <= KMX; ++k)
      for (int j = 0; j <= JMX; ++j)
        for (int i = 0; i <= IMX; ++i) {
          double T = *at(q, i, j, k, 5) / (*at(q, i, j, k, 1) * fl->R_gas);
          *at(mu, i, j, k, 1) = fl->mu_ref * (pow(T / fl->T_ref, 1.5)) *
                                ((fl->T_ref + fl->Sutherland_temp) / (T + fl->Sutherland_temp));
        }
  }
  if (is_sa(b)) {
    /* viscosity.f90:149-160: mu_t = rho tv fv1, xi = tv rho / mu */
    OMP_FOR
    for (int k = 0; k <= KMX; ++k)
      for (int j = 0; j <= JMX; ++j)
        for (int i = 0; i <= IMX; ++i) {
          double tv = *at(q, i, j, k, 6), density = *at(q, i, j, k, 1);
          double xi = tv * density / *at(mu, i, j, k, 1);
          double x3 = xi * xi * xi;
          double fv1 = x3 / (x3 + pow(cv1, 3.0));
          *at(mut, i, j, k, 1) = density * tv * fv1;
        }
    /* ghost copies (viscosity.f90:162-212): faces -1..-9 but -5 copy layer 1,
     * the wall negates it; interfaces keep their own */
    for (int f = 0; f < 6; ++f) {
      int id = b->bc.id[f];
      double sgn;
      if (id == -5) sgn = -1.0;
      else if (id >= -9 && id <= -1) sgn = 1.0;
      else continue;
      int na, nb;
      tang_range(b, f, &na, &nb);
      for (int tb = 1; tb <= nb; ++tb)
        for (int ta = 1; ta <= na; ++ta) {
          int gi, gj, gk, ii, ij, ik;
          ghost_ijk(b, f, 1, ta, tb, &gi, &gj, &gk);
          inner_ijk(b, f, 1, ta, tb, &ii, &ij, &ik);
          *at(mut, gi, gj, gk, 1) = sgn < 0 ? -*at(mut, ii, ij, ik, 1) : *at(mut, ii, ij, ik, 1);
        }
    }
    for (long p = 0; p < b->sz[FO_MU]; ++p)
      if (b->a[FO_MU][p] != b->a[FO_MU][p]) return FEST_ERR_NAN;
    return FEST_OK;
  }
  if (is_kkl(b)) {
    /* viscosity.f90:469-533: mu_t = cmu^0.25 rho kL / max(sqrt(k), 1e-20),
     * zero where k or kL is below 1e-14 */
    double c = pow(kkl_cmu, 0.25);
    OMP_FOR
    for (int k = 0; k <= KMX; ++k)
      for (int j = 0; j <= JMX; ++j)
        for (int i = 0; i <= IMX; ++i) {
          double density = *at(q, i, j, k, 1), tk = *at(q, i, j, k, 6), tkl = *at(q, i, j, k, 7);
          double m = c * density * tkl / (fmax2(sqrt(tk), 1.e-20));
          if (tkl < 1.e-14 || tk < 1.e-14) m = 0.0;
          *at(mut, i, j, k, 1) = m;
        }
    /* ghost copies: faces -1..-4, -6, -8, -9 copy layer 1, the wall negates it */
    for (int f = 0; f < 6; ++f) {
      int id = b->bc.id[f];
      double sgn;
      if (id == -5) sgn = -1.0;
      else if ((id >= -4 && id <= -1) || id == -6 || id == -8 || id == -9) sgn = 1.0;
      else continue;
      int na, nb;
      tang_range(b, f, &na, &nb);
      for (int tb = 1; tb <= nb; ++tb)
        for (int ta = 1; ta <= na; ++ta) {
          int gi, gj, gk, ii, ij, ik;
          ghost_ijk(b, f, 1, ta, tb, &gi, &gj, &gk);
          inner_ijk(b, f, 1, ta, tb, &ii, &ij, &ik);
          *at(mut, gi, gj, gk, 1) = sgn < 0 ? -*at(mut, ii, ij, ik, 1) : *at(mut, ii, ij, ik, 1);
        }
    }
    for (long p = 0; p < b->sz[FO_MU]; ++p)
      if (b->a[FO_MU][p] != b->a[FO_MU][p]) return FEST_ERR_NAN;
    return FEST_OK;
  }
  if (!is_sst(b)) return FEST_OK;
  int s2003 = b->sc.turbulence == FEST_TURB_SST2003;
  OMP_FOR
  for (int k = 0; k <= KMX; ++k)
    for (int j = 0; j <= JMX; ++j)
      for (int i = 0; i <= IMX; ++i) {
        double rho = *at(q, i, j, k, 1), tk = *at(q, i, j, k, 6), tw = *at(q, i, j, k, 7);
        double d = *at(dist, i, j, k, 1);
        double var1 = sqrt(tk) / (bstar * tw * d);
        double var2 = 500 * (*at(mu, i, j, k, 1) / rho) / ((d * d) * tw);
        double arg2 = fmax2(2 * var1, var2);
        double F = tanh(arg2 * arg2);
#define GR(c, l) (*at(g[c], i, j, k, l))
        double DENOM, NUM = rho * a1_sst * tk, CD;
        if (s2003) {
          double sxx = GR(0, 1), syy = GR(1, 2), szz = GR(2, 3);
          double syz = GR(1, 3) + GR(2, 2), szx = GR(2, 1) + GR(0, 3), sxy = GR(0, 2) + GR(1, 1);
          double SijSij = (2.0 * (sxx * sxx)) + (2.0 * (syy * syy)) + (2.0 * (szz * szz)) + syz * syz + szx * szx + sxy * sxy;
          double strain = sqrt(SijSij);
          DENOM = fmax2(fmax2((a1_sst * tw), strain * F), 1.0e-10);
        } else {
          double wx = GR(1, 3) - GR(2, 2), wy = GR(2, 1) - GR(0, 3), wz = GR(0, 2) - GR(1, 1);
          double vort = sqrt(wx * wx + wy * wy + wz * wz);
          DENOM = fmax2(fmax2((a1_sst * tw), vort * F), 1.e-20);
        }
        *at(mut, i, j, k, 1) = NUM / DENOM;
        CD = 2 * rho * sigma_w2 * (GR(0, 5) * GR(0, 6) + GR(1, 5) * GR(1, 6) + GR(2, 5) * GR(2, 6)) / tw;
        CD = fmax2(CD, s2003 ? 1.0e-10 : 1e-20);
#undef GR
        double right = 4 * (rho * sigma_w2 * tk) / (CD * (d * d));
        double left = fmax2(var1, var2);
        double arg1 = fmin2(left, right);
        double a2 = arg1 * arg1;
        *at(F1, i, j, k, 1) = tanh(a2 * a2);
      }
  if (is_lctm(b)) {
    /* viscosity.f90:265-280, 390-405: F1 raised to exp(-(var1/120)**8).
     * The loop there reads density and tk without setting them, so they
     * hold the last cell of the loop before it, (imx, jmx, kmx). */
    double rho_c = *at(q, IMX, JMX, KMX, 1), tk_c = *at(q, IMX, JMX, KMX, 6);
    OMP_FOR
    for (int k = 0; k <= KMX; ++k)
      for (int j = 0; j <= JMX; ++j)
        for (int i = 0; i <= IMX; ++i) {
          double var1 = rho_c * *at(dist, i, j, k, 1) * sqrt(tk_c) / *at(mu, i, j, k, 1);
          double x = var1 / 120, x2 = x * x, x4 = x2 * x2;
          double var2 = exp(-(x4 * x4));
          *at(F1, i, j, k, 1) = fmax2(*at(F1, i, j, k, 1), var2);
        }
  }
  /* ghost copies of mu_t and F1 (viscosity.f90:287-340, 405-460) */
  for (int f = 0; f < 6; ++f) {
    int id = b->bc.id[f];
    double sgn;
    if (id == -10 || id >= 0 || id == -11) continue;
    if (id == -5) sgn = -1.0;
    else if (id >= -9 && id <= -1) sgn = 1.0;
    else continue;
    int na, nb;
    tang_range(b, f, &na, &nb);
    for (int tb = 1; tb <= nb; ++tb)
      for (int ta = 1; ta <= na; ++ta) {
        int gi, gj, gk, ii, ij, ik;
        ghost_ijk(b, f, 1, ta, tb, &gi, &gj, &gk);
        inner_ijk(b, f, 1, ta, tb, &ii, &ij, &ik);
        *at(mut, gi, gj, gk, 1) = sgn < 0 ? -*at(mut, ii, ij, ik, 1) : *at(mut, ii, ij, ik, 1);
        *at(F1, gi, gj, gk, 1) = *at(F1, ii, ij, ik, 1);
      }
  }
  for (long p = 0; p < b->sz[FO_MU]; ++p)
    if (b->a[FO_MU][p] != b->a[FO_MU][p]) return FEST_ERR_NAN;
  return FEST_OK;
}

/* ======================================================================== */
/* viscous fluxes (viscous.f90:144-447) */
static void viscous_laminar(fo_block *b, int dir) {
  V q = vqp(b), mu = vpad(b, FO_MU), mut = vpad(b, FO_MUT), Fl = vflux(b, dir);
  V g[3] = {vgrad(b, 0), vgrad(b, 1), vgrad(b, 2)};
  R4 fa = vfaces(b, dir), cl = vcells(b);
  const fest_flow *fl = &b->flow;
  int ii = dir == 0, jj = dir == 1, kk = dir == 2;
  int turb = is_turb(b);
  OMP_FOR
  for (int k = 1; k <= KMX - 1 + kk; ++k)
    for (int j = 1; j <= JMX - 1 + jj; ++j)
      for (int i = 1; i <= IMX - 1 + ii; ++i) {
        int im = i - ii, jm = j - jj, km = k - kk;
        double G[3][4];
        for (int c = 0; c < 3; ++c)
          for (int l = 1; l <= 4; ++l) G[c][l - 1] = 0.5 * (*at(g[c], im, jm, km, l) + *at(g[c], i, j, k, l));
        const double *c1 = r4(cl, i, j, k), *c0 = r4(cl, im, jm, km);
        double delx = c1[1] - c0[1], dely = c1[2] - c0[2], delz = c1[3] - c0[3];
        double dLR = sqrt(delx * delx + dely * dely + delz * delz);
        double TLE = *at(q, im, jm, km, 5) / (*at(q, im, jm, km, 1) * fl->R_gas);
        double TRE = *at(q, i, j, k, 5) / (*at(q, i, j, k, 1) * fl->R_gas);
        double del[4] = {*at(q, i, j, k, 2) - *at(q, im, jm, km, 2), *at(q, i, j, k, 3) - *at(q, im, jm, km, 3),
                         *at(q, i, j, k, 4) - *at(q, im, jm, km, 4), TRE - TLE};
        for (int l = 0; l < 4; ++l) {
          double nc = (del[l] - (G[0][l] * delx + G[1][l] * dely + G[2][l] * delz)) / dLR;
          G[0][l] = G[0][l] + (nc * delx / dLR);
          G[1][l] = G[1][l] + (nc * dely / dLR);
          G[2][l] = G[2][l] + (nc * delz / dLR);
        }
        double dudx = G[0][0], dudy = G[1][0], dudz = G[2][0];
        double dvdx = G[0][1], dvdy = G[1][1], dvdz = G[2][1];
        double dwdx = G[0][2], dwdy = G[1][2], dwdz = G[2][2];
        double dTdx = G[0][3], dTdy = G[1][3], dTdz = G[2][3];
        double mu_f = 0.5 * (*at(mu, im, jm, km, 1) + *at(mu, i, j, k, 1));
        double mut_f = turb ? 0.5 * (*at(mut, im, jm, km, 1) + *at(mut, i, j, k, 1)) : 0.0;
        double tm = mu_f + mut_f;
        double Txx = 2. * tm * (dudx - ((dudx + dvdy + dwdz) / 3.));
        double Tyy = 2. * tm * (dvdy - ((dudx + dvdy + dwdz) / 3.));
        double Tzz = 2. * tm * (dwdz - ((dudx + dvdy + dwdz) / 3.));
        double Txy = tm * (dvdx + dudy), Txz = tm * (dwdx + dudz), Tyz = tm * (dwdy + dvdz);
        double Kh = (mu_f / fl->Pr + mut_f / fl->tPr) * fl->gm * fl->R_gas / (fl->gm - 1);
        double Qx = Kh * dTdx, Qy = Kh * dTdy, Qz = Kh * dTdz;
        const double *fc = r4(fa, i, j, k);
        double nx = fc[1], ny = fc[2], nz = fc[3], A = fc[0];
        double uf = 0.5 * (*at(q, im, jm, km, 2) + *at(q, i, j, k, 2));
        double vf = 0.5 * (*at(q, im, jm, km, 3) + *at(q, i, j, k, 3));
        double wf = 0.5 * (*at(q, im, jm, km, 4) + *at(q, i, j, k, 4));
        *at(Fl, i, j, k, 2) = *at(Fl, i, j, k, 2) - ((Txx * nx + Txy * ny + Txz * nz) * A);
        *at(Fl, i, j, k, 3) = *at(Fl, i, j, k, 3) - ((Txy * nx + Tyy * ny + Tyz * nz) * A);
        *at(Fl, i, j, k, 4) = *at(Fl, i, j, k, 4) - ((Txz * nx + Tyz * ny + Tzz * nz) * A);
        *at(Fl, i, j, k, 5) = *at(Fl, i, j, k, 5) -
                              (A * (((Txx * uf + Txy * vf + Txz * wf + Qx) * nx) + ((Txy * uf + Tyy * vf + Tyz * wf + Qy) * ny) +
                                    ((Txz * uf + Tyz * vf + Tzz * wf + Qz) * nz)));
      }
}

static void viscous_sst(fo_block *b, int dir) {
  V q = vqp(b), mu = vpad(b, FO_MU), mut = vpad(b, FO_MUT), F1v = vpad(b, FO_F1), Fl = vflux(b, dir);
  V g[3] = {vgrad(b, 0), vgrad(b, 1), vgrad(b, 2)};
  R4 fa = vfaces(b, dir), cl = vcells(b);
  int ii = dir == 0, jj = dir == 1, kk = dir == 2;
  OMP_FOR
  for (int k = 1; k <= KMX - 1 + kk; ++k)
    for (int j = 1; j <= JMX - 1 + jj; ++j)
      for (int i = 1; i <= IMX - 1 + ii; ++i) {
        int im = i - ii, jm = j - jj, km = k - kk;
        double G[3][2];
        for (int c = 0; c < 3; ++c)
          for (int l = 0; l < 2; ++l) G[c][l] = 0.5 * (*at(g[c], im, jm, km, 5 + l) + *at(g[c], i, j, k, 5 + l));
        const double *c1 = r4(cl, i, j, k), *c0 = r4(cl, im, jm, km);
        double delx = c1[1] - c0[1], dely = c1[2] - c0[2], delz = c1[3] - c0[3];
        double dLR = sqrt(delx * delx + dely * dely + delz * delz);
        double del[2] = {*at(q, i, j, k, 6) - *at(q, im, jm, km, 6), *at(q, i, j, k, 7) - *at(q, im, jm, km, 7)};
        for (int l = 0; l < 2; ++l) {
          double nc = (del[l] - (G[0][l] * delx + G[1][l] * dely + G[2][l] * delz)) / dLR;
          G[0][l] = G[0][l] + (nc * delx / dLR);
          G[1][l] = G[1][l] + (nc * dely / dLR);
          G[2][l] = G[2][l] + (nc * delz / dLR);
        }
        double mu_f = 0.5 * (*at(mu, im, jm, km, 1) + *at(mu, i, j, k, 1));
        double mut_f = 0.5 * (*at(mut, im, jm, km, 1) + *at(mut, i, j, k, 1));
        double F1 = 0.5 * (*at(F1v, im, jm, km, 1) + *at(F1v, i, j, k, 1));
        double skf = sigma_k1 * F1 + sigma_k2 * (1.0 - F1);
        double swf = sigma_w1 * F1 + sigma_w2 * (1.0 - F1);
        double rhof = 0.5 * (*at(q, im, jm, km, 1) + *at(q, i, j, k, 1));
        double tkf = 0.5 * (*at(q, im, jm, km, 6) + *at(q, i, j, k, 6));
        double Txx = -2.0 * rhof * tkf / 3.0;
        const double *fc = r4(fa, i, j, k);
        double nx = fc[1], ny = fc[2], nz = fc[3], A = fc[0];
        double dk = G[0][0] * nx + G[1][0] * ny + G[2][0] * nz;
        double dw = G[0][1] * nx + G[1][1] * ny + G[2][1] * nz;
        *at(Fl, i, j, k, 2) = *at(Fl, i, j, k, 2) - (Txx * nx * A);
        *at(Fl, i, j, k, 3) = *at(Fl, i, j, k, 3) - (Txx * ny * A);
        *at(Fl, i, j, k, 4) = *at(Fl, i, j, k, 4) - (Txx * nz * A);
        *at(Fl, i, j, k, 5) = *at(Fl, i, j, k, 5) - (A * ((mu_f + skf * mut_f) * dk));
        *at(Fl, i, j, k, 6) = *at(Fl, i, j, k, 6) - (A * ((mu_f + skf * mut_f) * dk));
        *at(Fl, i, j, k, 7) = *at(Fl, i, j, k, 7) - (A * ((mu_f + swf * mut_f) * dw));
      }
}

/* viscous.f90:570-656 compute_viscous_fluxes_sa */
static void viscous_sa(fo_block *b, int dir) {
  V q = vqp(b), mu = vpad(b, FO_MU), Fl = vflux(b, dir);
  V g[3] = {vgrad(b, 0), vgrad(b, 1), vgrad(b, 2)};
  R4 fa = vfaces(b, dir), cl = vcells(b);
  int ii = dir == 0, jj = dir == 1, kk = dir == 2;
  OMP_FOR
  for (int k = 1; k <= KMX - 1 + kk; ++k)
    for (int j = 1; j <= JMX - 1 + jj; ++j)
      for (int i = 1; i <= IMX - 1 + ii; ++i) {
        int im = i - ii, jm = j - jj, km = k - kk;
        double dtvdx = 0.5 * (*at(g[0], im, jm, km, 5) + *at(g[0], i, j, k, 5));
        double dtvdy = 0.5 * (*at(g[1], im, jm, km, 5) + *at(g[1], i, j, k, 5));
        double dtvdz = 0.5 * (*at(g[2], im, jm, km, 5) + *at(g[2], i, j, k, 5));
        const double *c1 = r4(cl, i, j, k), *c0 = r4(cl, im, jm, km);
        double delx = c1[1] - c0[1], dely = c1[2] - c0[2], delz = c1[3] - c0[3];
        double d_LR = sqrt(delx * delx + dely * dely + delz * delz);
        double deltv = *at(q, i, j, k, 6) - *at(q, im, jm, km, 6);
        double nc = (deltv - (dtvdx * delx + dtvdy * dely + dtvdz * delz)) / d_LR;
        dtvdx = dtvdx + (nc * delx / d_LR);
        dtvdy = dtvdy + (nc * dely / d_LR);
        dtvdz = dtvdz + (nc * delz / d_LR);
        double rhoface = 0.5 * (*at(q, im, jm, km, 1) + *at(q, i, j, k, 1));
        double mu_f = 0.5 * (*at(mu, im, jm, km, 1) + *at(mu, i, j, k, 1));
        double mut_f = 0.5 * (*at(q, im, jm, km, 6) + *at(q, i, j, k, 6)) * rhoface;
        const double *fc = r4(fa, i, j, k);
        double nx = fc[1], ny = fc[2], nz = fc[3], area = fc[0];
        *at(Fl, i, j, k, 6) = *at(Fl, i, j, k, 6) -
                              (area * ((mu_f + mut_f) * (dtvdx * nx + dtvdy * ny + dtvdz * nz))) / sigma_sa;
      }
}

/* viscous.f90:450-567 compute_viscous_fluxes_kkl */
/* viscous.f90:658-749 compute_viscous_fluxes_lctm2015: the intermittency's
 * diffusion with mu + mu_t, its face gradient corrected along the line of
 * centres as the other variables' are */
static void viscous_lctm(fo_block *b, int dir) {
  V q = vqp(b), mu = vpad(b, FO_MU), mut = vpad(b, FO_MUT), Fl = vflux(b, dir);
  V g[3] = {vgrad(b, 0), vgrad(b, 1), vgrad(b, 2)};
  R4 fa = vfaces(b, dir), cl = vcells(b);
  int ii = dir == 0, jj = dir == 1, kk = dir == 2;
  OMP_FOR
  for (int k = 1; k <= KMX - 1 + kk; ++k)
    for (int j = 1; j <= JMX - 1 + jj; ++j)
      for (int i = 1; i <= IMX - 1 + ii; ++i) {
        int im = i - ii, jm = j - jj, km = k - kk;
        double G[3];
        for (int c = 0; c < 3; ++c) G[c] = 0.5 * (*at(g[c], im, jm, km, 7) + *at(g[c], i, j, k, 7));
        const double *c1 = r4(cl, i, j, k), *c0 = r4(cl, im, jm, km);
        double delx = c1[1] - c0[1], dely = c1[2] - c0[2], delz = c1[3] - c0[3];
        double d_LR = sqrt(delx * delx + dely * dely + delz * delz);
        double deltgm = *at(q, i, j, k, 8) - *at(q, im, jm, km, 8);
        double nc = (deltgm - (G[0] * delx + G[1] * dely + G[2] * delz)) / d_LR;
        G[0] = G[0] + (nc * delx / d_LR);
        G[1] = G[1] + (nc * dely / d_LR);
        G[2] = G[2] + (nc * delz / d_LR);
        double mu_f = 0.5 * (*at(mu, im, jm, km, 1) + *at(mu, i, j, k, 1));
        double mut_f = 0.5 * (*at(mut, im, jm, km, 1) + *at(mut, i, j, k, 1));
        const double *fc = r4(fa, i, j, k);
        double nx = fc[1], ny = fc[2], nz = fc[3], area = fc[0];
        *at(Fl, i, j, k, 8) = *at(Fl, i, j, k, 8) - (area * ((mu_f + mut_f) * (G[0] * nx + G[1] * ny + G[2] * nz)));
      }
}

static void viscous_kkl(fo_block *b, int dir) {
  V q = vqp(b), mu = vpad(b, FO_MU), mut = vpad(b, FO_MUT), Fl = vflux(b, dir);
  V g[3] = {vgrad(b, 0), vgrad(b, 1), vgrad(b, 2)};
  R4 fa = vfaces(b, dir), cl = vcells(b);
  int ii = dir == 0, jj = dir == 1, kk = dir == 2;
  OMP_FOR
  for (int k = 1; k <= KMX - 1 + kk; ++k)
    for (int j = 1; j <= JMX - 1 + jj; ++j)
      for (int i = 1; i <= IMX - 1 + ii; ++i) {
        int im = i - ii, jm = j - jj, km = k - kk;
        double G[3][2];
        for (int c = 0; c < 3; ++c)
          for (int l = 0; l < 2; ++l) G[c][l] = 0.5 * (*at(g[c], im, jm, km, 5 + l) + *at(g[c], i, j, k, 5 + l));
        const double *c1 = r4(cl, i, j, k), *c0 = r4(cl, im, jm, km);
        double delx = c1[1] - c0[1], dely = c1[2] - c0[2], delz = c1[3] - c0[3];
        double d_LR = sqrt(delx * delx + dely * dely + delz * delz);
        double del[2] = {*at(q, i, j, k, 6) - *at(q, im, jm, km, 6), *at(q, i, j, k, 7) - *at(q, im, jm, km, 7)};
        for (int l = 0; l < 2; ++l) {
          double nc = (del[l] - (G[0][l] * delx + G[1][l] * dely + G[2][l] * delz)) / d_LR;
          G[0][l] = G[0][l] + (nc * delx / d_LR);
          G[1][l] = G[1][l] + (nc * dely / d_LR);
          G[2][l] = G[2][l] + (nc * delz / d_LR);
        }
        double mu_f = 0.5 * (*at(mu, im, jm, km, 1) + *at(mu, i, j, k, 1));
        double mut_f = 0.5 * (*at(mut, im, jm, km, 1) + *at(mut, i, j, k, 1));
        double rhoface = 0.5 * (*at(q, im, jm, km, 1) + *at(q, i, j, k, 1));
        double tkface = 0.5 * (*at(q, im, jm, km, 6) + *at(q, i, j, k, 6));
        double Tau_xx = -2.0 * rhoface * tkface / 3.0;
        const double *fc = r4(fa, i, j, k);
        double nx = fc[1], ny = fc[2], nz = fc[3], area = fc[0];
        double dk = G[0][0] * nx + G[1][0] * ny + G[2][0] * nz;
        double dkl = G[0][1] * nx + G[1][1] * ny + G[2][1] * nz;
        *at(Fl, i, j, k, 2) = *at(Fl, i, j, k, 2) - (Tau_xx * nx * area);
        *at(Fl, i, j, k, 3) = *at(Fl, i, j, k, 3) - (Tau_xx * ny * area);
        *at(Fl, i, j, k, 4) = *at(Fl, i, j, k, 4) - (Tau_xx * nz * area);
        *at(Fl, i, j, k, 5) = *at(Fl, i, j, k, 5) - (area * ((mu_f + kkl_sigma_k * mut_f) * dk));
        *at(Fl, i, j, k, 6) = *at(Fl, i, j, k, 6) - (area * ((mu_f + kkl_sigma_k * mut_f) * dk));
        *at(Fl, i, j, k, 7) = *at(Fl, i, j, k, 7) - (area * ((mu_f + kkl_sigma_phi * mut_f) * dkl));
      }
}

int fo_compute_viscous_fluxes(fo_block *b) {
  for (int dir = 0; dir < 3; ++dir) viscous_laminar(b, dir);
  if (is_kkl(b))
    for (int dir = 0; dir < 3; ++dir) viscous_kkl(b, dir);
  if (is_sa(b))
    for (int dir = 0; dir < 3; ++dir) viscous_sa(b, dir);
  if (is_sst(b)) {
    viscous_sst(b, 0);
    viscous_sst(b, 1);
    if (KMX != 2) viscous_sst(b, 2);
  }
  if (is_lctm(b)) { /* viscous.f90:115-125 */
    viscous_lctm(b, 0);
    viscous_lctm(b, 1);
    if (KMX != 2) viscous_lctm(b, 2);
  }
  for (int dir = 0; dir < 3; ++dir)
    for (long p = 0; p < b->sz[FO_F + dir]; ++p)
      if (b->a[FO_F + dir][p] != b->a[FO_F + dir][p]) return FEST_ERR_NAN;
  return FEST_OK;
}

/* source.f90:845-983 add_sa_source.  The density gradient comes from the
 * six face sums of the cell; the k faces' normal reads (nx, nx, nx) as the
 * reference does (source.f90:913). */
static void sa_source(fo_block *b) {
  V q = vqp(b), mu = vpad(b, FO_MU), dist = vpad(b, FO_DIST), r = vres(b);
  V g[3] = {vgrad(b, 0), vgrad(b, 1), vgrad(b, 2)};
  R4 If = vfaces(b, 0), Jf = vfaces(b, 1), Kf = vfaces(b, 2), cl = vcells(b);
  OMP_FOR
  for (int k = 1; k <= KMX - 1; ++k)
    for (int j = 1; j <= JMX - 1; ++j)
      for (int i = 1; i <= IMX - 1; ++i) {
#define GR(c, l) (*at(g[c], i, j, k, l))
        double density = *at(q, i, j, k, 1), tv = *at(q, i, j, k, 6);
        double RhoFace[6] = {*at(q, i - 1, j, k, 1) + density, *at(q, i, j - 1, k, 1) + density,
                             *at(q, i, j, k - 1, 1) + density, *at(q, i + 1, j, k, 1) + density,
                             *at(q, i, j + 1, k, 1) + density, *at(q, i, j, k + 1, 1) + density};
        const double *fI0 = r4(If, i, j, k), *fJ0 = r4(Jf, i, j, k), *fK0 = r4(Kf, i, j, k);
        const double *fI1 = r4(If, i + 1, j, k), *fJ1 = r4(Jf, i, j + 1, k), *fK1 = r4(Kf, i, j, k + 1);
        double Area[6] = {fI0[0], fJ0[0], fK0[0], fI1[0], fJ1[0], fK1[0]};
        double Normal[6][3] = {{fI0[1], fI0[2], fI0[3]}, {fJ0[1], fJ0[2], fJ0[3]}, {fK0[1], fK0[1], fK0[1]},
                               {fI1[1], fI1[2], fI1[3]}, {fJ1[1], fJ1[2], fJ1[3]}, {fK1[1], fK1[2], fK1[3]}};
        double vol = r4(cl, i, j, k)[0];
        double gr[3];
        for (int c = 0; c < 3; ++c)
          gr[c] = (-(RhoFace[0]) * Normal[0][c] * Area[0] - (RhoFace[1]) * Normal[1][c] * Area[1] -
                   (RhoFace[2]) * Normal[2][c] * Area[2] + (RhoFace[3]) * Normal[3][c] * Area[3] +
                   (RhoFace[4]) * Normal[4][c] * Area[4] + (RhoFace[5]) * Normal[5][c] * Area[5]) /
                  (2.0 * vol);
        double wa = GR(1, 3) - GR(2, 2), wb = GR(2, 1) - GR(0, 3), wc = GR(0, 2) - GR(1, 1);
        double vort = sqrt(((wa * wa) + (wb * wb) + (wc * wc)));
        double CD1 = cb2 * ((GR(0, 5) * GR(0, 5)) + (GR(1, 5) * GR(1, 5)) + (GR(2, 5) * GR(2, 5)));
        double CD2 = ((gr[0] * GR(0, 5)) + (gr[1] * GR(1, 5)) + (gr[2] * GR(2, 5)));
        double d = *at(dist, i, j, k, 1);
        double kd = kappa_sa * d, kd2 = kd * kd;
        double nu = *at(mu, i, j, k, 1) / density;
        double xi = tv / nu;
        double x3 = xi * xi * xi;
        double fv1 = x3 / (x3 + pow(cv1, 3.0));
        double fv2 = 1.0 - xi / (1.0 + (xi * fv1));
        double Scap = fmax2(vort + (tv * fv2 / (kd2)), 0.3 * vort);
        double rr = fmin2(tv / (Scap * kd2), 10.0);
        double gg = rr + cw2 * (pow6(rr) - rr);
        double fw = gg * pow((1.0 + pow6(cw3)) / (pow6(gg) + pow6(cw3)), 1.0 / 6.0);
        double td = tv / d;
        double D_v = density * CW1_SA * fw * (td * td);
        double P_v = density * cb1 * Scap * tv;
        double lamda = density * CD1 / sigma_sa - CD2 * (nu + tv) / sigma_sa;
        double S_v = (P_v - D_v + lamda) * vol;
        *at(r, i, j, k, 6) = *at(r, i, j, k, 6) - S_v;
#undef GR
      }
}

/* source.f90:607-832 add_kkl_source: production by the Reynolds stress,
 * the von Karman length from the velocity's second derivatives (Green-Gauss
 * sums of the gradients over the cell's faces) with its limiters, and the
 * wall damping */
static void kkl_source(fo_block *b) {
  V q = vqp(b), mu = vpad(b, FO_MU), mut = vpad(b, FO_MUT), dist = vpad(b, FO_DIST), r = vres(b);
  V g[3] = {vgrad(b, 0), vgrad(b, 1), vgrad(b, 2)};
  R4 If = vfaces(b, 0), Jf = vfaces(b, 1), Kf = vfaces(b, 2), cl = vcells(b);
  const double c075 = pow(kkl_cmu, 0.75);
  OMP_FOR
  for (int k = 1; k <= KMX - 1; ++k)
    for (int j = 1; j <= JMX - 1; ++j)
      for (int i = 1; i <= IMX - 1; ++i) {
#define GR(c, l) (*at(g[c], i, j, k, l))
        double density = *at(q, i, j, k, 1), tk = *at(q, i, j, k, 6), tkl = *at(q, i, j, k, 7);
        /* S(a, b) = (d u_a / d x_b + d u_b / d x_a) / 2 */
        double S[3][3];
        for (int a = 0; a < 3; ++a)
          for (int c = 0; c < 3; ++c) S[a][c] = 0.5 * (GR(c, a + 1) + GR(a, c + 1));
        double delv = GR(0, 1) + GR(1, 2) + GR(2, 3);
        double mt = *at(mut, i, j, k, 1);
        double Tau[3][3];
        for (int a = 0; a < 3; ++a)
          for (int c = 0; c < 3; ++c)
            Tau[a][c] = a == c ? mt * (2 * S[a][c] - (2.0 / 3.0) * delv) - (2.0 / 3.0) * density * tk
                               : mt * (2 * S[a][c]);
        double P_k = 0.;
        for (int a = 0; a < 3; ++a)
          P_k = P_k + Tau[a][0] * GR(0, a + 1) + Tau[a][1] * GR(1, a + 1) + Tau[a][2] * GR(2, a + 1);
        double D_k = c075 * density * (pow(tk, 2.5)) / fmax2(tkl, 1.e-20);
        P_k = fmin2(P_k, 20 * D_k);
        /* second derivatives d2(u_a)/d(x_c)2 */
        const double *fr[6] = {r4(If, i, j, k), r4(Jf, i, j, k), r4(Kf, i, j, k),
                               r4(If, i + 1, j, k), r4(Jf, i, j + 1, k), r4(Kf, i, j, k + 1)};
        const int nb[6][3] = {{i - 1, j, k}, {i, j - 1, k}, {i, j, k - 1}, {i + 1, j, k}, {i, j + 1, k}, {i, j, k + 1}};
        double vol2 = 2 * r4(cl, i, j, k)[0];
        double lap[3];
        for (int a = 0; a < 3; ++a) {
          double sum = 0.0;
          for (int c = 0; c < 3; ++c) {
            double gc = *at(g[c], i, j, k, a + 1);
            double t = -((*at(g[c], nb[0][0], nb[0][1], nb[0][2], a + 1) + gc) * fr[0][1 + c] * fr[0][0]);
            for (int f = 1; f < 6; ++f) {
              double v = (*at(g[c], nb[f][0], nb[f][1], nb[f][2], a + 1) + gc) * fr[f][1 + c] * fr[f][0];
              t = f < 3 ? t - v : t + v;
            }
            sum = c == 0 ? t / vol2 : sum + t / vol2;
          }
          lap[a] = sum;
        }
        double udd = sqrt((lap[0] * lap[0]) + (lap[1] * lap[1]) + (lap[2] * lap[2]));
        double s2 = 0.0;
        for (int a = 0; a < 3; ++a)
          for (int c = 0; c < 3; ++c) s2 = (a == 0 && c == 0) ? S[0][0] * S[0][0] : s2 + S[a][c] * S[a][c];
        double ud = sqrt(2 * s2);
        double Lvk = kkl_kappa * fabs(ud / fmax2(udd, 1.e-20));
        double fp = fmin2(fmax2(P_k / D_k, 0.5), 1.0);
        double d = *at(dist, i, j, k, 1), m = *at(mu, i, j, k, 1);
        Lvk = fmax2(Lvk, tkl / fmax2((tk * kkl_c11), 1.e-20));
        Lvk = fmin2(Lvk, kkl_c12 * kkl_kappa * d * fp);
        double eta = density * d * sqrt(0.3 * tk) / (20 * m);
        double e2 = eta * eta;
        double fphi = (1 + kkl_cd1 * eta) / (1 + e2 * e2);
        double cphi2 = kkl_zeta3;
        double rr = tkl / fmax2(tk * Lvk, 1.e-20);
        double cphi1 = (kkl_zeta1 - kkl_zeta2 * (rr * rr));
        double P_kl = cphi1 * tkl * P_k / fmax2(tk, 1.e-20);
        double D_kl = cphi2 * density * (pow(tk, 1.5));
        double S_k = P_k - D_k - 2 * m * tk / (d * d);
        double S_kl = P_kl - D_kl - 6 * m * tkl * fphi / (d * d);
        double vol = r4(cl, i, j, k)[0];
        S_k = S_k * vol;
        S_kl = S_kl * vol;
        *at(r, i, j, k, 6) = *at(r, i, j, k, 6) - S_k;
        *at(r, i, j, k, 7) = *at(r, i, j, k, 7) - S_kl;
#undef GR
      }
}

/* the free-stream Reynolds number of init_infinity_values (state.f90:89),
 * per unit length */
static double reynolds_number(const fo_block *b) {
  return b->flow.density_inf * b->flow.vel_mag * 1.0 / b->flow.mu_ref;
}

/* the 'bc' transition model's intermittency (source.f90:571-589 and
 * 1159-1170): from the momentum-thickness Reynolds number against its
 * transition value (Tu in percent) and the eddy viscosity against its
 * critical value */
static double gamma_bc(double re_v, double nu_bc, double Re, double tu) {
  const double chi_1 = 0.002, chi_2 = 5.0;
  double nu_cr = chi_2 / Re;
  double re_theta = re_v / 2.193;
  double re_theta_t = (803.73 * (pow((tu + 0.6067), (-1.027))));
  double term1 = sqrt(fmax2(re_theta - re_theta_t, 0.) / (chi_1 * re_theta_t));
  double term2 = sqrt(fmax2(nu_bc - nu_cr, 0.0) / nu_cr);
  double term_exponential = (term1 + term2);
  return 1.0 - exp(-term_exponential);
}

/* source.f90:985-1194 add_saBC_source: SA with the production scaled by
 * the 'bc' intermittency (S-hat floored at 1e-10) */
static void sa_bc_source(fo_block *b) {
  V q = vqp(b), mu = vpad(b, FO_MU), dist = vpad(b, FO_DIST), r = vres(b);
  V g[3] = {vgrad(b, 0), vgrad(b, 1), vgrad(b, 2)};
  R4 If = vfaces(b, 0), Jf = vfaces(b, 1), Kf = vfaces(b, 2), cl = vcells(b);
  const double Re = reynolds_number(b), tu = b->flow.tu_inf;
  OMP_FOR
  for (int k = 1; k <= KMX - 1; ++k)
    for (int j = 1; j <= JMX - 1; ++j)
      for (int i = 1; i <= IMX - 1; ++i) {
#define GR(c, l) (*at(g[c], i, j, k, l))
        double density = *at(q, i, j, k, 1), u = *at(q, i, j, k, 2), v = *at(q, i, j, k, 3), w = *at(q, i, j, k, 4);
        double tv = *at(q, i, j, k, 6);
        double vmag = sqrt(u * u + v * v + w * w);
        double RhoFace[6] = {*at(q, i - 1, j, k, 1) + density, *at(q, i, j - 1, k, 1) + density,
                             *at(q, i, j, k - 1, 1) + density, *at(q, i + 1, j, k, 1) + density,
                             *at(q, i, j + 1, k, 1) + density, *at(q, i, j, k + 1, 1) + density};
        const double *fI0 = r4(If, i, j, k), *fJ0 = r4(Jf, i, j, k), *fK0 = r4(Kf, i, j, k);
        const double *fI1 = r4(If, i + 1, j, k), *fJ1 = r4(Jf, i, j + 1, k), *fK1 = r4(Kf, i, j, k + 1);
        double Area[6] = {fI0[0], fJ0[0], fK0[0], fI1[0], fJ1[0], fK1[0]};
        double Normal[6][3] = {{fI0[1], fI0[2], fI0[3]}, {fJ0[1], fJ0[2], fJ0[3]}, {fK0[1], fK0[1], fK0[1]},
                               {fI1[1], fI1[2], fI1[3]}, {fJ1[1], fJ1[2], fJ1[3]}, {fK1[1], fK1[2], fK1[3]}};
        double vol = r4(cl, i, j, k)[0];
        double gr[3];
        for (int c = 0; c < 3; ++c)
          gr[c] = (-(RhoFace[0]) * Normal[0][c] * Area[0] - (RhoFace[1]) * Normal[1][c] * Area[1] -
                   (RhoFace[2]) * Normal[2][c] * Area[2] + (RhoFace[3]) * Normal[3][c] * Area[3] +
                   (RhoFace[4]) * Normal[4][c] * Area[4] + (RhoFace[5]) * Normal[5][c] * Area[5]) /
                  (2 * vol);
        double wa = GR(1, 3) - GR(2, 2), wb = GR(2, 1) - GR(0, 3), wc = GR(0, 2) - GR(1, 1);
        double Omega = sqrt(((wa * wa) + (wb * wb) + (wc * wc)));
        double CD1 = cb2 * ((GR(0, 5) * GR(0, 5)) + (GR(1, 5) * GR(1, 5)) + (GR(2, 5) * GR(2, 5)));
        double CD2 = ((gr[0] * GR(0, 5)) + (gr[1] * GR(1, 5)) + (gr[2] * GR(2, 5)));
        double dist_i = *at(dist, i, j, k, 1);
        double dist_i_2 = dist_i * dist_i;
        double k2 = kappa_sa * kappa_sa;
        double nu = *at(mu, i, j, k, 1) / density;
        double Ji = tv / nu, Ji_2 = Ji * Ji, Ji_3 = Ji_2 * Ji;
        double fv1 = (Ji_3) / ((Ji_3) + (pow(cv1, 3.0)));
        double fv2 = 1.0 - Ji / (1.0 + (Ji * fv1));
        double S = Omega;
        double inv_k2_d2 = 1.0 / (k2 * dist_i_2);
        double Shat = S + tv * fv2 * inv_k2_d2;
        Shat = fmax2(Shat, 1.0e-10);
        double inv_Shat = 1.0 / Shat;
        double nu_t = tv * fv1;
        double nu_bc = nu_t / (vmag * dist_i);
        double re_v = dist_i_2 * Omega / nu;
        double gBC = gamma_bc(re_v, nu_bc, Re, tu);
        double Production = gBC * cb1 * Shat * tv * vol;
        double rr = fmin2(tv * inv_Shat * inv_k2_d2, 10.0);
        double gg = rr + cw2 * (pow6(rr) - rr);
        double g_6 = pow6(gg);
        double glim = pow(((1.0 + pow6(cw3)) / (g_6 + pow6(cw3))), (1.0 / 6.0));
        double fw = gg * glim;
        double Destruction = (CW1_SA * fw * tv * tv / dist_i_2) * (vol);
        double lamda = (density * CD1 / sigma_sa - CD2 * (nu + tv) / sigma_sa) * vol;
        double S_v = (Production - Destruction + lamda);
        *at(r, i, j, k, 6) = *at(r, i, j, k, 6) - S_v;
#undef GR
      }
}

/* source.f90:467-604 add_sst_bc_source: SST with the production mu_t
 * Omega^2 (no divergence term, limited by 20 D_k), scaled by the 'bc'
 * intermittency after P_w is taken from it, and the cross diffusion
 * without its floor */
static void sst_bc_source(fo_block *b) {
  V q = vqp(b), mu = vpad(b, FO_MU), mut = vpad(b, FO_MUT), F1v = vpad(b, FO_F1), dist = vpad(b, FO_DIST);
  V r = vres(b);
  V g[3] = {vgrad(b, 0), vgrad(b, 1), vgrad(b, 2)};
  R4 cl = vcells(b);
  const double Re = reynolds_number(b), TuL = b->flow.tu_inf;
  double gama1 = (beta1 / bstar) - ((sigma_w1 * (kappa_sst * kappa_sst)) / sqrt(bstar));
  double gama2 = (beta2 / bstar) - ((sigma_w2 * (kappa_sst * kappa_sst)) / sqrt(bstar));
  OMP_FOR
  for (int k = 1; k <= KMX - 1; ++k)
    for (int j = 1; j <= JMX - 1; ++j)
      for (int i = 1; i <= IMX - 1; ++i) {
#define GR(c, l) (*at(g[c], i, j, k, l))
        double density = *at(q, i, j, k, 1), tk = *at(q, i, j, k, 6), tw = *at(q, i, j, k, 7);
        double wa = GR(1, 3) - GR(2, 2), wb = GR(2, 1) - GR(0, 3), wc = GR(0, 2) - GR(1, 1);
        double vort = sqrt(((wa * wa) + (wb * wb) + (wc * wc)));
        double CD = 2 * density * sigma_w2 * (GR(0, 5) * GR(0, 6) + GR(1, 5) * GR(1, 6) + GR(2, 5) * GR(2, 6)) / tw;
        double F1 = *at(F1v, i, j, k, 1);
        double gama = gama1 * F1 + gama2 * (1. - F1);
        double beta = beta1 * F1 + beta2 * (1. - F1);
        double D_k = bstar * density * tw * tk;
        double D_w = beta * density * (tw * tw);
        double mt = *at(mut, i, j, k, 1);
        double P_k = mt * (vort * vort);
        P_k = fmin2(P_k, 20.0 * D_k);
        double P_w = (density * gama / mt) * P_k;
        double lamda = (1. - F1) * CD;
        double u = *at(q, i, j, k, 2), v = *at(q, i, j, k, 3), w = *at(q, i, j, k, 4);
        double vmag = sqrt(u * u + v * v + w * w);
        double nu_t = mt / density;
        double d = *at(dist, i, j, k, 1);
        double nu_bc = nu_t / (vmag * d);
        double re_v = density * d * d * vort / *at(mu, i, j, k, 1);
        P_k = gamma_bc(re_v, nu_bc, Re, TuL) * P_k;
        double S_k = P_k - D_k;
        double S_w = P_w - D_w + lamda;
        double vol = r4(cl, i, j, k)[0];
        S_k = S_k * vol;
        S_w = S_w * vol;
        *at(r, i, j, k, 6) = *at(r, i, j, k, 6) - S_k;
        *at(r, i, j, k, 7) = *at(r, i, j, k, 7) - S_w;
#undef GR
      }
}

/* source.f90:273-465 add_sst_source_lctm2015: the SST source with the
 * production by vorticity times strain, scaled by the intermittency, its
 * limited extra production and the floored destruction, and the
 * intermittency's own source (onset from the vorticity Reynolds number
 * against 100 + 1000 exp(-Tu Fpg), Fpg from the wall-normal derivative of
 * the wall distance, CC.f90); the SST constants of the variant (sst2003's
 * gama1, gama2 and limiter 10) */
static void lctm_source(fo_block *b) {
  V q = vqp(b), mu = vpad(b, FO_MU), mut = vpad(b, FO_MUT), F1v = vpad(b, FO_F1), dist = vpad(b, FO_DIST);
  V r = vres(b);
  V g[3] = {vgrad(b, 0), vgrad(b, 1), vgrad(b, 2)};
  R4 fa[3] = {vfaces(b, 0), vfaces(b, 1), vfaces(b, 2)}, cl = vcells(b);
  const int s2003 = b->sc.turbulence == FEST_TURB_SST2003;
  const int limiter = s2003 ? 10 : 20;
  const double cdmin = s2003 ? 1.0e-10 : 1e-20; /* 10.0**(-limiter) */
  double gama1 = (beta1 / bstar) - ((sigma_w1 * (kappa_sst * kappa_sst)) / sqrt(bstar));
  double gama2 = (beta2 / bstar) - ((sigma_w2 * (kappa_sst * kappa_sst)) / sqrt(bstar));
  if (s2003) {
    gama1 = 5.0 / 9.0;
    gama2 = 0.44;
  }
  OMP_FOR
  for (int k = 1; k <= KMX - 1; ++k)
    for (int j = 1; j <= JMX - 1; ++j)
      for (int i = 1; i <= IMX - 1; ++i) {
#define GR(c, l) (*at(g[c], i, j, k, l))
        double density = *at(q, i, j, k, 1), tk = *at(q, i, j, k, 6), tw = *at(q, i, j, k, 7);
        double gm_ = *at(q, i, j, k, 8);
        double wa = GR(1, 3) - GR(2, 2), wb = GR(2, 1) - GR(0, 3), wc = GR(0, 2) - GR(1, 1);
        double vort = sqrt(((wa * wa) + (wb * wb) + (wc * wc)));
        double sa_ = GR(1, 3) + GR(2, 2), sb = GR(2, 1) + GR(0, 3), sc_ = GR(0, 2) + GR(1, 1);
        double strain = sqrt((sa_ * sa_) + (sb * sb) + (sc_ * sc_) + 2 * (GR(0, 1) * GR(0, 1)) +
                             2 * (GR(1, 2) * GR(1, 2)) + 2 * (GR(2, 3) * GR(2, 3)));
        double CD = 2 * density * sigma_w2 * (GR(0, 5) * GR(0, 6) + GR(1, 5) * GR(1, 6) + GR(2, 5) * GR(2, 6)) / tw;
        CD = fmax2(CD, cdmin);
        double F1 = *at(F1v, i, j, k, 1);
        double gama = gama1 * F1 + gama2 * (1. - F1);
        double beta = beta1 * F1 + beta2 * (1. - F1);
        double D_k = bstar * density * tw * tk;
        double D_w = beta * density * (tw * tw);
        double divergence = GR(0, 1) + GR(1, 2) + GR(2, 3);
        double mt = *at(mut, i, j, k, 1), m = *at(mu, i, j, k, 1), d = *at(dist, i, j, k, 1);
        double P_k = mt * (vort * strain) - ((2.0 / 3.0) * density * tk * divergence);
        P_k = fmin2(P_k, limiter * D_k);
        double P_w = (density * gama / mt) * P_k;
        double lamda = (1. - F1) * CD;
        /* CC.f90:56-75, 87-92: the gradient of the wall distance (the same
         * face sums as compute_gradient there) dotted with its unit vector */
        double dd[3];
        {
          const double d0 = d;
          const double dn[6] = {*at(dist, i - 1, j, k, 1), *at(dist, i, j - 1, k, 1), *at(dist, i, j, k - 1, 1),
                                *at(dist, i + 1, j, k, 1), *at(dist, i, j + 1, k, 1), *at(dist, i, j, k + 1, 1)};
          const double *fr[6] = {r4(fa[0], i, j, k), r4(fa[1], i, j, k), r4(fa[2], i, j, k),
                                 r4(fa[0], i + 1, j, k), r4(fa[1], i, j + 1, k), r4(fa[2], i, j, k + 1)};
          const double vol2 = 2 * r4(cl, i, j, k)[0];
          for (int c = 0; c < 3; ++c)
            dd[c] = (-(dn[0] + d0) * fr[0][1 + c] * fr[0][0] - (dn[1] + d0) * fr[1][1 + c] * fr[1][0] -
                     (dn[2] + d0) * fr[2][1 + c] * fr[2][0] + (dn[3] + d0) * fr[3][1 + c] * fr[3][0] +
                     (dn[4] + d0) * fr[4][1 + c] * fr[4][0] + (dn[5] + d0) * fr[5][1 + c] * fr[5][0]) /
                    vol2;
        }
        double Vn = sqrt(dd[0] * dd[0] + dd[1] * dd[1] + dd[2] * dd[2]);
        double dvdy = dd[0] * (dd[0] / (Vn + 1e-12)) + dd[1] * (dd[1] / (Vn + 1e-12)) + dd[2] * (dd[2] / (Vn + 1e-12));
        double lamd = (-7.57e-3) * (dvdy * d * d * density / m) + 0.0128;
        lamd = fmin2(fmax2(lamd, -1.0), 1.0);
        double Fpg = lamd >= 0.0 ? fmin2(1.0 + 14.68 * lamd, 1.5) : fmin2(1.0 - 7.34 * lamd, 3.0);
        Fpg = fmax2(Fpg, 0.0);
        double TuL = fmin2(100.0 * sqrt(2.0 * tk / 3.0) / (tw * d), 100.0);
        double Re_theta = 100.0 + 1000.0 * exp(-TuL * Fpg);
        double Rev = density * d * d * strain / m;
        double RT = density * tk / (m * tw);
        double h = 0.5 * RT, h2 = h * h;
        double Fturb = exp(-(h2 * h2));
        double Fonset1 = Rev / (2.2 * Re_theta);
        double Fonset2 = fmin2(Fonset1, 2.0);
        double t3 = RT / 3.5;
        double Fonset3 = fmax2(1.0 - (t3 * t3) * t3, 0.0);
        double Fonset = fmax2(Fonset2 - Fonset3, 0.0);
        double P_gm = 100 * density * strain * gm_ * (1.0 - gm_) * Fonset;
        double D_gm = 0.06 * density * vort * gm_ * Fturb * ((50.0 * gm_) - 1.0);
        double Fon_lim = fmin2(fmax2((Rev / (2.2 * 1100.0)) - 1.0, 0.0), 3.0);
        double Pk_lim = 5 * fmax2(gm_ - 0.2, 0.0) * (1.0 - gm_) * Fon_lim * fmax2(3 * m - mt, 0.0) * strain * vort;
        double S_k = gm_ * P_k - fmax2(gm_, 0.1) * D_k + Pk_lim;
        double S_w = P_w - D_w + lamda;
        double S_gm = P_gm - D_gm;
        double vol = r4(cl, i, j, k)[0];
        *at(r, i, j, k, 6) = *at(r, i, j, k, 6) - S_k * vol;
        *at(r, i, j, k, 7) = *at(r, i, j, k, 7) - S_w * vol;
        *at(r, i, j, k, 8) = *at(r, i, j, k, 8) - S_gm * vol;
#undef GR
      }
}

/* source.f90:94-155 add_source_term_residue: the SA (and saBC), k-kL and
 * SST (and SST-BC, LCTM2015) sources */
void fo_add_source_term_residue(fo_block *b) {
  const int bc_transition = b->sc.transition == FEST_TRANSITION_BC;
  if (is_sa(b)) {
    if (bc_transition) sa_bc_source(b);
    else sa_source(b);
    return;
  }
  if (is_sst(b) && bc_transition) {
    sst_bc_source(b);
    return;
  }
  if (is_sst(b) && is_lctm(b)) {
    lctm_source(b);
    return;
  }
  if (is_kkl(b)) {
    kkl_source(b);
    return;
  }
  if (!is_sst(b)) return;
  V q = vqp(b), mut = vpad(b, FO_MUT), F1v = vpad(b, FO_F1), r = vres(b);
  V g[3] = {vgrad(b, 0), vgrad(b, 1), vgrad(b, 2)};
  R4 cl = vcells(b);
  int limiter;
  double gama1, gama2;
  if (b->sc.turbulence == FEST_TURB_SST2003) {
    limiter = 10;
    gama1 = 5.0 / 9.0;
    gama2 = 0.44;
  } else {
    limiter = 20;
    gama1 = (beta1 / bstar) - ((sigma_w1 * (kappa_sst * kappa_sst)) / sqrt(bstar));
    gama2 = (beta2 / bstar) - ((sigma_w2 * (kappa_sst * kappa_sst)) / sqrt(bstar));
  }
  double cdmin = 1.0;
  for (int n = 0; n < limiter; ++n) cdmin *= 10.0;
  cdmin = 1.0 / cdmin;
  OMP_FOR
  for (int k = 1; k <= KMX - 1; ++k)
    for (int j = 1; j <= JMX - 1; ++j)
      for (int i = 1; i <= IMX - 1; ++i) {
#define GR(c, l) (*at(g[c], i, j, k, l))
        double rho = *at(q, i, j, k, 1), tk = *at(q, i, j, k, 6), tw = *at(q, i, j, k, 7);
        double a = GR(1, 3) - GR(2, 2), bb = GR(2, 1) - GR(0, 3), c = GR(0, 2) - GR(1, 1);
        double vort = sqrt(((a * a) + (bb * bb) + (c * c)));
        double CD = 2 * rho * sigma_w2 * (GR(0, 5) * GR(0, 6) + GR(1, 5) * GR(1, 6) + GR(2, 5) * GR(2, 6)) / tw;
        CD = fmax2(CD, cdmin);
        double F1 = *at(F1v, i, j, k, 1);
        double gama = gama1 * F1 + gama2 * (1. - F1);
        double beta = beta1 * F1 + beta2 * (1. - F1);
        double Dk = bstar * rho * tw * tk;
        double Dw = beta * rho * (tw * tw);
        double divergence = GR(0, 1) + GR(1, 2) + GR(2, 3);
        double mt = *at(mut, i, j, k, 1);
        double Pk = mt * (vort * vort) - ((2.0 / 3.0) * rho * tk * divergence);
        Pk = fmin2(Pk, limiter * Dk);
        double Pw = (rho * gama / mt) * Pk;
        double lamda = (1. - F1) * CD;
        double Sk = Pk - Dk;
        double Sw = Pw - Dw + lamda;
        double vol = r4(cl, i, j, k)[0];
        Sk = Sk * vol;
        Sw = Sw * vol;
        *at(r, i, j, k, 6) = *at(r, i, j, k, 6) - Sk;
        *at(r, i, j, k, 7) = *at(r, i, j, k, 7) - Sw;
#undef GR
      }
}

/* ======================================================================== */
/* time step (time.f90:122-334, 366-531) */
static void viscous_time(fo_block *b, int mut_part, double CFL) {
  V q = vqp(b), mu = vpad(b, mut_part ? FO_MUT : FO_MU), dt = vdt(b);
  R4 If = vfaces(b, 0), Jf = vfaces(b, 1), Kf = vfaces(b, 2), cl = vcells(b);
  double Pr = mut_part ? b->flow.tPr : b->flow.Pr, gm = b->flow.gm;
  OMP_FOR
  for (int k = 1; k <= KMX - 1; ++k)
    for (int j = 1; j <= JMX - 1; ++j)
      for (int i = 1; i <= IMX - 1; ++i) {
        const double *cc = r4(cl, i, j, k);
        double lmx[6];
        R4 fas[3] = {If, Jf, Kf};
        for (int d = 0; d < 3; ++d) {
          int di = d == 0, dj = d == 1, dk = d == 2;
          const double *cm = r4(cl, i - di, j - dj, k - dk), *cp = r4(cl, i + di, j + dj, k + dk);
          const double *f0 = r4(fas[d], i, j, k), *f1 = r4(fas[d], i + di, j + dj, k + dk);
          lmx[d] = *at(mu, i, j, k, 1) /
                   (*at(q, i, j, k, 1) * fabs(((cm[1] - cc[1]) * f0[1]) + ((cm[2] - cc[2]) * f0[2]) + ((cm[3] - cc[3]) * f0[3])));
          lmx[3 + d] = *at(mu, i + di, j + dj, k + dk, 1) /
                       (*at(q, i + di, j + dj, k + dk, 1) *
                        fabs(((cc[1] - cp[1]) * f1[1]) + ((cc[2] - cp[2]) * f1[2]) + ((cc[3] - cp[3]) * f1[3])));
        }
        double s = (r4(If, i, j, k)[0] * lmx[0]) + (r4(Jf, i, j, k)[0] * lmx[1]) + (r4(Kf, i, j, k)[0] * lmx[2]) +
                   (r4(If, i + 1, j, k)[0] * lmx[3]) + (r4(Jf, i, j + 1, k)[0] * lmx[4]) + (r4(Kf, i, j, k + 1)[0] * lmx[5]);
        s = gm * s / Pr;
        s = 2. / (s + (2. * CFL * cc[0] / *at(dt, i, j, k, 1)));
        *at(dt, i, j, k, 1) = CFL * (s * cc[0]);
      }
}

static void local_time_step(fo_block *b, double CFL) {
  V q = vqp(b), dt = vdt(b);
  R4 If = vfaces(b, 0), Jf = vfaces(b, 1), Kf = vfaces(b, 2), cl = vcells(b);
  double gm = b->flow.gm;
  V Ls[3], Rs[3];
  for (int d = 0; d < 3; ++d) { Ls[d] = vfs(b, FO_XL + 2 * d, d); Rs[d] = vfs(b, FO_XR + 2 * d, d); }
  OMP_FOR
  for (int k = 1; k <= KMX - 1; ++k)
    for (int j = 1; j <= JMX - 1; ++j)
      for (int i = 1; i <= IMX - 1; ++i) {
        double lmx[6];
        R4 fas[3] = {If, Jf, Kf};
        for (int d = 0; d < 3; ++d) {
          int di = d == 0, dj = d == 1, dk = d == 2;
          double c0 = 0.5 * (sqrt(gm * *at(Ls[d], i, j, k, 5) / *at(Ls[d], i, j, k, 1)) +
                             sqrt(gm * *at(Rs[d], i, j, k, 5) / *at(Rs[d], i, j, k, 1)));
          const double *f0 = r4(fas[d], i, j, k);
          lmx[d] = fabs((*at(q, i, j, k, 2) * f0[1]) + (*at(q, i, j, k, 3) * f0[2]) + (*at(q, i, j, k, 4) * f0[3])) + c0;
          double c1 = 0.5 * (sqrt(gm * *at(Ls[d], i + di, j + dj, k + dk, 5) / *at(Ls[d], i + di, j + dj, k + dk, 1)) +
                             sqrt(gm * *at(Rs[d], i + di, j + dj, k + dk, 5) / *at(Rs[d], i + di, j + dj, k + dk, 1)));
          const double *f1 = r4(fas[d], i + di, j + dj, k + dk);
          lmx[3 + d] = fabs((*at(q, i + di, j + dj, k + dk, 2) * f1[1]) + (*at(q, i + di, j + dj, k + dk, 3) * f1[2]) +
                            (*at(q, i + di, j + dj, k + dk, 4) * f1[3])) +
                       c1;
        }
        double s = (r4(If, i, j, k)[0] * lmx[0]) + (r4(Jf, i, j, k)[0] * lmx[1]) + (r4(Kf, i, j, k)[0] * lmx[2]) +
                   (r4(If, i + 1, j, k)[0] * lmx[3]) + (r4(Jf, i, j + 1, k)[0] * lmx[4]) + (r4(Kf, i, j, k + 1)[0] * lmx[5]);
        double t = 1. / s;
        *at(dt, i, j, k, 1) = t * r4(cl, i, j, k)[0] * CFL;
      }
  if (b->flow.mu_ref != 0.0) viscous_time(b, 0, CFL);
  if (b->flow.mu_ref != 0 && is_turb(b)) viscous_time(b, 1, CFL);
}

void fo_compute_time_step(fo_block *b, double CFL) {
  long N = b->sz[FO_DT];
  if (b->sc.time_stepping_method == 'g') {
    if (b->sc.global_time_step > 0) {
      for (long p = 0; p < N; ++p) b->a[FO_DT][p] = b->sc.global_time_step;
    } else {
      local_time_step(b, CFL);
      double m = b->a[FO_DT][0];
      for (long p = 1; p < N; ++p) m = fmin2(m, b->a[FO_DT][p]);
      for (long p = 0; p < N; ++p) b->a[FO_DT][p] = m;
    }
  } else {
    local_time_step(b, CFL);
  }
}

/* ======================================================================== */
/* update_with, conservative branch (update.f90:367-485) */
int fo_update_with(fo_block *b, double TF, double SF, int TU, int use_store) {
  V q = vqp(b), r = vres(b), dt = vdt(b), F1v = vpad(b, FO_F1);
  V Qu = use_store ? vpad(b, FO_USTORE) : q;
  if (use_store) Qu = mkv(b->a[FO_USTORE], -2, -2, -2, IMX + 5, JMX + 5, KMX + 5);
  V Rn = mkv(b->a[FO_RSTORE], 1, 1, 1, IMX - 1, JMX - 1, KMX - 1);
  R4 cl = vcells(b);
  double gm = b->flow.gm;
  int n = NV, sst = is_sst(b), sa = is_sa(b), kkl = is_kkl(b);
  V mu = vpad(b, FO_MU), dist = vpad(b, FO_DIST);
  V g[3] = {vgrad(b, 0), vgrad(b, 1), vgrad(b, 2)};
  int err = FEST_OK;
  OMP_FOR
  for (int k = 1; k <= KMX - 1; ++k)
    for (int j = 1; j <= JMX - 1; ++j)
      for (int i = 1; i <= IMX - 1; ++i) {
        double u1[8], u2[8], R[8];
        u1[0] = *at(Qu, i, j, k, 1);
        for (int l = 2; l <= n; ++l) u1[l - 1] = *at(Qu, i, j, k, l) * u1[0];
        double s1 = 0.0 + u1[1] * u1[1] + u1[2] * u1[2] + u1[3] * u1[3];
        u1[4] = (u1[4] / (gm - 1.) + 0.5 * s1) / u1[0] + 0.0;
        for (int l = 1; l <= n; ++l) R[l - 1] = *at(r, i, j, k, l);
        double dtc = *at(dt, i, j, k, 1);
        if (sst) {
          double F1 = *at(F1v, i, j, k, 1);
          double beta = beta1 * F1 + (1. - F1) * beta2;
          double w = *at(q, i, j, k, 7);
          R[5] = R[5] / (1 + (beta * w * dtc));
          R[6] = R[6] / (1 + (2 * beta * w * dtc));
        }
        if (kkl) {
          /* update.f90:399-404, with the conservative U1(6), U1(7) */
          double d = *at(dist, i, j, k, 1), m = *at(mu, i, j, k, 1);
          double eta = u1[0] * d * (sqrt(0.3 * u1[5]) / (20 * m));
          double e2 = eta * eta;
          double fphi = (1 + kkl_cd1 * eta) / (1 + e2 * e2);
          R[5] = R[5] / (1. + ((2.5 * ((pow(kkl_cmu, 0.75) * sqrt(u1[0]) * (pow(u1[5], 1.5))) / fmax2(u1[6], 1.e-20))) +
                               (2 * m / (d * d))) * dtc);
          R[6] = R[6] / (1. + (6 * m * fphi / (d * d)) * dtc);
        }
        if (sa) {
          /* update.f90:405-419: xi from the conservative U1(6) and the
           * stage state's density, as written there */
#define GR(c, l) (*at(g[c], i, j, k, l))
          double wa = GR(1, 3) - GR(2, 2), wb = GR(2, 1) - GR(0, 3), wc = GR(0, 2) - GR(1, 1);
          double vort = sqrt(((wa * wa) + (wb * wb) + (wc * wc)));
#undef GR
          double d = *at(dist, i, j, k, 1);
          double kd = kappa_sa * d, kd2 = kd * kd;
          double xi = u1[5] * *at(q, i, j, k, 1) / *at(mu, i, j, k, 1);
          double x3 = xi * xi * xi;
          double fv1 = x3 / (x3 + pow(cv1, 3.0));
          double fv2 = 1.0 - xi / (1 + xi * fv1);
          double scap = vort + u1[5] * fv2 / (kd2);
          double rsa = fmin2(u1[5] / (scap * kd2), 10.0);
          double gg = rsa + cw2 * (pow6(rsa) - rsa);
          double fw = gg * pow((1.0 + pow6(cw3)) / (pow6(gg) + pow6(cw3)), 1.0 / 6.0);
          R[5] = R[5] / (1. + ((-1.0 * u1[0] * cb1 * scap) + (2.0 * u1[0] * CW1_SA * fw * u1[5] / (d * d))) * dtc);
        }
        if (use_store) {
          for (int l = 1; l <= n; ++l) *at(Rn, i, j, k, l) = *at(Rn, i, j, k, l) + SF * R[l - 1];
          if (TU)
            for (int l = 1; l <= n; ++l) R[l - 1] = *at(Rn, i, j, k, l);
        }
        double fac = (TF * dtc / r4(cl, i, j, k)[0]);
        for (int l = 0; l < n; ++l) u2[l] = u1[l] - R[l] * fac;
        for (int l = 1; l < n; ++l) u2[l] = u2[l] / u2[0];
        double s2 = 0.0 + u2[1] * u2[1] + u2[2] * u2[2] + u2[3] * u2[3];
        u2[4] = (gm - 1.) * u2[0] * ((u2[4] - (0.5 * s2)) - 0.0);
        int bad = (u2[0] < 0.) || (u2[4] < 0.);
        for (int l = 0; l < n; ++l)
          if (u2[l] != u2[l]) bad = 1;
        if (bad) {
#ifdef _OPENMP
#pragma omp atomic write
#endif
          err = FEST_ERR_NEGATIVE_STATE;
          continue;
        }
        for (int l = 1; l <= 5; ++l) *at(q, i, j, k, l) = u2[l - 1];
        if (sst || kkl) { /* update.f90:456-470 */
          if (u2[5] >= 0.) *at(q, i, j, k, 6) = u2[5];
          if (u2[6] >= 0.) *at(q, i, j, k, 7) = u2[6];
        }
        if (sa) *at(q, i, j, k, 6) = fmax2(u2[5], 1.e-12); /* update.f90:474-475 */
      }
  return err;
}

/* ======================================================================== */
/* update.f90:495-547 get_total_conservative_Residue over all blocks */
int fo_get_total_conservative_residue(fo_block **bl, int nb, int it) {
  int err = FEST_OK, e;
  fo_apply_interface(bl, nb);
  for (int n = 0; n < nb; ++n) {
    fo_block *b = bl[n];
    fo_populate_ghost_primitive(b, it);
    if ((e = fo_compute_face_interpolant(b))) err = e;
    fo_reconstruct_boundary_state(b);
    if ((e = fo_compute_fluxes(b))) err = e;
    if (b->flow.mu_ref != 0.0) {
      if ((e = fo_evaluate_all_gradients(b))) err = e;
      if ((e = fo_calculate_viscosity(b))) err = e;
      if ((e = fo_compute_viscous_fluxes(b))) err = e;
    }
    fo_compute_residue(b);
    fo_add_source_term_residue(b);
  }
  return err;
}

static void blend(fo_block *b, double a, double c) {
  long n = b->sz[FO_QP];
  double *q = b->a[FO_QP], *u = b->a[FO_USTORE];
  for (long p = 0; p < n; ++p) q[p] = a * u[p] + c * q[p];
}

/* update.f90:129-226 get_next_solution */
int fo_get_next_solution(fo_block **bl, int nb, int it, double CFL) {
  int err = FEST_OK, e;
#define RES() do { if ((e = fo_get_total_conservative_residue(bl, nb, it))) err = e; } while (0)
#define EACH for (int n = 0; n < nb; ++n)
#define UPD(TF, SF, TU, ST) EACH { if ((e = fo_update_with(bl[n], TF, SF, TU, ST))) err = e; }
  EACH fo_compute_temperature(bl[n]);
  int acc = bl[0]->sc.time_step_accuracy;
  switch (acc) {
  case FEST_TIME_NONE:
    RES();
    EACH fo_compute_time_step(bl[n], CFL);
    UPD(1., 1., 0, 0);
    break;
  case FEST_TIME_RK4:
    EACH { memset(bl[n]->a[FO_RSTORE], 0, sizeof(double) * bl[n]->sz[FO_RSTORE]);
           memcpy(bl[n]->a[FO_USTORE], bl[n]->a[FO_QP], sizeof(double) * bl[n]->sz[FO_QP]); }
    RES();
    EACH fo_compute_time_step(bl[n], CFL);
    UPD(0.5, 1., 0, 1);
    RES(); UPD(0.5, 2., 0, 1);
    RES(); UPD(1.0, 2., 0, 1);
    RES(); UPD(1. / 6., 1., 1, 1);
    break;
  case FEST_TIME_RK2:
    EACH { memset(bl[n]->a[FO_RSTORE], 0, sizeof(double) * bl[n]->sz[FO_RSTORE]);
           memcpy(bl[n]->a[FO_USTORE], bl[n]->a[FO_QP], sizeof(double) * bl[n]->sz[FO_QP]); }
    RES();
    EACH fo_compute_time_step(bl[n], CFL);
    UPD(0.5, 1., 0, 1);
    RES(); UPD(0.5, 1., 1, 1);
    break;
  case FEST_TIME_TVDRK3:
    EACH memcpy(bl[n]->a[FO_USTORE], bl[n]->a[FO_QP], sizeof(double) * bl[n]->sz[FO_QP]);
    RES();
    EACH fo_compute_time_step(bl[n], CFL);
    UPD(1.0, 1., 0, 0);
    RES(); UPD(1.0, 1., 0, 0);
    EACH blend(bl[n], 0.75, 0.25);
    RES(); UPD(1.0, 1., 0, 0);
    EACH blend(bl[n], 1. / 3., 2. / 3.);
    break;
  case FEST_TIME_TVDRK2:
    EACH memcpy(bl[n]->a[FO_USTORE], bl[n]->a[FO_QP], sizeof(double) * bl[n]->sz[FO_QP]);
    RES();
    EACH fo_compute_time_step(bl[n], CFL);
    UPD(1.0, 1., 0, 0);
    RES(); UPD(1.0, 1., 0, 0);
    EACH blend(bl[n], 0.5, 0.5);
    break;
  default:
    return FEST_ERR_ARG;
  }
#undef RES
#undef EACH
#undef UPD
  return err;
}

/* ======================================================================== */
/* Implicit LU-SGS (lusgs.f90:186-683 laminar, 686-1196 k-omega SST).  Not
 * part of the explicit path: the reference runs its flat-plate test cases
 * with this integrator ("implicit", update.f90:215-218), and the oracle
 * restates it only to replay those runs iteration for iteration. */

/* one face seen from the cell being updated: area, outward normal, and the
 * means over the two cells of volume, laminar and eddy viscosity and the
 * SST blending F1 (lusgs.f90:278-324, 783-835) */
typedef struct { double A, nx, ny, nz, vol, mu, mut, F1; } lu_face;

/* lusgs.f90:491-630 Flux and 1027-1196 SSTFlux: the inviscid flux of the
 * neighbour state ql advanced by the conservative change du (k and omega
 * kept at ql's values where the advanced ones turn negative), less the
 * thin-layer viscous flux between that state and the cell state qr, times
 * the area; n = 5 (laminar), 7 (SST) or 8 (LCTM2015, lctm2015Flux of
 * lusgs.f90:2702-2856: the intermittency floored at zero, not kept, and
 * diffused with mu + mu_t) */
static void lu_flux(const fest_flow *fl, int n, const double *ql, const double *qr, const double *du,
                    const lu_face *f, double *out) {
  const double gm = fl->gm, R = fl->R_gas;
  double U[8], W[8];
  U[0] = ql[0];
  U[1] = ql[0] * ql[1];
  U[2] = ql[0] * ql[2];
  U[3] = ql[0] * ql[3];
  U[4] = (ql[4] / (gm - 1.0)) + (0.5 * ql[0] * (ql[1] * ql[1] + ql[2] * ql[2] + ql[3] * ql[3]));
  for (int l = 5; l < n; ++l) U[l] = ql[0] * ql[l];
  for (int l = 0; l < n; ++l) U[l] = U[l] + du[l];
  W[0] = U[0];
  W[1] = U[1] / U[0];
  W[2] = U[2] / U[0];
  W[3] = U[3] / U[0];
  W[4] = (gm - 1.0) * (U[4] - (0.5 * (U[1] * U[1] + U[2] * U[2] + U[3] * U[3]) / U[0]));
  for (int l = 5; l < n; ++l) {
    W[l] = U[l] / U[0];
    if (l < 7) W[l] = W[l] + 0.5 * (1. - fsign(1., W[l])) * (ql[l] - W[l]);
    else W[l] = fmax2(W[l], 0.0);
  }
  const double nx = f->nx, ny = f->ny, nz = f->nz;
  double vn = (W[1] * nx) + (W[2] * ny) + (W[3] * nz);
  double uf = 0.5 * (W[1] + qr[1]), vf = 0.5 * (W[2] + qr[2]), wf = 0.5 * (W[3] + qr[3]);
  out[0] = W[0] * vn;
  out[1] = (W[1] * out[0]) + (W[4] * nx);
  out[2] = (W[2] * out[0]) + (W[4] * ny);
  out[3] = (W[3] * out[0]) + (W[4] * nz);
  double half_rho_u2 = 0.5 * W[0] * (W[1] * W[1] + W[2] * W[2] + W[3] * W[3]);
  out[4] = (((gm / (gm - 1.0)) * W[4]) + half_rho_u2) * vn;
  for (int l = 5; l < n; ++l) out[l] = W[l] * out[0];
  /* differences across the face as the only gradient */
  const double mu = f->mu + f->mut, s = f->A;
  double T1 = W[4] / (W[0] * R), T2 = qr[4] / (qr[0] * R);
  double dT[3] = {(T2 - T1) * nx * s / f->vol, (T2 - T1) * ny * s / f->vol, (T2 - T1) * nz * s / f->vol};
  double g[6][3]; /* g[c][d]: d(u, v, w, k, omega, intermittency)/d(x_d) */
  for (int c = 0; c < 3 + (n - 5); ++c) {
    double dv = qr[c < 3 ? 1 + c : 2 + c] - W[c < 3 ? 1 + c : 2 + c];
    g[c][0] = dv * nx * s / f->vol;
    g[c][1] = dv * ny * s / f->vol;
    g[c][2] = dv * nz * s / f->vol;
  }
  double tr = g[0][0] + g[1][1] + g[2][2];
  double txx = 2. * mu * (g[0][0] - tr / 3.0), tyy = 2. * mu * (g[1][1] - tr / 3.0),
         tzz = 2. * mu * (g[2][2] - tr / 3.0);
  double txy = mu * (g[1][0] + g[0][1]), txz = mu * (g[2][0] + g[0][2]), tyz = mu * (g[2][1] + g[1][2]);
  double kh = (f->mu / fl->Pr + f->mut / fl->tPr) * gm * R / (gm - 1.0);
  out[1] = out[1] - (txx * nx + txy * ny + txz * nz);
  out[2] = out[2] - (txy * nx + tyy * ny + tyz * nz);
  out[3] = out[3] - (txz * nx + tyz * ny + tzz * nz);
  out[4] = out[4] - (txx * uf + txy * vf + txz * wf + kh * dT[0]) * nx;
  out[4] = out[4] - (txy * uf + tyy * vf + tyz * wf + kh * dT[1]) * ny;
  out[4] = out[4] - (txz * uf + tyz * vf + tzz * wf + kh * dT[2]) * nz;
  if (n == 7) {
    double sk = sigma_k1 * f->F1 + sigma_k2 * (1.0 - f->F1), sw = sigma_w1 * f->F1 + sigma_w2 * (1.0 - f->F1);
    /* added, as lusgs.f90:1190-1191 has it */
    out[5] = out[5] + (f->mu + sk * f->mut) * (g[3][0] * nx + g[3][1] * ny + g[3][2] * nz);
    out[6] = out[6] + (f->mu + sw * f->mut) * (g[4][0] * nx + g[4][1] * ny + g[4][2] * nz);
  }
  if (n == 8) {
    double sk = sigma_k1 * f->F1 + sigma_k2 * (1.0 - f->F1), sw = sigma_w1 * f->F1 + sigma_w2 * (1.0 - f->F1);
    out[5] = out[5] + (f->mu + sk * f->mut) * (g[3][0] * nx + g[3][1] * ny + g[3][2] * nz);
    out[6] = out[6] + (f->mu + sw * f->mut) * (g[4][0] * nx + g[4][1] * ny + g[4][2] * nz);
    out[7] = out[7] + (f->mu + f->mut) * (g[5][0] * nx + g[5][1] * ny + g[5][2] * nz);
  }
  for (int l = 0; l < n; ++l) out[l] = out[l] * s;
}

/* lusgs.f90:633-683 SpectralRadius: convective plus viscous spectral
 * radius of the face, times its area; ca, cb the two cell centres */
static double lu_radius(const fest_flow *fl, const double *qa, const double *qb, const lu_face *f,
                        const double *ca, const double *cb) {
  const double gm = fl->gm;
  double vn = fabs(0.5 * (((qa[1] + qb[1]) * f->nx) + ((qa[2] + qb[2]) * f->ny) + ((qa[3] + qb[3]) * f->nz)));
  double c = 0.5 * (sqrt(gm * qa[4] / qa[0]) + sqrt(gm * qb[4] / qb[0]));
  double rho = 0.5 * (qa[0] + qb[0]);
  double dx = ca[0] - cb[0], dy = ca[1] - cb[1], dz = ca[2] - cb[2];
  double dist = sqrt(dx * dx + dy * dy + dz * dz);
  double vis = gm * (f->mu / fl->Pr + f->mut / fl->tPr) / (rho * dist);
  return (vn + c + vis) * f->A;
}

/* plusgs.f90:723-776 SpectralRadius of the low-Mach preconditioned system:
 * eps is the cell's own min(1, max(M^2, Minf^2)), and the viscous part is
 * twice LU-SGS's */
static double plu_radius(const fest_flow *fl, const double *qa, const double *qb, const lu_face *f,
                         const double *ca, const double *cb, double eps) {
  const double gm = fl->gm;
  double vn = fabs(0.5 * (((qa[1] + qb[1]) * f->nx) + ((qa[2] + qb[2]) * f->ny) + ((qa[3] + qb[3]) * f->nz)));
  double c = 0.5 * (sqrt(gm * qa[4] / qa[0]) + sqrt(gm * qb[4] / qb[0]));
  double rho = 0.5 * (qa[0] + qb[0]);
  double dx = ca[0] - cb[0], dy = ca[1] - cb[1], dz = ca[2] - cb[2];
  double dist = sqrt(dx * dx + dy * dy + dz * dz);
  double vis = 2.0 * gm * (f->mu / fl->Pr + f->mut / fl->tPr) / (rho * dist);
  return (0.5 * ((1.0 + eps) * vn + sqrt(((eps - 1.0) * (eps - 1.0)) * (vn * vn) + 4 * eps * (c * c))) + vis) * f->A;
}

/* plusgs.f90:345-396 (laminar), 944-1014 (SST): the cell's eps and the
 * inverse preconditioner P = I - factor x c^T, x = (1, u, v, w, H[, k,
 * omega]), c = (|V|^2/2, -u, -v, -w, 1[, -1, 0]), H with the reference's
 * 0.5 |V| (not |V|^2), each entry in the reference's evaluation order */
static double plu_precond(const fest_flow *fl, int n, const double *q0, double P[8][8]) {
  const double gm = fl->gm;
  double r = q0[0], u = q0[1], v = q0[2], w = q0[3], p = q0[4];
  double VMag = sqrt(u * u + v * v + w * w);
  double SoundMag = sqrt(gm * p / r);
  double M = VMag / SoundMag;
  double H = (gm * p / (r * (gm - 1.0))) + 0.5 * (VMag);
  double eps = fmin(1.0, fmax(M * M, fl->MInf * fl->MInf));
  double factor = (1.0 - eps) * (gm - 1.0) / (SoundMag * SoundMag);
  /* plusgs.f90:2338-2355: LCTM2015 adds the intermittency to x, a zero to c */
  double x[8] = {1, u, v, w, H, n >= 7 ? q0[5] : 0, n >= 7 ? q0[6] : 0, n == 8 ? q0[7] : 0};
  for (int i = 0; i < n; ++i) {
    double fx = factor * x[i];
    P[i][0] = (i == 0 ? 1.0 : 0.0) - fx * VMag * VMag / 2.0;
    P[i][1] = (i == 1 ? 1.0 : 0.0) - fx * (-u);
    P[i][2] = (i == 2 ? 1.0 : 0.0) - fx * (-v);
    P[i][3] = (i == 3 ? 1.0 : 0.0) - fx * (-w);
    P[i][4] = (i == 4 ? 1.0 : 0.0) - fx * (1.);
    if (n >= 7) {
      P[i][5] = (i == 5 ? 1.0 : 0.0) - fx * (-1.);
      P[i][6] = (i == 6 ? 1.0 : 0.0) - fx * (0.);
    }
    if (n == 8) P[i][7] = (i == 7 ? 1.0 : 0.0) - fx * (0.);
  }
  return eps;
}

static void plu_apply(int n, double P[8][8], const double *y, double *out) {
  for (int i = 0; i < n; ++i) {
    double s = 0.0;
    for (int j = 0; j < n; ++j) s = s + P[i][j] * y[j];
    out[i] = s;
  }
}

/* lusgs.f90:186-488 update_laminar_variables, 686-1024
 * update_SST_variables: forward sweep for dQ*, back sweep for dQ, then the
 * conservative update of the interior cells (k and omega only where they
 * stay positive).  dQ is zero outside the block, so neighbouring blocks do
 * not couple.  With plus, the low-Mach preconditioned form of
 * plusgs.f90:191-577 and 779-1256: P applied to the residual and to the
 * flux differences, the preconditioned spectral radii. */
static void lu_sgs(fo_block *b, int plus) {
  const fest_flow *fl = &b->flow;
  const int imx = IMX, jmx = JMX, kmx = KMX, n = NV, sst = is_sst(b);
  V q = vqp(b), mu = vpad(b, FO_MU), mut = vpad(b, FO_MUT), F1 = vpad(b, FO_F1), r = vres(b), dt = vdt(b);
  V dist = vpad(b, FO_DIST);
  V g[3] = {vgrad(b, 0), vgrad(b, 1), vgrad(b, 2)};
  R4 cl = vcells(b), fa[3] = {vfaces(b, 0), vfaces(b, 1), vfaces(b, 2)};
  size_t cnt = (size_t)(imx + 1) * (jmx + 1) * (kmx + 1) * n;
  V dqs = mkv((double *)calloc(cnt, sizeof(double)), 0, 0, 0, imx + 1, jmx + 1, kmx + 1);
  V dq = mkv((double *)calloc(cnt, sizeof(double)), 0, 0, 0, imx + 1, jmx + 1, kmx + 1);
  static const int off[3][3] = {{1, 0, 0}, {0, 1, 0}, {0, 0, 1}};
  for (int pass = 0; pass < 2; ++pass) {
    /* forward: k, j, i ascending; back: i, j, k descending (lusgs.f90:363-365) */
    int ncell = (imx - 1) * (jmx - 1) * (kmx - 1);
    for (int c = 0; c < ncell; ++c) {
      int i, j, k;
      if (pass == 0) {
        i = 1 + c % (imx - 1);
        j = 1 + (c / (imx - 1)) % (jmx - 1);
        k = 1 + c / ((imx - 1) * (jmx - 1));
      } else {
        k = kmx - 1 - c % (kmx - 1);
        j = jmx - 1 - (c / (kmx - 1)) % (jmx - 1);
        i = imx - 1 - c / ((kmx - 1) * (jmx - 1));
      }
      double q0[8], qn[6][8], lam[6], sumlam = 0., P[8][8], eps = 0.0;
      lu_face fc[6];
      const double *c0 = r4(cl, i, j, k) + 1;
      for (int l = 0; l < n; ++l) q0[l] = *at(q, i, j, k, l + 1);
      if (plus) eps = plu_precond(fl, n, q0, P);
      for (int s = 0; s < 6; ++s) { /* 0..2 low i/j/k neighbour, 3..5 high */
        int d = s % 3, hi = s / 3;
        int ni = i + (hi ? off[d][0] : -off[d][0]), nj = j + (hi ? off[d][1] : -off[d][1]),
            nk = k + (hi ? off[d][2] : -off[d][2]);
        const double *f = r4(fa[d], i + hi * off[d][0], j + hi * off[d][1], k + hi * off[d][2]);
        double sg = hi ? 1.0 : -1.0;
        fc[s].A = f[0];
        fc[s].nx = sg * f[1];
        fc[s].ny = sg * f[2];
        fc[s].nz = sg * f[3];
        fc[s].vol = 0.5 * (r4(cl, ni, nj, nk)[0] + r4(cl, i, j, k)[0]);
        fc[s].mu = 0.5 * (*at(mu, ni, nj, nk, 1) + *at(mu, i, j, k, 1));
        fc[s].mut = sst ? 0.5 * (*at(mut, ni, nj, nk, 1) + *at(mut, i, j, k, 1)) : 0.0;
        fc[s].F1 = sst ? 0.5 * (*at(F1, ni, nj, nk, 1) + *at(F1, i, j, k, 1)) : 0.0;
        for (int l = 0; l < n; ++l) qn[s][l] = *at(q, ni, nj, nk, l + 1);
        lam[s] = plus ? plu_radius(fl, qn[s], q0, &fc[s], r4(cl, ni, nj, nk) + 1, c0, eps)
                      : lu_radius(fl, qn[s], q0, &fc[s], r4(cl, ni, nj, nk) + 1, c0);
      }
      for (int s = 0; s < 6; ++s) sumlam = sumlam + lam[s];
      const double vol = r4(cl, i, j, k)[0];
      double D[8];
      for (int l = 0; l < n; ++l) D[l] = (vol / *at(dt, i, j, k, 1)) + 0.5 * sumlam;
      if (sst) { /* lusgs.f90:860-862: the destruction terms of k and omega */
        double f1 = *at(F1, i, j, k, 1), beta = f1 * beta1 + (1.0 - f1) * beta2, w = q0[6];
        D[5] = (D[5] + (bstar * w) * vol);
        D[6] = (D[6] + 2.0 * beta * w * vol);
      }
      if (n == 8) { /* lusgs.f90:2455-2475: the intermittency's source, linearised */
#define GR(c, l) (*at(g[c], i, j, k, l))
        double density = q0[0], d = *at(dist, i, j, k, 1), m = *at(mu, i, j, k, 1);
        double wa = GR(1, 3) - GR(2, 2), wb = GR(2, 1) - GR(0, 3), wc = GR(0, 2) - GR(1, 1);
        double vort = sqrt(((wa * wa) + (wb * wb) + (wc * wc)));
        double sa_ = GR(1, 3) + GR(2, 2), sb = GR(2, 1) + GR(0, 3), sc_ = GR(0, 2) + GR(1, 1);
        double strain = sqrt((sa_ * sa_) + (sb * sb) + (sc_ * sc_) + 2 * (GR(0, 1) * GR(0, 1)) +
                             2 * (GR(1, 2) * GR(1, 2)) + 2 * (GR(2, 3) * GR(2, 3)));
#undef GR
        double TuL = fmin2(100.0 * sqrt(2.0 * q0[5] / 3.0) / (q0[6] * d), 100.0);
        double Re_theta = 100.0 + 1000.0 * exp(-TuL);
        double Rev = density * d * d * strain / m;
        double RT = density * q0[5] / (m * q0[6]);
        double h = 0.5 * RT, h2 = h * h;
        double Fturb = exp(-(h2 * h2));
        double Fonset2 = fmin2(Rev / (2.2 * Re_theta), 2.0);
        double t3 = RT / 3.5;
        double Fonset3 = fmax2(1.0 - (t3 * t3) * t3, 0.0);
        double Fonset = fmax2(Fonset2 - Fonset3, 0.0);
        double Dp = 100 * density * strain * Fonset * (1.0 - 2.0 * q0[7]);
        double De = 0.06 * vort * Fturb * density * (2.0 * 50.0 * q0[7] - 1.0);
        D[7] = (D[7] + (-Dp + De) * vol);
      }
      double acc[8] = {0, 0, 0, 0, 0, 0, 0, 0};
      for (int d = 0; d < 3; ++d) {
        int s = pass == 0 ? d : 3 + d;
        int ni = i + (pass ? off[d][0] : -off[d][0]), nj = j + (pass ? off[d][1] : -off[d][1]),
            nk = k + (pass ? off[d][2] : -off[d][2]);
        V src = pass == 0 ? dqs : dq;
        double dn[8], zero[8] = {0, 0, 0, 0, 0, 0, 0, 0}, fnew[8], fold[8];
        for (int l = 0; l < n; ++l) dn[l] = *at(src, ni, nj, nk, l + 1);
        lu_flux(fl, n, qn[s], q0, dn, &fc[s], fnew);
        lu_flux(fl, n, qn[s], q0, zero, &fc[s], fold);
        double df[8], pdf[8];
        for (int l = 0; l < n; ++l) df[l] = fnew[l] - fold[l];
        if (plus) plu_apply(n, P, df, pdf);
        for (int l = 0; l < n; ++l) acc[l] = acc[l] + ((plus ? pdf[l] : df[l]) - lam[s] * dn[l]);
      }
      double rr[8], pr[8];
      for (int l = 0; l < n; ++l) rr[l] = *at(r, i, j, k, l + 1);
      if (plus) plu_apply(n, P, rr, pr);
      for (int l = 0; l < n; ++l) {
        if (pass == 0)
          *at(dqs, i, j, k, l + 1) = (-(plus ? pr[l] : rr[l]) - 0.5 * acc[l]) / D[l];
        else
          *at(dq, i, j, k, l + 1) = *at(dqs, i, j, k, l + 1) - 0.5 * acc[l] / D[l];
      }
    }
  }
  const double gm = fl->gm;
  for (int k = 1; k <= kmx - 1; ++k)
    for (int j = 1; j <= jmx - 1; ++j)
      for (int i = 1; i <= imx - 1; ++i) {
        double *p[8], U[8];
        for (int l = 0; l < n; ++l) p[l] = at(q, i, j, k, l + 1);
        U[0] = *p[0];
        U[1] = *p[0] * *p[1];
        U[2] = *p[0] * *p[2];
        U[3] = *p[0] * *p[3];
        U[4] = (*p[4] / (gm - 1.0)) + (0.5 * *p[0] * (*p[1] * *p[1] + *p[2] * *p[2] + *p[3] * *p[3]));
        for (int l = 5; l < n; ++l) U[l] = *p[0] * *p[l];
        for (int l = 0; l < n; ++l) U[l] = U[l] + *at(dq, i, j, k, l + 1);
        *p[0] = U[0];
        *p[1] = U[1] / U[0];
        *p[2] = U[2] / U[0];
        *p[3] = U[3] / U[0];
        *p[4] = (gm - 1.0) * (U[4] - (0.5 * (U[1] * U[1] + U[2] * U[2] + U[3] * U[3]) / U[0]));
        for (int l = 5; l < n && l < 7; ++l)
          if (U[l] > 0) *p[l] = U[l] / U[0];
        if (n == 8) { /* lusgs.f90:2685-2687 */
          *p[7] = U[7] / U[0];
          *p[7] = fmax2(*p[7], 0.0);
        }
      }
  free(dqs.p);
  free(dq.p);
}

/* update.f90:215-218 (LU-SGS) and 219-222 (PLU-SGS): one implicit
 * iteration; laminar and k-omega SST blocks (lusgs.f90:158-164,
 * plusgs.f90:161-170) */
static int implicit_next_solution(fo_block **bl, int nb, int it, double CFL, int plus) {
  for (int n = 0; n < nb; ++n) {
    int t = bl[n]->sc.turbulence, lctm = is_lctm(bl[n]);
    if (!((t == FEST_TURB_NONE && bl[n]->d.n_var == 5) ||
          ((t == FEST_TURB_SST || t == FEST_TURB_SST2003) && bl[n]->d.n_var == 7 + lctm)))
      return FEST_ERR_ARG;
  }
  for (int n = 0; n < nb; ++n) fo_compute_temperature(bl[n]);
  int err = fo_get_total_conservative_residue(bl, nb, it);
  for (int n = 0; n < nb; ++n) {
    fo_compute_time_step(bl[n], CFL);
    lu_sgs(bl[n], plus);
  }
  return err;
}

int fo_lusgs_next_solution(fo_block **bl, int nb, int it, double CFL) {
  return implicit_next_solution(bl, nb, it, CFL, 0);
}

int fo_plusgs_next_solution(fo_block **bl, int nb, int it, double CFL) {
  return implicit_next_solution(bl, nb, it, CFL, 1);
}

/* resnorm.f90:128-225 */
void fo_find_resnorm(fo_block **bl, int nb, double *out) {
  int n = bl[0]->d.n_var;
  double acc[9] = {0};
  for (int bi = 0; bi < nb; ++bi) {
    fo_block *b = bl[bi];
    const fest_flow *fl = &b->flow;
    double sc[9];
    sc[0] = 1.;
    sc[1] = fl->density_inf * fl->vel_mag;
    sc[2] = sc[3] = sc[4] = fl->density_inf * fl->vel_mag * fl->vel_mag;
    sc[5] = (0.5 * fl->density_inf * (fl->vel_mag * fl->vel_mag * fl->vel_mag) + ((fl->gm / (fl->gm - 1.)) * fl->pressure_inf));
    sc[6] = fl->density_inf * fl->vel_mag * (b->sc.turbulence == FEST_TURB_SA ? fl->tv_inf : fl->tk_inf);
    sc[7] = fl->density_inf * fl->vel_mag * (b->sc.turbulence == FEST_TURB_KKL ? fl->tkl_inf : fl->tw_inf);
    /* the intermittency's scale: setup_scale (resnorm.f90:128-167) leaves
     * Res_scale(8) unset, so the norm of the eighth residual is taken
     * unscaled */
    sc[8] = 1.0;
    V r = vres(b), F = vflux(b, 0), G = vflux(b, 1), H = vflux(b, 2);
    for (int l = 1; l <= n; ++l) {
      double s = 0.0;
      for (int k = 1; k <= b->d.kmx - 1; ++k)
        for (int j = 1; j <= b->d.jmx - 1; ++j)
          for (int i = 1; i <= b->d.imx - 1; ++i) {
            double v = *at(r, i, j, k, l);
            s += v * v;
          }
      acc[l] += s / (sc[l] * sc[l]);
    }
    double s1 = 0, s2 = 0, s3 = 0, s4 = 0, s5 = 0, s6 = 0;
    for (int k = 1; k <= b->d.kmx - 1; ++k)
      for (int j = 1; j <= b->d.jmx - 1; ++j) { s1 += *at(F, 1, j, k, 1); s2 += *at(F, b->d.imx, j, k, 1); }
    for (int k = 1; k <= b->d.kmx - 1; ++k)
      for (int i = 1; i <= b->d.imx - 1; ++i) { s3 += *at(G, i, 1, k, 1); s4 += *at(G, i, b->d.jmx, k, 1); }
    for (int j = 1; j <= b->d.jmx - 1; ++j)
      for (int i = 1; i <= b->d.imx - 1; ++i) { s5 += *at(H, i, j, 1, 1); s6 += *at(H, i, j, b->d.kmx, 1); }
    acc[0] += (s1 - s2 + s3 - s4 + s5 - s6) / sc[0];
  }
  out[0] = fabs(acc[0]);
  for (int l = 1; l <= n; ++l) out[l] = sqrt(acc[l]);
}
