/* CPU oracle for the curvilinear (topography) part of the elastic time step --
 * TEST INFRASTRUCTURE ONLY.
 *
 * A plain-C restatement of the reference's curvilinear kernels, used by tests/,
 * __graft_entry__.smoke() and bench.py's CPU leg as the checker; the product
 * never links it.  Each function names the reference code it follows.
 *
 * Grid conventions are the reference's: inclusive 1-based bounds with 2 ghost
 * points, i fastest; 3-component fields and the 4-component metric stored
 * component-major (soa=1, the _rev kernels) or point-major (soa=0).
 */
#ifndef _GNU_SOURCE
#define _GNU_SOURCE
#endif
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include "sw4_oracle.h"

typedef struct {
   int ib, ie, jb, je, kb, ke;
   long ni, nij, npts;
   long cs, ps;   /* 3-component field: component / point stride */
   long mcs, mps; /* metric: component / point stride */
} cbox;

static cbox make_cbox(int soa, int ib, int ie, int jb, int je, int kb, int ke)
{
   cbox b;
   b.ib = ib; b.ie = ie; b.jb = jb; b.je = je; b.kb = kb; b.ke = ke;
   b.ni = ie - ib + 1;
   b.nij = b.ni * (je - jb + 1);
   b.npts = b.nij * (ke - kb + 1);
   b.cs = soa ? b.npts : 1;
   b.ps = soa ? 1 : 3;
   b.mcs = soa ? b.npts : 1;
   b.mps = soa ? 1 : 4;
   return b;
}

static inline long P(const cbox* b, int i, int j, int k)
{
   return (i - b->ib) + b->ni * (j - b->jb) + b->nij * (long)(k - b->kb);
}

/* ------------------------------------------------------------------------ */
/* Curvilinear divergence of stress (rhs4sgcurv_rev.C:34 / rhs4sgcurv.C:34). */
/*                                                                          */
/* With metric m1 = sqrt(z_r), m2 = -z_p/m1, m3 = -z_q/m1, m4 = h/m1 and      */
/* J = h^2 z_r (index-space derivatives), the operator is                    */
/*   Lu_c = (sx sy / J) * sum of                                            */
/*     same-axis terms   D_a(C D_a u_d) : 4th-order variable-coefficient    */
/*                       second differences (SBP acof/ghcof rows in r at a  */
/*                       one-sided top);                                    */
/*     cross terms       D_a(C D_b u_d), a != b : 4th-order centred first    */
/*                       differences (SBP bope rows in r at the top).       */
/* The coefficient C of each (equation, axis pair, component) and its scale  */
/* by 1/sx, 1/sy are the reference's; they are tabulated below.              */
/* ------------------------------------------------------------------------ */

typedef struct {
   const cbox* b;
   const double *u, *mu, *la, *met, *jac, *sx, *sy;
} curv_in;

static inline double MU(const curv_in* a, int i, int j, int k) { return a->mu[P(a->b, i, j, k)]; }
static inline double LA(const curv_in* a, int i, int j, int k) { return a->la[P(a->b, i, j, k)]; }
static inline double MET(const curv_in* a, int c, int i, int j, int k)
{
   return a->met[c * a->b->mcs + a->b->mps * P(a->b, i, j, k)];
}
static inline double UU(const curv_in* a, int c, int i, int j, int k)
{
   return a->u[c * a->b->cs + a->b->ps * P(a->b, i, j, k)];
}
static inline double SX(const curv_in* a, int i) { return a->sx[i - a->b->ib]; }
static inline double SY(const curv_in* a, int j) { return a->sy[j - a->b->jb]; }

/* Coefficient kinds at a point (i,j,k); sx, sy taken at that point's i, j. */
enum {
   K_2ML_11_SX, /* (2mu+la) m1^2 sx */
   K_MU_11_SX,  /* mu m1^2 sx */
   K_MU_11_SY,  /* mu m1^2 sy */
   K_2ML_11_SY, /* (2mu+la) m1^2 sy */
   K_MU_11,     /* mu m1^2 */
   K_LA_11,     /* la m1^2 */
   K_2ML_21_SX, /* (2mu+la) m2 m1 sx */
   K_MU_31,     /* mu m3 m1 */
   K_MU_41,     /* mu m4 m1 */
   K_LA_31_SY,  /* la m3 m1 sy */
   K_LA_41,     /* la m4 m1 */
   K_MU_31_SY,  /* mu m3 m1 sy */
   K_LA_21,     /* la m2 m1 */
   K_MU_21,     /* mu m2 m1 */
   K_LA_31,     /* la m3 m1 */
   K_MU_21_SX,  /* mu m2 m1 sx */
   K_2ML_31_SY, /* (2mu+la) m3 m1 sy */
};

static double coef(const curv_in* a, int kind, int i, int j, int k)
{
   const double mu = MU(a, i, j, k), la = LA(a, i, j, k);
   const double m1 = MET(a, 0, i, j, k);
   switch (kind) {
      case K_2ML_11_SX: return (2 * mu + la) * m1 * m1 * SX(a, i);
      case K_MU_11_SX: return mu * m1 * m1 * SX(a, i);
      case K_MU_11_SY: return mu * m1 * m1 * SY(a, j);
      case K_2ML_11_SY: return (2 * mu + la) * m1 * m1 * SY(a, j);
      case K_MU_11: return mu * m1 * m1;
      case K_LA_11: return la * m1 * m1;
      case K_2ML_21_SX: return (2 * mu + la) * MET(a, 1, i, j, k) * m1 * SX(a, i);
      case K_MU_31: return mu * MET(a, 2, i, j, k) * m1;
      case K_MU_41: return mu * MET(a, 3, i, j, k) * m1;
      case K_LA_31_SY: return la * MET(a, 2, i, j, k) * m1 * SY(a, j);
      case K_LA_41: return la * MET(a, 3, i, j, k) * m1;
      case K_MU_31_SY: return mu * MET(a, 2, i, j, k) * m1 * SY(a, j);
      case K_LA_21: return la * MET(a, 1, i, j, k) * m1;
      case K_MU_21: return mu * MET(a, 1, i, j, k) * m1;
      case K_LA_31: return la * MET(a, 2, i, j, k) * m1;
      case K_MU_21_SX: return mu * MET(a, 1, i, j, k) * m1 * SX(a, i);
      case K_2ML_31_SY: return (2 * mu + la) * MET(a, 2, i, j, k) * m1 * SY(a, j);
   }
   return 0;
}

/* The r-r coefficient matrix A_cd at (i,j,k), with the stretching of the
 * column (sxc, syc). */
static double rr_coef(const curv_in* a, int c, int d, int i, int j, int k, double sxc, double syc)
{
   const double mu = MU(a, i, j, k), la = LA(a, i, j, k);
   const double m2 = MET(a, 1, i, j, k) * sxc, m3 = MET(a, 2, i, j, k) * syc, m4 = MET(a, 3, i, j, k);
   if (c > d) { const int t = c; c = d; d = t; }
   if (c == d) {
      const double m[3] = {m2, m3, m4};
      double o = 0;
      for (int q = 0; q < 3; q++)
         if (q != c) o += m[q] * m[q];
      return (2 * mu + la) * m[c] * m[c] + mu * o;
   }
   const double mm[3] = {MET(a, 1, i, j, k), MET(a, 2, i, j, k), MET(a, 3, i, j, k)};
   return (mu + la) * mm[c] * mm[d];
}

/* A cross-term entry: coefficient kind, inner component, scale (0: 1, 1: 1/sx,
 * 2: 1/sy) */
typedef struct { int kind, comp, scale; } xent;
typedef struct { int n; xent e[3]; } xterm;

/* axis pairs: outer, inner; 0 p (i), 1 q (j), 2 r (k) */
enum { PQ, QP, PR, RP, QR, RQ, NPAIR };
static const int pair_outer[NPAIR] = {1, 0, 2, 0, 2, 1};
static const int pair_inner[NPAIR] = {0, 1, 0, 2, 1, 2};

/* [equation][pair] */
static const xterm xtab[3][NPAIR] = {
   { /* u */
      {1, {{K_MU_11, 1, 0}}},
      {1, {{K_LA_11, 1, 0}}},
      {3, {{K_2ML_21_SX, 0, 2}, {K_MU_31, 1, 0}, {K_MU_41, 2, 2}}},
      {3, {{K_2ML_21_SX, 0, 2}, {K_LA_31_SY, 1, 2}, {K_LA_41, 2, 2}}},
      {2, {{K_MU_31_SY, 0, 1}, {K_LA_21, 1, 0}}},
      {2, {{K_MU_31_SY, 0, 1}, {K_MU_21, 1, 0}}},
   },
   { /* v */
      {1, {{K_LA_11, 0, 0}}},
      {1, {{K_MU_11, 0, 0}}},
      {2, {{K_LA_31, 0, 0}, {K_MU_21_SX, 1, 2}}},
      {2, {{K_MU_31, 0, 0}, {K_MU_21_SX, 1, 2}}},
      {3, {{K_MU_21, 0, 0}, {K_2ML_31_SY, 1, 1}, {K_MU_41, 2, 1}}},
      {3, {{K_LA_21, 0, 0}, {K_2ML_31_SY, 1, 1}, {K_LA_41, 2, 1}}},
   },
   { /* w */
      {0, {{0}}},
      {0, {{0}}},
      {2, {{K_LA_41, 0, 2}, {K_MU_21_SX, 2, 2}}},
      {2, {{K_MU_41, 0, 2}, {K_MU_21_SX, 2, 2}}},
      {2, {{K_MU_31_SY, 2, 1}, {K_LA_41, 1, 1}}},
      {2, {{K_MU_31_SY, 2, 1}, {K_MU_41, 1, 1}}},
   },
};

/* same-axis coefficient kinds [equation][axis p, q] */
static const int same_kind[3][2] = {
   {K_2ML_11_SX, K_MU_11_SY}, {K_MU_11_SX, K_2ML_11_SY}, {K_MU_11_SX, K_MU_11_SY}};

static inline void step_axis(int ax, int m, int* i, int* j, int* k)
{
   if (ax == 0) *i += m;
   else if (ax == 1) *j += m;
   else *k += m;
}

/* 4th-order variable-coefficient second difference from the 5 coefficient and
 * field values at offsets -2..2 (the same formula as the Cartesian operator). */
static double d2v(const double c[5], const double f[5])
{
   const double w1 = c[1] - 0.75 * (c[2] + c[0]);
   const double w2 = c[0] + c[3] + 3 * (c[2] + c[1]);
   const double w3 = c[1] + c[4] + 3 * (c[3] + c[2]);
   const double w4 = c[3] - 0.75 * (c[2] + c[4]);
   return (w1 * (f[0] - f[2]) + w2 * (f[1] - f[2]) + w3 * (f[3] - f[2]) + w4 * (f[4] - f[2])) / 6;
}

static const double C1 = 2.0 / 3, C2 = -1.0 / 12;

void sw4o_rhs4sgcurv(int soa, int ib, int ie, int jb, int je, int kb, int ke, const double* u,
                     const double* mu, const double* la, const double* met, const double* jac,
                     double* lu, const int* onesided, const double* strx, const double* stry)
{
   double acof[384], ghcof[6], bope[48], sbop[5];
   sw4o_stencil_coefficients(acof, ghcof, bope, sbop);
   const cbox b = make_cbox(soa, ib, ie, jb, je, kb, ke);
   curv_in A = {&b, u, mu, la, met, jac, strx, stry};
   const curv_in* a = &A;
   const int top = onesided[4] == 1;
   const int k1 = top ? 1 : kb + 2;
#pragma omp parallel for collapse(2)
   for (int k = k1; k <= ke - 2; k++)
      for (int j = jb + 2; j <= je - 2; j++)
         for (int i = ib + 2; i <= ie - 2; i++) {
            const int bnd = top && k <= 6;
            const double sxc = SX(a, i), syc = SY(a, j);
            const double istrx = 1 / sxc, istry = 1 / syc, istrxy = istry * istrx;
            const double scl[3] = {1, istrx, istry};
            double r[3] = {0, 0, 0};
            /* same-axis p and q */
            for (int c = 0; c < 3; c++)
               for (int ax = 0; ax < 2; ax++) {
                  double cf[5], f[5];
                  for (int m = -2; m <= 2; m++) {
                     int ii = i, jj = j, kk = k;
                     step_axis(ax, m, &ii, &jj, &kk);
                     cf[m + 2] = coef(a, same_kind[c][ax], ii, jj, kk);
                     f[m + 2] = UU(a, c, ii, jj, kk);
                  }
                  r[c] += d2v(cf, f) * (ax == 0 ? istry : istrx);
               }
            /* same-axis r: 3x3 coefficient matrix */
            const double rs[3][3] = {{istrxy, 1, istry}, {1, istrxy, istrx}, {istry, istrx, istrxy}};
            for (int c = 0; c < 3; c++)
               for (int d = 0; d < 3; d++) {
                  double s = 0;
                  if (!bnd) {
                     double cf[5], f[5];
                     for (int m = -2; m <= 2; m++) {
                        cf[m + 2] = rr_coef(a, c, d, i, j, k + m, sxc, syc);
                        f[m + 2] = UU(a, d, i, j, k + m);
                     }
                     s = d2v(cf, f);
                  } else {
                     for (int q = 1; q <= 8; q++) {
                        double cq = 0;
                        for (int m = 1; m <= 8; m++)
                           cq += acof[(k - 1) + 6 * (q - 1) + 48 * (m - 1)] *
                                 rr_coef(a, c, d, i, j, m, sxc, syc);
                        s += cq * UU(a, d, i, j, q);
                     }
                     s += ghcof[k - 1] * rr_coef(a, c, d, i, j, 1, sxc, syc) * UU(a, d, i, j, 0);
                  }
                  r[c] += rs[c][d] * s;
               }
            /* cross terms */
            for (int c = 0; c < 3; c++)
               for (int pr = 0; pr < NPAIR; pr++) {
                  const xterm* t = &xtab[c][pr];
                  if (t->n == 0) continue;
                  const int ao = pair_outer[pr], ai = pair_inner[pr];
                  /* G(o) = sum_e coef_e(o) * scale_e * D_inner u_comp(o), at outer offsets */
                  double G[9];
                  const int useb_outer = bnd && ao == 2, useb_inner = bnd && ai == 2;
                  const int nq = useb_outer ? 8 : 5;
                  for (int s = 0; s < nq; s++) {
                     int ii = i, jj = j, kk = k;
                     if (useb_outer) kk = s + 1;
                     else step_axis(ao, s - 2, &ii, &jj, &kk);
                     double g = 0;
                     for (int e = 0; e < t->n; e++) {
                        const xent* x = &t->e[e];
                        double du;
                        if (useb_inner) {
                           du = 0;
                           for (int q = 1; q <= 8; q++) du += bope[(k - 1) + 6 * (q - 1)] * UU(a, x->comp, ii, jj, q);
                        } else {
                           double f[5];
                           for (int m = -2; m <= 2; m++) {
                              int i2 = ii, j2 = jj, k2 = kk;
                              step_axis(ai, m, &i2, &j2, &k2);
                              f[m + 2] = UU(a, x->comp, i2, j2, k2);
                           }
                           du = C2 * (f[4] - f[0]) + C1 * (f[3] - f[1]);
                        }
                        g += coef(a, x->kind, ii, jj, kk) * scl[x->scale] * du;
                     }
                     G[s] = g;
                  }
                  double d;
                  if (useb_outer) {
                     d = 0;
                     for (int q = 1; q <= 8; q++) d += bope[(k - 1) + 6 * (q - 1)] * G[q - 1];
                  } else {
                     d = C2 * (G[4] - G[0]) + C1 * (G[3] - G[1]);
                  }
                  r[c] += d;
               }
            const double ijac = sxc * syc / a->jac[P(&b, i, j, k)];
            for (int c = 0; c < 3; c++) lu[c * b.cs + b.ps * P(&b, i, j, k)] = r[c] * ijac;
         }
}

/* ------------------------------------------------------------------------ */
/* Metric from the grid's z (EW::metric_rev, curvilinear-c.C:175): index-space */
/* derivatives z_p, z_q, z_r by the 4th-order centred difference, with        */
/* 6-point one-sided 4th-order differences on the two outermost points of     */
/* each line; J = h^2 z_r, met = (sqrt(z_r), -z_p/sqrt(z_r), -z_q/sqrt(z_r),   */
/* h/sqrt(z_r)).  Returns -1 if z_r <= 0 anywhere (the grid folds over).      */
/* ------------------------------------------------------------------------ */

/* derivative along a line of n >= 6 values at position q (0-based) */
static double line_diff(const double* f, long st, int q, int n)
{
#define F(m) f[(long)(q + (m)) * st]
   if (q >= 2 && q <= n - 3) return C2 * (F(2) - F(-2)) + C1 * (F(1) - F(-1));
   if (q == 0)
      return -2.25 * F(0) + (4 + 5.0 / 6) * F(1) - 14.0 / 3 * F(2) + 3 * F(3) - (1 + 1.0 / 12) * F(4) +
             F(5) / 6;
   if (q == 1)
      return -F(-1) / 6 - 1.25 * F(0) + (1 + 4.0 / 3) * F(1) - 4.0 / 3 * F(2) + 0.5 * F(3) - F(4) / 12;
   if (q == n - 2)
      return F(1) / 6 + 1.25 * F(0) - (1 + 4.0 / 3) * F(-1) + 4.0 / 3 * F(-2) - 0.5 * F(-3) + F(-4) / 12;
   return 2.25 * F(0) - (4 + 5.0 / 6) * F(-1) + 14.0 / 3 * F(-2) - 3 * F(-3) + (1 + 1.0 / 12) * F(-4) -
          F(-5) / 6;
#undef F
}

int sw4o_metric(int soa, int ib, int ie, int jb, int je, int kb, int ke, double h, const double* z,
                double* met, double* jac)
{
   const cbox b = make_cbox(soa, ib, ie, jb, je, kb, ke);
   const int ni = ie - ib + 1, nj = je - jb + 1, nk = ke - kb + 1;
   int bad = 0;
#pragma omp parallel for collapse(2) reduction(| : bad)
   for (int k = kb; k <= ke; k++)
      for (int j = jb; j <= je; j++)
         for (int i = ib; i <= ie; i++) {
            const long p = P(&b, i, j, k);
            const double zr = line_diff(z + (p - (long)(k - kb) * b.nij), b.nij, k - kb, nk);
            const double zq = line_diff(z + (p - (long)(j - jb) * b.ni), b.ni, j - jb, nj);
            const double zp = line_diff(z + (p - (i - ib)), 1, i - ib, ni);
            if (!(zr > 0)) {
               bad = 1;
               continue;
            }
            const double s = sqrt(zr);
            jac[p] = h * h * zr;
            met[0 * b.mcs + b.mps * p] = s;
            met[1 * b.mcs + b.mps * p] = -zp / s;
            met[2 * b.mcs + b.mps * p] = -zq / s;
            met[3 * b.mcs + b.mps * p] = h / s;
         }
   return bad ? -1 : 0;
}

/* ------------------------------------------------------------------------ */
/* Curvilinear grid over a Gaussian hill (EW::grid_mapping, EW.C:5694;         */
/* interpolate_topography's analytic branch, EW.C:5619-5627): x = (i-1)h,     */
/* y = (j-1)h, surface z_s = -A exp(-((x-xc)/lx)^2 - ((y-yc)/ly)^2), and      */
/*   z(k) = zmax - (nz-k)h - (1-sa)^order (zmax - (nz-1)h - z_s),  sa < 1     */
/*   z(k) = zmax - (nz-k)h,                                        sa >= 1    */
/* with sa = (k-1)/(zeta_break (nz-1)).                                       */
/* ------------------------------------------------------------------------ */
void sw4o_gaussian_hill_z(int ib, int ie, int jb, int je, int kb, int ke, int nz, double h,
                          double zmax, double zeta_break, int order, double amp, double xc,
                          double yc, double lx, double ly, double* z)
{
   const long ni = ie - ib + 1, nij = ni * (je - jb + 1);
   const double izb = 1.0 / (zeta_break * (nz - 1));
   for (int k = kb; k <= ke; k++)
      for (int j = jb; j <= je; j++)
         for (int i = ib; i <= ie; i++) {
            const double x = (i - 1.0) * h, y = (j - 1.0) * h;
            const double zs = -amp * exp(-(x - xc) * (x - xc) / (lx * lx) - (y - yc) * (y - yc) / (ly * ly));
            const double sa = (k - 1) * izb;
            double om = 1 - sa;
            for (int l = 2; l <= order; l++) om *= (1 - sa);
            double zz = zmax - (nz - k) * h;
            if (sa < 1) zz -= om * (zmax - (nz - 1) * h - zs);
            z[(i - ib) + ni * (j - jb) + nij * (k - kb)] = zz;
         }
}

/* ------------------------------------------------------------------------ */
/* Free-surface ghost plane of a curvilinear grid (EW::freesurfcurvisg_rev,   */
/* curvilinear-c.C:621): at k = 1 (side 5) or k = nz (side 6) the traction     */
/* condition sum_q sbop[q] u(k -/+ 1 + q) + normal-derivative coupling =      */
/* forcing is solved for the ghost value, for i, j in [b+2, e-2].             */
/* The tangential part of the traction is the operator's pr + qr flux at k.   */
/* forcing: 3 x ni x nj, point-major (may be NULL for zero forcing).          */
/* ------------------------------------------------------------------------ */
void sw4o_freesurfcurvisg(int soa, int ib, int ie, int jb, int je, int kb, int ke, int nz, int side,
                          double* u, const double* mu, const double* la, const double* met,
                          const double* sbop, const double* forcing, const double* strx,
                          const double* stry)
{
   const cbox b = make_cbox(soa, ib, ie, jb, je, kb, ke);
   curv_in A = {&b, u, mu, la, met, NULL, strx, stry};
   const curv_in* a = &A;
   const int k = side == 5 ? 1 : nz, kl = side == 5 ? 1 : -1;
   const double s0i = 1 / sbop[0];
#pragma omp parallel for
   for (int j = jb + 2; j <= je - 2; j++)
      for (int i = ib + 2; i <= ie - 2; i++) {
         const double istrx = 1 / SX(a, i), istry = 1 / SY(a, j);
         const double scl[3] = {1, istrx, istry};
         double rhs[3];
         for (int c = 0; c < 3; c++) {
            double g = 0;
            for (int pr = PR; pr <= QR; pr += 2) { /* PR and QR: outer r */
               const xterm* t = &xtab[c][pr];
               const int ai = pair_inner[pr];
               for (int e = 0; e < t->n; e++) {
                  const xent* x = &t->e[e];
                  double f[5];
                  for (int m = -2; m <= 2; m++) {
                     int i2 = i, j2 = j, k2 = k;
                     step_axis(ai, m, &i2, &j2, &k2);
                     f[m + 2] = UU(a, x->comp, i2, j2, k2);
                  }
                  g += coef(a, x->kind, i, j, k) * scl[x->scale] * (C2 * (f[4] - f[0]) + C1 * (f[3] - f[1]));
               }
            }
            const double fo = forcing ? forcing[3 * ((i - ib) + b.ni * (j - jb)) + c] : 0.0;
            rhs[c] = g - fo;
         }
         const double m2 = MET(a, 1, i, j, k), m3 = MET(a, 2, i, j, k), m4 = MET(a, 3, i, j, k);
         const double sx = SX(a, i), sy = SY(a, j), mu0 = MU(a, i, j, k), la0 = LA(a, i, j, k);
         const double ac = sx * istry * m2 * m2 + sy * istrx * m3 * m3 + m4 * m4 * istry * istrx;
         const double bc = 1 / (mu0 * ac);
         const double cc = (mu0 + la0) / (2 * mu0 + la0) * bc / ac;
         const double xoy = sqrt(sx * istry), yox = 1 / xoy, ixy = istrx * xoy;
         const double dc = cc * (xoy * m2 * rhs[0] + yox * m3 * rhs[1] + ixy * m4 * rhs[2]);
         const double nrm[3] = {m2 * xoy, m3 * yox, m4 * ixy};
         for (int c = 0; c < 3; c++) {
            double s = 0;
            for (int q = 1; q <= 4; q++) s += sbop[q] * UU(a, c, i, j, k + (q - 1) * kl);
            u[c * b.cs + b.ps * P(&b, i, j, k - kl)] = -s0i * (s + bc * rhs[c] - dc * nrm[c]);
         }
      }
}

/* ------------------------------------------------------------------------ */
/* Supergrid damping on a curvilinear grid (EW::addsgd4cfort_indrev,          */
/* ew-cfromfort.C:1323): x and y only, each 4th difference weighted by         */
/* rho*dc*J and the whole by beta/(rho J).                                    */
/* ------------------------------------------------------------------------ */
void sw4o_addsgd4c(int soa, int ib, int ie, int jb, int je, int kb, int ke, double* up,
                   const double* u, const double* um, const double* rho, const double* dcx,
                   const double* dcy, const double* strx, const double* stry, const double* jac,
                   const double* cox, const double* coy, double beta)
{
   if (beta == 0) return;
   const cbox b = make_cbox(soa, ib, ie, jb, je, kb, ke);
#pragma omp parallel for collapse(2)
   for (int k = kb + 2; k <= ke - 2; k++)
      for (int j = jb + 2; j <= je - 2; j++)
         for (int i = ib + 2; i <= ie - 2; i++) {
            const long p = P(&b, i, j, k);
            const double irhoj = beta / (rho[p] * jac[p]);
            for (int c = 0; c < 3; c++) {
               const long o = c * b.cs;
               double acc = 0;
               for (int ax = 0; ax < 2; ax++) {
                  const long st = ax == 0 ? 1 : b.ni;
                  const double* dc = ax == 0 ? dcx : dcy;
                  const int q = ax == 0 ? i - ib : j - jb;
                  const double w = ax == 0 ? strx[i - ib] * coy[j - jb] : stry[j - jb] * cox[i - ib];
                  double s = 0;
                  for (int m = -1; m <= 1; m++) {
                     const long pm = p + m * st;
                     const double e = rho[pm] * dc[q + m] * jac[pm];
                     const double du = u[o + b.ps * (pm + st)] - 2 * u[o + b.ps * pm] + u[o + b.ps * (pm - st)];
                     const double dm = um[o + b.ps * (pm + st)] - 2 * um[o + b.ps * pm] + um[o + b.ps * (pm - st)];
                     s += (m == 0 ? -2 : 1) * e * (du - dm);
                  }
                  acc += w * s;
               }
               up[o + b.ps * p] -= irhoj * acc;
            }
         }
}

/* ------------------------------------------------------------------------ */
/* Sixth-order supergrid damping on a curvilinear grid (EW::addsgd6cfort and  */
/* _indrev, ew-cfromfort.C:1241-1322, :1405): x and y only; along each axis    */
/* the sum over the four half points of +-(1, 3) x (e_a + e_b) x the third     */
/* difference of u - um across them, e = rho dc J; the whole times             */
/* beta / (2 rho J), over the points 3 away from every array edge.             */
/* ------------------------------------------------------------------------ */
void sw4o_addsgd6c(int soa, int ib, int ie, int jb, int je, int kb, int ke, double* up,
                   const double* u, const double* um, const double* rho, const double* dcx,
                   const double* dcy, const double* strx, const double* stry, const double* jac,
                   const double* cox, const double* coy, double beta)
{
   if (beta == 0) return;
   const cbox b = make_cbox(soa, ib, ie, jb, je, kb, ke);
   /* half point m + 1/2 for m = -2..1: sign and weight, and the offsets of the third
      difference (u(m+2) - 3u(m+1) + 3u(m) - u(m-1)) */
   static const double wgt[4] = {-1, 3, -3, 1};
#pragma omp parallel for collapse(2)
   for (int k = kb + 3; k <= ke - 3; k++)
      for (int j = jb + 3; j <= je - 3; j++)
         for (int i = ib + 3; i <= ie - 3; i++) {
            const long p = P(&b, i, j, k);
            const double birhoj = 0.5 * beta / (rho[p] * jac[p]);
            for (int c = 0; c < 3; c++) {
               const long o = c * b.cs;
               double acc = 0;
               for (int ax = 0; ax < 2; ax++) {
                  const long st = ax == 0 ? 1 : b.ni;
                  const double* dc = ax == 0 ? dcx : dcy;
                  const int q = ax == 0 ? i - ib : j - jb;
                  const double w = ax == 0 ? strx[i - ib] * coy[j - jb] : stry[j - jb] * cox[i - ib];
                  double s = 0;
                  for (int m = -2; m <= 1; m++) {
                     const long pa = p + m * st, pb = p + (m + 1) * st;
                     const double e = rho[pb] * dc[q + m + 1] * jac[pb] + rho[pa] * dc[q + m] * jac[pa];
                     double d3 = 0;
                     for (int t = -1; t <= 2; t++) {
                        static const double c3[4] = {-1, 3, -3, 1};
                        const long pt = o + b.ps * (p + (m + t) * st);
                        d3 += c3[t + 1] * (u[pt] - um[pt]);
                     }
                     s += wgt[m + 2] * e * d3;
                  }
                  acc += w * s;
               }
               up[o + b.ps * p] += birhoj * acc;
            }
         }
}

/* ------------------------------------------------------------------------ */
/* Time step limit of a curvilinear grid (EW::computeDT, EW.C:5066-5125): the  */
/* largest -lambda_min(A)/(4 rho) over the grid, A the symmetric 3x3 matrix    */
/* built from the metric and material; dt = cfl / sqrt(max).  The reference     */
/* calls LAPACK dspev for lambda_min; here it is the closed form for the       */
/* eigenvalues of a symmetric 3x3 matrix by the trigonometric method (O. K.    */
/* Smith, "Eigenvalues of a symmetric 3x3 matrix", Commun. ACM 4(4), 1961).    */
/* ------------------------------------------------------------------------ */
double sw4o_sym3_min_eig(const double a[6])
{
   /* a = [a00, a01, a02, a11, a12, a22] */
   const double a00 = a[0], a01 = a[1], a02 = a[2], a11 = a[3], a12 = a[4], a22 = a[5];
   const double p1 = a01 * a01 + a02 * a02 + a12 * a12;
   const double q = (a00 + a11 + a22) / 3;
   if (p1 == 0) {
      double m = a00 < a11 ? a00 : a11;
      return m < a22 ? m : a22;
   }
   const double p2 = (a00 - q) * (a00 - q) + (a11 - q) * (a11 - q) + (a22 - q) * (a22 - q) + 2 * p1;
   const double p = sqrt(p2 / 6);
   const double b00 = (a00 - q) / p, b11 = (a11 - q) / p, b22 = (a22 - q) / p;
   const double b01 = a01 / p, b02 = a02 / p, b12 = a12 / p;
   double r = 0.5 * (b00 * (b11 * b22 - b12 * b12) - b01 * (b01 * b22 - b12 * b02) +
                     b02 * (b01 * b12 - b11 * b02));
   r = r < -1 ? -1 : (r > 1 ? 1 : r);
   const double phi = acos(r) / 3;
   /* eigenvalues q + 2p cos(phi + 2 pi m / 3); the smallest is m = 1 */
   return q + 2 * p * cos(phi + 2 * M_PI / 3);
}

double sw4o_curv_dt(int soa, int ib, int ie, int jb, int je, int kb, int ke, const double* rho,
                    const double* mu, const double* la, const double* met, const double* jac,
                    double cfl)
{
   const cbox b = make_cbox(soa, ib, ie, jb, je, kb, ke);
   double eigmax = -1;
   for (long p = 0; p < b.npts; p++) {
      const double l = la[p], m = mu[p], l2m = l + 2 * m, ji = 1 / jac[p];
      const double m1 = met[b.mps * p], m2 = met[b.mcs + b.mps * p], m3 = met[2 * b.mcs + b.mps * p],
                   m4 = met[3 * b.mcs + b.mps * p];
      const double A[6] = {
          -4 * (m1 * m1 * l2m + m1 * m1 * m + m2 * m2 * l2m + m3 * m3 * m + m4 * m4 * m) * ji,
          -4 * m2 * m3 * (m + l) * ji,
          -4 * m2 * m4 * (m + l) * ji,
          -4 * (m1 * m1 * m + m1 * m1 * l2m + m2 * m2 * m + m3 * m3 * l2m + m4 * m4 * m) * ji,
          -4 * m3 * m4 * (m + l) * ji,
          -4 * (m1 * m1 * m + m1 * m1 * m + m2 * m2 * m + m3 * m3 * m + m4 * m4 * l2m) * ji};
      const double e = -sw4o_sym3_min_eig(A) / (4 * rho[p]);
      if (e > eigmax) eigmax = e;
   }
   return cfl / sqrt(eigmax);
}


/* ------------------------------------------------------------------------ */
/* Two-grid time step over topography.                                       */
/* ------------------------------------------------------------------------ */
void sw4o_cart_topo(const sw4o_problem* cart, const sw4o_curv* cv, double* ucart, double* ucurv)
{
   const cbox bc = make_cbox(1, cart->ib, cart->ie, cart->jb, cart->je, cart->kb, cart->ke);
   const cbox bv = make_cbox(1, cv->ib, cv->ie, cv->jb, cv->je, cv->kb, cv->ke);
   const int nzc = cv->nz;
   for (int c = 0; c < 3; c++)
      for (int j = cart->jb; j <= cart->je; j++)
         for (int i = cart->ib; i <= cart->ie; i++) {
            for (int q = 0; q < 2; q++)
               ucart[c * bc.cs + P(&bc, i, j, cart->kb + q)] = ucurv[c * bv.cs + P(&bv, i, j, nzc - 2 + q)];
            for (int q = 0; q <= 2; q++)
               ucurv[c * bv.cs + P(&bv, i, j, cv->ke - q)] = ucart[c * bc.cs + P(&bc, i, j, cart->kb + 4 - q)];
         }
}

static void topo_bc(const sw4o_problem* p, const sw4o_curv* cv, const double* sbop, double* up,
                    double* cup)
{
   double* nob[6] = {NULL, NULL, NULL, NULL, NULL, NULL};
   sw4o_bcfortsg(1, p->ib, p->ie, p->jb, p->je, p->kb, p->ke, p->wind, p->nx, p->ny, p->nz, up,
                 p->h, p->bccnd, sbop, p->mu, p->la, nob, p->strx, p->stry);
   sw4o_bcfortsg(1, cv->ib, cv->ie, cv->jb, cv->je, cv->kb, cv->ke, cv->wind, cv->nx, cv->ny, cv->nz,
                 cup, cv->h, cv->bccnd, sbop, cv->mu, cv->la, nob, cv->strx, cv->stry);
   if (cv->bccnd[4] == 0)
      sw4o_freesurfcurvisg(1, cv->ib, cv->ie, cv->jb, cv->je, cv->kb, cv->ke, cv->nz, 5, cup, cv->mu,
                           cv->la, cv->met, sbop, NULL, cv->strx, cv->stry);
   sw4o_cart_topo(p, cv, up, cup);
}

void sw4o_step_topo(const sw4o_problem* p, const sw4o_curv* cv, double t, double* up,
                    const double* u, const double* um, double* lu, double* f, double* uacc,
                    double* cup, const double* cu, const double* cum, double* clu, double* cf,
                    double* cuacc)
{
   double acof[384], ghcof[6], bope[48], sbop[5];
   sw4o_stencil_coefficients(acof, ghcof, bope, sbop);
   const long npts = (long)(p->ie - p->ib + 1) * (p->je - p->jb + 1) * (p->ke - p->kb + 1);
   const long cnpts = (long)(cv->ie - cv->ib + 1) * (cv->je - cv->jb + 1) * (cv->ke - cv->kb + 1);
   const double dt = p->dt;
   const int onesided_c[6] = {0, 0, 0, 0, cv->bccnd[4] == 0, 0};
   sw4o_force(1, cv->ib, cv->ie, cv->jb, cv->je, cv->kb, cv->ke, cf, cv->nsrc, cv->src_ijk,
              cv->src_amp, cv->src_freq, cv->src_t0, cv->src_kind, t, 0);

   sw4o_force(1, p->ib, p->ie, p->jb, p->je, p->kb, p->ke, f, p->nsrc, p->src_ijk, p->src_amp,
              p->src_freq, p->src_t0, p->src_kind, t, 0);
   memset(lu, 0, 3 * npts * sizeof(double));
   memset(clu, 0, 3 * cnpts * sizeof(double));
   sw4o_rhs4sg(1, p->ib, p->ie, p->jb, p->je, p->kb, p->ke, p->nz, p->onesided, acof, bope, ghcof,
               lu, u, p->mu, p->la, p->h, p->strx, p->stry, p->strz);
   sw4o_rhs4sgcurv(1, cv->ib, cv->ie, cv->jb, cv->je, cv->kb, cv->ke, cu, cv->mu, cv->la, cv->met,
                   cv->jac, clu, onesided_c, cv->strx, cv->stry);
   sw4o_predfort(1, p->ib, p->ie, p->jb, p->je, p->kb, p->ke, up, u, um, lu, f, p->rho, dt * dt);
   sw4o_predfort(1, cv->ib, cv->ie, cv->jb, cv->je, cv->kb, cv->ke, cup, cu, cum, clu, cf, cv->rho,
                 dt * dt);
   topo_bc(p, cv, sbop, up, cup);

   sw4o_force(1, p->ib, p->ie, p->jb, p->je, p->kb, p->ke, f, p->nsrc, p->src_ijk, p->src_amp,
              p->src_freq, p->src_t0, p->src_kind, t, 1);
   sw4o_force(1, cv->ib, cv->ie, cv->jb, cv->je, cv->kb, cv->ke, cf, cv->nsrc, cv->src_ijk,
              cv->src_amp, cv->src_freq, cv->src_t0, cv->src_kind, t, 1);
   sw4o_dpdmtfort(p->ib, p->ie, p->jb, p->je, p->kb, p->ke, up, u, um, uacc, 1.0 / (dt * dt));
   sw4o_dpdmtfort(cv->ib, cv->ie, cv->jb, cv->je, cv->kb, cv->ke, cup, cu, cum, cuacc, 1.0 / (dt * dt));
   sw4o_rhs4sg(1, p->ib, p->ie, p->jb, p->je, p->kb, p->ke, p->nz, p->onesided, acof, bope, ghcof,
               lu, uacc, p->mu, p->la, p->h, p->strx, p->stry, p->strz);
   sw4o_rhs4sgcurv(1, cv->ib, cv->ie, cv->jb, cv->je, cv->kb, cv->ke, cuacc, cv->mu, cv->la, cv->met,
                   cv->jac, clu, onesided_c, cv->strx, cv->stry);
   sw4o_corrfort(1, p->ib, p->ie, p->jb, p->je, p->kb, p->ke, up, lu, f, p->rho, dt * dt * dt * dt);
   sw4o_corrfort(1, cv->ib, cv->ie, cv->jb, cv->je, cv->kb, cv->ke, cup, clu, cf, cv->rho,
                 dt * dt * dt * dt);
   if (p->sg_beta != 0) {
      if (p->sg_order == 6) {
         sw4o_addsgd6(1, p->ib, p->ie, p->jb, p->je, p->kb, p->ke, up, u, um, p->rho, p->dcx, p->dcy,
                      p->dcz, p->strx, p->stry, p->strz, p->cox, p->coy, p->coz, p->sg_beta);
         sw4o_addsgd6c(1, cv->ib, cv->ie, cv->jb, cv->je, cv->kb, cv->ke, cup, cu, cum, cv->rho,
                       cv->dcx, cv->dcy, cv->strx, cv->stry, cv->jac, cv->cox, cv->coy, p->sg_beta);
      } else {
         sw4o_addsgd4(1, p->ib, p->ie, p->jb, p->je, p->kb, p->ke, up, u, um, p->rho, p->dcx, p->dcy,
                      p->dcz, p->strx, p->stry, p->strz, p->cox, p->coy, p->coz, p->sg_beta);
         sw4o_addsgd4c(1, cv->ib, cv->ie, cv->jb, cv->je, cv->kb, cv->ke, cup, cu, cum, cv->rho,
                       cv->dcx, cv->dcy, cv->strx, cv->stry, cv->jac, cv->cox, cv->coy, p->sg_beta);
      }
   }
   topo_bc(p, cv, sbop, up, cup);
}
