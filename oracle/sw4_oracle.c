/*
 * CPU oracle for the sw4lite elastic time step -- TEST INFRASTRUCTURE ONLY.
 * See sw4_oracle.h for the contract.  Each function restates the reference
 * algorithm cited beside it; the arithmetic is grouped for readability (stencil
 * weights as small arrays, sums as loops) rather than in the reference's
 * unrolled order, so results agree with the reference to rounding, not bitwise.
 */
#define _GNU_SOURCE
#include "sw4_oracle.h"

#include <math.h>
#include <stddef.h>
#include <stdlib.h>
#include <string.h>

/* ------------------------------------------------------------------------ */
/* SBP coefficients.  The values are the published 4th-order SBP operator of  */
/* Sjogreen & Petersson (J. Sci. Comput. 2012) as tabulated by the reference   */
/* in src/ew-cfromfort.C:1487-1944; they are listed here sparsely as exact     */
/* rationals (row, column, second column, numerator, denominator).            */
/* ------------------------------------------------------------------------ */
typedef struct { int q, k, m; double num, den; } sbp_entry;

static const sbp_entry acof_nz[] = {
   {1,1,1,104,289},{1,1,2,-2476335,2435692},{1,1,3,-16189,84966},{1,1,4,-9,3332},
   {1,2,1,-516,289},{1,2,2,544521,1217846},{1,2,3,2509879,3653538},
   {1,3,1,312,289},{1,3,2,1024279,2435692},{1,3,3,-687797,1217846},{1,3,4,177,3332},
   {1,4,1,-104,289},{1,4,2,181507,1217846},{1,4,3,241309,3653538},
   {1,5,3,5,2193},{1,5,4,-48,833},{1,6,4,6,833},
   {2,1,1,12,17},{2,1,2,544521,4226642},{2,1,3,2509879,12679926},
   {2,2,1,-59,68},{2,2,2,-1633563,4226642},{2,2,3,-21510077,25359852},{2,2,4,-12655,372939},
   {2,3,1,2,17},{2,3,2,1633563,4226642},{2,3,3,2565299,4226642},{2,3,4,40072,372939},
   {2,4,1,3,68},{2,4,2,-544521,4226642},{2,4,3,987685,25359852},{2,4,4,-14762,124313},
   {2,5,3,1630,372939},{2,5,4,18976,372939},{2,6,4,-1,177},
   {3,1,1,-96,731},{3,1,2,1024279,6160868},{3,1,3,-687797,3080434},{3,1,4,177,8428},
   {3,2,1,118,731},{3,2,2,1633563,3080434},{3,2,3,2565299,3080434},{3,2,4,40072,271803},
   {3,3,1,-16,731},{3,3,2,-5380447,6160868},{3,3,3,-3569115,3080434},{3,3,4,-331815,362404},
   {3,3,5,-283,6321},
   {3,4,1,-6,731},{3,4,2,544521,3080434},{3,4,3,2193521,3080434},{3,4,4,8065,12943},
   {3,4,5,381,2107},
   {3,5,3,-14762,90601},{3,5,4,32555,271803},{3,5,5,-283,2107},
   {3,6,4,9,2107},{3,6,5,-11,6321},
   {4,1,1,-36,833},{4,1,2,181507,3510262},{4,1,3,241309,10530786},
   {4,2,1,177,3332},{4,2,2,-544521,3510262},{4,2,3,987685,21061572},{4,2,4,-14762,103243},
   {4,3,1,-6,833},{4,3,2,544521,3510262},{4,3,3,2193521,3510262},{4,3,4,8065,14749},
   {4,3,5,381,2401},
   {4,4,1,-9,3332},{4,4,2,-181507,3510262},{4,4,3,-2647979,3008796},{4,4,4,-80793,103243},
   {4,4,5,-1927,2401},{4,4,6,-2,49},
   {4,5,3,57418,309729},{4,5,4,51269,103243},{4,5,5,1143,2401},{4,5,6,8,49},
   {4,6,4,-283,2401},{4,6,5,403,2401},{4,6,6,-6,49},
   {5,1,3,5,6192},{5,1,4,-1,49},
   {5,2,3,815,151704},{5,2,4,1186,18963},
   {5,3,3,-7381,50568},{5,3,4,32555,303408},{5,3,5,-283,2352},
   {5,4,3,28709,151704},{5,4,4,51269,101136},{5,4,5,381,784},{5,4,6,1,6},
   {5,5,3,-349,7056},{5,5,4,-247951,303408},{5,5,5,-577,784},{5,5,6,-5,6},{5,5,7,-1,24},
   {5,6,4,1135,7056},{5,6,5,1165,2352},{5,6,6,1,2},{5,6,7,1,6},
   {5,7,5,-1,8},{5,7,6,1,6},{5,7,7,-1,8},
   {6,1,4,1,392},{6,2,4,-1,144},{6,3,4,3,784},{6,3,5,-11,7056},
   {6,4,4,-283,2352},{6,4,5,403,2352},{6,4,6,-1,8},
   {6,5,4,1135,7056},{6,5,5,1165,2352},{6,5,6,1,2},{6,5,7,1,6},
   {6,6,4,-47,1176},{6,6,5,-5869,7056},{6,6,6,-3,4},{6,6,7,-5,6},{6,6,8,-1,24},
   {6,7,5,1,6},{6,7,6,1,2},{6,7,7,1,2},{6,7,8,1,6},
   {6,8,6,-1,8},{6,8,7,1,6},{6,8,8,-1,8},
};

static const sbp_entry bope_nz[] = {
   {1,1,0,-24,17},{1,2,0,59,34},{1,3,0,-4,17},{1,4,0,-3,34},
   {2,1,0,-1,2},{2,3,0,1,2},
   {3,1,0,4,43},{3,2,0,-59,86},{3,4,0,59,86},{3,5,0,-4,43},
   {4,1,0,3,98},{4,3,0,-59,98},{4,5,0,32,49},{4,6,0,-4,49},
   {5,3,0,1,12},{5,4,0,-2,3},{5,6,0,2,3},{5,7,0,-1,12},
   {6,4,0,1,12},{6,5,0,-2,3},{6,7,0,2,3},{6,8,0,-1,12},
};

void sw4o_stencil_coefficients(double acof[384], double ghcof[6], double bope[48], double sbop[5])
{
   memset(acof, 0, 384 * sizeof(double));
   memset(bope, 0, 48 * sizeof(double));
   memset(ghcof, 0, 6 * sizeof(double));
   for (size_t n = 0; n < sizeof(acof_nz) / sizeof(acof_nz[0]); n++) {
      const sbp_entry* e = &acof_nz[n];
      acof[(e->q - 1) + 6 * (e->k - 1) + 48 * (e->m - 1)] = e->num / e->den;
   }
   for (size_t n = 0; n < sizeof(bope_nz) / sizeof(bope_nz[0]); n++) {
      const sbp_entry* e = &bope_nz[n];
      bope[(e->q - 1) + 6 * (e->k - 1)] = e->num / e->den;
   }
   ghcof[0] = 12.0 / 17;
   sbop[0] = -1.0 / 4;
   sbop[1] = -5.0 / 6;
   sbop[2] = 3.0 / 2;
   sbop[3] = -1.0 / 2;
   sbop[4] = 1.0 / 12;
}

/* ------------------------------------------------------------------------ */
/* Indexing helpers                                                          */
/* ------------------------------------------------------------------------ */
typedef struct {
   int ib, jb, kb;
   long ni, nij, npts;
   long cs, ps; /* component stride, point stride */
} box;

static box make_box(int soa, int ib, int ie, int jb, int je, int kb, int ke)
{
   box b;
   b.ib = ib;
   b.jb = jb;
   b.kb = kb;
   b.ni = ie - ib + 1;
   b.nij = b.ni * (je - jb + 1);
   b.npts = b.nij * (ke - kb + 1);
   b.cs = soa ? b.npts : 1;
   b.ps = soa ? 1 : 3;
   return b;
}

static inline long PT(const box* b, int i, int j, int k)
{
   return (i - b->ib) + b->ni * (j - b->jb) + b->nij * (k - b->kb);
}
static inline long CX(const box* b, int c, int i, int j, int k)
{
   return c * b->cs + b->ps * PT(b, i, j, k);
}

/* 4th-order variable-coefficient second difference (a f_x)_x on 5 points,
 * times 6: weights built from a[-2..2] as in src/rhs4sg_rev.C:114-136. */
static inline double d2var(const double a[5], const double f[5])
{
   const double tf = 0.75;
   double wm2 = a[1] - tf * (a[2] + a[0]);
   double wm1 = a[0] + a[3] + 3 * (a[2] + a[1]);
   double wp1 = a[1] + a[4] + 3 * (a[3] + a[2]);
   double wp2 = a[3] - tf * (a[2] + a[4]);
   return wm2 * (f[0] - f[2]) + wm1 * (f[1] - f[2]) + wp1 * (f[3] - f[2]) + wp2 * (f[4] - f[2]);
}

/* 12h * centred 4th-order first difference. */
static const double DW[5] = {1, -8, 0, 8, -1};

/* Strided forms used by the centred rows: `mst` is the point stride of the
 * material arrays along the axis, `fst` the stride of the field. */
static inline double d2v_axis(const double* mu, const double* la, long mst, const double* sa,
                              const double* f, long fst, int twomu)
{
   double a[5], ff[5];
   for (int m = -2; m <= 2; m++) {
      const double c = twomu ? 2 * mu[m * mst] + la[m * mst] : mu[m * mst];
      a[m + 2] = c * sa[m];
      ff[m + 2] = f[m * fst];
   }
   return d2var(a, ff);
}

/* sum_m DW[m] coef(m along outer) * (12h d/d inner of f at that point) */
static inline double mixed_axis(const double* coef, long cst, const double* f, long fo, long fi)
{
   double s = 0;
   for (int m = -2; m <= 2; m++) {
      if (m == 0) continue;
      const double* g = f + m * fo;
      const double inner = (g[-2 * fi] - g[2 * fi]) + 8 * (g[fi] - g[-fi]);
      s += DW[m + 2] * coef[m * cst] * inner;
   }
   return s;
}

/* ------------------------------------------------------------------------ */
/* rhs4sg: src/rhs4sg_rev.C:44-864 (SoA) and src/rhs4sg.C:38-849 (AoS).      */
/* ------------------------------------------------------------------------ */
typedef struct {
   const box* b;
   const double *u, *mu, *la, *sx, *sy, *sz;
   int ifirst, jfirst, kfirst;
} opctx;

/* u component c at (i,j,k) offset by m along axis ax (0,1,2) */
static inline double uat(const opctx* o, int c, int i, int j, int k)
{
   return o->u[CX(o->b, c, i, j, k)];
}
static inline double coefat(const double* a, const opctx* o, int i, int j, int k)
{
   return a[PT(o->b, i, j, k)];
}

/* Sum over the outer axis `ao` of DW * coef * (12h d/d(ai) of component c):
 * the mixed term (coef * f_ai)_ao times 144 h^2 (src/rhs4sg_rev.C:221-347). */
static double mixed(const opctx* o, const double* coef, int ao, int ai, int c, int i, int j, int k)
{
   double s = 0;
   for (int m = -2; m <= 2; m++) {
      if (m == 0) continue;
      int io = i + (ao == 0) * m, jo = j + (ao == 1) * m, ko = k + (ao == 2) * m;
      double inner = 0;
      for (int n = -2; n <= 2; n++) {
         if (n == 0) continue;
         inner += DW[n + 2] * uat(o, c, io + (ai == 0) * n, jo + (ai == 1) * n, ko + (ai == 2) * n);
      }
      s += DW[m + 2] * coefat(coef, o, io, jo, ko) * inner;
   }
   return s;
}

/* Second-derivative part along axis ax for component c, coefficient either
 * mu (twomu=0) or 2mu+lambda (twomu=1), stretched by the axis profile. */
static double secder(const opctx* o, int ax, int twomu, int c, int i, int j, int k)
{
   double a[5], f[5];
   for (int m = -2; m <= 2; m++) {
      int ii = i + (ax == 0) * m, jj = j + (ax == 1) * m, kk = k + (ax == 2) * m;
      long p = PT(o->b, ii, jj, kk);
      double s = ax == 0 ? o->sx[ii - o->ifirst] : ax == 1 ? o->sy[jj - o->jfirst]
                                                            : o->sz[kk - o->kfirst];
      double coef = twomu ? 2 * o->mu[p] + o->la[p] : o->mu[p];
      a[m + 2] = coef * s;
      f[m + 2] = uat(o, c, ii, jj, kk);
   }
   return d2var(a, f);
}

typedef struct {
   /* z-direction one-sided operators for a boundary row:
    *   second derivative  sum_q (sum_m acof[q][m] * coef(km[m])) u(kq[q]) + gh * coef(kbnd) u(kgh)
    *   first derivative   sum_q wz[q] f(kq[q])                                   */
   int kq[8], km[8];
   double ac[8][8], wz[8], gh;
   int kbnd, kgh;
} zrow;

static void make_zrow(zrow* z, int k, int nk, const double* acof, const double* bope,
                      const double* ghcof)
{
   int top = k <= 6;
   int kk = top ? k : nk - k + 1; /* row index into the SBP tables */
   for (int q = 1; q <= 8; q++) {
      z->kq[q - 1] = top ? q : nk - q + 1;
      z->km[q - 1] = top ? q : nk - q + 1;
      double bo = bope[(kk - 1) + 6 * (q - 1)];
      z->wz[q - 1] = top ? bo : -bo;
      for (int m = 1; m <= 8; m++)
         z->ac[q - 1][m - 1] = acof[(kk - 1) + 6 * (q - 1) + 48 * (m - 1)];
   }
   z->gh = ghcof[kk - 1];
   z->kbnd = top ? 1 : nk;
   z->kgh = top ? 0 : nk + 1;
}

static double zz_row(const opctx* o, const zrow* z, int twomu, int c, int i, int j)
{
   double coefm[8];
   for (int m = 0; m < 8; m++) {
      long p = PT(o->b, i, j, z->km[m]);
      coefm[m] = twomu ? 2 * o->mu[p] + o->la[p] : o->mu[p];
   }
   double s = 0;
   for (int q = 0; q < 8; q++) {
      double cq = 0;
      for (int m = 0; m < 8; m++) cq += z->ac[q][m] * coefm[m];
      s += cq * uat(o, c, i, j, z->kq[q]);
   }
   long pb = PT(o->b, i, j, z->kbnd);
   double cb = twomu ? 2 * o->mu[pb] + o->la[pb] : o->mu[pb];
   return s + z->gh * cb * uat(o, c, i, j, z->kgh);
}

/* (coef * f_z)_a with the outer difference along a (0 or 1), f_z one-sided:
 * i12 * sum_m DW[m] coef(i+m) * Dz f(i+m)   (src/rhs4sg_rev.C:496-505). */
static double outer_of_dz(const opctx* o, const zrow* z, const double* coef, int a, int c, int i,
                          int j, int k)
{
   double s = 0;
   for (int m = -2; m <= 2; m++) {
      if (m == 0) continue;
      int ii = i + (a == 0) * m, jj = j + (a == 1) * m;
      double dz = 0;
      for (int q = 0; q < 8; q++) dz += z->wz[q] * uat(o, c, ii, jj, z->kq[q]);
      s += DW[m + 2] * coefat(coef, o, ii, jj, k) * dz;
   }
   return s / 12.0;
}

/* Dz( coef * f_a ) one-sided in z, centred along a (src/rhs4sg_rev.C:507-512). */
static double dz_of_inner(const opctx* o, const zrow* z, const double* coef, int a, int c, int i,
                          int j)
{
   double s = 0;
   for (int q = 0; q < 8; q++) {
      int kq = z->kq[q];
      double inner = 0;
      for (int n = -2; n <= 2; n++) {
         if (n == 0) continue;
         inner += DW[n + 2] * uat(o, c, i + (a == 0) * n, j + (a == 1) * n, kq);
      }
      s += z->wz[q] * coefat(coef, o, i, j, kq) * inner / 12.0;
   }
   return s;
}

void sw4o_rhs4sg(int soa, int ifirst, int ilast, int jfirst, int jlast, int kfirst, int klast,
                 int nk, const int onesided[6], const double* acof, const double* bope,
                 const double* ghcof, double* lu, const double* u, const double* mu,
                 const double* la, double h, const double* strx, const double* stry,
                 const double* strz)
{
   box b = make_box(soa, ifirst, ilast, jfirst, jlast, kfirst, klast);
   opctx o = {&b, u, mu, la, strx, stry, strz, ifirst, jfirst, kfirst};
   const double i6 = 1.0 / 6, i144 = 1.0 / 144, cof = 1.0 / (h * h);
   int k1 = onesided[4] == 1 ? 7 : kfirst + 2;
   int k2 = onesided[5] == 1 ? nk - 6 : klast - 2;

   /* Centred rows, src/rhs4sg_rev.C:111-348. */
   const long fx = b.ps, fy = b.ps * b.ni, fz = b.ps * b.nij; /* field strides */
   const long mx = 1, my = b.ni, mz = b.nij;                  /* material strides */
#pragma omp parallel for collapse(2) schedule(static)
   for (int k = k1; k <= k2; k++)
      for (int j = jfirst + 2; j <= jlast - 2; j++)
         for (int i = ifirst + 2; i <= ilast - 2; i++) {
            const long p = PT(&b, i, j, k);
            const double* sxp = strx + (i - ifirst);
            const double* syp = stry + (j - jfirst);
            const double* szp = strz + (k - kfirst);
            const double sx = *sxp, sy = *syp, sz = *szp;
            const double* m0 = mu + p;
            const double* l0 = la + p;
            const double* U0 = u + b.ps * p;            /* component 0 */
            const double* U1 = U0 + b.cs;
            const double* U2 = U0 + 2 * b.cs;
            double r[3];
            r[0] = i6 * (sx * d2v_axis(m0, l0, mx, sxp, U0, fx, 1) +
                         sy * d2v_axis(m0, l0, my, syp, U0, fy, 0) +
                         sz * d2v_axis(m0, l0, mz, szp, U0, fz, 0));
            r[1] = i6 * (sx * d2v_axis(m0, l0, mx, sxp, U1, fx, 0) +
                         sy * d2v_axis(m0, l0, my, syp, U1, fy, 1) +
                         sz * d2v_axis(m0, l0, mz, szp, U1, fz, 0));
            r[2] = i6 * (sx * d2v_axis(m0, l0, mx, sxp, U2, fx, 0) +
                         sy * d2v_axis(m0, l0, my, syp, U2, fy, 0) +
                         sz * d2v_axis(m0, l0, mz, szp, U2, fz, 1));
            r[0] += i144 * (sx * sy * (mixed_axis(l0, mx, U1, fx, fy) + mixed_axis(m0, my, U1, fy, fx)) +
                            sx * sz * (mixed_axis(l0, mx, U2, fx, fz) + mixed_axis(m0, mz, U2, fz, fx)));
            r[1] += i144 * (sx * sy * (mixed_axis(m0, mx, U0, fx, fy) + mixed_axis(l0, my, U0, fy, fx)) +
                            sy * sz * (mixed_axis(l0, my, U2, fy, fz) + mixed_axis(m0, mz, U2, fz, fy)));
            r[2] += i144 * (sx * sz * (mixed_axis(m0, mx, U0, fx, fz) + mixed_axis(l0, mz, U0, fz, fx)) +
                            sy * sz * (mixed_axis(m0, my, U1, fy, fz) + mixed_axis(l0, mz, U1, fz, fy)));
            for (int c = 0; c < 3; c++) lu[c * b.cs + b.ps * p] = cof * r[c];
         }

   /* One-sided SBP rows at the top (k=1..6, src/rhs4sg_rev.C:349-600) and the
    * bottom (k=nk-5..nk, src/rhs4sg_rev.C:602-856).  The z-stretching strz is
    * not applied on these rows, as in the reference. */
   for (int side = 0; side < 2; side++) {
      if (onesided[4 + side] != 1) continue;
      int kr0 = side == 0 ? 1 : nk - 5, kr1 = side == 0 ? 6 : nk;
#pragma omp parallel for collapse(2) schedule(static)
      for (int k = kr0; k <= kr1; k++)
         for (int j = jfirst + 2; j <= jlast - 2; j++) {
            zrow z;
            make_zrow(&z, k, nk, acof, bope, ghcof);
            for (int i = ifirst + 2; i <= ilast - 2; i++) {
               double sx = strx[i - ifirst], sy = stry[j - jfirst];
               double r[3];
               r[0] = i6 * (sx * secder(&o, 0, 1, 0, i, j, k) + sy * secder(&o, 1, 0, 0, i, j, k)) +
                      zz_row(&o, &z, 0, 0, i, j);
               r[1] = i6 * (sx * secder(&o, 0, 0, 1, i, j, k) + sy * secder(&o, 1, 1, 1, i, j, k)) +
                      zz_row(&o, &z, 0, 1, i, j);
               r[2] = i6 * (sx * secder(&o, 0, 0, 2, i, j, k) + sy * secder(&o, 1, 0, 2, i, j, k)) +
                      zz_row(&o, &z, 1, 2, i, j);
               r[0] += sx * sy * i144 * (mixed(&o, la, 0, 1, 1, i, j, k) + mixed(&o, mu, 1, 0, 1, i, j, k));
               r[0] += sx * outer_of_dz(&o, &z, la, 0, 2, i, j, k);
               r[0] += sx * dz_of_inner(&o, &z, mu, 0, 2, i, j);
               r[1] += sx * sy * i144 * (mixed(&o, mu, 0, 1, 0, i, j, k) + mixed(&o, la, 1, 0, 0, i, j, k));
               r[1] += sy * outer_of_dz(&o, &z, la, 1, 2, i, j, k);
               r[1] += sy * dz_of_inner(&o, &z, mu, 1, 2, i, j);
               r[2] += sx * outer_of_dz(&o, &z, mu, 0, 0, i, j, k);
               r[2] += sy * outer_of_dz(&o, &z, mu, 1, 1, i, j, k);
               r[2] += sx * dz_of_inner(&o, &z, la, 0, 0, i, j);
               r[2] += sy * dz_of_inner(&o, &z, la, 1, 1, i, j);
               for (int c = 0; c < 3; c++) lu[CX(&b, c, i, j, k)] = cof * r[c];
            }
         }
   }
}

/* ------------------------------------------------------------------------ */
/* Pointwise updates: src/ew-cfromfort.C:40-142.                             */
/* ------------------------------------------------------------------------ */
void sw4o_predfort(int soa, int ib, int ie, int jb, int je, int kb, int ke, double* up,
                   const double* u, const double* um, const double* lu, const double* fo,
                   const double* rho, double dt2)
{
   box b = make_box(soa, ib, ie, jb, je, kb, ke);
#pragma omp parallel for schedule(static)
   for (long p = 0; p < b.npts; p++) {
      double c0 = dt2 / rho[p];
      for (int c = 0; c < 3; c++) {
         long q = c * b.cs + b.ps * p;
         up[q] = 2 * u[q] - um[q] + c0 * (lu[q] + fo[q]);
      }
   }
}

void sw4o_corrfort(int soa, int ib, int ie, int jb, int je, int kb, int ke, double* up,
                   const double* lu, const double* fo, const double* rho, double dt4)
{
   box b = make_box(soa, ib, ie, jb, je, kb, ke);
   const double dt4i12 = dt4 / 12;
#pragma omp parallel for schedule(static)
   for (long p = 0; p < b.npts; p++) {
      double c0 = dt4i12 / rho[p];
      for (int c = 0; c < 3; c++) {
         long q = c * b.cs + b.ps * p;
         up[q] += c0 * (lu[q] + fo[q]);
      }
   }
}

void sw4o_dpdmtfort(int ib, int ie, int jb, int je, int kb, int ke, const double* up,
                    const double* u, const double* um, double* u2, double dt2i)
{
   long n = 3L * (ie - ib + 1) * (je - jb + 1) * (ke - kb + 1);
#pragma omp parallel for schedule(static)
   for (long q = 0; q < n; q++) u2[q] = dt2i * (up[q] - 2 * u[q] + um[q]);
}

/* ------------------------------------------------------------------------ */
/* Supergrid damping.  addsgd4: src/ew-cfromfort.C:748-850 (AoS) and :952-1057 */
/* (SoA): up -= beta/rho * sum_axes str*co*co * D+D-( rho*dc * D+D-(u-um) ).   */
/* addsgd6: :852-950, :1059-1158, the 6th-order analogue with a plus sign.    */
/* ------------------------------------------------------------------------ */
void sw4o_addsgd4(int soa, int ifirst, int ilast, int jfirst, int jlast, int kfirst, int klast,
                  double* up, const double* u, const double* um, const double* rho,
                  const double* dcx, const double* dcy, const double* dcz, const double* strx,
                  const double* stry, const double* strz, const double* cox, const double* coy,
                  const double* coz, double beta)
{
   if (beta == 0) return;
   box b = make_box(soa, ifirst, ilast, jfirst, jlast, kfirst, klast);
   const long fst[3] = {b.ps, b.ps * b.ni, b.ps * b.nij}, mst[3] = {1, b.ni, b.nij};
#pragma omp parallel for collapse(2) schedule(static)
   for (int k = kfirst + 2; k <= klast - 2; k++)
      for (int j = jfirst + 2; j <= jlast - 2; j++)
         for (int i = ifirst + 2; i <= ilast - 2; i++) {
            const long p = PT(&b, i, j, k);
            const double birho = beta / rho[p];
            const double w[3] = {strx[i - ifirst] * coy[j - jfirst] * coz[k - kfirst],
                                 stry[j - jfirst] * cox[i - ifirst] * coz[k - kfirst],
                                 strz[k - kfirst] * cox[i - ifirst] * coy[j - jfirst]};
            const double* dcp[3] = {dcx + (i - ifirst), dcy + (j - jfirst), dcz + (k - kfirst)};
            for (int c = 0; c < 3; c++) {
               const long q = c * b.cs + b.ps * p;
               double tot = 0;
               for (int ax = 0; ax < 3; ax++) {
                  const long f = fst[ax], ms = mst[ax];
                  double d[5];
                  for (int m = -2; m <= 2; m++) d[m + 2] = u[q + m * f] - um[q + m * f];
                  const double e0 = rho[p - ms] * dcp[ax][-1], e1 = rho[p] * dcp[ax][0],
                               e2 = rho[p + ms] * dcp[ax][1];
                  const double sgx = e2 * (d[4] - 2 * d[3] + d[2]) - 2 * e1 * (d[3] - 2 * d[2] + d[1]) +
                                     e0 * (d[2] - 2 * d[1] + d[0]);
                  tot += w[ax] * sgx;
               }
               up[q] -= birho * tot;
            }
         }
}

void sw4o_addsgd6(int soa, int ifirst, int ilast, int jfirst, int jlast, int kfirst, int klast,
                  double* up, const double* u, const double* um, const double* rho,
                  const double* dcx, const double* dcy, const double* dcz, const double* strx,
                  const double* stry, const double* strz, const double* cox, const double* coy,
                  const double* coz, double beta)
{
   if (beta == 0) return;
   box b = make_box(soa, ifirst, ilast, jfirst, jlast, kfirst, klast);
#pragma omp parallel for collapse(2) schedule(static)
   for (int k = kfirst + 3; k <= klast - 3; k++)
      for (int j = jfirst + 3; j <= jlast - 3; j++)
         for (int i = ifirst + 3; i <= ilast - 3; i++) {
            double birho = 0.5 * beta / rho[PT(&b, i, j, k)];
            double wx = strx[i - ifirst] * coy[j - jfirst] * coz[k - kfirst];
            double wy = stry[j - jfirst] * cox[i - ifirst] * coz[k - kfirst];
            double wz = strz[k - kfirst] * cox[i - ifirst] * coy[j - jfirst];
            for (int c = 0; c < 3; c++) {
               double tot = 0;
               for (int ax = 0; ax < 3; ax++) {
                  int di = ax == 0, dj = ax == 1, dk = ax == 2;
                  const double* dc = ax == 0 ? dcx : ax == 1 ? dcy : dcz;
                  int off = ax == 0 ? i - ifirst : ax == 1 ? j - jfirst : k - kfirst;
                  double d[7], e[5];
                  for (int m = -3; m <= 3; m++) {
                     long q = CX(&b, c, i + di * m, j + dj * m, k + dk * m);
                     d[m + 3] = u[q] - um[q];
                  }
                  for (int m = -2; m <= 2; m++)
                     e[m + 2] = rho[PT(&b, i + di * m, j + dj * m, k + dk * m)] * dc[off + m];
                  /* third differences at half points m+1/2, m = -2..1 */
                  double s = 0;
                  const double w4[4] = {-1, 3, -3, 1};
                  for (int m = -2; m <= 1; m++) {
                     double d3 = d[m + 5] - 3 * d[m + 4] + 3 * d[m + 3] - d[m + 2];
                     s += w4[m + 2] * (e[m + 3] + e[m + 2]) * d3;
                  }
                  tot += (ax == 0 ? wx : ax == 1 ? wy : wz) * s;
               }
               up[CX(&b, c, i, j, k)] += birho * tot;
            }
         }
}

/* ------------------------------------------------------------------------ */
/* Boundary windows: src/EW.C:3347-3444.                                      */
/* ------------------------------------------------------------------------ */
void sw4o_boundary_windows(int ib, int ie, int jb, int je, int kb, int ke, int nx, int ny,
                           int nz, const int bccnd[6], int wind[36], int npts[6])
{
   (void)nx;
   (void)ny;
   (void)nz;
   const int ng = 2;
   for (int s = 0; s < 6; s++) {
      npts[s] = 0;
      for (int q = 0; q < 6; q++) wind[6 * s + q] = (q % 2 == 0) ? 999 : -999;
      int t = bccnd[s];
      if (!(t == 0 || t == 1 || t == 2 || t == 3)) continue;
      int w[6] = {ib, ie, jb, je, kb, ke};
      int nghost = t == 0 ? 1 : ng;
      /* side plane of nghost layers */
      if (s == 0) w[1] = w[0] + nghost - 1;
      else if (s == 1) w[0] = w[1] - (nghost - 1);
      else if (s == 2) w[3] = w[2] + nghost - 1;
      else if (s == 3) w[2] = w[3] - (nghost - 1);
      else if (s == 4) w[5] = w[4] + nghost - 1;
      else w[4] = w[5] - (nghost - 1);
      if (t == 0) {
         /* free surface: the plane just inside the ghost points */
         if (s == 0) { w[0] += ng; w[1] = w[0]; }
         else if (s == 1) { w[0] -= ng; w[1] = w[0]; }
         else if (s == 2) { w[2] += ng; w[3] = w[2]; }
         else if (s == 3) { w[2] -= ng; w[3] = w[2]; }
         else if (s == 4) { w[4] += ng; w[5] = w[4]; }
         else { w[4] -= ng; w[5] = w[4]; }
      }
      for (int q = 0; q < 6; q++) wind[6 * s + q] = w[q];
      npts[s] = (w[5] - w[4] + 1) * (w[3] - w[2] + 1) * (w[1] - w[0] + 1);
   }
}

/* ------------------------------------------------------------------------ */
/* bcfortsg: src/ew-cfromfort.C:205-476 (AoS), :480-746 (SoA).                */
/* ------------------------------------------------------------------------ */
void sw4o_bcfortsg(int soa, int ib, int ie, int jb, int je, int kb, int ke, const int wind[36],
                   int nx, int ny, int nz, double* u, double h, const int bccnd[6],
                   const double sbop[5], const double* mu, const double* la,
                   double* const bforce[6], const double* strx, const double* stry)
{
   box b = make_box(soa, ib, ie, jb, je, kb, ke);
   const double d4a = 2.0 / 3.0, d4b = -1.0 / 12.0;
   for (int s = 0; s < 6; s++) {
      const int* w = wind + 6 * s;
      if (bccnd[s] == 1 || bccnd[s] == 2) {
         /* Dirichlet / supergrid: copy the boundary data into the ghost points */
         long idel = 1 + w[1] - w[0], ijdel = idel * (1 + w[3] - w[2]);
         for (int k = w[4]; k <= w[5]; k++)
            for (int j = w[2]; j <= w[3]; j++)
               for (int i = w[0]; i <= w[1]; i++) {
                  long qq = (k - w[4]) * ijdel + (j - w[2]) * idel + (i - w[0]);
                  for (int c = 0; c < 3; c++)
                     u[CX(&b, c, i, j, k)] = bforce[s] ? bforce[s][3 * qq + c] : 0.0;
               }
      } else if (bccnd[s] == 3) {
         /* periodic: copy from the point one period inside */
         int di = s == 0 ? nx : s == 1 ? -nx : 0;
         int dj = s == 2 ? ny : s == 3 ? -ny : 0;
         int dk = s == 4 ? nz : s == 5 ? -nz : 0;
         for (int k = w[4]; k <= w[5]; k++)
            for (int j = w[2]; j <= w[3]; j++)
               for (int i = w[0]; i <= w[1]; i++)
                  for (int c = 0; c < 3; c++)
                     u[CX(&b, c, i, j, k)] = u[CX(&b, c, i + di, j + dj, k + dk)];
      } else if (bccnd[s] == 0 && (s == 4 || s == 5)) {
         /* free surface: solve for the ghost plane from the traction condition */
         int k = s == 4 ? 1 : nz, kl = s == 4 ? 1 : -1;
         const double* bf = bforce[s];
         for (int j = jb + 2; j <= je - 2; j++)
            for (int i = ib + 2; i <= ie - 2; i++) {
               long qq = (i - ib) + b.ni * (j - jb);
               long p = PT(&b, i, j, k);
               double sx = strx[i - ib], sy = stry[j - jb];
#define UU(c, ii, jj, kk) u[CX(&b, c, ii, jj, kk)]
               double wx = sx * (d4a * (UU(2, i + 1, j, k) - UU(2, i - 1, j, k)) +
                                 d4b * (UU(2, i + 2, j, k) - UU(2, i - 2, j, k)));
               double ux = sx * (d4a * (UU(0, i + 1, j, k) - UU(0, i - 1, j, k)) +
                                 d4b * (UU(0, i + 2, j, k) - UU(0, i - 2, j, k)));
               double wy = sy * (d4a * (UU(2, i, j + 1, k) - UU(2, i, j - 1, k)) +
                                 d4b * (UU(2, i, j + 2, k) - UU(2, i, j - 2, k)));
               double vy = sy * (d4a * (UU(1, i, j + 1, k) - UU(1, i, j - 1, k)) +
                                 d4b * (UU(1, i, j + 2, k) - UU(1, i, j - 2, k)));
               double uz = 0, vz = 0, wz = 0;
               for (int q = 1; q <= 4; q++) {
                  int kq = k + kl * (q - 1);
                  uz += sbop[q] * UU(0, i, j, kq);
                  vz += sbop[q] * UU(1, i, j, kq);
                  wz += sbop[q] * UU(2, i, j, kq);
               }
               double f0 = bf ? bf[3 * qq] : 0, f1 = bf ? bf[3 * qq + 1] : 0,
                      f2 = bf ? bf[3 * qq + 2] : 0;
               UU(0, i, j, k - kl) = (-uz - kl * wx + kl * h * f0 / mu[p]) / sbop[0];
               UU(1, i, j, k - kl) = (-vz - kl * wy + kl * h * f1 / mu[p]) / sbop[0];
               UU(2, i, j, k - kl) =
                   (-wz + (-kl * la[p] * (ux + vy) + kl * h * f2) / (2 * mu[p] + la[p])) / sbop[0];
#undef UU
            }
      }
   }
}

/* ------------------------------------------------------------------------ */
/* Supergrid profiles: src/SuperGrid.C:52-198, assignment src/EW.C:4745-4781. */
/* ------------------------------------------------------------------------ */
static double psi0(double xi)
{
   if (xi <= 0) return 0;
   if (xi >= 1) return 1;
   /* C5 smooth step: 462 x^6 - 1980 x^7 + 3465 x^8 - 3080 x^9 + 1386 x^10 - 252 x^11.
    * Evaluated as monomials in the reference's order: near xi=1 the sum cancels
    * to ~1 and the stretching 1-(1-epsL)psi cancels again, so a different
    * evaluation order changes dc = psi/phi at the 1e-9 level. */
   return xi * xi * xi * xi * xi * xi *
          (462 - 1980 * xi + 3465 * xi * xi - 3080 * xi * xi * xi + 1386 * xi * xi * xi * xi -
           252 * xi * xi * xi * xi * xi);
}

void sw4o_supergrid_profile(int first, int last, double h, double xmin, int left, int right,
                            double x0, double x1, double width, double* dc, double* str,
                            double* corner)
{
   const double epsL = 1e-4, cmin = 0.33;
   double trans = 0.5 * width;
   for (int q = first; q <= last; q++) {
      double x = (q - 1) * h + xmin;
      double psi_aux = 0, psi_damp = 0, lin = 0;
      if (left && x < x0 + width) {
         psi_aux = psi0((x0 + width - x) / width);
         psi_damp = psi0((x0 + width - x) / trans);
         lin = (x0 + width - x) / width;
      } else if (right && x > x1 - width) {
         psi_aux = psi0((x - (x1 - width)) / width);
         psi_damp = psi0((x - (x1 - width)) / trans);
         lin = (x - (x1 - width)) / width;
      }
      double phi = 1 - (1 - epsL) * psi_aux;
      str[q - first] = phi;
      dc[q - first] = psi_damp / phi;
      corner[q - first] = 1.0 - (1.0 - cmin) * lin;
   }
}

/* ------------------------------------------------------------------------ */
/* Time functions and forcing.                                               */
/* ------------------------------------------------------------------------ */
double sw4o_timefunc(int kind, double freq, double t)
{
   if (kind == 0) { /* Gaussian, src/time_functions.C:284-291 (cutoff exponent -700) */
      double f = (t * freq) * (t * freq) / 2;
      return (-f > -700.0) ? freq / sqrt(2 * M_PI) * exp(-f) : 0.0;
   }
   /* C6SmoothBump, src/time_functions.C:1637-1648 */
   double x = t * freq;
   if (x < 0 || x > 1) return 0.0;
   return 51480 * pow(x * (1 - x), 7);
}

double sw4o_timefunc_tt(int kind, double freq, double t)
{
   if (kind == 0) { /* src/time_functions.C:311-318 */
      double f = (t * freq) * (t * freq) / 2;
      return (-f > -700.0) ? freq / sqrt(2 * M_PI) * freq * freq * (2 * f - 1) * exp(-f) : 0.0;
   }
   /* src/time_functions.C:1676-1687 */
   double x = t * freq;
   if (x < 0 || x > 1) return 0.0;
   double y = x * (1 - x);
   return 51480 * freq * freq * 7 * (6 * (1 - 2 * x) * (1 - 2 * x) * pow(y, 5) - 2 * pow(y, 6));
}

void sw4o_force(int soa, int ib, int ie, int jb, int je, int kb, int ke, double* f, int nsrc,
                const int* src_ijk, const double* src_amp, const double* src_freq,
                const double* src_t0, const int* src_kind, double t, int tt)
{
   box b = make_box(soa, ib, ie, jb, je, kb, ke);
   memset(f, 0, 3 * b.npts * sizeof(double));
   /* sequential accumulation in source order, as the reference does per unique point */
   for (int s = 0; s < nsrc; s++) {
      double g = tt ? sw4o_timefunc_tt(src_kind[s], src_freq[s], t - src_t0[s])
                    : sw4o_timefunc(src_kind[s], src_freq[s], t - src_t0[s]);
      for (int c = 0; c < 3; c++)
         f[CX(&b, c, src_ijk[3 * s], src_ijk[3 * s + 1], src_ijk[3 * s + 2])] += src_amp[3 * s + c] * g;
   }
}

/* ------------------------------------------------------------------------ */
/* One step, CPU phase order of src/EW.C:2537-2756 for one Cartesian grid.   */
/* ------------------------------------------------------------------------ */
static void enforce_bc(const sw4o_problem* p, int soa, double* u)
{
   double acof[384], ghcof[6], bope[48], sbop[5];
   sw4o_stencil_coefficients(acof, ghcof, bope, sbop);
   double* bf[6] = {0, 0, 0, 0, 0, 0};
   sw4o_bcfortsg(soa, p->ib, p->ie, p->jb, p->je, p->kb, p->ke, p->wind, p->nx, p->ny, p->nz, u,
                 p->h, p->bccnd, sbop, p->mu, p->la, bf, p->strx, p->stry);
}

void sw4o_step(const sw4o_problem* p, int soa, double t, double* up, const double* u,
               const double* um, double* lu, double* f, double* uacc)
{
   sw4o_step_pred(p, soa, t, up, u, um, lu, f, uacc, NULL);
}

void sw4o_step_pred(const sw4o_problem* p, int soa, double t, double* up, const double* u,
                    const double* um, double* lu, double* f, double* uacc, double* pred)
{
   double acof[384], ghcof[6], bope[48], sbop[5];
   sw4o_stencil_coefficients(acof, ghcof, bope, sbop);
   const long npts = (long)(p->ie - p->ib + 1) * (p->je - p->jb + 1) * (p->ke - p->kb + 1);
   const double dt = p->dt;

   sw4o_force(soa, p->ib, p->ie, p->jb, p->je, p->kb, p->ke, f, p->nsrc, p->src_ijk, p->src_amp,
              p->src_freq, p->src_t0, p->src_kind, t, 0);
   memset(lu, 0, 3 * npts * sizeof(double));
   sw4o_rhs4sg(soa, p->ib, p->ie, p->jb, p->je, p->kb, p->ke, p->nz, p->onesided, acof, bope,
               ghcof, lu, u, p->mu, p->la, p->h, p->strx, p->stry, p->strz);
   sw4o_predfort(soa, p->ib, p->ie, p->jb, p->je, p->kb, p->ke, up, u, um, lu, f, p->rho, dt * dt);
   enforce_bc(p, soa, up);
   if (pred) memcpy(pred, up, 3 * npts * sizeof(double));

   sw4o_force(soa, p->ib, p->ie, p->jb, p->je, p->kb, p->ke, f, p->nsrc, p->src_ijk, p->src_amp,
              p->src_freq, p->src_t0, p->src_kind, t, 1);
   sw4o_dpdmtfort(p->ib, p->ie, p->jb, p->je, p->kb, p->ke, up, u, um, uacc, 1.0 / (dt * dt));
   sw4o_rhs4sg(soa, p->ib, p->ie, p->jb, p->je, p->kb, p->ke, p->nz, p->onesided, acof, bope,
               ghcof, lu, uacc, p->mu, p->la, p->h, p->strx, p->stry, p->strz);
   sw4o_corrfort(soa, p->ib, p->ie, p->jb, p->je, p->kb, p->ke, up, lu, f, p->rho,
                 dt * dt * dt * dt);
   if (p->sg_beta != 0) {
      if (p->sg_order == 6)
         sw4o_addsgd6(soa, p->ib, p->ie, p->jb, p->je, p->kb, p->ke, up, u, um, p->rho, p->dcx,
                      p->dcy, p->dcz, p->strx, p->stry, p->strz, p->cox, p->coy, p->coz,
                      p->sg_beta);
      else
         sw4o_addsgd4(soa, p->ib, p->ie, p->jb, p->je, p->kb, p->ke, up, u, um, p->rho, p->dcx,
                      p->dcy, p->dcz, p->strx, p->stry, p->strz, p->cox, p->coy, p->coz,
                      p->sg_beta);
   }
   enforce_bc(p, soa, up);
}


/* ------------------------------------------------------------------------ */
/* Analytic point-source solution.                                           */
/*                                                                          */
/* Time history g(s) of the source (force X0(t) or moment M_pq(t) = M_pq g(t)),   */
/* its derivative, and I(s) = int_{R/a}^{R/b} tau g(s - tau) dtau, the         */
/* near-field integral.  The whole-space Green's functions are the published  */
/* ones (Aki & Richards, Quantitative Seismology, eq. 4.23 for a force and     */
/* eq. 4.29 for a moment tensor).                                              */
/* ------------------------------------------------------------------------ */

/* bump B(x) on (0,1) and B'(x): C6SmoothBump 51480 x^7 (1-x)^7 and
 * VerySmoothBump 1024 x^5 (1-x)^5 */
static double bump(int kind, double x, int deriv)
{
   if (!(x > 0 && x < 1)) return 0.0;
   const double y = x * (1 - x);
   if (kind == 1) return deriv ? 51480.0 * 7 * pow(y, 6) * (1 - 2 * x) : 51480.0 * pow(y, 7);
   return deriv ? 1024.0 * 5 * pow(y, 4) * (1 - 2 * x) : 1024.0 * pow(y, 5);
}

static double hist(int kind, double freq, double s)
{
   if (kind == 0) return freq / sqrt(2 * M_PI) * exp(-(s * freq) * (s * freq) / 2);
   return bump(kind, freq * s, 0);
}

static double hist_dt(int kind, double freq, double s)
{
   if (kind == 0) return -s * freq * freq * hist(0, freq, s);
   return freq * bump(kind, freq * s, 1);
}

/* Gauss-Legendre nodes and weights on [-1, 1] by Newton iteration on P_n */
#define GL_N 10
static double gl_x[GL_N], gl_w[GL_N];
static int gl_ready = 0;

static void gl_init(void)
{
   if (gl_ready) return;
   for (int i = 0; i < GL_N; i++) {
      double x = cos(M_PI * (i + 0.75) / (GL_N + 0.5)), dp = 1;
      for (int it = 0; it < 100; it++) {
         double p0 = 1, p1 = x;
         for (int k = 2; k <= GL_N; k++) {
            const double p2 = ((2 * k - 1) * x * p1 - (k - 1) * p0) / k;
            p0 = p1;
            p1 = p2;
         }
         dp = GL_N * (x * p1 - p0) / (x * x - 1);
         const double dx = p1 / dp;
         x -= dx;
         if (fabs(dx) < 1e-16) break;
      }
      gl_x[i] = x;
      gl_w[i] = 2 / ((1 - x * x) * dp * dp);
   }
   gl_ready = 1;
}

static double near_integral(int kind, double freq, double s, double lo, double hi)
{
   if (kind == 0) {
      /* tau = s - v:  int (s - v) phi(v) dv over v in [s-hi, s-lo], phi the
       * Gaussian density with sigma = 1/freq: s (Phi(U) - Phi(L)) + sigma^2 (phi(U) - phi(L)) */
      const double sig = 1 / freq, U = s - lo, L = s - hi;
      const double Phi = 0.5 * (erf(U / (sig * sqrt(2.0))) - erf(L / (sig * sqrt(2.0))));
      return s * Phi + sig * sig * (hist(0, freq, U) - hist(0, freq, L));
   }
   /* the bump is a polynomial of degree 14 on s - tau in (0, 1/freq): integrate
    * tau * g(s - tau) exactly over the part of [lo, hi] where it is nonzero */
   const double a = fmax(lo, s - 1 / freq), b = fmin(hi, s);
   if (!(b > a)) return 0.0;
   gl_init();
   const double c = 0.5 * (a + b), d = 0.5 * (b - a);
   double acc = 0;
   for (int q = 0; q < GL_N; q++) {
      const double tau = c + d * gl_x[q];
      acc += gl_w[q] * tau * hist(kind, freq, s - tau);
   }
   return d * acc;
}

void sw4o_exact_point_source(int ib, int ie, int jb, int je, int kb, int ke, double h, double zmin,
                             double rho, double cp, double cs, double x0, double y0, double z0,
                             int moment, const double* f, const double* m, int kind, double freq,
                             double t0, double t, double* u)
{
   const long ni = ie - ib + 1, nij = ni * (je - jb + 1), npts = nij * (ke - kb + 1);
   const double a = cp, b = cs, s = t - t0, eps = 1e-3 * h, c4 = 1 / (4 * M_PI * rho);
   double M[3][3] = {{0}};
   if (moment) {
      M[0][0] = m[0]; M[0][1] = M[1][0] = m[1]; M[0][2] = M[2][0] = m[2];
      M[1][1] = m[3]; M[1][2] = M[2][1] = m[4]; M[2][2] = m[5];
   }
   gl_init();
#pragma omp parallel for collapse(2)
   for (int k = kb; k <= ke; k++)
      for (int j = jb; j <= je; j++)
         for (int i = ib; i <= ie; i++) {
            const long p = (i - ib) + ni * (j - jb) + nij * (k - kb);
            const double d[3] = {(i - 1) * h - x0, (j - 1) * h - y0, zmin + (k - 1) * h - z0};
            const double R = sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
            double out[3] = {0, 0, 0};
            if (R >= eps) {
               const double g[3] = {d[0] / R, d[1] / R, d[2] / R};
               const double ga = hist(kind, freq, s - R / a), gb = hist(kind, freq, s - R / b);
               const double I = near_integral(kind, freq, s, R / a, R / b);
               if (!moment) {
                  /* A&R 4.23 */
                  const double gf = g[0] * f[0] + g[1] * f[1] + g[2] * f[2];
                  for (int n = 0; n < 3; n++)
                     out[n] = c4 * (g[n] * gf * (3 * I / (R * R * R) + ga / (a * a * R) - gb / (b * b * R)) +
                                    f[n] * (gb / (b * b * R) - I / (R * R * R)));
               } else {
                  /* A&R 4.29 contracted with the symmetric M */
                  const double da = hist_dt(kind, freq, s - R / a), db = hist_dt(kind, freq, s - R / b);
                  double Mg[3], gMg = 0, tr = M[0][0] + M[1][1] + M[2][2];
                  for (int n = 0; n < 3; n++) {
                     Mg[n] = M[n][0] * g[0] + M[n][1] * g[1] + M[n][2] * g[2];
                     gMg += g[n] * Mg[n];
                  }
                  const double R2 = R * R, R4 = R2 * R2;
                  for (int n = 0; n < 3; n++)
                     out[n] = c4 * ((15 * g[n] * gMg - 3 * g[n] * tr - 6 * Mg[n]) * I / R4 +
                                    (6 * g[n] * gMg - g[n] * tr - 2 * Mg[n]) * ga / (a * a * R2) -
                                    (6 * g[n] * gMg - g[n] * tr - 3 * Mg[n]) * gb / (b * b * R2) +
                                    g[n] * gMg * da / (a * a * a * R) -
                                    (g[n] * gMg - Mg[n]) * db / (b * b * b * R));
               }
            }
            for (int c = 0; c < 3; c++) u[c * npts + p] = out[c];
         }
}

void sw4o_solerr3(int ib, int ie, int jb, int je, int kb, int ke, double h, double zmin,
                  const double* uex, const double* u, double x0, double y0, double z0,
                  double radius, int imin, int imax, int jmin, int jmax, int kmin, int kmax,
                  double* li, double* l2, double* xli)
{
   const long ni = ie - ib + 1, nij = ni * (je - jb + 1), npts = nij * (ke - kb + 1);
   const double r2 = radius < 0 ? -radius * radius : radius * radius, h3 = h * h * h;
   double mx = 0, sq = 0, xm = 0;
   for (int c = 0; c < 3; c++)
      for (int k = kmin; k <= kmax; k++)
         for (int j = jmin; j <= jmax; j++)
            for (int i = imin; i <= imax; i++) {
               const double dx = (i - 1) * h - x0, dy = (j - 1) * h - y0, dz = (k - 1) * h + zmin - z0;
               if (!(dx * dx + dy * dy + dz * dz > r2)) continue;
               const long q = c * npts + (i - ib) + ni * (j - jb) + nij * (k - kb);
               const double e = u[q] - uex[q];
               if (fabs(e) > mx) mx = fabs(e);
               if (uex[q] > xm) xm = uex[q];
               sq += h3 * e * e;
            }
   *li = mx;
   *l2 = sqrt(sq);
   *xli = xm;
}
