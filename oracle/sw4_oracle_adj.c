/* CPU oracle for the discrete adjoint of the Cartesian time step --
 * TEST INFRASTRUCTURE ONLY (tests/ and the bench's CPU leg use it as a checker).
 *
 * The reference has no material-gradient adjoint (sw4lite computes source
 * gradients only, src/GridPointSource.C:659); these functions restate the exact
 * transpose of the oracle's own step (sw4o_step) for grids whose ghost points
 * are zero after every boundary pass (Dirichlet / supergrid sides with zero
 * boundary data) or, on the z sides, set by the free-surface condition from the
 * interior (src/ew-cfromfort.C:415-476), so the state is the interior points I.
 *
 * Step (on I, R = diag(1/rho)):
 *   up = 2u - um + dt^2 R L(u) + dt^2 R F
 *   u+ = up + dt^2/12 R L(up - 2u + um) - beta R SG(u - um) + dt^4/12 R F_tt
 * Transposes:
 *   L^T = W L W^-1 with W = 1/(sx sy sz) (W L is symmetric: the stretched
 *   elastic operator is self-adjoint in the stretched volume);
 *   SG = sum_ax diag(w_ax) D2 E_ax D2 with E_ax = rho dc_ax, so
 *   SG^T y = sum_ax D2 E_ax D2 (w_ax y).
 * Adjoint recursion a^n = g^n + A^T a^{n+1} + B^T a^{n+2}:
 *   s = L^T R a1, m = a1 + dt^2/12 s, t = L^T R m,
 *   a^n = g^n + 2m + dt^2 t - dt^2/6 s - a2 - beta SG^T R (a1 - a2).
 * Gradient of a1 . u+ with respect to (rho, mu, lambda) at fixed (u, um):
 *   mu, lambda: G(R a1 dt^2/12, up - 2u + um) + G(R m dt^2, u), G(v, w) the
 *   coefficient gradient of v . L(w);
 *   rho: -(1/rho)[m.(up - 2u + um) + a1.(u+ - up)] - beta dSG/drho terms.
 * Free surface on a z side: L is the operator with the one-sided SBP rows
 * (src/rhs4sg_rev.C:349-856) applied after the ghost plane is solved from the
 * traction condition.  D L is symmetric for D = H W, H the SBP norm weights
 * (17/48, 59/48, 43/48, 49/48 on the four planes next to the side, 1 elsewhere),
 * provided the z stretching is 1 on the rows next to the side (the reference does
 * not apply it there; with no supergrid layer on a free-surface side it is 1), so
 * L^T = D L D^-1.  L stays linear in (mu, lambda): the ghost plane enters the first
 * row only through ghcof (2mu + lambda) w_ghost (mu u_ghost), and the traction
 * condition makes that product linear in the material of the boundary point.
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
} abox;

static abox mk(int ib, int ie, int jb, int je, int kb, int ke)
{
   abox b = {ib, ie, jb, je, kb, ke, ie - ib + 1, 0, 0};
   b.nij = b.ni * (je - jb + 1);
   b.npts = b.nij * (ke - kb + 1);
   return b;
}

static inline long IX(const abox* b, int i, int j, int k)
{
   return (i - b->ib) + b->ni * (j - b->jb) + b->nij * (long)(k - b->kb);
}

static inline int interior(const abox* b, int i, int j, int k)
{
   return i >= b->ib + 2 && i <= b->ie - 2 && j >= b->jb + 2 && j <= b->je - 2 && k >= b->kb + 2 &&
          k <= b->ke - 2;
}

/* lt = L^T y = W L (W^-1 y) on I (SoA, zero outside I).  onesided must be all 0. */
void sw4o_apply_lt(int ib, int ie, int jb, int je, int kb, int ke, int nz, const double* y,
                   const double* mu, const double* la, double h, const double* strx,
                   const double* stry, const double* strz, double* lt)
{
   double acof[384], ghcof[6], bope[48], sbop[5];
   sw4o_stencil_coefficients(acof, ghcof, bope, sbop);
   const abox b = mk(ib, ie, jb, je, kb, ke);
   double* wy = (double*)calloc(3 * b.npts, sizeof(double));
   for (int k = kb; k <= ke; k++)
      for (int j = jb; j <= je; j++)
         for (int i = ib; i <= ie; i++) {
            if (!interior(&b, i, j, k)) continue;
            const long p = IX(&b, i, j, k);
            const double iw = strx[i - ib] * stry[j - jb] * strz[k - kb];
            for (int c = 0; c < 3; c++) wy[c * b.npts + p] = iw * y[c * b.npts + p];
         }
   memset(lt, 0, 3 * b.npts * sizeof(double));
   const int os[6] = {0, 0, 0, 0, 0, 0};
   sw4o_rhs4sg(1, ib, ie, jb, je, kb, ke, nz, os, acof, bope, ghcof, lt, wy, mu, la, h, strx, stry,
               strz);
   for (int k = kb; k <= ke; k++)
      for (int j = jb; j <= je; j++)
         for (int i = ib; i <= ie; i++) {
            const long p = IX(&b, i, j, k);
            const double w = interior(&b, i, j, k) ? 1 / (strx[i - ib] * stry[j - jb] * strz[k - kb]) : 0;
            for (int c = 0; c < 3; c++) lt[c * b.npts + p] *= w;
         }
   free(wy);
}

/* weights w_ax of the damping terms at a point (sw4o_addsgd4) */
static void sg_w(const abox* b, int i, int j, int k, const double* strx, const double* stry,
                 const double* strz, const double* cox, const double* coy, const double* coz,
                 double w[3])
{
   w[0] = strx[i - b->ib] * coy[j - b->jb] * coz[k - b->kb];
   w[1] = stry[j - b->jb] * cox[i - b->ib] * coz[k - b->kb];
   w[2] = strz[k - b->kb] * cox[i - b->ib] * coy[j - b->jb];
}

/* z = SG^T (y / rho) on I: sum_ax D2 E D2 (w_ax y / rho), with the vector zero
 * outside I. */
void sw4o_sg_adjoint(int ib, int ie, int jb, int je, int kb, int ke, const double* y,
                     const double* rho, const double* dcx, const double* dcy, const double* dcz,
                     const double* strx, const double* stry, const double* strz, const double* cox,
                     const double* coy, const double* coz, double* z)
{
   const abox b = mk(ib, ie, jb, je, kb, ke);
   const double* dcs[3] = {dcx, dcy, dcz};
   const long st[3] = {1, b.ni, b.nij};
   memset(z, 0, 3 * b.npts * sizeof(double));
#pragma omp parallel for collapse(2)
   for (int k = kb + 2; k <= ke - 2; k++)
      for (int j = jb + 2; j <= je - 2; j++)
         for (int i = ib + 2; i <= ie - 2; i++) {
            const long p = IX(&b, i, j, k);
            const int qa[3] = {i - ib, j - jb, k - kb};
            for (int c = 0; c < 3; c++) {
               double tot = 0;
               for (int ax = 0; ax < 3; ax++) {
                  double v[5];
                  for (int m = -2; m <= 2; m++) {
                     int ii = i + (ax == 0) * m, jj = j + (ax == 1) * m, kk = k + (ax == 2) * m;
                     if (!interior(&b, ii, jj, kk)) {
                        v[m + 2] = 0;
                        continue;
                     }
                     double w[3];
                     sg_w(&b, ii, jj, kk, strx, stry, strz, cox, coy, coz, w);
                     const long q = IX(&b, ii, jj, kk);
                     v[m + 2] = w[ax] * y[c * b.npts + q] / rho[q];
                  }
                  const double* dc = dcs[ax] + qa[ax];
                  const double e0 = rho[p - st[ax]] * dc[-1], e1 = rho[p] * dc[0], e2 = rho[p + st[ax]] * dc[1];
                  tot += e2 * (v[4] - 2 * v[3] + v[2]) - 2 * e1 * (v[3] - 2 * v[2] + v[1]) +
                         e0 * (v[2] - 2 * v[1] + v[0]);
               }
               z[c * b.npts + p] = tot;
            }
         }
}

/* Sixth-order damping (sw4o_addsgd6, src/ew-cfromfort.C:1059-1158), applied at the
 * points three away from every array edge (the set Q) from u - um anywhere:
 *   SG6 d = 1/2 P_Q sum_ax diag(w_ax) D3^T E~ D3 d,
 * D3 the third difference at the half points, E~(q+1/2) = E(q) + E(q+1), E = rho dc.
 * Its transpose on I applies the same stencil at every point of I to a vector that
 * is zero outside Q:  SG6^T y = 1/2 P_I sum_ax D3^T E~ D3 P_Q (w_ax y).
 * T(v, h) below is the third difference of v at the half point h = q + 1/2. */
static inline int in_q(const abox* b, int i, int j, int k)
{
   return i >= b->ib + 3 && i <= b->ie - 3 && j >= b->jb + 3 && j <= b->je - 3 && k >= b->kb + 3 &&
          k <= b->ke - 3;
}

/* z = SG6^T (y / rho) on I (zero elsewhere). */
void sw4o_sg6_adjoint(int ib, int ie, int jb, int je, int kb, int ke, const double* y,
                      const double* rho, const double* dcx, const double* dcy, const double* dcz,
                      const double* strx, const double* stry, const double* strz, const double* cox,
                      const double* coy, const double* coz, double* z)
{
   const abox b = mk(ib, ie, jb, je, kb, ke);
   const double* dcs[3] = {dcx, dcy, dcz};
   const int lo[3] = {ib, jb, kb};
   memset(z, 0, 3 * b.npts * sizeof(double));
   static const double sm[4] = {-1, 3, -3, 1}; /* s_m of the half points p-3/2 .. p+3/2 */
#pragma omp parallel for collapse(2)
   for (int k = kb + 2; k <= ke - 2; k++)
      for (int j = jb + 2; j <= je - 2; j++)
         for (int i = ib + 2; i <= ie - 2; i++) {
            const long p = IX(&b, i, j, k);
            const int pc[3] = {i, j, k};
            for (int c = 0; c < 3; c++) {
               double tot = 0;
               for (int ax = 0; ax < 3; ax++) {
                  double v[7], e[5];
                  for (int m = -3; m <= 3; m++) {
                     int q[3] = {i, j, k};
                     q[ax] += m;
                     v[m + 3] = 0;
                     if (!in_q(&b, q[0], q[1], q[2])) continue;
                     double w[3];
                     sg_w(&b, q[0], q[1], q[2], strx, stry, strz, cox, coy, coz, w);
                     const long qi = IX(&b, q[0], q[1], q[2]);
                     v[m + 3] = w[ax] * y[c * b.npts + qi] / rho[qi];
                  }
                  for (int m = -2; m <= 2; m++) {
                     int q[3] = {i, j, k};
                     q[ax] += m;
                     e[m + 2] = rho[IX(&b, q[0], q[1], q[2])] * dcs[ax][pc[ax] + m - lo[ax]];
                  }
                  double s = 0;
                  for (int m = -2; m <= 1; m++) {
                     const double t3 = v[m + 5] - 3 * v[m + 4] + 3 * v[m + 3] - v[m + 2];
                     s += sm[m + 2] * (e[m + 3] + e[m + 2]) * t3;
                  }
                  tot += s;
               }
               z[c * b.npts + p] = -0.5 * tot;
            }
         }
}

/* rho gradient of the sixth-order damping term: -beta (R a1) . dSG6(d)/drho at fixed
 * R, added into grho: -beta/2 sum_ax dc(q) [T(v, q-1/2) T(d, q-1/2) + T(v, q+1/2)
 * T(d, q+1/2)], v = P_Q w_ax a1 / rho along the axis. */
void sw4o_sg6_rho_gradient(int ib, int ie, int jb, int je, int kb, int ke, const double* a1,
                           const double* d, const double* rho, const double* dcx, const double* dcy,
                           const double* dcz, const double* strx, const double* stry,
                           const double* strz, const double* cox, const double* coy,
                           const double* coz, double beta, double* grho)
{
   const abox b = mk(ib, ie, jb, je, kb, ke);
   const double* dcs[3] = {dcx, dcy, dcz};
   const int lo[3] = {ib, jb, kb}, hi[3] = {ie, je, ke};
#pragma omp parallel for collapse(2)
   for (int k = kb; k <= ke; k++)
      for (int j = jb; j <= je; j++)
         for (int i = ib; i <= ie; i++) {
            const int pc[3] = {i, j, k};
            double g = 0;
            for (int ax = 0; ax < 3; ax++) {
               const double dcq = dcs[ax][pc[ax] - lo[ax]];
               if (dcq == 0) continue;
               for (int c = 0; c < 3; c++) {
                  /* values at q-2 .. q+2 along the axis */
                  double vv[5], dd[5];
                  for (int m = -2; m <= 2; m++) {
                     int q[3] = {i, j, k};
                     q[ax] += m;
                     vv[m + 2] = dd[m + 2] = 0;
                     if (q[ax] < lo[ax] || q[ax] > hi[ax]) continue;
                     const long qi = IX(&b, q[0], q[1], q[2]);
                     dd[m + 2] = d[c * b.npts + qi];
                     if (in_q(&b, q[0], q[1], q[2])) {
                        double w[3];
                        sg_w(&b, q[0], q[1], q[2], strx, stry, strz, cox, coy, coz, w);
                        vv[m + 2] = w[ax] * a1[c * b.npts + qi] / rho[qi];
                     }
                  }
                  /* third differences at q-1/2 (points q-2..q+1) and q+1/2 (q-1..q+2) */
                  const double tvm = vv[3] - 3 * vv[2] + 3 * vv[1] - vv[0];
                  const double tdm = dd[3] - 3 * dd[2] + 3 * dd[1] - dd[0];
                  const double tvp = vv[4] - 3 * vv[3] + 3 * vv[2] - vv[1];
                  const double tdp = dd[4] - 3 * dd[3] + 3 * dd[2] - dd[1];
                  g += dcq * (tvm * tdm + tvp * tdp);
               }
            }
            grho[IX(&b, i, j, k)] -= 0.5 * beta * g;
         }
}

/* G(v, w): gradient of v . L(w) with respect to mu and lambda at every array
 * point, added into gmu, gla.  v zero outside I; w zero at ghost points. */
static const double DW[5] = {1, -8, 0, 8, -1};

/* The centred rows' part of G(v, w); the z-involving terms skip the rows k <= zlo
 * and k >= zhi (the one-sided rows next to a free surface). */
static void coef_gradient_central(int ib, int ie, int jb, int je, int kb, int ke, const double* v,
                                  const double* w, double h, const double* strx, const double* stry,
                                  const double* strz, int zlo, int zhi, double* gmu, double* gla)
{
   const abox b = mk(ib, ie, jb, je, kb, ke);
   const double* sp[3] = {strx, stry, strz};
   const int lo[3] = {ib, jb, kb}, hi[3] = {ie, je, ke};
   const double c6 = 1.0 / (6 * h * h), c144 = 1.0 / (144 * h * h);
   /* mixed terms: (equation c, component d, outer, inner, 0 mu / 1 lambda) */
   static const int mix[12][5] = {{0, 1, 0, 1, 1}, {0, 1, 1, 0, 0}, {0, 2, 0, 2, 1}, {0, 2, 2, 0, 0},
                                  {1, 0, 0, 1, 0}, {1, 0, 1, 0, 1}, {1, 2, 1, 2, 1}, {1, 2, 2, 1, 0},
                                  {2, 0, 0, 2, 0}, {2, 0, 2, 0, 1}, {2, 1, 1, 2, 0}, {2, 1, 2, 1, 1}};
#pragma omp parallel for collapse(2)
   for (int k = kb; k <= ke; k++)
      for (int j = jb; j <= je; j++)
         for (int i = ib; i <= ie; i++) {
            const int pc[3] = {i, j, k};
            const long p = IX(&b, i, j, k);
            double gm = 0, gl = 0;
            /* same-axis second differences: rows q = p - n e_ax */
            for (int ax = 0; ax < 3; ax++)
               for (int n = -2; n <= 2; n++) {
                  int qc[3] = {i, j, k};
                  qc[ax] -= n;
                  if (!interior(&b, qc[0], qc[1], qc[2])) continue;
                  if (ax == 2 && (qc[2] <= zlo || qc[2] >= zhi)) continue;
                  const long q = IX(&b, qc[0], qc[1], qc[2]);
                  const long st = ax == 0 ? 1 : ax == 1 ? b.ni : b.nij;
                  for (int c = 0; c < 3; c++) {
                     const double vq = v[c * b.npts + q];
                     if (vq == 0) continue;
                     const double* wq = w + c * b.npts + q;
                     double d[5];
                     for (int m = -2; m <= 2; m++) d[m + 2] = wq[m * st] - wq[0];
                     double K;
                     switch (n) {
                        case -2: K = -0.75 * d[0] + d[1]; break;
                        case -1: K = d[0] + 3 * d[1] + d[3]; break;
                        case 0: K = -0.75 * (d[0] + d[4]) + 3 * (d[1] + d[3]); break;
                        case 1: K = d[1] + 3 * d[3] + d[4]; break;
                        default: K = d[3] - 0.75 * d[4]; break;
                     }
                     const double f = c6 * vq * sp[ax][qc[ax] - lo[ax]] * K * sp[ax][pc[ax] - lo[ax]];
                     if (c == ax) {
                        gm += 2 * f;
                        gl += f;
                     } else {
                        gm += f;
                     }
                  }
               }
            /* mixed terms: -(1/144h^2) s_ai(p) (DW.w_d along ai)(p) (DW.(s_ao v_c) along ao)(p) */
            for (int t = 0; t < 12; t++) {
               const int c = mix[t][0], d = mix[t][1], ao = mix[t][2], ai = mix[t][3];
               if (pc[ai] < lo[ai] + 2 || pc[ai] > hi[ai] - 2) continue;
               if (ai == 2 && (k <= zlo || k >= zhi)) continue; /* rows in this plane */
               double inner = 0, outer = 0;
               for (int m = -2; m <= 2; m++) {
                  if (m == 0) continue;
                  int a[3] = {i, j, k};
                  a[ai] += m;
                  inner += DW[m + 2] * w[d * b.npts + IX(&b, a[0], a[1], a[2])];
                  int o[3] = {i, j, k};
                  o[ao] += m;
                  if (o[ao] < lo[ao] || o[ao] > hi[ao] || !interior(&b, o[0], o[1], o[2])) continue;
                  if (ao == 2 && (o[2] <= zlo || o[2] >= zhi)) continue;
                  outer += DW[m + 2] * sp[ao][o[ao] - lo[ao]] * v[c * b.npts + IX(&b, o[0], o[1], o[2])];
               }
               const double g = -c144 * sp[ai][pc[ai] - lo[ai]] * inner * outer;
               if (mix[t][4]) gl += g;
               else gm += g;
            }
            gmu[p] += gm;
            gla[p] += gl;
         }
}

void sw4o_coef_gradient(int ib, int ie, int jb, int je, int kb, int ke, const double* v,
                        const double* w, double h, const double* strx, const double* stry,
                        const double* strz, double* gmu, double* gla)
{
   coef_gradient_central(ib, ie, jb, je, kb, ke, v, w, h, strx, stry, strz, kb - 10, ke + 10, gmu, gla);
}

/* The z-involving terms of the six one-sided rows next to a free-surface z side
 * (top: rows 1..6, bottom: nz-5..nz), differentiated term by term
 * (src/rhs4sg_rev.C:349-600 top, :602-856 bottom; the ghost plane from the
 * traction condition, src/ew-cfromfort.C:415-476):
 *   zz   sum_q (sum_m acof(k,q,m) coef(m)) f(q) + ghcof coef(bnd) f(ghost);
 *   dz_of_inner  s_a Dz(coef D_a f) / 12,  outer_of_dz  s_a D_a(coef Dz f) / 12,
 * Dz the one-sided bope rows, D_a the centred DW stencil along x or y. */
static void coef_gradient_rows(const abox* b, int nz, int top, const double* v, const double* w, double h,
                               const double* strx, const double* stry, double* gmu, double* gla)
{
   double acof[384], ghcof[6], bope[48], sbop[5];
   sw4o_stencil_coefficients(acof, ghcof, bope, sbop);
   const double cof = 1.0 / (h * h), d4a = 2.0 / 3.0, d4b = -1.0 / 12.0;
   const int kl = top ? 1 : -1, kbnd = top ? 1 : nz, kgh = top ? 0 : nz + 1;
   const long n = b->npts;
#define W_(c, i, j, k) w[(c) * n + IX(b, i, j, k)]
   for (int kk = 1; kk <= 6; kk++) {
      const int k = top ? kk : nz - kk + 1;
      int kq[8];
      double wz[8];
      for (int q = 1; q <= 8; q++) {
         kq[q - 1] = top ? q : nz - q + 1;
         wz[q - 1] = top ? bope[(kk - 1) + 6 * (q - 1)] : -bope[(kk - 1) + 6 * (q - 1)];
      }
      for (int j = b->jb + 2; j <= b->je - 2; j++)
         for (int i = b->ib + 2; i <= b->ie - 2; i++) {
            const long r = IX(b, i, j, k);
            const double V[3] = {v[r], v[n + r], v[2 * n + r]};
            if (V[0] == 0 && V[1] == 0 && V[2] == 0) continue;
            const double sx = strx[i - b->ib], sy = stry[j - b->jb];
            /* zz rows: coefficient mu (components 0, 1) or 2mu + lambda (component 2) */
            for (int m = 1; m <= 8; m++) {
               double t[3] = {0, 0, 0};
               for (int q = 1; q <= 8; q++) {
                  const double a = acof[(kk - 1) + 6 * (q - 1) + 48 * (m - 1)];
                  if (a == 0) continue;
                  for (int c = 0; c < 3; c++) t[c] += a * W_(c, i, j, kq[q - 1]);
               }
               const long pm = IX(b, i, j, kq[m - 1]);
               gmu[pm] += cof * (V[0] * t[0] + V[1] * t[1] + 2 * V[2] * t[2]);
               gla[pm] += cof * V[2] * t[2];
            }
            if (ghcof[kk - 1] != 0) {
               /* ghost plane: u, v ghosts do not depend on the material; (2mu + la) w_gh =
                * -[(2mu + la) Sw + kl la (ux + vy)] / sbop0 */
               const double gh = ghcof[kk - 1];
               double S[3] = {0, 0, 0};
               for (int q = 1; q <= 4; q++)
                  for (int c = 0; c < 3; c++) S[c] += sbop[q] * W_(c, i, j, k + kl * (q - 1));
               const double wx = sx * (d4a * (W_(2, i + 1, j, k) - W_(2, i - 1, j, k)) +
                                       d4b * (W_(2, i + 2, j, k) - W_(2, i - 2, j, k)));
               const double wy = sy * (d4a * (W_(2, i, j + 1, k) - W_(2, i, j - 1, k)) +
                                       d4b * (W_(2, i, j + 2, k) - W_(2, i, j - 2, k)));
               const double ux = sx * (d4a * (W_(0, i + 1, j, k) - W_(0, i - 1, j, k)) +
                                       d4b * (W_(0, i + 2, j, k) - W_(0, i - 2, j, k)));
               const double vy = sy * (d4a * (W_(1, i, j + 1, k) - W_(1, i, j - 1, k)) +
                                       d4b * (W_(1, i, j + 2, k) - W_(1, i, j - 2, k)));
               const double ugh = (-S[0] - kl * wx) / sbop[0], vgh = (-S[1] - kl * wy) / sbop[0];
               const long pb = IX(b, i, j, kbnd);
               (void)kgh;
               gmu[pb] += cof * gh * (V[0] * ugh + V[1] * vgh - 2 * V[2] * S[2] / sbop[0]);
               gla[pb] += cof * gh * V[2] * (-(S[2] + kl * (ux + vy)) / sbop[0]);
            }
            /* dz_of_inner: s_a Dz(coef D_a f) / 12 */
            for (int q = 1; q <= 8; q++) {
               if (wz[q - 1] == 0) continue;
               const int kk2 = kq[q - 1];
               double dx[3], dy[3];
               for (int c = 0; c < 3; c++) {
                  dx[c] = dy[c] = 0;
                  for (int e = -2; e <= 2; e++) {
                     dx[c] += DW[e + 2] * W_(c, i + e, j, kk2);
                     dy[c] += DW[e + 2] * W_(c, i, j + e, kk2);
                  }
               }
               const long pq = IX(b, i, j, kk2);
               const double f = cof * wz[q - 1] / 12;
               gmu[pq] += f * (V[0] * sx * dx[2] + V[1] * sy * dy[2]);
               gla[pq] += f * V[2] * (sx * dx[0] + sy * dy[1]);
            }
            /* outer_of_dz: s_a D_a(coef Dz f) / 12 with the coefficient at the row's
             * neighbours along a */
            for (int e = -2; e <= 2; e++) {
               if (e == 0) continue;
               double zx[3] = {0, 0, 0}, zy[3] = {0, 0, 0};
               for (int q = 1; q <= 8; q++)
                  for (int c = 0; c < 3; c++) {
                     zx[c] += wz[q - 1] * W_(c, i + e, j, kq[q - 1]);
                     zy[c] += wz[q - 1] * W_(c, i, j + e, kq[q - 1]);
                  }
               const double f = cof * DW[e + 2] / 12;
               const long px = IX(b, i + e, j, k), py = IX(b, i, j + e, k);
               gla[px] += f * V[0] * sx * zx[2];
               gla[py] += f * V[1] * sy * zy[2];
               gmu[px] += f * V[2] * sx * zx[0];
               gmu[py] += f * V[2] * sy * zy[1];
            }
         }
   }
#undef W_
}

/* G(v, w) with free-surface z sides (onesided[4], onesided[5]): the centred rows'
 * terms (z-involving ones without the one-sided rows) plus the one-sided rows'. */
void sw4o_coef_gradient_fs(int ib, int ie, int jb, int je, int kb, int ke, int nz, const int onesided[6],
                           const double* v, const double* w, double h, const double* strx,
                           const double* stry, const double* strz, double* gmu, double* gla)
{
   const abox b = mk(ib, ie, jb, je, kb, ke);
   const int zlo = onesided[4] ? 6 : kb - 10, zhi = onesided[5] ? nz - 5 : ke + 10;
   coef_gradient_central(ib, ie, jb, je, kb, ke, v, w, h, strx, stry, strz, zlo, zhi, gmu, gla);
   if (onesided[4]) coef_gradient_rows(&b, nz, 1, v, w, h, strx, stry, gmu, gla);
   if (onesided[5]) coef_gradient_rows(&b, nz, 0, v, w, h, strx, stry, gmu, gla);
}

/* The SBP norm weight of plane k next to free-surface z sides (1 elsewhere). */
static double norm_h(int k, int nz, const int onesided[6])
{
   static const double om[4] = {17.0 / 48, 59.0 / 48, 43.0 / 48, 49.0 / 48};
   if (onesided[4] && k >= 1 && k <= 4) return om[k - 1];
   if (onesided[5] && k <= nz && k >= nz - 3) return om[nz - k];
   return 1;
}

/* lt = L^T y = D L (D^-1 y) on I with free-surface z sides, D = H W: the ghost
 * planes of D^-1 y from the traction condition (the lateral sides' ghosts zero). */
void sw4o_apply_lt_fs(int ib, int ie, int jb, int je, int kb, int ke, int nx, int ny, int nz,
                      const int onesided[6], const double* y, const double* mu, const double* la,
                      double h, const double* strx, const double* stry, const double* strz, double* lt)
{
   double acof[384], ghcof[6], bope[48], sbop[5];
   sw4o_stencil_coefficients(acof, ghcof, bope, sbop);
   const abox b = mk(ib, ie, jb, je, kb, ke);
   double* wy = (double*)calloc(3 * b.npts, sizeof(double));
   for (int k = kb; k <= ke; k++)
      for (int j = jb; j <= je; j++)
         for (int i = ib; i <= ie; i++) {
            if (!interior(&b, i, j, k)) continue;
            const long p = IX(&b, i, j, k);
            const double iw = strx[i - ib] * stry[j - jb] * strz[k - kb] / norm_h(k, nz, onesided);
            for (int c = 0; c < 3; c++) wy[c * b.npts + p] = iw * y[c * b.npts + p];
         }
   const int bccnd[6] = {1, 1, 1, 1, onesided[4] ? 0 : 1, onesided[5] ? 0 : 1};
   int wind[36], npts[6];
   sw4o_boundary_windows(ib, ie, jb, je, kb, ke, nx, ny, nz, bccnd, wind, npts);
   double* const bf[6] = {NULL, NULL, NULL, NULL, NULL, NULL};
   sw4o_bcfortsg(1, ib, ie, jb, je, kb, ke, wind, nx, ny, nz, wy, h, bccnd, sbop, mu, la, bf, strx, stry);
   memset(lt, 0, 3 * b.npts * sizeof(double));
   sw4o_rhs4sg(1, ib, ie, jb, je, kb, ke, nz, onesided, acof, bope, ghcof, lt, wy, mu, la, h, strx, stry,
               strz);
   for (int k = kb; k <= ke; k++)
      for (int j = jb; j <= je; j++)
         for (int i = ib; i <= ie; i++) {
            const long p = IX(&b, i, j, k);
            const double w = interior(&b, i, j, k)
                                 ? norm_h(k, nz, onesided) / (strx[i - ib] * stry[j - jb] * strz[k - kb])
                                 : 0;
            for (int c = 0; c < 3; c++) lt[c * b.npts + p] *= w;
         }
   free(wy);
}

/* rho gradient of the damping term: -beta * (R a1) . dSG(d)/drho at every point,
 * added into grho; d = u - um (zero ghosts), a1 zero outside I. */
void sw4o_sg_rho_gradient(int ib, int ie, int jb, int je, int kb, int ke, const double* a1,
                          const double* d, const double* rho, const double* dcx, const double* dcy,
                          const double* dcz, const double* strx, const double* stry,
                          const double* strz, const double* cox, const double* coy,
                          const double* coz, double beta, double* grho)
{
   const abox b = mk(ib, ie, jb, je, kb, ke);
   const double* dcs[3] = {dcx, dcy, dcz};
   const int lo[3] = {ib, jb, kb}, hi[3] = {ie, je, ke};
#pragma omp parallel for collapse(2)
   for (int k = kb; k <= ke; k++)
      for (int j = jb; j <= je; j++)
         for (int i = ib; i <= ie; i++) {
            const int pc[3] = {i, j, k};
            double g = 0;
            for (int ax = 0; ax < 3; ax++) {
               if (pc[ax] - 1 < lo[ax] || pc[ax] + 1 > hi[ax]) continue;
               for (int c = 0; c < 3; c++) {
                  double vv[3], dd[3];
                  for (int m = -1; m <= 1; m++) {
                     int q[3] = {i, j, k};
                     q[ax] += m;
                     const long qi = IX(&b, q[0], q[1], q[2]);
                     dd[m + 1] = d[c * b.npts + qi];
                     if (interior(&b, q[0], q[1], q[2])) {
                        double w[3];
                        sg_w(&b, q[0], q[1], q[2], strx, stry, strz, cox, coy, coz, w);
                        vv[m + 1] = w[ax] * a1[c * b.npts + qi] / rho[qi];
                     } else {
                        vv[m + 1] = 0;
                     }
                  }
                  g += dcs[ax][pc[ax] - lo[ax]] * (dd[2] - 2 * dd[1] + dd[0]) * (vv[2] - 2 * vv[1] + vv[0]);
               }
            }
            grho[IX(&b, i, j, k)] -= beta * g;
         }
}
