/*
 * fe_oracle.c -- FP64 CPU restatement of FEDDLib's element-assembly path.
 *
 * TEST INFRASTRUCTURE ONLY: the checker for the GPU engine (see fe_oracle.h
 * for the parity status).  All citations are relative to the FEDDLib tree.
 */
#include "fe_oracle.h"
#include <math.h>
#include <stdlib.h>
#include <string.h>

/* ======================================================================== */
/* Quadrature: Helper::getQuadratureValues, 3D tetrahedra                    */
/* feddlib/core/FE/Helper.cpp:1300-1517 (1-, 5- and 15-point rules) and the   */
/* AceGen 4-point rule, code 18 (AceInterface/SMSUtility.f:344-352).          */
/* ======================================================================== */
int orc_quad(int npts, double *pts, double *w)
{
    int i;
    if (npts == 1) {            /* Helper.cpp:1310-1317 */
        pts[0] = pts[1] = pts[2] = 0.25;
        w[0] = 1.0 / 6.0;
        return 1;
    }
    if (npts == 4) {            /* SMSUtility.f:344-352 (code 18) */
        const double a = 0.585410196624968454, b = 0.138196601125010515;
        const double P[4][3] = {{a, b, b}, {b, a, b}, {b, b, a}, {b, b, b}};
        for (i = 0; i < 4; i++) {
            pts[3 * i] = P[i][0]; pts[3 * i + 1] = P[i][1]; pts[3 * i + 2] = P[i][2];
            w[i] = 1.0 / 24.0;
        }
        return 4;
    }
    if (npts == 5) {            /* Helper.cpp:1319-1350 (== AceGen code 19) */
        const double a = 0.25, b = 1.0 / 6.0, c = 0.5;
        const double P[5][3] = {{a, a, a}, {b, b, b}, {b, b, c}, {b, c, b}, {c, b, b}};
        for (i = 0; i < 5; i++) {
            pts[3 * i] = P[i][0]; pts[3 * i + 1] = P[i][1]; pts[3 * i + 2] = P[i][2];
            w[i] = (i == 0) ? -2.0 / 15.0 : 3.0 / 40.0;
        }
        return 5;
    }
    if (npts == 15) {           /* Helper.cpp:1423-1517 */
        const double s = sqrt(15.0);
        const double a = 0.25, b1 = (7. + s) / 34., b2 = (7. - s) / 34.;
        const double c1 = (13. - 3. * s) / 34., c2 = (13. + 3. * s) / 34.;
        const double d = (5. - s) / 20., e = (5. + s) / 20.;
        const double P[15][3] = {{a, a, a},    {b1, b1, b1}, {b1, b1, c1}, {b1, c1, b1},
                                 {c1, b1, b1}, {b2, b2, b2}, {b2, b2, c2}, {b2, c2, b2},
                                 {c2, b2, b2}, {d, d, e},    {d, e, d},    {e, d, d},
                                 {d, e, e},    {e, d, e},    {e, e, d}};
        const double P1 = (2665. - 14. * s) / 226800., P2 = (2665. + 14. * s) / 226800.;
        for (i = 0; i < 15; i++) {
            pts[3 * i] = P[i][0]; pts[3 * i + 1] = P[i][1]; pts[3 * i + 2] = P[i][2];
            w[i] = (i == 0) ? 8. / 405. : (i <= 4) ? P1 : (i <= 8) ? P2 : 5. / 567.;
        }
        return 15;
    }
    return -1;
}

/* Helper.cpp:1302-1305: in 3D a requested degree 2 becomes 3 and 4 becomes 5.
 * Degree 4's 11-point case (1351-1422) falls through into case 5 (no break),
 * so it is unreachable; degree 3 -> 5 points, degree 5 -> 15 points. */
int orc_quad_points_for_degree(int degree)
{
    if (degree == 2) degree = 3;
    if (degree == 4) degree = 5;
    switch (degree) {
    case 1: return 1;
    case 3: return 5;
    case 5: return 15;
    default: return -1;
    }
}

/* Helper::determineDegree(dim, FEType, UN degFunc), Helper.cpp:7-25 */
int orc_degree_un(int fe_order, unsigned deg_func)
{
    int deg = fe_order + (int)deg_func;
    return deg == 0 ? 1 : deg;
}

/* Helper::determineDegree(dim, FE1, FE2, type1, type2, extra), Helper.cpp:57-135
 * type: 0 = Std, 1 = Grad (Helper.hpp:21). */
int orc_degree_pair(int fe1, int fe2, int type1, int type2, int extra)
{
    int d1 = (type1 == 0) ? fe1 : fe1 - 1;
    int d2 = (type2 == 0) ? fe2 : fe2 - 1;
    int deg = d1 + d2 + extra;
    return deg == 0 ? 1 : deg;
}

/* Helper::phi, 3D P1/P2, Helper.cpp:703-745.  Local P2 order:
 * 0-3 vertices, 4 = e01, 5 = e12, 6 = e02, 7 = e03, 8 = e13, 9 = e23. */
void orc_phi(int fe_order, const double *p, double *v)
{
    const double x = p[0], y = p[1], z = p[2], l = 1.0 - x - y - z;
    if (fe_order == 1) {
        v[0] = l; v[1] = x; v[2] = y; v[3] = z;
        return;
    }
    v[0] = l * (1 - 2 * x - 2 * y - 2 * z);
    v[1] = x * (2 * x - 1);
    v[2] = y * (2 * y - 1);
    v[3] = z * (2 * z - 1);
    v[4] = 4 * x * l;
    v[5] = 4 * x * y;
    v[6] = 4 * y * l;
    v[7] = 4 * z * l;
    v[8] = 4 * x * z;
    v[9] = 4 * y * z;
}

/* Helper::gradPhi, 3D P1/P2, Helper.cpp:503-590 */
void orc_dphi(int fe_order, const double *p, double *g)
{
    const double x = p[0], y = p[1], z = p[2];
    int i;
    if (fe_order == 1) {
        const double G[12] = {-1, -1, -1, 1, 0, 0, 0, 1, 0, 0, 0, 1};
        for (i = 0; i < 12; i++) g[i] = G[i];
        return;
    }
    {
        const double t = -3. + 4. * x + 4. * y + 4. * z;
        double G[30] = {t, t, t,
                        4. * x - 1, 0., 0.,
                        0., 4. * y - 1, 0.,
                        0., 0., 4. * z - 1,
                        4. - 8. * x - 4. * y - 4. * z, -4. * x, -4. * x,
                        4. * y, 4. * x, 0.,
                        -4. * y, 4. - 4. * x - 8. * y - 4. * z, -4. * y,
                        -4. * z, -4. * z, 4. - 4. * x - 4. * y - 8. * z,
                        4. * z, 0., 4. * x,
                        0., 4. * z, 4. * y};
        for (i = 0; i < 30; i++) g[i] = G[i];
    }
}

/* ======================================================================== */
/* Structured mesh: MeshStructured::buildMesh3D, 1 rank, unit cube           */
/* P1 points :700-735, P1 elements :770-804, P2 points :832-858,             */
/* P2 elements :899-992 (feddlib/core/Mesh/MeshStructured_def.hpp).          */
/* ======================================================================== */
void orc_mesh_sizes(int M, int fe_order, int64_t *nn, int64_t *ne)
{
    int64_t n = (fe_order == 1) ? (M + 1) : (2 * M + 1);
    *nn = n * n * n;
    *ne = 6LL * M * M * M;
}

void orc_mesh_structured(int M, int fe_order, double *xyz, int32_t *conn)
{
    const double h = 1.0 / M;
    int64_t c = 0;
    int r, s, t;
    if (fe_order == 1) {
        const int n = M + 1;
        for (t = 0; t < n; t++)
            for (s = 0; s < n; s++)
                for (r = 0; r < n; r++) {
                    xyz[3 * c] = r * h; xyz[3 * c + 1] = s * h; xyz[3 * c + 2] = t * h;
                    c++;
                }
        c = 0;
#define P1(rr, ss, tt) ((int32_t)((rr) + n * (ss) + (int64_t)n * n * (tt)))
        for (t = 0; t < M; t++)
            for (s = 0; s < M; s++)
                for (r = 0; r < M; r++) {
                    int32_t *e = conn + 24 * c;
                    e[0] = P1(r + 1, s, t);     e[1] = P1(r, s, t);     e[2] = P1(r + 1, s, t + 1);     e[3] = P1(r + 1, s + 1, t + 1);
                    e[4] = P1(r, s, t + 1);     e[5] = P1(r, s, t);     e[6] = P1(r + 1, s, t + 1);     e[7] = P1(r + 1, s + 1, t + 1);
                    e[8] = P1(r + 1, s, t);     e[9] = P1(r, s, t);     e[10] = P1(r + 1, s + 1, t);    e[11] = P1(r + 1, s + 1, t + 1);
                    e[12] = P1(r, s, t);        e[13] = P1(r, s + 1, t); e[14] = P1(r + 1, s + 1, t);   e[15] = P1(r + 1, s + 1, t + 1);
                    e[16] = P1(r, s, t);        e[17] = P1(r, s + 1, t); e[18] = P1(r, s + 1, t + 1);   e[19] = P1(r + 1, s + 1, t + 1);
                    e[20] = P1(r, s, t);        e[21] = P1(r, s, t + 1); e[22] = P1(r, s + 1, t + 1);   e[23] = P1(r + 1, s + 1, t + 1);
                    c++;
                }
#undef P1
        return;
    }
    {
        const int P = 2 * M + 1;
        const int64_t PP = (int64_t)P * P;
        for (t = 0; t < P; t++)
            for (s = 0; s < P; s++)
                for (r = 0; r < P; r++) {
                    xyz[3 * c] = r * h / 2.0; xyz[3 * c + 1] = s * h / 2.0; xyz[3 * c + 2] = t * h / 2.0;
                    c++;
                }
        c = 0;
        for (t = 0; t < M; t++)
            for (s = 0; s < M; s++)
                for (r = 0; r < M; r++) {
                    const int64_t R0 = 2 * r, R1 = 2 * (r + 1), S = 2 * P * (int64_t)s, S1 = 2 * P * (int64_t)(s + 1);
                    const int64_t T = 2 * PP * t, T1 = 2 * PP * (int64_t)(t + 1);
                    int32_t *e = conn + 60 * c;
                    /* tet 0 */
                    e[0] = R1 + S + T;      e[1] = R0 + S + T;      e[2] = R1 + S + T1;     e[3] = R1 + S1 + T1;
                    e[4] = R0 + 1 + S + T;  e[6] = R1 + S + T + PP; e[7] = R1 + S + P + T + PP;
                    e[5] = R0 + 1 + S + T + PP; e[8] = R0 + 1 + S + P + T + PP; e[9] = R1 + S + P + T1;
                    e += 10;
                    /* tet 1 */
                    e[0] = R0 + S + T1;     e[1] = R0 + S + T;      e[2] = R1 + S + T1;     e[3] = R1 + S1 + T1;
                    e[4] = R0 + S + T + PP; e[6] = R0 + 1 + S + T1; e[7] = R0 + 1 + S + P + T1;
                    e[5] = R0 + 1 + S + T + PP; e[8] = R0 + 1 + S + P + T + PP; e[9] = R1 + S + P + T1;
                    e += 10;
                    /* tet 2 */
                    e[0] = R1 + S + T;      e[1] = R0 + S + T;      e[2] = R1 + S1 + T;     e[3] = R1 + S1 + T1;
                    e[4] = R0 + 1 + S + T;  e[6] = R1 + S + P + T;  e[7] = R1 + S + P + T + PP;
                    e[5] = R0 + 1 + S + P + T; e[8] = R0 + 1 + S + P + T + PP; e[9] = R1 + S1 + T + PP;
                    e += 10;
                    /* tet 3 */
                    e[0] = R0 + S + T;      e[1] = R0 + S1 + T;     e[2] = R1 + S1 + T;     e[3] = R1 + S1 + T1;
                    e[4] = R0 + S + P + T;  e[6] = R0 + 1 + S + P + T; e[7] = R0 + 1 + S + P + T + PP;
                    e[5] = R0 + 1 + S1 + T; e[8] = R0 + 1 + S1 + T + PP; e[9] = R1 + S1 + T + PP;
                    e += 10;
                    /* tet 4 */
                    e[0] = R0 + S + T;      e[1] = R0 + S1 + T;     e[2] = R0 + S1 + T1;    e[3] = R1 + S1 + T1;
                    e[4] = R0 + S + P + T;  e[6] = R0 + S + P + T + PP; e[7] = R0 + 1 + S + P + T + PP;
                    e[5] = R0 + S1 + T + PP; e[8] = R0 + 1 + S1 + T + PP; e[9] = R0 + 1 + S1 + T1;
                    e += 10;
                    /* tet 5 */
                    e[0] = R0 + S + T;      e[1] = R0 + S + T1;     e[2] = R0 + S1 + T1;    e[3] = R1 + S1 + T1;
                    e[4] = R0 + S + T + PP; e[6] = R0 + S + P + T + PP; e[7] = R0 + 1 + S + P + T + PP;
                    e[5] = R0 + S + P + T1; e[8] = R0 + 1 + S + P + T1; e[9] = R0 + 1 + S1 + T1;
                    c++;
                }
    }
}

/* Seeded jitter of interior P1 vertices (input generator, not reference
 * code).  splitmix64 stream; three draws per interior vertex in P1 lattice
 * order (x fastest); each coordinate moves by (2u-1)*amp*h. */
static uint64_t sm64(uint64_t *s)
{
    uint64_t z = (*s += 0x9E3779B97F4A7C15ULL);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    return z ^ (z >> 31);
}
static double u01(uint64_t *s) { return (double)(sm64(s) >> 11) * (1.0 / 9007199254740992.0); }

void orc_mesh_jitter(int M, int fe_order, uint64_t seed, double amp, double *xyz)
{
    const double h = 1.0 / M;
    const int n = M + 1, P = 2 * M + 1;
    uint64_t st = seed;
    int r, s, t, d;
    for (t = 0; t < n; t++)
        for (s = 0; s < n; s++)
            for (r = 0; r < n; r++) {
                int64_t idx;
                if (r == 0 || s == 0 || t == 0 || r == M || s == M || t == M) continue;
                idx = (fe_order == 1) ? (r + (int64_t)n * s + (int64_t)n * n * t)
                                      : (2 * r + (int64_t)P * 2 * s + (int64_t)P * P * 2 * t);
                for (d = 0; d < 3; d++) xyz[3 * idx + d] += (2.0 * u01(&st) - 1.0) * amp * h;
            }
}

/* P2 edge nodes at the midpoint of their (jittered) edge, edge order of
 * Helper.cpp:537-590: 4=e01, 5=e12, 6=e02, 7=e03, 8=e13, 9=e23. */
void orc_mesh_p2_midpoints(int64_t ne, const int32_t *conn, double *xyz)
{
    static const int E[6][2] = {{0, 1}, {1, 2}, {0, 2}, {0, 3}, {1, 3}, {2, 3}};
    int64_t e;
    int k, d;
    for (e = 0; e < ne; e++) {
        const int32_t *c = conn + 10 * e;
        for (k = 0; k < 6; k++)
            for (d = 0; d < 3; d++)
                xyz[3 * (int64_t)c[4 + k] + d] =
                    0.5 * (xyz[3 * (int64_t)c[E[k][0]] + d] + xyz[3 * (int64_t)c[E[k][1]] + d]);
    }
}

/* B = [x1-x0, x2-x0, x3-x0] (Helper.cpp:196-222), det by the rule of Sarrus
 * and inverse by cofactors / det (General/SmallMatrix.hpp:317-368).
 * Row-major B[i*3+j] = B[i][j]. */
double orc_geometry(const double *x0, const double *x1, const double *x2, const double *x3,
                    double *B, double *Bi)
{
    const double *X[3] = {x1, x2, x3};
    double v[9], det;
    int i, j;
    for (j = 0; j < 3; j++)
        for (i = 0; i < 3; i++) v[3 * i + j] = X[j][i] - x0[i];
    if (B) memcpy(B, v, sizeof v);
    det = v[0] * v[4] * v[8] + v[1] * v[5] * v[6] + v[2] * v[3] * v[7] - v[6] * v[4] * v[2] -
          v[7] * v[5] * v[0] - v[8] * v[3] * v[1];
    if (Bi) {
        Bi[0] = (v[4] * v[8] - v[5] * v[7]) / det;
        Bi[1] = (v[2] * v[7] - v[1] * v[8]) / det;
        Bi[2] = (v[1] * v[5] - v[2] * v[4]) / det;
        Bi[3] = (v[5] * v[6] - v[3] * v[8]) / det;
        Bi[4] = (v[0] * v[8] - v[2] * v[6]) / det;
        Bi[5] = (v[2] * v[3] - v[0] * v[5]) / det;
        Bi[6] = (v[3] * v[7] - v[4] * v[6]) / det;
        Bi[7] = (v[1] * v[6] - v[0] * v[7]) / det;
        Bi[8] = (v[0] * v[4] - v[1] * v[3]) / det;
    }
    return det;
}

/* Mesh::correctElementOrientation + flipElement (Mesh_def.hpp:543-577,
 * 648-735): elements with det B < 0 get nodes 1<->2 swapped (P2 also
 * 4<->6 and 8<->9). Returns the number of flipped elements. */
int64_t orc_mesh_orient(int fe_order, int64_t ne, const double *xyz, int32_t *conn)
{
    const int npe = fe_order == 1 ? 4 : 10;
    int64_t e, nflip = 0;
    for (e = 0; e < ne; e++) {
        int32_t *c = conn + npe * e, t;
        double det = orc_geometry(xyz + 3 * (int64_t)c[0], xyz + 3 * (int64_t)c[1],
                                  xyz + 3 * (int64_t)c[2], xyz + 3 * (int64_t)c[3], NULL, NULL);
        if (det < 0) {
            t = c[1]; c[1] = c[2]; c[2] = t;
            if (npe == 10) {
                t = c[4]; c[4] = c[6]; c[6] = t;
                t = c[8]; c[8] = c[9]; c[9] = t;
            }
            nflip++;
        }
    }
    return nflip;
}

/* physical gradients at a point: dphi_phys[i][d1] = sum_d2 dphi_ref[i][d2] * Binv[d2][d1]
 * (Helper::applyBTinv, Helper.cpp:258-271) */
static void grad_phys(int nloc, const double *gref, const double *Bi, double *g)
{
    int i, a, b;
    for (i = 0; i < nloc; i++)
        for (a = 0; a < 3; a++) {
            double s = 0;
            for (b = 0; b < 3; b++) s += gref[3 * i + b] * Bi[3 * b + a];
            g[3 * i + a] = s;
        }
}

/* AssembleFE_Laplace::assemblyLaplacian (AssembleFE_Laplace_def.hpp:53-96)
 * and FE::assemblyLaplace (FE_def.hpp:2437-2500): K_ij = |detB| sum_q w_q
 * grad phi_i . grad phi_j.  npts is the rule the caller's degree selects. */
void orc_elem_laplace(int fe_order, int npts, const double *xe, double *K)
{
    const int n = fe_order == 1 ? 4 : 10;
    double pts[45], w[15], gref[30], g[30], B[9], Bi[9], det, adet;
    int q, i, j, d;
    det = orc_geometry(xe, xe + 3, xe + 6, xe + 9, B, Bi);
    adet = fabs(det);
    orc_quad(npts, pts, w);
    memset(K, 0, sizeof(double) * n * n);
    for (q = 0; q < npts; q++) {
        orc_dphi(fe_order, pts + 3 * q, gref);
        grad_phys(n, gref, Bi, g);
        for (i = 0; i < n; i++)
            for (j = 0; j < n; j++) {
                double s = 0;
                for (d = 0; d < 3; d++) s += g[3 * i + d] * g[3 * j + d];
                K[n * i + j] += w[q] * s;
            }
    }
    for (i = 0; i < n * n; i++) K[i] *= adet;
}

/* FE::assemblyRHS with a constant scalar source (FE_def.hpp:7303-7400):
 * b_i = |detB| sum_q w_q phi_i(q) f. */
void orc_elem_rhs_const(int fe_order, int npts, const double *xe, double f, double *b)
{
    const int n = fe_order == 1 ? 4 : 10;
    double pts[45], w[15], phi[10], det;
    int q, i;
    det = orc_geometry(xe, xe + 3, xe + 6, xe + 9, NULL, NULL);
    orc_quad(npts, pts, w);
    for (i = 0; i < n; i++) b[i] = 0;
    for (q = 0; q < npts; q++) {
        orc_phi(fe_order, pts + 3 * q, phi);
        for (i = 0; i < n; i++) b[i] += w[q] * phi[i] * f;
    }
    for (i = 0; i < n; i++) b[i] *= fabs(det);
}

/* AssembleFENavierStokes (AssembleFENavierStokes_def.hpp):
 *  A  assemblyLaplacian      :149-196  (15-point rule, dof-diagonal)
 *  N  assemblyAdvection      :227-298  (15-point rule, dof-diagonal)
 *  W  assemblyAdvectionInU   :301-369  (15-point rule, full 3x3 blocks)
 *  B  assemblyDivAndDivT     :373-461  (5-point rule, P1 pressure basis)
 *  J = nu*rho*A - B - B^T + rho*N (+ rho*W if Linearization != FixedPoint) :66-112
 *  res = (coeff .* ANB) x, ANB = nu*rho*A - B - B^T + rho*N             :199-224
 * Element dofs: 30 velocity (3*i+d, node-wise) then 4 pressure.
 * Optional outputs A, N, W, Bd (34x34 each) hold the unscaled parts. */
void orc_elem_ns(const double *xe, const double *u, const double *p, double visc, double dens,
                 int newton, const double *coeff, double *J, double *res, double *Ao, double *No,
                 double *Wo, double *Bo)
{
    enum { ND = 34 };
    double pts[45], w[15], gref[30], g[15][30], phi[15][10], Bm[9], Bi[9], det, adet;
    double A[100], N[100], W[900], Bd[120]; /* Bd[i][3j+d] = int psi_i d_d phi_j */
    double ul[15][3], du[15][9];
    double ANB[ND * ND];
    double x[ND];
    int q, i, j, d, d1, d2, k, nq;
    det = orc_geometry(xe, xe + 3, xe + 6, xe + 9, Bm, Bi);
    adet = fabs(det);
    nq = orc_quad(15, pts, w);
    for (q = 0; q < nq; q++) {
        orc_dphi(2, pts + 3 * q, gref);
        grad_phys(10, gref, Bi, g[q]);
        orc_phi(2, pts + 3 * q, phi[q]);
        for (d = 0; d < 3; d++) {
            double s = 0;
            for (k = 0; k < 10; k++) s += u[3 * k + d] * phi[q][k];
            ul[q][d] = s;
        }
        for (d1 = 0; d1 < 3; d1++)
            for (d2 = 0; d2 < 3; d2++) {
                double s = 0; /* du[q][d2][d1] = sum_k u_{k,d1} d_{d2} phi_k */
                for (k = 0; k < 10; k++) s += u[3 * k + d1] * g[q][3 * k + d2];
                du[q][3 * d2 + d1] = s;
            }
    }
    for (i = 0; i < 10; i++)
        for (j = 0; j < 10; j++) {
            double sa = 0, sn = 0;
            for (q = 0; q < nq; q++) {
                double gg = 0, ug = 0;
                for (d = 0; d < 3; d++) {
                    gg += g[q][3 * i + d] * g[q][3 * j + d];
                    ug += ul[q][d] * g[q][3 * j + d];
                }
                sa += w[q] * gg;
                sn += w[q] * ug * phi[q][i];
            }
            A[10 * i + j] = sa * adet;
            N[10 * i + j] = sn * adet;
            for (d1 = 0; d1 < 3; d1++)
                for (d2 = 0; d2 < 3; d2++) {
                    double s = 0;
                    for (q = 0; q < nq; q++) s += w[q] * du[q][3 * d2 + d1] * phi[q][i] * phi[q][j];
                    W[(3 * i + d1) * 30 + 3 * j + d2] = s * adet;
                }
        }
    /* divergence block with the 5-point rule */
    {
        double pts5[15], w5[5], psi[4], gr5[30], g5[30];
        int n5 = orc_quad(5, pts5, w5);
        memset(Bd, 0, sizeof Bd);
        for (q = 0; q < n5; q++) {
            orc_dphi(2, pts5 + 3 * q, gr5);
            grad_phys(10, gr5, Bi, g5);
            orc_phi(1, pts5 + 3 * q, psi);
            for (i = 0; i < 4; i++)
                for (j = 0; j < 10; j++)
                    for (d = 0; d < 3; d++) Bd[30 * i + 3 * j + d] += w5[q] * psi[i] * g5[3 * j + d];
        }
        for (i = 0; i < 120; i++) Bd[i] *= adet;
    }
    memset(ANB, 0, sizeof ANB);
    for (i = 0; i < 10; i++)
        for (j = 0; j < 10; j++)
            for (d = 0; d < 3; d++)
                ANB[(3 * i + d) * ND + 3 * j + d] = visc * dens * A[10 * i + j] + dens * N[10 * i + j];
    for (i = 0; i < 4; i++)
        for (k = 0; k < 30; k++) {
            ANB[(30 + i) * ND + k] -= Bd[30 * i + k];
            ANB[k * ND + 30 + i] -= Bd[30 * i + k];
        }
    if (J) {
        memcpy(J, ANB, sizeof ANB);
        if (newton)
            for (i = 0; i < 30; i++)
                for (j = 0; j < 30; j++) J[i * ND + j] += dens * W[30 * i + j];
    }
    if (res) {
        for (i = 0; i < 30; i++) x[i] = u[i];
        for (i = 0; i < 4; i++) x[30 + i] = p ? p[i] : 0.0;
        for (i = 0; i < ND; i++) {
            double s = 0;
            int si = i >= 30;
            for (j = 0; j < ND; j++) s += ANB[i * ND + j] * x[j] * coeff[2 * si + (j >= 30)];
            res[i] = s;
        }
    }
    if (Ao) {
        memset(Ao, 0, sizeof(double) * ND * ND);
        for (i = 0; i < 10; i++)
            for (j = 0; j < 10; j++)
                for (d = 0; d < 3; d++) Ao[(3 * i + d) * ND + 3 * j + d] = A[10 * i + j];
    }
    if (No) {
        memset(No, 0, sizeof(double) * ND * ND);
        for (i = 0; i < 10; i++)
            for (j = 0; j < 10; j++)
                for (d = 0; d < 3; d++) No[(3 * i + d) * ND + 3 * j + d] = N[10 * i + j];
    }
    if (Wo) {
        memset(Wo, 0, sizeof(double) * ND * ND);
        for (i = 0; i < 30; i++)
            for (j = 0; j < 30; j++) Wo[i * ND + j] = W[30 * i + j];
    }
    if (Bo) {
        memset(Bo, 0, sizeof(double) * ND * ND);
        for (i = 0; i < 4; i++)
            for (k = 0; k < 30; k++) {
                Bo[(30 + i) * ND + k] = Bd[30 * i + k];
                Bo[k * ND + 30 + i] = Bd[30 * i + k];
            }
    }
}

/* ---- generalized-Newtonian element ---------------------------------------- */
/* Viscosity laws: CarreauYasuda_def.hpp:25-57, PowerLaw_def.hpp:27-63,
 * Dimless_Carreau_def.hpp:26-43 (GeneralizedNewtonianModels).
 *
 * Those sources test abs(x) against small thresholds (the a = 2 branch of
 * Carreau-Yasuda: abs(a - 2) < DBL_EPSILON; the shear-rate floor:
 * abs(gamma) <= Numerical_ZeroValue_ShearRate).  Compiled with the headers
 * they include, that abs is the integer function, so the tests read
 * |trunc(x)|: the a = 2 formula is taken for every a in (1, 3), and every
 * shear rate below 1 is replaced by the floor.  Verified against the
 * reference compiled from its own sources; restated here as it computes. */
static double ref_abs_int(double x) { return fabs(trunc(x)); }

double orc_gn_eta(const orc_visc_law *L, double g)
{
    const double *c = L->prm;
    if (L->model == ORC_GN_CARREAU_YASUDA)
        return c[3] + (c[2] - c[3]) * pow(1.0 + pow(c[0] * g, c[4]), (c[1] - 1.0) / c[4]);
    if (L->model == ORC_GN_POWER_LAW) {
        double eta = c[0] * pow(g, c[1] - 1.0);
        if (eta < c[3])
            eta = c[3];
        else if (fabs(eta) > c[2])
            eta = c[2];
        return eta;
    }
    return c[4] * (c[3] + (c[2] - c[3]) * pow(1.0 + pow(c[0] * g, 2.0), (c[1] - 1.0) / 2.0));
}

double orc_gn_dterm(const orc_visc_law *L, double g)
{
    const double *c = L->prm;
    if (L->model == ORC_GN_CARREAU_YASUDA) {
        const double a = c[4];
        if (ref_abs_int(a - 2.0) < 2.220446049250313e-16)
            return -2.0 * (c[2] - c[3]) * (c[1] - 1.0) * pow(c[0], a) *
                   pow(1.0 + pow(c[0] * g, a), (c[1] - 1.0 - a) / a);
        if (ref_abs_int(g) <= L->gamma_min) g = L->gamma_min;
        return -2.0 * (c[2] - c[3]) * (c[1] - 1.0) * pow(c[0], a) * pow(g, a - 2.0) *
               pow(1.0 + pow(c[0] * g, a), (c[1] - 1.0 - a) / a);
    }
    if (L->model == ORC_GN_POWER_LAW) {
        if (ref_abs_int(g) <= L->gamma_min) g = L->gamma_min;
        return -2.0 * c[0] * (c[1] - 1.0) * pow(g, c[1] - 3.0);
    }
    return c[4] * (-2.0 * (c[2] - c[3]) * (c[1] - 1.0) * pow(c[0], 2) *
                   pow(1.0 + pow(c[0] * g, 2.0), (c[1] - 3.0) / 2.0));
}

/* velocity gradient du[a][b] = d u_a / d x_b at one point */
static void gn_velgrad(const double *u, const double *g, double du[3][3])
{
    int a, b, k;
    for (a = 0; a < 3; a++)
        for (b = 0; b < 3; b++) {
            double s = 0;
            for (k = 0; k < 10; k++) s += u[3 * k + a] * g[3 * k + b];
            du[a][b] = s;
        }
}

static double gn_shear_rate(double du[3][3])
{
    return sqrt(2.0 * du[0][0] * du[0][0] + 2.0 * du[1][1] * du[1][1] + 2.0 * du[2][2] * du[2][2] +
                (du[0][1] + du[1][0]) * (du[0][1] + du[1][0]) + (du[0][2] + du[2][0]) * (du[0][2] + du[2][0]) +
                (du[1][2] + du[2][1]) * (du[1][2] + du[2][1]));
}

/* AssembleFEGeneralizedNewtonian (feddlib/core/AceFemAssembly/specific/
 * AssembleFEGeneralizedNewtonian_def.hpp) without an outflow Neumann term:
 *   J   = -B - B^T + rho N + S(eta)  [+ D + rho W with Newton]      :72-170
 *   res = (-B - B^T + rho N + S(eta)) x                             :932-996
 * S (assemblyStress, :225-416, degree 3 -> 5-point rule):
 *   S_(ik)(jl) = |detB| sum_q w_q eta(gamma_q) (d_kl g_i.g_j + g_i,l g_j,k)
 * D (assemblyStressDev, :418-695, degree 4 -> 15-point rule):
 *   D_(ik)(jl) = |detB| sum_q w_q (-2 c_q) G_j^l F_i^k, c_q = -(2/gamma) deta/dgamma,
 *   F_i^k = row k of sym(grad u) contracted with g_i, and G_j^l the same for
 *   the column, except that the reference's third column factor reads
 *   g_j,3 * (du_13 + du_31)/2 where the symmetric gradient gives g_j,1 * ...;
 *   restated as the reference computes it.
 * gamma_q = sqrt(2 (u11^2 + u22^2 + u33^2) + (u12 + u21)^2 + (u13 + u31)^2
 *           + (u23 + u32)^2)  (computeShearRate, :998-1083). */
void orc_elem_gn(const double *xe, const double *u, const double *p, const orc_visc_law *L, double dens,
                 int newton, double *J, double *res)
{
    enum { ND = 34 };
    static const double ones[4] = {1, 1, 1, 1};
    double Jns[ND * ND], S[900], D[900], Bm[9], Bi[9], det, adet, x[ND];
    double pts[45], w[15], gref[30], g[30], du[3][3];
    int q, n, i, j, k, l;
    orc_elem_ns(xe, u, p, 0.0, dens, newton, ones, Jns, NULL, NULL, NULL, NULL, NULL);
    det = orc_geometry(xe, xe + 3, xe + 6, xe + 9, Bm, Bi);
    adet = fabs(det);
    memset(S, 0, sizeof S);
    memset(D, 0, sizeof D);
    n = orc_quad(5, pts, w);
    for (q = 0; q < n; q++) {
        double eta;
        orc_dphi(2, pts + 3 * q, gref);
        grad_phys(10, gref, Bi, g);
        gn_velgrad(u, g, du);
        eta = orc_gn_eta(L, gn_shear_rate(du));
        for (i = 0; i < 10; i++)
            for (j = 0; j < 10; j++) {
                const double gg = g[3 * i] * g[3 * j] + g[3 * i + 1] * g[3 * j + 1] + g[3 * i + 2] * g[3 * j + 2];
                for (k = 0; k < 3; k++)
                    for (l = 0; l < 3; l++)
                        S[(3 * i + k) * 30 + 3 * j + l] +=
                            eta * w[q] * ((k == l ? gg : 0.0) + g[3 * i + l] * g[3 * j + k]);
            }
    }
    if (newton) {
        n = orc_quad(15, pts, w);
        for (q = 0; q < n; q++) {
            double c, xy, xz, yz, F[30], G[30];
            orc_dphi(2, pts + 3 * q, gref);
            grad_phys(10, gref, Bi, g);
            gn_velgrad(u, g, du);
            c = orc_gn_dterm(L, gn_shear_rate(du));
            xy = 0.5 * (du[0][1] + du[1][0]);
            xz = 0.5 * (du[2][0] + du[0][2]);
            yz = 0.5 * (du[2][1] + du[1][2]);
            for (i = 0; i < 10; i++) {
                const double *gi = g + 3 * i;
                F[3 * i] = gi[0] * du[0][0] + gi[1] * xy + gi[2] * xz;
                F[3 * i + 1] = gi[0] * xy + gi[1] * du[1][1] + gi[2] * yz;
                F[3 * i + 2] = gi[0] * xz + gi[1] * yz + gi[2] * du[2][2];
                G[3 * i] = F[3 * i];
                G[3 * i + 1] = F[3 * i + 1];
                G[3 * i + 2] = gi[2] * xz + gi[1] * yz + gi[2] * du[2][2];
            }
            for (i = 0; i < 30; i++)
                for (j = 0; j < 30; j++) D[30 * i + j] += -2.0 * c * w[q] * G[j] * F[i];
        }
    }
    for (i = 0; i < 900; i++) {
        S[i] *= adet;
        D[i] *= adet;
    }
    for (i = 0; i < 30; i++)
        for (j = 0; j < 30; j++) Jns[i * ND + j] += S[30 * i + j];
    if (res) {
        /* ANB = J without the Newton terms: rebuild it from the FixedPoint NS part */
        double Afp[ND * ND];
        orc_elem_ns(xe, u, p, 0.0, dens, 0, ones, Afp, NULL, NULL, NULL, NULL, NULL);
        for (i = 0; i < 30; i++)
            for (j = 0; j < 30; j++) Afp[i * ND + j] += S[30 * i + j];
        for (i = 0; i < 30; i++) x[i] = u[i];
        for (i = 0; i < 4; i++) x[30 + i] = p ? p[i] : 0.0;
        for (i = 0; i < ND; i++) {
            double s = 0;
            for (j = 0; j < ND; j++) s += Afp[i * ND + j] * x[j];
            res[i] = s;
        }
    }
    if (J) {
        memcpy(J, Jns, sizeof Jns);
        if (newton)
            for (i = 0; i < 30; i++)
                for (j = 0; j < 30; j++) J[i * ND + j] += D[30 * i + j];
    }
}

/* The outflow Neumann boundary term of AssembleFEGeneralizedNewtonian
 * (assemblyOutflowNeumannBoundaryTerm, AssembleFEGeneralizedNewtonian_def.hpp:
 * 697-920) for one element whose flagged face has the vertex coordinates
 * face[0..8] (the face's own node order).  The surface data are those that
 * Domain::setSurfaceNormalsForFE (Domain_def.hpp:1148-1180) and
 * Domain::setSurfaceQuadraturePointsWeights(flag, 8) (:1214-1255) attach to a
 * P2 face in 3D:
 *   n   = unit((f0 - f1) x (f0 - f2))        (Helper::computeSurfaceNormal, Helper.cpp:161-194)
 *   s   = |(f1 - f0) x (f2 - f0)|            (Helper::buildTransformationSurface, SmallMatrix::computeScaling)
 *   x_q = the 7-point triangle rule in barycentric form, weights w_q
 *         (Helper::getQuadraturePointsOnSurfaceInGlobalSpace, Helper.cpp:1762-1893)
 * and the element maps each point back to its reference coordinates,
 * xi_q = B^-1 (x_q - x_0), to evaluate phi and its physical gradient there:
 *   K[(i,d)][(j,e)] = -s sum_q eta(gamma_q) w_q (d phi_j / d x_d)(xi_q) n_e phi_i(xi_q),
 * gamma_q from the element's velocity as in the stress term.  K (30 x 30,
 * row-major) enters the Jacobian (Newton and FixedPoint alike: its Newton
 * derivative is left out in the reference) and the residual's operator. */
void orc_gn_outflow(const double *xe, const double *face, const double *u, const orc_visc_law *L, double *K)
{
    static const double qa = 0.470142064105115, qb = 0.101286507323456;
    static const double wP1 = 0.066197076394253, wP2 = 0.062969590272413;
    const double lam[7][3] = {{1 / 3., 1 / 3., 1 / 3.},  {1 - 2 * qa, qa, qa}, {qa, 1 - 2 * qa, qa},
                              {qa, qa, 1 - 2 * qa},       {1 - 2 * qb, qb, qb}, {qb, 1 - 2 * qb, qb},
                              {qb, qb, 1 - 2 * qb}};
    const double wq[7] = {9 / 80., wP1, wP1, wP1, wP2, wP2, wP2};
    double B[9], Bi[9], p1[3], p2[3], n[3], c[3], nn, scale, gref[30], g[30], phi[10], du[3][3];
    int q, i, j, d, e, k;
    orc_geometry(xe, xe + 3, xe + 6, xe + 9, B, Bi);
    for (k = 0; k < 3; k++) {
        p1[k] = face[k] - face[3 + k];
        p2[k] = face[k] - face[6 + k];
    }
    n[0] = p1[1] * p2[2] - p1[2] * p2[1];
    n[1] = p1[2] * p2[0] - p1[0] * p2[2];
    n[2] = p1[0] * p2[1] - p1[1] * p2[0];
    nn = sqrt(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]);
    for (k = 0; k < 3; k++) n[k] /= nn;
    {
        double a[3], b[3];
        for (k = 0; k < 3; k++) {
            a[k] = face[3 + k] - face[k];
            b[k] = face[6 + k] - face[k];
        }
        c[0] = a[1] * b[2] - a[2] * b[1];
        c[1] = a[2] * b[0] - a[0] * b[2];
        c[2] = a[0] * b[1] - a[1] * b[0];
        scale = sqrt(c[0] * c[0] + c[1] * c[1] + c[2] * c[2]);
    }
    memset(K, 0, sizeof(double) * 900);
    for (q = 0; q < 7; q++) {
        double xg[3], xi[3], eta;
        for (k = 0; k < 3; k++)
            xg[k] = lam[q][0] * face[k] + lam[q][1] * face[3 + k] + lam[q][2] * face[6 + k];
        for (k = 0; k < 3; k++) {
            xi[k] = 0;
            for (d = 0; d < 3; d++) xi[k] += Bi[3 * k + d] * (xg[d] - xe[d]);
        }
        orc_phi(2, xi, phi);
        orc_dphi(2, xi, gref);
        grad_phys(10, gref, Bi, g);
        gn_velgrad(u, g, du);
        eta = orc_gn_eta(L, gn_shear_rate(du));
        for (i = 0; i < 10; i++)
            for (j = 0; j < 10; j++)
                for (d = 0; d < 3; d++)
                    for (e = 0; e < 3; e++)
                        K[(3 * i + d) * 30 + 3 * j + e] += -(eta * wq[q] * g[3 * j + d] * n[e] * phi[i]);
    }
    for (k = 0; k < 900; k++) K[k] *= scale;
}

/* FE::assemblyLinElasXDim (FE_def.hpp:4701-): K = |detB| sum_q w_q
 * [2 mu eps(phi_a e_i):eps(phi_b e_j) + lambda div div]; degree from
 * determineDegree(P2,P2,Grad,Grad) = 2 -> 5-point rule. */
void orc_elem_linelas_classic(int npts, const double *xe, double lambda, double mu, double *K)
{
    double pts[45], w[15], gref[30], g[30], B[9], Bi[9], det, adet;
    int q, a, b, i, j;
    det = orc_geometry(xe, xe + 3, xe + 6, xe + 9, B, Bi);
    adet = fabs(det);
    orc_quad(npts, pts, w);
    memset(K, 0, sizeof(double) * 900);
    for (q = 0; q < npts; q++) {
        orc_dphi(2, pts + 3 * q, gref);
        grad_phys(10, gref, Bi, g);
        for (a = 0; a < 10; a++)
            for (b = 0; b < 10; b++) {
                double gg = g[3 * a] * g[3 * b] + g[3 * a + 1] * g[3 * b + 1] + g[3 * a + 2] * g[3 * b + 2];
                for (i = 0; i < 3; i++)
                    for (j = 0; j < 3; j++)
                        K[(3 * a + i) * 30 + 3 * b + j] +=
                            adet * w[q] * (mu * ((i == j) * gg + g[3 * a + j] * g[3 * b + i]) +
                                           lambda * g[3 * a + i] * g[3 * b + j]);
            }
    }
}

/* ======================================================================== */
/* Hyperelastic laws as Psi(I1, J, I4a, I4b).                                */
/*  skr1 (AceInterface/NeoHookQuadraticTets.f:27-32, 481-483):              */
/*     Psi = mu/2 (I1-3) - mu lnJ + lambda/4 (J^2 - 1 - 2 lnJ)              */
/*     (P = mu F + (lambda J/2 - (lambda+2mu)/(2J)) cof F)                  */
/*  skr2 (NeoHookQuadraticTets2.f:28-30, 490-512):                          */
/*     Psi = mu/2 (I1-3) - mu lnJ + lambda/2 (lnJ)^2                        */
/*  skr3 (NeoHookQuadraticTets3.f:25-31, 491-496; v(208), v(214), v(561)    */
/*  are the derivatives with respect to I3 = J^2), "lambda" = kappa:        */
/*     Psi = mu/2 (J^-2/3 I1 - 3) + kappa/2 (J-1)^2,                        */
/*     mu = E/(2(1+nu)), kappa = E/(3(1-2nu))                               */
/*  aniso (no reference counterpart): skr1 matrix + two exponential fibre    */
/*     families, k1/(2 k2) (exp(k2 (I4-1)^2) - 1), active only for I4 > 1.   */
/*  mlp   (no reference counterpart): surrogate for the aniso law.          */
/* ======================================================================== */
static double sp_(double z) { return z > 30 ? z : log1p(exp(z)); }
static double sg_(double z) { return 1.0 / (1.0 + exp(-z)); }

void orc_mlp_eval(int H, const double *W1, const double *b1, const double *W2, const double *b2,
                  const double *w3, double b3, const double *x, double *y, double *g, double *h)
{
    double *z1 = malloc(sizeof(double) * H * 18), *h1 = z1 + H, *s1 = h1 + H, *t1 = s1 + H;
    double *dh1 = t1 + H /* 4H */, *d2h1 = dh1 + 4 * H /* 10H */;
    int i, j, k, l, kl;
    for (i = 0; i < H; i++) {
        double z = b1[i];
        for (k = 0; k < 4; k++) z += W1[4 * i + k] * x[k];
        z1[i] = z; h1[i] = sp_(z); s1[i] = sg_(z); t1[i] = s1[i] * (1 - s1[i]);
        for (k = 0; k < 4; k++) dh1[k * H + i] = s1[i] * W1[4 * i + k];
        kl = 0;
        for (k = 0; k < 4; k++)
            for (l = k; l < 4; l++, kl++) d2h1[kl * H + i] = t1[i] * W1[4 * i + k] * W1[4 * i + l];
    }
    {
        double yy = b3, gg[4] = {0, 0, 0, 0}, hh[10] = {0};
        for (j = 0; j < H; j++) {
            double z = b2[j], dz[4], d2z[10], s, t;
            for (k = 0; k < 4; k++) dz[k] = 0;
            for (kl = 0; kl < 10; kl++) d2z[kl] = 0;
            for (i = 0; i < H; i++) {
                double wji = W2[H * j + i];
                z += wji * h1[i];
                for (k = 0; k < 4; k++) dz[k] += wji * dh1[k * H + i];
                for (kl = 0; kl < 10; kl++) d2z[kl] += wji * d2h1[kl * H + i];
            }
            s = sg_(z); t = s * (1 - s);
            yy += w3[j] * sp_(z);
            for (k = 0; k < 4; k++) gg[k] += w3[j] * s * dz[k];
            kl = 0;
            for (k = 0; k < 4; k++)
                for (l = k; l < 4; l++, kl++) hh[kl] += w3[j] * (t * dz[k] * dz[l] + s * d2z[kl]);
        }
        *y = yy;
        if (g) for (k = 0; k < 4; k++) g[k] = gg[k];
        if (h) {
            kl = 0;
            for (k = 0; k < 4; k++)
                for (l = k; l < 4; l++, kl++) { h[4 * k + l] = hh[kl]; h[4 * l + k] = hh[kl]; }
        }
    }
    free(z1);
}

double orc_mlp_loss(int H, const double *W1, const double *b1, const double *W2, const double *b2,
                    const double *w3, double b3, int64_t n, const double *X, const double *tpsi,
                    const double *tgrad, double wpsi, double wgrad, double *gW1, double *gb1,
                    double *gW2, double *gb2, double *gw3, double *gb3)
{
    double *buf = malloc(sizeof(double) * H * 40);
    double *z1 = buf, *h1 = z1 + H, *s1 = h1 + H, *t1 = s1 + H, *dh1 = t1 + H; /* 4H */
    double *z2 = dh1 + 4 * H, *h2 = z2 + H, *s2 = h2 + H, *t2 = s2 + H, *dz2 = t2 + H; /* 4H */
    double *dlz2 = dz2 + 4 * H, *dldz2 = dlz2 + H /* 4H */, *dlh1 = dldz2 + 4 * H;
    double *dldh1 = dlh1 + H /* 4H */, *dlz1 = dldh1 + 4 * H;
    double loss = 0;
    int64_t s;
    int i, j, k;
    if (gW1) {
        memset(gW1, 0, sizeof(double) * 4 * H); memset(gb1, 0, sizeof(double) * H);
        memset(gW2, 0, sizeof(double) * H * H); memset(gb2, 0, sizeof(double) * H);
        memset(gw3, 0, sizeof(double) * H); *gb3 = 0;
    }
    for (s = 0; s < n; s++) {
        const double *x = X + 4 * s;
        double y = b3, g[4] = {0, 0, 0, 0}, ey, eg[4];
        for (i = 0; i < H; i++) {
            double z = b1[i];
            for (k = 0; k < 4; k++) z += W1[4 * i + k] * x[k];
            z1[i] = z; h1[i] = sp_(z); s1[i] = sg_(z); t1[i] = s1[i] * (1 - s1[i]);
            for (k = 0; k < 4; k++) dh1[k * H + i] = s1[i] * W1[4 * i + k];
        }
        for (j = 0; j < H; j++) {
            double z = b2[j];
            for (k = 0; k < 4; k++) dz2[k * H + j] = 0;
            for (i = 0; i < H; i++) {
                z += W2[H * j + i] * h1[i];
                for (k = 0; k < 4; k++) dz2[k * H + j] += W2[H * j + i] * dh1[k * H + i];
            }
            z2[j] = z; h2[j] = sp_(z); s2[j] = sg_(z); t2[j] = s2[j] * (1 - s2[j]);
            y += w3[j] * h2[j];
            for (k = 0; k < 4; k++) g[k] += w3[j] * s2[j] * dz2[k * H + j];
        }
        ey = 2 * wpsi * (y - tpsi[s]);
        loss += wpsi * (y - tpsi[s]) * (y - tpsi[s]);
        for (k = 0; k < 4; k++) {
            eg[k] = 2 * wgrad * (g[k] - tgrad[4 * s + k]);
            loss += wgrad * (g[k] - tgrad[4 * s + k]) * (g[k] - tgrad[4 * s + k]);
        }
        if (!gW1) continue;
        /* backward (derivation in the module docstring of the GPU trainer) */
        *gb3 += ey;
        for (j = 0; j < H; j++) {
            double a = ey * w3[j] * s2[j];
            gw3[j] += ey * h2[j];
            for (k = 0; k < 4; k++) {
                gw3[j] += eg[k] * s2[j] * dz2[k * H + j];
                a += eg[k] * w3[j] * t2[j] * dz2[k * H + j];
                dldz2[k * H + j] = eg[k] * w3[j] * s2[j];
            }
            dlz2[j] = a;
            gb2[j] += a;
        }
        for (j = 0; j < H; j++)
            for (i = 0; i < H; i++) {
                double gsum = dlz2[j] * h1[i];
                for (k = 0; k < 4; k++) gsum += dldz2[k * H + j] * dh1[k * H + i];
                gW2[H * j + i] += gsum;
            }
        for (i = 0; i < H; i++) {
            double a = 0;
            for (j = 0; j < H; j++) a += W2[H * j + i] * dlz2[j];
            dlh1[i] = a;
            for (k = 0; k < 4; k++) {
                double b = 0;
                for (j = 0; j < H; j++) b += W2[H * j + i] * dldz2[k * H + j];
                dldh1[k * H + i] = b;
            }
        }
        for (i = 0; i < H; i++) {
            double a = dlh1[i] * s1[i];
            for (k = 0; k < 4; k++) {
                a += dldh1[k * H + i] * t1[i] * W1[4 * i + k];
                gW1[4 * i + k] += dldh1[k * H + i] * s1[i];
            }
            dlz1[i] = a;
            gb1[i] += a;
            for (k = 0; k < 4; k++) gW1[4 * i + k] += a * x[k];
        }
    }
    free(buf);
    if (gW1 && n > 0) {
        double r = 1.0 / (double)n;
        for (i = 0; i < 4 * H; i++) gW1[i] *= r;
        for (i = 0; i < H; i++) { gb1[i] *= r; gb2[i] *= r; gw3[i] *= r; }
        for (i = 0; i < H * H; i++) gW2[i] *= r;
        *gb3 *= r;
    }
    return n > 0 ? loss / (double)n : 0.0;
}

void orc_law_invariants(const orc_law *L, const double *F, double *inv)
{
    double I1 = 0, J, fa[3], fb[3];
    int i, k;
    for (i = 0; i < 9; i++) I1 += F[i] * F[i];
    J = F[0] * (F[4] * F[8] - F[5] * F[7]) - F[1] * (F[3] * F[8] - F[5] * F[6]) +
        F[2] * (F[3] * F[7] - F[4] * F[6]);
    for (i = 0; i < 3; i++) {
        fa[i] = fb[i] = 0;
        for (k = 0; k < 3; k++) { fa[i] += F[3 * i + k] * L->a1[k]; fb[i] += F[3 * i + k] * L->a2[k]; }
    }
    inv[0] = I1; inv[1] = J;
    inv[2] = fa[0] * fa[0] + fa[1] * fa[1] + fa[2] * fa[2];
    inv[3] = fb[0] * fb[0] + fb[1] * fb[1] + fb[2] * fb[2];
}

/* psi and its derivatives with respect to (I1, J, I4a, I4b); d2 is 4x4 */
void orc_law_dpsi(const orc_law *L, const double *inv, double *psi, double *d1, double *d2)
{
    const double mu = L->mu, lam = L->lambda, I1 = inv[0], J = inv[1];
    double lnJ = log(J), P = 0;
    int k;
    for (k = 0; k < 4; k++) d1[k] = 0;
    for (k = 0; k < 16; k++) d2[k] = 0;
    if (L->law == ORC_LAW_SKR3) {
        const double j23 = pow(J, -2.0 / 3.0), j53 = j23 / J, j83 = j53 / J;
        P = 0.5 * mu * (j23 * I1 - 3) + 0.5 * lam * (J - 1) * (J - 1);
        d1[0] = 0.5 * mu * j23;
        d1[1] = -(mu / 3.0) * I1 * j53 + lam * (J - 1);
        d2[1] = d2[4] = -(mu / 3.0) * j53;
        d2[5] = (5.0 * mu / 9.0) * I1 * j83 + lam;
    } else if (L->law == ORC_LAW_SKR2) {
        P = 0.5 * mu * (I1 - 3) - mu * lnJ + 0.5 * lam * lnJ * lnJ;
        d1[0] = 0.5 * mu;
        d1[1] = (-mu + lam * lnJ) / J;
        d2[5] = (mu + lam - lam * lnJ) / (J * J);
    } else if (L->law == ORC_LAW_SKR1 || L->law == ORC_LAW_ANISO ||
               (L->law == ORC_LAW_MLP && L->mlp_add_matrix)) {
        P = 0.5 * mu * (I1 - 3) - mu * lnJ + 0.25 * lam * (J * J - 1 - 2 * lnJ);
        d1[0] = 0.5 * mu;
        d1[1] = -mu / J + 0.5 * lam * (J - 1 / J);
        d2[5] = mu / (J * J) + 0.5 * lam * (1 + 1 / (J * J));
    }
    if (L->law == ORC_LAW_ANISO) {
        for (k = 2; k < 4; k++) {
            double e = inv[k] - 1;
            if (e > 0) {
                double ex = exp(L->k2 * e * e);
                P += L->k1 / (2 * L->k2) * (ex - 1);
                d1[k] = L->k1 * e * ex;
                d2[5 * k] = L->k1 * ex * (1 + 2 * L->k2 * e * e);
            }
        }
    }
    if (L->law == ORC_LAW_MLP) {
        double x[4], y, g[4], h[16];
        int l;
        double dk[4], d2k[4];
        for (k = 0; k < 4; k++) {
            /* a clamped input enters squared and vanishes, with its
               derivatives, at or below its shift */
            double e = inv[k] - L->in_shift[k];
            if ((L->in_clamp >> k) & 1) {
                if (e > 0) {
                    x[k] = e * e * L->in_scale[k];
                    dk[k] = 2 * e * L->in_scale[k];
                    d2k[k] = 2 * L->in_scale[k];
                } else {
                    x[k] = dk[k] = d2k[k] = 0;
                }
            } else {
                x[k] = e * L->in_scale[k];
                dk[k] = L->in_scale[k];
                d2k[k] = 0;
            }
        }
        orc_mlp_eval(L->hidden, L->W1, L->b1, L->W2, L->b2, L->w3, L->b3, x, &y, g, h);
        P += L->out_scale * y;
        for (k = 0; k < 4; k++) {
            d1[k] += L->out_scale * g[k] * dk[k];
            for (l = 0; l < 4; l++)
                d2[4 * k + l] += L->out_scale * (h[4 * k + l] * dk[k] * dk[l] + (k == l ? g[k] * d2k[k] : 0));
        }
    }
    *psi = P;
}

/* First Piola P = dPsi/dF and A = d2Psi/dF dF (A[((i*3+k)*3+j)*3+l]). */
void orc_law_PA(const orc_law *L, const double *F, double *psi, double *P, double *A)
{
    double inv[4], d1[4], d2[16], cof[9], D[4][9], J, fa[3], fb[3];
    const double *af[2] = {L->a1, L->a2};
    int i, k, j, l, m, n;
    orc_law_invariants(L, F, inv);
    orc_law_dpsi(L, inv, psi, d1, d2);
    J = inv[1];
    cof[0] = F[4] * F[8] - F[5] * F[7]; cof[1] = F[5] * F[6] - F[3] * F[8]; cof[2] = F[3] * F[7] - F[4] * F[6];
    cof[3] = F[2] * F[7] - F[1] * F[8]; cof[4] = F[0] * F[8] - F[2] * F[6]; cof[5] = F[1] * F[6] - F[0] * F[7];
    cof[6] = F[1] * F[5] - F[2] * F[4]; cof[7] = F[2] * F[3] - F[0] * F[5]; cof[8] = F[0] * F[4] - F[1] * F[3];
    for (i = 0; i < 3; i++) {
        fa[i] = fb[i] = 0;
        for (k = 0; k < 3; k++) { fa[i] += F[3 * i + k] * L->a1[k]; fb[i] += F[3 * i + k] * L->a2[k]; }
    }
    for (i = 0; i < 3; i++)
        for (k = 0; k < 3; k++) {
            D[0][3 * i + k] = 2 * F[3 * i + k];
            D[1][3 * i + k] = cof[3 * i + k];
            D[2][3 * i + k] = 2 * fa[i] * L->a1[k];
            D[3][3 * i + k] = 2 * fb[i] * L->a2[k];
        }
    for (m = 0; m < 9; m++) {
        double s = 0;
        for (n = 0; n < 4; n++) s += d1[n] * D[n][m];
        P[m] = s;
    }
    if (!A) return;
    for (i = 0; i < 3; i++)
        for (k = 0; k < 3; k++)
            for (j = 0; j < 3; j++)
                for (l = 0; l < 3; l++) {
                    double s = 0;
                    int f;
                    for (m = 0; m < 4; m++)
                        for (n = 0; n < 4; n++) s += d2[4 * m + n] * D[m][3 * i + k] * D[n][3 * j + l];
                    if (i == j) s += d1[0] * 2.0 * (k == l);
                    s += d1[1] * (cof[3 * i + k] * cof[3 * j + l] - cof[3 * i + l] * cof[3 * j + k]) / J;
                    for (f = 0; f < 2; f++)
                        if (i == j) s += d1[2 + f] * 2.0 * af[f][k] * af[f][l];
                    A[((i * 3 + k) * 3 + j) * 3 + l] = s;
                }
}

/* Element tangent and residual with the conventions FEDDLib applies to the
 * AceGen kernels (AssembleFE_LinElas_def.hpp:117-121,167;
 * AssembleFE_NonLinElas_def.hpp:119,171-172): AceGen accumulates with the
 * signed isoparametric determinant of its (xi, eta, zeta, lambda0) map,
 * which is -det B for FEDDLib's node order (an odd permutation,
 * NeoHookQuadraticTets.f:132,584-586); FEDDLib negates and transposes s and
 * copies p.  Net result for an element with FEDDLib det B:
 *   K = det B sum_q w_q G_a A G_b,     r = -det B sum_q w_q P : G_a.
 * Geometry is affine (straight-edged P2), so G = B^-T grad_ref phi. */
void orc_elem_hyper(const orc_law *L, int npts, const double *xe, const double *u, double *K,
                    double *r)
{
    double pts[45], w[15], gref[30], g[30], Bm[9], Bi[9], det, F[9], P[9], A[81], psi;
    int q, a, b, i, j, k, l;
    det = orc_geometry(xe, xe + 3, xe + 6, xe + 9, Bm, Bi);
    orc_quad(npts, pts, w);
    if (K) memset(K, 0, sizeof(double) * 900);
    if (r) memset(r, 0, sizeof(double) * 30);
    for (q = 0; q < npts; q++) {
        orc_dphi(2, pts + 3 * q, gref);
        grad_phys(10, gref, Bi, g);
        for (i = 0; i < 3; i++)
            for (k = 0; k < 3; k++) {
                double s = (i == k);
                if (u)
                    for (a = 0; a < 10; a++) s += u[3 * a + i] * g[3 * a + k];
                F[3 * i + k] = s;
            }
        orc_law_PA(L, F, &psi, P, K ? A : NULL);
        if (r)
            for (a = 0; a < 10; a++)
                for (i = 0; i < 3; i++) {
                    double s = 0;
                    for (k = 0; k < 3; k++) s += P[3 * i + k] * g[3 * a + k];
                    r[3 * a + i] -= det * w[q] * s;
                }
        if (K)
            for (a = 0; a < 10; a++)
                for (b = 0; b < 10; b++)
                    for (i = 0; i < 3; i++)
                        for (j = 0; j < 3; j++) {
                            double s = 0;
                            for (k = 0; k < 3; k++)
                                for (l = 0; l < 3; l++)
                                    s += g[3 * a + k] * A[((i * 3 + k) * 3 + j) * 3 + l] * g[3 * b + l];
                            K[(3 * a + i) * 30 + 3 * b + j] += det * w[q] * s;
                        }
    }
}

/* ======================================================================== */
/* Global assembly with Tpetra semantics: insertGlobalValues accumulates,   */
/* fillComplete sorts columns ascending and sums duplicates, explicit zeros  */
/* stay (Matrix_def.hpp:86-91, FE_def.hpp:1419-1442, 982-1062).  Duplicates */
/* are summed in insertion (element) order.                                  */
/* ======================================================================== */
typedef struct { int64_t row, col, ord; } coo_key;
static int cmp_key(const void *a, const void *b)
{
    const coo_key *x = a, *y = b;
    if (x->row != y->row) return x->row < y->row ? -1 : 1;
    if (x->col != y->col) return x->col < y->col ? -1 : 1;
    return x->ord < y->ord ? -1 : (x->ord > y->ord);
}

int64_t orc_coo_to_csr(int64_t nrows, int64_t ncoo, const int64_t *rows, const int64_t *cols,
                       const double *vals, int64_t *rowptr, int32_t *colind, double *values)
{
    coo_key *k = malloc(sizeof(coo_key) * (ncoo > 0 ? ncoo : 1));
    int64_t i, nnz = 0, r;
    for (i = 0; i < ncoo; i++) { k[i].row = rows[i]; k[i].col = cols[i]; k[i].ord = i; }
    qsort(k, ncoo, sizeof(coo_key), cmp_key);
    for (r = 0; r <= nrows; r++) rowptr[r] = 0;
    for (i = 0; i < ncoo; i++) {
        if (i == 0 || k[i].row != k[i - 1].row || k[i].col != k[i - 1].col) {
            colind[nnz] = (int32_t)k[i].col;
            values[nnz] = vals[k[i].ord];
            rowptr[k[i].row + 1]++;
            nnz++;
        } else {
            values[nnz - 1] += vals[k[i].ord];
        }
    }
    for (r = 0; r < nrows; r++) rowptr[r + 1] += rowptr[r];
    free(k);
    return nnz;
}

static void gather_x(const double *xyz, const int32_t *c, int n, double *xe)
{
    int i, d;
    for (i = 0; i < n; i++)
        for (d = 0; d < 3; d++) xe[3 * i + d] = xyz[3 * (int64_t)c[i] + d];
}

/* FE::assemblyLaplace: row-wise insertGlobalValues (FE_def.hpp:2470-2490) */
int64_t orc_assemble_laplace_coo(int fe_order, int npts, int64_t ne, const double *xyz,
                                 const int32_t *conn, int64_t *rows, int64_t *cols, double *vals)
{
    const int n = fe_order == 1 ? 4 : 10;
    double xe[30], K[100];
    int64_t e, c = 0;
    int i, j;
    for (e = 0; e < ne; e++) {
        const int32_t *ce = conn + n * e;
        gather_x(xyz, ce, n, xe);
        orc_elem_laplace(fe_order, npts, xe, K);
        for (i = 0; i < n; i++)
            for (j = 0; j < n; j++) {
                rows[c] = ce[i]; cols[c] = ce[j]; vals[c] = K[n * i + j]; c++;
            }
    }
    return c;
}

/* FE::assemblyRHS, scalar field, constant f (FE_def.hpp:7303-7400) */
void orc_assemble_rhs(int fe_order, int npts, int64_t ne, const double *xyz, const int32_t *conn,
                      double f, double *rhs)
{
    const int n = fe_order == 1 ? 4 : 10;
    double xe[30], b[10];
    int64_t e;
    int i;
    for (e = 0; e < ne; e++) {
        const int32_t *ce = conn + n * e;
        gather_x(xyz, ce, n, xe);
        orc_elem_rhs_const(fe_order, npts, xe, f, b);
        for (i = 0; i < n; i++) rhs[ce[i]] += b[i];
    }
}

/* Vector-valued P2 problems through FE::addFeBlock (FE_def.hpp:1419-1442):
 * every dof pair of every node pair is inserted, zeros included.
 * kind 0: classic linear elasticity (lambda = L->lambda, mu = L->mu, 5-pt)
 * kind 1: hyperelastic law L with the rule npts (skr1: 4, skr2: 5)
 * Residual (kind 1) is scattered with addFeBlockMv (FE_def.hpp:630-640). */
int64_t orc_assemble_vec_coo(int kind, const orc_law *L, int npts, int64_t ne, const double *xyz,
                             const int32_t *conn, const double *u, int64_t *rows, int64_t *cols,
                             double *vals, double *res)
{
    double xe[30], ue[30], K[900], r[30];
    int64_t e, c = 0;
    int i, j, di, d;
    for (e = 0; e < ne; e++) {
        const int32_t *ce = conn + 10 * e;
        gather_x(xyz, ce, 10, xe);
        for (i = 0; i < 10; i++)
            for (d = 0; d < 3; d++) ue[3 * i + d] = u ? u[3 * (int64_t)ce[i] + d] : 0.0;
        if (kind == 0)
            orc_elem_linelas_classic(npts, xe, L->lambda, L->mu, K);
        else
            orc_elem_hyper(L, npts, xe, u ? ue : NULL, K, res ? r : NULL);
        if (rows)
            for (i = 0; i < 10; i++)
                for (di = 0; di < 3; di++)
                    for (d = 0; d < 3; d++)
                        for (j = 0; j < 10; j++) {
                            rows[c] = 3LL * ce[i] + di;
                            cols[c] = 3LL * ce[j] + d;
                            vals[c] = K[(3 * i + di) * 30 + 3 * j + d];
                            c++;
                        }
        if (res && kind == 1)
            for (i = 0; i < 10; i++)
                for (d = 0; d < 3; d++) res[3 * (int64_t)ce[i] + d] += r[3 * i + d];
    }
    return c;
}

/* FE::assemblyNavierStokes first assembly (reAssemble = false) through
 * addFeBlockMatrix (FE_def.hpp:982-1062) and the residual through
 * addFeBlockMv (FE_def.hpp:1381-1403).  block selects which COO is
 * returned: 0 -> (0,0), 1 -> (0,1), 2 -> (1,0), 3 -> (1,1) (|v| > 1e-13). */
int64_t orc_assemble_ns_coo(int64_t ne, const double *xyz, const int32_t *conn2,
                            const int32_t *conn1, const double *u, const double *p, double visc,
                            double dens, int newton, int block, int64_t *rows, int64_t *cols,
                            double *vals, double *res_u, double *res_p)
{
    static const double coeff[4] = {1, 1, 1, 1};
    double *J = malloc(sizeof(double) * 34 * 34), res[34], xe[30], ue[30], pe[4];
    int64_t e, c = 0;
    int i, j, di, d;
    for (e = 0; e < ne; e++) {
        const int32_t *c2 = conn2 + 10 * e, *c1 = conn1 + 4 * e;
        gather_x(xyz, c2, 10, xe);
        for (i = 0; i < 10; i++)
            for (d = 0; d < 3; d++) ue[3 * i + d] = u[3 * (int64_t)c2[i] + d];
        for (i = 0; i < 4; i++) pe[i] = p ? p[c1[i]] : 0.0;
        orc_elem_ns(xe, ue, pe, visc, dens, newton, coeff, J, res, NULL, NULL, NULL, NULL);
        if (rows) {
            if (block == 0)
                for (i = 0; i < 10; i++)
                    for (di = 0; di < 3; di++)
                        for (d = 0; d < 3; d++)
                            for (j = 0; j < 10; j++) {
                                rows[c] = 3LL * c2[i] + di; cols[c] = 3LL * c2[j] + d;
                                vals[c] = J[(3 * i + di) * 34 + 3 * j + d]; c++;
                            }
            if (block == 3)
                for (i = 0; i < 4; i++)
                    for (j = 0; j < 4; j++) {
                        double v = J[(30 + i) * 34 + 30 + j];
                        if (fabs(v) > 1e-13) { rows[c] = c1[i]; cols[c] = c1[j]; vals[c] = v; c++; }
                    }
            if (block == 1)
                for (i = 0; i < 10; i++)
                    for (di = 0; di < 3; di++)
                        for (j = 0; j < 4; j++) {
                            rows[c] = 3LL * c2[i] + di; cols[c] = c1[j];
                            vals[c] = J[(3 * i + di) * 34 + 30 + j]; c++;
                        }
            if (block == 2)
                for (j = 0; j < 4; j++)
                    for (d = 0; d < 3; d++)
                        for (i = 0; i < 10; i++) {
                            rows[c] = c1[j]; cols[c] = 3LL * c2[i] + d;
                            vals[c] = J[(30 + j) * 34 + 3 * i + d]; c++;
                        }
        }
        if (res_u)
            for (i = 0; i < 10; i++)
                for (d = 0; d < 3; d++) res_u[3 * (int64_t)c2[i] + d] += res[3 * i + d];
        if (res_p)
            for (i = 0; i < 4; i++) res_p[c1[i]] += res[30 + i];
    }
    free(J);
    return c;
}

/* ======================================================================== */
/* Reference-shaped CPU baseline for the Navier-Stokes Jacobian + residual.  */
/* Per element: rebuild quadrature/basis tables (Helper::getDPhi per call,   */
/* AssembleFENavierStokes_def.hpp:163,245), heap-allocate element matrices   */
/* (SmallMatrix per call, :69-75), insert row-wise into growable per-row     */
/* buffers (Tpetra dynamic profile), then sort + merge at "fillComplete".    */
/* Returns a checksum so the work cannot be optimised away.                  */
/* ======================================================================== */
typedef struct { int64_t *c; double *v; int64_t n, cap; } rowbuf;
static void rb_push(rowbuf *b, int64_t c, double v)
{
    if (b->n == b->cap) {
        b->cap = b->cap ? 2 * b->cap : 64;
        b->c = realloc(b->c, sizeof(int64_t) * b->cap);
        b->v = realloc(b->v, sizeof(double) * b->cap);
    }
    b->c[b->n] = c; b->v[b->n] = v; b->n++;
}
typedef struct { int64_t c; double v; int64_t o; } cv;
static int cmp_cv(const void *a, const void *b)
{
    const cv *x = a, *y = b;
    if (x->c != y->c) return x->c < y->c ? -1 : 1;
    return x->o < y->o ? -1 : (x->o > y->o);
}
static double fill_complete(rowbuf *rb, int64_t nrows)
{
    double chk = 0;
    int64_t r, i;
    for (r = 0; r < nrows; r++) {
        cv *t;
        int64_t m = 0;
        if (!rb[r].n) continue;
        t = malloc(sizeof(cv) * rb[r].n);
        for (i = 0; i < rb[r].n; i++) { t[i].c = rb[r].c[i]; t[i].v = rb[r].v[i]; t[i].o = i; }
        qsort(t, rb[r].n, sizeof(cv), cmp_cv);
        for (i = 0; i < rb[r].n; i++) {
            if (i && t[i].c == t[m - 1].c) t[m - 1].v += t[i].v;
            else t[m++] = t[i];
        }
        for (i = 0; i < m; i++) chk += t[i].v * (double)((i & 7) + 1);
        free(t);
        free(rb[r].c); free(rb[r].v);
        rb[r].c = NULL; rb[r].v = NULL; rb[r].n = rb[r].cap = 0;
    }
    return chk;
}
double orc_cpu_baseline_ns(int64_t ne, const double *xyz, const int32_t *conn2,
                           const int32_t *conn1, const double *u, const double *p, double visc,
                           double dens, int64_t nru, int64_t nrp)
{
    static const double coeff[4] = {1, 1, 1, 1};
    rowbuf *r00 = calloc(nru, sizeof(rowbuf)), *r01 = calloc(nru, sizeof(rowbuf));
    rowbuf *r10 = calloc(nrp, sizeof(rowbuf));
    double *resu = calloc(nru, sizeof(double)), *resp = calloc(nrp, sizeof(double)), chk = 0;
    int64_t e, r;
    int i, j, di, d;
    for (e = 0; e < ne; e++) {
        const int32_t *c2 = conn2 + 10 * e, *c1 = conn1 + 4 * e;
        double *xe = malloc(sizeof(double) * 30), *ue = malloc(sizeof(double) * 30);
        double *pe = malloc(sizeof(double) * 4), *J = malloc(sizeof(double) * 34 * 34);
        double *res = malloc(sizeof(double) * 34);
        double *Aw = malloc(sizeof(double) * 34 * 34 * 4);
        gather_x(xyz, c2, 10, xe);
        for (i = 0; i < 10; i++)
            for (d = 0; d < 3; d++) ue[3 * i + d] = u[3 * (int64_t)c2[i] + d];
        for (i = 0; i < 4; i++) pe[i] = p[c1[i]];
        /* Jacobian call, then the residual call recomputes the advection */
        orc_elem_ns(xe, ue, pe, visc, dens, 1, coeff, J, NULL, Aw, NULL, NULL, NULL);
        orc_elem_ns(xe, ue, pe, visc, dens, 0, coeff, NULL, res, NULL, NULL, NULL, NULL);
        for (i = 0; i < 10; i++)
            for (di = 0; di < 3; di++) {
                int64_t row = 3LL * c2[i] + di;
                for (d = 0; d < 3; d++)
                    for (j = 0; j < 10; j++) rb_push(&r00[row], 3LL * c2[j] + d, J[(3 * i + di) * 34 + 3 * j + d]);
                for (j = 0; j < 4; j++) rb_push(&r01[row], c1[j], J[(3 * i + di) * 34 + 30 + j]);
            }
        for (j = 0; j < 4; j++)
            for (d = 0; d < 3; d++)
                for (i = 0; i < 10; i++) rb_push(&r10[c1[j]], 3LL * c2[i] + d, J[(30 + j) * 34 + 3 * i + d]);
        for (i = 0; i < 30; i++) resu[3 * (int64_t)c2[i / 3] + i % 3] += res[i];
        for (i = 0; i < 4; i++) resp[c1[i]] += res[30 + i];
        free(xe); free(ue); free(pe); free(J); free(res); free(Aw);
    }
    chk += fill_complete(r00, nru) + fill_complete(r01, nru) + fill_complete(r10, nrp);
    for (r = 0; r < nru; r++) chk += resu[r];
    for (r = 0; r < nrp; r++) chk += resp[r];
    free(r00); free(r01); free(r10); free(resu); free(resp);
    return chk;
}

/* Seeded input fields (same stream as the engine's generator, so the CPU
 * reference arm assembles the very same inputs): sum of 8 Fourier modes
 * a_m sin(2 pi k_m.x + phi_m), k_m in {kmin..kmax}^3, |a_m| = 1, and
 * uniform values in [lo, hi). */
void orc_field_fourier(uint64_t seed, int kmin, int kmax, int64_t n, const double *xyz, double scale, double *u)
{
    uint64_t st = seed;
    double K[8][3], A[8][3], PH[8];
    const double pi = 3.14159265358979323846;
    int m, d;
    int64_t i;
    for (m = 0; m < 8; m++) {
        double nr = 0;
        for (d = 0; d < 3; d++) K[m][d] = kmin + (int)(u01(&st) * (kmax - kmin + 1));
        for (d = 0; d < 3; d++) { A[m][d] = 2.0 * u01(&st) - 1.0; nr += A[m][d] * A[m][d]; }
        nr = sqrt(nr > 0 ? nr : 1.0);
        for (d = 0; d < 3; d++) A[m][d] /= nr;
        PH[m] = 2.0 * pi * u01(&st);
    }
    for (i = 0; i < n; i++) {
        const double *x = xyz + 3 * i;
        double v[3] = {0, 0, 0};
        for (m = 0; m < 8; m++) {
            double sn = sin(2.0 * pi * (K[m][0] * x[0] + K[m][1] * x[1] + K[m][2] * x[2]) + PH[m]);
            for (d = 0; d < 3; d++) v[d] += A[m][d] * sn;
        }
        for (d = 0; d < 3; d++) u[3 * i + d] = scale * v[d];
    }
}

void orc_field_uniform(uint64_t seed, int64_t n, double lo, double hi, double *v)
{
    uint64_t st = seed;
    int64_t i;
    for (i = 0; i < n; i++) v[i] = lo + (hi - lo) * u01(&st);
}

/* ======================================================================== */
/* Rows at full mesh size.  A row of a global block is the sum, over the     */
/* elements incident to the row's node, of that node's rows of the element   */
/* matrix: the element loop of FE::assembly* (FE_def.hpp:1153-1213 for       */
/* Navier-Stokes, 362-434 / 449-523 for elasticity), addFeBlock /            */
/* addFeBlockMatrix inserting every dof pair of every node pair              */
/* (FE_def.hpp:1419-1442, 982-1062) and Tpetra's fillComplete summing the    */
/* duplicates of sorted columns (Matrix_def.hpp:86-91).  The functions below */
/* rebuild the complete rows of chosen nodes from all of their incident      */
/* elements (ascending element order, FP64), and check a whole CSR pattern   */
/* node by node, without assembling the rest of the mesh: that is what       */
/* parity at the configurations' full sizes needs.                           */
/* ======================================================================== */

/* node -> incident elements, ascending element id per node */
void orc_node_elements(int64_t ne, const int32_t *conn, int npe, int64_t nn, int64_t *ptr, int64_t *elems)
{
    int64_t e, n, *cur = calloc(nn + 1, sizeof(int64_t));
    int a;
    memset(ptr, 0, sizeof(int64_t) * (nn + 1));
    for (e = 0; e < ne; e++)
        for (a = 0; a < npe; a++) ptr[conn[npe * e + a] + 1]++;
    for (n = 0; n < nn; n++) ptr[n + 1] += ptr[n];
    for (e = 0; e < ne; e++)
        for (a = 0; a < npe; a++) {
            int64_t node = conn[npe * e + a];
            elems[ptr[node] + cur[node]++] = e;
        }
    free(cur);
}

static int cmp_i64(const void *a, const void *b)
{
    int64_t x = *(const int64_t *)a, y = *(const int64_t *)b;
    return (x > y) - (x < y);
}

/* sorted unique column nodes of the elements elems[0..m): returns K */
static int col_union(const int64_t *elems, int m, const int32_t *conn, int npe, int64_t *buf)
{
    int k, a, K = 0;
    for (k = 0; k < m; k++)
        for (a = 0; a < npe; a++) buf[k * npe + a] = conn[(int64_t)npe * elems[k] + a];
    qsort(buf, (size_t)m * npe, sizeof(int64_t), cmp_i64);
    for (k = 0; k < m * npe; k++)
        if (K == 0 || buf[k] != buf[K - 1]) buf[K++] = buf[k];
    return K;
}

static int find_col(const int64_t *cols, int K, int64_t c)
{
    int lo = 0, hi = K - 1;
    while (lo <= hi) {
        int mid = (lo + hi) / 2;
        if (cols[mid] == c) return mid;
        if (cols[mid] < c) lo = mid + 1; else hi = mid - 1;
    }
    return -1;
}

/* Checks a CSR block whose rows are (row node, dr < dofs_r) and columns
 * (column node, dc < dofs_c), node-wise numbering, against the node
 * adjacency through the elements (the pattern addFeBlock* + fillComplete
 * produce).  Returns -1 when every row matches, else the first row that
 * differs. */
int64_t orc_check_block_pattern(int64_t ne, const int32_t *row_conn, int npe_r, const int32_t *col_conn,
                                int npe_c, int64_t nrow_nodes, const int64_t *node_ptr, const int64_t *node_elems,
                                int dofs_r, int dofs_c, const int64_t *rowptr, const int32_t *colind)
{
    int64_t n, bad = -1;
    int64_t *buf = malloc(sizeof(int64_t) * 64 * 16 * 16);
    (void)ne; (void)row_conn; (void)npe_r;
    if (rowptr[0] != 0) { free(buf); return 0; }
    for (n = 0; n < nrow_nodes && bad < 0; n++) {
        int m = (int)(node_ptr[n + 1] - node_ptr[n]), K, k, dr, dc;
        if (m > 64 * 16 * 16 / npe_c) { bad = (int64_t)dofs_r * n; break; }
        K = col_union(node_elems + node_ptr[n], m, col_conn, npe_c, buf);
        for (dr = 0; dr < dofs_r && bad < 0; dr++) {
            int64_t r = (int64_t)dofs_r * n + dr, o = rowptr[r];
            if (rowptr[r + 1] - o != (int64_t)K * dofs_c) { bad = r; break; }
            for (k = 0; k < K && bad < 0; k++)
                for (dc = 0; dc < dofs_c; dc++)
                    if ((int64_t)colind[o + (int64_t)k * dofs_c + dc] != buf[k] * dofs_c + dc) { bad = r; break; }
        }
    }
    free(buf);
    return bad;
}

/* Elasticity rows (kind 0: classic linear elasticity with (lambda, mu) from
 * L; kind 1: the hyperelastic law L at displacement u) of the nodes sel[]:
 * per node k, cols[k * kmax + s] = column node of slot s (sorted, -1 beyond
 * its count), vals[((k * 3 + di) * kmax + s) * 3 + d] = value of row
 * 3 n + di, column 3 cols[s] + d; res[3 k + di] = residual entry (kind 1).
 * Returns 0, or -1 when a node has more than kmax columns. */
int orc_rows_vec(int kind, const orc_law *L, int npts, int64_t ne, const double *xyz, const int32_t *conn,
                 const double *u, const int64_t *node_ptr, const int64_t *node_elems, int64_t nsel,
                 const int64_t *sel, int kmax, int64_t *cols, double *vals, double *res)
{
    double xe[30], ue[30], K[900], r[30];
    int64_t *buf = malloc(sizeof(int64_t) * 64 * 10);
    int64_t k;
    int rc = 0;
    memset(vals, 0, sizeof(double) * nsel * 9 * kmax);
    if (res) memset(res, 0, sizeof(double) * nsel * 3);
    for (k = 0; k < nsel && rc == 0; k++) {
        const int64_t n = sel[k], *E = node_elems + node_ptr[n];
        const int m = (int)(node_ptr[n + 1] - node_ptr[n]);
        int s, t, a, b, di, d, Kc;
        if (m > 64) { rc = -1; break; }
        Kc = col_union(E, m, conn, 10, buf);
        if (Kc > kmax) { rc = -1; break; }
        for (s = 0; s < kmax; s++) cols[k * kmax + s] = s < Kc ? buf[s] : -1;
        for (t = 0; t < m; t++) {
            const int32_t *ce = conn + 10 * E[t];
            int i;
            gather_x(xyz, ce, 10, xe);
            for (i = 0; i < 10; i++)
                for (d = 0; d < 3; d++) ue[3 * i + d] = u ? u[3 * (int64_t)ce[i] + d] : 0.0;
            if (kind == 0)
                orc_elem_linelas_classic(npts, xe, L->lambda, L->mu, K);
            else
                orc_elem_hyper(L, npts, xe, u ? ue : NULL, K, r);
            for (a = 0; a < 10; a++) {
                if (ce[a] != n) continue;
                for (b = 0; b < 10; b++) {
                    const int slot = find_col(buf, Kc, ce[b]);
                    for (di = 0; di < 3; di++)
                        for (d = 0; d < 3; d++)
                            vals[((k * 3 + di) * kmax + slot) * 3 + d] += K[(3 * a + di) * 30 + 3 * b + d];
                }
                if (res && kind == 1)
                    for (di = 0; di < 3; di++) res[3 * k + di] += r[3 * a + di];
            }
        }
    }
    free(buf);
    return rc;
}

/* Navier-Stokes rows (FE::assemblyNavierStokes, first assembly): velocity
 * row nodes vsel[] give block (0,0) rows (cols00/vals00 as in orc_rows_vec,
 * P2 column nodes), block (0,1) rows (cols01[k * kpmax + s] = P1 column
 * node, vals01[(k * 3 + di) * kpmax + s]) and the velocity residual
 * res_u[3 k + di]; pressure row nodes psel[] give block (1,0) rows
 * (cols10 as cols00, vals10[(k * kmax + s) * 3 + d]) and the pressure
 * residual res_p[k].  ptr2/el2 and ptr1/el1: incident elements of the P2
 * and the P1 nodes.  Returns 0, or -1 when a node exceeds kmax / kpmax. */
static int rows_ns_impl(const double *xyz, const int32_t *conn2, const int32_t *conn1, const double *u,
                        const double *p, double visc, double dens, int newton, const orc_visc_law *L,
                        const int64_t *ptr2, const int64_t *el2, const int64_t *ptr1, const int64_t *el1, int64_t nv,
                        const int64_t *vsel, int64_t np, const int64_t *psel, int kmax, int kpmax, int64_t *cols00,
                        double *vals00, int64_t *cols01, double *vals01, double *res_u, int64_t *cols10,
                        double *vals10, double *res_p);

int orc_rows_ns(int64_t ne, const double *xyz, const int32_t *conn2, const int32_t *conn1, const double *u,
                const double *p, double visc, double dens, int newton, const int64_t *ptr2, const int64_t *el2,
                const int64_t *ptr1, const int64_t *el1, int64_t nv, const int64_t *vsel, int64_t np,
                const int64_t *psel, int kmax, int kpmax, int64_t *cols00, double *vals00, int64_t *cols01,
                double *vals01, double *res_u, int64_t *cols10, double *vals10, double *res_p)
{
    (void)ne;
    return rows_ns_impl(xyz, conn2, conn1, u, p, visc, dens, newton, NULL, ptr2, el2, ptr1, el1, nv, vsel, np, psel,
                        kmax, kpmax, cols00, vals00, cols01, vals01, res_u, cols10, vals10, res_p);
}

/* the same complete rows for the generalized-Newtonian element (orc_elem_gn,
 * no outflow term) with viscosity law L */
int orc_rows_gn(int64_t ne, const double *xyz, const int32_t *conn2, const int32_t *conn1, const double *u,
                const double *p, const orc_visc_law *L, double dens, int newton, const int64_t *ptr2,
                const int64_t *el2, const int64_t *ptr1, const int64_t *el1, int64_t nv, const int64_t *vsel,
                int64_t np, const int64_t *psel, int kmax, int kpmax, int64_t *cols00, double *vals00,
                int64_t *cols01, double *vals01, double *res_u, int64_t *cols10, double *vals10, double *res_p)
{
    (void)ne;
    return rows_ns_impl(xyz, conn2, conn1, u, p, 0.0, dens, newton, L, ptr2, el2, ptr1, el1, nv, vsel, np, psel,
                        kmax, kpmax, cols00, vals00, cols01, vals01, res_u, cols10, vals10, res_p);
}

static int rows_ns_impl(const double *xyz, const int32_t *conn2, const int32_t *conn1, const double *u,
                        const double *p, double visc, double dens, int newton, const orc_visc_law *L,
                        const int64_t *ptr2, const int64_t *el2, const int64_t *ptr1, const int64_t *el1, int64_t nv,
                        const int64_t *vsel, int64_t np, const int64_t *psel, int kmax, int kpmax, int64_t *cols00,
                        double *vals00, int64_t *cols01, double *vals01, double *res_u, int64_t *cols10,
                        double *vals10, double *res_p)
{
    static const double coeff[4] = {1, 1, 1, 1};
    double *J = malloc(sizeof(double) * 34 * 34), res[34], xe[30], ue[30], pe[4];
    int64_t *buf = malloc(sizeof(int64_t) * 64 * 10), *pbuf = malloc(sizeof(int64_t) * 64 * 4);
    int64_t k;
    int rc = 0;
    memset(vals00, 0, sizeof(double) * nv * 9 * kmax);
    memset(vals01, 0, sizeof(double) * nv * 3 * kpmax);
    memset(res_u, 0, sizeof(double) * nv * 3);
    memset(vals10, 0, sizeof(double) * np * 3 * kmax);
    memset(res_p, 0, sizeof(double) * np);
    for (k = 0; k < nv + np && rc == 0; k++) {
        const int vel = k < nv;
        const int64_t n = vel ? vsel[k] : psel[k - nv];
        const int64_t *E = vel ? el2 + ptr2[n] : el1 + ptr1[n];
        const int m = (int)(vel ? ptr2[n + 1] - ptr2[n] : ptr1[n + 1] - ptr1[n]);
        const int64_t kk = vel ? k : k - nv;
        int s, t, a, b, di, d, Kc, Kp = 0;
        if (m > 64) { rc = -1; break; }
        Kc = col_union(E, m, conn2, 10, buf);
        if (Kc > kmax) { rc = -1; break; }
        if (vel) {
            Kp = col_union(E, m, conn1, 4, pbuf);
            if (Kp > kpmax) { rc = -1; break; }
            for (s = 0; s < kmax; s++) cols00[kk * kmax + s] = s < Kc ? buf[s] : -1;
            for (s = 0; s < kpmax; s++) cols01[kk * kpmax + s] = s < Kp ? pbuf[s] : -1;
        } else {
            for (s = 0; s < kmax; s++) cols10[kk * kmax + s] = s < Kc ? buf[s] : -1;
        }
        for (t = 0; t < m; t++) {
            const int32_t *c2 = conn2 + 10 * E[t], *c1 = conn1 + 4 * E[t];
            int i;
            gather_x(xyz, c2, 10, xe);
            for (i = 0; i < 10; i++)
                for (d = 0; d < 3; d++) ue[3 * i + d] = u[3 * (int64_t)c2[i] + d];
            for (i = 0; i < 4; i++) pe[i] = p ? p[c1[i]] : 0.0;
            if (L)
                orc_elem_gn(xe, ue, pe, L, dens, newton, J, res);
            else
                orc_elem_ns(xe, ue, pe, visc, dens, newton, coeff, J, res, NULL, NULL, NULL, NULL);
            if (vel) {
                for (a = 0; a < 10; a++) {
                    if (c2[a] != n) continue;
                    for (b = 0; b < 10; b++) {
                        const int slot = find_col(buf, Kc, c2[b]);
                        for (di = 0; di < 3; di++)
                            for (d = 0; d < 3; d++)
                                vals00[((kk * 3 + di) * kmax + slot) * 3 + d] += J[(3 * a + di) * 34 + 3 * b + d];
                    }
                    for (b = 0; b < 4; b++) {
                        const int slot = find_col(pbuf, Kp, c1[b]);
                        for (di = 0; di < 3; di++)
                            vals01[(kk * 3 + di) * kpmax + slot] += J[(3 * a + di) * 34 + 30 + b];
                    }
                    for (di = 0; di < 3; di++) res_u[3 * kk + di] += res[3 * a + di];
                }
            } else {
                for (a = 0; a < 4; a++) {
                    if (c1[a] != n) continue;
                    for (b = 0; b < 10; b++) {
                        const int slot = find_col(buf, Kc, c2[b]);
                        for (d = 0; d < 3; d++) vals10[(kk * kmax + slot) * 3 + d] += J[(30 + a) * 34 + 3 * b + d];
                    }
                    res_p[kk] += res[30 + a];
                }
            }
        }
    }
    free(J); free(buf); free(pbuf);
    return rc;
}

/* Reference-shaped CPU baseline for the elasticity problems:
 * FE::assemblyLinearElasticity (FE_def.hpp:362-434, Jacobian only: one
 * kernel call per element, AssembleFE_LinElas_def.hpp:109) and
 * FE::assemblyNonLinearElasticity (FE_def.hpp:449-523: assembleJacobian and
 * assembleRHS each call the kernel, AssembleFE_NonLinElas_def.hpp:109,168).
 * Per element: heap copies of coordinates and displacements (the element
 * object, FE_def.hpp:1455-1474), heap element matrices, 90 row inserts of 10
 * values (addFeBlock, FE_def.hpp:1419-1442) into growable per-row buffers,
 * the residual through addFeBlockMv; fillComplete sorts and merges.  Returns
 * a checksum. */
double orc_cpu_baseline_vec(const orc_law *L, int npts, int64_t ne, const double *xyz, const int32_t *conn,
                            const double *u, int want_res, int64_t nrows)
{
    rowbuf *rb = calloc(nrows, sizeof(rowbuf));
    double *res = calloc(nrows, sizeof(double)), chk = 0;
    int64_t e, r;
    int i, j, di, d;
    for (e = 0; e < ne; e++) {
        const int32_t *ce = conn + 10 * e;
        double *xe = malloc(sizeof(double) * 30), *ue = malloc(sizeof(double) * 30);
        double *K = malloc(sizeof(double) * 900), *re = malloc(sizeof(double) * 30);
        gather_x(xyz, ce, 10, xe);
        for (i = 0; i < 10; i++)
            for (d = 0; d < 3; d++) ue[3 * i + d] = u ? u[3 * (int64_t)ce[i] + d] : 0.0;
        orc_elem_hyper(L, npts, xe, ue, K, NULL);                  /* assembleJacobian */
        if (want_res) orc_elem_hyper(L, npts, xe, ue, NULL, re);    /* assembleRHS      */
        for (i = 0; i < 10; i++)
            for (di = 0; di < 3; di++) {
                const int64_t row = 3LL * ce[i] + di;
                for (d = 0; d < 3; d++)
                    for (j = 0; j < 10; j++) rb_push(&rb[row], 3LL * ce[j] + d, K[(3 * i + di) * 30 + 3 * j + d]);
            }
        if (want_res)
            for (i = 0; i < 30; i++) res[3 * (int64_t)ce[i / 3] + i % 3] += re[i];
        free(xe); free(ue); free(K); free(re);
    }
    chk += fill_complete(rb, nrows);
    for (r = 0; r < nrows; r++) chk += res[r];
    free(rb); free(res);
    return chk;
}

/* min / max of det F over the quadrature points (npts-point rule) of the
 * elements [0, ne) for displacement u (3 per node): the CPU side of the
 * hyperelastic field bisection (det F kept in [0.7, 1.4]). */
void orc_detF_range(int npts, int64_t ne, const double *xyz, const int32_t *conn, const double *u,
                    double *jmin, double *jmax)
{
    double pts[45], w[15], gref[30], g[30], Bm[9], Bi[9], xe[30], F[9], lo = 1e300, hi = -1e300;
    int64_t e;
    int q, a, i, k;
    orc_quad(npts, pts, w);
    for (e = 0; e < ne; e++) {
        const int32_t *ce = conn + 10 * e;
        gather_x(xyz, ce, 10, xe);
        orc_geometry(xe, xe + 3, xe + 6, xe + 9, Bm, Bi);
        for (q = 0; q < npts; q++) {
            double J;
            orc_dphi(2, pts + 3 * q, gref);
            grad_phys(10, gref, Bi, g);
            for (i = 0; i < 3; i++)
                for (k = 0; k < 3; k++) {
                    double s = (i == k);
                    for (a = 0; a < 10; a++) s += u[3 * (int64_t)ce[a] + i] * g[3 * a + k];
                    F[3 * i + k] = s;
                }
            J = F[0] * (F[4] * F[8] - F[5] * F[7]) - F[1] * (F[3] * F[8] - F[5] * F[6]) +
                F[2] * (F[3] * F[7] - F[4] * F[6]);
            if (J < lo) lo = J;
            if (J > hi) hi = J;
        }
    }
    *jmin = lo;
    *jmax = hi;
}
