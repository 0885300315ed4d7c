// tables.cpp -- quadrature rules, P1/P2 bases and the Navier-Stokes reference
// tensors, evaluated once on the host in FP64.
//
// Rules follow Helper::getQuadratureValues (feddlib/core/FE/Helper.cpp:
// 1310-1317 one point, 1319-1350 five points, 1423-1517 fifteen points) and
// the AceGen 4-point rule, integration code 18
// (feddlib/core/AceFemAssembly/AceInterface/SMSUtility.f:344-352).  Bases
// follow Helper::phi / Helper::gradPhi (Helper.cpp:503-590, 703-745), local
// P2 order 0-3 vertices, 4=e01, 5=e12, 6=e02, 7=e03, 8=e13, 9=e23.
#include <cmath>
#include <cstring>

#include "engine.hpp"

namespace fedd {

Rule make_rule(int npts) {
    Rule r;
    auto set = [&](int i, double x, double y, double z, double w) {
        r.pts[i][0] = x; r.pts[i][1] = y; r.pts[i][2] = z; r.w[i] = w;
    };
    if (npts == 1) {
        r.n = 1;
        set(0, 0.25, 0.25, 0.25, 1.0 / 6.0);
    } else if (npts == 4) {
        const double a = 0.585410196624968454, b = 0.138196601125010515;
        r.n = 4;
        set(0, a, b, b, 1.0 / 24); set(1, b, a, b, 1.0 / 24);
        set(2, b, b, a, 1.0 / 24); set(3, b, b, b, 1.0 / 24);
    } else if (npts == 5) {
        const double a = 0.25, b = 1.0 / 6.0, c = 0.5;
        r.n = 5;
        set(0, a, a, a, -2.0 / 15.0);
        set(1, b, b, b, 3.0 / 40.0); set(2, b, b, c, 3.0 / 40.0);
        set(3, b, c, b, 3.0 / 40.0); set(4, c, b, b, 3.0 / 40.0);
    } else if (npts == 15) {
        const double s = std::sqrt(15.0);
        const double a = 0.25, b1 = (7. + s) / 34., b2 = (7. - s) / 34.;
        const double c1 = (13. - 3. * s) / 34., c2 = (13. + 3. * s) / 34.;
        const double d = (5. - s) / 20., e = (5. + s) / 20.;
        const double P1 = (2665. - 14. * s) / 226800., P2 = (2665. + 14. * s) / 226800., W3 = 5. / 567.;
        r.n = 15;
        set(0, a, a, a, 8. / 405.);
        set(1, b1, b1, b1, P1); set(2, b1, b1, c1, P1); set(3, b1, c1, b1, P1); set(4, c1, b1, b1, P1);
        set(5, b2, b2, b2, P2); set(6, b2, b2, c2, P2); set(7, b2, c2, b2, P2); set(8, c2, b2, b2, P2);
        set(9, d, d, e, W3); set(10, d, e, d, W3); set(11, e, d, d, W3);
        set(12, d, e, e, W3); set(13, e, d, e, W3); set(14, e, e, d, W3);
    }
    return r;
}

void basis_phi(int order, const double *p, double *v) {
    const double x = p[0], y = p[1], z = p[2], l = 1.0 - x - y - z;
    if (order == 1) {
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

void basis_dphi(int order, const double *p, double *g) {
    const double x = p[0], y = p[1], z = p[2];
    if (order == 1) {
        const double G[12] = {-1, -1, -1, 1, 0, 0, 0, 1, 0, 0, 0, 1};
        std::memcpy(g, G, sizeof G);
        return;
    }
    const double t = -3. + 4. * x + 4. * y + 4. * z;
    const double G[30] = {t, t, t,
                          4. * x - 1, 0., 0.,
                          0., 4. * y - 1, 0.,
                          0., 0., 4. * z - 1,
                          4. - 8. * x - 4. * y - 4. * z, -4. * x, -4. * x,
                          4. * y, 4. * x, 0.,
                          -4. * y, 4. - 4. * x - 8. * y - 4. * z, -4. * y,
                          -4. * z, -4. * z, 4. - 4. * x - 4. * y - 8. * z,
                          4. * z, 0., 4. * x,
                          0., 4. * z, 4. * y};
    std::memcpy(g, G, sizeof G);
}

void make_ns_tables(NSTables *t) {
    Rule q15 = make_rule(15), q5 = make_rule(5);
    static double phi[15][10], dphi[15][10][3], lam[15][4];
    for (int q = 0; q < 15; q++) {
        basis_phi(2, q15.pts[q], phi[q]);
        basis_dphi(2, q15.pts[q], &dphi[q][0][0]);
        basis_phi(1, q15.pts[q], lam[q]);
    }
    static const int SC[6] = {0, 1, 2, 0, 0, 1}, SD[6] = {0, 1, 2, 1, 2, 2};
    for (int a = 0; a < 10; a++)
        for (int b = 0; b < 10; b++) {
            for (int s = 0; s < 6; s++) {
                double v = 0;
                for (int q = 0; q < 15; q++) {
                    double x = dphi[q][a][SC[s]] * dphi[q][b][SD[s]];
                    if (SC[s] != SD[s]) x += dphi[q][a][SD[s]] * dphi[q][b][SC[s]];
                    v += q15.w[q] * x;
                }
                t->KS[a][b][s] = (float)v;
            }
            for (int m = 0; m < 4; m++) {
                double v = 0;
                for (int q = 0; q < 15; q++) v += q15.w[q] * lam[q][m] * phi[q][a] * phi[q][b];
                t->R[a][b][m] = (float)v;
            }
            for (int c = 0; c < 3; c++)
                for (int k = 0; k < 10; k++) {
                    double v = 0;
                    for (int q = 0; q < 15; q++) v += q15.w[q] * phi[q][a] * phi[q][k] * dphi[q][b][c];
                    t->T[c][a][b][k] = (float)v;
                }
        }
    for (int c = 0; c < 3; c++)
        for (int pn = 0; pn < 4; pn++)
            for (int b = 0; b < 10; b++) {
                double v = 0;
                for (int q = 0; q < 5; q++) {
                    double ps[4], dp[10][3];
                    basis_phi(1, q5.pts[q], ps);
                    basis_dphi(2, q5.pts[q], &dp[0][0]);
                    v += q5.w[q] * ps[pn] * dp[b][c];
                }
                t->Y[c][pn][b] = (float)v;
            }
    for (int a = 0; a < 10; a++)
        for (int q = 0; q < 16; q++) {
            t->WPHI[a][q] = q < 15 ? (float)(q15.w[q] * phi[q][a]) : 0.0f;
            for (int c = 0; c < 3; c++) t->DQ[a][c][q] = q < 15 ? (float)dphi[q][a][c] : 0.0f;
        }
    for (int q = 0; q < 15; q++)
        for (int k = 0; k < 10; k++) t->PHIQ[q][k] = (float)phi[q][k];
    const double V[4][3] = {{0, 0, 0}, {1, 0, 0}, {0, 1, 0}, {0, 0, 1}};
    for (int m = 0; m < 4; m++) {
        double dp[10][3];
        basis_dphi(2, V[m], &dp[0][0]);
        for (int k = 0; k < 10; k++)
            for (int c = 0; c < 3; c++) t->DV[m][k][c] = (float)dp[k][c];
    }
}

void make_hyper_tables(int npts, HyperTables *t) {
    Rule r = make_rule(npts);
    t->nq = r.n;
    for (int q = 0; q < r.n; q++) {
        double dp[10][3];
        basis_dphi(2, r.pts[q], &dp[0][0]);
        t->w[q] = (float)r.w[q];
        for (int a = 0; a < 10; a++)
            for (int c = 0; c < 3; c++) t->dphi[q][a][c] = (float)dp[a][c];
    }
}

}  // namespace fedd
