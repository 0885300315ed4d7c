// gen.cpp -- seeded synthetic inputs: FEDDLib's structured unit-cube tet mesh
// and smooth random fields.
//
// Mesh numbering and the 6-tet split follow MeshStructured::buildMesh3D
// (feddlib/core/Mesh/MeshStructured_def.hpp: P1 points 700-735, P1 elements
// 770-804, P2 points 832-858, P2 elements 899-992) for one rank on the unit
// cube; orientation follows Mesh::correctElementOrientation / flipElement
// (feddlib/core/Mesh/Mesh_def.hpp:543-577, 648-735).
#include <cmath>
#include <cstring>

#include "../../include/feddgpu.h"

namespace {

uint64_t splitmix(uint64_t &s) {
    uint64_t z = (s += 0x9E3779B97F4A7C15ULL);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    return z ^ (z >> 31);
}
double unit(uint64_t &s) { return (double)(splitmix(s) >> 11) * (1.0 / 9007199254740992.0); }

double det_b(const double *xyz, const int32_t *c) {
    const double *x0 = xyz + 3 * (int64_t)c[0];
    double v[9];
    for (int j = 0; j < 3; j++)
        for (int i = 0; i < 3; i++) v[3 * i + j] = xyz[3 * (int64_t)c[j + 1] + i] - x0[i];
    return v[0] * v[4] * v[8] + v[1] * v[5] * v[6] + v[2] * v[3] * v[7] - v[6] * v[4] * v[2] - v[7] * v[5] * v[0] -
           v[8] * v[3] * v[1];
}

}  // namespace

extern "C" {

fedd_status fedd_mesh_sizes(int32_t M, int32_t fe_order, int64_t *num_nodes, int64_t *num_elements) {
    if (M < 1 || (fe_order != 1 && fe_order != 2) || !num_nodes || !num_elements) return FEDD_ERR_ARG;
    int64_t n = fe_order == 1 ? (M + 1) : (2 * M + 1);
    *num_nodes = n * n * n;
    *num_elements = 6LL * M * M * M;
    return FEDD_OK;
}

fedd_status fedd_mesh_structured(int32_t M, int32_t fe_order, uint64_t seed, double amp, double *xyz, int32_t *conn) {
    if (M < 1 || (fe_order != 1 && fe_order != 2) || !xyz || !conn) return FEDD_ERR_ARG;
    if (6LL * M * M * M >= (1LL << 28)) return FEDD_ERR_ARG;
    const double h = 1.0 / M;
    const int n1 = M + 1, P = 2 * M + 1;
    const int64_t PP = (int64_t)P * P;
    int64_t c = 0;
    if (fe_order == 1) {
        for (int t = 0; t < n1; t++)
            for (int s = 0; s < n1; s++)
                for (int r = 0; r < n1; r++, c++) {
                    xyz[3 * c] = r * h; xyz[3 * c + 1] = s * h; xyz[3 * c + 2] = t * h;
                }
    } else {
        for (int t = 0; t < P; t++)
            for (int s = 0; s < P; s++)
                for (int r = 0; r < P; r++, c++) {
                    xyz[3 * c] = r * h / 2.0; xyz[3 * c + 1] = s * h / 2.0; xyz[3 * c + 2] = t * h / 2.0;
                }
    }
    // elements: 6 tets per hex in the reference's order
    c = 0;
    for (int t = 0; t < M; t++)
        for (int s = 0; s < M; s++)
            for (int r = 0; r < M; r++) {
                if (fe_order == 1) {
                    auto I = [&](int rr, int ss, int tt) { return (int32_t)(rr + n1 * ss + (int64_t)n1 * n1 * tt); };
                    const int32_t T[6][4] = {
                        {I(r + 1, s, t), I(r, s, t), I(r + 1, s, t + 1), I(r + 1, s + 1, t + 1)},
                        {I(r, s, t + 1), I(r, s, t), I(r + 1, s, t + 1), I(r + 1, s + 1, t + 1)},
                        {I(r + 1, s, t), I(r, s, t), I(r + 1, s + 1, t), I(r + 1, s + 1, t + 1)},
                        {I(r, s, t), I(r, s + 1, t), I(r + 1, s + 1, t), I(r + 1, s + 1, t + 1)},
                        {I(r, s, t), I(r, s + 1, t), I(r, s + 1, t + 1), I(r + 1, s + 1, t + 1)},
                        {I(r, s, t), I(r, s, t + 1), I(r, s + 1, t + 1), I(r + 1, s + 1, t + 1)}};
                    std::memcpy(conn + 24 * c, T, sizeof T);
                } else {
                    // lattice node (x, y, z) of the P2 grid
                    auto N = [&](int64_t x, int64_t y, int64_t z) { return (int32_t)(x + P * y + PP * z); };
                    const int64_t x0 = 2 * r, y0 = 2 * s, z0 = 2 * t;
                    // vertices of each tet as lattice offsets (in half-steps), then edge
                    // nodes at the lattice midpoints, in Helper's local edge order
                    static const int V[6][4][3] = {
                        {{2, 0, 0}, {0, 0, 0}, {2, 0, 2}, {2, 2, 2}}, {{0, 0, 2}, {0, 0, 0}, {2, 0, 2}, {2, 2, 2}},
                        {{2, 0, 0}, {0, 0, 0}, {2, 2, 0}, {2, 2, 2}}, {{0, 0, 0}, {0, 2, 0}, {2, 2, 0}, {2, 2, 2}},
                        {{0, 0, 0}, {0, 2, 0}, {0, 2, 2}, {2, 2, 2}}, {{0, 0, 0}, {0, 0, 2}, {0, 2, 2}, {2, 2, 2}}};
                    static const int E[6][2] = {{0, 1}, {1, 2}, {0, 2}, {0, 3}, {1, 3}, {2, 3}};
                    for (int k = 0; k < 6; k++) {
                        int32_t *e = conn + 60 * c + 10 * k;
                        for (int v = 0; v < 4; v++) e[v] = N(x0 + V[k][v][0], y0 + V[k][v][1], z0 + V[k][v][2]);
                        for (int m = 0; m < 6; m++) {
                            const int *A = V[k][E[m][0]], *B = V[k][E[m][1]];
                            e[4 + m] = N(x0 + (A[0] + B[0]) / 2, y0 + (A[1] + B[1]) / 2, z0 + (A[2] + B[2]) / 2);
                        }
                    }
                }
                c++;
            }
    const int64_t ne = 6LL * M * M * M;
    const int npe = fe_order == 1 ? 4 : 10;
    // jitter interior P1 vertices
    if (amp != 0.0) {
        uint64_t st = seed;
        for (int t = 0; t < n1; t++)
            for (int s = 0; s < n1; s++)
                for (int r = 0; r < n1; r++) {
                    if (r == 0 || s == 0 || t == 0 || r == M || s == M || t == M) continue;
                    int64_t idx = fe_order == 1 ? (r + (int64_t)n1 * s + (int64_t)n1 * n1 * t)
                                                : (2 * r + (int64_t)P * 2 * s + PP * 2 * t);
                    for (int d = 0; d < 3; d++) xyz[3 * idx + d] += (2.0 * unit(st) - 1.0) * amp * h;
                }
        if (fe_order == 2) {
            static const int E[6][2] = {{0, 1}, {1, 2}, {0, 2}, {0, 3}, {1, 3}, {2, 3}};
            for (int64_t e = 0; e < ne; e++) {
                const int32_t *ce = conn + 10 * e;
                for (int k = 0; k < 6; k++)
                    for (int d = 0; d < 3; d++)
                        xyz[3 * (int64_t)ce[4 + k] + d] =
                            0.5 * (xyz[3 * (int64_t)ce[E[k][0]] + d] + xyz[3 * (int64_t)ce[E[k][1]] + d]);
            }
        }
    }
    // orientation fix: det B < 0 -> swap 1<->2 (P2 also 4<->6, 8<->9)
    for (int64_t e = 0; e < ne; e++) {
        int32_t *ce = conn + npe * e;
        if (det_b(xyz, ce) < 0) {
            int32_t tmp = ce[1]; ce[1] = ce[2]; ce[2] = tmp;
            if (npe == 10) {
                tmp = ce[4]; ce[4] = ce[6]; ce[6] = tmp;
                tmp = ce[8]; ce[8] = ce[9]; ce[9] = tmp;
            }
        }
    }
    return FEDD_OK;
}

fedd_status fedd_field_fourier(uint64_t seed, int32_t kmin, int32_t kmax, int64_t num_nodes, const double *coords,
                               double scale, double *u) {
    if (!coords || !u || num_nodes < 0 || kmax < kmin) return FEDD_ERR_ARG;
    uint64_t st = seed;
    double K[8][3], A[8][3], PH[8];
    for (int m = 0; m < 8; m++) {
        for (int d = 0; d < 3; d++) K[m][d] = kmin + (int)(unit(st) * (kmax - kmin + 1));
        double n = 0;
        for (int d = 0; d < 3; d++) {
            A[m][d] = 2.0 * unit(st) - 1.0;
            n += A[m][d] * A[m][d];
        }
        n = std::sqrt(n > 0 ? n : 1.0);
        for (int d = 0; d < 3; d++) A[m][d] /= n;
        PH[m] = 2.0 * M_PI * unit(st);
    }
    for (int64_t i = 0; i < num_nodes; i++) {
        const double *x = coords + 3 * i;
        double v[3] = {0, 0, 0};
        for (int m = 0; m < 8; m++) {
            double sn = std::sin(2.0 * M_PI * (K[m][0] * x[0] + K[m][1] * x[1] + K[m][2] * x[2]) + PH[m]);
            for (int d = 0; d < 3; d++) v[d] += A[m][d] * sn;
        }
        for (int d = 0; d < 3; d++) u[3 * i + d] = scale * v[d];
    }
    return FEDD_OK;
}

fedd_status fedd_field_uniform(uint64_t seed, int64_t n, double lo, double hi, double *v) {
    if (!v || n < 0) return FEDD_ERR_ARG;
    uint64_t st = seed;
    for (int64_t i = 0; i < n; i++) v[i] = lo + (hi - lo) * unit(st);
    return FEDD_OK;
}

}  // extern "C"
