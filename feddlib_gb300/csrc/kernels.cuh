// kernels.cuh -- device-side declarations shared by the kernel translation
// units and the C ABI layer.
#pragma once
#include "engine.hpp"

namespace fedd {

// ---------------------------------------------------------------- laws ----
enum LawKind : int { kLawSKR1 = 1, kLawSKR2 = 2, kLawAniso = 3, kLawMLP = 4, kLawSKR3 = 5 };
// element-kernel instance of kLawMLP for a network whose I1 and J inputs are
// frozen (LawParams::mlp_fibre): the fibre-block Hessian only
constexpr int kLawMLPF = 6;

struct LawParams {
    int kind;
    float mu, lam, k1, k2;  // skr3: lam holds the bulk modulus kappa = E / (3 (1 - 2 nu))
    float a1[3], a2[3];
    int mlp_fibre;  // surrogate with frozen I1, J inputs: its Hessian lives in the (I4a, I4b) block
    // per element E_e / E (fedd_set_element_moduli), or null: the neo-Hooke
    // energies are linear in E at fixed Poisson ratio
    const float *escale;
};

// per-QP law derivatives with respect to (I1, J, I4a, I4b); d2 packed
// symmetric (00,01,02,03,11,12,13,22,23,33)
struct QPDerivs {
    float d1[4];
    float d2[10];
};

// The small tensors of a width-64 network as FP32 values (the bf16 weights
// widened exactly), passed by value so the quadrature-point kernel reads them
// from the constant bank: W1 by unit, its columns of the active inputs
// (those with a non-zero input scale, ascending) by input, biases, w3.
struct MlpConst {
    float W1[64][4];
    float Wact[4][64];
    float b1[64], b2[64], w3[64];
    int nact;           // number of active inputs
    int act[4];         // their indices
};

// MLP surrogate on the device: bf16 weights, FP32 biases and scalars.
struct MLPDev {
    int hidden;          // H (multiple of 16, <= 128)
    const void *W1;      // bf16, H x 4
    const float *b1;     // H
    const void *W2;      // bf16, H x H (row-major out x in)
    const float *b2;     // H
    const void *w3;      // bf16, H
    float b3, out_scale;
    float in_shift[4], in_scale[4];
    float inv_lo[4], inv_hi[4];
    int in_clamp;        // bit k: input k is max(inv_k - in_shift_k, 0)^2 in_scale_k
    MlpConst c;          // filled for hidden == 64
};

// ------------------------------------------------------- staging sizes ----
// Element stage of the elasticity paths: the 30 x 30 element matrix
// row-major with rows padded to 32 floats (128-byte aligned, so a row gather
// moves whole 16-byte chunks); column 30 of row p holds entry p of the
// element residual, so a row's gather brings its residual along, and column
// 31 is zero.  (The tangent is symmetric, but a packed upper triangle of
// 3 x 3 blocks, padded to 48 bytes for 16-byte copies, measured slower: the
// row gather is bound by the bytes it stages per incidence, 480 for ten
// padded blocks against 384 for three rows, and the two nodes that read an
// off-diagonal block are too far apart in the sweep for L2 to keep it.)
constexpr int kElemStride = 960;   // floats per element
constexpr int kElemResCol = 30;    // column of each row holding its residual entry
// The generalized-Newtonian stage keeps a separate residual row: 30 rows of
// 32 floats (columns 30 and 31 zero), then the 30 residual entries.  Its
// element kernel writes each row from the lanes that own the columns, so a
// residual column would need a cross-lane move per row; that measured 5 %
// slower than the separate row.
constexpr int kGNStride = 992;     // floats per element
constexpr int kGNRes = 960;        // offset of the residual row
constexpr int kNSRecord = 228;     // floats per element record (Navier-Stokes): 128 + NA[10][10]
constexpr int kLapStrideP1 = 16;   // doubles: 10 packed K + 4 load + pad
constexpr int kLapStrideP2 = 72;   // doubles: 55 packed K + 10 load + pad

// ------------------------------------------------------------ launches ----
struct LaunchCounter {
    int64_t n = 0;
};

// The element-stage launchers take an element range [e_begin, e_end) (e_end
// -1: ne); ne stays the stride of the connectivity arrays.
// hyperelastic / elasticity
void launch_hyper_elem(const double *xyz, const int32_t *conn, int64_t ne, const double *u, const LawParams &law,
                       const HyperTables &tab, const QPDerivs *qpd, const uint8_t *qp_fallback, float *stage,
                       int want_res, int *d_err, cudaStream_t s, LaunchCounter &lc, int64_t e_begin = 0,
                       int64_t e_end = -1);
void launch_hyper_rows(const Graph &g, const float *stage, const int64_t *rowptr, double *vals, double *res,
                       int64_t nnodes, cudaStream_t s, LaunchCounter &lc,
                       int64_t n_begin = 0);
void launch_hyper_invariants(const double *xyz, const int32_t *conn, int64_t ne, const double *u,
                             const LawParams &law, const HyperTables &tab, float *inv, int *d_err, cudaStream_t s,
                             LaunchCounter &lc, int64_t e_begin = 0, int64_t e_end = -1);
void launch_mlp_qp(const MLPDev &m, const LawParams &law, const float *inv, int64_t nqp, QPDerivs *out,
                   uint8_t *fallback, int *d_count, int *d_err, cudaStream_t s, LaunchCounter &lc);
void launch_law_qp_plain(const LawParams &law, const float *inv, int64_t nqp, QPDerivs *out, cudaStream_t s,
                         LaunchCounter &lc);
void launch_law_eval(const LawParams &law, const MLPDev *m, int64_t n, const double *F, double *psi, double *P,
                     double *A, cudaStream_t s);
void launch_hyper_dense(const float *stage, int64_t first, int64_t count, double *Ke, double *re, cudaStream_t s);

// Navier-Stokes
void ns_upload_tables(const NSTables &t, float **d_tables);
void launch_ns_record(const double *xyz, const int32_t *conn2, const int32_t *conn1, int64_t ne, const double *u,
                      const double *p, const float *d_tables, float visc_dens, float dens, float *rec, int *d_err,
                      cudaStream_t s, LaunchCounter &lc, int64_t e_begin = 0, int64_t e_end = -1);
// per velocity-row node: first incidence, vertex P1 node, neighbour and
// incidence counts (one int4; built once per mesh)
void launch_ns_node_info(const Graph &g, const int64_t *padj_ptr, const int32_t *vmap, int4 *info, cudaStream_t s);
// FE::assemblyNavierStokes' coeff (AssembleFENavierStokes::setCoeff,
// AssembleFENavierStokes_def.hpp:56-64): the residual's block factors,
// r_u = uu (ANB_uu u) + up (ANB_up p) and r_p = pu (ANB_pu u) (:199-224;
// ANB_pp is empty).  The matrices are not scaled.
struct NSCoeff {
    double uu = 1.0, up = 1.0, pu = 1.0;
};
void launch_ns_vel_rows(const Graph &g, const int4 *ninfo, const float *rec, const float *d_tables,
                        const int64_t *rowptr00, const int64_t *rowptr01, double *vals00, double *vals01,
                        double *res_u, float visc_dens, float dens, int newton, int want_jac, int max_adj,
                        int max_padj, const int32_t *vmap, const int64_t *rowptr10, double *vals10, double *res_p,
                        const float *gstage, cudaStream_t s, LaunchCounter &lc,
                        int64_t n_begin = 0, int64_t n_end = -1, unsigned long long *work = nullptr,
                        const NSCoeff &co = NSCoeff{});
void launch_ns_pres_rows(const Graph &gp, const float *rec, const float *d_tables, const int64_t *rowptr10,
                         double *vals10, double *res_p, int want_jac, int max_adj, cudaStream_t s,
                         LaunchCounter &lc, const NSCoeff &co = NSCoeff{});
void launch_ns_dense(const float *rec, const float *d_tables, int64_t first, int64_t count, float visc_dens,
                     float dens, int newton, double *Ke, double *re, cudaStream_t s, const NSCoeff &co = NSCoeff{});

// FE::assemblyRHS with a source function (FP64): the rule's reference
// points, weights and basis values (1 point for P1, 5 for P2)
struct RhsRule {
    int nq, npe;
    double xhat[5][3];
    double w[5];
    double phi[5][10];
};
RhsRule make_rhs_rule(int order);
// physical quadrature points, element-major (ne x nq x 3)
void launch_rhs_points(const double *xyz, const int32_t *conn, int64_t ne, const RhsRule &R, double *xq,
                       cudaStream_t s);
// the load vector from the source values at those points (ne x nq x ncomp)
void launch_rhs_assemble(const Graph &g, const double *xyz, const int32_t *conn, int64_t ne, const RhsRule &R,
                         const double *fq, int ncomp, double *stage, double *rhs, int *d_err, cudaStream_t s);

// Laplace (FP64)
void lap_make_tables(int order, std::vector<double> &out);
void launch_lap_elem(const double *xyz, const int32_t *conn, int64_t ne, int order, const double *d_tables, double f,
                     double *stage, int *d_err, cudaStream_t s, LaunchCounter &lc, int64_t e_begin = 0,
                     int64_t e_end = -1);
void launch_lap_rows(const Graph &g, const double *stage, int order, const int64_t *rowptr, double *vals,
                     double *load, int64_t nnodes, cudaStream_t s, LaunchCounter &lc);
void launch_lap_dense(const double *stage, int order, int64_t first, int64_t count, double *Ke, double *re,
                      cudaStream_t s);

// ---------------------------------------------------- Dirichlet rows ----
void launch_dirichlet_rows(const int64_t *rows, int64_t nrows, const int64_t *rowptr, const int32_t *colind,
                           double *vals, bool diagonal_block, cudaStream_t s, LaunchCounter &lc);
void launch_dirichlet_rhs(const int64_t *rows, int64_t n, const double *g, const double *sub, double *res,
                          cudaStream_t s, LaunchCounter &lc);

// ---------------------------------------------- generalized Newtonian ----
// Viscosity law of FEDDLib's generalized-Newtonian models: model 0
// Carreau-Yasuda (lambda, n, eta0, etaInf, a), 1 Power-Law (K, n, eta_max,
// eta_min), 2 Dimless-Carreau (lambda, n, eta0, etaInf, reference viscosity).
struct ViscLaw {
    int model;
    float prm[5];
    float gamma_min;
};
// Elements flagged for the outflow Neumann term (fedd_set_outflow_faces):
// element ids ascending, and per element the three vertex node ids of the
// face it takes, in the face's own order (which sets the normal's sign).
struct GNOutflow {
    const int32_t *elem = nullptr;
    const int32_t *face = nullptr;
    int64_t n = 0;
    int matrix = 0;  // 1: the term enters the element matrix too (the fixed-point matrix)
};
// Viscous part (stress term, and its derivative with Newton) of every
// element into the element stage (kGNStride floats per element), then the
// outflow Neumann term of the flagged elements into their residual rows.
void launch_gn_elem(const double *xyz, const int32_t *conn, int64_t ne, const double *u, const ViscLaw &law,
                    int newton, float *stage, int *d_err, cudaStream_t s, LaunchCounter &lc, int64_t e_begin = 0,
                    int64_t e_end = -1, const GNOutflow &outflow = GNOutflow{});
void launch_gn_dense(const float *stage, int64_t first, int64_t count, double *Ke, double *re, cudaStream_t s,
                     double coeff_uu = 1.0);

}  // namespace fedd
