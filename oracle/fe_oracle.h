/*
 * fe_oracle.h -- FP64 CPU restatement of FEDDLib's element-assembly path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the checker for the GPU engine:
 * only tests/, __graft_entry__.smoke() and bench.py's cpu_baseline leg load it.
 * Nothing in feddlib_gb300/ links, loads or calls it.
 *
 * Parity status: pinned where the reference's own code could be compiled
 * here (oracle/_ref, see oracle/build_ref.sh): Helper quadrature/basis
 * tables, the AssembleFE_Laplace, AssembleFENavierStokes and
 * AssembleFEGeneralizedNewtonian element classes (compiled against stub
 * Trilinos headers), and the classic elasticity members of FE_def.hpp
 * (assemblyLinElasXDim and nh3d through assemblyElasticityJacobianAceFEM /
 * assemblyElasticityStressesAceFEM, extracted by extract_fe_members.py and
 * compiled against a stub FE class).  The AceGen Fortran kernels
 * (skr1/skr2/skr3) cannot be compiled here (no Fortran compiler); the
 * hyperelastic laws are restated from the strain energies identified in
 * those files and pinned through the reference's own cross-path identities
 * with those classic elements (skr1 at u = 0 == assemblyLinElasXDim,
 * fe_test_linElas.cpp; skr2 == nh3d, fe_test_nonLinElas.cpp), to ~1e-15.
 * skr3 is pinned by its linear-elastic limit and finite differences.  The
 * anisotropic two-fibre law and the MLP surrogate have no reference
 * counterpart: parity unpinned for those two.
 *
 * Every function cites the reference file:line it restates (paths relative
 * to the FEDDLib source tree).
 */
#ifndef FE_ORACLE_H
#define FE_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- quadrature and basis (feddlib/core/FE/Helper.cpp) ------------------ */
int orc_quad(int npts, double *pts, double *w);
int orc_quad_points_for_degree(int degree);
int orc_degree_un(int fe_order, unsigned deg_func);
int orc_degree_pair(int fe1, int fe2, int type1, int type2, int extra);
void orc_phi(int fe_order, const double *p, double *val);
void orc_dphi(int fe_order, const double *p, double *val);

/* ---- structured mesh (feddlib/core/Mesh/MeshStructured_def.hpp) --------- */
void orc_mesh_sizes(int M, int fe_order, int64_t *num_nodes, int64_t *num_elements);
void orc_mesh_structured(int M, int fe_order, double *xyz, int32_t *conn);
void orc_mesh_jitter(int M, int fe_order, uint64_t seed, double amp, double *xyz);
void orc_mesh_p2_midpoints(int64_t ne, const int32_t *conn, double *xyz);
int64_t orc_mesh_orient(int fe_order, int64_t ne, const double *xyz, int32_t *conn);
double orc_geometry(const double *x0, const double *x1, const double *x2,
                    const double *x3, double *B, double *Binv);

/* ---- element kernels ------------------------------------------------------ */
void orc_elem_laplace(int fe_order, int npts, const double *xe, double *K);
void orc_elem_rhs_const(int fe_order, int npts, const double *xe, double f, double *b);
void orc_elem_ns(const double *xe, const double *u, const double *p, double visc,
                 double dens, int newton, const double *coeff, double *J, double *res,
                 double *A, double *N, double *W, double *Bd);
void orc_elem_linelas_classic(int npts, const double *xe, double lambda, double mu,
                              double *K);

/* Generalized-Newtonian viscosity laws (feddlib/core/AceFemAssembly/specific/
 * GeneralizedNewtonianModels): prm for Carreau-Yasuda = (lambda, n, eta0,
 * etaInf, a); Power-Law = (K, n, eta_max, eta_min); Dimless-Carreau =
 * (lambda, n, eta0, etaInf, reference viscosity).  gamma_min is
 * "Numerical_ZeroValue_ShearRate". */
enum { ORC_GN_CARREAU_YASUDA = 0, ORC_GN_POWER_LAW = 1, ORC_GN_DIMLESS_CARREAU = 2 };
typedef struct {
    int model;
    double prm[5];
    double gamma_min;
} orc_visc_law;
double orc_gn_eta(const orc_visc_law *L, double gamma);
double orc_gn_dterm(const orc_visc_law *L, double gamma); /* -(2/gamma) d eta / d gamma */
void orc_elem_gn(const double *xe, const double *u, const double *p, const orc_visc_law *L,
                 double dens, int newton, double *J, double *res);
/* outflow Neumann boundary term of one element with one flagged face (face:
 * its three vertex coordinates in the face's node order); K is 30 x 30 */
void orc_gn_outflow(const double *xe, const double *face, const double *u, const orc_visc_law *L, double *K);

/* Hyperelastic laws, written as Psi(I1, J, I4a, I4b). */
enum { ORC_LAW_SKR1 = 1, ORC_LAW_SKR2 = 2, ORC_LAW_ANISO = 3, ORC_LAW_MLP = 4, ORC_LAW_SKR3 = 5 };
typedef struct {
    int law;
    double mu, lambda;
    double k1, k2;
    double a1[3], a2[3];
    /* MLP surrogate (law == ORC_LAW_MLP): invariants -> H -> H -> Psi */
    int hidden;
    const double *W1, *b1, *W2, *b2, *w3; double b3;
    const double *in_shift, *in_scale;  /* x_k = (inv_k - shift_k) * scale_k */
    double out_scale;                   /* Psi_mlp = out_scale * net(x) */
    int mlp_add_matrix;                 /* 1: Psi = Psi_skr1(I1,J) + mlp */
    int in_clamp;                       /* bit k: x_k = max(inv_k - shift_k, 0)^2 * scale_k */
} orc_law;

void orc_law_invariants(const orc_law *L, const double *F, double *inv);
void orc_law_dpsi(const orc_law *L, const double *inv, double *psi, double *d1, double *d2);
void orc_law_PA(const orc_law *L, const double *F, double *psi, double *P, double *A);
void orc_elem_hyper(const orc_law *L, int npts, const double *xe, const double *u,
                    double *K, double *r);

/* MLP surrogate forward with first/second derivatives w.r.t. the 4 inputs. */
void orc_mlp_eval(int H, const double *W1, const double *b1, const double *W2,
                  const double *b2, const double *w3, double b3, const double *x,
                  double *y, double *g, double *h);
/* Loss used for training and its parameter gradient (for gradient checks). */
double orc_mlp_loss(int H, const double *W1, const double *b1, const double *W2,
                    const double *b2, const double *w3, double b3, int64_t n,
                    const double *x, const double *tpsi, const double *tgrad,
                    double wpsi, double wgrad, double *gW1, double *gb1, double *gW2,
                    double *gb2, double *gw3, double *gb3);

/* ---- global assembly with Tpetra insert/fillComplete semantics ----------- */
int64_t orc_coo_to_csr(int64_t nrows, int64_t ncoo, const int64_t *rows,
                       const int64_t *cols, const double *vals, int64_t *rowptr,
                       int32_t *colind, double *values);

/* Batched element assembly over a whole mesh into COO triples, in the
 * reference's insertion order (element by element). */
int64_t orc_assemble_laplace_coo(int fe_order, int npts, int64_t ne, const double *xyz,
                                 const int32_t *conn, int64_t *rows, int64_t *cols,
                                 double *vals);
void orc_assemble_rhs(int fe_order, int npts, int64_t ne, const double *xyz,
                      const int32_t *conn, double f, double *rhs);
int64_t orc_assemble_vec_coo(int kind, const orc_law *L, int npts, int64_t ne,
                             const double *xyz, const int32_t *conn, const double *u,
                             int64_t *rows, int64_t *cols, double *vals, double *res);
int64_t orc_assemble_ns_coo(int64_t ne, const double *xyz, const int32_t *conn2,
                            const int32_t *conn1, const double *u, const double *p,
                            double visc, double dens, int newton, int block,
                            int64_t *rows, int64_t *cols, double *vals, double *res_u,
                            double *res_p);

/* Reference-shaped CPU baseline: keeps FEDDLib's algorithm shape (per-element
 * table rebuild and heap element matrices, growable per-row insert buffers,
 * sort + merge at fillComplete).  Used only as the timed CPU stand-in. */
double orc_cpu_baseline_ns(int64_t ne_sample, const double *xyz, const int32_t *conn2,
                           const int32_t *conn1, const double *u, const double *p,
                           double visc, double dens, int64_t nrows_u, int64_t nrows_p);

/* ---- rows at full mesh size ------------------------------------------------
 * Node -> incident elements (ascending), a node-by-node check of a CSR block
 * pattern against the element adjacency, and the complete rows of chosen
 * nodes rebuilt from all of their incident elements (FP64), so that parity
 * is checked at the configurations' own sizes without assembling the whole
 * mesh on the CPU. */
void orc_node_elements(int64_t ne, const int32_t *conn, int npe, int64_t nn, int64_t *ptr, int64_t *elems);
int64_t orc_check_block_pattern(int64_t ne, const int32_t *row_conn, int npe_r, const int32_t *col_conn,
                                int npe_c, int64_t nrow_nodes, const int64_t *node_ptr, const int64_t *node_elems,
                                int dofs_r, int dofs_c, const int64_t *rowptr, const int32_t *colind);
int orc_rows_vec(int kind, const orc_law *L, int npts, int64_t ne, const double *xyz, const int32_t *conn,
                 const double *u, const int64_t *node_ptr, const int64_t *node_elems, int64_t nsel,
                 const int64_t *sel, int kmax, int64_t *cols, double *vals, double *res);
int orc_rows_ns(int64_t ne, const double *xyz, const int32_t *conn2, const int32_t *conn1, const double *u,
                const double *p, double visc, double dens, int newton, const int64_t *ptr2, const int64_t *el2,
                const int64_t *ptr1, const int64_t *el1, int64_t nv, const int64_t *vsel, int64_t np,
                const int64_t *psel, int kmax, int kpmax, int64_t *cols00, double *vals00, int64_t *cols01,
                double *vals01, double *res_u, int64_t *cols10, double *vals10, double *res_p);
/* orc_rows_ns for the generalized-Newtonian element (orc_elem_gn) */
int orc_rows_gn(int64_t ne, const double *xyz, const int32_t *conn2, const int32_t *conn1, const double *u,
                const double *p, const orc_visc_law *L, double dens, int newton, const int64_t *ptr2,
                const int64_t *el2, const int64_t *ptr1, const int64_t *el1, int64_t nv, const int64_t *vsel,
                int64_t np, const int64_t *psel, int kmax, int kpmax, int64_t *cols00, double *vals00,
                int64_t *cols01, double *vals01, double *res_u, int64_t *cols10, double *vals10, double *res_p);

/* Reference-shaped CPU baseline for the elasticity problems (one kernel call
 * per element for the Jacobian, a second for the residual when want_res),
 * with per-row inserts and fillComplete; returns a checksum. */
double orc_cpu_baseline_vec(const orc_law *L, int npts, int64_t ne, const double *xyz, const int32_t *conn,
                            const double *u, int want_res, int64_t nrows);

/* min / max of det F over the quadrature points of elements [0, ne) */
void orc_detF_range(int npts, int64_t ne, const double *xyz, const int32_t *conn, const double *u,
                    double *jmin, double *jmax);

void orc_field_fourier(uint64_t seed, int kmin, int kmax, int64_t n, const double *xyz, double scale,
                       double *u);
void orc_field_uniform(uint64_t seed, int64_t n, double lo, double hi, double *v);

#ifdef __cplusplus
}
#endif
#endif
