/*
 * feddgpu.h -- C ABI of the GB300 finite-element assembly engine.
 *
 * The engine replaces FEDDLib's element loop + scatter for one mesh/problem:
 * the FE::assembly* drivers (feddlib/core/FE/FE_decl.hpp) with their
 * AssembleFE element kernels (feddlib/core/AceFemAssembly/AssembleFE_decl.hpp)
 * and the Tpetra insertGlobalValues/fillComplete scatter.  It hands back CSR
 * blocks in Tpetra's layout (size_t row offsets, int32 column indices sorted
 * ascending per row, double values, node-wise dof numbering dof = dofs*node+d)
 * and residual vectors on the unique (non-repeated) numbering.
 *
 * Conventions
 *  - Plain pointers and sizes only.  "host" buffers are ordinary memory;
 *    "device" buffers are CUDA device pointers.  `stream` is a cudaStream_t
 *    passed as void* (NULL = legacy default stream).
 *  - Every call returns a fedd_status.  No exception crosses the ABI.
 *    fedd_last_error() gives a message for the last failing call on a handle.
 *  - A handle is not re-entrant: serialise calls on one handle.  All device
 *    work is stream-ordered; host-buffer calls synchronise their stream.
 *  - Results are deterministic: each CSR value is written once, as the sum of
 *    its element contributions in ascending element order.
 */
#ifndef FEDDGPU_H
#define FEDDGPU_H
#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define FEDDGPU_ABI_VERSION 1

typedef enum {
    FEDD_OK = 0,
    FEDD_ERR_ARG = 1,         /* bad argument (null pointer, size, unknown key)      */
    FEDD_ERR_CUDA = 2,        /* a CUDA runtime call failed                           */
    FEDD_ERR_MESH = 3,        /* invalid mesh: bad node index, det B <= 0 where       */
                              /* orientation matters                                  */
    FEDD_ERR_NONFINITE = 4,   /* a non-finite value appeared (e.g. det F <= 0)        */
    FEDD_ERR_TIMEOUT = 5,     /* a bounded device wait gave up                        */
    FEDD_ERR_NOMEM = 6,       /* device allocation failed                             */
    FEDD_ERR_STATE = 7,       /* call not valid in the handle's current state         */
    FEDD_ERR_UNSUPPORTED = 8, /* combination not implemented                          */
    FEDD_ERR_CAPACITY = 9     /* a per-node adjacency exceeds the engine's limits     */
} fedd_status;

/* Problem keys of AssembleFEFactory::build
 * (feddlib/core/AceFemAssembly/AssembleFEFactory_def.hpp:22-62). */
typedef enum {
    FEDD_LAPLACE = 1,               /* "Laplace": scalar stiffness (+ load vector)   */
    FEDD_LINEAR_ELASTICITY = 2,     /* "LinearElasticity": AceGen skr1 law, 4 points */
    FEDD_NONLINEAR_ELASTICITY = 3,  /* "NonLinearElasticity": AceGen skr2 law, 5 pts */
    FEDD_NAVIER_STOKES = 4,         /* "NavierStokes": P2-P1 Taylor-Hood             */
    FEDD_ANISO_FIBER = 5,           /* two-fibre exponential law (no FEDDLib key)    */
    FEDD_NONLINEAR_ELASTICITY2 = 6  /* "NonLinearElasticity2" ("Neo-Hooke Modell" != 1):
                                       AceGen skr3, isochoric neo-Hooke, 5 pts       */
} fedd_problem;

/* what-flags for fedd_assemble*: */
#define FEDD_JACOBIAN 1u
#define FEDD_RESIDUAL 2u

/* Block ids of the 2x2 Navier-Stokes BlockMatrix (FE_def.hpp:982-1062);
 * single-field problems only have FEDD_BLOCK_00. */
#define FEDD_BLOCK_00 0
#define FEDD_BLOCK_01 1
#define FEDD_BLOCK_10 2
#define FEDD_BLOCK_11 3

/* fedd_mesh.flags: coords, elements and elements_p are device pointers (a
 * mesh made or refined on the device never visits the host). */
#define FEDD_MESH_DEVICE 1u

typedef struct {
    int64_t num_nodes;          /* nodes of the primary mesh (P1 or P2)              */
    int64_t num_elements;
    int32_t fe_order;           /* 1 = "P1" (4 nodes), 2 = "P2" (10 nodes)            */
    uint32_t flags;             /* 0 (host arrays) or FEDD_MESH_DEVICE                */
    const double *coords;       /* num_nodes x 3                                      */
    const int32_t *elements;    /* num_elements x (4|10), FEDDLib local order         */
    int64_t num_nodes_p;        /* Navier-Stokes: P1 pressure mesh nodes, else 0      */
    const int32_t *elements_p;  /* Navier-Stokes: num_elements x 4, same element order*/
} fedd_mesh;

typedef struct {
    int32_t problem;            /* fedd_problem                                       */
    int32_t linearization;      /* NS "General/Linearization": 0 FixedPoint, 1 Newton;
                                   2 the fixed-point matrix of FE::assemblyNavierStokes'
                                   assembleMode "FixedPoint" (FE_def.hpp:1178-1191), the
                                   same as 0 except that a generalized-Newtonian element's
                                   outflow term also enters the matrix                  */
    int32_t quad_points;        /* 0 = the reference's rule for this problem          */
    int32_t surrogate;          /* FEDD_ANISO_FIBER: 0 plain law, 1 MLP surrogate     */
    double viscosity;           /* "Parameter/Viscosity"                              */
    double density;             /* "Parameter/Density"                                */
    double E;                   /* "Parameter/E"                                      */
    double poisson_ratio;       /* "Parameter/Poisson Ratio"                          */
    double k1, k2;              /* fibre law parameters                               */
    double fiber_angle_deg;     /* fibres at +-angle in the xy-plane                  */
    double source;              /* Laplace load: constant f                           */
} fedd_params;

typedef struct fedd_assembler fedd_assembler;

/* ---- lifetime ------------------------------------------------------------ */
/* Replaces FE::initAssembleFEElements (FE_def.hpp:1455-1474) + the BlockMatrix
 * allocation with getApproxEntriesPerRow (NavierStokesAssFE_def.hpp:143-165):
 * uploads the mesh, checks it, and builds every CSR pattern on the device. */
fedd_status fedd_create(const fedd_mesh *mesh, const fedd_params *params, int device,
                        fedd_assembler **out);
fedd_status fedd_destroy(fedd_assembler *h);
/* h = NULL: the message of the calling thread's last failing call that takes
 * no handle (mesh front end, medit files). */
fedd_status fedd_last_error(const fedd_assembler *h, char *buf, size_t len);
const char *fedd_status_string(fedd_status s);
int fedd_abi_version(void);

/* ---- pattern (fillComplete's column map, Matrix_decl.hpp:133-138) ------- */
fedd_status fedd_block_info(const fedd_assembler *h, int block, int64_t *nrows, int64_t *ncols,
                            int64_t *nnz);
fedd_status fedd_get_pattern(fedd_assembler *h, int block, int64_t *rowptr_host,
                             int32_t *colind_host);
fedd_status fedd_device_pattern(fedd_assembler *h, int block, const int64_t **d_rowptr,
                                const int32_t **d_colind);
fedd_status fedd_residual_sizes(const fedd_assembler *h, int64_t *n_u, int64_t *n_p);

/* ---- assembly ------------------------------------------------------------ */
/* Host-buffer entry point: one call = FE::assemblyNavierStokes("Jacobian")
 * (FE_def.hpp:1078-1239) followed by its "Rhs" call, or
 * FE::assemblyLinearElasticity / assemblyNonLinearElasticity
 * (FE_def.hpp:362-434, 449-523), or FE::assemblyLaplace + assemblyRHS
 * (FE_def.hpp:2437-2500, 7303-7400).  u: dofs*num_nodes values (node-wise);
 * p: num_nodes_p values (NS only).  vals[b] receives block b's values;
 * with FEDD_JACOBIAN every block of the problem is required (00; NS: 00, 01
 * and 10), the unused ones NULL.  res_u/res_p receive the residual blocks
 * (both for NS) with FEDD_RESIDUAL.  Laplace: res_u is the load vector and u
 * is ignored. */
fedd_status fedd_assemble(fedd_assembler *h, unsigned what, const double *u, const double *p,
                          double *vals00, double *vals01, double *vals10, double *res_u,
                          double *res_p, void *stream);
/* Device-buffer entry point, same meaning; nothing is copied and the call
 * returns after enqueueing the work on `stream`. */
fedd_status fedd_assemble_device(fedd_assembler *h, unsigned what, const double *d_u,
                                 const double *d_p, double *d_vals00, double *d_vals01,
                                 double *d_vals10, double *d_res_u, double *d_res_p, void *stream);
/* Reads the device error word written by the last assembly on this handle
 * (non-finite values, det F <= 0, timeouts); synchronises `stream`. */
fedd_status fedd_check(fedd_assembler *h, void *stream);

/* ---- generalized-Newtonian fluids ---------------------------------------- */
/* Makes a Navier-Stokes handle a generalized-Newtonian one, FEDDLib's
 * AssembleFEGeneralizedNewtonian (feddlib/core/AceFemAssembly/specific/
 * AssembleFEGeneralizedNewtonian_def.hpp, chosen by "Material/
 * ShearThinningModel"): the Newtonian Laplacian is replaced by the
 * stress-divergence term with viscosity eta(shear rate) and, with Newton
 * linearization, its derivative; advection, its Newton term and B / B^T stay.
 * model 0 "Carreau-Yasuda": prm = (CharacteristicTime_Lambda, FluidIndex_n,
 *   ZeroShearRateViscosity_eta0, InftyShearRateViscosity_etaInfty,
 *   InflectionPoint_a); 1 "Power-Law": (PowerLawParameter K, PowerLaw index n,
 *   Numerical_ZeroShearRateViscosity, Numerical_InftyShearRateViscosity, -);
 *   2 "Dimless-Carreau": (Dimless_CharacteristicTime_Lambda,
 *   Carreau_FluidIndex_n, Dimless_ZeroShearRateViscosity_eta0,
 *   Dimless_InftyShearRateViscosity_etaInfty, Reference_Viscosity);
 * gamma_min = "Numerical_ZeroValue_ShearRate".  model < 0 returns to the
 * Newtonian fluid.  The outflow Neumann boundary term applies to the elements
 * flagged by fedd_set_outflow_faces. */
fedd_status fedd_set_viscosity_law(fedd_assembler *h, int32_t model, const double *prm,
                                   double gamma_min);

/* The faces flagged for the generalized-Newtonian outflow Neumann term, the
 * boundary sub-elements that Domain::setSurfaceQuadraturePointsWeights(flag,
 * degree) marks (feddlib/core/FE/Domain_def.hpp:1214-1255) and
 * AssembleFEGeneralizedNewtonian::assemblyOutflowNeumannBoundaryTerm
 * integrates (AssembleFEGeneralizedNewtonian_def.hpp:697-920): faces holds
 * nfaces x 3 vertex node ids (P2 mesh numbering) in the sub-element's own
 * order, which sets the normal (f0 - f1) x (f0 - f2) as FEDDLib's
 * Helper::computeSurfaceNormal does.  Each face must be a face of exactly one
 * element (FEDD_ERR_ARG otherwise, with a message); an element listed more
 * than once takes its last face, as the reference keeps the data of an
 * element's last flagged sub-element.  The surface rule is the 7-point one
 * FEDDLib's P2 faces get in 3D.  As in the reference, the term enters the
 * velocity residual; it enters the matrix only with linearization 2, the
 * fixed-point matrix (assembleJacobian forms the element Jacobian before it
 * adds the term; assembleFixedPoint's matrix holds it, :172-221).  It applies
 * while a viscosity law is set.  Each call matches the faces to their
 * elements on the host (a hash of every element's four vertex faces), so
 * set the list once, not per Newton step.  nfaces = 0 clears.
 * Navier-Stokes handles only (FEDD_ERR_STATE otherwise). */
fedd_status fedd_set_outflow_faces(fedd_assembler *h, const int32_t *faces, int64_t nfaces);

/* FE::assemblyNavierStokes' coeff argument, which FEDDLib hands to every
 * element through AssembleFENavierStokes::setCoeff
 * (feddlib/core/FE/FE_def.hpp:1206, AssembleFENavierStokes_def.hpp:56-64):
 * the 2 x 2 block factors of the residual r = (coeff .* ANB) x
 * (AssembleFENavierStokes_def.hpp:199-224 and, for the generalized-Newtonian
 * element, AssembleFEGeneralizedNewtonian_def.hpp:928-970), row-major
 * {c_uu, c_up, c_pu, c_pp}: r_u = c_uu (ANB_uu u) + c_up (ANB_up p) and
 * r_p = c_pu (ANB_pu u); c_pp multiplies the empty pressure block.  The
 * matrices are not scaled.  Applies to the residuals of fedd_assemble*,
 * fedd_element_matrices and fedd_element_matrices_noalloc until the next
 * call; all ones (the default) reproduces the unscaled residual bit for bit.
 * Non-finite factors give FEDD_ERR_ARG.  Navier-Stokes handles only
 * (FEDD_ERR_STATE otherwise). */
fedd_status fedd_set_coeff(fedd_assembler *h, const double coeff[4]);

/* The E-field variant of FE::assemblyNonLinearElasticity
 * (feddlib/core/FE/FE_def.hpp:538-614): a Young's modulus per element (host
 * array of num_elements values), which FEDDLib hands to each element with
 * updateParameter("E", eModVec[T]) (AssembleFE_NonLinElas_def.hpp:175-180);
 * the Poisson ratio stays the handle's.  The elasticity energies are linear
 * in E at a fixed Poisson ratio (mu, lambda and the bulk modulus all scale
 * with E), so each element's tangent and residual are its terms at the
 * handle's E times E_e / E (that factor rounded to FP32).  Kept until the
 * next call; E = NULL returns to the handle's E.  Values must be finite and
 * positive (FEDD_ERR_ARG).  Linear elasticity and neo-Hooke handles only
 * (FEDD_ERR_STATE otherwise). */
fedd_status fedd_set_element_moduli(fedd_assembler *h, const double *E);

/* ---- load vector from a source function ---------------------------------- */
/* FE::assemblyRHS (feddlib/core/FE/FE_def.hpp:7303-7400) evaluates its
 * source function at the physical quadrature points of every element, on
 * the rule Helper::determineDegree(dim, FEType, Std) selects (1 point for P1
 * meshes, the 5-point rule for P2).  fedd_rhs_points gives those points,
 * x_q = B xhat_q + x_0 in FP64, element-major (num_elements x nq x 3, host);
 * *nq receives the points per element, and xq = NULL asks for nq only.  The
 * caller evaluates its function there and fedd_assemble_rhs forms
 *     rhs[ncomp node + c] = sum over the node's elements (ascending) of
 *                           |det B| sum_q w_q phi_a(q) f[e][q][c]
 * from fq (num_elements x nq x ncomp, host): ncomp 1 is fieldType "Scalar",
 * 3 "Vector" (node-wise dofs).  rhs (host, ncomp x num_nodes) is
 * overwritten.  The handle's mesh is used: the velocity mesh of a
 * Navier-Stokes handle.  Synchronous. */
fedd_status fedd_rhs_points(fedd_assembler *h, double *xq, int32_t *nq);
fedd_status fedd_assemble_rhs(fedd_assembler *h, const double *fq, int32_t ncomp, double *rhs);

/* ---- Dirichlet rows on the device ---------------------------------------- */
/* The Dirichlet dofs of the problem, FEDDLib's BC flags resolved to dofs
 * (BCBuilder, feddlib/core/General/BCBuilder_decl.hpp:128-172): host masks
 * over the dofs of block row 0 (n_u, node-wise) and, for Navier-Stokes,
 * block row 1 (n_p; may be NULL).  Nonzero = Dirichlet.  Kept on the device
 * until the next call. */
fedd_status fedd_dirichlet_set(fedd_assembler *h, const uint8_t *mask_u, const uint8_t *mask_p);
/* BCBuilder::setSystem (BCBuilder_def.hpp:590-700) on device CSR values:
 * each Dirichlet row becomes zero except a one at its diagonal entry in the
 * diagonal block (a row whose pattern lacks the diagonal entry stays zero)
 * and zero in the off-diagonal blocks of its block row.  Navier-Stokes needs
 * all three value arrays.  Enqueued on `stream`. */
fedd_status fedd_dirichlet_system(fedd_assembler *h, double *d_vals00, double *d_vals01,
                                  double *d_vals10, void *stream);
/* BCBuilder::setRHS (BCBuilder_def.hpp:93-200) and setBCMinusVector
 * (:232-350) on device vectors: res[k] = g[k] - sub[k] at the Dirichlet dofs
 * of each block (g NULL: zero boundary values; sub NULL: setRHS).  Other
 * entries are untouched.  Enqueued on `stream`. */
fedd_status fedd_dirichlet_rhs(fedd_assembler *h, const double *d_g_u, const double *d_g_p,
                               const double *d_sub_u, const double *d_sub_p, double *d_res_u,
                               double *d_res_p, void *stream);

/* Element-level output, the AssembleFE::getJacobian()/getRHS() view
 * (AssembleFE_decl.hpp:100,112): dense element matrices (nd x nd, row-major,
 * nd = 4|10 Laplace, 30 elasticity, 34 NS) and element vectors for elements
 * [first, first+count).  Host buffers.  newton_step 0 vs >0 does not change
 * values (FEDDLib caches A and B at step 0; the engine recomputes them). */
fedd_status fedd_element_matrices(fedd_assembler *h, const double *u, const double *p,
                                  int64_t first, int64_t count, double *Ke, double *re);

/* fedd_element_matrices without allocation.  No counterpart in FEDDLib.
 * For callers that may not allocate device memory per call: a host that
 * keeps other streams busy cannot take the device-wide synchronisation of
 * cudaFree, and a host that reserved its device memory once at start-up
 * must not see the footprint grow.  Fields are DEVICE pointers (d_u: n_u
 * doubles, d_p: n_p doubles, as fedd_assemble_device); Ke/re are host
 * buffers as in fedd_element_matrices, staged through a 4 MiB file-scope
 * device array; the element stage runs over [first, first + count) only.
 * Limits: count * nd * (nd + 1) <= 524288 doubles, i.e. at most 440
 * elements (Navier-Stokes), 563 (elasticity), 4766 (Laplace P2), 26214
 * (Laplace P1) per call; more is rejected with FEDD_ERR_ARG and a message.
 * Generalized-Newtonian handles (fedd_set_viscosity_law) are rejected with
 * FEDD_ERR_UNSUPPORTED.  The first call on a device may load the module
 * there: make it before any stream capture.  Nothing in the scratch must
 * start at zero; the call clears the handle's error word itself.  One
 * scratch array per device is shared by all handles: calls that overlap in
 * time on one device race, so serialise them; the call also writes the
 * handle's element stage, so it must not overlap any other call on the same
 * handle.  Synchronises `stream` before returning. */
fedd_status fedd_element_matrices_noalloc(fedd_assembler *h, const double *d_u,
                                          const double *d_p, int64_t first, int64_t count,
                                          double *Ke, double *re, void *stream);

/* Element geometry exactly as the element kernels use it, the
 * Helper::buildTransformation + SmallMatrix::computeDet/computeInverse step
 * (feddlib/core/FE/Helper.cpp:196-222, feddlib/core/General/SmallMatrix.hpp:
 * 317-368): B = [x1 - x0, x2 - x0, x3 - x0], det B and B^-1 = adj(B) / det B
 * formed in FP64, each entry of B^-1 then rounded once to FP32.  For elements
 * [first, first + count): det (count doubles, signed) and binv (count x 9
 * floats, row-major).  Host buffers. */
fedd_status fedd_element_geometry(fedd_assembler *h, int64_t first, int64_t count, double *det,
                                  float *binv);

/* Number of kernel launches the last fedd_assemble* enqueued. */
fedd_status fedd_launch_count(const fedd_assembler *h, int64_t *launches);

/* Stage timing with CUDA events recorded on the caller's stream around each
 * kernel of fedd_assemble* (up to 256 calls are kept).  A diagnostic with no
 * FEDDLib counterpart; FEDDLib times its loops on the host with
 * Teuchos::TimeMonitor (feddlib/core/Utils/FEDDUtils.hpp:7-12).
 * fedd_stage_times synchronises, returns per-stage totals in ms over the
 * recorded calls and clears them. */
fedd_status fedd_set_profiling(fedd_assembler *h, int on);
fedd_status fedd_stage_times(fedd_assembler *h, int max_stages, double *ms_total, int *nstages,
                             int64_t *calls);
const char *fedd_stage_name(const fedd_assembler *h, int stage);

/* ---- MLP strain-energy surrogate (FEDD_ANISO_FIBER with surrogate = 1) -- */
/* Psi(I1, J, I4a, I4b) = Psi_skr1(I1, J) + out_scale * net(x),
 * x_k = (inv_k - in_shift_k) * in_scale_k, net: 4 -> H -> H -> 1, softplus.
 * Weights are uploaded as bf16 (rounded to nearest even); host arrays FP32.
 * W1: H x 4, W2: H x H (row-major, out x in), w3: H. */
typedef struct {
    int32_t hidden;
    int32_t in_clamp;  /* bit k: input k enters as max(inv_k - in_shift_k, 0)^2 * in_scale_k, so
                          the surrogate and its first derivative vanish continuously at and
                          below in_shift_k (a one-sided law such as fibres in tension only);
                          0: (inv_k - in_shift_k) * in_scale_k */
    const float *W1, *b1, *W2, *b2, *w3;
    float b3;
    float out_scale;
    float in_shift[4];
    float in_scale[4];
    float inv_lo[4], inv_hi[4]; /* per-QP invariant box; outside it -> plain law */
} fedd_mlp_desc;
fedd_status fedd_set_surrogate(fedd_assembler *h, const fedd_mlp_desc *mlp);
/* Fraction of quadrature points that fell back to the plain law in the last
 * assembly, and the number of such points. */
fedd_status fedd_surrogate_fallbacks(fedd_assembler *h, int64_t *count, int64_t *total);

/* Invariants (I1, J, I4a, I4b) at every quadrature point of every element
 * for displacement u (host, 3 per node): out is num_elements x nq x 4 FP32
 * (host).  Hyperelastic problems only; the training-data generator of the
 * surrogate samples these over load steps.  No FEDDLib counterpart. */
fedd_status fedd_qp_invariants(fedd_assembler *h, const double *u, float *out);

/* Law evaluation at given deformation gradients (n x 9 row-major, host):
 * psi (n), first Piola P (n x 9) and tangent A = dP/dF (n x 81), for the
 * handle's law (plain or surrogate).  Measures the surrogate against the plain law. */
fedd_status fedd_law_eval(fedd_assembler *h, int64_t n, const double *F, double *psi,
                          double *P, double *A);

/* Training of the surrogate on the device with the project's own kernels:
 * Sobolev loss  mean( wpsi (y - tpsi)^2 + wgrad |dy/dx - tgrad|^2 )  in the
 * network's normalised units, Adam, full-batch or mini-batch.  Parameters
 * are FP32 masters (host in/out); the caller rounds to bf16 for inference. */
typedef struct fedd_trainer fedd_trainer;
fedd_status fedd_trainer_create(int32_t hidden, int64_t n, const float *x, const float *tpsi,
                                const float *tgrad, int device, fedd_trainer **out);
fedd_status fedd_trainer_set_params(fedd_trainer *t, const float *W1, const float *b1,
                                    const float *W2, const float *b2, const float *w3, float b3);
fedd_status fedd_trainer_get_params(fedd_trainer *t, float *W1, float *b1, float *W2,
                                    float *b2, float *w3, float *b3);
/* One pass of `steps` Adam updates over mini-batches of `batch` samples
 * (batch = n: full batch); returns the mean loss of the last step. */
fedd_status fedd_trainer_run(fedd_trainer *t, int32_t steps, int64_t batch, float lr,
                             float wpsi, float wgrad, uint64_t seed, float *last_loss);
/* Loss and parameter gradient at the current parameters (full data set),
 * for checking the backward kernels against the oracle. */
fedd_status fedd_trainer_grad(fedd_trainer *t, float wpsi, float wgrad, float *loss, float *gW1,
                              float *gb1, float *gW2, float *gb2, float *gw3, float *gb3);
fedd_status fedd_trainer_destroy(fedd_trainer *t);

/* ---- input generators (MeshStructured::buildMesh3D, MeshStructured_def.hpp:
 *      622-1010, plus the orientation fix Mesh_def.hpp:543-735) ------------ */
/* Unit cube, M^3 hexes x 6 tets, FEDDLib numbering; interior P1 vertices
 * jittered by (2u-1)*amp*h (splitmix64 stream from `seed`, 3 draws per
 * vertex in lattice order); P2 edge nodes at their edge midpoints; elements
 * with det B < 0 flipped as flipElement does.  Sizes first, then fill. */
fedd_status fedd_mesh_sizes(int32_t M, int32_t fe_order, int64_t *num_nodes,
                            int64_t *num_elements);
fedd_status fedd_mesh_structured(int32_t M, int32_t fe_order, uint64_t seed, double amp,
                                 double *coords, int32_t *elements);
/* The same mesh written straight into device buffers (coords num_nodes x 3,
 * elements num_elements x (4|10), sizes from fedd_mesh_sizes), bit-identical
 * to fedd_mesh_structured; `stream` is a cudaStream_t, synchronised before
 * the call returns. */
fedd_status fedd_mesh_structured_device(int32_t M, int32_t fe_order, uint64_t seed, double amp,
                                        double *coords, int32_t *elements, void *stream);

/* ---- unstructured meshes (the mesh front end) ------------------------------ */
/* P2 mesh of a P1 tetrahedral mesh, built on the device as
 * MeshUnstructured::buildP2ofP1MeshEdge does (MeshUnstructured_def.hpp:
 * 122-233): the P2 nodes are the P1 nodes followed by one node per edge at
 * its midpoint, edges numbered in the lexicographic order of their (min, max)
 * vertex pair (EdgeElements::sortUniqueAndSetGlobalIDs via
 * MeshPartitioner::buildEdgeListParallel, MeshPartitioner_def.hpp:737-775);
 * P2 element e lists the P1 element's vertices, then its edge nodes at
 * positions 4=e01 5=e12 6=e02 7=e03 8=e13 9=e23
 * (determinePositionInElementP2, MeshUnstructured_def.hpp:690-736).
 * flags & FEDD_MESH_DEVICE: coords / elements are device pointers.
 * *num_nodes_p2 receives the P2 node count; fedd_p2_copy fills caller buffers
 * (coords num_nodes_p2 x 3, elements num_elements x 10; host or device per
 * flags). The P1 mesh stays the pressure mesh of a Taylor-Hood pair. */
typedef struct fedd_p2mesh fedd_p2mesh;
fedd_status fedd_p2_of_p1(int64_t num_nodes, int64_t num_elements, const double *coords,
                          const int32_t *elements, uint32_t flags, int device, fedd_p2mesh **out,
                          int64_t *num_nodes_p2);
fedd_status fedd_p2_copy(const fedd_p2mesh *m, double *coords, int32_t *elements, uint32_t flags);
fedd_status fedd_p2_destroy(fedd_p2mesh *m);

/* medit (.mesh) files as FEDDLib reads them (MeshFileReader.cpp:16-106,
 * MeshFileReader.hpp:80-128): "Dimension 3", "Vertices" (x y z flag),
 * "Tetrahedra" (4 one-based node ids + flag), "Triangles" (3 ids + flag);
 * other sections are skipped.  Ids come back zero-based; any output pointer
 * may be NULL.  The writer prints 17 significant digits (exact round trip). */
fedd_status fedd_medit_sizes(const char *path, int64_t *num_nodes, int64_t *num_tets,
                             int64_t *num_tris);
fedd_status fedd_medit_read(const char *path, double *coords, int32_t *node_flags, int32_t *tets,
                            int32_t *tet_flags, int32_t *tris, int32_t *tri_flags);
fedd_status fedd_medit_write(const char *path, int64_t num_nodes, const double *coords,
                             const int32_t *node_flags, int64_t num_tets, const int32_t *tets,
                             const int32_t *tet_flags, int64_t num_tris, const int32_t *tris,
                             const int32_t *tri_flags);

/* Seeded velocity field: sum of 8 Fourier modes a_m sin(2 pi k_m.x + phi_m),
 * k_m in {kmin..kmax}^3, |a_m| = 1; written node-wise (3 per node). */
fedd_status fedd_field_fourier(uint64_t seed, int32_t kmin, int32_t kmax, int64_t num_nodes,
                               const double *coords, double scale, double *u);
/* Uniform[lo, hi) values (pressure field). */
fedd_status fedd_field_uniform(uint64_t seed, int64_t n, double lo, double hi, double *v);

#ifdef __cplusplus
}
#endif
#endif
