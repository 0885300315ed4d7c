/*
 * feddgpu_fe.hpp -- C++ facade over the C ABI (feddgpu.h), header only, C++17.
 *
 * It mirrors the FEDDLib interfaces the engine replaces, with plain CSR and
 * vector types in place of Tpetra/Xpetra:
 *   feddgpu::FE                 FE::assembly* (feddlib/core/FE/FE_decl.hpp:181-186,
 *                               453-458, 475-490, 560-595)
 *   feddgpu::AssembleFE         AssembleFE (feddlib/core/AceFemAssembly/
 *                               AssembleFE_decl.hpp:61-299)
 *   feddgpu::AssembleFEFactory  AssembleFEFactory::build
 *                               (AssembleFEFactory_decl.hpp:56, keys of
 *                               AssembleFEFactory_def.hpp:22-62)
 *   feddgpu::ParameterList      the Teuchos::ParameterList entries these calls read
 *
 * Status codes of the C ABI become feddgpu::Error exceptions, as FEDDLib's
 * TEUCHOS_TEST_FOR_EXCEPTION sites throw std::runtime_error / logic_error.
 */
#ifndef FEDDGPU_FE_HPP
#define FEDDGPU_FE_HPP

#include <array>
#include <cstdint>
#include <functional>
#include <map>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "feddgpu.h"

namespace feddgpu {

class Error : public std::runtime_error {
  public:
    Error(fedd_status code, const std::string &what) : std::runtime_error(what), code(code) {}
    fedd_status code;
};

inline void check(fedd_status s, const fedd_assembler *h = nullptr) {
    if (s == FEDD_OK) return;
    std::string msg = fedd_status_string(s);
    if (h) {
        char buf[512] = {0};
        if (fedd_last_error(h, buf, sizeof buf) == FEDD_OK && buf[0]) msg += std::string(": ") + buf;
    }
    throw Error(s, msg);
}

// The Teuchos::ParameterList entries read by the assembly calls:
// sublist("Parameter"): "Viscosity", "Density", "E", "Poisson Ratio";
// sublist("General"): "Linearization" ("FixedPoint" | "Newton");
// sublist("Material"): "Newtonian" (bool), "ShearThinningModel" and each
// model's parameters, as FEDDLib's generalized-Newtonian models read them.
class ParameterList {
  public:
    ParameterList &sublist(const std::string &name) {
        auto &p = subs_[name];
        if (!p) p = std::make_unique<ParameterList>();
        return *p;
    }
    const ParameterList *findSublist(const std::string &name) const {
        auto it = subs_.find(name);
        return it == subs_.end() ? nullptr : it->second.get();
    }
    ParameterList &set(const std::string &key, double v) { num_[key] = v; return *this; }
    ParameterList &set(const std::string &key, bool v) { bool_[key] = v; return *this; }
    ParameterList &set(const std::string &key, const std::string &v) { str_[key] = v; return *this; }
    ParameterList &set(const std::string &key, const char *v) { str_[key] = v; return *this; }
    double get(const std::string &key, double def) const {
        auto it = num_.find(key);
        return it == num_.end() ? def : it->second;
    }
    std::string get(const std::string &key, const std::string &def) const {
        auto it = str_.find(key);
        return it == str_.end() ? def : it->second;
    }
    std::string get(const std::string &key, const char *def) const { return get(key, std::string(def)); }
    bool get(const std::string &key, bool def) const {
        auto it = bool_.find(key);
        return it == bool_.end() ? def : it->second;
    }
    // value of sublist(sub).get(key, def) without creating the sublist
    template <class T> T at(const std::string &sub, const std::string &key, T def) const {
        const ParameterList *s = findSublist(sub);
        return s ? s->get(key, def) : def;
    }

  private:
    std::map<std::string, std::unique_ptr<ParameterList>> subs_;
    std::map<std::string, double> num_;
    std::map<std::string, std::string> str_;
    std::map<std::string, bool> bool_;
};

// What FEDDLib's Domain hands the FE class: node coordinates and element
// connectivity in FEDDLib's local node order.
struct Domain {
    std::string FEType = "P2";      // "P1" (4 nodes) | "P2" (10 nodes)
    // boundary faces that Domain::setSurfaceQuadraturePointsWeights(flag, 8)
    // flags for the generalized-Newtonian outflow term: three vertex node ids
    // per face in the sub-element's order (Domain_def.hpp:1214-1255)
    std::vector<int32_t> outflowFaces;
    std::vector<double> coords;     // num_nodes x 3
    std::vector<int32_t> elements;  // num_elements x nodes per element

    int nodesPerElement() const { return FEType == "P1" ? 4 : 10; }
    int64_t numNodes() const { return (int64_t)coords.size() / 3; }
    int64_t numElements() const { return (int64_t)elements.size() / nodesPerElement(); }

    // MeshStructured::buildMesh3D on the unit cube (M^3 hexes x 6 tets),
    // interior vertices jittered by +-jitter*h from `seed`.
    static Domain structured(int M, const std::string &FEType, uint64_t seed, double jitter = 0.1) {
        Domain d;
        d.FEType = FEType;
        const int order = FEType == "P1" ? 1 : 2;
        int64_t nn = 0, ne = 0;
        check(fedd_mesh_sizes(M, order, &nn, &ne));
        d.coords.resize((size_t)nn * 3);
        d.elements.resize((size_t)ne * d.nodesPerElement());
        check(fedd_mesh_structured(M, order, seed, jitter, d.coords.data(), d.elements.data()));
        return d;
    }
};

struct CsrMatrix {  // a fill-completed CrsMatrix: sorted columns, node-wise dofs
    int64_t nrows = 0, ncols = 0;
    std::vector<int64_t> rowptr;
    std::vector<int32_t> colind;
    std::vector<double> values;
    int64_t nnz() const { return (int64_t)colind.size(); }
};

struct BlockMatrix {  // BlockMatrix_Type: present[i][j] marks an assembled block
    std::array<std::array<CsrMatrix, 2>, 2> block;
    std::array<std::array<bool, 2>, 2> present{};
};

struct BlockMultiVector {  // BlockMultiVector_Type on unique maps
    std::vector<std::vector<double>> block;
};

// RAII owner of one engine handle.
class Assembler {
  public:
    Assembler(const Domain &d, const Domain *pressure, const fedd_params &prm, int device) {
        fedd_mesh m{};
        m.num_nodes = d.numNodes();
        m.num_elements = d.numElements();
        m.fe_order = d.FEType == "P1" ? 1 : 2;
        m.coords = d.coords.data();
        m.elements = d.elements.data();
        if (pressure) {
            m.num_nodes_p = pressure->numNodes();
            m.elements_p = pressure->elements.data();
        }
        check(fedd_create(&m, &prm, device, &h_));
        check(fedd_residual_sizes(h_, &n_u_, &n_p_), h_);
        ne_ = d.numElements();
    }
    Assembler(const Assembler &) = delete;
    Assembler &operator=(const Assembler &) = delete;
    ~Assembler() { fedd_destroy(h_); }

    fedd_assembler *handle() const { return h_; }
    int64_t n_u() const { return n_u_; }
    int64_t n_p() const { return n_p_; }

    void pattern(int b, CsrMatrix &A) const {
        int64_t nr = 0, nc = 0, nnz = 0;
        check(fedd_block_info(h_, b, &nr, &nc, &nnz), h_);
        A.nrows = nr;
        A.ncols = nc;
        A.rowptr.resize((size_t)nr + 1);
        A.colind.resize((size_t)nnz);
        A.values.assign((size_t)nnz, 0.0);
        check(fedd_get_pattern(h_, b, A.rowptr.data(), A.colind.data()), h_);
    }
    // blocks: which of 00, 01, 10 receive values (their pattern must be set)
    void assemble(unsigned what, const double *u, const double *p, CsrMatrix *b00, CsrMatrix *b01,
                  CsrMatrix *b10, double *res_u, double *res_p) {
        auto v = [](CsrMatrix *m) { return m ? m->values.data() : nullptr; };
        check(fedd_assemble(h_, what, u, p, v(b00), v(b01), v(b10), res_u, res_p, nullptr), h_);
    }
    void elementMatrices(const double *u, const double *p, int64_t first, int64_t count, double *Ke,
                         double *re) {
        check(fedd_element_matrices(h_, u, p, first, count, Ke, re), h_);
    }
    void viscosityLaw(int model, const double prm[5], double gamma_min) {
        check(fedd_set_viscosity_law(h_, model, prm, gamma_min), h_);
    }
    // a Young's modulus per element, or null for the handle's E
    void elementModuli(const std::vector<double> *E) {
        if (E && (int64_t)E->size() != ne_) throw Error(FEDD_ERR_ARG, "element moduli: one value per element");
        check(fedd_set_element_moduli(h_, E ? E->data() : nullptr), h_);
    }
    // the residual's 2 x 2 block factors (AssembleFENavierStokes::setCoeff)
    void coeff(const std::array<std::array<double, 2>, 2> &c) {
        const double v[4] = {c[0][0], c[0][1], c[1][0], c[1][1]};
        check(fedd_set_coeff(h_, v), h_);
    }
    // the face list is matched to its elements once; repeated calls with the
    // same list (every Newton step) do nothing
    void outflowFaces(const std::vector<int32_t> &faces) {
        if (faces_set_ && faces == faces_) return;
        check(fedd_set_outflow_faces(h_, faces.empty() ? nullptr : faces.data(), (int64_t)faces.size() / 3), h_);
        faces_ = faces;
        faces_set_ = true;
    }

  private:
    fedd_assembler *h_ = nullptr;
    int64_t n_u_ = 0, n_p_ = 0, ne_ = 0;
    std::vector<int32_t> faces_;
    bool faces_set_ = false;
};

namespace detail {
inline int fe_order(const std::string &FEType) {
    if (FEType == "P1") return 1;
    if (FEType == "P2") return 2;
    throw Error(FEDD_ERR_UNSUPPORTED, "FEType " + FEType + " not supported (P1, P2)");
}
inline void require_dim3(int dim) {
    if (dim != 3) throw Error(FEDD_ERR_UNSUPPORTED, "only dim = 3 is supported");
}
// The generalized-Newtonian viscosity model of sublist("Material") as
// FEDDLib's models read it (GeneralizedNewtonianModels/CarreauYasuda_def.hpp:
// 14-20, PowerLaw_def.hpp:14-19, Dimless_Carreau_def.hpp:14-20): the engine's
// model index (-1: Newtonian), its five parameters and the shear-rate floor.
// With `always` the model is read whatever Material/Newtonian says (the
// factory's "GeneralizedNewtonian" key builds that element directly).
inline int viscosity_model(const ParameterList &params, double prm[5], double &gamma_min, bool always = false) {
    for (int k = 0; k < 5; k++) prm[k] = 0.0;
    gamma_min = params.at<double>("Material", "Numerical_ZeroValue_ShearRate", 1e-8);
    if (!always && params.at<bool>("Material", "Newtonian", true)) return -1;
    const std::string m = params.at<std::string>("Material", "ShearThinningModel", "");
    auto g = [&](const char *key, double def) { return params.at<double>("Material", key, def); };
    if (m == "Carreau-Yasuda") {
        prm[0] = g("CharacteristicTime_Lambda", 0.0);
        prm[1] = g("FluidIndex_n", 1.0);
        prm[2] = g("ZeroShearRateViscosity_eta0", 0.0);
        prm[3] = g("InftyShearRateViscosity_etaInfty", 0.0);
        prm[4] = g("InflectionPoint_a", 1.0);
        return 0;
    }
    if (m == "Power-Law") {
        prm[0] = g("PowerLawParameter K", 0.0);
        prm[1] = g("PowerLaw index n", 1.0);
        prm[2] = g("Numerical_ZeroShearRateViscosity", 1.0);
        prm[3] = g("Numerical_InftyShearRateViscosity", 1.0);
        return 1;
    }
    if (m == "Dimless-Carreau") {
        prm[0] = g("Dimless_CharacteristicTime_Lambda", 0.0);
        prm[1] = g("Carreau_FluidIndex_n", 1.0);
        prm[2] = g("Dimless_ZeroShearRateViscosity_eta0", 0.0);
        prm[3] = g("Dimless_InftyShearRateViscosity_etaInfty", 0.0);
        prm[4] = g("Reference_Viscosity", 0.0);
        return 2;
    }
    throw Error(FEDD_ERR_UNSUPPORTED, "ShearThinningModel " + m + " (Carreau-Yasuda, Power-Law, Dimless-Carreau)");
}
}  // namespace detail

// FE::assembly* with plain outputs.  addFE(domain) registers the domains in
// FEDDLib's order (0: velocity / displacement / scalar, 1: pressure).  One
// engine handle per (problem, parameters) is kept, like FEDDLib's
// assemblyFEElements_, so Newton steps reuse the device-resident pattern.
class FE {
  public:
    explicit FE(int device = 0) : device_(device) {}

    void addFE(const Domain &d) { domains_.push_back(d); }

    // FE::assemblyLaplace (FE_def.hpp:2437-2500)
    void assemblyLaplace(int dim, const std::string &FEType, int degree, CsrMatrix &A,
                         bool callFillComplete = true, int FELocExternal = -1) {
        (void)degree; (void)callFillComplete;
        detail::require_dim3(dim);
        const Domain &d = domain(FELocExternal < 0 ? 0 : FELocExternal, FEType);
        fedd_params prm{};
        prm.problem = FEDD_LAPLACE;
        Assembler &a = get("Laplace/" + FEType, d, nullptr, prm);
        a.pattern(FEDD_BLOCK_00, A);
        a.assemble(FEDD_JACOBIAN, nullptr, nullptr, &A, nullptr, nullptr, nullptr, nullptr);
    }

    // FE::assemblyLaplaceAssFE (FE_def.hpp:1818-1853): the same stiffness
    // through FEDDLib's AssembleFE_Laplace elements, into block (0,0).  Its
    // 5-point rule and assemblyLaplace's 1-point rule both integrate the
    // P1 (and, with 5 points, the P2) gradient products exactly, and the
    // engine forms those integrals in closed form, so both calls give the
    // same values.
    void assemblyLaplaceAssFE(int dim, const std::string &FEType, int degree, int dofs, BlockMatrix &A,
                              bool callFillComplete = true, int FELocExternal = -1) {
        if (dofs != 1) throw Error(FEDD_ERR_UNSUPPORTED, "assemblyLaplaceAssFE: scalar Laplace, dofs = 1");
        assemblyLaplace(dim, FEType, degree, A.block[0][0], callFillComplete, FELocExternal);
        A.present[0][0] = true;
    }

    // FEDDLib's RhsFunc_Type (FEDDCore.hpp:124): func(x, res, parameters)
    // writes the source at the point x into res (one value per component)
    using RhsFunc = std::function<void(double *x, double *res, double *parameters)>;

    // FE::assemblyRHS (FE_def.hpp:7303-7400) with a source function: func
    // is evaluated on the host at the physical quadrature points of every
    // element (fedd_rhs_points), the engine integrates and sums per node
    // (fedd_assemble_rhs); fieldType "Scalar" (one value) or "Vector" (three,
    // node-wise dofs).
    void assemblyRHS(int dim, const std::string &FEType, std::vector<double> &a, const std::string &fieldType,
                     const RhsFunc &func, std::vector<double> &funcParameter) {
        detail::require_dim3(dim);
        if (fieldType != "Scalar" && fieldType != "Vector")
            throw Error(FEDD_ERR_ARG, "assemblyRHS: fieldType " + fieldType);
        const int ncomp = fieldType == "Scalar" ? 1 : 3;
        const Domain &d = domain(0, FEType);
        fedd_params prm{};
        prm.problem = FEDD_LAPLACE;
        Assembler &as = get("Laplace/" + FEType, d, nullptr, prm);
        int32_t nq = 0;
        check(fedd_rhs_points(as.handle(), nullptr, &nq), as.handle());
        std::vector<double> xq((size_t)d.numElements() * nq * 3), fq((size_t)d.numElements() * nq * ncomp);
        check(fedd_rhs_points(as.handle(), xq.data(), &nq), as.handle());
        double *par = funcParameter.empty() ? nullptr : funcParameter.data();
        for (size_t k = 0; k < xq.size() / 3; k++) {
            double res[3] = {0.0, 0.0, 0.0};
            func(&xq[3 * k], res, par);
            for (int c = 0; c < ncomp; c++) fq[k * ncomp + c] = res[c];
        }
        a.assign((size_t)d.numNodes() * ncomp, 0.0);
        check(fedd_assemble_rhs(as.handle(), fq.data(), ncomp, a.data()), as.handle());
    }

    // FE::assemblyRHS (FE_def.hpp:7303-7400) for fieldType "Scalar" and a
    // constant source f (the reference's rhs function evaluated as constant)
    void assemblyRHS(int dim, const std::string &FEType, std::vector<double> &a, const std::string &fieldType,
                     double f) {
        detail::require_dim3(dim);
        if (fieldType != "Scalar") throw Error(FEDD_ERR_UNSUPPORTED, "assemblyRHS: fieldType Scalar only");
        const Domain &d = domain(0, FEType);
        fedd_params prm{};
        prm.problem = FEDD_LAPLACE;
        prm.source = f;
        Assembler &as = get("RHS/" + FEType + "/" + std::to_string(f), d, nullptr, prm);
        a.assign((size_t)as.n_u(), 0.0);
        as.assemble(FEDD_RESIDUAL, nullptr, nullptr, nullptr, nullptr, nullptr, a.data(), nullptr);
    }

    // FE::assemblyLinearElasticity (FE_def.hpp:362-434): AceGen skr1.
    // assembleMode "Jacobian" fills A(0,0), "Rhs" fills resVec (needs d_rep).
    void assemblyLinearElasticity(int dim, const std::string &FEType, int degree, int dofs,
                                  const std::vector<double> *d_rep, BlockMatrix &A, BlockMultiVector &resVec,
                                  const ParameterList &params, bool reAssemble, const std::string &assembleMode,
                                  bool callFillComplete = true, int FELocExternal = -1) {
        (void)reAssemble;
        elasticity(FEDD_LINEAR_ELASTICITY, dim, FEType, degree, dofs, d_rep, A, resVec, params, assembleMode,
                   callFillComplete, FELocExternal);
    }

    // FE::assemblyNonLinearElasticity (FE_def.hpp:449-523): "Parameter/
    // Neo-Hooke Modell" 1 (the default) is "NonLinearElasticity" (AceGen
    // skr2), any other value "NonLinearElasticity2" (skr3) (:483-487);
    // tangent and residual in one call, as the reference does.
    void assemblyNonLinearElasticity(int dim, const std::string &FEType, int degree, int dofs,
                                     const std::vector<double> &d_rep, BlockMatrix &A, BlockMultiVector &resVec,
                                     const ParameterList &params, bool callFillComplete = true,
                                     int FELocExternal = -1) {
        const int model = (int)params.at<double>("Parameter", "Neo-Hooke Modell", 1.0);
        elasticity(model == 1 ? FEDD_NONLINEAR_ELASTICITY : FEDD_NONLINEAR_ELASTICITY2, dim, FEType, degree, dofs,
                   &d_rep, A, resVec, params, "Jacobian+Rhs", callFillComplete, FELocExternal);
    }

    // The E-field variant (FE_def.hpp:538-614): the elements of `domain`
    // with a Young's modulus each, eModVec[T], which FEDDLib hands to the
    // element with updateParameter("E", ...) before it assembles.
    void assemblyNonLinearElasticity(int dim, const std::string &FEType, int degree, int dofs,
                                     const std::vector<double> &d_rep, BlockMatrix &A, BlockMultiVector &resVec,
                                     const ParameterList &params, const Domain &domain,
                                     const std::vector<double> &eModVec, bool callFillComplete = true,
                                     int FELocExternal = -1) {
        (void)FELocExternal;
        const int model = (int)params.at<double>("Parameter", "Neo-Hooke Modell", 1.0);
        elasticity(model == 1 ? FEDD_NONLINEAR_ELASTICITY : FEDD_NONLINEAR_ELASTICITY2, dim, FEType, degree, dofs,
                   &d_rep, A, resVec, params, "Jacobian+Rhs", callFillComplete, -1, &domain, &eModVec);
    }

    // FE::assemblyNavierStokes (FE_def.hpp:1078-1239).  assembleMode:
    // "Jacobian" (Linearization from params: Newton adds W), "FixedPoint"
    // (no W), "Rhs" (residual into resVec blocks 0 and 1).  reAssemble
    // reuses A's patterns and refreshes its values in place (FEDDLib
    // re-assembles block (0,0) in Newton steps; the other blocks do not
    // depend on u and come out unchanged).  coeff scales the residual's
    // blocks, as FEDDLib hands it to every element with setCoeff
    // (FE_def.hpp:1206; AssembleFENavierStokes_def.hpp:56-64, 199-224).
    void assemblyNavierStokes(int dim, const std::string &FETypeVelocity, const std::string &FETypePressure,
                              int degree, int dofsVelocity, int dofsPressure, const std::vector<double> &u_rep,
                              const std::vector<double> &p_rep, BlockMatrix &A, BlockMultiVector &resVec,
                              const std::array<std::array<double, 2>, 2> &coeff, const ParameterList &params,
                              bool reAssemble, const std::string &assembleMode, bool callFillComplete = true,
                              int FELocExternal = -1) {
        (void)degree; (void)callFillComplete; (void)FELocExternal;
        detail::require_dim3(dim);
        if (FETypeVelocity != "P2" || FETypePressure != "P1" || dofsVelocity != 3 || dofsPressure != 1)
            throw Error(FEDD_ERR_UNSUPPORTED, "assemblyNavierStokes: P2-P1 Taylor-Hood, 3 + 1 dofs only");
        if (domains_.size() < 2) throw Error(FEDD_ERR_STATE, "assemblyNavierStokes: addFE velocity and pressure");
        const double visc = params.at<double>("Parameter", "Viscosity", 1.0);
        const double dens = params.at<double>("Parameter", "Density", 1.0);
        bool newton = params.at<std::string>("General", "Linearization", "FixedPoint") != "FixedPoint";
        // assembleMode "FixedPoint" takes the element's fixed-point matrix
        // (FE_def.hpp:1178-1191), linearization 2; it differs from the
        // FixedPoint Jacobian only by a generalized-Newtonian outflow term
        const bool fp_matrix = assembleMode == "FixedPoint";
        if (fp_matrix) newton = false;
        if (assembleMode != "Jacobian" && assembleMode != "FixedPoint" && assembleMode != "Rhs")
            throw Error(FEDD_ERR_ARG, "assemblyNavierStokes: assembleMode " + assembleMode);
        // Material/Newtonian = false selects AssembleFEGeneralizedNewtonian (FE_def.hpp:1134-1138)
        double vprm[5], gamma_min;
        const int model = detail::viscosity_model(params, vprm, gamma_min);
        fedd_params prm{};
        prm.problem = FEDD_NAVIER_STOKES;
        prm.linearization = newton ? 1 : (fp_matrix ? 2 : 0);
        prm.viscosity = visc;
        prm.density = dens;
        Assembler &a = get("NS/" + std::to_string(visc) + "/" + std::to_string(dens) +
                               (newton ? "/N" : (fp_matrix ? "/M" : "/F")),
                           domain(0, "P2"), &domain(1, "P1"), prm);
        a.viscosityLaw(model, vprm, gamma_min);
        a.outflowFaces(domain(0, "P2").outflowFaces);
        if ((int64_t)u_rep.size() != a.n_u() || (int64_t)p_rep.size() != a.n_p())
            throw Error(FEDD_ERR_ARG, "assemblyNavierStokes: u_rep / p_rep sizes");
        if (assembleMode == "Rhs") {
            a.coeff(coeff);
            resVec.block.resize(2);
            resVec.block[0].assign((size_t)a.n_u(), 0.0);
            resVec.block[1].assign((size_t)a.n_p(), 0.0);
            a.assemble(FEDD_RESIDUAL, u_rep.data(), p_rep.data(), nullptr, nullptr, nullptr,
                       resVec.block[0].data(), resVec.block[1].data());
            return;
        }
        // the engine writes the three blocks in one pass; with reAssemble the
        // (0,1)/(1,0) blocks, which do not depend on u, are refreshed in place
        const bool have = A.present[0][0] && A.present[0][1] && A.present[1][0] &&
                          (int64_t)A.block[0][0].values.size() == A.block[0][0].nnz() &&
                          (int64_t)A.block[0][1].values.size() == A.block[0][1].nnz() &&
                          (int64_t)A.block[1][0].values.size() == A.block[1][0].nnz();
        if (!reAssemble || !have) {
            a.pattern(FEDD_BLOCK_00, A.block[0][0]);
            a.pattern(FEDD_BLOCK_01, A.block[0][1]);
            a.pattern(FEDD_BLOCK_10, A.block[1][0]);
            a.pattern(FEDD_BLOCK_11, A.block[1][1]);  // empty for P2-P1 (FE_def.hpp:1024)
            A.present[0][0] = A.present[0][1] = A.present[1][0] = A.present[1][1] = true;
        }
        a.assemble(FEDD_JACOBIAN, u_rep.data(), p_rep.data(), &A.block[0][0], &A.block[0][1], &A.block[1][0],
                   nullptr, nullptr);
    }

  private:
    const Domain &domain(int k, const std::string &FEType) const {
        if (k < 0 || k >= (int)domains_.size()) throw Error(FEDD_ERR_STATE, "FE: domain not added (addFE)");
        if (domains_[k].FEType != FEType)
            throw Error(FEDD_ERR_ARG, "FE: domain " + std::to_string(k) + " is " + domains_[k].FEType +
                                          ", call asks for " + FEType);
        detail::fe_order(FEType);
        return domains_[k];
    }
    Assembler &get(const std::string &key, const Domain &d, const Domain *p, const fedd_params &prm) {
        auto &slot = cache_[key];
        if (!slot) slot = std::make_unique<Assembler>(d, p, prm, device_);
        return *slot;
    }
    void elasticity(int problem, int dim, const std::string &FEType, int degree, int dofs,
                    const std::vector<double> *d_rep, BlockMatrix &A, BlockMultiVector &resVec,
                    const ParameterList &params, const std::string &mode, bool callFillComplete, int FELoc,
                    const Domain *own = nullptr, const std::vector<double> *eMod = nullptr) {
        (void)degree; (void)callFillComplete;
        detail::require_dim3(dim);
        if (FEType != "P2" || dofs != 3) throw Error(FEDD_ERR_UNSUPPORTED, "elasticity: P2 with 3 dofs only");
        const double E = params.at<double>("Parameter", "E", 1000.0);
        const double nu = params.at<double>("Parameter", "Poisson Ratio", 0.4);
        fedd_params prm{};
        prm.problem = problem;
        prm.E = E;
        prm.poisson_ratio = nu;
        // a domain passed by the call (the E-field variant) gets its own handle
        const std::string where = own ? "/at" + std::to_string(reinterpret_cast<uintptr_t>(own)) : std::string();
        if (own && own->FEType != FEType) throw Error(FEDD_ERR_ARG, "elasticity: the domain is " + own->FEType);
        Assembler &a = get("Elas/" + std::to_string(problem) + "/" + std::to_string(E) + "/" + std::to_string(nu) +
                               where,
                           own ? *own : domain(FELoc < 0 ? 0 : FELoc, FEType), nullptr, prm);
        a.elementModuli(eMod);
        const bool jac = mode.find("Jacobian") != std::string::npos;
        const bool res = mode.find("Rhs") != std::string::npos;
        if (!jac && !res) throw Error(FEDD_ERR_ARG, "elasticity: assembleMode " + mode);
        if (res && !d_rep) throw Error(FEDD_ERR_ARG, "elasticity: the residual needs d_rep");
        if (d_rep && (int64_t)d_rep->size() != a.n_u()) throw Error(FEDD_ERR_ARG, "elasticity: d_rep size");
        if (jac) {
            if (!A.present[0][0] || A.block[0][0].nnz() == 0) a.pattern(FEDD_BLOCK_00, A.block[0][0]);
            A.present[0][0] = true;
        }
        if (res) {
            resVec.block.resize(1);
            resVec.block[0].assign((size_t)a.n_u(), 0.0);
        }
        a.assemble((jac ? FEDD_JACOBIAN : 0u) | (res ? FEDD_RESIDUAL : 0u), d_rep ? d_rep->data() : nullptr,
                   nullptr, jac ? &A.block[0][0] : nullptr, nullptr, nullptr,
                   res ? resVec.block[0].data() : nullptr, nullptr);
    }

    int device_;
    std::vector<Domain> domains_;
    std::map<std::string, std::unique_ptr<Assembler>> cache_;
};

// ----------------------------------------------------------- AssembleFE ----
// FEDDLib builds one AssembleFE object per element.  Here the objects built
// by one factory share an ElementBatch: the first assemble* call on any of
// them computes every element of the batch in one device call (a mesh of
// the batch's elements, each with its own nodes), and getJacobian()/getRHS()
// return that element's slice.  This is the compatibility path; the fast
// path is FE above.
class ElementBatch {
  public:
    // gn: the generalized-Newtonian element, its viscosity model read from
    // params' sublist("Material")
    ElementBatch(int problem, const ParameterList &params, int device, bool gn = false)
        : problem_(problem), params_(params_copy(params)), device_(device) {
        if (gn) vmodel_ = detail::viscosity_model(params, vprm_, vgmin_, true);
    }

    int problem() const { return problem_; }
    bool generalizedNewtonian() const { return vmodel_ >= 0; }
    int nodesPerElement() const { return problem_ == FEDD_LAPLACE ? npe_ : 10; }
    int dofsPerElement() const {
        return problem_ == FEDD_LAPLACE ? npe_ : problem_ == FEDD_NAVIER_STOKES ? 34 : 30;
    }

    int64_t add(const std::vector<std::array<double, 3>> &nodes) {
        if (asm_) throw Error(FEDD_ERR_STATE, "AssembleFE: batch already evaluated; build a new factory");
        if (problem_ == FEDD_LAPLACE) {
            if (nodes.size() != 4 && nodes.size() != 10) throw Error(FEDD_ERR_ARG, "Laplace: 4 or 10 nodes");
            if (n_ == 0) npe_ = (int)nodes.size();
            if ((int)nodes.size() != npe_) throw Error(FEDD_ERR_ARG, "AssembleFE: mixed element types in a batch");
        } else if (nodes.size() != 10) {
            throw Error(FEDD_ERR_ARG, "AssembleFE: P2 elements (10 nodes) expected");
        }
        for (auto &x : nodes) coords_.insert(coords_.end(), x.begin(), x.end());
        sol_.resize((size_t)(n_ + 1) * dofsPerElement(), 0.0);
        E_.push_back(params_.at<double>("Parameter", "E", -1.0));
        coeff_.push_back({{{1.0, 1.0}, {1.0, 1.0}}});
        lin_.push_back(params_.at<std::string>("General", "Linearization", "FixedPoint"));
        return n_++;
    }

    // AssembleFE_NonLinElas{,2}::updateParameter (AssembleFE_NonLinElas_def.hpp:175-180):
    // "E" sets the element's Young's modulus; other names, and the other
    // element types, keep the base class's no-op.  The engine assembles a
    // batch with one material, so evaluate() rejects a batch whose elements
    // carry different values.
    void setParameter(int64_t e, const std::string &type, double value) {
        if (type != "E" || (problem_ != FEDD_NONLINEAR_ELASTICITY && problem_ != FEDD_NONLINEAR_ELASTICITY2)) return;
        if (E_[(size_t)e] != value) fresh_ = false;
        E_[(size_t)e] = value;
    }
    // AssembleFE::changeLinearization (AssembleFE_decl.hpp:245): "Newton" adds
    // the Navier-Stokes W term (AssembleFENavierStokes_def.hpp:96-98); one
    // value per batch when it is evaluated, as for E.
    void setLinearization(int64_t e, const std::string &lin) {
        if (lin_[(size_t)e] != lin) fresh_ = false;
        lin_[(size_t)e] = lin;
    }
    // AssembleFENavierStokes::setCoeff (AssembleFENavierStokes_def.hpp:56-64):
    // the residual's block factors; one value per batch, as for E
    void setCoeff(int64_t e, const std::array<std::array<double, 2>, 2> &c) {
        if (problem_ != FEDD_NAVIER_STOKES) throw Error(FEDD_ERR_STATE, "setCoeff: Navier-Stokes elements only");
        if (coeff_[(size_t)e] != c) fresh_ = false;
        coeff_[(size_t)e] = c;
    }
    const std::vector<double> &solution() const { return sol_; }

    void setSolution(int64_t e, const std::vector<double> &s) {
        if ((int)s.size() != dofsPerElement()) throw Error(FEDD_ERR_ARG, "updateSolution: wrong size");
        std::copy(s.begin(), s.end(), sol_.begin() + (size_t)e * dofsPerElement());
        fresh_ = false;
    }

    void evaluate() {
        if (fresh_) return;
        const int nd = dofsPerElement();
        for (int64_t e = 1; e < n_; e++) {
            if (E_[(size_t)e] != E_[0])
                throw Error(FEDD_ERR_UNSUPPORTED, "AssembleFE: the elements of one batch carry different E");
            if (lin_[(size_t)e] != lin_[0])
                throw Error(FEDD_ERR_UNSUPPORTED, "AssembleFE: the elements of one batch carry different linearizations");
            if (coeff_[(size_t)e] != coeff_[0])
                throw Error(FEDD_ERR_UNSUPPORTED, "AssembleFE: the elements of one batch carry different coefficients");
        }
        if (asm_ && n_ > 0 && (E_[0] != made_E_ || lin_[0] != made_lin_)) asm_.reset();  // material or linearization changed
        if (!asm_) create();
        std::vector<double> u, p;
        if (problem_ != FEDD_LAPLACE) {  // element-local dofs -> the batch's node-wise vectors
            u.resize((size_t)n_ * 30);
            for (int64_t e = 0; e < n_; e++)
                for (int k = 0; k < 30; k++) u[(size_t)e * 30 + k] = sol_[(size_t)e * nd + k];
            if (problem_ == FEDD_NAVIER_STOKES) {
                p.resize((size_t)n_ * 4);
                for (int64_t e = 0; e < n_; e++)
                    for (int k = 0; k < 4; k++) p[(size_t)e * 4 + k] = sol_[(size_t)e * nd + 30 + k];
            }
        }
        if (problem_ == FEDD_NAVIER_STOKES && n_ > 0) asm_->coeff(coeff_[0]);
        K_.assign((size_t)n_ * nd * nd, 0.0);
        r_.assign((size_t)n_ * nd, 0.0);
        asm_->elementMatrices(u.empty() ? nullptr : u.data(), p.empty() ? nullptr : p.data(), 0, n_, K_.data(),
                              r_.data());
        fresh_ = true;
    }

    const double *jacobian(int64_t e) const { return K_.data() + (size_t)e * dofsPerElement() * dofsPerElement(); }
    const double *rhs(int64_t e) const { return r_.data() + (size_t)e * dofsPerElement(); }

  private:
    static ParameterList params_copy(const ParameterList &p) {
        ParameterList q;
        for (const char *k : {"Viscosity", "Density", "E", "Poisson Ratio"})
            if (p.findSublist("Parameter")) q.sublist("Parameter").set(k, p.at<double>("Parameter", k, -1.0));
        q.sublist("General").set("Linearization", p.at<std::string>("General", "Linearization", "FixedPoint"));
        return q;
    }
    void create() {
        Domain d;
        d.FEType = nodesPerElement() == 4 ? "P1" : "P2";
        d.coords = coords_;
        d.elements.resize((size_t)n_ * nodesPerElement());
        for (size_t k = 0; k < d.elements.size(); k++) d.elements[k] = (int32_t)k;
        Domain dp;
        fedd_params prm{};
        prm.problem = problem_;
        auto par = [&](const char *k, double def) {
            const double v = params_.at<double>("Parameter", k, -1.0);
            return v < 0 ? def : v;
        };
        prm.viscosity = par("Viscosity", 1.0);
        prm.density = par("Density", 1.0);
        made_E_ = n_ > 0 ? E_[0] : -1.0;
        made_lin_ = n_ > 0 ? lin_[0] : std::string("FixedPoint");
        prm.E = made_E_ < 0 ? par("E", 1000.0) : made_E_;
        prm.poisson_ratio = par("Poisson Ratio", 0.4);
        prm.linearization = made_lin_ == "Newton";
        if (problem_ == FEDD_NAVIER_STOKES) {
            dp.FEType = "P1";
            dp.coords.resize((size_t)n_ * 4 * 3);
            dp.elements.resize((size_t)n_ * 4);
            for (int64_t e = 0; e < n_; e++)
                for (int k = 0; k < 4; k++) {
                    dp.elements[(size_t)e * 4 + k] = (int32_t)(e * 4 + k);
                    for (int c = 0; c < 3; c++)
                        dp.coords[((size_t)e * 4 + k) * 3 + c] = coords_[((size_t)e * 10 + k) * 3 + c];
                }
        }
        asm_ = std::make_unique<Assembler>(d, problem_ == FEDD_NAVIER_STOKES ? &dp : nullptr, prm, device_);
        if (vmodel_ >= 0) asm_->viscosityLaw(vmodel_, vprm_, vgmin_);
    }

    int problem_;
    ParameterList params_;
    int device_;
    int npe_ = 10;
    int64_t n_ = 0;
    std::vector<double> coords_, sol_, K_, r_;
    std::vector<double> E_;          // per element (-1: the parameter list's)
    std::vector<std::string> lin_;   // per element
    std::vector<std::array<std::array<double, 2>, 2>> coeff_;  // per element
    double made_E_ = -1.0;           // what the current assembler was made with
    std::string made_lin_;
    std::unique_ptr<Assembler> asm_;
    bool fresh_ = false;
    int vmodel_ = -1;
    double vprm_[5] = {0, 0, 0, 0, 0}, vgmin_ = 1e-8;
};

class AssembleFE {
  public:
    AssembleFE(std::shared_ptr<ElementBatch> batch, int64_t index) : batch_(std::move(batch)), e_(index) {}

    // AssembleFE_decl.hpp:82, 94: compute (the whole batch, once per solution change)
    void assembleJacobian() { batch_->evaluate(); }
    void assembleRHS() { batch_->evaluate(); }
    // :89 -- a no-op for the element types of this path; the
    // generalized-Newtonian element throws (AssembleFEGeneralizedNewtonian_decl.hpp:58)
    void assembleJacobianBlock(int64_t i) {
        (void)i;
        if (batch_->generalizedNewtonian()) throw Error(FEDD_ERR_UNSUPPORTED, "assembleJacobianBlock: no implementation");
    }
    // :100, 112 -- row-major nd x nd (SmallMatrix order) and nd values
    std::vector<double> getJacobian() const {
        const int nd = batch_->dofsPerElement();
        return std::vector<double>(batch_->jacobian(e_), batch_->jacobian(e_) + (size_t)nd * nd);
    }
    std::vector<double> getRHS() const {
        const int nd = batch_->dofsPerElement();
        return std::vector<double>(batch_->rhs(e_), batch_->rhs(e_) + nd);
    }
    // :159 -- element-local solution in FEDDLib's order (velocity 3*i+d, then pressure)
    void updateSolution(const std::vector<double> &solution) { batch_->setSolution(e_, solution); }
    std::vector<double> getSolution() const {
        const int nd = batch_->dofsPerElement();
        const double *s = batch_->solution().data() + (size_t)e_ * nd;
        return std::vector<double>(s, s + nd);
    }
    // :131 (AssembleFE_NonLinElas_def.hpp:175-180) and :245
    void updateParameter(const std::string &type, double value) { batch_->setParameter(e_, type, value); }
    void changeLinearization(const std::string &linearization) { batch_->setLinearization(e_, linearization); }
    // AssembleFENavierStokes::setCoeff (Navier-Stokes elements)
    void setCoeff(const std::array<std::array<double, 2>, 2> &coeff) { batch_->setCoeff(e_, coeff); }
    // :136, :146 (AssembleFE_def.hpp:79-101): the time and Newton counters.
    // The engine recomputes every term on each evaluation, so the Newton
    // step only counts (FEDDLib's NS element caches its constant part at
    // step 0).
    void advanceInTime(double dt) {
        timeIncrement_ = dt;
        timeStep_ += dt;
    }
    double getTimeStep() const { return timeStep_; }
    double getTimeIncrement() const { return timeIncrement_; }
    void advanceNewtonStep() { newtonStep_++; }
    int getNewtonStep() const { return newtonStep_; }
    int64_t index() const { return e_; }

  private:
    std::shared_ptr<ElementBatch> batch_;
    int64_t e_;
    double timeStep_ = 0.0, timeIncrement_ = 0.0;
    int newtonStep_ = 0;
};

class AssembleFEFactory {
  public:
    explicit AssembleFEFactory(int device = 0) : device_(device) {}

    // AssembleFEFactory::build(problemType, flag, nodesRefConfig, params, tuple)
    // (AssembleFEFactory_def.hpp:16-70); keys "Laplace", "LinearElasticity",
    // "NonLinearElasticity", "NonLinearElasticity2", "NavierStokes",
    // "GeneralizedNewtonian" (the viscosity model from params'
    // sublist("Material")).  All elements built by one factory with one key
    // form one batch.
    std::shared_ptr<AssembleFE> build(const std::string &problemType, int flag,
                                      const std::vector<std::array<double, 3>> &nodesRefConfig,
                                      const ParameterList &params) {
        (void)flag;
        int problem = 0;
        if (problemType == "Laplace") problem = FEDD_LAPLACE;
        else if (problemType == "LinearElasticity") problem = FEDD_LINEAR_ELASTICITY;
        else if (problemType == "NonLinearElasticity") problem = FEDD_NONLINEAR_ELASTICITY;
        else if (problemType == "NonLinearElasticity2") problem = FEDD_NONLINEAR_ELASTICITY2;
        else if (problemType == "NavierStokes" || problemType == "GeneralizedNewtonian") problem = FEDD_NAVIER_STOKES;
        else throw Error(FEDD_ERR_UNSUPPORTED, "AssembleFEFactory: unknown problem type " + problemType);
        auto &b = batches_[problemType];
        if (!b) b = std::make_shared<ElementBatch>(problem, params, device_, problemType == "GeneralizedNewtonian");
        const int64_t e = b->add(nodesRefConfig);
        return std::make_shared<AssembleFE>(b, e);
    }

  private:
    int device_;
    std::map<std::string, std::shared_ptr<ElementBatch>> batches_;
};

}  // namespace feddgpu

#endif  // FEDDGPU_FE_HPP
