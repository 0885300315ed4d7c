// Drives FEDDLib's own element classes, compiled from the reference sources
// where they lie (see build_ref.sh), so the FP64 restatement can be checked
// against the reference itself.  Test infrastructure only.
#include "feddlib/core/AceFemAssembly/AssembleFE_def.hpp"
#include "feddlib/core/AceFemAssembly/specific/AssembleFE_Laplace_def.hpp"
#include "feddlib/core/AceFemAssembly/specific/AssembleFENavierStokes_def.hpp"
#include "feddlib/core/General/InputToOutputMappingClass_def.hpp"
#include "feddlib/core/General/DifferentiableFuncClass_def.hpp"
#include "feddlib/core/AceFemAssembly/specific/GeneralizedNewtonianModels/CarreauYasuda_def.hpp"
#include "feddlib/core/AceFemAssembly/specific/GeneralizedNewtonianModels/PowerLaw_def.hpp"
#include "feddlib/core/AceFemAssembly/specific/GeneralizedNewtonianModels/Dimless_Carreau_def.hpp"
#include "feddlib/core/AceFemAssembly/specific/GeneralizedNewtonianModels/GNF_Const_Hematocrit_def.hpp"
#include "feddlib/core/AceFemAssembly/specific/AssembleFEGeneralizedNewtonian_decl.hpp"
#include "feddlib/core/AceFemAssembly/specific/AssembleFEGeneralizedNewtonian_def.hpp"

using namespace FEDD;
typedef AssembleFENavierStokes<double, int, long long, default_no> NS;
typedef AssembleFE_Laplace<double, int, long long, default_no> LAP;

// The element constructors are protected (only the factory may call them);
// a derived class with a public constructor is the minimal way in.
struct NSElem : NS {
    NSElem(vec2D_dbl_Type n, ParameterListPtr_Type p, tuple_disk_vec_ptr_Type t) : NS(0, n, p, t) {}
};
typedef AssembleFEGeneralizedNewtonian<double, int, long long, default_no> GN;
struct GNElem : GN {
    GNElem(vec2D_dbl_Type n, ParameterListPtr_Type p, tuple_disk_vec_ptr_Type t) : GN(0, n, p, t) {}
};
struct LapElem : LAP {
    LapElem(vec2D_dbl_Type n, ParameterListPtr_Type p, tuple_disk_vec_ptr_Type t) : LAP(0, n, p, t) {}
    // assembleRHS assigns through rhsVec_, which the base constructor leaves null
    void allocRHS(int n) { this->rhsVec_ = Teuchos::rcp(new vec_dbl_Type(n, 0.0)); }
};

static vec2D_dbl_Type nodes_of(const double *x, int n) {
    vec2D_dbl_Type v(n, vec_dbl_Type(3));
    for (int i = 0; i < n; i++)
        for (int d = 0; d < 3; d++) v[i][d] = x[3 * i + d];
    return v;
}

extern "C" {

// Helper::getQuadratureValues (dim 3, P-type); returns the number of points
int ref_quad(int degree, double *pts, double *w) {
    vec2D_dbl_ptr_Type qp;
    vec_dbl_ptr_Type qw = Teuchos::rcp(new vec_dbl_Type(0));
    Helper::getQuadratureValues(3, degree, qp, qw, "P2");
    for (size_t i = 0; i < qw->size(); i++) {
        w[i] = (*qw)[i];
        for (int d = 0; d < 3; d++) pts[3 * i + d] = (*qp)[i][d];
    }
    return (int)qw->size();
}

// Helper::getDPhi / getPhi at the rule for `degree`
int ref_dphi(const char *fe, int degree, double *dphi, double *phi) {
    vec3D_dbl_ptr_Type D;
    vec2D_dbl_ptr_Type P;
    vec_dbl_ptr_Type w = Teuchos::rcp(new vec_dbl_Type(0));
    Helper::getDPhi(D, w, 3, fe, degree);
    Helper::getPhi(P, w, 3, fe, degree);
    int nq = (int)D->size(), nb = (int)(*D)[0].size();
    for (int q = 0; q < nq; q++)
        for (int i = 0; i < nb; i++) {
            phi[q * nb + i] = (*P)[q][i];
            for (int d = 0; d < 3; d++) dphi[(q * nb + i) * 3 + d] = (*D)[q][i][d];
        }
    return nq;
}

// AssembleFENavierStokes: assembleJacobian (newtonStep 0) then assembleRHS.
// sol = 30 velocity (node-wise) + 4 pressure values; J is 34x34 row-major.
int ref_ns_element(const double *x10, const double *sol, double visc, double dens, int newton,
                   double *J, double *rhs) {
    try {
        ParameterListPtr_Type p = Teuchos::rcp(new Teuchos::ParameterList());
        p->sublist("Parameter").set("Dimension", 3);
        p->sublist("Parameter").set("Viscosity", visc);
        p->sublist("Parameter").set("Density", dens);
        p->sublist("General").set("Linearization", newton ? "Newton" : "FixedPoint");
        tuple_disk_vec_ptr_Type t = Teuchos::rcp(new tuple_disk_vec_Type());
        t->push_back(tuple_ssii_Type("Velocity", "P2", 3, 10));
        t->push_back(tuple_ssii_Type("Pressure", "P1", 1, 4));
        NSElem e(nodes_of(x10, 10), p, t);
        e.updateSolution(vec_dbl_Type(sol, sol + 34));
        e.assembleJacobian();
        auto Jm = e.getJacobian();
        for (int i = 0; i < 34; i++)
            for (int j = 0; j < 34; j++) J[34 * i + j] = (*Jm)[i][j];
        e.assembleRHS();
        auto r = e.getRHS();
        for (int i = 0; i < 34; i++) rhs[i] = (*r)[i];
        return 0;
    } catch (const std::exception &ex) {
        return 1;
    }
}

// AssembleFENavierStokes with FE::assemblyNavierStokes' coeff handed over by
// setCoeff (AssembleFENavierStokes_def.hpp:56-64): assembleJacobian (which
// caches the constant part), then assembleRHS, r = (coeff .* ANB) x.
// coeff row-major {c_uu, c_up, c_pu, c_pp}.
int ref_ns_element_coeff(const double *x10, const double *sol, double visc, double dens, const double *coeff,
                         double *rhs) {
    try {
        ParameterListPtr_Type p = Teuchos::rcp(new Teuchos::ParameterList());
        p->sublist("Parameter").set("Dimension", 3);
        p->sublist("Parameter").set("Viscosity", visc);
        p->sublist("Parameter").set("Density", dens);
        tuple_disk_vec_ptr_Type t = Teuchos::rcp(new tuple_disk_vec_Type());
        t->push_back(tuple_ssii_Type("Velocity", "P2", 3, 10));
        t->push_back(tuple_ssii_Type("Pressure", "P1", 1, 4));
        NSElem e(nodes_of(x10, 10), p, t);
        e.updateSolution(vec_dbl_Type(sol, sol + 34));
        e.assembleJacobian();
        SmallMatrix<double> c(2);
        c[0][0] = coeff[0]; c[0][1] = coeff[1];
        c[1][0] = coeff[2]; c[1][1] = coeff[3];
        e.setCoeff(c);
        e.assembleRHS();
        auto r = e.getRHS();
        for (int i = 0; i < 34; i++) rhs[i] = (*r)[i];
        return 0;
    } catch (const std::exception &ex) {
        return 1;
    }
}

// AssembleFEGeneralizedNewtonian: assembleJacobian (newtonStep 0) then
// assembleRHS.  model 0 "Carreau-Yasuda" (mp: lambda, n, eta0, etaInf, a),
// 1 "Power-Law" (mp: K, n, eta_max, eta_min), 2 "Dimless-Carreau"
// (mp: lambda, n, eta0, etaInf, reference viscosity).
static int gn_element(const double *x10, const double *face, const double *sol, int model, const double *mp,
                      double dens, int newton, double *J, double *rhs, bool fixed_point_matrix = false) {
    try {
        ParameterListPtr_Type p = Teuchos::rcp(new Teuchos::ParameterList());
        p->sublist("Parameter").set("Dimension", 3);
        p->sublist("Parameter").set("Viscosity", 1.0);
        p->sublist("Parameter").set("Density", dens);
        p->sublist("General").set("Linearization", newton ? "Newton" : "FixedPoint");
        Teuchos::ParameterList &m = p->sublist("Material");
        if (model == 0) {
            m.set("ShearThinningModel", "Carreau-Yasuda");
            m.set("CharacteristicTime_Lambda", mp[0]);
            m.set("FluidIndex_n", mp[1]);
            m.set("ZeroShearRateViscosity_eta0", mp[2]);
            m.set("InftyShearRateViscosity_etaInfty", mp[3]);
            m.set("InflectionPoint_a", mp[4]);
        } else if (model == 1) {
            m.set("ShearThinningModel", "Power-Law");
            m.set("PowerLawParameter K", mp[0]);
            m.set("PowerLaw index n", mp[1]);
            m.set("Numerical_ZeroShearRateViscosity", mp[2]);
            m.set("Numerical_InftyShearRateViscosity", mp[3]);
        } else {
            m.set("ShearThinningModel", "Dimless-Carreau");
            m.set("Dimless_CharacteristicTime_Lambda", mp[0]);
            m.set("Carreau_FluidIndex_n", mp[1]);
            m.set("Dimless_ZeroShearRateViscosity_eta0", mp[2]);
            m.set("Dimless_InftyShearRateViscosity_etaInfty", mp[3]);
            m.set("Reference_Viscosity", mp[4]);
        }
        tuple_disk_vec_ptr_Type t = Teuchos::rcp(new tuple_disk_vec_Type());
        t->push_back(tuple_ssii_Type("Velocity", "P2", 3, 10));
        t->push_back(tuple_ssii_Type("Pressure", "P1", 1, 4));
        GNElem e(nodes_of(x10, 10), p, t);
        FiniteElement fe;
        if (face) {
            // the element is flagged for the outflow Neumann term: one
            // boundary sub-element carrying the surface data that
            // Domain::setSurfaceNormalsForFE and
            // Domain::setSurfaceQuadraturePointsWeights(flag, 8) attach
            // (Domain_def.hpp:1148-1180, 1214-1255), computed by the same
            // Helper and SmallMatrix routines they call
            vec2D_dbl_ptr_Type pts = Teuchos::rcp(new vec2D_dbl_Type(nodes_of(face, 3)));
            vec_int_Type ids = {0, 1, 2};
            vec_dbl_Type nv(3, 1.0);
            double nn = 1.0;
            Helper::computeSurfaceNormal(3, pts, ids, nv, nn);
            for (int k = 0; k < 3; k++) nv[k] *= 1.0 / nn;
            SmallMatrix<double> Bs(3);
            vec_dbl_Type bs(3);
            Helper::buildTransformationSurface(ids, pts, Bs, bs, "P2");
            vec_dbl_Type qw(7);
            vec2D_dbl_Type qp(7, vec_dbl_Type(3));
            Helper::getQuadraturePointsOnSurfaceInGlobalSpace(3, "P2", qw, qp, vec_LO_Type(ids.begin(), ids.end()), pts);
            FiniteElement sub;
            sub.setNeumannBCElement(true);
            sub.setSurfaceNormal(nv);
            sub.setElementScaling(Bs.computeScaling());
            sub.setQuadratureWeightsReference(qw);
            sub.setQuadraturePointsGlobal(qp);
            Teuchos::RCP<Elements> subs = Teuchos::rcp(new Elements());
            subs->addElement(sub);
            fe.setSubElements(subs);
            fe.setNeumannBCElement(true);
        }
        e.setFiniteElement(fe);
        e.updateSolution(vec_dbl_Type(sol, sol + 34));
        Teuchos::RCP<SmallMatrix<double>> Jm;
        if (fixed_point_matrix) {
            // FE::assemblyNavierStokes with assembleMode "FixedPoint"
            // (FE_def.hpp:1178-1191): assembleFixedPoint, getFixedPointMatrix
            e.assembleFixedPoint();
            Jm = e.getFixedPointMatrix();
        } else {
            e.assembleJacobian();
            Jm = e.getJacobian();
        }
        for (int i = 0; i < 34; i++)
            for (int j = 0; j < 34; j++) J[34 * i + j] = (*Jm)[i][j];
        e.assembleRHS();
        auto r = e.getRHS();
        for (int i = 0; i < 34; i++) rhs[i] = (*r)[i];
        return 0;
    } catch (const std::exception &ex) {
        return 1;
    }
}

int ref_gn_element(const double *x10, const double *sol, int model, const double *mp, double dens, int newton,
                   double *J, double *rhs) {
    return gn_element(x10, nullptr, sol, model, mp, dens, newton, J, rhs);
}

// The same element flagged for the outflow Neumann term on one face, given by
// its three vertex coordinates face[0..8] in the face's node order.
int ref_gn_element_outflow(const double *x10, const double *face, const double *sol, int model, const double *mp,
                           double dens, int newton, double *J, double *rhs) {
    return gn_element(x10, face, sol, model, mp, dens, newton, J, rhs);
}

// The fixed-point matrix of the element (assembleFixedPoint + getFixedPointMatrix,
// what FE::assemblyNavierStokes takes in assembleMode "FixedPoint"), with the
// outflow term on one face when face is not NULL, and the residual.
int ref_gn_element_fixed_point(const double *x10, const double *face, const double *sol, int model,
                               const double *mp, double dens, double *J, double *rhs) {
    return gn_element(x10, face, sol, model, mp, dens, 0, J, rhs, true);
}

// AssembleFE_Laplace: assembleJacobian and assembleRHS with f = fval.
int ref_laplace_element(const char *fe, const double *x, double fval, double *K, double *rhs) {
    try {
        int n = (fe[1] == '1') ? 4 : 10;
        ParameterListPtr_Type p = Teuchos::rcp(new Teuchos::ParameterList());
        p->sublist("Parameter").set("Dimension", 3);
        tuple_disk_vec_ptr_Type t = Teuchos::rcp(new tuple_disk_vec_Type());
        t->push_back(tuple_ssii_Type("Laplace", fe, 1, n));
        LapElem e(nodes_of(x, n), p, t);
        e.assembleJacobian();
        auto Km = e.getJacobian();
        for (int i = 0; i < n; i++)
            for (int j = 0; j < n; j++) K[n * i + j] = (*Km)[i][j];
        e.addRHSFunc([fval](double *, double *res, double *) { res[0] = fval; res[1] = fval; res[2] = fval; });
        e.updateSolution(vec_dbl_Type(n, 0.0));
        e.allocRHS(n);
        e.assembleRHS();
        auto r = e.getRHS();
        for (int i = 0; i < n; i++) rhs[i] = (*r)[i];
        return 0;
    } catch (const std::exception &ex) {
        return 1;
    }
}
}
