// Runs FE member functions extracted from the reference's FE_def.hpp
// (extract_fe_members.py -> oracle/_ref/fe_members.inc) on a given P2 mesh
// and hands back the assembled values, so the oracle's elasticity elements
// can be checked against the reference's own classic elasticity code:
// FE::assemblyLinElasXDim (linear elasticity with lambda, mu) and
// FE::assemblyElasticityJacobianAceFEM / assemblyElasticityStressesAceFEM
// with "Neo-Hooke" (the AceGen law nh3d).  Test infrastructure only.
#include "ref_fe_stub.hpp"
#include "feddlib/core/FE/sms.hpp"

namespace FEDD {
using std::cout;
using std::endl;
#include "fe_members.inc"
}  // namespace FEDD

using namespace FEDD;
typedef FE<double, int, long long, default_no> FEd;

static void make_domain(FEd &fe, int nn, const double *xyz, int ne, const int *conn, int npe = 10) {
    auto d = Teuchos::rcp(new RefDomain());
    d->points = Teuchos::rcp(new vec2D_dbl_Type(nn, vec_dbl_Type(3)));
    for (int i = 0; i < nn; i++)
        for (int k = 0; k < 3; k++) (*d->points)[i][k] = xyz[3 * i + k];
    d->elems = Teuchos::rcp(new vec2D_int_Type(ne, vec_int_Type(npe)));
    d->elemsC = Teuchos::rcp(new RefElements());
    d->elemsC->el.resize(ne);
    for (int e = 0; e < ne; e++) {
        for (int a = 0; a < npe; a++) (*d->elems)[e][a] = conn[npe * e + a];
        d->elemsC->el[e].nodes = (*d->elems)[e];
    }
    fe.domainVec_.push_back(d);
}

// The source functions of the load-vector check, FEDDLib's RhsFunc_Type
// signature f(x, res, parameters): a scalar one and a vector one.  The
// reference also calls the function once, before its element loop, with a
// pointer to a single double, so these read the first coordinate only.
static void rhs_scalar(double *x, double *res, double *par) { res[0] = std::sin(3.0 * x[0]) + par[0]; }
static void rhs_vector(double *x, double *res, double *par) {
    res[0] = x[0] * x[0];
    res[1] = 2.0 * x[0] * par[0];
    res[2] = 1.0 + x[0];
}

static int to_coo(const RefMatrix &A, long long *rows, long long *cols, double *vals, int cap) {
    int k = 0;
    for (const auto &kv : A.v) {
        if (k >= cap) return -1;
        rows[k] = kv.first.first;
        cols[k] = kv.first.second;
        vals[k] = kv.second;
        k++;
    }
    return k;
}

extern "C" {

// FE::assemblyLinElasXDim on a P2 mesh: the assembled matrix as sorted COO
// (row, col ascending); returns the entry count or -1.
int ref_linelas_xdim(int nn, const double *xyz, int ne, const int *conn, double lambda, double mu, long long *rows,
                     long long *cols, double *vals, int cap) {
    try {
        FEd fe;
        make_domain(fe, nn, xyz, ne, conn);
        auto A = Teuchos::rcp(new RefMatrix());
        fe.assemblyLinElasXDim(3, "P2", A, lambda, mu, true);
        return to_coo(*A, rows, cols, vals, cap);
    } catch (...) {
        return -1;
    }
}

// FE::assemblyElasticityJacobianAceFEM and assemblyElasticityStressesAceFEM
// with "Neo-Hooke" (nh3d) at displacement u (3 per node): matrix as sorted
// COO, stress vector f (3 per node); returns the entry count or -1.
int ref_nh3d_acefem(int nn, const double *xyz, int ne, const int *conn, const double *u, double E, double nu,
                    long long *rows, long long *cols, double *vals, int cap, double *f) {
    try {
        FEd fe;
        make_domain(fe, nn, xyz, ne, conn);
        auto A = Teuchos::rcp(new RefMatrix());
        auto U = Teuchos::rcp(new RefMultiVector());
        U->d.assign(u, u + 3 * nn);
        auto Fv = Teuchos::rcp(new RefMultiVector());
        Fv->d.assign(3 * nn, 0.0);
        fe.assemblyElasticityJacobianAceFEM(3, "P2", A, U, "Neo-Hooke", E, nu, 1.0, true);
        fe.assemblyElasticityStressesAceFEM(3, "P2", Fv, U, "Neo-Hooke", E, nu, 1.0, true);
        for (int i = 0; i < 3 * nn; i++) f[i] = Fv->d[i];
        return to_coo(*A, rows, cols, vals, cap);
    } catch (...) {
        return -1;
    }
}

// FE::assemblyRHS with rhs_scalar (ncomp 1, "Scalar") or rhs_vector (3,
// "Vector") on a P1 (npe 4) or P2 (npe 10) mesh: the load vector into out
// (ncomp per node); parameters {0.5, degree 0}.  Returns 0, or -1.
int ref_assembly_rhs(int npe, int nn, const double *xyz, int ne, const int *conn, int ncomp, double *out) {
    try {
        FEd fe;
        make_domain(fe, nn, xyz, ne, conn, npe);
        auto a = Teuchos::rcp(new RefMultiVector());
        a->d.assign((size_t)nn * ncomp, 0.0);
        std::vector<double> par = {0.5, 0.0};
        fe.assemblyRHS(3, npe == 4 ? "P1" : "P2", a, ncomp == 1 ? "Scalar" : "Vector",
                       ncomp == 1 ? RhsFunc_Type(rhs_scalar) : RhsFunc_Type(rhs_vector), par);
        for (size_t i = 0; i < a->d.size(); i++) out[i] = a->d[i];
        return 0;
    } catch (...) {
        return -1;
    }
}

// nh3d at one deformation gradient F (row-major 3x3): P and A (81, A[i][j][k][l])
void ref_nh3d(double E, double nu, const double *F9, double *P9, double *A81) {
    FEd fe;
    double v[466];
    double Fr[3][3], Pr[3][3], Ar[3][3][3][3];
    double *Fp[3], *Pp[3], **Ap2[3][3], *Ap1[3][3][3], ***Ap3[3], ****A = Ap3;
    for (int i = 0; i < 3; i++) {
        Fp[i] = Fr[i];
        Pp[i] = Pr[i];
        for (int j = 0; j < 3; j++) {
            Fr[i][j] = F9[3 * i + j];
            for (int k = 0; k < 3; k++) Ap1[i][j][k] = Ar[i][j][k];
            Ap2[i][j] = Ap1[i][j];
        }
        Ap3[i] = Ap2[i];
    }
    fe.nh3d(v, &E, &nu, Fp, Pp, A);
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) {
            P9[3 * i + j] = Pr[i][j];
            for (int k = 0; k < 3; k++)
                for (int l = 0; l < 3; l++) A81[((3 * i + j) * 3 + k) * 3 + l] = Ar[i][j][k][l];
        }
}

}  // extern "C"
