// Stub of FEDDLib's FE class template, just large enough for member
// functions extracted from feddlib/core/FE/FE_def.hpp (extract_fe_members.py)
// to compile as they are: nh3d, epsilonTensor, applyBTinv, buildFullDPhi,
// fillMatrixArray, assemblyLinElasXDim, assemblyElasticityJacobianAceFEM,
// assemblyElasticityStressesAceFEM and assemblyRHS.  The domain, map, matrix and vector
// types below are this project's own minimal stand-ins: a one-rank domain
// given as arrays, an identity map, and a matrix that records
// insertGlobalValues calls.  Test infrastructure only.
#ifndef REF_FE_STUB_HPP
#define REF_FE_STUB_HPP
#include <cmath>
#include <map>

#include "feddlib/core/FE/Helper.hpp"
#include "feddlib/core/General/SmallMatrix.hpp"

namespace Teuchos {
enum ETransp { NO_TRANS, TRANS };
// column-major BLAS subset (reference semantics, plain loops)
template <class O, class T> struct BLAS {
    void GEMM(ETransp ta, ETransp tb, O m, O n, O k, T alpha, const T *A, O lda, const T *B, O ldb, T beta, T *C,
              O ldc) const {
        for (O j = 0; j < n; j++)
            for (O i = 0; i < m; i++) {
                T s = 0;
                for (O l = 0; l < k; l++) {
                    const T a = ta == NO_TRANS ? A[i + l * lda] : A[l + i * lda];
                    const T b = tb == NO_TRANS ? B[l + j * ldb] : B[j + l * ldb];
                    s += a * b;
                }
                C[i + j * ldc] = alpha * s + (beta == T(0) ? T(0) : beta * C[i + j * ldc]);
            }
    }
    void GEMV(ETransp ta, O m, O n, T alpha, const T *A, O lda, const T *x, O incx, T beta, T *y, O incy) const {
        const O ny = ta == NO_TRANS ? m : n, nx = ta == NO_TRANS ? n : m;
        for (O i = 0; i < ny; i++) {
            T s = 0;
            for (O l = 0; l < nx; l++) s += (ta == NO_TRANS ? A[i + l * lda] : A[l + i * lda]) * x[l * incx];
            y[i * incy] = alpha * s + (beta == T(0) ? T(0) : beta * y[i * incy]);
        }
    }
};
template <class T> struct ArrayRCP {
    T *p = nullptr;
    T &operator[](long long i) const { return p[i]; }
};
}  // namespace Teuchos

namespace FEDD {

struct RefElement {
    vec_int_Type nodes;
    int getNode(int i) const { return nodes.at(i); }
    const vec_int_Type &getVectorNodeList() const { return nodes; }
};
struct RefElements {
    std::vector<RefElement> el;
    int numberElements() const { return (int)el.size(); }
    const RefElement &getElement(int T) const { return el.at(T); }
};
struct RefMap {
    long long getGlobalElement(int i) const { return i; }
};
struct RefDomain {
    vec2D_int_ptr_Type elems;
    vec2D_dbl_ptr_Type points;
    Teuchos::RCP<RefElements> elemsC;
    vec2D_int_ptr_Type getElements() const { return elems; }
    Teuchos::RCP<RefElements> getElementsC() const { return elemsC; }
    vec2D_dbl_ptr_Type getPointsRepeated() const { return points; }
    Teuchos::RCP<const RefMap> getMapRepeated() const { return Teuchos::rcp(new RefMap()); }
};
// records insertGlobalValues as Tpetra would sum them (duplicates added)
struct RefMatrix {
    std::map<std::pair<long long, long long>, double> v;
    void insertGlobalValues(long long row, const std::vector<long long> &cols, const std::vector<double> &vals) {
        for (size_t k = 0; k < cols.size(); k++) v[{row, cols[k]}] += vals[k];
    }
    void fillComplete() {}
};
struct RefMultiVector {
    std::vector<double> d;
    int getNumVectors() const { return 1; }
    Teuchos::ArrayRCP<const double> getData(int) const { return {d.data()}; }
    Teuchos::ArrayRCP<double> getDataNonConst(int) { return {d.data()}; }
};

template <class SC, class LO, class GO, class NO> class FE {
  public:
    typedef Teuchos::RCP<RefMatrix> MatrixPtr_Type;
    typedef Teuchos::RCP<RefMultiVector> MultiVectorPtr_Type;
    typedef Teuchos::RCP<const RefMap> MapConstPtr_Type;
    typedef Teuchos::RCP<RefElements> ElementsPtr_Type;
    enum VarType { Std = 0, Grad = 1 };  // as FE declares it (FE_decl.hpp:51)
    std::vector<Teuchos::RCP<RefDomain>> domainVec_;
    int checkFE(int, std::string) { return 0; }

    void nh3d(double *v, double(*E), double(*Nu), double **F, double **Pmat, double ****Amat);
    void mr3d(double *, double *, double *, double *, double **, double **, double ****) {
        TEUCHOS_TEST_FOR_EXCEPTION(true, std::logic_error, "Mooney-Rivlin is not part of the checker");
    }
    void epsilonTensor(vec_dbl_Type &basisValues, SmallMatrix<SC> &epsilonValues, int activeDof);
    void applyBTinv(vec3D_dbl_ptr_Type &dPhiIn, vec3D_dbl_Type &dPhiOut, SmallMatrix<SC> &Binv);
    void buildFullDPhi(vec3D_dbl_ptr_Type dPhi, Teuchos::Array<SmallMatrix<double>> &dPhiMat);
    void fillMatrixArray(SmallMatrix<double> &matIn, double *matArrayOut, std::string order, int offset = 0);
    void assemblyLinElasXDim(int dim, std::string FEType, MatrixPtr_Type &A, double lambda, double mu,
                             bool callFillComplete = true);
    void assemblyElasticityJacobianAceFEM(int dim, std::string FEType, MatrixPtr_Type &A, MultiVectorPtr_Type u,
                                          std::string material_model, double E, double nu, double C,
                                          bool callFillComplete = true);
    void assemblyElasticityStressesAceFEM(int dim, std::string FEType, MultiVectorPtr_Type &f, MultiVectorPtr_Type u,
                                          std::string material_model, double E, double nu, double C,
                                          bool callFillComplete = true);
    void assemblyRHS(int dim, std::string FEType, MultiVectorPtr_Type a, std::string fieldType, RhsFunc_Type func,
                     std::vector<SC> &funcParameter);
};

}  // namespace FEDD
#endif
