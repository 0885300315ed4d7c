#ifndef FINITEELEMENT_hpp
#define FINITEELEMENT_hpp
#include "feddlib/core/FEDDCore.hpp"
// Stand-in for FEDDLib's FiniteElement as the element classes use it: the
// outflow Neumann flag of an element and, on its boundary sub-elements, the
// surface data (normal, reference quadrature weights, global quadrature
// points, area scaling) that the generalized-Newtonian element's boundary
// integral reads.  A driver sets them as FEDDLib's Domain would.
namespace FEDD {
class Elements;
class FiniteElement {
  public:
    bool getNeumannBCElement() const { return neumann_; }
    void setNeumannBCElement(bool b) { neumann_ = b; }
    Teuchos::RCP<Elements> getSubElements() const { return sub_; }
    void setSubElements(const Teuchos::RCP<Elements> &s) { sub_ = s; }
    int numSubElements() const;
    std::vector<double> getSurfaceNormal() const { return normal_; }
    void setSurfaceNormal(const std::vector<double> &n) { normal_ = n; }
    std::vector<double> getQuadratureWeightsReference() const { return weights_; }
    void setQuadratureWeightsReference(const std::vector<double> &w) { weights_ = w; }
    std::vector<std::vector<double>> getQuadraturePointsGlobal() const { return points_; }
    void setQuadraturePointsGlobal(const std::vector<std::vector<double>> &q) { points_ = q; }
    double getElementScaling() const { return scaling_; }
    void setElementScaling(double s) { scaling_ = s; }

  private:
    bool neumann_ = false;
    Teuchos::RCP<Elements> sub_;
    std::vector<double> normal_, weights_;
    std::vector<std::vector<double>> points_;
    double scaling_ = 0.0;
};
class Elements {
  public:
    FiniteElement getElement(int i) const { return el_.at(i); }
    void addElement(const FiniteElement &f) { el_.push_back(f); }
    int numberElements() const { return (int)el_.size(); }

  private:
    std::vector<FiniteElement> el_;
};
inline int FiniteElement::numSubElements() const { return sub_.is_null() ? 0 : sub_->numberElements(); }
}  // namespace FEDD
#endif
