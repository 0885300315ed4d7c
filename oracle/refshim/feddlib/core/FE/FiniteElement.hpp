#ifndef FINITEELEMENT_hpp
#define FINITEELEMENT_hpp
#include "feddlib/core/FEDDCore.hpp"
// Stand-in for FEDDLib's FiniteElement as the element classes use it: no
// element is flagged for a Neumann outflow term, so the boundary integral of
// the generalized-Newtonian element is never taken and these accessors only
// need to exist.
namespace FEDD {
class Elements;
class FiniteElement {
  public:
    bool getNeumannBCElement() const { return false; }
    Teuchos::RCP<Elements> getSubElements() const { return Teuchos::RCP<Elements>(); }
    int numSubElements() const { return 0; }
    std::vector<double> getSurfaceNormal() const { return {}; }
    std::vector<double> getQuadratureWeightsReference() const { return {}; }
    std::vector<std::vector<double>> getQuadraturePointsGlobal() const { return {}; }
    double getElementScaling() const { return 0.0; }
};
class Elements {
  public:
    FiniteElement getElement(int) const { return FiniteElement(); }
};
}  // namespace FEDD
#endif
