#ifndef FINITEELEMENT_hpp
#define FINITEELEMENT_hpp
#include "feddlib/core/FEDDCore.hpp"
namespace FEDD { class FiniteElement {}; }
#endif
