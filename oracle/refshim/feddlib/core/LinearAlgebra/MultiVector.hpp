#ifndef MULTIVECTOR_hpp
#define MULTIVECTOR_hpp
#include "feddlib/core/FEDDCore.hpp"
namespace FEDD { template <class SC, class LO, class GO, class NO> class MultiVector {}; }
#endif
