#ifndef MATRIX_hpp
#define MATRIX_hpp
#include "feddlib/core/FEDDCore.hpp"
using std::string;
using std::cout;
using std::endl;
namespace FEDD { template <class SC, class LO, class GO, class NO> class Matrix {}; }
#endif
