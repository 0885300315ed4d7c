#ifndef DEFAULTTYPEDEFS_hpp
#define DEFAULTTYPEDEFS_hpp
#include "teuchos_stub.hpp"
struct stub_default_node {};
typedef double default_sc;
typedef int default_lo;
typedef long long default_go;
typedef stub_default_node default_no;
#endif
