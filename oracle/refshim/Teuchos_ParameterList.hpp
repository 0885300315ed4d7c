#include "teuchos_stub.hpp"
