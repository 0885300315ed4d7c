#include <functional>
namespace boost { template <class F> using function = std::function<F>; }
