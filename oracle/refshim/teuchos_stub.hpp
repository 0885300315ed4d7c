// Minimal stand-ins for the Teuchos types FEDDLib's element classes use.
#ifndef TEUCHOS_STUB_HPP
#define TEUCHOS_STUB_HPP
#include <map>
#include <memory>
#include <sstream>
#include <stdexcept>
#include <string>
#include <vector>
#include <limits>
#include <functional>

#define TEUCHOS_TEST_FOR_EXCEPTION(cond, Exc, msg)                     \
    do { if (cond) { std::ostringstream os_; os_ << msg;               \
                     throw Exc(os_.str()); } } while (0)

namespace Teuchos {
template <class T> class RCP {
  public:
    RCP() {}
    RCP(std::nullptr_t) {}
    RCP(int) {}
    explicit RCP(T *p, bool owns = true) {
        if (owns) p_.reset(p); else p_ = std::shared_ptr<T>(p, [](T *) {});
    }
    template <class U> RCP(const RCP<U> &o) : p_(o.sp()) {}
    T *operator->() const { return p_.get(); }
    T &operator*() const { return *p_; }
    T *get() const { return p_.get(); }
    void reset(T *p = nullptr) { p_.reset(p); }
    bool is_null() const { return !p_; }
    const std::shared_ptr<T> &sp() const { return p_; }
    explicit RCP(std::shared_ptr<T> p) : p_(std::move(p)) {}
  private:
    std::shared_ptr<T> p_;
};
template <class T> RCP<T> rcp(T *p) { return RCP<T>(p); }
template <class T, class U> RCP<T> rcp_dynamic_cast(const RCP<U> &o) {
    return RCP<T>(std::dynamic_pointer_cast<T>(o.sp()));
}
template <class T> RCP<T> rcpFromRef(T &r) { return RCP<T>(&r, false); }

template <class T> class Array : public std::vector<T> {
  public:
    using std::vector<T>::vector;
    std::vector<T> &operator()() { return *this; }
};

template <class T> struct ScalarTraits {
    static T zero() { return T(0); }
    static T one() { return T(1); }
    static T eps() { return std::numeric_limits<T>::epsilon(); }
};

class ParameterList {
  public:
    ParameterList &sublist(const std::string &n) {
        auto &p = subs_[n];
        if (!p) p = std::make_shared<ParameterList>();
        return *p;
    }
    template <class T> T get(const std::string &n, T def) {
        auto it = d_.find(n);
        return it == d_.end() ? def : T(it->second);
    }
    std::string get(const std::string &n, const char *def) {
        auto it = s_.find(n);
        return it == s_.end() ? std::string(def) : it->second;
    }
    bool get(const std::string &n, bool def) {
        auto it = d_.find(n);
        return it == d_.end() ? def : it->second != 0.0;
    }
    void set(const std::string &n, double v) { d_[n] = v; }
    void set(const std::string &n, int v) { d_[n] = v; }
    void set(const std::string &n, const std::string &v) { s_[n] = v; }
    void set(const std::string &n, const char *v) { s_[n] = v; }
  private:
    std::map<std::string, double> d_;
    std::map<std::string, std::string> s_;
    std::map<std::string, std::shared_ptr<ParameterList>> subs_;
};
class Time {};
class TimeMonitor {};
class CommandLineProcessor {};
}  // namespace Teuchos
#endif
