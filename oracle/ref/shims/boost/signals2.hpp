// Minimal stand-in for the part of Boost.Signals2 and Boost.Bind that the
// reference engine uses: signal<void()> with connect(F) and operator(), and
// boost::bind(&Class::method, object). Only for building the oracle.
#pragma once
#include <functional>
#include <utility>
#include <vector>

namespace boost {
namespace signals2 {
template <class Signature> class signal;

template <class R, class... A>
class signal<R(A...)> {
 public:
  struct connection {};
  template <class F>
  connection connect(F&& f) {
    slots_.emplace_back(std::forward<F>(f));
    return connection{};
  }
  void operator()(A... a) {
    for (auto& s : slots_) s(a...);
  }

 private:
  std::vector<std::function<R(A...)>> slots_;
};
}  // namespace signals2

template <class M, class C>
auto bind(M method, C* object) {
  return [method, object]() { return (object->*method)(); };
}
}  // namespace boost
