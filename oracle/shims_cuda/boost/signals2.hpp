// Reference-CUDA build shim (test infrastructure only): the reference's render
// translation unit is compiled here for its device code alone (a cubin), so
// its host-side property-change plumbing only has to type-check.
#pragma once
#include <functional>
#include <map> // the real header pulls in <map>; the reference's VsControllerInput.hpp relies on it
namespace boost {
namespace signals2 {
class connection {
public:
    void disconnect() const {}
};
template <class Sig> class signal;
template <class R, class... A> class signal<R(A...)> {
public:
    template <class F> connection connect(F&&) { return {}; }
    void disconnect(const connection&) {}
    void operator()(A...) const {}
};
} // namespace signals2
} // namespace boost
