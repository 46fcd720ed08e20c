// Oracle build shim: boost::range::transform.
#pragma once
#include <algorithm>
#include <iterator>
namespace boost { namespace range {
template <class R, class O, class F> inline O transform(const R& r, O out, F f) { return std::transform(std::begin(r), std::end(r), out, f); }
template <class R, class O, class F> inline O transform(R& r, O out, F f) { return std::transform(std::begin(r), std::end(r), out, f); }
} }
