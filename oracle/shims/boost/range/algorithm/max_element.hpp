// Oracle build shim: boost::range::max_element.
#pragma once
#include <algorithm>
#include <iterator>
namespace boost { namespace range {
template <class R> inline auto max_element(R& r) { return std::max_element(std::begin(r), std::end(r)); }
template <class R, class P> inline auto max_element(R& r, P p) { return std::max_element(std::begin(r), std::end(r), p); }
} }
