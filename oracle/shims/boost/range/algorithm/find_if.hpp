// Shim (test infrastructure): boost::range::find_if over a range.
#pragma once
#include <algorithm>
#include <iterator>
namespace boost {
namespace range {
template <class R, class P> auto find_if(R& r, P p) { return std::find_if(std::begin(r), std::end(r), p); }
template <class R, class P> auto find_if(const R& r, P p) { return std::find_if(std::begin(r), std::end(r), p); }
} // namespace range
using range::find_if;
} // namespace boost
