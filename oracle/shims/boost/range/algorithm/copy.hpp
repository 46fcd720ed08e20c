// Oracle build shim: boost::range::copy.
#pragma once
#include <algorithm>
#include <iterator>
namespace boost { namespace range {
template <class R, class O> inline O copy(const R& r, O out) { return std::copy(std::begin(r), std::end(r), out); }
} }
