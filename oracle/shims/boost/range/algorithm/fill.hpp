// Oracle build shim: boost::range::fill.
#pragma once
#include <algorithm>
#include <iterator>
namespace boost { namespace range {
template <class R, class V> inline R& fill(R& r, const V& v) { std::fill(std::begin(r), std::end(r), v); return r; }
} }
