// Oracle build shim: boost::ignore_unused.
#pragma once
namespace boost {
template <class... T> inline void ignore_unused(T const&...) {}
template <class... T> inline void ignore_unused() {}
} // namespace boost
