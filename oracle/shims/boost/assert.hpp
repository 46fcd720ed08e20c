// Oracle build shim (test infrastructure only): minimal stand-in for the Boost
// header of the same name, written for compiling the reference's header-only
// hot-path code without Boost installed.
#pragma once
#include <cassert>
#ifndef BOOST_ASSERT
#define BOOST_ASSERT(expr) assert(expr)
#endif
#ifndef BOOST_ASSERT_MSG
#define BOOST_ASSERT_MSG(expr, msg) assert((expr) && (msg))
#endif
