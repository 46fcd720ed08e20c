// Oracle build shim: BOOST_STATIC_ASSERT on top of C++ static_assert.
#pragma once
#ifndef BOOST_STATIC_ASSERT
#define BOOST_STATIC_ASSERT(expr) static_assert(expr, #expr)
#endif
