// Shim (test infrastructure): boost::any as std::any, enough for the
// reference's ImageData.hpp to compile in the dataset fixture generator.
#pragma once
#include <any>
namespace boost {
using std::any;
using std::any_cast;
} // namespace boost
