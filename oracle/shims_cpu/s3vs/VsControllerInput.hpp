// Oracle build shim: the only name ColorTransferFunction.hpp needs from the
// reference's VsControllerInput.hpp is the control-point map type
// (VsControllerInput.hpp:84); the property classes behind it need
// boost::signals2 and silver_bullets, which are not installed.
#pragma once
#include "s3vs/types.hpp"
#include <cstring>
#include <map>
namespace s3vs {
using ColorTransferFunction = std::map<s3dmm::real_type, Vec4r>;
} // namespace s3vs
