// Oracle build shim: the reference's s3vs/types.hpp names vl::Matrix3/4 only in
// type aliases; the hot-path headers built here never use their members.
#pragma once
namespace vl {
template <class T> class Matrix3 {};
template <class T> class Matrix4 {};
} // namespace vl
