// Reference-CUDA build shim (test infrastructure only): the VisualizationLibrary
// vector/matrix names the reference's render unit uses in host code.  Only its
// device code is kept (a cubin), so these are plain, untuned implementations.
#pragma once
#include <cmath>
namespace vl {
template <class T> struct Vector3 {
    T v[3] = {0, 0, 0};
    Vector3() = default;
    Vector3(T x, T y, T z) : v{x, y, z} {}
    T& operator[](int i) { return v[i]; }
    const T& operator[](int i) const { return v[i]; }
    T x() const { return v[0]; }
    T y() const { return v[1]; }
    T z() const { return v[2]; }
    T length() const { return std::sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]); }
    Vector3& normalize() { T l = length(); if (l > 0) { v[0] /= l; v[1] /= l; v[2] /= l; } return *this; }
    Vector3 operator*(T s) const { return {v[0] * s, v[1] * s, v[2] * s}; }
    Vector3 operator-() const { return {-v[0], -v[1], -v[2]}; }
    Vector3 operator+(const Vector3& o) const { return {v[0] + o.v[0], v[1] + o.v[1], v[2] + o.v[2]}; }
    Vector3 operator-(const Vector3& o) const { return {v[0] - o.v[0], v[1] - o.v[1], v[2] - o.v[2]}; }
};
template <class T> struct Vector4 {
    T v[4] = {0, 0, 0, 0};
    Vector4() = default;
    Vector4(T x, T y, T z, T w) : v{x, y, z, w} {}
    T& operator[](int i) { return v[i]; }
    const T& operator[](int i) const { return v[i]; }
    T x() const { return v[0]; }
    T y() const { return v[1]; }
    T z() const { return v[2]; }
    T w() const { return v[3]; }
};
template <class T> struct Matrix3 {
    T e[3][3] = {};
    Matrix3 operator-() const
    {
        Matrix3 m;
        for (int c = 0; c < 3; ++c)
            for (int r = 0; r < 3; ++r) m.e[c][r] = -e[c][r];
        return m;
    }
    Vector3<T> operator*(const Vector3<T>& x) const
    {
        Vector3<T> r;
        for (int i = 0; i < 3; ++i) r[i] = e[0][i] * x[0] + e[1][i] * x[1] + e[2][i] * x[2];
        return r;
    }
};
// column-major: e[c][r]
template <class T> struct Matrix4 {
    T e[4][4] = {{1, 0, 0, 0}, {0, 1, 0, 0}, {0, 0, 1, 0}, {0, 0, 0, 1}};
    T* ptr() { return &e[0][0]; }
    const T* ptr() const { return &e[0][0]; }
    Vector3<T> getX() const { return {e[0][0], e[0][1], e[0][2]}; }
    Vector3<T> getY() const { return {e[1][0], e[1][1], e[1][2]}; }
    Vector3<T> getZ() const { return {e[2][0], e[2][1], e[2][2]}; }
    Vector3<T> getT() const { return {e[3][0], e[3][1], e[3][2]}; }
    Matrix3<T> get3x3() const
    {
        Matrix3<T> m;
        for (int c = 0; c < 3; ++c)
            for (int r = 0; r < 3; ++r) m.e[c][r] = e[c][r];
        return m;
    }
    // rigid-motion inverse (rotation + translation)
    Matrix4 getInverse() const
    {
        Matrix4 m;
        for (int c = 0; c < 3; ++c)
            for (int r = 0; r < 3; ++r) m.e[c][r] = e[r][c];
        for (int r = 0; r < 3; ++r) m.e[3][r] = -(m.e[0][r] * e[3][0] + m.e[1][r] * e[3][1] + m.e[2][r] * e[3][2]);
        return m;
    }
    Vector4<T> operator*(const Vector4<T>& x) const
    {
        Vector4<T> r;
        for (int i = 0; i < 4; ++i) r[i] = e[0][i] * x[0] + e[1][i] * x[1] + e[2][i] * x[2] + e[3][i] * x[3];
        return r;
    }
};
} // namespace vl
