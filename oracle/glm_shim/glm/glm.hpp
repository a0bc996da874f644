// Minimal stand-in for the few GLM pieces the reference's CPU geodesic mirror uses
// (src/physics/Geodesic.h, tests/geodesic_tests.cpp): glm::dvec3 arithmetic, dot, cross,
// length and normalize. GLM 1.0.1 itself is not in the image (the reference fetches it at
// configure time). The formulas below are GLM's documented definitions:
//   dot(a, b)      = (a.x*b.x + a.y*b.y) + a.z*b.z
//   length(v)      = sqrt(dot(v, v))
//   normalize(v)   = v * (1 / sqrt(dot(v, v)))
//   cross(a, b)    = (a.y*b.z - b.y*a.z, a.z*b.x - b.z*a.x, a.x*b.y - b.x*a.y)
// Test infrastructure only: used to build the reference's own sources into oracle/_ref.
#pragma once
#include <cmath>

namespace glm {

struct dvec3 {
    double x, y, z;
    dvec3() : x(0), y(0), z(0) {}
    explicit dvec3(double s) : x(s), y(s), z(s) {}
    dvec3(double a, double b, double c) : x(a), y(b), z(c) {}
    dvec3& operator+=(const dvec3& o) { x += o.x; y += o.y; z += o.z; return *this; }
    dvec3& operator-=(const dvec3& o) { x -= o.x; y -= o.y; z -= o.z; return *this; }
};

inline dvec3 operator+(const dvec3& a, const dvec3& b) { return dvec3(a.x + b.x, a.y + b.y, a.z + b.z); }
inline dvec3 operator-(const dvec3& a, const dvec3& b) { return dvec3(a.x - b.x, a.y - b.y, a.z - b.z); }
inline dvec3 operator-(const dvec3& a) { return dvec3(-a.x, -a.y, -a.z); }
inline dvec3 operator*(const dvec3& a, double s) { return dvec3(a.x * s, a.y * s, a.z * s); }
inline dvec3 operator*(double s, const dvec3& a) { return dvec3(s * a.x, s * a.y, s * a.z); }
inline dvec3 operator/(const dvec3& a, double s) { return dvec3(a.x / s, a.y / s, a.z / s); }

inline double dot(const dvec3& a, const dvec3& b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline double length(const dvec3& v) { return std::sqrt(dot(v, v)); }
inline dvec3 normalize(const dvec3& v) { return v * (1.0 / std::sqrt(dot(v, v))); }
inline dvec3 cross(const dvec3& a, const dvec3& b) {
    return dvec3(a.y * b.z - b.y * a.z, a.z * b.x - b.z * a.x, a.x * b.y - b.x * a.y);
}

}  // namespace glm
