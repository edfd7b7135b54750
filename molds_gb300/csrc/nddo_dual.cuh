// Forward-mode dual numbers with three partial derivatives: a value and its
// gradient with respect to the relative position vector of an atom pair.
// Running the templated pair mathematics (nddo_math.cuh) on this type gives
// the exact derivatives of the implemented formulas (the analytic energy
// gradient), not finite differences.
#pragma once
#include <cmath>

namespace nddo {
// in their own namespace: found by argument-dependent lookup for Dual3
// arguments only, so they never hide ::sqrt / ::exp for doubles in nddo
namespace ad {

struct Dual3 {
  double v;
  double d[3];
  __host__ __device__ Dual3() : v(0.0), d{0.0, 0.0, 0.0} {}
  __host__ __device__ Dual3(double x) : v(x), d{0.0, 0.0, 0.0} {}   // NOLINT: implicit, as a scalar
  __host__ __device__ Dual3(double x, double g0, double g1, double g2) : v(x), d{g0, g1, g2} {}

  __host__ __device__ Dual3& operator+=(const Dual3& b) { v += b.v; d[0] += b.d[0]; d[1] += b.d[1]; d[2] += b.d[2]; return *this; }
  __host__ __device__ Dual3& operator-=(const Dual3& b) { v -= b.v; d[0] -= b.d[0]; d[1] -= b.d[1]; d[2] -= b.d[2]; return *this; }
  __host__ __device__ Dual3& operator*=(const Dual3& b) {
    d[0] = d[0] * b.v + v * b.d[0];
    d[1] = d[1] * b.v + v * b.d[1];
    d[2] = d[2] * b.v + v * b.d[2];
    v *= b.v;
    return *this;
  }
  __host__ __device__ Dual3& operator/=(const Dual3& b) {
    const double r = 1.0 / b.v, q = v * r;
    d[0] = (d[0] - q * b.d[0]) * r;
    d[1] = (d[1] - q * b.d[1]) * r;
    d[2] = (d[2] - q * b.d[2]) * r;
    v = q;
    return *this;
  }
};

__host__ __device__ inline Dual3 operator-(const Dual3& a) { return Dual3(-a.v, -a.d[0], -a.d[1], -a.d[2]); }
__host__ __device__ inline Dual3 operator+(Dual3 a, const Dual3& b) { return a += b; }
__host__ __device__ inline Dual3 operator-(Dual3 a, const Dual3& b) { return a -= b; }
__host__ __device__ inline Dual3 operator*(Dual3 a, const Dual3& b) { return a *= b; }
__host__ __device__ inline Dual3 operator/(Dual3 a, const Dual3& b) { return a /= b; }
__host__ __device__ inline Dual3 operator+(Dual3 a, double b) { a.v += b; return a; }
__host__ __device__ inline Dual3 operator+(double b, Dual3 a) { a.v += b; return a; }
__host__ __device__ inline Dual3 operator-(Dual3 a, double b) { a.v -= b; return a; }
__host__ __device__ inline Dual3 operator-(double b, const Dual3& a) { return Dual3(b - a.v, -a.d[0], -a.d[1], -a.d[2]); }
__host__ __device__ inline Dual3 operator*(const Dual3& a, double b) { return Dual3(a.v * b, a.d[0] * b, a.d[1] * b, a.d[2] * b); }
__host__ __device__ inline Dual3 operator*(double b, const Dual3& a) { return a * b; }
__host__ __device__ inline Dual3 operator/(const Dual3& a, double b) { return a * (1.0 / b); }
__host__ __device__ inline Dual3 operator/(double b, const Dual3& a) { return Dual3(b) /= a; }

__host__ __device__ inline bool operator<(const Dual3& a, const Dual3& b) { return a.v < b.v; }
__host__ __device__ inline bool operator>(const Dual3& a, const Dual3& b) { return a.v > b.v; }
__host__ __device__ inline bool operator<=(const Dual3& a, const Dual3& b) { return a.v <= b.v; }
__host__ __device__ inline bool operator>=(const Dual3& a, const Dual3& b) { return a.v >= b.v; }
__host__ __device__ inline bool operator==(const Dual3& a, const Dual3& b) { return a.v == b.v; }
__host__ __device__ inline bool operator!=(const Dual3& a, const Dual3& b) { return a.v != b.v; }

__host__ __device__ inline Dual3 fabs(const Dual3& a) { return a.v < 0.0 ? -a : a; }
__host__ __device__ inline Dual3 sqrt(const Dual3& a) {
  const double s = ::sqrt(a.v), h = 0.5 / s;
  return Dual3(s, a.d[0] * h, a.d[1] * h, a.d[2] * h);
}
__host__ __device__ inline Dual3 exp(const Dual3& a) {
  const double e = ::exp(a.v);
  return Dual3(e, a.d[0] * e, a.d[1] * e, a.d[2] * e);
}

}  // namespace ad
using ad::Dual3;
}  // namespace nddo
