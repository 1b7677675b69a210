// Exact squared forms of float-radius decisions.  sqrtf is correctly rounded
// and monotonic, so a test on sqrtf(r2) against a float bound is the same as
// a test of r2 against a float threshold found once on the host; the kernels
// then skip the square root where only the decision needs it.
#pragma once
#include <cmath>
#include <cstdint>
#include <cstring>

namespace simrecon {

// smallest float t with sqrtf(t) >= c: for every float r2, r2 < t <=> sqrtf(r2) < c
inline float r2_below(float c)
{
  float t = c * c;
  while (t > 0.f && std::sqrt(t) >= c) t = std::nextafter(t, 0.f);
  while (std::sqrt(t) < c) t = std::nextafter(t, INFINITY);
  return t;
}

// largest float t with sqrtf(t) <= c: r2 <= t <=> sqrtf(r2) <= c
inline float r2_atmost(float c)
{
  if (!(c >= 0.f)) return -1.f;
  float t = c * c;
  while (t > 0.f && std::sqrt(t) > c) t = std::nextafter(t, 0.f);
  while (std::sqrt(std::nextafter(t, INFINITY)) <= c) t = std::nextafter(t, INFINITY);
  return t;
}

// smallest non-negative float m with sqrtf(m) * f > c (float product), or
// +inf if none: m >= t <=> sqrtf(m) * f > c for m >= 0 (f > 0; the product
// is non-decreasing in m, so a bisection over the float bit patterns finds it)
inline float m_above_scaled_root(float c, float f)
{
  auto pred = [&](uint32_t bits) {
    float m;
    std::memcpy(&m, &bits, 4);
    return std::sqrt(m) * f > c;
  };
  uint32_t lo = 0, hi = 0x7f800000u;  // 0 .. +inf
  if (!pred(hi)) return INFINITY;
  if (pred(lo)) return 0.f;
  while (hi - lo > 1) {  // pred(lo) false, pred(hi) true
    const uint32_t mid = lo + (hi - lo) / 2;
    if (pred(mid)) hi = mid;
    else lo = mid;
  }
  float t;
  std::memcpy(&t, &hi, 4);
  return t;
}

}  // namespace simrecon
