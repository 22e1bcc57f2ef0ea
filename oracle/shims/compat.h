/* Forced-include header for compiling the reference solver with g++ 13.
 * The reference spells libm calls with the glibc _Float64 names (sqrtf64, ...);
 * mapping them to the double overloads changes no arithmetic (both are the
 * same IEEE binary64 functions) but keeps std::max<double> type-correct. */
#pragma once
#ifdef __cplusplus
#include <cmath>
#include <cstdlib>
#include <stdexcept>
#define sqrtf64 sqrt
#define fabsf64 fabs
#define powf64 pow
#define tanhf64 tanh
#define cosf64 cos
#define sinf64 sin
namespace std { template <class T> inline T abs(T x) { return x < 0 ? -x : x; } }
#endif
