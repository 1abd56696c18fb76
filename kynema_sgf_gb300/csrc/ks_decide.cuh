// Branch decisions of the Godunov / PPM passes in the arithmetic type of the
// pass: FP64 operands are compared on the integer pipe (ks_common.cuh), FP32
// operands with plain compares.  The forward kernels and their reverse
// (adjoint) kernels take every decision through these functions, so a reverse
// kernel re-evaluates exactly the branch its forward took.
#pragma once

#include "ks_common.cuh"

namespace ks {

#ifdef __CUDACC__
__device__ inline bool same_sign(double a, double b) { return isame_sign(a, b); }
__device__ inline bool same_sign(float a, float b) { return a * b > 0.0f; }
__device__ inline bool abs_lt(double a, double b) { return iabs_lt2(a, b); }  // |a| < |b|
__device__ inline bool abs_lt(float a, float b) { return fabsf(a) < fabsf(b); }
__device__ inline double mag_sign(double m, double s) { return isign(iabs(m), s); }  // |m| with the sign of s
__device__ inline float mag_sign(float m, float s) { return copysignf(fabsf(m), s); }
__device__ inline double clip2(double e, double a, double b) { return imin(imax(e, imin(a, b)), imax(a, b)); }
__device__ inline float clip2(float e, float a, float b) { return fminf(fmaxf(e, fminf(a, b)), fmaxf(a, b)); }
__device__ inline bool gt0(double x) { return igt0(x); }
__device__ inline bool gt0(float x) { return x > 0.0f; }
__device__ inline bool le0(double x) { return ile0(x); }
__device__ inline bool le0(float x) { return x <= 0.0f; }
__device__ inline bool ge0(double x) { return ige0(x); }
__device__ inline bool ge0(float x) { return x >= 0.0f; }
__device__ inline bool above_small(double u) { return dbits(u) > dbits(kSmallVel); }          // u > small_vel
__device__ inline bool above_small(float u) { return u > (float)kSmallVel; }
__device__ inline bool below_msmall(double u) { return okey(u) < okey(-kSmallVel); }      // u < -small_vel
__device__ inline bool below_msmall(float u) { return u < -(float)kSmallVel; }
__device__ inline bool below_small_abs(double u) { return iabs_lt(u, kSmallVel); }        // |u| < small_vel
__device__ inline bool below_small_abs(float u) { return fabsf(u) < (float)kSmallVel; }
__device__ inline double absv(double x) { return iabs(x); }
__device__ inline float absv(float x) { return fabsf(x); }
__device__ inline double neg_if(bool c, double x) { return c ? bitsd(dbits(x) ^ ~kMag) : x; }
__device__ inline float neg_if(bool c, float x) { return c ? -x : x; }
__device__ inline double min2(double a, double b) { return imin(a, b); }
__device__ inline float min2(float a, float b) { return fminf(a, b); }
__device__ inline double max2(double a, double b) { return imax(a, b); }
__device__ inline float max2(float a, float b) { return fmaxf(a, b); }
__device__ inline bool lt(double a, double b) { return ilt(a, b); }  // a < b
__device__ inline bool lt(float a, float b) { return a < b; }
__device__ inline bool nonzero(double x) { return (dbits(x) & kMag) != 0; }
__device__ inline bool nonzero(float x) { return x != 0.0f; }

#endif

}  // namespace ks
