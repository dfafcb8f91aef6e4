// tfs_device.cuh -- device-side RPY pair arithmetic shared by the kernels.
//
// Units: every pair routine returns velocities multiplied by 8*pi*mu, i.e. in
// units of c = 1/(8 pi mu); kernels scale their sums by c once at the end.
// Only the far-field routine runs per pair in practice; the near-field one
// covers the overlapping and nested regimes of the reference's pair function
// (src/cilia/cuda_functions.cu:205-356) and the self term (r = 0).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace tfs {

constexpr double kPi = 3.14159265358979323846264338327950288;

// ---------------------------------------------------------------------------
// FP64 reciprocal square root for far-field separations.
//
// Seed: the FP32 hardware reciprocal square root of x rounded to FP32 by bit
// manipulation (exponent rebias, mantissa truncated to 20 bits), so the seed
// costs no FP64 instruction; relative seed error |e0| < 1e-6.
// Refinement: one third-order Householder step for y = x^(-1/2),
//   e = 1 - x y0^2,  y = y0 (1 + e/2 + 3 e^2 / 8),
// the second-order truncation of the binomial series of (1 - e)^(-1/2), whose
// truncation error is about (5/16) e^3 < 1e-18: the result is within a few
// ulp of the correctly rounded value, for 5 FP64 operations.
// Valid for x in the FP32 normal range [1.2e-38, 1.7e38] (far-field r^2 of
// any physical configuration); the kernels never call it for r^2 = 0.
// ---------------------------------------------------------------------------
__device__ __forceinline__ double rsqrt_far(double x) {
  const int hi = __double2hiint(x);
  const float xf = __int_as_float((hi - (896 << 20)) << 3);
  const float yf = rsqrtf(xf);
  const int fb = __float_as_int(yf);
  const double y0 = __hiloint2double((fb >> 3) + (896 << 20), fb << 29);
  const double t = x * y0;
  const double e = fma(-t, y0, 1.0);
  const double p = fma(e, 0.375, 0.5);
  const double g = y0 * e;
  return fma(g, p, y0);
}

__device__ __forceinline__ float rsqrt_far(float x) { return rsqrtf(x); }

template <typename T>
__device__ __forceinline__ T sqrt_t(T x);
template <>
__device__ __forceinline__ double sqrt_t<double>(double x) {
  return sqrt(x);
}
template <>
__device__ __forceinline__ float sqrt_t<float>(float x) {
  return sqrtf(x);
}

// Pair constants of one (target kind, source kind) block.
template <typename T>
struct PairConst {
  T ai, aj;     // target and source radii
  T asum2;      // (ai + aj)^2: r^2 above it is the far field
  T s;          // (ai^2 + aj^2) / 3
  T s3;         // -(ai^2 + aj^2) = -3 s
};

// ---------------------------------------------------------------------------
// Far field (r > ai + aj), cuda_functions.cu:224-234, :264-266, :288-290,
// :311-316, with d = x_i - x_j unnormalised and c = 1/(8 pi mu) factored out:
//   v_t += (rm1 + s rm3) F + rm3 (1 - 3 s rm2) (d.F) d + rm3 (T x d)
//   v_r += rm3 (F x d) - rm3/2 T + (3/2) rm5 (d.T) d
// ---------------------------------------------------------------------------
template <typename T, int VD, int FD>
__device__ __forceinline__ void far_pair(T *__restrict__ v, T dx, T dy, T dz, T rm1,
                                         const T *__restrict__ f, const PairConst<T> &pc) {
  const T rm2 = rm1 * rm1;
  const T rm3 = rm1 * rm2;
  const T rm5 = rm3 * rm2;
  const T A = fma(pc.s, rm3, rm1);
  const T B = fma(pc.s3, rm5, rm3);
  const T dF = fma(dx, f[0], fma(dy, f[1], dz * f[2]));
  const T Bd = B * dF;
  v[0] = fma(A, f[0], fma(Bd, dx, v[0]));
  v[1] = fma(A, f[1], fma(Bd, dy, v[1]));
  v[2] = fma(A, f[2], fma(Bd, dz, v[2]));
  if (FD == 6 || VD == 6) {
    const T ex = rm3 * dx, ey = rm3 * dy, ez = rm3 * dz;
    if (FD == 6) {  // translation from torque: rm3 (T x d)
      v[0] = fma(f[4], ez, fma(-f[5], ey, v[0]));
      v[1] = fma(f[5], ex, fma(-f[3], ez, v[1]));
      v[2] = fma(f[3], ey, fma(-f[4], ex, v[2]));
    }
    if (VD == 6) {  // rotation from force: rm3 (F x d)
      v[3] = fma(f[1], ez, fma(-f[2], ey, v[3]));
      v[4] = fma(f[2], ex, fma(-f[0], ez, v[4]));
      v[5] = fma(f[0], ey, fma(-f[1], ex, v[5]));
      if (FD == 6) {  // rotation from torque
        const T h = T(-0.5) * rm3;
        const T dT = fma(dx, f[3], fma(dy, f[4], dz * f[5]));
        const T q = (T(1.5) * rm5) * dT;
        v[3] = fma(h, f[3], fma(q, dx, v[3]));
        v[4] = fma(h, f[4], fma(q, dy, v[4]));
        v[5] = fma(h, f[5], fma(q, dz, v[5]));
      }
    }
  }
}

// ---------------------------------------------------------------------------
// Near field: the full three-regime pair of cuda_functions.cu:205-356, used
// when r^2 <= (ai + aj)^2 (overlap, nesting, self). Coefficients are the
// reference's multiplied by 8 pi mu. Branches on r as the reference does.
// ---------------------------------------------------------------------------
template <typename T, int VD, int FD>
__device__ __forceinline__ void near_pair(T *__restrict__ v, T dx, T dy, T dz, T r2,
                                       const T *__restrict__ f, const PairConst<T> &pc) {
  const T ai = pc.ai, aj = pc.aj;
  const T r = sqrt_t<T>(r2);
  const T inv_r = T(1) / (r + T(1e-20));  // :213, r = 0 gives e = 0
  const T ex = dx * inv_r, ey = dy * inv_r, ez = dz * inv_r;
  const T asum = ai + aj;
  const T adiff = ai > aj ? ai - aj : aj - ai;
  const T amax = ai > aj ? ai : aj;
  T A, B;
  T e_dot = ex * f[0] + ey * f[1] + ez * f[2];
  if (r > asum) {
    const T s = inv_r * inv_r * (ai * ai + aj * aj) / T(3);
    A = (T(1) + s) * inv_r;
    B = (T(1) - T(3) * s) * inv_r * e_dot;
  } else if (r > adiff) {
    const T r3x32 = T(32) * r * r * r;
    const T p = adiff * adiff + T(3) * r * r;
    const T q = adiff * adiff - r * r;
    const T c = T(4) / (T(3) * ai * aj);
    A = (T(0.5) * asum - p * p / r3x32) * c;
    B = (T(3) * q * q / r3x32) * c * e_dot;
  } else {
    A = T(4) / (T(3) * amax);
    B = T(0);
  }
  v[0] += A * f[0] + B * ex;
  v[1] += A * f[1] + B * ey;
  v[2] += A * f[2] + B * ez;
  if (FD == 6) {
    if (r > asum) {
      A = inv_r * inv_r;
    } else if (r > adiff) {
      const T g = aj - ai + r;
      A = inv_r * inv_r * g * g * (ai * ai + T(2) * ai * (r + aj) - T(3) * (aj - r) * (aj - r)) /
          (T(16) * ai * aj * aj * aj);
    } else {
      A = (aj > ai ? T(1) : T(0)) * r / (aj * aj * aj);
    }
    v[0] += A * (f[4] * ez - f[5] * ey);
    v[1] += A * (f[5] * ex - f[3] * ez);
    v[2] += A * (f[3] * ey - f[4] * ex);
  }
  if (VD == 6) {
    if (r > asum) {
      A = inv_r * inv_r;
    } else if (r > adiff) {
      const T g = ai - aj + r;
      A = inv_r * inv_r * g * g * (aj * aj + T(2) * aj * (r + ai) - T(3) * (ai - r) * (ai - r)) /
          (T(16) * aj * ai * ai * ai);
    } else {
      A = (ai > aj ? T(1) : T(0)) * r / (ai * ai * ai);
    }
    v[3] += A * (f[1] * ez - f[2] * ey);
    v[4] += A * (f[2] * ex - f[0] * ez);
    v[5] += A * (f[0] * ey - f[1] * ex);
    if (FD == 6) {
      e_dot = ex * f[3] + ey * f[4] + ez * f[5];
      if (r > asum) {
        A = T(-0.5) * inv_r * inv_r * inv_r;
        B = T(-3) * e_dot * A;
      } else if (r > adiff) {
        const T rr2 = r * r, r3 = rr2 * r;
        const T ai2 = ai * ai, aj2 = aj * aj, ai3 = ai2 * ai, aj3 = aj2 * aj;
        const T ad4 = adiff * adiff * adiff * adiff;
        const T num = T(5) * r3 * r3 - T(27) * rr2 * rr2 * (ai2 + aj2) + T(32) * r3 * (ai3 + aj3) -
                      T(9) * rr2 * (ai2 - aj2) * (ai2 - aj2) - ad4 * (ai2 + aj2 + T(4) * ai * aj);
        const T q = (ai - aj) * (ai - aj) - rr2;
        const T den = T(1) / (T(64) * r3 * ai3 * aj3);
        A = num * den;
        B = T(3) * q * q * (ai2 + aj2 + T(4) * ai * aj - rr2) * den * e_dot;
      } else {
        A = T(1) / (amax * amax * amax);
        B = T(0);
      }
      v[3] += A * f[3] + B * ex;
      v[4] += A * f[4] + B * ey;
      v[5] += A * f[5] + B * ez;
    }
  }
}

// One pair, branch-selected. The far branch is taken by every pair of the
// configurations of interest except self pairs and touching particles.
template <typename T, int VD, int FD>
__device__ __forceinline__ void rpy_pair(T *__restrict__ v, T dx, T dy, T dz,
                                         const T *__restrict__ f, const PairConst<T> &pc) {
  const T r2 = fma(dx, dx, fma(dy, dy, dz * dz));
  if (r2 > pc.asum2) {
    far_pair<T, VD, FD>(v, dx, dy, dz, rsqrt_far(r2), f, pc);
  } else {
    near_pair<T, VD, FD>(v, dx, dy, dz, r2, f, pc);
  }
}

// Knuth's TwoSum: hi + lo = a + b exactly (round-to-nearest).
__device__ __forceinline__ void two_sum(float &hi, float &lo, float b) {
  const float s = hi + b;
  const float bp = s - hi;
  const float err = (hi - (s - bp)) + (b - bp);
  hi = s;
  lo += err;
}

}  // namespace tfs
