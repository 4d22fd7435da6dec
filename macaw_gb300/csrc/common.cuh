// Shared device helpers for the G-MCTDH propagation core (sm_103a).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

typedef double2 cplx;    // FP64 complex, interleaved (re, im) like Fortran double complex
typedef float2 cplxf;    // FP32 complex for the split-precision contractions

__host__ __device__ __forceinline__ cplx mkc(double r, double i) { return make_double2(r, i); }
__host__ __device__ __forceinline__ cplx cadd(cplx a, cplx b) { return make_double2(a.x + b.x, a.y + b.y); }
__host__ __device__ __forceinline__ cplx csub(cplx a, cplx b) { return make_double2(a.x - b.x, a.y - b.y); }
__host__ __device__ __forceinline__ cplx cmul(cplx a, cplx b) {
  return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__host__ __device__ __forceinline__ cplx cconj(cplx a) { return make_double2(a.x, -a.y); }
__host__ __device__ __forceinline__ cplx cscale(cplx a, double s) { return make_double2(a.x * s, a.y * s); }
// acc += a * b
__host__ __device__ __forceinline__ void cfma(cplx& acc, cplx a, cplx b) {
  acc.x = fma(a.x, b.x, acc.x);
  acc.x = fma(-a.y, b.y, acc.x);
  acc.y = fma(a.x, b.y, acc.y);
  acc.y = fma(a.y, b.x, acc.y);
}
// acc += conj(a) * b
__host__ __device__ __forceinline__ void cfma_conj(cplx& acc, cplx a, cplx b) {
  acc.x = fma(a.x, b.x, acc.x);
  acc.x = fma(a.y, b.y, acc.x);
  acc.y = fma(a.x, b.y, acc.y);
  acc.y = fma(-a.y, b.x, acc.y);
}
__host__ __device__ __forceinline__ double cabs2(cplx a) { return a.x * a.x + a.y * a.y; }

__device__ __forceinline__ cplxf cfmaf_(cplxf acc, cplxf a, cplxf b) {
  acc.x = fmaf(a.x, b.x, acc.x);
  acc.x = fmaf(-a.y, b.y, acc.x);
  acc.y = fmaf(a.x, b.y, acc.y);
  acc.y = fmaf(a.y, b.x, acc.y);
  return acc;
}

// Exact FP64 -> FP32 hi + lo split and FP32 -> FP64 widening with integer
// operations only.  On GB300 the F2F conversions run on the FP64 pipe, which is
// 1/64 of the FP32 rate; these keep the split-precision kernels off that pipe.
// hi takes the leading 24 mantissa bits (truncated), lo the next 24, so
// hi + lo = x to 2^-48 relative.  Magnitudes below 2^-126 are flushed to zero.
__device__ __forceinline__ void split_d2f(double x, float& hi, float& lo) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(x);
  const unsigned int sign = (unsigned int)(b >> 63) << 31;
  const int E = (int)((b >> 52) & 0x7FF) - 1023;
  const unsigned long long m = b & 0xFFFFFFFFFFFFFULL;
  if (E < -126) { hi = 0.f; lo = 0.f; return; }
  if (E > 127) { hi = __uint_as_float(sign | 0x7F800000u | (m ? 1u : 0u)); lo = 0.f; return; }
  hi = __uint_as_float(sign | ((unsigned int)(E + 127) << 23) | (unsigned int)(m >> 29));
  const unsigned int rem = (unsigned int)(m & 0x1FFFFFFFu);
  if (rem == 0) { lo = 0.f; return; }
  const int p = 31 - __clz(rem);              // top bit of the remainder, 0..28
  const int el = E - 52 + p + 127;            // biased exponent of lo
  if (el <= 0) { lo = 0.f; return; }
  const unsigned int mant = (p <= 23) ? (rem << (23 - p)) : (rem >> (p - 23));
  lo = __uint_as_float(sign | ((unsigned int)el << 23) | (mant & 0x7FFFFFu));
}
__device__ __forceinline__ double f2d_exact(float f) {
  const unsigned int u = __float_as_uint(f);
  const unsigned long long sign = (unsigned long long)(u >> 31) << 63;
  const unsigned int e = (u >> 23) & 0xFF;
  const unsigned long long m = u & 0x7FFFFFu;
  if (e == 0) return __longlong_as_double((long long)sign);
  if (e == 0xFF) return __longlong_as_double((long long)(sign | (0x7FFULL << 52) | (m << 29)));
  return __longlong_as_double((long long)(sign | ((unsigned long long)(e - 127 + 1023) << 52) | (m << 29)));
}

// Element i of a tensor in any storage format: 0 complex128, 1 FP32 split pairs
// (re hi, im hi, re lo, im lo) in 16 bytes, 2 complex FP32 (re, im) in 8 bytes.
__device__ __forceinline__ cplx load_c(const cplx* p, long long i, int fmt) {
  if (!fmt) return p[i];
  if (fmt == 2) {
    const float2 v = reinterpret_cast<const float2*>(p)[i];
    return make_double2(f2d_exact(v.x), f2d_exact(v.y));
  }
  const float4 w = reinterpret_cast<const float4*>(p)[i];
  return make_double2(f2d_exact(w.x) + f2d_exact(w.z), f2d_exact(w.y) + f2d_exact(w.w));
}
// ... as an FP32 (re hi, im hi, re lo, im lo) split
__device__ __forceinline__ float4 load_split(const cplx* p, long long i, int fmt) {
  if (fmt == 2) {
    const float2 v = reinterpret_cast<const float2*>(p)[i];
    return make_float4(v.x, v.y, 0.f, 0.f);
  }
  if (fmt) return reinterpret_cast<const float4*>(p)[i];
  const cplx v = p[i];
  float4 w;
  split_d2f(v.x, w.x, w.z);
  split_d2f(v.y, w.y, w.w);
  return w;
}

// (l, r) of fibre p < nfib = L * R (l fastest): 32-bit division whenever the
// fibre count fits, the 64-bit one otherwise.
__device__ __forceinline__ void fibre_lr(long long p, long long L, long long nfib, long long& l, long long& r) {
  if (nfib <= 0xFFFFFFFFLL) {
    const unsigned pu = (unsigned)p, Lu = (unsigned)L;
    const unsigned ru = pu / Lu;
    r = ru;
    l = pu - ru * Lu;
  } else {
    r = p / L;
    l = p - r * L;
  }
}

// Status codes returned through the C-ABI (negative = error).
enum {
  MCTDH_OK = 0,
  MCTDH_EUNSUPPORTED = -1,
  MCTDH_EEIG = -2,
  MCTDH_EKRYLOV = -3,
  MCTDH_ESTEP = -4,
  MCTDH_ENONFINITE = -5,
  MCTDH_ECUDA = -6,
  MCTDH_EARG = -7,
};

// Device status word bits written by kernels whose iteration caps ran out.
enum { DEVST_EIG_NOCONV = 1, DEVST_CHOL_FAIL = 2, DEVST_NONFINITE = 4 };

#define MAXN_SPF 32   // largest SPF count per mode handled by the small dense kernels
