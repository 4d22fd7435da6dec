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
