// Allocation-free density matrix of one mode.
//
// Some callers cannot call cudaMalloc at the point where they need a density
// matrix: code running while a CUDA stream is being captured into a graph
// (allocation calls are not capturable), host programs that hand the GPU a fixed
// memory budget and forbid further allocations, or a Fortran time loop that has
// already placed A in device memory it manages itself.  For them this file
// computes rho(j1, j2) = sum conj(A(.., j1, ..)) A(.., j2, ..) over all modes but
// one -- the contraction of Calc_rho1mode for a grid mode -- with the caller's
// input and output buffers and a fixed scratch area that the library reserves
// once as a file-scope __device__ array (every GPU that loads the library holds
// it until the process exits).
#include <cuda_runtime.h>
#include <stdio.h>
#include <string.h>

#include "../../include/macaw_gb300.h"
#include "common.cuh"

#define NOALLOC_MAX_N MAXN_SPF        // largest SPF count of the contracted mode
#define NOALLOC_MAX_BLOCKS 128         // block partials held in the scratch area
#define NOALLOC_TILE 32
#define NOALLOC_THREADS 256
#define NOALLOC_MAX_DEVICES 64

// Block partials of the contraction: NOALLOC_MAX_BLOCKS x 32 x 32 complex = 2 MiB.
static __device__ __align__(256) cplx g_noalloc_scratch[NOALLOC_MAX_BLOCKS * NOALLOC_MAX_N * NOALLOC_MAX_N];

// Device addresses of g_noalloc_scratch, looked up once per device.  In host
// code the symbol name stands for a host-side shadow, not a device address.
static cplx* g_scratch_addr[NOALLOC_MAX_DEVICES];

void mctdh_set_global_error(const char* msg);

// Block b sums the fibre tiles b, b + nblk, ... into its own n x n partial; every
// partial entry read by the second kernel is written by this launch first.
__global__ void __launch_bounds__(NOALLOC_THREADS)
noalloc_rho_partial(const cplx* __restrict__ A, long long L, long long R, int n, int nblk, cplx* scratch) {
  __shared__ cplx Xs[NOALLOC_TILE * NOALLOC_MAX_N];
  const int b = blockIdx.x;
  const int npairs = n * n;
  const long long nfib = L * R;
  const long long ntiles = (nfib + NOALLOC_TILE - 1) / NOALLOC_TILE;
  const int tid = threadIdx.x;
  const bool small = npairs <= NOALLOC_THREADS;
  const int G = small ? NOALLOC_THREADS / npairs : 1;
  const int pair0 = small ? tid % npairs : tid;
  const int g = small ? tid / npairs : 0;
  cplx acc[4] = {mkc(0, 0), mkc(0, 0), mkc(0, 0), mkc(0, 0)};
  for (long long tile = b; tile < ntiles; tile += nblk) {
    const long long p0 = tile * NOALLOC_TILE;
    for (int e = tid; e < NOALLOC_TILE * n; e += NOALLOC_THREADS) {
      const int q = e % NOALLOC_TILE, j = e / NOALLOC_TILE;
      const long long p = p0 + q;
      cplx v = mkc(0, 0);
      if (p < nfib) {
        const long long l = p % L, r = p / L;
        v = A[l + L * (j + (long long)n * r)];
      }
      Xs[q * NOALLOC_MAX_N + j] = v;
    }
    __syncthreads();
    if (small) {
      if (g < G) {
        const int j1 = pair0 % n, j2 = pair0 / n;
        for (int q = g; q < NOALLOC_TILE; q += G)
          cfma_conj(acc[0], Xs[q * NOALLOC_MAX_N + j1], Xs[q * NOALLOC_MAX_N + j2]);
      }
    } else {
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        const int pr = pair0 + NOALLOC_THREADS * k;
        if (pr < npairs) {
          const int j1 = pr % n, j2 = pr / n;
          for (int q = 0; q < NOALLOC_TILE; ++q)
            cfma_conj(acc[k], Xs[q * NOALLOC_MAX_N + j1], Xs[q * NOALLOC_MAX_N + j2]);
        }
      }
    }
    __syncthreads();
  }
  cplx* out = scratch + (long long)b * npairs;
  if (small) {
    cplx* red = Xs;
    red[tid] = acc[0];
    __syncthreads();
    if (tid < npairs) {
      cplx s = mkc(0, 0);
      for (int gg = 0; gg < G; ++gg) s = cadd(s, red[gg * npairs + tid]);
      out[tid] = s;
    }
  } else {
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      const int pr = pair0 + NOALLOC_THREADS * k;
      if (pr < npairs) out[pr] = acc[k];
    }
  }
}

// rho = 1/2 (S + S^H), S = sum of the block partials in a fixed order.
__global__ void noalloc_rho_finish(const cplx* __restrict__ scratch, int nblk, int n, cplx* rho, long long ld) {
  const int npairs = n * n;
  for (int pr = threadIdx.x; pr < npairs; pr += blockDim.x) {
    const int j1 = pr % n, j2 = pr / n;
    const int prT = j2 + n * j1;
    cplx s = mkc(0, 0), sT = mkc(0, 0);
    for (int b = 0; b < nblk; ++b) {
      s = cadd(s, scratch[(long long)b * npairs + pr]);
      sT = cadd(sT, scratch[(long long)b * npairs + prT]);
    }
    rho[j1 + ld * j2] = cscale(cadd(s, cconj(sT)), 0.5);
  }
}

// True for device memory of device `dev` and for managed memory; host memory,
// unregistered pointers and buffers of another GPU are refused (a kernel given a
// peer buffer would fault without peer access or silently read over the link).
static bool device_pointer(const void* p, int dev) {
  cudaPointerAttributes at;
  if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
    cudaGetLastError();   // the query's own error (unregistered host pointer)
    return false;
  }
  if (at.type == cudaMemoryTypeManaged) return true;
  return at.type == cudaMemoryTypeDevice && at.device == dev;
}

extern "C" int64_t mctdh_density_matrix_noalloc(const double* A, const int64_t* nspf, int64_t nmodes,
                                                int64_t mode, double* rho, int64_t ld, void* stream) {
  char msg[256];
  if (!A || !nspf || !rho) {
    mctdh_set_global_error("mctdh_density_matrix_noalloc: null pointer");
    return MCTDH_EARG;
  }
  if (nmodes < 1 || mode < 0 || mode >= nmodes) {
    mctdh_set_global_error("mctdh_density_matrix_noalloc: mode outside 0..nmodes-1");
    return MCTDH_EARG;
  }
  const int64_t n = nspf[mode];
  if (n < 1 || n > NOALLOC_MAX_N) {
    snprintf(msg, sizeof msg,
             "mctdh_density_matrix_noalloc: %lld SPFs on the contracted mode exceed the maximum of %d",
             (long long)n, NOALLOC_MAX_N);
    mctdh_set_global_error(msg);
    return MCTDH_EARG;
  }
  if (ld < n) {
    mctdh_set_global_error("mctdh_density_matrix_noalloc: leading dimension of rho smaller than n");
    return MCTDH_EARG;
  }
  long long L = 1, R = 1;
  for (int64_t m = 0; m < nmodes; ++m) {
    if (nspf[m] < 1) {
      mctdh_set_global_error("mctdh_density_matrix_noalloc: non-positive SPF count");
      return MCTDH_EARG;
    }
    if (m < mode) L *= nspf[m];
    if (m > mode) R *= nspf[m];
  }
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= NOALLOC_MAX_DEVICES) {
    cudaGetLastError();
    mctdh_set_global_error("mctdh_density_matrix_noalloc: no usable CUDA device");
    return MCTDH_ECUDA;
  }
  // an error left by an earlier, unrelated call stays with its owner: report it
  // without clearing it rather than taking it for a failure of this call
  const cudaError_t pending = cudaPeekAtLastError();
  if (pending != cudaSuccess) {
    snprintf(msg, sizeof msg, "mctdh_density_matrix_noalloc: a CUDA error of an earlier call is pending: %s",
             cudaGetErrorString(pending));
    mctdh_set_global_error(msg);
    return MCTDH_ECUDA;
  }
  if (!device_pointer(A, dev) || !device_pointer(rho, dev)) {
    mctdh_set_global_error("mctdh_density_matrix_noalloc: A and rho must be device memory of the current device");
    return MCTDH_EARG;
  }
  // once per device, with that device current: the device address of the scratch
  // area.  The cached address assumes the device is not reset (cudaDeviceReset)
  // while the library is loaded.
  if (!g_scratch_addr[dev]) {
    cplx* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress((void**)&p, g_noalloc_scratch);
    if (e != cudaSuccess || !p) {
      snprintf(msg, sizeof msg, "mctdh_density_matrix_noalloc: cudaGetSymbolAddress failed: %s",
               cudaGetErrorString(e));
      mctdh_set_global_error(msg);
      return MCTDH_ECUDA;
    }
    g_scratch_addr[dev] = p;
  }
  const long long ntiles = (L * R + NOALLOC_TILE - 1) / NOALLOC_TILE;
  long long nb = ntiles / 8;
  if (nb < 1) nb = 1;
  if (nb > NOALLOC_MAX_BLOCKS) nb = NOALLOC_MAX_BLOCKS;
  const int nblk = (int)nb;
  cudaStream_t st = (cudaStream_t)stream;
  noalloc_rho_partial<<<nblk, NOALLOC_THREADS, 0, st>>>((const cplx*)A, L, R, (int)n, nblk, g_scratch_addr[dev]);
  noalloc_rho_finish<<<1, 256, 0, st>>>(g_scratch_addr[dev], nblk, (int)n, (cplx*)rho, (long long)ld);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    snprintf(msg, sizeof msg, "mctdh_density_matrix_noalloc: launch failed: %s", cudaGetErrorString(e));
    mctdh_set_global_error(msg);
    return MCTDH_ECUDA;
  }
  return MCTDH_OK;
}
