// Tensor-core (tcgen05, TF32 with FP32 accumulation in TMEM) kernels of the
// split-FP32 path for sm_103a.
//
// Batched mode product (Mult_HeM_MatV / Mult_GM_MatV, gmctdh_objects.f90:1407-1468)
// as a GEMM: the 128 fibres (l, :, r) of a tile are the rows, the complex
// matrix is a real 2 nin x 2 nout block [[Mr, Mi], [-Mi, Mr]] acting on the
// interleaved (re, im) columns, so D(fibre, 2 jo + c) is the real (c = 0) or
// imaginary (c = 1) part of output jo.  Every FP32 operand is split exactly into
// three TF32 numbers, x = hi + mid + lo (11 + 11 + 2 significant bits), and a
// tile takes six MMAs per K step (every part product down to 2^-22 of the
// leading one: lo*hi, mid*mid, hi*lo, mid*hi, hi*mid, hi*hi): each product is
// carried to ~2^-33, so the FP32 accumulation in TMEM is the only rounding, as
// in the FP32 CUDA-core products this replaces.
//
// Persistent CTAs of 4 warps (128 threads) walk the tiles of all descriptors
// (tile b of the batch = fibres 128 (b - block_start) ... of its descriptor, the
// CUDA-core kernel's block mapping): thread t loads fibre t of a tile (coalesced
// along l), splits it and writes the K-major operand tiles of its stage; thread
// 0 issues the MMAs into that stage's 32-column TMEM accumulator and commits
// them to the stage's mbarrier; every warp then reads its 32 TMEM lanes (= its
// 32 fibres) and stores them.  With two stages the loads of tile i run while
// the MMAs of tile i - 1 finish, and tile i - 1 is drained after them; with one
// stage a CTA drains each tile before loading the next, and twice as many CTAs
// share an SM.
#include <algorithm>
#include <stdlib.h>

#include "../../include/macaw_gb300.h"
#include "kernels.cuh"
#include "tc.cuh"

#define TC_ROWS 128
#define TC_MAXN 16          // largest nin / nout of the tensor-core mode product
#define TC_NPART 3          // hi, mid, lo

// set when a tensor-core kernel gave up waiting for its MMAs (never expected)
__device__ int g_tc_timeout = 0;

__device__ __forceinline__ int tc_find_tile(const ProdDesc* descs, int ndesc, long long b) {
  int lo = 0, hi = ndesc - 1;
  while (lo < hi) {
    int mid = (lo + hi + 1) >> 1;
    if (descs[mid].block_start <= b) lo = mid; else hi = mid - 1;
  }
  return lo;
}

__global__ void __launch_bounds__(TC_ROWS) prod_tc_kernel(const ProdDesc* __restrict__ descs, int ndesc,
                                                          long long ntiles, int K, int N, int nstage) {
  extern __shared__ __align__(128) unsigned char tc_smem[];
  __shared__ __align__(8) uint64_t bar[2];
  __shared__ uint32_t s_tmem;
  const int tid = threadIdx.x, warp = tid >> 5;
  // stage layout: A parts (128 x K floats each), then B parts (N x K floats each)
  const uint32_t abytes = (uint32_t)TC_ROWS * K * 4, bbytes = (uint32_t)N * K * 4;
  const uint32_t sbytes = TC_NPART * (abytes + bbytes);
  const uint32_t base = tc_smem_addr(tc_smem);
  if (tid == 0) {
    tc_bar_init(&bar[0], 1);
    tc_bar_init(&bar[1], 1);
  }
  if (warp == 0) tc_alloc(&s_tmem, 64);
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = s_tmem;
  const uint32_t idesc = tc_idesc_tf32(TC_ROWS, N);
  const uint32_t sbo = (uint32_t)K * 32;
  bool ok = true;
  int prev_di = -1;          // the tile loaded in the previous iteration
  long long prev_p = 0;
  int it = 0;
  for (long long tile = blockIdx.x;; tile += gridDim.x, ++it) {
    const bool have = tile < ntiles;
    const int s = (nstage == 2) ? (it & 1) : 0;
    int di = -1;
    long long p = 0;
    if (have) {
      di = tc_find_tile(descs, ndesc, tile);
      const ProdDesc& d = descs[di];
      const int nin = d.nin, nout = d.nout;
      unsigned char* sb = tc_smem + s * sbytes;
      // B(n, k): n = 2 jo + c', k = 2 ji + c; y_re = sum Mr x_re - Mi x_im, y_im = sum Mi x_re + Mr x_im
      for (int e = tid; e < N * K; e += TC_ROWS) {
        const int n = e % N, k = e / N;
        const int jo = n >> 1, ji = k >> 1;
        float v = 0.f;
        if (jo < nout && ji < nin) {
          const cplx m = d.conjT ? cconj(d.M[ji + (long long)d.ldm * jo]) : d.M[jo + (long long)d.ldm * ji];
          const int cout = n & 1, cin = k & 1;
          const float mr = (float)m.x, mi = (float)m.y;
          v = (cout == cin) ? mr : (cout ? mi : -mi);
        }
        float h, m_, l;
        tc_split3(v, h, m_, l);
        const uint32_t o = TC_NPART * abytes + tc_off(n, k, K);
        *reinterpret_cast<float*>(sb + o) = h;
        *reinterpret_cast<float*>(sb + o + bbytes) = m_;
        *reinterpret_cast<float*>(sb + o + 2 * bbytes) = l;
      }
      // A: fibre tid of the tile
      const long long L = d.L, nfib = d.L * d.R;
      p = (tile - d.block_start) * TC_ROWS + tid;
      const bool valid = p < nfib;
      long long l = 0, r = 0;
      if (valid) fibre_lr(p, L, nfib, l, r);
      const long long xi0 = l + L * (long long)nin * r;
      for (int k4 = 0; k4 < K; k4 += 4) {
        float x[4];
#pragma unroll
        for (int q = 0; q < 2; ++q) {
          const int ji = (k4 >> 1) + q;
          float re = 0.f, im = 0.f;
          if (valid && ji < nin) {
            const float4 w = load_split(d.X, xi0 + L * ji, d.xfmt);
            re = w.x + w.z;
            im = w.y + w.w;
          }
          x[2 * q] = re;
          x[2 * q + 1] = im;
        }
        float4 hv, mv, lv;
        tc_split3(x[0], hv.x, mv.x, lv.x);
        tc_split3(x[1], hv.y, mv.y, lv.y);
        tc_split3(x[2], hv.z, mv.z, lv.z);
        tc_split3(x[3], hv.w, mv.w, lv.w);
        const uint32_t o = tc_off(tid, k4, K);
        *reinterpret_cast<float4*>(sb + o) = hv;
        *reinterpret_cast<float4*>(sb + o + abytes) = mv;
        *reinterpret_cast<float4*>(sb + o + 2 * abytes) = lv;
      }
    }
    tc_fence_smem();
    tc_fence_before();
    __syncthreads();
    if (have && tid == 0) {
      tc_fence_after();
      const uint32_t dt = tmem + 32u * s;
      const uint32_t sa = base + s * sbytes, sbb = sa + TC_NPART * abytes;
      // part products in increasing size: (A part, B part) = (lo, hi), (mid, mid),
      // (hi, lo), (mid, hi), (hi, mid), (hi, hi); part 0 = hi, 1 = mid, 2 = lo
      uint32_t acc = 0;
      for (int k8 = 0; k8 < K / 8; ++k8) {
        const uint32_t o = 256u * k8;
#pragma unroll
        for (int q = 0; q < 6; ++q) {
          const uint32_t pa = (q == 0) ? 2u : ((q == 1 || q == 3) ? 1u : 0u);
          const uint32_t pb = (q == 2) ? 2u : ((q == 1 || q == 4) ? 1u : 0u);
          tc_mma_tf32(dt, tc_smem_desc(sa + pa * abytes + o, 128, sbo), tc_smem_desc(sbb + pb * bbytes + o, 128, sbo),
                      idesc, acc);
          acc = 1;
        }
      }
      tc_commit(&bar[s]);
    }
    // Drain: with two stages the previous tile (the other stage) while this one
    // runs, with one stage this tile.  Uniform across the CTA.
    const bool do_drain = (nstage == 2) ? (prev_di >= 0) : have;
    if (do_drain) {
      const int ps = (nstage == 2) ? ((it - 1) & 1) : 0;
      const uint32_t parity = (nstage == 2) ? ((uint32_t)((it - 1) >> 1) & 1u) : ((uint32_t)it & 1u);
      const int dd = (nstage == 2) ? prev_di : di;
      const long long dpf = (nstage == 2) ? prev_p : p;
      // every thread polls the mbarrier; the verdict is made uniform across the
      // CTA so that all threads leave the loop together if a wait ran out
      const bool w = __syncthreads_and(tc_wait(&bar[ps], parity));
      tc_fence_after();
      if (!w) {
        ok = false;
      } else {
        const ProdDesc& d = descs[dd];
        const int nout = d.nout;
        float acc[32];
        const uint32_t trow = tmem + 32u * ps + ((uint32_t)(warp * 32) << 16);
        tc_ld16(trow, acc);
        if (N > 16) tc_ld16(trow + 16, acc + 16);
        const long long L = d.L, nfib = d.L * d.R;
        if (dpf < nfib) {
          long long l, r;
          fibre_lr(dpf, L, nfib, l, r);
          cplx* y0 = d.Y + l + L * (long long)nout * r;
          float4* y0f = reinterpret_cast<float4*>(y0);
          const bool unit_alpha = (d.alpha.x == 1.0 && d.alpha.y == 0.0);
#pragma unroll
          for (int jo = 0; jo < TC_MAXN; ++jo) {
            if (jo >= nout) break;
            const float re = acc[2 * jo], im = acc[2 * jo + 1];
            if (d.yfmt == TF_F32) {
              reinterpret_cast<float2*>(d.Y)[l + L * ((long long)nout * r + jo)] = make_float2(re, im);
            } else if (d.yfmt) {
              y0f[L * jo] = make_float4(re, im, 0.f, 0.f);
            } else {
              const cplx a = mkc(f2d_exact(re), f2d_exact(im));
              cplx v = unit_alpha ? a : cmul(d.alpha, a);
              if (d.accumulate) v = cadd(v, y0[L * jo]);
              y0[L * jo] = v;
            }
          }
        }
      }
    }
    if (!have || !ok) break;
    prev_di = di;
    prev_p = p;
  }
  if (!ok && tid == 0) atomicExch(&g_tc_timeout, 1);
  tc_fence_before();
  __syncthreads();
  if (warp == 0) {
    tc_fence_after();
    tc_dealloc(tmem, 64);
  }
}

static int g_tc_nsm = 0;
// pipeline stages of the tensor-core mode product (MACAW_GB300_TC_STAGES=1 or 2)
static int g_tc_stages = 1;
// smallest largest-SPF-count of a batch that single contexts send to the tensor
// cores (MACAW_GB300_TC_MIN_N or mctdh_tensor_core_config).  Default 17, i.e.
// none: on the benchmark model the FP32 CUDA-core kernel is faster at 8 and at
// 12 SPFs and its round-to-nearest sums drift less over long propagations.
static int g_tc_min_n = 17;

// Once per process, outside any stream capture (context creation calls it): the
// SM count and the dynamic shared-memory limit of the tensor-core kernel.
void tc_prepare() {
  if (g_tc_nsm) return;
  int dev = 0, nsm = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  cudaFuncSetAttribute(prod_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                       2 * TC_NPART * (TC_ROWS * 2 * TC_MAXN * 4 + 2 * TC_MAXN * 2 * TC_MAXN * 4));
  const char* e = getenv("MACAW_GB300_TC_STAGES");
  g_tc_stages = (e && e[0] == '2') ? 2 : 1;
  const char* m = getenv("MACAW_GB300_TC_MIN_N");
  if (m && atoi(m) > 0) g_tc_min_n = atoi(m);
  g_tc_nsm = nsm > 0 ? nsm : 152;
}

// Tensor-core path for FP32 products of nin, nout <= 16, from the threshold on
// (force: any size up to 16); false: not taken
bool launch_prod_tc(const ProdDesc* d_descs, int ndesc, long long nblocks, int maxn, cudaStream_t st, bool force) {
  if (maxn > TC_MAXN || (!force && maxn < g_tc_min_n) || ndesc <= 0 || nblocks <= 0 || !g_tc_nsm) return false;
  const int K = ((2 * maxn + 7) / 8) * 8;
  const int N = 2 * maxn <= 16 ? 16 : 32;
  const size_t stage = (size_t)TC_NPART * ((size_t)TC_ROWS * K * 4 + (size_t)N * K * 4);
  const int nstage = g_tc_stages;
  const size_t smem = stage * nstage;
  const int per_sm = std::max(1, std::min(8, (int)((220 * 1024) / smem)));
  const long long grid = std::min<long long>(nblocks, (long long)g_tc_nsm * per_sm);
  prod_tc_kernel<<<(unsigned)grid, TC_ROWS, smem, st>>>(d_descs, ndesc, nblocks, K, N, nstage);
  return true;
}

// the timeout flag (cleared when `clear`), or -1 when it could not be read
int tc_timeout_flag(bool clear) {
  int v = 0;
  if (cudaMemcpyFromSymbol(&v, g_tc_timeout, sizeof(int)) != cudaSuccess) return -1;
  if (clear && v) {
    const int z = 0;
    if (cudaMemcpyToSymbol(g_tc_timeout, &z, sizeof(int)) != cudaSuccess) return -1;
  }
  return v;
}

extern "C" int64_t mctdh_tensor_core_status(int64_t* enabled, int64_t* timeouts) {
  if (enabled) *enabled = tc_enabled() ? 1 : 0;
  if (timeouts) {
    const int v = tc_timeout_flag(true);
    if (v < 0) return MCTDH_ECUDA;
    *timeouts = v;
  }
  return MCTDH_OK;
}

extern "C" int64_t mctdh_tensor_core_config(int64_t min_n, int64_t stages) {
  if (min_n < 0 || stages < 0 || stages > 2) return MCTDH_EARG;
  if (min_n > 0) g_tc_min_n = (int)min_n;
  if (stages > 0) g_tc_stages = (int)stages;
  return MCTDH_OK;
}
