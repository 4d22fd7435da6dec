// FP64 kernels of the G-MCTDH equation-of-motion path for sm_103a.
//
// On GB300 FP64 runs on the CUDA cores at a small fraction of the FP32 rate, so
// these kernels are written to spend FP64 FMAs only on the algebra the EOM needs:
// each fibre of a tensor is read once into registers (mode products), fibre tiles
// are staged in shared memory for the single-hole contractions, and reductions
// are two-stage with a fixed summation order so reruns are bitwise identical.
#include <algorithm>

#include "kernels.cuh"
#include <stdio.h>
#include <stdlib.h>

// ---------------------------------------------------------------------------
// descriptor lookup: descriptors are sorted by block_start
// ---------------------------------------------------------------------------
template <typename D>
__device__ __forceinline__ int find_desc_at(const D* descs, int ndesc, long long b) {
  int lo = 0, hi = ndesc - 1;
  while (lo < hi) {
    int mid = (lo + hi + 1) >> 1;
    if (descs[mid].block_start <= b) lo = mid; else hi = mid - 1;
  }
  return lo;
}
template <typename D>
__device__ __forceinline__ int find_desc(const D* descs, int ndesc) {
  return find_desc_at(descs, ndesc, (long long)blockIdx.x);
}

// ---------------------------------------------------------------------------
// Batched mode product (Mult_HeM_MatV / Mult_GM_MatV, gmctdh_objects.f90:1407-1468)
// One thread owns one fibre (l, :, r): it reads the nin inputs once into
// registers and writes the nout outputs.
// ---------------------------------------------------------------------------
// acc (hi, lo) += a * b for FP32 pairs a = ah + al, b = bh + bl: the leading
// product is split exactly with an FMA, the sum keeps its rounding error in lo.
__device__ __forceinline__ void df_fma(float& sh, float& sl, float ah, float al, float bh, float bl) {
  const float p = ah * bh;
  float e = fmaf(ah, bh, -p);
  e = fmaf(ah, bl, e);
  e = fmaf(al, bh, e);
  const float s = sh + p;
  const float bp = s - sh;
  const float t = (sh - (s - bp)) + (p - bp);
  sh = s;
  sl += t + e;
}

// acc (hi, lo) += a * b for plain FP32 a, b (no low parts): the same compensated
// sum as df_fma without the two correction products that vanish.
__device__ __forceinline__ void df_fma0(float& sh, float& sl, float a, float b) {
  const float p = a * b;
  const float e = fmaf(a, b, -p);
  const float s = sh + p;
  const float bp = s - sh;
  const float t = (sh - (s - bp)) + (p - bp);
  sh = s;
  sl += t + e;
}

// acc += conj(x) y for complex split operands (re hi, im hi, re lo, im lo):
// re = xr yr + xi yi, im = xr yi - xi yr, each real product compensated
__device__ __forceinline__ void df_cfma(float* h, float* l, const float4& x, const float4& y) {
  df_fma(h[0], l[0], x.x, x.z, y.x, y.z);
  df_fma(h[0], l[0], x.y, x.w, y.y, y.w);
  df_fma(h[1], l[1], x.x, x.z, y.y, y.w);
  df_fma(h[1], l[1], -x.y, -x.w, y.x, y.z);
}
// the same for complex FP32 operands (no low parts)
__device__ __forceinline__ void df_cfma0(float* h, float* l, const float2& x, const float2& y) {
  df_fma0(h[0], l[0], x.x, y.x);
  df_fma0(h[0], l[0], x.y, y.y);
  df_fma0(h[1], l[1], x.x, y.y);
  df_fma0(h[1], l[1], -x.y, y.x);
}

// PREC 0: FP64.  PREC 1: FP32 -- the products of the FP32-rounded x and M are
// accumulated in FP32 (~1e-7 relative; the split's correction products would sit
// at the accumulation's own rounding level), outputs complex FP32 (TF_F32) or
// FP64.  PREC 2: x and M split into hi + lo FP32 parts, x*M = xh*Mh + xh*Ml + xl*Mh
// with the sum carried as an FP32 hi/lo pair (compensated), ~1e-13 relative.
// Block `bb` of the batch (blockIdx.x of the plain launch; persistent CTAs walk
// the blocks).
template <int MAXN, int PREC>
__device__ __forceinline__ void prod_block(const ProdDesc* __restrict__ descs, int ndesc, long long bb) {
  __shared__ int s_di;
  __shared__ cplx Ms[PREC == 0 ? MAXN * MAXN : 1];
  __shared__ cplxf Mh[PREC == 0 ? 1 : MAXN * MAXN];
  __shared__ cplxf Ml[PREC == 0 ? 1 : MAXN * MAXN];
  if (threadIdx.x == 0) s_di = find_desc_at(descs, ndesc, bb);
  __syncthreads();
  const ProdDesc& d = descs[s_di];
  const int nin = d.nin, nout = d.nout;
  for (int e = threadIdx.x; e < nin * nout; e += blockDim.x) {
    int jo = e % nout, ji = e / nout;
    cplx v = d.conjT ? cconj(d.M[ji + (long long)d.ldm * jo]) : d.M[jo + (long long)d.ldm * ji];
    if (PREC == 0) {
      Ms[jo + MAXN * ji] = v;
    } else {
      float hx, lx, hy, ly;
      split_d2f(v.x, hx, lx);
      split_d2f(v.y, hy, ly);
      if (PREC == 1) {
        Mh[jo + MAXN * ji] = make_float2(hx + lx, hy + ly);   // rounded to nearest
      } else {
        Mh[jo + MAXN * ji] = make_float2(hx, hy);
        Ml[jo + MAXN * ji] = make_float2(lx, ly);
      }
    }
  }
  __syncthreads();
  const long long p = (bb - d.block_start) * blockDim.x + threadIdx.x;
  const long long L = d.L, nfib = L * d.R;
  if (p >= nfib) return;
  long long l, r;
  fibre_lr(p, L, nfib, l, r);
  const long long xi0 = l + L * (long long)nin * r;
  cplx* y0 = d.Y + l + L * (long long)nout * r;
  const cplx alpha = d.alpha;
  if (PREC == 0) {
    cplx x[MAXN];
#pragma unroll
    for (int j = 0; j < MAXN; ++j) x[j] = (j < nin) ? load_c(d.X, xi0 + L * j, d.xfmt) : mkc(0.0, 0.0);
    for (int jo = 0; jo < nout; ++jo) {
      cplx acc = mkc(0.0, 0.0);
#pragma unroll
      for (int j = 0; j < MAXN; ++j)
        if (j < nin) cfma(acc, Ms[jo + MAXN * j], x[j]);
      cplx v = cmul(alpha, acc);
      if (d.accumulate) v = cadd(v, y0[L * jo]);
      y0[L * jo] = v;
    }
  } else {
    cplxf xh[MAXN], xl[MAXN];
#pragma unroll
    for (int j = 0; j < MAXN; ++j) {
      const float4 w = (j < nin) ? load_split(d.X, xi0 + L * j, d.xfmt) : make_float4(0.f, 0.f, 0.f, 0.f);
      if (PREC == 1) {
        xh[j] = make_float2(w.x + w.z, w.y + w.w);   // rounded to nearest
      } else {
        xh[j] = make_float2(w.x, w.y);
        xl[j] = make_float2(w.z, w.w);
      }
    }
    const bool unit_alpha = (alpha.x == 1.0 && alpha.y == 0.0);
    float4* y0f = reinterpret_cast<float4*>(y0);
    for (int jo = 0; jo < nout; ++jo) {
      cplx accd;
      if (PREC == 1) {
        // FP32 values rounded to nearest: hi + lo of the split, added in FP32
        cplxf acc = make_float2(0.f, 0.f);
#pragma unroll
        for (int j = 0; j < MAXN; ++j)
          if (j < nin) acc = cfmaf_(acc, Mh[jo + MAXN * j], xh[j]);
        if (d.yfmt == TF_F32) {   // 8-byte elements: index from the tensor's base
          reinterpret_cast<float2*>(d.Y)[l + L * ((long long)nout * r + jo)] = acc;
          continue;
        }
        if (d.yfmt) {
          y0f[L * jo] = make_float4(acc.x, acc.y, 0.f, 0.f);
          continue;
        }
        accd = mkc(f2d_exact(acc.x), f2d_exact(acc.y));
      } else {
        float rh = 0.f, rl = 0.f, ih = 0.f, il = 0.f;
#pragma unroll
        for (int j = 0; j < MAXN; ++j)
          if (j < nin) {
            const cplxf mh = Mh[jo + MAXN * j], ml = Ml[jo + MAXN * j];
            // real: mr*xr - mi*xi ; imag: mr*xi + mi*xr
            df_fma(rh, rl, mh.x, ml.x, xh[j].x, xl[j].x);
            df_fma(rh, rl, -mh.y, -ml.y, xh[j].y, xl[j].y);
            df_fma(ih, il, mh.x, ml.x, xh[j].y, xl[j].y);
            df_fma(ih, il, mh.y, ml.y, xh[j].x, xl[j].x);
          }
        if (d.yfmt) {
          y0f[L * jo] = make_float4(rh, ih, rl, il);
          continue;
        }
        accd = mkc(f2d_exact(rh) + f2d_exact(rl), f2d_exact(ih) + f2d_exact(il));
      }
      cplx v = unit_alpha ? accd : cmul(alpha, accd);
      if (d.accumulate) v = cadd(v, y0[L * jo]);
      y0[L * jo] = v;
    }
  }
}

template <int MAXN, int PREC>
__global__ void __launch_bounds__(128) prod_kernel(const ProdDesc* __restrict__ descs, int ndesc) {
  prod_block<MAXN, PREC>(descs, ndesc, (long long)blockIdx.x);
}

// Persistent form: gridDim.x CTAs walk the batch's blocks in a fixed stride.
template <int MAXN, int PREC>
__global__ void __launch_bounds__(128) prod_kernel_persistent(const ProdDesc* __restrict__ descs, int ndesc,
                                                              long long nblocks) {
  for (long long bb = blockIdx.x; bb < nblocks; bb += gridDim.x) {
    prod_block<MAXN, PREC>(descs, ndesc, bb);
    __syncthreads();   // the block's shared operands are rewritten by the next one
  }
}

// Tensor-core kernels (tc.cu) may serve the FP32 products unless
// MACAW_GB300_TC=0 selects the CUDA-core kernels (read once per process).
bool tc_enabled() {
  static int on = -1;
  if (on < 0) {
    const char* e = getenv("MACAW_GB300_TC");
    on = (e && e[0] == '0') ? 0 : 1;
  }
  return on == 1;
}

// tc: 0 CUDA-core kernel, 1 tensor cores from the configured SPF count on,
// 2 tensor cores for every size they take (the ensemble autotuner's candidate).
// persist > 0: at most that many persistent CTAs walk the blocks.
void launch_prod(const ProdDesc* d_descs, int ndesc, long long nblocks, int maxn, cudaStream_t st, int prec,
                 int tc, int persist) {
  if (ndesc <= 0 || nblocks <= 0) return;
  if (prec == 1 && tc && tc_enabled() && launch_prod_tc(d_descs, ndesc, nblocks, maxn, st, tc == 2)) return;
  if (persist > 0 && nblocks > persist) {
    const unsigned g = (unsigned)persist;
    if (maxn <= 8) {
      if (prec == 0) prod_kernel_persistent<8, 0><<<g, 128, 0, st>>>(d_descs, ndesc, nblocks);
      else if (prec == 1) prod_kernel_persistent<8, 1><<<g, 128, 0, st>>>(d_descs, ndesc, nblocks);
      else prod_kernel_persistent<8, 2><<<g, 128, 0, st>>>(d_descs, ndesc, nblocks);
    } else if (maxn <= 12) {
      if (prec == 0) prod_kernel_persistent<12, 0><<<g, 128, 0, st>>>(d_descs, ndesc, nblocks);
      else if (prec == 1) prod_kernel_persistent<12, 1><<<g, 128, 0, st>>>(d_descs, ndesc, nblocks);
      else prod_kernel_persistent<12, 2><<<g, 128, 0, st>>>(d_descs, ndesc, nblocks);
    } else {
      if (prec == 0) prod_kernel_persistent<MAXN_SPF, 0><<<g, 128, 0, st>>>(d_descs, ndesc, nblocks);
      else if (prec == 1) prod_kernel_persistent<MAXN_SPF, 1><<<g, 128, 0, st>>>(d_descs, ndesc, nblocks);
      else prod_kernel_persistent<MAXN_SPF, 2><<<g, 128, 0, st>>>(d_descs, ndesc, nblocks);
    }
    return;
  }
  const unsigned nb = (unsigned)nblocks;
  // register arrays sized for the batch's largest SPF count: no dead unrolled
  // iterations and fewer registers (more resident warps) at 8 SPFs and below
  if (maxn <= 8) {
    if (prec == 0) prod_kernel<8, 0><<<nb, 128, 0, st>>>(d_descs, ndesc);
    else if (prec == 1) prod_kernel<8, 1><<<nb, 128, 0, st>>>(d_descs, ndesc);
    else prod_kernel<8, 2><<<nb, 128, 0, st>>>(d_descs, ndesc);
  } else if (maxn <= 12) {
    if (prec == 0) prod_kernel<12, 0><<<nb, 128, 0, st>>>(d_descs, ndesc);
    else if (prec == 1) prod_kernel<12, 1><<<nb, 128, 0, st>>>(d_descs, ndesc);
    else prod_kernel<12, 2><<<nb, 128, 0, st>>>(d_descs, ndesc);
  } else {
    if (prec == 0) prod_kernel<MAXN_SPF, 0><<<nb, 128, 0, st>>>(d_descs, ndesc);
    else if (prec == 1) prod_kernel<MAXN_SPF, 1><<<nb, 128, 0, st>>>(d_descs, ndesc);
    else prod_kernel<MAXN_SPF, 2><<<nb, 128, 0, st>>>(d_descs, ndesc);
  }
}

// ---------------------------------------------------------------------------
// Batched single-hole contraction, first stage (zher2k / zgemm('T','N') loops of
// Calc_rho1mode and Calc_MeanField, gmctdh_objects.f90:452-457, :595-600).
// Block b of a descriptor handles fibre tiles b, b + nblk, ...; every thread owns
// one (j1, j2) pair and a fibre group; groups are summed in shared memory.
// ---------------------------------------------------------------------------
// 1 x 1 contractions (inner products): every thread strides over elements with
// coalesced loads, the block reduces in shared memory.
template <int PREC>
__device__ void dot_block(const HoleDesc& d, int b, cplx* red) {
  const long long n = d.L * d.R;
  const int tid = threadIdx.x;
  cplx acc = mkc(0, 0);
  for (long long i = (long long)b * HOLE_THREADS + tid; i < n; i += (long long)d.nblk * HOLE_THREADS)
    cfma_conj(acc, load_c(d.X, i, d.xfmt), load_c(d.Y, i, d.yfmt));
  red[tid] = acc;
  __syncthreads();
  for (int s = HOLE_THREADS / 2; s > 0; s >>= 1) {
    if (tid < s) red[tid] = cadd(red[tid], red[tid + s]);
    __syncthreads();
  }
  if (tid == 0) d.partial[b] = red[0];
}

// PREC 0: FP64.  PREC 2: operands split into FP32 hi + lo parts, products and sums
// carried as compensated FP32 pairs (df_fma), ~1e-13 relative; complex-FP32
// operands on both sides skip the vanishing low-part products (df_fma0).
// PREC 1: FP32 operands (rounded to nearest), FP32 products and sums (~1e-7
// relative), the block partials widened to FP64 for the deterministic reduction.
template <int PREC>
__device__ __forceinline__ void hole_block(const HoleDesc* __restrict__ descs, int ndesc, long long bb) {
  __shared__ int s_di;
  __shared__ cplx Xs[HOLE_TILE * MAXN_SPF];
  __shared__ cplx Ys[HOLE_TILE * MAXN_SPF];
  float4* Xf = reinterpret_cast<float4*>(Xs);   // PREC 2: (re hi, im hi, re lo, im lo)
  float4* Yf = reinterpret_cast<float4*>(Ys);
  float2* X1 = reinterpret_cast<float2*>(Xs);   // PREC 1 and complex-FP32 operands: (re, im)
  float2* Y1 = reinterpret_cast<float2*>(Ys);
  if (threadIdx.x == 0) s_di = find_desc_at(descs, ndesc, bb);
  __syncthreads();
  const HoleDesc& d = descs[s_di];
  const int b = (int)(bb - d.block_start);
  const int n1 = d.n1, n2 = d.n2, npairs = n1 * n2;
  if (npairs == 1 && d.L * d.R >= HOLE_THREADS) {
    dot_block<PREC>(d, b, Xs);
    return;
  }
  const long long L = d.L, nfib = d.L * d.R;
  const long long ntiles = (nfib + HOLE_TILE - 1) / HOLE_TILE;
  const int tid = threadIdx.x;
  // PREC 2 with complex-FP32 operands on both sides: exact products of plain FP32
  // numbers into the compensated sums (the staging keeps (re, im) pairs)
  const bool f32in = PREC == 2 && d.xfmt == TF_F32 && d.yfmt == TF_F32;
  const bool small = npairs <= HOLE_THREADS;
  const int G = small ? HOLE_THREADS / npairs : 1;
  const int pair0 = small ? tid % npairs : tid;
  const int g = small ? tid / npairs : 0;
  // PREC 2 with even n1, n2: every thread owns a 2 x 2 block of (j1, j2) pairs, so
  // each staged value it reads feeds two products (half the shared-memory reads
  // per product and four independent accumulation chains)
  const bool quad = PREC == 2 && small && ((n1 | n2) & 1) == 0;
  // X = Y (density matrices, SPF overlaps): C is Hermitian, so only the blocks on
  // and above the diagonal are computed (the others are their conjugates) and the
  // tensor is staged once
  const bool sym = quad && d.X == d.Y && n1 == n2 && d.xfmt == d.yfmt;
  const int h1 = n1 >> 1, nq = sym ? h1 * (h1 + 1) / 2 : h1 * (n2 >> 1);
  const int Gq = quad ? HOLE_THREADS / nq : 0;
  const int qd = quad ? tid % nq : 0, gq = quad ? tid / nq : 0;
  int i1 = 2 * (qd % (h1 > 0 ? h1 : 1)), i2 = 2 * (qd / (h1 > 0 ? h1 : 1));
  if (sym) {   // qd -> (qi <= qj), qj-major: qd = qj (qj + 1) / 2 + qi
    int rem = qd, qj = 0;
    while (rem > qj) { rem -= qj + 1; ++qj; }
    i1 = 2 * rem;
    i2 = 2 * qj;
  }
  cplx acc[4] = {mkc(0, 0), mkc(0, 0), mkc(0, 0), mkc(0, 0)};
  float ah[4][2] = {{0.f, 0.f}, {0.f, 0.f}, {0.f, 0.f}, {0.f, 0.f}};
  float al[4][2] = {{0.f, 0.f}, {0.f, 0.f}, {0.f, 0.f}, {0.f, 0.f}};
  // Staging: thread tid always loads fibre q = tid % HOLE_TILE of a tile and the
  // columns j = tid / HOLE_TILE, + HOLE_THREADS / HOLE_TILE, ...; its fibre's
  // (l, r) is carried from tile to tile instead of divided out per element.
  static_assert(HOLE_THREADS % HOLE_TILE == 0, "staging assumes whole tiles per thread row");
  static_assert(4 * HOLE_THREADS <= HOLE_TILE * MAXN_SPF, "the 2 x 2 partials fit the staging tile");
  const int qt = tid % HOLE_TILE, jt = tid / HOLE_TILE, jstep = HOLE_THREADS / HOLE_TILE;
  long long pcur = (long long)b * HOLE_TILE + qt;
  long long lcur = pcur % L, rcur = pcur / L;
  const long long pstep = (long long)d.nblk * HOLE_TILE;
  const long long dl = pstep % L, dr = pstep / L;
  for (long long tile = b; tile < ntiles; tile += d.nblk) {
    const bool in_range = pcur < nfib;
    const long long xb = lcur + L * (long long)n1 * rcur, yb = lcur + L * (long long)n2 * rcur;
    pcur += pstep;
    lcur += dl;
    rcur += dr;
    if (lcur >= L) { lcur -= L; rcur += 1; }
    const int q = qt;
    for (int j = jt; j < n1; j += jstep) {
      const long long idx = in_range ? xb + L * j : -1;
      if (PREC == 0) {
        Xs[q * MAXN_SPF + j] = (idx >= 0) ? load_c(d.X, idx, d.xfmt) : mkc(0, 0);
      } else if (PREC == 1 || f32in) {
        const float4 w = (idx >= 0) ? load_split(d.X, idx, d.xfmt) : make_float4(0.f, 0.f, 0.f, 0.f);
        X1[q * MAXN_SPF + j] = make_float2(w.x + w.z, w.y + w.w);
      } else {
        Xf[q * MAXN_SPF + j] = (idx >= 0) ? load_split(d.X, idx, d.xfmt) : make_float4(0.f, 0.f, 0.f, 0.f);
      }
    }
    for (int j = jt; j < (sym ? 0 : n2); j += jstep) {
      const long long idx = in_range ? yb + L * j : -1;
      if (PREC == 0) {
        Ys[q * MAXN_SPF + j] = (idx >= 0) ? load_c(d.Y, idx, d.yfmt) : mkc(0, 0);
      } else if (PREC == 1 || f32in) {
        const float4 w = (idx >= 0) ? load_split(d.Y, idx, d.yfmt) : make_float4(0.f, 0.f, 0.f, 0.f);
        Y1[q * MAXN_SPF + j] = make_float2(w.x + w.z, w.y + w.w);
      } else {
        Yf[q * MAXN_SPF + j] = (idx >= 0) ? load_split(d.Y, idx, d.yfmt) : make_float4(0.f, 0.f, 0.f, 0.f);
      }
    }
    __syncthreads();
    if (quad) {
      // pairs (i1, i2), (i1 + 1, i2), (i1, i2 + 1), (i1 + 1, i2 + 1) in ah/al[0..3]
      const float2* Y1r = sym ? X1 : Y1;
      const float4* Yfr = sym ? Xf : Yf;
      if (gq < Gq) {
        for (int q = gq; q < HOLE_TILE; q += Gq) {
          if (f32in) {
            const float2 xa = X1[q * MAXN_SPF + i1], xb = X1[q * MAXN_SPF + i1 + 1];
            const float2 ya = Y1r[q * MAXN_SPF + i2], yb = Y1r[q * MAXN_SPF + i2 + 1];
            df_cfma0(ah[0], al[0], xa, ya);
            df_cfma0(ah[1], al[1], xb, ya);
            df_cfma0(ah[2], al[2], xa, yb);
            df_cfma0(ah[3], al[3], xb, yb);
          } else {
            const float4 xa = Xf[q * MAXN_SPF + i1], xb = Xf[q * MAXN_SPF + i1 + 1];
            const float4 ya = Yfr[q * MAXN_SPF + i2], yb = Yfr[q * MAXN_SPF + i2 + 1];
            df_cfma(ah[0], al[0], xa, ya);
            df_cfma(ah[1], al[1], xb, ya);
            df_cfma(ah[2], al[2], xa, yb);
            df_cfma(ah[3], al[3], xb, yb);
          }
        }
      }
      __syncthreads();
      continue;
    }
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      int pr, q0, qs;
      if (small) {
        if (k > 0 || g >= G) break;
        pr = pair0; q0 = g; qs = G;
      } else {
        pr = pair0 + HOLE_THREADS * k;
        if (pr >= npairs) break;
        q0 = 0; qs = 1;
      }
      const int j1 = pr % n1, j2 = pr / n1;
      for (int q = q0; q < HOLE_TILE; q += qs) {
        if (PREC == 0) {
          cfma_conj(acc[k], Xs[q * MAXN_SPF + j1], Ys[q * MAXN_SPF + j2]);
        } else if (PREC == 1) {
          const float2 x = X1[q * MAXN_SPF + j1], y = Y1[q * MAXN_SPF + j2];
          ah[k][0] = fmaf(x.x, y.x, ah[k][0]);
          ah[k][0] = fmaf(x.y, y.y, ah[k][0]);
          ah[k][1] = fmaf(x.x, y.y, ah[k][1]);
          ah[k][1] = fmaf(-x.y, y.x, ah[k][1]);
        } else if (f32in) {
          // complex FP32 operands on both sides (no low parts)
          const float2 x = X1[q * MAXN_SPF + j1], y = Y1[q * MAXN_SPF + j2];
          df_fma0(ah[k][0], al[k][0], x.x, y.x);
          df_fma0(ah[k][0], al[k][0], x.y, y.y);
          df_fma0(ah[k][1], al[k][1], x.x, y.y);
          df_fma0(ah[k][1], al[k][1], -x.y, y.x);
        } else {
          // conj(x) y: re = xr yr + xi yi, im = xr yi - xi yr
          const float4 x = Xf[q * MAXN_SPF + j1], y = Yf[q * MAXN_SPF + j2];
          df_fma(ah[k][0], al[k][0], x.x, x.z, y.x, y.z);
          df_fma(ah[k][0], al[k][0], x.y, x.w, y.y, y.w);
          df_fma(ah[k][1], al[k][1], x.x, x.z, y.y, y.w);
          df_fma(ah[k][1], al[k][1], -x.y, -x.w, y.x, y.z);
        }
      }
    }
    __syncthreads();
  }
  if (PREC != 0) {
#pragma unroll
    for (int k = 0; k < 4; ++k)
      acc[k] = mkc(f2d_exact(ah[k][0]) + f2d_exact(al[k][0]), f2d_exact(ah[k][1]) + f2d_exact(al[k][1]));
  }
  cplx* out = d.partial + (long long)b * npairs;
  if (quad) {
    cplx* red = Xs;   // 4 * HOLE_THREADS <= HOLE_TILE * MAXN_SPF entries
#pragma unroll
    for (int k = 0; k < 4; ++k) red[4 * tid + k] = acc[k];
    __syncthreads();
    if (tid < npairs) {
      int j1 = tid % n1, j2 = tid / n1;
      const bool lower = sym && (j1 >> 1) > (j2 >> 1);   // conj of the transposed pair
      if (lower) { const int tmp = j1; j1 = j2; j2 = tmp; }
      const int qq = sym ? (j2 >> 1) * ((j2 >> 1) + 1) / 2 + (j1 >> 1) : (j1 >> 1) + h1 * (j2 >> 1);
      const int k = (j1 & 1) + 2 * (j2 & 1);
      cplx s = mkc(0, 0);
      for (int gg = 0; gg < Gq; ++gg) s = cadd(s, red[4 * (gg * nq + qq) + k]);
      out[tid] = lower ? cconj(s) : s;
    }
  } else if (small) {
    cplx* red = Xs;   // reuse (HOLE_TILE*MAXN_SPF >= HOLE_THREADS)
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
      int pr = pair0 + HOLE_THREADS * k;
      if (pr < npairs) out[pr] = acc[k];
    }
  }
}

template <int PREC>
__global__ void __launch_bounds__(HOLE_THREADS, 4) hole_kernel(const HoleDesc* __restrict__ descs, int ndesc) {
  hole_block<PREC>(descs, ndesc, (long long)blockIdx.x);
}

// Persistent form: gridDim.x CTAs walk the batch's blocks in a fixed stride (each
// block still writes its own partial, so the sums do not depend on the grid).
template <int PREC>
__global__ void __launch_bounds__(HOLE_THREADS, 4) hole_kernel_persistent(const HoleDesc* __restrict__ descs,
                                                                       int ndesc, long long nblocks) {
  for (long long bb = blockIdx.x; bb < nblocks; bb += gridDim.x) {
    hole_block<PREC>(descs, ndesc, bb);
    __syncthreads();   // the staging tiles are rewritten by the next block
  }
}

void launch_hole(const HoleDesc* d_descs, int ndesc, long long nblocks, cudaStream_t st, int prec, int persist) {
  if (ndesc <= 0 || nblocks <= 0) return;
  if (persist > 0 && nblocks > persist) {
    const unsigned g = (unsigned)persist;
    if (prec == 0) hole_kernel_persistent<0><<<g, HOLE_THREADS, 0, st>>>(d_descs, ndesc, nblocks);
    else if (prec == 1) hole_kernel_persistent<1><<<g, HOLE_THREADS, 0, st>>>(d_descs, ndesc, nblocks);
    else hole_kernel_persistent<2><<<g, HOLE_THREADS, 0, st>>>(d_descs, ndesc, nblocks);
    return;
  }
  if (prec == 0)
    hole_kernel<0><<<(unsigned)nblocks, HOLE_THREADS, 0, st>>>(d_descs, ndesc);
  else if (prec == 1)
    hole_kernel<1><<<(unsigned)nblocks, HOLE_THREADS, 0, st>>>(d_descs, ndesc);
  else
    hole_kernel<2><<<(unsigned)nblocks, HOLE_THREADS, 0, st>>>(d_descs, ndesc);
}

// ---------------------------------------------------------------------------
// Second stage: deterministic sum of partials into the target matrices.
// ---------------------------------------------------------------------------
// One block per target; the partial blocks of every term are spread over G thread
// groups (G = blockDim / (n1 n2) when that is > 1), each group sums its share in a
// fixed order, then the groups are added in group order (deterministic).
__global__ void __launch_bounds__(256) reduce_kernel(const RedTarget* __restrict__ tg,
                                                     const RedTerm* __restrict__ terms) {
  __shared__ cplx red[256], redT[256];
  const RedTarget& t = tg[blockIdx.x];
  const int npairs = t.n1 * t.n2;
  const int G = (npairs <= (int)blockDim.x / 2) ? (int)blockDim.x / npairs : 1;
  const int g = (G > 1) ? (int)threadIdx.x / npairs : 0;
  const int p0 = (G > 1) ? (int)threadIdx.x % npairs : (int)threadIdx.x;
  for (int base = 0; base < npairs; base += (G > 1 ? npairs : (int)blockDim.x)) {
    const int pr = base + p0;
    const bool act = (G > 1) ? (g < G) : (pr < npairs);
    cplx s = mkc(0, 0), sT = mkc(0, 0);
    if (act) {
      const int j1 = pr % t.n1, j2 = pr / t.n1;
      const int prT = j2 + t.n1 * j1;
      const int prC = j2 + t.n2 * j1;   // element (j2, j1) of an n2 x n1 source (conjT terms)
      for (int k = 0; k < t.count; ++k) {
        const RedTerm& rt = terms[t.first + k];
        cplx a = mkc(0, 0), aT = mkc(0, 0);
        for (int bb = g; bb < rt.nblk; bb += G) {
          if (rt.conjT) {
            a = cadd(a, cconj(rt.partial[(long long)bb * npairs + prC]));
            if (t.hermitize) aT = cadd(aT, cconj(rt.partial[(long long)bb * npairs + pr]));
          } else {
            a = cadd(a, rt.partial[(long long)bb * npairs + pr]);
            if (t.hermitize) aT = cadd(aT, rt.partial[(long long)bb * npairs + prT]);
          }
        }
        s = cadd(s, cmul(rt.alpha, a));
        if (t.hermitize) sT = cadd(sT, cmul(rt.alpha, aT));
      }
    }
    if (G > 1) {
      red[threadIdx.x] = s;
      redT[threadIdx.x] = sT;
      __syncthreads();
      if (g == 0) {
        for (int q = 1; q < G; ++q) {
          s = cadd(s, red[q * npairs + p0]);
          sT = cadd(sT, redT[q * npairs + p0]);
        }
      }
      __syncthreads();
    }
    if (act && g == 0) {
      const int j1 = pr % t.n1, j2 = pr / t.n1;
      if (t.hermitize) s = cscale(cadd(s, cconj(sT)), 0.5);
      cplx* o = t.out + j1 + (long long)t.ld * j2;
      *o = t.accumulate ? cadd(*o, s) : s;
    }
  }
}

void launch_reduce(const RedTarget* d_tg, int ntg, const RedTerm* d_terms, cudaStream_t st) {
  if (ntg <= 0) return;
  reduce_kernel<<<ntg, 256, 0, st>>>(d_tg, d_terms);
}

// ---------------------------------------------------------------------------
// h1mode and operator-applied SPFs for DVR modes (Calc_h1mode, hamilton.f90:416-482;
// MultTens / MultTensDiag, :577-629).  One block per (mode, operator).
// ---------------------------------------------------------------------------
// One block per (operator, SPF column j2): the primitive DOF operators act
// within each SPF, so a column is transformed in shared memory on its own
// (MultTens / MultTensDiag, hamilton.f90:577-629).  The DVR matrices of p, qp
// (i x real) and d^2/dq^2 (real) are applied with real arithmetic.  Then, when
// h1mode is wanted, the column j2 of phi_l^H (O phi_r), one warp per row j1.
__global__ void __launch_bounds__(256) h1_kernel(const H1Desc* __restrict__ descs) {
  extern __shared__ cplx sm[];
  const H1Desc& d = descs[blockIdx.x];
  const int j2 = blockIdx.y;
  if (j2 >= d.n2) return;
  const int G = d.G, n1 = d.n1;
  cplx* bufA = sm;
  cplx* bufB = sm + G;
  const cplx* src = d.phi_r + (long long)G * j2;
  for (int e = threadIdx.x; e < G; e += blockDim.x) bufA[e] = src[e];
  __syncthreads();
  int ll = 1;
  for (int k = 0; k < d.ndof; ++k) {
    const int ng = d.ng[k];
    const int ot = d.optype[k];
    if (ot != 0) {
      const cplx* M = d.mat[k];
      for (int e = threadIdx.x; e < G; e += blockDim.x) {
        const int a = e % ll;
        const int gg = (e / ll) % ng;
        const int bidx = e / (ll * ng);
        cplx v;
        if (ot == 2) {
          v = cscale(bufA[e], M[gg].x);
        } else {
          // psi(.., g, ..) <- sum_g' psi(.., g', ..) M(g', g)   (zlacrm from the right)
          const cplx* in = bufA + a + (long long)ll * ng * bidx;
          const cplx* mc = M + (long long)ng * gg;
          double sx = 0.0, sy = 0.0;
          if (ot == 1) {
            for (int gp = 0; gp < ng; ++gp) {
              const cplx x = in[(long long)ll * gp];
              sx = fma(mc[gp].x, x.x, sx);
              sy = fma(mc[gp].x, x.y, sy);
            }
            v = mkc(sx, sy);
          } else {
            for (int gp = 0; gp < ng; ++gp) {
              const cplx x = in[(long long)ll * gp];
              sx = fma(mc[gp].y, x.x, sx);
              sy = fma(mc[gp].y, x.y, sy);
            }
            v = mkc(-sy, sx);   // i * (real matrix x column)
          }
        }
        bufB[e] = v;
      }
      __syncthreads();
      cplx* t = bufA; bufA = bufB; bufB = t;
    }
    ll *= ng;
  }
  cplx* dst = d.ophi + (long long)G * j2;
  for (int e = threadIdx.x; e < G; e += blockDim.x) dst[e] = bufA[e];
  if (d.h == nullptr) return;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  for (int j1 = warp; j1 < n1; j1 += (int)(blockDim.x >> 5)) {
    const cplx* pl = d.phi_l + (long long)G * j1;
    cplx s = mkc(0, 0);
    for (int gg = lane; gg < G; gg += 32) cfma_conj(s, pl[gg], bufA[gg]);
    for (int o = 16; o > 0; o >>= 1) {
      s.x += __shfl_down_sync(0xffffffffu, s.x, o);
      s.y += __shfl_down_sync(0xffffffffu, s.y, o);
    }
    if (lane == 0) {
      if (d.same_state) d.X[j1 + n1 * j2] = s;
      else d.h[j1 + n1 * j2] = s;
    }
  }
}

// Split-FP32 variant of h1_kernel (precision modes 1 and 2): the column is held
// as FP32 (hi, lo) pairs, the DOF matrices come pre-split, every product is
// accumulated as a compensated FP32 pair (df_fma, ~1e-13 relative).
__global__ void __launch_bounds__(256) h1_split_kernel(const H1Desc* __restrict__ descs) {
  extern __shared__ float4 smf[];
  const H1Desc& d = descs[blockIdx.x];
  const int j2 = blockIdx.y;
  if (j2 >= d.n2) return;
  const int G = d.G, n1 = d.n1;
  float4* bufA = smf;
  float4* bufB = smf + G;
  const cplx* src = d.phi_r + (long long)G * j2;
  for (int e = threadIdx.x; e < G; e += blockDim.x) {
    const cplx v = src[e];
    float hx, lx, hy, ly;
    split_d2f(v.x, hx, lx);
    split_d2f(v.y, hy, ly);
    bufA[e] = make_float4(hx, hy, lx, ly);
  }
  __syncthreads();
  int ll = 1;
  for (int k = 0; k < d.ndof; ++k) {
    const int ng = d.ng[k];
    const int ot = d.optype[k];
    if (ot != 0) {
      const float2* Mf = d.matf[k];
      for (int e = threadIdx.x; e < G; e += blockDim.x) {
        const int a = e % ll;
        const int gg = (e / ll) % ng;
        const int bidx = e / (ll * ng);
        float rh = 0.f, rl = 0.f, ih = 0.f, il = 0.f;
        if (ot == 2) {
          const float4 x = bufA[e];
          const float2 m = Mf[gg];
          df_fma(rh, rl, m.x, m.y, x.x, x.z);
          df_fma(ih, il, m.x, m.y, x.y, x.w);
        } else {
          const float4* in = bufA + a + (long long)ll * ng * bidx;
          const float2* mc = Mf + (long long)ng * gg;
          for (int gp = 0; gp < ng; ++gp) {
            const float4 x = in[(long long)ll * gp];
            const float2 m = mc[gp];
            df_fma(rh, rl, m.x, m.y, x.x, x.z);
            df_fma(ih, il, m.x, m.y, x.y, x.w);
          }
        }
        bufB[e] = (ot == 3) ? make_float4(-ih, rh, -il, rl) : make_float4(rh, ih, rl, il);
      }
      __syncthreads();
      float4* t = bufA; bufA = bufB; bufB = t;
    }
    ll *= ng;
  }
  cplx* dst = d.ophi + (long long)G * j2;
  for (int e = threadIdx.x; e < G; e += blockDim.x) {
    const float4 x = bufA[e];
    dst[e] = mkc(f2d_exact(x.x) + f2d_exact(x.z), f2d_exact(x.y) + f2d_exact(x.w));
  }
  if (d.h == nullptr) return;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  for (int j1 = warp; j1 < n1; j1 += (int)(blockDim.x >> 5)) {
    const cplx* pl = d.phi_l + (long long)G * j1;
    float rh = 0.f, rl = 0.f, ih = 0.f, il = 0.f;
    for (int gg = lane; gg < G; gg += 32) {
      const cplx p = pl[gg];
      float phx, plx, phy, ply;
      split_d2f(p.x, phx, plx);
      split_d2f(p.y, phy, ply);
      const float4 x = bufA[gg];
      // conj(p) * x
      df_fma(rh, rl, phx, plx, x.x, x.z);
      df_fma(rh, rl, phy, ply, x.y, x.w);
      df_fma(ih, il, phx, plx, x.y, x.w);
      df_fma(ih, il, -phy, -ply, x.x, x.z);
    }
    cplx s = mkc(f2d_exact(rh) + f2d_exact(rl), f2d_exact(ih) + f2d_exact(il));
    for (int o = 16; o > 0; o >>= 1) {
      s.x += __shfl_down_sync(0xffffffffu, s.x, o);
      s.y += __shfl_down_sync(0xffffffffu, s.y, o);
    }
    if (lane == 0) {
      if (d.same_state) d.X[j1 + n1 * j2] = s;
      else d.h[j1 + n1 * j2] = s;
    }
  }
}

// Same-state h1mode = (X + X^H) / 2 (the zher2k form, hamilton.f90:500-506).
__global__ void h1_herm_kernel(const H1Desc* __restrict__ descs) {
  const H1Desc& d = descs[blockIdx.x];
  if (d.h == nullptr || !d.same_state) return;
  const int n1 = d.n1;
  for (int pr = threadIdx.x; pr < n1 * d.n2; pr += blockDim.x) {
    const int j1 = pr % n1, j2 = pr / n1;
    d.h[pr] = cscale(cadd(d.X[pr], cconj(d.X[j2 + n1 * j1])), 0.5);
  }
}

void launch_h1(const H1Desc* d_descs, int ndesc, int maxn2, size_t smem_bytes, bool with_h, cudaStream_t st,
               int prec) {
  if (ndesc <= 0) return;
  static size_t configured = 0;
  if (smem_bytes > 48 * 1024 && smem_bytes > configured) {
    cudaFuncSetAttribute(h1_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_bytes);
    cudaFuncSetAttribute(h1_split_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_bytes);
    configured = smem_bytes;
  }
  if (prec > 0) h1_split_kernel<<<dim3(ndesc, maxn2), 256, smem_bytes, st>>>(d_descs);
  else h1_kernel<<<dim3(ndesc, maxn2), 256, smem_bytes, st>>>(d_descs);
  if (with_h) h1_herm_kernel<<<ndesc, 128, 0, st>>>(d_descs);
}

// ---------------------------------------------------------------------------
// Parallel complex Jacobi eigen-decomposition of a Hermitian matrix (n <= 32)
// held in shared memory, run by one warp: the work zheev does inside StdRegInv
// (maths.f90:36).  Each round rotates the n/2 disjoint index pairs of a
// round-robin schedule at once (column rotations A J, then row rotations J^H (A J);
// rotations of disjoint pairs commute), so a sweep is n-1 rounds.  A pair is
// rotated when |a_pq|^2 > 1e-38 ||A||_F^2 and |a_pq|^2 > 1e-32 |a_pp a_qq|; the
// sweep count is capped.  A[i + ld*j], V likewise.  *ok: the sweeps converged.
// ---------------------------------------------------------------------------
#define JAC_MAX_SWEEPS 40
struct JacRot {
  double c, s, tm, app, aqq;
  cplx u;
  int p, q, rot;
};

__device__ void jacobi_herm(cplx* A, cplx* V, int n, int ld, JacRot* R, bool* ok) {
  const int lane = threadIdx.x;   // blockDim.x == 32
  for (int e = lane; e < n * n; e += 32) {
    int i = e % n, j = e / n;
    V[i + ld * j] = mkc(i == j ? 1.0 : 0.0, 0.0);
  }
  __syncwarp();
  double fro2 = 0.0;
  for (int e = 0; e < n * n; ++e) { int i = e % n, j = e / n; fro2 += cabs2(A[i + ld * j]); }
  const int m = n + (n & 1);      // even count; index n is a dummy for odd n
  const int npair = m / 2;
  bool converged = (n <= 1);
  for (int sweep = 0; sweep < JAC_MAX_SWEEPS && !converged; ++sweep) {
    bool any = false;
    for (int r = 0; r < m - 1; ++r) {
      int rot = 0;
      if (lane < npair) {
        // circle schedule: (r, m-1) and ((r+j) mod (m-1), (r-j) mod (m-1))
        int a = (lane == 0) ? r : (r + lane) % (m - 1);
        int b = (lane == 0) ? m - 1 : (r - lane + (m - 1)) % (m - 1);
        const int p = min(a, b), q = max(a, b);
        JacRot& J = R[lane];
        J.p = p;
        J.q = q;
        if (q < n) {
          const cplx apq = A[p + ld * q];
          const double m2 = cabs2(apq);
          const double app = A[p + ld * p].x, aqq = A[q + ld * q].x;
          rot = (m2 > 1e-38 * fro2) && (m2 > 1e-32 * fabs(app * aqq));
          if (rot) {
            // one reciprocal square root for |a_pq| (the FP64 pipe is the bottleneck here)
            const double rm = rsqrt(m2);
            const double mag = m2 * rm;
            const double tau = (aqq - app) * 0.5 * rm;
            const double t = (tau >= 0.0 ? 1.0 : -1.0) / (fabs(tau) + sqrt(1.0 + tau * tau));
            J.c = rsqrt(1.0 + t * t);
            J.s = t * J.c;
            J.u = mkc(apq.x * rm, apq.y * rm);
            J.tm = t * mag;
            J.app = app;
            J.aqq = aqq;
          }
        }
        J.rot = rot;
      }
      const unsigned ballot = __ballot_sync(0xffffffffu, rot);
      __syncwarp();
      if (ballot == 0) continue;
      any = true;
      // column rotations: work items (row, pair) spread over the lanes (one item per
      // lane for n <= 8); pairs are disjoint, so items never share an element
      for (int it = lane; it < n * npair; it += 32) {
        const int row = it % n;
        const JacRot& J = R[it / n];
        if (!J.rot) continue;
        const cplx uc = cconj(J.u);
        cplx ap = A[row + ld * J.p], aq = A[row + ld * J.q];
        A[row + ld * J.p] = csub(cscale(ap, J.c), cscale(cmul(uc, aq), J.s));
        A[row + ld * J.q] = cadd(cscale(cmul(J.u, ap), J.s), cscale(aq, J.c));
        cplx vp = V[row + ld * J.p], vq = V[row + ld * J.q];
        V[row + ld * J.p] = csub(cscale(vp, J.c), cscale(cmul(uc, vq), J.s));
        V[row + ld * J.q] = cadd(cscale(cmul(J.u, vp), J.s), cscale(vq, J.c));
      }
      __syncwarp();
      // row rotations: items (column, pair)
      for (int it = lane; it < n * npair; it += 32) {
        const int col = it % n;
        const JacRot& J = R[it / n];
        if (!J.rot) continue;
        cplx ap = A[J.p + ld * col], aq = A[J.q + ld * col];
        A[J.p + ld * col] = csub(cscale(ap, J.c), cscale(cmul(J.u, aq), J.s));
        A[J.q + ld * col] = cadd(cscale(cmul(cconj(J.u), ap), J.s), cscale(aq, J.c));
      }
      __syncwarp();
      // the rotated 2x2 blocks in closed form (other pairs never touch them)
      if (lane < npair && rot) {
        const JacRot& J = R[lane];
        A[J.p + ld * J.p] = mkc(J.app - J.tm, 0.0);
        A[J.q + ld * J.q] = mkc(J.aqq + J.tm, 0.0);
        A[J.p + ld * J.q] = mkc(0, 0);
        A[J.q + ld * J.p] = mkc(0, 0);
      }
      __syncwarp();
    }
    converged = !any;
  }
  *ok = converged;
}

// Four warps per (mode, state): the Jacobi sweeps run on the first (its
// rotations are one round per warp-wide step), the warm-start products, the
// regularised inverse and the rho^-1 MF products on all four (independent
// FP64 dot products, so more of them in flight against the FP64 latency).
__global__ void __launch_bounds__(128) reginv_kernel(const RegInvDesc* __restrict__ descs, const MFOp* __restrict__ ops,
                                                     int* status) {
  __shared__ cplx A[MAXN_SPF * MAXN_SPF];
  __shared__ cplx V[MAXN_SPF * MAXN_SPF];
  __shared__ cplx Inv[MAXN_SPF * MAXN_SPF];
  __shared__ double w[MAXN_SPF];
  __shared__ JacRot R[MAXN_SPF / 2];
  const RegInvDesc& d = descs[blockIdx.x];
  const int n = d.n, ld = MAXN_SPF;
  for (int e = threadIdx.x; e < n * n; e += blockDim.x) {
    int i = e % n, j = e / n;
    // upper triangle is authoritative (zheev 'U'): mirror it
    cplx v = (i <= j) ? d.A[i + n * j] : cconj(d.A[j + n * i]);
    if (i == j) v.y = 0.0;
    A[i + ld * j] = v;
  }
  __syncthreads();
  // Warm start: rho changes little between consecutive calls (the mean-field
  // evaluations of one propagation), so the previous eigenvectors Vp nearly
  // diagonalise it; Jacobi then runs on Vp^H A Vp and the eigenvectors are Vp V.
  // The same eigen-decomposition up to rounding, in one or two sweeps instead of
  // a cold start's six to ten.  Every 64th call starts cold, which bounds the
  // drift of the accumulated product from unitarity.
  const int wcount = d.vprev ? *d.vcount : 0;
  const bool warm = wcount > 0 && wcount < 64;
  if (warm) {
    for (int e = threadIdx.x; e < n * n; e += blockDim.x) {   // Inv <- A Vp
      const int i = e % n, j = e / n;
      cplx s = mkc(0, 0);
      for (int k = 0; k < n; ++k) cfma(s, A[i + ld * k], d.vprev[k + n * j]);
      Inv[i + ld * j] = s;
    }
    __syncthreads();
    for (int e = threadIdx.x; e < n * n; e += blockDim.x) {   // V <- Vp^H Inv
      const int i = e % n, j = e / n;
      cplx s = mkc(0, 0);
      for (int k = 0; k < n; ++k) cfma_conj(s, d.vprev[k + n * i], Inv[k + ld * j]);
      V[i + ld * j] = s;
    }
    __syncthreads();
    for (int e = threadIdx.x; e < n * n; e += blockDim.x) {   // Hermitian from the upper triangle
      const int i = e % n, j = e / n;
      cplx v = (i <= j) ? V[i + ld * j] : cconj(V[j + ld * i]);
      if (i == j) v.y = 0.0;
      A[i + ld * j] = v;
    }
    __syncthreads();
  }
  bool ok = true;
  if (threadIdx.x < 32) jacobi_herm(A, V, n, ld, R, &ok);
  __syncthreads();
  if (!ok && threadIdx.x == 0) atomicOr(status, DEVST_EIG_NOCONV);
  if (warm) {
    for (int e = threadIdx.x; e < n * n; e += blockDim.x) {   // Inv <- Vp V
      const int i = e % n, j = e / n;
      cplx s = mkc(0, 0);
      for (int k = 0; k < n; ++k) cfma(s, d.vprev[i + n * k], V[k + ld * j]);
      Inv[i + ld * j] = s;
    }
    __syncthreads();
    for (int e = threadIdx.x; e < n * n; e += blockDim.x) V[e % n + ld * (e / n)] = Inv[e % n + ld * (e / n)];
    __syncthreads();
  }
  if (d.vprev) {
    for (int e = threadIdx.x; e < n * n; e += blockDim.x) d.vprev[e] = V[e % n + ld * (e / n)];
    if (threadIdx.x == 0) *d.vcount = (warm && ok) ? wcount + 1 : (ok ? 1 : 0);
  }
  if (threadIdx.x < n) {
    double wv = A[threadIdx.x + ld * threadIdx.x].x;
    double f;
    if (d.regtype == 0) {   // 'poly'
      double eps = d.eps;
      double wr = (wv < eps) ? 0.5 * (eps + wv * wv / eps) : wv;
      f = 1.0 / wr;
    } else {                // 'tikh'
      f = wv / (wv * wv + d.eps * d.eps);
    }
    w[threadIdx.x] = f;
  }
  __syncthreads();
  for (int e = threadIdx.x; e < n * n; e += blockDim.x) {
    int i = e % n, j = e / n;
    cplx s = mkc(0, 0);
    for (int k = 0; k < n; ++k) {
      cplx vik = V[i + ld * k], vjk = V[j + ld * k];
      s = cadd(s, cscale(cmul(vik, cconj(vjk)), w[k]));
    }
    Inv[i + ld * j] = s;
    if (d.inv_out) d.inv_out[i + n * j] = s;
  }
  __syncthreads();
  for (int o = 0; o < d.op_count; ++o) {
    const MFOp& op = ops[d.op_first + o];
    for (int e = threadIdx.x; e < n * op.n2; e += blockDim.x) {
      int i = e % n, j = e / n;
      cplx s = mkc(0, 0);
      for (int k = 0; k < n; ++k) cfma(s, Inv[i + ld * k], op.mf[k + n * j]);
      op.out[i + n * j] = s;
    }
  }
}

void launch_reginv(const RegInvDesc* d_descs, int ndesc, const MFOp* d_ops, int* d_status, cudaStream_t st) {
  if (ndesc <= 0) return;
  reginv_kernel<<<ndesc, 128, 0, st>>>(d_descs, d_ops, d_status);
}

// ---------------------------------------------------------------------------
// Natural populations (output.f90:88-140), one warp per (mode, state) block:
// eigenvalues of rho (zheev on the upper triangle) in decreasing order; for a
// Gaussian mode of conj(S^1/2) rho conj(S^1/2) with S^1/2 = sum_j sqrt(w_j) u_j u_j^H
// (SquareRoot, maths.f90:556-585; zlacgv; two zhemm 'R' on upper triangles), the
// gross Gaussian populations sum_j2 Re(rho S)(j1, j2) and the population errors
// |sum_j2 2 Re(rho S)(j1, j2) - rho(j1, j1)| (decreasing), all from upper triangles.
// ---------------------------------------------------------------------------
__device__ __forceinline__ cplx herm_up(const cplx* X, int n, int i, int j) {
  cplx v = (i <= j) ? X[i + n * j] : cconj(X[j + n * i]);
  if (i == j) v.y = 0.0;
  return v;
}

// position of v[i] in decreasing order (ties keep their index order)
__device__ __forceinline__ int rank_desc(const double* v, int n, int i) {
  int r = 0;
  for (int j = 0; j < n; ++j) r += (v[j] > v[i]) || (v[j] == v[i] && j < i);
  return r;
}

__global__ void __launch_bounds__(32) natpop_kernel(const NatpopDesc* __restrict__ descs, int* status) {
  __shared__ cplx A[MAXN_SPF * MAXN_SPF];
  __shared__ cplx V[MAXN_SPF * MAXN_SPF];
  __shared__ double w[MAXN_SPF];
  __shared__ JacRot R[MAXN_SPF / 2];
  const NatpopDesc& d = descs[blockIdx.x];
  const int n = d.n, ld = MAXN_SPF, lane = threadIdx.x;
  bool ok = true, ok2 = true;
  if (d.S) {
    for (int e = lane; e < n * n; e += 32) A[e % n + ld * (e / n)] = herm_up(d.S, n, e % n, e / n);
    __syncwarp();
    jacobi_herm(A, V, n, ld, R, &ok);
    if (lane < n) w[lane] = sqrt(A[lane + ld * lane].x);
    __syncwarp();
    cplx* S12 = d.work;
    cplx* T = d.work + n * n;
    for (int e = lane; e < n * n; e += 32) {
      const int i = e % n, j = e / n;
      cplx v = mkc(0.0, 0.0);
      for (int k = 0; k < n; ++k) v = cadd(v, cscale(cmul(V[i + ld * k], cconj(V[j + ld * k])), w[k]));
      S12[e] = cconj(v);
    }
    __syncwarp();
    for (int e = lane; e < n * n; e += 32) {   // T = S12 rho
      const int i = e % n, j = e / n;
      cplx v = mkc(0.0, 0.0);
      for (int q = 0; q < n; ++q) v = cadd(v, cmul(S12[i + n * q], herm_up(d.rho, n, q, j)));
      T[e] = v;
    }
    __syncwarp();
    for (int e = lane; e < n * n; e += 32) {   // M = T S12, S12 Hermitian from its upper triangle
      const int i = e % n, j = e / n;
      cplx v = mkc(0.0, 0.0);
      for (int q = 0; q < n; ++q) v = cadd(v, cmul(T[i + n * q], herm_up(S12, n, q, j)));
      A[i + ld * j] = v;
    }
    __syncwarp();
    for (int e = lane; e < n * n; e += 32) {   // zheev reads the upper triangle
      const int i = e % n, j = e / n;
      if (i > j) A[i + ld * j] = cconj(A[j + ld * i]);
      if (i == j) A[i + ld * j].y = 0.0;
    }
  } else {
    for (int e = lane; e < n * n; e += 32) A[e % n + ld * (e / n)] = herm_up(d.rho, n, e % n, e / n);
  }
  __syncwarp();
  jacobi_herm(A, V, n, ld, R, &ok2);
  if (lane < n) w[lane] = A[lane + ld * lane].x;
  __syncwarp();
  if (lane < n) d.natpop[rank_desc(w, n, lane)] = w[lane];
  __syncwarp();
  if (d.S) {
    double g = 0.0, e = 0.0;
    if (lane < n) {
      const int j1 = lane;
      for (int j2 = 0; j2 < j1; ++j2) {
        const double v = cmul(d.rho[j2 + n * j1], d.S[j2 + n * j1]).x;
        g += v;
        e += 2.0 * v;
      }
      e -= d.rho[j1 + n * j1].x;
      for (int j2 = j1; j2 < n; ++j2) {
        const double v = cmul(d.rho[j1 + n * j2], d.S[j1 + n * j2]).x;
        g += v;
        e += 2.0 * v;
      }
      e = fabs(e);
      d.ggp[j1] = g;
      w[lane] = e;
    }
    __syncwarp();
    if (lane < n) d.poperr[rank_desc(w, n, lane)] = e;
  }
  if (lane == 0 && !(ok && ok2)) atomicOr(status, DEVST_EIG_NOCONV);
}
void launch_natpop(const NatpopDesc* d, int nd, int* status, cudaStream_t st) {
  if (nd <= 0) return;
  natpop_kernel<<<nd, 32, 0, st>>>(d, status);
}

// ---------------------------------------------------------------------------
// <a|b> over a whole vector in FP64 (zdotc): each of DOT_BLOCKS blocks sums a
// grid-stride range (warp shuffles, then warps in order), and the last block to
// finish adds the block sums in block order, so the result does not depend on
// the blocks' timing.  The counter is reset for the next launch (graph replays).
// ---------------------------------------------------------------------------
__device__ __forceinline__ cplx warp_sum_c(cplx v) {
  for (int off = 16; off > 0; off >>= 1) {
    v.x += __shfl_down_sync(0xffffffffu, v.x, off);
    v.y += __shfl_down_sync(0xffffffffu, v.y, off);
  }
  return v;
}

__global__ void __launch_bounds__(256) dot_kernel(const cplx* __restrict__ a, const cplx* __restrict__ b,
                                                  long long n, cplx* partial, unsigned* counter, cplx* out) {
  __shared__ cplx ws[8];
  __shared__ bool last;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  cplx s = mkc(0.0, 0.0);
  for (long long i = (long long)blockIdx.x * blockDim.x + tid; i < n; i += (long long)gridDim.x * blockDim.x) {
    const cplx x = a[i], y = b[i];
    s.x = fma(x.x, y.x, fma(x.y, y.y, s.x));
    s.y = fma(x.x, y.y, fma(-x.y, y.x, s.y));
  }
  s = warp_sum_c(s);
  if (lane == 0) ws[warp] = s;
  __syncthreads();
  if (tid == 0) {
    cplx t = ws[0];
    for (int w = 1; w < (int)(blockDim.x >> 5); ++w) t = cadd(t, ws[w]);
    partial[blockIdx.x] = t;
    __threadfence();
    last = (atomicAdd(counter, 1u) == gridDim.x - 1);
  }
  __syncthreads();
  if (!last) return;
  __threadfence();
  if (warp == 0) {
    cplx t = mkc(0.0, 0.0);
    for (int q = lane; q < (int)gridDim.x; q += 32) {
      const volatile double* pv = (const volatile double*)partial;
      t = cadd(t, mkc(pv[2 * q], pv[2 * q + 1]));
    }
    t = warp_sum_c(t);
    if (lane == 0) {
      *out = t;
      *counter = 0u;
    }
  }
}
void launch_dot(const cplx* a, const cplx* b, long long n, cplx* partial, unsigned* counter, cplx* out,
                cudaStream_t st) {
  dot_kernel<<<DOT_BLOCKS, 256, 0, st>>>(a, b, n, partial, counter, out);
}

// Tridiagonal eigenproblem of the Lanczos matrix (dstev, cmf2_integration.f90:85)
__global__ void tridiag_kernel(const double* alpha, const double* beta, int n, double* evals, double* evecs,
                               int* status) {
  __shared__ cplx A[MAXN_SPF * MAXN_SPF];
  __shared__ cplx V[MAXN_SPF * MAXN_SPF];
  __shared__ JacRot R[MAXN_SPF / 2];
  const int ld = MAXN_SPF;
  for (int e = threadIdx.x; e < n * n; e += blockDim.x) {
    int i = e % n, j = e / n;
    double v = 0.0;
    if (i == j) v = alpha[i];
    else if (j == i + 1) v = beta[i];
    else if (i == j + 1) v = beta[j];
    A[i + ld * j] = mkc(v, 0.0);
  }
  __syncthreads();
  bool ok;
  jacobi_herm(A, V, n, ld, R, &ok);
  if (!ok && threadIdx.x == 0) atomicOr(status, DEVST_EIG_NOCONV);
  for (int e = threadIdx.x; e < n * n; e += blockDim.x) {
    int i = e % n, j = e / n;
    evecs[i + n * j] = V[i + ld * j].x;   // real symmetric input keeps V real
  }
  if (threadIdx.x < n) evals[threadIdx.x] = A[threadIdx.x + ld * threadIdx.x].x;
}

void launch_jacobi_tridiag(const double* alpha, const double* beta, int n, double* evals, double* evecs,
                           int* d_status, cudaStream_t st) {
  tridiag_kernel<<<1, 32, 0, st>>>(alpha, beta, n, evals, evecs, d_status);
}

// ---------------------------------------------------------------------------
// DVR SPF derivative with the (1 - P) projector (derivatives.f90:96-153), tiled
// over the grid so every (mode, state) block spreads over many SMs:
//  (1) spf_tile_kernel: dphi rows = f * sum_k ophi_k rhom1MF_k^T for SPF_TILE grid
//      rows, plus this tile's share of phi^H phi and phi^H dphi;
//  (2) spf_solve_kernel: sum the tile shares (fixed order), Cholesky solve
//      (phi^H phi) X = phi^H dphi  (zposv 'U');
//  (3) spf_proj_kernel: dphi rows -= phi rows * X.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256) spf_tile_kernel(const SpfDesc* __restrict__ descs, int ndesc,
                                                       const SpfOp* __restrict__ ops, cplx* __restrict__ out,
                                                       cplx der) {
  __shared__ int s_di;
  __shared__ cplx phs[SPF_TILE * MAXN_SPF];
  __shared__ cplx dps[SPF_TILE * MAXN_SPF];
  if (threadIdx.x == 0) s_di = find_desc(descs, ndesc);
  __syncthreads();
  const SpfDesc& d = descs[s_di];
  const int t = (int)(blockIdx.x - d.block_start);
  const int G = d.G, n = d.n;
  const int g0 = t * SPF_TILE;
  const int rows = min(SPF_TILE, G - g0);
  cplx* o = out + d.out_offset;
  for (int e = threadIdx.x; e < rows * n; e += blockDim.x) {
    const int r = e % rows, j1 = e / rows;
    const int g = g0 + r;
    phs[r + SPF_TILE * j1] = d.phi[g + (long long)G * j1];
    cplx acc = mkc(0, 0);
    for (int q = 0; q < d.op_count; ++q) {
      const SpfOp& op = ops[d.op_first + q];
      const cplx* oph = op.ophi + g;
      for (int j2 = 0; j2 < op.n2; ++j2) cfma(acc, oph[(long long)G * j2], op.rm[j1 + n * j2]);
    }
    acc = cmul(der, acc);
    dps[r + SPF_TILE * j1] = acc;
    o[g + (long long)G * j1] = acc;
  }
  __syncthreads();
  cplx* part = d.partial + (long long)t * 2 * n * n;
  for (int pr = threadIdx.x; pr < 2 * n * n; pr += blockDim.x) {
    const int which = pr / (n * n), q = pr % (n * n);
    const int j1 = q % n, j2 = q / n;
    const cplx* a = phs + SPF_TILE * j1;
    const cplx* b = (which == 0 ? phs : dps) + SPF_TILE * j2;
    cplx s = mkc(0, 0);
    for (int r = 0; r < rows; ++r) cfma_conj(s, a[r], b[r]);
    part[pr] = s;
  }
}

// Split-FP32 variant of spf_tile_kernel (precision modes 1 and 2): per operator,
// the tile rows of ophi and the matrix rhom1MF are split once into FP32 hi/lo
// pairs in shared memory, and every product is accumulated as a compensated
// FP32 pair (df_fma, ~1e-13 relative), leaving the FP64 pipe one add per output.
// PREC 1: the products of FP32-rounded operands accumulated in FP32 (~1e-7
// relative); PREC 2: compensated pairs.  The tile's shares of phi^H phi and
// phi^H dphi are compensated FP32 sums in both.
template <int PREC>
__global__ void __launch_bounds__(256) spf_tile_split_kernel(const SpfDesc* __restrict__ descs, int ndesc,
                                                             const SpfOp* __restrict__ ops, cplx* __restrict__ out,
                                                             cplx der) {
  __shared__ int s_di;
  // operator phase: ophi tile and rhom1MF as (hx, hy, lx, ly); epilogue: phi and dphi rows
  __shared__ __align__(16) cplx smem_u[2 * SPF_TILE * MAXN_SPF];
  float4* ops_s = reinterpret_cast<float4*>(smem_u);
  float4* rm_s = ops_s + SPF_TILE * MAXN_SPF;
  float4* phf = reinterpret_cast<float4*>(smem_u);                    // epilogue: phi rows, split
  float4* dpf = reinterpret_cast<float4*>(smem_u) + SPF_TILE * MAXN_SPF; // epilogue: dphi rows, split
  if (threadIdx.x == 0) s_di = find_desc(descs, ndesc);
  __syncthreads();
  const SpfDesc& d = descs[s_di];
  const int t = (int)(blockIdx.x - d.block_start);
  const int G = d.G, n = d.n;
  const int g0 = t * SPF_TILE;
  const int rows = min(SPF_TILE, G - g0);
  cplx* o = out + d.out_offset;
  // each thread owns up to 4 outputs (r, j1); SPF_TILE * MAXN_SPF <= 4 * 256
  float ah[4][2], al[4][2];
#pragma unroll
  for (int u = 0; u < 4; ++u) ah[u][0] = ah[u][1] = al[u][0] = al[u][1] = 0.f;
  for (int q = 0; q < d.op_count; ++q) {
    const SpfOp& op = ops[d.op_first + q];
    const int n2 = op.n2;
    __syncthreads();
    for (int e = threadIdx.x; e < rows * n2; e += blockDim.x) {
      const int r = e % rows, j2 = e / rows;
      const cplx v = op.ophi[g0 + r + (long long)G * j2];
      float hx, lx, hy, ly;
      split_d2f(v.x, hx, lx);
      split_d2f(v.y, hy, ly);
      ops_s[r + SPF_TILE * j2] = (PREC == 1) ? make_float4(hx + lx, hy + ly, 0.f, 0.f) : make_float4(hx, hy, lx, ly);
    }
    for (int e = threadIdx.x; e < n * n2; e += blockDim.x) {
      const cplx v = op.rm[e];
      float hx, lx, hy, ly;
      split_d2f(v.x, hx, lx);
      split_d2f(v.y, hy, ly);
      rm_s[e] = (PREC == 1) ? make_float4(hx + lx, hy + ly, 0.f, 0.f) : make_float4(hx, hy, lx, ly);
    }
    __syncthreads();
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      const int e = threadIdx.x + u * blockDim.x;
      if (e >= rows * n) continue;
      const int r = e % rows, j1 = e / rows;
      for (int j2 = 0; j2 < n2; ++j2) {
        const float4 x = ops_s[r + SPF_TILE * j2];
        const float4 m = rm_s[j1 + n * j2];
        // (x.r + i x.i)(m.r + i m.i)
        if (PREC == 1) {
          ah[u][0] = fmaf(x.x, m.x, fmaf(-x.y, m.y, ah[u][0]));
          ah[u][1] = fmaf(x.x, m.y, fmaf(x.y, m.x, ah[u][1]));
        } else {
          df_fma(ah[u][0], al[u][0], x.x, x.z, m.x, m.z);
          df_fma(ah[u][0], al[u][0], -x.y, -x.w, m.y, m.w);
          df_fma(ah[u][1], al[u][1], x.x, x.z, m.y, m.w);
          df_fma(ah[u][1], al[u][1], x.y, x.w, m.x, m.z);
        }
      }
    }
  }
  __syncthreads();
#pragma unroll
  for (int u = 0; u < 4; ++u) {
    const int e = threadIdx.x + u * blockDim.x;
    if (e >= rows * n) continue;
    const int r = e % rows, j1 = e / rows;
    const int g = g0 + r;
    const cplx acc = cmul(der, mkc(f2d_exact(ah[u][0]) + f2d_exact(al[u][0]),
                                   f2d_exact(ah[u][1]) + f2d_exact(al[u][1])));
    const cplx ph = d.phi[g + (long long)G * j1];
    float4 w;
    split_d2f(ph.x, w.x, w.z);
    split_d2f(ph.y, w.y, w.w);
    phf[r + SPF_TILE * j1] = w;
    split_d2f(acc.x, w.x, w.z);
    split_d2f(acc.y, w.y, w.w);
    dpf[r + SPF_TILE * j1] = w;
    o[g + (long long)G * j1] = acc;
  }
  __syncthreads();
  cplx* part = d.partial + (long long)t * 2 * n * n;
  for (int pr = threadIdx.x; pr < 2 * n * n; pr += blockDim.x) {
    const int which = pr / (n * n), q = pr % (n * n);
    const int j1 = q % n, j2 = q / n;
    const float4* a = phf + SPF_TILE * j1;
    const float4* b = (which == 0 ? phf : dpf) + SPF_TILE * j2;
    // conj(a) b as compensated FP32 pairs on the pre-split rows (the FP64 pipe is ~64x slower)
    float rh = 0.f, rl = 0.f, ih = 0.f, il = 0.f;
    for (int r = 0; r < rows; ++r) {
      const float4 x = a[r], y = b[r];
      df_fma(rh, rl, x.x, x.z, y.x, y.z);
      df_fma(rh, rl, x.y, x.w, y.y, y.w);
      df_fma(ih, il, x.x, x.z, y.y, y.w);
      df_fma(ih, il, -x.y, -x.w, y.x, y.z);
    }
    part[pr] = mkc(f2d_exact(rh) + f2d_exact(rl), f2d_exact(ih) + f2d_exact(il));
  }
}

// spf_tile_split_kernel<2> with the operator sum split between two groups of 256
// threads (operators 0, 2, 4, .. and 1, 3, 5, ..; both groups pass every barrier),
// for n <= 16: twice the warps per tile, the same compensated arithmetic; the
// second group's (hi, lo) sums are added to the first's at the end.
#define SPF_G2_N 16
__global__ void __launch_bounds__(512) spf_tile_split2_kernel(const SpfDesc* __restrict__ descs, int ndesc,
                                                              const SpfOp* __restrict__ ops,
                                                              cplx* __restrict__ out, cplx der) {
  __shared__ int s_di;
  // per group: ophi tile [SPF_TILE][16] and rhom1MF [16][16], split; epilogue: phi and
  // dphi rows alias them; red: the second group's sums
  __shared__ __align__(16) float4 buf[2 * (SPF_TILE * SPF_G2_N + SPF_G2_N * SPF_G2_N)];
  __shared__ __align__(16) float4 red[2 * 256];
  const int grp = threadIdx.x >> 8, loc = threadIdx.x & 255;
  float4* ops_s = buf + grp * (SPF_TILE * SPF_G2_N + SPF_G2_N * SPF_G2_N);
  float4* rm_s = ops_s + SPF_TILE * SPF_G2_N;
  float4* phf = buf;
  float4* dpf = buf + SPF_TILE * SPF_G2_N;
  if (threadIdx.x == 0) s_di = find_desc(descs, ndesc);
  __syncthreads();
  const SpfDesc& d = descs[s_di];
  const int t = (int)(blockIdx.x - d.block_start);
  const int G = d.G, n = d.n;
  const int g0 = t * SPF_TILE;
  const int rows = min(SPF_TILE, G - g0);
  cplx* o = out + d.out_offset;
  // each thread owns up to 2 outputs (r, j1) = loc, loc + 256 of its group
  float ah[2][2], al[2][2];
#pragma unroll
  for (int u = 0; u < 2; ++u) ah[u][0] = ah[u][1] = al[u][0] = al[u][1] = 0.f;
  const int iters = (d.op_count + 1) / 2;
  for (int it = 0; it < iters; ++it) {
    const int q = 2 * it + grp;
    const bool act = q < d.op_count;
    const SpfOp* op = act ? &ops[d.op_first + q] : nullptr;
    const int n2 = act ? op->n2 : 0;
    __syncthreads();
    for (int e = loc; e < rows * n2; e += 256) {
      const int r = e % rows, j2 = e / rows;
      const cplx v = op->ophi[g0 + r + (long long)G * j2];
      float hx, lx, hy, ly;
      split_d2f(v.x, hx, lx);
      split_d2f(v.y, hy, ly);
      ops_s[r + SPF_TILE * j2] = make_float4(hx, hy, lx, ly);
    }
    for (int e = loc; e < n * n2; e += 256) {
      const cplx v = op->rm[e];
      float hx, lx, hy, ly;
      split_d2f(v.x, hx, lx);
      split_d2f(v.y, hy, ly);
      rm_s[e] = make_float4(hx, hy, lx, ly);
    }
    __syncthreads();
#pragma unroll
    for (int u = 0; u < 2; ++u) {
      const int e = loc + u * 256;
      if (e >= rows * n) continue;
      const int r = e % rows, j1 = e / rows;
      for (int j2 = 0; j2 < n2; ++j2) {
        const float4 x = ops_s[r + SPF_TILE * j2];
        const float4 m = rm_s[j1 + n * j2];
        df_fma(ah[u][0], al[u][0], x.x, x.z, m.x, m.z);
        df_fma(ah[u][0], al[u][0], -x.y, -x.w, m.y, m.w);
        df_fma(ah[u][1], al[u][1], x.x, x.z, m.y, m.w);
        df_fma(ah[u][1], al[u][1], x.y, x.w, m.x, m.z);
      }
    }
  }
  if (grp == 1) {
#pragma unroll
    for (int u = 0; u < 2; ++u) red[loc + 256 * u] = make_float4(ah[u][0], ah[u][1], al[u][0], al[u][1]);
  }
  __syncthreads();   // the operator tiles are dead; red holds the second group's sums
  if (grp == 0) {
#pragma unroll
    for (int u = 0; u < 2; ++u) {
      const int e = loc + u * 256;
      if (e >= rows * n) continue;
      const float4 b = red[e];
      float sh = ah[u][0], sl = al[u][0], th = ah[u][1], tl = al[u][1];
      {
        const float x = sh + b.x, bp = x - sh;
        sl += ((sh - (x - bp)) + (b.x - bp)) + b.z;
        sh = x;
      }
      {
        const float x = th + b.y, bp = x - th;
        tl += ((th - (x - bp)) + (b.y - bp)) + b.w;
        th = x;
      }
      const int r = e % rows, j1 = e / rows;
      const int g = g0 + r;
      const cplx acc = cmul(der, mkc(f2d_exact(sh) + f2d_exact(sl), f2d_exact(th) + f2d_exact(tl)));
      const cplx ph = d.phi[g + (long long)G * j1];
      float4 w;
      split_d2f(ph.x, w.x, w.z);
      split_d2f(ph.y, w.y, w.w);
      phf[r + SPF_TILE * j1] = w;
      split_d2f(acc.x, w.x, w.z);
      split_d2f(acc.y, w.y, w.w);
      dpf[r + SPF_TILE * j1] = w;
      o[g + (long long)G * j1] = acc;
    }
  }
  __syncthreads();
  cplx* part = d.partial + (long long)t * 2 * n * n;
  for (int pr = threadIdx.x; pr < 2 * n * n; pr += blockDim.x) {
    const int which = pr / (n * n), qq = pr % (n * n);
    const int j1 = qq % n, j2 = qq / n;
    const float4* a = phf + SPF_TILE * j1;
    const float4* b = (which == 0 ? phf : dpf) + SPF_TILE * j2;
    float rh = 0.f, rl = 0.f, ih = 0.f, il = 0.f;
    for (int r = 0; r < rows; ++r) {
      const float4 x = a[r], y = b[r];
      df_fma(rh, rl, x.x, x.z, y.x, y.z);
      df_fma(rh, rl, x.y, x.w, y.y, y.w);
      df_fma(ih, il, x.x, x.z, y.y, y.w);
      df_fma(ih, il, -x.y, -x.w, y.x, y.z);
    }
    part[pr] = mkc(f2d_exact(rh) + f2d_exact(rl), f2d_exact(ih) + f2d_exact(il));
  }
}

// (phi^H phi) X = phi^H dphi (zposv 'U') by Gauss-Jordan elimination of [S | O]
// without pivoting, which is stable for the Hermitian positive definite S: each of
// the n steps is one pivot reciprocal, then one scale and one update per element
// across all threads (a short dependent path, unlike the column-serial Cholesky
// and the per-right-hand-side triangular solves).  A non-positive pivot is the
// zposv failure (DEVST_CHOL_FAIL).
__global__ void __launch_bounds__(256) spf_solve_kernel(const SpfDesc* __restrict__ descs, int* status) {
  __shared__ cplx M[MAXN_SPF * 2 * MAXN_SPF];   // M[i + ld * c], c < n: S, c >= n: O
  __shared__ cplx s_pinv;
  __shared__ int s_fail;
  const SpfDesc& d = descs[blockIdx.x];
  const int n = d.n, ld = MAXN_SPF;
  if (threadIdx.x == 0) s_fail = 0;
  for (int pr = threadIdx.x; pr < 2 * n * n; pr += blockDim.x) {
    const int which = pr / (n * n), q = pr % (n * n);
    const int j1 = q % n, j2 = q / n;
    cplx s = mkc(0, 0);
    for (int t = 0; t < d.ntile; ++t) s = cadd(s, d.partial[(long long)t * 2 * n * n + pr]);
    M[j1 + ld * (j2 + which * n)] = s;
  }
  __syncthreads();
  for (int k = 0; k < n; ++k) {
    if (threadIdx.x == 0) {
      const cplx p = M[k + ld * k];
      if (!(p.x > 0.0)) s_fail = 1;
      const double den = p.x * p.x + p.y * p.y;
      s_pinv = (den > 0.0) ? mkc(p.x / den, -p.y / den) : mkc(0.0, 0.0);
    }
    __syncthreads();
    for (int c = k + 1 + (int)threadIdx.x; c < 2 * n; c += blockDim.x) M[k + ld * c] = cmul(s_pinv, M[k + ld * c]);
    __syncthreads();
    for (int e = threadIdx.x; e < n * 2 * n; e += blockDim.x) {
      const int i = e % n, c = e / n;
      if (i == k || c <= k) continue;
      M[i + ld * c] = csub(M[i + ld * c], cmul(M[i + ld * k], M[k + ld * c]));
    }
    __syncthreads();
  }
  if (threadIdx.x == 0 && s_fail) atomicOr(status, DEVST_CHOL_FAIL);
  for (int e = threadIdx.x; e < n * n; e += blockDim.x) d.X[e] = M[(e % n) + ld * (n + e / n)];
}

__global__ void __launch_bounds__(256) spf_proj_kernel(const SpfDesc* __restrict__ descs, int ndesc,
                                                       cplx* __restrict__ out) {
  __shared__ int s_di;
  __shared__ cplx Xs[MAXN_SPF * MAXN_SPF];
  if (threadIdx.x == 0) s_di = find_desc(descs, ndesc);
  __syncthreads();
  const SpfDesc& d = descs[s_di];
  const int n = d.n, G = d.G;
  for (int e = threadIdx.x; e < n * n; e += blockDim.x) Xs[e] = d.X[e];
  __syncthreads();
  const int t = (int)(blockIdx.x - d.block_start);
  const int g0 = t * SPF_TILE;
  const int rows = min(SPF_TILE, G - g0);
  cplx* o = out + d.out_offset;
  for (int e = threadIdx.x; e < rows * n; e += blockDim.x) {
    const int r = e % rows, j = e / rows;
    const int g = g0 + r;
    cplx v = o[g + (long long)G * j];
    for (int k = 0; k < n; ++k) v = csub(v, cmul(d.phi[g + (long long)G * k], Xs[k + n * j]));
    o[g + (long long)G * j] = v;
  }
}

// Split modes: dphi -= phi X with the products as compensated FP32 pairs on split
// operands (~1e-13 relative) and one FP64 subtraction per element.
__global__ void __launch_bounds__(256) spf_proj_split_kernel(const SpfDesc* __restrict__ descs, int ndesc,
                                                             cplx* __restrict__ out) {
  __shared__ int s_di;
  __shared__ float4 Xs[MAXN_SPF * MAXN_SPF];
  if (threadIdx.x == 0) s_di = find_desc(descs, ndesc);
  __syncthreads();
  const SpfDesc& d = descs[s_di];
  const int n = d.n, G = d.G;
  for (int e = threadIdx.x; e < n * n; e += blockDim.x) {
    const cplx v = d.X[e];
    float4 w4;
    split_d2f(v.x, w4.x, w4.z);
    split_d2f(v.y, w4.y, w4.w);
    Xs[e] = w4;
  }
  __syncthreads();
  const int t = (int)(blockIdx.x - d.block_start);
  const int g0 = t * SPF_TILE;
  const int rows = min(SPF_TILE, G - g0);
  cplx* o = out + d.out_offset;
  for (int e = threadIdx.x; e < rows * n; e += blockDim.x) {
    const int r = e % rows, j = e / rows;
    const int g = g0 + r;
    float rh = 0.f, rl = 0.f, ih = 0.f, il = 0.f;
    for (int k = 0; k < n; ++k) {
      const cplx ph = d.phi[g + (long long)G * k];
      float xh, xl, yh, yl;
      split_d2f(ph.x, xh, xl);
      split_d2f(ph.y, yh, yl);
      const float4 m = Xs[k + n * j];
      df_fma(rh, rl, xh, xl, m.x, m.z);
      df_fma(rh, rl, -yh, -yl, m.y, m.w);
      df_fma(ih, il, xh, xl, m.y, m.w);
      df_fma(ih, il, yh, yl, m.x, m.z);
    }
    const cplx v = o[g + (long long)G * j];
    o[g + (long long)G * j] = mkc(v.x - (f2d_exact(rh) + f2d_exact(rl)), v.y - (f2d_exact(ih) + f2d_exact(il)));
  }
}

void launch_spf(const SpfDesc* d_descs, int ndesc, long long ntiles, const SpfOp* d_ops, cplx* out,
                cplx der_factor, int* d_status, cudaStream_t st, int prec, int nf) {
  if (ndesc <= 0) return;
  // both split modes: compensated (FP32 accumulation here makes the SPF error
  // estimate noisier and the adaptive SPF integration take more steps)
  if (prec > 0 && nf > 0 && nf <= SPF_G2_N)
    spf_tile_split2_kernel<<<(unsigned)ntiles, 512, 0, st>>>(d_descs, ndesc, d_ops, out, der_factor);
  else if (prec > 0)
    spf_tile_split_kernel<2><<<(unsigned)ntiles, 256, 0, st>>>(d_descs, ndesc, d_ops, out, der_factor);
  else
    spf_tile_kernel<<<(unsigned)ntiles, 256, 0, st>>>(d_descs, ndesc, d_ops, out, der_factor);
  spf_solve_kernel<<<ndesc, 256, 0, st>>>(d_descs, d_status);
  if (prec > 0) spf_proj_split_kernel<<<(unsigned)ntiles, 256, 0, st>>>(d_descs, ndesc, out);
  else spf_proj_kernel<<<(unsigned)ntiles, 256, 0, st>>>(d_descs, ndesc, out);
}

// ---------------------------------------------------------------------------
// Elementwise helpers
// ---------------------------------------------------------------------------
// The launch-wide sum of one complex value per thread, in a fixed order: warps,
// then the block's warps into partial[blockIdx.x]; the last block to finish adds
// the block sums in block order into *out and resets the counter (graph replays).
// Every thread of every block calls it (no early returns before it).
__device__ __forceinline__ cplx warp_sum_cd(cplx v) {
  for (int off = 16; off > 0; off >>= 1) {
    v.x += __shfl_down_sync(0xffffffffu, v.x, off);
    v.y += __shfl_down_sync(0xffffffffu, v.y, off);
  }
  return v;
}
__device__ void grid_sum_c(cplx v, cplx* partial, unsigned* counter, cplx* out) {
  __shared__ cplx ws[32];
  __shared__ bool last;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, nw = (blockDim.x + 31) >> 5;
  v = warp_sum_cd(v);
  if (lane == 0) ws[warp] = v;
  __syncthreads();
  if (tid == 0) {
    cplx t = ws[0];
    for (int w = 1; w < nw; ++w) t = cadd(t, ws[w]);
    partial[blockIdx.x] = t;
    __threadfence();
    last = (atomicAdd(counter, 1u) == gridDim.x - 1);
  }
  __syncthreads();
  if (!last) return;
  __threadfence();
  const volatile double* pv = (const volatile double*)partial;
  cplx t = mkc(0.0, 0.0);
  for (int q = tid; q < (int)gridDim.x; q += blockDim.x) t = cadd(t, mkc(pv[2 * q], pv[2 * q + 1]));
  t = warp_sum_cd(t);
  __syncthreads();
  if (lane == 0) ws[warp] = t;
  __syncthreads();
  if (tid == 0) {
    cplx r = ws[0];
    for (int w = 1; w < nw; ++w) r = cadd(r, ws[w]);
    *out = r;
    *counter = 0u;
  }
}

// out[i] = sum_k coeff_k src_k[i - offset] over the sources of the state range
// holding i; with dot.v also the launch-wide <dot.v|out> (FP64 products of the
// values written) into dot.res.  Each block streams a contiguous chunk of the
// elements with the current range's source descriptors cached in shared memory.
// PREC 0: FP64.  PREC 1: FP32 coefficients times FP32-rounded sources accumulated
// in FP32 (the sources are FP32 products there).  PREC 2: compensated FP32 pairs
// (df_fma, ~1e-13 relative).
#define TERMSUM_CACHE 64
template <int PREC>
__global__ void __launch_bounds__(256) termsum_kernel(cplx* __restrict__ out, const SumRange* __restrict__ ranges,
                                                      int nr, const SumSrc* __restrict__ srcs, long long total,
                                                      FusedDot dot) {
  __shared__ SumSrc ss[TERMSUM_CACHE];
  __shared__ int s_rg;
  const long long chunk = (total + gridDim.x - 1) / gridDim.x;
  const long long start = (long long)blockIdx.x * chunk, end = min(total, start + chunk);
  cplx d = mkc(0, 0);
  long long base = start;
  while (base < end) {
    if (threadIdx.x == 0) {
      int lo = 0, hi = nr - 1;   // last range starting at or before base (ranges sorted by offset)
      while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (ranges[mid].offset <= base) lo = mid; else hi = mid - 1;
      }
      s_rg = lo;
    }
    __syncthreads();
    const SumRange rg = ranges[s_rg];
    long long seg_end = min(end, rg.offset + rg.n);
    if (base < rg.offset || base >= rg.offset + rg.n) {
      // outside every range: skip to the next range start
      seg_end = (s_rg + 1 < nr) ? min(end, ranges[s_rg + 1].offset) : end;
      __syncthreads();
      base = max(seg_end, base + 1);
      continue;
    }
    const bool cached = rg.count <= TERMSUM_CACHE;
    if (cached)
      for (int k = threadIdx.x; k < rg.count; k += blockDim.x) ss[k] = srcs[rg.first + k];
    __syncthreads();
    const SumSrc* sp = cached ? ss : srcs + rg.first;
    if (PREC == 1) {
      // four elements per thread in flight: per source, four independent loads
      const long long stride = (long long)blockDim.x;
      for (long long i0 = base + threadIdx.x; i0 < seg_end; i0 += 4 * stride) {
        float ar[4] = {0.f, 0.f, 0.f, 0.f}, ai[4] = {0.f, 0.f, 0.f, 0.f};
        for (int k = 0; k < rg.count; ++k) {
          const float cr = sp[k].cs[0] + sp[k].cs[1], ci = sp[k].cs[2] + sp[k].cs[3];
          const cplx* src = sp[k].src;
          const int fmt = sp[k].fmt;
#pragma unroll
          for (int e = 0; e < 4; ++e) {
            const long long i = i0 + e * stride;
            if (i >= seg_end) break;
            const float4 x = load_split(src, i - rg.offset, fmt);
            const float xr = x.x + x.z, xi = x.y + x.w;
            ar[e] = fmaf(cr, xr, fmaf(-ci, xi, ar[e]));
            ai[e] = fmaf(cr, xi, fmaf(ci, xr, ai[e]));
          }
        }
#pragma unroll
        for (int e = 0; e < 4; ++e) {
          const long long i = i0 + e * stride;
          if (i >= seg_end) break;
          const cplx val = mkc(f2d_exact(ar[e]), f2d_exact(ai[e]));
          out[i] = val;
          if (dot.v) cfma_conj(d, dot.v[i], val);
        }
      }
      __syncthreads();
      base = seg_end;
      continue;
    }
    for (long long i = base + threadIdx.x; i < seg_end; i += blockDim.x) {
      const long long li = i - rg.offset;
      cplx val;
      if (PREC == 0) {
        val = mkc(0, 0);
        for (int k = 0; k < rg.count; ++k) cfma(val, sp[k].coeff, load_c(sp[k].src, li, sp[k].fmt));
      } else {
        float rh = 0.f, rl = 0.f, ih = 0.f, il = 0.f;
        for (int k = 0; k < rg.count; ++k) {
          const float ch = sp[k].cs[0], cl = sp[k].cs[1], dh = sp[k].cs[2], dl = sp[k].cs[3];
          const float4 x = load_split(sp[k].src, li, sp[k].fmt);
          // (c + i d)(xr + i xi)
          df_fma(rh, rl, ch, cl, x.x, x.z);
          df_fma(rh, rl, -dh, -dl, x.y, x.w);
          df_fma(ih, il, ch, cl, x.y, x.w);
          df_fma(ih, il, dh, dl, x.x, x.z);
        }
        val = mkc(f2d_exact(rh) + f2d_exact(rl), f2d_exact(ih) + f2d_exact(il));
      }
      out[i] = val;
      if (dot.v) cfma_conj(d, dot.v[i], val);
    }
    __syncthreads();
    base = seg_end;
  }
  if (dot.v) grid_sum_c(d, dot.partial, dot.counter, dot.res);
}

void launch_termsum(cplx* out, const SumRange* d_ranges, int nranges, const SumSrc* d_srcs, long long total,
                    cudaStream_t st, int prec, FusedDot dot) {
  if (total <= 0) return;
  const unsigned nb = (unsigned)std::min<long long>((total + 255) / 256, FUSED_BLOCKS);
  if (prec == 1)
    termsum_kernel<1><<<nb, 256, 0, st>>>(out, d_ranges, nranges, d_srcs, total, dot);
  else if (prec > 1)
    termsum_kernel<2><<<nb, 256, 0, st>>>(out, d_ranges, nranges, d_srcs, total, dot);
  else
    termsum_kernel<0><<<nb, 256, 0, st>>>(out, d_ranges, nranges, d_srcs, total, dot);
}

__global__ void stage_kernel(cplx* __restrict__ out, const cplx* __restrict__ base, StageArgs a, double dt,
                             long long n) {
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  cplx s = mkc(0, 0);
  for (int k = 0; k < a.nk; ++k) {
    cplx v = a.k[k][i];
    s.x = fma(a.c[k], v.x, s.x);
    s.y = fma(a.c[k], v.y, s.y);
  }
  cplx b = base[i];
  out[i] = mkc(fma(dt, s.x, b.x), fma(dt, s.y, b.y));
}

// Ensemble stage: every member m (elements off[m] .. off[m+1]) with its own dt.
__device__ __forceinline__ int member_of(const long long* __restrict__ off, int nm, long long i) {
  int lo = 0, hi = nm - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (off[mid] <= i) lo = mid; else hi = mid - 1;
  }
  return lo;
}
__global__ void ens_stage_kernel(cplx* __restrict__ out, const cplx* __restrict__ base, StageArgs a,
                                 const double* __restrict__ dt, const long long* __restrict__ off, int nm,
                                 long long n) {
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double h = dt[member_of(off, nm, i)];
  cplx s = mkc(0, 0);
  for (int k = 0; k < a.nk; ++k) {
    cplx v = a.k[k][i];
    s.x = fma(a.c[k], v.x, s.x);
    s.y = fma(a.c[k], v.y, s.y);
  }
  cplx b = base[i];
  out[i] = mkc(fma(h, s.x, b.x), fma(h, s.y, b.y));
}
void launch_ens_stage(cplx* out, const cplx* base, const StageArgs& a, const double* dt, const long long* off, int nm,
                      long long n, cudaStream_t st) {
  if (n <= 0) return;
  ens_stage_kernel<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(out, base, a, dt, off, nm, n);
}
__global__ void ens_accept_kernel(cplx* __restrict__ y, const cplx* __restrict__ src, const int* __restrict__ accept,
                                  const long long* __restrict__ off, int nm, long long n) {
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  if (accept[member_of(off, nm, i)]) y[i] = src[i];
}
void launch_ens_accept(cplx* y, const cplx* src, const int* accept, const long long* off, int nm, long long n,
                       cudaStream_t st) {
  if (n <= 0) return;
  ens_accept_kernel<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(y, src, accept, off, nm, n);
}

__global__ void bs_final_kernel(cplx* __restrict__ out, const cplx* __restrict__ am, const cplx* __restrict__ an,
                                const cplx* __restrict__ d, double dt, long long n) {
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const cplx a = am[i], b = an[i], g = d[i];
  out[i] = mkc(0.5 * ((a.x + b.x) + dt * g.x), 0.5 * ((a.y + b.y) + dt * g.y));
}
void launch_bs_final(cplx* out, const cplx* am, const cplx* an, const cplx* d, double dt, long long n, cudaStream_t st) {
  if (n <= 0) return;
  bs_final_kernel<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(out, am, an, d, dt, n);
}
__global__ void bs_extr_kernel(BsExtr e, const cplx* __restrict__ est, cplx* __restrict__ a0, cplx* __restrict__ a1,
                               long long n) {
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const cplx x = est[i];
  if (e.iest == 1) {
    e.q[1][i] = x;
    a0[i] = x;
    a1[i] = x;
    return;
  }
  cplx A0 = x, A1 = x, At = x;
  for (int k1 = 1; k1 < e.iest; ++k1) {
    const cplx cd = e.q[k1][i];
    e.q[k1][i] = A1;
    const cplx del = csub(At, cd);
    A1 = cscale(del, e.f1[k1]);
    At = cscale(del, e.f2[k1]);
    A0 = cadd(A0, A1);
  }
  e.q[e.iest][i] = A1;
  a0[i] = A0;
  a1[i] = cadd(A0, A1);
}
void launch_bs_extr(const BsExtr& e, const cplx* est, cplx* a0, cplx* a1, long long n, cudaStream_t st) {
  if (n <= 0) return;
  bs_extr_kernel<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(e, est, a0, a1, n);
}

void launch_stage(cplx* out, const cplx* base, const StageArgs& a, double dt, long long n, cudaStream_t st) {
  if (n <= 0) return;
  stage_kernel<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(out, base, a, dt, n);
}

__global__ void copy_scale_kernel(cplx* out, const cplx* in, cplx s, long long n) {
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] = cmul(s, in[i]);
}
void launch_copy_scale(cplx* out, const cplx* in, cplx s, long long n, cudaStream_t st) {
  if (n <= 0) return;
  copy_scale_kernel<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(out, in, s, n);
}

__global__ void axpy_kernel(cplx* y, const cplx* x, cplx a, long long n) {
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) { cplx v = y[i]; cfma(v, a, x[i]); y[i] = v; }
}
// complex FP64 -> complex FP32 rounded to nearest (the FP64 pipe stays idle)
__global__ void to_f32_kernel(float2* __restrict__ out, const cplx* __restrict__ in, long long n) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const cplx v = in[i];
  float hx, lx, hy, ly;
  split_d2f(v.x, hx, lx);
  split_d2f(v.y, hy, ly);
  out[i] = make_float2(hx + lx, hy + ly);
}
// complex128 -> FP32 split pairs (re hi, im hi, re lo, im lo), the exact split
// of load_split done once per element
__global__ void to_split_kernel(float4* __restrict__ out, const cplx* __restrict__ in, long long n) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const cplx v = in[i];
  float4 w;
  split_d2f(v.x, w.x, w.z);
  split_d2f(v.y, w.y, w.w);
  out[i] = w;
}
void launch_to_split(cplx* out, const cplx* in, long long n, cudaStream_t st) {
  if (n <= 0) return;
  to_split_kernel<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(reinterpret_cast<float4*>(out), in, n);
}
void launch_to_f32(cplx* out, const cplx* in, long long n, cudaStream_t st) {
  if (n <= 0) return;
  to_f32_kernel<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(reinterpret_cast<float2*>(out), in, n);
}

void launch_axpy(cplx* y, const cplx* x, cplx a, long long n, cudaStream_t st) {
  if (n <= 0) return;
  axpy_kernel<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(y, x, a, n);
}

__global__ void gemv_cols_kernel(cplx* out, const cplx* basis, long long ld, const cplx* coef, int ncol, long long n) {
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  cplx s = mkc(0, 0);
  for (int j = 0; j < ncol; ++j) cfma(s, coef[j], basis[i + ld * j]);
  out[i] = s;
}
void launch_gemv_cols(cplx* out, const cplx* basis, long long ld, const cplx* coef, int ncol, long long n,
                      cudaStream_t st) {
  if (n <= 0) return;
  gemv_cols_kernel<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(out, basis, ld, coef, ncol, n);
}

__global__ void matsum_kernel(const MatSumDesc* __restrict__ descs, const MatSumSrc* __restrict__ srcs) {
  const MatSumDesc& d = descs[blockIdx.x];
  for (int e = threadIdx.x; e < d.n1 * d.n2; e += blockDim.x) {
    cplx acc = mkc(0, 0);
    for (int k = 0; k < d.count; ++k) cfma(acc, srcs[d.first + k].coeff, srcs[d.first + k].src[e]);
    d.out[e] = acc;
  }
}
void launch_matsum(const MatSumDesc* d_descs, int ndesc, const MatSumSrc* d_srcs, cudaStream_t st) {
  if (ndesc <= 0) return;
  matsum_kernel<<<ndesc, 128, 0, st>>>(d_descs, d_srcs);
}

// ---------------------------------------------------------------------------
// FP64 FMA throughput calibration (independent FMA chains, no memory traffic).
// ---------------------------------------------------------------------------
__global__ void fp64_peak_kernel(double* out, int iters, double a) {
  double x0 = threadIdx.x * 1e-3, x1 = x0 + 1, x2 = x0 + 2, x3 = x0 + 3, x4 = x0 + 4, x5 = x0 + 5, x6 = x0 + 6,
         x7 = x0 + 7;
  for (int i = 0; i < iters; ++i) {
    x0 = fma(x0, a, 1e-9); x1 = fma(x1, a, 1e-9); x2 = fma(x2, a, 1e-9); x3 = fma(x3, a, 1e-9);
    x4 = fma(x4, a, 1e-9); x5 = fma(x5, a, 1e-9); x6 = fma(x6, a, 1e-9); x7 = fma(x7, a, 1e-9);
  }
  double s = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
  if (s == 12345.678) out[0] = s;
}

double measure_fp64_tflops() {
  double* d = nullptr;
  if (cudaMalloc(&d, 64) != cudaSuccess) return 0.0;
  int dev = 0, nsm = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  const int blocks = nsm * 8, threads = 256, iters = 4096;
  fp64_peak_kernel<<<blocks, threads>>>(d, 16, 0.999999);
  cudaEvent_t a, b;
  cudaEventCreate(&a);
  cudaEventCreate(&b);
  float best = 1e30f;
  for (int r = 0; r < 5; ++r) {
    cudaEventRecord(a);
    fp64_peak_kernel<<<blocks, threads>>>(d, iters, 0.999999);
    cudaEventRecord(b);
    cudaEventSynchronize(b);
    float ms;
    cudaEventElapsedTime(&ms, a, b);
    best = ms < best ? ms : best;
  }
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  cudaFree(d);
  const double flops = 2.0 * 8.0 * (double)iters * blocks * threads;
  return flops / (best * 1e-3) / 1e12;
}

// ---------------------------------------------------------------------------
// Lockstep SPF integration of all DVR modes (rk_SPF_ck with frozen mean fields,
// cmf2_integration.f90:105-253): every psi element carries its mode, each mode its
// own step length (0 for a mode that has finished its interval).
// ---------------------------------------------------------------------------
__global__ void stage_modes_kernel(cplx* __restrict__ out, const cplx* __restrict__ base, StageArgs a,
                                   const double* __restrict__ dt_mode, const unsigned char* __restrict__ elem_mode,
                                   long long off, long long n) {
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const long long g = off + i;
  const double dt = dt_mode[elem_mode[i]];
  cplx s = mkc(0, 0);
  for (int k = 0; k < a.nk; ++k) {
    cplx v = a.k[k][g];
    s.x = fma(a.c[k], v.x, s.x);
    s.y = fma(a.c[k], v.y, s.y);
  }
  cplx b = base[g];
  out[g] = mkc(fma(dt, s.x, b.x), fma(dt, s.y, b.y));
}
void launch_stage_modes(cplx* out, const cplx* base, const StageArgs& a, const double* dt_mode,
                        const unsigned char* elem_mode, long long off, long long n, cudaStream_t st) {
  if (n <= 0) return;
  stage_modes_kernel<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(out, base, a, dt_mode, elem_mode, off, n);
}

// y <- src on the elements of accepted modes
__global__ void masked_copy_kernel(cplx* __restrict__ y, const cplx* __restrict__ src,
                                   const unsigned char* __restrict__ elem_mode, const int* __restrict__ accept,
                                   long long off, long long n) {
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  if (accept[elem_mode[i]]) y[off + i] = src[off + i];
}
void launch_masked_copy(cplx* y, const cplx* src, const unsigned char* elem_mode, const int* accept, long long off,
                        long long n, cudaStream_t st) {
  if (n <= 0) return;
  masked_copy_kernel<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(y, src, elem_mode, accept, off, n);
}

// Calc_Err_SPF (cmf2_derivatives.f90:239-283): err_m = sqrt|sum_blocks Tr(rho dS)| with
// the reference's upper-triangle evaluation; one thread per mode.
// err_m = sqrt|sum over the mode's blocks of Tr(rho . dS)| (Calc_Err_SPF,
// cmf2_derivatives.f90:239-338): one warp per block (lane-strided entries,
// shuffle sum), then one thread per mode adds its blocks in descriptor order.
__global__ void __launch_bounds__(1024) spf_err_kernel(const SpfErrDesc* __restrict__ d, int nd, double* err_mode,
                                                       int nmodes) {
  __shared__ double part[256];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int nw = blockDim.x >> 5;
  for (int q = warp; q < nd && q < 256; q += nw) {
    const int n = d[q].n;
    const cplx* r = d[q].rho;
    const cplx* o = d[q].ds;
    double e = 0.0;
    for (int pr = lane; pr < n * n; pr += 32) {
      const int j1 = pr % n, j2 = pr / n;
      if (j1 > j2) continue;
      const cplx rv = r[pr], ov = o[pr];
      e += (j1 < j2) ? 2.0 * (rv.x * ov.x + rv.y * ov.y) : (rv.x * ov.x - rv.y * ov.y);
    }
    for (int off = 16; off > 0; off >>= 1) e += __shfl_down_sync(0xffffffffu, e, off);
    if (lane == 0) part[q] = e;
  }
  __syncthreads();
  const int m = threadIdx.x;
  if (m >= nmodes) return;
  double e = 0.0;
  bool any = false;
  for (int q = 0; q < nd && q < 256; ++q) {
    if (d[q].mode != m) continue;
    any = true;
    e += part[q];
  }
  err_mode[m] = any ? sqrt(fabs(e)) : 0.0;
}
void launch_spf_err(const SpfErrDesc* d, int nd, double* err_mode, int nmodes, cudaStream_t st) {
  // nd <= 256 blocks (checked when the plan is built), nmodes <= 64
  const int warps = std::max(std::min(nd, 32), (nmodes + 31) / 32);
  spf_err_kernel<<<1, 32 * warps, 0, st>>>(d, nd, err_mode, nmodes);
}

// ---------------------------------------------------------------------------
// Lanczos recurrence with device-resident scalars (cmf2_integration.f90:53-79):
// Kn <- (Kn - beta_prev * Kp) - alpha * Kj, alpha = Re <Kj|Kn> (two zaxpy in the
// reference order), then Kn <- Kn / ||Kn||.
// ---------------------------------------------------------------------------
// ... and with nrm.res the launch-wide ||Kn||^2 of the new Kn (the next normalisation)
__global__ void lan_axpy_kernel(cplx* __restrict__ Kn, const cplx* __restrict__ Kj, const cplx* __restrict__ Kp,
                                const cplx* __restrict__ dot_alpha, const double* __restrict__ beta_prev,
                                double* alpha_out, long long n, FusedDot nrm) {
  const long long i0 = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const double alpha = dot_alpha->x;
  if (i0 == 0) *alpha_out = alpha;
  const double b = Kp ? *beta_prev : 0.0;
  double s2 = 0.0;
  for (long long i = i0; i < n; i += (long long)gridDim.x * blockDim.x) {
    cplx v = Kn[i];
    if (Kp) {
      cplx p = Kp[i];
      v = mkc(fma(-b, p.x, v.x), fma(-b, p.y, v.y));
    }
    cplx q = Kj[i];
    const cplx w = mkc(fma(-alpha, q.x, v.x), fma(-alpha, q.y, v.y));
    Kn[i] = w;
    s2 = fma(w.x, w.x, fma(w.y, w.y, s2));
  }
  if (nrm.res) grid_sum_c(mkc(s2, 0.0), nrm.partial, nrm.counter, nrm.res);
}
void launch_lan_axpy(cplx* Kn, const cplx* Kj, const cplx* Kp, const cplx* dot_alpha, const double* beta_prev,
                     double* alpha_out, long long n, cudaStream_t st, FusedDot nrm) {
  const unsigned nb = (unsigned)std::max<long long>(1, std::min<long long>((n + 255) / 256, FUSED_BLOCKS));
  lan_axpy_kernel<<<nb, 256, 0, st>>>(Kn, Kj, Kp, dot_alpha, beta_prev, alpha_out, n, nrm);
}

// Grid-stride: the norm and its reciprocal once per thread (FP64 square roots and
// divisions are expensive on this GPU), then one multiply per component.
// ... optionally also into copy (FP64) and f32 (complex FP32 rounded to nearest):
// the input of the next H_B application, written in the same pass.
__global__ void lan_normalize_kernel(cplx* __restrict__ out, const cplx* __restrict__ in, const cplx* __restrict__ nrm2,
                                     double* beta_out, long long n, cplx* __restrict__ copy,
                                     float2* __restrict__ f32) {
  const long long i0 = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const double beta = sqrt(nrm2->x);
  if (i0 == 0 && beta_out) *beta_out = beta;
  const double s = 1.0 / beta;
  for (long long i = i0; i < n; i += (long long)gridDim.x * blockDim.x) {
    const cplx v = in[i];
    const cplx w = mkc(v.x * s, v.y * s);
    out[i] = w;
    if (copy) copy[i] = w;
    if (f32) {
      float hx, lx, hy, ly;
      split_d2f(w.x, hx, lx);
      split_d2f(w.y, hy, ly);
      f32[i] = make_float2(hx + lx, hy + ly);
    }
  }
}
void launch_lan_normalize(cplx* out, const cplx* in, const cplx* nrm2, double* beta_out, long long n, cudaStream_t st,
                          cplx* copy, cplx* f32) {
  const long long want = (n + 255) / 256;
  const unsigned nb = (unsigned)std::max<long long>(1, std::min<long long>(want, 152 * 4));
  lan_normalize_kernel<<<nb, 256, 0, st>>>(out, in, nrm2, beta_out, n, copy, reinterpret_cast<float2*>(f32));
}

// ---------------------------------------------------------------------------
// Mean-field snapshots for the learned extrapolator: all density matrices and
// mean fields of the grid modes gathered into one complex vector (and back;
// scatter 2: the mean fields only).
// ---------------------------------------------------------------------------
__global__ void snap_gather_kernel(const SnapSeg* __restrict__ segs, int nseg, cplx* __restrict__ flat, long long E,
                                   int scatter) {
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= E) return;
  int lo = 0, hi = nseg - 1;
  while (lo < hi) {
    int mid = (lo + hi + 1) >> 1;
    if (segs[mid].offset <= i) lo = mid; else hi = mid - 1;
  }
  cplx* p = segs[lo].ptr + (i - segs[lo].offset);
  if (scatter == 2 && segs[lo].density) return;
  if (scatter) *p = flat[i]; else flat[i] = *p;
}
void launch_snap(const SnapSeg* segs, int nseg, cplx* flat, long long E, int scatter, cudaStream_t st) {
  if (E <= 0) return;
  snap_gather_kernel<<<(unsigned)((E + 255) / 256), 256, 0, st>>>(segs, nseg, flat, E, scatter);
}

// Learned mean-field extrapolation.  Each entry z of the snapshot has its values
// z_0..z_4 at the last five step starts.  Newton increments at tau:
// inc_o(tau) = P_o(tau) - P_{o-1}(tau), P_o the Lagrange polynomial through the
// last o+1 values (P_0 = z_4), with host-computed weights c.inc[tau][o-1][j].
// The scale S is the RMS over all entries of |inc_1| at the step end.

// S = sqrt(mean |inc_1(end)|^2): one block, fixed-order grid-stride sums.
__global__ void __launch_bounds__(1024) mfx_scale_kernel(MfxHist hz, MfxCoef c, double* __restrict__ S,
                                                         long long E) {
  __shared__ double red[1024];
  double acc = 0.0;
  for (long long i = threadIdx.x; i < E; i += blockDim.x) {
    cplx v = mkc(0, 0);
#pragma unroll
    for (int j = 0; j < MFX_NHIST; ++j) {
      const cplx z = hz.z[j][i];
      v.x += c.inc[1][0][j] * z.x;
      v.y += c.inc[1][0][j] * z.y;
    }
    acc += cabs2(v);
  }
  red[threadIdx.x] = acc;
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if ((int)threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) S[0] = fmax(sqrt(red[0] / (double)(E > 0 ? E : 1)), 1e-300);
}

// The entry's own scale: |inc_1| + |inc_2| at the step end plus 1e-12 S.
__device__ __forceinline__ double mfx_entry_scale(const cplx* z, const MfxCoef& c, double S) {
  cplx v1 = mkc(0, 0), v2 = mkc(0, 0);
#pragma unroll
  for (int j = 0; j < MFX_NHIST; ++j) {
    v1.x += c.inc[1][0][j] * z[j].x;
    v1.y += c.inc[1][0][j] * z[j].y;
    v2.x += c.inc[1][1][j] * z[j].x;
    v2.y += c.inc[1][1][j] * z[j].y;
  }
  return sqrt(cabs2(v1)) + sqrt(cabs2(v2)) + 1e-12 * S + 1e-300;
}

// Network inputs per entry: Re/Im of inc_1..inc_4 at the half step and the step
// end divided by the entry's scale, then the step-length ratios; each divided by
// its column scale.
__global__ void mfx_features_kernel(MfxHist hz, MfxCoef c, const double* __restrict__ S, float* __restrict__ X,
                                    long long E) {
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= E) return;
  cplx z[MFX_NHIST];
#pragma unroll
  for (int j = 0; j < MFX_NHIST; ++j) z[j] = hz.z[j][i];
  const double q = 1.0 / mfx_entry_scale(z, c, S[0]);
  float* x = X + (long long)MFX_NFEAT * i;
  int col = 0;
#pragma unroll
  for (int tau = 0; tau < 2; ++tau) {
#pragma unroll
    for (int o = 0; o < MFX_NHIST - 1; ++o) {
      cplx v = mkc(0, 0);
#pragma unroll
      for (int j = 0; j < MFX_NHIST; ++j) {
        v.x += c.inc[tau][o][j] * z[j].x;
        v.y += c.inc[tau][o][j] * z[j].y;
      }
      x[col] = (float)(v.x * q / c.fscale[col]);
      ++col;
      x[col] = (float)(v.y * q / c.fscale[col]);
      ++col;
    }
  }
#pragma unroll
  for (int r = 0; r < MFX_NHIST - 1; ++r, ++col) x[col] = (float)(c.ratio[r] / c.fscale[col]);
}

// z(tau) = polynomial extrapolation + s * tscale * y at the half step and the step
// end (s the entry's scale)
__global__ void mfx_combine_kernel(MfxHist hz, MfxCoef c, const float* __restrict__ Y, const double* __restrict__ S,
                                   cplx* __restrict__ half, cplx* __restrict__ full, long long E) {
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= E) return;
  cplx z[MFX_NHIST];
#pragma unroll
  for (int j = 0; j < MFX_NHIST; ++j) z[j] = hz.z[j][i];
  const float* y = Y + (long long)MFX_NOUT * i;
  const double s = mfx_entry_scale(z, c, S[0]);
  cplx out[2];
#pragma unroll
  for (int tau = 0; tau < 2; ++tau) {
    cplx v = mkc(0, 0);
#pragma unroll
    for (int j = 0; j < MFX_NHIST; ++j) {
      v.x += c.base[tau][j] * z[j].x;
      v.y += c.base[tau][j] * z[j].y;
    }
    v.x += s * c.tscale[2 * tau] * (double)y[2 * tau];
    v.y += s * c.tscale[2 * tau + 1] * (double)y[2 * tau + 1];
    out[tau] = v;
  }
  half[i] = out[0];
  full[i] = out[1];
}

void launch_mfx_features(const MfxHist& hz, const MfxCoef& c, double* S, float* X, long long E, cudaStream_t st) {
  if (E <= 0) return;
  mfx_scale_kernel<<<1, 1024, 0, st>>>(hz, c, S, E);
  mfx_features_kernel<<<(unsigned)((E + 255) / 256), 256, 0, st>>>(hz, c, S, X, E);
}
void launch_mfx_combine(const MfxHist& hz, const MfxCoef& c, const float* Y, const double* S, cplx* half, cplx* full,
                        long long E, cudaStream_t st) {
  if (E <= 0) return;
  mfx_combine_kernel<<<(unsigned)((E + 255) / 256), 256, 0, st>>>(hz, c, Y, S, half, full, E);
}

// ---------------------------------------------------------------------------
// Statistical mixtures and dissipation
// ---------------------------------------------------------------------------

// Partial sums of <X_i|Y_j> (one row of PK_GRAM_BLOCKS blocks per pair).
__global__ void __launch_bounds__(256) pk_gram_kernel(const PkGramPair* __restrict__ pairs,
                                                      const PkState* __restrict__ st, int nstates,
                                                      cplx* __restrict__ partial) {
  const PkGramPair pr = pairs[blockIdx.y];
  double re = 0.0, im = 0.0;
  for (int s = 0; s < nstates; ++s) {
    const PkState q = st[s];
    const cplx* x = pr.X + q.off + (long long)pr.i * q.n;
    const cplx* y = pr.Y + q.off + (long long)pr.j * q.n;
    for (long long c = blockIdx.x * 256LL + threadIdx.x; c < q.n; c += 256LL * gridDim.x) {
      const cplx a = x[c], b = y[c];
      re = fma(a.x, b.x, fma(a.y, b.y, re));
      im = fma(a.x, b.y, fma(-a.y, b.x, im));
    }
  }
  __shared__ double sr[8], si[8];
  for (int o = 16; o > 0; o >>= 1) {
    re += __shfl_down_sync(0xffffffffu, re, o);
    im += __shfl_down_sync(0xffffffffu, im, o);
  }
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  if (l == 0) { sr[w] = re; si[w] = im; }
  __syncthreads();
  if (threadIdx.x == 0) {
    double r = 0.0, i2 = 0.0;
    for (int k = 0; k < 8; ++k) { r += sr[k]; i2 += si[k]; }
    partial[(long long)blockIdx.y * PK_GRAM_BLOCKS + blockIdx.x] = make_double2(r, i2);
  }
}

void launch_pk_gram(const PkGramPair* d_pairs, int npairs, const PkState* d_st, int nstates, cplx* partial,
                    cudaStream_t st) {
  if (npairs <= 0) return;
  pk_gram_kernel<<<dim3(PK_GRAM_BLOCKS, npairs), 256, 0, st>>>(d_pairs, d_st, nstates, partial);
}

__device__ __forceinline__ cplx pk_mul(cplx a, cplx b) { return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x); }
__device__ __forceinline__ cplx pk_conj(cplx a) { return make_double2(a.x, -a.y); }

// Packet populations, Lagrange multipliers and mixing matrices (one block).
// WPpopm1 = p / (p^2 + (eps exp(-(p/eps)^2))^2) (gmctdh_objects.f90:616-619);
// type 1 (:661-692): AVA = <A_i|V A_j>, multLagDiag -= aeD1 sum |AVA_ij|^2 WPpopm1_i,
// multLag_ij += aeD1 (AVA AVA^H)_ij (WPpopm1_i + WPpopm1_j) for i > j, D_W += aeD1 WPpopm1_W
// sum_j V A_j conj(AVA_Wj), AuxA_W = i aeD1 WPpopm1_W sum_j A_j conj(AVA_Wj);
// type 2 (:805-818) with G_ij = <A_i|X A_j>, X = sum_t f i aeD2 ae_t W_t:
// multLagDiag -= Re sum_W G_WW, multLag_ij += G_ij + conj(G_ji) for i > j;
// then multLag_ij *= i dw / (dw^2 + (eps exp(-(dw/eps)^2))^2), dw = p_i - p_j (:1128-1137).
__global__ void __launch_bounds__(256) pk_coef_kernel(PkCoefArgs a) {
  extern __shared__ cplx g[];   // [npairs]
  __shared__ double pop[MAX_PACKETS], wpm1[MAX_PACKETS];
  __shared__ cplx M[MAX_PACKETS * MAX_PACKETS];
  __shared__ double dterm[MAX_PACKETS * MAX_PACKETS];
  // one warp per pair: the PK_GRAM_BLOCKS (= 32) block sums, one per lane, added by
  // a fixed shuffle tree
  const int lane = threadIdx.x & 31, tid = threadIdx.x;
  for (int p = tid >> 5; p < a.npairs; p += blockDim.x >> 5) {
    const cplx v = a.partial[(long long)p * PK_GRAM_BLOCKS + lane];
    double r = v.x, i2 = v.y;
    for (int o = 16; o > 0; o >>= 1) {
      r += __shfl_down_sync(0xffffffffu, r, o);
      i2 += __shfl_down_sync(0xffffffffu, i2, o);
    }
    if (lane == 0) g[p] = make_double2(r, i2);
  }
  const int P = a.P, PP = P * P;
  if (tid < P) {
    const double p = P > 1 ? a.norms[3 * tid].x : 1.0;
    const double r = a.eps_pop * exp(-(p / a.eps_pop) * (p / a.eps_pop));
    pop[tid] = p;
    wpm1[tid] = p / (p * p + r * r);
    a.pop[tid] = p;
  }
  // thread (i, j) = (tid % P, tid / P) owns M[i + P j] and its share of multLagDiag
  const int i = tid % P, j = tid / P;
  const bool own = tid < PP;
  if (own) {
    M[tid] = make_double2(0.0, 0.0);
    dterm[tid] = 0.0;
  }
  __syncthreads();
  int base = a.has2 ? PP : 0;
  for (int k = 0; k < a.ndiss1; ++k, base += PP) {
    const cplx* V = g + base;   // V[i + P j] = <A_i|V_k A_j>
    const double ae = a.aeD1[k];
    if (own) {
      const cplx v = V[tid];
      dterm[tid] -= ae * (v.x * v.x + v.y * v.y) * wpm1[i];
      if (i > j) {
        cplx h = make_double2(0.0, 0.0);
        for (int l = 0; l < P; ++l) {
          const cplx t = pk_mul(V[i + P * l], pk_conj(V[j + P * l]));
          h.x += t.x;
          h.y += t.y;
        }
        const double f = ae * (wpm1[i] + wpm1[j]);
        M[tid].x += h.x * f;
        M[tid].y += h.y * f;
      }
      // C[j' + P w] with (j', w) = (i, j): conj(V[w + P j']) scaled by aeD1 WPpopm1_w
      const cplx v2 = pk_conj(V[j + P * i]);
      const double f = ae * wpm1[j];
      a.C1[(long long)k * PP + tid] = make_double2(v2.x * f, v2.y * f);
      a.C2[(long long)k * PP + tid] = make_double2(-v2.y * f, v2.x * f);
    }
  }
  if (a.has2 && own) {
    const cplx* G = g;
    if (i == j) dterm[tid] -= G[tid].x;
    if (i > j) {
      M[tid].x += G[i + P * j].x + G[j + P * i].x;
      M[tid].y += G[i + P * j].y - G[j + P * i].y;
    }
  }
  if (own && i > j) {
    const double dw = pop[i] - pop[j];
    const double r = a.eps_pop * exp(-(dw / a.eps_pop) * (dw / a.eps_pop));
    const double f = dw / (dw * dw + r * r);
    const cplx m = M[tid];
    M[tid] = make_double2(-m.y * f, m.x * f);   // times i f
  }
  __syncthreads();
  if (own) {
    // multLagDiag: the owners' shares added in a fixed order
    double mdiag = 0.0;
    if (i == j)
      for (int q = 0; q < PP; ++q) mdiag += dterm[q];
    // ML = multLagDiag I + i H, H Hermitian from the lower triangle with a zero diagonal
    const cplx h = i > j ? M[tid] : (i < j ? pk_conj(M[j + P * i]) : make_double2(0.0, 0.0));
    a.ML[tid] = make_double2(-h.y + (i == j ? mdiag : 0.0), h.x);
  }
}

void launch_pk_coef(const PkCoefArgs& a, cudaStream_t st) {
  pk_coef_kernel<<<1, 256, sizeof(cplx) * (a.npairs + 1), st>>>(a);
}

__global__ void __launch_bounds__(256) pk_mix_kernel(const PkMix* __restrict__ mix, int nmix,
                                                     const PkState* __restrict__ st, int nstates,
                                                     long long n1tot, int P, cplx* out0) {
  extern __shared__ cplx cm[];   // [nmix][P][P]
  for (int q = threadIdx.x; q < nmix * P * P; q += blockDim.x) cm[q] = mix[q / (P * P)].C[q % (P * P)];
  __syncthreads();
  for (long long e = blockIdx.x * 256LL + threadIdx.x; e < n1tot; e += 256LL * gridDim.x) {
    long long c = e;
    int s = 0;
    while (s + 1 < nstates && c >= st[s].n) c -= st[s++].n;
    const long long off = st[s].off + c, n = st[s].n;
    for (int d = 0; d < nmix; ++d) {
      const cplx* in = mix[d].in + off;
      cplx* out = (out0 ? out0 : mix[d].out) + off;
      const cplx* C = cm + d * P * P;
      cplx x[MAX_PACKETS];
      for (int j = 0; j < P; ++j) x[j] = in[j * n];
      for (int w = 0; w < P; ++w) {
        double re = 0.0, im = 0.0;
        for (int j = 0; j < P; ++j) {
          const cplx cc = C[j + P * w];
          re = fma(x[j].x, cc.x, fma(-x[j].y, cc.y, re));
          im = fma(x[j].x, cc.y, fma(x[j].y, cc.x, im));
        }
        if (mix[d].accumulate) {
          const cplx o = out[w * n];
          re += o.x;
          im += o.y;
        }
        out[w * n] = make_double2(re, im);
      }
    }
  }
}

void launch_pk_mix(const PkMix* d_mix, int nmix, const PkState* d_st, int nstates, long long n1tot, int P,
                   cplx* out0, cudaStream_t st) {
  if (nmix <= 0 || n1tot <= 0) return;
  const long long nb = std::min<long long>((n1tot + 255) / 256, FUSED_BLOCKS);
  pk_mix_kernel<<<(int)nb, 256, sizeof(cplx) * nmix * P * P, st>>>(d_mix, nmix, d_st, nstates, n1tot, P, out0);
}
