// Gaussian (G-MCTDH) block of the equations of motion on the device:
//  - normalised overlaps of multi-dimensional Gaussians (GauOvlMultiD,
//    gmctdh_objects.f90:1497-1519) for S00 and for <Psi1|Psi2>;
//  - one-dimensional integrals <g1|op|g2>/<g1|g2> and <dg1/dxi|op|g2>/<g1|g2>
//    (GauInt1D / Gau10Int1D, hamilton.f90:745-902) and h1mode of a Gaussian
//    mode (hamilton.f90:494-524);
//  - Calc_CY (gmctdh_objects.f90:1198-1333): Sa0, Sa0 S^-1, the matrix C and the
//    vector Y of the parameter equations;
//  - the Tikhonov-regularised solve C x = Y (StdRegSol 'tikh', maths.f90:87-162),
//    dxi = der_factor * x (derivatives.f90:158-173) and the tau matrices of the
//    coefficient correction (derivatives.f90:201-234).
//
// The reference solves C x = Y through the eigen-decomposition of C,
// x = sum_j u_j w_j / (w_j^2 + eps^2) (u_j^H Y).  That is the minimiser of
// |C x - Y|^2 + eps^2 |x|^2, which this file computes as the least-squares
// solution of the stacked system [C; eps I] x = [Y; 0] by Householder QR: the
// same x, with the conditioning of C/eps instead of (C/eps)^2 of the normal
// equations, and no iterative eigen-solver.  The QR runs in panels of
// GWP_QR_PW columns: every block of a launch factors the panel in shared memory
// and applies its reflectors to its own trailing columns (one warp per column),
// so no block reads what another block of the same launch writes.
#include <float.h>

#include <algorithm>

#include "kernels.cuh"

namespace {

__device__ __forceinline__ cplx cexp_(cplx z) {
  const double e = exp(z.x);
  double s, c;
  sincos(z.y, &s, &c);
  return mkc(e * c, e * s);
}
__device__ __forceinline__ cplx neg_i(cplx z) { return mkc(z.y, -z.x); }   // -i z
__device__ __forceinline__ cplx cdivr(cplx z, double r) { return mkc(z.x / r, z.y / r); }
__device__ __forceinline__ cplx cdiv(cplx a, cplx b) {
  const double d = b.x * b.x + b.y * b.y;
  return mkc((a.x * b.x + a.y * b.y) / d, (a.y * b.x - a.x * b.y) / d);
}

// T(k, n) = binomial(n, 2k) * (2k-1)!!, the moment coefficients of hamilton.f90:761-785
// (every intermediate of the product formula is an exact integer below 2^53).
__device__ double gau_coeff(int k, int n) {
  double b = 1.0;
  for (int i = 0; i < 2 * k; ++i) b = b * (double)(n - i) / (double)(i + 1);
  double df = 1.0;
  for (int x = 2 * k - 1; x > 0; x -= 2) df *= (double)x;
  return b * df;
}
__device__ cplx cpow_int(cplx z, int m) {
  cplx r = mkc(1.0, 0.0);
  for (int i = 0; i < m; ++i) r = cmul(r, z);
  return r;
}
__device__ double rpow_int(double z, int m) {
  double r = 1.0;
  for (int i = 0; i < m; ++i) r *= z;
  return r;
}

// <g1|op|g2>/<g1|g2> for g = exp(a x^2 + xi x) and the primitive operator code iop
// (0 identity, -1 p, -2 d^2/dq^2, -3 qp, k >= 1: q^k).
__device__ cplx gau_int_1d(double a1, double a2, cplx xi1, cplx xi2, int iop) {
  const cplx x1c = cconj(xi1);
  const double a12 = a1 + a2;
  switch (iop) {
    case 0:
      return mkc(1.0, 0.0);
    case -1: {
      const cplx num = csub(cscale(xi2, a1), cscale(x1c, a2));
      return cdivr(neg_i(num), a12);
    }
    case -2: {
      const cplx u = cdivr(csub(cscale(x1c, a2), cscale(xi2, a1)), a12);
      return cadd(cmul(u, u), mkc(2.0 * a1 * a2 / a12, 0.0));
    }
    case -3: {
      const cplx g = cadd(mkc(a1 * a1 - a2 * a2, 0.0), cmul(csub(cscale(x1c, a2), cscale(xi2, a1)), cadd(x1c, xi2)));
      return cdivr(neg_i(g), a12 * a12);
    }
    case 1:
      return cdivr(cadd(x1c, xi2), -2.0 * a12);
    case 2: {
      const double a = 2.0 * a12;
      const cplx v = cdivr(cadd(x1c, xi2), a);
      return csub(cmul(v, v), mkc(1.0 / a, 0.0));
    }
    default:
      break;
  }
  const cplx c1 = cadd(x1c, xi2);
  const double an = -2.0 * a12;
  if (iop >= 3 && iop <= 19 && (iop & 1)) {
    cplx g = mkc(0.0, 0.0);
    for (int k = 0; k <= iop / 2; ++k) {
      const double f = gau_coeff(k, iop) / rpow_int(an, iop - k);
      g = cadd(g, cscale(cpow_int(c1, iop - 2 * k), f));
    }
    return g;
  }
  if (iop >= 4 && iop <= 20 && !(iop & 1)) {
    const cplx c2 = cdivr(cmul(c1, c1), an);
    cplx p = mkc(1.0, 0.0);
    cplx g = mkc(0.0, 0.0);
    for (int k = iop / 2; k >= 0; --k) {
      g = cadd(g, cscale(p, gau_coeff(k, iop)));
      p = cmul(p, c2);
    }
    return cdivr(g, rpow_int(an, iop / 2));
  }
  return mkc(nan(""), 0.0);   // unsupported codes are rejected when the plan is built
}

// <dg1/dxi1|op|g2>/<g1|g2> (Gau10Int1D)
__device__ cplx gau10_int_1d(double a1, double a2, cplx xi1, cplx xi2, int iop) {
  if (iop == -1) {
    const cplx t1 = neg_i(cmul(xi2, gau_int_1d(a1, a2, xi1, xi2, 1)));
    const cplx t2 = cscale(neg_i(gau_int_1d(a1, a2, xi1, xi2, 2)), 2.0 * a2);
    return cadd(t1, t2);
  }
  if (iop == -2) {
    const cplx g1 = gau_int_1d(a1, a2, xi1, xi2, 1);
    const cplx g2 = gau_int_1d(a1, a2, xi1, xi2, 2);
    const cplx g3 = gau_int_1d(a1, a2, xi1, xi2, 3);
    cplx r = cmul(cadd(mkc(a2 + a2, 0.0), cmul(xi2, xi2)), g1);
    r = cadd(r, cmul(cscale(xi2, 4.0 * a2), g2));
    return cadd(r, cscale(g3, 4.0 * a2 * a2));
  }
  if (iop == -3) {
    const cplx g1 = gau_int_1d(a1, a2, xi1, xi2, 1);
    const cplx g2 = gau_int_1d(a1, a2, xi1, xi2, 2);
    const cplx g3 = gau_int_1d(a1, a2, xi1, xi2, 3);
    return neg_i(cadd(cadd(g1, cmul(cscale(xi2, 2.0), g2)), cscale(g3, 4.0 * a2)));
  }
  return gau_int_1d(a1, a2, xi1, xi2, iop + 1);
}

// Normalised overlap of two nmd-dimensional Gaussians.
__device__ cplx gau_ovl(const double* a1, const double* a2, const cplx* xi1, const cplx* xi2, int nmd) {
  bool same = true;
  for (int k = 0; k < nmd; ++k)
    if (!(fabs(a1[k] - a2[k]) < DBL_EPSILON)) same = false;
  cplx c = mkc(0.0, 0.0);
  if (same) {
    for (int k = 0; k < nmd; ++k) {
      const cplx s = cadd(cconj(xi1[k]), xi2[k]);
      const cplx t = csub(mkc(xi1[k].x * xi1[k].x + xi2[k].x * xi2[k].x, 0.0), cscale(cmul(s, s), 0.5));
      c = cadd(c, cdivr(t, a1[k]));
    }
    return cexp_(cscale(c, 0.25));
  }
  double d = 1.0;
  for (int k = 0; k < nmd; ++k) {
    const cplx s = cadd(cconj(xi1[k]), xi2[k]);
    const double a12 = a1[k] + a2[k];
    c = cadd(c, mkc(xi1[k].x * xi1[k].x / a1[k] + xi2[k].x * xi2[k].x / a2[k], 0.0));
    c = csub(c, cdivr(cmul(s, s), a12));
    d *= 4.0 * a1[k] * a2[k] / (a12 * a12);
  }
  return cscale(cexp_(cscale(c, 0.25)), sqrt(sqrt(d)));
}

__global__ void gwp_ovl_kernel(const GwpOvlDesc* __restrict__ descs) {
  const GwpOvlDesc& d = descs[blockIdx.x];
  for (int e = threadIdx.x; e < d.n1 * d.n2; e += blockDim.x) {
    const int j1 = e % d.n1, j2 = e / d.n1;
    cplx v;
    if (d.kind == 3) {
      // Calc_Err_SPF (cmf2_derivatives.f90:301-315): 2 - 2 Re<g(x)|g(y)> on the
      // diagonal, S(x,x) + S(y,y) - S(x,y) - S(y,x) above it
      if (j1 > j2) continue;
      const double* a1 = d.a + d.lda * j1;
      const double* a2 = d.a + d.lda * j2;
      const cplx* x1 = d.xi1 + d.nmd * j1;
      const cplx* x2 = d.xi1 + d.nmd * j2;
      const cplx* y1 = d.xi2 + d.nmd * j1;
      const cplx* y2 = d.xi2 + d.nmd * j2;
      if (j1 == j2) {
        v = mkc(2.0 - 2.0 * gau_ovl(a1, a1, x1, y1, d.nmd).x, 0.0);
      } else {
        v = cadd(gau_ovl(a1, a2, x1, x2, d.nmd), gau_ovl(a1, a2, y1, y2, d.nmd));
        v = csub(v, gau_ovl(a1, a2, x1, y2, d.nmd));
        v = csub(v, gau_ovl(a1, a2, y1, x2, d.nmd));
      }
    } else if (d.kind == 0 && j1 == j2) {
      v = mkc(1.0, 0.0);
    } else if (d.kind == 0 && j1 > j2) {
      v = cconj(gau_ovl(d.a + d.lda * j2, d.a + d.lda * j1, d.xi1 + d.nmd * j2, d.xi2 + d.nmd * j1, d.nmd));
    } else if (d.kind == 2) {
      v = cconj(gau_ovl(d.a + d.lda * j2, d.a + d.lda * j1, d.xi2 + d.nmd * j2, d.xi1 + d.nmd * j1, d.nmd));
    } else {
      v = gau_ovl(d.a + d.lda * j1, d.a + d.lda * j2, d.xi1 + d.nmd * j1, d.xi2 + d.nmd * j2, d.nmd);
    }
    d.out[e] = v;
  }
}

__device__ cplx gwp_h1_entry(const GwpH1Desc& d, int j1, int j2) {
  cplx g = mkc(1.0, 0.0);
  for (int k = 0; k < d.nmd; ++k)
    g = cmul(g, gau_int_1d(d.a[k + d.lda * j1], d.a[k + d.lda * j2], d.xi1[k + d.nmd * j1], d.xi2[k + d.nmd * j2],
                           d.ops[k]));
  return cmul(d.S[j1 + d.n1 * j2], g);
}

__global__ void gwp_h1_kernel(const GwpH1Desc* __restrict__ descs) {
  const GwpH1Desc& d = descs[blockIdx.x];
  for (int e = threadIdx.x; e < d.n1 * d.n2; e += blockDim.x) {
    const int j1 = e % d.n1, j2 = e / d.n1;
    d.out[e] = (d.same_state && j1 > j2) ? cconj(gwp_h1_entry(d, j2, j1)) : gwp_h1_entry(d, j1, j2);
  }
}

// Sa0 (nG x n): <dg_j1/dxi_k | g_j2> / normalisation, upper blocks from the
// integrals and the lower ones as conjugates (gmctdh_objects.f90:1218-1240).
__global__ void gwp_sa0_kernel(const GwpCYDesc* __restrict__ descs) {
  const GwpCYDesc& d = descs[blockIdx.y];
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= d.nG * d.n) return;
  const int r = e % d.nG, j2 = e / d.nG;
  const int j1 = r / d.nmd, k = r % d.nmd;
  cplx v;
  if (j1 <= j2) {
    v = cmul(d.S[j1 + d.n * j2], gau_int_1d(d.a[k + d.lda * j1], d.a[k + d.lda * j2], d.xi[k + d.nmd * j1],
                                            d.xi[k + d.nmd * j2], 1));
  } else {
    v = cconj(cmul(d.S[j2 + d.n * j1], gau_int_1d(d.a[k + d.lda * j2], d.a[k + d.lda * j1], d.xi[k + d.nmd * j2],
                                                  d.xi[k + d.nmd * j1], 1)));
  }
  d.Sa0[e] = v;
}

// Sa0Sm1 = Sa0 * S^-1 (nG x n)
__global__ void gwp_sa0sm1_kernel(const GwpCYDesc* __restrict__ descs) {
  const GwpCYDesc& d = descs[blockIdx.y];
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= d.nG * d.n) return;
  const int r = e % d.nG, j = e / d.nG;
  cplx s = mkc(0.0, 0.0);
  for (int l = 0; l < d.n; ++l) cfma(s, d.Sa0[r + d.nG * l], d.Sm1[l + d.n * j]);
  d.Sa0Sm1[e] = s;
}

// Upper-triangle entry (r <= c) of C = rho o (Sab - (Sa0Sm1 Sa0^H + Sa0 Sa0Sm1^H)/2)
// (gmctdh_objects.f90:1242-1283).
__device__ cplx gwp_c_entry(const GwpCYDesc& d, int r, int c) {
  const int j1 = r / d.nmd, k1 = r % d.nmd, j2 = c / d.nmd, k2 = c % d.nmd;
  const double* a = d.a;
  const cplx* xi = d.xi;
  cplx v;
  if (k1 == k2) {
    v = gau_int_1d(a[k1 + d.lda * j1], a[k2 + d.lda * j2], xi[k1 + d.nmd * j1], xi[k2 + d.nmd * j2], 2);
  } else {
    const cplx g1 = gau_int_1d(a[k1 + d.lda * j1], a[k1 + d.lda * j2], xi[k1 + d.nmd * j1], xi[k1 + d.nmd * j2], 1);
    const cplx g2 = gau_int_1d(a[k2 + d.lda * j1], a[k2 + d.lda * j2], xi[k2 + d.nmd * j1], xi[k2 + d.nmd * j2], 1);
    v = cmul(g1, g2);
  }
  cplx sab = cmul(d.S[j1 + d.n * j2], v);
  cplx s1 = mkc(0.0, 0.0), s2 = mkc(0.0, 0.0);
  for (int j = 0; j < d.n; ++j) {
    cfma(s1, d.Sa0Sm1[r + d.nG * j], cconj(d.Sa0[c + d.nG * j]));
    cfma(s2, d.Sa0[r + d.nG * j], cconj(d.Sa0Sm1[c + d.nG * j]));
  }
  sab = csub(sab, cscale(cadd(s1, s2), 0.5));
  return cmul(d.rho[j1 + d.n * j2], sab);
}

// The stacked least-squares system [C, Y; eps I, 0]: the Hermitian C from its
// upper triangle, the Tikhonov block below it.
__global__ void gwp_c_kernel(const GwpCYDesc* __restrict__ descs) {
  const GwpCYDesc& d = descs[blockIdx.z];
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  const int c = blockIdx.y * blockDim.y + threadIdx.y;
  if (r >= d.nG || c >= d.nG) return;
  const long long ld = 2LL * d.nG;
  d.M[r + ld * c] = (r <= c) ? gwp_c_entry(d, r, c) : cconj(gwp_c_entry(d, c, r));
  d.M[d.nG + r + ld * c] = mkc(r == c ? d.eps : 0.0, 0.0);
}

// Y (gmctdh_objects.f90:1285-1326): per entry r = j1*nmd + k,
// sum over operators (outer) and j2 (inner) of MF(j1,j2) (Ha0 - Sa0Sm1 h)(r, j2).
// Stage 1: one thread per (j1, j2, operator) computes the nmd one-dimensional
// integrals of the pair once, shares them between the k entries through
// prefix/suffix products, and writes the nmd terms to part[((o*n2 + j2)*nG + r)].
// Stage 2: one thread per r adds its terms in the reference's order.
__global__ void gwp_y_part_kernel(const GwpCYDesc* __restrict__ descs, const GwpYOp* __restrict__ ops,
                                  cplx* __restrict__ part, long long part_ld, int maxn2) {
  const GwpCYDesc& d = descs[blockIdx.y];
  const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= (long long)d.n * maxn2 * d.op_count) return;
  const int j1 = (int)(e % d.n);
  const int j2 = (int)((e / d.n) % maxn2);
  const int o = (int)(e / ((long long)d.n * maxn2));
  const GwpYOp& op = ops[d.op_first + o];
  if (j2 >= op.n2) return;
  const int nmd = d.nmd;
  const double* a = d.a;
  cplx g[GWP_MAXDOF], pre[GWP_MAXDOF + 1];
  for (int q = 0; q < nmd; ++q)
    g[q] = gau_int_1d(a[q + d.lda * j1], a[q + d.lda * j2], d.xi[q + d.nmd * j1], op.xi2[q + d.nmd * j2], op.ops[q]);
  pre[0] = mkc(1.0, 0.0);
  for (int q = 0; q < nmd; ++q) pre[q + 1] = cmul(pre[q], g[q]);
  const cplx s12 = op.S12[j1 + d.n * j2];
  const cplx mf = op.mf[j1 + d.n * j2];
  cplx* out = part + (long long)blockIdx.y * part_ld + ((long long)o * maxn2 + j2) * d.nG;
  for (int k = 0; k < nmd; ++k) {
    cplx right = mkc(1.0, 0.0);   // prod_{q > k} g[q] in order (np.prod over gi[k+1:])
    for (int q = k + 1; q < nmd; ++q) right = cmul(right, g[q]);
    const cplx g10 = gau10_int_1d(a[k + d.lda * j1], a[k + d.lda * j2], d.xi[k + d.nmd * j1],
                                  op.xi2[k + d.nmd * j2], op.ops[k]);
    const cplx ha0 = cmul(cmul(s12, cmul(pre[k], right)), g10);
    const int r = j1 * nmd + k;
    cplx sh = mkc(0.0, 0.0);
    for (int j = 0; j < d.n; ++j) cfma(sh, d.Sa0Sm1[r + d.nG * j], op.h[j + d.n * j2]);
    out[r] = cmul(mf, csub(ha0, sh));
  }
}

__global__ void gwp_y_sum_kernel(const GwpCYDesc* __restrict__ descs, const GwpYOp* __restrict__ ops,
                                 const cplx* __restrict__ part, long long part_ld, int maxn2) {
  const GwpCYDesc& d = descs[blockIdx.y];
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= d.nG) return;
  const cplx* base = part + (long long)blockIdx.y * part_ld;
  cplx acc = mkc(0.0, 0.0);
  for (int o = 0; o < d.op_count; ++o) {
    const int n2 = ops[d.op_first + o].n2;
    for (int j2 = 0; j2 < n2; ++j2) acc = cadd(acc, base[((long long)o * maxn2 + j2) * d.nG + r]);
  }
  const long long ld = 2LL * d.nG;
  d.M[r + ld * d.nG] = acc;
  d.M[d.nG + r + ld * d.nG] = mkc(0.0, 0.0);
}

// Fixed-order block reduction of a double over 256 threads.
__device__ double block_sum(double v, double* red) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  __syncthreads();
  if (lane == 0) red[warp] = v;
  __syncthreads();
  double t = 0.0;
  if (threadIdx.x == 0) {
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += red[w];
    red[32] = t;
  }
  __syncthreads();
  return red[32];
}
__device__ cplx warp_sum(cplx v) {
  for (int o = 16; o > 0; o >>= 1) {
    v.x += __shfl_down_sync(0xffffffffu, v.x, o);
    v.y += __shfl_down_sync(0xffffffffu, v.y, o);
  }
  v.x = __shfl_sync(0xffffffffu, v.x, 0);
  v.y = __shfl_sync(0xffffffffu, v.y, 0);
  return v;
}

// One panel of the Householder QR of M (2nG x (nG+1), the last column the
// right-hand side).  Shared: the panel rows j0.. of columns j0..j0+pw-1.
// cpb: trailing columns per block (one warp each, cpb <= 8)
__global__ void __launch_bounds__(256) gwp_qr_panel_kernel(const GwpCYDesc* __restrict__ descs, int j0, int cpb) {
  extern __shared__ cplx P[];
  __shared__ double red[33];
  __shared__ cplx s_alpha[GWP_QR_PW];
  __shared__ double s_tau[GWP_QR_PW];
  const GwpCYDesc& d = descs[blockIdx.y];
  const int nG = d.nG;
  if (j0 >= nG) return;
  const int pw = min(GWP_QR_PW, nG - j0);
  const int ncol = nG + 1;
  const int trailing = ncol - (j0 + pw);
  const int nblk = (trailing + cpb - 1) / cpb;
  if ((int)blockIdx.x > 0 && (int)blockIdx.x >= nblk) return;
  const long long ld = 2LL * nG;
  const int rows = 2 * nG - j0;
  for (int e = threadIdx.x; e < rows * pw; e += blockDim.x) {
    const int rr = e % rows, jj = e / rows;
    P[e] = d.M[(j0 + rr) + ld * (j0 + jj)];
  }
  __syncthreads();
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  for (int jj = 0; jj < pw; ++jj) {
    cplx* col = P + (long long)rows * jj;
    // reflector j0+jj has no support below row nG + j0 + jj: the eps I block below C
    // only fills in down to that row (panel-relative: nG + jj)
    const int rend = min(rows, nG + jj + 1);
    double part = 0.0;
    for (int rr = jj + threadIdx.x; rr < rend; rr += blockDim.x) part += cabs2(col[rr]);
    const double nrm2 = block_sum(part, red);
    if (threadIdx.x == 0) {
      const double nrm = sqrt(nrm2);
      const cplx x0 = col[jj];
      const double ax0 = sqrt(cabs2(x0));
      if (nrm == 0.0) {
        s_alpha[jj] = mkc(0.0, 0.0);
        s_tau[jj] = 0.0;
      } else {
        const cplx ph = (ax0 > 0.0) ? cdivr(x0, ax0) : mkc(1.0, 0.0);
        const cplx alpha = cscale(ph, -nrm);
        col[jj] = csub(x0, alpha);
        s_alpha[jj] = alpha;
        s_tau[jj] = 2.0 / (2.0 * nrm2 + 2.0 * nrm * ax0);
      }
    }
    __syncthreads();
    // apply the reflector to the later panel columns, one warp per column
    const int c = jj + 1 + warp;
    if (c < pw && s_tau[jj] != 0.0) {
      cplx* y = P + (long long)rows * c;
      cplx w = mkc(0.0, 0.0);
      for (int rr = jj + lane; rr < rend; rr += 32) cfma_conj(w, col[rr], y[rr]);
      w = warp_sum(w);
      const cplx f = cscale(w, s_tau[jj]);
      for (int rr = jj + lane; rr < rend; rr += 32) y[rr] = csub(y[rr], cmul(col[rr], f));
    }
    __syncthreads();
  }
  // trailing columns of this block (the right-hand side is column nG)
  const int c = j0 + pw + blockIdx.x * cpb + warp;
  if (warp < cpb && c < ncol) {
    cplx* y = d.M + ld * c;
    for (int jj = 0; jj < pw; ++jj) {
      if (s_tau[jj] == 0.0) continue;
      const cplx* v = P + (long long)rows * jj;
      cplx w = mkc(0.0, 0.0);
      const int rend = min(rows, nG + jj + 1);
      for (int rr = jj + lane; rr < rend; rr += 32) cfma_conj(w, v[rr], y[j0 + rr]);
      w = warp_sum(w);
      const cplx f = cscale(w, s_tau[jj]);
      for (int rr = jj + lane; rr < rend; rr += 32) y[j0 + rr] = csub(y[j0 + rr], cmul(v[rr], f));
      __syncwarp();
    }
  }
  // the R entries of the panel columns (rows j0.., above and on the diagonal)
  if (blockIdx.x == 0) {
    for (int e = threadIdx.x; e < pw * pw; e += blockDim.x) {
      const int rr = e % pw, jj = e / pw;
      if (rr > jj) continue;
      d.R[(j0 + rr) + (long long)nG * (j0 + jj)] = (rr == jj) ? s_alpha[jj] : P[rr + (long long)rows * jj];
    }
  }
}

// Back substitution R x = (Q^H b)[0:nG], then dxi = der * x and tau.
__global__ void __launch_bounds__(256) gwp_backsub_kernel(const GwpCYDesc* __restrict__ descs, cplx der,
                                                          cplx* __restrict__ out, int* status) {
  extern __shared__ cplx sh[];
  const GwpCYDesc& d = descs[blockIdx.x];
  const int nG = d.nG;
  const long long ld = 2LL * nG;
  cplx* b = sh;
  cplx* xs = sh + nG;
  for (int r = threadIdx.x; r < nG; r += blockDim.x) b[r] = d.M[r + ld * nG];
  __syncthreads();
  for (int c = nG - 1; c >= 0; --c) {
    if (threadIdx.x == 0) {
      const cplx rc = d.R[c + (long long)nG * c];
      cplx xv = cdiv(b[c], rc);
      if (!isfinite(xv.x) || !isfinite(xv.y)) {
        atomicOr(status, DEVST_NONFINITE);
        xv = mkc(0.0, 0.0);
      }
      xs[c] = xv;
    }
    __syncthreads();
    const int pstart = (c / GWP_QR_PW) * GWP_QR_PW;
    const cplx xc = xs[c];
    for (int r = threadIdx.x; r < c; r += blockDim.x) {
      const cplx rv = (r >= pstart) ? d.R[r + (long long)nG * c] : d.M[r + ld * c];
      b[r] = csub(b[r], cmul(rv, xc));
    }
    __syncthreads();
  }
  for (int r = threadIdx.x; r < nG; r += blockDim.x) {
    d.x[r] = xs[r];
    out[d.dxi_offset + r] = cmul(der, xs[r]);
  }
  __syncthreads();
  // tau(j1, j2) = sum_k conj(Sa0Sm1(j2*nmd+k, j1)) dxi(k, j2) + diagonal phase term
  const int n = d.n, nmd = d.nmd;
  for (int e = threadIdx.x; e < n * n; e += blockDim.x) {
    const int j1 = e % n, j2 = e / n;
    cplx t = mkc(0.0, 0.0);
    for (int k = 0; k < nmd; ++k) cfma_conj(t, d.Sa0Sm1[(j2 * nmd + k) + (long long)nG * j1], cmul(der, xs[k + nmd * j2]));
    if (j1 == j2) {
      double dd = 0.0;
      for (int k = 0; k < nmd; ++k) {
        const cplx dx = cmul(der, xs[k + nmd * j2]);
        dd += d.xi[k + nmd * j2].x * dx.x / d.a[k + d.lda * j2];
      }
      t.x += dd * 0.5;
    }
    d.tau[e] = t;
  }
}

// Tikhonov-regularised inverse of a Hermitian n x n matrix (n <= 32) as the
// least-squares solution of [A; eps I] X = [I; 0]: X = (A^2 + eps^2)^-1 A, the
// matrix StdRegInv 'tikh' (maths.f90:8-83) builds from the eigen-decomposition
// U w/(w^2 + eps^2) U^H.  Householder QR of the 2n x n stack in shared memory
// with the 2n x n right-hand side carried along, one warp per column.
__global__ void __launch_bounds__(256) tikh_inv_kernel(const RegInvDesc* __restrict__ descs) {
  extern __shared__ cplx smq[];
  const RegInvDesc& d = descs[blockIdx.x];
  const int n = d.n, m = 2 * n, ld = 2 * MAXN_SPF;
  cplx* A = smq;                       // m x n (ld)
  cplx* B = smq + (size_t)ld * MAXN_SPF;  // m x n (ld)
  __shared__ cplx s_alpha[MAXN_SPF];
  __shared__ double s_tau[MAXN_SPF];
  for (int e = threadIdx.x; e < m * n; e += blockDim.x) {
    const int i = e % m, j = e / m;
    cplx a, b;
    if (i < n) {
      // the upper triangle is authoritative (zheev 'U'): mirror it, real diagonal
      a = (i <= j) ? d.A[i + n * j] : cconj(d.A[j + n * i]);
      if (i == j) a.y = 0.0;
      b = mkc(i == j ? 1.0 : 0.0, 0.0);
    } else {
      a = mkc((i - n) == j ? d.eps : 0.0, 0.0);
      b = mkc(0.0, 0.0);
    }
    A[i + ld * j] = a;
    B[i + ld * j] = b;
  }
  __syncthreads();
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int nw = blockDim.x >> 5;
  for (int j = 0; j < n; ++j) {
    cplx* col = A + ld * j;
    if (warp == 0) {
      double part = 0.0;
      for (int r = j + lane; r < m; r += 32) part += cabs2(col[r]);
      for (int o = 16; o > 0; o >>= 1) part += __shfl_down_sync(0xffffffffu, part, o);
      if (lane == 0) {
        const double nrm = sqrt(part);
        const cplx x0 = col[j];
        const double ax0 = sqrt(cabs2(x0));
        if (nrm == 0.0) {
          s_alpha[j] = mkc(0.0, 0.0);
          s_tau[j] = 0.0;
        } else {
          const cplx ph = (ax0 > 0.0) ? mkc(x0.x / ax0, x0.y / ax0) : mkc(1.0, 0.0);
          const cplx alpha = cscale(ph, -nrm);
          col[j] = csub(x0, alpha);
          s_alpha[j] = alpha;
          s_tau[j] = 2.0 / (2.0 * part + 2.0 * nrm * ax0);
        }
      }
    }
    __syncthreads();
    const double tau = s_tau[j];
    if (tau != 0.0) {
      // columns j+1..n-1 of A, then all n columns of B
      for (int c = warp; c < (n - j - 1) + n; c += nw) {
        cplx* y = (c < n - j - 1) ? A + ld * (j + 1 + c) : B + ld * (c - (n - j - 1));
        cplx w = mkc(0.0, 0.0);
        for (int r = j + lane; r < m; r += 32) cfma_conj(w, col[r], y[r]);
        w = warp_sum(w);
        const cplx f = cscale(w, tau);
        for (int r = j + lane; r < m; r += 32) y[r] = csub(y[r], cmul(col[r], f));
      }
    }
    __syncthreads();
  }
  // back substitution R X = (Q^H [I; 0])[0:n], one thread per right-hand side
  for (int c = threadIdx.x; c < n; c += blockDim.x) {
    cplx* x = B + ld * c;
    for (int i = n - 1; i >= 0; --i) {
      cplx v = x[i];
      for (int k = i + 1; k < n; ++k) v = csub(v, cmul(A[i + ld * k], x[k]));
      x[i] = cdiv(v, s_alpha[i]);
    }
  }
  __syncthreads();
  for (int e = threadIdx.x; e < n * n; e += blockDim.x) {
    const int i = e % n, j = e / n;
    d.inv_out[i + n * j] = B[i + ld * j];
  }
}

}  // namespace

void launch_tikh_inv(const RegInvDesc* d, int nd, cudaStream_t st) {
  if (nd <= 0) return;
  const size_t smem = sizeof(cplx) * 2 * (size_t)(2 * MAXN_SPF) * MAXN_SPF;
  static bool configured = false;
  if (!configured) {
    cudaFuncSetAttribute(tikh_inv_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    configured = true;
  }
  tikh_inv_kernel<<<nd, 256, smem, st>>>(d);
}

// ---------------------------------------------------------------------------
// CMF2 with Gaussian modes
// ---------------------------------------------------------------------------
// D = S^-1/2 in the Cholesky form of InverseSquareRootU (maths.f90:621-644):
// S = U^H U (zpotrf 'U', column by column as the unblocked zpotf2), D = U^-1
// (ztrtri 'U','N', columns from the already inverted leading block as ztrti2),
// zeros below the diagonal; and DhS = D^H S, the matrix of A_to_B
// (cmf2_base.f90:288-292, B = (S D)^H A).  One block per (mode, set), n <= 32.
__global__ void __launch_bounds__(1024) gwp_isqrt_kernel(const GwpIsqrtDesc* __restrict__ descs, int* status) {
  const GwpIsqrtDesc& d = descs[blockIdx.x];
  const int n = d.n;
  __shared__ cplx U[MAXN_SPF][MAXN_SPF + 1];   // U[row][col]
  __shared__ cplx X[MAXN_SPF][MAXN_SPF + 1];   // U^-1
  __shared__ int bad;
  const int tid = threadIdx.x;
  if (tid == 0) bad = 0;
  for (int e = tid; e < MAXN_SPF * MAXN_SPF; e += blockDim.x) {
    const int r = e % MAXN_SPF, col = e / MAXN_SPF;
    U[r][col] = (r < n && col < n && r <= col) ? d.S[r + n * col] : mkc(0.0, 0.0);
    X[r][col] = mkc(0.0, 0.0);
  }
  __syncthreads();
  for (int j = 0; j < n; ++j) {
    if (tid < 32) {
      // U(j,j) = sqrt(S(j,j) - sum_{q<j} |U(q,j)|^2)
      double part = 0.0;
      for (int q = tid; q < j; q += 32) part += U[q][j].x * U[q][j].x + U[q][j].y * U[q][j].y;
      for (int off = 16; off > 0; off >>= 1) part += __shfl_down_sync(0xffffffffu, part, off);
      if (tid == 0) {
        const double ajj = U[j][j].x - part;
        if (!(ajj > 0.0)) bad = 1;
        U[j][j] = mkc(sqrt(fabs(ajj)), 0.0);
      }
    }
    __syncthreads();
    // row j right of the diagonal: (S(j,k) - sum_{q<j} conj(U(q,j)) U(q,k)) / U(j,j)
    const double rinv = 1.0 / U[j][j].x;
    for (int k = j + 1 + tid; k < n; k += blockDim.x) {
      cplx v = U[j][k];
      for (int q = 0; q < j; ++q) v = csub(v, cmul(cconj(U[q][j]), U[q][k]));
      U[j][k] = cscale(v, rinv);
    }
    __syncthreads();
  }
  for (int j = tid; j < n; j += blockDim.x) X[j][j] = mkc(1.0 / U[j][j].x, 0.0);
  __syncthreads();
  for (int j = 1; j < n; ++j) {
    // X(0:j-1, j) = -X(0:j-1, 0:j-1) U(0:j-1, j) X(j,j)
    for (int i = tid; i < j; i += blockDim.x) {
      cplx v = mkc(0.0, 0.0);
      for (int q = i; q < j; ++q) v = cadd(v, cmul(X[i][q], U[q][j]));
      X[i][j] = cscale(v, -X[j][j].x);
    }
    __syncthreads();
  }
  for (int e = tid; e < n * n; e += blockDim.x) {
    const int r = e % n, col = e / n;
    d.D[e] = X[r][col];
    // (D^H S)(r, col) = sum_q conj(D(q, r)) S(q, col), S Hermitian from its upper triangle
    cplx v = mkc(0.0, 0.0);
    for (int q = 0; q <= r; ++q) {
      const cplx sq = (q <= col) ? d.S[q + n * col] : cconj(d.S[col + n * q]);
      v = cadd(v, cmul(cconj(X[q][r]), sq));
    }
    d.DhS[e] = v;
  }
  if (tid == 0 && bad) atomicOr(status, DEVST_CHOL_FAIL);
}

// Calc_DHD (hamilton.f90:535-574): same state, 1/2 (D^H (h D) + (h D)^H D) with h
// Hermitian from its upper triangle (zhemm + zher2k), real diagonal; across
// states (D1^H h) D2.  Entries of modulus <= DBL_EPSILON become zero (the
// reference's clean-up, on the upper triangle for the Hermitian case, which is
// then mirrored into the full matrix the mode products use).
__global__ void __launch_bounds__(1024) gwp_dhd_kernel(const GwpDhdDesc* __restrict__ descs) {
  const GwpDhdDesc& d = descs[blockIdx.x];
  const int n1 = d.n1, n2 = d.n2;
  __shared__ cplx aux[MAXN_SPF][MAXN_SPF + 1];
  __shared__ cplx res[MAXN_SPF][MAXN_SPF + 1];
  const int tid = threadIdx.x;
  if (d.same_state) {
    for (int e = tid; e < n1 * n2; e += blockDim.x) {   // aux = h D
      const int a = e % n1, b = e / n1;
      cplx v = mkc(0.0, 0.0);
      for (int q = 0; q < n1; ++q) {
        const cplx hq = (a <= q) ? d.h[a + n1 * q] : cconj(d.h[q + n1 * a]);
        v = cadd(v, cmul(hq, d.D2[q + n2 * b]));
      }
      aux[a][b] = v;
    }
    __syncthreads();
    for (int e = tid; e < n1 * n2; e += blockDim.x) {
      const int a = e % n1, b = e / n1;
      if (a > b) continue;
      cplx v = mkc(0.0, 0.0);
      for (int q = 0; q < n1; ++q) {
        v = cadd(v, cmul(cconj(d.D1[q + n1 * a]), aux[q][b]));
        v = cadd(v, cmul(cconj(aux[q][a]), d.D1[q + n1 * b]));
      }
      v = cscale(v, 0.5);
      if (a == b) v.y = 0.0;
      if (!(sqrt(v.x * v.x + v.y * v.y) > DBL_EPSILON)) v = mkc(0.0, 0.0);
      res[a][b] = v;
    }
    __syncthreads();
    for (int e = tid; e < n1 * n2; e += blockDim.x) {
      const int a = e % n1, b = e / n1;
      d.out[e] = (a <= b) ? res[a][b] : cconj(res[b][a]);
    }
  } else {
    for (int e = tid; e < n1 * n2; e += blockDim.x) {   // aux = D1^H h
      const int a = e % n1, b = e / n1;
      cplx v = mkc(0.0, 0.0);
      for (int q = 0; q < n1; ++q) v = cadd(v, cmul(cconj(d.D1[q + n1 * a]), d.h[q + n1 * b]));
      aux[a][b] = v;
    }
    __syncthreads();
    for (int e = tid; e < n1 * n2; e += blockDim.x) {
      const int a = e % n1, b = e / n1;
      cplx v = mkc(0.0, 0.0);
      for (int q = 0; q < n2; ++q) v = cadd(v, cmul(aux[a][q], d.D2[q + n2 * b]));
      if (!(sqrt(v.x * v.x + v.y * v.y) > DBL_EPSILON)) v = mkc(0.0, 0.0);
      d.out[e] = v;
    }
  }
}

// dD = -tau D per (mode, set) block of the D vectors (cmf2_derivatives.f90:228)
__global__ void gwp_dderiv_kernel(const GwpDDerivDesc* __restrict__ descs, const cplx* __restrict__ Din,
                                  cplx* __restrict__ Dout) {
  const GwpDDerivDesc& d = descs[blockIdx.x];
  const int n = d.n;
  const cplx* D = Din + d.off;
  for (int e = threadIdx.x; e < n * n; e += blockDim.x) {
    const int a = e % n, b = e / n;
    cplx v = mkc(0.0, 0.0);
    for (int q = 0; q < n; ++q) v = cadd(v, cmul(d.tau[a + n * q], D[q + n * b]));
    Dout[d.off + e] = mkc(-v.x, -v.y);
  }
}

void launch_gwp_isqrt(const GwpIsqrtDesc* d, int nd, int* status, cudaStream_t st) {
  if (nd <= 0) return;
  gwp_isqrt_kernel<<<nd, 1024, 0, st>>>(d, status);
}
void launch_gwp_dhd(const GwpDhdDesc* d, int nd, cudaStream_t st) {
  if (nd <= 0) return;
  gwp_dhd_kernel<<<nd, 1024, 0, st>>>(d);
}
void launch_gwp_dderiv(const GwpDDerivDesc* d, int nd, const cplx* Din, cplx* Dout, cudaStream_t st) {
  if (nd <= 0) return;
  gwp_dderiv_kernel<<<nd, 256, 0, st>>>(d, Din, Dout);
}

// ---------------------------------------------------------------------------
// Calc_Density (output.f90:332-445)
// ---------------------------------------------------------------------------
// GauOvl1D (gmctdh_objects.f90:1476-1493): <g1|g2> of normalised 1D Gaussians
__device__ cplx gau_ovl_1d(double a1, double a2, cplx xi1, cplx xi2) {
  const cplx s = cadd(cconj(xi1), xi2);
  cplx c = mkc(xi1.x * xi1.x / a1 + xi2.x * xi2.x / a2, 0.0);
  c = csub(c, cdivr(cmul(s, s), a1 + a2));
  const double a12 = a1 + a2;
  return cscale(cexp_(cscale(c, 0.25)), sqrt(sqrt(4.0 * a1 * a2 / (a12 * a12))));
}

__device__ __forceinline__ cplx herm_el(const cplx* X, int n, int i, int j) {
  cplx v = (i <= j) ? X[i + n * j] : cconj(X[j + n * i]);
  if (i == j) v.y = 0.0;
  return v;
}

// Grid DOF: Y_j = sum_j' rho(j, j') phi_j' (rho Hermitian from its upper
// triangle), DM(kg1, kg2) = sum_r sum_j conj(phi_j(r, kg2)) Y_j(r, kg1) with r the
// other DOFs of the mode (MatricisePsi, hamilton.f90:664-699), density = Re DM(kg, kg),
// basis populations Re sum_ab T(kg, a) DM(a, b) T(kg, b).  One block.
__global__ void __launch_bounds__(256) density_grid_kernel(DensGridArgs a) {
  const int n = a.n, nG = a.nG, ll = a.ll, nl = a.nl;
  const long long G = (long long)ll * nG * nl;
  for (long long e = threadIdx.x; e < G * n; e += blockDim.x) {
    const long long g = e % G;
    const int j = (int)(e / G);
    cplx v = mkc(0.0, 0.0);
    for (int q = 0; q < n; ++q) v = cadd(v, cmul(herm_el(a.rho, n, j, q), a.phi[g + G * q]));
    a.Y[e] = v;
  }
  __syncthreads();
  for (int e = threadIdx.x; e < nG * nG; e += blockDim.x) {
    const int k1 = e % nG, k2 = e / nG;
    cplx v = mkc(0.0, 0.0);
    for (int j = 0; j < n; ++j)
      for (int ro = 0; ro < nl; ++ro)
        for (int ri = 0; ri < ll; ++ri) {
          const long long b = ri + (long long)ll * nG * ro + G * j;
          v = cadd(v, cmul(cconj(a.phi[b + (long long)ll * k2]), a.Y[b + (long long)ll * k1]));
        }
    a.DM[e] = v;
  }
  __syncthreads();
  for (int kg = threadIdx.x; kg < nG; kg += blockDim.x) {
    a.dens[kg] = a.DM[kg + nG * kg].x;
    if (a.trafo) {
      double p = 0.0;
      for (int q = 0; q < nG; ++q) {
        cplx v = mkc(0.0, 0.0);
        for (int b = 0; b < nG; ++b) v = cadd(v, cscale(a.DM[q + nG * b], a.trafo[kg + a.ldt * b]));
        p += a.trafo[kg + a.ldt * q] * v.x;
      }
      a.pop[kg] = p;
    }
  }
}

// Gaussian DOF k: density(x) = delta Re sum_{j1,j2} c(j1,j2) exp(x^2 (a1 + a2) + x (conj xi1 + xi2))
// with c = rho(j1,j2) (4/pi^2 a1 a2 exp(Re xi1^2/a1 + Re xi2^2/a2))^(1/4) times the 1D
// overlaps of the other DOFs (rho Hermitian from its upper triangle).  One block.
__global__ void __launch_bounds__(256) density_gwp_kernel(DensGwpArgs a) {
  __shared__ cplx cf[MAXN_SPF * MAXN_SPF];
  const int n = a.n, k = a.k;
  const double pi24 = 1.0 / (asin(1.0) * asin(1.0));
  for (int e = threadIdx.x; e < n * n; e += blockDim.x) {
    const int j1 = e % n, j2 = e / n;
    const double a1 = a.a[k + a.lda * j1], a2 = a.a[k + a.lda * j2];
    const cplx x1 = a.xi[k + a.nmd * j1], x2 = a.xi[k + a.nmd * j2];
    cplx c = cscale(herm_el(a.rho, n, j1, j2), pow(pi24 * a1 * a2 * exp(x1.x * x1.x / a1 + x2.x * x2.x / a2), 0.25));
    for (int q = 0; q < a.nmd; ++q) {
      if (q == k) continue;
      c = cmul(c, gau_ovl_1d(a.a[q + a.lda * j1], a.a[q + a.lda * j2], a.xi[q + a.nmd * j1], a.xi[q + a.nmd * j2]));
    }
    cf[e] = c;
  }
  __syncthreads();
  for (int kg = threadIdx.x; kg < a.nG; kg += blockDim.x) {
    const double x = a.x0 + a.delta * kg;
    double d = 0.0;
    for (int j2 = 0; j2 < n; ++j2)
      for (int j1 = 0; j1 < n; ++j1) {
        const double a12 = a.a[k + a.lda * j1] + a.a[k + a.lda * j2];
        const cplx xs = cadd(cconj(a.xi[k + a.nmd * j1]), a.xi[k + a.nmd * j2]);
        const cplx ex = cexp_(mkc(x * x * a12 + x * xs.x, x * xs.y));
        d += cmul(cf[j1 + n * j2], ex).x;
      }
    a.dens[kg] = d * a.delta;
  }
}

void launch_density_grid(const DensGridArgs& a, cudaStream_t st) { density_grid_kernel<<<1, 256, 0, st>>>(a); }
void launch_density_gwp(const DensGwpArgs& a, cudaStream_t st) { density_gwp_kernel<<<1, 256, 0, st>>>(a); }

void launch_gwp_ovl(const GwpOvlDesc* d, int nd, cudaStream_t st) {
  if (nd <= 0) return;
  gwp_ovl_kernel<<<nd, 256, 0, st>>>(d);
}

void launch_gwp_h1(const GwpH1Desc* d, int nd, cudaStream_t st) {
  if (nd <= 0) return;
  gwp_h1_kernel<<<nd, 256, 0, st>>>(d);
}

void launch_gwp_cy(const GwpCYDesc* d, int nd, int maxG, int maxn, int maxops, const GwpYOp* ops, cplx* part,
                   cudaStream_t st) {
  if (nd <= 0) return;
  const unsigned ne = (unsigned)((maxG * maxn + 255) / 256);
  gwp_sa0_kernel<<<dim3(ne, nd), 256, 0, st>>>(d);
  gwp_sa0sm1_kernel<<<dim3(ne, nd), 256, 0, st>>>(d);
  const unsigned nt = (unsigned)((maxG + 15) / 16);
  gwp_c_kernel<<<dim3(nt, nt, nd), dim3(16, 16), 0, st>>>(d);
  const long long part_ld = (long long)maxG * maxn * std::max(maxops, 1);
  const long long nthr = (long long)maxn * maxn * std::max(maxops, 1);
  gwp_y_part_kernel<<<dim3((unsigned)((nthr + 127) / 128), nd), 128, 0, st>>>(d, ops, part, part_ld, maxn);
  gwp_y_sum_kernel<<<dim3((maxG + 127) / 128, nd), 128, 0, st>>>(d, ops, part, part_ld, maxn);
}

void launch_gwp_solve(const GwpCYDesc* d, int nd, int maxG, cplx der, cplx* out, int* status, cudaStream_t st) {
  if (nd <= 0) return;
  const size_t smem = sizeof(cplx) * (size_t)(2 * maxG) * GWP_QR_PW;
  static size_t configured = 0;
  if (smem > 48 * 1024 && smem > configured) {
    cudaFuncSetAttribute(gwp_qr_panel_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    configured = smem;
  }
  // the trailing columns spread over at most one block per SM (every block
  // factors the panel itself, so more blocks than SMs would share an SM's FP64
  // pipe), at most eight per block
  static int nsm = 0;
  if (!nsm) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    if (nsm <= 0) nsm = 152;
  }
  for (int j0 = 0; j0 < maxG; j0 += GWP_QR_PW) {
    const int trailing = maxG + 1 - j0 - GWP_QR_PW;
    const int per_desc = std::max(1, nsm / nd);
    const int cpb = std::min(8, std::max(1, (trailing + per_desc - 1) / per_desc));
    const unsigned nblk = (unsigned)std::max(1, (trailing + cpb - 1) / cpb);
    gwp_qr_panel_kernel<<<dim3(nblk, nd), 256, smem, st>>>(d, j0, cpb);
  }
  gwp_backsub_kernel<<<nd, 256, sizeof(cplx) * 2 * maxG, st>>>(d, der, out, status);
}
