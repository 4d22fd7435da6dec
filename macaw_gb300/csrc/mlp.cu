// Multilayer perceptron of the learned mean-field extrapolator (BF16 weights and
// activations, FP32 accumulation), with hand-written forward, backward and Adam
// kernels.  Layout: row-major matrices; a layer maps X (M x K) to
// Y = act(X W^T + b) with W (N x K).
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <math.h>
#include <string.h>

#include <string>
#include <vector>

#include "../../include/macaw_gb300.h"
#include "kernels.cuh"

void mctdh_set_global_error(const char* msg);

namespace {

#define GT 64       // output tile (rows and columns) of the GEMM kernels
#define GK 16       // reduction slice staged in shared memory

// C (M x N) = A (M x K) * B^T (B: N x K), FP32 accumulation; A and B are BF16 or
// FP32 (template).  Epilogue: + bias, optional tanh, store FP32 and/or BF16.
template <typename TA, typename TB>
__global__ void __launch_bounds__(256) gemm_nt_kernel(const TA* __restrict__ A, const TB* __restrict__ B,
                                                      const float* __restrict__ bias, float* C32,
                                                      __nv_bfloat16* C16, int M, int N, int K, int act) {
  __shared__ float As[GK][GT + 1];
  __shared__ float Bs[GK][GT + 1];
  const int tx = threadIdx.x % 16, ty = threadIdx.x / 16;
  const int row0 = blockIdx.y * GT, col0 = blockIdx.x * GT;
  float acc[4][4] = {};
  for (int k0 = 0; k0 < K; k0 += GK) {
    for (int e = threadIdx.x; e < GK * GT; e += 256) {
      const int kk = e % GK, rr = e / GK;
      const int r = row0 + rr, k = k0 + kk;
      As[kk][rr] = (r < M && k < K) ? (float)A[(long long)r * K + k] : 0.f;
      const int cidx = col0 + rr;
      Bs[kk][rr] = (cidx < N && k < K) ? (float)B[(long long)cidx * K + k] : 0.f;
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < GK; ++kk) {
      float a[4], b[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) a[i] = As[kk][ty + 16 * i];
#pragma unroll
      for (int j = 0; j < 4; ++j) b[j] = Bs[kk][tx + 16 * j];
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] = fmaf(a[i], b[j], acc[i][j]);
    }
    __syncthreads();
  }
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const int r = row0 + ty + 16 * i;
    if (r >= M) continue;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int cidx = col0 + tx + 16 * j;
      if (cidx >= N) continue;
      float v = acc[i][j] + (bias ? bias[cidx] : 0.f);
      if (act) v = tanhf(v);
      if (C32) C32[(long long)r * N + cidx] = v;
      if (C16) C16[(long long)r * N + cidx] = __float2bfloat16(v);
    }
  }
}

// C (M x N) = A (M x K) * B (K x N), FP32 accumulation (for dX = dY W).
template <typename TA, typename TB>
__global__ void __launch_bounds__(256) gemm_nn_kernel(const TA* __restrict__ A, const TB* __restrict__ B,
                                                      float* __restrict__ C, int M, int N, int K) {
  __shared__ float As[GK][GT + 1];
  __shared__ float Bs[GK][GT + 1];
  const int tx = threadIdx.x % 16, ty = threadIdx.x / 16;
  const int row0 = blockIdx.y * GT, col0 = blockIdx.x * GT;
  float acc[4][4] = {};
  for (int k0 = 0; k0 < K; k0 += GK) {
    for (int e = threadIdx.x; e < GK * GT; e += 256) {
      const int kk = e % GK, rr = e / GK;
      const int r = row0 + rr, k = k0 + kk;
      As[kk][rr] = (r < M && k < K) ? (float)A[(long long)r * K + k] : 0.f;
      const int cc = e % GT, kb = e / GT;
      const int cidx = col0 + cc, k2 = k0 + kb;
      Bs[kb][cc] = (cidx < N && k2 < K) ? (float)B[(long long)k2 * N + cidx] : 0.f;
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < GK; ++kk) {
      float a[4], b[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) a[i] = As[kk][ty + 16 * i];
#pragma unroll
      for (int j = 0; j < 4; ++j) b[j] = Bs[kk][tx + 16 * j];
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] = fmaf(a[i], b[j], acc[i][j]);
    }
    __syncthreads();
  }
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const int r = row0 + ty + 16 * i;
    if (r >= M) continue;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int cidx = col0 + tx + 16 * j;
      if (cidx < N) C[(long long)r * N + cidx] = acc[i][j];
    }
  }
}

// dW (N x K) = dY^T (N x M) * X (M x K) and db = sum_m dY: reduction over the
// batch in fixed-order M slices per block, FP32.
template <typename TX>
__global__ void __launch_bounds__(256) grad_w_kernel(const float* __restrict__ dY, const TX* __restrict__ X,
                                                     float* __restrict__ dW, float* __restrict__ db, int M, int N,
                                                     int K) {
  __shared__ float Ds[GK][GT + 1];
  __shared__ float Xs[GK][GT + 1];
  const int tx = threadIdx.x % 16, ty = threadIdx.x / 16;
  const int n0 = blockIdx.y * GT, k0 = blockIdx.x * GT;
  float acc[4][4] = {};
  float bacc[4] = {};
  for (int m0 = 0; m0 < M; m0 += GK) {
    for (int e = threadIdx.x; e < GK * GT; e += 256) {
      const int mm = e / GT, cc = e % GT;
      const int m = m0 + mm;
      Ds[mm][cc] = (m < M && n0 + cc < N) ? dY[(long long)m * N + n0 + cc] : 0.f;
      Xs[mm][cc] = (m < M && k0 + cc < K) ? (float)X[(long long)m * K + k0 + cc] : 0.f;
    }
    __syncthreads();
#pragma unroll
    for (int mm = 0; mm < GK; ++mm) {
      float a[4], b[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) a[i] = Ds[mm][ty + 16 * i];
#pragma unroll
      for (int j = 0; j < 4; ++j) b[j] = Xs[mm][tx + 16 * j];
#pragma unroll
      for (int i = 0; i < 4; ++i) {
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] = fmaf(a[i], b[j], acc[i][j]);
        if (blockIdx.x == 0 && tx == 0) bacc[i] += a[i];
      }
    }
    __syncthreads();
  }
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const int n = n0 + ty + 16 * i;
    if (n >= N) continue;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int k = k0 + tx + 16 * j;
      if (k < K) dW[(long long)n * K + k] = acc[i][j];
    }
    if (blockIdx.x == 0 && tx == 0) db[n] = bacc[i];
  }
}

// dZ = dH * (1 - H^2) (tanh), in place on the FP32 gradient
__global__ void tanh_back_kernel(float* dH, const __nv_bfloat16* H, long long n) {
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float h = __bfloat162float(H[i]);
  dH[i] *= (1.f - h * h);
}

// dY = 2 (Y - T) / (M * Dout); per-block partial sums of the squared error
__global__ void mse_kernel(const float* Y, const float* T, float* dY, double* part, long long n, float scale) {
  __shared__ double red[256];
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  double e2 = 0.0;
  if (i < n) {
    const float d = Y[i] - T[i];
    dY[i] = 2.f * d * scale;
    e2 = (double)d * d;
  }
  red[threadIdx.x] = e2;
  __syncthreads();
  for (int s = 128; s > 0; s >>= 1) {
    if (threadIdx.x < s) red[threadIdx.x] += red[threadIdx.x + s];
    __syncthreads();
  }
  if (threadIdx.x == 0) part[blockIdx.x] = red[0];
}

__global__ void adam_kernel(float* w, __nv_bfloat16* w16, const float* g, float* m1, float* m2, long long n, float lr,
                            float b1, float b2, float c1, float c2, float eps) {
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float gi = g[i];
  const float a = b1 * m1[i] + (1.f - b1) * gi;
  const float b = b2 * m2[i] + (1.f - b2) * gi * gi;
  m1[i] = a;
  m2[i] = b;
  const float v = w[i] - lr * (a / c1) / (sqrtf(b / c2) + eps);
  w[i] = v;
  if (w16) w16[i] = __float2bfloat16(v);
}

__global__ void to_bf16_kernel(const float* in, __nv_bfloat16* out, long long n) {
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] = __float2bfloat16(in[i]);
}

struct Layer {
  int K, N, act;
  float* W = nullptr;          // FP32 master (N x K)
  __nv_bfloat16* W16 = nullptr;
  float* b = nullptr;
  float *gW = nullptr, *gb = nullptr;
  float *mW = nullptr, *vW = nullptr, *mb = nullptr, *vb = nullptr;
};

#define MLP_CK(call)                                                                 \
  do {                                                                               \
    cudaError_t e_ = (call);                                                         \
    if (e_ != cudaSuccess) throw std::string(#call) + ": " + cudaGetErrorString(e_); \
  } while (0)

}  // namespace

struct mctdh_mlp {
  std::vector<Layer> L;
  cudaStream_t st = nullptr;
  long long cap = 0;             // rows the activation buffers hold
  float* X = nullptr;            // input (cap x Din), FP32
  float* T = nullptr;            // targets (cap x Dout)
  std::vector<__nv_bfloat16*> H; // activations (BF16) per hidden layer
  float* Y = nullptr;            // output (cap x Dout)
  float* dA = nullptr;           // gradient buffer (cap x 256)
  float* dB = nullptr;
  double* part = nullptr;
  long long step = 0;
  std::vector<void*> allocs;
  std::string err;
  void* alloc(size_t bytes) {
    void* p = nullptr;
    MLP_CK(cudaMalloc(&p, bytes));
    MLP_CK(cudaMemset(p, 0, bytes));
    allocs.push_back(p);
    return p;
  }
  void ensure(long long rows) {
    if (rows <= cap) return;
    const long long r = std::max(rows, 1024LL);
    X = (float*)alloc(sizeof(float) * r * L[0].K);
    T = (float*)alloc(sizeof(float) * r * L.back().N);
    Y = (float*)alloc(sizeof(float) * r * L.back().N);
    H.clear();
    int wmax = 0;
    for (size_t i = 0; i < L.size(); ++i) {
      wmax = std::max(wmax, std::max(L[i].N, L[i].K));
      if (i + 1 < L.size()) H.push_back((__nv_bfloat16*)alloc(sizeof(__nv_bfloat16) * r * L[i].N));
    }
    dA = (float*)alloc(sizeof(float) * r * wmax);
    dB = (float*)alloc(sizeof(float) * r * wmax);
    part = (double*)alloc(sizeof(double) * (r * L.back().N / 256 + 2));
    cap = r;
  }
  void forward(long long M) { forward_on(M, st); }
  void forward_on(long long M, cudaStream_t st) {
    const int nl = (int)L.size();
    for (int i = 0; i < nl; ++i) {
      dim3 grid((L[i].N + GT - 1) / GT, (unsigned)((M + GT - 1) / GT));
      const bool last = (i == nl - 1);
      if (i == 0)
        gemm_nt_kernel<float, __nv_bfloat16><<<grid, 256, 0, st>>>(X, L[i].W16, L[i].b, last ? Y : nullptr,
                                                                    last ? nullptr : H[i], (int)M, L[i].N, L[i].K,
                                                                    L[i].act);
      else
        gemm_nt_kernel<__nv_bfloat16, __nv_bfloat16><<<grid, 256, 0, st>>>(
            H[i - 1], L[i].W16, L[i].b, last ? Y : nullptr, last ? nullptr : H[i], (int)M, L[i].N, L[i].K,
            L[i].act);
    }
  }
  double backward(long long M) {
    const int nl = (int)L.size();
    const long long n = M * L.back().N;
    const int nb = (int)((n + 255) / 256);
    mse_kernel<<<nb, 256, 0, st>>>(Y, T, dA, part, n, 1.f / (float)n);
    float* g = dA;
    float* o = dB;
    for (int i = nl - 1; i >= 0; --i) {
      dim3 gw((L[i].K + GT - 1) / GT, (L[i].N + GT - 1) / GT);
      if (i == 0)
        grad_w_kernel<float><<<gw, 256, 0, st>>>(g, X, L[i].gW, L[i].gb, (int)M, L[i].N, L[i].K);
      else
        grad_w_kernel<__nv_bfloat16><<<gw, 256, 0, st>>>(g, H[i - 1], L[i].gW, L[i].gb, (int)M, L[i].N, L[i].K);
      if (i == 0) break;
      dim3 gx((L[i].K + GT - 1) / GT, (unsigned)((M + GT - 1) / GT));
      gemm_nn_kernel<float, __nv_bfloat16><<<gx, 256, 0, st>>>(g, L[i].W16, o, (int)M, L[i].K, L[i].N);
      const long long nh = M * L[i].K;
      tanh_back_kernel<<<(unsigned)((nh + 255) / 256), 256, 0, st>>>(o, H[i - 1], nh);
      std::swap(g, o);
    }
    std::vector<double> hp(nb);
    MLP_CK(cudaMemcpyAsync(hp.data(), part, sizeof(double) * nb, cudaMemcpyDeviceToHost, st));
    MLP_CK(cudaStreamSynchronize(st));
    double s = 0;
    for (double v : hp) s += v;
    return s / (double)n;
  }
  void adam(float lr) {
    ++step;
    const float b1 = 0.9f, b2 = 0.999f;
    const float c1 = 1.f - powf(b1, (float)step), c2 = 1.f - powf(b2, (float)step);
    for (auto& l : L) {
      const long long nw = (long long)l.N * l.K;
      adam_kernel<<<(unsigned)((nw + 255) / 256), 256, 0, st>>>(l.W, l.W16, l.gW, l.mW, l.vW, nw, lr, b1, b2, c1,
                                                                 c2, 1e-8f);
      adam_kernel<<<(unsigned)((l.N + 255) / 256), 256, 0, st>>>(l.b, nullptr, l.gb, l.mb, l.vb, l.N, lr, b1, b2,
                                                                  c1, c2, 1e-8f);
    }
  }
  long long nparams() const {
    long long n = 0;
    for (auto& l : L) n += (long long)l.N * l.K + l.N;
    return n;
  }
  ~mctdh_mlp() {
    if (st) cudaStreamSynchronize(st);
    for (void* p : allocs) cudaFree(p);
    if (st) cudaStreamDestroy(st);
  }
};

namespace {

template <typename F>
int64_t mlp_guard(mctdh_mlp_t* m, F&& fn) {
  try {
    fn();
    return MCTDH_OK;
  } catch (const std::string& e) {
    if (m) m->err = e;
    mctdh_set_global_error(e.c_str());
    return MCTDH_ECUDA;
  }
}

// weights of layer l in the flat parameter vector: W (N x K, row-major) then b (N)
void set_params_host(mctdh_mlp_t* m, const float* p) {
  long long off = 0;
  for (auto& l : m->L) {
    const long long nw = (long long)l.N * l.K;
    MLP_CK(cudaMemcpy(l.W, p + off, sizeof(float) * nw, cudaMemcpyHostToDevice));
    to_bf16_kernel<<<(unsigned)((nw + 255) / 256), 256>>>(l.W, l.W16, nw);
    off += nw;
    MLP_CK(cudaMemcpy(l.b, p + off, sizeof(float) * l.N, cudaMemcpyHostToDevice));
    off += l.N;
  }
  MLP_CK(cudaDeviceSynchronize());
}

}  // namespace

extern "C" {

int64_t mctdh_mlp_create(const int64_t* widths, int64_t nlayers, uint64_t seed, mctdh_mlp_t** out) {
  if (!widths || !out || nlayers < 1 || nlayers > 16) return MCTDH_EARG;
  *out = nullptr;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
    mctdh_set_global_error("no CUDA device available (this core has no CPU fallback)");
    return MCTDH_ECUDA;
  }
  mctdh_mlp_t* m = new mctdh_mlp_t();
  int64_t rc = mlp_guard(m, [&] {
    MLP_CK(cudaStreamCreateWithFlags(&m->st, cudaStreamNonBlocking));
    for (int64_t i = 0; i < nlayers; ++i) {
      Layer l;
      l.K = (int)widths[i];
      l.N = (int)widths[i + 1];
      l.act = (i + 1 < nlayers) ? 1 : 0;
      const long long nw = (long long)l.N * l.K;
      l.W = (float*)m->alloc(sizeof(float) * nw);
      l.W16 = (__nv_bfloat16*)m->alloc(sizeof(__nv_bfloat16) * nw);
      l.b = (float*)m->alloc(sizeof(float) * l.N);
      l.gW = (float*)m->alloc(sizeof(float) * nw);
      l.gb = (float*)m->alloc(sizeof(float) * l.N);
      l.mW = (float*)m->alloc(sizeof(float) * nw);
      l.vW = (float*)m->alloc(sizeof(float) * nw);
      l.mb = (float*)m->alloc(sizeof(float) * l.N);
      l.vb = (float*)m->alloc(sizeof(float) * l.N);
      m->L.push_back(l);
    }
    // Glorot-uniform initialisation from a 64-bit LCG on the host
    std::vector<float> p((size_t)m->nparams());
    uint64_t s = seed * 6364136223846793005ULL + 1442695040888963407ULL;
    long long off = 0;
    for (auto& l : m->L) {
      const float lim = sqrtf(6.f / (float)(l.K + l.N));
      for (long long i = 0; i < (long long)l.N * l.K; ++i) {
        s = s * 6364136223846793005ULL + 1442695040888963407ULL;
        const float u = (float)((s >> 11) * (1.0 / 9007199254740992.0));
        p[off++] = (2.f * u - 1.f) * lim;
      }
      for (int i = 0; i < l.N; ++i) p[off++] = 0.f;
    }
    set_params_host(m, p.data());
  });
  if (rc != MCTDH_OK) {
    delete m;
    return rc;
  }
  *out = m;
  return MCTDH_OK;
}

int64_t mctdh_mlp_destroy(mctdh_mlp_t* m) {
  if (!m) return MCTDH_EARG;
  delete m;
  return MCTDH_OK;
}

int64_t mctdh_mlp_nparams(mctdh_mlp_t* m, int64_t* n) {
  if (!m || !n) return MCTDH_EARG;
  *n = m->nparams();
  return MCTDH_OK;
}

int64_t mctdh_mlp_set_params(mctdh_mlp_t* m, const float* p) {
  if (!m || !p) return MCTDH_EARG;
  return mlp_guard(m, [&] { set_params_host(m, p); });
}

int64_t mctdh_mlp_get_params(mctdh_mlp_t* m, float* p) {
  if (!m || !p) return MCTDH_EARG;
  return mlp_guard(m, [&] {
    long long off = 0;
    for (auto& l : m->L) {
      MLP_CK(cudaMemcpy(p + off, l.W, sizeof(float) * l.N * l.K, cudaMemcpyDeviceToHost));
      off += (long long)l.N * l.K;
      MLP_CK(cudaMemcpy(p + off, l.b, sizeof(float) * l.N, cudaMemcpyDeviceToHost));
      off += l.N;
    }
  });
}

int64_t mctdh_mlp_predict(mctdh_mlp_t* m, const float* X, float* Y, int64_t M) {
  if (!m || !X || !Y || M < 1) return MCTDH_EARG;
  return mlp_guard(m, [&] {
    m->ensure(M);
    MLP_CK(cudaMemcpyAsync(m->X, X, sizeof(float) * M * m->L[0].K, cudaMemcpyHostToDevice, m->st));
    m->forward(M);
    MLP_CK(cudaMemcpyAsync(Y, m->Y, sizeof(float) * M * m->L.back().N, cudaMemcpyDeviceToHost, m->st));
    MLP_CK(cudaStreamSynchronize(m->st));
  });
}

// Loss and gradient of the mean squared error on one batch (no update).
int64_t mctdh_mlp_grad(mctdh_mlp_t* m, const float* X, const float* T, int64_t M, float* grad, double* loss) {
  if (!m || !X || !T || !grad || !loss || M < 1) return MCTDH_EARG;
  return mlp_guard(m, [&] {
    m->ensure(M);
    MLP_CK(cudaMemcpyAsync(m->X, X, sizeof(float) * M * m->L[0].K, cudaMemcpyHostToDevice, m->st));
    MLP_CK(cudaMemcpyAsync(m->T, T, sizeof(float) * M * m->L.back().N, cudaMemcpyHostToDevice, m->st));
    m->forward(M);
    *loss = m->backward(M);
    long long off = 0;
    for (auto& l : m->L) {
      MLP_CK(cudaMemcpy(grad + off, l.gW, sizeof(float) * l.N * l.K, cudaMemcpyDeviceToHost));
      off += (long long)l.N * l.K;
      MLP_CK(cudaMemcpy(grad + off, l.gb, sizeof(float) * l.N, cudaMemcpyDeviceToHost));
      off += l.N;
    }
  });
}

// Adam training over the data set: epochs x ceil(M / batch) updates on
// consecutive batches.  Returns the mean loss of the last epoch.
int64_t mctdh_mlp_train(mctdh_mlp_t* m, const float* X, const float* T, int64_t M, int64_t batch, int64_t epochs,
                        double lr, double* loss) {
  if (!m || !X || !T || M < 1 || batch < 1 || epochs < 1) return MCTDH_EARG;
  return mlp_guard(m, [&] {
    const int din = m->L[0].K, dout = m->L.back().N;
    m->ensure(batch);
    double last = 0.0;
    for (int64_t ep = 0; ep < epochs; ++ep) {
      double acc = 0.0;
      int64_t nb = 0;
      for (int64_t s = 0; s < M; s += batch) {
        const int64_t b = std::min(batch, M - s);
        MLP_CK(cudaMemcpyAsync(m->X, X + s * din, sizeof(float) * b * din, cudaMemcpyHostToDevice, m->st));
        MLP_CK(cudaMemcpyAsync(m->T, T + s * dout, sizeof(float) * b * dout, cudaMemcpyHostToDevice, m->st));
        m->forward(b);
        acc += m->backward(b);
        ++nb;
        m->adam((float)lr);
      }
      last = acc / (double)nb;
    }
    MLP_CK(cudaStreamSynchronize(m->st));
    if (loss) *loss = last;
  });
}

}  // extern "C"

float* mlp_input_buffer(mctdh_mlp* m, long long M) {
  m->ensure(M);
  return m->X;
}

const float* mlp_forward_on(mctdh_mlp* m, long long M, cudaStream_t st) {
  m->forward_on(M, st);
  return m->Y;
}

bool mlp_has_shape(const mctdh_mlp* m, int din, int dout) {
  return !m->L.empty() && m->L[0].K == din && m->L.back().N == dout;
}
