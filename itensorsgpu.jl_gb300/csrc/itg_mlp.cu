// Learned Davidson preconditioner: a per-element MLP with hand-written
// forward, backward and Adam kernels.
//
// Network (F inputs, width 128, BF16 weights, FP32 accumulation):
//   z1 = W1 x + b1, a1 = relu(z1)        W1: 128 x F
//   z2 = W2 a1 + b2, a2 = relu(z2)       W2: 128 x 128
//   g  = w3 . a2 + b3                    w3: 128
// Davidson uses it as a correction of the diagonal preconditioner: with
// m_e = r_e / (diag_e - theta) (normalised, clipped), the correction is
// t_e = (1 + g(features_e)) m_e, so g = 0 (the initial output layer) is the
// diagonal preconditioner.  Training minimises
//   loss = mean_e (g_e * m_e - y_e)^2
// with m the (scaled) diagonal correction and y the part of the ideal
// correction it misses, on samples that the plain solver generates.
//
// Master weights are FP32; the forward and backward passes read a BF16 copy
// (rounded to nearest even) and accumulate in FP32.  Per-CTA partial weight
// gradients are reduced in a fixed order, so gradients are deterministic.
#include "itg_internal.cuh"

#include <cuda_bf16.h>

#include <cmath>
#include <vector>

namespace {

constexpr int MW = 128;        // width
constexpr int MAXF = 8;        // max input features
constexpr int EPB = 64;        // elements per CTA
constexpr int MTHREADS = 256;

struct Mlp {
  int F = 0;
  int64_t nparam = 0;
  float* master = nullptr;     // FP32 parameters
  __nv_bfloat16* w16 = nullptr; // BF16 copy
  float* m = nullptr;          // Adam first moment
  float* v = nullptr;          // Adam second moment
  float* grad = nullptr;       // reduced gradient
  float* partial = nullptr;    // per-CTA gradient partials
  int64_t partial_ctas = 0;
  float* loss_part = nullptr;
  int64_t step = 0;
};

// parameter layout offsets
__host__ __device__ inline int64_t oW1(int) { return 0; }
__host__ __device__ inline int64_t ob1(int F) { return (int64_t)MW * F; }
__host__ __device__ inline int64_t oW2(int F) { return ob1(F) + MW; }
__host__ __device__ inline int64_t ob2(int F) { return oW2(F) + (int64_t)MW * MW; }
__host__ __device__ inline int64_t ow3(int F) { return ob2(F) + MW; }
__host__ __device__ inline int64_t ob3(int F) { return ow3(F) + MW; }
__host__ __device__ inline int64_t nparams(int F) { return ob3(F) + 1; }

__global__ void k_to_bf16(const float* __restrict__ x, int64_t n, __nv_bfloat16* __restrict__ y) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    y[i] = __float2bfloat16_rn(x[i]);
}

// Shared memory of the fused forward/backward kernel (floats):
//   W2 [128 x 128] | a1 [128 x EPB] | z2 [128 x EPB] | W1 [128 x F] | b1 b2 w3 [128 each] | x [EPB x F] | g [EPB]
constexpr size_t mlp_smem_floats(int F) {
  return (size_t)MW * MW + 2 * (size_t)MW * EPB + (size_t)MW * F + 3 * MW + (size_t)EPB * F + EPB + 8;
}

// Persistent over element chunks: each CTA stages the weights once and walks
// chunks blockIdx.x, blockIdx.x + gridDim.x, ...
// mode 0: forward only (write g).  mode 1: forward + backward: the CTA's
// gradient partial (accumulated over its chunks, each entry owned by one
// thread, so the sum order is fixed) and its loss partial.
__global__ void __launch_bounds__(MTHREADS)
k_mlp_fused(const __nv_bfloat16* __restrict__ w16, const float* __restrict__ master, int F, int64_t n,
            const float* __restrict__ X, const float* __restrict__ mult, const float* __restrict__ target,
            float* __restrict__ g_out, int mode, float inv_n, float* __restrict__ partial,
            float* __restrict__ loss_part) {
  extern __shared__ float sm[];
  float* W2 = sm;
  float* A1 = W2 + MW * MW;       // [h][e]
  float* Z2 = A1 + MW * EPB;      // [h][e]
  float* W1 = Z2 + MW * EPB;      // [h][f]
  float* b1 = W1 + MW * F;
  float* b2 = b1 + MW;
  float* w3 = b2 + MW;
  float* xs = w3 + MW;            // [e][f]
  float* gs = xs + EPB * F;       // [e]
  __shared__ float red[MTHREADS / 32];
  const int t = threadIdx.x;
  for (int i = t; i < MW * MW; i += MTHREADS) W2[i] = __bfloat162float(w16[oW2(F) + i]);
  for (int i = t; i < MW * F; i += MTHREADS) W1[i] = __bfloat162float(w16[oW1(F) + i]);
  for (int i = t; i < MW; i += MTHREADS) {
    b1[i] = master[ob1(F) + i];
    b2[i] = master[ob2(F) + i];
    w3[i] = __bfloat162float(w16[ow3(F) + i]);
  }
  const float b3 = master[ob3(F)];
  const int64_t nchunks = (n + EPB - 1) / EPB;
  float* P = (mode == 1) ? partial + (int64_t)blockIdx.x * nparams(F) : nullptr;
  for (int64_t chunk = blockIdx.x; chunk < nchunks; chunk += gridDim.x) {
    const int64_t e0 = chunk * EPB;
    const bool first = chunk == (int64_t)blockIdx.x;
    for (int i = t; i < EPB * F; i += MTHREADS) {
      const int64_t e = e0 + i / F;
      xs[i] = (e < n) ? X[e0 * F + i] : 0.f;
    }
    __syncthreads();
    // layer 1: A1[h][e] = relu(W1[h] . x[e] + b1[h])
    for (int i = t; i < MW * EPB; i += MTHREADS) {
      const int hh = i / EPB, e = i % EPB;
      float z = b1[hh];
      for (int f = 0; f < F; ++f) z = fmaf(W1[hh * F + f], xs[e * F + f], z);
      A1[hh * EPB + e] = z > 0.f ? z : 0.f;
    }
    __syncthreads();
    // layer 2: Z2[h][e] = W2[h] . A1[:, e] + b2[h]; 16 x 16 threads, each 8 h x 4 e
    {
      const int th = t / 16, te = t % 16;
      float acc[8][4];
#pragma unroll
      for (int a = 0; a < 8; ++a)
#pragma unroll
        for (int b = 0; b < 4; ++b) acc[a][b] = 0.f;
      for (int k = 0; k < MW; ++k) {
        float wv[8], av[4];
#pragma unroll
        for (int a = 0; a < 8; ++a) wv[a] = W2[(th * 8 + a) * MW + k];
#pragma unroll
        for (int b = 0; b < 4; ++b) av[b] = A1[k * EPB + te * 4 + b];
#pragma unroll
        for (int a = 0; a < 8; ++a)
#pragma unroll
          for (int b = 0; b < 4; ++b) acc[a][b] = fmaf(wv[a], av[b], acc[a][b]);
      }
#pragma unroll
      for (int a = 0; a < 8; ++a)
#pragma unroll
        for (int b = 0; b < 4; ++b) Z2[(th * 8 + a) * EPB + te * 4 + b] = acc[a][b] + b2[th * 8 + a];
    }
    __syncthreads();
    // output: g[e] = w3 . relu(Z2[:, e]) + b3   (one warp per 8 elements)
    {
      const int warp = t >> 5, lane = t & 31;
      for (int e = warp; e < EPB; e += MTHREADS / 32) {
        float s = 0.f;
        for (int hh = lane; hh < MW; hh += 32) {
          const float z = Z2[hh * EPB + e];
          s = fmaf(w3[hh], z > 0.f ? z : 0.f, s);
        }
        for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
        if (lane == 0) gs[e] = s + b3;
      }
    }
    __syncthreads();
    if (mode == 0) {
      for (int e = t; e < EPB; e += MTHREADS)
        if (e0 + e < n) g_out[e0 + e] = gs[e];
      __syncthreads();
      continue;
    }
    // -------------------------------------------------------------- backward
    // dg[e] = 2 (g m - y) m / n ; loss partial
    float lsum = 0.f;
    for (int e = t; e < EPB; e += MTHREADS) {
      float dg = 0.f;
      if (e0 + e < n) {
        const float mm = mult[e0 + e];
        const float diff = gs[e] * mm - target[e0 + e];
        lsum += diff * diff;
        dg = 2.f * diff * mm * inv_n;
      }
      gs[e] = dg;  // gs now holds dL/dg
    }
    for (int o = 16; o > 0; o >>= 1) lsum += __shfl_xor_sync(0xffffffffu, lsum, o);
    if ((t & 31) == 0) red[t >> 5] = lsum;
    __syncthreads();
    if (t == 0) {
      float s = 0.f;
      for (int i = 0; i < MTHREADS / 32; ++i) s += red[i];
      loss_part[blockIdx.x] = first ? s : loss_part[blockIdx.x] + s;
      float db3 = 0.f;
      for (int e = 0; e < EPB; ++e) db3 += gs[e];
      P[ob3(F)] = first ? db3 : P[ob3(F)] + db3;
    }
    // dw3[h] = sum_e dg[e] relu(Z2[h][e]);  dZ2[h][e] = dg[e] w3[h] [Z2 > 0] (in place in Z2)
    for (int hh = t; hh < MW; hh += MTHREADS) {
      float s = 0.f;
      for (int e = 0; e < EPB; ++e) {
        const float z = Z2[hh * EPB + e];
        s = fmaf(gs[e], z > 0.f ? z : 0.f, s);
      }
      P[ow3(F) + hh] = first ? s : P[ow3(F) + hh] + s;
    }
    __syncthreads();
    for (int i = t; i < MW * EPB; i += MTHREADS) {
      const int hh = i / EPB, e = i % EPB;
      const float z = Z2[i];
      Z2[i] = z > 0.f ? gs[e] * w3[hh] : 0.f;
    }
    __syncthreads();
    // db2[h] = sum_e dZ2 ; dW2[h][k] = sum_e dZ2[h][e] A1[k][e]
    for (int hh = t; hh < MW; hh += MTHREADS) {
      float s = 0.f;
      for (int e = 0; e < EPB; ++e) s += Z2[hh * EPB + e];
      P[ob2(F) + hh] = first ? s : P[ob2(F) + hh] + s;
    }
    for (int i = t; i < MW * MW; i += MTHREADS) {
      const int hh = i / MW, k = i % MW;
      float s = 0.f;
      for (int e = 0; e < EPB; ++e) s = fmaf(Z2[hh * EPB + e], A1[k * EPB + e], s);
      P[oW2(F) + i] = first ? s : P[oW2(F) + i] + s;
    }
    __syncthreads();
    // dA1[k][e] = sum_h W2[h][k] dZ2[h][e]; dZ1 = dA1 [A1 > 0], stored in place of A1
    for (int i = t; i < MW * EPB; i += MTHREADS) {
      const int k = i / EPB, e = i % EPB;
      float s = 0.f;
      for (int hh = 0; hh < MW; ++hh) s = fmaf(W2[hh * MW + k], Z2[hh * EPB + e], s);
      // relu mask: A1 > 0 exactly where z1 > 0; each (k, e) is read and
      // rewritten only by this thread, and dW2 already consumed A1 above
      A1[i] = (A1[i] > 0.f) ? s : 0.f;
    }
    __syncthreads();
    // db1[h] = sum_e dZ1[h][e]; dW1[h][f] = sum_e dZ1[h][e] x[e][f]
    for (int hh = t; hh < MW; hh += MTHREADS) {
      float s = 0.f;
      for (int e = 0; e < EPB; ++e) s += A1[hh * EPB + e];
      P[ob1(F) + hh] = first ? s : P[ob1(F) + hh] + s;
    }
    for (int i = t; i < MW * F; i += MTHREADS) {
      const int hh = i / F, f = i % F;
      float s = 0.f;
      for (int e = 0; e < EPB; ++e) s = fmaf(A1[hh * EPB + e], xs[e * F + f], s);
      P[oW1(F) + i] = first ? s : P[oW1(F) + i] + s;
    }
    __syncthreads();
  }
}

// grad[p] = sum_c partial[c][p] in CTA order (deterministic)
__global__ void k_reduce_partials(const float* __restrict__ partial, int64_t nctas, int64_t np,
                                  float* __restrict__ grad) {
  for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < np; p += (int64_t)gridDim.x * blockDim.x) {
    float s = 0.f;
    for (int64_t c = 0; c < nctas; ++c) s += partial[c * np + p];
    grad[p] = s;
  }
}

__global__ void k_adam(float* __restrict__ w, float* __restrict__ m, float* __restrict__ v,
                       const float* __restrict__ g, int64_t np, float lr, float b1, float b2, float eps,
                       float c1, float c2, __nv_bfloat16* __restrict__ w16) {
  for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < np; p += (int64_t)gridDim.x * blockDim.x) {
    const float gg = g[p];
    const float mm = b1 * m[p] + (1.f - b1) * gg;
    const float vv = b2 * v[p] + (1.f - b2) * gg * gg;
    m[p] = mm;
    v[p] = vv;
    const float upd = lr * (mm / c1) / (sqrtf(vv / c2) + eps);
    const float nw = w[p] - upd;
    w[p] = nw;
    w16[p] = __float2bfloat16_rn(nw);
  }
}

// One CTA per SM (the kernel's shared memory allows one), at most one chunk each.
int64_t mlp_grid(itg_handle* h, int64_t n) {
  const int64_t chunks = (n + EPB - 1) / EPB;
  return chunks < h->num_sms ? chunks : (int64_t)h->num_sms;
}

}  // namespace

extern "C" int itg_mlp_create(itg_handle* h, int in_dim, uint64_t seed, void** out) {
  if (!h || !out || in_dim < 1 || in_dim > MAXF) return ITG_ERR_INVALID;
  Mlp* M = new Mlp();
  M->F = in_dim;
  M->nparam = nparams(in_dim);
  const size_t bytes = sizeof(float) * M->nparam;
  if (cudaMalloc(&M->master, bytes) != cudaSuccess || cudaMalloc(&M->m, bytes) != cudaSuccess ||
      cudaMalloc(&M->v, bytes) != cudaSuccess || cudaMalloc(&M->grad, bytes) != cudaSuccess ||
      cudaMalloc(&M->w16, sizeof(__nv_bfloat16) * M->nparam) != cudaSuccess) {
    delete M;
    return itg_fail(h, ITG_ERR_ALLOC, "mlp allocation failed");
  }
  // He-style initialisation from a host LCG (deterministic per seed)
  std::vector<float> w(M->nparam, 0.f);
  uint64_t st = seed * 6364136223846793005ull + 1442695040888963407ull;
  auto uni = [&]() {
    st = st * 6364136223846793005ull + 1442695040888963407ull;
    return ((st >> 11) * (1.0 / 9007199254740992.0)) * 2.0 - 1.0;
  };
  const int F = in_dim;
  for (int64_t i = 0; i < (int64_t)MW * F; ++i) w[oW1(F) + i] = (float)(uni() * std::sqrt(6.0 / F));
  for (int64_t i = 0; i < (int64_t)MW * MW; ++i) w[oW2(F) + i] = (float)(uni() * std::sqrt(6.0 / MW));
  // output layer starts at zero: g = 0, i.e. the learned preconditioner
  // starts as the diagonal one (the first Adam step moves w3 off zero)
  for (int64_t i = 0; i < MW; ++i) w[ow3(F) + i] = 0.f;
  ITG_CUDA(h, cudaMemcpy(M->master, w.data(), bytes, cudaMemcpyHostToDevice));
  ITG_CUDA(h, cudaMemset(M->m, 0, bytes));
  ITG_CUDA(h, cudaMemset(M->v, 0, bytes));
  k_to_bf16<<<64, 256, 0, h->stream>>>(M->master, M->nparam, M->w16);
  ITG_CHECK_LAUNCH(h);
  static bool attr = false;
  if (!attr) {
    ITG_CUDA(h, cudaFuncSetAttribute(k_mlp_fused, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)(sizeof(float) * mlp_smem_floats(MAXF))));
    attr = true;
  }
  *out = M;
  return ITG_OK;
}

extern "C" int itg_mlp_destroy(itg_handle* h, void* mlp) {
  if (!h || !mlp) return ITG_ERR_INVALID;
  Mlp* M = (Mlp*)mlp;
  cudaStreamSynchronize(h->stream);
  cudaFree(M->master);
  cudaFree(M->m);
  cudaFree(M->v);
  cudaFree(M->grad);
  cudaFree(M->w16);
  if (M->partial) cudaFree(M->partial);
  if (M->loss_part) cudaFree(M->loss_part);
  delete M;
  return ITG_OK;
}

extern "C" int itg_mlp_num_params(void* mlp, int64_t* n) {
  if (!mlp || !n) return ITG_ERR_INVALID;
  *n = ((Mlp*)mlp)->nparam;
  return ITG_OK;
}

extern "C" int itg_mlp_get_params(itg_handle* h, void* mlp, float* host) {
  if (!h || !mlp || !host) return ITG_ERR_INVALID;
  Mlp* M = (Mlp*)mlp;
  ITG_CUDA(h, cudaMemcpyAsync(host, M->master, sizeof(float) * M->nparam, cudaMemcpyDeviceToHost, h->stream));
  ITG_CUDA(h, cudaStreamSynchronize(h->stream));
  return ITG_OK;
}

extern "C" int itg_mlp_set_params(itg_handle* h, void* mlp, const float* host) {
  if (!h || !mlp || !host) return ITG_ERR_INVALID;
  Mlp* M = (Mlp*)mlp;
  ITG_CUDA(h, cudaMemcpyAsync(M->master, host, sizeof(float) * M->nparam, cudaMemcpyHostToDevice, h->stream));
  k_to_bf16<<<64, 256, 0, h->stream>>>(M->master, M->nparam, M->w16);
  ITG_CHECK_LAUNCH(h);
  ITG_CUDA(h, cudaStreamSynchronize(h->stream));
  return ITG_OK;
}

namespace itg {
int mlp_forward(itg_handle* h, void* mlp, int64_t n, const float* X, float* g) {
  Mlp* M = (Mlp*)mlp;
  if (n <= 0) return ITG_OK;
  const int64_t ctas = mlp_grid(h, n);
  k_mlp_fused<<<(unsigned)ctas, MTHREADS, sizeof(float) * mlp_smem_floats(M->F), h->stream>>>(
      M->w16, M->master, M->F, n, X, nullptr, nullptr, g, 0, 0.f, nullptr, nullptr);
  ITG_CHECK_LAUNCH(h);
  return ITG_OK;
}
}  // namespace itg

extern "C" int itg_mlp_forward(itg_handle* h, void* mlp, int64_t n, const float* X, float* g) {
  if (!h || !mlp || n < 0 || (n > 0 && (!X || !g))) return ITG_ERR_INVALID;
  return itg::mlp_forward(h, mlp, n, X, g);
}

// Gradient of the loss w.r.t. the master parameters (device array `grad_out`
// of num_params floats, may be NULL) and the loss (host, may be NULL); with
// lr > 0 an Adam step (beta1 0.9, beta2 0.999, eps 1e-8) follows.
extern "C" int itg_mlp_train_step(itg_handle* h, void* mlp, int64_t n, const float* X, const float* mult,
                                  const float* target, float lr, float* grad_out, float* loss) {
  if (!h || !mlp || n <= 0 || !X || !mult || !target) return ITG_ERR_INVALID;
  Mlp* M = (Mlp*)mlp;
  const int64_t ctas = mlp_grid(h, n);
  if (ctas > M->partial_ctas) {
    if (M->partial) cudaFree(M->partial);
    if (M->loss_part) cudaFree(M->loss_part);
    M->partial = nullptr;
    M->loss_part = nullptr;
    ITG_CUDA(h, cudaStreamSynchronize(h->stream));
    if (cudaMalloc(&M->partial, sizeof(float) * ctas * M->nparam) != cudaSuccess ||
        cudaMalloc(&M->loss_part, sizeof(float) * ctas) != cudaSuccess)
      return itg_fail(h, ITG_ERR_ALLOC, "mlp gradient buffers");
    M->partial_ctas = ctas;
  }
  k_mlp_fused<<<(unsigned)ctas, MTHREADS, sizeof(float) * mlp_smem_floats(M->F), h->stream>>>(
      M->w16, M->master, M->F, n, X, mult, target, nullptr, 1, 1.f / (float)n, M->partial, M->loss_part);
  k_reduce_partials<<<itg_blocks_for(M->nparam, 256, 256), 256, 0, h->stream>>>(M->partial, ctas, M->nparam,
                                                                                M->grad);
  ITG_CHECK_LAUNCH(h);
  if (grad_out)
    ITG_CUDA(h, cudaMemcpyAsync(grad_out, M->grad, sizeof(float) * M->nparam, cudaMemcpyDeviceToDevice, h->stream));
  if (lr > 0.f) {
    M->step++;
    const float b1 = 0.9f, b2 = 0.999f;
    const float c1 = 1.f - std::pow(b1, (float)M->step), c2 = 1.f - std::pow(b2, (float)M->step);
    k_adam<<<itg_blocks_for(M->nparam, 256, 256), 256, 0, h->stream>>>(M->master, M->m, M->v, M->grad, M->nparam,
                                                                       lr, b1, b2, 1e-8f, c1, c2, M->w16);
    ITG_CHECK_LAUNCH(h);
  }
  if (loss) {
    std::vector<float> lp(ctas);
    ITG_CUDA(h, cudaMemcpyAsync(lp.data(), M->loss_part, sizeof(float) * ctas, cudaMemcpyDeviceToHost, h->stream));
    ITG_CUDA(h, cudaStreamSynchronize(h->stream));
    double s = 0.0;
    for (float x : lp) s += x;
    *loss = (float)(s / (double)n);
  }
  return ITG_OK;
}
