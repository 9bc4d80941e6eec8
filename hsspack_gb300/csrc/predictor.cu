// predictor.cu -- learned initial iterate for the secular solver.
//
// For a non-last root j of f(x) = 1/rho + sum_i z_i^2/(d_i - x), with
// delta = d_{j+1} - d_j and x = d_j + t*delta, delta*f = c(t) - a/t + b/(1-t)
// where a = z_j^2, b = z_{j+1}^2 and c(t) collects 1/rho and every far pole.
// The midpoint pass (k_secular_mid, secular.cu) evaluates the full sums at
// t = 1/2 -- exactly the first evaluation of the standard method -- and gives
// c0 = c(1/2), c1 = c'(1/2).  Features:
//   f0 = log(a/|c0|), f1 = log(b/|c0|), f2 = c1/|c0|, f3 = sign(c0),
//   f4/f5 = log of the neighbouring pole gaps over delta,
//   f6 = logit t0 (two-pole root with c = c0, the standard guess),
//   f7 = logit t1 (two-pole root with c = c0 + c1 (t0 - 1/2)).
// A 3 x 64 MLP (ReLU) predicts the residual logit(t*) - f7; the learned start
// is sigmoid(f7 + mlp(f)) kept inside the half interval that the sign of
// f(midpoint) selects.  Weights are stored in BF16, arithmetic in FP32.  The
// FP64 secular iteration starts there and always runs to convergence inside
// its bracket (restarting from the standard guess if the start fails its
// residual check), so a poor prediction costs iterations only.
//
// Training (hand-written): forward / backward of the same network in FP32
// (one thread per sample, gradients reduced per CTA in shared memory, then one
// atomic per parameter per CTA), mean squared error, Adam update.
#include <cuda_bf16.h>

#include "hss_common.cuh"
#include "hss_kernels.h"

namespace hss {

constexpr int NF = 8;       // features
constexpr int NH = 64;      // hidden width
constexpr int WIN = 6;      // pole window each side for local sums
// parameter layout (floats): W1[NF][NH], b1[NH], W2[NH][NH], b2[NH], W3[NH][NH],
// b3[NH], W4[NH], b4
constexpr int P_W1 = 0, P_B1 = P_W1 + NF * NH, P_W2 = P_B1 + NH, P_B2 = P_W2 + NH * NH,
              P_W3 = P_B2 + NH, P_B3 = P_W3 + NH * NH, P_W4 = P_B3 + NH, P_B4 = P_W4 + NH,
              NPARAM = P_B4 + 1;

__device__ __forceinline__ float clampf(float x, float lo, float hi) {
  return fminf(fmaxf(x, lo), hi);
}

// y = mlp(f) with weights given as FP32 (training) or read from BF16 (inference)
template <class WT>
__device__ float mlp_forward(const float *f, const WT *__restrict__ P, float *h1, float *h2,
                             float *h3) {
  auto w = [&](int i) -> float { return (float)P[i]; };
  for (int o = 0; o < NH; ++o) {
    float s = w(P_B1 + o);
#pragma unroll
    for (int i = 0; i < NF; ++i) s = fmaf(f[i], w(P_W1 + i * NH + o), s);
    h1[o] = fmaxf(s, 0.f);
  }
  for (int o = 0; o < NH; ++o) {
    float s = w(P_B2 + o);
    for (int i = 0; i < NH; ++i) s = fmaf(h1[i], w(P_W2 + i * NH + o), s);
    h2[o] = fmaxf(s, 0.f);
  }
  for (int o = 0; o < NH; ++o) {
    float s = w(P_B3 + o);
    for (int i = 0; i < NH; ++i) s = fmaf(h2[i], w(P_W3 + i * NH + o), s);
    h3[o] = fmaxf(s, 0.f);
  }
  float y = w(P_B4);
  for (int i = 0; i < NH; ++i) y = fmaf(h3[i], w(P_W4 + i), y);
  return y;
}

struct bf16w {
  __nv_bfloat16 v;
  __device__ operator float() const { return __bfloat162float(v); }
};

// Inference: feat[(s+j)*(NF+1) + i] from the midpoint pass (slot NF holds the
// side: 0 root in (d_j, midpoint], 1 in (midpoint, d_{j+1}), -1 no prediction).
// One thread per position.  The weights (converted to FP32) sit in shared
// memory and are read as broadcasts; each thread keeps its activation row in
// a padded shared-memory row (stride NH + 1: conflict-free) and computes 16
// outputs at a time in registers, so every activation load feeds 16 FMAs.
// The sums run in the same order as mlp_forward (bias, then inputs ascending).
constexpr int PT = 128;          // positions per CTA
constexpr int AST = NH + 1;      // activation row stride (floats)
constexpr int OB = 16;           // outputs per register block
constexpr size_t PREDICT_SMEM = sizeof(float) * ((size_t)((NPARAM + 3) / 4 * 4) + 2 * PT * AST);

template <int NIN>
__device__ __forceinline__ void dense_relu_rows(const float *__restrict__ in, int in_stride,
                                                const float *__restrict__ W, const float *__restrict__ b,
                                                float *__restrict__ out) {
#pragma unroll 1
  for (int o0 = 0; o0 < NH; o0 += OB) {
    float acc[OB];
#pragma unroll
    for (int j = 0; j < OB; ++j) acc[j] = b[o0 + j];
#pragma unroll 4
    for (int i = 0; i < NIN; ++i) {
      const float x = in[i * in_stride];
      const float *w = W + i * NH + o0;
#pragma unroll
      for (int j = 0; j < OB; ++j) acc[j] = fmaf(x, w[j], acc[j]);
    }
#pragma unroll
    for (int j = 0; j < OB; ++j) out[o0 + j] = fmaxf(acc[j], 0.f);
  }
}

__global__ void __launch_bounds__(PT)
k_predict(int n, const float *__restrict__ feat, const __nv_bfloat16 *__restrict__ Wb,
          const float *__restrict__ norm, float *__restrict__ guess) {
  extern __shared__ float psm[];
  float *sW = psm;
  float *A = psm + (NPARAM + 3) / 4 * 4;
  float *B = A + PT * AST;
  for (int i = threadIdx.x; i < NPARAM; i += blockDim.x) sW[i] = __bfloat162float(Wb[i]);
  __syncthreads();
  const int r = blockIdx.x * PT + threadIdx.x;
  if (r >= n) return;
  const float *f = feat + (long long)r * (NF + 1);
  const float side = f[NF];
  if (side < 0.f) { guess[r] = 2.0f; return; }  // no prediction
  float *a = A + threadIdx.x * AST, *bb = B + threadIdx.x * AST;
  // normalised features in this thread's row of B (stride 1)
#pragma unroll
  for (int i = 0; i < NF; ++i) bb[i] = (f[i] - norm[i]) / norm[NF + i];
  dense_relu_rows<NF>(bb, 1, sW + P_W1, sW + P_B1, a);
  dense_relu_rows<NH>(a, 1, sW + P_W2, sW + P_B2, bb);
  dense_relu_rows<NH>(bb, 1, sW + P_W3, sW + P_B3, a);
  float y = sW[P_B4];
  for (int i = 0; i < NH; ++i) y = fmaf(a[i], sW[P_W4 + i], y);
  const float l = f[NF - 1] + clampf(y, -1.f, 1.f);
  // signed distance to the nearer pole: +u (left pole), -u (right pole)
  float u;
  if (side == 0.f) u = (l <= 0.f) ? __expf(l) / (1.f + __expf(l)) : 0.5f;
  else u = (l > 0.f) ? __expf(-l) / (1.f + __expf(-l)) : 0.5f;
  u = fminf(fmaxf(u, 1e-20f), side == 0.f ? 0.5f : 0.49999f);
  guess[r] = side == 0.f ? u : -u;
}

// Training targets: T[j] = clamp(logit(difl_j / delta_j) - f7_j), from the
// midpoint features of one solved secular problem (non-last roots).
__global__ void k_train_targets(int K, const double *__restrict__ d,
                                const double *__restrict__ difl, const double *__restrict__ difr,
                                const float *__restrict__ feat, float *__restrict__ X,
                                float *__restrict__ T) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= K - 1) return;
  const float *f = feat + (long long)j * (NF + 1);
  for (int i = 0; i < NF; ++i) X[(long long)j * NF + i] = f[i];
  // logit of the root's position: log(t / (1 - t)) = log(difl / -difr)
  const double l = log(fmax(difl[j], 1e-300) / fmax(-difr[j], 1e-300));
  // only small refinements of the analytic start are learned; larger
  // residuals are rare and left to the FP64 iteration
  T[j] = clampf((float)(l - (double)f[NF - 1]), -1.f, 1.f);
}

// One training pass over n samples: loss = mean (mlp(xn) - t)^2; gradients
// accumulated into G (NPARAM floats, zeroed by the caller) and loss into L.
__global__ void __launch_bounds__(128)
k_mlp_grad(int n, const float *__restrict__ X, const float *__restrict__ T,
           const float *__restrict__ norm, const float *__restrict__ W, float *__restrict__ G,
           float *__restrict__ L) {
  __shared__ float sG[NPARAM];
  __shared__ float sL;
  const float *sW = W;  // weights through the read-only cache
  for (int i = threadIdx.x; i < NPARAM; i += blockDim.x) sG[i] = 0.f;
  if (threadIdx.x == 0) sL = 0.f;
  __syncthreads();
  const int idx = blockIdx.x * blockDim.x + threadIdx.x;
  if (idx < n) {
    float fn[NF];
#pragma unroll
    for (int i = 0; i < NF; ++i) fn[i] = (X[(long long)idx * NF + i] - norm[i]) / norm[NF + i];
    float h1[NH], h2[NH], h3[NH];
    const float y = mlp_forward(fn, sW, h1, h2, h3);
    const float e = y - T[idx];
    atomicAdd(&sL, e * e / n);
    const float dy = 2.f * e / n;
    // layer 4
    atomicAdd(&sG[P_B4], dy);
    float d3[NH];
    for (int i = 0; i < NH; ++i) {
      atomicAdd(&sG[P_W4 + i], dy * h3[i]);
      d3[i] = (h3[i] > 0.f) ? dy * sW[P_W4 + i] : 0.f;
    }
    // layer 3: h3 = relu(h2 W3 + b3)
    float d2[NH];
    for (int i = 0; i < NH; ++i) d2[i] = 0.f;
    for (int o = 0; o < NH; ++o) {
      if (d3[o] == 0.f) continue;
      atomicAdd(&sG[P_B3 + o], d3[o]);
      for (int i = 0; i < NH; ++i) {
        atomicAdd(&sG[P_W3 + i * NH + o], h2[i] * d3[o]);
        d2[i] = fmaf(sW[P_W3 + i * NH + o], d3[o], d2[i]);
      }
    }
    for (int i = 0; i < NH; ++i) if (h2[i] <= 0.f) d2[i] = 0.f;
    // layer 2
    float d1[NH];
    for (int i = 0; i < NH; ++i) d1[i] = 0.f;
    for (int o = 0; o < NH; ++o) {
      if (d2[o] == 0.f) continue;
      atomicAdd(&sG[P_B2 + o], d2[o]);
      for (int i = 0; i < NH; ++i) {
        atomicAdd(&sG[P_W2 + i * NH + o], h1[i] * d2[o]);
        d1[i] = fmaf(sW[P_W2 + i * NH + o], d2[o], d1[i]);
      }
    }
    for (int i = 0; i < NH; ++i) if (h1[i] <= 0.f) d1[i] = 0.f;
    // layer 1
    for (int o = 0; o < NH; ++o) {
      if (d1[o] == 0.f) continue;
      atomicAdd(&sG[P_B1 + o], d1[o]);
#pragma unroll
      for (int i = 0; i < NF; ++i) atomicAdd(&sG[P_W1 + i * NH + o], fn[i] * d1[o]);
    }
  }
  __syncthreads();
  for (int i = threadIdx.x; i < NPARAM; i += blockDim.x)
    if (sG[i] != 0.f) atomicAdd(&G[i], sG[i]);
  if (threadIdx.x == 0) atomicAdd(L, sL);
}

// Adam step (Kingma & Ba 2015) on the FP32 master weights; refreshes the BF16 copy.
__global__ void k_adam(int np, float *__restrict__ W, const float *__restrict__ G,
                       float *__restrict__ M, float *__restrict__ V, float lr, float b1, float b2,
                       float eps, int step, __nv_bfloat16 *__restrict__ Wb) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= np) return;
  const float g = G[i];
  const float m = b1 * M[i] + (1.f - b1) * g;
  const float v = b2 * V[i] + (1.f - b2) * g * g;
  M[i] = m;
  V[i] = v;
  const float mh = m / (1.f - powf(b1, (float)step)), vh = v / (1.f - powf(b2, (float)step));
  W[i] -= lr * mh / (sqrtf(vh) + eps);
  if (Wb) Wb[i] = __float2bfloat16_rn(W[i]);
}

int mlp_nparam() { return NPARAM; }
int mlp_nfeat() { return NF; }

void launch_predict(int n, const float *feat, const void *Wb, const float *norm, float *guess,
                    cudaStream_t st) {
  if (n <= 0) return;
  static bool attr = false;
  if (!attr) {
    cudaFuncSetAttribute(k_predict, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)PREDICT_SMEM);
    attr = true;
  }
  k_predict<<<(n + PT - 1) / PT, PT, PREDICT_SMEM, st>>>(n, feat, (const __nv_bfloat16 *)Wb, norm,
                                                         guess);
}

void launch_train_targets(int K, const double *d, const double *difl, const double *difr,
                          const float *feat, float *X, float *T, cudaStream_t st) {
  if (K < 2) return;
  k_train_targets<<<(K + 127) / 128, 128, 0, st>>>(K, d, difl, difr, feat, X, T);
}

void launch_mlp_grad(int n, const float *X, const float *T, const float *norm, const float *W,
                     float *G, float *L, cudaStream_t st) {
  if (n <= 0) return;
  k_mlp_grad<<<(n + 127) / 128, 128, 0, st>>>(n, X, T, norm, W, G, L);
}

void launch_adam(int np, float *W, const float *G, float *M, float *V, float lr, int step,
                 void *Wb, cudaStream_t st) {
  k_adam<<<(np + 255) / 256, 256, 0, st>>>(np, W, G, M, V, lr, 0.9f, 0.999f, 1e-8f, step,
                                          (__nv_bfloat16 *)Wb);
}

}  // namespace hss
