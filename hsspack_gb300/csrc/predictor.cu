// predictor.cu -- learned initial iterate for the secular solver.
//
// For a non-last root j of f(x) = 1/rho + sum_i z_i^2/(d_i - x), with
// delta = d_{j+1} - d_j, the target is x* = (lam_j - d_j)/delta in (0, 1).
// Local features (O(W) work per root, W = 6 poles each side):
//   f0 = log(z_j^2/delta), f1 = log(z_{j+1}^2/delta), f2 = log(delta/rho),
//   f3/f4 = windowed left/right far sums at the midpoint (times delta),
//   f5/f6 = log gaps to the next pole on each side (over delta),
//   f7 = logit of the analytic two-pole guess with the windowed far sum.
// A 3 x 64 MLP (ReLU) maps the features to a logit correction; the guess is
// sigmoid(f7 + mlp(f)).  Weights are stored in BF16, all arithmetic in FP32.
// The FP64 secular iteration starts from this guess and always runs to
// convergence inside its bracket, so a poor prediction costs iterations only.
//
// Training (hand-written): forward / backward of the same network over a batch
// in FP32 (one thread per sample, gradients reduced per CTA in shared memory,
// then one atomic per parameter per CTA), mean squared error on the logit,
// Adam update.
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

// Features of root j (non-last) of the secular problem (d, z, rho, K).
__device__ void root_features(const double *__restrict__ d, const double *__restrict__ z, int K,
                             double rho, int j, float *f) {
  const double dj = d[j], dj1 = d[j + 1];
  const double delta = dj1 - dj;
  const double mid = dj + 0.5 * delta;
  const double a = z[j] * z[j] / delta, b = z[j + 1] * z[j + 1] / delta;
  double sl = 0.0, sr = 0.0;
  for (int i = max(0, j - WIN); i < j; ++i) sl += z[i] * z[i] / (d[i] - mid);
  for (int i = j + 2; i <= min(K - 1, j + 1 + WIN); ++i) sr += z[i] * z[i] / (d[i] - mid);
  sl *= delta;
  sr *= delta;
  // two-pole model  c - a/x + b/(1-x) = 0  (units of 1/delta), c = delta/rho + sl + sr
  const double c = delta / rho + sl + sr;
  // c x (1 - x) - a (1 - x) + b x = 0  ->  -c x^2 + (c + a + b) x - a = 0
  double x0;
  {
    const double A = -c, B = c + a + b, C = -a;
    if (fabs(A) < 1e-300) {
      x0 = a / (a + b);
    } else {
      double disc = B * B - 4.0 * A * C;
      disc = disc < 0.0 ? 0.0 : disc;
      const double q = -0.5 * (B + copysign(sqrt(disc), B));
      const double r1 = q / A, r2 = (q != 0.0) ? C / q : r1;
      x0 = (r1 > 0.0 && r1 < 1.0) ? r1 : r2;
      if (!(x0 > 0.0 && x0 < 1.0)) x0 = 0.5;
    }
  }
  x0 = fmin(fmax(x0, 1e-7), 1.0 - 1e-7);
  const double gl = (j > 0) ? (dj - d[j - 1]) / delta : 1e3;
  const double gr = (j + 2 < K) ? (d[j + 2] - dj1) / delta : 1e3;
  f[0] = clampf((float)log(a + 1e-300), -80.f, 80.f);
  f[1] = clampf((float)log(b + 1e-300), -80.f, 80.f);
  f[2] = clampf((float)log(delta / rho + 1e-300), -80.f, 80.f);
  f[3] = clampf((float)sl, -1e4f, 1e4f);
  f[4] = clampf((float)sr, -1e4f, 1e4f);
  f[5] = clampf((float)log(gl), -40.f, 40.f);
  f[6] = clampf((float)log(gr), -40.f, 40.f);
  f[7] = (float)log(x0 / (1.0 - x0));
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

// Inference over the roots of a level: guess[s + j] for j < K-1 of every merge.
// Features are normalised by (mu, sigma) before the network.
__global__ void __launch_bounds__(128)
k_predict(LevelView lv, const double *__restrict__ dl, const double *__restrict__ zw,
          const __nv_bfloat16 *__restrict__ Wb, const float *__restrict__ norm,
          float *__restrict__ guess) {
  __shared__ __nv_bfloat16 sW[NPARAM];
  for (int i = threadIdx.x; i < NPARAM; i += blockDim.x) sW[i] = Wb[i];
  __syncthreads();
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= __ldg(lv.rootoff + lv.P)) return;
  int lo = 0, hi = lv.P;
  while (hi - lo > 1) { int md = (lo + hi) >> 1; if (__ldg(lv.rootoff + md) <= r) lo = md; else hi = md; }
  const int j = r - __ldg(lv.rootoff + lo);
  const int s = __ldg(lv.s + lo), K = __ldg(lv.K + lo);
  if (j >= K - 1 || K < 3) { guess[s + j] = -1.0f; return; }
  float f[NF];
  root_features(dl + s, zw + s, K, __ldg(lv.rho + lo), j, f);
  float fn[NF];
#pragma unroll
  for (int i = 0; i < NF; ++i) fn[i] = (f[i] - norm[i]) / norm[NF + i];
  float h1[NH], h2[NH], h3[NH];
  const float y = mlp_forward(fn, reinterpret_cast<const bf16w *>(sW), h1, h2, h3);
  const float logit = clampf(f[7] + y, -16.f, 16.f);
  guess[s + j] = 1.f / (1.f + __expf(-logit));
}

// Training features and targets for one secular problem solved by the plain
// solver: X[j] = features, T[j] = logit(difl_j / delta_j) - f7 (the correction).
__global__ void k_train_features(int K, const double *__restrict__ d, const double *__restrict__ z,
                                 double rho, const double *__restrict__ difl, float *__restrict__ X,
                                 float *__restrict__ T) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= K - 1) return;
  float f[NF];
  root_features(d, z, K, rho, j, f);
  for (int i = 0; i < NF; ++i) X[(long long)j * NF + i] = f[i];
  double x = difl[j] / (d[j + 1] - d[j]);
  x = fmin(fmax(x, 1e-7), 1.0 - 1e-7);
  T[j] = (float)log(x / (1.0 - x)) - f[7];
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

void launch_predict(const LevelView &lv, int total, const double *dl, const double *zw,
                    const void *Wb, const float *norm, float *guess, cudaStream_t st) {
  if (total <= 0) return;
  k_predict<<<(total + 127) / 128, 128, 0, st>>>(lv, dl, zw, (const __nv_bfloat16 *)Wb, norm,
                                                 guess);
}

void launch_train_features(int K, const double *d, const double *z, double rho,
                           const double *difl, float *X, float *T, cudaStream_t st) {
  if (K < 2) return;
  k_train_features<<<(K + 127) / 128, 128, 0, st>>>(K, d, z, rho, difl, X, T);
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
