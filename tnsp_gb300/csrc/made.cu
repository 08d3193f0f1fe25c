// Learned proposal: an autoregressive masked MLP (MADE, Germain et al., ICML 2015) over n binary sites,
// trained by maximum likelihood on configurations of the plain sweep and sampled site by site; the
// sampler uses it as a Metropolis-Hastings independence proposal with exact PEPS amplitudes.
//
// x (n) -> h1 = relu(W1 x + b1) (H) -> h2 = relu(W2 h1 + b2) (H) -> o = W3 h2 + b3 (n),
// p(x_i = 1 | x_<i) = sigmoid(o_i).  Degrees: input / output i -> i + 1, hidden k -> (k mod (n-1)) + 1;
// masks W1: d_h >= d_in, W2: d_h >= d_h, W3: d_out > d_h, so o_i sees x_0..x_{i-1} only.
// Weights are kept in float32 (master copy, Adam moments) and used by every product as bfloat16;
// activations and accumulations are float32.  The networks are small (n <= a few hundred, H = 256):
// every kernel computes one output element per thread.
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>
#include <cmath>
#include <random>
#include <string>
#include <vector>

#include "../../include/tnsp_gb300.h"

struct tnsp_made {
  int device = 0, n = 0, H = 0, cap = 0;
  long long P = 0;                 // parameters: W1 (H x n), b1 (H), W2 (H x H), b2 (H), W3 (n x H), b3 (n)
  long long oW1 = 0, ob1 = 0, oW2 = 0, ob2 = 0, oW3 = 0, ob3 = 0;
  float *p = nullptr, *m = nullptr, *v = nullptr, *g = nullptr;
  __nv_bfloat16* w = nullptr;      // bfloat16 copy of p
  float *x = nullptr, *a1 = nullptr, *h1 = nullptr, *a2 = nullptr, *h2 = nullptr, *o = nullptr;
  float *d_o = nullptr, *dh2 = nullptr, *dh1 = nullptr;
  int32_t* conf = nullptr;
  double* lq = nullptr;
  int step = 0;
  uint64_t seed = 0, draws = 0;
  cudaStream_t stream = nullptr;
  std::string err;
};

namespace {

enum { MASK_IN_H = 1, MASK_H_H = 2, MASK_H_OUT = 3 };

__device__ __forceinline__ int deg_h(int k, int n) { return (k % (n > 1 ? n - 1 : 1)) + 1; }

// mask of weight (row r, column c) of the layer: 1 where the connection is allowed
__device__ __forceinline__ bool allowed(int mode, int r, int c, int n) {
  if (mode == MASK_IN_H) return deg_h(r, n) >= c + 1;
  if (mode == MASK_H_H) return deg_h(r, n) >= deg_h(c, n);
  return r + 1 > deg_h(c, n);
}

__global__ void k_to_bf16(const float* __restrict__ p, __nv_bfloat16* __restrict__ w, long long P) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < P; i += (long long)gridDim.x * blockDim.x)
    w[i] = __float2bfloat16_rn(p[i]);
}

// out[b][r] = act(sum_c in[b][c] W[r][c] mask + bias[r]); pre[b][r] keeps the value before the relu
__global__ void k_linear(const float* __restrict__ in, int K, const __nv_bfloat16* __restrict__ W,
                         const float* __restrict__ bias, int R, int mode, int n, int B, float* __restrict__ pre,
                         float* __restrict__ out, int relu) {
  const long long total = (long long)B * R;
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < total; t += (long long)gridDim.x * blockDim.x) {
    const int b = (int)(t / R), r = (int)(t % R);
    const float* xi = in + (long long)b * K;
    const __nv_bfloat16* wr = W + (long long)r * K;
    float acc = bias[r];
    for (int c = 0; c < K; ++c)
      if (allowed(mode, r, c, n)) acc = fmaf(xi[c], __bfloat162float(wr[c]), acc);
    if (pre) pre[t] = acc;
    out[t] = relu ? fmaxf(acc, 0.f) : acc;
  }
}

// log q(x) per sample and (when d_o != null) the gradient of the mean negative log-likelihood with
// respect to the logits: (sigmoid(o) - x) / B
__global__ void k_logq(const float* __restrict__ o, const float* __restrict__ x, int B, int n, double* __restrict__ lq,
                       float* __restrict__ d_o) {
  for (int b = blockIdx.x * blockDim.x + threadIdx.x; b < B; b += gridDim.x * blockDim.x) {
    double s = 0.0;
    for (int i = 0; i < n; ++i) {
      const float oi = o[(long long)b * n + i], xi = x[(long long)b * n + i];
      // log sigmoid(o) = -log(1 + e^-o), log(1 - sigmoid(o)) = -log(1 + e^o), evaluated stably
      const double l1p = log1p(exp(-fabs((double)oi)));
      const double lp = -(fmax(-(double)oi, 0.0) + l1p), lm = -(fmax((double)oi, 0.0) + l1p);
      s += xi > 0.5f ? lp : lm;
      if (d_o) d_o[(long long)b * n + i] = (1.f / (1.f + expf(-oi)) - xi) / (float)B;
    }
    lq[b] = s;
  }
}

// din[b][c] = (sum_r dout[b][r] W[r][c] mask) * (pre[b][c] > 0)
__global__ void k_backprop(const float* __restrict__ dout, int R, const __nv_bfloat16* __restrict__ W, int K, int mode,
                           int n, int B, const float* __restrict__ pre, float* __restrict__ din) {
  const long long total = (long long)B * K;
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < total; t += (long long)gridDim.x * blockDim.x) {
    const int b = (int)(t / K), c = (int)(t % K);
    float acc = 0.f;
    for (int r = 0; r < R; ++r)
      if (allowed(mode, r, c, n)) acc = fmaf(dout[(long long)b * R + r], __bfloat162float(W[(long long)r * K + c]), acc);
    din[t] = pre[t] > 0.f ? acc : 0.f;
  }
}

// gW[r][c] = mask ? sum_b dout[b][r] in[b][c] : 0; gb[r] = sum_b dout[b][r]
__global__ void k_wgrad(const float* __restrict__ dout, int R, const float* __restrict__ in, int K, int mode, int n,
                        int B, float* __restrict__ gW, float* __restrict__ gb) {
  const long long total = (long long)R * (K + 1);
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < total; t += (long long)gridDim.x * blockDim.x) {
    const int r = (int)(t / (K + 1)), c = (int)(t % (K + 1));
    if (c == K) {
      float s = 0.f;
      for (int b = 0; b < B; ++b) s += dout[(long long)b * R + r];
      gb[r] = s;
    } else {
      float s = 0.f;
      if (allowed(mode, r, c, n))
        for (int b = 0; b < B; ++b) s = fmaf(dout[(long long)b * R + r], in[(long long)b * K + c], s);
      gW[(long long)r * K + c] = s;
    }
  }
}

__global__ void k_adam(float* __restrict__ p, const float* __restrict__ g, float* __restrict__ m, float* __restrict__ v,
                       long long P, float lr, float bc1, float bc2) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < P; i += (long long)gridDim.x * blockDim.x) {
    const float gi = g[i];
    const float mi = 0.9f * m[i] + 0.1f * gi;
    const float vi = 0.999f * v[i] + 0.001f * gi * gi;
    m[i] = mi;
    v[i] = vi;
    p[i] -= lr * (mi / bc1) / (sqrtf(vi / bc2) + 1e-8f);
  }
}

__global__ void k_conf_to_x(const int32_t* __restrict__ conf, long long N, float* __restrict__ x) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < N; i += (long long)gridDim.x * blockDim.x)
    x[i] = conf[i] ? 1.f : 0.f;
}

__global__ void k_x_to_conf(const float* __restrict__ x, long long N, int32_t* __restrict__ conf) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < N; i += (long long)gridDim.x * blockDim.x)
    conf[i] = x[i] > 0.5f ? 1 : 0;
}

// SplitMix64 (S. Vigna) of a counter: one uniform in [0, 1) per (seed, draw, sample)
__device__ __forceinline__ double uniform01(uint64_t seed, uint64_t draw, int b) {
  uint64_t z = seed + 0x9E3779B97F4A7C15ull * (draw * 0x100000001B3ull + (uint64_t)b + 1);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  z ^= z >> 31;
  return (double)(z >> 11) * (1.0 / 9007199254740992.0);
}

// x[b][i] ~ Bernoulli(sigmoid(o[b][i]))
__global__ void k_sample_site(const float* __restrict__ o, float* __restrict__ x, int B, int n, int i, uint64_t seed,
                              uint64_t draw) {
  for (int b = blockIdx.x * blockDim.x + threadIdx.x; b < B; b += gridDim.x * blockDim.x) {
    const double p1 = 1.0 / (1.0 + exp(-(double)o[(long long)b * n + i]));
    x[(long long)b * n + i] = uniform01(seed, draw, b) < p1 ? 1.f : 0.f;
  }
}

int fail(tnsp_made* h, int code, const std::string& msg) {
  if (h) h->err = msg;
  return code;
}

#define MK(call)                                                                                    \
  do {                                                                                              \
    cudaError_t e_ = (call);                                                                        \
    if (e_ != cudaSuccess)                                                                          \
      return fail(h, e_ == cudaErrorMemoryAllocation ? TNSP_E_NOMEM : TNSP_E_CUDA,                  \
                  std::string(#call) + ": " + cudaGetErrorString(e_));                              \
  } while (0)

int grid_for(long long n) { return (int)std::min<long long>(std::max<long long>((n + 255) / 256, 1), 4096); }

int forward(tnsp_made* h, int B) {
  const int n = h->n, H = h->H;
  k_linear<<<grid_for((long long)B * H), 256, 0, h->stream>>>(h->x, n, h->w + h->oW1, h->p + h->ob1, H, MASK_IN_H, n, B,
                                                            h->a1, h->h1, 1);
  k_linear<<<grid_for((long long)B * H), 256, 0, h->stream>>>(h->h1, H, h->w + h->oW2, h->p + h->ob2, H, MASK_H_H, n, B,
                                                            h->a2, h->h2, 1);
  k_linear<<<grid_for((long long)B * n), 256, 0, h->stream>>>(h->h2, H, h->w + h->oW3, h->p + h->ob3, n, MASK_H_OUT, n, B,
                                                            nullptr, h->o, 0);
  MK(cudaGetLastError());
  return TNSP_OK;
}

int load_batch(tnsp_made* h, const int32_t* configs, int B) {
  if (B < 1 || B > h->cap) return fail(h, TNSP_E_ARG, "batch size outside 1..capacity");
  for (long long i = 0; i < (long long)B * h->n; ++i)
    if (configs[i] != 0 && configs[i] != 1) return fail(h, TNSP_E_ARG, "configurations must be 0/1 per site");
  MK(cudaMemcpyAsync(h->conf, configs, sizeof(int32_t) * (size_t)B * h->n, cudaMemcpyHostToDevice, h->stream));
  k_conf_to_x<<<grid_for((long long)B * h->n), 256, 0, h->stream>>>(h->conf, (long long)B * h->n, h->x);
  MK(cudaGetLastError());
  return TNSP_OK;
}

}  // namespace

extern "C" {

int tnsp_made_create(tnsp_made** out, int device, int n_sites, int hidden, uint64_t seed, int batch_capacity) {
  if (!out || n_sites < 2 || hidden < 1 || batch_capacity < 1) return TNSP_E_ARG;
  tnsp_made* h = new tnsp_made();
  *out = h;
  h->device = device;
  h->n = n_sites;
  h->H = hidden;
  h->cap = batch_capacity;
  h->seed = seed;
  const long long n = n_sites, H = hidden;
  h->oW1 = 0;
  h->ob1 = h->oW1 + H * n;
  h->oW2 = h->ob1 + H;
  h->ob2 = h->oW2 + H * H;
  h->oW3 = h->ob2 + H;
  h->ob3 = h->oW3 + n * H;
  h->P = h->ob3 + n;
  MK(cudaSetDevice(device));
  MK(cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking));
  for (float** q : {&h->p, &h->m, &h->v, &h->g}) MK(cudaMalloc((void**)q, sizeof(float) * h->P));
  MK(cudaMalloc((void**)&h->w, sizeof(__nv_bfloat16) * h->P));
  const long long B = batch_capacity;
  for (float** q : {&h->x, &h->o, &h->d_o}) MK(cudaMalloc((void**)q, sizeof(float) * B * n));
  for (float** q : {&h->a1, &h->h1, &h->a2, &h->h2, &h->dh2, &h->dh1}) MK(cudaMalloc((void**)q, sizeof(float) * B * H));
  MK(cudaMalloc((void**)&h->conf, sizeof(int32_t) * B * n));
  MK(cudaMalloc((void**)&h->lq, sizeof(double) * B));
  // weights N(0, 1/fan_in) (masked entries are never used), biases zero
  std::mt19937_64 gen(seed);
  std::vector<float> p(h->P, 0.f);
  auto fill = [&](long long off, long long count, double fan_in) {
    std::normal_distribution<double> d(0.0, 1.0 / std::sqrt(fan_in));
    for (long long i = 0; i < count; ++i) p[off + i] = (float)d(gen);
  };
  fill(h->oW1, H * n, (double)n);
  fill(h->oW2, H * H, (double)H);
  fill(h->oW3, n * H, (double)H);
  MK(cudaMemcpy(h->p, p.data(), sizeof(float) * h->P, cudaMemcpyHostToDevice));
  MK(cudaMemset(h->m, 0, sizeof(float) * h->P));
  MK(cudaMemset(h->v, 0, sizeof(float) * h->P));
  k_to_bf16<<<grid_for(h->P), 256, 0, h->stream>>>(h->p, h->w, h->P);
  MK(cudaGetLastError());
  MK(cudaStreamSynchronize(h->stream));
  return TNSP_OK;
}

int tnsp_made_destroy(tnsp_made* h) {
  if (!h) return TNSP_E_ARG;
  cudaSetDevice(h->device);
  for (void* q : {(void*)h->p, (void*)h->m, (void*)h->v, (void*)h->g, (void*)h->w, (void*)h->x, (void*)h->o,
                  (void*)h->d_o, (void*)h->a1, (void*)h->h1, (void*)h->a2, (void*)h->h2, (void*)h->dh2,
                  (void*)h->dh1, (void*)h->conf, (void*)h->lq})
    if (q) cudaFree(q);
  if (h->stream) cudaStreamDestroy(h->stream);
  delete h;
  return TNSP_OK;
}

const char* tnsp_made_error(tnsp_made* h) { return h ? h->err.c_str() : "null handle"; }

int tnsp_made_params(tnsp_made* h, float* params, int write) {
  if (!h || !params) return TNSP_E_ARG;
  MK(cudaSetDevice(h->device));
  if (write) {
    MK(cudaMemcpyAsync(h->p, params, sizeof(float) * h->P, cudaMemcpyHostToDevice, h->stream));
    k_to_bf16<<<grid_for(h->P), 256, 0, h->stream>>>(h->p, h->w, h->P);
    MK(cudaGetLastError());
  } else {
    MK(cudaMemcpyAsync(params, h->p, sizeof(float) * h->P, cudaMemcpyDeviceToHost, h->stream));
  }
  MK(cudaStreamSynchronize(h->stream));
  return TNSP_OK;
}

int tnsp_made_train(tnsp_made* h, const int32_t* configs, int B, double lr, double* loss) {
  if (!h || !configs) return TNSP_E_ARG;
  MK(cudaSetDevice(h->device));
  int r = load_batch(h, configs, B);
  if (!r) r = forward(h, B);
  if (r) return r;
  const int n = h->n, H = h->H;
  k_logq<<<grid_for(B), 256, 0, h->stream>>>(h->o, h->x, B, n, h->lq, h->d_o);
  // layer 3, then 2, then 1: weight gradients from the layer input, input gradients through W
  k_wgrad<<<grid_for((long long)n * (H + 1)), 256, 0, h->stream>>>(h->d_o, n, h->h2, H, MASK_H_OUT, n, B, h->g + h->oW3,
                                                                  h->g + h->ob3);
  k_backprop<<<grid_for((long long)B * H), 256, 0, h->stream>>>(h->d_o, n, h->w + h->oW3, H, MASK_H_OUT, n, B, h->a2,
                                                              h->dh2);
  k_wgrad<<<grid_for((long long)H * (H + 1)), 256, 0, h->stream>>>(h->dh2, H, h->h1, H, MASK_H_H, n, B, h->g + h->oW2,
                                                                  h->g + h->ob2);
  k_backprop<<<grid_for((long long)B * H), 256, 0, h->stream>>>(h->dh2, H, h->w + h->oW2, H, MASK_H_H, n, B, h->a1,
                                                              h->dh1);
  k_wgrad<<<grid_for((long long)H * (n + 1)), 256, 0, h->stream>>>(h->dh1, H, h->x, n, MASK_IN_H, n, B, h->g + h->oW1,
                                                                  h->g + h->ob1);
  ++h->step;
  const float bc1 = 1.f - powf(0.9f, (float)h->step), bc2 = 1.f - powf(0.999f, (float)h->step);
  k_adam<<<grid_for(h->P), 256, 0, h->stream>>>(h->p, h->g, h->m, h->v, h->P, (float)lr, bc1, bc2);
  k_to_bf16<<<grid_for(h->P), 256, 0, h->stream>>>(h->p, h->w, h->P);
  MK(cudaGetLastError());
  if (loss) {
    std::vector<double> lq(B);
    MK(cudaMemcpyAsync(lq.data(), h->lq, sizeof(double) * B, cudaMemcpyDeviceToHost, h->stream));
    MK(cudaStreamSynchronize(h->stream));
    double s = 0.0;
    for (double v : lq) s += v;
    *loss = -s / B;  // before this step's update
  }
  MK(cudaStreamSynchronize(h->stream));
  return TNSP_OK;
}

int tnsp_made_gradient(tnsp_made* h, const int32_t* configs, int B, float* grad) {
  if (!h || !configs || !grad) return TNSP_E_ARG;
  MK(cudaSetDevice(h->device));
  int r = load_batch(h, configs, B);
  if (!r) r = forward(h, B);
  if (r) return r;
  const int n = h->n, H = h->H;
  k_logq<<<grid_for(B), 256, 0, h->stream>>>(h->o, h->x, B, n, h->lq, h->d_o);
  k_wgrad<<<grid_for((long long)n * (H + 1)), 256, 0, h->stream>>>(h->d_o, n, h->h2, H, MASK_H_OUT, n, B, h->g + h->oW3,
                                                                  h->g + h->ob3);
  k_backprop<<<grid_for((long long)B * H), 256, 0, h->stream>>>(h->d_o, n, h->w + h->oW3, H, MASK_H_OUT, n, B, h->a2,
                                                              h->dh2);
  k_wgrad<<<grid_for((long long)H * (H + 1)), 256, 0, h->stream>>>(h->dh2, H, h->h1, H, MASK_H_H, n, B, h->g + h->oW2,
                                                                  h->g + h->ob2);
  k_backprop<<<grid_for((long long)B * H), 256, 0, h->stream>>>(h->dh2, H, h->w + h->oW2, H, MASK_H_H, n, B, h->a1,
                                                              h->dh1);
  k_wgrad<<<grid_for((long long)H * (n + 1)), 256, 0, h->stream>>>(h->dh1, H, h->x, n, MASK_IN_H, n, B, h->g + h->oW1,
                                                                  h->g + h->ob1);
  MK(cudaGetLastError());
  MK(cudaMemcpyAsync(grad, h->g, sizeof(float) * h->P, cudaMemcpyDeviceToHost, h->stream));
  MK(cudaStreamSynchronize(h->stream));
  return TNSP_OK;
}

int tnsp_made_logq(tnsp_made* h, const int32_t* configs, int B, double* logq) {
  if (!h || !configs || !logq) return TNSP_E_ARG;
  MK(cudaSetDevice(h->device));
  int r = load_batch(h, configs, B);
  if (!r) r = forward(h, B);
  if (r) return r;
  k_logq<<<grid_for(B), 256, 0, h->stream>>>(h->o, h->x, B, h->n, h->lq, nullptr);
  MK(cudaGetLastError());
  MK(cudaMemcpyAsync(logq, h->lq, sizeof(double) * B, cudaMemcpyDeviceToHost, h->stream));
  MK(cudaStreamSynchronize(h->stream));
  return TNSP_OK;
}

int tnsp_made_sample(tnsp_made* h, int B, int32_t* configs, double* logq) {
  if (!h || !configs || B < 1 || B > h->cap) return TNSP_E_ARG;
  MK(cudaSetDevice(h->device));
  const int n = h->n;
  MK(cudaMemsetAsync(h->x, 0, sizeof(float) * (size_t)B * n, h->stream));
  for (int i = 0; i < n; ++i) {  // o_i depends on x_0..x_{i-1} only: one forward pass per site
    int r = forward(h, B);
    if (r) return r;
    k_sample_site<<<grid_for(B), 256, 0, h->stream>>>(h->o, h->x, B, n, i, h->seed, h->draws++);
  }
  int r = forward(h, B);
  if (r) return r;
  k_logq<<<grid_for(B), 256, 0, h->stream>>>(h->o, h->x, B, n, h->lq, nullptr);
  k_x_to_conf<<<grid_for((long long)B * n), 256, 0, h->stream>>>(h->x, (long long)B * n, h->conf);
  MK(cudaGetLastError());
  MK(cudaMemcpyAsync(configs, h->conf, sizeof(int32_t) * (size_t)B * n, cudaMemcpyDeviceToHost, h->stream));
  if (logq) MK(cudaMemcpyAsync(logq, h->lq, sizeof(double) * B, cudaMemcpyDeviceToHost, h->stream));
  MK(cudaStreamSynchronize(h->stream));
  return TNSP_OK;
}

}  // extern "C"
