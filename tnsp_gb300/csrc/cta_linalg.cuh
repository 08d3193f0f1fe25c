// CTA-cooperative dense linear algebra for one Markov chain per thread block.
//
// Every routine here is called by all threads of the block with identical arguments and ends
// with a __syncthreads(); operands live in global memory (this block's scratch slot) and are
// row-major unless stated.  The element type T is double (the FP64 sampler), dd (double-float,
// ddfloat.cuh) or float; reductions that decide control flow are done in the element type.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "ddfloat.cuh"

namespace tnsp {

constexpr int kThreads = 128;
constexpr int kWarps = kThreads / 32;

template <class T> struct Eps;
template <> struct Eps<double> {
  static __device__ __forceinline__ double value() { return 1.1102230246251565e-16; }
};
template <> struct Eps<float> {
  static __device__ __forceinline__ float value() { return 5.9604645e-08f; }
};
// double-float: 2^-44.  Its dot products err by up to ~2^-46 of the operands' magnitudes (float64's
// fused multiply-add rounds once, relative to the result), so the Jacobi stopping test
// |g| <= eps*len*sqrt(ab) needs this margin on the 216-long sector vectors of a Dcut=36, D=6 lattice
template <> struct Eps<dd> {
  static __device__ __forceinline__ dd value() { return dd(5.684342e-14f, 0.f); }
};

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}
__device__ __forceinline__ float warp_sum(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}
__device__ __forceinline__ dd warp_sum(dd v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = v + shfl_xor(v, o);
  return v;
}
template <class T> __device__ __forceinline__ T warp_max(T v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
  return v;
}
__device__ __forceinline__ dd warp_max(dd v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fmax(v, shfl_xor(v, o));
  return v;
}

// Tangent of the one-sided Jacobi rotation angle, t = sign(zeta) / (|zeta| + sqrt(1 + zeta^2)).  For
// double-float, zeta^2 overflows float's exponent range on strongly graded pairs (|zeta| ~ 1e21 next
// to the noise floor), which would make t = 0 and the pair never converge; above 2^40 the series
// value t = 1 / (2 zeta) is used (relative error below zeta^-2).
template <class T> __device__ __forceinline__ T jacobi_tan(T zeta) {
  return (zeta >= 0 ? (T)1 : (T)-1) / (fabs(zeta) + sqrt((T)1 + zeta * zeta));
}
__device__ __forceinline__ dd jacobi_tan(dd zeta) {
  if (fabs(zeta) > dd(1.0995116e12f, 0.f)) return dd(1.f, 0.f) / (dd(2.f, 0.f) * zeta);
  return (zeta >= dd(0.f, 0.f) ? dd(1.f, 0.f) : dd(-1.f, 0.f)) / (fabs(zeta) + sqrt(dd(1.f, 0.f) + zeta * zeta));
}

// Plane rotation of one element pair: (u, v) -> (c u - s v, s u + c v).
template <class T> __device__ __forceinline__ void rotate_pair(T c, T s, T& u, T& v) {
  const T x = u, y = v;
  u = c * x - s * y;
  v = s * x + c * y;
}
__device__ __forceinline__ void rotate_pair(dd c, dd s, dd& u, dd& v) {
  const dd x = u, y = v;
  u = dd_lincomb(c, x, -s, y);
  v = dd_lincomb(s, x, c, y);
}

// Rotates the element pairs (x[r], y[r]), r = lane, lane + 32, ... < n, two per step so that the
// dependent chains of two elements interleave (the same arithmetic per element as one at a time).
template <class T> __device__ __forceinline__ void rotate_vectors(T c, T s, T* x, T* y, int n, int lane) {
  int r = lane;
  for (; r + 32 < n; r += 64) {
    T u0 = x[r], v0 = y[r], u1 = x[r + 32], v1 = y[r + 32];
    rotate_pair(c, s, u0, v0);
    rotate_pair(c, s, u1, v1);
    x[r] = u0;
    y[r] = v0;
    x[r + 32] = u1;
    y[r + 32] = v1;
  }
  if (r < n) rotate_pair(c, s, x[r], y[r]);
}

// Shared-memory accumulation of a threshold estimate (order-independent to rounding only).
__device__ __forceinline__ void shared_accumulate(double* p, double v) { atomicAdd(p, v); }
__device__ __forceinline__ void shared_accumulate(float* p, float v) { atomicAdd(p, v); }
__device__ __forceinline__ void shared_accumulate(dd* p, dd v) { atomicAdd(&p->hi, v.hi + v.lo); }

// Block-wide sum; `red` is shared scratch of kWarps doubles.  Result broadcast to all threads.
template <class T> __device__ T block_sum(T v, T* red) {
  v = warp_sum(v);
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  __syncthreads();
  if (lane == 0) red[w] = v;
  __syncthreads();
  T r = 0;
#pragma unroll
  for (int i = 0; i < kWarps; ++i) r += red[i];
  __syncthreads();
  return r;
}

template <class T> __device__ T block_max(T v, T* red) {
  v = warp_max(v);
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  __syncthreads();
  if (lane == 0) red[w] = v;
  __syncthreads();
  T r = 0;
#pragma unroll
  for (int i = 0; i < kWarps; ++i) r = fmax(r, red[i]);
  __syncthreads();
  return r;
}

// Rescales x[0..n) by a power of two so that max|x| lies in [0.5, 1); returns the exponent e with
// x_old = x_new * 2^e (exact: a power-of-two scaling never rounds).  All-zero input: e = 0.
template <class T> __device__ int block_normalize(T* x, long n, T* red) {
  T m = 0;
  for (long i = threadIdx.x; i < n; i += blockDim.x) m = fmax(m, fabs(x[i]));
  m = block_max(m, red);
  if (!(m > 0) || !isfinite(m)) return 0;
  int e;
  frexp((double)m, &e);
  const T s = (T)ldexp(1.0, -e);
  for (long i = threadIdx.x; i < n; i += blockDim.x) x[i] *= s;
  __syncthreads();
  return e;
}

// C[m x n] = A[m x k] * B[k x n]; A has row stride lda, B row stride ldb, C row stride ldc.
// Each thread owns a 2x2 register tile of C.
template <class T>
__device__ void block_gemm(int m, int n, int k, const T* __restrict__ A, int lda, const T* __restrict__ B, int ldb,
                           T* __restrict__ C, int ldc) {
  const int tm = (m + 1) >> 1, tn = (n + 1) >> 1;
  const long tiles = (long)tm * tn;
  for (long t = threadIdx.x; t < tiles; t += blockDim.x) {
    const int i0 = (int)(t / tn) * 2, j0 = (int)(t % tn) * 2;
    const bool i1ok = i0 + 1 < m, j1ok = j0 + 1 < n;
    T c00 = 0, c01 = 0, c10 = 0, c11 = 0;
    const T* a0 = A + (long)i0 * lda;
    const T* a1 = A + (long)(i1ok ? i0 + 1 : i0) * lda;
    for (int p = 0; p < k; ++p) {
      const T* b = B + (long)p * ldb;
      const T b0 = b[j0], b1 = j1ok ? b[j0 + 1] : (T)0;
      const T x0 = a0[p], x1 = a1[p];
      c00 = fma(x0, b0, c00);
      c01 = fma(x0, b1, c01);
      c10 = fma(x1, b0, c10);
      c11 = fma(x1, b1, c11);
    }
    C[(long)i0 * ldc + j0] = c00;
    if (j1ok) C[(long)i0 * ldc + j0 + 1] = c01;
    if (i1ok) {
      C[(long)(i0 + 1) * ldc + j0] = c10;
      if (j1ok) C[(long)(i0 + 1) * ldc + j0 + 1] = c11;
    }
  }
  __syncthreads();
}

// Householder QR of the row-major m x n matrix M (overwritten).  Writes Q (m x kk, row-major,
// kk = min(m, n)) to Q and R (kk x n, row-major) to R.  tau: kk scratch values.
// Reflector j: H_j = I - tau_j v v^T, v_j = 1, v below the diagonal stored in column j of M
// (the LAPACK dgeqrf convention; any orthogonal gauge is acceptable to the callers).
template <class T>
__device__ void block_qr(int m, int n, T* M, T* Q, T* R, T* tau, T* red) {
  const int kk = m < n ? m : n;
  __shared__ T s_beta, s_tau, s_scale;
  for (int j = 0; j < kk; ++j) {
    // norm of M[j+1:m, j]
    T part = 0;
    for (int r = j + 1 + threadIdx.x; r < m; r += blockDim.x) {
      const T x = M[(long)r * n + j];
      part = fma(x, x, part);
    }
    const T sigma = block_sum(part, red);
    if (threadIdx.x == 0) {
      const T alpha = M[(long)j * n + j];
      if (sigma == (T)0) {
        s_tau = 0;
        s_beta = alpha;
        s_scale = 0;
      } else {
        T beta = sqrt(alpha * alpha + sigma);
        if (alpha > 0) beta = -beta;
        s_tau = (beta - alpha) / beta;
        s_scale = (T)1 / (alpha - beta);
        s_beta = beta;
      }
      tau[j] = s_tau;
    }
    __syncthreads();
    const T tj = s_tau, sc = s_scale;
    if (tj != (T)0) {
      for (int r = j + 1 + threadIdx.x; r < m; r += blockDim.x) M[(long)r * n + j] *= sc;
    }
    __syncthreads();
    if (threadIdx.x == 0) M[(long)j * n + j] = s_beta;
    // apply H_j to columns j+1..n-1: warp per column
    if (tj != (T)0) {
      const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
      for (int c = j + 1 + w; c < n; c += kWarps) {
        T d = lane == 0 ? M[(long)j * n + c] : (T)0;
        for (int r = j + 1 + lane; r < m; r += 32) d = fma(M[(long)r * n + j], M[(long)r * n + c], d);
        d = warp_sum(d) * tj;
        if (lane == 0) M[(long)j * n + c] -= d;
        for (int r = j + 1 + lane; r < m; r += 32) M[(long)r * n + c] -= d * M[(long)r * n + j];
      }
    }
    __syncthreads();
  }
  // R = upper triangle of the first kk rows
  for (long t = threadIdx.x; t < (long)kk * n; t += blockDim.x) {
    const int i = (int)(t / n), c = (int)(t % n);
    R[t] = c >= i ? M[(long)i * n + c] : (T)0;
  }
  // Q = H_0 ... H_{kk-1} [I; 0], accumulated backwards
  for (long t = threadIdx.x; t < (long)m * kk; t += blockDim.x) {
    const int i = (int)(t / kk), c = (int)(t % kk);
    Q[t] = i == c ? (T)1 : (T)0;
  }
  __syncthreads();
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  for (int j = kk - 1; j >= 0; --j) {
    const T tj = tau[j];
    if (tj != (T)0) {
      for (int c = j + w; c < kk; c += kWarps) {
        T d = lane == 0 ? Q[(long)j * kk + c] : (T)0;
        for (int r = j + 1 + lane; r < m; r += 32) d = fma(M[(long)r * n + j], Q[(long)r * kk + c], d);
        d = warp_sum(d) * tj;
        if (lane == 0) Q[(long)j * kk + c] -= d;
        for (int r = j + 1 + lane; r < m; r += 32) Q[(long)r * kk + c] -= d * M[(long)r * n + j];
      }
    }
    __syncthreads();
  }
}

// One-sided (Hestenes) Jacobi on nv vectors X[j][0..len) (vector-major), accumulating the same
// rotations into Vr[j][0..nv) (initialised to the identity here).  Pairs are visited in the
// round-robin (circle) order, one warp per pair.  Returns the number of sweeps, or -1 if the
// sweep limit was reached without convergence.
template <class T>
__device__ int block_jacobi(int nv, int len, T* X, T* Vr, int max_sweeps) {
  __shared__ int s_rot;
  for (long t = threadIdx.x; t < (long)nv * nv; t += blockDim.x) Vr[t] = (t / nv == t % nv) ? (T)1 : (T)0;
  __syncthreads();
  if (nv < 2) return 0;
  const int np = nv + (nv & 1);  // padded to even; index nv is a dummy
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  // Relative orthogonality target eps*max(len, 32) (rounding of a dot product of short vectors
  // would otherwise hover at the target).  A vector whose squared norm is below tol^2 *
  // max_j |x_j|^2 is rounding noise (a numerically zero singular value, which the callers
  // discard); pairs involving one are not rotated, which keeps graded noise-vs-signal pairs from
  // oscillating at the tolerance.
  const T tol = Eps<T>::value() * (T)(len > 32 ? len : 32);
  __shared__ T s_red[kWarps];
  for (int sweep = 0; sweep < max_sweeps; ++sweep) {
    T mx = 0;
    for (int j = w; j < nv; j += kWarps) {
      T a = 0;
      for (int r = lane; r < len; r += 32) a = fma(X[(long)j * len + r], X[(long)j * len + r], a);
      mx = fmax(mx, warp_sum(a));
    }
    mx = block_max(mx, s_red);
    const T noise2 = mx * tol * tol;
    if (threadIdx.x == 0) s_rot = 0;
    __syncthreads();
    int rot = 0;
    for (int round = 0; round < np - 1; ++round) {
      for (int k = w; k < np / 2; k += kWarps) {
        const int i = k == 0 ? 0 : ((k + round - 1) % (np - 1)) + 1;
        const int j = ((np - 1 - k + round - 1) % (np - 1)) + 1;
        if (i >= nv || j >= nv) continue;
        T* xi = X + (long)i * len;
        T* xj = X + (long)j * len;
        T a = 0, b = 0, g = 0;
        for (int r = lane; r < len; r += 32) {
          const T u = xi[r], v = xj[r];
          a = fma(u, u, a);
          b = fma(v, v, b);
          g = fma(u, v, g);
        }
        a = warp_sum(a);
        b = warp_sum(b);
        g = warp_sum(g);
        if (a <= noise2 || b <= noise2) continue;
        if (!(fabs(g) > tol * sqrt(a) * sqrt(b))) continue;
        rot = 1;
        const T zeta = (b - a) / ((T)2 * g);
        const T t = jacobi_tan(zeta);
        const T c = (T)1 / sqrt((T)1 + t * t);
        const T s = c * t;
        rotate_vectors(c, s, xi, xj, len, lane);
        T* vi = Vr + (long)i * nv;
        T* vj = Vr + (long)j * nv;
        rotate_vectors(c, s, vi, vj, nv, lane);
      }
      __syncthreads();
    }
    if (rot) s_rot = 1;  // benign race: every writer stores 1
    __syncthreads();
    const int any = s_rot;
    __syncthreads();
    if (!any) return sweep + 1;
  }
  return -1;
}


// ---------------------------------------------------------------------------------------------
// block-wide integer scan and stable compaction
// ---------------------------------------------------------------------------------------------
// Inclusive prefix sum of one int per thread; `sh` is shared scratch of kWarps + 1 ints.  The block
// total is returned in *total.
__device__ __forceinline__ int block_inclusive_scan(int v, int* sh, int* total) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int y = __shfl_up_sync(0xffffffffu, v, o);
    if (lane >= o) v += y;
  }
  __syncthreads();
  if (lane == 31) sh[w] = v;
  __syncthreads();
  if (threadIdx.x == 0) {
    int acc = 0;
    for (int i = 0; i < kWarps; ++i) {
      const int t = sh[i];
      sh[i] = acc;
      acc += t;
    }
    sh[kWarps] = acc;
  }
  __syncthreads();
  v += sh[w];
  *total = sh[kWarps];
  __syncthreads();
  return v;
}

// Writes, in increasing order, every i in [0, n) with pred(i) to out; returns the count.
template <class Pred> __device__ int block_compact(int n, Pred pred, int* out, int* sh) {
  const int chunk = (n + (int)blockDim.x - 1) / (int)blockDim.x;
  const int beg = threadIdx.x * chunk;
  const int end = beg + chunk < n ? beg + chunk : n;
  int cnt = 0;
  for (int i = beg; i < end; ++i) cnt += pred(i) ? 1 : 0;
  int total;
  int pos = block_inclusive_scan(cnt, sh, &total) - cnt;
  for (int i = beg; i < end; ++i)
    if (pred(i)) out[pos++] = i;
  __syncthreads();
  return total;
}

// ---------------------------------------------------------------------------------------------
// column-major Householder QR (LAPACK geqr2 / org2r conventions, any orthogonal gauge is fine)
// ---------------------------------------------------------------------------------------------
// G: m x n column-major (ld = m), overwritten by R (upper triangle) and the reflectors below it.
template <class T> __device__ void block_geqrf_cm(int m, int n, T* G, T* tau, T* red) {
  const int kk = m < n ? m : n;
  __shared__ T s_beta, s_tau, s_scale;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  for (int j = 0; j < kk; ++j) {
    T* gj = G + (long)j * m;
    T part = 0;
    for (int r = j + 1 + threadIdx.x; r < m; r += blockDim.x) part = fma(gj[r], gj[r], part);
    const T sigma = block_sum(part, red);
    if (threadIdx.x == 0) {
      const T alpha = gj[j];
      if (sigma == (T)0) {
        s_tau = 0;
        s_beta = alpha;
        s_scale = 0;
      } else {
        T beta = sqrt(alpha * alpha + sigma);
        if (alpha > 0) beta = -beta;
        s_tau = (beta - alpha) / beta;
        s_scale = (T)1 / (alpha - beta);
        s_beta = beta;
      }
      tau[j] = s_tau;
    }
    __syncthreads();
    const T tj = s_tau, sc = s_scale;
    if (tj != (T)0)
      for (int r = j + 1 + threadIdx.x; r < m; r += blockDim.x) gj[r] *= sc;
    __syncthreads();
    if (threadIdx.x == 0) gj[j] = s_beta;
    if (tj != (T)0) {
      for (int c = j + 1 + w; c < n; c += kWarps) {
        T* gc = G + (long)c * m;
        T d = lane == 0 ? gc[j] : (T)0;
        for (int r = j + 1 + lane; r < m; r += 32) d = fma(gj[r], gc[r], d);
        d = warp_sum(d) * tj;
        if (lane == 0) gc[j] -= d;
        for (int r = j + 1 + lane; r < m; r += 32) gc[r] -= d * gj[r];
      }
    }
    __syncthreads();
  }
}

// Forms Q (m x k, first k columns of G, column-major) in place from block_geqrf_cm's reflectors.
template <class T> __device__ void block_orgqr_cm(int m, int k, T* G, const T* tau) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  for (int i = k - 1; i >= 0; --i) {
    T* gi = G + (long)i * m;
    const T ti = tau[i];
    if (i < k - 1) {
      if (threadIdx.x == 0) gi[i] = (T)1;
      __syncthreads();
      if (ti != (T)0) {
        for (int c = i + 1 + w; c < k; c += kWarps) {
          T* gc = G + (long)c * m;
          T d = 0;
          for (int r = i + lane; r < m; r += 32) d = fma(gi[r], gc[r], d);
          d = warp_sum(d) * ti;
          for (int r = i + lane; r < m; r += 32) gc[r] -= d * gi[r];
        }
      }
      __syncthreads();
    }
    for (int r = i + 1 + threadIdx.x; r < m; r += blockDim.x) gi[r] *= -ti;
    for (int r = threadIdx.x; r < i; r += blockDim.x) gi[r] = (T)0;
    if (threadIdx.x == 0) gi[i] = (T)1 - ti;
    __syncthreads();
  }
}



// ---------------------------------------------------------------------------------------------
// one-sided Jacobi on several independent vector sets at once
// ---------------------------------------------------------------------------------------------
// Set t has nv[t] vectors of length len[t] at Xs[t] (vector-major) and accumulates its rotations
// into Vs[t] (nv[t] x nv[t], set to the identity here); each set may live in shared or global memory.  Every set follows its own
// circle ordering and convergence test (rotation rule and tolerance of block_jacobi, noise floor
// tol^2 * |A|_F^2), but all sets advance together: a block barrier ends one round of every set, so
// the number of barriers is set by the largest set instead of the sum over sets.  Pairs of a round
// are spread over the warps.  Returns the largest sweep count, or -1 if a set hit max_sweeps.
template <class T, int MAXS>
__device__ int block_jacobi_multi(int ns, const int* nv, const int* len, T* const* Xs, T* const* Vs, int max_sweeps) {
  __shared__ int s_np[MAXS], s_pp[MAXS + 1], s_rot[MAXS], s_done[MAXS], s_sweeps[MAXS];
  __shared__ T s_noise[MAXS];
  __shared__ int s_active, s_fail;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  for (int t = 0; t < ns; ++t)
    for (long e = threadIdx.x; e < (long)nv[t] * nv[t]; e += blockDim.x)
      Vs[t][e] = (e / nv[t] == e % nv[t]) ? (T)1 : (T)0;
  // squared Frobenius norm of each set (invariant under the rotations, >= sigma_max^2): the noise
  // floor below which a vector is left alone is tol^2 * |A|_F^2
  if (threadIdx.x < MAXS) s_noise[threadIdx.x] = 0;
  __syncthreads();
  for (int t = 0; t < ns; ++t) {
    T acc = 0;
    for (long e = threadIdx.x; e < (long)nv[t] * len[t]; e += blockDim.x) acc = fma(Xs[t][e], Xs[t][e], acc);
    acc = warp_sum(acc);
    if (lane == 0) shared_accumulate(&s_noise[t], acc);
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    int pp = 0;
    for (int t = 0; t < ns; ++t) {
      const T tol = Eps<T>::value() * (T)(len[t] > 32 ? len[t] : 32);
      s_noise[t] = s_noise[t] * tol * tol;
      s_np[t] = nv[t] + (nv[t] & 1);
      s_pp[t] = pp;
      pp += nv[t] >= 2 ? s_np[t] / 2 : 0;
      s_rot[t] = 0;
      s_done[t] = nv[t] < 2;
      s_sweeps[t] = 0;
    }
    s_pp[ns] = pp;
    s_fail = 0;
  }
  __syncthreads();
  for (int g = 0;; ++g) {
    // pairs of round g of every unfinished set
    const int total = s_pp[ns];
    for (int p = w; p < total; p += kWarps) {
      int t = 0;
      while (p >= s_pp[t + 1]) ++t;
      if (s_done[t]) continue;
      const int np = s_np[t], k = p - s_pp[t], rounds = np - 1;
      const int round = g % rounds;
      const int i = k == 0 ? 0 : ((k + round - 1) % rounds) + 1;
      const int j = ((np - 1 - k + round - 1) % rounds) + 1;
      if (i >= nv[t] || j >= nv[t]) continue;
      const int L = len[t];
      T* xi = Xs[t] + (long)i * L;
      T* xj = Xs[t] + (long)j * L;
      T a = 0, b = 0, c2 = 0;
      for (int r = lane; r < L; r += 32) {
        const T u = xi[r], v = xj[r];
        a = fma(u, u, a);
        b = fma(v, v, b);
        c2 = fma(u, v, c2);
      }
      a = warp_sum(a);
      b = warp_sum(b);
      c2 = warp_sum(c2);
      const T tol = Eps<T>::value() * (T)(L > 32 ? L : 32);
      if (a <= s_noise[t] || b <= s_noise[t]) continue;
      if (!(fabs(c2) > tol * sqrt(a) * sqrt(b))) continue;
      if (lane == 0) s_rot[t] = 1;
      const T zeta = (b - a) / ((T)2 * c2);
      const T tt = jacobi_tan(zeta);
      const T c = (T)1 / sqrt((T)1 + tt * tt);
      const T sn = c * tt;
      rotate_vectors(c, sn, xi, xj, L, lane);
      const int n = nv[t];
      T* vi = Vs[t] + (long)i * n;
      T* vj = Vs[t] + (long)j * n;
      rotate_vectors(c, sn, vi, vj, n, lane);
    }
    __syncthreads();
    // end of a sweep of some sets: converged or next sweep
    if (threadIdx.x == 0) {
      int active = 0;
      for (int t = 0; t < ns; ++t) {
        if (s_done[t]) continue;
        const int rounds = s_np[t] - 1;
        if ((g + 1) % rounds == 0) {
          ++s_sweeps[t];
          if (!s_rot[t]) {
            s_done[t] = 1;
          } else if (s_sweeps[t] >= max_sweeps) {
            s_done[t] = 1;
            s_fail = 1;
          }
          s_rot[t] = 0;
        }
        active += !s_done[t];
      }
      s_active = active;
    }
    __syncthreads();
    if (s_active == 0) break;
  }
  int mx = 0;
  for (int t = 0; t < ns; ++t) mx = max(mx, s_sweeps[t]);
  const int fail = s_fail;
  __syncthreads();
  return fail ? -1 : mx;
}


// ---------------------------------------------------------------------------------------------
// Householder QR with column pivoting (column-major), the preconditioner of the Jacobi SVD
// ---------------------------------------------------------------------------------------------
// G: m x n column-major (m >= n).  At step j the remaining column of largest norm (rows j..m) is
// swapped into position j (ties to the lower index); perm[j] records the original column.  On exit
// R is in the upper triangle and the reflectors below it, as in block_geqrf_cm.
template <class T> __device__ void block_geqp3_cm(int m, int n, T* G, T* tau, int* perm, T* red) {
  __shared__ T s_beta, s_tau, s_scale;
  __shared__ int s_piv;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  for (int j = threadIdx.x; j < n; j += blockDim.x) perm[j] = j;
  __syncthreads();
  for (int j = 0; j < n; ++j) {
    // pivot: largest trailing column norm (warp per column, thread 0 picks)
    if (threadIdx.x == 0) s_piv = j;
    __syncthreads();
    {
      __shared__ T s_best[kWarps];
      __shared__ int s_bidx[kWarps];
      T best = -1;
      int bidx = j;
      for (int c = j + w; c < n; c += kWarps) {
        const T* gc = G + (long)c * m;
        T a = 0;
        for (int r = j + lane; r < m; r += 32) a = fma(gc[r], gc[r], a);
        a = warp_sum(a);
        if (a > best) {
          best = a;
          bidx = c;
        }
      }
      if (lane == 0) {
        s_best[w] = best;
        s_bidx[w] = bidx;
      }
      __syncthreads();
      if (threadIdx.x == 0) {
        T b = -1;
        int bi = j;
        for (int k = 0; k < kWarps; ++k)
          if (s_best[k] > b || (s_best[k] == b && s_bidx[k] < bi)) {
            b = s_best[k];
            bi = s_bidx[k];
          }
        s_piv = bi;
      }
      __syncthreads();
    }
    const int p = s_piv;
    if (p != j) {
      T* gj = G + (long)j * m;
      T* gp = G + (long)p * m;
      for (int r = threadIdx.x; r < m; r += blockDim.x) {
        const T t = gj[r];
        gj[r] = gp[r];
        gp[r] = t;
      }
      if (threadIdx.x == 0) {
        const int t = perm[j];
        perm[j] = perm[p];
        perm[p] = t;
      }
      __syncthreads();
    }
    // Householder step j (as block_geqrf_cm)
    T* gj = G + (long)j * m;
    T part = 0;
    for (int r = j + 1 + threadIdx.x; r < m; r += blockDim.x) part = fma(gj[r], gj[r], part);
    const T sigma = block_sum(part, red);
    if (threadIdx.x == 0) {
      const T alpha = gj[j];
      if (sigma == (T)0) {
        s_tau = 0;
        s_beta = alpha;
        s_scale = 0;
      } else {
        T beta = sqrt(alpha * alpha + sigma);
        if (alpha > 0) beta = -beta;
        s_tau = (beta - alpha) / beta;
        s_scale = (T)1 / (alpha - beta);
        s_beta = beta;
      }
      tau[j] = s_tau;
    }
    __syncthreads();
    const T tj = s_tau, sc = s_scale;
    if (tj != (T)0)
      for (int r = j + 1 + threadIdx.x; r < m; r += blockDim.x) gj[r] *= sc;
    __syncthreads();
    if (threadIdx.x == 0) gj[j] = s_beta;
    if (tj != (T)0) {
      for (int c = j + 1 + w; c < n; c += kWarps) {
        T* gc = G + (long)c * m;
        T d = lane == 0 ? gc[j] : (T)0;
        for (int r = j + 1 + lane; r < m; r += 32) d = fma(gj[r], gc[r], d);
        d = warp_sum(d) * tj;
        if (lane == 0) gc[j] -= d;
        for (int r = j + 1 + lane; r < m; r += 32) gc[r] -= d * gj[r];
      }
    }
    __syncthreads();
  }
}

}  // namespace tnsp
