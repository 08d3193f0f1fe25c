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

// Lane-group primitives of the Jacobi routines: a rotation pair is handled by a group of kJG lanes, so
// a warp works on 32 / kJG pairs at once and the latency-bound parts of a pair step (the reductions
// of its three dot products and the scalar angle computation) run for all of them in the same
// instructions.
constexpr int kJG = 8;
__device__ __forceinline__ double shfl_xor(double v, int o) { return __shfl_xor_sync(0xffffffffu, v, o); }
__device__ __forceinline__ float shfl_xor(float v, int o) { return __shfl_xor_sync(0xffffffffu, v, o); }
// Sum over the aligned group of G lanes (every lane of the warp must call it).
template <int G, class T> __device__ __forceinline__ T group_sum(T v) {
#pragma unroll
  for (int o = G / 2; o > 0; o >>= 1) v = v + shfl_xor(v, o);
  return v;
}
// Rotates the element pairs (x[r], y[r]) of a G-lane group, r = sl, sl + G, ... < n, two per step so
// that the dependent chains of two elements interleave (the same arithmetic per element).
template <int G, class T> __device__ __forceinline__ void rotate_group(T c, T s, T* x, T* y, int n, int sl) {
  int r = sl;
  for (; r + G < n; r += 2 * G) {
    T u0 = x[r], v0 = y[r], u1 = x[r + G], v1 = y[r + G];
    rotate_pair(c, s, u0, v0);
    rotate_pair(c, s, u1, v1);
    x[r] = u0;
    y[r] = v0;
    x[r + G] = u1;
    y[r + G] = v1;
  }
  if (r < n) rotate_pair(c, s, x[r], y[r]);
}
// One pair step of one-sided Jacobi on vectors xi, xj (length len) with their accumulated rotations
// vi, vj (length n), by a G-lane group (sub-lane sl).  Every lane of the warp calls it; groups without
// a pair pass act = false (their pointers are not touched).  Returns true if the pair was rotated.
// Pairs where either vector is below the noise floor, or that are orthogonal to tol, are left alone.
template <int G, class T>
__device__ __forceinline__ bool jacobi_pair(bool act, T* xi, T* xj, int len, T* vi, T* vj, int n, T noise2, T tol,
                                            int sl) {
  T a = 0, b = 0, g = 0;
  if (act) {
    for (int r = sl; r < len; r += G) {
      const T u = xi[r], v = xj[r];
      a = fma(u, u, a);
      b = fma(v, v, b);
      g = fma(u, v, g);
    }
  }
  a = group_sum<G>(a);
  b = group_sum<G>(b);
  g = group_sum<G>(g);
  if (!act || a <= noise2 || b <= noise2) return false;
  if (!(fabs(g) > tol * sqrt(a) * sqrt(b))) return false;
  const T zeta = (b - a) / ((T)2 * g);
  const T t = jacobi_tan(zeta);
  const T c = (T)1 / sqrt((T)1 + t * t);
  const T s = c * t;
  rotate_group<G>(c, s, xi, xj, len, sl);
  if (vi) rotate_group<G>(c, s, vi, vj, n, sl);  // no accumulation when the caller passes none
  return true;
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
template <class T> __device__ __noinline__ int block_normalize(T* x, long n, T* red) {
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

// One-sided (Hestenes) Jacobi on nv vectors X[j][0..len) (vector-major), accumulating the same
// rotations into Vr[j][0..nv) (initialised to the identity here; Vr = nullptr: not accumulated).  Pairs are visited in the
// round-robin (circle) order, one kJG-lane group per pair.  Returns the number of sweeps, or -1 if
// the sweep limit was reached without convergence.
template <class T>
__device__ __noinline__ int block_jacobi(int nv, int len, T* X, T* Vr, int max_sweeps) {
  __shared__ int s_rot;
  if (Vr)
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
    const int grp = lane / kJG, sl = lane % kJG;
    for (int round = 0; round < np - 1; ++round) {
      for (int base = w * (32 / kJG); base < np / 2; base += kWarps * (32 / kJG)) {  // warp-uniform
        const int k = base + grp;
        int i = 0, j = 0;
        bool act = k < np / 2;
        if (act) {
          i = k == 0 ? 0 : ((k + round - 1) % (np - 1)) + 1;
          j = ((np - 1 - k + round - 1) % (np - 1)) + 1;
          act = i < nv && j < nv;
        }
        if (!act) i = j = 0;
        if (jacobi_pair<kJG>(act, X + (long)i * len, X + (long)j * len, len, Vr ? Vr + (long)i * nv : nullptr,
                             Vr ? Vr + (long)j * nv : nullptr, nv, noise2, tol, sl))
          rot = 1;
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
// column-major Householder QR (LAPACK geqr2 conventions, any orthogonal gauge is fine); Q is never
// formed: its reflectors are applied where it is used (block_ormqr_panel in sampler_kernels.cuh)
// ---------------------------------------------------------------------------------------------
// Applies the reflector H = I - tau v v^T to columns c0..n-1 of the column-major m-row matrix G, one
// kJG-lane group per column.  v occupies rows r0..m-1 of column-major storage `v`; with unit_head
// its row-r0 entry is an implicit 1 (geqrf layout: R's diagonal sits there), else it is stored.
template <class T>
__device__ __forceinline__ void apply_reflector_cm(int m, int r0, const T* v, bool unit_head, T tau, T* G, int c0,
                                                   int n) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, grp = lane / kJG, sl = lane % kJG;
  const int rs = unit_head ? r0 + 1 : r0;
  for (int base = c0 + w * (32 / kJG); base < n; base += kWarps * (32 / kJG)) {  // warp-uniform
    const int c = base + grp;
    const bool act = c < n;
    T* gc = G + (long)(act ? c : base) * m;
    T d = (act && unit_head && sl == 0) ? gc[r0] : (T)0;
    if (act)
      for (int r = rs + sl; r < m; r += kJG) d = fma(v[r], gc[r], d);
    d = group_sum<kJG>(d) * tau;
    if (act) {
      if (unit_head && sl == 0) gc[r0] -= d;
      for (int r = rs + sl; r < m; r += kJG) gc[r] -= d * v[r];
    }
  }
}

// G: m x n column-major (ld = m), overwritten by R (upper triangle) and the reflectors below it.
template <class T> __device__ __noinline__ void block_geqrf_cm(int m, int n, T* G, T* tau, T* red) {
  const int kk = m < n ? m : n;
  __shared__ T s_beta, s_tau, s_scale;
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
    if (tj != (T)0) apply_reflector_cm(m, j, gj, true, tj, G, j + 1, n);
    __syncthreads();
  }
}

// ---------------------------------------------------------------------------------------------
// blocked Householder QR for matrices staged in global memory (compact WY form of a panel:
// H_0 H_1 ... H_{b-1} = I - V Tw V^T, LAPACK larft / larfb)
// ---------------------------------------------------------------------------------------------
// The unblocked routines above read and write the whole trailing matrix once per reflector; from
// global memory that is one latency-bound pass per column.  The panel routines factorise (or apply)
// up to kNB columns at a time in shared memory and apply them to the rest of the matrix as one block
// reflector: two reads and one write of each trailing column per panel, with kNB independent dot
// products per lane in flight.  Results equal the unblocked ones up to rounding (same reflectors).
constexpr int kNB = 8;

// Tw (jb x jb upper triangular, row stride kNB) of the explicit unit-lower panel V (pm x jb,
// column-major, ld pm; zeros above the unit diagonal) and its scalars tau:
//   Tw[i][i] = tau_i,   Tw[0:i][i] = -tau_i Tw[0:i][0:i] (V[:, 0:i]^T v_i).
// Y (kNB x kNB) is scratch for the Gram entries v_a . v_b, a < b.  Both live in shared memory.
template <class T> __device__ void panel_tw(int pm, int jb, const T* V, const T* tau, T* Y, T* Tw) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, grp = lane / kJG, sl = lane % kJG;
  const int npairs = jb * (jb - 1) / 2;
  for (int base = w * (32 / kJG); base < npairs; base += kWarps * (32 / kJG)) {  // warp-uniform
    const int p = base + grp;
    const bool act = p < npairs;
    int a = 0, b = 1;
    if (act) {  // pairs enumerated by b = 1, 2, ... with a = 0 .. b-1
      int q = p;
      while (q >= b) {
        q -= b;
        ++b;
      }
      a = q;
    }
    T d = 0;
    if (act)  // v_b is zero above row b and 1 at it: the overlap starts at row b
      for (int r = b + sl; r < pm; r += kJG) d = fma(V[(long)a * pm + r], V[(long)b * pm + r], d);
    d = group_sum<kJG>(d);
    if (act && sl == 0) Y[a * kNB + b] = d;
  }
  __syncthreads();
  // column i of Tw from its columns < i; lane a owns row a (it reads only its own row and Y)
  if (threadIdx.x < 32) {
    for (int i = 0; i < jb; ++i) {
      if (lane < i) {
        T s = 0;
        for (int c = lane; c < i; ++c) s = fma(Tw[lane * kNB + c], Y[c * kNB + i], s);
        Tw[lane * kNB + i] = -tau[i] * s;
      } else if (lane == i) {
        Tw[i * kNB + i] = tau[i];
      }
    }
  }
  __syncthreads();
}

// A <- (I - V op(Tw) V^T) A on columns c0..n-1 of A (pm rows, column-major, ld lda); op(Tw) = Tw^T
// applies Q^T of the panel (the factorisation's trailing update), op(Tw) = Tw applies Q (forming Q).
// One kJG-lane group per column.  No barrier at the end.
template <class T, bool TRANS>
__device__ void apply_panel(int pm, int jb, const T* V, const T* Tw, T* A, long lda, int c0, int n) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, grp = lane / kJG, sl = lane % kJG;
  for (int base = c0 + w * (32 / kJG); base < n; base += kWarps * (32 / kJG)) {  // warp-uniform
    const int c = base + grp;
    const bool act = c < n;
    T* ac = A + (long)(act ? c : base) * lda;
    T y[kNB];
#pragma unroll
    for (int i = 0; i < kNB; ++i) y[i] = 0;
    if (act)
      for (int r = sl; r < pm; r += kJG) {
        const T x = ac[r];
#pragma unroll
        for (int i = 0; i < kNB; ++i)
          if (i < jb) y[i] = fma(V[(long)i * pm + r], x, y[i]);
      }
#pragma unroll
    for (int i = 0; i < kNB; ++i) y[i] = group_sum<kJG>(y[i]);
    // y <- op(Tw) y in place: Tw^T y (lower triangular) from the last entry down, Tw y (upper) up
    if (TRANS) {
#pragma unroll
      for (int i = kNB - 1; i >= 0; --i) {
        T s = 0;
#pragma unroll
        for (int a = 0; a <= i; ++a)
          if (i < jb) s = fma(Tw[a * kNB + i], y[a], s);
        y[i] = s;
      }
    } else {
#pragma unroll
      for (int i = 0; i < kNB; ++i) {
        T s = 0;
#pragma unroll
        for (int b = i; b < kNB; ++b)
          if (b < jb) s = fma(Tw[i * kNB + b], y[b], s);
        y[i] = s;
      }
    }
    if (act)
      for (int r = sl; r < pm; r += kJG) {
        T s = 0;
#pragma unroll
        for (int i = 0; i < kNB; ++i)
          if (i < jb) s = fma(V[(long)i * pm + r], y[i], s);
        ac[r] -= s;
      }
  }
}

// Panel width for an m-row matrix with pcap elements of shared staging (0 or 1: not blocked).
__device__ __forceinline__ int panel_width(int m, long pcap) {
  const long room = pcap - 2L * kNB * kNB;
  if (m <= 0 || room < 2L * m) return 0;
  return room / m < kNB ? (int)(room / m) : kNB;
}

// Copies the panel G[r0.., c0..c0+jb) (pm rows, G column-major with ld m) to P (ld pm) or back.
template <class T> __device__ void panel_copy(int m, int pm, int jb, T* G, long goff, T* P, bool to_panel) {
  for (long e = threadIdx.x; e < (long)pm * jb; e += blockDim.x) {
    const int c = (int)(e / pm), r = (int)(e % pm);
    T* g = G + goff + (long)c * m + r;
    if (to_panel)
      P[e] = *g;
    else
      *g = P[e];
  }
}

// Zeros above the diagonal and ones on it: the explicit unit-lower V of a geqrf-layout panel.
template <class T> __device__ void panel_explicit(int pm, int jb, T* P) {
  for (int e = threadIdx.x; e < jb * jb; e += blockDim.x) {
    const int c = e / jb, r = e % jb;
    if (r <= c) P[(long)c * pm + r] = r == c ? (T)1 : (T)0;
  }
}

// block_geqrf_cm for G in global memory, blocked through the shared staging P (pcap elements).  With
// TwOut, the Tw factor of every panel (kNB x kNB, in panel order) is also written there.
template <class T>
__device__ __noinline__ void block_geqrf_panel(int m, int n, T* G, T* tau, T* red, T* P, long pcap, T* TwOut) {
  const int nb = panel_width(m, pcap);
  if (nb < 2) {
    block_geqrf_cm(m, n, G, tau, red);
    return;
  }
  const int kk = m < n ? m : n;
  for (int j0 = 0; j0 < kk; j0 += nb) {
    const int jb = kk - j0 < nb ? kk - j0 : nb, pm = m - j0;
    const long goff = (long)j0 * m + j0;
    T* Y = P + (long)pm * jb;
    T* Tw = Y + kNB * kNB;
    panel_copy(m, pm, jb, G, goff, P, true);
    __syncthreads();
    block_geqrf_cm(pm, jb, P, tau + j0, red);  // ends with a barrier
    panel_copy(m, pm, jb, G, goff, P, false);  // R's rows of the panel and its reflectors
    __syncthreads();
    if (j0 + jb < n || TwOut) {
      panel_explicit(pm, jb, P);
      __syncthreads();
      panel_tw(pm, jb, P, tau + j0, Y, Tw);  // ends with a barrier
      if (TwOut)
        for (int e = threadIdx.x; e < kNB * kNB; e += blockDim.x) TwOut[(long)(j0 / nb) * kNB * kNB + e] = Tw[e];
      if (j0 + jb < n) apply_panel<T, true>(pm, jb, P, Tw, G + j0, m, j0 + jb, n);
      __syncthreads();
    }
  }
}

// ---------------------------------------------------------------------------------------------
// one-sided Jacobi on several independent vector sets at once
// ---------------------------------------------------------------------------------------------
// Set t has nv[t] vectors of length len[t] at Xs[t] (vector-major) and accumulates its rotations
// into Vs[t] (nv[t] x nv[t], set to the identity here; Vs = nullptr: not accumulated); each set may
// live in shared or global memory.  Every set follows its own
// circle ordering and convergence test (rotation rule and tolerance of block_jacobi, noise floor
// tol^2 * |A|_F^2), but all sets advance together: a block barrier ends one round of every set, so
// the number of barriers is set by the largest set instead of the sum over sets.  Pairs of a round
// are spread over kJG-lane groups of all warps.  Returns the largest sweep count, or -1 if a set hit max_sweeps.
template <class T, int MAXS>
__device__ __noinline__ int block_jacobi_multi(int ns, const int* nv, const int* len, T* const* Xs, T* const* Vs, int max_sweeps) {
  __shared__ int s_np[MAXS], s_pp[MAXS + 1], s_rot[MAXS], s_done[MAXS], s_sweeps[MAXS];
  __shared__ T s_noise[MAXS];
  __shared__ int s_active, s_fail;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  if (Vs)
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
    // pairs of round g of every unfinished set, one kJG-lane group per pair
    const int total = s_pp[ns];
    const int grp = lane / kJG, sl = lane % kJG;
    for (int base = w * (32 / kJG); base < total; base += kWarps * (32 / kJG)) {  // warp-uniform
      const int p = base + grp;
      bool act = p < total;
      int t = 0, i = 0, j = 0;
      if (act) {
        while (p >= s_pp[t + 1]) ++t;
        act = !s_done[t];
      }
      if (act) {
        const int np = s_np[t], k = p - s_pp[t], rounds = np - 1;
        const int round = g % rounds;
        i = k == 0 ? 0 : ((k + round - 1) % rounds) + 1;
        j = ((np - 1 - k + round - 1) % rounds) + 1;
        act = i < nv[t] && j < nv[t];
      }
      const int L = act ? len[t] : 0, n = act ? nv[t] : 0;
      T* xi = act ? Xs[t] + (long)i * L : nullptr;
      T* xj = act ? Xs[t] + (long)j * L : nullptr;
      T* vi = (act && Vs) ? Vs[t] + (long)i * n : nullptr;
      T* vj = (act && Vs) ? Vs[t] + (long)j * n : nullptr;
      const T tol = Eps<T>::value() * (T)(L > 32 ? L : 32);
      const T noise = act ? s_noise[t] : (T)0;
      if (jacobi_pair<kJG>(act, xi, xj, L, vi, vj, n, noise, tol, sl) && sl == 0) s_rot[t] = 1;
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
template <class T> __device__ __noinline__ void block_geqp3_cm(int m, int n, T* G, T* tau, int* perm, T* red) {
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
    if (tj != (T)0) apply_reflector_cm(m, j, gj, true, tj, G, j + 1, n);
    __syncthreads();
  }
}

}  // namespace tnsp
