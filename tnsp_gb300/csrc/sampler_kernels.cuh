// Sweep sampling, local energy and gradient holes of a PEPS on one GPU (kernel templates; the
// instantiations live in sampler_f64.cu, sampler_dd.cu, sampler_f32.cu and sampler_mixed.cu).
//
// Two element types: T, the arithmetic of the factorisations (per-sector QR, pivoted QR and one-sided
// Jacobi SVD, their staging and factors), and S, the storage and arithmetic of everything else (site
// tensors, boundary lines, compression tensors, strip environments and their contractions).  The
// float64, double-float and float32 samplers use one type for both; the mixed sampler keeps the
// factorisations in double-float and stores and contracts in float32.
//
// One thread block owns one Markov chain at a time (persistent blocks stride over thousands of
// chains).  Inside a block the chain's boundary MPSs, strip environments and compression
// workspace live in the block's scratch slot in HBM; a lazily-validated cache mirrors the
// reference's lazy DAG (lazy_graph/lazy/__init__.py, tetragono/tetragono/auxiliaries/
// single_layer_auxiliaries.py:106-244): every cached tensor is a deterministic function of the
// chain's current configuration, so recomputing it yields the value the reference would read.
//
// Reference semantics restated here (file:line in USTC-TNS/TNSP):
//  * _two_line_to_one_line: contraction, QR sweep, truncating SVD sweep
//      (tetragono/tetragono/auxiliaries/single_layer_auxiliaries.py:462-498)
//  * strips, replace (two-site) and hole (single_layer_auxiliaries.py:254-312, 568-692, 710-729)
//  * SweepSampling._single_term / __call__ (tetragono/tetragono/sampling_lattice/sampling.py:117-154)
//  * Observer.__call__ (tetragono/tetragono/sampling_lattice/observer.py:313-415)
//  * TAT.random: std::mt19937_64 with libstdc++'s uniform_int / uniform_real (PyTAT/PyTAT.hpp:86-113)
#pragma once
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#include "cta_linalg.cuh"

namespace tnsp {

constexpr int kMaxL = 16;       // lattice extent limit (rows or columns)
constexpr int kMaxSites = kMaxL * kMaxL;
constexpr int kMtN = 312;
constexpr int kMaxSweepsJacobi = 60;   // default sweep limit of the one-sided Jacobi SVD
constexpr int kMaxSec = 96;     // charge sectors per factorised matrix
constexpr int kMaxChi = 1024;   // cut * Dmax
constexpr int kCounters = 16;   // per-slot counters: 4 flop classes + 12 phase cycle counters
enum { PH_TWOLINE = 0, PH_SECTORS, PH_QR, PH_RABSORB, PH_JACOBI, PH_SVDOUT, PH_USABSORB, PH_STRIP, PH_HOLE,
       PH_OBSERVE, PH_NORMALIZE, PH_OTHER };
// counter slots 12..15 (phases HOLE, NORMALIZE, OTHER are not timed) hold event counts
enum { CT_COMPRESS = 12, CT_JACOBI_CALLS = 14, CT_JACOBI_SWEEPS = 15 };

enum { ST_SVD_NOCONV = 1, ST_NONFINITE = 2, ST_UNSUPPORTED = 4, ST_ZERO_WS = 8 };
enum { F_UP = 0, F_DOWN = 1, F_LEFT = 2, F_RIGHT = 3 };

struct Model {
  int L1, L2, P, cut, Dmax;
  const int* dims;          // [site][4] = U, D, L, R extents
  const long long* off;     // [site] element offset of A[site]
  const void* A;            // element type T, A[site][p][u][d][l][r]
  int n_terms;
  const int* term_sites;    // [t][4]
  const int* hterm;         // [site]: term on (l1,l2)-(l1,l2+1) or -1
  const int* vterm;         // [site]: term on (l1,l2)-(l1+1,l2) or -1
  const int* hflip;         // [t]: 1 if positions[0] is the second (right/lower) site
  const int* tab_off;       // [t][P*P]
  const int* tab_cnt;       // [t][P*P], -1 = input absent from the table
  const int* tab_out;       // [entries]
  const double* tab_val;    // [entries]
  long long n_params;       // total elements of all site tensors
  // charges (all zero without symmetry): every nonzero element of site tensor A[p][u][d][l][r]
  // satisfies qphys[p] + qU[u] + qD[d] + qL[l] + qR[r] == sflux[site]
  const int* qleg;          // [site][4][Dmax]: charge of each index of the U, D, L, R legs
  const int* qphys;         // [P]
  const int* sflux;         // [site]
  // fermionic lattice: A holds eight slices per site, [family][n][prefix parity][u][d][l][r] (family 0
  // for the row orientations, 1 for the column ones), and the gradient accumulators / hole rows use
  // the two-slice parameter layout at poff (null: the layout of off)
  int fermion;
  int pT;                   // parity of the T leg's charge
  const long long* poff;
  int jacobi_max;           // sweep limit of the one-sided Jacobi SVD
  // the sweep's proposal tables (SweepSampling's hopping Hamiltonians; the energy tables above unless
  // replaced), laid out like hterm .. tab_out; allow flags per table entry (null: every entry allowed):
  // a proposal or an E_loc term whose entry is not allowed is skipped, as a restricted subspace makes
  // the reference skip it
  const int* s_hterm;
  const int* s_vterm;
  const int* s_hflip;
  const int* s_tab_off;
  const int* s_tab_cnt;
  const int* s_tab_out;
  const unsigned char* s_allow;
  const unsigned char* e_allow;
};

struct Chains {
  int B;
  int32_t* conf;            // [B][L1*L2]
  uint64_t* mt;             // [B][312]
  int32_t* mti;             // [B]
  double* ws_m;             // [B] carried amplitude of the last sweep (mantissa)
  int32_t* ws_e;            // [B]
  int64_t* accepted;        // [B]
  double* acc;              // [B][8] observer scalars (see tnsp_observer_read)
  double* rec_eloc;         // [nsamples][B]
  double* rec_logws;
  double* rec_rw;
  int32_t* status;
  // optional per-sample hole rows for the natural gradient: row hole_row0 + sweep * B + chain holds
  // <psi|s|d psi / d A> / <psi|s|psi> for every parameter (zero outside the sampled physical slices;
  // the rows are zeroed before the launch)
  double* rec_hole;
  long long hole_row0;
};

struct Slots {
  long long stride;         // bytes per slot
  long long o_lines[4];     // line storage per family: [line][site][capB] (S); every o_* is a byte offset
  long long capB, capT, capR, capE, capS, capH;  // capacities in elements
  // S-typed: o_lines, o_T, o_E, o_F, o_t1, o_t2, o_w0, o_w1, o_h; T-typed: o_G, o_R, o_tau, o_X, o_V, o_W, o_sig
  long long o_T, o_G, o_R, o_tau, o_X, o_V, o_W, o_sig, o_E, o_F, o_t1, o_t2, o_w0, o_w1, o_h;
  // implicit Q of the QR sweep per site: o_qsec (int) [site][1 + 6 kMaxSec]: sector count, then per
  // sector rows, reflectors, bond offset, row-list offset, reflector offset, Tw offset (-1: none);
  // o_qrow (int) [site][chi*Dmax]: row lists; o_qtau (T) [site][chi]: reflector scalars; o_qtw (T)
  // [site][(chi + kMaxSec) kNB^2]: the Tw factor of every panel of the sectors factorised in panels
  long long o_qsec, o_qrow, o_qtau, o_qtw;
  int* ldims;               // [slot][4][kMaxL][kMaxL][3]
  int* lexp;                // [slot][4][kMaxL]
  int* order;               // [slot][cut*(Dmax+1)]: kept singular values, then pivots
  double* delta;            // [slot][n_params]
  double* edelta;           // [slot][n_params]
  double* contrib;          // [slot][n_terms]
  double* flops;            // [slot][4]: algorithmic flops of contractions, QR, SVD, strip/hole work
  int* lq;                  // [slot][4][kMaxL][kMaxL][2][cut]: charges of the left/right bond of line sites
  int* lfl;                 // [slot][4][kMaxL][kMaxL]: flux of line sites
  int* tq;                  // [slot][kMaxL][3][chi]: charges of the left/right/open legs of compression tensors
  int* tfl;                 // [slot][kMaxL]
  int* ilist;               // [slot][chi*Dmax + chi]: packed sector row lists, then column lists
  long long smem_elems;     // dynamic shared memory available to a block, in elements of T
};

// element conversion between the two types of an engine
template <class To> struct Cvt {
  template <class From> static __device__ __forceinline__ To from(From x) { return (To)x; }
};
template <> struct Cvt<float> {
  static __device__ __forceinline__ float from(float x) { return x; }
  static __device__ __forceinline__ float from(double x) { return (float)x; }
  static __device__ __forceinline__ float from(dd x) { return x.hi + x.lo; }
};
template <> struct Cvt<dd> {
  static __device__ __forceinline__ dd from(dd x) { return x; }
  static __device__ __forceinline__ dd from(float x) { return dd(x); }
  static __device__ __forceinline__ dd from(double x) { return dd(x); }
};
template <class To, class From> __device__ __forceinline__ To cvt(From x) { return Cvt<To>::from(x); }

// B <- Q B for the m x nc column-major matrix B (ld m), Q = H_0 H_1 ... H_{k-1} from block_geqrf_cm's
// reflectors V (m x k column-major, stored as S; the unit diagonal is implicit and the entries above it
// are not read) and their scalars tau (LAPACK ormqr, side L, no transpose).  Panels of up to kNB
// reflectors, the last panel first, are staged in shared memory P (pcap elements) and applied as one
// block reflector each; without room for a panel, one reflector at a time.  TwIn, when given, holds
// the panels' Tw factors (kNB x kNB each, in panel order) kept by the factorisation, which are then not
// recomputed.  Ends with a barrier.
template <class T, class S>
__device__ __noinline__ void block_ormqr_panel(int m, int k, const S* V, const T* tau, T* B, int nc, T* P, long pcap,
                                               const T* TwIn) {
  const int nb = panel_width(m, pcap);
  if (nb < 2) {
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, grp = lane / kJG, sl = lane % kJG;
    for (int y = k - 1; y >= 0; --y) {
      const T ty = tau[y];
      if (ty != (T)0) {
        const S* v = V + (long)y * m;
        for (int base = w * (32 / kJG); base < nc; base += kWarps * (32 / kJG)) {  // warp-uniform
          const int c = base + grp;
          const bool act = c < nc;
          T* bc = B + (long)(act ? c : base) * m;
          T d = (act && sl == 0) ? bc[y] : (T)0;
          if (act)
            for (int r = y + 1 + sl; r < m; r += kJG) d = fma(cvt<T>(v[r]), bc[r], d);
          d = group_sum<kJG>(d) * ty;
          if (act) {
            if (sl == 0) bc[y] -= d;
            for (int r = y + 1 + sl; r < m; r += kJG) bc[r] -= d * cvt<T>(v[r]);
          }
        }
      }
      __syncthreads();
    }
    return;
  }
  for (int j0 = ((k - 1) / nb) * nb; j0 >= 0; j0 -= nb) {
    const int jb = k - j0 < nb ? k - j0 : nb, pm = m - j0;
    T* Y = P + (long)pm * jb;
    T* Tw = Y + kNB * kNB;
    for (long e = threadIdx.x; e < (long)pm * jb; e += blockDim.x) {  // explicit unit-lower panel
      const int c = (int)(e / pm), r = (int)(e % pm);
      P[e] = r < c ? (T)0 : (r == c ? (T)1 : cvt<T>(V[(long)(j0 + c) * m + j0 + r]));
    }
    __syncthreads();
    const T* tw = Tw;
    if (TwIn)
      tw = TwIn + (long)(j0 / nb) * kNB * kNB;
    else
      panel_tw(pm, jb, P, tau + j0, Y, Tw);
    apply_panel<T, false>(pm, jb, P, tw, B + j0, m, 0, nc);
    __syncthreads();
  }
}

// ------------------------------------------------------------------------------------------
// random numbers: std::mt19937_64 + libstdc++ 13 distributions (thread 0 only)
// ------------------------------------------------------------------------------------------
__device__ inline uint64_t mt_next(uint64_t* mt, int& mti) {
  if (mti >= kMtN) {
    for (int i = 0; i < kMtN; ++i) {
      const uint64_t x = (mt[i] & 0xFFFFFFFF80000000ull) | (mt[(i + 1) % kMtN] & 0x7FFFFFFFull);
      uint64_t xa = x >> 1;
      if (x & 1ull) xa ^= 0xB5026F5AA96619E9ull;
      mt[i] = mt[(i + 156) % kMtN] ^ xa;
    }
    mti = 0;
  }
  uint64_t y = mt[mti++];
  y ^= (y >> 29) & 0x5555555555555555ull;
  y ^= (y << 17) & 0x71D67FFFEDA60000ull;
  y ^= (y << 37) & 0xFFF7EEE000000000ull;
  y ^= y >> 43;
  return y;
}

// std::uniform_int_distribution<int>(0, n-1): Lemire's nearly-divisionless downscaling on a
// 128-bit product (bits/uniform_int_dist.h, _S_nd).
__device__ inline int draw_uniform_int(uint64_t* mt, int& mti, int n) {
  const uint64_t range = (uint64_t)n;
  uint64_t x = mt_next(mt, mti);
  uint64_t lo = x * range;
  uint64_t hi = __umul64hi(x, range);
  if (lo < range) {
    const uint64_t threshold = (0ull - range) % range;
    while (lo < threshold) {
      x = mt_next(mt, mti);
      lo = x * range;
      hi = __umul64hi(x, range);
    }
  }
  return (int)hi;
}

// std::uniform_real_distribution<double>(0, 1): generate_canonical<double, 53> with one 64-bit
// word: round-to-nearest conversion, division by 2^64, clamp to below 1.
__device__ inline double draw_uniform_real(uint64_t* mt, int& mti) {
  const uint64_t x = mt_next(mt, mti);
  double r = __ull2double_rn(x) * 5.421010862427522e-20;  // 2^-64, exact
  if (r >= 1.0) r = 0.99999999999999989;
  return r;
}

// ------------------------------------------------------------------------------------------
// views
// ------------------------------------------------------------------------------------------
// which of a fermionic site's eight slices [family][n][prefix parity] a view reads: family 0 for the row
// orientations (0, 1), 1 for the column ones (2, 3)
__host__ __device__ __forceinline__ long long fermion_slice(int orient, int s, int mp) {
  return (long long)((orient >= 2 ? 2 : 0) + s) * 2 + (mp & 1);
}

// particles before strip position c of line idx: the sites of row idx left of column c (kind 0) or the
// sites of column idx above row c (kind 1)
__host__ __device__ inline int strip_prefix_of(const short* conf, int L2, int kind, int idx, int c) {
  int n = 0;
  for (int k = 0; k < c; ++k) n += kind == 0 ? conf[idx * L2 + k] : conf[k * L2 + idx];
  return n;
}

struct SiteView {  // a projected site tensor seen as W(u, d, l, r)
  long long base;
  int du, dd, dl, dr;
  int su, sd, sl, sr;
  const int *qu, *qd, *ql, *qr;  // index charges of the four roles
  int flux;                      // sum of the four leg charges of every nonzero element
};

struct Dims3 {
  int a, p, b;
};

template <class T, class S> struct Chain {
  const Model& md;
  const Slots& sl;
  unsigned char* slot;
  const S* A;
  int* ldims;
  int* lexp;
  int* order;
  // shared state (pointers into shared memory)
  short* conf;
  unsigned char* valid;   // [4][kMaxL]
  int* eE;                // [kMaxL + 1]
  int* eF;
  T* red;
  double* dred;
  double* fl;             // shared [kCounters]: flop counters [0..3], phase cycles [4..]

  // typed view of a byte offset in the slot
  template <class X> __device__ X* at(long long off) const { return reinterpret_cast<X*>(slot + off); }
  // block-reduction scratch for S-typed sums (red holds kWarps elements of T, sizeof(S) <= sizeof(T))
  __device__ S* sred() const { return reinterpret_cast<S*>(red); }

  __device__ void count(int k, double f) const {
    if (threadIdx.x == 0) fl[k] += f;
  }
  // phase timer: thread 0 reads the SM clock at phase boundaries (already barrier points)
  __device__ long long tic() const { return clock64(); }
  __device__ void toc(int phase, long long t0) const {
    if (threadIdx.x == 0) fl[4 + phase] += (double)(clock64() - t0);
  }

  __device__ S* line(int f, int idx, int i) const {
    const int ns = (f < 2) ? md.L2 : md.L1;
    return at<S>(sl.o_lines[f]) + ((long long)idx * ns + i) * sl.capB;
  }
  __device__ int* ldim(int f, int idx, int i) const { return ldims + (((f * kMaxL) + idx) * kMaxL + i) * 3; }

  // site (l1, l2) at physical index s in one of four orientations:
  //   0: (U, D, L, R)   1: (D, U, L, R)   2: (L, R, U, D)   3: (R, L, U, D)
  //   fermionic lattices: ``mp`` is the number of particles before the site along its row (orientations
  //   0, 1) or column (2, 3) in the configuration being evaluated; its parity picks the slice
  __device__ SiteView site(int l1, int l2, int s, int orient, int mp = 0) const {
    const int id = l1 * md.L2 + l2;
    const int* d = md.dims + id * 4;
    const int U = d[0], D = d[1], L = d[2], R = d[3];
    const int sR = 1, sL = R, sD = L * R, sU = D * L * R;
    SiteView v;
    const long long slice = md.fermion ? fermion_slice(orient, s, mp) : (long long)s;
    v.base = md.off[id] + slice * U * D * L * R;
    const int* q = md.qleg + (long long)id * 4 * md.Dmax;
    const int *qU = q, *qD = q + md.Dmax, *qL = q + 2 * md.Dmax, *qR = q + 3 * md.Dmax;
    v.flux = md.sflux[id] - md.qphys[s];
    switch (orient) {
      case 0: v.du = U; v.su = sU; v.qu = qU; v.dd = D; v.sd = sD; v.qd = qD; v.dl = L; v.sl = sL; v.ql = qL; v.dr = R; v.sr = sR; v.qr = qR; break;
      case 1: v.du = D; v.su = sD; v.qu = qD; v.dd = U; v.sd = sU; v.qd = qU; v.dl = L; v.sl = sL; v.ql = qL; v.dr = R; v.sr = sR; v.qr = qR; break;
      case 2: v.du = L; v.su = sL; v.qu = qL; v.dd = R; v.sd = sR; v.qd = qR; v.dl = U; v.sl = sU; v.ql = qU; v.dr = D; v.sr = sD; v.qr = qD; break;
      default: v.du = R; v.su = sR; v.qu = qR; v.dd = L; v.sd = sL; v.qd = qL; v.dl = U; v.sl = sU; v.ql = qU; v.dr = D; v.sr = sD; v.qr = qD; break;
    }
    return v;
  }
};

// ------------------------------------------------------------------------------------------
// contractions
// ------------------------------------------------------------------------------------------
// Every contraction below gives each thread kCB outputs that share one operand load (a run of the
// fastest output index, or of another free index where that one is short): the kCB multiply-add
// chains are independent, so a thread keeps kCB operations in flight instead of waiting on each
// result, and the shared operand is read once per kCB outputs.  Tails are handled by clamped reads
// and guarded writes; each output's sum runs over its terms in the same order as a one-output loop.
constexpr int kCB = 4;

// out[(x*l + y), dd, (z*r + w)] = sum_p line[x, p, z] * W(p, dd, y, w).
// With `dense`, every output (a thread computes kCB values of dd).  Otherwise only the charge-allowed
// outputs, qa[x] + ql[y] + qd[dd] + qb[z] + qr[w] == F (qa, qb null: zero), are computed and written,
// and the other entries of `out` are left as they are: the compression reads this tensor only at
// allowed entries (its sector gathers and the R absorption's column lists), and a block tensor has
// most of its entries outside them.  A thread takes one (row, column) pair and its allowed dd, kTL at
// a time.
constexpr int kTL = 2;
template <class T>
__device__ __noinline__ void two_line(const T* __restrict__ line, Dims3 ld, const T* __restrict__ A, SiteView w,
                                      T* __restrict__ out, const int* qa, const int* qb, int F, bool dense) {
  const int Am = ld.a * w.dl, Bm = ld.b * w.dr;
  if (!dense) {
    const long long n = (long long)Am * Bm;
    for (long long t = threadIdx.x; t < n; t += blockDim.x) {
      const int col = (int)(t % Bm), row = (int)(t / Bm);
      const int x = row / w.dl, y = row % w.dl, z = col / w.dr, ww = col % w.dr;
      const int want = F - (qa ? qa[x] : 0) - w.ql[y] - (qb ? qb[z] : 0) - w.qr[ww];
      const T* lp = line + (long long)x * ld.p * ld.b + z;
      const T* wb = A + w.base + (long long)y * w.sl + (long long)ww * w.sr;
      int d0 = 0;
      while (true) {
        int ds[kTL];
#pragma unroll
        for (int v = 0; v < kTL; ++v) {  // the next kTL allowed dd from d0 on (-1: none)
          while (d0 < w.dd && w.qd[d0] != want) ++d0;
          ds[v] = d0 < w.dd ? d0++ : -1;
        }
        if (ds[0] < 0) break;
        T acc[kTL];
        const T* wp[kTL];
#pragma unroll
        for (int v = 0; v < kTL; ++v) {
          acc[v] = 0;
          wp[v] = wb + (long long)(ds[v] >= 0 ? ds[v] : ds[0]) * w.sd;
        }
        for (int p = 0; p < ld.p; ++p) {
          const T lv = lp[(long long)p * ld.b];
#pragma unroll
          for (int v = 0; v < kTL; ++v) acc[v] = fma(lv, wp[v][(long long)p * w.su], acc[v]);
        }
#pragma unroll
        for (int v = 0; v < kTL; ++v)
          if (ds[v] >= 0) out[((long long)row * w.dd + ds[v]) * Bm + col] = acc[v];
        if (ds[kTL - 1] < 0) break;
      }
    }
    __syncthreads();
    return;
  }
  const int ddb = (w.dd + kCB - 1) / kCB;
  const long long n = (long long)Am * ddb * Bm;
  for (long long t = threadIdx.x; t < n; t += blockDim.x) {
    const int col = (int)(t % Bm);
    const long long rest = t / Bm;
    const int d0 = (int)(rest % ddb) * kCB;
    const int row = (int)(rest / ddb);
    const int x = row / w.dl, y = row % w.dl, z = col / w.dr, ww = col % w.dr;
    T acc[kCB];
    const T* wp[kCB];
#pragma unroll
    for (int v = 0; v < kCB; ++v) {
      acc[v] = 0;
      const int d = d0 + v < w.dd ? d0 + v : w.dd - 1;
      wp[v] = A + w.base + (long long)d * w.sd + (long long)y * w.sl + (long long)ww * w.sr;
    }
    const T* lp = line + (long long)x * ld.p * ld.b + z;
    for (int p = 0; p < ld.p; ++p) {
      const T lv = lp[(long long)p * ld.b];
#pragma unroll
      for (int v = 0; v < kCB; ++v) acc[v] = fma(lv, wp[v][(long long)p * w.su], acc[v]);
    }
#pragma unroll
    for (int v = 0; v < kCB; ++v)
      if (d0 + v < w.dd) out[((long long)row * w.dd + d0 + v) * Bm + col] = acc[v];
  }
  __syncthreads();
}

// E'[a, r, b] = sum E[x, y, z] up[x, u, a] W(u, d, y, r) dn[z, d, b]
template <class T>
__device__ __noinline__ void strip_left(const T* E, int X, int Y, int Z, const T* up, Dims3 ud, const T* A, SiteView w,
                           const T* dn, Dims3 dd, T* t1, T* t2, T* out) {
  const int U = ud.p, Aa = ud.b, D = dd.p, Bb = dd.b, R = w.dr;
  const int ab = (Aa + kCB - 1) / kCB, bb = (Bb + kCB - 1) / kCB;
  // t1[y, z, u, a] = sum_x E[x, y, z] up[x, u, a]   (kCB consecutive a)
  long long n = (long long)Y * Z * U * ab;
  for (long long t = threadIdx.x; t < n; t += blockDim.x) {
    const int a0 = (int)(t % ab) * kCB;
    long long r = t / ab;
    const int u = (int)(r % U);
    r /= U;
    const int z = (int)(r % Z);
    const int y = (int)(r / Z);
    T acc[kCB];
#pragma unroll
    for (int v = 0; v < kCB; ++v) acc[v] = 0;
    for (int x = 0; x < X; ++x) {
      const T e = E[((long long)x * Y + y) * Z + z];
      const T* uu = up + ((long long)x * U + u) * Aa;
#pragma unroll
      for (int v = 0; v < kCB; ++v) acc[v] = fma(e, uu[a0 + v < Aa ? a0 + v : Aa - 1], acc[v]);
    }
    T* o = t1 + (((long long)y * Z + z) * U + u) * Aa;
#pragma unroll
    for (int v = 0; v < kCB; ++v)
      if (a0 + v < Aa) o[a0 + v] = acc[v];
  }
  __syncthreads();
  // t2[z, a, d, r] = sum_{y,u} t1[y, z, u, a] W(u, d, y, r)   (kCB consecutive a)
  n = (long long)Z * ab * D * R;
  for (long long t = threadIdx.x; t < n; t += blockDim.x) {
    const int rr = (int)(t % R);
    long long q = t / R;
    const int d = (int)(q % D);
    q /= D;
    const int a0 = (int)(q % ab) * kCB;
    const int z = (int)(q / ab);
    T acc[kCB];
#pragma unroll
    for (int v = 0; v < kCB; ++v) acc[v] = 0;
    for (int y = 0; y < Y; ++y)
      for (int u = 0; u < U; ++u) {
        const T wv = A[w.base + (long long)u * w.su + (long long)d * w.sd + (long long)y * w.sl + (long long)rr * w.sr];
        const T* tt = t1 + (((long long)y * Z + z) * U + u) * Aa;
#pragma unroll
        for (int v = 0; v < kCB; ++v) acc[v] = fma(tt[a0 + v < Aa ? a0 + v : Aa - 1], wv, acc[v]);
      }
#pragma unroll
    for (int v = 0; v < kCB; ++v)
      if (a0 + v < Aa) t2[(((long long)z * Aa + a0 + v) * D + d) * R + rr] = acc[v];
  }
  __syncthreads();
  // out[a, r, b] = sum_{z,d} t2[z, a, d, r] dn[z, d, b]   (kCB consecutive b)
  n = (long long)Aa * R * bb;
  for (long long t = threadIdx.x; t < n; t += blockDim.x) {
    const int b0 = (int)(t % bb) * kCB;
    long long q = t / bb;
    const int rr = (int)(q % R);
    const int a = (int)(q / R);
    T acc[kCB];
#pragma unroll
    for (int v = 0; v < kCB; ++v) acc[v] = 0;
    for (int z = 0; z < Z; ++z)
      for (int d = 0; d < D; ++d) {
        const T tv = t2[(((long long)z * Aa + a) * D + d) * R + rr];
        const T* dp = dn + ((long long)z * D + d) * Bb;
#pragma unroll
        for (int v = 0; v < kCB; ++v) acc[v] = fma(tv, dp[b0 + v < Bb ? b0 + v : Bb - 1], acc[v]);
      }
    T* o = out + ((long long)a * R + rr) * Bb;
#pragma unroll
    for (int v = 0; v < kCB; ++v)
      if (b0 + v < Bb) o[b0 + v] = acc[v];
  }
  __syncthreads();
}

// F'[x, l, z] = sum F[a, r, b] up[x, u, a] W(u, d, l, r) dn[z, d, b]
template <class T>
__device__ __noinline__ void strip_right(const T* F, int Aa, int R, int Bb, const T* up, Dims3 ud, const T* A, SiteView w,
                            const T* dn, Dims3 dd, T* s1, T* s2, T* out) {
  const int X = ud.a, U = ud.p, Z = dd.a, D = dd.p, L = w.dl;
  const int bb = (Bb + kCB - 1) / kCB, zb = (Z + kCB - 1) / kCB;
  // s1[x, u, r, b] = sum_a up[x, u, a] F[a, r, b]   (kCB consecutive b)
  long long n = (long long)X * U * R * bb;
  for (long long t = threadIdx.x; t < n; t += blockDim.x) {
    const int b0 = (int)(t % bb) * kCB;
    long long q = t / bb;
    const int rr = (int)(q % R);
    q /= R;
    const int u = (int)(q % U);
    const int x = (int)(q / U);
    T acc[kCB];
#pragma unroll
    for (int v = 0; v < kCB; ++v) acc[v] = 0;
    for (int a = 0; a < Aa; ++a) {
      const T uv = up[((long long)x * U + u) * Aa + a];
      const T* fp = F + ((long long)a * R + rr) * Bb;
#pragma unroll
      for (int v = 0; v < kCB; ++v) acc[v] = fma(uv, fp[b0 + v < Bb ? b0 + v : Bb - 1], acc[v]);
    }
    T* o = s1 + (((long long)x * U + u) * R + rr) * Bb;
#pragma unroll
    for (int v = 0; v < kCB; ++v)
      if (b0 + v < Bb) o[b0 + v] = acc[v];
  }
  __syncthreads();
  // s2[x, l, d, b] = sum_{u,r} s1[x, u, r, b] W(u, d, l, r)   (kCB consecutive b)
  n = (long long)X * L * D * bb;
  for (long long t = threadIdx.x; t < n; t += blockDim.x) {
    const int b0 = (int)(t % bb) * kCB;
    long long q = t / bb;
    const int d = (int)(q % D);
    q /= D;
    const int l = (int)(q % L);
    const int x = (int)(q / L);
    T acc[kCB];
#pragma unroll
    for (int v = 0; v < kCB; ++v) acc[v] = 0;
    for (int u = 0; u < U; ++u)
      for (int rr = 0; rr < R; ++rr) {
        const T wv = A[w.base + (long long)u * w.su + (long long)d * w.sd + (long long)l * w.sl + (long long)rr * w.sr];
        const T* sp = s1 + (((long long)x * U + u) * R + rr) * Bb;
#pragma unroll
        for (int v = 0; v < kCB; ++v) acc[v] = fma(sp[b0 + v < Bb ? b0 + v : Bb - 1], wv, acc[v]);
      }
    T* o = s2 + (((long long)x * L + l) * D + d) * Bb;
#pragma unroll
    for (int v = 0; v < kCB; ++v)
      if (b0 + v < Bb) o[b0 + v] = acc[v];
  }
  __syncthreads();
  // out[x, l, z] = sum_{d,b} s2[x, l, d, b] dn[z, d, b]   (kCB consecutive z)
  n = (long long)X * L * zb;
  for (long long t = threadIdx.x; t < n; t += blockDim.x) {
    const int z0 = (int)(t % zb) * kCB;
    long long q = t / zb;
    const int l = (int)(q % L);
    const int x = (int)(q / L);
    T acc[kCB];
    const T* dp[kCB];
#pragma unroll
    for (int v = 0; v < kCB; ++v) {
      acc[v] = 0;
      dp[v] = dn + (long long)(z0 + v < Z ? z0 + v : Z - 1) * D * Bb;
    }
    const T* sp = s2 + ((long long)x * L + l) * D * Bb;
    for (int e = 0; e < D * Bb; ++e) {
      const T sv = sp[e];
#pragma unroll
      for (int v = 0; v < kCB; ++v) acc[v] = fma(sv, dp[v][e], acc[v]);
    }
    T* o = out + ((long long)x * L + l) * Z;
#pragma unroll
    for (int v = 0; v < kCB; ++v)
      if (z0 + v < Z) o[z0 + v] = acc[v];
  }
  __syncthreads();
}

// h[u, d, l, r] = sum E[x, l, z] up[x, u, a] dn[z, d, b] F[a, r, b]
template <class T>
__device__ __noinline__ void strip_hole(const T* E, int X, int L, int Z, const T* up, Dims3 ud, const T* dn, Dims3 dd, const T* F,
                           int R, T* h1, T* h2, T* out) {
  const int U = ud.p, Aa = ud.b, D = dd.p, Bb = dd.b;
  const int ab = (Aa + kCB - 1) / kCB, bb = (Bb + kCB - 1) / kCB, rb = (R + kCB - 1) / kCB;
  // h1[l, z, u, a] = sum_x E[x, l, z] up[x, u, a]   (kCB consecutive a)
  long long n = (long long)L * Z * U * ab;
  for (long long t = threadIdx.x; t < n; t += blockDim.x) {
    const int a0 = (int)(t % ab) * kCB;
    long long q = t / ab;
    const int u = (int)(q % U);
    q /= U;
    const int z = (int)(q % Z);
    const int l = (int)(q / Z);
    T acc[kCB];
#pragma unroll
    for (int v = 0; v < kCB; ++v) acc[v] = 0;
    for (int x = 0; x < X; ++x) {
      const T e = E[((long long)x * L + l) * Z + z];
      const T* uu = up + ((long long)x * U + u) * Aa;
#pragma unroll
      for (int v = 0; v < kCB; ++v) acc[v] = fma(e, uu[a0 + v < Aa ? a0 + v : Aa - 1], acc[v]);
    }
    T* o = h1 + (((long long)l * Z + z) * U + u) * Aa;
#pragma unroll
    for (int v = 0; v < kCB; ++v)
      if (a0 + v < Aa) o[a0 + v] = acc[v];
  }
  __syncthreads();
  // h2[l, u, a, d, b] = sum_z h1[l, z, u, a] dn[z, d, b]   (kCB consecutive b)
  n = (long long)L * U * Aa * D * bb;
  for (long long t = threadIdx.x; t < n; t += blockDim.x) {
    const int b0 = (int)(t % bb) * kCB;
    long long q = t / bb;
    const int d = (int)(q % D);
    q /= D;
    const int a = (int)(q % Aa);
    q /= Aa;
    const int u = (int)(q % U);
    const int l = (int)(q / U);
    T acc[kCB];
#pragma unroll
    for (int v = 0; v < kCB; ++v) acc[v] = 0;
    for (int z = 0; z < Z; ++z) {
      const T hv = h1[(((long long)l * Z + z) * U + u) * Aa + a];
      const T* dp = dn + ((long long)z * D + d) * Bb;
#pragma unroll
      for (int v = 0; v < kCB; ++v) acc[v] = fma(hv, dp[b0 + v < Bb ? b0 + v : Bb - 1], acc[v]);
    }
    T* o = h2 + ((((long long)l * U + u) * Aa + a) * D + d) * Bb;
#pragma unroll
    for (int v = 0; v < kCB; ++v)
      if (b0 + v < Bb) o[b0 + v] = acc[v];
  }
  __syncthreads();
  // out[u, d, l, r] = sum_{a,b} h2[l, u, a, d, b] F[a, r, b]   (kCB consecutive r)
  n = (long long)U * D * L * rb;
  for (long long t = threadIdx.x; t < n; t += blockDim.x) {
    const int r0 = (int)(t % rb) * kCB;
    long long q = t / rb;
    const int l = (int)(q % L);
    q /= L;
    const int d = (int)(q % D);
    const int u = (int)(q / D);
    T acc[kCB];
#pragma unroll
    for (int v = 0; v < kCB; ++v) acc[v] = 0;
    for (int a = 0; a < Aa; ++a) {
      const T* hp = h2 + ((((long long)l * U + u) * Aa + a) * D + d) * Bb;
      const T* fp = F + (long long)a * R * Bb;
      for (int b = 0; b < Bb; ++b) {
        const T hv = hp[b];
#pragma unroll
        for (int v = 0; v < kCB; ++v) acc[v] = fma(hv, fp[(long long)(r0 + v < R ? r0 + v : R - 1) * Bb + b], acc[v]);
      }
    }
    T* o = out + (((long long)u * D + d) * L + l) * R;
#pragma unroll
    for (int v = 0; v < kCB; ++v)
      if (r0 + v < R) o[r0 + v] = acc[v];
  }
  __syncthreads();
}

template <class T> __device__ T block_dot(const T* x, const T* y, long long n, T* red) {
  T acc = 0;
  for (long long t = threadIdx.x; t < n; t += blockDim.x) acc = fma(x[t], y[t], acc);
  return block_sum(acc, red);
}

// ------------------------------------------------------------------------------------------
// the chain engine
// ------------------------------------------------------------------------------------------
template <class T, class S> struct Engine : Chain<T, S> {
  using Chain<T, S>::md;
  using Chain<T, S>::sl;
  using Chain<T, S>::slot;
  using Chain<T, S>::A;
  using Chain<T, S>::conf;
  using Chain<T, S>::valid;
  using Chain<T, S>::eE;
  using Chain<T, S>::eF;
  using Chain<T, S>::red;
  using Chain<T, S>::line;
  using Chain<T, S>::ldim;
  using Chain<T, S>::site;
  using Chain<T, S>::lexp;
  using Chain<T, S>::order;
  using Chain<T, S>::tic;
  using Chain<T, S>::toc;
  using Chain<T, S>::sred;
  template <class X> __device__ X* at(long long off) const { return Chain<T, S>::template at<X>(off); }
  const S* ones;
  int32_t* status;
  int* lq;
  int* lfl;
  int* tq;
  int* tfl;
  int* ilist;
  T* smem;
  // strip currently held in E/F: kind 0 = row, 1 = column, -1 none
  int* strip_kind;
  int* strip_idx;
  int* strip_eupto;       // E[0..eupto] valid
  int* strip_ffrom;       // F[ffrom..n] valid

  __device__ int nsites_along(int f) const { return f < 2 ? md.L2 : md.L1; }
  __device__ int nlines(int f) const { return f < 2 ? md.L1 : md.L2; }

  // line family f at index idx, or the all-ones line beyond the lattice edge
  __device__ bool is_ones(int f, int idx) const { return idx < 0 || idx >= nlines(f); }
  __device__ const S* lsite(int f, int idx, int i) const { return is_ones(f, idx) ? ones : line(f, idx, i); }
  __device__ Dims3 lsdim(int f, int idx, int i) const {
    if (is_ones(f, idx)) return Dims3{1, 1, 1};
    const int* d = ldim(f, idx, i);
    return Dims3{d[0], d[1], d[2]};
  }
  __device__ int lexpo(int f, int idx) const { return is_ones(f, idx) ? 0 : lexp[f * kMaxL + idx]; }

  __device__ S* Tbuf(int k) const { return at<S>(sl.o_T) + (long long)k * sl.capT; }

  // charges of line sites and of compression tensors
  __device__ int* lqa(int f, int idx, int i) const {
    return lq + ((((long long)f * kMaxL + idx) * kMaxL + i) * 2 + 0) * md.cut;
  }
  __device__ int* lqb(int f, int idx, int i) const {
    return lq + ((((long long)f * kMaxL + idx) * kMaxL + i) * 2 + 1) * md.cut;
  }
  __device__ int* lflux(int f, int idx, int i) const { return lfl + ((long long)f * kMaxL + idx) * kMaxL + i; }
  __device__ int chi() const { return md.cut * md.Dmax; }
  __device__ int* tqL(int i) const { return tq + ((long long)i * 3 + 0) * chi(); }
  __device__ int* tqR(int i) const { return tq + ((long long)i * 3 + 1) * chi(); }
  __device__ int* tqD(int i) const { return tq + ((long long)i * 3 + 2) * chi(); }

  // Sector table of a matrix whose rows carry charges qrow(x), columns qcol(z), and whose
  // nonzeros satisfy qrow + qcol == F: one sector per row charge r (ascending) with matching
  // columns F - r.  Row and column index lists are packed into ilist.
  struct Sectors {
    int n;
    int r[kMaxSec], m[kMaxSec], c[kMaxSec], ro[kMaxSec], co[kMaxSec];
  };

  template <class QR, class QC>
  __device__ void sectors(int rows, int cols, QR qrow, QC qcol, int F, Sectors* sec, int* sh) {
    __shared__ int s_lo, s_hi;
    if (threadIdx.x == 0) {
      s_lo = 1 << 30;
      s_hi = -(1 << 30);
    }
    __syncthreads();
    int lo = 1 << 30, hi = -(1 << 30);
    for (int x = threadIdx.x; x < rows; x += blockDim.x) {
      const int q = qrow(x);
      lo = q < lo ? q : lo;
      hi = q > hi ? q : hi;
    }
    atomicMin(&s_lo, lo);
    atomicMax(&s_hi, hi);
    __syncthreads();
    const int qlo = s_lo, qhi = s_hi;
    int* rl = ilist;
    int* cl = ilist + (long long)chi() * md.Dmax;
    int nr = 0, nc = 0, ns = 0;
    for (int q = qlo; q <= qhi; ++q) {
      const int mr = block_compact(rows, [&](int x) { return qrow(x) == q; }, rl + nr, sh);
      if (mr == 0) continue;
      const int mc = block_compact(cols, [&](int z) { return qcol(z) == F - q; }, cl + nc, sh);
      if (mc == 0) continue;
      if (ns >= kMaxSec) {
        if (threadIdx.x == 0) atomicOr(status, ST_UNSUPPORTED);
        break;
      }
      if (threadIdx.x == 0) {
        sec->r[ns] = q;
        sec->m[ns] = mr;
        sec->c[ns] = mc;
        sec->ro[ns] = nr;
        sec->co[ns] = nc;
      }
      nr += mr;
      nc += mc;
      ++ns;
    }
    if (threadIdx.x == 0) sec->n = ns;
    __syncthreads();
  }

  // _two_line_to_one_line for family f producing line idx (single_layer_auxiliaries.py:462-498).
  // Every QR and SVD is done per charge sector (TAT/include/TAT/implement/qr.hpp:310-510,
  // svd.hpp:259-532); the SVD truncation keeps the `cut` largest singular values over all
  // sectors (svd.hpp:429-470).  Without symmetry every charge is zero: one sector.
  __device__ __noinline__ void compress(int f, int idx) {
    this->count(CT_COMPRESS, 1.0);
    const int n = nsites_along(f);
    const int prev = (f == F_UP || f == F_LEFT) ? idx - 1 : idx + 1;
    const int orient = f;  // 0: UDLR, 1: DULR, 2: LRUD, 3: RLUD
    __shared__ int s_buf[kMaxL + 2];
    __shared__ int s_dA[kMaxL], s_dd[kMaxL], s_dB[kMaxL], s_fl[kMaxL];
    __shared__ int s_sh[kWarps + 1];
    __shared__ Sectors s_sec;
    __shared__ short s_kmap[kMaxChi];  // new bond index -> sector
    __shared__ short s_kloc[kMaxChi];  // new bond index -> local index in its sector
    __shared__ int s_roffs[kMaxSec];
    __shared__ int s_xo[kMaxSec], s_vo[kMaxSec], s_so[kMaxSec];
    const bool ones_prev = is_ones(f, prev);
    if (threadIdx.x < n + 2) s_buf[threadIdx.x] = threadIdx.x;
    __syncthreads();
    int expo = lexpo(f, prev);
    long long t0 = tic();
    int prefix = 0;
    for (int i = 0; i < n; ++i) {
      const int l1 = (f < 2) ? idx : i, l2 = (f < 2) ? i : idx;
      const SiteView w = site(l1, l2, conf[l1 * md.L2 + l2], orient, prefix);
      prefix += conf[l1 * md.L2 + l2];
      const Dims3 ld = lsdim(f, prev, i);
      const int* qa = ones_prev ? nullptr : lqa(f, prev, i);
      const int* qb = ones_prev ? nullptr : lqb(f, prev, i);
      // a one-site line is stored as is (its zeros included); longer ones only read allowed entries
      two_line(lsite(f, prev, i), ld, A, w, Tbuf(s_buf[i]), qa, qb,
               (ones_prev ? 0 : *lflux(f, prev, i)) + w.flux, n == 1);
      this->count(0, 2.0 * ld.a * w.dl * w.dd * ld.b * w.dr * ld.p);
      int* L = tqL(i);
      int* Rr = tqR(i);
      int* Dd = tqD(i);
      for (int x = threadIdx.x; x < ld.a * w.dl; x += blockDim.x) L[x] = (qa ? qa[x / w.dl] : 0) + w.ql[x % w.dl];
      for (int z = threadIdx.x; z < ld.b * w.dr; z += blockDim.x) Rr[z] = (qb ? qb[z / w.dr] : 0) + w.qr[z % w.dr];
      for (int d = threadIdx.x; d < w.dd; d += blockDim.x) Dd[d] = w.qd[d];
      if (threadIdx.x == 0) {
        s_dA[i] = ld.a * w.dl;
        s_dd[i] = w.dd;
        s_dB[i] = ld.b * w.dr;
        s_fl[i] = (ones_prev ? 0 : *lflux(f, prev, i)) + w.flux;
      }
      __syncthreads();
    }
    toc(PH_TWOLINE, t0);
    T* Rb = at<T>(sl.o_R);
    T* tau = at<T>(sl.o_tau);
    T* sm = smem;
    const long long smcap = sl.smem_elems;
    int* rl = ilist;
    int* cl = ilist + (long long)chi() * md.Dmax;
    // ---------------- QR sweep, per sector ----------------
    for (int i = 0; i < n - 1; ++i) {
      const int d = s_dd[i], rows = s_dA[i] * d, cols = s_dB[i], F = s_fl[i];
      const int* qL = tqL(i);
      const int* qD = tqD(i);
      const int* qR = tqR(i);
      t0 = tic();
      sectors(rows, cols, [&](int x) { return qL[x / d] + qD[x % d]; }, [&](int z) { return qR[z]; }, F, &s_sec, s_sh);
      toc(PH_SECTORS, t0);
      t0 = tic();
      const int ns = s_sec.n;
      int ktot = 0;
      for (int t = 0; t < ns; ++t) ktot += min(s_sec.m[t], s_sec.c[t]);
      const int spare = s_buf[n], spare2 = s_buf[n + 1];
      // new T[i] = Q is kept implicit: the buffer holds the sectors' reflectors, packed, and Q is applied
      // to U*S in the SVD sweep (the only use of T[i] before it is replaced), so it is never formed
      S* Tq = Tbuf(spare);
      S* G = Tbuf(spare2);   // new T[i+1] = R T[i+1]
      T* Gs = at<T>(sl.o_G);  // sector staging when shared memory is too small
      int* qsec = at<int>(sl.o_qsec) + (long long)i * (1 + 6 * kMaxSec);
      int* qrow = at<int>(sl.o_qrow) + (long long)i * chi() * md.Dmax;
      T* qtau = at<T>(sl.o_qtau) + (long long)i * chi();
      T* qtw = at<T>(sl.o_qtw) + (long long)i * (chi() + kMaxSec) * kNB * kNB;
      if (threadIdx.x == 0) {
        int o = 0, ko = 0, ro = 0, vo = 0, wo = 0;
        qsec[0] = ns;
        for (int t = 0; t < ns; ++t) {
          const int kr = min(s_sec.m[t], s_sec.c[t]);
          s_roffs[t] = o;
          o += kr * s_sec.c[t];
          int* q = qsec + 1 + 6 * t;
          q[0] = s_sec.m[t];
          q[1] = kr;
          q[2] = ko;
          q[3] = ro;
          q[4] = vo;
          // the panels' Tw factors are kept where the sector is factorised in panels and its reflectors
          // are stored at the factorisation's precision (they must match the panels the factors belong to)
          const int nb = panel_width(s_sec.m[t], smcap);
          const bool panels = (long long)s_sec.m[t] * s_sec.c[t] > smcap && nb >= 2 && sizeof(S) == sizeof(T);
          q[5] = panels ? wo : -1;
          if (panels) wo += (kr + nb - 1) / nb * kNB * kNB;
          ko += kr;
          ro += s_sec.m[t];
          vo += s_sec.m[t] * kr;
        }
      }
      __syncthreads();
      int koff = 0;
      double rsz = 0;
      for (int t = 0; t < ns; ++t) {
        const int mr = s_sec.m[t], mc = s_sec.c[t], kr = min(mr, mc);
        const int* R_ = rl + s_sec.ro[t];
        const int* C_ = cl + s_sec.co[t];
        const S* M = Tbuf(s_buf[i]);
        T* g = ((long long)mr * mc <= smcap) ? sm : Gs;
        for (long long e = threadIdx.x; e < (long long)mr * mc; e += blockDim.x) {
          const int y = (int)(e / mr), x = (int)(e % mr);
          g[e] = cvt<T>(M[(long long)R_[x] * cols + C_[y]]);
        }
        __syncthreads();
        // power-of-two scaling of the sector to max |g| in [0.5, 1): exact, so Q and R / 2^es are the
        // factors of the unscaled block; it keeps the squared norms of a sector that is small next to
        // the tensor's largest one inside the exponent range of float-based element types
        const int es = block_normalize(g, (long long)mr * mc, red);
        const T rsc = (T)ldexp(1.0, es);
        // a sector staged in the slot is factorised in panels through the (then unused) shared memory
        if (g == sm)
          block_geqrf_cm(mr, mc, g, tau, red);
        else
          block_geqrf_panel(mr, mc, g, tau, red, sm, smcap, qsec[1 + 6 * t + 5] >= 0 ? qtw + qsec[1 + 6 * t + 5] : nullptr);
        {
          const double mm = mr > mc ? mr : mc, nn = kr;
          this->count(1, 2.0 * mm * nn * nn - 2.0 * nn * nn * nn / 3.0);
        }
        // R (kr x mc, row-major) into Rb
        T* rb = Rb + s_roffs[t];
        for (long long e = threadIdx.x; e < (long long)kr * mc; e += blockDim.x) {
          const int y = (int)(e / mc), z = (int)(e % mc);
          rb[e] = z >= y ? g[(long long)z * mr + y] * rsc : (T)0;
        }
        // the reflectors (the first kr columns of g; R above their diagonal is not read again), their
        // scalars and the sector's rows are kept for the application of Q in the SVD sweep
        {
          const int* q = qsec + 1 + 6 * t;
          S* vq = Tq + q[4];
          for (long long e = threadIdx.x; e < (long long)mr * kr; e += blockDim.x) vq[e] = cvt<S>(g[e]);
          for (int x = threadIdx.x; x < mr; x += blockDim.x) qrow[q[3] + x] = R_[x];
          for (int y = threadIdx.x; y < kr; y += blockDim.x) qtau[koff + y] = tau[y];
        }
        for (int y = threadIdx.x; y < kr; y += blockDim.x) {
          s_kmap[koff + y] = (short)t;
          s_kloc[koff + y] = (short)y;
        }
        __syncthreads();
        koff += kr;
        rsz += (double)kr * mc;
      }
      toc(PH_QR, t0);
      t0 = tic();
      // the power-of-two normalisation is applied to the small factor R before the product instead
      // of to the product (exact either way): the product is not read and written a second time
      expo += block_normalize(Rb, (long long)rsz, red);
      // new T[i+1] (ktot x d'B') = R * T[i+1], sector by sector, into G; each thread owns a 4x4
      // output tile (4 rows of one sector's R x 4 columns), so one load of T feeds 4 FMAs.  The rows
      // C_ of T[i+1] that a sector's R reads share one left charge, so only the columns (d', b') with
      // charge F_{i+1} minus it can be nonzero in those rows (and in the sector's output rows): they
      // are listed (in rl, free after the Q scatter) and only they are computed; G starts zeroed.
      const int dB = s_dd[i + 1] * s_dB[i + 1];
      {
        const S* Tn = Tbuf(s_buf[i + 1]);
        const int Bn = s_dB[i + 1], Fn = s_fl[i + 1];
        const int* qLo = tqL(i + 1);  // left charges of T[i+1] before this step
        const int* qDn = tqD(i + 1);
        const int* qRn = tqR(i + 1);
        for (long long e = threadIdx.x; e < (long long)ktot * dB; e += blockDim.x) G[e] = (S)0;
        __syncthreads();
        int kof = 0;
        double fl = 0;
        for (int t = 0; t < ns; ++t) {
          const int mc = s_sec.c[t], kr = min(s_sec.m[t], mc);
          const T* rb = Rb + s_roffs[t];
          const int* C_ = cl + s_sec.co[t];
          const int want = Fn - qLo[C_[0]];
          const int nc = block_compact(
              dB, [&](int col) { return qDn[col / Bn] + qRn[col % Bn] == want; }, rl, s_sh);
          const int tr = (kr + 3) / 4, tc = (nc + 3) / 4;
          for (long long tile = threadIdx.x; tile < (long long)tr * tc; tile += blockDim.x) {
            const int y0 = (int)(tile / tc) * 4, c0 = (int)(tile % tc) * 4;
            int col[4];
#pragma unroll
            for (int u = 0; u < 4; ++u) col[u] = rl[c0 + u < nc ? c0 + u : nc - 1];
            S acc[4][4];
#pragma unroll
            for (int v = 0; v < 4; ++v)
#pragma unroll
              for (int u = 0; u < 4; ++u) acc[v][u] = (S)0;
            for (int z = y0; z < mc; ++z) {
              const S* trow = Tn + (long long)C_[z] * dB;
              S tv[4];
#pragma unroll
              for (int u = 0; u < 4; ++u) tv[u] = trow[col[u]];
#pragma unroll
              for (int v = 0; v < 4; ++v) {
                const S rv = (y0 + v < kr) ? cvt<S>(rb[(long long)(y0 + v) * mc + z]) : (S)0;
#pragma unroll
                for (int u = 0; u < 4; ++u) acc[v][u] = fma(rv, tv[u], acc[v][u]);
              }
            }
#pragma unroll
            for (int v = 0; v < 4; ++v)
              if (y0 + v < kr)
#pragma unroll
                for (int u = 0; u < 4; ++u)
                  if (c0 + u < nc) G[(long long)(kof + y0 + v) * dB + col[u]] = acc[v][u];
          }
          kof += kr;
          fl += 2.0 * nc * kr * mc;
          __syncthreads();  // rl is rewritten by the next sector's list
        }
        this->count(0, fl);
      }
      __syncthreads();
      // charges and flux of the new bond: Q side -r, R side +r
      {
        int* qRi = tqR(i);
        int* qLn = tqL(i + 1);
        for (int k = threadIdx.x; k < ktot; k += blockDim.x) {
          const int r = s_sec.r[s_kmap[k]];
          qRi[k] = -r;
          qLn[k] = r;
        }
      }
      __syncthreads();
      if (threadIdx.x == 0) {
        const int old_i = s_buf[i], old_n = s_buf[i + 1];
        s_buf[i] = spare;
        s_buf[i + 1] = spare2;
        s_buf[n] = old_i;
        s_buf[n + 1] = old_n;
        s_dB[i] = ktot;
        s_dA[i + 1] = ktot;
        s_fl[i + 1] += s_fl[i];
        s_fl[i] = 0;
      }
      __syncthreads();
      toc(PH_RABSORB, t0);
    }
    // ---------------- truncating SVD sweep, per sector, global cut ----------------
    T* X = at<T>(sl.o_X);
    T* V = at<T>(sl.o_V);
    T* sig = at<T>(sl.o_sig);
    for (int i = n - 1; i >= 1; --i) {
      const int d = s_dd[i], Bc = s_dB[i], rows = s_dA[i], cols = d * Bc, F = s_fl[i];
      const int* qL = tqL(i);
      const int* qD = tqD(i);
      const int* qR = tqR(i);
      t0 = tic();
      sectors(rows, cols, [&](int x) { return qL[x]; }, [&](int z) { return qD[z / Bc] + qR[z % Bc]; }, F, &s_sec,
              s_sh);
      toc(PH_SECTORS, t0);
      t0 = tic();
      const int ns = s_sec.n;
      if (threadIdx.x == 0) {
        int xo = 0, vo = 0, so = 0;
        for (int t = 0; t < ns; ++t) {
          const int nv = min(s_sec.m[t], s_sec.c[t]), len = max(s_sec.m[t], s_sec.c[t]);
          s_xo[t] = xo;
          s_vo[t] = vo;
          s_so[t] = so;
          xo += nv * len;
          vo += nv * nv;
          so += nv;
        }
      }
      __syncthreads();
      int nsv = 0;
      for (int t = 0; t < ns; ++t) nsv += min(s_sec.m[t], s_sec.c[t]);
      const S* M = Tbuf(s_buf[i]);
      // QR-preconditioned one-sided Jacobi (Drmac-Veselic): per sector, A (len x nv, its columns are
      // the block's columns when it is tall, its rows when wide) = Q R P^T by Householder QR with
      // column pivoting, then one-sided Jacobi on the nv columns of R^T, which converges in fewer
      // sweeps and on vectors of length nv.  With B = R^T and B J = W (J the product of the rotations):
      //   A = (Q J) Sigma (P W Sigma^-1)^T,  sigma_j = |W_j|.
      // Outputs per value j: nvvec_j = P W_j (nv-dim, sigma_j times unit) and, for the kept values only,
      // lenvec_j = (Q J)_j = A nvvec_j / sigma_j^2 (len-dim, unit), so neither J nor Q is formed.
      // Sector data sit in shared memory while it has room (the Jacobi vectors first), else in the slot.
      __shared__ int s_nvv[kMaxSec], s_lenv[kMaxSec], s_esec[kMaxSec];
      __shared__ T* s_xp[kMaxSec];  // A, then R and the reflectors (len x nv, column-major)
      __shared__ T* s_bp[kMaxSec];  // B = R^T vectors, rotated into W (nv x nv)
      T* Wl = at<T>(sl.o_W);                         // lenvec, packed at s_xo
      T* Wn = at<T>(sl.o_W) + (long long)chi() * chi();  // nvvec, packed at s_vo
      int* perm = order + md.cut;                    // pivots of the current sector (<= chi entries)
      if (threadIdx.x == 0) {
        long long used = 0;
        for (int t = 0; t < ns; ++t) {  // the Jacobi vectors first: every sweep reads and rotates them
          const int nv = min(s_sec.m[t], s_sec.c[t]), len = max(s_sec.m[t], s_sec.c[t]);
          s_nvv[t] = nv;
          s_lenv[t] = len;
          const long long nb = (long long)nv * nv;
          if (used + nb <= smcap) {
            s_bp[t] = sm + used;
            used += nb;
          } else {
            s_bp[t] = V + s_vo[t];
          }
        }
        for (int t = 0; t < ns; ++t) {  // then the blocks of the pivoted QR
          const long long nx = (long long)s_nvv[t] * s_lenv[t];
          if (used + nx <= smcap) {
            s_xp[t] = sm + used;
            used += nx;
          } else {
            s_xp[t] = X + s_xo[t];
          }
        }
      }
      __syncthreads();
      for (int t = 0; t < ns; ++t) {
        const int mr = s_sec.m[t], mc = s_sec.c[t];
        const bool caseA = mc <= mr;
        const int nv = caseA ? mc : mr, len = caseA ? mr : mc;
        const int* R_ = rl + s_sec.ro[t];
        const int* C_ = cl + s_sec.co[t];
        T* x = s_xp[t];
        for (long long e = threadIdx.x; e < (long long)nv * len; e += blockDim.x) {
          const int j = (int)(e / len), q = (int)(e % len);
          x[e] = cvt<T>(caseA ? M[(long long)R_[q] * cols + C_[j]] : M[(long long)R_[j] * cols + C_[q]]);
        }
        const double mm = len, nn = nv;
        this->count(2, 4.0 * mm * mm * nn + 8.0 * mm * nn * nn + 9.0 * nn * nn * nn);
      }
      __syncthreads();
      // QR with column pivoting per sector; B = R^T as nv vectors of length nv (vector i = row i of R)
      for (int t = 0; t < ns; ++t) {
        const int nv = s_nvv[t], len = s_lenv[t];
        T* x = s_xp[t];
        // exact power-of-two scaling of the sector (as in the QR sweep); sigma and P W are scaled back
        const int es = block_normalize(x, (long long)nv * len, red);
        if (threadIdx.x == 0) s_esec[t] = es;
        block_geqp3_cm(len, nv, x, tau + 0, perm, red);
        T* b = s_bp[t];
        for (long long e = threadIdx.x; e < (long long)nv * nv; e += blockDim.x) {
          const int i = (int)(e / nv), k = (int)(e % nv);
          b[e] = k >= i ? x[(long long)k * len + i] : (T)0;
        }
        // keep the pivots of this sector in its packed nvvec area, which is written last
        int* pk = reinterpret_cast<int*>(Wn + s_vo[t]);
        for (int k = threadIdx.x; k < nv; k += blockDim.x) pk[k] = perm[k];
        __syncthreads();
      }
      toc(PH_SVDOUT, t0);  // gather + pivoted QR
      t0 = tic();
      const int sweeps = ns == 1 ? block_jacobi(s_nvv[0], s_nvv[0], s_bp[0], (T*)nullptr, md.jacobi_max)
                                 : block_jacobi_multi<T, kMaxSec>(ns, s_nvv, s_nvv, s_bp, nullptr, md.jacobi_max);
      toc(PH_JACOBI, t0);
      t0 = tic();
      if (sweeps < 0 && threadIdx.x == 0) atomicOr(status, ST_SVD_NOCONV);
      this->count(CT_JACOBI_CALLS, 1.0);
      this->count(CT_JACOBI_SWEEPS, (double)(sweeps > 0 ? sweeps : 0));
      {
        const int lane = threadIdx.x & 31, wp = threadIdx.x >> 5;
        for (int t = 0; t < ns; ++t) {
          const int nv = s_nvv[t];
          const T* b = s_bp[t];
          const T ssc = (T)ldexp(1.0, s_esec[t]);
          for (int j = wp; j < nv; j += kWarps) {
            T s2 = 0;
            for (int q = lane; q < nv; q += 32) s2 = fma(b[(long long)j * nv + q], b[(long long)j * nv + q], s2);
            s2 = warp_sum(s2);
            if (lane == 0) sig[s_so[t] + j] = sqrt(s2) * ssc;
          }
        }
      }
      __syncthreads();
      const int c = md.cut < nsv ? md.cut : nsv;
      // global selection: descending value, ties to the earlier sector / lower index
      for (int j = threadIdx.x; j < nsv; j += blockDim.x) {
        const T sj = sig[j];
        int rank = 0;
        for (int k = 0; k < nsv; ++k) {
          const T sk = sig[k];
          rank += (sk > sj) || (sk == sj && k < j);
        }
        if (rank < c) order[rank] = j;
      }
      __syncthreads();
      // kept index -> (sector, local)
      for (int k = threadIdx.x; k < c; k += blockDim.x) {
        const int j = order[k];
        int t = 0;
        while (t + 1 < ns && s_so[t + 1] <= j) ++t;
        s_kmap[k] = (short)t;
        s_kloc[k] = (short)(j - s_so[t]);
      }
      __syncthreads();
      T smax = 0;
      for (int j = threadIdx.x; j < nsv; j += blockDim.x) smax = fmax(smax, sig[j]);
      smax = block_max(smax, red);
      int lmaxi = 1;
      for (int t = 0; t < ns; ++t) lmaxi = max(lmaxi, max(s_sec.m[t], s_sec.c[t]));
      const T thr = smax * Eps<T>::value() * (T)lmaxi;
      // per sector: nvvec = P W for every value; lenvec_j = A nvvec_j / sigma_j^2 for the kept ones
      // (zero below the noise floor thr, where the value carries no direction), A read back from the
      // compression tensor; each thread computes kCB kept vectors at one position (one load of A each)
      for (int t = 0; t < ns; ++t) {
        const int nv = s_nvv[t], len = s_lenv[t];
        const bool caseA = s_sec.c[t] <= s_sec.m[t];
        const int* R_ = rl + s_sec.ro[t];
        const int* C_ = cl + s_sec.co[t];
        const int* pk = reinterpret_cast<const int*>(Wn + s_vo[t]);
        for (int k = threadIdx.x; k < nv; k += blockDim.x) perm[k] = pk[k];
        __syncthreads();
        const T* b = s_bp[t];
        T* lv = Wl + s_xo[t];
        T* nvv = Wn + s_vo[t];
        const T ssc = (T)ldexp(1.0, s_esec[t]);
        for (long long e = threadIdx.x; e < (long long)nv * nv; e += blockDim.x) {
          const int j = (int)(e / nv), k = (int)(e % nv);
          nvv[(long long)j * nv + perm[k]] = b[e] * ssc;
        }
        int* kl = order;  // kept vectors of this sector (order is free after the selection)
        const int nk = block_compact(c, [&](int k) { return s_kmap[k] == t; }, kl, s_sh);  // ends with a barrier
        const int kb = (nk + kCB - 1) / kCB;
        for (long long e = threadIdx.x; e < (long long)kb * len; e += blockDim.x) {
          const int p0 = (int)(e / len) * kCB, q = (int)(e % len);
          int jv[kCB];
          T acc[kCB];
          const T* nj[kCB];
#pragma unroll
          for (int v = 0; v < kCB; ++v) {
            jv[v] = s_kloc[kl[p0 + v < nk ? p0 + v : nk - 1]];
            nj[v] = nvv + (long long)jv[v] * nv;
            acc[v] = 0;
          }
          for (int r = 0; r < nv; ++r) {
            const T a = cvt<T>(caseA ? M[(long long)R_[q] * cols + C_[r]] : M[(long long)R_[r] * cols + C_[q]]);
#pragma unroll
            for (int v = 0; v < kCB; ++v) acc[v] = fma(a, nj[v][r], acc[v]);
          }
#pragma unroll
          for (int v = 0; v < kCB; ++v)
            if (p0 + v < nk) {
              const T sv = sig[s_so[t] + jv[v]];
              lv[(long long)jv[v] * len + q] = sv > thr ? acc[v] / (sv * sv) : (T)0;
            }
        }
        __syncthreads();
      }
      const int spare = s_buf[n], spare2 = s_buf[n + 1];
      S* Tn = Tbuf(spare);  // new T[i] (c x cols)
      for (long long e = threadIdx.x; e < (long long)c * cols; e += blockDim.x) Tn[e] = (S)0;
      for (long long e = threadIdx.x; e < (long long)rows * c; e += blockDim.x) Rb[e] = (T)0;
      __syncthreads();
      const int span = max(rows, cols);
      for (long long e = threadIdx.x; e < (long long)c * span; e += blockDim.x) {
        const int k = (int)(e / span), q = (int)(e % span);
        const int t = s_kmap[k], j = s_kloc[k];
        const int mr = s_sec.m[t], mc = s_sec.c[t];
        const bool caseA = mc <= mr;
        const int nv = caseA ? mc : mr, len = caseA ? mr : mc;
        const T sv = sig[s_so[t] + j];
        const T* lj = Wl + s_xo[t] + (long long)j * len;   // unit, len-dim
        const T* nj = Wn + s_vo[t] + (long long)j * nv;    // sigma * unit, nv-dim
        // tall block (case A): columns are the nv side; wide block: rows are the nv side
        if (q < mc) {  // right singular vector component at column C[q]
          const T val = caseA ? (sv > thr ? nj[q] / sv : (T)0) : lj[q];
          Tn[(long long)k * cols + cl[s_sec.co[t] + q]] = cvt<S>(val);
        }
        if (q < mr) {  // U*S component at row R[q]
          const T val = caseA ? lj[q] * sv : nj[q];
          Rb[(long long)rl[s_sec.ro[t] + q] * c + k] = val;
        }
      }
      __syncthreads();
      toc(PH_SVDOUT, t0);
      t0 = tic();
      // U*S normalised before the absorption (exact; the product needs no second pass)
      expo += block_normalize(Rb, (long long)rows * c, red);
      // new T[i-1] (A d x c) = Q_{i-1} US with Q_{i-1} from its reflectors (LAPACK ormqr): per QR sector
      // of step i-1, the rows of US on its bonds are nonzero only in the kept columns of the bonds'
      // charge; that block is staged (in the G area), padded to the sector's rows, Q_t is applied to it
      // and the result goes to the sector's rows of T[i-1].  Rows in no sector stay zero.
      {
        const int Ad = s_dA[i - 1] * s_dd[i - 1];
        const S* Vq = Tbuf(s_buf[i - 1]);
        S* out = Tbuf(spare2);
        const int* qsec = at<int>(sl.o_qsec) + (long long)(i - 1) * (1 + 6 * kMaxSec);
        const int* qrow = at<int>(sl.o_qrow) + (long long)(i - 1) * chi() * md.Dmax;
        const T* qtau = at<T>(sl.o_qtau) + (long long)(i - 1) * chi();
        const T* qtw = at<T>(sl.o_qtw) + (long long)(i - 1) * (chi() + kMaxSec) * kNB * kNB;
        const int* qbond = tqL(i);  // charges of the bonds (the rows of T[i] and of US)
        T* Bs = at<T>(sl.o_G);
        int* kl = order;  // free after the selection above
        for (long long e = threadIdx.x; e < (long long)Ad * c; e += blockDim.x) out[e] = (S)0;
        __syncthreads();
        const int nq = qsec[0];
        double fl = 0;
        for (int t = 0; t < nq; ++t) {
          const int* q = qsec + 1 + 6 * t;
          const int mr = q[0], kr = q[1], ko = q[2];
          const int* Rq = qrow + q[3];
          const int rq = qbond[ko];
          const int nk = block_compact(c, [&](int k) { return s_sec.r[s_kmap[k]] == rq; }, kl, s_sh);
          if (nk == 0) continue;
          for (long long e = threadIdx.x; e < (long long)mr * nk; e += blockDim.x) {
            const int j = (int)(e / mr), x = (int)(e % mr);
            Bs[e] = x < kr ? Rb[(long long)(ko + x) * c + kl[j]] : (T)0;
          }
          __syncthreads();
          block_ormqr_panel(mr, kr, Vq + q[4], qtau + ko, Bs, nk, sm, smcap, q[5] >= 0 ? qtw + q[5] : (const T*)nullptr);
          for (long long e = threadIdx.x; e < (long long)mr * nk; e += blockDim.x) {
            const int j = (int)(e / mr), x = (int)(e % mr);
            out[(long long)Rq[x] * c + kl[j]] = cvt<S>(Bs[e]);
          }
          fl += 4.0 * mr * kr * nk;
          __syncthreads();  // Bs and the column list are reused by the next sector
        }
        this->count(1, fl);
      }
      {
        int* qLi = tqL(i);
        int* qRp = tqR(i - 1);
        for (int k = threadIdx.x; k < c; k += blockDim.x) {
          const int r = s_sec.r[s_kmap[k]];
          qLi[k] = r;
          qRp[k] = -r;
        }
      }
      __syncthreads();
      if (threadIdx.x == 0) {
        const int old_i = s_buf[i], old_p = s_buf[i - 1];
        s_buf[i] = spare;
        s_buf[i - 1] = spare2;
        s_buf[n] = old_i;
        s_buf[n + 1] = old_p;
        s_dA[i] = c;
        s_dB[i - 1] = c;
      }
      __syncthreads();
      toc(PH_USABSORB, t0);
    }
    if (n == 1) expo += block_normalize(Tbuf(s_buf[0]), (long long)s_dA[0] * s_dd[0] * s_dB[0], sred());
    // store the line with its charges
    for (int i = 0; i < n; ++i) {
      const long long cnt = (long long)s_dA[i] * s_dd[i] * s_dB[i];
      const S* src = Tbuf(s_buf[i]);
      S* dst = line(f, idx, i);
      for (long long t = threadIdx.x; t < cnt; t += blockDim.x) dst[t] = src[t];
      int* qa = lqa(f, idx, i);
      int* qb = lqb(f, idx, i);
      const int* sa = tqL(i);
      const int* sb = tqR(i);
      for (int x = threadIdx.x; x < s_dA[i]; x += blockDim.x) qa[x] = sa[x];
      for (int x = threadIdx.x; x < s_dB[i]; x += blockDim.x) qb[x] = sb[x];
      if (threadIdx.x == 0) {
        int* dd = ldim(f, idx, i);
        dd[0] = s_dA[i];
        dd[1] = s_dd[i];
        dd[2] = s_dB[i];
        *lflux(f, idx, i) = s_fl[i];
      }
    }
    if (threadIdx.x == 0) lexp[f * kMaxL + idx] = expo;
    __syncthreads();
  }

  // make line (f, idx) valid for the current configuration (recomputing its invalid upstreams)
  __device__ __noinline__ void ensure(int f, int idx) {
    if (is_ones(f, idx)) return;
    const bool forward = (f == F_UP || f == F_LEFT);
    if (valid[f * kMaxL + idx]) return;
    // first invalid index in the dependency chain
    int start = idx;
    if (forward) {
      while (start - 1 >= 0 && !valid[f * kMaxL + start - 1]) --start;
      for (int k = start; k <= idx; ++k) {
        compress(f, k);
        if (threadIdx.x == 0) valid[f * kMaxL + k] = 1;
        __syncthreads();
      }
    } else {
      while (start + 1 < nlines(f) && !valid[f * kMaxL + start + 1]) ++start;
      for (int k = start; k >= idx; --k) {
        compress(f, k);
        if (threadIdx.x == 0) valid[f * kMaxL + k] = 1;
        __syncthreads();
      }
    }
  }

  // sites changed: invalidate every line that contains them and the strip cache
  __device__ void invalidate_site(int l1, int l2) {
    if (threadIdx.x == 0) {
      for (int k = l1; k < md.L1; ++k) valid[F_UP * kMaxL + k] = 0;
      for (int k = 0; k <= l1; ++k) valid[F_DOWN * kMaxL + k] = 0;
      for (int k = l2; k < md.L2; ++k) valid[F_LEFT * kMaxL + k] = 0;
      for (int k = 0; k <= l2; ++k) valid[F_RIGHT * kMaxL + k] = 0;
    }
  }

  // strip geometry: kind 0 = row idx (lines up/down, orientation 0), 1 = column idx (left/right, orientation 2)
  __device__ int strip_len(int kind) const { return kind == 0 ? md.L2 : md.L1; }
  __device__ void strip_site_rc(int kind, int idx, int c, int& l1, int& l2) const {
    if (kind == 0) { l1 = idx; l2 = c; } else { l1 = c; l2 = idx; }
  }
  __device__ int fup(int kind) const { return kind == 0 ? F_UP : F_LEFT; }
  __device__ int fdn(int kind) const { return kind == 0 ? F_DOWN : F_RIGHT; }

  __device__ S* Ebuf(int c) const { return at<S>(sl.o_E) + (long long)c * sl.capE; }
  __device__ S* Fbuf(int c) const { return at<S>(sl.o_F) + (long long)c * sl.capE; }
  __device__ Dims3 Edims(int kind, int idx, int c) const {
    // E[c] = columns 0..c-1 : (up bond, site bond, down bond) at cut c
    if (c == 0) return Dims3{1, 1, 1};
    int l1, l2;
    strip_site_rc(kind, idx, c - 1, l1, l2);
    const SiteView w = site(l1, l2, 0, kind == 0 ? 0 : 2);
    return Dims3{lsdim(fup(kind), idx - 1, c - 1).b, w.dr, lsdim(fdn(kind), idx + 1, c - 1).b};
  }
  __device__ Dims3 Fdims(int kind, int idx, int c) const {
    const int n = strip_len(kind);
    if (c == n) return Dims3{1, 1, 1};
    int l1, l2;
    strip_site_rc(kind, idx, c, l1, l2);
    const SiteView w = site(l1, l2, 0, kind == 0 ? 0 : 2);
    return Dims3{lsdim(fup(kind), idx - 1, c).a, w.dl, lsdim(fdn(kind), idx + 1, c).a};
  }

  // E[c+1] = E[c] x column c (physical index s); writes into dst with exponent returned
  __device__ __noinline__ int step_left(int kind, int idx, int c, const S* Ein, Dims3 e, int s, S* dst, int mp = 0) {
    const long long t0 = tic();
    int l1, l2;
    strip_site_rc(kind, idx, c, l1, l2);
    const SiteView w = site(l1, l2, s, kind == 0 ? 0 : 2, mp);
    strip_left(Ein, e.a, e.p, e.b, lsite(fup(kind), idx - 1, c), lsdim(fup(kind), idx - 1, c), A, w,
               lsite(fdn(kind), idx + 1, c), lsdim(fdn(kind), idx + 1, c), at<S>(sl.o_t1), at<S>(sl.o_t2), dst);
    const Dims3 up = lsdim(fup(kind), idx - 1, c), dn = lsdim(fdn(kind), idx + 1, c);
    this->count(3, 2.0 * ((double)e.a * e.p * e.b * up.p * up.b + (double)e.b * up.b * dn.p * w.dr * e.p * up.p +
                          (double)up.b * w.dr * dn.b * e.b * dn.p));
    const int ex = block_normalize(dst, (long long)up.b * w.dr * dn.b, sred());
    toc(PH_STRIP, t0);
    return ex;
  }
  __device__ __noinline__ int step_right(int kind, int idx, int c, const S* Fin, Dims3 f, int s, S* dst, int mp = 0) {
    const long long t0 = tic();
    int l1, l2;
    strip_site_rc(kind, idx, c, l1, l2);
    const SiteView w = site(l1, l2, s, kind == 0 ? 0 : 2, mp);
    strip_right(Fin, f.a, f.p, f.b, lsite(fup(kind), idx - 1, c), lsdim(fup(kind), idx - 1, c), A, w,
                lsite(fdn(kind), idx + 1, c), lsdim(fdn(kind), idx + 1, c), at<S>(sl.o_t1), at<S>(sl.o_t2), dst);
    const Dims3 up = lsdim(fup(kind), idx - 1, c), dn = lsdim(fdn(kind), idx + 1, c);
    this->count(3, 2.0 * ((double)up.a * up.p * f.a * f.p * f.b + (double)up.a * w.dl * dn.p * f.b * up.p * f.p +
                          (double)up.a * w.dl * dn.a * dn.p * f.b));
    const int ex = block_normalize(dst, (long long)up.a * w.dl * dn.a, sred());
    toc(PH_STRIP, t0);
    return ex;
  }

  __device__ int conf_at(int kind, int idx, int c) const {
    int l1, l2;
    strip_site_rc(kind, idx, c, l1, l2);
    return conf[l1 * md.L2 + l2];
  }

  // particles at strip positions before c (0 for a bosonic lattice, where it is not used)
  __device__ int strip_prefix(int kind, int idx, int c) const {
    return md.fermion ? strip_prefix_of(conf, md.L2, kind, idx, c) : 0;
  }

  // build the strip (kind, idx) for the current configuration: all F, E[0]
  __device__ __noinline__ void strip_begin(int kind, int idx) {
    ensure(fup(kind), idx - 1);
    ensure(fdn(kind), idx + 1);
    const int n = strip_len(kind);
    S* F = Fbuf(n);
    if (threadIdx.x == 0) F[0] = (S)1;
    S* E = Ebuf(0);
    if (threadIdx.x == 0) E[0] = (S)1;
    if (threadIdx.x == 0) {
      eF[n] = 0;
      eE[0] = 0;
    }
    __syncthreads();
    for (int c = n - 1; c >= 0; --c) {
      const int e = step_right(kind, idx, c, Fbuf(c + 1), Fdims(kind, idx, c + 1), conf_at(kind, idx, c), Fbuf(c),
                               strip_prefix(kind, idx, c));
      if (threadIdx.x == 0) eF[c] = eF[c + 1] + e;
      __syncthreads();
    }
    if (threadIdx.x == 0) {
      *strip_kind = kind;
      *strip_idx = idx;
      *strip_eupto = 0;
      *strip_ffrom = 0;
    }
    __syncthreads();
  }

  __device__ __noinline__ void strip_advance(int kind, int idx, int c) {
    // make E[c] valid
    while (*strip_eupto < c) {
      const int k = *strip_eupto;
      const int e = step_left(kind, idx, k, Ebuf(k), Edims(kind, idx, k), conf_at(kind, idx, k), Ebuf(k + 1),
                              strip_prefix(kind, idx, k));
      if (threadIdx.x == 0) {
        eE[k + 1] = eE[k] + e;
        *strip_eupto = k + 1;
      }
      __syncthreads();
    }
  }

  // amplitude with columns c, c+1 of the strip set to s0, s1 (E[c] and F[c+2] valid)
  __device__ __noinline__ void strip_replace2(int kind, int idx, int c, int s0, int s1, double& m, int& ex) {
    S* w0 = at<S>(sl.o_w0);
    S* w1 = at<S>(sl.o_w1);
    const int mp0 = strip_prefix(kind, idx, c);  // the pair's second site counts the first one's new value
    const int e0 = step_left(kind, idx, c, Ebuf(c), Edims(kind, idx, c), s0, w0, mp0);
    const int e1 = step_left(kind, idx, c + 1, w0, Edims(kind, idx, c + 1), s1, w1, mp0 + s0);
    const Dims3 fd = Fdims(kind, idx, c + 2);
    const S v = block_dot(w1, Fbuf(c + 2), (long long)fd.a * fd.p * fd.b, sred());
    m = (double)v;
    ex = eE[c] + e0 + e1 + eF[c + 2] + lexpo(fup(kind), idx - 1) + lexpo(fdn(kind), idx + 1);
  }

  // hole(()) = _inline_right_to_left[0, 0]: the row-0 strip (single_layer_auxiliaries.py:710-720)
  __device__ __noinline__ void hole0(double& m, int& ex) {
    ensure(F_DOWN, 1);
    const int n = md.L2;
    S* f0 = at<S>(sl.o_w0);
    S* f1 = at<S>(sl.o_w1);
    if (threadIdx.x == 0) f0[0] = (S)1;
    __syncthreads();
    int e = 0;
    Dims3 fd{1, 1, 1};
    for (int c = n - 1; c >= 0; --c) {
      e += step_right(0, 0, c, f0, fd, conf_at(0, 0, c), f1, strip_prefix(0, 0, c));
      fd = Fdims(0, 0, c);
      S* t = f0;
      f0 = f1;
      f1 = t;
    }
    m = (double)f0[0];
    ex = e + lexpo(F_DOWN, 1);
    __syncthreads();
  }
};

// per-slot integer arrays and the dynamic shared-memory staging area of this block
template <class T, class S> __device__ void bind_slot(Engine<T, S>& eng, const Slots& sl, const Model& md) {
  extern __shared__ __align__(16) unsigned char dyn_smem[];
  const long long chi = (long long)md.cut * md.Dmax;
  eng.lq = sl.lq + (long long)blockIdx.x * 4 * kMaxL * kMaxL * 2 * md.cut;
  eng.lfl = sl.lfl + (long long)blockIdx.x * 4 * kMaxL * kMaxL;
  eng.tq = sl.tq + (long long)blockIdx.x * kMaxL * 3 * chi;
  eng.tfl = sl.tfl + (long long)blockIdx.x * kMaxL;
  eng.ilist = sl.ilist + (long long)blockIdx.x * (chi * md.Dmax + chi);
  eng.smem = reinterpret_cast<T*>(dyn_smem);
}

__device__ __forceinline__ double ratio_of(double m1, int e1, double m0, int e0) {
  return ldexp(m1 / m0, e1 - e0);
}

// occupation of site i of a fermionic configuration with sites ia, ib replaced by na, nb
__host__ __device__ __forceinline__ int occ_after(const short* conf, int i, int ia, int na, int ib, int nb) {
  return i == ia ? na : i == ib ? nb : conf[i];
}

// parity bit of the configuration sign prod_k (-1)^((N_<k + p_T)(N_<=k + p_T)) over the cuts between rows
// (rows = 1) or columns (rows = 0), of the configuration with sites ia, ib replaced
__host__ __device__ inline int config_sign_bit(const short* conf, int L1, int L2, int pT, int rows, int ia, int na, int ib, int nb) {
  const int nk = rows ? L1 : L2, len = rows ? L2 : L1;
  int s = 0, before = pT & 1;
  for (int k = 0; k + 1 < nk; ++k) {
    int cnt = 0;
    for (int j = 0; j < len; ++j) cnt += occ_after(conf, rows ? k * L2 + j : j * L2 + k, ia, na, ib, nb);
    const int upto = (before + cnt) & 1;
    s ^= before & upto;
    before = upto;
  }
  return s;
}

// sign of one E_loc term of a fermionic lattice, for amplitudes ws from the row strips and wss from the
// row (horizontal pair) or column (vertical pair) strips of the bosonized slices: the hop's string of
// particles between the two sites in row-major order (-1 more for a forward move) and, for a vertical
// pair, the column and row configuration signs and the parity of the order inversions of the new
// configuration
__host__ __device__ inline double fermion_term_sign(const short* conf, int L1, int L2, int pT, int ia, int na, int ib, int nb,
                                    int vertical) {
  const int i = ia < ib ? ia : ib, j = ia < ib ? ib : ia;
  const int new_i = i == ia ? na : nb;
  int s = 0;
  for (int k = i + 1; k < j; ++k) s ^= conf[k] & 1;
  if (conf[i] == 1 && new_i == 0) s ^= 1;
  if (vertical) {
    s ^= config_sign_bit(conf, L1, L2, pT, 0, ia, na, ib, nb);
    s ^= config_sign_bit(conf, L1, L2, pT, 1, -1, 0, -1, 0);
    int inv = 0;
    for (int a = 1; a < L1; ++a)
      for (int b = 0; b + 1 < L2; ++b) {
        if (!occ_after(conf, a * L2 + b, ia, na, ib, nb)) continue;
        for (int a2 = 0; a2 < a; ++a2)
          for (int b2 = b + 1; b2 < L2; ++b2) inv += occ_after(conf, a2 * L2 + b2, ia, na, ib, nb);
      }
    s ^= inv & 1;
  }
  return s ? -1.0 : 1.0;
}

// one Metropolis proposal on the term at (kind, idx, c)-(kind, idx, c+1)
template <class T, class S>
__device__ __noinline__ void single_term(Engine<T, S>& eng, const Model& md, int kind, int idx, int c, int t, uint64_t* mt, int* s_mti,
                            double* s_ws_m, int* s_ws_e, int* s_h0_valid, double* s_h0_m, int* s_h0_e, int64_t* accepted) {
  __shared__ int s_sel, s_nn, s_acc, s_skip;
  __shared__ double s_m;
  __shared__ int s_e;
  const int P = md.P;
  int l1a, l2a, l1b, l2b;
  eng.strip_site_rc(kind, idx, c, l1a, l2a);
  eng.strip_site_rc(kind, idx, c + 1, l1b, l2b);
  const int flip = md.s_hflip[t];
  const int sa = eng.conf[l1a * md.L2 + l2a], sb = eng.conf[l1b * md.L2 + l2b];
  const int in0 = flip ? sb : sa, in1 = flip ? sa : sb;
  const int key = in0 * P + in1;
  const int cnt = md.s_tab_cnt[t * P * P + key];
  if (cnt <= 0) return;  // not in the element pool, or no hopping
  __shared__ int s_ok;
  if (threadIdx.x == 0) {
    int mti = *s_mti;
    const int pick = draw_uniform_int(mt, mti, cnt);
    *s_mti = mti;
    const int entry = md.s_tab_off[t * P * P + key] + pick;
    const int out = md.s_tab_out[entry];
    s_sel = out;
    s_nn = md.s_tab_cnt[t * P * P + out];
    // a restricted subspace rejects the proposal before its ratio and its uniform draw (sampling.py:133-136)
    s_ok = md.s_allow ? md.s_allow[entry] : 1;
  }
  __syncthreads();
  if (!s_ok) return;
  const int out = s_sel;
  const int o0 = out / P, o1 = out % P;
  const int na = flip ? o1 : o0, nb = flip ? o0 : o1;
  double m;
  int ex;
  if (na == sa && nb == sb) {
    // replace({}) returns hole(()) (single_layer_auxiliaries.py:501-509)
    if (!*s_h0_valid) {
      eng.hole0(m, ex);
      if (threadIdx.x == 0) {
        *s_h0_m = m;
        *s_h0_e = ex;
        *s_h0_valid = 1;
      }
      __syncthreads();
    }
    m = *s_h0_m;
    ex = *s_h0_e;
  } else if (na != sa && nb != sb) {
    eng.strip_advance(kind, idx, c);
    eng.strip_replace2(kind, idx, c, na, nb, m, ex);
  } else {
    if (threadIdx.x == 0) atomicOr(eng.status, ST_UNSUPPORTED);
    return;
  }
  if (threadIdx.x == 0) {
    const double r = ratio_of(m, ex, *s_ws_m, *s_ws_e);
    const double a = sqrt(r * r);
    const double p = a * a * (double)cnt / (double)s_nn;
    int mti = *s_mti;
    const double u = draw_uniform_real(mt, mti);
    *s_mti = mti;
    // IEEE semantics as in the reference: ws == 0 gives p = inf (accepted) or, for 0/0, NaN
    // (rejected); the event is recorded in the status word, not treated as a failure
    s_acc = u < p;
    if (*s_ws_m == 0.0) atomicOr(eng.status, ST_ZERO_WS);
    s_m = m;
    s_e = ex;
    s_skip = (na == sa && nb == sb);
  }
  __syncthreads();
  if (s_acc) {
    if (threadIdx.x == 0) {
      *s_ws_m = s_m;
      *s_ws_e = s_e;
    }
    if (!s_skip) {
      if (threadIdx.x == 0) {
        eng.conf[l1a * md.L2 + l2a] = (short)na;
        eng.conf[l1b * md.L2 + l2b] = (short)nb;
        *s_h0_valid = 0;
        *accepted += 1;
        // E[c] stays valid, E[c+1..] do not; F[c+2..] stays valid
        if (*eng.strip_eupto > c) *eng.strip_eupto = c;
      }
      eng.invalidate_site(l1a, l2a);
      eng.invalidate_site(l1b, l2b);
    }
  }
  __syncthreads();
}

template <class T, class S>
__global__ void __launch_bounds__(kThreads) sweep_kernel(Model md, Chains ch, Slots sl, unsigned char* scratch,
                                                         const S* ones, int nsweeps, int observe, int rec_base) {
  // nsweeps == 0 with observe: observe the current configurations once, without sweeping
  const bool observe_only = nsweeps == 0 && observe;
  const int nsteps = observe_only ? 1 : nsweeps;
  __shared__ short s_conf[kMaxSites];
  __shared__ unsigned char s_valid[4 * kMaxL];
  __shared__ int s_eE[kMaxL + 1], s_eF[kMaxL + 1];
  __shared__ T s_red[kWarps];
  __shared__ double s_dred[kWarps];
  __shared__ int s_mti, s_ws_e, s_h0_valid, s_h0_e;
  __shared__ double s_ws_m, s_h0_m;
  __shared__ int s_strip_kind, s_strip_idx, s_strip_eupto, s_strip_ffrom;
  __shared__ int64_t s_accepted;
  __shared__ double s_fl[kCounters];
  if (threadIdx.x < kCounters) s_fl[threadIdx.x] = 0.0;
  __syncthreads();
  const int nsite = md.L1 * md.L2;
  Engine<T, S> eng{{md, sl, scratch + (long long)blockIdx.x * sl.stride, (const S*)md.A,
                    sl.ldims + (long long)blockIdx.x * 4 * kMaxL * kMaxL * 3, sl.lexp + (long long)blockIdx.x * 4 * kMaxL,
                    sl.order + (long long)blockIdx.x * md.cut * (md.Dmax + 1), s_conf, s_valid, s_eE, s_eF, s_red, s_dred,
                    s_fl},
                   ones, ch.status};
  eng.strip_kind = &s_strip_kind;
  eng.strip_idx = &s_strip_idx;
  eng.strip_eupto = &s_strip_eupto;
  eng.strip_ffrom = &s_strip_ffrom;
  bind_slot(eng, sl, md);
  double* delta = sl.delta + (long long)blockIdx.x * md.n_params;
  double* edelta = sl.edelta + (long long)blockIdx.x * md.n_params;
  double* contrib = sl.contrib + (long long)blockIdx.x * md.n_terms;
  for (int b = blockIdx.x; b < ch.B; b += gridDim.x) {
    for (int i = threadIdx.x; i < nsite; i += blockDim.x) s_conf[i] = (short)ch.conf[(long long)b * nsite + i];
    for (int i = threadIdx.x; i < 4 * kMaxL; i += blockDim.x) s_valid[i] = 0;
    if (threadIdx.x == 0) {
      s_mti = ch.mti[b];
      s_h0_valid = 0;
      s_strip_kind = -1;
      s_accepted = 0;
    }
    __syncthreads();
    uint64_t* mt = ch.mt + (long long)b * kMtN;
    for (int sw = 0; sw < nsteps; ++sw) {
      // ws = hole(())  (sampling.py:146-148)
      {
        double m;
        int e;
        eng.hole0(m, e);
        if (threadIdx.x == 0) {
          s_ws_m = m;
          s_ws_e = e;
          s_h0_m = m;
          s_h0_e = e;
          s_h0_valid = 1;
        }
        __syncthreads();
      }
      // horizontal bonds, row-major (sampling.py:159-177)
      for (int l1 = 0; l1 < md.L1 && !observe_only; ++l1) {
        bool any = false;
        for (int l2 = 0; l2 + 1 < md.L2; ++l2) any |= md.s_hterm[l1 * md.L2 + l2] >= 0;
        if (!any) continue;
        eng.strip_begin(0, l1);
        for (int l2 = 0; l2 + 1 < md.L2; ++l2) {
          const int t = md.s_hterm[l1 * md.L2 + l2];
          if (t < 0) continue;
          single_term(eng, md, 0, l1, l2, t, mt, &s_mti, &s_ws_m, &s_ws_e, &s_h0_valid, &s_h0_m, &s_h0_e, &s_accepted);
        }
      }
      // vertical bonds, column-major (sampling.py:178-186)
      for (int l2 = 0; l2 < md.L2 && !observe_only; ++l2) {
        bool any = false;
        for (int l1 = 0; l1 + 1 < md.L1; ++l1) any |= md.s_vterm[l1 * md.L2 + l2] >= 0;
        if (!any) continue;
        eng.strip_begin(1, l2);
        for (int l1 = 0; l1 + 1 < md.L1; ++l1) {
          const int t = md.s_vterm[l1 * md.L2 + l2];
          if (t < 0) continue;
          single_term(eng, md, 1, l2, l1, t, mt, &s_mti, &s_ws_m, &s_ws_e, &s_h0_valid, &s_h0_m, &s_h0_e, &s_accepted);
        }
      }
      if (!observe) continue;
      // ---------------- Observer.__call__ (observer.py:313-415) ----------------
      double ws_m;
      int ws_e;
      eng.hole0(ws_m, ws_e);
      __shared__ double s_rw;
      if (threadIdx.x == 0) {
        const double r = ratio_of(ws_m, ws_e, s_ws_m, s_ws_e);  // ws / ws_sweep
        s_rw = r * r;                                          // |ws|^2 / possibility
        if (ws_m == 0.0) atomicOr(ch.status, ST_ZERO_WS);
      }
      for (int t = threadIdx.x; t < md.n_terms; t += blockDim.x) contrib[t] = 0.0;
      __syncthreads();
      const double rw = s_rw;
      const bool zero_ws = (ws_m == 0.0);
      // energy terms, grouped by strip; contributions kept per term and summed in term order
      for (int kind = 0; kind < 2 && !zero_ws; ++kind) {
        const int nl = kind == 0 ? md.L1 : md.L2;
        const int len = kind == 0 ? md.L2 : md.L1;
        for (int idx = 0; idx < nl; ++idx) {
          eng.strip_begin(kind, idx);
          eng.strip_advance(kind, idx, len);
          for (int c = 0; c + 1 < len; ++c) {
            int l1a, l2a, l1b, l2b;
            eng.strip_site_rc(kind, idx, c, l1a, l2a);
            eng.strip_site_rc(kind, idx, c + 1, l1b, l2b);
            const int t = kind == 0 ? md.hterm[l1a * md.L2 + l2a] : md.vterm[l1a * md.L2 + l2a];
            if (t < 0) continue;
            const int flip = md.hflip[t];
            const int sa = s_conf[l1a * md.L2 + l2a], sb = s_conf[l1b * md.L2 + l2b];
            const int key = (flip ? sb : sa) * md.P + (flip ? sa : sb);
            const int cnt = md.tab_cnt[t * md.P * md.P + key];
            double total = 0.0;
            for (int k = 0; k < cnt; ++k) {
              const int entry = md.tab_off[t * md.P * md.P + key] + k;
              if (md.e_allow && !md.e_allow[entry]) continue;  // outside the restricted subspace (observer.py:364-367)
              const int out = md.tab_out[entry];
              const double v = md.tab_val[entry];
              const int o0 = out / md.P, o1 = out % md.P;
              const int na = flip ? o1 : o0, nb = flip ? o0 : o1;
              if (na == sa && nb == sb) {
                total += v;
              } else if (na != sa && nb != sb) {
                double m;
                int e;
                eng.strip_replace2(kind, idx, c, na, nb, m, e);
                const double sg = md.fermion ? fermion_term_sign(s_conf, md.L1, md.L2, md.pT, l1a * md.L2 + l2a, na,
                                                                 l1b * md.L2 + l2b, nb, kind)
                                             : 1.0;
                if (m != 0.0) total += sg * v * ratio_of(m, e, ws_m, ws_e);
              } else {
                if (threadIdx.x == 0) atomicOr(ch.status, ST_UNSUPPORTED);
              }
            }
            if (threadIdx.x == 0) contrib[t] = total;
          }
        }
      }
      __syncthreads();
      __shared__ double s_eloc;
      if (threadIdx.x == 0) {
        double e = 0.0;
        for (int t = 0; t < md.n_terms; ++t) e += contrib[t];
        s_eloc = e;
      }
      __syncthreads();
      const double eloc = s_eloc;
      const long long t_obs = eng.tic();
      if (!zero_ws) {
        // holes: d psi / d A[l1,l2] / ws, accumulated with weight rw and E_loc * rw
        for (int l1 = 0; l1 < md.L1; ++l1) {
          eng.strip_begin(0, l1);
          eng.strip_advance(0, l1, md.L2);
          for (int l2 = 0; l2 < md.L2; ++l2) {
            const Dims3 ed = eng.Edims(0, l1, l2);
            const Dims3 fd = eng.Fdims(0, l1, l2 + 1);
            S* h = eng.template at<S>(sl.o_h);
            S* h1 = eng.template at<S>(sl.o_t1);
            S* h2 = eng.template at<S>(sl.o_t2);
            strip_hole(eng.Ebuf(l2), ed.a, ed.p, ed.b, eng.lsite(F_UP, l1 - 1, l2), eng.lsdim(F_UP, l1 - 1, l2),
                       eng.lsite(F_DOWN, l1 + 1, l2), eng.lsdim(F_DOWN, l1 + 1, l2), eng.Fbuf(l2 + 1), fd.p, h1, h2, h);
            {
              const Dims3 ud = eng.lsdim(F_UP, l1 - 1, l2), dd = eng.lsdim(F_DOWN, l1 + 1, l2);
              eng.count(3, 2.0 * ((double)ed.p * ed.b * ud.p * ud.b * ed.a + (double)ed.p * ud.p * ud.b * dd.p * dd.b * ed.b +
                                  (double)ud.p * dd.p * ed.p * fd.p * ud.b * dd.b));
            }
            const int ex = s_eE[l2] + s_eF[l2 + 1] + eng.lexpo(F_UP, l1 - 1) + eng.lexpo(F_DOWN, l1 + 1);
            const double fh = ldexp(1.0 / ws_m, ex - ws_e);  // hole / ws
            const double f = fh * rw;
            const int id = l1 * md.L2 + l2;
            const int* d = md.dims + id * 4;
            const long long n = (long long)d[0] * d[1] * d[2] * d[3];
            const long long base = (md.poff ? md.poff : md.off)[id] + (long long)s_conf[id] * n;
            // fermionic lattice: the hole of a slice read with an odd row prefix carries the prefix parity
            // on its odd D indices
            const int* qD = md.qleg + (long long)id * 4 * md.Dmax + md.Dmax;
            const int LR = d[2] * d[3];
            const bool odd_prefix = md.fermion && (eng.strip_prefix(0, l1, l2) & 1);
            for (long long q = threadIdx.x; q < n; q += blockDim.x) {
              double hv = (double)h[q] * f;
              if (odd_prefix && (qD[(q / LR) % d[1]] & 1)) hv = -hv;
              delta[base + q] += hv;
              edelta[base + q] += eloc * hv;
            }
            if (ch.rec_hole) {
              double* row = ch.rec_hole + (ch.hole_row0 + (long long)(rec_base + sw) * ch.B + b) * md.n_params;
              for (long long q = threadIdx.x; q < n; q += blockDim.x) {
                const double hv = (double)h[q] * fh;
                row[base + q] = (odd_prefix && (qD[(q / LR) % d[1]] & 1)) ? -hv : hv;
              }
            }
            __syncthreads();
          }
        }
      }
      eng.toc(PH_OBSERVE, t_obs);
      if (threadIdx.x == 0) {
        double* acc = ch.acc + (long long)b * 8;
        acc[0] += 1.0;
        if (!zero_ws) {
          acc[1] += rw;
          acc[2] += rw * rw;
          acc[3] += log(fabs(ws_m)) + (double)ws_e * 0.6931471805599453;
          acc[4] += eloc * rw;
          acc[5] += eloc * rw * rw;
          acc[6] += eloc * eloc * rw * rw;
        }
        const long long r = (long long)(rec_base + sw) * ch.B + b;
        if (ch.rec_eloc) {
          ch.rec_eloc[r] = eloc;
          ch.rec_logws[r] = log(fabs(ws_m)) + (double)ws_e * 0.6931471805599453;
          ch.rec_rw[r] = rw;
        }
      }
      __syncthreads();
    }
    // write back the chain
    for (int i = threadIdx.x; i < nsite; i += blockDim.x) ch.conf[(long long)b * nsite + i] = s_conf[i];
    if (threadIdx.x == 0) {
      ch.mti[b] = s_mti;
      ch.ws_m[b] = s_ws_m;
      ch.ws_e[b] = s_ws_e;
      ch.accepted[b] += s_accepted;
      ch.acc[(long long)b * 8 + 7] += (double)s_accepted;
    }
    __syncthreads();
  }
  if (threadIdx.x < kCounters) sl.flops[(long long)blockIdx.x * kCounters + threadIdx.x] += s_fl[threadIdx.x];
}

// amplitude hole(()) of arbitrary configurations (no RNG, no accumulators)
template <class T, class S>
__global__ void __launch_bounds__(kThreads) amplitude_kernel(Model md, Slots sl, unsigned char* scratch, const S* ones,
                                                             int B, const int32_t* confs, double* out_m, int32_t* out_e,
                                                             int32_t* status) {
  __shared__ short s_conf[kMaxSites];
  __shared__ unsigned char s_valid[4 * kMaxL];
  __shared__ int s_eE[kMaxL + 1], s_eF[kMaxL + 1];
  __shared__ T s_red[kWarps];
  __shared__ double s_dred[kWarps];
  __shared__ int s_strip_kind, s_strip_idx, s_strip_eupto, s_strip_ffrom;
  __shared__ double s_fl[kCounters];
  if (threadIdx.x < kCounters) s_fl[threadIdx.x] = 0.0;
  __syncthreads();
  const int nsite = md.L1 * md.L2;
  Engine<T, S> eng{{md, sl, scratch + (long long)blockIdx.x * sl.stride, (const S*)md.A,
                    sl.ldims + (long long)blockIdx.x * 4 * kMaxL * kMaxL * 3, sl.lexp + (long long)blockIdx.x * 4 * kMaxL,
                    sl.order + (long long)blockIdx.x * md.cut * (md.Dmax + 1), s_conf, s_valid, s_eE, s_eF, s_red, s_dred,
                    s_fl},
                   ones, status};
  eng.strip_kind = &s_strip_kind;
  eng.strip_idx = &s_strip_idx;
  eng.strip_eupto = &s_strip_eupto;
  eng.strip_ffrom = &s_strip_ffrom;
  bind_slot(eng, sl, md);
  for (int b = blockIdx.x; b < B; b += gridDim.x) {
    for (int i = threadIdx.x; i < nsite; i += blockDim.x) s_conf[i] = (short)confs[(long long)b * nsite + i];
    for (int i = threadIdx.x; i < 4 * kMaxL; i += blockDim.x) s_valid[i] = 0;
    __syncthreads();
    double m;
    int e;
    eng.hole0(m, e);
    if (threadIdx.x == 0) {
      out_m[b] = m;
      out_e[b] = e;
    }
    __syncthreads();
  }
}

}  // namespace tnsp
