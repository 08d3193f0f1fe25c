// C ABI of the sampler (declared in include/tnsp_gb300.h): host-side plan, buffers and launches.
// The kernels are instantiated in sampler_f64.cu / sampler_dd.cu / sampler_f32.cu and reached
// through launch.h.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdio>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/tnsp_gb300.h"
#include "capi_internal.h"

using namespace tnsp;

namespace tnsp {
// sum the per-slot gradient accumulators in slot order (deterministic)
__global__ void reduce_slots(const double* __restrict__ src, int nslots, long long n, double* __restrict__ dst) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    double s = 0.0;
    for (int k = 0; k < nslots; ++k) s += src[(long long)k * n + i];
    dst[i] = s;
  }
}

// y[s] = sum_p H[s][p] x[p] over the kept hole rows: one block per row, fixed-order reduction
__global__ void holes_gemv_rows(const double* __restrict__ H, long long np, long long rows, const double* __restrict__ x,
                                double* __restrict__ y) {
  __shared__ double red[8];
  for (long long s = blockIdx.x; s < rows; s += gridDim.x) {
    const double* h = H + s * np;
    double acc = 0.0;
    for (long long p = threadIdx.x; p < np; p += blockDim.x) acc = fma(h[p], x[p], acc);
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
      double t = 0.0;
      for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += red[w];
      y[s] = t;
    }
    __syncthreads();
  }
}

// y[p] = sum_s H[s][p] u[s]: one thread per parameter, rows in order (coalesced along a row)
// G = H H^T over the kept hole rows (rows x np, row-major): one 32 x 32 tile of G per block of 32 x 8
// threads, the rows of both tiles staged in shared memory 32 parameters at a time; each thread
// accumulates four entries of its column (float64, the parameters in order).
__global__ void holes_gram(const double* __restrict__ H, long long np, long long rows, double* __restrict__ G) {
  __shared__ double a[32][33], b[32][33];
  const int tx = threadIdx.x, ty = threadIdx.y;
  const long long i0 = (long long)blockIdx.y * 32, j0 = (long long)blockIdx.x * 32;
  double acc[4] = {0.0, 0.0, 0.0, 0.0};
  for (long long k0 = 0; k0 < np; k0 += 32) {
    for (int r = ty; r < 32; r += 8) {
      const long long k = k0 + tx;
      a[r][tx] = (i0 + r < rows && k < np) ? H[(i0 + r) * np + k] : 0.0;
      b[r][tx] = (j0 + r < rows && k < np) ? H[(j0 + r) * np + k] : 0.0;
    }
    __syncthreads();
#pragma unroll 8
    for (int c = 0; c < 32; ++c) {
      const double bv = b[tx][c];
#pragma unroll
      for (int m = 0; m < 4; ++m) acc[m] = fma(a[ty + 8 * m][c], bv, acc[m]);
    }
    __syncthreads();
  }
  for (int m = 0; m < 4; ++m) {
    const long long i = i0 + ty + 8 * m, j = j0 + tx;
    if (i < rows && j < rows) G[i * rows + j] = acc[m];
  }
}

__global__ void holes_gemv_cols(const double* __restrict__ H, long long np, long long rows, const double* __restrict__ u,
                                double* __restrict__ y) {
  for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < np; p += (long long)gridDim.x * blockDim.x) {
    double acc = 0.0;
    for (long long s = 0; s < rows; ++s) acc = fma(H[s * np + p], u[s], acc);
    y[p] = acc;
  }
}

template <class T> __global__ void fill_ones(T* p) {
  if (threadIdx.x == 0 && blockIdx.x == 0) p[0] = (T)1;
}

// float and double-float copies of the float64 site tensors (round to nearest; hi + lo carries
// the float64 value to about 2^-48 relative)
__global__ void convert_tensors(const double* __restrict__ a, long long n, float* __restrict__ a32,
                                dd* __restrict__ add) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const double x = a[i];
    a32[i] = (float)x;
    add[i] = dd(x);
  }
}
}  // namespace tnsp

namespace {

int fail(tnsp_ctx* c, int code, const std::string& msg) {
  if (c) c->err = msg;
  return code;
}

#define CK(call)                                                                                       \
  do {                                                                                                 \
    cudaError_t e_ = (call);                                                                           \
    if (e_ != cudaSuccess) return fail(ctx, e_ == cudaErrorMemoryAllocation ? TNSP_E_NOMEM : TNSP_E_CUDA, \
                                       std::string(#call) + ": " + cudaGetErrorString(e_));            \
  } while (0)

template <class T> void dfree(T*& p) {
  if (p) cudaFree((void*)p);
  p = nullptr;
}

void free_slots(tnsp_ctx* c) {
  dfree(c->d_scratch);
  dfree(c->d_ones);
  dfree(c->d_ldims);
  dfree(c->d_lexp);
  dfree(c->d_order);
  dfree(c->d_delta);
  dfree(c->d_edelta);
  dfree(c->d_contrib);
  dfree(c->d_red);
  dfree(c->d_flops);
  dfree(c->d_lq);
  dfree(c->d_lfl);
  dfree(c->d_tq);
  dfree(c->d_tfl);
  dfree(c->d_ilist);
  c->nslots = 0;
}

void free_chains(tnsp_ctx* c) {
  dfree(c->d_conf);
  dfree(c->d_mt);
  dfree(c->d_mti);
  dfree(c->d_ws_m);
  dfree(c->d_ws_e);
  dfree(c->d_accepted);
  dfree(c->d_acc);
  dfree(c->d_rec);
  c->rec_cap = 0;
  c->rec_n = 0;
  dfree(c->d_holes);
  c->holes_rows = c->holes_cap = 0;
  dfree(c->d_gemv);
  c->gemv_cap = 0;
  c->B = 0;
}

void free_hopping(tnsp_ctx* c) {
  dfree(c->d_s_hterm);
  dfree(c->d_s_vterm);
  dfree(c->d_s_hflip);
  dfree(c->d_s_tab_off);
  dfree(c->d_s_tab_cnt);
  dfree(c->d_s_tab_out);
  dfree(c->d_s_allow);
  c->has_hop = false;
  c->hop_entries = 0;
}

void free_model(tnsp_ctx* c) {
  dfree(c->d_term_sites);
  dfree(c->d_hterm);
  dfree(c->d_vterm);
  dfree(c->d_hflip);
  dfree(c->d_tab_off);
  dfree(c->d_tab_cnt);
  dfree(c->d_tab_out);
  dfree(c->d_tab_val);
  dfree(c->d_e_allow);
  free_hopping(c);
  c->has_model = false;
}

// Checks a term table (nearest-neighbour two-site terms in the reference's dictionary order) and maps
// every bond to its term: hterm / vterm [site] = term on (l1,l2)-(l1,l2+1) / (l1,l2)-(l1+1,l2) or -1;
// hflip[t] = 1 when positions[0] is the second site.  Returns TNSP_OK or a failure code.
int plan_terms(tnsp_ctx* ctx, int n_terms, const int* sites, const int* offsets, const int* counts, int n_entries,
               const int* out_index, std::vector<int>& hterm, std::vector<int>& vterm, std::vector<int>& hflip) {
  const int L1 = ctx->L1, L2 = ctx->L2, P = ctx->P;
  hterm.assign(L1 * L2, -1);
  vterm.assign(L1 * L2, -1);
  hflip.assign(std::max(1, n_terms), 0);
  for (int t = 0; t < n_terms; ++t) {
    const int a1 = sites[t * 4], a2 = sites[t * 4 + 1], b1 = sites[t * 4 + 2], b2 = sites[t * 4 + 3];
    if (a1 < 0 || a1 >= L1 || b1 < 0 || b1 >= L1 || a2 < 0 || a2 >= L2 || b2 < 0 || b2 >= L2)
      return fail(ctx, TNSP_E_ARG, "term site out of range");
    int f1 = a1, f2 = a2, flip = 0;
    if (b1 < a1 || (b1 == a1 && b2 < a2)) {
      f1 = b1;
      f2 = b2;
      flip = 1;
    }
    const int g1 = flip ? a1 : b1, g2 = flip ? a2 : b2;
    int* slot = nullptr;
    if (g1 == f1 && g2 == f2 + 1)
      slot = &hterm[f1 * L2 + f2];
    else if (g2 == f2 && g1 == f1 + 1)
      slot = &vterm[f1 * L2 + f2];
    else
      return fail(ctx, TNSP_E_ARG, "only nearest-neighbour two-site terms are supported");
    if (*slot >= 0) return fail(ctx, TNSP_E_ARG, "several terms on one bond");
    *slot = t;
    hflip[t] = flip;
    for (int i = 0; i < P * P; ++i) {
      const int cnt = counts[t * P * P + i];
      if (cnt > 0 && (offsets[t * P * P + i] < 0 || offsets[t * P * P + i] + cnt > n_entries))
        return fail(ctx, TNSP_E_ARG, "table entry range out of bounds");
    }
  }
  for (int e = 0; e < n_entries; ++e)
    if (out_index[e] < 0 || out_index[e] >= P * P) return fail(ctx, TNSP_E_ARG, "table output index out of range");
  return TNSP_OK;
}

void free_fermion(tnsp_ctx* c) {
  dfree(c->dF64);
  dfree(c->dF32);
  dfree(c->dFdd);
  dfree(c->d_foff);
  c->fermion = false;
}

void free_lattice(tnsp_ctx* c) {
  free_fermion(c);
  dfree(c->dA64);
  dfree(c->dA32);
  dfree(c->dAdd);
  dfree(c->d_dims);
  dfree(c->d_off);
  dfree(c->d_qleg);
  dfree(c->d_qphys);
  dfree(c->d_sflux);
  c->has_lattice = false;
}

Model make_model(tnsp_ctx* c) {
  Model m{};
  m.L1 = c->L1;
  m.L2 = c->L2;
  m.P = c->P;
  m.cut = c->cut;
  m.Dmax = c->Dmax;
  m.dims = c->d_dims;
  m.off = c->d_off;
  // site tensors in the storage type: float64, double-float, or float32 (TNSP_FP32 and TNSP_MIXED)
  m.A = c->precision == TNSP_FP64 ? (const void*)c->dA64
        : c->precision == TNSP_DD  ? (const void*)c->dAdd
                                   : (const void*)c->dA32;
  if (c->fermion) {
    m.fermion = 1;
    m.pT = c->fermion_pT;
    m.poff = c->d_off;
    m.off = c->d_foff;
    m.A = c->precision == TNSP_FP64 ? (const void*)c->dF64
          : c->precision == TNSP_DD  ? (const void*)c->dFdd
                                     : (const void*)c->dF32;
  }
  m.n_terms = c->n_terms;
  m.term_sites = c->d_term_sites;
  m.hterm = c->d_hterm;
  m.vterm = c->d_vterm;
  m.hflip = c->d_hflip;
  m.tab_off = c->d_tab_off;
  m.tab_cnt = c->d_tab_cnt;
  m.tab_out = c->d_tab_out;
  m.tab_val = c->d_tab_val;
  m.n_params = c->n_params;
  m.qleg = c->d_qleg;
  m.qphys = c->d_qphys;
  m.sflux = c->d_sflux;
  m.jacobi_max = c->jacobi_max;
  m.s_hterm = c->has_hop ? c->d_s_hterm : c->d_hterm;
  m.s_vterm = c->has_hop ? c->d_s_vterm : c->d_vterm;
  m.s_hflip = c->has_hop ? c->d_s_hflip : c->d_hflip;
  m.s_tab_off = c->has_hop ? c->d_s_tab_off : c->d_tab_off;
  m.s_tab_cnt = c->has_hop ? c->d_s_tab_cnt : c->d_tab_cnt;
  m.s_tab_out = c->has_hop ? c->d_s_tab_out : c->d_tab_out;
  m.s_allow = c->d_s_allow;
  m.e_allow = c->d_e_allow;
  return m;
}

Chains make_chains(tnsp_ctx* c) {
  Chains ch{};
  ch.B = c->B;
  ch.conf = c->d_conf;
  ch.mt = c->d_mt;
  ch.mti = c->d_mti;
  ch.ws_m = c->d_ws_m;
  ch.ws_e = c->d_ws_e;
  ch.accepted = c->d_accepted;
  ch.acc = c->d_acc;
  ch.status = c->d_status;
  if (c->d_rec) {
    ch.rec_eloc = c->d_rec;
    ch.rec_logws = c->d_rec + (size_t)c->rec_cap * c->B;
    ch.rec_rw = c->d_rec + 2 * (size_t)c->rec_cap * c->B;
  }
  return ch;
}

int ensure_slots(tnsp_ctx* ctx) {
  if (ctx->nslots > 0) return 0;
  int sms = 0;
  CK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, ctx->device));
  Slots s{};
  long long tsize = 8, ssize = 8;
  precision_sizes(ctx->precision, &tsize, &ssize);
  plan_slots(ctx, s, tsize, ssize);
  ctx->elem = (size_t)tsize;
  // dynamic shared memory for sector staging.  Per block: 56 KB + ~15 KB static + 1 KB reserved, so
  // three blocks fit in an SM's 228 KB (64 KB allowed only two); the register budget of the sweep
  // kernel (168 per thread) also allows three 128-thread blocks.  With TNSP_OPT_BLOCKS_PER_SM = b the
  // SM's shared memory is split b ways instead (fewer chains at once, larger sectors staged on chip).
  ctx->smem_bytes = 56 * 1024;
  if (ctx->blocks_per_sm > 0) {
    const long long share = 228LL * 1024 / ctx->blocks_per_sm - 20LL * 1024;  // static + reserved margin
    ctx->smem_bytes = (size_t)std::max(0LL, std::min(200LL * 1024, share / 1024 * 1024));
  }
  int occ = 0;
  if (ctx->precision == TNSP_FP64) {
    CK(set_smem_limit_f64((int)ctx->smem_bytes));
    CK(occupancy_f64((int)ctx->smem_bytes, &occ));
  } else if (ctx->precision == TNSP_DD) {
    CK(set_smem_limit_dd((int)ctx->smem_bytes));
    CK(occupancy_dd((int)ctx->smem_bytes, &occ));
  } else if (ctx->precision == TNSP_MIXED) {
    CK(set_smem_limit_mx((int)ctx->smem_bytes));
    CK(occupancy_mx((int)ctx->smem_bytes, &occ));
  } else {
    CK(set_smem_limit_f32((int)ctx->smem_bytes));
    CK(occupancy_f32((int)ctx->smem_bytes, &occ));
  }
  if (ctx->blocks_per_sm > 0 && occ < ctx->blocks_per_sm)
    return fail(ctx, TNSP_E_ARG, "TNSP_OPT_BLOCKS_PER_SM exceeds the blocks an SM can hold for this kernel");
  if (ctx->blocks_per_sm > 0) occ = ctx->blocks_per_sm;
  // one resident wave of blocks (the occupancy limit per SM), bounded by a scratch budget: 60 % of the
  // device memory free at this point (the large lattices' slots hold hundreds of MB each; the rest stays
  // for the caller and for other contexts)
  long long want = (long long)std::max(1, occ) * sms;
  const long long per = s.stride + 2LL * ctx->n_params * 8;
  size_t free_b = 0, total_b = 0;
  CK(cudaMemGetInfo(&free_b, &total_b));
  const long long budget = (long long)(0.6 * (double)free_b);
  want = std::min(want, std::max(1LL, budget / std::max(1LL, per)));
  want = std::min<long long>(want, std::max(1, ctx->B));
  ctx->nslots = (int)want;
  CK(cudaMalloc(&ctx->d_scratch, (size_t)s.stride * ctx->nslots));
  CK(cudaMalloc(&ctx->d_ones, 16));
  CK(cudaMalloc((void**)&ctx->d_ldims, sizeof(int) * 4 * kMaxL * kMaxL * 3 * ctx->nslots));
  CK(cudaMalloc((void**)&ctx->d_lexp, sizeof(int) * 4 * kMaxL * ctx->nslots));
  CK(cudaMalloc((void**)&ctx->d_order, sizeof(int) * ctx->cut * (ctx->Dmax + 1) * ctx->nslots));
  CK(cudaMalloc((void**)&ctx->d_delta, sizeof(double) * ctx->n_params * ctx->nslots));
  CK(cudaMalloc((void**)&ctx->d_edelta, sizeof(double) * ctx->n_params * ctx->nslots));
  CK(cudaMalloc((void**)&ctx->d_contrib, sizeof(double) * std::max(1, ctx->n_terms) * ctx->nslots));
  CK(cudaMalloc((void**)&ctx->d_red, sizeof(double) * ctx->n_params * 2));
  CK(cudaMalloc((void**)&ctx->d_flops, sizeof(double) * kCounters * ctx->nslots));
  {
    const long long chi = (long long)ctx->cut * ctx->Dmax;
    CK(cudaMalloc((void**)&ctx->d_lq, sizeof(int) * 4 * kMaxL * kMaxL * 2 * ctx->cut * ctx->nslots));
    CK(cudaMalloc((void**)&ctx->d_lfl, sizeof(int) * 4 * kMaxL * kMaxL * ctx->nslots));
    CK(cudaMalloc((void**)&ctx->d_tq, sizeof(int) * kMaxL * 3 * chi * ctx->nslots));
    CK(cudaMalloc((void**)&ctx->d_tfl, sizeof(int) * kMaxL * ctx->nslots));
    CK(cudaMalloc((void**)&ctx->d_ilist, sizeof(int) * (chi * ctx->Dmax + chi) * ctx->nslots));
  }
  CK(cudaMemsetAsync(ctx->d_flops, 0, sizeof(double) * kCounters * ctx->nslots, ctx->stream));
  CK(cudaMemsetAsync(ctx->d_delta, 0, sizeof(double) * ctx->n_params * ctx->nslots, ctx->stream));
  CK(cudaMemsetAsync(ctx->d_edelta, 0, sizeof(double) * ctx->n_params * ctx->nslots, ctx->stream));
  if (ctx->precision == TNSP_FP64)
    fill_ones<double><<<1, 32, 0, ctx->stream>>>((double*)ctx->d_ones);
  else if (ctx->precision == TNSP_DD)
    fill_ones<dd><<<1, 32, 0, ctx->stream>>>((dd*)ctx->d_ones);
  else  // float32 storage (TNSP_FP32, TNSP_MIXED)
    fill_ones<float><<<1, 32, 0, ctx->stream>>>((float*)ctx->d_ones);
  CK(cudaGetLastError());
  s.ldims = ctx->d_ldims;
  s.lexp = ctx->d_lexp;
  s.order = ctx->d_order;
  s.delta = ctx->d_delta;
  s.edelta = ctx->d_edelta;
  s.contrib = ctx->d_contrib;
  s.flops = ctx->d_flops;
  s.lq = ctx->d_lq;
  s.lfl = ctx->d_lfl;
  s.tq = ctx->d_tq;
  s.tfl = ctx->d_tfl;
  s.ilist = ctx->d_ilist;
  s.smem_elems = (long long)(ctx->smem_bytes / ctx->elem);
  ctx->slots = s;
  return 0;
}

void seed_mt(uint64_t seed, uint64_t* mt) {
  mt[0] = seed;
  for (int i = 1; i < kMtN; ++i) mt[i] = 6364136223846793005ull * (mt[i - 1] ^ (mt[i - 1] >> 62)) + (uint64_t)i;
}

uint64_t host_mt_next(uint64_t* mt, int& mti) {
  if (mti >= kMtN) {
    for (int i = 0; i < kMtN; ++i) {
      const uint64_t x = (mt[i] & 0xFFFFFFFF80000000ull) | (mt[(i + 1) % kMtN] & 0x7FFFFFFFull);
      uint64_t xa = x >> 1;
      if (x & 1ull) xa ^= 0xB5026F5AA96619E9ull;
      mt[i] = mt[(i + 156) % kMtN] ^ xa;
    }
    mti = 0;
  }
  return mt[mti++];  // tempering not needed for discarded draws
}

}  // namespace

extern "C" {

int tnsp_ctx_create(tnsp_ctx** out, int device, void* stream) {
  if (!out) return TNSP_E_ARG;
  tnsp_ctx* ctx = new tnsp_ctx();
  ctx->device = device;
  ctx->stream = (cudaStream_t)stream;
  cudaError_t e = cudaSetDevice(device);
  if (e != cudaSuccess) {
    delete ctx;
    *out = nullptr;
    return TNSP_E_CUDA;
  }
  if (cudaEventCreate(&ctx->ev0) != cudaSuccess || cudaEventCreate(&ctx->ev1) != cudaSuccess) {
    delete ctx;
    *out = nullptr;
    return TNSP_E_CUDA;
  }
  if (cudaMalloc((void**)&ctx->d_status, sizeof(int32_t)) != cudaSuccess ||
      cudaMemset(ctx->d_status, 0, sizeof(int32_t)) != cudaSuccess) {
    delete ctx;
    *out = nullptr;
    return TNSP_E_CUDA;
  }
  *out = ctx;
  return TNSP_OK;
}

int tnsp_ctx_destroy(tnsp_ctx* ctx) {
  if (!ctx) return TNSP_E_ARG;
  cudaSetDevice(ctx->device);
  cudaStreamSynchronize(ctx->stream);
  free_slots(ctx);
  free_chains(ctx);
  free_model(ctx);
  free_lattice(ctx);
  dfree(ctx->d_status);
  if (ctx->ev0) cudaEventDestroy(ctx->ev0);
  if (ctx->ev1) cudaEventDestroy(ctx->ev1);
  delete ctx;
  return TNSP_OK;
}

const char* tnsp_last_error(tnsp_ctx* ctx) { return ctx ? ctx->err.c_str() : tnsp_noalloc_error(); }

int tnsp_resident_chains(tnsp_ctx* ctx, int* n) {
  if (!ctx || !n) return TNSP_E_ARG;
  if (!ctx->B) return fail(ctx, TNSP_E_STATE, "no chains");
  CK(cudaSetDevice(ctx->device));
  const int r = ensure_slots(ctx);
  if (r) return r;
  *n = ctx->nslots;
  return TNSP_OK;
}

int tnsp_set_option(tnsp_ctx* ctx, int option, int value) {
  if (!ctx) return TNSP_E_ARG;
  switch (option) {
    case TNSP_OPT_JACOBI_SWEEPS:
      if (value < 1 || value > 1000) return fail(ctx, TNSP_E_ARG, "Jacobi sweep limit out of range (1..1000)");
      ctx->jacobi_max = value;
      return TNSP_OK;
    case TNSP_OPT_BLOCKS_PER_SM:
      if (value < 0 || value > 32) return fail(ctx, TNSP_E_ARG, "blocks per SM out of range (0..32)");
      if (value != ctx->blocks_per_sm) {
        CK(cudaSetDevice(ctx->device));
        CK(cudaDeviceSynchronize());
        free_slots(ctx);  // re-planned at the next use
        ctx->blocks_per_sm = value;
      }
      return TNSP_OK;
    default:
      return fail(ctx, TNSP_E_ARG, "unknown option");
  }
}

int tnsp_lattice_upload(tnsp_ctx* ctx, int L1, int L2, int P, const int* dims, const double* tensors, int cut) {
  if (!ctx) return TNSP_E_ARG;
  if (L1 < 1 || L2 < 1 || L1 > kMaxL || L2 > kMaxL) return fail(ctx, TNSP_E_ARG, "lattice extent out of range (1..16)");
  if (P < 1 || P > 64) return fail(ctx, TNSP_E_ARG, "physical dimension out of range");
  if (cut < 1) return fail(ctx, TNSP_E_ARG, "cut dimension must be positive");
  if (!dims || !tensors) return fail(ctx, TNSP_E_ARG, "null dims or tensors");
  CK(cudaSetDevice(ctx->device));
  std::vector<int> dv(dims, dims + (size_t)L1 * L2 * 4);
  int Dmax = 1;
  std::vector<long long> off(L1 * L2);
  long long total = 0;
  for (int l1 = 0; l1 < L1; ++l1)
    for (int l2 = 0; l2 < L2; ++l2) {
      const int id = l1 * L2 + l2;
      const int* d = &dv[id * 4];
      for (int k = 0; k < 4; ++k) {
        if (d[k] < 1) return fail(ctx, TNSP_E_ARG, "bond extents must be >= 1");
        Dmax = std::max(Dmax, d[k]);
      }
      if ((l1 == 0 && d[0] != 1) || (l1 == L1 - 1 && d[1] != 1) || (l2 == 0 && d[2] != 1) ||
          (l2 == L2 - 1 && d[3] != 1))
        return fail(ctx, TNSP_E_ARG, "bonds leaving the open lattice must have extent 1");
      if (l2 + 1 < L2 && d[3] != dv[(id + 1) * 4 + 2]) return fail(ctx, TNSP_E_ARG, "R/L bond extents differ");
      if (l1 + 1 < L1 && d[1] != dv[(id + L2) * 4 + 0]) return fail(ctx, TNSP_E_ARG, "D/U bond extents differ");
      off[id] = total;
      total += (long long)P * d[0] * d[1] * d[2] * d[3];
    }
  for (long long i = 0; i < total; ++i)
    if (!std::isfinite(tensors[i])) return fail(ctx, TNSP_E_ARG, "non-finite element in the site tensors");
  if ((long long)cut * Dmax > kMaxChi) return fail(ctx, TNSP_E_ARG, "cut * max bond extent exceeds 1024");
  const bool reshape = ctx->has_lattice && (L1 != ctx->L1 || L2 != ctx->L2 || P != ctx->P || cut != ctx->cut ||
                                            Dmax != ctx->Dmax || dv != ctx->dims);
  if (reshape) {
    free_slots(ctx);
    free_chains(ctx);
    free_model(ctx);
  }
  free_fermion(ctx);  // a new upload describes a bosonic lattice until tnsp_lattice_fermion is called again
  if (!ctx->has_lattice || reshape) {
    free_lattice(ctx);
    CK(cudaMalloc((void**)&ctx->dA64, sizeof(double) * total));
    CK(cudaMalloc((void**)&ctx->dA32, sizeof(float) * total));
    CK(cudaMalloc((void**)&ctx->dAdd, sizeof(dd) * total));
    CK(cudaMalloc((void**)&ctx->d_dims, sizeof(int) * dv.size()));
    CK(cudaMalloc((void**)&ctx->d_off, sizeof(long long) * off.size()));
    CK(cudaMalloc((void**)&ctx->d_qleg, sizeof(int) * (size_t)L1 * L2 * 4 * Dmax));
    CK(cudaMalloc((void**)&ctx->d_qphys, sizeof(int) * P));
    CK(cudaMalloc((void**)&ctx->d_sflux, sizeof(int) * (size_t)L1 * L2));
    CK(cudaMemset(ctx->d_qleg, 0, sizeof(int) * (size_t)L1 * L2 * 4 * Dmax));
    CK(cudaMemset(ctx->d_qphys, 0, sizeof(int) * P));
    CK(cudaMemset(ctx->d_sflux, 0, sizeof(int) * (size_t)L1 * L2));
    ctx->charged = false;
  }
  ctx->hostA.assign(tensors, tensors + total);
  CK(cudaMemcpyAsync(ctx->dA64, tensors, sizeof(double) * total, cudaMemcpyHostToDevice, ctx->stream));
  convert_tensors<<<(int)std::min<long long>(1024, (total + 255) / 256), 256, 0, ctx->stream>>>(ctx->dA64, total,
                                                                                               ctx->dA32, ctx->dAdd);
  CK(cudaGetLastError());
  CK(cudaMemcpyAsync(ctx->d_dims, dv.data(), sizeof(int) * dv.size(), cudaMemcpyHostToDevice, ctx->stream));
  CK(cudaMemcpyAsync(ctx->d_off, off.data(), sizeof(long long) * off.size(), cudaMemcpyHostToDevice, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  ctx->L1 = L1;
  ctx->L2 = L2;
  ctx->P = P;
  ctx->cut = cut;
  ctx->Dmax = Dmax;
  ctx->dims = dv;
  ctx->off = off;
  ctx->n_params = total;
  ctx->has_lattice = true;
  return TNSP_OK;
}

int tnsp_lattice_charges(tnsp_ctx* ctx, const int* leg_charges, const int* phys_charges, const int* site_flux) {
  if (!ctx) return TNSP_E_ARG;
  if (!ctx->has_lattice) return fail(ctx, TNSP_E_STATE, "upload the lattice first");
  if (!leg_charges || !phys_charges || !site_flux) return fail(ctx, TNSP_E_ARG, "null charge array");
  CK(cudaSetDevice(ctx->device));
  const int L1 = ctx->L1, L2 = ctx->L2, P = ctx->P, Dm = ctx->Dmax;
  // every nonzero element must conserve charge, otherwise the sector factorisation would drop it
  for (int id = 0; id < L1 * L2; ++id) {
    const int* d = &ctx->dims[id * 4];
    const int* q = leg_charges + (size_t)id * 4 * Dm;
    const double* a = ctx->hostA.data() + ctx->off[id];
    long long e = 0;
    for (int p = 0; p < P; ++p)
      for (int u = 0; u < d[0]; ++u)
        for (int dd = 0; dd < d[1]; ++dd)
          for (int l = 0; l < d[2]; ++l)
            for (int r = 0; r < d[3]; ++r, ++e)
              if (a[e] != 0.0 &&
                  phys_charges[p] + q[u] + q[Dm + dd] + q[2 * Dm + l] + q[3 * Dm + r] != site_flux[id]) {
                char buf[160];
                snprintf(buf, sizeof buf, "site %d: element (%d,%d,%d,%d,%d) violates charge conservation", id, p, u,
                         dd, l, r);
                return fail(ctx, TNSP_E_ARG, buf);
              }
  }
  // bonds must carry opposite charges on their two ends
  for (int l1 = 0; l1 < L1; ++l1)
    for (int l2 = 0; l2 < L2; ++l2) {
      const int id = l1 * L2 + l2;
      const int* q = leg_charges + (size_t)id * 4 * Dm;
      if (l2 + 1 < L2) {
        const int* qn = leg_charges + (size_t)(id + 1) * 4 * Dm;
        for (int x = 0; x < ctx->dims[id * 4 + 3]; ++x)
          if (q[3 * Dm + x] != -qn[2 * Dm + x]) return fail(ctx, TNSP_E_ARG, "R/L bond charges are not opposite");
      }
      if (l1 + 1 < L1) {
        const int* qn = leg_charges + (size_t)(id + L2) * 4 * Dm;
        for (int x = 0; x < ctx->dims[id * 4 + 1]; ++x)
          if (q[Dm + x] != -qn[x]) return fail(ctx, TNSP_E_ARG, "D/U bond charges are not opposite");
      }
    }
  CK(cudaMemcpy(ctx->d_qleg, leg_charges, sizeof(int) * (size_t)L1 * L2 * 4 * Dm, cudaMemcpyHostToDevice));
  CK(cudaMemcpy(ctx->d_qphys, phys_charges, sizeof(int) * P, cudaMemcpyHostToDevice));
  CK(cudaMemcpy(ctx->d_sflux, site_flux, sizeof(int) * (size_t)L1 * L2, cudaMemcpyHostToDevice));
  ctx->charged = true;
  return TNSP_OK;
}

int tnsp_lattice_fermion(tnsp_ctx* ctx, const double* slices, int total_charge) {
  if (!ctx) return TNSP_E_ARG;
  if (!ctx->has_lattice) return fail(ctx, TNSP_E_STATE, "upload the lattice first");
  if (!ctx->charged) return fail(ctx, TNSP_E_STATE, "declare the charges first");
  if (ctx->P != 2) return fail(ctx, TNSP_E_ARG, "a fermionic site has two physical slices (empty, occupied)");
  if (!slices) return fail(ctx, TNSP_E_ARG, "null slices");
  CK(cudaSetDevice(ctx->device));
  const int nsite = ctx->L1 * ctx->L2;
  std::vector<long long> foff(nsite);
  long long total = 0;
  for (int id = 0; id < nsite; ++id) {
    const int* d = &ctx->dims[id * 4];
    foff[id] = total;
    total += 8LL * d[0] * d[1] * d[2] * d[3];
  }
  for (long long i = 0; i < total; ++i)
    if (!std::isfinite(slices[i])) return fail(ctx, TNSP_E_ARG, "non-finite element in the slices");
  free_fermion(ctx);
  CK(cudaMalloc((void**)&ctx->dF64, sizeof(double) * total));
  CK(cudaMalloc((void**)&ctx->dF32, sizeof(float) * total));
  CK(cudaMalloc((void**)&ctx->dFdd, sizeof(dd) * total));
  CK(cudaMalloc((void**)&ctx->d_foff, sizeof(long long) * nsite));
  CK(cudaMemcpyAsync(ctx->dF64, slices, sizeof(double) * total, cudaMemcpyHostToDevice, ctx->stream));
  convert_tensors<<<(int)std::min<long long>(1024, (total + 255) / 256), 256, 0, ctx->stream>>>(ctx->dF64, total,
                                                                                               ctx->dF32, ctx->dFdd);
  CK(cudaGetLastError());
  CK(cudaMemcpyAsync(ctx->d_foff, foff.data(), sizeof(long long) * nsite, cudaMemcpyHostToDevice, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  ctx->fermion = true;
  ctx->fermion_pT = total_charge & 1;
  return TNSP_OK;
}

int tnsp_model_upload(tnsp_ctx* ctx, int n_terms, const int* sites, const int* offsets, const int* counts,
                      int n_entries, const int* out_index, const double* values) {
  if (!ctx) return TNSP_E_ARG;
  if (!ctx->has_lattice) return fail(ctx, TNSP_E_STATE, "upload the lattice first");
  if (n_terms < 0 || n_entries < 0) return fail(ctx, TNSP_E_ARG, "negative sizes");
  if (n_entries > 0 && (!out_index || !values)) return fail(ctx, TNSP_E_ARG, "null table arrays");
  if (n_terms > 0 && (!sites || !offsets || !counts)) return fail(ctx, TNSP_E_ARG, "null table arrays");
  CK(cudaSetDevice(ctx->device));
  const int L1 = ctx->L1, L2 = ctx->L2, P = ctx->P;
  std::vector<int> hterm, vterm, hflip;
  const int r = plan_terms(ctx, n_terms, sites, offsets, counts, n_entries, out_index, hterm, vterm, hflip);
  if (r) return r;
  const bool terms_changed = !ctx->has_model || n_terms != ctx->n_terms;
  free_model(ctx);
  const size_t tp = (size_t)std::max(1, n_terms) * P * P;
  CK(cudaMalloc((void**)&ctx->d_term_sites, sizeof(int) * std::max(1, n_terms) * 4));
  CK(cudaMalloc((void**)&ctx->d_hterm, sizeof(int) * L1 * L2));
  CK(cudaMalloc((void**)&ctx->d_vterm, sizeof(int) * L1 * L2));
  CK(cudaMalloc((void**)&ctx->d_hflip, sizeof(int) * hflip.size()));
  CK(cudaMalloc((void**)&ctx->d_tab_off, sizeof(int) * tp));
  CK(cudaMalloc((void**)&ctx->d_tab_cnt, sizeof(int) * tp));
  CK(cudaMalloc((void**)&ctx->d_tab_out, sizeof(int) * std::max(1, n_entries)));
  CK(cudaMalloc((void**)&ctx->d_tab_val, sizeof(double) * std::max(1, n_entries)));
  if (n_terms > 0) {
    CK(cudaMemcpy(ctx->d_term_sites, sites, sizeof(int) * n_terms * 4, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(ctx->d_tab_off, offsets, sizeof(int) * n_terms * P * P, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(ctx->d_tab_cnt, counts, sizeof(int) * n_terms * P * P, cudaMemcpyHostToDevice));
  }
  if (n_entries > 0) {
    CK(cudaMemcpy(ctx->d_tab_out, out_index, sizeof(int) * n_entries, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(ctx->d_tab_val, values, sizeof(double) * n_entries, cudaMemcpyHostToDevice));
  }
  CK(cudaMemcpy(ctx->d_hterm, hterm.data(), sizeof(int) * L1 * L2, cudaMemcpyHostToDevice));
  CK(cudaMemcpy(ctx->d_vterm, vterm.data(), sizeof(int) * L1 * L2, cudaMemcpyHostToDevice));
  CK(cudaMemcpy(ctx->d_hflip, hflip.data(), sizeof(int) * hflip.size(), cudaMemcpyHostToDevice));
  ctx->n_terms = n_terms;
  ctx->n_entries = n_entries;
  ctx->has_model = true;
  if (terms_changed) free_slots(ctx);  // the contribution buffer depends on n_terms
  return TNSP_OK;
}

int tnsp_model_hopping(tnsp_ctx* ctx, int n_terms, const int* sites, const int* offsets, const int* counts,
                       int n_entries, const int* out_index, const unsigned char* allowed) {
  if (!ctx) return TNSP_E_ARG;
  if (!ctx->has_model) return fail(ctx, TNSP_E_STATE, "upload the model first");
  if (n_terms < 0 || n_entries < 0) return fail(ctx, TNSP_E_ARG, "negative sizes");
  CK(cudaSetDevice(ctx->device));
  free_hopping(ctx);
  const int L1 = ctx->L1, L2 = ctx->L2, P = ctx->P;
  if (n_terms == 0) {
    // the energy tables propose; only the allow flags are new
    if (!allowed) return TNSP_OK;
    CK(cudaMalloc((void**)&ctx->d_s_allow, std::max(1, ctx->n_entries)));
    if (ctx->n_entries > 0) CK(cudaMemcpy(ctx->d_s_allow, allowed, ctx->n_entries, cudaMemcpyHostToDevice));
    ctx->hop_entries = ctx->n_entries;
    return TNSP_OK;
  }
  if (!sites || !offsets || !counts || (n_entries > 0 && !out_index)) return fail(ctx, TNSP_E_ARG, "null table arrays");
  std::vector<int> hterm, vterm, hflip;
  const int r = plan_terms(ctx, n_terms, sites, offsets, counts, n_entries, out_index, hterm, vterm, hflip);
  if (r) return r;
  const size_t tp = (size_t)n_terms * P * P;
  CK(cudaMalloc((void**)&ctx->d_s_hterm, sizeof(int) * L1 * L2));
  CK(cudaMalloc((void**)&ctx->d_s_vterm, sizeof(int) * L1 * L2));
  CK(cudaMalloc((void**)&ctx->d_s_hflip, sizeof(int) * hflip.size()));
  CK(cudaMalloc((void**)&ctx->d_s_tab_off, sizeof(int) * tp));
  CK(cudaMalloc((void**)&ctx->d_s_tab_cnt, sizeof(int) * tp));
  CK(cudaMalloc((void**)&ctx->d_s_tab_out, sizeof(int) * std::max(1, n_entries)));
  CK(cudaMemcpy(ctx->d_s_hterm, hterm.data(), sizeof(int) * L1 * L2, cudaMemcpyHostToDevice));
  CK(cudaMemcpy(ctx->d_s_vterm, vterm.data(), sizeof(int) * L1 * L2, cudaMemcpyHostToDevice));
  CK(cudaMemcpy(ctx->d_s_hflip, hflip.data(), sizeof(int) * hflip.size(), cudaMemcpyHostToDevice));
  CK(cudaMemcpy(ctx->d_s_tab_off, offsets, sizeof(int) * tp, cudaMemcpyHostToDevice));
  CK(cudaMemcpy(ctx->d_s_tab_cnt, counts, sizeof(int) * tp, cudaMemcpyHostToDevice));
  if (n_entries > 0) CK(cudaMemcpy(ctx->d_s_tab_out, out_index, sizeof(int) * n_entries, cudaMemcpyHostToDevice));
  if (allowed) {
    CK(cudaMalloc((void**)&ctx->d_s_allow, std::max(1, n_entries)));
    if (n_entries > 0) CK(cudaMemcpy(ctx->d_s_allow, allowed, n_entries, cudaMemcpyHostToDevice));
  }
  ctx->has_hop = true;
  ctx->hop_entries = n_entries;
  return TNSP_OK;
}

int tnsp_model_energy_restrict(tnsp_ctx* ctx, const unsigned char* allowed) {
  if (!ctx) return TNSP_E_ARG;
  if (!ctx->has_model) return fail(ctx, TNSP_E_STATE, "upload the model first");
  CK(cudaSetDevice(ctx->device));
  dfree(ctx->d_e_allow);
  if (!allowed) return TNSP_OK;
  CK(cudaMalloc((void**)&ctx->d_e_allow, std::max(1, ctx->n_entries)));
  if (ctx->n_entries > 0) CK(cudaMemcpy(ctx->d_e_allow, allowed, ctx->n_entries, cudaMemcpyHostToDevice));
  return TNSP_OK;
}

int tnsp_chains_init(tnsp_ctx* ctx, int B, const int32_t* configs, const uint64_t* seeds, int discard,
                     int precision) {
  if (!ctx) return TNSP_E_ARG;
  if (!ctx->has_lattice || !ctx->has_model) return fail(ctx, TNSP_E_STATE, "upload the lattice and the model first");
  if (B < 1) return fail(ctx, TNSP_E_ARG, "need at least one chain");
  if (precision != TNSP_FP64 && precision != TNSP_FP32 && precision != TNSP_DD && precision != TNSP_MIXED)
    return fail(ctx, TNSP_E_ARG, "unknown precision");
  if (!configs || !seeds) return fail(ctx, TNSP_E_ARG, "null configs or seeds");
  const int ns = ctx->L1 * ctx->L2;
  for (long long i = 0; i < (long long)B * ns; ++i)
    if (configs[i] < 0 || configs[i] >= ctx->P) return fail(ctx, TNSP_E_ARG, "configuration index out of range");
  if ((precision == TNSP_DD || precision == TNSP_MIXED) && !ctx->charged) {
    // block-sparse tensors passed densely without their charges: the structural zeros make
    // rank-deficient boundaries that double-float resolves only to ~1e-3 (float64 is exact there)
    for (int id = 0; id < ns; ++id) {
      const long long n = (id + 1 < ns ? ctx->off[id + 1] : ctx->n_params) - ctx->off[id];
      long long zeros = 0;
      for (long long i = 0; i < n; ++i) zeros += ctx->hostA[ctx->off[id] + i] == 0.0;
      if (4 * zeros > n)
        return fail(ctx, TNSP_E_ARG,
                    "double-float needs the charges of block-sparse tensors: site " + std::to_string(id) +
                        " is more than a quarter exact zeros and no charges were declared (call "
                        "tnsp_lattice_charges, or use TNSP_FP64)");
    }
  }
  CK(cudaSetDevice(ctx->device));
  if (B != ctx->B || precision != ctx->precision) {
    free_chains(ctx);
    free_slots(ctx);
    ctx->precision = precision;
    CK(cudaMalloc((void**)&ctx->d_conf, sizeof(int32_t) * B * ns));
    CK(cudaMalloc((void**)&ctx->d_mt, sizeof(uint64_t) * B * kMtN));
    CK(cudaMalloc((void**)&ctx->d_mti, sizeof(int32_t) * B));
    CK(cudaMalloc((void**)&ctx->d_ws_m, sizeof(double) * B));
    CK(cudaMalloc((void**)&ctx->d_ws_e, sizeof(int32_t) * B));
    CK(cudaMalloc((void**)&ctx->d_accepted, sizeof(int64_t) * B));
    CK(cudaMalloc((void**)&ctx->d_acc, sizeof(double) * B * 8));
    ctx->B = B;
  }
  std::vector<uint64_t> mt((size_t)B * kMtN);
  std::vector<int32_t> mti(B);
  for (int b = 0; b < B; ++b) {
    seed_mt(seeds[b], &mt[(size_t)b * kMtN]);
    int k = kMtN;
    for (int d = 0; d < discard; ++d) host_mt_next(&mt[(size_t)b * kMtN], k);
    mti[b] = k;
  }
  CK(cudaMemcpy(ctx->d_conf, configs, sizeof(int32_t) * B * ns, cudaMemcpyHostToDevice));
  CK(cudaMemcpy(ctx->d_mt, mt.data(), sizeof(uint64_t) * mt.size(), cudaMemcpyHostToDevice));
  CK(cudaMemcpy(ctx->d_mti, mti.data(), sizeof(int32_t) * B, cudaMemcpyHostToDevice));
  CK(cudaMemset(ctx->d_accepted, 0, sizeof(int64_t) * B));
  CK(cudaMemset(ctx->d_acc, 0, sizeof(double) * B * 8));
  CK(cudaMemset(ctx->d_ws_m, 0, sizeof(double) * B));
  CK(cudaMemset(ctx->d_ws_e, 0, sizeof(int32_t) * B));
  return ensure_slots(ctx);
}

int tnsp_chains_write(tnsp_ctx* ctx, const int32_t* configs) {
  if (!ctx || !configs) return TNSP_E_ARG;
  if (!ctx->B) return fail(ctx, TNSP_E_STATE, "no chains");
  const long long n = (long long)ctx->B * ctx->L1 * ctx->L2;
  for (long long i = 0; i < n; ++i)
    if (configs[i] < 0 || configs[i] >= ctx->P) return fail(ctx, TNSP_E_ARG, "configuration index out of range");
  CK(cudaSetDevice(ctx->device));
  CK(cudaMemcpy(ctx->d_conf, configs, sizeof(int32_t) * n, cudaMemcpyHostToDevice));
  return TNSP_OK;
}

int tnsp_observer_reset(tnsp_ctx* ctx) {
  if (!ctx) return TNSP_E_ARG;
  if (!ctx->B) return fail(ctx, TNSP_E_STATE, "no chains");
  CK(cudaSetDevice(ctx->device));
  int r = ensure_slots(ctx);
  if (r) return r;
  CK(cudaMemsetAsync(ctx->d_acc, 0, sizeof(double) * ctx->B * 8, ctx->stream));
  CK(cudaMemsetAsync(ctx->d_delta, 0, sizeof(double) * ctx->n_params * ctx->nslots, ctx->stream));
  CK(cudaMemsetAsync(ctx->d_edelta, 0, sizeof(double) * ctx->n_params * ctx->nslots, ctx->stream));
  ctx->rec_n = 0;
  ctx->holes_rows = 0;
  return TNSP_OK;
}

namespace {

// one sweep call, split so that tnsp_sweep_batch can enqueue several contexts into one graph
struct SweepPlan {
  Model md;
  Chains ch;
  int nrec = 0;
  long long new_rows = 0;
};

// host-side preparation: buffers, per-sample records, kept hole rows (may allocate, enqueues memsets
// on the context stream)
int sweep_prepare(tnsp_ctx* ctx, int nsweeps, int observe, SweepPlan& p) {
  if (!ctx) return TNSP_E_ARG;
  if (!ctx->B) return fail(ctx, TNSP_E_STATE, "no chains");
  if (nsweeps < 0) return fail(ctx, TNSP_E_ARG, "negative sweep count");
  CK(cudaSetDevice(ctx->device));
  int r = ensure_slots(ctx);
  if (r) return r;
  p.nrec = (nsweeps == 0 && observe) ? 1 : nsweeps;
  if (observe) {
    // the per-sample record holds the samples of this call
    if (ctx->rec_cap < p.nrec) {
      dfree(ctx->d_rec);
      CK(cudaMalloc((void**)&ctx->d_rec, sizeof(double) * 3 * (size_t)std::max(1, p.nrec) * ctx->B));
      ctx->rec_cap = std::max(1, p.nrec);
    }
    ctx->rec_n = p.nrec;
  }
  p.md = make_model(ctx);
  p.ch = make_chains(ctx);
  if (!observe) {
    p.ch.rec_eloc = p.ch.rec_logws = p.ch.rec_rw = nullptr;
  }
  p.new_rows = (observe && ctx->keep_holes) ? (long long)p.nrec * ctx->B : 0;
  if (p.new_rows > 0) {
    // append after the rows kept since the last observer reset (grow by doubling, keep the old rows)
    const long long need = ctx->holes_rows + p.new_rows;
    if (need > ctx->holes_cap) {
      const long long cap = std::max(need, 2 * ctx->holes_cap);
      double* grown = nullptr;
      CK(cudaMalloc((void**)&grown, sizeof(double) * (size_t)cap * ctx->n_params));
      if (ctx->holes_rows > 0)
        CK(cudaMemcpyAsync(grown, ctx->d_holes, sizeof(double) * (size_t)ctx->holes_rows * ctx->n_params,
                           cudaMemcpyDeviceToDevice, ctx->stream));
      CK(cudaStreamSynchronize(ctx->stream));
      dfree(ctx->d_holes);
      ctx->d_holes = grown;
      ctx->holes_cap = cap;
    }
    CK(cudaMemsetAsync(ctx->d_holes + (size_t)ctx->holes_rows * ctx->n_params, 0,
                       sizeof(double) * (size_t)p.new_rows * ctx->n_params, ctx->stream));
    p.ch.rec_hole = ctx->d_holes;
    p.ch.hole_row0 = ctx->holes_rows;
  }
  return TNSP_OK;
}

// the sweep launch itself on stream st (no synchronisation: capturable)
int sweep_enqueue(tnsp_ctx* ctx, const SweepPlan& p, int nsweeps, int observe, cudaStream_t st) {
  if (p.nrec == 0) return TNSP_OK;
  const int grid = ctx->nslots;
  if (ctx->precision == TNSP_FP64)
    launch_sweep_f64(grid, ctx->smem_bytes, st, p.md, p.ch, ctx->slots, ctx->d_scratch, ctx->d_ones, nsweeps, observe,
                     0);
  else if (ctx->precision == TNSP_DD)
    launch_sweep_dd(grid, ctx->smem_bytes, st, p.md, p.ch, ctx->slots, ctx->d_scratch, ctx->d_ones, nsweeps, observe,
                    0);
  else if (ctx->precision == TNSP_MIXED)
    launch_sweep_mx(grid, ctx->smem_bytes, st, p.md, p.ch, ctx->slots, ctx->d_scratch, ctx->d_ones, nsweeps, observe,
                    0);
  else
    launch_sweep_f32(grid, ctx->smem_bytes, st, p.md, p.ch, ctx->slots, ctx->d_scratch, ctx->d_ones, nsweeps, observe,
                     0);
  CK(cudaGetLastError());
  return TNSP_OK;
}

// after the launch completed: the device status word
int sweep_finish(tnsp_ctx* ctx, const SweepPlan& p) {
  int32_t st = 0;
  CK(cudaMemcpy(&st, ctx->d_status, sizeof(int32_t), cudaMemcpyDeviceToHost));
  if (st & (TNSP_ST_SVD_NOCONV | TNSP_ST_NONFINITE | TNSP_ST_UNSUPPORTED)) {
    char buf[128];
    snprintf(buf, sizeof buf, "device status 0x%x (see TNSP_ST_* bits)", st);
    return fail(ctx, TNSP_E_DEVICE, buf);
  }
  ctx->holes_rows += p.new_rows;
  return TNSP_OK;
}

}  // namespace

int tnsp_sweep(tnsp_ctx* ctx, int nsweeps, int observe) {
  SweepPlan p;
  int r = sweep_prepare(ctx, nsweeps, observe, p);
  if (r) return r;
  CK(cudaEventRecord(ctx->ev0, ctx->stream));
  r = sweep_enqueue(ctx, p, nsweeps, observe, ctx->stream);
  if (r) return r;
  CK(cudaEventRecord(ctx->ev1, ctx->stream));
  CK(cudaEventSynchronize(ctx->ev1));
  float ms = 0;
  CK(cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1));
  ctx->last_ms = ms;
  ctx->last_launches = p.nrec > 0 ? 1 : 0;
  return sweep_finish(ctx, p);
}

int tnsp_sweep_batch(tnsp_ctx* const* ctxs, int n, int nsweeps, int observe) {
  if (!ctxs || n < 1) return TNSP_E_ARG;
  tnsp_ctx* ctx = ctxs[0];  // error messages of the batch go to the first context
  for (int i = 0; i < n; ++i)
    if (!ctxs[i] || ctxs[i]->device != ctx->device) return fail(ctx, TNSP_E_ARG, "contexts must share one device");
  std::vector<SweepPlan> plans(n);
  for (int i = 0; i < n; ++i) {
    int r = sweep_prepare(ctxs[i], nsweeps, observe, plans[i]);
    if (r) return r;
    CK(cudaStreamSynchronize(ctxs[i]->stream));  // its memsets precede the graph
  }
  CK(cudaSetDevice(ctx->device));
  // capture: fork from a capture stream to one stream per context, one sweep launch each, join
  struct Res {
    cudaStream_t cs = nullptr;
    std::vector<cudaStream_t> side;
    cudaEvent_t fork = nullptr, t0 = nullptr, t1 = nullptr;
    std::vector<cudaEvent_t> join;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    ~Res() {
      if (exec) cudaGraphExecDestroy(exec);
      if (graph) cudaGraphDestroy(graph);
      for (auto e : join) if (e) cudaEventDestroy(e);
      for (auto e : {fork, t0, t1}) if (e) cudaEventDestroy(e);
      for (auto s : side) if (s) cudaStreamDestroy(s);
      if (cs) cudaStreamDestroy(cs);
    }
  } res;
  res.side.assign(n, nullptr);
  res.join.assign(n, nullptr);
  CK(cudaStreamCreateWithFlags(&res.cs, cudaStreamNonBlocking));
  CK(cudaEventCreateWithFlags(&res.fork, cudaEventDisableTiming));
  CK(cudaEventCreate(&res.t0));
  CK(cudaEventCreate(&res.t1));
  for (int i = 0; i < n; ++i) {
    CK(cudaStreamCreateWithFlags(&res.side[i], cudaStreamNonBlocking));
    CK(cudaEventCreateWithFlags(&res.join[i], cudaEventDisableTiming));
  }
  CK(cudaStreamBeginCapture(res.cs, cudaStreamCaptureModeThreadLocal));
  int launched = 0, r = TNSP_OK;
  if (cudaEventRecord(res.fork, res.cs) != cudaSuccess) r = fail(ctx, TNSP_E_CUDA, "fork event");
  for (int i = 0; i < n && r == TNSP_OK; ++i) {
    if (cudaStreamWaitEvent(res.side[i], res.fork, 0) != cudaSuccess) {
      r = fail(ctx, TNSP_E_CUDA, "fork wait");
      break;
    }
    r = sweep_enqueue(ctxs[i], plans[i], nsweeps, observe, res.side[i]);
    launched += plans[i].nrec > 0 ? 1 : 0;
    if (r == TNSP_OK && (cudaEventRecord(res.join[i], res.side[i]) != cudaSuccess ||
                         cudaStreamWaitEvent(res.cs, res.join[i], 0) != cudaSuccess))
      r = fail(ctx, TNSP_E_CUDA, "join");
  }
  const cudaError_t ec = cudaStreamEndCapture(res.cs, &res.graph);
  if (r) return r;
  if (ec != cudaSuccess) return fail(ctx, TNSP_E_CUDA, std::string("stream capture: ") + cudaGetErrorString(ec));
  CK(cudaGraphInstantiate(&res.exec, res.graph, 0));
  CK(cudaEventRecord(res.t0, res.cs));
  CK(cudaGraphLaunch(res.exec, res.cs));
  CK(cudaEventRecord(res.t1, res.cs));
  CK(cudaEventSynchronize(res.t1));
  float ms = 0;
  CK(cudaEventElapsedTime(&ms, res.t0, res.t1));
  int first = TNSP_OK;
  for (int i = 0; i < n; ++i) {
    ctxs[i]->last_ms = ms;
    ctxs[i]->last_launches = launched;
    const int ri = sweep_finish(ctxs[i], plans[i]);
    if (ri && first == TNSP_OK) {
      first = ri;
      if (i) ctx->err = ctxs[i]->err;
    }
  }
  return first;
}

int tnsp_holes_keep(tnsp_ctx* ctx, int enable) {
  if (!ctx) return TNSP_E_ARG;
  CK(cudaSetDevice(ctx->device));
  ctx->keep_holes = enable != 0;
  if (!ctx->keep_holes) {
    dfree(ctx->d_holes);
    ctx->holes_rows = ctx->holes_cap = 0;
  }
  return TNSP_OK;
}

int tnsp_holes_count(tnsp_ctx* ctx, int64_t* rows) {
  if (!ctx || !rows) return TNSP_E_ARG;
  *rows = ctx->holes_rows;
  return TNSP_OK;
}

int tnsp_holes_gemv(tnsp_ctx* ctx, int transpose, const double* x, double* y) {
  if (!ctx || !x || !y) return TNSP_E_ARG;
  if (!ctx->holes_rows) return fail(ctx, TNSP_E_STATE, "no hole rows kept (tnsp_holes_keep before an observed sweep)");
  CK(cudaSetDevice(ctx->device));
  const long long rows = ctx->holes_rows, np = ctx->n_params;
  const long long nx = transpose ? rows : np, ny = transpose ? np : rows;
  if (ctx->gemv_cap < nx + ny) {
    dfree(ctx->d_gemv);
    CK(cudaMalloc((void**)&ctx->d_gemv, sizeof(double) * (size_t)(nx + ny)));
    ctx->gemv_cap = nx + ny;
  }
  double* dx = ctx->d_gemv;
  double* dy = ctx->d_gemv + nx;
  CK(cudaMemcpyAsync(dx, x, sizeof(double) * (size_t)nx, cudaMemcpyHostToDevice, ctx->stream));
  if (transpose) {
    const int grid = (int)std::min<long long>((np + 255) / 256, 65535);
    holes_gemv_cols<<<grid, 256, 0, ctx->stream>>>(ctx->d_holes, np, rows, dx, dy);
  } else {
    const int grid = (int)std::min<long long>(rows, 65535);
    holes_gemv_rows<<<grid, 256, 0, ctx->stream>>>(ctx->d_holes, np, rows, dx, dy);
  }
  CK(cudaGetLastError());
  CK(cudaMemcpyAsync(y, dy, sizeof(double) * (size_t)ny, cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  return TNSP_OK;
}

int tnsp_holes_gram(tnsp_ctx* ctx, double* gram) {
  if (!ctx || !gram) return TNSP_E_ARG;
  if (!ctx->holes_rows) return fail(ctx, TNSP_E_STATE, "no hole rows kept (tnsp_holes_keep before an observed sweep)");
  CK(cudaSetDevice(ctx->device));
  const long long rows = ctx->holes_rows, np = ctx->n_params;
  double* dg = nullptr;
  CK(cudaMalloc((void**)&dg, sizeof(double) * (size_t)rows * rows));
  const long long tiles = (rows + 31) / 32;
  if (tiles > 65535) {
    cudaFree(dg);
    return fail(ctx, TNSP_E_ARG, "too many kept hole rows for the Gram product");
  }
  holes_gram<<<dim3((unsigned)tiles, (unsigned)tiles), dim3(32, 8), 0, ctx->stream>>>(ctx->d_holes, np, rows, dg);
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaMemcpyAsync(gram, dg, sizeof(double) * (size_t)rows * rows, cudaMemcpyDeviceToHost,
                                            ctx->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
  cudaFree(dg);
  CK(e);
  return TNSP_OK;
}

int tnsp_observer_read(tnsp_ctx* ctx, double* scalars, double* delta, double* edelta) {
  if (!ctx) return TNSP_E_ARG;
  if (!ctx->B || !ctx->nslots) return fail(ctx, TNSP_E_STATE, "no chains");
  CK(cudaSetDevice(ctx->device));
  CK(cudaStreamSynchronize(ctx->stream));
  std::vector<double> acc((size_t)ctx->B * 8);
  CK(cudaMemcpy(acc.data(), ctx->d_acc, sizeof(double) * acc.size(), cudaMemcpyDeviceToHost));
  if (scalars) {
    for (int k = 0; k < 8; ++k) {
      double s = 0;
      for (int b = 0; b < ctx->B; ++b) s += acc[(size_t)b * 8 + k];
      scalars[k] = s;
    }
  }
  const long long n = ctx->n_params;
  const int threads = 256;
  const int blocks = (int)std::min<long long>((n + threads - 1) / threads, 4096);
  if (delta) {
    reduce_slots<<<blocks, threads, 0, ctx->stream>>>(ctx->d_delta, ctx->nslots, n, ctx->d_red);
    CK(cudaGetLastError());
    CK(cudaMemcpyAsync(delta, ctx->d_red, sizeof(double) * n, cudaMemcpyDeviceToHost, ctx->stream));
  }
  if (edelta) {
    reduce_slots<<<blocks, threads, 0, ctx->stream>>>(ctx->d_edelta, ctx->nslots, n, ctx->d_red + n);
    CK(cudaGetLastError());
    CK(cudaMemcpyAsync(edelta, ctx->d_red + n, sizeof(double) * n, cudaMemcpyDeviceToHost, ctx->stream));
  }
  CK(cudaStreamSynchronize(ctx->stream));
  return TNSP_OK;
}

int tnsp_samples_read(tnsp_ctx* ctx, double* eloc, double* log_ws, double* reweight) {
  if (!ctx) return TNSP_E_ARG;
  if (!ctx->d_rec) return fail(ctx, TNSP_E_STATE, "no observed sweeps recorded");
  CK(cudaSetDevice(ctx->device));
  CK(cudaStreamSynchronize(ctx->stream));
  const size_t n = (size_t)ctx->rec_n * ctx->B;
  const size_t cap = (size_t)ctx->rec_cap * ctx->B;
  if (eloc) CK(cudaMemcpy(eloc, ctx->d_rec, sizeof(double) * n, cudaMemcpyDeviceToHost));
  if (log_ws) CK(cudaMemcpy(log_ws, ctx->d_rec + cap, sizeof(double) * n, cudaMemcpyDeviceToHost));
  if (reweight) CK(cudaMemcpy(reweight, ctx->d_rec + 2 * cap, sizeof(double) * n, cudaMemcpyDeviceToHost));
  return TNSP_OK;
}

int tnsp_chains_read(tnsp_ctx* ctx, int32_t* configs, double* log_possibility) {
  if (!ctx) return TNSP_E_ARG;
  if (!ctx->B) return fail(ctx, TNSP_E_STATE, "no chains");
  CK(cudaSetDevice(ctx->device));
  CK(cudaStreamSynchronize(ctx->stream));
  if (configs)
    CK(cudaMemcpy(configs, ctx->d_conf, sizeof(int32_t) * ctx->B * ctx->L1 * ctx->L2, cudaMemcpyDeviceToHost));
  if (log_possibility) {
    std::vector<double> m(ctx->B);
    std::vector<int32_t> e(ctx->B);
    CK(cudaMemcpy(m.data(), ctx->d_ws_m, sizeof(double) * ctx->B, cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(e.data(), ctx->d_ws_e, sizeof(int32_t) * ctx->B, cudaMemcpyDeviceToHost));
    for (int b = 0; b < ctx->B; ++b) log_possibility[b] = 2.0 * (std::log(std::fabs(m[b])) + e[b] * 0.6931471805599453);
  }
  return TNSP_OK;
}

int tnsp_amplitude(tnsp_ctx* ctx, int B, const int32_t* configs, double* mantissa, int32_t* exponent) {
  if (!ctx) return TNSP_E_ARG;
  if (!ctx->has_lattice || !ctx->has_model) return fail(ctx, TNSP_E_STATE, "upload the lattice and the model first");
  if (B < 1 || !configs || !mantissa || !exponent) return fail(ctx, TNSP_E_ARG, "bad arguments");
  const int ns = ctx->L1 * ctx->L2;
  for (long long i = 0; i < (long long)B * ns; ++i)
    if (configs[i] < 0 || configs[i] >= ctx->P) return fail(ctx, TNSP_E_ARG, "configuration index out of range");
  CK(cudaSetDevice(ctx->device));
  int r = ensure_slots(ctx);
  if (r) return r;
  int32_t* dconf = nullptr;
  double* dm = nullptr;
  int32_t* de = nullptr;
  CK(cudaMalloc((void**)&dconf, sizeof(int32_t) * B * ns));
  CK(cudaMalloc((void**)&dm, sizeof(double) * B));
  CK(cudaMalloc((void**)&de, sizeof(int32_t) * B));
  CK(cudaMemcpyAsync(dconf, configs, sizeof(int32_t) * B * ns, cudaMemcpyHostToDevice, ctx->stream));
  Model md = make_model(ctx);
  const int grid = std::min(ctx->nslots, B);
  if (ctx->precision == TNSP_FP64)
    launch_amplitude_f64(grid, ctx->smem_bytes, ctx->stream, md, ctx->slots, ctx->d_scratch, ctx->d_ones, B, dconf,
                         dm, de, ctx->d_status);
  else if (ctx->precision == TNSP_DD)
    launch_amplitude_dd(grid, ctx->smem_bytes, ctx->stream, md, ctx->slots, ctx->d_scratch, ctx->d_ones, B, dconf,
                        dm, de, ctx->d_status);
  else if (ctx->precision == TNSP_MIXED)
    launch_amplitude_mx(grid, ctx->smem_bytes, ctx->stream, md, ctx->slots, ctx->d_scratch, ctx->d_ones, B, dconf,
                        dm, de, ctx->d_status);
  else
    launch_amplitude_f32(grid, ctx->smem_bytes, ctx->stream, md, ctx->slots, ctx->d_scratch, ctx->d_ones, B, dconf,
                         dm, de, ctx->d_status);
  CK(cudaGetLastError());
  CK(cudaMemcpyAsync(mantissa, dm, sizeof(double) * B, cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaMemcpyAsync(exponent, de, sizeof(int32_t) * B, cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  cudaFree(dconf);
  cudaFree(dm);
  cudaFree(de);
  return TNSP_OK;
}

int tnsp_device_status(tnsp_ctx* ctx, int32_t* status) {
  if (!ctx || !status) return TNSP_E_ARG;
  CK(cudaSetDevice(ctx->device));
  CK(cudaStreamSynchronize(ctx->stream));
  CK(cudaMemcpy(status, ctx->d_status, sizeof(int32_t), cudaMemcpyDeviceToHost));
  CK(cudaMemset(ctx->d_status, 0, sizeof(int32_t)));
  return TNSP_OK;
}

int tnsp_last_timing(tnsp_ctx* ctx, double* ms, int64_t* launches) {
  if (!ctx) return TNSP_E_ARG;
  if (ms) *ms = ctx->last_ms;
  if (launches) *launches = ctx->last_launches;
  return TNSP_OK;
}

int tnsp_counters_read(tnsp_ctx* ctx, double* flops, int reset) {
  if (!ctx || !flops) return TNSP_E_ARG;
  if (!ctx->nslots) return fail(ctx, TNSP_E_STATE, "no chains");
  CK(cudaSetDevice(ctx->device));
  CK(cudaStreamSynchronize(ctx->stream));
  std::vector<double> f((size_t)kCounters * ctx->nslots);
  CK(cudaMemcpy(f.data(), ctx->d_flops, sizeof(double) * f.size(), cudaMemcpyDeviceToHost));
  for (int k = 0; k < kCounters; ++k) {
    double s = 0;
    for (int i = 0; i < ctx->nslots; ++i) s += f[(size_t)i * kCounters + k];
    flops[k] = s;
  }
  if (reset) CK(cudaMemset(ctx->d_flops, 0, sizeof(double) * f.size()));
  return TNSP_OK;
}

}  // extern "C"

