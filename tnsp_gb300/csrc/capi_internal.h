// Host-side context of the C ABI and the per-slot scratch plan, shared by tnsp_capi.cu and noalloc.cu.
#pragma once
#include <cuda_runtime.h>

#include <algorithm>
#include <string>
#include <vector>

#include "../../include/tnsp_gb300.h"
#include "launch.h"

struct tnsp_ctx {
  int device = 0;
  cudaStream_t stream = nullptr;
  std::string err;
  // lattice
  bool has_lattice = false, has_model = false;
  int L1 = 0, L2 = 0, P = 0, cut = 0, Dmax = 0;
  std::vector<int> dims;
  std::vector<long long> off;
  long long n_params = 0;
  double* dA64 = nullptr;
  float* dA32 = nullptr;           // float copy (TNSP_FP32)
  tnsp::dd* dAdd = nullptr;        // double-float copy (TNSP_DD)
  int* d_dims = nullptr;
  long long* d_off = nullptr;
  std::vector<double> hostA;       // host copy of the site tensors (charge validation)
  int* d_qleg = nullptr;           // [site][4][Dmax]
  int* d_qphys = nullptr;          // [P]
  int* d_sflux = nullptr;          // [site]
  bool charged = false;
  // fermionic lattice (tnsp_lattice_fermion): eight sign-folded slices per site and their offsets
  bool fermion = false;
  int fermion_pT = 0;
  double* dF64 = nullptr;
  float* dF32 = nullptr;
  tnsp::dd* dFdd = nullptr;
  long long* d_foff = nullptr;
  // model
  int n_terms = 0;
  int* d_term_sites = nullptr;
  int* d_hterm = nullptr;
  int* d_vterm = nullptr;
  int* d_hflip = nullptr;
  int* d_tab_off = nullptr;
  int* d_tab_cnt = nullptr;
  int* d_tab_out = nullptr;
  double* d_tab_val = nullptr;
  int n_entries = 0;
  unsigned char* d_e_allow = nullptr;  // energy-table entries inside the observer's restricted subspace
  // the sweep's proposal tables (tnsp_model_hopping; the energy tables when absent) and their allow flags
  bool has_hop = false;
  int hop_entries = 0;
  int* d_s_hterm = nullptr;
  int* d_s_vterm = nullptr;
  int* d_s_hflip = nullptr;
  int* d_s_tab_off = nullptr;
  int* d_s_tab_cnt = nullptr;
  int* d_s_tab_out = nullptr;
  unsigned char* d_s_allow = nullptr;
  // chains
  int B = 0, precision = TNSP_FP64;
  int32_t* d_conf = nullptr;
  uint64_t* d_mt = nullptr;
  int32_t* d_mti = nullptr;
  double* d_ws_m = nullptr;
  int32_t* d_ws_e = nullptr;
  int64_t* d_accepted = nullptr;
  double* d_acc = nullptr;
  int32_t* d_status = nullptr;
  double* d_rec = nullptr;  // 3 x rec_cap x B
  int rec_cap = 0, rec_n = 0;
  // per-sample hole rows kept for the natural gradient (tnsp_holes_keep): holes_rows x n_params
  bool keep_holes = false;
  double* d_holes = nullptr;
  long long holes_rows = 0, holes_cap = 0;
  double* d_gemv = nullptr;  // operand / result staging of tnsp_holes_gemv
  long long gemv_cap = 0;
  // slots
  int nslots = 0;
  tnsp::Slots slots{};
  size_t elem = 8;    // bytes of the factorisation type T (shared-memory staging)
  void* d_scratch = nullptr;
  void* d_ones = nullptr;
  int* d_ldims = nullptr;
  int* d_lexp = nullptr;
  int* d_order = nullptr;
  double* d_delta = nullptr;
  double* d_edelta = nullptr;
  double* d_contrib = nullptr;
  double* d_red = nullptr;
  double* d_flops = nullptr;
  int* d_lq = nullptr;
  int* d_lfl = nullptr;
  int* d_tq = nullptr;
  int* d_tfl = nullptr;
  int* d_ilist = nullptr;
  size_t smem_bytes = 0;
  // options (tnsp_set_option)
  int jacobi_max = tnsp::kMaxSweepsJacobi;  // sweep limit of the one-sided Jacobi SVD
  int blocks_per_sm = 0;                    // resident sampler blocks per SM (0: the occupancy limit)
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  double last_ms = 0;
  long long last_launches = 0;
};


// message of the calling thread's last failed tnsp_amplitude_noalloc call (noalloc.cu); returned by
// tnsp_last_error(NULL)
const char* tnsp_noalloc_error();

namespace tnsp {

// scratch layout of one slot: byte offsets of its areas, S-typed (storage / contraction type, ssize
// bytes per element) or T-typed (factorisation type, tsize bytes), each aligned to 256 bytes
inline void plan_slots(const tnsp_ctx* c, Slots& s, long long tsize, long long ssize) {
  const long long cut = c->cut, D = c->Dmax, Lmax = std::max(c->L1, c->L2);
  const long long chi = cut * D;
  s.capB = cut * D * cut;
  s.capT = chi * D * chi;
  s.capR = chi * chi;
  s.capE = cut * D * cut;
  s.capS = D * D * D * cut * cut;
  s.capH = D * D * D * D;
  long long o = 0;
  auto take = [&](long long n, long long esize) {
    const long long r = o;
    o += (n * esize + 255) / 256 * 256;
    return r;
  };
  s.o_lines[F_UP] = take((long long)c->L1 * c->L2 * s.capB, ssize);
  s.o_lines[F_DOWN] = take((long long)c->L1 * c->L2 * s.capB, ssize);
  s.o_lines[F_LEFT] = take((long long)c->L2 * c->L1 * s.capB, ssize);
  s.o_lines[F_RIGHT] = take((long long)c->L2 * c->L1 * s.capB, ssize);
  s.o_T = take((Lmax + 2) * s.capT, ssize);
  s.o_G = take(s.capT, tsize);
  s.o_R = take(s.capR, tsize);
  s.o_tau = take(chi, tsize);
  s.o_X = take(chi * chi, tsize);
  s.o_V = take(chi * chi, tsize);
  s.o_W = take(2 * chi * chi, tsize);
  s.o_sig = take(chi, tsize);
  // Q of each QR-sweep step, kept implicit (the reflectors stay in the site's compression buffer):
  // per site its sector table, the sectors' row lists, the reflector scalars and the panels' Tw factors
  s.o_qsec = take(Lmax * (1 + 6LL * kMaxSec), 4);
  s.o_qrow = take(Lmax * chi * D, 4);
  s.o_qtau = take(Lmax * chi, tsize);
  s.o_qtw = take(Lmax * (chi + kMaxSec) * kNB * kNB, tsize);
  s.o_E = take((Lmax + 1) * s.capE, ssize);
  s.o_F = take((Lmax + 1) * s.capE, ssize);
  s.o_t1 = take(s.capS, ssize);
  s.o_t2 = take(s.capS, ssize);
  s.o_w0 = take(s.capE, ssize);
  s.o_w1 = take(s.capE, ssize);
  s.o_h = take(s.capH, ssize);
  s.stride = o;
}

// element sizes of a precision mode: factorisation type T, storage / contraction type S
inline void precision_sizes(int precision, long long* tsize, long long* ssize) {
  *tsize = precision == TNSP_FP32 ? 4 : 8;
  *ssize = (precision == TNSP_FP32 || precision == TNSP_MIXED) ? 4 : 8;
}

}  // namespace tnsp
