// tnsp_amplitude_noalloc: the amplitude hole(()) of a batch of configurations without any
// device allocation.
//
// Who needs it: callers that must not allocate device memory once they are running -- a host
// application whose device memory is all reserved by its own pool or caching allocator (a
// cudaMalloc behind the allocator's back fails or fragments the pool), and latency-bound or
// real-time hosts, where cudaMalloc and cudaFree can synchronise the device and take unbounded
// time.  The regular entry points allocate their per-chain scratch slots with cudaMalloc; this one
// takes every input and output as a caller-owned device pointer and uses a fixed scratch arena
// compiled into the library instead.
//
// The arena is a file-scope __device__ array of kNoAllocArenaBytes (64 MiB).  Every GPU that loads
// the library holds it until the process exits.  A problem whose scratch (metadata plus one
// per-chain slot) does not fit is rejected with TNSP_E_TOO_LARGE before anything is launched.
//
// Sharing: all calls on a device use the same arena, and it keeps the contents of the last call.
// Everything that must start at a known value (status word, the all-ones boundary element, site
// metadata, the all-zero charges: this entry point treats every matrix as one block) is rewritten
// by every call before the kernel runs.  Two calls whose work overlaps on the GPU (different
// streams, or different host threads) race on the arena and give undefined results: serialise them.
//
// Set-up: the first call on each device resolves the arena's device address with
// cudaGetSymbolAddress (with that device current) and caches it.  Every call copies small host
// arrays to the arena and waits for its stream before it returns, so no call can be captured into a
// CUDA graph.
//
// Errors: the reason of the calling thread's last failure is kept in a thread-local buffer and is
// returned by tnsp_last_error(NULL).
#include <cuda_runtime.h>

#include <cstdio>
#include <mutex>

#include "capi_internal.h"

namespace tnsp_noalloc {

constexpr size_t kNoAllocArenaBytes = 64ull << 20;
constexpr int kMaxDevices = 64;

static __device__ __align__(256) unsigned char g_arena[kNoAllocArenaBytes];

struct DeviceArena {
  bool ready = false;
  unsigned char* ptr = nullptr;
};

static DeviceArena g_dev[kMaxDevices];
static std::mutex g_mu;

// device address of the arena for the current device (resolved once per device)
static cudaError_t arena_for_current_device(unsigned char** out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
  std::lock_guard<std::mutex> lock(g_mu);
  if (!g_dev[dev].ready) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_arena);
    if (e != cudaSuccess) return e;
    g_dev[dev].ptr = (unsigned char*)p;
    g_dev[dev].ready = true;
  }
  *out = g_dev[dev].ptr;
  return cudaSuccess;
}

static size_t align256(size_t n) { return (n + 255) / 256 * 256; }

static thread_local char g_err[160] = "";

// records the reason of a failure for tnsp_last_error(NULL) and returns its code
static int fail(int code, const char* what, cudaError_t e = cudaSuccess) {
  if (e != cudaSuccess)
    snprintf(g_err, sizeof g_err, "tnsp_amplitude_noalloc: %s (%s)", what, cudaGetErrorString(e));
  else
    snprintf(g_err, sizeof g_err, "tnsp_amplitude_noalloc: %s", what);
  return code;
}

}  // namespace tnsp_noalloc

const char* tnsp_noalloc_error() { return tnsp_noalloc::g_err; }

extern "C" int tnsp_amplitude_noalloc(int L1, int L2, int P, const int* dims, const double* tensors, int cut, int B,
                                      const int32_t* configs, double* mantissa, int32_t* exponent, void* stream) {
  using namespace tnsp;
  using namespace tnsp_noalloc;
  auto err = [](int code, const char* what, cudaError_t e = cudaSuccess) { return fail(code, what, e); };
  if (L1 < 1 || L2 < 1 || L1 > kMaxL || L2 > kMaxL) return err(TNSP_E_ARG, "lattice extent out of range (1..16)");
  if (P < 1 || cut < 1 || B < 1) return err(TNSP_E_ARG, "P, cut and B must be positive");
  if (!dims || !tensors || !configs || !mantissa || !exponent) return err(TNSP_E_ARG, "null pointer argument");
  // host-side plan: offsets and the largest bond extent
  const int ns = L1 * L2;
  int Dmax = 1;
  long long off_host[kMaxSites];
  long long total = 0;
  for (int id = 0; id < ns; ++id) {
    const int* d = dims + id * 4;
    for (int k = 0; k < 4; ++k) {
      if (d[k] < 1) return err(TNSP_E_ARG, "bond extents must be >= 1");
      if (d[k] > Dmax) Dmax = d[k];
    }
    off_host[id] = total;
    total += (long long)P * d[0] * d[1] * d[2] * d[3];
  }
  // the same per-chain slot layout as the allocating entry points
  tnsp_ctx shape;
  shape.L1 = L1;
  shape.L2 = L2;
  shape.cut = cut;
  shape.Dmax = Dmax;
  Slots s{};
  plan_slots(&shape, s, sizeof(double), sizeof(double));
  const long long chi = (long long)cut * Dmax;
  if (chi > kMaxChi) return err(TNSP_E_TOO_LARGE, "cut * max bond extent exceeds 1024");
  // arena layout: metadata, then one array per kind with an exact per-slot stride (the kernels
  // index every per-slot array as base + blockIdx.x * stride)
  const size_t meta = align256(sizeof(int32_t))                      // status word
                      + align256(sizeof(double))                     // boundary "ones"
                      + align256(sizeof(int) * ns * 4)               // dims
                      + align256(sizeof(long long) * ns)             // offsets
                      + align256(sizeof(int) * (size_t)ns * 4 * Dmax) // leg charges (zero)
                      + align256(sizeof(int) * (size_t)P)            // physical charges (zero)
                      + align256(sizeof(int) * (size_t)ns);          // site flux (zero)
  const size_t scratch_slot = align256((size_t)s.stride);
  const size_t ints_slot = sizeof(int) * ((size_t)4 * kMaxL * kMaxL * 3 + 4 * kMaxL + (size_t)cut * (Dmax + 1) +
                                          (size_t)4 * kMaxL * kMaxL * 2 * cut + 4 * kMaxL * kMaxL +
                                          (size_t)kMaxL * 3 * chi + kMaxL + (size_t)(chi * Dmax + chi));
  const size_t per_slot = scratch_slot + ints_slot;
  const size_t slack = 16 * 256;  // alignment of the eight per-slot arrays
  if (meta + per_slot + slack > kNoAllocArenaBytes)
    return err(TNSP_E_TOO_LARGE, "one chain slot of this lattice/cut does not fit in the 64 MiB arena");
  int nslots = (int)((kNoAllocArenaBytes - meta - slack) / per_slot);
  if (nslots > B) nslots = B;
  int dev = 0, sms = 0;
  if (cudaGetDevice(&dev) == cudaSuccess &&
      cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) == cudaSuccess && sms > 0 &&
      nslots > 4 * sms)
    nslots = 4 * sms;
  unsigned char* base = nullptr;
  cudaError_t e = arena_for_current_device(&base);
  if (e != cudaSuccess) return err(TNSP_E_CUDA, "cudaGetSymbolAddress failed", e);
  cudaStream_t st = (cudaStream_t)stream;
  size_t o = 0;
  auto carve = [&](size_t bytes) {
    o = align256(o);
    unsigned char* r = base + o;
    o += bytes;
    return r;
  };
  int32_t* d_status = (int32_t*)carve(sizeof(int32_t));
  double* d_ones = (double*)carve(sizeof(double));
  int* d_dims = (int*)carve(sizeof(int) * ns * 4);
  long long* d_off = (long long*)carve(sizeof(long long) * ns);
  int* d_qleg = (int*)carve(sizeof(int) * (size_t)ns * 4 * Dmax);
  int* d_qphys = (int*)carve(sizeof(int) * (size_t)P);
  int* d_sflux = (int*)carve(sizeof(int) * (size_t)ns);
  s.stride = (long long)scratch_slot;
  double* d_scratch = (double*)carve(scratch_slot * nslots);
  s.ldims = (int*)carve(sizeof(int) * 4 * kMaxL * kMaxL * 3 * (size_t)nslots);
  s.lexp = (int*)carve(sizeof(int) * 4 * kMaxL * (size_t)nslots);
  s.order = (int*)carve(sizeof(int) * (size_t)cut * (Dmax + 1) * nslots);
  s.lq = (int*)carve(sizeof(int) * (size_t)4 * kMaxL * kMaxL * 2 * cut * nslots);
  s.lfl = (int*)carve(sizeof(int) * (size_t)4 * kMaxL * kMaxL * nslots);
  s.tq = (int*)carve(sizeof(int) * (size_t)kMaxL * 3 * chi * nslots);
  s.tfl = (int*)carve(sizeof(int) * (size_t)kMaxL * nslots);
  s.ilist = (int*)carve(sizeof(int) * (size_t)(chi * Dmax + chi) * nslots);
  s.smem_elems = 0;  // no dynamic shared memory: sector blocks are staged in the arena
  if (o > kNoAllocArenaBytes) return err(TNSP_E_TOO_LARGE, "arena layout overflow");
  const double one = 1.0;
  if ((e = cudaMemsetAsync(d_status, 0, sizeof(int32_t), st)) != cudaSuccess ||
      (e = cudaMemcpyAsync(d_ones, &one, sizeof(double), cudaMemcpyHostToDevice, st)) != cudaSuccess ||
      (e = cudaMemcpyAsync(d_dims, dims, sizeof(int) * ns * 4, cudaMemcpyHostToDevice, st)) != cudaSuccess ||
      (e = cudaMemcpyAsync(d_off, off_host, sizeof(long long) * ns, cudaMemcpyHostToDevice, st)) != cudaSuccess ||
      (e = cudaMemsetAsync(d_qleg, 0, sizeof(int) * (size_t)ns * 4 * Dmax, st)) != cudaSuccess ||
      (e = cudaMemsetAsync(d_qphys, 0, sizeof(int) * (size_t)P, st)) != cudaSuccess ||
      (e = cudaMemsetAsync(d_sflux, 0, sizeof(int) * (size_t)ns, st)) != cudaSuccess)
    return err(TNSP_E_CUDA, "arena set-up copy failed", e);
  Model md{};
  md.L1 = L1;
  md.L2 = L2;
  md.P = P;
  md.cut = cut;
  md.Dmax = Dmax;
  md.dims = d_dims;
  md.off = d_off;
  md.A = tensors;
  md.n_params = total;
  md.qleg = d_qleg;
  md.qphys = d_qphys;
  md.sflux = d_sflux;
  md.jacobi_max = kMaxSweepsJacobi;
  launch_amplitude_f64(nslots, 0, st, md, s, d_scratch, d_ones, B, configs, mantissa, exponent, d_status);
  if ((e = cudaGetLastError()) != cudaSuccess) return err(TNSP_E_CUDA, "kernel launch failed", e);
  int32_t status = 0;
  if ((e = cudaMemcpyAsync(&status, d_status, sizeof(int32_t), cudaMemcpyDeviceToHost, st)) != cudaSuccess ||
      (e = cudaStreamSynchronize(st)) != cudaSuccess)
    return err(TNSP_E_CUDA, "stream synchronisation failed", e);
  if (status & (TNSP_ST_SVD_NOCONV | TNSP_ST_NONFINITE)) {
    char buf[96];
    snprintf(buf, sizeof buf, "device status 0x%x (see TNSP_ST_* bits)", status);
    return err(TNSP_E_DEVICE, buf);
  }
  g_err[0] = 0;
  return TNSP_OK;
}
