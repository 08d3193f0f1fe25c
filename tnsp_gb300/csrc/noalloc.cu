// tnsp_amplitude_noalloc: the amplitude hole(()) of a batch of configurations without any
// device allocation.
//
// Who needs it: callers that cannot call cudaMalloc -- code running inside a CUDA-graph capture
// or another library's stream callback, processes whose device memory is entirely owned by a
// caching allocator they must not bypass, and embedded hosts that forbid allocation after start-up.
// The regular entry points allocate their per-chain scratch slots with cudaMalloc; this one takes
// every input and output as a caller-owned device pointer and uses a fixed scratch arena compiled
// into the library instead.
//
// The arena is a file-scope __device__ array of kNoAllocArenaBytes (64 MiB).  Every GPU that loads
// the library holds it until the process exits.  A problem whose scratch (metadata plus one
// per-chain slot) does not fit is rejected with TNSP_E_TOO_LARGE before anything is launched.
//
// Sharing: all calls on a device use the same arena, and it keeps the contents of the last call.
// Everything that must start at a known value (status word, the all-ones boundary element, site
// metadata) is rewritten by every call before the kernel runs.  Two calls whose work overlaps on
// the GPU (different streams, or different host threads) race on the arena and give undefined
// results: serialise them.
//
// Set-up: the first call on each device resolves the arena's device address with
// cudaGetSymbolAddress (with that device current) and caches it; make that first call before any
// stream capture begins.
#include <cuda_runtime.h>

#include <mutex>

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

}  // namespace tnsp_noalloc

extern "C" int tnsp_amplitude_noalloc(int L1, int L2, int P, const int* dims, const double* tensors, int cut, int B,
                                      const int32_t* configs, double* mantissa, int32_t* exponent, void* stream) {
  using namespace tnsp;
  using namespace tnsp_noalloc;
  auto err = [](int code, const char*) { return code; };  // the second argument documents the cause
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
  plan_slots(&shape, s);
  const size_t meta = align256(sizeof(int32_t))                      // status word
                      + align256(sizeof(double))                     // boundary "ones"
                      + align256(sizeof(int) * ns * 4)               // dims
                      + align256(sizeof(long long) * ns);            // offsets
  const size_t per_slot = align256((size_t)s.stride * sizeof(double)) + align256(sizeof(int) * 4 * kMaxL * kMaxL * 3) +
                          align256(sizeof(int) * 4 * kMaxL) + align256(sizeof(int) * (size_t)cut * Dmax);
  if (meta + per_slot > kNoAllocArenaBytes)
    return err(TNSP_E_TOO_LARGE, "one chain slot of this lattice/cut does not fit in the 64 MiB arena");
  int nslots = (int)((kNoAllocArenaBytes - meta) / per_slot);
  if (nslots > B) nslots = B;
  int dev = 0, sms = 0;
  if (cudaGetDevice(&dev) == cudaSuccess &&
      cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) == cudaSuccess && sms > 0 &&
      nslots > 2 * sms)
    nslots = 2 * sms;
  unsigned char* base = nullptr;
  cudaError_t e = arena_for_current_device(&base);
  if (e != cudaSuccess) return err(TNSP_E_CUDA, "cudaGetSymbolAddress failed");
  cudaStream_t st = (cudaStream_t)stream;
  unsigned char* p = base;
  int32_t* d_status = (int32_t*)p;
  p += align256(sizeof(int32_t));
  double* d_ones = (double*)p;
  p += align256(sizeof(double));
  int* d_dims = (int*)p;
  p += align256(sizeof(int) * ns * 4);
  long long* d_off = (long long*)p;
  p += align256(sizeof(long long) * ns);
  double* d_scratch = (double*)p;
  p += align256((size_t)s.stride * sizeof(double)) * nslots;
  s.ldims = (int*)p;
  p += align256(sizeof(int) * 4 * kMaxL * kMaxL * 3) * nslots;
  s.lexp = (int*)p;
  p += align256(sizeof(int) * 4 * kMaxL) * nslots;
  s.order = (int*)p;
  // per-slot arrays are indexed with the kernel's own strides: make the carved strides match
  // (stride in elements for scratch, fixed sizes for the integer arrays)
  s.stride = (long long)(align256((size_t)s.stride * sizeof(double)) / sizeof(double));
  const double one = 1.0;
  if ((e = cudaMemsetAsync(d_status, 0, sizeof(int32_t), st)) != cudaSuccess ||
      (e = cudaMemcpyAsync(d_ones, &one, sizeof(double), cudaMemcpyHostToDevice, st)) != cudaSuccess ||
      (e = cudaMemcpyAsync(d_dims, dims, sizeof(int) * ns * 4, cudaMemcpyHostToDevice, st)) != cudaSuccess ||
      (e = cudaMemcpyAsync(d_off, off_host, sizeof(long long) * ns, cudaMemcpyHostToDevice, st)) != cudaSuccess)
    return err(TNSP_E_CUDA, "arena set-up copy failed");
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
  amplitude_kernel<double><<<nslots, kThreads, 0, st>>>(md, s, d_scratch, d_ones, B, configs, mantissa, exponent,
                                                        d_status);
  if ((e = cudaGetLastError()) != cudaSuccess) return err(TNSP_E_CUDA, "kernel launch failed");
  int32_t status = 0;
  if ((e = cudaMemcpyAsync(&status, d_status, sizeof(int32_t), cudaMemcpyDeviceToHost, st)) != cudaSuccess ||
      (e = cudaStreamSynchronize(st)) != cudaSuccess)
    return err(TNSP_E_CUDA, "stream synchronisation failed");
  if (status & (TNSP_ST_SVD_NOCONV | TNSP_ST_NONFINITE)) return err(TNSP_E_DEVICE, "device status word set");
  return TNSP_OK;
}
