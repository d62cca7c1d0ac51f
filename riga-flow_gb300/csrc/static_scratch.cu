// static_scratch.cu — pricing without any device allocation.
//
// Some callers cannot allocate device memory: hosts whose allocator owns every device byte (a
// serving framework's memory pool, a process started under a hard device-memory budget), or
// plugins that must not call cudaMalloc/cudaFree behind their host's back (cudaFree synchronises
// the whole device, and both take memory outside the host's accounting).  rg_price_put_leg_static serves
// them: it runs the same pipeline and kernels as rg_price_put_leg, but every device buffer it needs
// (request tables, calibration scratch, per-block partial sums, the reduced sums, optional
// per-path KO steps) is carved out of one file-scope __device__ array of RG_STATIC_SCRATCH_BYTES,
// and it creates no engine, stream or event.  Requests whose buffers do not fit are rejected with
// "invalid_argument".
//
// The array is a module global: with lazy module loading (the CUDA default) it is reserved on a
// GPU the first time the library's kernels are used there; with CUDA_MODULE_LOADING=EAGER every
// context that loads the library reserves it, whether or not this entry point is called.  Either
// way it stays reserved until the process exits.
//
// The array is process state shared by every call on a device and keeps the last call's contents;
// every region the pipeline reads is written by the same call first, so nothing needs clearing.
// Calls on one device are serialised by that device's lock and each returns only after its work
// on the legacy default stream has finished; work of two calls that overlapped on the GPU would
// race on the array, which is why the lock exists.  The first call on a device resolves the
// array's device address with cudaGetSymbolAddress while that device is current.
#include <mutex>
#include <new>

#include "rg_internal.h"

#define RG_STATIC_SCRATCH_BYTES (16u << 20)
#define RG_STATIC_MAX_DEVICES 64

static __device__ __align__(256) unsigned char g_static_scratch[RG_STATIC_SCRATCH_BYTES];

namespace {

std::mutex g_static_mu[RG_STATIC_MAX_DEVICES];
void* g_static_ptr[RG_STATIC_MAX_DEVICES];
int g_static_sms[RG_STATIC_MAX_DEVICES];

// Bump allocation in the static array; restarts at every fused launch.
struct StaticWorkspace : rg::Workspace {
  uint8_t* base = nullptr;
  size_t cap = 0, off = 0;
  double sums[RG_MAX_SCEN * RG_ACC];
  void begin_launch() override { off = 0; }
  bool persistent() const override { return false; }
  bool may_tune() const override { return false; }
  void* device(int slot, size_t bytes) override {
    (void)slot;
    const size_t o = (off + 255) & ~(size_t)255;
    if (bytes > cap || o > cap - bytes)
      rg::raise(RG_ERR_INVALID_ARGUMENT,
                "this request needs more device scratch than the 16 MiB static region of "
                "rg_price_put_leg_static holds (fewer paths, no trace events or rg_price_put_leg)");
    off = o + bytes;
    return base + o;
  }
  void* host(size_t bytes) override {
    if (bytes > sizeof sums) rg::raise(RG_ERR_INVALID_ARGUMENT, "too many scenarios for the static region");
    return sums;
  }
};

}  // namespace

extern "C" int32_t rg_price_put_leg_static(const rg_price_request* request, rg_price_result* out) {
  try {
    if (!request || !out) rg::raise(RG_ERR_INVALID_ARGUMENT, "null argument");
    int32_t g = rg_guard_device();
    if (g) return g;
    int dev = 0;
    rg::cuda_check(cudaGetDevice(&dev), "cudaGetDevice");
    if (dev < 0 || dev >= RG_STATIC_MAX_DEVICES) rg::raise(RG_ERR_INVALID_ARGUMENT, "device index out of range");
    std::lock_guard<std::mutex> lock(g_static_mu[dev]);
    if (!g_static_ptr[dev]) {
      // one-time set-up on this device (the current one): the array's device address and the
      // device's own SM count, which sizes the FP32 grid and the partial-sum region
      void* p = nullptr;
      int sms = 0;
      rg::cuda_check(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev),
                     "cudaDeviceGetAttribute");
      rg::cuda_check(cudaGetSymbolAddress(&p, g_static_scratch), "cudaGetSymbolAddress");
      g_static_sms[dev] = sms;
      g_static_ptr[dev] = p;
    }
    StaticWorkspace W;
    W.base = static_cast<uint8_t*>(g_static_ptr[dev]);
    W.cap = RG_STATIC_SCRATCH_BYTES;
    W.stream = 0;  // legacy default stream; the call is synchronous
    W.sm_count = g_static_sms[dev];
    rg::price_with(W, request, nullptr, 0, out);
    return RG_OK;
  } catch (const rg::Error& e) {
    rg::set_last_error(e.message);
    return e.status;
  } catch (const std::bad_alloc&) {
    rg::set_last_error("host allocation failed");
    return RG_ERR_GPU_ERROR;
  }
}
