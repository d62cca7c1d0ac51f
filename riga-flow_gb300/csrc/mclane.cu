// mclane.cu — the reference's pseudo-random lane on the device: ChaCha8Rng::seed_from_u64(seed)
// feeding rand_distr's StandardNormal (rand_chacha 0.9.0, rand_core 0.9.5, rand_distr 0.5.1; the
// reference draws it in crates/riga-engine/src/note.rs:58,123-127 and pathcube.rs:37-66).
//
// The stream is sequential: a normal consumes one 64-bit word, or more when the ziggurat rejects,
// so where the k-th normal starts depends on every earlier draw.  The device reproduces it exactly
// by a parallel parse:
//   1. keystream — ChaCha8 is counter-based: one thread per 64-byte block writes its 8 words
//      (next_u64 = low word | high word << 32 of consecutive output words);
//   2. transfer — the words are cut into segments of B words; for every segment and every entry
//      offset e < E (where the previous segment's last normal may end) one thread simulates the
//      ziggurat's consumption through the segment and records the exit offset and the count;
//   3. scan — one thread chains the segments from word 0 and prefix-sums the counts;
//   4. emit — one thread per segment re-runs from its true entry and writes the normals whose
//      global index falls in the requested range.
// The ziggurat is Doornik's ZIGNOR with 256 layers (R = 3.6541528853610088, V = 0.00492867323399);
// its tables are regenerated from that recurrence and rounded to the 18 decimals of the crate's
// table literals.  Compiled with -fmad=false so every product and sum rounds as on the host; the
// wedge test's exp and the tail's log are CUDA's (an accept/reject decision could differ from the
// host's libm only for a value within an ulp of the threshold).
#include <cmath>
#include <cstdio>
#include <cstdlib>

#include "rg_internal.h"

namespace rg {

namespace {

constexpr double kZigR = 3.6541528853610088;
constexpr int kSegWords = 2048;  // B
constexpr int kEntries = 32;     // E: a normal spans at most E words past a segment end
constexpr int kTailIters = 64;   // tail-loop bound (each pass succeeds with probability > 0.9)

struct ZigTables {
  double x[257], f[257];
};

double round18(double v) {
  char b[64];
  snprintf(b, sizeof b, "%.18f", v);
  return strtod(b, nullptr);
}

const ZigTables& zig_tables() {
  static ZigTables t;
  static std::once_flag once;
  std::call_once(once, [] {
    const double r = kZigR, v = 0.00492867323399;
    double x[257];
    x[0] = v / std::exp(-r * r / 2.0);
    x[1] = r;
    for (int i = 2; i < 256; ++i) {
      const double last = x[i - 1];
      x[i] = std::sqrt(-2.0 * std::log(v / last + std::exp(-last * last / 2.0)));
    }
    x[256] = 0.0;
    for (int i = 0; i < 257; ++i) {
      t.x[i] = round18(x[i]);
      t.f[i] = round18(std::exp(-x[i] * x[i] / 2.0));
    }
  });
  return t;
}

struct ChaKey {
  uint32_t k[8];
};

// seed_from_u64: eight PCG32 (XSH-RR) outputs of the seed state (rand_core 0.9.5).
ChaKey chacha_key(uint64_t state) {
  ChaKey key;
  for (int i = 0; i < 8; ++i) {
    state = state * 6364136223846793005ULL + 11634580027462260723ULL;
    const uint32_t xs = (uint32_t)(((state >> 18) ^ state) >> 27);
    const uint32_t rot = (uint32_t)(state >> 59);
    key.k[i] = (xs >> rot) | (xs << ((32 - rot) & 31));
  }
  return key;
}

__device__ __forceinline__ uint32_t rotl(uint32_t v, int c) { return (v << c) | (v >> (32 - c)); }

#define RG_QR(a, b, c, d)               \
  x[a] += x[b]; x[d] = rotl(x[d] ^ x[a], 16); \
  x[c] += x[d]; x[b] = rotl(x[b] ^ x[c], 12); \
  x[a] += x[b]; x[d] = rotl(x[d] ^ x[a], 8);  \
  x[c] += x[d]; x[b] = rotl(x[b] ^ x[c], 7);

// ChaCha with 8 rounds, 64-bit block counter in words 12-13, stream 0 in words 14-15.
__global__ void chacha8_stream_kernel(ChaKey key, uint64_t nblocks, uint64_t* __restrict__ out) {
  const uint64_t b = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= nblocks) return;
  uint32_t s[16] = {0x61707865u, 0x3320646eu, 0x79622d32u, 0x6b206574u};
#pragma unroll
  for (int i = 0; i < 8; ++i) s[4 + i] = key.k[i];
  s[12] = (uint32_t)b;
  s[13] = (uint32_t)(b >> 32);
  s[14] = 0;
  s[15] = 0;
  uint32_t x[16];
#pragma unroll
  for (int i = 0; i < 16; ++i) x[i] = s[i];
#pragma unroll
  for (int r = 0; r < 4; ++r) {
    RG_QR(0, 4, 8, 12) RG_QR(1, 5, 9, 13) RG_QR(2, 6, 10, 14) RG_QR(3, 7, 11, 15)
    RG_QR(0, 5, 10, 15) RG_QR(1, 6, 11, 12) RG_QR(2, 7, 8, 13) RG_QR(3, 4, 9, 14)
  }
#pragma unroll
  for (int i = 0; i < 8; ++i)
    out[b * 8 + i] = (uint64_t)(x[2 * i] + s[2 * i]) | ((uint64_t)(x[2 * i + 1] + s[2 * i + 1]) << 32);
}
#undef RG_QR

__device__ __forceinline__ double from_bits(uint64_t frac52, int e) {
  return __longlong_as_double((long long)(frac52 | ((uint64_t)(1023 + e) << 52)));
}

// One StandardNormal draw starting at word `pos`: returns the words consumed (0 if the stream or
// the tail-loop bound ran out) and the value.
__device__ int zig_draw(const uint64_t* __restrict__ U, uint64_t pos, uint64_t limit,
                        const double* __restrict__ zx, const double* __restrict__ zf, double* value) {
  uint64_t p = pos;
  for (int attempt = 0; attempt < kTailIters; ++attempt) {
    if (p >= limit) return 0;
    const uint64_t bits = U[p++];
    const int i = (int)(bits & 0xff);
    const double u = from_bits(bits >> 12, 1) - 3.0;
    const double x = u * zx[i];
    if (fabs(x) < zx[i + 1]) {
      *value = x;
      return (int)(p - pos);
    }
    if (i == 0) {
      double xx = 1.0, y = 0.0;
      int it = 0;
      while (-2.0 * y < xx * xx) {
        if (p + 2 > limit || ++it > kTailIters) return 0;
        const double x_ = from_bits(U[p++] >> 12, 0) - (1.0 - 2.220446049250313e-16 / 2.0);
        const double y_ = from_bits(U[p++] >> 12, 0) - (1.0 - 2.220446049250313e-16 / 2.0);
        xx = log(x_) / kZigR;
        y = log(y_);
      }
      *value = u < 0.0 ? xx - kZigR : kZigR - xx;
      return (int)(p - pos);
    }
    if (p >= limit) return 0;
    const double uu = (double)(U[p++] >> 11) * (1.0 / 9007199254740992.0);
    if (zf[i + 1] + (zf[i] - zf[i + 1]) * uu < exp(-x * x / 2.0)) {
      *value = x;
      return (int)(p - pos);
    }
  }
  return 0;
}

__global__ void zig_transfer_kernel(const uint64_t* __restrict__ U, uint64_t limit, uint64_t segs,
                                    const double* __restrict__ zt, int32_t* __restrict__ exit_off,
                                    int32_t* __restrict__ count, int* __restrict__ status) {
  const uint64_t t = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= segs * kEntries) return;
  const uint64_t g = t / kEntries;
  const int e = (int)(t % kEntries);
  const uint64_t end = (g + 1) * kSegWords;
  uint64_t pos = g * kSegWords + e;
  int cnt = 0;
  double v;
  while (pos < end) {
    const int used = zig_draw(U, pos, limit, zt, zt + 257, &v);
    if (used == 0) {
      atomicExch(status, 1);
      break;
    }
    pos += used;
    ++cnt;
  }
  const int64_t ex = (int64_t)pos - (int64_t)end;
  if (ex < 0 || ex >= kEntries) atomicExch(status, 2);
  exit_off[t] = (int32_t)(ex < 0 ? 0 : (ex >= kEntries ? kEntries - 1 : ex));
  count[t] = cnt;
}

// Chains the segments from word 0: entry[g] and the global index of segment g's first normal.
__global__ void zig_scan_kernel(const int32_t* __restrict__ exit_off, const int32_t* __restrict__ count,
                                uint64_t segs, int32_t* __restrict__ entry, uint64_t* __restrict__ base,
                                uint64_t* __restrict__ total) {
  if (blockIdx.x != 0 || threadIdx.x != 0) return;
  int e = 0;
  uint64_t k = 0;
  for (uint64_t g = 0; g < segs; ++g) {
    entry[g] = e;
    base[g] = k;
    k += (uint64_t)count[g * kEntries + e];
    e = exit_off[g * kEntries + e];
  }
  *total = k;
}

__global__ void zig_emit_kernel(const uint64_t* __restrict__ U, uint64_t limit, uint64_t segs,
                                const double* __restrict__ zt, const int32_t* __restrict__ entry,
                                const uint64_t* __restrict__ base, uint64_t first, uint64_t n,
                                double* __restrict__ out, int* __restrict__ status) {
  const uint64_t g = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= segs) return;
  uint64_t k = base[g];
  if (k >= first + n) return;
  const uint64_t end = (g + 1) * kSegWords;
  uint64_t pos = g * kSegWords + entry[g];
  double v;
  while (pos < end && k < first + n) {
    const int used = zig_draw(U, pos, limit, zt, zt + 257, &v);
    if (used == 0) {
      atomicExch(status, 1);
      return;
    }
    if (k >= first) out[k - first] = v;
    pos += used;
    ++k;
  }
}

}  // namespace

void mc_normals(uint64_t seed, uint64_t first, uint64_t count, double* d_out, Workspace& W) {
  if (count == 0) return;
  const ZigTables& zt = zig_tables();
  const ChaKey key = chacha_key(seed);
  cudaStream_t s = W.stream;
  // words: the normals need about 1.0125 words each (ziggurat acceptance); grow until they fit
  uint64_t need = first + count;
  uint64_t words = need + need / 16 + 8192;
  for (int attempt = 0; attempt < 4; ++attempt) {
    const uint64_t segs = (words + kSegWords - 1) / kSegWords;
    const uint64_t blocks = (segs * kSegWords + 8 * 64 + 7) / 8;  // keystream padding past the last segment
    const uint64_t limit = blocks * 8;
    uint8_t* aux = static_cast<uint8_t*>(W.device(WS_MCAUX, 4096 + sizeof(double) * 514 + segs * kEntries * 8 +
                                                                segs * 16 + 256));
    uint64_t* U = static_cast<uint64_t*>(W.device(WS_MCKEYS, limit * sizeof(uint64_t)));
    double* d_zt = reinterpret_cast<double*>(aux + 4096);
    int32_t* exit_off = reinterpret_cast<int32_t*>(aux + 4096 + sizeof(double) * 514);
    int32_t* cnt = exit_off + segs * kEntries;
    int32_t* entry = cnt + segs * kEntries;
    uint64_t* base = reinterpret_cast<uint64_t*>(((uintptr_t)(entry + segs) + 15) & ~(uintptr_t)15);
    int* status = reinterpret_cast<int*>(aux);
    uint64_t* total = reinterpret_cast<uint64_t*>(aux + 64);
    double host_zt[514];
    memcpy(host_zt, zt.x, sizeof zt.x);
    memcpy(host_zt + 257, zt.f, sizeof zt.f);
    cuda_check(cudaMemsetAsync(aux, 0, 128, s), "mc status");
    cuda_check(cudaMemcpyAsync(d_zt, host_zt, sizeof host_zt, cudaMemcpyHostToDevice, s), "mc tables");
    chacha8_stream_kernel<<<(unsigned)((blocks + 127) / 128), 128, 0, s>>>(key, blocks, U);
    cuda_check(cudaGetLastError(), "chacha8_stream_kernel launch");
    const uint64_t threads = segs * kEntries;
    zig_transfer_kernel<<<(unsigned)((threads + 127) / 128), 128, 0, s>>>(U, limit, segs, d_zt, exit_off, cnt, status);
    cuda_check(cudaGetLastError(), "zig_transfer_kernel launch");
    zig_scan_kernel<<<1, 1, 0, s>>>(exit_off, cnt, segs, entry, base, total);
    cuda_check(cudaGetLastError(), "zig_scan_kernel launch");
    uint64_t host_total = 0;
    int host_status = 0;
    cuda_check(cudaMemcpyAsync(&host_total, total, sizeof host_total, cudaMemcpyDeviceToHost, s), "D2H");
    cuda_check(cudaMemcpyAsync(&host_status, status, sizeof host_status, cudaMemcpyDeviceToHost, s), "D2H");
    cuda_check(cudaStreamSynchronize(s), "mc parse");
    if (host_status) raise(RG_ERR_GPU_ERROR, "ChaCha8 normal stream: ziggurat parse overflow");
    if (host_total < need) {
      words = words * 2;
      continue;
    }
    zig_emit_kernel<<<(unsigned)((segs + 127) / 128), 128, 0, s>>>(U, limit, segs, d_zt, entry, base, first, count,
                                                                   d_out, status);
    cuda_check(cudaGetLastError(), "zig_emit_kernel launch");
    cuda_check(cudaMemcpyAsync(&host_status, status, sizeof host_status, cudaMemcpyDeviceToHost, s), "D2H");
    cuda_check(cudaStreamSynchronize(s), "mc emit");
    if (host_status) raise(RG_ERR_GPU_ERROR, "ChaCha8 normal stream: ziggurat emit overflow");
    return;
  }
  raise(RG_ERR_GPU_ERROR, "ChaCha8 normal stream: could not size the keystream");
}

// ------------------------------------------------------------------ PathCube (pathcube.rs) ----
namespace {

// y = L·z per (path, time) in the reference's order (Cholesky::apply_into), stored as f32.
__global__ void correlate_block_kernel(const double* __restrict__ z, const double* __restrict__ L, int F,
                                       uint64_t cells, float* __restrict__ out) {
  const uint64_t c = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= cells) return;
  const double* zc = z + c * F;
  for (int i = 0; i < F; ++i) {
    double acc = 0.0;
    for (int j = 0; j <= i; ++j) acc += L[i * F + j] * zc[j];
    out[c * F + i] = (float)acc;
  }
}

// gbm_evolve (pathcube.rs:146-187): one thread per (path, factor), log-space FP64, f32 output.
__global__ void gbm_evolve_kernel(const double* __restrict__ s0, const double* __restrict__ vols, double rate,
                                  const double* __restrict__ q, int F, double dt, double sqrt_dt,
                                  const float* __restrict__ block, uint64_t paths, uint64_t times,
                                  float* __restrict__ out) {
  const uint64_t t = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= paths * (uint64_t)F) return;
  const uint64_t p = t / F;
  const int f = (int)(t % F);
  double log_s = log(s0[f]);
  const double drift = (rate - q[f] - 0.5 * vols[f] * vols[f]) * dt;
  const double diffusion = vols[f] * sqrt_dt;
  for (uint64_t i = 0; i < times; ++i) {
    const uint64_t at = (p * times + i) * F + f;
    log_s += drift + diffusion * (double)block[at];
    out[at] = (float)exp(log_s);
  }
}

// Scratch for the engine-less entry points: plain device allocations freed on exit.
struct TempWorkspace : Workspace {
  DevBuf bufs[WS_NSLOTS];
  TempWorkspace() { sm_count = device_sm_count(); }
  void* device(int slot, size_t bytes) override {
    bufs[slot].ensure(bytes);
    return bufs[slot].ptr;
  }
  void* host(size_t) override { raise(RG_ERR_INVALID_ARGUMENT, "no host sums here"); }
};

}  // namespace

}  // namespace rg

using namespace rg;

extern "C" int32_t rg_chacha8_normals(uint64_t seed, uint64_t first, uint64_t count, double* out) {
  RG_TRY({
    int32_t g = rg_guard_device();
    if (g) return g;
    if (!out && count) raise(RG_ERR_INVALID_ARGUMENT, "null output");
    if (count > (uint64_t(1) << 31) || first > (uint64_t(1) << 40))
      raise(RG_ERR_INVALID_ARGUMENT, "at most 2^31 normals per call");
    TempWorkspace W;
    double* d = static_cast<double*>(W.device(WS_MCZ, sizeof(double) * (count ? count : 1)));
    mc_normals(seed, first, count, d, W);
    if (count) cuda_check(cudaMemcpy(out, d, sizeof(double) * count, cudaMemcpyDeviceToHost), "D2H normals");
  })
}

extern "C" int32_t rg_generate_correlated_block(uint64_t seed, int64_t paths, int64_t times, int32_t factors,
                                                const double* chol, float* out) {
  RG_TRY({
    int32_t g = rg_guard_device();
    if (g) return g;
    if (paths < 0 || times < 0 || factors < 1 || factors > RG_BOOK_MAX_UNIVERSE || !chol || (!out && paths && times))
      raise(RG_ERR_SHAPE_MISMATCH, "paths and times must be non-negative, 1..32 factors, non-null buffers");
    const uint64_t cells = (uint64_t)paths * (uint64_t)times, n = cells * (uint64_t)factors;
    if (n == 0) return RG_OK;
    if (n > (uint64_t(1) << 31)) raise(RG_ERR_INVALID_ARGUMENT, "at most 2^31 normals per block");
    TempWorkspace W;
    double* z = static_cast<double*>(W.device(WS_MCZ, sizeof(double) * n));
    mc_normals(seed, 0, n, z, W);
    DevBuf dl, dout;
    dl.ensure(sizeof(double) * factors * factors);
    dout.ensure(sizeof(float) * n);
    cuda_check(cudaMemcpy(dl.ptr, chol, sizeof(double) * factors * factors, cudaMemcpyHostToDevice), "H2D");
    correlate_block_kernel<<<(unsigned)((cells + 127) / 128), 128>>>(z, static_cast<double*>(dl.ptr), factors, cells,
                                                                    static_cast<float*>(dout.ptr));
    cuda_check(cudaGetLastError(), "correlate_block_kernel launch");
    cuda_check(cudaMemcpy(out, dout.ptr, sizeof(float) * n, cudaMemcpyDeviceToHost), "D2H block");
  })
}

extern "C" int32_t rg_gbm_evolve(const double* s0, const double* vols, double rate, const double* dividend_yields,
                                 int32_t factors, double dt, const float* block, int64_t paths, int64_t times,
                                 float* out) {
  RG_TRY({
    int32_t g = rg_guard_device();
    if (g) return g;
    if (factors < 1 || !s0 || !vols || !dividend_yields)
      raise(RG_ERR_SHAPE_MISMATCH, "s0, vols and dividend_yields must have equal length");
    if (paths < 0 || times < 0 || ((paths && times) && (!block || !out)))
      raise(RG_ERR_SHAPE_MISMATCH, "Brownian block factor count must match the spot count");
    const uint64_t n = (uint64_t)paths * (uint64_t)times * (uint64_t)factors;
    if (n == 0) return RG_OK;
    DevBuf ds, dv, dq, db, dout;
    ds.ensure(sizeof(double) * factors);
    dv.ensure(sizeof(double) * factors);
    dq.ensure(sizeof(double) * factors);
    db.ensure(sizeof(float) * n);
    dout.ensure(sizeof(float) * n);
    cuda_check(cudaMemcpy(ds.ptr, s0, sizeof(double) * factors, cudaMemcpyHostToDevice), "H2D");
    cuda_check(cudaMemcpy(dv.ptr, vols, sizeof(double) * factors, cudaMemcpyHostToDevice), "H2D");
    cuda_check(cudaMemcpy(dq.ptr, dividend_yields, sizeof(double) * factors, cudaMemcpyHostToDevice), "H2D");
    cuda_check(cudaMemcpy(db.ptr, block, sizeof(float) * n, cudaMemcpyHostToDevice), "H2D");
    const uint64_t threads = (uint64_t)paths * factors;
    gbm_evolve_kernel<<<(unsigned)((threads + 127) / 128), 128>>>(
        static_cast<double*>(ds.ptr), static_cast<double*>(dv.ptr), rate, static_cast<double*>(dq.ptr), factors, dt,
        std::sqrt(dt), static_cast<float*>(db.ptr), (uint64_t)paths, (uint64_t)times, static_cast<float*>(dout.ptr));
    cuda_check(cudaGetLastError(), "gbm_evolve_kernel launch");
    cuda_check(cudaMemcpy(out, dout.ptr, sizeof(float) * n, cudaMemcpyDeviceToHost), "D2H cube");
  })
}
