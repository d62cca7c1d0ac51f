// backend.cu — the final fixed-order reduction and the drop-ins for the reference's `gpu`
// backend (crates/riga-engine/src/gpu.rs): worst_of, lv_terminal_spots and the resident objects.
#include <cstring>
#include <mutex>
#include <new>

#include "rg_internal.h"

namespace rg {

// partial[rows][S][RG_ACC] -> out[S][RG_ACC] in two fixed-order passes, so that the FP64 adds
// spread over every SM (GB300's FP64 pipe is narrow; one CTA per scenario kept 16 SMs busy for
// about 1 ms on 32,768 rows).  Pass 1: CTA (s, g) sums rows [g·kReduceRows, (g+1)·kReduceRows) of
// scenario s — thread i adds rows i, i + 256, ... of the range in order with Neumaier
// compensation, all RG_ACC quantities of a row at once (one 128-byte line), then a pairwise tree
// over the threads in shared memory — into group row g.  Pass 2: the same over the group rows.
// The order depends only on the row count, so repeated launches — and every launch shape of the
// kernels that wrote the rows — give the same bits.
constexpr int kReduceRows = 512;

__global__ void __launch_bounds__(256) reduce_kernel(const double* __restrict__ partial, int rows, int per_cta,
                                                     int S, double* __restrict__ out) {
  __shared__ double sh[RG_ACC][256];
  const int s = blockIdx.x, g = blockIdx.y, tid = threadIdx.x;
  const int r0 = g * per_cta, r1 = min(rows, r0 + per_cta);
  double sum[RG_ACC], comp[RG_ACC];
#pragma unroll
  for (int k = 0; k < RG_ACC; ++k) sum[k] = comp[k] = 0.0;
  for (int b = r0 + tid; b < r1; b += blockDim.x) {
    const double2* row = reinterpret_cast<const double2*>(partial + ((size_t)b * S + s) * RG_ACC);
#pragma unroll
    for (int k2 = 0; k2 < RG_ACC / 2; ++k2) {
      const double2 v2 = __ldg(row + k2);
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        const int k = 2 * k2 + h;
        const double v = h ? v2.y : v2.x;
        const double t = sum[k] + v;
        comp[k] += fabs(sum[k]) >= fabs(v) ? (sum[k] - t) + v : (v - t) + sum[k];
        sum[k] = t;
      }
    }
  }
#pragma unroll
  for (int k = 0; k < RG_ACC; ++k) sh[k][tid] = sum[k] + comp[k];
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if (tid < w)
#pragma unroll
      for (int k = 0; k < RG_ACC; ++k) sh[k][tid] += sh[k][tid + w];
    __syncthreads();
  }
  if (tid < RG_ACC) out[((size_t)g * S + s) * RG_ACC + tid] = sh[tid][0];
}

int reduce_groups(int rows) { return rows > kReduceRows ? (rows + kReduceRows - 1) / kReduceRows : 0; }

void launch_reduce(const double* partial, int rows, int S, double* out, cudaStream_t st) {
  const int G = reduce_groups(rows);
  if (G == 0) {
    reduce_kernel<<<dim3(S, 1), 256, 0, st>>>(partial, rows, rows, S, out);
  } else {
    double* groups = out + (size_t)S * RG_ACC;  // the caller's reduce_scratch_doubles beyond out[S][RG_ACC]
    reduce_kernel<<<dim3(S, G), 256, 0, st>>>(partial, rows, kReduceRows, S, groups);
    cuda_check(cudaGetLastError(), "reduce_kernel launch");
    reduce_kernel<<<dim3(S, 1), 256, 0, st>>>(groups, G, G, S, out);
  }
  cuda_check(cudaGetLastError(), "reduce_kernel launch");
}

size_t reduce_scratch_doubles(int rows, int S) { return (size_t)reduce_groups(rows) * S * RG_ACC; }

// ------------------------------------------------------------------ worst_of ------------------
// o = min(a, b) elementwise (gpu.rs:28-31); float4 loads for the aligned body.
__global__ void worst_of_kernel(const float* __restrict__ a, const float* __restrict__ b, float* __restrict__ o,
                                int64_t n) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  const int64_t n4 = n / 4;
  const float4* a4 = reinterpret_cast<const float4*>(a);
  const float4* b4 = reinterpret_cast<const float4*>(b);
  float4* o4 = reinterpret_cast<float4*>(o);
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n4; i += stride) {
    float4 x = __ldg(a4 + i), y = __ldg(b4 + i);
    o4[i] = make_float4(x.x < y.x ? x.x : y.x, x.y < y.y ? x.y : y.y, x.z < y.z ? x.z : y.z,
                        x.w < y.w ? x.w : y.w);
  }
  for (int64_t i = n4 * 4 + (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride)
    o[i] = a[i] < b[i] ? a[i] : b[i];
}

static void launch_worst_of(const float* a, const float* b, float* o, int64_t n, cudaStream_t st) {
  int64_t blocks = (n / 4 + 255) / 256;
  if (blocks < 1) blocks = 1;
  if (blocks > 152 * 8) blocks = 152 * 8;
  worst_of_kernel<<<(int)blocks, 256, 0, st>>>(a, b, o, n);
  cuda_check(cudaGetLastError(), "worst_of_kernel launch");
}

// ------------------------------------------------------------------ lv_propagate -------------
// Log-space FP32 local-vol Euler for two factors with first-autocall detection, the function of
// the reference's lv_propagate (gpu.rs:37-75): sigma is linear in log-spot on a uniform axis,
// ls += (r - q - sigma^2/2) dt + sigma sqrt(dt) n, KO at the first step where both
// exp(ls_f) / ref_f >= barrier.  The [path, step, 2] normals are staged through shared memory in
// tiles of LV_TS steps with warp-contiguous loads, so HBM reads are coalesced although each path's
// row is contiguous only along time.
#define LV_PATHS 128
#define LV_TS 32

struct LvArgs {
  const float* normals;
  const float* rows;
  const float* ls_axis;
  const float* s0;
  float* out;
  int32_t* ko_out;
  float ref0, ref1, ko_bar;
  int64_t paths, steps;
  int gx;
  float dt, rate, q0, q1;
};

__global__ void __launch_bounds__(LV_PATHS) lv_propagate_kernel(LvArgs A) {
  __shared__ float2 nz[LV_PATHS][LV_TS + 1];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int64_t p0 = (int64_t)blockIdx.x * LV_PATHS;
  const int64_t p = p0 + tid;
  const int gx = A.gx;
  float ls0 = logf(A.s0[0]), ls1 = logf(A.s0[1]);
  const float sq = sqrtf(A.dt);
  const float lo0 = A.ls_axis[0], inv0 = 1.0f / (A.ls_axis[gx - 1] - lo0);
  const float lo1 = A.ls_axis[gx], inv1 = 1.0f / (A.ls_axis[2 * gx - 1] - lo1);
  const float span = (float)(gx - 1);
  int ko = -1;
  const float2* n2 = reinterpret_cast<const float2*>(A.normals);
  for (int64_t t0 = 0; t0 < A.steps; t0 += LV_TS) {
    const int tn = (int)(A.steps - t0 < LV_TS ? A.steps - t0 : LV_TS);
    __syncthreads();
    // each warp copies whole path rows of the tile: lane j loads step t0 + j of the row
    for (int r = warp; r < LV_PATHS; r += LV_PATHS / 32) {
      const int64_t pr = p0 + r;
      if (pr < A.paths && lane < tn) nz[r][lane] = __ldg(n2 + pr * A.steps + t0 + lane);
    }
    __syncthreads();
    if (p < A.paths) {
      for (int j = 0; j < tn; ++j) {
        const int64_t s = t0 + j;
        float x0 = (ls0 - lo0) * inv0 * span;
        x0 = fminf(fmaxf(x0, 0.0f), span);
        int j0 = min((int)x0, gx - 2);
        float w0 = x0 - (float)j0;
        const float* r0 = A.rows + s * gx;
        float sig0 = __ldg(r0 + j0) * (1.0f - w0) + __ldg(r0 + j0 + 1) * w0;
        float x1 = (ls1 - lo1) * inv1 * span;
        x1 = fminf(fmaxf(x1, 0.0f), span);
        int j1 = min((int)x1, gx - 2);
        float w1 = x1 - (float)j1;
        const float* r1 = A.rows + (A.steps + s) * gx;
        float sig1 = __ldg(r1 + j1) * (1.0f - w1) + __ldg(r1 + j1 + 1) * w1;
        const float2 z = nz[tid][j];
        ls0 += (A.rate - A.q0 - 0.5f * sig0 * sig0) * A.dt + sig0 * sq * z.x;
        ls1 += (A.rate - A.q1 - 0.5f * sig1 * sig1) * A.dt + sig1 * sq * z.y;
        if (ko < 0 && expf(ls0) / A.ref0 >= A.ko_bar && expf(ls1) / A.ref1 >= A.ko_bar) ko = (int)s;
      }
    }
  }
  if (p < A.paths) {
    A.out[p * 2] = expf(ls0);
    A.out[p * 2 + 1] = expf(ls1);
    A.ko_out[p] = ko;
  }
}

static void launch_lv(const LvArgs& A, cudaStream_t st) {
  int64_t blocks = (A.paths + LV_PATHS - 1) / LV_PATHS;
  if (blocks < 1) return;
  lv_propagate_kernel<<<(unsigned)blocks, LV_PATHS, 0, st>>>(A);
  cuda_check(cudaGetLastError(), "lv_propagate_kernel launch");
}

}  // namespace rg

// ==================================================================== C ABI ===================
using namespace rg;

namespace {
template <class T>
T* dev_copy(const T* host, size_t count, cudaStream_t st) {
  T* d = nullptr;
  cuda_check(cudaMalloc(&d, sizeof(T) * (count ? count : 1)), "cudaMalloc");
  if (count) cuda_check(cudaMemcpyAsync(d, host, sizeof(T) * count, cudaMemcpyHostToDevice, st), "H2D");
  return d;
}
template <class T>
T* dev_alloc(size_t count) {
  T* d = nullptr;
  cuda_check(cudaMalloc(&d, sizeof(T) * (count ? count : 1)), "cudaMalloc");
  return d;
}
}  // namespace

extern "C" int32_t rg_worst_of(const float* a, const float* b, float* out, int64_t n) {
  RG_TRY({
    if (n < 0 || (n > 0 && (!a || !b || !out))) raise(RG_ERR_INVALID_ARGUMENT, "null buffer or negative length");
    int32_t g = rg_guard_device();
    if (g) raise(g, "no usable CUDA device");
    if (n == 0) return RG_OK;
    cudaStream_t st = 0;
    float* da = dev_copy(a, (size_t)n, st);
    float* db = dev_copy(b, (size_t)n, st);
    float* dout = dev_alloc<float>((size_t)n);
    launch_worst_of(da, db, dout, n, st);
    cuda_check(cudaMemcpyAsync(out, dout, sizeof(float) * n, cudaMemcpyDeviceToHost, st), "D2H");
    cuda_check(cudaStreamSynchronize(st), "worst_of sync");
    cudaFree(da);
    cudaFree(db);
    cudaFree(dout);
  })
}

static void check_lv_args(const float* normals, const float* rows, const float* ls_axis, int64_t gx,
                          int64_t paths, int64_t steps) {
  if (!normals || !rows || !ls_axis) raise(RG_ERR_INVALID_ARGUMENT, "null buffer");
  if (gx < 2) raise(RG_ERR_SHAPE_MISMATCH, "the local-vol grid needs at least two points");
  if (paths < 0 || steps < 1) raise(RG_ERR_SHAPE_MISMATCH, "paths must be >= 0 and steps >= 1");
}

extern "C" int32_t rg_lv_terminal_spots(const float* normals, const float* rows, const float* ls_axis,
                                        int64_t gx, const float* s0, const float* references,
                                        float call_barrier, int64_t paths, int64_t steps, float dt,
                                        float rate, const float* dividends, float* out_terminal,
                                        int32_t* out_ko) {
  RG_TRY({
    check_lv_args(normals, rows, ls_axis, gx, paths, steps);
    if (!s0 || !references || !dividends || !out_terminal || !out_ko)
      raise(RG_ERR_INVALID_ARGUMENT, "null buffer");
    int32_t g = rg_guard_device();
    if (g) raise(g, "no usable CUDA device");
    if (paths == 0) return RG_OK;
    cudaStream_t st = 0;
    LvArgs A{};
    float* dn = dev_copy(normals, (size_t)paths * steps * 2, st);
    float* dr = dev_copy(rows, (size_t)2 * steps * gx, st);
    float* dl = dev_copy(ls_axis, (size_t)2 * gx, st);
    float* ds = dev_copy(s0, 2, st);
    float* dout = dev_alloc<float>((size_t)paths * 2);
    int32_t* dko = dev_alloc<int32_t>((size_t)paths);
    A.normals = dn; A.rows = dr; A.ls_axis = dl; A.s0 = ds; A.out = dout; A.ko_out = dko;
    A.ref0 = references[0]; A.ref1 = references[1]; A.ko_bar = call_barrier;
    A.paths = paths; A.steps = steps; A.gx = (int)gx;
    A.dt = dt; A.rate = rate; A.q0 = dividends[0]; A.q1 = dividends[1];
    // s0 is read by the kernel from device memory; copy it in before launch
    launch_lv(A, st);
    cuda_check(cudaMemcpyAsync(out_terminal, dout, sizeof(float) * paths * 2, cudaMemcpyDeviceToHost, st), "D2H");
    cuda_check(cudaMemcpyAsync(out_ko, dko, sizeof(int32_t) * paths, cudaMemcpyDeviceToHost, st), "D2H");
    cuda_check(cudaStreamSynchronize(st), "lv sync");
    cudaFree(dn); cudaFree(dr); cudaFree(dl); cudaFree(ds); cudaFree(dout); cudaFree(dko);
  })
}

// ResidentLv (gpu.rs:409-488): scenario-independent buffers stay on the device; each run ships
// only the scenario's spots.  The object owns one stream; run enqueues, download blocks.
struct rg_resident_lv {
  cudaStream_t st = nullptr;
  float *normals = nullptr, *rows = nullptr, *ls = nullptr, *s0 = nullptr, *out = nullptr;
  int32_t* ko = nullptr;
  int64_t paths = 0, steps = 0, gx = 0;
  float dt = 0;
};

extern "C" int32_t rg_resident_lv_create(const float* normals, const float* rows, const float* ls_axis,
                                         int64_t gx, int64_t paths, int64_t steps, float dt,
                                         rg_resident_lv** out) {
  RG_TRY({
    if (!out) raise(RG_ERR_INVALID_ARGUMENT, "null output handle");
    *out = nullptr;
    check_lv_args(normals, rows, ls_axis, gx, paths, steps);
    int32_t g = rg_guard_device();
    if (g) raise(g, "no usable CUDA device");
    rg_resident_lv* r = new rg_resident_lv();
    try {
      cuda_check(cudaStreamCreateWithFlags(&r->st, cudaStreamNonBlocking), "stream");
      r->normals = dev_copy(normals, (size_t)paths * steps * 2, r->st);
      r->rows = dev_copy(rows, (size_t)2 * steps * gx, r->st);
      r->ls = dev_copy(ls_axis, (size_t)2 * gx, r->st);
      r->s0 = dev_alloc<float>(2);
      r->out = dev_alloc<float>((size_t)paths * 2 + 1);
      r->ko = dev_alloc<int32_t>((size_t)paths + 1);
      r->paths = paths; r->steps = steps; r->gx = gx; r->dt = dt;
      cuda_check(cudaStreamSynchronize(r->st), "resident upload");
    } catch (...) {
      rg_resident_lv_destroy(r);
      throw;
    }
    *out = r;
  })
}

extern "C" int32_t rg_resident_lv_run(rg_resident_lv* r, const float* s0, const float* references,
                                      float call_barrier, float rate, const float* dividends) {
  RG_TRY({
    if (!r || !s0 || !references || !dividends) raise(RG_ERR_INVALID_ARGUMENT, "null argument");
    cuda_check(cudaMemcpyAsync(r->s0, s0, sizeof(float) * 2, cudaMemcpyHostToDevice, r->st), "H2D s0");
    LvArgs A{};
    A.normals = r->normals; A.rows = r->rows; A.ls_axis = r->ls; A.s0 = r->s0; A.out = r->out;
    A.ko_out = r->ko; A.ref0 = references[0]; A.ref1 = references[1]; A.ko_bar = call_barrier;
    A.paths = r->paths; A.steps = r->steps; A.gx = (int)r->gx; A.dt = r->dt; A.rate = rate;
    A.q0 = dividends[0]; A.q1 = dividends[1];
    launch_lv(A, r->st);
  })
}

extern "C" int32_t rg_resident_lv_download(rg_resident_lv* r, float* out_terminal, int32_t* out_ko) {
  RG_TRY({
    if (!r || !out_terminal || !out_ko) raise(RG_ERR_INVALID_ARGUMENT, "null argument");
    if (r->paths) {
      cuda_check(cudaMemcpyAsync(out_terminal, r->out, sizeof(float) * r->paths * 2, cudaMemcpyDeviceToHost, r->st), "D2H");
      cuda_check(cudaMemcpyAsync(out_ko, r->ko, sizeof(int32_t) * r->paths, cudaMemcpyDeviceToHost, r->st), "D2H");
    }
    cuda_check(cudaStreamSynchronize(r->st), "resident download");
  })
}

extern "C" int32_t rg_resident_lv_synchronize(rg_resident_lv* r) {
  RG_TRY({
    if (!r) raise(RG_ERR_INVALID_ARGUMENT, "null handle");
    cuda_check(cudaStreamSynchronize(r->st), "resident synchronize");
  })
}

extern "C" void rg_resident_lv_destroy(rg_resident_lv* r) {
  if (!r) return;
  if (r->st) cudaStreamSynchronize(r->st);
  cudaFree(r->normals); cudaFree(r->rows); cudaFree(r->ls); cudaFree(r->s0); cudaFree(r->out); cudaFree(r->ko);
  if (r->st) cudaStreamDestroy(r->st);
  delete r;
}

// ResidentWorstOf (gpu.rs:362-405)
struct rg_resident_worst_of {
  cudaStream_t st = nullptr;
  float *a = nullptr, *b = nullptr, *out = nullptr;
  int64_t n = 0;
};

extern "C" int32_t rg_resident_worst_of_create(const float* a, const float* b, int64_t n,
                                               rg_resident_worst_of** out) {
  RG_TRY({
    if (!out) raise(RG_ERR_INVALID_ARGUMENT, "null output handle");
    *out = nullptr;
    if (n < 0 || (n > 0 && (!a || !b))) raise(RG_ERR_INVALID_ARGUMENT, "null buffer or negative length");
    int32_t g = rg_guard_device();
    if (g) raise(g, "no usable CUDA device");
    rg_resident_worst_of* w = new rg_resident_worst_of();
    try {
      cuda_check(cudaStreamCreateWithFlags(&w->st, cudaStreamNonBlocking), "stream");
      w->a = dev_copy(a, (size_t)n, w->st);
      w->b = dev_copy(b, (size_t)n, w->st);
      w->out = dev_alloc<float>((size_t)n);
      w->n = n;
      cuda_check(cudaStreamSynchronize(w->st), "resident upload");
    } catch (...) {
      rg_resident_worst_of_destroy(w);
      throw;
    }
    *out = w;
  })
}

extern "C" int32_t rg_resident_worst_of_reduce(rg_resident_worst_of* w) {
  RG_TRY({
    if (!w) raise(RG_ERR_INVALID_ARGUMENT, "null handle");
    if (w->n) launch_worst_of(w->a, w->b, w->out, w->n, w->st);
  })
}

extern "C" int32_t rg_resident_worst_of_download(rg_resident_worst_of* w, float* out) {
  RG_TRY({
    if (!w || (w->n && !out)) raise(RG_ERR_INVALID_ARGUMENT, "null argument");
    if (w->n) cuda_check(cudaMemcpyAsync(out, w->out, sizeof(float) * w->n, cudaMemcpyDeviceToHost, w->st), "D2H");
    cuda_check(cudaStreamSynchronize(w->st), "resident download");
  })
}

extern "C" int32_t rg_resident_worst_of_synchronize(rg_resident_worst_of* w) {
  RG_TRY({
    if (!w) raise(RG_ERR_INVALID_ARGUMENT, "null handle");
    cuda_check(cudaStreamSynchronize(w->st), "resident synchronize");
  })
}

extern "C" void rg_resident_worst_of_destroy(rg_resident_worst_of* w) {
  if (!w) return;
  if (w->st) cudaStreamSynchronize(w->st);
  cudaFree(w->a); cudaFree(w->b); cudaFree(w->out);
  if (w->st) cudaStreamDestroy(w->st);
  delete w;
}
