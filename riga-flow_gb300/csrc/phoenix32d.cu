// phoenix32d.cu — the FP32 kernel for single-scenario launches: one thread per (path, scenario),
// everything in registers, no shared-memory time tiles and no CTA barriers.
//
// The tiled kernel (phoenix32.cu) stages a tile's normals and Brownian increments in shared
// memory so that the scenarios of a path share one generation; with one scenario there is nothing
// to share and the staging only costs occupancy.  (Measured on the 3-asset local-vol trade at 2^20
// paths: 17.5 ms here against 24.4 ms for the tiled kernel on four padded scenario slots; the
// tiled kernel wins with two or more scenarios, and below about 2^18 paths, where one path per
// thread leaves too few warps to hide the per-step latency.)  Here a warp walks 32 consecutive
// paths of one scenario through time:
//   * Sobol points from consumption-order tables staged for the launch (host_prep.cu,
//     direct_sobol_tables): the warp's 32 points lie in at most two aligned 32-point blocks, and
//     Gray codes are linear over XOR, so a point is the block's high-bit term X(gray(a)) — one
//     coalesced row of transposed directions per set bit of gray(a), for a batch of the next
//     32 / N nodes' dimensions at once, kept in shared memory — XOR the lane's low-bit term, one
//     coalesced 128-byte row per dimension; without the tables (another offset within a block),
//     by warp cooperation: x(n) for the warp's first point as a shuffle reduction over the set bits
//     of its Gray code, and the Gray recurrence x(n) = x(n-1) ^ v[ctz(n)] as an XOR scan over the
//     lanes;
//   * the digital shift (or Owen scramble) and the FP32 inverse normal of rg_common.cuh;
//   * the streamed Brownian bridge per factor with its anchor stack in shared memory, laid out
//     [depth][factor][thread] so that a warp's accesses (the depth is warp-uniform) hit 32 banks;
//   * the correlation with the scenario's Cholesky factor, the log-space GBM / Dupire step and the
//     Phoenix state machine.
// Every operation of the per-path arithmetic is the one phoenix32.cu performs, in the same order,
// so a path's FP32 payoff values are identical in both kernels.  The 32 paths of a warp are one
// chunk of the sums, added by the same FP32 shuffle butterfly and written as FP64 to
// partial[chunk][scenario] as the tiled kernel writes them, so both kernels — and every launch
// shape of either — give the same sums.
#include "p32_path.cuh"
#include "rg_internal.h"

namespace rg {

#define P32D_THREADS 256
#define P32D_WARPS (P32D_THREADS / 32)

// Up to three assets the state fits 64 registers (four CTAs per SM, measured 2.3% faster on three
// assets); four or five assets keep 80 registers at three CTAs per SM (four spilled, 12% slower).
template <int N, bool LV, bool REC>
__global__ void __launch_bounds__(P32D_THREADS, N <= 3 ? 4 : 3) phoenix32d_kernel(
    DevTrade tr, DevTables tb, const DevScenario* __restrict__ scen,
    const DevScen32* __restrict__ scen32, int S, float ln_ko, float ln_cb, float ln_ki, uint64_t path0,
    uint64_t npaths, double* __restrict__ partial, int32_t* __restrict__ ko_steps,
    rg_path_record* __restrict__ records) {
  __shared__ float4 s_lv[32 * RG_NMAX];
  // per warp: the high-bit Sobol terms of a batch of consumption indices q (q0 + l for lane l):
  // [0, 32) for lanes whose point lies in the warp's first 32-point block, [33, 65) for the next
  __shared__ uint32_t s_hi[P32D_WARPS][66];
  extern __shared__ float s_stk[];  // [stack depth][N][P32D_THREADS]
  const int tid = threadIdx.x, lane = tid & 31, wib = tid >> 5;
  const int T = (int)tr.steps;
  const int gx = tr.gx;
  const float gxm1 = (float)(gx - 1);
  const float nhdt = tr.neg_half_dt_f;
  // the grid holds a multiple of S warps: warp w serves scenario w % S, path groups w / S + k·(W / S)
  const int gw = blockIdx.x * P32D_WARPS + wib;
  const int nw = gridDim.x * P32D_WARPS;
  const int s = gw % S;
  for (int i = tid; i < S * N; i += blockDim.x) {
    const DevScen32& s3 = scen32[i / N];
    const int f = i % N;
    const float inv_gxm1 = 1.0f / (float)(tr.gx - 1);
    s_lv[i] = make_float4(s3.a_u[f] * inv_gxm1, s3.inv_h[f] * inv_gxm1,
                          __int_as_float((int)((uint32_t)s3.surf_off[f] - 0x4B000000u)), s3.x0[f]);
  }
  float Lf[N * (N + 1) / 2], mu[N], sig[N];
  {
    const DevScen32& s3 = scen32[s];
    int q = 0;
#pragma unroll
    for (int a = 0; a < N; ++a)
#pragma unroll
      for (int b = 0; b <= a; ++b) Lf[q++] = s3.L[a * N + b];
#pragma unroll
    for (int f = 0; f < N; ++f) {
      mu[f] = s3.mu_dt[f];
      sig[f] = s3.sig[f];
    }
  }
  const float4* lvc = s_lv + s * N;
  __syncthreads();

  const uint64_t groups = (npaths + 31) / 32;
  // Sobol points from the staged consumption-order tables when they were built for this launch's
  // offset within a 32-point block (else the warp cooperation of rg_warp_sobol)
  const bool lut = tr.vr == RG_VR_SOBOL && tb.sob_lut != nullptr && (int32_t)((path0 + 1) & 31) == tb.sob_lut_o;
  const bool upper = (uint32_t)tb.sob_lut_o + (uint32_t)lane >= 32u;  // point in the next 32-block
  constexpr int kNb = 32 / N;  // nodes per batch of high-bit terms
  for (uint64_t grp = (uint64_t)(gw / S); grp < groups; grp += (uint64_t)(nw / S)) {
    const uint64_t gi = grp * 32 + lane;
    const bool ok = gi < npaths;
    const uint64_t n1 = path0 + grp * 32 + 1;  // Sobol point of the warp's first path
    const uint32_t ga = (uint32_t)((n1 & ~(uint64_t)31) ^ ((n1 & ~(uint64_t)31) >> 1));  // gray(a)
    const int cw = __ffsll((long long)((n1 >> 5) + 1)) - 1 + 5;  // a / 32 + 1: its lowest set bit + 5
    int cb = -kNb;  // first node of the batch in s_hi
    // the lanes' low-bit terms of the next node, loaded a node ahead so that their latency
    // overlaps the current step
    uint32_t lnext[N];
#pragma unroll
    for (int f = 0; f < N; ++f) lnext[f] = lut ? __ldg(tb.sob_lut + (size_t)f * 32 + lane) : 0u;
    float x[N], wcur[N];
    float* const stk = s_stk + tid;  // entry (depth d, factor f) at stk[(d * N + f) * P32D_THREADS]
#pragma unroll
    for (int f = 0; f < N; ++f) {
      x[f] = lvc[f].w;
      wcur[f] = 0.0f;
    }
    int sp = 0;
    P32Phoenix ph;
    float worst = 0.0f;
    for (int t = 0; t < T; ++t) {
      // bridge nodes consumed at this step: normals, then the streamed bridge (qmc.rs:158-191)
      const int c0 = __ldg(tb.node_off + t), c1 = __ldg(tb.node_off + t + 1);
      for (int c = c0; c < c1; ++c) {
        const float cf = __ldg(tb.node_cf + c);
        float zf[N];
        if (lut) {
          if (c >= cb + kNb) {
            // the high-bit terms X(gray(a)) of q = c·N .. (c + kNb)·N - 1, lane l holding q0 + l:
            // one coalesced row of transposed directions per set bit of gray(a)
            cb = c;
            __syncwarp();  // every lane has read the previous batch
            const int q = c * N + lane;
            if (lane < kNb * N && q < tb.sob_nq) {
              uint32_t h = 0;
              for (uint32_t g = ga; g; g &= g - 1u) h ^= __ldg(tb.sob_t + (size_t)(__ffs(g) - 1) * tb.sob_nq + q);
              s_hi[wib][lane] = h;
              s_hi[wib][33 + lane] = h ^ __ldg(tb.sob_t + (size_t)cw * tb.sob_nq + q);
            }
            __syncwarp();
          }
          const int hb = (c - cb) * N + (upper ? 33 : 0);
          uint32_t lcur[N];
          const bool more = (c + 1) * N < tb.sob_nq;
#pragma unroll
          for (int f = 0; f < N; ++f) {
            lcur[f] = lnext[f];
            if (more) lnext[f] = __ldg(tb.sob_lut + ((size_t)(c + 1) * N + f) * 32 + lane);
          }
#pragma unroll
          for (int f = 0; f < N; ++f) {
            const uint32_t xs = s_hi[wib][hb + f] ^ lcur[f];
            zf[f] = rg_probit32(tr.scrambler == RG_SCRAMBLE_DIGITAL_SHIFT
                                    ? xs
                                    : rg_owen(xs, (uint64_t)__ldg(tb.node_k + c) * N + f, tr.seed));
          }
        } else if (tr.vr == RG_VR_SOBOL) {
#pragma unroll
          for (int f = 0; f < N; ++f) {
            const uint32_t xs = rg_warp_sobol(tb.sobol + 32 * (size_t)__ldg(tb.nf_row + c * N + f), n1, lane);
            zf[f] = rg_probit32(tr.scrambler == RG_SCRAMBLE_DIGITAL_SHIFT
                                    ? xs ^ __ldg(tb.nf_shift + c * N + f)
                                    : rg_owen(xs, (uint64_t)__ldg(tb.node_k + c) * N + f, tr.seed));
          }
        } else {
#pragma unroll
          for (int f = 0; f < N; ++f)
            zf[f] = rg_qmc_normal32(tr, tb, path0 + gi, (uint64_t)__ldg(tb.node_k + c) * N + f);
        }
#pragma unroll
        for (int f = 0; f < N; ++f)
          stk[(sp * N + f) * P32D_THREADS] =
              c == 0 ? zf[f] * cf : fmaf(zf[f], cf, 0.5f * (wcur[f] + stk[((sp - 1) * N + f) * P32D_THREADS]));
        ++sp;
      }
      --sp;
      float d[N], y[N];
#pragma unroll
      for (int f = 0; f < N; ++f) {
        const float wn = stk[(sp * N + f) * P32D_THREADS];
        d[f] = wn - wcur[f];
        wcur[f] = wn;
      }
      const int tg = t * gx;
      int q = 0;
#pragma unroll
      for (int a = 0; a < N; ++a) {
        float acc_y = 0.0f;
#pragma unroll
        for (int b = 0; b <= a; ++b) acc_y = fmaf(Lf[q++], d[b], acc_y);
        y[a] = acc_y;
      }
      float wmin = INFINITY;
#pragma unroll
      for (int f = 0; f < N; ++f) {
        float sg;
        if (LV) {
          // the saturating grid lookup of the tiled kernel: u01 clamped by the FMA's saturation, the
          // grid index from a round-down FMA's bit pattern (bias folded into c4.z), one gather of
          // the cell's line (c, d) and sigma = c + u01·d
          const float4 c4 = lvc[f];
          const float u01 = __saturatef(fmaf(x[f], c4.y, c4.x));
          const float fl = __fmaf_rd(u01, gxm1, 8388608.0f);
          const uint32_t idx = (uint32_t)__float_as_int(c4.z) + (uint32_t)tg + (uint32_t)__float_as_int(fl);
          const float2 r = __ldg(tb.lv_rows + idx);
          sg = fmaf(u01, r.y, r.x);
        } else {
          sg = sig[f];
        }
        x[f] = fmaf(sg, fmaf(nhdt, sg, y[f]), x[f]) + mu[f];
        wmin = fminf(wmin, x[f]);
      }
      worst = wmin;
      if (ph.alive)  // Phoenix state machine (note.rs:150-218)
        p32_phoenix_step<REC>(ph, __ldg(tb.step_flags + t), t, wmin, ln_cb, ln_ko, tr, tb, tb.df_f + (size_t)s * T,
                              [&] { return __ldg(tb.step_period + t); });
    }
    // path close (note.rs:221-258)
    float out[RG_ACC];
    p32_close_path<REC>(tr, tb, s, T, ok, s == 0, path0, gi, ph.ko_step, worst, ln_ki, ph.cpv, ph.mpv,
                        ph.received, ph.qualified, ph.paid, ko_steps, records, out);
    // the same FP32 butterfly over the warp's 32 paths (one chunk) as phoenix32.cu, then lane k
    // writes the chunk's quantity k as FP64 to partial[chunk][scenario]
#pragma unroll
    for (int off = 16; off > 0; off >>= 1)
#pragma unroll
      for (int k = 0; k < RG_ACC; ++k) out[k] += __shfl_xor_sync(0xffffffffu, out[k], off);
    float mine = 0.0f;
#pragma unroll
    for (int k = 0; k < RG_ACC; ++k) mine = lane == k ? out[k] : mine;
    if (lane < RG_ACC) partial[((size_t)grp * S + s) * RG_ACC + lane] = (double)mine;
  }
}

static size_t stack_bytes(const Prepared& P) {
  return (size_t)P.stack_max * P.n * P32D_THREADS * sizeof(float);
}

template <int N, bool LV, bool REC>
static void launch_n(const Prepared& P, const DevTables& tb, const DevScenario* scen, const DevScen32* scen32,
                     uint64_t path0, uint64_t npaths, int grid, const LaunchOut& out, cudaStream_t st) {
  phoenix32d_kernel<N, LV, REC><<<grid, P32D_THREADS, stack_bytes(P), st>>>(
      P.trade, tb, scen, scen32, P.n_scen, (float)P.ln_ko, (float)P.ln_cb, (float)P.ln_ki, path0, npaths,
      out.partial, out.ko_steps, out.records);
}

template <int N, bool LV>
static const void* kernel_ptr(bool rec) {
  return rec ? reinterpret_cast<const void*>(&phoenix32d_kernel<N, LV, true>)
             : reinterpret_cast<const void*>(&phoenix32d_kernel<N, LV, false>);
}

static const void* select_kernel(int n, bool lv, bool rec) {
  switch (n) {
    case 1: return lv ? kernel_ptr<1, true>(rec) : kernel_ptr<1, false>(rec);
    case 2: return lv ? kernel_ptr<2, true>(rec) : kernel_ptr<2, false>(rec);
    case 3: return lv ? kernel_ptr<3, true>(rec) : kernel_ptr<3, false>(rec);
    case 4: return lv ? kernel_ptr<4, true>(rec) : kernel_ptr<4, false>(rec);
    case 5: return lv ? kernel_ptr<5, true>(rec) : kernel_ptr<5, false>(rec);
    default: raise(RG_ERR_INVALID_MARKET_SHAPE, "unsupported asset count");
  }
}

// Grid of the direct kernel: enough warps for every (path group, scenario) pair up to a few waves
// of resident CTAs, rounded so that the warp count is a multiple of the scenario count.
int phoenix32d_grid(const Prepared& P, uint64_t npaths, int sm_count) {
  const int S = P.n_scen;
  if (S < 1 || S > 32) raise(RG_ERR_INVALID_ARGUMENT, "1 to 32 scenarios per fused launch");
  // function attributes are process-wide: raise every instantiation's dynamic shared-memory limit
  // to the device maximum once, so concurrent engines never lower it under each other
  {
    static std::mutex mu;
    static std::vector<char> done;
    int dev = 0;
    cuda_check(cudaGetDevice(&dev), "cudaGetDevice");
    std::lock_guard<std::mutex> lock(mu);
    if ((int)done.size() <= dev) done.resize(dev + 1, 0);
    if (!done[dev]) {
      int optin = 0;
      cuda_check(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev), "smem opt-in");
      for (int n = 1; n <= RG_NMAX; ++n)
        for (int lv = 0; lv < 2; ++lv)
          for (int rec = 0; rec < 2; ++rec) {
            const void* k = select_kernel(n, lv != 0, rec != 0);
            cudaFuncAttributes fa{};
            cuda_check(cudaFuncGetAttributes(&fa, k), "phoenix32d attributes");
            cuda_check(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                            optin - (int)fa.sharedSizeBytes),
                       "phoenix32d smem attribute");
          }
      done[dev] = 1;
    }
  }
  int per_sm = 0;
  cuda_check(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, select_kernel(P.n, P.trade.has_lv != 0, false),
                                                           P32D_THREADS, stack_bytes(P)),
             "phoenix32d occupancy");
  if (per_sm < 1) raise(RG_ERR_GPU_ERROR, "phoenix32d: launch shape does not fit on an SM");
  int step = 1;  // CTAs per repeat of the scenario cycle: the smallest k with k·P32D_WARPS % S == 0
  while ((step * P32D_WARPS) % S) ++step;
  const uint64_t units = (npaths + 31) / 32 * (uint64_t)S;
  uint64_t ctas = (units + P32D_WARPS - 1) / P32D_WARPS;
  const uint64_t cap = (uint64_t)sm_count * per_sm * 4;  // up to 4 waves of resident CTAs
  if (ctas > cap) ctas = cap;
  ctas = (ctas + step - 1) / step * step;
  return (int)(ctas < 1 ? step : ctas);
}

void launch_phoenix32d(const Prepared& P, const DevTables& tb, const DevScenario* scen, const DevScen32* scen32,
                       uint64_t path0, uint64_t npaths, int grid, const LaunchOut& out, cudaStream_t st) {
  const bool lv = P.trade.has_lv != 0, rec = out.records != nullptr;
#define RG_CASE(NN)                                                                          \
  case NN:                                                                                   \
    if (lv) {                                                                                \
      if (rec) launch_n<NN, true, true>(P, tb, scen, scen32, path0, npaths, grid, out, st);  \
      else launch_n<NN, true, false>(P, tb, scen, scen32, path0, npaths, grid, out, st);     \
    } else {                                                                                 \
      if (rec) launch_n<NN, false, true>(P, tb, scen, scen32, path0, npaths, grid, out, st); \
      else launch_n<NN, false, false>(P, tb, scen, scen32, path0, npaths, grid, out, st);    \
    }                                                                                        \
    break;
  switch (P.n) {
    RG_CASE(1) RG_CASE(2) RG_CASE(3) RG_CASE(4) RG_CASE(5)
    default: raise(RG_ERR_INVALID_MARKET_SHAPE, "unsupported asset count");
  }
#undef RG_CASE
  cuda_check(cudaGetLastError(), "phoenix32d_kernel launch");
}

}  // namespace rg
