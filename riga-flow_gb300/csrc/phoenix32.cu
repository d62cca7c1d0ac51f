// phoenix32.cu — the FP32 production kernel: one fused launch prices S common-random-number
// scenarios of one trade.
//
// A CTA owns Pb consecutive paths × Sb scenario slots (Sb = S rounded up to a power of two, at least
// 4; a single scenario runs on the direct kernel of phoenix32d.cu); thread
// t serves scenario t / Pb and path t % Pb, so a warp is 32 paths of one scenario and its
// local-vol lookups all read one surface.  Time is walked in tiles of TT steps, each in three
// phases separated by CTA barriers:
//   G. generation — every thread takes (bridge node, factor, 8-path run) tasks: the Sobol integer
//      of the run's first point from its Gray code, the next seven by the Gray recurrence
//      x(n) = x(n-1) ^ v[ctz(n)] (one load each), the digital shift (or Owen scramble) and the
//      FP32 inverse normal; the standard normals of every node the tile consumes land in shared
//      memory.  The step schedule of the tile is staged next to them.
//   B. bridge — one chain per (path, factor) walks the tile's steps through the streamed
//      Brownian bridge and writes the uncorrelated increments dW[step][factor][path].
//   S. scenario stepping — every (path, scenario) thread correlates dW with its own Cholesky
//      factor (the bridge is linear, so L·bridge(z) = bridge(L·z)), steps ln(S/S0) under flat vol
//      or its scenario's Dupire surface and runs the Phoenix state machine.
// Generation is paid once per path, not once per scenario.  Path state and a path's payoff values
// are FP32; the 32 paths of a warp are summed in FP32 by a fixed shuffle butterfly, and every
// sum above that (warps in index order, tiles, blocks in the final reduce kernel) is FP64, so a
// launch of a given shape is bit-reproducible.  With 16 scenarios a CTA is 1024 threads (64 paths
// × 16 scenarios, one CTA per SM): each scenario has two warps on the same paths, which share
// its local-vol rows in L1.
#include <algorithm>
#include <map>
#include <mutex>
#include <vector>

#include "p32_path.cuh"
#include "rg_internal.h"

namespace rg {

#define GEN_CH 8  // consecutive paths per generation task (one Gray-code run)

// Byte offsets of the kernel's dynamic shared-memory regions, 16-byte aligned, and their total.
// Computed by the same function on the host (to size the launch) and in the kernel (to carve).
struct P32Layout {
  uint32_t acc, lv, flags, per, noff, ncf, wcur, stack, z, dw, total;
};

__host__ __device__ inline P32Layout p32_layout(int S, int N, int Pb, int TT, int NNmax, int stack_max,
                                                int threads) {
  P32Layout L;
  uint32_t o = 0;
  auto put = [&o](uint32_t& field, uint32_t bytes) {
    field = o;
    o += (bytes + 15u) & ~15u;
  };
  const uint32_t PbN = (uint32_t)(Pb * N);
  const int g = Pb < 32 ? Pb : 32;
  // normals of the tile's bridge nodes, one row of Pb + 4 floats per (node, factor): the padding
  // spreads a generation pass's stores (lanes stride GEN_CH·nch apart) over distinct banks
  const uint32_t zb = (uint32_t)NNmax * (uint32_t)N * (uint32_t)(Pb + 4) * 4u;
  const uint32_t rb = (uint32_t)(threads / g) * RG_ACC * 8u;  // per-tile reduction, aliases Z
  put(L.acc, (uint32_t)S * RG_ACC * 8u);
  put(L.lv, (uint32_t)(S * N) * 16u);
  put(L.flags, (uint32_t)TT * 4u);
  put(L.per, (uint32_t)TT * 4u);
  put(L.noff, (uint32_t)(TT + 1) * 4u);
  put(L.ncf, (uint32_t)NNmax * 4u);
  put(L.wcur, PbN * 4u);
  put(L.stack, (uint32_t)stack_max * PbN * 4u);
  put(L.z, zb > rb ? zb : rb);
  put(L.dw, (uint32_t)TT * PbN * 4u);
  L.total = o;
  return L;
}

template <int N, bool LV, bool REC>
__global__ void __launch_bounds__(1024, 1) phoenix32_kernel(
    DevTrade tr, DevTables tb, const DevScenario* __restrict__ scen,
    const DevScen32* __restrict__ scen32, int S, int Pb, int TT, int NNmax, int stack_max,
    float ln_ko, float ln_cb, float ln_ki, uint64_t path0, uint64_t npaths,
    double* __restrict__ partial, int32_t* __restrict__ ko_steps, rg_path_record* __restrict__ records) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int tid = threadIdx.x, lane = tid & 31;
  const int PbN = Pb * N;
  const int nch = Pb / GEN_CH;
  const int T = (int)tr.steps;
  // ---- shared-memory carve-up (the host sizes the launch from the same layout)
  const P32Layout L = p32_layout(S, N, Pb, TT, NNmax, stack_max, (int)blockDim.x);
  uint32_t dyn_bytes;
  asm("mov.u32 %0, %%dynamic_smem_size;" : "=r"(dyn_bytes));
  if (L.total > dyn_bytes) {
    // launched with less shared memory than the layout needs: touch none of it, poison this
    // block's sums so the host reports the launch as failed
    for (int k = tid; k < S * RG_ACC; k += blockDim.x)
      partial[(size_t)blockIdx.x * S * RG_ACC + k] = __longlong_as_double(0x7ff8000000000000LL);
    return;
  }
  double* acc = reinterpret_cast<double*>(smem_raw + L.acc);
  // per (scenario, asset): (a_u/(gx-1), inv_h/(gx-1), row offset - 0x4B000000 as bits, x0)
  float4* s_lv = reinterpret_cast<float4*>(smem_raw + L.lv);
  uint32_t* s_flags = reinterpret_cast<uint32_t*>(smem_raw + L.flags);
  int32_t* s_per = reinterpret_cast<int32_t*>(smem_raw + L.per);
  int32_t* s_noff = reinterpret_cast<int32_t*>(smem_raw + L.noff);
  float* s_ncf = reinterpret_cast<float*>(smem_raw + L.ncf);
  float* wcur = reinterpret_cast<float*>(smem_raw + L.wcur);
  float* stack = reinterpret_cast<float*>(smem_raw + L.stack);
  float* Z = reinterpret_cast<float*>(smem_raw + L.z);
  float* dW = reinterpret_cast<float*>(smem_raw + L.dw);
  double* red = reinterpret_cast<double*>(Z);  // reduction scratch, reused after the time loop

  for (int k = tid; k < S * RG_ACC; k += blockDim.x) acc[k] = 0.0;

  const int s = tid / Pb, pl = tid % Pb;
  const bool lane_ok = s < S;
  const int gx = tr.gx;
  const float gxm1 = (float)(gx - 1);
  const float nhdt = (float)(-0.5 * tr.dt);

  // scenario constants: the Cholesky factor and drifts in registers; the per-asset local-vol
  // constants (warp-uniform) in shared memory
  for (int i = tid; i < S * N; i += blockDim.x) {
    const DevScen32& s3 = scen32[i / N];
    const int f = i % N;
    const float inv_gxm1 = 1.0f / (float)(tr.gx - 1);
    s_lv[i] = make_float4(s3.a_u[f] * inv_gxm1, s3.inv_h[f] * inv_gxm1,
                          __int_as_float((int)((uint32_t)s3.surf_off[f] - 0x4B000000u)), s3.x0[f]);
  }
  float Lf[N * (N + 1) / 2], mu[N], sig[N];
  const int ss = lane_ok ? s : 0;
  {
    const DevScenario& sc = scen[ss];
    const DevScen32& s3 = scen32[ss];
    int q = 0;
#pragma unroll
    for (int a = 0; a < N; ++a)
#pragma unroll
      for (int b = 0; b <= a; ++b) Lf[q++] = (float)sc.L[a * N + b];
#pragma unroll
    for (int f = 0; f < N; ++f) {
      mu[f] = s3.mu_dt[f];
      sig[f] = s3.sig[f];
    }
  }
  const float4* lvc = s_lv + ss * N;
  __syncthreads();

  const uint64_t ntiles = (npaths + Pb - 1) / Pb;
  for (uint64_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    const uint64_t tile0 = tile * Pb;
    for (int c = tid; c < PbN; c += blockDim.x) wcur[c] = 0.0f;
    const uint64_t gi = tile0 + pl;
    const bool ok = lane_ok && gi < npaths;
    float x[N];
#pragma unroll
    for (int f = 0; f < N; ++f) x[f] = lvc[f].w;
    P32Phoenix ph;
    float worst = 0.0f;
    int sp = 0;
    for (int t0 = 0; t0 < T; t0 += TT) {
      const int tn = min(TT, T - t0);
      const int n0 = __ldg(tb.node_off + t0), n1 = __ldg(tb.node_off + t0 + tn);
      const int nn = n1 - n0;
      // ---- G: standard normals of the tile's bridge nodes, and the tile's step schedule
      for (int i = tid; i < tn; i += blockDim.x) {
        s_flags[i] = __ldg(tb.step_flags + t0 + i);
        s_per[i] = __ldg(tb.step_period + t0 + i);
      }
      for (int i = tid; i <= tn; i += blockDim.x) s_noff[i] = __ldg(tb.node_off + t0 + i);
      for (int i = tid; i < nn; i += blockDim.x) s_ncf[i] = __ldg(tb.node_cf + n0 + i);
      const int ntask = nn * N * nch;
      for (int task = tid; task < ntask; task += blockDim.x) {
        const int c = task % nch, rem = task / nch, f = rem % N, j = rem / N;
        const int nd = n0 + j;
        const uint64_t g0 = tile0 + (uint64_t)c * GEN_CH;
        if (g0 >= npaths) continue;  // these paths are never read
        float* zo = Z + (size_t)(j * N + f) * (Pb + 4) + c;
        if (tr.vr == RG_VR_SOBOL) {
          const uint32_t* row = tb.sobol + 32 * (size_t)__ldg(tb.nf_row + nd * N + f);
          uint64_t n = path0 + g0 + 1;
          uint32_t xs = rg_sobol_gray(row, n);
          if (tr.scrambler == RG_SCRAMBLE_DIGITAL_SHIFT) {
            const uint32_t shift = __ldg(tb.nf_shift + nd * N + f);
#pragma unroll
            for (int q = 0; q < GEN_CH; ++q) {
              if (q) {
                ++n;
                xs ^= __ldg(row + (__ffsll((long long)n) - 1));
              }
              zo[q * nch] = rg_probit32(xs ^ shift);
            }
          } else {
            const uint64_t dim = (uint64_t)__ldg(tb.node_k + nd) * N + f;
            for (int q = 0; q < GEN_CH; ++q) {
              if (q) {
                ++n;
                xs ^= __ldg(row + (__ffsll((long long)n) - 1));
              }
              zo[q * nch] = rg_probit32(rg_owen(xs, dim, tr.seed));
            }
          }
        } else {
          const uint64_t dim = (uint64_t)__ldg(tb.node_k + nd) * N + f;
          for (int q = 0; q < GEN_CH; ++q) zo[q * nch] = rg_qmc_normal32(tr, tb, path0 + g0 + q, dim);
        }
      }
      __syncthreads();
      // ---- B: streamed bridge, one chain per (path, factor)
      for (int c = tid; c < PbN; c += blockDim.x) {
        const int p = c % Pb, f = c / Pb;
        if (tile0 + p >= npaths) continue;
        const int pc = p / GEN_CH, pq = p % GEN_CH;
        float wc = wcur[c];
        int lsp = sp;
        for (int tt = 0; tt < tn; ++tt) {
          const int e0 = s_noff[tt], e1 = s_noff[tt + 1];
          for (int nd = e0; nd < e1; ++nd) {
            const int j = nd - n0;
            const float z = Z[(size_t)(j * N + f) * (Pb + 4) + pq * nch + pc];
            const float cf = s_ncf[j];
            const float w = nd == 0 ? z * cf : fmaf(z, cf, 0.5f * (wc + stack[(lsp - 1) * PbN + c]));
            stack[lsp * PbN + c] = w;
            ++lsp;
          }
          --lsp;
          const float wn = stack[lsp * PbN + c];
          dW[(tt * N + f) * Pb + p] = wn - wc;
          wc = wn;
        }
        wcur[c] = wc;
      }
      sp += nn - tn;
      __syncthreads();
      // ---- S: scenario stepping
      if (ok) {
        for (int tt = 0; tt < tn; ++tt) {
          const int tg = (t0 + tt) * gx;
          float d[N], y[N];
#pragma unroll
          for (int f = 0; f < N; ++f) d[f] = dW[(tt * N + f) * Pb + pl];
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
              // sigma at the step's time row, linear in log-spot.  u01 = the grid position scaled
              // to [0, 1], clamped by the FMA's saturation (NaN -> 0); 2^23 + floor(u01·(gx-1))
              // by one round-down FMA, whose bit pattern minus 0x4B000000 is the grid index —
              // that bias is folded into the row offset c4.z; then one (value, slope) gather
              const float4 c4 = lvc[f];
              const float u01 = __saturatef(fmaf(x[f], c4.y, c4.x));
              const float fl = __fmaf_rd(u01, gxm1, 8388608.0f);
              const float w = fmaf(u01, gxm1, 8388608.0f - fl);
              const uint32_t idx = (uint32_t)__float_as_int(c4.z) + (uint32_t)tg + (uint32_t)__float_as_int(fl);
              const float2 r = __ldg(tb.lv_rows + idx);
              sg = fmaf(w, r.y, r.x);
            } else {
              sg = sig[f];
            }
            x[f] = fmaf(sg, fmaf(nhdt, sg, y[f]), x[f]) + mu[f];
            wmin = fminf(wmin, x[f]);
          }
          worst = wmin;
          if (ph.alive)
            p32_phoenix_step<REC>(ph, s_flags[tt], t0 + tt, wmin, ln_cb, ln_ko, tr, tb, tb.df_f + (size_t)ss * T,
                                  [&] { return s_per[tt]; });
        }
      }
      __syncthreads();
    }
    // ---- path close (note.rs:221-258) and the per-tile reduction
    float out[RG_ACC];
    p32_close_path<REC>(tr, tb, ss, T, ok, s == 0, path0, gi, ph.ko_step, worst, ln_ki, ph.cpv, ph.mpv,
                        ph.received, ph.qualified, ph.paid, ko_steps, records, out);
    // butterfly within each group of lanes that share a scenario (g = min(32, Pb) lanes)
    const int g = Pb < 32 ? Pb : 32;
    for (int off = g >> 1; off > 0; off >>= 1)
#pragma unroll
      for (int k = 0; k < RG_ACC; ++k) out[k] += __shfl_xor_sync(0xffffffffu, out[k], off);
    if ((lane % g) == 0)
#pragma unroll
      for (int k = 0; k < RG_ACC; ++k) red[(size_t)(tid / g) * RG_ACC + k] = (double)out[k];
    __syncthreads();
    const int groups_per_scen = Pb / g;
    for (int jx = tid; jx < S * RG_ACC; jx += blockDim.x) {
      const int ss = jx / RG_ACC, k = jx % RG_ACC;
      double v = 0.0;
      for (int w = 0; w < groups_per_scen; ++w) v += red[(size_t)(ss * groups_per_scen + w) * RG_ACC + k];
      acc[jx] += v;
    }
    __syncthreads();
  }
  for (int jx = tid; jx < S * RG_ACC; jx += blockDim.x) partial[(size_t)blockIdx.x * S * RG_ACC + jx] = acc[jx];
}

template <int N, bool LV>
static const void* kernel_ptr(bool rec) {
  return rec ? reinterpret_cast<const void*>(&phoenix32_kernel<N, LV, true>)
             : reinterpret_cast<const void*>(&phoenix32_kernel<N, LV, false>);
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

Fp32Shape phoenix32_shape(const Prepared& P, uint64_t npaths, int sm_count) {
  Fp32Shape sh{};
  if (P.n_scen > 32) raise(RG_ERR_INVALID_ARGUMENT, "at most 32 scenarios per fused launch");
  if (p32_direct(P, npaths)) {
    // nothing for the scenarios to share: the per-thread kernel without shared-memory tiles
    sh.direct = 1;
    sh.Sb = P.n_scen;
    sh.threads = 256;
    sh.grid = phoenix32d_grid(P, npaths, sm_count);
    sh.smem = P.stack_max * P.n * 256 * (int)sizeof(float);  // the bridge stacks (dynamic)
    return sh;
  }
  // scenario slots: S rounded up to a power of two, at least 4 (two scenarios run padded: a CTA
  // of 1024 threads on half the slots beats both the direct kernel and a smaller CTA); the
  // largest block of 1024, 512 or 256 threads whose shared-memory layout fits
  int sb = 4;
  while (sb < P.n_scen) sb <<= 1;
  sh.Sb = sb;
  const int N = P.n;
  for (int threads = 1024; threads >= 256; threads >>= 1) {
    sh.threads = threads;
    sh.Pb = threads / sb;
    const int PbN = sh.Pb * N;
    int tt = (32768 / PbN - P.stack_max) / 2;
    tt = tt < 8 ? 8 : (tt > 64 ? 64 : tt);
    sh.TT = tt;
    sh.smem = (int)p32_layout(P.n_scen, N, sh.Pb, tt, tt + P.stack_max, P.stack_max, threads).total;
    if (sh.smem <= 227 * 1024 || threads == 256) break;
  }
  // Function attributes are process-wide: raise every instantiation's dynamic shared-memory limit
  // to the device maximum once, so engines pricing concurrently never lower it under each other.
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
            const void* kr = select_kernel(n, lv != 0, rec != 0);
            cuda_check(cudaFuncSetAttribute(kr, cudaFuncAttributeMaxDynamicSharedMemorySize, optin),
                       "phoenix32 smem attribute");
            cuda_check(cudaFuncSetAttribute(kr, cudaFuncAttributePreferredSharedMemoryCarveout, 100),
                       "phoenix32 carveout");
          }
      done[dev] = 1;
    }
  }
  const void* k = select_kernel(P.n, P.trade.has_lv != 0, false);
  int per_sm = 0;
  cuda_check(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k, sh.threads, sh.smem),
             "phoenix32 occupancy");
  if (per_sm < 1) raise(RG_ERR_GPU_ERROR, "phoenix32: launch shape does not fit on an SM");
  uint64_t tiles = (npaths + sh.Pb - 1) / sh.Pb;
  uint64_t cap = (uint64_t)sm_count * per_sm;
  sh.grid = (int)(tiles < cap ? tiles : cap);
  if (sh.grid < 1) sh.grid = 1;
  return sh;
}

// ---------------------------------------------------------------------- tile-depth autotuner --
namespace {
std::mutex g_tune_mu;
std::map<std::vector<int64_t>, int> g_tuned;  // launch shape -> tile depth
bool g_tune_enabled = true;

// Sets the tile depth of a tiled-kernel shape if its layout fits next to the same block size.
bool p32_with_tt(const Prepared& P, Fp32Shape& sh, int tt) {
  const int smem = (int)p32_layout(P.n_scen, P.n, sh.Pb, tt, tt + P.stack_max, P.stack_max, sh.threads).total;
  if (smem > 227 * 1024) return false;
  sh.TT = tt;
  sh.smem = smem;
  return true;
}
}  // namespace

void p32_set_autotune(bool enabled) {
  std::lock_guard<std::mutex> lock(g_tune_mu);
  g_tune_enabled = enabled;
  g_tuned.clear();
}

Fp32Shape phoenix32_tune(const Prepared& P, const DevTables& tb, const DevScenario* scen,
                         const DevScen32* scen32, uint64_t path0, uint64_t npaths, Fp32Shape sh,
                         const LaunchOut& out, bool may_tune, cudaStream_t st) {
  // only the 1024-thread shapes, which hold one CTA per SM whatever the tile depth (the grid, the
  // partial-sum buffer and the block's path grouping stay as they are)
  if (sh.direct || sh.threads != 1024) return sh;
  int dev = 0;
  cuda_check(cudaGetDevice(&dev), "cudaGetDevice");
  const std::vector<int64_t> key{dev, P.n, P.trade.has_lv, P.n_scen, sh.Sb, P.T, P.stack_max,
                                 P.trade.vr, P.trade.scrambler, P.trade.gx};
  {
    std::lock_guard<std::mutex> lock(g_tune_mu);
    if (!g_tune_enabled) return sh;
    auto it = g_tuned.find(key);
    if (it != g_tuned.end()) {
      Fp32Shape t = sh;
      if (p32_with_tt(P, t, it->second)) t.tuned = 1;
      return t.tuned ? t : sh;
    }
  }
  // a tuning pass costs about (candidates × 2) launches over two waves of tiles: only for
  // launches of at least eight waves
  const uint64_t prefix = (uint64_t)sh.grid * (uint64_t)sh.Pb * 2;
  if (!may_tune || npaths < prefix * 4) return sh;
  std::vector<int> cand;
  for (int tt : {sh.TT, 24, 32, 48, 64, 80, 96, 128}) {
    Fp32Shape c = sh;
    if (std::find(cand.begin(), cand.end(), tt) == cand.end() && p32_with_tt(P, c, tt)) cand.push_back(tt);
  }
  LaunchOut lo = out;  // the partial sums are overwritten by the real launch afterwards
  lo.ko_steps = nullptr;
  lo.records = nullptr;
  cudaEvent_t e0, e1;
  cuda_check(cudaEventCreate(&e0), "event");
  cuda_check(cudaEventCreate(&e1), "event");
  std::vector<float> best(cand.size(), 1e30f);
  for (int rep = 0; rep < 2; ++rep)
    for (size_t i = 0; i < cand.size(); ++i) {
      Fp32Shape c = sh;
      p32_with_tt(P, c, cand[i]);
      cuda_check(cudaEventRecord(e0, st), "event");
      launch_phoenix32(P, tb, scen, scen32, path0, prefix, c, lo, st);
      cuda_check(cudaEventRecord(e1, st), "event");
      cuda_check(cudaEventSynchronize(e1), "autotune");
      float ms = 0.f;
      cuda_check(cudaEventElapsedTime(&ms, e0, e1), "event time");
      best[i] = std::min(best[i], ms);
    }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  const size_t win = (size_t)(std::min_element(best.begin(), best.end()) - best.begin());
  Fp32Shape t = sh;
  p32_with_tt(P, t, cand[win]);
  t.tuned = 1;
  std::lock_guard<std::mutex> lock(g_tune_mu);
  g_tuned[key] = cand[win];
  return t;
}

void launch_phoenix32(const Prepared& P, const DevTables& tb, const DevScenario* scen,
                      const DevScen32* scen32, uint64_t path0, uint64_t npaths, const Fp32Shape& sh,
                      const LaunchOut& out, cudaStream_t st) {
  if (sh.direct) {
    launch_phoenix32d(P, tb, scen, scen32, path0, npaths, sh.grid, out, st);
    return;
  }
  const float ln_ko = (float)P.ln_ko, ln_cb = (float)P.ln_cb, ln_ki = (float)P.ln_ki;
  const int NNmax = sh.TT + P.stack_max;
#define RG_LAUNCH(NN, LVV)                                                                        \
  if (out.records) RG_LAUNCH_R(NN, LVV, true) else RG_LAUNCH_R(NN, LVV, false)
#define RG_LAUNCH_R(NN, LVV, REC)                                                                 \
  phoenix32_kernel<NN, LVV, REC><<<sh.grid, sh.threads, sh.smem, st>>>(                           \
      P.trade, tb, scen, scen32, P.n_scen, sh.Pb, sh.TT, NNmax, P.stack_max, ln_ko, ln_cb, ln_ki, \
      path0, npaths, out.partial, out.ko_steps, out.records);
  const bool lv = P.trade.has_lv != 0;
  switch (P.n) {
    case 1: if (lv) { RG_LAUNCH(1, true) } else { RG_LAUNCH(1, false) } break;
    case 2: if (lv) { RG_LAUNCH(2, true) } else { RG_LAUNCH(2, false) } break;
    case 3: if (lv) { RG_LAUNCH(3, true) } else { RG_LAUNCH(3, false) } break;
    case 4: if (lv) { RG_LAUNCH(4, true) } else { RG_LAUNCH(4, false) } break;
    case 5: if (lv) { RG_LAUNCH(5, true) } else { RG_LAUNCH(5, false) } break;
    default: raise(RG_ERR_INVALID_MARKET_SHAPE, "unsupported asset count");
  }
#undef RG_LAUNCH
#undef RG_LAUNCH_R
  cuda_check(cudaGetLastError(), "phoenix32_kernel launch");
}

}  // namespace rg
