// phoenix32.cu — the FP32 production kernel: one fused launch prices S common-random-number
// scenarios of one trade.
//
// A CTA owns Pb paths × Sb scenario lanes (Sb = S rounded up to a power of two, Sb·Pb = 256) and
// walks time in tiles of TT steps:
//   1. chain phase — one "chain" per (path, factor) generates the Sobol coordinates of the bridge
//      nodes the tile consumes, maps them through the inverse normal and advances the streamed
//      Brownian bridge of that factor; the uncorrelated increments dW[tile][factor][path] land in
//      shared memory.  Generation is paid once per path, not once per scenario.
//   2. scenario phase — every (path, scenario) thread correlates the increments with its own
//      Cholesky factor (the bridge is linear, so L·bridge(z) = bridge(L·z)), steps ln(S/S0) under
//      flat vol or its scenario's Dupire surface and runs the Phoenix state machine.
// Path state is FP32; event cash flows, discount factors and every reduction are FP64.
// Reductions are fixed-order (shuffle butterfly, then warps in index order, then blocks in the
// final reduce kernel), so results are bit-reproducible for a given launch shape.
#include "rg_internal.h"

namespace rg {

template <int N, bool LV>
__global__ void __launch_bounds__(256, 2) phoenix32_kernel(
    DevTrade tr, DevTables tb, const DevScenario* __restrict__ scen,
    const DevScen32* __restrict__ scen32, int S, int Sb, int Pb, int TT, int stack_max, float ln_ko,
    float ln_cb, float ln_ki, uint64_t path0, uint64_t npaths, double* __restrict__ partial,
    int32_t* __restrict__ ko_steps, rg_path_record* __restrict__ records) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int nwarps = blockDim.x >> 5;
  const int PbN = Pb * N;
  double* acc = reinterpret_cast<double*>(smem_raw);                  // [S][RG_ACC]
  unsigned char* region = smem_raw + (((size_t)S * RG_ACC * 8 + 15) & ~(size_t)15);
  float* wcur = reinterpret_cast<float*>(region);                    // [N*Pb]
  float* stack = wcur + PbN;                                         // [stack_max][N*Pb]
  float* dW = stack + (size_t)stack_max * PbN;                       // [TT][N][Pb]
  double* red = reinterpret_cast<double*>(region);                   // [nwarps][Sb][RG_ACC]

  for (int k = tid; k < S * RG_ACC; k += blockDim.x) acc[k] = 0.0;

  const int s = tid % Sb, pl = tid / Sb;
  const bool lane_ok = s < S;
  const int T = (int)tr.steps;
  const int gx = tr.gx;
  const float gxm1 = (float)(gx - 1);
  const float nhdt = (float)(-0.5 * tr.dt);

  // scenario constants in registers
  float Lf[N * (N + 1) / 2], mu[N], sig[N], x0[N], a_u[N], inv_h[N];
  int soff[N];
  const double* df_s = tb.df;
  double df_mat = 1.0;
  if (lane_ok) {
    const DevScenario& sc = scen[s];
    const DevScen32& s3 = scen32[s];
    int q = 0;
#pragma unroll
    for (int a = 0; a < N; ++a)
#pragma unroll
      for (int b = 0; b <= a; ++b) Lf[q++] = (float)sc.L[a * N + b];
#pragma unroll
    for (int f = 0; f < N; ++f) {
      mu[f] = s3.mu_dt[f];
      sig[f] = s3.sig[f];
      x0[f] = s3.x0[f];
      a_u[f] = s3.a_u[f];
      inv_h[f] = s3.inv_h[f];
      soff[f] = s3.surf_off[f];
    }
    df_s = tb.df + (size_t)s * T;
    df_mat = tb.df_mat[s];
  }

  const uint64_t ntiles = (npaths + Pb - 1) / Pb;
  for (uint64_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    const uint64_t tile0 = tile * Pb;
    for (int c = tid; c < PbN; c += blockDim.x) wcur[c] = 0.0f;
    const uint64_t gi = tile0 + pl;
    const bool ok = lane_ok && gi < npaths;
    float x[N];
#pragma unroll
    for (int f = 0; f < N; ++f) x[f] = x0[f];
    bool alive = true, received = false;
    int qual = 0, unpaid = 0, ko_step = -1, qualified = 0, paid = 0;
    double cpv = 0.0, mpv = 0.0;
    float worst = 0.0f;
    int sp = 0;
    __syncthreads();
    for (int t0 = 0; t0 < T; t0 += TT) {
      const int tn = min(TT, T - t0);
      // ---- chain phase: Sobol → inverse normal → streamed bridge, one chain per (path, factor)
      for (int c = tid; c < PbN; c += blockDim.x) {
        const int p = c % Pb, f = c / Pb;
        const uint64_t cgi = tile0 + p;
        if (cgi < npaths) {
          const uint64_t path = path0 + cgi;
          float wc = wcur[c];
          int lsp = sp;
          for (int tt = 0; tt < tn; ++tt) {
            const int t = t0 + tt;
            const int n0 = __ldg(tb.node_off + t), n1 = __ldg(tb.node_off + t + 1);
            for (int nd = n0; nd < n1; ++nd) {
              const int k = __ldg(tb.node_k + nd);
              const float cf = __ldg(tb.node_cf + nd);
              const float z = rg_qmc_normal32(tr, tb, path, (uint64_t)k * N + f);
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
      }
      sp += (__ldg(tb.node_off + t0 + tn) - __ldg(tb.node_off + t0)) - tn;
      __syncthreads();
      // ---- scenario phase
      if (ok) {
        for (int tt = 0; tt < tn; ++tt) {
          const int t = t0 + tt;
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
              const int2 ti = __ldg(tb.lv_ti + f * T + t);
              const float wt = __ldg(tb.lv_twf + f * T + t);
              float u = fmaf(x[f], inv_h[f], a_u[f]);
              u = fminf(fmaxf(u, 0.0f), gxm1);
              const int j = min((int)u, gx - 2);
              const float w = u - (float)j;
              const float2* base = tb.lv_vf + soff[f] + j;
              const float2 lo = __ldg(base + ti.x * gx), hi = __ldg(base + ti.y * gx);
              const float v0 = fmaf(w, lo.y, lo.x), v1 = fmaf(w, hi.y, hi.x);
              sg = fmaf(wt, v1 - v0, v0);
            } else {
              sg = sig[f];
            }
            x[f] += fmaf(sg, y[f], fmaf(nhdt * sg, sg, mu[f]));
            wmin = fminf(wmin, x[f]);
          }
          worst = wmin;
          if (alive) {
            const uint32_t fl = __ldg(tb.step_flags + t);
            if (fl & STEP_PERIOD_RESET) qual = 0;
            if ((fl & STEP_ACCRUE) && wmin >= ln_cb) {
              ++qual;
              ++qualified;
            }
            if ((fl & STEP_CALL_ACTIVE) && wmin >= ln_ko) {
              alive = false;
              ko_step = t;
              const double due = (fl & STEP_FIXED_DUE) ? tr.coupon_rate
                                                       : (double)qual * __ldg(tb.accr_inc + __ldg(tb.step_period + t));
              const double carry = due > 0.0 ? (double)unpaid * tr.coupon_rate : 0.0;
              if (due + carry > 0.0) {
                const double df = __ldg(df_s + t);
                cpv += due * df;
                mpv += carry * df;
                received = true;
                ++paid;
              }
            } else if (fl & STEP_PERIOD_END) {
              const double due = (fl & STEP_FIXED_DUE) ? tr.coupon_rate
                                                       : (double)qual * __ldg(tb.accr_inc + __ldg(tb.step_period + t));
              if (due > 0.0) {
                const double df = __ldg(df_s + t);
                cpv += due * df;
                mpv += (double)unpaid * tr.coupon_rate * df;
                unpaid = 0;
                received = true;
                ++paid;
              } else if (tr.memory) {
                ++unpaid;
              }
            }
          }
        }
      }
      __syncthreads();
    }
    // ---- path close (note.rs:221-258) and the per-tile reduction
    double out[RG_ACC];
#pragma unroll
    for (int k = 0; k < RG_ACC; ++k) out[k] = 0.0;
    if (ok) {
      const bool ko = ko_step >= 0;
      const double funding = ko ? __ldg(df_s + ko_step) : df_mat;
      const bool hit_ki = worst <= ln_ki;
      const bool put_ok = hit_ki && !ko;
      const double wf = exp((double)worst);
      const double put = put_ok ? fmax(tr.strike - wf, 0.0) * df_mat : 0.0;
      const double cn = cpv + mpv;
      const double pv = funding + cn - put;
      out[ACC_PV] = pv - 1.0;
      out[ACC_PV2] = (pv - 1.0) * (pv - 1.0);
      if (ko) {
        out[ACC_KOF] = funding - 1.0;
        out[ACC_KOF2] = (funding - 1.0) * (funding - 1.0);
        out[ACC_NKO] = 1.0;
      }
      if (hit_ki) {
        out[ACC_KIPUT] = put;
        out[ACC_KIPUT2] = put * put;
        out[ACC_NKI] = 1.0;
      }
      if (received) {
        out[ACC_CPN] = cn;
        out[ACC_CPN2] = cn * cn;
        out[ACC_NCPN] = 1.0;
      }
      out[ACC_PUT] = put;
      out[ACC_FUND] = funding;
      out[ACC_CQ] = cn * 10.0 - mpv * 10.0;
      out[ACC_MQ] = mpv * 10.0;
      out[ACC_NPUT] = put_ok ? 1.0 : 0.0;
      if (s == 0 && ko_steps) ko_steps[gi] = ko_step;
      if (s == 0 && records) {
        rg_path_record r;
        r.path_id = path0 + gi;
        r.rng_seed = tr.seed;
        r.sobol_index = path0 + gi + 1;
        r.worst_final = wf;
        r.knocked_out = ko;
        r.ko_step = ko_step;
        r.ko_time = ko ? (double)(ko_step + 1) * tr.dt : __longlong_as_double(0x7ff8000000000000LL);
        r.ki_hit = hit_ki;
        r.qualified_steps = qualified;
        r.paid_periods = paid;
        r.put_payoff = put;
        r.coupon_pv = cn;
        r.memory_coupon_pv = mpv;
        r.funding = funding;
        r.pv = pv;
        records[gi] = r;
      }
    }
    // butterfly across the paths of this warp that share a scenario lane
    for (int off = Sb; off < 32; off <<= 1)
#pragma unroll
      for (int k = 0; k < RG_ACC; ++k) out[k] += __shfl_xor_sync(0xffffffffu, out[k], off);
    if (lane < Sb)
#pragma unroll
      for (int k = 0; k < RG_ACC; ++k) red[((size_t)warp * Sb + lane) * RG_ACC + k] = out[k];
    __syncthreads();
    for (int j = tid; j < S * RG_ACC; j += blockDim.x) {
      const int ss = j / RG_ACC, k = j % RG_ACC;
      double v = 0.0;
      for (int w = 0; w < nwarps; ++w) v += red[((size_t)w * Sb + ss) * RG_ACC + k];
      acc[j] += v;
    }
    __syncthreads();
  }
  for (int j = tid; j < S * RG_ACC; j += blockDim.x) partial[(size_t)blockIdx.x * S * RG_ACC + j] = acc[j];
}

template <int N, bool LV>
static const void* kernel_ptr() {
  return reinterpret_cast<const void*>(&phoenix32_kernel<N, LV>);
}

static const void* select_kernel(int n, bool lv) {
  switch (n) {
    case 1: return lv ? kernel_ptr<1, true>() : kernel_ptr<1, false>();
    case 2: return lv ? kernel_ptr<2, true>() : kernel_ptr<2, false>();
    case 3: return lv ? kernel_ptr<3, true>() : kernel_ptr<3, false>();
    case 4: return lv ? kernel_ptr<4, true>() : kernel_ptr<4, false>();
    case 5: return lv ? kernel_ptr<5, true>() : kernel_ptr<5, false>();
    default: raise(RG_ERR_INVALID_MARKET_SHAPE, "unsupported asset count");
  }
}

Fp32Shape phoenix32_shape(const Prepared& P, uint64_t npaths, int sm_count) {
  Fp32Shape sh{};
  if (P.n_scen > 32) raise(RG_ERR_INVALID_ARGUMENT, "at most 32 scenarios per fused launch");
  int sb = 1;
  while (sb < P.n_scen) sb <<= 1;
  sh.Sb = sb;
  sh.threads = 256;
  sh.Pb = 256 / sb;
  const int PbN = sh.Pb * P.n;
  int tt = 8192 / PbN;
  tt = tt < 8 ? 8 : (tt > 64 ? 64 : tt);
  sh.TT = tt;
  size_t acc_bytes = ((size_t)P.n_scen * RG_ACC * 8 + 15) & ~(size_t)15;
  size_t chain = ((size_t)(1 + P.stack_max) * PbN + (size_t)tt * PbN) * 4;
  size_t red = (size_t)(256 / 32) * sb * RG_ACC * 8;
  sh.smem = (int)(acc_bytes + (chain > red ? chain : red));
  const void* k = select_kernel(P.n, P.trade.has_lv != 0);
  cuda_check(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, sh.smem),
             "phoenix32 smem attribute");
  int per_sm = 0;
  cuda_check(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k, sh.threads, sh.smem),
             "phoenix32 occupancy");
  if (per_sm < 1) per_sm = 1;
  uint64_t tiles = (npaths + sh.Pb - 1) / sh.Pb;
  uint64_t cap = (uint64_t)sm_count * per_sm;
  sh.grid = (int)(tiles < cap ? tiles : cap);
  if (sh.grid < 1) sh.grid = 1;
  return sh;
}

void launch_phoenix32(const Prepared& P, const DevTables& tb, const DevScenario* scen,
                      const DevScen32* scen32, uint64_t path0, uint64_t npaths, const Fp32Shape& sh,
                      const LaunchOut& out, cudaStream_t st) {
  const float ln_ko = (float)P.ln_ko, ln_cb = (float)P.ln_cb, ln_ki = (float)P.ln_ki;
#define RG_LAUNCH(NN, LVV)                                                                       \
  phoenix32_kernel<NN, LVV><<<sh.grid, sh.threads, sh.smem, st>>>(                               \
      P.trade, tb, scen, scen32, P.n_scen, sh.Sb, sh.Pb, sh.TT, P.stack_max, ln_ko, ln_cb, ln_ki, \
      path0, npaths, out.partial, out.ko_steps, out.records)
  const bool lv = P.trade.has_lv != 0;
  switch (P.n) {
    case 1: if (lv) RG_LAUNCH(1, true); else RG_LAUNCH(1, false); break;
    case 2: if (lv) RG_LAUNCH(2, true); else RG_LAUNCH(2, false); break;
    case 3: if (lv) RG_LAUNCH(3, true); else RG_LAUNCH(3, false); break;
    case 4: if (lv) RG_LAUNCH(4, true); else RG_LAUNCH(4, false); break;
    case 5: if (lv) RG_LAUNCH(5, true); else RG_LAUNCH(5, false); break;
    default: raise(RG_ERR_INVALID_MARKET_SHAPE, "unsupported asset count");
  }
#undef RG_LAUNCH
  cuda_check(cudaGetLastError(), "phoenix32_kernel launch");
}

}  // namespace rg
