// phoenix64.cu — the FP64 parity kernel: generation + bridge + step + payoff fused per path.
//
// One thread prices one path of one scenario in the reference's own operation order
// (crates/riga-engine/src/note.rs:81-259): QMC normals per step, y = L·z, the depth-first
// Brownian bridge of each factor (or, in the pseudo-random lane, the path's slice of the ChaCha8
// normal stream and y = L·z with no bridge, note.rs:123-127), the multiplicative GBM/Dupire step, the Phoenix state machine
// and the path close.  The bridge is streamed: an in-order traversal of the bisection tree needs
// only the current point and a stack of right anchors, so no per-path O(T) buffer exists.  The
// node schedule (which preorder index and standard deviation each step consumes) is a host table
// shared by every thread, so the traversal is warp-uniform.
//
// Compiled with -fmad=false: products and sums round separately, as in the reference; exp and
// log are the deterministic rg_exp64/rg_log64 shared with the host tables.
#include "rg_internal.h"

namespace rg {

// DupireLocalVol::sigma with a precomputed tenor row/weight (riga-market/src/lib.rs:305-343).
__device__ __forceinline__ double lv_sigma64(const double* __restrict__ v, const double* __restrict__ ls,
                                             int gx, int ti, int ti1, double wt, double spot) {
  double x = rg_log64(spot > 1e-12 ? spot : 1e-12);
  int lo, hi;
  if (x <= __ldg(ls)) {
    lo = 0; hi = 0;
  } else if (x >= __ldg(ls + gx - 1)) {
    lo = gx - 1; hi = gx - 1;
  } else {
    // first j with x <= ls[j+1]: start from the uniform-axis estimate and correct
    double l0 = __ldg(ls), l1 = __ldg(ls + gx - 1);
    int j = (int)((x - l0) / (l1 - l0) * (double)(gx - 1));
    j = j < 0 ? 0 : (j > gx - 2 ? gx - 2 : j);
    while (j > 0 && x <= __ldg(ls + j)) --j;
    while (j + 1 < gx - 1 && x > __ldg(ls + j + 1)) ++j;
    lo = j; hi = j + 1;
  }
  double wx = hi == lo ? 0.0 : (x - __ldg(ls + lo)) / (__ldg(ls + hi) - __ldg(ls + lo));
  double v0 = (1.0 - wx) * __ldg(v + ti * gx + lo) + wx * __ldg(v + ti * gx + hi);
  double v1 = (1.0 - wx) * __ldg(v + ti1 * gx + lo) + wx * __ldg(v + ti1 * gx + hi);
  return (1.0 - wt) * v0 + wt * v1;
}

template <int N, bool LV, bool MC>
__global__ void __launch_bounds__(128) phoenix64_kernel(DevTrade tr, DevTables tb,
                                                        const DevScenario* __restrict__ scen,
                                                        uint64_t path0, uint64_t npaths,
                                                        double* __restrict__ partial,
                                                        int32_t* __restrict__ ko_steps,
                                                        rg_path_record* __restrict__ records,
                                                        const double* __restrict__ mcz,
                                                        float* __restrict__ cube) {
  __shared__ double red[128][RG_ACC + 1];
  __shared__ double acc_blk[RG_ACC];
  const int tid = threadIdx.x;
  if (tid < RG_ACC) acc_blk[tid] = 0.0;
  const DevScenario& sc = scen[0];
  double L[N * N], s0[N], vol[N], qd[N];
  int surf_off[N], logs_off[N];
#pragma unroll
  for (int i = 0; i < N * N; ++i) L[i] = sc.L[i];
#pragma unroll
  for (int f = 0; f < N; ++f) {
    s0[f] = sc.spots[f];
    vol[f] = sc.vols[f];
    qd[f] = sc.q[f];
    surf_off[f] = LV ? sc.surf_off[f] : 0;
    logs_off[f] = LV ? sc.surf[f] * tr.gx : 0;
  }
  const double rate = sc.rate, dt = tr.dt, inv_sqrt_dt = tr.inv_sqrt_dt, sqrt_dt = tr.sqrt_dt;
  const int64_t T = tr.steps;
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  const uint64_t rounds = (npaths + stride - 1) / stride;
  for (uint64_t rd = 0; rd < rounds; ++rd) {
    const uint64_t i = rd * stride + (uint64_t)blockIdx.x * blockDim.x + tid;
    double out[RG_ACC];
#pragma unroll
    for (int k = 0; k < RG_ACC; ++k) out[k] = 0.0;
    if (i < npaths) {
      const uint64_t path = path0 + i;
      double spots[N], wcur[N], stk[RG_STACK_MAX][N];
#pragma unroll
      for (int f = 0; f < N; ++f) {
        spots[f] = s0[f];
        wcur[f] = 0.0;
      }
      int sp = 0;
      int ko = 0, received = 0, ko_step = -1, qualified = 0, paid = 0;
      double accrual = 0.0, unpaid = 0.0, cpv = 0.0, mpv = 0.0, final_worst = 1.0;
      for (int64_t t = 0; t < T; ++t) {
        double shock[N];
        if (MC) {
          // pseudo-random lane (note.rs:123-127): n draws of the sequential stream, then L·z
          const double* zp = mcz + (i * (uint64_t)T + (uint64_t)t) * N;
          double z[N];
#pragma unroll
          for (int f = 0; f < N; ++f) z[f] = zp[f];
#pragma unroll
          for (int a = 0; a < N; ++a) {
            double s = 0.0;
#pragma unroll
            for (int b = 0; b <= a; ++b) s += L[a * N + b] * z[b];
            shock[a] = s;
          }
        } else {
          // bridge nodes consumed at this step (note.rs:89-105 and qmc.rs:158-191)
          const int c0 = __ldg(tb.node_off + t), c1 = __ldg(tb.node_off + t + 1);
          for (int c = c0; c < c1; ++c) {
            const int k = __ldg(tb.node_k + c);
            const double cc = __ldg(tb.node_c + c);
            double z[N], y[N];
#pragma unroll
            for (int f = 0; f < N; ++f) z[f] = rg_qmc_normal64(tr, tb, path, (uint64_t)k * N + f);
#pragma unroll
            for (int a = 0; a < N; ++a) {  // Cholesky::apply_into (correlation.rs:196-206)
              double s = 0.0;
#pragma unroll
              for (int b = 0; b <= a; ++b) s += L[a * N + b] * z[b];
              y[a] = s;
            }
            if (c == 0) {
#pragma unroll
              for (int f = 0; f < N; ++f) stk[sp][f] = y[f] * cc;
            } else {
#pragma unroll
              for (int f = 0; f < N; ++f) stk[sp][f] = 0.5 * (wcur[f] + stk[sp - 1][f]) + y[f] * cc;
            }
            ++sp;
          }
          --sp;
#pragma unroll
          for (int f = 0; f < N; ++f) {
            double wn = stk[sp][f];
            shock[f] = (wn - wcur[f]) * inv_sqrt_dt;
            wcur[f] = wn;
          }
        }
        // GBM / Dupire step (note.rs:133-142)
        int2 tix[N];
        double tw[N];
        if (LV) {
#pragma unroll
          for (int f = 0; f < N; ++f) {
            tix[f] = __ldg(tb.lv_ti + f * T + t);
            tw[f] = __ldg(tb.lv_tw + f * T + t);
          }
        }
#pragma unroll
        for (int f = 0; f < N; ++f) {
          double v = LV ? lv_sigma64(tb.lv_v + surf_off[f], tb.lv_logs + logs_off[f], tr.gx, tix[f].x,
                                     tix[f].y, tw[f], spots[f])
                        : vol[f];
          double drift = (rate - qd[f] - 0.5 * v * v) * dt;
          spots[f] *= rg_exp64(drift + v * sqrt_dt * shock[f]);
        }
        if (cube) {  // PathCube slice: the spots this step leaves (pathcube.rs:19-35 layout)
          float* cp = cube + (i * (uint64_t)T + (uint64_t)t) * N;
#pragma unroll
          for (int f = 0; f < N; ++f) cp[f] = (float)spots[f];
        }
        double worst = spots[0] / tr.init[0];
#pragma unroll
        for (int f = 1; f < N; ++f) worst = fmin(worst, spots[f] / tr.init[f]);
        final_worst = worst;
        if (ko) continue;
        // Phoenix state machine (note.rs:150-218)
        const uint32_t fl = __ldg(tb.step_flags + t);
        const int per = __ldg(tb.step_period + t);
        if (fl & STEP_PERIOD_RESET) accrual = 0.0;
        if ((fl & STEP_ACCRUE) && worst >= tr.coupon_barrier) {
          accrual += __ldg(tb.accr_inc + per);
          ++qualified;
        }
        bool up = (fl & STEP_CALL_ACTIVE) != 0;
#pragma unroll
        for (int f = 0; f < N; ++f) up = up && (spots[f] / tr.init[f] >= tr.call_barrier);
        if (up) {
          ko = 1;
          ko_step = (int)t;
          double due = (fl & STEP_FIXED_DUE) ? tr.coupon_rate : accrual;
          double carry = due > 0.0 ? unpaid : 0.0;
          if (due + carry > 0.0) {
            double df = __ldg(tb.df + t);
            cpv += due * df;
            mpv += carry * df;
            received = 1;
            ++paid;
          }
          continue;
        }
        if (fl & STEP_PERIOD_END) {
          double due = (fl & STEP_FIXED_DUE) ? tr.coupon_rate : accrual;
          if (due > 0.0) {
            double df = __ldg(tb.df + t);
            cpv += due * df;
            mpv += unpaid * df;
            received = 1;
            unpaid = 0.0;
            ++paid;
          } else if (tr.memory) {
            unpaid += tr.coupon_rate;
          }
        }
      }
      // path close (note.rs:221-258)
      const double dfm = __ldg(tb.df_mat);
      const double funding = ko ? __ldg(tb.df + ko_step) : dfm;
      const int hit_ki = final_worst <= tr.ki;
      const int put_ok = hit_ki && !ko;
      const double put = put_ok ? fmax(tr.strike - final_worst, 0.0) * dfm : 0.0;
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
      if (ko_steps) ko_steps[i] = ko_step;
      if (records) {
        rg_path_record r;
        r.path_id = path;
        r.rng_seed = tr.seed;
        r.sobol_index = MC ? 0 : path + 1;
        r.worst_final = final_worst;
        r.knocked_out = ko;
        r.ko_step = ko_step;
        r.ko_time = ko ? (double)(ko_step + 1) * dt : __longlong_as_double(0x7ff8000000000000LL);
        r.ki_hit = hit_ki;
        r.qualified_steps = qualified;
        r.paid_periods = paid;
        r.put_payoff = put;
        r.coupon_pv = cn;
        r.memory_coupon_pv = mpv;
        r.funding = funding;
        r.pv = pv;
        records[i] = r;
      }
    }
    // fixed-order block reduction of this round
#pragma unroll
    for (int k = 0; k < RG_ACC; ++k) red[tid][k] = out[k];
    __syncthreads();
    for (int s = 64; s > 0; s >>= 1) {
      if (tid < s)
        for (int k = 0; k < RG_ACC; ++k) red[tid][k] += red[tid + s][k];
      __syncthreads();
    }
    if (tid < RG_ACC) acc_blk[tid] += red[0][tid];
    __syncthreads();
  }
  if (tid < RG_ACC) partial[(size_t)blockIdx.x * RG_ACC + tid] = acc_blk[tid];
}

int phoenix64_grid(const Prepared& P, uint64_t npaths) {
  (void)P;
  uint64_t blocks = (npaths + 127) / 128;
  const uint64_t cap = 152 * 16;  // a few rounds of resident CTAs on 152 SMs
  return (int)(blocks < cap ? blocks : cap);
}

template <int N, bool LV>
static void launch_n(const Prepared& P, const DevTables& tb, const DevScenario* scen, uint64_t path0,
                     uint64_t npaths, const LaunchOut& out, cudaStream_t s) {
  if (out.mcz)
    phoenix64_kernel<N, LV, true><<<out.grid, 128, 0, s>>>(P.trade, tb, scen, path0, npaths, out.partial,
                                                           out.ko_steps, out.records, out.mcz,
                                                           out.cube);
  else
    phoenix64_kernel<N, LV, false><<<out.grid, 128, 0, s>>>(P.trade, tb, scen, path0, npaths, out.partial,
                                                            out.ko_steps, out.records, nullptr,
                                                            out.cube);
}

void launch_phoenix64(const Prepared& P, const DevTables& tb, const DevScenario* scen,
                      uint64_t path0, uint64_t npaths, const LaunchOut& out, cudaStream_t s) {
  const bool lv = P.trade.has_lv != 0;
#define RG_CASE(NN)                                                   \
  case NN:                                                            \
    if (lv) launch_n<NN, true>(P, tb, scen, path0, npaths, out, s);   \
    else launch_n<NN, false>(P, tb, scen, path0, npaths, out, s);     \
    break;
  switch (P.n) {
    RG_CASE(1) RG_CASE(2) RG_CASE(3) RG_CASE(4) RG_CASE(5)
    default: raise(RG_ERR_INVALID_MARKET_SHAPE, "unsupported asset count");
  }
#undef RG_CASE
  cuda_check(cudaGetLastError(), "phoenix64_kernel launch");
}

}  // namespace rg
