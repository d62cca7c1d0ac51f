// book64.cu — FP64 parity kernels of a book: universe path generation and the per-trade scan.
//
// Generation: one thread per (path, universe asset u).  At every bridge node the thread forms the
// correlated normal y_u = Σ_{b<=u} L[u][b]·z_b from the QMC normals of dimensions U·k + b
// (Cholesky::apply_into, crates/riga-market/src/correlation.rs:196-206, in the reference's
// order), streams the depth-first Brownian bridge of asset u (crates/riga-engine/src/qmc.rs:
// 158-191) in order, and writes ΔW/√dt of every step to incr[t][u][p] — exactly the array
// note.rs:83-106 builds for a U-asset trade on the universe grid.
//
// Scan: one thread per ((trade, scenario), path) runs note.rs:129-259 on the first T_j steps of
// the trade's assets' increments: the multiplicative step, the Phoenix state machine and the
// path close, then a fixed-order tree over each block of 128 paths.
//
// Compiled with -fmad=false: products and sums round separately as in the reference; exp is the
// deterministic rg_exp64 shared with the oracle.
#include "rg_internal.h"

namespace rg {

__global__ void __launch_bounds__(128) book_gen64_kernel(DevTrade gen, DevTables tb,
                                                         const double* __restrict__ L, int U,
                                                         uint64_t path0, uint64_t npaths,
                                                         double* __restrict__ incr) {
  const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= npaths * (uint64_t)U) return;
  const uint64_t p = i % npaths;
  const int u = (int)(i / npaths);
  const uint64_t point = path0 + p;
  const int64_t T = gen.steps;
  double wcur = 0.0, stk[RG_STACK_MAX];
  int sp = 0;
  for (int64_t t = 0; t < T; ++t) {
    const int c0 = __ldg(tb.node_off + t), c1 = __ldg(tb.node_off + t + 1);
    for (int c = c0; c < c1; ++c) {
      const int k = __ldg(tb.node_k + c);
      const double cc = __ldg(tb.node_c + c);
      double y = 0.0;
      for (int b = 0; b <= u; ++b)
        y += __ldg(L + u * U + b) * rg_qmc_normal64(gen, tb, point, (uint64_t)k * (uint64_t)U + (uint64_t)b);
      stk[sp] = c == 0 ? y * cc : 0.5 * (wcur + stk[sp - 1]) + y * cc;
      ++sp;
    }
    --sp;
    const double wn = stk[sp];
    incr[((uint64_t)t * U + u) * npaths + p] = (wn - wcur) * gen.inv_sqrt_dt;
    wcur = wn;
  }
}

void launch_book_gen64(const DevTrade& gen, const DevTables& tb, const double* L, int U,
                       uint64_t path0, uint64_t npaths, double* incr, cudaStream_t s) {
  const uint64_t n = npaths * (uint64_t)U;
  book_gen64_kernel<<<(unsigned)((n + 127) / 128), 128, 0, s>>>(gen, tb, L, U, path0, npaths, incr);
  cuda_check(cudaGetLastError(), "book_gen64_kernel launch");
}

__global__ void __launch_bounds__(128) book_trade64_kernel(DevTrade gen, BookDev bk,
                                                           const double* __restrict__ incr,
                                                           uint64_t path0, uint64_t npaths,
                                                           double* __restrict__ partial,
                                                           int blocks, rg_path_record* __restrict__ records) {
  __shared__ double red[128][RG_ACC + 1];
  const int tid = threadIdx.x;
  const int pair = (int)(blockIdx.x / (unsigned)blocks), blk = (int)(blockIdx.x % (unsigned)blocks);
  const int pairs = bk.n_trades * bk.S;
  const int j = pair / bk.S, s = pair % bk.S;
  const BookTradeDev& tr = bk.trades[j];
  const BookPair32& pc = bk.pair32[(size_t)j * bk.S + s];
  const BookScenDev& sc = bk.scen[pc.mkt];
  const uint64_t p = (uint64_t)blk * blockDim.x + tid;
  double out[RG_ACC];
#pragma unroll
  for (int k = 0; k < RG_ACC; ++k) out[k] = 0.0;
  if (p < npaths) {
    const int n = tr.n;
    const int64_t T = tr.T;
    const double dt = gen.dt, sqrt_dt = gen.sqrt_dt, rate = sc.rate;
    const int64_t periods = tr.periods;
    double spots[RG_NMAX], vol[RG_NMAX], qd[RG_NMAX];
    const double* row[RG_NMAX];
    for (int f = 0; f < n; ++f) {
      const int a = tr.idx[f];
      spots[f] = sc.spots[a];
      vol[f] = sc.vols[a];
      qd[f] = sc.q[a];
      row[f] = incr + (uint64_t)a * npaths + p;
    }
    const uint64_t step_stride = (uint64_t)bk.U * npaths;
    const double* df = bk.df + (size_t)pc.dfrow * bk.TU;
    int ko = 0, received = 0, ko_step = -1, qualified = 0, paid = 0;
    double accrual = 0.0, unpaid = 0.0, cpv = 0.0, mpv = 0.0, final_worst = 1.0;
    int64_t current = 0;
    for (int64_t t = 0; t < T; ++t) {
      // step (note.rs:133-142)
      for (int f = 0; f < n; ++f) {
        const double v = vol[f];
        const double drift = (rate - qd[f] - 0.5 * v * v) * dt;
        spots[f] *= rg_exp64(drift + v * sqrt_dt * row[f][(uint64_t)t * step_stride]);
      }
      double worst = spots[0] / tr.init[0];
      for (int f = 1; f < n; ++f) worst = fmin(worst, spots[f] / tr.init[f]);
      final_worst = worst;
      if (ko) continue;
      // Phoenix state machine (note.rs:150-218)
      int64_t period = (t * periods) / T;
      if (period > periods - 1) period = periods - 1;
      if (period != current) {
        current = period;
        accrual = 0.0;
      }
      const bool fixed = period == 0 && tr.fixed_first;
      if (!fixed && worst >= tr.coupon_barrier) {
        const int64_t a = T * (period + 1) / periods, b = T * period / periods;
        int64_t ps = a > b ? a - b : 0;
        if (ps < 1) ps = 1;
        accrual += tr.coupon_rate / (double)ps;
        ++qualified;
      }
      bool up = t >= tr.call_start;
      for (int f = 0; f < n; ++f) up = up && (spots[f] / tr.init[f] >= tr.call_barrier);
      if (up) {
        ko = 1;
        ko_step = (int)t;
        const double due = fixed ? tr.coupon_rate : accrual;
        const double carry = due > 0.0 ? unpaid : 0.0;
        if (due + carry > 0.0) {
          const double d = __ldg(df + t);
          cpv += due * d;
          mpv += carry * d;
          received = 1;
          ++paid;
        }
        continue;
      }
      int64_t next;
      if (t + 1 == T) {
        next = periods;
      } else {
        next = ((t + 1) * periods) / T;
        if (next > periods - 1) next = periods - 1;
      }
      if (t + 1 == T || next != period) {
        const double due = fixed ? tr.coupon_rate : accrual;
        if (due > 0.0) {
          const double d = __ldg(df + t);
          cpv += due * d;
          mpv += unpaid * d;
          received = 1;
          unpaid = 0.0;
          ++paid;
        } else if (tr.memory) {
          unpaid += tr.coupon_rate;
        }
      }
    }
    // path close (note.rs:221-258)
    const double dfm = bk.dfm[(size_t)j * bk.S + s];
    const double funding = ko ? __ldg(df + ko_step) : dfm;
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
    if (records) {
      rg_path_record r;
      r.path_id = path0 + p;
      r.rng_seed = gen.seed;
      r.sobol_index = path0 + p + 1;
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
      records[p * (uint64_t)pairs + pair] = r;
    }
  }
  // fixed-order tree over the block's 128 paths
#pragma unroll
  for (int k = 0; k < RG_ACC; ++k) red[tid][k] = out[k];
  __syncthreads();
  for (int w = 64; w > 0; w >>= 1) {
    if (tid < w)
      for (int k = 0; k < RG_ACC; ++k) red[tid][k] += red[tid + w][k];
    __syncthreads();
  }
  if (tid < RG_ACC) partial[((size_t)pair * blocks + blk) * RG_ACC + tid] = red[0][tid];
}

void launch_book_trade64(const DevTrade& gen, const BookDev& bk, const double* incr, uint64_t path0,
                         uint64_t npaths, double* partial, int blocks, rg_path_record* records,
                         cudaStream_t s) {
  const uint64_t grid = (uint64_t)blocks * (uint64_t)(bk.n_trades * bk.S);
  if (grid > 0x7fffffffULL) raise(RG_ERR_INVALID_ARGUMENT, "book too large for one FP64 launch");
  book_trade64_kernel<<<(unsigned)grid, 128, 0, s>>>(gen, bk, incr, path0, npaths, partial, blocks, records);
  cuda_check(cudaGetLastError(), "book_trade64_kernel launch");
}

}  // namespace rg
