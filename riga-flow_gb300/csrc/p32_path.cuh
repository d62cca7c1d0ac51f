// p32_path.cuh — the path close shared by the FP32 kernels (phoenix32.cu, phoenix32d.cu).
#pragma once
#include "rg_common.cuh"

namespace rg {

// The Phoenix state of one FP32 path of one scenario.
struct P32Phoenix {
  bool alive = true, received = false;
  int qual = 0, unpaid = 0, ko_step = -1, qualified = 0, paid = 0;
  float cpv = 0.0f, mpv = 0.0f;
};

// One step of the Phoenix state machine (crates/riga-engine/src/note.rs:150-218) for a live path:
// `fl` is the step's schedule flags, `wmin` the log worst-of performance after the step, `df` the
// scenario's discount factors by step, `period()` the step's coupon period (read only when a
// coupon is due).  Barriers compare in log space (ln_cb, ln_ko).
template <bool REC, class Period>
__device__ __forceinline__ void p32_phoenix_step(P32Phoenix& st, uint32_t fl, int t, float wmin, float ln_cb,
                                                 float ln_ko, const DevTrade& tr, const DevTables& tb,
                                                 const float* __restrict__ df, Period period) {
  if (fl & STEP_PERIOD_RESET) st.qual = 0;
  if ((fl & STEP_ACCRUE) && wmin >= ln_cb) {
    ++st.qual;
    if (REC) ++st.qualified;
  }
  if ((fl & STEP_CALL_ACTIVE) && wmin >= ln_ko) {
    st.alive = false;
    st.ko_step = t;
    const float due = (fl & STEP_FIXED_DUE) ? tr.coupon_f : (float)st.qual * __ldg(tb.accr_f + period());
    const float carry = due > 0.0f ? (float)st.unpaid * tr.coupon_f : 0.0f;
    if (due + carry > 0.0f) {
      const float d = __ldg(df + t);
      st.cpv = fmaf(due, d, st.cpv);
      st.mpv = fmaf(carry, d, st.mpv);
      st.received = true;
      if (REC) ++st.paid;
    }
  } else if (fl & STEP_PERIOD_END) {
    const float due = (fl & STEP_FIXED_DUE) ? tr.coupon_f : (float)st.qual * __ldg(tb.accr_f + period());
    if (due > 0.0f) {
      const float d = __ldg(df + t);
      st.cpv = fmaf(due, d, st.cpv);
      st.mpv = fmaf((float)st.unpaid * tr.coupon_f, d, st.mpv);
      st.unpaid = 0;
      st.received = true;
      if (REC) ++st.paid;
    } else if (tr.memory) {
      ++st.unpaid;
    }
  }
}

// Path close (crates/riga-engine/src/note.rs:221-258) of one FP32 path of scenario `sc`: its
// payoff values into out[RG_ACC] (zero when `ok` is false), and for scenario 0 (`first`) its KO
// step for the trace events and, in the records variant, its PathRecord (explain.rs:90-316) with
// the discounting and put in FP64 as the parity kernel forms them.
template <bool REC>
__device__ __forceinline__ void p32_close_path(const DevTrade& tr, const DevTables& tb, int sc, int T, bool ok,
                                               bool first, uint64_t path0, uint64_t gi, int ko_step, float worst,
                                               float ln_ki, float cpv, float mpv, bool received, int qualified,
                                               int paid, int32_t* __restrict__ ko_steps,
                                               rg_path_record* __restrict__ records, float (&out)[RG_ACC]) {
#pragma unroll
  for (int k = 0; k < RG_ACC; ++k) out[k] = 0.0f;
  if (!ok) return;
  const bool ko = ko_step >= 0;
  const float df_mat = __ldg(tb.df_mat_f + sc);
  const float funding = ko ? __ldg(tb.df_f + (size_t)sc * T + ko_step) : df_mat;
  const bool hit_ki = worst <= ln_ki;
  const bool put_ok = hit_ki && !ko;
  const float put = put_ok ? fmaxf(tr.strike_f - expf(worst), 0.0f) * df_mat : 0.0f;
  const float cn = cpv + mpv;
  const float pv1 = (funding - 1.0f) + cn - put;
  out[ACC_PV] = pv1;
  out[ACC_PV2] = pv1 * pv1;
  if (ko) {
    out[ACC_KOF] = funding - 1.0f;
    out[ACC_KOF2] = (funding - 1.0f) * (funding - 1.0f);
    out[ACC_NKO] = 1.0f;
  }
  if (hit_ki) {
    out[ACC_KIPUT] = put;
    out[ACC_KIPUT2] = put * put;
    out[ACC_NKI] = 1.0f;
  }
  if (received) {
    out[ACC_CPN] = cn;
    out[ACC_CPN2] = cn * cn;
    out[ACC_NCPN] = 1.0f;
  }
  out[ACC_PUT] = put;
  out[ACC_FUND] = funding;
  out[ACC_CQ] = cpv * 10.0f;
  out[ACC_MQ] = mpv * 10.0f;
  out[ACC_NPUT] = put_ok ? 1.0f : 0.0f;
  if (first && ko_steps) ko_steps[gi] = ko_step;
  if (REC && first && records) {
    const double df_mat64 = __ldg(tb.df_mat + sc);
    const double funding64 = ko ? __ldg(tb.df + (size_t)sc * T + ko_step) : df_mat64;
    const double wf = exp((double)worst);
    const double put64 = put_ok ? fmax(tr.strike - wf, 0.0) * df_mat64 : 0.0;
    const double cn64 = (double)cpv + (double)mpv;
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
    r.put_payoff = put64;
    r.coupon_pv = cn64;
    r.memory_coupon_pv = (double)mpv;
    r.funding = funding64;
    r.pv = funding64 + cn64 - put64;
    records[gi] = r;
  }
}

}  // namespace rg
