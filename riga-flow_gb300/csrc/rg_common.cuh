// rg_common.cuh — shared device definitions for the GB300 Phoenix engine (sm_103a).
//
// Layout of everything the fused kernels read lives here: the per-trade step schedule, the
// per-scenario market block, the Brownian-bridge node schedule and the QMC tables.  All tables
// are built once per request on the host (integer/FP64 work) or by the FP64 prologue kernels
// (Cholesky, Dupire calibration) and stay resident in HBM for every kernel of the request.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/riga_gb300.h"
#include "rg_math.cuh"

#define RG_NMAX RG_MAX_ASSETS
#define RG_ACC 16          // FP64 accumulators per (block, scenario)
#define RG_STACK_MAX 24    // Brownian-bridge anchor stack depth (T <= 2^22)
#define RG_MAX_SCEN 64     // scenarios in one fused CRN launch
#define RG_BPLAN_MAX 8     // tile depths with a bridge plan: the formula depth and the tuner's candidates

// Accumulator slots (per scenario).  Second moments are of shifted values so that the FP64
// sums keep their precision: pv and KO funding are shifted by 1.
enum {
  ACC_PV = 0, ACC_PV2, ACC_KOF, ACC_KOF2, ACC_KIPUT, ACC_KIPUT2, ACC_CPN, ACC_CPN2,
  ACC_PUT, ACC_FUND, ACC_CQ, ACC_MQ, ACC_NKO, ACC_NKI, ACC_NPUT, ACC_NCPN
};

// Per-step flags of the Phoenix schedule (note.rs:150-218), identical for every path.
enum : uint32_t {
  STEP_PERIOD_END = 1u,    // a coupon period closes at this step
  STEP_CALL_ACTIVE = 2u,   // step >= call_start_step
  STEP_ACCRUE = 4u,        // daily accrual allowed (not the fixed first period)
  STEP_PERIOD_RESET = 8u,  // the period index changed at this step
  STEP_FIXED_DUE = 16u     // the due amount is the fixed coupon (period 0, fixed first coupon)
};

struct DevTrade {
  int32_t n, vr, scrambler, has_lv;
  int64_t steps, periods;
  int64_t sob_dim;     // rows of the Sobol table (the wrap modulus)
  int32_t hal_dim;
  int32_t hal_hash;    // 1: the production Halton lane (hashed affine digit scrambling, no wrap)
  int32_t gx;          // Dupire log-strike points
  uint64_t seed;
  double dt, sqrt_dt, inv_sqrt_dt, maturity;
  double init[RG_NMAX];
  double call_barrier, coupon_barrier, coupon_rate, strike, ki;
  float coupon_f, strike_f;  // coupon_rate and strike rounded to FP32 for the FP32 kernels
  float neg_half_dt_f;       // -dt / 2 rounded to FP32 (the FP32 kernels' Euler drift term)
  int32_t memory;
};

struct DevScenario {
  double spots[RG_NMAX], vols[RG_NMAX], q[RG_NMAX];
  double rate;
  double L[RG_NMAX * RG_NMAX];  // written by the FP64 Cholesky kernel
  int32_t surf[RG_NMAX];         // calibrated Dupire surface per asset (-1 = flat vol)
  int32_t surf_off[RG_NMAX];     // first cell of that surface in the packed local-vol grids
  int32_t status;                // Cholesky status
};

// Device pointers of one request's resident tables.
struct DevTables {
  const uint32_t* sobol;       // [sob_dim][32]
  const uint32_t* hal_base;    // [hal_dim]
  const uint32_t* hal_off;     // [hal_dim] offsets into hal_perm
  const uint32_t* hal_perm;
  const uint32_t* step_flags;  // [T]
  const int32_t* step_period;  // [T]
  const double* accr_inc;      // [periods] coupon_rate / period_steps
  const int32_t* node_off;     // [T+1] first bridge node consumed at step t
  const int32_t* node_k;       // [T] preorder index (QMC step) of each node, consumption order
  const double* node_c;        // [T] bridge standard deviation of each node
  const float* node_cf;        // [T] the same in FP32
  const int32_t* nf_row;       // [T][n] Sobol table row of (node, factor)
  const uint32_t* nf_shift;    // [T][n] digital-shift mask of (node, factor)
  const int2* lv_ti;           // [n][T] (tenor row at or below step t's time, next row)
  const double* lv_tw;         // [n][T] tenor weight
  const float* lv_twf;         // [n][T] tenor weight in FP32
  const double* lv_v;          // [surfaces][n_t][gx] FP64 local vol
  const float2* lv_vf;         // [surfaces][n_t][gx] (v, v[j+1]-v[j]) FP32
  const float2* lv_rows;       // [surfaces][T][gx] the row at each step's time: cell j's line (c, d) in
                               // the grid position u in [0, 1], v = c + u·d, FP32
  const double* lv_logs;       // [surfaces][gx] log-strike axis
  const double* df;            // [scenarios][T] exp(-r_s * (t+1) dt)
  const double* df_mat;        // [scenarios] exp(-r_s * maturity)
  const float* accr_f;         // accr_inc, df and df_mat rounded to FP32 for the FP32 kernels
  const float* df_f;
  const float* df_mat_f;
  int32_t lv_nt;
  // the direct FP32 kernel's Sobol tables in consumption order q = node·n + factor (phoenix32d.cu):
  // directions transposed [32][n·T], and per q the 32 lanes' low-bit terms for points starting at
  // offset sob_lut_o within a 32-point block (digital shift folded in); null when not staged
  const uint32_t* sob_t;
  const uint32_t* sob_lut;
  int32_t sob_nq, sob_lut_o;
  // level-ordered bridge plans of the FP32 tiled kernel (phoenix32.cu), one per tile depth
  const uint32_t* bplan;
  int32_t bplan_tt[RG_BPLAN_MAX], bplan_at[RG_BPLAN_MAX];
  int32_t n_bplan;
};

// ------------------------------------------------------------------ integer QMC primitives ----
__host__ __device__ __forceinline__ uint64_t rg_mix64(uint64_t z) {
  // SplitMix64 finaliser (crates/riga-engine/src/qmc.rs:310-314)
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
  return z ^ (z >> 31);
}

// Nested (Owen) scramble keyed on the scrambled prefix (qmc.rs:292-308).  The loop-invariant key
// part seed ^ dim*C1 is hoisted; bit*C2 is a running sum.
__device__ __forceinline__ uint32_t rg_owen(uint32_t x, uint64_t dim, uint64_t seed) {
  const uint64_t base = seed ^ (dim * 0x9E3779B97F4A7C15ULL);
  uint32_t result = 0, prefix = 0;
#pragma unroll 4
  for (int bit = 31; bit >= 0; --bit) {
    uint32_t b = (x >> bit) & 1u;
    uint64_t h = rg_mix64(base ^ ((uint64_t)bit * 0xD6E8FEB86659FD93ULL) ^
                          ((uint64_t)prefix * 0xA24BAED4963EE407ULL));
    uint32_t s = b ^ (uint32_t)(h >> 63);
    result |= s << bit;
    prefix = (prefix << 1) | s;
  }
  return result;
}

// Digital shift: the engine's production scrambler (one XOR mask per dimension).
__host__ __device__ __forceinline__ uint32_t rg_digital_shift(uint64_t dim, uint64_t seed) {
  return (uint32_t)(rg_mix64(seed ^ ((dim + 1) * 0xD1B54A32D192ED03ULL)) >> 32);
}

// Gray-code Sobol integer of 1-based point n: XOR of row[k] over the set bits of n ^ (n >> 1)
// (qmc.rs:269-279: an odd count (n>>k)-(n>>(k+1)) is exactly bit k of the Gray code).
__device__ __forceinline__ uint32_t rg_sobol_gray(const uint32_t* __restrict__ row, uint64_t n) {
  uint64_t g = n ^ (n >> 1);
  uint32_t x = 0;
  uint32_t gl = (uint32_t)g;
  while (gl) {
    int k = __ffs(gl) - 1;
    x ^= __ldg(row + k);
    gl &= gl - 1;
  }
  return x;
}

// Sobol integers x(n1 + lane) of one QMC dimension (direction numbers `row`) for the 32 lanes of a
// warp: x(n1) is the XOR of the direction numbers at the set bits of n1's Gray code (lane k
// contributes bit k, a shuffle reduction), and x(n1 + lane) follows by the Gray recurrence
// x(n) = x(n-1) ^ v[ctz(n)] as an inclusive XOR scan over the lanes.  All 32 lanes must call it.
__device__ __forceinline__ uint32_t rg_warp_sobol(const uint32_t* __restrict__ row, uint64_t n1, int lane) {
  const uint32_t g = (uint32_t)(n1 ^ (n1 >> 1));
  uint32_t v = ((g >> lane) & 1u) ? __ldg(row + lane) : 0u;
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) v ^= __shfl_xor_sync(0xffffffffu, v, off);
  // lanes past the request's last point may reach n = 2^32 (ctz 32); their values are never used
  uint32_t d = lane == 0 ? v : __ldg(row + ((__ffsll((long long)(n1 + (uint64_t)lane)) - 1) & 31));
#pragma unroll
  for (int off = 1; off < 32; off <<= 1) {
    const uint32_t t = __shfl_up_sync(0xffffffffu, d, off);
    if (lane >= off) d ^= t;
  }
  return d;
}

// ------------------------------------------------------------------ inverse normal ------------
// Acklam's rational approximation (qmc.rs:37-91), FP64, reference operation order.
__device__ __forceinline__ double rg_probit64(double p) {
  const double a0 = -3.969683028665376e1, a1 = 2.209460984245205e2, a2 = -2.759285104469687e2,
               a3 = 1.383577518672690e2, a4 = -3.066479806614716e1, a5 = 2.506628277459239e0;
  const double b0 = -5.447609879822406e1, b1 = 1.615858368580409e2, b2 = -1.556989798598866e2,
               b3 = 6.680131188771972e1, b4 = -1.328068155288572e1;
  const double c0 = -7.784894002430293e-3, c1 = -3.223964580411365e-1, c2 = -2.400758277161838e0,
               c3 = -2.549732539343734e0, c4 = 4.374664141464968e0, c5 = 2.938163982698783e0;
  const double d0 = 7.784695709041462e-3, d1 = 3.224671290700398e-1, d2 = 2.445134137142996e0,
               d3 = 3.754408661907416e0;
  if (p <= 0.0) return -INFINITY;
  if (p >= 1.0) return INFINITY;
  const double plow = 0.02425, phigh = 1.0 - plow;
  if (p < plow) {
    double q = sqrt(-2.0 * rg_log64(p));
    return (((((c0 * q + c1) * q + c2) * q + c3) * q + c4) * q + c5) /
           ((((d0 * q + d1) * q + d2) * q + d3) * q + 1.0);
  } else if (p <= phigh) {
    double q = p - 0.5, r = q * q;
    return (((((a0 * r + a1) * r + a2) * r + a3) * r + a4) * r + a5) * q /
           (((((b0 * r + b1) * r + b2) * r + b3) * r + b4) * r + 1.0);
  } else {
    double q = sqrt(-2.0 * rg_log64(1.0 - p));
    return -(((((c0 * q + c1) * q + c2) * q + c3) * q + c4) * q + c5) /
           ((((d0 * q + d1) * q + d2) * q + d3) * q + 1.0);
  }
}

// -Φ^-1(p) >= 0 in FP32 for a lower-tail probability p in [1e-12, 1/2], given p2 = 2p and
// s = 1 - 2p (each formed exactly or to FP32 rounding by the caller).  With
// w = -ln(4p(1-p)) = -ln(p2·(1 + s)), -Φ^-1(p) = s · g(w) for a smooth g (g(0) = sqrt(π/2)); g is
// this project's own near-minimax polynomial fit (csrc/probit32_fit.py): degree 8 in w - 2.5 for
// w < 5 (p >= 0.0017, 99.6% of draws, so nearly every warp stays on one branch) and degree 11 in
// sqrt(w) - 3.7161102 beyond.  No division, one fast logarithm, no FP64; within 4e-7 relative of
// the exact inverse normal, which the reference's Acklam approximation (qmc.rs:37-91) matches to
// 1.15e-9.
__device__ __forceinline__ float rg_ninv32_lower(float p2, float s) {
  const float w = -__logf(fmaf(p2, s, p2));
  float g;
  if (w < 5.0f) {
    const float t = w - 2.5f;
    g = 4.035466097e-08f;
    g = fmaf(g, t, 4.861039695e-07f);
    g = fmaf(g, t, -4.990565522e-06f);
    g = fmaf(g, t, -6.217993119e-06f);
    g = fmaf(g, t, 3.091502040e-04f);
    g = fmaf(g, t, -1.773010155e-03f);
    g = fmaf(g, t, -5.908170971e-03f);
    g = fmaf(g, t, 3.488026599e-01f);
    g = fmaf(g, t, 2.123313567e+00f);
  } else {
    const float v = sqrtf(w) - 3.716110200f;
    g = 5.467908077e-06f;
    g = fmaf(g, v, -1.174909974e-05f);
    g = fmaf(g, v, -2.363354380e-05f);
    g = fmaf(g, v, 9.947906459e-05f);
    g = fmaf(g, v, -1.555746239e-04f);
    g = fmaf(g, v, 2.347132999e-04f);
    g = fmaf(g, v, -4.239792245e-04f);
    g = fmaf(g, v, 8.495624679e-04f);
    g = fmaf(g, v, -1.928687814e-03f);
    g = fmaf(g, v, 3.093904488e-03f);
    g = fmaf(g, v, 1.426282266e+00f);
    g = fmaf(g, v, 5.025157229e+00f);
  }
  return s * g;
}

// The FP32 inverse normal of u = (x + 1/2) / 2^32: twice the lower-tail probability
// p = min(u, 1 - u) and s = 1 - 2p formed from x or ~x (s from the integer distance to the centre,
// exact for points near it), rg_ninv32_lower, and the sign by symmetry.  It tracks the exact inverse normal, so
// the FP32 lanes' normals agree with the FP64 lanes' Acklam normals to a few FP32 ulps.
__device__ __forceinline__ float rg_probit32(uint32_t x) {
  const bool lower = x < 0x80000000u;
  const uint32_t xl = lower ? x : ~x;
  const float p2 = fmaf((float)xl, 4.656612873077393e-10f, 2.3283064365386963e-10f);
  const float s = fmaf((float)(0x7FFFFFFFu - xl), 4.656612873077393e-10f, 2.3283064365386963e-10f);
  const float q = rg_ninv32_lower(p2, s);
  return lower ? -q : q;
}

// ------------------------------------------------------------------ Halton -------------------
// Digit-permuted radical inverse (qmc.rs:143-153) in FP64.
__device__ __forceinline__ double rg_halton_u(uint64_t index, uint32_t base, const uint32_t* perm) {
  double inv = 1.0 / (double)base, factor = inv, result = 0.0;
  while (index > 0) {
    result += factor * (double)__ldg(perm + (index % base));
    index /= base;
    factor *= inv;
  }
  return result;
}

// The QMC integer for (point, dim) before the probit: scrambled Sobol (Owen or digital shift).
__device__ __forceinline__ uint32_t rg_sobol_scrambled(const DevTrade& tr, const uint32_t* __restrict__ sobol,
                                                       uint64_t point, uint64_t dim) {
  const uint32_t* row = sobol + 32 * (dim % (uint64_t)tr.sob_dim);
  uint32_t x = rg_sobol_gray(row, point + 1);
  return tr.scrambler == RG_SCRAMBLE_DIGITAL_SHIFT ? x ^ rg_digital_shift(dim, tr.seed)
                                                   : rg_owen(x, dim, tr.seed);
}

// The production Halton lane (dimension mode "full"; the engine's own construction, with no
// counterpart in the reference, whose Halton lane wraps at its first 512 primes): dimension d uses
// the (d+1)-th prime b and no wrap; the point's base-b digits (least significant first, digit i)
// are each scrambled by the affine map x -> (a·x + c) mod b, with a in [1, b-1] and c in [0, b-1]
// drawn from a SplitMix64 hash of (seed, d, i); u = Σ σ_i(d_i) b^-(i+1) formed exactly as an
// integer over b^k.  Random affine digit scrambling decorrelates the high bases, whose first digits
// would otherwise rise in lockstep along the points.
__host__ __device__ __forceinline__ uint64_t rg_halton_key(uint64_t seed, uint64_t dim) {
  return seed ^ ((dim + 1) * 0xA0761D6478BD642FULL);
}
// The scrambled radical inverse as the exact fraction R / Bk (Bk = b^k, k the point's digit count).
__host__ __device__ __forceinline__ void rg_halton_hashed_rb(uint32_t n, uint32_t b, uint64_t key, uint64_t& R_,
                                                             uint64_t& Bk_) {
  uint64_t R = 0, Bk = 1;
  for (uint32_t i = 0; n; ++i) {
    const uint32_t q = n / b, d = n - q * b;
    const uint64_t h = rg_mix64(key ^ ((uint64_t)(i + 1) * 0xE7037ED1A0B428DBULL));
    const uint64_t a = 1u + ((uint64_t)(uint32_t)h * (uint64_t)(b - 1u) >> 32);
    const uint64_t cc = (h >> 32) * (uint64_t)b >> 32;
    // exact either way; 32-bit arithmetic while a·d + c fits (bases below 2^16)
    R = R * b + (b < 65536u ? (uint64_t)((uint32_t)(a * d + cc) % b) : (a * d + cc) % b);
    Bk *= b;
    n = q;
  }
  R_ = R;
  Bk_ = Bk;
}
__host__ __device__ __forceinline__ double rg_halton_hashed_u(uint32_t n, uint32_t b, uint64_t key) {
  uint64_t R, Bk;
  rg_halton_hashed_rb(n, b, key, R, Bk);
  return (double)R / (double)Bk;
}

// The FP32 inverse normal of u = R / Bk: twice the lower-tail probability p = min(R, Bk - R) / Bk
// and s = |Bk - 2R| / Bk formed in FP32 from the exact integers by one reciprocal (no FP64), p
// clamped below at the reference's 1e-12, rg_ninv32_lower and the sign by symmetry (as
// rg_probit32).
__device__ __forceinline__ float rg_probit32_frac(uint64_t R, uint64_t Bk) {
  const bool lower = 2 * R < Bk;
  const float inv = __frcp_rn((float)Bk);
  const float p2 = fmaxf((float)(2 * (lower ? R : Bk - R)) * inv, 2.0e-12f);
  const float s = (float)(lower ? Bk - 2 * R : 2 * R - Bk) * inv;
  const float q = rg_ninv32_lower(p2, s);
  return lower ? -q : q;
}

// FP64 normal of the QMC lanes (Ladder::normal, qmc.rs:119-125, 284-289).
__device__ __forceinline__ double rg_qmc_normal64(const DevTrade& tr, const DevTables& tb,
                                                  uint64_t point, uint64_t dim) {
  double u;
  if (tr.vr == RG_VR_SOBOL) {
    uint32_t x = rg_sobol_scrambled(tr, tb.sobol, point, dim);
    u = ((double)x + 0.5) / 4294967296.0;
  } else if (tr.hal_hash) {
    u = rg_halton_hashed_u((uint32_t)(point + 1), __ldg(tb.hal_base + dim), rg_halton_key(tr.seed, dim));
  } else {
    uint32_t idx = (uint32_t)(dim % (uint64_t)tr.hal_dim);
    u = rg_halton_u(point + 1, __ldg(tb.hal_base + idx), tb.hal_perm + __ldg(tb.hal_off + idx));
  }
  u = u < 1.0e-12 ? 1.0e-12 : (u > 1.0 - 1.0e-12 ? 1.0 - 1.0e-12 : u);
  return rg_probit64(u);
}

// The scrambled Halton normal of the FP32 lanes.  The reference's permuted radical inverse
// (qmc.rs:143-153) is the sum over the k digits d_i of the point (least significant first) of
// perm[d_i] / b^(i+1); here it is accumulated exactly as the integer R = Σ perm[d_i] b^(k-1-i)
// (Horner over the digits, 32-bit divisions) over b^k; then the FP32 inverse normal of the
// lower-tail probability min(R, b^k - R) / b^k (rg_probit32_frac: no FP64 operation), clamped
// below at 1e-12 as the reference's clamp of u to [1e-12, 1 - 1e-12].  The FP64 parity lane keeps
// the reference's own accumulation (rg_halton_u).
__device__ __forceinline__ float rg_halton_normal32(uint32_t n, uint32_t b, const uint32_t* __restrict__ perm) {
  uint64_t R = 0, Bk = 1;
  while (n) {
    const uint32_t q = n / b;
    R = R * b + __ldg(perm + (n - q * b));
    Bk *= b;
    n = q;
  }
  return rg_probit32_frac(R, Bk);
}

// FP32 normal of the QMC lanes.
__device__ __forceinline__ float rg_qmc_normal32(const DevTrade& tr, const DevTables& tb,
                                                 uint64_t point, uint64_t dim) {
  if (tr.vr == RG_VR_SOBOL) {
    uint32_t x = rg_sobol_scrambled(tr, tb.sobol, point, dim);
    return rg_probit32(x);
  }
  if (tr.hal_hash) {
    uint64_t R, Bk;
    rg_halton_hashed_rb((uint32_t)(point + 1), __ldg(tb.hal_base + dim), rg_halton_key(tr.seed, dim), R, Bk);
    return rg_probit32_frac(R, Bk);
  }
  const uint32_t idx = (uint32_t)(dim % (uint64_t)tr.hal_dim);
  return rg_halton_normal32((uint32_t)(point + 1), __ldg(tb.hal_base + idx), tb.hal_perm + __ldg(tb.hal_off + idx));
}

// ------------------------------------------------------------------ kernels (launchers) -------
struct DevRecordOut;  // forward

// Status word a kernel raises instead of trapping.
enum { KSTAT_OK = 0, KSTAT_BAD_LAUNCH = 1, KSTAT_TIMEOUT = 2 };
