// p32_tiled.cuh — the tiled FP32 CRN kernel (phoenix32_kernel): shared-memory layout, the kernel
// template and the entry points per (asset count, paths per thread).  Each pair's instantiations
// live in their own translation unit (phoenix32_n<N>p<PPT>.cu) so that they compile in parallel;
// the host side (shapes, bridge plans, autotuner, launch) is phoenix32.cu.
//
// The FP32 production kernel: one fused launch prices S common-random-number scenarios of one
// trade.
//
// A CTA owns Pb consecutive paths × Sb scenario slots (Sb = S rounded up to a power of two, at least
// 4; Pb = 1024 / Sb; a single scenario runs on the direct kernel of phoenix32d.cu).  In the
// stepping phase a thread serves one scenario and PPT paths: PPT = 2 (512 threads) steps a pair of
// paths in packed FP32x2 arithmetic (fma/add .f32x2, one instruction for both paths), PPT = 1
// (1024 threads) one path; a warp is 32·PPT paths of one scenario, so its local-vol lookups all
// read one surface.  Time is walked in tiles of TT steps, each in three phases separated by CTA
// barriers:
//   G. generation — warp-wide items (bridge node, 32-path group): the Sobol integers of the group's
//      32 consecutive points by a warp cooperation (rg_warp_sobol: shuffle reduction of the first
//      point's Gray code, XOR scan of the Gray recurrence), the digital shift (or Owen scramble) and
//      the FP32 inverse normal, for every factor; the standard normals of every node the tile
//      consumes land in shared memory, 32 consecutive floats per store.  The tile's step schedule
//      is staged beside them.
//   B. bridge — the tile's bridge nodes level by level from a host plan of the streamed Brownian
//      bridge's dependencies, each level's (node, factor, 32-path group) items spread over all
//      warps; then the uncorrelated increments dW[step][factor][path] and the state carried to
//      the next tile.
//   S. scenario stepping — every (path, scenario) correlates dW with its scenario's Cholesky
//      factor (the bridge is linear, so L·bridge(z) = bridge(L·z)), steps ln(S/S0) under flat vol
//      or its scenario's Dupire surface and runs the Phoenix state machine.
// Generation is paid once per path, not once per scenario.  Path state and a path's payoff values
// are FP32; each 32-path chunk is summed in FP32 by a fixed shuffle butterfly and written as FP64
// to partial[chunk][scenario], and the chunks are reduced in chunk order, so the sums — and the
// prices — are the same for every launch shape (paths per thread, tile depth, block).
#pragma once
#include "p32_path.cuh"
#include "rg_internal.h"

namespace rg {

// Byte offsets of the kernel's dynamic shared-memory regions, 16-byte aligned, and their total.
// Computed by the same function on the host (to size the launch) and in the kernel (to carve).
struct P32Layout {
  uint32_t flags, per, thr, noff, ncf, qmc, node4, plan, z, dw, total;
};

// Floats per row of the Z array: N·(Pb + 4) and one more, so that rows start in different banks.
__host__ __device__ inline int p32_zrow(int N, int Pb) { return N * (Pb + 4) + 1; }
// Floats per step of the dW array: odd for one path per thread, even for two, whose (path,
// path + 1) pairs are read as one aligned 8-byte load.
__host__ __device__ inline int p32_dwstep(int N, int Pb, int ppt) { return Pb * N + (ppt == 2 ? 2 : 1); }

__host__ __device__ inline P32Layout p32_layout(int N, int Pb, int TT, int NNmax, int stack_max, int ppt) {
  P32Layout L;
  uint32_t o = 0;
  auto put = [&o](uint32_t& field, uint32_t bytes) {
    field = o;
    o += (bytes + 15u) & ~15u;
  };
  // rows of p32_zrow(N, Pb) floats, factor f's paths at columns f·(Pb + 4) + path: the normals of
  // the tile's bridge nodes (rows 0 .. NNmax-1, overwritten by their bridge values), then the
  // bridge state carried between tiles: the value at the tile start (row NNmax) and the stack
  // (rows NNmax + 1 + slot)
  const uint32_t zb = (uint32_t)(NNmax + 1 + stack_max) * (uint32_t)p32_zrow(N, Pb) * 4u;
  put(L.flags, (uint32_t)TT * 4u);
  put(L.per, (uint32_t)TT * 4u);
  put(L.thr, (uint32_t)TT * 8u);  // per step (coupon threshold, knock-out threshold) or +inf
  put(L.noff, (uint32_t)(TT + 1) * 4u);
  put(L.ncf, (uint32_t)NNmax * 4u);
  // per (tile node, factor): Sobol row and digital-shift mask; per tile node: preorder index
  put(L.qmc, (uint32_t)NNmax * (uint32_t)(2 * N + 1) * 4u);
  // the tile's bridge plan: node words, level offsets, step codes, stack entries
  put(L.node4, (uint32_t)NNmax * 16u);  // per tile node in level order: Z offsets and coefficient
  put(L.plan, (uint32_t)(NNmax + (NNmax + 1) + (TT + 1) + stack_max) * 4u);
  put(L.z, zb);
  put(L.dw, (uint32_t)TT * (uint32_t)p32_dwstep(N, Pb, ppt) * 4u);  // dW[step][factor][path]
  L.total = o;
  return L;
}

// PPT path values of one thread: a float (one path per thread) or a float pair (two), so that the
// stepping arithmetic of two paths issues as one packed FP32x2 instruction (__ffma2_rn etc.).
template <int PPT> struct PVec;
template <> struct PVec<1> {
  float v[1];
  __device__ __forceinline__ static PVec splat(float a) { return {{a}}; }
  __device__ __forceinline__ static PVec fma(PVec a, PVec b, PVec c) { return {{fmaf(a.v[0], b.v[0], c.v[0])}}; }
  __device__ __forceinline__ static PVec fma_rd(PVec a, PVec b, PVec c) { return {{__fmaf_rd(a.v[0], b.v[0], c.v[0])}}; }
  __device__ __forceinline__ static PVec add(PVec a, PVec b) { return {{a.v[0] + b.v[0]}}; }
};
template <> struct PVec<2> {
  float v[2];
  __device__ __forceinline__ static PVec splat(float a) { return {{a, a}}; }
  __device__ __forceinline__ static PVec from(float2 f) { return {{f.x, f.y}}; }
  __device__ __forceinline__ float2 f2() const { return make_float2(v[0], v[1]); }
  __device__ __forceinline__ static PVec fma(PVec a, PVec b, PVec c) { return from(__ffma2_rn(a.f2(), b.f2(), c.f2())); }
  __device__ __forceinline__ static PVec fma_rd(PVec a, PVec b, PVec c) { return from(__ffma2_rd(a.f2(), b.f2(), c.f2())); }
  __device__ __forceinline__ static PVec add(PVec a, PVec b) { return from(__fadd2_rn(a.f2(), b.f2())); }
};

// The knock-out branch of the Phoenix state machine (p32_phoenix_step) for one live path.
template <bool REC>
__device__ __forceinline__ void p32_knock_out(P32Phoenix& st, uint32_t fl, int t, const DevTrade& tr,
                                              const DevTables& tb, const float* __restrict__ df, int period) {
  st.alive = false;
  st.ko_step = t;
  const float due = (fl & STEP_FIXED_DUE) ? tr.coupon_f : (float)st.qual * __ldg(tb.accr_f + period);
  const float carry = due > 0.0f ? (float)st.unpaid * tr.coupon_f : 0.0f;
  if (due + carry > 0.0f) {
    const float d = __ldg(df + t);
    st.cpv = fmaf(due, d, st.cpv);
    st.mpv = fmaf(carry, d, st.mpv);
    st.received = true;
    if (REC) ++st.paid;
  }
}

// Phase clocks, a build option (RG_PHASE_CLOCKS, see riga_gb300/build.py): thread 0 of every CTA
// reads clock64 at each phase boundary — the CTA's wall time in generation (0), bridge (1),
// stepping (2) and path close (3) — and adds its totals to g_p32_phase_clocks at exit
// (rg_phase_clocks).  Off in the product build.
#ifdef RG_PHASE_CLOCKS
static __device__ unsigned long long g_p32_phase_clocks[4];  // one per translation unit
#define RG_PHASE_BEGIN()                        \
  unsigned long long rg_pc[4] = {0, 0, 0, 0}; \
  long long rg_pt = clock64();
#define RG_PHASE_MARK(k)                                \
  if (threadIdx.x == 0) {                               \
    const long long rg_now = clock64();                 \
    rg_pc[k] += (unsigned long long)(rg_now - rg_pt);   \
    rg_pt = rg_now;                                     \
  }
#define RG_PHASE_END()         \
  if (threadIdx.x == 0)        \
    for (int rg_k = 0; rg_k < 4; ++rg_k) atomicAdd(&g_p32_phase_clocks[rg_k], rg_pc[rg_k]);
#else
#define RG_PHASE_BEGIN()
#define RG_PHASE_MARK(k)
#define RG_PHASE_END()
#endif

// This translation unit's phase clocks (the kernels of one asset count).
static inline int p32_phase_clocks_tu(unsigned long long out[4], bool reset) {
#ifdef RG_PHASE_CLOCKS
  cuda_check(cudaMemcpyFromSymbol(out, g_p32_phase_clocks, sizeof(unsigned long long) * 4), "phase clocks");
  if (reset) {
    const unsigned long long zero[4] = {0, 0, 0, 0};
    cuda_check(cudaMemcpyToSymbol(g_p32_phase_clocks, zero, sizeof zero), "phase clocks");
  }
  return 1;
#else
  (void)out;
  (void)reset;
  return 0;
#endif
}

template <int N, bool LV, bool REC, int PPT>
__global__ void __launch_bounds__(PPT == 1 ? 1024 : 512, 1) phoenix32_kernel(
    DevTrade tr, DevTables tb, const DevScenario* __restrict__ scen,
    const DevScen32* __restrict__ scen32, int S, int Pb, int TT, int NNmax, int stack_max,
    float ln_ko, float ln_cb, float ln_ki, uint64_t path0, uint64_t npaths, const uint32_t* __restrict__ plan,
    double* __restrict__ partial, int32_t* __restrict__ ko_steps, rg_path_record* __restrict__ records) {
  using V = PVec<PPT>;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int tid = threadIdx.x, lane = tid & 31;
  const int lg_pb = __ffs(Pb) - 1;  // Pb is a power of two, at least 32
  const int zs = p32_zrow(N, Pb);    // floats per Z row
  const int dws = p32_dwstep(N, Pb, PPT);
  const int T = (int)tr.steps;
  const uint64_t nchunks = (npaths + 31) / 32;
  // ---- shared-memory carve-up (the host sizes the launch from the same layout)
  const P32Layout L = p32_layout(N, Pb, TT, NNmax, stack_max, PPT);
  uint32_t dyn_bytes;
  asm("mov.u32 %0, %%dynamic_smem_size;" : "=r"(dyn_bytes));
  if (L.total > dyn_bytes) {
    // launched with less shared memory than the layout needs: touch none of it, poison the sums
    // of this block's first chunk so the host reports the launch as failed
    if ((uint64_t)blockIdx.x * Pb < npaths)
      for (int k = tid; k < S * RG_ACC; k += blockDim.x)
        partial[(size_t)((uint64_t)blockIdx.x * Pb / 32) * S * RG_ACC + k] = __longlong_as_double(0x7ff8000000000000LL);
    return;
  }
  uint32_t* s_flags = reinterpret_cast<uint32_t*>(smem_raw + L.flags);
  int32_t* s_per = reinterpret_cast<int32_t*>(smem_raw + L.per);
  float2* s_thr = reinterpret_cast<float2*>(smem_raw + L.thr);
  int32_t* s_noff = reinterpret_cast<int32_t*>(smem_raw + L.noff);
  float* s_ncf = reinterpret_cast<float*>(smem_raw + L.ncf);
  uint32_t* s_nfrow = reinterpret_cast<uint32_t*>(smem_raw + L.qmc);  // [node][factor]
  uint32_t* s_nfsh = s_nfrow + NNmax * N;                              // [node][factor]
  uint32_t* s_nodek = s_nfsh + NNmax * N;                              // [node]
  // node q of the tile in level order: (its Z row offset, left and right anchor row offsets, cf bits),
  // bit 31 of the first field set for the bridge's first node (no anchors)
  int4* s_node4 = reinterpret_cast<int4*>(smem_raw + L.node4);
  uint32_t* s_pnode = reinterpret_cast<uint32_t*>(smem_raw + L.plan);
  uint32_t* s_plev = s_pnode + NNmax;
  int32_t* s_poff = reinterpret_cast<int32_t*>(s_plev + NNmax + 1);  // Z row offset of W at step k (k = 0: tile start)
  uint32_t* s_pstk = reinterpret_cast<uint32_t*>(s_poff + TT + 1);
  float* Z = reinterpret_cast<float*>(smem_raw + L.z);
  float* dW = reinterpret_cast<float*>(smem_raw + L.dw);

  // stepping: thread tid serves scenario s and paths pl0 .. pl0 + PPT - 1 of each tile
  const int tps = Pb / PPT;  // threads per scenario
  const int s = tid / tps, pl0 = (tid % tps) * PPT;
  const bool lane_ok = s < S;
  const int ss = lane_ok ? s : 0;
  // a warp whose first thread has no scenario (padded scenario slots) skips the stepping phase
  const bool warp_on = ((tid & ~31) / tps) < S;
  const int gx = tr.gx;
  const V gxm1 = V::splat((float)(gx - 1));
  const V two23 = V::splat(8388608.0f);
  const V nhdt = V::splat(tr.neg_half_dt_f);
  // generation and bridge: warp-wide items over 32-path groups of the tile
  const int ngrp = Pb >> 5, lg_ngrp = lg_pb - 5;
  const int nwarp = (int)(blockDim.x >> 5), wid = tid >> 5;

  // scenario constants in registers: the Cholesky factor, drifts, flat vols and the per-asset
  // local-vol lookup constants (a_u/(gx-1), inv_h/(gx-1), row offset - 0x4B000000, x0)
  V Lf[N * (N + 1) / 2], mu[N], sig[N];
  float lva[N], lvb[N], x0[N];
  uint32_t lvo[N];
  {
    const DevScen32& s3 = scen32[ss];
    const float inv_gxm1 = 1.0f / (float)(gx - 1);
    int q = 0;
#pragma unroll
    for (int a = 0; a < N; ++a)
#pragma unroll
      for (int b = 0; b <= a; ++b) Lf[q++] = V::splat(s3.L[a * N + b]);
#pragma unroll
    for (int f = 0; f < N; ++f) {
      mu[f] = V::splat(s3.mu_dt[f]);
      sig[f] = V::splat(s3.sig[f]);
      lva[f] = s3.a_u[f] * inv_gxm1;
      lvb[f] = s3.inv_h[f] * inv_gxm1;
      lvo[f] = (uint32_t)s3.surf_off[f] - 0x4B000000u;
      x0[f] = s3.x0[f];
    }
  }
  const float* __restrict__ dfs = tb.df_f + (size_t)ss * T;

  // Sobol points from the staged consumption-order tables (as phoenix32d.cu) when they were built
  // for this launch's offset within a 32-point block; a lane's point may lie in the next block
  const bool sob_lut = tr.vr == RG_VR_SOBOL && tb.sob_lut != nullptr && (int32_t)((path0 + 1) & 31) == tb.sob_lut_o;
  const bool upper = (uint32_t)tb.sob_lut_o + (uint32_t)lane >= 32u;
  RG_PHASE_BEGIN();
  const uint64_t ntiles = (npaths + Pb - 1) / Pb;
  for (uint64_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    const uint64_t tile0 = tile * Pb;
    for (int i = tid; i < zs; i += blockDim.x) Z[(size_t)NNmax * zs + i] = 0.0f;  // W(0)
    bool ok[PPT];
    V x[N];
    P32Phoenix ph[PPT];
    float worst[PPT];
#pragma unroll
    for (int j = 0; j < PPT; ++j) {
      ok[j] = lane_ok && tile0 + pl0 + j < npaths;
      ph[j].alive = ok[j];
      worst[j] = 0.0f;
    }
#pragma unroll
    for (int f = 0; f < N; ++f) x[f] = V::splat(x0[f]);
    for (int t0 = 0; t0 < T; t0 += TT) {
      const int tn = min(TT, T - t0);
      const int n0 = __ldg(tb.node_off + t0), n1 = __ldg(tb.node_off + t0 + tn);
      const int nn = n1 - n0;
      // ---- G: standard normals of the tile's bridge nodes, and the tile's step schedule
      for (int i = tid; i < tn; i += blockDim.x) {
        const uint32_t fl = __ldg(tb.step_flags + t0 + i);
        s_flags[i] = fl;
        s_per[i] = __ldg(tb.step_period + t0 + i);
        s_thr[i] = make_float2((fl & STEP_ACCRUE) ? ln_cb : INFINITY, (fl & STEP_CALL_ACTIVE) ? ln_ko : INFINITY);
      }
      for (int i = tid; i <= tn; i += blockDim.x) s_noff[i] = __ldg(tb.node_off + t0 + i);
      for (int i = tid; i < nn; i += blockDim.x) {
        s_ncf[i] = __ldg(tb.node_cf + n0 + i);
        s_nodek[i] = (uint32_t)__ldg(tb.node_k + n0 + i);
      }
      if (tr.vr == RG_VR_SOBOL)
        for (int i = tid; i < nn * N; i += blockDim.x) {
          s_nfrow[i] = (uint32_t)__ldg(tb.nf_row + n0 * N + i);
          s_nfsh[i] = __ldg(tb.nf_shift + n0 * N + i);
        }
      __syncthreads();
      const uint32_t* hd = plan + 1 + (size_t)(t0 / TT) * 6;
      const uint32_t nlev = __ldg(hd + 2), stk_cnt = __ldg(hd + 4);
      {
        const uint32_t node_base = __ldg(hd), lev_base = __ldg(hd + 1), stk_base = __ldg(hd + 3),
                       steps_base = __ldg(hd + 5);
        for (int i = tid; i < nn; i += blockDim.x) {
          const uint32_t e = __ldg(plan + node_base + i);
          s_pnode[i] = e;
          s_node4[i] = make_int4((int)(e & 511u) * zs | (int)((e >> 27) << 31), (int)((e >> 9) & 511u) * zs,
                                 (int)((e >> 18) & 511u) * zs, __float_as_int(__ldg(tb.node_cf + n0 + (e & 511u))));
        }
        for (int i = tid; i <= (int)nlev; i += blockDim.x) s_plev[i] = __ldg(plan + lev_base + i);
        for (int i = tid; i <= tn; i += blockDim.x)
          s_poff[i] = i == 0 ? NNmax * zs : (int)__ldg(plan + steps_base + t0 + i - 1) * zs;
        for (int i = tid; i < (int)stk_cnt; i += blockDim.x) s_pstk[i] = __ldg(plan + stk_base + i);
      }
      // the high-bit Sobol terms X(gray(a)) of every (32-path group, tile dimension q), in the dW
      // region (free until the bridge phase): rows [group][block 0 / next block][q], q = jj·N + f;
      // a warp item is (group, 32 consecutive q), one coalesced row of transposed directions per
      // set bit of the group's gray(a)
      const int nq = nn * N, hs = ((nq + 31) & ~31) + 1;
      const bool lut_tile = sob_lut && ngrp * 2 * hs <= TT * dws;
      uint32_t* s_hq = reinterpret_cast<uint32_t*>(dW);
      if (lut_tile) {
        const int nb = (nq + 31) >> 5;
        for (int it = wid; it < ngrp * nb; it += nwarp) {
          const int hh = it / nb, ql = ((it - hh * nb) << 5) + lane;
          const uint64_t n1 = path0 + tile0 + ((uint64_t)hh << 5) + 1;
          const uint64_t a = n1 & ~(uint64_t)31;
          const uint32_t ga = (uint32_t)(a ^ (a >> 1));
          const int cw = __ffsll((long long)((n1 >> 5) + 1)) - 1 + 5;
          if (ql < nq) {
            const int q = n0 * N + ql;
            uint32_t h = 0;
            for (uint32_t g = ga; g; g &= g - 1u) h ^= __ldg(tb.sob_t + (size_t)(__ffs(g) - 1) * tb.sob_nq + q);
            s_hq[(hh * 2) * hs + ql] = h;
            s_hq[(hh * 2 + 1) * hs + ql] = h ^ __ldg(tb.sob_t + (size_t)cw * tb.sob_nq + q);
          }
        }
        __syncthreads();
      }
      {
        // kGB items per warp at a time in straight-line code, so that their global loads, shuffles
        // and inverse normals overlap (three: four spilled registers, measured 0.7% slower); a
        // warp's surplus slots recompute its last item (the same values stored twice), and items
        // of paths past the request compute values nobody reads
        constexpr int kGB = 3;
        const int nitems = nn << lg_ngrp;
        const bool shift_lane = tr.vr == RG_VR_SOBOL && tr.scrambler == RG_SCRAMBLE_DIGITAL_SHIFT;
        for (int base = wid; base < nitems; base += kGB * nwarp) {
          int jj[kGB], hh[kGB];
#pragma unroll
          for (int u = 0; u < kGB; ++u) {
            const int it = min(base + u * nwarp, nitems - 1);
            jj[u] = it >> lg_ngrp;
            hh[u] = it & (ngrp - 1);
          }
          if (lut_tile) {
            // x = the group's high-bit term (this lane's block) ^ the lane's low-bit term, with the
            // digital shift folded into the low-bit table
            uint32_t xs[kGB][N];
#pragma unroll
            for (int u = 0; u < kGB; ++u) {
              const int hb = (hh[u] * 2 + (upper ? 1 : 0)) * hs + jj[u] * N;
              const uint32_t* lt = tb.sob_lut + (size_t)(n0 + jj[u]) * N * 32 + lane;
#pragma unroll
              for (int f = 0; f < N; ++f) xs[u][f] = s_hq[hb + f] ^ __ldg(lt + f * 32);
            }
#pragma unroll
            for (int u = 0; u < kGB; ++u)
#pragma unroll
              for (int f = 0; f < N; ++f)
                Z[(size_t)jj[u] * zs + f * (Pb + 4) + (hh[u] << 5) + lane] =
                    rg_probit32(shift_lane ? xs[u][f] : rg_owen(xs[u][f], (uint64_t)s_nodek[jj[u]] * N + f, tr.seed));
          } else if (shift_lane) {
            uint32_t xs[kGB][N];
#pragma unroll
            for (int u = 0; u < kGB; ++u) {
              const uint64_t n1 = path0 + tile0 + ((uint64_t)hh[u] << 5) + 1;  // Sobol point of lane 0
#pragma unroll
              for (int f = 0; f < N; ++f)
                xs[u][f] = rg_warp_sobol(tb.sobol + 32 * (size_t)s_nfrow[jj[u] * N + f], n1, lane) ^ s_nfsh[jj[u] * N + f];
            }
#pragma unroll
            for (int u = 0; u < kGB; ++u)
#pragma unroll
              for (int f = 0; f < N; ++f)
                Z[(size_t)jj[u] * zs + f * (Pb + 4) + (hh[u] << 5) + lane] = rg_probit32(xs[u][f]);
          } else {
#pragma unroll
            for (int u = 0; u < kGB; ++u) {
              const uint64_t g0 = tile0 + ((uint64_t)hh[u] << 5);
              float* zo = Z + (size_t)jj[u] * zs + (hh[u] << 5) + lane;
              if (tr.vr == RG_VR_SOBOL) {
                const uint64_t n1 = path0 + g0 + 1;
#pragma unroll
                for (int f = 0; f < N; ++f) {
                  const uint32_t xs = rg_warp_sobol(tb.sobol + 32 * (size_t)s_nfrow[jj[u] * N + f], n1, lane);
                  zo[f * (Pb + 4)] = rg_probit32(rg_owen(xs, (uint64_t)s_nodek[jj[u]] * N + f, tr.seed));
                }
              } else {
#pragma unroll
                for (int f = 0; f < N; ++f)
                  zo[f * (Pb + 4)] = rg_qmc_normal32(tr, tb, path0 + g0 + lane, (uint64_t)s_nodek[jj[u]] * N + f);
              }
            }
          }
        }
      }
      __syncthreads();
      RG_PHASE_MARK(0);
      // ---- B: the tile's bridge nodes level by level from the plan (every node after its
      // anchors), W = z·c + (W_left + W_right) / 2 on the streamed bridge's anchors — so the
      // values are its values — each written over its normal in Z.  A chain (factor, path) is one
      // column of Z served by two lanes of one warp (16 chains a warp): each takes every other node
      // of a level, kB at a time loaded before any is stored (a level's nodes never read each
      // other), with a warp barrier between levels.  Then the chain's dW of every step (the two
      // lanes alternate steps), and the state it carries to the next tile (the value at the tile
      // end, the stack entries pushed in the tile).
      {
        constexpr int kB = 4;
        const int slot = lane >> 4;
        const int nch = N * Pb;  // chains
        for (int cb = wid * 16; cb < nch; cb += nwarp * 16) {
          const int ch = cb + (lane & 15);
          const bool chain_on = ch < nch;
          const int c = chain_on ? (ch >> lg_pb) * (Pb + 4) + (ch & (Pb - 1)) : 0;
          for (uint32_t lv = 0; lv < nlev; ++lv) {
            const int a = (int)s_plev[lv], b = (int)s_plev[lv + 1];
            for (int q = a + slot; q < b; q += 2 * kB) {
              float val[kB];
              int dst[kB];
#pragma unroll
              for (int u = 0; u < kB; ++u) {
                // surplus slots recompute the lane's last node of the level (the same value)
                const int qq = min(q + 2 * u, q + 2 * ((b - 1 - q) >> 1));
                const int4 nd = s_node4[qq];
                dst[u] = (nd.x & 0x7fffffff) + c;
                const float z = Z[dst[u]], cf = __int_as_float(nd.w);
                const float l = Z[nd.y + c], r = Z[nd.z + c];
                val[u] = nd.x < 0 ? z * cf : fmaf(z, cf, 0.5f * (l + r));
              }
              if (chain_on)
#pragma unroll
                for (int u = 0; u < kB; ++u) Z[dst[u]] = val[u];
            }
            __syncwarp();
          }
          float* dwc = dW + ch;
          for (int t1 = slot; t1 < tn; t1 += 2 * kB) {
            float dv[kB];
            int tt[kB];
#pragma unroll
            for (int u = 0; u < kB; ++u) {
              tt[u] = min(t1 + 2 * u, t1 + 2 * ((tn - 1 - t1) >> 1));
              dv[u] = Z[s_poff[tt[u] + 1] + c] - Z[s_poff[tt[u]] + c];
            }
            if (chain_on)
#pragma unroll
              for (int u = 0; u < kB; ++u) dwc[tt[u] * dws] = dv[u];
          }
          __syncwarp();
          if (chain_on && slot == 0) {
            const float wend = Z[s_poff[tn] + c];  // the value at the tile end
            for (uint32_t k = 0; k < stk_cnt; ++k) {
              const uint32_t e = s_pstk[k];  // (destination row, tile node)
              Z[(int)(e >> 9) * zs + c] = Z[(int)(e & 511u) * zs + c];
            }
            Z[NNmax * zs + c] = wend;
          }
        }
      }
      __syncthreads();
      RG_PHASE_MARK(1);
      // ---- S: scenario stepping.  Every thread of a warp with a scenario runs it (threads of
      // padded slots and paths past the request with their Phoenix state dead), so the
      // knock-out test can vote warp-wide.  Steps go in pairs: the Euler steps of both, then the
      // Phoenix machine of both in order, so that the second step's local-vol lookups overlap the
      // first step's barrier tests and one vote serves two steps.
      if (warp_on) {
        // one Euler step of every asset (correlated increment, local-vol lookup, log-space update);
        // returns the worst-of log performance of each path after the step
        auto euler = [&](int tt, float (&wmin)[PPT]) {
          const int tg = (t0 + tt) * gx;
          V d[N], y[N];
#pragma unroll
          for (int f = 0; f < N; ++f) {
            const float* dp = dW + tt * dws + f * Pb + pl0;
            if constexpr (PPT == 2) d[f] = V::from(*reinterpret_cast<const float2*>(dp));
            else d[f] = V::splat(*dp);
          }
          int q = 0;
#pragma unroll
          for (int a = 0; a < N; ++a) {
            V acc_y = V::fma(Lf[q++], d[0], V::splat(0.0f));
#pragma unroll
            for (int b = 1; b <= a; ++b) acc_y = V::fma(Lf[q++], d[b], acc_y);
            y[a] = acc_y;
          }
#pragma unroll
          for (int j = 0; j < PPT; ++j) wmin[j] = INFINITY;
#pragma unroll
          for (int f = 0; f < N; ++f) {
            V sg;
            if (LV) {
              // sigma at the step's time row, linear in log-spot.  u01 = the grid position scaled
              // to [0, 1], clamped by the FMA's saturation (NaN -> 0); 2^23 + floor(u01·(gx-1))
              // by one round-down FMA, whose bit pattern minus 0x4B000000 is the grid index —
              // that bias is folded into the row offset lvo; then one gather of the cell's line
              // (c, d) in u01 and sigma = c + u01·d
              V u01;
#pragma unroll
              for (int j = 0; j < PPT; ++j) u01.v[j] = __saturatef(fmaf(x[f].v[j], lvb[f], lva[f]));
              const V fl = V::fma_rd(u01, gxm1, two23);
#pragma unroll
              for (int j = 0; j < PPT; ++j) {
                const uint32_t idx = lvo[f] + (uint32_t)tg + (uint32_t)__float_as_int(fl.v[j]);
                const float2 r = __ldg(tb.lv_rows + idx);
                sg.v[j] = fmaf(u01.v[j], r.y, r.x);
              }
            } else {
              sg = sig[f];
            }
            x[f] = V::add(V::fma(sg, V::fma(nhdt, sg, y[f]), x[f]), mu[f]);
#pragma unroll
            for (int j = 0; j < PPT; ++j) wmin[j] = fminf(wmin[j], x[f].v[j]);
          }
        };
        // Phoenix state machine (note.rs:150-218) of one step in full: steps that reset or close a
        // coupon period take p32_phoenix_step; on the others a live path accrues and tests the
        // knock-out branch-free against the step's thresholds (+inf where the step does not accrue
        // or cannot call), and the knock-out branch runs when some path of the warp knocks out
        auto phoenix = [&](int tt, const float (&wmin)[PPT]) {
          const int t = t0 + tt;
          const uint32_t fl = s_flags[tt];
          if (fl & (STEP_PERIOD_RESET | STEP_PERIOD_END)) {
#pragma unroll
            for (int j = 0; j < PPT; ++j)
              if (ph[j].alive)
                p32_phoenix_step<REC>(ph[j], fl, t, wmin[j], ln_cb, ln_ko, tr, tb, dfs, [&] { return s_per[tt]; });
          } else {
            const float2 th = s_thr[tt];
            bool hit[PPT], any = false;
#pragma unroll
            for (int j = 0; j < PPT; ++j) {
              const bool a = ph[j].alive;
              const bool acc = a & (wmin[j] >= th.x);
              ph[j].qual += acc;
              if (REC) ph[j].qualified += acc;
              hit[j] = a & (wmin[j] >= th.y);
              any |= hit[j];
            }
            if (__any_sync(0xffffffffu, any)) {
#pragma unroll
              for (int j = 0; j < PPT; ++j)
                if (hit[j]) p32_knock_out<REC>(ph[j], fl, t, tr, tb, dfs, s_per[tt]);
            }
          }
        };
        int tt = 0;
        for (; tt + 1 < tn; tt += 2) {
          float w0[PPT], w1[PPT];
          euler(tt, w0);
          euler(tt + 1, w1);
#pragma unroll
          for (int j = 0; j < PPT; ++j) worst[j] = w1[j];
          const uint32_t f0 = s_flags[tt], f1 = s_flags[tt + 1];
          if ((f0 | f1) & (STEP_PERIOD_RESET | STEP_PERIOD_END)) {
            phoenix(tt, w0);
            phoenix(tt + 1, w1);
          } else {
            // two plain steps: when no path of the warp knocks out in either, both only accrue
            const float2 th0 = s_thr[tt], th1 = s_thr[tt + 1];
            bool any = false;
#pragma unroll
            for (int j = 0; j < PPT; ++j) any |= ph[j].alive & ((w0[j] >= th0.y) | (w1[j] >= th1.y));
            if (__any_sync(0xffffffffu, any)) {
              phoenix(tt, w0);
              phoenix(tt + 1, w1);
            } else {
#pragma unroll
              for (int j = 0; j < PPT; ++j) {
                const bool a = ph[j].alive;
                const int acc = (int)(a & (w0[j] >= th0.x)) + (int)(a & (w1[j] >= th1.x));
                ph[j].qual += acc;
                if (REC) ph[j].qualified += acc;
              }
            }
          }
        }
        if (tt < tn) {
          float w0[PPT];
          euler(tt, w0);
#pragma unroll
          for (int j = 0; j < PPT; ++j) worst[j] = w0[j];
          phoenix(tt, w0);
        }
      }
      __syncthreads();
      RG_PHASE_MARK(2);
    }
    // ---- path close (note.rs:221-258) and the sums of each 32-path chunk: FP32 values per path,
    // a fixed FP32 shuffle butterfly over the chunk (path offsets 16, 8, 4, 2, 1 — with two paths
    // per thread the last offset is the thread's own pair, so the tree is the same), the chunk's
    // 16 sums as FP64 to partial[chunk][scenario] by its first 16 lanes.  The chunk sums, and the
    // reduction over chunks in chunk order, do not depend on the launch shape.
    if (warp_on) {
      float out[PPT][RG_ACC];
#pragma unroll
      for (int j = 0; j < PPT; ++j)
        p32_close_path<REC>(tr, tb, ss, T, ok[j], s == 0, path0, tile0 + pl0 + j, ph[j].ko_step, worst[j],
                            ln_ki, ph[j].cpv, ph[j].mpv, ph[j].received, ph[j].qualified, ph[j].paid,
                            ko_steps, records, out[j]);
      constexpr int LG = 32 / PPT;  // lanes per chunk
      for (int off = LG >> 1; off > 0; off >>= 1)
#pragma unroll
        for (int j = 0; j < PPT; ++j)
#pragma unroll
          for (int k = 0; k < RG_ACC; ++k) out[j][k] += __shfl_xor_sync(0xffffffffu, out[j][k], off);
      float mine = 0.0f;
      const int lk = lane & (LG - 1);
#pragma unroll
      for (int k = 0; k < RG_ACC; ++k) {
        const float v = PPT == 2 ? out[0][k] + out[PPT - 1][k] : out[0][k];
        mine = lk == k ? v : mine;
      }
      const uint64_t chunk = (tile0 + (uint64_t)(pl0 & ~31)) >> 5;
      if (lane_ok && lk < RG_ACC && chunk < nchunks)
        partial[((size_t)chunk * S + s) * RG_ACC + lk] = (double)mine;
    }
    RG_PHASE_MARK(3);
  }
  RG_PHASE_END();
}

// The arguments of one tiled launch.
struct P32Args {
  DevTrade tr;
  DevTables tb;
  const DevScenario* scen;
  const DevScen32* scen32;
  int S, Pb, TT, NNmax, stack_max;
  float ln_ko, ln_cb, ln_ki;
  uint64_t path0, npaths;
  const uint32_t* plan;
  double* partial;
  int32_t* ko_steps;
  rg_path_record* records;
};

// Per asset count N and paths per thread PPT (phoenix32_n<N>p<PPT>.cu): the kernel of (lv: local
// vol; rec: path records), its launch, and the phase clocks of that translation unit's kernels
// (RG_PHASE_CLOCKS builds).
#define RG_P32_DECLARE(NN, PP)                                                                      \
  const void* p32_kernel_ptr_n##NN##p##PP(bool lv, bool rec);                                      \
  void p32_kernel_launch_n##NN##p##PP(bool lv, bool rec, int grid, int threads, int smem,           \
                                      cudaStream_t st, const P32Args& a);                          \
  int p32_phase_clocks_n##NN##p##PP(unsigned long long out[4], bool reset);
RG_P32_DECLARE(1, 1) RG_P32_DECLARE(1, 2)
RG_P32_DECLARE(2, 1) RG_P32_DECLARE(2, 2)
RG_P32_DECLARE(3, 1) RG_P32_DECLARE(3, 2)
RG_P32_DECLARE(4, 1) RG_P32_DECLARE(4, 2)
RG_P32_DECLARE(5, 1) RG_P32_DECLARE(5, 2)
#undef RG_P32_DECLARE

// The definitions of one (N, PPT)'s entry points (one use per translation unit).
#define RG_P32_DEFINE(NN, PP)                                                                       \
  const void* p32_kernel_ptr_n##NN##p##PP(bool lv, bool rec) {                                     \
    if (lv) return rec ? reinterpret_cast<const void*>(&phoenix32_kernel<NN, true, true, PP>)      \
                       : reinterpret_cast<const void*>(&phoenix32_kernel<NN, true, false, PP>);    \
    return rec ? reinterpret_cast<const void*>(&phoenix32_kernel<NN, false, true, PP>)             \
               : reinterpret_cast<const void*>(&phoenix32_kernel<NN, false, false, PP>);           \
  }                                                                                                 \
  template <bool LV, bool REC>                                                                      \
  static void p32_go(int grid, int threads, int smem, cudaStream_t st, const P32Args& a) {          \
    phoenix32_kernel<NN, LV, REC, PP><<<grid, threads, smem, st>>>(                                 \
        a.tr, a.tb, a.scen, a.scen32, a.S, a.Pb, a.TT, a.NNmax, a.stack_max, a.ln_ko, a.ln_cb,     \
        a.ln_ki, a.path0, a.npaths, a.plan, a.partial, a.ko_steps, a.records);                      \
  }                                                                                                 \
  void p32_kernel_launch_n##NN##p##PP(bool lv, bool rec, int grid, int threads, int smem,           \
                                      cudaStream_t st, const P32Args& a) {                         \
    if (lv) {                                                                                       \
      if (rec) p32_go<true, true>(grid, threads, smem, st, a);                                      \
      else p32_go<true, false>(grid, threads, smem, st, a);                                         \
    } else {                                                                                        \
      if (rec) p32_go<false, true>(grid, threads, smem, st, a);                                     \
      else p32_go<false, false>(grid, threads, smem, st, a);                                        \
    }                                                                                               \
  }                                                                                                 \
  int p32_phase_clocks_n##NN##p##PP(unsigned long long out[4], bool reset) { return p32_phase_clocks_tu(out, reset); }

}  // namespace rg
