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
//   B. bridge — the tile's bridge nodes of every (path, factor) chain, evaluated level by level
//      from a host plan of the streamed Brownian bridge's dependencies (each warp owns a slice of
//      the chains, its lanes take one level's nodes at once), then the uncorrelated increments
//      dW[step][factor][path] and the state carried to the next tile.
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
  uint32_t acc, lv, flags, per, noff, ncf, plan, z, dw, total;
};

// Floats per row of the Z array: N·(Pb + 4) and one more, so that rows start in different banks.
__host__ __device__ inline int p32_zrow(int N, int Pb) { return N * (Pb + 4) + 1; }

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
  // rows of p32_zrow(N, Pb) floats, N·(Pb + 4) of them one per (factor, path): the normals of the
  // tile's bridge nodes (rows 0 .. NNmax-1, overwritten by their bridge values), then the bridge
  // state carried between tiles: the value at the tile start (row NNmax) and the stack (rows
  // NNmax + 1 + slot).  The padding spreads a generation pass's stores (lanes stride GEN_CH·nch
  // apart) over distinct banks, and the odd row length the bridge phase's loads of several rows
  const uint32_t zb = (uint32_t)(NNmax + 1 + stack_max) * (uint32_t)p32_zrow(N, Pb) * 4u;
  const uint32_t rb = (uint32_t)(threads / g) * RG_ACC * 8u;  // per-tile reduction, aliases Z
  put(L.acc, (uint32_t)S * RG_ACC * 8u);
  put(L.lv, (uint32_t)(S * N) * 16u);
  put(L.flags, (uint32_t)TT * 4u);
  put(L.per, (uint32_t)TT * 4u);
  put(L.noff, (uint32_t)(TT + 1) * 4u);
  put(L.ncf, (uint32_t)NNmax * 4u);
  // the tile's bridge plan: node words, level offsets, step codes, stack entries
  put(L.plan, (uint32_t)(NNmax + (NNmax + 1) + TT + stack_max) * 4u);
  put(L.z, zb > rb ? zb : rb);
  put(L.dw, (uint32_t)TT * (PbN + 1) * 4u);  // dW[step][factor][path], odd step stride
  L.total = o;
  return L;
}

template <int N, bool LV, bool REC>
__global__ void __launch_bounds__(1024, 1) phoenix32_kernel(
    DevTrade tr, DevTables tb, const DevScenario* __restrict__ scen,
    const DevScen32* __restrict__ scen32, int S, int Pb, int TT, int NNmax, int stack_max,
    float ln_ko, float ln_cb, float ln_ki, uint64_t path0, uint64_t npaths, const uint32_t* __restrict__ plan,
    double* __restrict__ partial, int32_t* __restrict__ ko_steps, rg_path_record* __restrict__ records) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int tid = threadIdx.x, lane = tid & 31;
  const int PbN = Pb * N;
  const int nch = Pb / GEN_CH;
  const int lg_pb = __ffs(Pb) - 1;  // Pb is a power of two
  const int zs = p32_zrow(N, Pb);    // floats per Z row
  const int dws = PbN + 1;           // floats per dW step
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
  uint32_t* s_pnode = reinterpret_cast<uint32_t*>(smem_raw + L.plan);
  uint32_t* s_plev = s_pnode + NNmax;
  uint32_t* s_pstep = s_plev + NNmax + 1;
  uint32_t* s_pstk = s_pstep + TT;
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
    for (int i = tid; i < zs; i += blockDim.x) Z[(size_t)NNmax * zs + i] = 0.0f;  // W(0)
    const uint64_t gi = tile0 + pl;
    const bool ok = lane_ok && gi < npaths;
    float x[N];
#pragma unroll
    for (int f = 0; f < N; ++f) x[f] = lvc[f].w;
    P32Phoenix ph;
    float worst = 0.0f;
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
      const uint32_t* hd = plan + 1 + (size_t)(t0 / TT) * 6;
      const uint32_t nlev = __ldg(hd + 2), stk_cnt = __ldg(hd + 4);
      {
        const uint32_t node_base = __ldg(hd), lev_base = __ldg(hd + 1), stk_base = __ldg(hd + 3),
                       steps_base = __ldg(hd + 5);
        for (int i = tid; i < nn; i += blockDim.x) s_pnode[i] = __ldg(plan + node_base + i);
        for (int i = tid; i <= (int)nlev; i += blockDim.x) s_plev[i] = __ldg(plan + lev_base + i);
        for (int i = tid; i < tn; i += blockDim.x) s_pstep[i] = __ldg(plan + steps_base + t0 + i);
        for (int i = tid; i < (int)stk_cnt; i += blockDim.x) s_pstk[i] = __ldg(plan + stk_base + i);
      }
      const int ntask = nn * N * nch;
      for (int task = tid; task < ntask; task += blockDim.x) {
        const int c = task % nch, rem = task / nch, f = rem % N, j = rem / N;
        const int nd = n0 + j;
        const uint64_t g0 = tile0 + (uint64_t)c * GEN_CH;
        if (g0 >= npaths) continue;  // these paths are never read
        float* zo = Z + (size_t)j * zs + f * (Pb + 4) + c;
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
      // ---- B: the tile's bridge nodes in the plan's dependency levels, then the increments.  Warp
      // w owns chains [w·cpw, w·cpw + nc) (chain c = path c % Pb, factor c / Pb): its lanes
      // evaluate one level's nodes of those chains at once, W = z·c + (W_left + W_right) / 2 —
      // the streamed bridge's arithmetic on the same anchors, so the values are identical — each
      // written over its normal in Z; then dW of every step, and the state carried to the next
      // tile (the value at the tile end, the stack entries pushed in the tile).  Every anchor is
      // a row of Z, so an evaluation is four loads and one FMA.
      {
        const int nwarp = (int)(blockDim.x >> 5);
        const int cpw = (PbN + nwarp - 1) / nwarp;  // at most 64 (host-checked)
        const int c_lo = (tid >> 5) * cpw;
        const int nc = max(0, min(cpw, PbN - c_lo));
        const int nc1 = nc < 32 ? max(nc, 1) : 32;
        const int G = 32 / nc1, q0 = lane / nc1;  // G node slots at once; this lane's first
        const bool lane_on = nc > 0 && lane < G * nc1;
        const int cA = c_lo + lane % nc1, cB = cA + 32;  // this lane's chains (B when nc > 32)
        const bool hasB = lane_on && cB < c_lo + nc;
        auto zoff_of = [&](int c) {
          const int p = c & (Pb - 1);
          return (c >> lg_pb) * (Pb + 4) + (p & (GEN_CH - 1)) * nch + (p >> 3);
        };
        const int zA = zoff_of(cA), zB = zoff_of(cB);
        auto eval = [&](uint32_t e, float cf, int zo) {
          float* zp = Z + (int)(e & 511u) * zs + zo;
          const float z = *zp;
          const float l = Z[(int)((e >> 9) & 511u) * zs + zo], r = Z[(int)((e >> 18) & 511u) * zs + zo];
          *zp = (e >> 27) ? z * cf : fmaf(z, cf, 0.5f * (l + r));
        };
        for (uint32_t L = 0; L < nlev; ++L) {
          const int a = (int)s_plev[L], b = (int)s_plev[L + 1];
          if (lane_on)
            for (int q = a + q0; q < b; q += G) {
              const uint32_t e = s_pnode[q];
              const float cf = s_ncf[e & 511u];
              eval(e, cf, zA);
              if (hasB) eval(e, cf, zB);
            }
          __syncwarp();
        }
        if (lane_on)
          for (int tt = q0; tt < tn; tt += G) {
            const int hi = (int)s_pstep[tt] * zs;
            const int lo = tt == 0 ? NNmax * zs : (int)s_pstep[tt - 1] * zs;
            dW[tt * dws + cA] = Z[hi + zA] - Z[lo + zA];
            if (hasB) dW[tt * dws + cB] = Z[hi + zB] - Z[lo + zB];
          }
        __syncwarp();
        if (lane_on && q0 == 0) {
          const int wrow = (int)s_pstep[tn - 1] * zs;
          const float wnA = Z[wrow + zA], wnB = hasB ? Z[wrow + zB] : 0.0f;
          for (uint32_t k = 0; k < stk_cnt; ++k) {
            const uint32_t e = s_pstk[k];  // (destination row, tile node)
            Z[(int)(e >> 9) * zs + zA] = Z[(int)(e & 511u) * zs + zA];
            if (hasB) Z[(int)(e >> 9) * zs + zB] = Z[(int)(e & 511u) * zs + zB];
          }
          Z[NNmax * zs + zA] = wnA;
          if (hasB) Z[NNmax * zs + zB] = wnB;
        }
      }
      __syncthreads();
      // ---- S: scenario stepping
      if (ok) {
        for (int tt = 0; tt < tn; ++tt) {
          const int tg = (t0 + tt) * gx;
          float d[N], y[N];
#pragma unroll
          for (int f = 0; f < N; ++f) d[f] = dW[tt * dws + f * Pb + pl];
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

// The tiled kernel's block and formula tile depth.  Scenario slots: S rounded up to a power of
// two, at least 4 (two scenarios run padded: a CTA of 1024 threads on half the slots beats both
// the direct kernel and a smaller CTA); the largest block of 1024, 512 or 256 threads whose
// shared-memory layout fits.
static void tiled_shape(const Prepared& P, Fp32Shape& sh) {
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
}

// Tile depths the autotuner times besides the formula depth.
static const int kTileCandidates[] = {24, 32, 48, 64, 80, 96, 128};

// ----------------------------------------------------------------------- bridge plans --------
// The plan of one tile depth TT, word offsets relative to its start:
//   [0] tiles; then per tile 6 words (node list, level offsets, level count, stack entries,
//   stack entry count, step codes); the step codes of all T steps; per tile its nodes in level
//   order, its level offsets and its stack entries.
// Values are named by their row in the kernel's Z array: tile node j is row j, the value at the
// tile start row NNmax = TT + stack_max, stack slot d (as the tile found it) row NNmax + 1 + d.
// A node word packs (tile node j, left anchor row, right anchor row) in 9-bit fields, and bit 27
// for the bridge's first node (no anchors: W = z·c; its anchor fields name row NNmax).  A step
// code is the row of W at the step's end.  A stack entry packs (destination row NNmax + 1 + d,
// tile node) for each entry pushed in the tile and still on the stack at its end.
// The plan comes from running the streamed bridge (qmc.rs:158-191 in the order of
// bridge_schedule_into) on node ids: a node pushed at step t has the value at t as its left anchor
// and the stack's top as its right one; its level is one more than the deepest in-tile anchor.
static void build_bridge_plan(const std::vector<int32_t>& node_off, int64_t T, int TT, int stack_max,
                              std::vector<uint32_t>& w) {
  const uint32_t NNmax = (uint32_t)(TT + stack_max);
  if (NNmax + 1 + (uint32_t)stack_max > 511u) raise(RG_ERR_INVALID_SCHEDULE, "bridge plan: tile too deep");
  const size_t base = w.size();
  const int64_t ntiles = (T + TT - 1) / TT;
  w.push_back((uint32_t)ntiles);
  const size_t hdr = w.size();
  w.resize(hdr + (size_t)ntiles * 6);
  const size_t steps_at = w.size();
  w.resize(steps_at + (size_t)T);
  std::vector<int32_t> stk;  // node ids on the stack
  int32_t wc = -1;           // node id of the value at the current time (-1: W(0) = 0)
  std::vector<int> level((size_t)node_off[T], 0);
  std::vector<std::pair<int, uint32_t>> recs;
  for (int64_t k = 0; k < ntiles; ++k) {
    const int64_t t0 = k * TT, tn = std::min<int64_t>(TT, T - t0);
    const int32_t n0 = node_off[t0], n1 = node_off[t0 + tn];
    if ((uint32_t)(n1 - n0) > NNmax) raise(RG_ERR_INVALID_SCHEDULE, "bridge plan: tile too deep");
    const std::vector<int32_t> stk0 = stk;
    const int32_t wc0 = wc;
    auto code = [&](int32_t id) -> uint32_t {
      if (id >= n0 && id < n1) return (uint32_t)(id - n0);
      if (id == wc0) return NNmax;
      for (size_t d = 0; d < stk0.size(); ++d)
        if (stk0[d] == id) return NNmax + 1u + (uint32_t)d;
      raise(RG_ERR_INVALID_SCHEDULE, "bridge plan: an anchor is outside the tile's state");
    };
    recs.clear();
    for (int64_t tt = 0; tt < tn; ++tt) {
      for (int32_t nd = node_off[t0 + tt]; nd < node_off[t0 + tt + 1]; ++nd) {
        uint32_t lc = NNmax, rc = NNmax, first = 1u;
        int lev = 0;
        if (nd != 0) {
          first = 0u;
          if (stk.empty()) raise(RG_ERR_INVALID_SCHEDULE, "bridge plan: empty stack");
          const int32_t top = stk.back();
          lc = code(wc);
          rc = code(top);
          if (lc < NNmax) lev = std::max(lev, level[wc] + 1);
          if (rc < NNmax) lev = std::max(lev, level[top] + 1);
        }
        level[nd] = lev;
        recs.push_back({lev, (uint32_t)(nd - n0) | (lc << 9) | (rc << 18) | (first << 27)});
        stk.push_back(nd);
        if ((int)stk.size() > stack_max) raise(RG_ERR_INVALID_SCHEDULE, "bridge plan: stack overflow");
      }
      if (stk.empty()) raise(RG_ERR_INVALID_SCHEDULE, "bridge plan: empty stack");
      wc = stk.back();
      stk.pop_back();
      w[steps_at + t0 + tt] = code(wc);
    }
    // nodes in level order (stable), and the level offsets
    int nlev = 0;
    for (const auto& r : recs) nlev = std::max(nlev, r.first + 1);
    std::stable_sort(recs.begin(), recs.end(),
                     [](const std::pair<int, uint32_t>& a, const std::pair<int, uint32_t>& b) { return a.first < b.first; });
    const size_t node_at = w.size();
    for (const auto& r : recs) w.push_back(r.second);
    const size_t lev_at = w.size();
    {
      size_t i = 0;
      for (int L = 0; L <= nlev; ++L) {
        while (i < recs.size() && recs[i].first < L) ++i;
        w.push_back((uint32_t)i);
      }
    }
    // entries pushed in this tile and still on the stack; the rest kept their slots
    const size_t stk_at = w.size();
    for (size_t d = 0; d < stk.size(); ++d) {
      if (stk[d] >= n0 && stk[d] < n1) {
        w.push_back(((NNmax + 1u + (uint32_t)d) << 9) | (uint32_t)(stk[d] - n0));
      } else if (d >= stk0.size() || stk0[d] != stk[d]) {
        raise(RG_ERR_INVALID_SCHEDULE, "bridge plan: a carried stack entry moved");
      }
    }
    uint32_t* h = w.data() + hdr + (size_t)k * 6;
    h[0] = (uint32_t)(node_at - base);
    h[1] = (uint32_t)(lev_at - base);
    h[2] = (uint32_t)nlev;
    h[3] = (uint32_t)(stk_at - base);
    h[4] = (uint32_t)(w.size() - stk_at);
    h[5] = (uint32_t)(steps_at - base);
  }
}

std::shared_ptr<const BridgePlans> p32_bridge_plans(const Prepared& P) {
  Fp32Shape sh{};
  tiled_shape(P, sh);
  static std::mutex mu;
  static std::map<std::pair<int64_t, int>, std::shared_ptr<const BridgePlans>> cache;
  const std::pair<int64_t, int> key{P.T, sh.TT};
  {
    std::lock_guard<std::mutex> lock(mu);
    auto it = cache.find(key);
    if (it != cache.end()) return it->second;
  }
  auto out = std::make_shared<BridgePlans>();
  std::vector<int> tts{sh.TT};
  for (int tt : kTileCandidates)
    if (std::find(tts.begin(), tts.end(), tt) == tts.end()) tts.push_back(tt);
  for (int tt : tts) {
    if (out->n == RG_BPLAN_MAX) break;
    out->tt[out->n] = tt;
    out->at[out->n] = (int32_t)out->words.size();
    build_bridge_plan(P.node_off, P.T, tt, P.stack_max, out->words);
    ++out->n;
  }
  std::lock_guard<std::mutex> lock(mu);
  if (cache.size() >= 256) cache.clear();  // bounded: one entry per step count in use
  cache[key] = out;
  return out;
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
  tiled_shape(P, sh);
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
  std::vector<int> tts{sh.TT};
  tts.insert(tts.end(), std::begin(kTileCandidates), std::end(kTileCandidates));
  for (int tt : tts) {
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
  const uint32_t* plan = nullptr;
  for (int i = 0; i < tb.n_bplan; ++i)
    if (tb.bplan_tt[i] == sh.TT) plan = tb.bplan + tb.bplan_at[i];
  if (!plan) raise(RG_ERR_GPU_ERROR, "phoenix32: no bridge plan staged for the tile depth");
  // the bridge phase gives each warp at most 64 chains (two per lane)
  if ((sh.Pb * P.n + sh.threads / 32 - 1) / (sh.threads / 32) > 64)
    raise(RG_ERR_GPU_ERROR, "phoenix32: too many bridge chains per warp");
#define RG_LAUNCH(NN, LVV)                                                                        \
  if (out.records) RG_LAUNCH_R(NN, LVV, true) else RG_LAUNCH_R(NN, LVV, false)
#define RG_LAUNCH_R(NN, LVV, REC)                                                                 \
  phoenix32_kernel<NN, LVV, REC><<<sh.grid, sh.threads, sh.smem, st>>>(                           \
      P.trade, tb, scen, scen32, P.n_scen, sh.Pb, sh.TT, NNmax, P.stack_max, ln_ko, ln_cb, ln_ki, \
      path0, npaths, plan, out.partial, out.ko_steps, out.records);
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
