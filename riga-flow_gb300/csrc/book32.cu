// book32.cu — FP32 production kernels of a book.
//
// book_gen32_kernel: the universe's correlated Brownian increments of a chunk of paths,
// incr[t][u][p] = ΔW (variance dt), FP32, written once to HBM and read by every trade.  A CTA is
// 32 paths × U assets (threadIdx.x = path lane, threadIdx.y = asset): at every bridge node each
// thread draws its asset's QMC normal once into shared memory, then forms its correlated normal
// y_u = Σ_{b<=u} L[u][b]·z_b from the shared row and advances the streamed bridge of (path, u).
// The bridge is applied after the correlation, as in the reference (note.rs:89-106).  Each warp
// writes 32 consecutive paths of one (step, asset): 128-byte coalesced stores.
//
// book_trade32_kernel: persistent.  Work items are (path block, trade), taken from an atomic
// counter in path-block-major order with trades longest first, so the CTAs in flight read the
// same block of increments (L2-resident) and the tail is short.  A CTA is Sb scenario slots × Pb
// paths (a warp is 32 paths of one scenario); the increments each (path tile, time tile) stage
// needs are staged in shared memory by TMA, double-buffered on mbarriers, and thread (s, p) steps
// the trade's assets in log space — x_f += σ_f·ΔW + (r - q_f - σ_f²/2)·dt — from shared memory
// and runs the Phoenix state machine of note.rs:150-218 with the period schedule advanced
// incrementally.  Per path the payoff values are FP32;
// a warp's 32 paths are summed by a fixed butterfly and every sum above that is FP64 in a fixed
// order, so an item's sums do not depend on which CTA ran it.
#include <algorithm>
#include <mutex>

#include "rg_async.cuh"
#include "rg_internal.h"

namespace rg {

__global__ void __launch_bounds__(1024) book_gen32_kernel(DevTrade gen, DevTables tb,
                                                          const float* __restrict__ L32, int U,
                                                          uint64_t path0, uint64_t npaths, uint64_t rowlen,
                                                          float* __restrict__ incr) {
  __shared__ float zs[2][RG_BOOK_MAX_UNIVERSE][33];
  const int lane = threadIdx.x, u = threadIdx.y;
  const uint64_t p = (uint64_t)blockIdx.x * 32 + lane;
  const bool ok = p < npaths;
  const uint64_t point = path0 + (ok ? p : 0);
  const int64_t T = gen.steps;
  float lrow[RG_BOOK_MAX_UNIVERSE];
#pragma unroll
  for (int b = 0; b < RG_BOOK_MAX_UNIVERSE; ++b) lrow[b] = b <= u && b < U ? __ldg(L32 + u * U + b) : 0.0f;
  float wcur = 0.0f, stk[RG_STACK_MAX];
  int sp = 0, buf = 0;
  for (int64_t t = 0; t < T; ++t) {
    const int c0 = __ldg(tb.node_off + t), c1 = __ldg(tb.node_off + t + 1);
    for (int c = c0; c < c1; ++c) {
      const int k = __ldg(tb.node_k + c);
      zs[buf][u][lane] = rg_qmc_normal32(gen, tb, point, (uint64_t)k * (uint64_t)U + (uint64_t)u);
      __syncthreads();
      float y = 0.0f;
#pragma unroll
      for (int b = 0; b < RG_BOOK_MAX_UNIVERSE; ++b)
        if (b <= u) y = fmaf(lrow[b], zs[buf][b][lane], y);
      const float cf = __ldg(tb.node_cf + c);
      stk[sp] = c == 0 ? y * cf : fmaf(y, cf, 0.5f * (wcur + stk[sp - 1]));
      ++sp;
      buf ^= 1;  // the next node writes the other row: one barrier per node suffices
    }
    --sp;
    const float wn = stk[sp];
    if (ok) incr[((uint64_t)t * U + u) * rowlen + p] = wn - wcur;
    wcur = wn;
  }
}

void launch_book_gen32(const DevTrade& gen, const DevTables& tb, const float* L32, int U,
                       uint64_t path0, uint64_t npaths, uint64_t rowlen, float* incr, cudaStream_t s) {
  const unsigned blocks = (unsigned)((npaths + 31) / 32);
  book_gen32_kernel<<<blocks, dim3(32, U), 0, s>>>(gen, tb, L32, U, path0, npaths, rowlen, incr);
  cuda_check(cudaGetLastError(), "book_gen32_kernel launch");
}

// ------------------------------------------------------------------ TMA-staged scan ----------
// The increments a (trade, path tile) stage needs — for each of the trade's N underlyings, TT
// steps × Pb paths — are one 3-D tensor-map box each (paths innermost).  One elected thread
// issues the next stage's boxes into the other shared-memory buffer (cp.async.bulk.tensor,
// completion counted on that buffer's "full" mbarrier) while every warp consumes the current
// buffer, and each warp releases a buffer on its "empty" mbarrier when it is done with it.
// Every wait is bounded: a wait that runs out sets the status word and the kernel returns.

// Bounded wait for the phase of `bar` with the given parity to complete; sets the status word
// when it runs out.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, int* status) {
  if (mbar_wait_bounded(bar, parity)) return true;
  atomicExch(status, KSTAT_TIMEOUT);
  return false;
}
__device__ __forceinline__ void tma_load_3d(void* dst, const CUtensorMap* map, uint64_t* bar, int x, int y, int z) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%3, %4, %5}], [%2];"
      ::"r"(smem_u32(dst)), "l"(reinterpret_cast<uint64_t>(map)), "r"(smem_u32(bar)), "r"(x), "r"(y), "r"(z)
      : "memory");
}

struct BookStage {
  int tile, k;  // path tile within the item, time tile within the trade
};

template <int N>
__device__ __forceinline__ bool book_scan32_tma(const BookDev& bk, const BookTradeDev& tr, int j, int s, bool lane_ok,
                                                int pl, int Pb, int TT, uint64_t p_lo, uint64_t p_hi,
                                                const CUtensorMap* tmap, float* bufs, uint64_t* full,
                                                uint64_t* empty, uint32_t& G, int* status, double& acc) {
  const int lane = threadIdx.x & 31;
  const int tid = threadIdx.x;
  const int ss = lane_ok ? s : 0;
  const BookPair32 pc = bk.pair32[(size_t)j * bk.S + ss];
  float drift[N], sig[N];
#pragma unroll
  for (int f = 0; f < N; ++f) {
    drift[f] = pc.drift[f];
    sig[f] = pc.sig[f];
  }
  const float* df = bk.df_f + (size_t)pc.dfrow * bk.TU;
  const float dfm = bk.dfm_f[(size_t)j * bk.S + ss];
  const int T = tr.T, PER = tr.periods;
  const int ntiles = (int)((p_hi - p_lo + Pb - 1) / Pb);
  const int ntt = (T + TT - 1) / TT;
  const int nst = ntiles * ntt;
  const uint32_t stage_floats = (uint32_t)(N * TT * Pb);
  const uint32_t bytes = (uint32_t)(N * TT * Pb * 4);
  // the producer: stage st of this item into buffer g & 1 (the (g >> 1)-th use of that buffer)
  auto produce = [&](uint32_t g, int st) -> bool {
    const uint32_t b = g & 1u, u = g >> 1;
    if (u >= 1 && !mbar_wait(&empty[b], (u - 1) & 1u, status)) return false;
    const int tile = st / ntt, k = st % ntt;
    mbar_expect_tx(&full[b], bytes);
    float* dst = bufs + b * stage_floats;
#pragma unroll
    for (int f = 0; f < N; ++f)
      tma_load_3d(dst + f * TT * Pb, tmap, &full[b], (int)(p_lo + (uint64_t)tile * Pb), tr.idx[f], k * TT);
    return true;
  };
  if (tid == 0 && !produce(G, 0)) return false;
  float x[N];
  bool alive = true, received = false, ok = false;
  int qual = 0, unpaid = 0, ko_step = -1, per = 0, pend = 0;
  float cpv = 0.0f, mpv = 0.0f, worst = 0.0f, inc = 0.0f;
  bool fixed = false;
  auto accr = [&](int q) {
    const int64_t a = (int64_t)T * (q + 1) / PER, b = (int64_t)T * q / PER;
    return a - b <= tr.ps_a ? tr.inc_a : tr.inc_b;  // coupon_rate / max(1, a - b), rounded to FP32
  };
  for (int st = 0; st < nst; ++st, ++G) {
    const int tile = st / ntt, k = st % ntt;
    if (tid == 0 && st + 1 < nst && !produce(G + 1, st + 1)) return false;
    if (k == 0) {
      // a new path tile: fresh path state
      ok = lane_ok && p_lo + (uint64_t)tile * Pb + pl < p_hi;
#pragma unroll
      for (int f = 0; f < N; ++f) x[f] = pc.x0[f];
      alive = true;
      received = false;
      qual = unpaid = 0;
      ko_step = -1;
      cpv = mpv = worst = 0.0f;
      per = 0;
      pend = PER > 1 ? (int)(((int64_t)T + PER - 1) / PER) - 1 : T - 1;
      inc = accr(0);
      fixed = tr.fixed_first != 0;
    }
    const uint32_t b = G & 1u;
    if (!mbar_wait(&full[b], (G >> 1) & 1u, status)) return false;
    const float* buf = bufs + b * stage_floats;
    const int t0 = k * TT, tn = min(TT, T - t0);
    // one step of the path: log-space Euler on the staged increments, the worst-of performance
    auto advance = [&](int tt) -> float {
      float wmin = INFINITY;
#pragma unroll
      for (int f = 0; f < N; ++f) {
        x[f] = fmaf(sig[f], buf[(f * TT + tt) * Pb + pl], x[f]) + drift[f];
        wmin = fminf(wmin, x[f]);
      }
      worst = wmin;
      return wmin;
    };
    auto knock_out = [&](int t) {
      alive = false;
      ko_step = t;
      const float due = fixed ? tr.coupon_f : (float)qual * inc;
      const float carry = due > 0.0f ? (float)unpaid * tr.coupon_f : 0.0f;
      if (due + carry > 0.0f) {
        const float d = __ldg(df + t);
        cpv = fmaf(due, d, cpv);
        mpv = fmaf(carry, d, mpv);
        received = true;
      }
    };
    // The schedule is the trade's, the same for every thread: the stage splits into runs of plain
    // steps (no period end) before and after the call start, and the period-end step, which alone
    // pays coupons and moves to the next period.
    int tt = 0;
    while (tt < tn) {
      const int seg = min(tn, pend - t0 + 1);           // through the next period end, or the stage end
      const int plain = pend - t0 < tn ? seg - 1 : seg;  // steps [tt, plain) are not a period end
      const int ko_from = max(tt, min(plain, tr.call_start - t0));
      for (; tt < ko_from; ++tt) {
        const float wmin = advance(tt);
        if (alive && !fixed && wmin >= tr.ln_cb) ++qual;
      }
      for (; tt < plain; ++tt) {
        const float wmin = advance(tt);
        if (alive) {
          if (!fixed && wmin >= tr.ln_cb) ++qual;
          if (wmin >= tr.ln_ko) knock_out(t0 + tt);
        }
      }
      if (tt < seg) {
        // the period-end step (note.rs:150-218 at a period boundary)
        const int t = t0 + tt;
        const float wmin = advance(tt);
        if (alive) {
          if (!fixed && wmin >= tr.ln_cb) ++qual;
          if (t >= tr.call_start && wmin >= tr.ln_ko) {
            knock_out(t);
          } else {
            const float due = fixed ? tr.coupon_f : (float)qual * inc;
            if (due > 0.0f) {
              const float d = __ldg(df + t);
              cpv = fmaf(due, d, cpv);
              mpv = fmaf((float)unpaid * tr.coupon_f, d, mpv);
              unpaid = 0;
              received = true;
            } else if (tr.memory) {
              ++unpaid;
            }
          }
        }
        if (t + 1 < T) {
          int64_t q = (int64_t)(t + 1) * PER / T;
          if (q > PER - 1) q = PER - 1;
          per = (int)q;
          pend = per == PER - 1 ? T - 1 : (int)(((int64_t)T * (per + 1) + PER - 1) / PER) - 1;
          inc = accr(per);
          fixed = false;
          qual = 0;
        }
        ++tt;
      }
    }
    // this warp is done with the buffer
    __syncwarp();
    if (lane == 0) mbar_arrive(&empty[b]);
    if (k == ntt - 1) {
      // path close (note.rs:221-258) in FP32; each slot summed over the warp's 32 paths by a
      // fixed butterfly and kept by lane k
      const bool ko = ko_step >= 0;
      const float funding = ok ? (ko ? __ldg(df + ko_step) : dfm) : 0.0f;
      const bool hit_ki = ok && worst <= tr.ln_ki;
      const bool put_ok = hit_ki && !ko;
      const float put = put_ok ? fmaxf(tr.strike_f - expf(worst), 0.0f) * dfm : 0.0f;
      const float cn = cpv + mpv;
      const float pv1 = ok ? (funding - 1.0f) + cn - put : 0.0f;
      const bool kof = ok && ko, rec = ok && received;
      float mine = 0.0f;
#pragma unroll
      for (int kk = 0; kk < RG_ACC; ++kk) {
        float v;
        switch (kk) {
          case ACC_PV: v = pv1; break;
          case ACC_PV2: v = pv1 * pv1; break;
          case ACC_KOF: v = kof ? funding - 1.0f : 0.0f; break;
          case ACC_KOF2: v = kof ? (funding - 1.0f) * (funding - 1.0f) : 0.0f; break;
          case ACC_KIPUT: v = hit_ki ? put : 0.0f; break;
          case ACC_KIPUT2: v = hit_ki ? put * put : 0.0f; break;
          case ACC_CPN: v = rec ? cn : 0.0f; break;
          case ACC_CPN2: v = rec ? cn * cn : 0.0f; break;
          case ACC_PUT: v = put; break;
          case ACC_FUND: v = funding; break;
          case ACC_CQ: v = ok ? cpv * 10.0f : 0.0f; break;
          case ACC_MQ: v = ok ? mpv * 10.0f : 0.0f; break;
          case ACC_NKO: v = kof ? 1.0f : 0.0f; break;
          case ACC_NKI: v = hit_ki ? 1.0f : 0.0f; break;
          case ACC_NPUT: v = put_ok ? 1.0f : 0.0f; break;
          default: v = rec ? 1.0f : 0.0f; break;  // ACC_NCPN
        }
#pragma unroll
        for (int w = 16; w > 0; w >>= 1) v += __shfl_xor_sync(0xffffffffu, v, w);
        if (lane == kk) mine = v;
      }
      acc += (double)mine;
    }
  }
  return true;
}

// One persistent launch per underlying count N over that group of trades (order[g_lo, g_lo + ng)),
// so each instantiation gets the registers its N needs.
template <int N>
__global__ void __launch_bounds__(1024, 1) book_trade32_kernel(const __grid_constant__ CUtensorMap tmap, BookDev bk,
                                                               uint64_t npaths, uint64_t block0, int blk_paths,
                                                               int Pb, int TT, int g_lo, int ng,
                                                               double* __restrict__ partial,
                                                               int32_t* __restrict__ counter, int* __restrict__ status) {
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  __shared__ int s_item;
  __shared__ double s_red[32][RG_ACC];
  float* bufs = reinterpret_cast<float*>(smem_raw);
  uint64_t* bars = reinterpret_cast<uint64_t*>(smem_raw + (size_t)2 * N * TT * Pb * 4);
  uint64_t* full = bars;
  uint64_t* empty = bars + 2;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int nwarps = blockDim.x >> 5;
  const int s = tid / Pb, pl = tid % Pb;
  const bool lane_ok = s < bk.S;
  const int warps_per_scen = Pb / 32;
  const int64_t nblk = (int64_t)((npaths + blk_paths - 1) / blk_paths);
  const int64_t n_items = nblk * ng;
  if (tid == 0) {
    mbar_init(&full[0], 1);
    mbar_init(&full[1], 1);
    mbar_init(&empty[0], (uint32_t)nwarps);
    mbar_init(&empty[1], (uint32_t)nwarps);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();
  uint32_t G = 0;
  for (;;) {
    if (tid == 0) s_item = atomicAdd(counter, 1);
    __syncthreads();
    const int64_t item = s_item;
    __syncthreads();
    if (item >= n_items || *(volatile int*)status != 0) break;
    const int64_t b = item / ng;
    const int j = bk.order[g_lo + item % ng];
    const BookTradeDev& tr = bk.trades[j];
    if (tr.n != N) {
      if (tid == 0) atomicExch(status, KSTAT_BAD_LAUNCH);
      return;
    }
    const uint64_t p_lo = (uint64_t)b * blk_paths;
    const uint64_t p_hi = p_lo + blk_paths < npaths ? p_lo + blk_paths : npaths;
    double acc = 0.0;
    if (!book_scan32_tma<N>(bk, tr, j, s, lane_ok, pl, Pb, TT, p_lo, p_hi, &tmap, bufs, full, empty, G, status, acc))
      return;  // a bounded wait ran out (status set): nothing more is issued
    // the scenario's warps in index order
    if (lane < RG_ACC) s_red[warp][lane] = acc;
    __syncthreads();
    if (tid < bk.S * RG_ACC) {
      const int sc = tid / RG_ACC, k = tid % RG_ACC;
      double v = 0.0;
      for (int w = 0; w < warps_per_scen; ++w) v += s_red[sc * warps_per_scen + w][k];
      partial[(((size_t)(block0 + b) * bk.n_trades + j) * bk.S + sc) * RG_ACC + k] = v;
    }
  }
}

Book32Shape book32_shape(int S, int sm_count, uint64_t paths, int min_group_trades) {
  Book32Shape sh{};
  if (S > 32) raise(RG_ERR_INVALID_ARGUMENT, "at most 32 scenarios per book launch");
  int sb = 1;
  while (sb < S) sb <<= 1;
  sh.Sb = sb;
  sh.threads = sb >= 8 ? 1024 : 256;
  sh.Pb = sh.threads / sb;
  // stage depth for five underlyings: 64 steps where the two stage buffers fit 168 KB
  sh.TT = 64;
  while (sh.TT > 8 && 2 * 5 * sh.TT * sh.Pb * 4 > 168 * 1024) sh.TT >>= 1;
  sh.grid = sm_count * (sh.threads == 1024 ? 1 : 4);
  // a work item is one trade over a block of 32 path tiles; a small book (few paths, or an
  // underlying-count group of few trades) takes smaller blocks, so that the smallest group's launch
  // still has two items per SM instead of running as long as one long item
  int k = 32;
  const uint64_t g = (uint64_t)(min_group_trades > 0 ? min_group_trades : 1);
  while (k > 1 && (paths + (uint64_t)sh.Pb * k - 1) / ((uint64_t)sh.Pb * k) * g < 2 * (uint64_t)sm_count) k >>= 1;
  sh.blk_paths = sh.Pb * k;
  sh.smem = 2 * 5 * sh.TT * sh.Pb * 4 + 64;
  return sh;
}

// Steps per stage for trades on n underlyings: the stage buffers hold 5 × base steps of one
// underlying, so fewer underlyings take proportionally deeper stages (fewer hand-overs per step) in
// the same shared memory; at most 160 steps (a box edge may not exceed 256).
int book_stage_steps(int n, int base) {
  const int tt = base * 5 / (n > 0 ? n : 1);
  return tt < 160 ? tt : 160;
}

template <int N>
static void launch_group(const BookDev& bk, const Book32Shape& sh, const CUtensorMap& tmap, uint64_t npaths,
                         uint64_t block0, int g_lo, int ng, double* partial, int32_t* counter, int* status,
                         cudaStream_t s) {
  // process-wide attribute, raised once per device to cover every shape's stage buffers
  {
    static std::mutex mu;
    static std::vector<char> done;
    int dev = 0;
    cuda_check(cudaGetDevice(&dev), "cudaGetDevice");
    std::lock_guard<std::mutex> lock(mu);
    if ((int)done.size() <= dev) done.resize(dev + 1, 0);
    if (!done[dev]) {
      cuda_check(cudaFuncSetAttribute(book_trade32_kernel<N>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      176 * 1024),
                 "book smem attribute");
      done[dev] = 1;
    }
  }
  const int tt = book_stage_steps(N, sh.TT);
  const int smem = 2 * N * tt * sh.Pb * 4 + 64;
  if (smem > 176 * 1024) raise(RG_ERR_GPU_ERROR, "book stage buffers exceed the shared-memory limit");
  cuda_check(cudaMemsetAsync(counter, 0, sizeof(int32_t), s), "book counter reset");
  book_trade32_kernel<N><<<sh.grid, sh.threads, smem, s>>>(tmap, bk, npaths, block0, sh.blk_paths, sh.Pb, tt,
                                                           g_lo, ng, partial, counter, status);
  cuda_check(cudaGetLastError(), "book_trade32_kernel launch");
}

void launch_book_trade32(const BookDev& bk, const Book32Shape& sh, const CUtensorMap* maps, uint64_t npaths,
                         uint64_t block0, const int* group_lo, const int* group_n, double* partial,
                         int32_t* counter, int* status, cudaStream_t s) {
  for (int n = 1; n <= RG_NMAX; ++n) {
    const int lo = group_lo[n - 1], ng = group_n[n - 1];
    if (ng == 0) continue;
    const CUtensorMap& tmap = maps[n - 1];
    switch (n) {
      case 1: launch_group<1>(bk, sh, tmap, npaths, block0, lo, ng, partial, counter, status, s); break;
      case 2: launch_group<2>(bk, sh, tmap, npaths, block0, lo, ng, partial, counter, status, s); break;
      case 3: launch_group<3>(bk, sh, tmap, npaths, block0, lo, ng, partial, counter, status, s); break;
      case 4: launch_group<4>(bk, sh, tmap, npaths, block0, lo, ng, partial, counter, status, s); break;
      default: launch_group<5>(bk, sh, tmap, npaths, block0, lo, ng, partial, counter, status, s); break;
    }
  }
}

__global__ void book_l32_kernel(const double* __restrict__ L, int n, float* __restrict__ L32) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) L32[i] = (float)L[i];
}

void launch_book_l32(const double* L, int U, float* L32, cudaStream_t s) {
  book_l32_kernel<<<(U * U + 255) / 256, 256, 0, s>>>(L, U * U, L32);
  cuda_check(cudaGetLastError(), "book_l32_kernel launch");
}

// out[pair][k] = Σ_b partial[b·stride_b + pair·stride_pair + k], b in order.
__global__ void book_reduce_kernel(const double* __restrict__ partial, int64_t blocks, int64_t stride_b,
                                   int64_t stride_pair, int pairs, double* __restrict__ out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= pairs * RG_ACC) return;
  const int pair = i / RG_ACC, k = i % RG_ACC;
  double v = 0.0;
  for (int64_t b = 0; b < blocks; ++b) v += partial[b * stride_b + (int64_t)pair * stride_pair + k];
  out[i] = v;
}

void launch_book_reduce_strided(const double* partial, int64_t blocks, int64_t stride_b, int64_t stride_pair,
                                int pairs, double* out, cudaStream_t s) {
  const int n = pairs * RG_ACC;
  book_reduce_kernel<<<(n + 255) / 256, 256, 0, s>>>(partial, blocks, stride_b, stride_pair, pairs, out);
  cuda_check(cudaGetLastError(), "book_reduce_kernel launch");
}

}  // namespace rg
