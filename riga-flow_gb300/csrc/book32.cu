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
// paths (a warp is 32 paths of one scenario); thread (s, p) steps the trade's assets in log space
// — x_f += σ_f·ΔW + (r - q_f - σ_f²/2)·dt, reading ΔW of its assets with coalesced loads that
// the Sb scenario warps share through L1 — and runs the Phoenix state machine of note.rs:
// 150-218 with the period schedule advanced incrementally.  Per path the payoff values are FP32;
// a warp's 32 paths are summed by a fixed butterfly and every sum above that is FP64 in a fixed
// order, so an item's sums do not depend on which CTA ran it.
#include "rg_internal.h"

namespace rg {

__global__ void __launch_bounds__(1024) book_gen32_kernel(DevTrade gen, DevTables tb,
                                                          const float* __restrict__ L32, int U,
                                                          uint64_t path0, uint64_t npaths,
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
    if (ok) incr[((uint64_t)t * U + u) * npaths + p] = wn - wcur;
    wcur = wn;
  }
}

void launch_book_gen32(const DevTrade& gen, const DevTables& tb, const float* L32, int U,
                       uint64_t path0, uint64_t npaths, float* incr, cudaStream_t s) {
  const unsigned blocks = (unsigned)((npaths + 31) / 32);
  book_gen32_kernel<<<blocks, dim3(32, U), 0, s>>>(gen, tb, L32, U, path0, npaths, incr);
  cuda_check(cudaGetLastError(), "book_gen32_kernel launch");
}

// One (trade, block) item for N underlyings: steps every tile of Pb paths of the block and adds
// the tiles' FP32 warp sums into `acc` (lane k holds slot k of this warp's FP64 sums).
template <int N>
__device__ __forceinline__ void book_scan32(const BookDev& bk, const BookTradeDev& tr, int j, int s,
                                            bool lane_ok, int pl, int Pb, const float* __restrict__ incr,
                                            uint64_t npaths, uint64_t p_lo, uint64_t p_hi, double& acc) {
  const int lane = threadIdx.x & 31;
  const int ss = lane_ok ? s : 0;
  const BookPair32 pc = bk.pair32[(size_t)j * bk.S + ss];
  float drift[N], sig[N];
  uint32_t off[N];  // asset rows within a step: idx·npaths < 2^32 for every chunk the budget allows
#pragma unroll
  for (int f = 0; f < N; ++f) {
    drift[f] = pc.drift[f];
    sig[f] = pc.sig[f];
    off[f] = (uint32_t)tr.idx[f] * (uint32_t)npaths;
  }
  const uint64_t step_stride = (uint64_t)bk.U * npaths;
  const double* df = bk.df + (size_t)ss * bk.TU;
  const double dfm_d = bk.dfm[(size_t)j * bk.S + ss];
  const float dfm = (float)dfm_d;
  const int T = tr.T, PER = tr.periods;
  for (uint64_t p0 = p_lo; p0 < p_hi; p0 += Pb) {
    const uint64_t p = p0 + pl;
    const bool ok = lane_ok && p < p_hi;
    const float* base = incr + (ok ? p : p_lo);
    float x[N];
#pragma unroll
    for (int f = 0; f < N; ++f) x[f] = pc.x0[f];
    bool alive = true, received = false;
    int qual = 0, unpaid = 0, ko_step = -1;
    float cpv = 0.0f, mpv = 0.0f, worst = 0.0f;
    // period schedule (note.rs:150-218): current period, its last step, its accrual increment
    // the last step of period 0: the largest s with min(s·PER/T, PER-1) == 0
    int per = 0;
    int pend = PER > 1 ? (int)(((int64_t)T + PER - 1) / PER) - 1 : T - 1;
    auto accr = [&](int q) {
      const int64_t a = (int64_t)T * (q + 1) / PER, b = (int64_t)T * q / PER;
      int64_t ps = a > b ? a - b : 0;
      if (ps < 1) ps = 1;
      return (float)(tr.coupon_rate / (double)ps);
    };
    float inc = accr(0);
    bool fixed = tr.fixed_first != 0;
    // ΔW of the next step is loaded one step ahead when registers allow (N <= 3)
    constexpr bool kAhead = N <= 3;
    float y[N];
#pragma unroll
    for (int f = 0; f < N; ++f) y[f] = kAhead ? __ldg(base + off[f]) : 0.0f;
    for (int t = 0; t < T; ++t) {
      float yn[N];
      if (kAhead) {
        const float* nb = base + (uint64_t)(t + 1 < T ? t + 1 : t) * step_stride;
#pragma unroll
        for (int f = 0; f < N; ++f) yn[f] = __ldg(nb + off[f]);
      } else {
        const float* cb = base + (uint64_t)t * step_stride;
#pragma unroll
        for (int f = 0; f < N; ++f) y[f] = __ldg(cb + off[f]);
      }
      float wmin = INFINITY;
#pragma unroll
      for (int f = 0; f < N; ++f) {
        x[f] = fmaf(sig[f], y[f], x[f]) + drift[f];
        wmin = fminf(wmin, x[f]);
      }
      worst = wmin;
      if (alive) {
        if (!fixed && wmin >= tr.ln_cb) ++qual;
        if (t >= tr.call_start && wmin >= tr.ln_ko) {
          alive = false;
          ko_step = t;
          const float due = fixed ? tr.coupon_f : (float)qual * inc;
          const float carry = due > 0.0f ? (float)unpaid * tr.coupon_f : 0.0f;
          if (due + carry > 0.0f) {
            const float d = (float)__ldg(df + t);
            cpv = fmaf(due, d, cpv);
            mpv = fmaf(carry, d, mpv);
            received = true;
          }
        } else if (t == pend) {
          const float due = fixed ? tr.coupon_f : (float)qual * inc;
          if (due > 0.0f) {
            const float d = (float)__ldg(df + t);
            cpv = fmaf(due, d, cpv);
            mpv = fmaf((float)unpaid * tr.coupon_f, d, mpv);
            unpaid = 0;
            received = true;
          } else if (tr.memory) {
            ++unpaid;
          }
        }
      }
      if (t == pend && t + 1 < T) {
        // the next step opens period min((t+1)·PER/T, PER-1); find where it ends
        int64_t q = (int64_t)(t + 1) * PER / T;
        if (q > PER - 1) q = PER - 1;
        per = (int)q;
        pend = per == PER - 1 ? T - 1 : (int)(((int64_t)T * (per + 1) + PER - 1) / PER) - 1;
        inc = accr(per);
        fixed = false;
        qual = 0;
      }
      if (kAhead) {
#pragma unroll
        for (int f = 0; f < N; ++f) y[f] = yn[f];
      }
    }
    // path close (note.rs:221-258) in FP32; each accumulator slot is formed, summed over the
    // warp's 32 paths by a fixed butterfly and kept by lane k, one slot at a time
    const bool ko = ko_step >= 0;
    const float funding = ok ? (ko ? (float)__ldg(df + ko_step) : dfm) : 0.0f;
    const bool hit_ki = ok && worst <= tr.ln_ki;
    const bool put_ok = hit_ki && !ko;
    const float put = put_ok ? fmaxf((float)tr.strike - expf(worst), 0.0f) * dfm : 0.0f;
    const float cn = cpv + mpv;
    const float pv1 = ok ? (funding - 1.0f) + cn - put : 0.0f;
    const bool kof = ok && ko, rec = ok && received;
    float mine = 0.0f;
#pragma unroll
    for (int k = 0; k < RG_ACC; ++k) {
      float v;
      switch (k) {
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
      if (lane == k) mine = v;
    }
    acc += (double)mine;
  }
}

__global__ void __launch_bounds__(1024, 1) book_trade32_kernel(BookDev bk, const float* __restrict__ incr,
                                                               uint64_t npaths, uint64_t block0, int blk_paths,
                                                               int Pb, double* __restrict__ partial,
                                                               int32_t* __restrict__ counter,
                                                               int* __restrict__ status) {
  __shared__ int s_item;
  __shared__ double s_red[32][RG_ACC];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int s = tid / Pb, pl = tid % Pb;
  const bool lane_ok = s < bk.S;
  const int warps_per_scen = Pb / 32;
  const int64_t nblk = (int64_t)((npaths + blk_paths - 1) / blk_paths);
  const int64_t n_items = nblk * bk.n_trades;
  for (;;) {
    if (tid == 0) s_item = atomicAdd(counter, 1);
    __syncthreads();
    const int64_t item = s_item;
    __syncthreads();
    if (item >= n_items) break;
    const int64_t b = item / bk.n_trades;
    const int j = bk.order[item % bk.n_trades];
    const BookTradeDev& tr = bk.trades[j];
    const uint64_t p_lo = (uint64_t)b * blk_paths;
    const uint64_t p_hi = p_lo + blk_paths < npaths ? p_lo + blk_paths : npaths;
    double acc = 0.0;
    switch (tr.n) {
      case 1: book_scan32<1>(bk, tr, j, s, lane_ok, pl, Pb, incr, npaths, p_lo, p_hi, acc); break;
      case 2: book_scan32<2>(bk, tr, j, s, lane_ok, pl, Pb, incr, npaths, p_lo, p_hi, acc); break;
      case 3: book_scan32<3>(bk, tr, j, s, lane_ok, pl, Pb, incr, npaths, p_lo, p_hi, acc); break;
      case 4: book_scan32<4>(bk, tr, j, s, lane_ok, pl, Pb, incr, npaths, p_lo, p_hi, acc); break;
      case 5: book_scan32<5>(bk, tr, j, s, lane_ok, pl, Pb, incr, npaths, p_lo, p_hi, acc); break;
      default:
        if (tid == 0) atomicExch(status, KSTAT_BAD_LAUNCH);
        break;
    }
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

Book32Shape book32_shape(int S, int sm_count) {
  Book32Shape sh{};
  if (S > 32) raise(RG_ERR_INVALID_ARGUMENT, "at most 32 scenarios per book launch");
  int sb = 1;
  while (sb < S) sb <<= 1;
  sh.Sb = sb;
  sh.threads = sb >= 8 ? 1024 : 256;
  sh.Pb = sh.threads / sb;
  sh.grid = sm_count * (sh.threads == 1024 ? 1 : 4);
  sh.blk_paths = sh.Pb * 32;
  return sh;
}

void launch_book_trade32(const BookDev& bk, const Book32Shape& sh, const float* incr, uint64_t npaths,
                         uint64_t block0, double* partial, int32_t* counter, int* status, cudaStream_t s) {
  cuda_check(cudaMemsetAsync(counter, 0, sizeof(int32_t), s), "book counter reset");
  book_trade32_kernel<<<sh.grid, sh.threads, 0, s>>>(bk, incr, npaths, block0, sh.blk_paths, sh.Pb,
                                                     partial, counter, status);
  cuda_check(cudaGetLastError(), "book_trade32_kernel launch");
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
