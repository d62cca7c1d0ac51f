// phoenix32.cu — host side of the tiled FP32 CRN kernel (p32_tiled.cuh): launch shapes, the
// level-ordered bridge plans, the launch-shape autotuner and the launch.  The kernel's
// instantiations are compiled per (asset count, paths per thread) in phoenix32_n<N>p<PPT>.cu.
#include <algorithm>
#include <map>
#include <mutex>
#include <vector>

#include "p32_tiled.cuh"

namespace rg {

static const void* select_kernel(int n, bool lv, bool rec, int ppt) {
#define RG_SEL(NN) return ppt == 2 ? p32_kernel_ptr_n##NN##p2(lv, rec) : p32_kernel_ptr_n##NN##p1(lv, rec);
  switch (n) {
    case 1: RG_SEL(1)
    case 2: RG_SEL(2)
    case 3: RG_SEL(3)
    case 4: RG_SEL(4)
    case 5: RG_SEL(5)
    default: raise(RG_ERR_INVALID_MARKET_SHAPE, "unsupported asset count");
  }
#undef RG_SEL
}

// Paths per thread of the formula shape: two (packed FP32x2 stepping, 512 threads) unless the
// autotuner measured one faster for the launch shape.
static constexpr int kDefaultPpt = 2;

// Formula tile depth of a block of Pb paths.
static int formula_tt(const Prepared& P, int Pb) {
  int tt = (32768 / (Pb * P.n) - P.stack_max) / 2;
  return tt < 8 ? 8 : (tt > 64 ? 64 : tt);
}

// Shared-memory bytes of a tiled shape: Pb paths per tile at `ppt` paths per thread, `tt` steps per
// tile.
static uint32_t p32_smem(const Prepared& P, int Pb, int ppt, int tt) {
  return p32_layout(P.n, Pb, tt, tt + P.stack_max, P.stack_max, ppt).total;
}
// Whether the shape fits in 227 KB of shared memory.
static bool p32_fits(const Prepared& P, int Pb, int ppt, int tt) { return p32_smem(P, Pb, ppt, tt) <= 227u * 1024u; }

// The tiled kernel's block and formula tile depth.  Scenario slots: S rounded up to a power of
// two, at least 4 (two scenarios run padded: a CTA on half the slots beats both the direct kernel
// and a smaller CTA); Pb = 1024 / slots paths per tile (at least 32: the path chunks of the sums
// lie inside one tile), served by 1024 threads (one path per thread) or 512 (two).
static void tiled_shape(const Prepared& P, Fp32Shape& sh, int ppt) {
  int sb = 4;
  while (sb < P.n_scen) sb <<= 1;
  sh.Sb = sb;
  sh.Pb = 1024 / sb;
  sh.TT = formula_tt(P, sh.Pb);
  if (ppt == 2 && !p32_fits(P, sh.Pb, 2, sh.TT)) ppt = 1;
  sh.ppt = ppt;
  sh.threads = sb * sh.Pb / ppt;
  sh.smem = (int)p32_smem(P, sh.Pb, ppt, sh.TT);
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
  tiled_shape(P, sh, kDefaultPpt);
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

// Function attributes are process-wide: raise every instantiation's dynamic shared-memory limit to
// the device maximum once per device, so engines pricing concurrently never lower it under each other.
static void p32_set_attributes() {
  static std::mutex mu;
  static std::vector<char> done;
  int dev = 0;
  cuda_check(cudaGetDevice(&dev), "cudaGetDevice");
  std::lock_guard<std::mutex> lock(mu);
  if ((int)done.size() <= dev) done.resize(dev + 1, 0);
  if (done[dev]) return;
  int optin = 0;
  cuda_check(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev), "smem opt-in");
  for (int ppt = 1; ppt <= 2; ++ppt)
    for (int n = 1; n <= RG_NMAX; ++n)
      for (int lv = 0; lv < 2; ++lv)
        for (int rec = 0; rec < 2; ++rec) {
          const void* kr = select_kernel(n, lv != 0, rec != 0, ppt);
          cuda_check(cudaFuncSetAttribute(kr, cudaFuncAttributeMaxDynamicSharedMemorySize, optin),
                     "phoenix32 smem attribute");
          cuda_check(cudaFuncSetAttribute(kr, cudaFuncAttributePreferredSharedMemoryCarveout, 100),
                     "phoenix32 carveout");
        }
  done[dev] = 1;
}

// Grid of a tiled shape: as many CTAs as are resident on the SMs, at most one per tile.
static int tiled_grid(const Prepared& P, const Fp32Shape& sh, uint64_t npaths, int sm_count) {
  const void* k = select_kernel(P.n, P.trade.has_lv != 0, false, sh.ppt);
  int per_sm = 0;
  cuda_check(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k, sh.threads, sh.smem),
             "phoenix32 occupancy");
  if (per_sm < 1) raise(RG_ERR_GPU_ERROR, "phoenix32: launch shape does not fit on an SM");
  const uint64_t tiles = (npaths + sh.Pb - 1) / sh.Pb;
  const uint64_t cap = (uint64_t)sm_count * per_sm;
  const int grid = (int)(tiles < cap ? tiles : cap);
  return grid < 1 ? 1 : grid;
}

Fp32Shape phoenix32_shape(const Prepared& P, uint64_t npaths, int sm_count) {
  Fp32Shape sh{};
  if (P.n_scen > 32) raise(RG_ERR_INVALID_ARGUMENT, "at most 32 scenarios per fused launch");
  if (p32_direct(P, npaths)) {
    // nothing for the scenarios to share: the per-thread kernel without shared-memory tiles
    sh.direct = 1;
    sh.Sb = P.n_scen;
    sh.threads = 256;
    sh.ppt = 1;
    sh.grid = phoenix32d_grid(P, npaths, sm_count);
    sh.smem = P.stack_max * P.n * 256 * (int)sizeof(float);  // the bridge stacks (dynamic)
    return sh;
  }
  tiled_shape(P, sh, kDefaultPpt);
  if (sh.smem > 227 * 1024) raise(RG_ERR_GPU_ERROR, "phoenix32: the tile does not fit in shared memory");
  p32_set_attributes();
  sh.grid = tiled_grid(P, sh, npaths, sm_count);
  return sh;
}

// Rows of the FP32 kernels' partial sums: one per 32-path chunk of the launch.
uint64_t p32_chunks(uint64_t npaths) { return (npaths + 31) / 32; }

// ---------------------------------------------------------------------- tiled-shape autotuner --
namespace {
// A tiled launch shape: paths per CTA tile, paths per thread, tile depth.
struct TiledKnobs {
  int pb, ppt, tt;
  bool operator==(const TiledKnobs& o) const { return pb == o.pb && ppt == o.ppt && tt == o.tt; }
};

// Sets the block (Pb paths per tile), paths per thread and tile depth of a tiled shape if the
// block keeps a warp on 32·ppt paths of one scenario and its layout fits.
bool p32_with(const Prepared& P, Fp32Shape& sh, TiledKnobs k) {
  if (k.pb < 32 * k.ppt || (k.pb & (k.pb - 1)) || k.pb * sh.Sb > 1024 || !p32_fits(P, k.pb, k.ppt, k.tt)) return false;
  sh.Pb = k.pb;
  sh.ppt = k.ppt;
  sh.threads = sh.Sb * k.pb / k.ppt;
  sh.TT = k.tt;
  sh.smem = (int)p32_smem(P, k.pb, k.ppt, k.tt);
  return true;
}

std::mutex g_tune_mu;
std::map<std::vector<int64_t>, TiledKnobs> g_tuned;  // launch shape -> (block, paths per thread, tile depth)
bool g_tune_enabled = true;
TiledKnobs g_forced{0, 0, 0};  // the shape every tiled launch takes, or none (ppt 0); pb 0: the
                               // formula block


}  // namespace

void p32_set_autotune(bool enabled) {
  std::lock_guard<std::mutex> lock(g_tune_mu);
  g_tune_enabled = enabled;
  g_tuned.clear();
}

void p32_force_shape(int ppt, int tt, int pb) {
  if (!((ppt == 0 && tt == 0 && pb == 0) || ((ppt == 1 || ppt == 2) && tt > 0 && pb >= 0)))
    raise(RG_ERR_INVALID_ARGUMENT, "tiled shape: paths per thread 1 or 2, a tile depth and a block, or (0, 0, 0)");
  if (pb != 0 && (pb < 32 * ppt || pb > 1024 || (pb & (pb - 1))))
    raise(RG_ERR_INVALID_ARGUMENT, "tiled shape: the block must be a power of two of 32 x paths per thread to 1024 paths");
  bool plan = tt == 0;
  for (int c : kTileCandidates) plan = plan || c == tt;
  if (!plan) raise(RG_ERR_INVALID_ARGUMENT, "tiled shape: the tile depth must be one of the autotuner's candidates");
  std::lock_guard<std::mutex> lock(g_tune_mu);
  g_forced = TiledKnobs{pb, ppt, tt};
}

// Times every (block, paths per thread, tile depth) candidate on a prefix of the launch's paths and
// keeps the fastest for the launch shape.  No knob changes a path's arithmetic or the 32-path
// chunks of the sums, so prices are identical whichever wins.  Blocks: the formula's Pb paths per
// tile and half of it (two smaller CTAs per SM where they fit).
Fp32Shape phoenix32_tune(const Prepared& P, const DevTables& tb, const DevScenario* scen,
                         const DevScen32* scen32, uint64_t path0, uint64_t npaths, Fp32Shape sh,
                         const LaunchOut& out, bool may_tune, int sm_count, cudaStream_t st) {
  if (sh.direct) return sh;
  int dev = 0;
  cuda_check(cudaGetDevice(&dev), "cudaGetDevice");
  const std::vector<int64_t> key{dev, sm_count, P.n, P.trade.has_lv, P.n_scen, sh.Sb, P.T, P.stack_max,
                                 P.trade.vr, P.trade.scrambler, P.trade.gx};
  auto apply = [&](TiledKnobs c, uint64_t paths) {
    Fp32Shape t = sh;
    if (!p32_with(P, t, c)) return sh;
    t.grid = tiled_grid(P, t, paths, sm_count);
    t.tuned = 1;
    return t;
  };
  {
    std::lock_guard<std::mutex> lock(g_tune_mu);
    if (g_forced.ppt) {
      Fp32Shape t = apply({g_forced.pb ? g_forced.pb : sh.Pb, g_forced.ppt, g_forced.tt}, npaths);
      if (!t.tuned) raise(RG_ERR_INVALID_ARGUMENT, "tiled shape: the forced tile does not fit in shared memory");
      return t;
    }
    if (!g_tune_enabled) return sh;
    auto it = g_tuned.find(key);
    if (it != g_tuned.end()) return apply(it->second, npaths);
  }
  // a tuning pass costs about (candidates × 2) launches over two waves of tiles: only for
  // launches of at least eight waves
  const uint64_t prefix = (uint64_t)sh.grid * (uint64_t)sh.Pb * 2;
  if (!may_tune || npaths < prefix * 4) return sh;
  std::vector<TiledKnobs> cand;
  std::vector<int> tts{sh.TT};
  tts.insert(tts.end(), std::begin(kTileCandidates), std::end(kTileCandidates));
  for (int pb : {sh.Pb, sh.Pb / 2})
    for (int ppt = 1; ppt <= 2; ++ppt)
      for (int tt : tts) {
        Fp32Shape c = sh;
        const TiledKnobs k{pb, ppt, tt};
        if (std::find(cand.begin(), cand.end(), k) == cand.end() && p32_with(P, c, k)) cand.push_back(k);
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
      const Fp32Shape c = apply(cand[i], prefix);
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
  {
    std::lock_guard<std::mutex> lock(g_tune_mu);
    g_tuned[key] = cand[win];
  }
  return apply(cand[win], npaths);
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
  if (sh.Pb < 32 || (sh.Pb & (sh.Pb - 1)) || sh.threads * sh.ppt != sh.Sb * sh.Pb || (sh.ppt != 1 && sh.ppt != 2))
    raise(RG_ERR_GPU_ERROR, "phoenix32: invalid tile shape");
  const bool lvk = P.trade.has_lv != 0;
  const P32Args a{P.trade, tb, scen, scen32, P.n_scen, sh.Pb, sh.TT, NNmax, P.stack_max, ln_ko, ln_cb, ln_ki,
                  path0, npaths, plan, out.partial, out.ko_steps, out.records};
  const bool rec = out.records != nullptr;
#define RG_GO(NN)                                                                         \
  if (sh.ppt == 2) p32_kernel_launch_n##NN##p2(lvk, rec, sh.grid, sh.threads, sh.smem, st, a); \
  else p32_kernel_launch_n##NN##p1(lvk, rec, sh.grid, sh.threads, sh.smem, st, a);
  switch (P.n) {
    case 1: RG_GO(1) break;
    case 2: RG_GO(2) break;
    case 3: RG_GO(3) break;
    case 4: RG_GO(4) break;
    case 5: RG_GO(5) break;
    default: raise(RG_ERR_INVALID_MARKET_SHAPE, "unsupported asset count");
  }
#undef RG_GO
  cuda_check(cudaGetLastError(), "phoenix32_kernel launch");
}

int p32_phase_clocks(unsigned long long out[4], bool reset) {
  int (*const tus[10])(unsigned long long*, bool) = {
      p32_phase_clocks_n1p1, p32_phase_clocks_n1p2, p32_phase_clocks_n2p1, p32_phase_clocks_n2p2,
      p32_phase_clocks_n3p1, p32_phase_clocks_n3p2, p32_phase_clocks_n4p1, p32_phase_clocks_n4p2,
      p32_phase_clocks_n5p1, p32_phase_clocks_n5p2};
  for (int k = 0; k < 4; ++k) out[k] = 0;
  int have = 0;
  for (auto f : tus) {
    unsigned long long v[4];
    have = f(v, reset);
    if (have)
      for (int k = 0; k < 4; ++k) out[k] += v[k];
  }
  return have;
}

}  // namespace rg
