// Host-only check of the FP32 tiled kernel's bridge plans (phoenix32.cu): evaluating a plan level by
// level — every anchor of a level read before any of its values is written, as the kernel's lanes
// do — gives the streamed Brownian bridge's increments bit for bit, for many step counts and every
// tile depth the kernel may launch with.  Both sides use the same single-precision arithmetic
// (without the fused multiply-add, identically on both sides).  Built and run by
// tests/test_bridge_plan.py against the engine library.
#include <cstdio>
#include <cstring>
#include <random>
#include "rg_internal.h"
using namespace rg;

static int check(int64_t T) {
  Prepared P;
  P.T = T;
  P.n = 3;
  P.n_scen = 16;
  bridge_schedule_into(T, 1.0 / 252, P);
  const std::shared_ptr<const BridgePlans> bpp = p32_bridge_plans(P);
  const BridgePlans& bp = *bpp;
  std::mt19937 rng(1234 + (unsigned)T);
  std::normal_distribution<float> nd(0.f, 1.f);
  const int64_t NN = P.node_off[T];
  std::vector<float> z(NN);
  for (auto& v : z) v = nd(rng);
  // streamed bridge (the former B phase, one chain)
  std::vector<float> ref(T), stack(P.stack_max + 1);
  {
    float wc = 0.f;
    int lsp = 0;
    for (int64_t t = 0; t < T; ++t) {
      for (int nd2 = P.node_off[t]; nd2 < P.node_off[t + 1]; ++nd2) {
        const float cf = P.node_cf[nd2];
        const float w = nd2 == 0 ? z[nd2] * cf : z[nd2] * cf + 0.5f * (wc + stack[lsp - 1]);
        stack[lsp++] = w;
      }
      --lsp;
      const float wn = stack[lsp];
      ref[t] = wn - wc;
      wc = wn;
    }
  }
  int bad = 0;
  for (int pi = 0; pi < bp.n; ++pi) {
    const int TT = bp.tt[pi];
    const uint32_t* plan = bp.words.data() + bp.at[pi];
    const int NNmax = TT + P.stack_max;
    std::vector<float> got(T), Zv(NNmax + 1 + P.stack_max, 0.f);
    for (int64_t t0 = 0; t0 < T; t0 += TT) {
      const int tn = (int)std::min<int64_t>(TT, T - t0);
      const int n0 = P.node_off[t0], n1 = P.node_off[t0 + tn];
      for (int j = 0; j < n1 - n0; ++j) Zv[j] = z[n0 + j];
      const uint32_t* hd = plan + 1 + (t0 / TT) * 6;
      auto anchor = [&](uint32_t code) -> float { return Zv[code]; };
      for (uint32_t L = 0; L < hd[2]; ++L) {
        const uint32_t a = plan[hd[1] + L], b = plan[hd[1] + L + 1];
        // evaluate a level "in parallel": read all anchors first, then write
        std::vector<std::pair<int, float>> outv;
        for (uint32_t q = a; q < b; ++q) {
          const uint32_t e = plan[hd[0] + q];
          const int j = e & 511u;
          const uint32_t lc = (e >> 9) & 511u, rc = (e >> 18) & 511u;
          const float cf = P.node_cf[n0 + j];
          const float zz = Zv[j];
          const float w = (e >> 27) ? zz * cf : zz * cf + 0.5f * (anchor(lc) + anchor(rc));
          outv.push_back({j, w});
        }
        for (auto& o : outv) Zv[o.first] = o.second;
      }
      for (int tt = 0; tt < tn; ++tt) {
        const float hi = anchor(plan[hd[5] + t0 + tt]);
        const float lo = tt == 0 ? Zv[NNmax] : anchor(plan[hd[5] + t0 + tt - 1]);
        got[t0 + tt] = hi - lo;
      }
      const float wn = anchor(plan[hd[5] + t0 + tn - 1]);
      for (uint32_t k = 0; k < hd[4]; ++k) {
        const uint32_t e = plan[hd[3] + k];
        Zv[e >> 9] = Zv[e & 511u];
      }
      Zv[NNmax] = wn;
    }
    for (int64_t t = 0; t < T; ++t)
      if (memcmp(&got[t], &ref[t], 4) != 0) {
        if (bad < 5) printf("T=%lld TT=%d step %lld: plan %.9g streamed %.9g\n", (long long)T, TT, (long long)t, got[t], ref[t]);
        ++bad;
        break;
      }
  }
  return bad;
}

int main() {
  int bad = 0, n = 0;
  for (int64_t T : {1, 2, 3, 4, 5, 7, 8, 9, 15, 16, 17, 31, 63, 64, 65, 100, 126, 127, 128, 129, 252, 255, 256, 257,
                    500, 756, 1000, 1023, 1024, 1025, 1260, 2520, 5000}) {
    bad += check(T);
    ++n;
  }
  printf("%d schedules checked, %d mismatching plans\n", n, bad);
  return bad != 0;
}
