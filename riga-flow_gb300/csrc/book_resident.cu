// book_resident.cu — resident books: rg_book_create / rg_book_price / rg_book_destroy.
//
// A resident book is uploaded once: its trade tables, QMC tables, bridge schedule and universe
// Cholesky factor stay on the device, and so do the universe's FP32 increments of every path
// (generated once at creation; they do not depend on the scenarios).  Each rg_book_price call
// then only prices: it plans the scenario tables on the host, writes them to a pinned staging
// buffer and replays a CUDA graph of the device work — the scenario upload, one persistent TMA
// scan per underlying count, the fixed-order reduction and the download of the sums — captured
// on the first call for that scenario count.  Before the capture, an autotuner times the scan's
// stage depth (time steps per TMA stage) on a prefix of the paths and keeps the fastest; the
// stage depth changes only the schedule, never the arithmetic, so results equal rg_price_book's
// for the same book and scenarios bit for bit.
#include <chrono>
#include <map>
#include <memory>

#include "rg_book.h"

namespace rg {
namespace {

// Device bytes of increments a resident book may keep (they are 80 B per path-step for a
// 20-asset universe: 26 GB at 2^18 paths × 1260 steps).
constexpr size_t kResidentBudget = size_t(96) << 30;

// One captured graph per scenario count, with the buffers it was captured on (a graph holds
// their addresses, so they are never reallocated).
struct GraphEntry {
  cudaGraphExec_t exec = nullptr;
  Book32Shape sh{};
  size_t scen_bytes = 0;
  DevBuf scen_dev, partial, sums;
  HostBuf scen_host, sums_host;
  ~GraphEntry() {
    if (exec) cudaGraphExecDestroy(exec);
  }
};

}  // namespace
}  // namespace rg

struct rg_book {
  rg_engine* E = nullptr;
  // the universe market (for the default scenario) and the request's config
  std::string as_of;
  std::vector<double> spots, vols, q, corr;
  rg_market_snapshot universe{};
  rg_simulation_config config{};
  rg::bk::BookPlan B;
  rg::bk::BookStaged st;
  rg::DevBuf tables, incr, scratch;
  uint64_t P = 0, rowlen = 0;
  std::map<int, rg::GraphEntry> graphs;
  std::map<int, int> tuned;  // scenario count → stage depth
};

namespace rg {
namespace {

using namespace bk;

// Times the scan of a prefix of the paths for each candidate stage depth; returns the fastest.
int autotune_stage(rg_book* b, const Book32Shape& base) {
  rg_engine* E = b->E;
  const int S = b->B.S;
  std::vector<int> cands;
  for (int tt : {8, 16, 32, 64})
    if (2 * 5 * tt * base.Pb * 4 <= 168 * 1024) cands.push_back(tt);
  const uint64_t np = std::min<uint64_t>(b->P, (uint64_t)base.blk_paths * 4);
  const size_t pbytes = sizeof(double) * ((np + base.blk_paths - 1) / base.blk_paths) * b->B.n_trades * S * RG_ACC;
  DevBuf tpartial;
  tpartial.ensure(pbytes);
  cudaEvent_t e0, e1;
  cuda_check(cudaEventCreate(&e0), "event");
  cuda_check(cudaEventCreate(&e1), "event");
  int best = cands.empty() ? base.TT : cands.back();
  float best_ms = 1e30f;
  BookDev bkd = b->st.bk;
  for (int tt : cands) {
    Book32Shape sh = base;
    sh.TT = tt;
    sh.smem = 2 * 5 * tt * sh.Pb * 4 + 64;
    CUtensorMap maps[RG_NMAX];
    increments_maps(static_cast<float*>(b->incr.ptr), b->P, b->rowlen, b->B.U, b->B.TU, sh, maps);
    int32_t* scr = static_cast<int32_t*>(b->scratch.ptr);
    float ms = 0;
    for (int rep = 0; rep < 2; ++rep) {  // the first run warms the caches
      cuda_check(cudaMemsetAsync(scr, 0, 256, E->stream), "tune status");
      cuda_check(cudaEventRecord(e0, E->stream), "event");
      launch_book_trade32(bkd, sh, maps, np, 0, b->B.group_lo, b->B.group_n, static_cast<double*>(tpartial.ptr),
                          scr, scr + 1, E->stream);
      cuda_check(cudaEventRecord(e1, E->stream), "event");
      cuda_check(cudaEventSynchronize(e1), "tune");
      cuda_check(cudaEventElapsedTime(&ms, e0, e1), "event time");
    }
    int st = 0;
    cuda_check(cudaMemcpy(&st, scr + 1, sizeof st, cudaMemcpyDeviceToHost), "D2H");
    if (st) raise(st == KSTAT_TIMEOUT ? RG_ERR_TIMEOUT : RG_ERR_GPU_ERROR, "book autotune launch failed");
    if (ms < best_ms) {
      best_ms = ms;
      best = tt;
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  return best;
}

void price_resident(rg_book* b, const BookScenarios& spec, rg_price_result* out) {
  rg_engine* E = b->E;
  validate_book_scenarios(b->universe, spec);
  rg_book_request view{};
  view.universe = b->universe;
  plan_book_scenarios(&view, spec, b->B);
  const int S = b->B.S;
  if (S > 32) raise(RG_ERR_INVALID_ARGUMENT, "at most 32 scenarios per book price");
  const int pairs = b->B.n_trades * S;
  const ScenarioPack sp = pack_book_scenarios(b->B);
  const size_t scen_bytes = sp.pk.host.size();
  // one graph per scenario count, per-trade bump sets apart; tables of another size (other bump
  // sizes can merge or split markets) are captured again
  GraphEntry& g = b->graphs[spec.per_trade ? 1000 + S : S];
  if (g.exec && scen_bytes != g.scen_bytes) {
    cudaGraphExecDestroy(g.exec);
    g.exec = nullptr;
  }
  if (!g.exec) {
    // this scenario count's buffers, then tune the stage depth, then capture
    g.scen_dev.release();
    g.scen_host.release();
    g.scen_dev.ensure(scen_bytes);
    g.scen_host.ensure(scen_bytes);
    memcpy(g.scen_host.ptr, sp.pk.host.data(), scen_bytes);
    cuda_check(cudaMemcpyAsync(g.scen_dev.ptr, g.scen_host.ptr, scen_bytes, cudaMemcpyHostToDevice, E->stream), "H2D");
    point_scenarios(sp, static_cast<uint8_t*>(g.scen_dev.ptr), S, b->st.bk);
    Book32Shape sh = book32_shape(S, device_sm_count(), b->P, b->B.min_group());
    sh.TT = autotune_stage(b, sh);
    sh.smem = 2 * 5 * sh.TT * sh.Pb * 4 + 64;
    b->tuned[spec.per_trade ? 1000 + S : S] = sh.TT;
    const uint64_t blocks = (b->P + sh.blk_paths - 1) / sh.blk_paths;
    g.partial.ensure(sizeof(double) * blocks * pairs * RG_ACC);
    g.sums.ensure(sizeof(double) * pairs * RG_ACC);
    g.sums_host.ensure(sizeof(double) * pairs * RG_ACC + 64);
    CUtensorMap maps[RG_NMAX];
    increments_maps(static_cast<float*>(b->incr.ptr), b->P, b->rowlen, b->B.U, b->B.TU, sh, maps);
    int32_t* scr = static_cast<int32_t*>(b->scratch.ptr);
    cuda_check(cudaStreamSynchronize(E->stream), "book before capture");
    cudaGraph_t graph = nullptr;
    cuda_check(cudaStreamBeginCapture(E->stream, cudaStreamCaptureModeThreadLocal), "begin capture");
    try {
      cuda_check(cudaMemcpyAsync(g.scen_dev.ptr, g.scen_host.ptr, scen_bytes, cudaMemcpyHostToDevice, E->stream),
                 "scenarios H2D");
      cuda_check(cudaMemsetAsync(scr, 0, 256, E->stream), "status reset");
      launch_book_trade32(b->st.bk, sh, maps, b->P, 0, b->B.group_lo, b->B.group_n, static_cast<double*>(g.partial.ptr),
                          scr, scr + 1, E->stream);
      launch_book_reduce_strided(static_cast<double*>(g.partial.ptr), (int64_t)blocks, (int64_t)pairs * RG_ACC, RG_ACC,
                                 pairs, static_cast<double*>(g.sums.ptr), E->stream);
      cuda_check(cudaMemcpyAsync(g.sums_host.ptr, g.sums.ptr, sizeof(double) * pairs * RG_ACC, cudaMemcpyDeviceToHost,
                                 E->stream), "sums D2H");
      cuda_check(cudaMemcpyAsync(static_cast<uint8_t*>(g.sums_host.ptr) + sizeof(double) * pairs * RG_ACC, scr + 1,
                                 sizeof(int), cudaMemcpyDeviceToHost, E->stream), "status D2H");
    } catch (...) {
      cudaStreamEndCapture(E->stream, &graph);
      if (graph) cudaGraphDestroy(graph);
      throw;
    }
    cuda_check(cudaStreamEndCapture(E->stream, &graph), "end capture");
    const cudaError_t inst = cudaGraphInstantiate(&g.exec, graph, 0);
    cudaGraphDestroy(graph);
    cuda_check(inst, "graph instantiate");
    g.sh = sh;
    g.scen_bytes = scen_bytes;
  }
  if (scen_bytes != g.scen_bytes) raise(RG_ERR_GPU_ERROR, "resident book: scenario tables changed size");
  memcpy(g.scen_host.ptr, sp.pk.host.data(), scen_bytes);
  cuda_check(cudaGraphLaunch(g.exec, E->stream), "graph launch");
  cuda_check(cudaStreamSynchronize(E->stream), "book price");
  const double* hs = static_cast<const double*>(g.sums_host.ptr);
  int kst = 0;
  memcpy(&kst, static_cast<const uint8_t*>(g.sums_host.ptr) + sizeof(double) * pairs * RG_ACC, sizeof kst);
  if (kst == KSTAT_TIMEOUT) raise(RG_ERR_TIMEOUT, "book scan: a bounded stage wait ran out");
  if (kst) raise(RG_ERR_GPU_ERROR, "book scan reported a bad work item");
  for (int k = 0; k < pairs * RG_ACC; ++k)
    if (!std::isfinite(hs[k])) raise(RG_ERR_GPU_ERROR, "book: non-finite path sums");
  for (int p = 0; p < pairs; ++p) finish(hs + (size_t)p * RG_ACC, b->P, b->config.seed, &out[p]);
}

}  // namespace
}  // namespace rg

using namespace rg;

extern "C" int32_t rg_book_create(rg_engine* e, const rg_book_request* request, rg_book** out) {
  RG_TRY({
    if (!e || !request || !out) raise(RG_ERR_INVALID_ARGUMENT, "null argument");
    *out = nullptr;
    int32_t g = rg_guard_device();
    if (g) return g;
    if (request->config.precision != RG_PRECISION_FP32)
      raise(RG_ERR_UNSUPPORTED, "resident books run the FP32 production kernels (use rg_price_book for FP64 parity)");
    bk::validate_book(request, bk::BookScenarios{});
    std::lock_guard<std::mutex> lock(e->mu);
    cuda_check(cudaSetDevice(e->device), "cudaSetDevice");
    std::unique_ptr<rg_book> b(new rg_book());
    b->E = e;
    const rg_market_snapshot& u = request->universe;
    const int U = u.n_assets;
    b->as_of = u.as_of;
    b->spots.assign(u.spots, u.spots + U);
    b->vols.assign(u.vols, u.vols + U);
    b->q.assign(u.dividend_yields, u.dividend_yields + U);
    b->corr.assign(u.correlation, u.correlation + (size_t)U * U);
    b->universe = u;
    b->universe.as_of = b->as_of.c_str();
    b->universe.spots = b->spots.data();
    b->universe.vols = b->vols.data();
    b->universe.dividend_yields = b->q.data();
    b->universe.correlation = b->corr.data();
    b->config = request->config;
    bk::plan_book(request, bk::BookScenarios{}, b->B);
    b->st = bk::stage_book_static(b->tables, e->stream, request, b->B);
    b->P = request->config.paths;
    b->rowlen = (b->P + 63) / 64 * 64;
    const size_t ibytes = sizeof(float) * (size_t)U * (size_t)b->B.TU * (size_t)b->rowlen;
    if (ibytes > kResidentBudget)
      raise(RG_ERR_INVALID_ARGUMENT, "the book's increments (" + std::to_string(ibytes >> 30) +
                                         " GiB) exceed the resident budget; price it with rg_price_book");
    b->incr.ensure(ibytes);
    b->scratch.ensure(256);
    launch_book_gen32(b->B.gen, b->st.tb, b->st.L32, U, request->config.first_path, b->P, b->rowlen,
                      static_cast<float*>(b->incr.ptr), e->stream);
    cuda_check(cudaStreamSynchronize(e->stream), "book generation");
    *out = b.release();
  })
}

extern "C" int32_t rg_book_price(rg_book* book, const rg_market_snapshot* scenarios, int32_t n_scenarios,
                                 rg_price_result* out) {
  RG_TRY({
    if (!book || !out) raise(RG_ERR_INVALID_ARGUMENT, "null argument");
    std::lock_guard<std::mutex> lock(book->E->mu);
    cuda_check(cudaSetDevice(book->E->device), "cudaSetDevice");
    bk::BookScenarios sc;
    sc.sc = scenarios;
    sc.n = n_scenarios;
    price_resident(book, sc, out);
  })
}

extern "C" int32_t rg_book_price_trade_bumps(rg_book* book, const rg_book_bumps* sizes, rg_price_result* out) {
  RG_TRY({
    if (!book || !out) raise(RG_ERR_INVALID_ARGUMENT, "null argument");
    std::lock_guard<std::mutex> lock(book->E->mu);
    cuda_check(cudaSetDevice(book->E->device), "cudaSetDevice");
    bk::BookScenarios sc;
    sc.bumps = sizes;
    sc.per_trade = true;
    price_resident(book, sc, out);
  })
}

extern "C" int32_t rg_book_tuned_stage(rg_book* book, int32_t n_scenarios, int32_t* steps_per_stage) {
  RG_TRY({
    if (!book || !steps_per_stage) raise(RG_ERR_INVALID_ARGUMENT, "null argument");
    const int S = n_scenarios > 0 ? n_scenarios : 1;
    auto it = book->tuned.find(S);
    *steps_per_stage = it == book->tuned.end() ? 0 : it->second;
  })
}

extern "C" void rg_book_destroy(rg_book* book) {
  if (!book) return;
  {
    std::lock_guard<std::mutex> lock(book->E->mu);
    cudaStreamSynchronize(book->E->stream);
  }
  delete book;
}
