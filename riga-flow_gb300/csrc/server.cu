// server.cu — the continuous-batching request server (rg_server_*).
//
// Slots: one engine (CUDA stream + growable workspace) and one worker thread per slot.  Requests
// are deep-copied at submission into owned storage and queued in arrival order.  A worker takes the
// head of the queue when the head's device-memory estimate fits: the budget is compared with the
// sum over slots of what each holds (a running slot counts max(held, its request's estimate)); when
// the head does not fit, idle slots release their buffers first.  Requests therefore enter as
// slots and memory free up, and the ones admitted run concurrently on their own streams.  Requests
// whose work (paths × steps × scenarios, summed over a book's trades) reaches the large-work mark
// may hold at most max_large_slots slots at once; a worker takes the first queued request it may
// start, so small requests pass large ones that are waiting for a large slot.  A request that waits
// for memory is passed only by requests whose estimate is at most a sixteenth of the budget (single
// trades beside a waiting book), which can hold back little of the memory it waits for.  Each
// request runs through the same entry points as a direct call (rg_price_scenarios,
// rg_price_risk_batch, rg_price_book, rg_price_book_trade_bumps), so its results are independent of
// what runs beside it.
#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <deque>
#include <memory>
#include <thread>
#include <unordered_map>

#include "rg_internal.h"

namespace rg {
namespace {

using Clock = std::chrono::steady_clock;

// ------------------------------------------------------------------ owned request copies -------
struct OwnedMarket {
  std::string as_of;
  std::vector<double> spots, vols, q, corr;
  bool has_corr = false;
  rg_market_snapshot m{};
  void copy(const rg_market_snapshot& s) {
    const int n = s.n_assets > 0 ? s.n_assets : 0;
    as_of = s.as_of ? s.as_of : "";
    auto take = [n](const double* p, size_t cnt, std::vector<double>& v) {
      if (p) v.assign(p, p + cnt);
      else v.clear();
    };
    take(s.spots, n, spots);
    take(s.vols, n, vols);
    take(s.dividend_yields, n, q);
    has_corr = s.correlation != nullptr;
    take(s.correlation, (size_t)n * n, corr);
    m = s;
    m.as_of = s.as_of ? as_of.c_str() : nullptr;
    m.spots = s.spots ? spots.data() : nullptr;
    m.vols = s.vols ? vols.data() : nullptr;
    m.dividend_yields = s.dividend_yields ? q.data() : nullptr;
    m.correlation = has_corr ? corr.data() : nullptr;
  }
};

struct OwnedTrade {
  std::string id;
  std::vector<double> init;
  rg_phoenix_trade t{};
  void copy(const rg_phoenix_trade& s) {
    id = s.trade_id ? s.trade_id : "";
    const int n = s.n_assets > 0 ? s.n_assets : 0;
    if (s.initial_spots) init.assign(s.initial_spots, s.initial_spots + n);
    t = s;
    t.trade_id = s.trade_id ? id.c_str() : nullptr;
    t.initial_spots = s.initial_spots ? init.data() : nullptr;
  }
};

struct OwnedRequest {
  OwnedTrade trade;
  OwnedMarket market;
  std::string as_of;
  std::vector<std::vector<double>> grid_data;  // per grid: maturities, strikes, vols
  std::vector<rg_implied_vol_grid> grids;
  rg_price_request r{};
  void copy(const rg_price_request& s) {
    trade.copy(s.trade);
    market.copy(s.market);
    as_of = s.as_of ? s.as_of : "";
    r = s;
    r.trade = trade.t;
    r.market = market.m;
    r.as_of = s.as_of ? as_of.c_str() : nullptr;
    grids.clear();
    grid_data.clear();
    if (s.n_local_vol > 0 && s.local_vol) {
      grids.resize(s.n_local_vol);
      grid_data.resize((size_t)s.n_local_vol * 3);
      for (int f = 0; f < s.n_local_vol; ++f) {
        const rg_implied_vol_grid& g = s.local_vol[f];
        const size_t nt = g.n_maturities > 0 ? g.n_maturities : 0, nk = g.n_strikes > 0 ? g.n_strikes : 0;
        auto& a = grid_data[f * 3], &b = grid_data[f * 3 + 1], &c = grid_data[f * 3 + 2];
        if (g.maturities_years) a.assign(g.maturities_years, g.maturities_years + nt);
        if (g.strikes) b.assign(g.strikes, g.strikes + nk);
        if (g.vols) c.assign(g.vols, g.vols + nt * nk);
        grids[f] = g;
        grids[f].maturities_years = g.maturities_years ? a.data() : nullptr;
        grids[f].strikes = g.strikes ? b.data() : nullptr;
        grids[f].vols = g.vols ? c.data() : nullptr;
      }
      r.local_vol = grids.data();
    } else {
      r.local_vol = nullptr;
    }
  }
};

struct OwnedScenario {
  OwnedMarket market;
  std::vector<double> shift;
  rg_scenario s{};
};

struct OwnedBook {
  OwnedMarket universe;
  std::vector<OwnedTrade> trades;
  std::vector<std::vector<int32_t>> under;
  std::vector<rg_book_trade> views;
  rg_book_request r{};
  void copy(const rg_book_request& s) {
    universe.copy(s.universe);
    const int n = s.n_trades > 0 && s.trades ? s.n_trades : 0;
    trades.resize(n);
    under.resize(n);
    views.resize(n);
    for (int j = 0; j < n; ++j) {
      trades[j].copy(s.trades[j].terms);
      const int k = s.trades[j].terms.n_assets > 0 ? s.trades[j].terms.n_assets : 0;
      if (s.trades[j].underlyings) under[j].assign(s.trades[j].underlyings, s.trades[j].underlyings + k);
      views[j].terms = trades[j].t;
      views[j].underlyings = s.trades[j].underlyings ? under[j].data() : nullptr;
    }
    r = s;
    r.universe = universe.m;
    r.trades = n ? views.data() : s.trades;
  }
};

// ------------------------------------------------------------------ jobs and the server --------
struct Job {
  uint64_t id = 0;
  int kind = RG_JOB_PRICE;
  OwnedRequest req;
  std::vector<OwnedScenario> scen;
  std::vector<rg_scenario> scen_views;
  rg_central_difference_config risk_cfg{};
  OwnedBook book;
  rg_book_bumps bumps{};  // per-trade bump sizes of an RG_JOB_BOOK_BUMPS request
  bool has_bumps = false;
  std::vector<OwnedMarket> book_scen;
  std::vector<rg_market_snapshot> book_scen_views;
  size_t est = 0;
  double work = 0;     // path-steps × scenarios the request prices
  bool large = false;  // work at or above the server's large-work mark
  bool waited_memory = false;  // was passed over at least once because it did not fit the budget
  uint64_t n_results = 0;
  int state = RG_JOB_QUEUED;
  int32_t status = RG_OK;
  std::string error;
  int slot = -1;
  bool cancel = false;
  std::vector<rg_price_result> results;
  std::unique_ptr<rg_batch_risk_report> report;
  double t_submit = 0, t_start = 0, t_end = 0;
};

struct Slot {
  rg_engine* engine = nullptr;
  size_t held = 0;      // device bytes the engine's workspace holds
  size_t running = 0;   // estimate of the request it runs (0 when idle)
  bool busy = false;
  bool busy_large = false;  // running a large request
  bool trimming = false;    // another worker releases this idle engine's buffers (outside the lock)
};

}  // namespace
}  // namespace rg

struct rg_server {
  int device = 0;
  size_t budget = 0;
  std::chrono::steady_clock::time_point t0;
  std::mutex mu;
  std::condition_variable cv_work, cv_done;
  std::vector<rg::Slot> slots;
  std::vector<std::thread> workers;
  std::deque<rg::Job*> queue;
  std::unordered_map<uint64_t, std::unique_ptr<rg::Job>> jobs;
  uint64_t next_id = 1;
  bool stopping = false;
  uint64_t submitted = 0, completed = 0, failed = 0, cancelled = 0;
  std::vector<double> latencies_ms;
  int n_running = 0;
  double busy_s = 0, busy_since = 0;
  int max_large = 1;        // slots large requests may hold at once
  double large_work = 0;    // work at which a request counts as large
  int large_sms = 0;        // SMs a large request's grids are sized for (0: all)
  int n_large = 0;          // large requests running
  uint64_t memory_waits = 0;  // requests that waited at the head of the queue for device memory
  size_t peak_reserved = 0;   // largest reservation (the slots' holdings and running estimates)
};

namespace rg {
namespace {

double now_s(const rg_server* S) {
  return std::chrono::duration<double>(Clock::now() - S->t0).count();
}

size_t reserved(const rg_server* S) {
  size_t b = 0;
  for (const Slot& s : S->slots) b += s.busy ? std::max(s.held, s.running) : s.held;
  return b;
}

// Under S->mu: whether `job` can start on slot k now, counting as free the buffers of the idle
// slots listed in `trim` (the smallest set, in slot order, that makes room).  Releasing buffers
// (cudaFree) waits for the device, so the caller does it after dropping the lock.
bool admit(rg_server* S, int k, const Job* job, std::vector<int>& trim) {
  trim.clear();
  size_t freed = 0;
  auto need = [&]() {
    return reserved(S) - freed - S->slots[k].held + std::max(S->slots[k].held, job->est);
  };
  if (need() <= S->budget) return true;
  for (size_t i = 0; i < S->slots.size(); ++i) {
    const Slot& s = S->slots[i];
    if ((int)i == k || s.busy || s.trimming || s.held == 0) continue;
    trim.push_back((int)i);
    freed += s.held;
    if (need() <= S->budget) return true;
  }
  trim.clear();
  return false;
}

void run_job(rg_engine* E, Job* job) {
  int32_t st = RG_OK;
  switch (job->kind) {
    case RG_JOB_PRICE:
      if (job->scen_views.empty()) st = rg_price_put_leg(E, &job->req.r, job->results.data());
      else st = rg_price_scenarios(E, &job->req.r, job->scen_views.data(), (int32_t)job->scen_views.size(), job->results.data());
      break;
    case RG_JOB_RISK:
      job->report.reset(new rg_batch_risk_report());
      st = rg_price_risk_batch(E, &job->req.r, &job->risk_cfg, job->report.get());
      break;
    case RG_JOB_BOOK:
      st = rg_price_book(E, &job->book.r, job->book_scen_views.empty() ? nullptr : job->book_scen_views.data(),
                         (int32_t)job->book_scen_views.size(), job->results.data());
      break;
    case RG_JOB_BOOK_BUMPS:
      st = rg_price_book_trade_bumps(E, &job->book.r, job->has_bumps ? &job->bumps : nullptr, job->results.data());
      break;
    default:
      st = RG_ERR_INVALID_ARGUMENT;
  }
  job->status = st;
  if (st != RG_OK) {
    char buf[1024];
    rg_last_error(buf, sizeof buf);
    job->error = buf;
  }
}

// Under S->mu: the queued request slot k starts next, or null.  Requests go in arrival order,
// except that a large one waiting for a large slot is passed, and one that does not fit the memory
// budget is passed only by requests of at most a sixteenth of the budget (later requests with larger
// estimates never overtake it on memory).
// A request larger than a sixteenth of the budget goes to a slot whose buffers already hold most
// of its estimate (80%; estimates are upper bounds) when there is one — waiting for it if it is
// running a short request — so that no buffers are released and allocated again (cudaFree and a
// large cudaMalloc wait for the whole device).
Job* next_job(rg_server* S, int k, std::vector<int>& trim) {
  if (S->slots[k].trimming) return nullptr;
  bool waiting = false;  // an earlier request waits for memory
  for (Job* j : S->queue) {
    if (j->large && S->n_large >= S->max_large) continue;
    if (waiting && j->est > S->budget / 16) continue;
    auto holds = [&](const Slot& s) { return s.held / 4 >= j->est / 5; };
    if (j->est > S->budget / 16 && !holds(S->slots[k])) {
      bool other = false;
      for (size_t i = 0; i < S->slots.size(); ++i) {
        const Slot& s = S->slots[i];
        other = other || ((int)i != k && !s.trimming && !s.busy_large && holds(s));
      }
      if (other) {  // left to that slot's worker; nothing larger than small requests passes it
        waiting = true;
        continue;
      }
    }
    if (admit(S, k, j, trim)) return j;
    if (!j->waited_memory) {
      j->waited_memory = true;
      ++S->memory_waits;
    }
    waiting = true;
  }
  return nullptr;
}

void worker(rg_server* S, int k) {
  std::unique_lock<std::mutex> lock(S->mu);
  std::vector<int> trim;
  for (;;) {
    Job* job = nullptr;
    S->cv_work.wait(lock, [&] {
      if (S->stopping) return true;
      job = next_job(S, k, trim);
      return job != nullptr;
    });
    if (S->stopping) return;
    S->queue.erase(std::find(S->queue.begin(), S->queue.end(), job));
    if (job->large) ++S->n_large;
    Slot& slot = S->slots[k];
    slot.busy = true;
    slot.busy_large = job->large;
    slot.running = job->est;
    for (int i : trim) {  // counted free from now on; released below, outside the lock
      S->slots[i].trimming = true;
      S->slots[i].held = 0;
    }
    S->peak_reserved = std::max(S->peak_reserved, reserved(S));
    job->state = RG_JOB_RUNNING;
    job->slot = k;
    job->t_start = now_s(S);
    if (S->n_running++ == 0) S->busy_since = job->t_start;
    // the head may have changed: let another idle worker look at the new head
    S->cv_work.notify_all();
    lock.unlock();
    if (!trim.empty()) {
      for (int i : trim) engine_trim(S->slots[i].engine);
      lock.lock();
      for (int i : trim) S->slots[i].trimming = false;
      S->cv_work.notify_all();
      lock.unlock();
    }
    // large requests run at default priority on a share of the SMs; small ones at the highest
    // priority on all of them, so they pass a large request's kernels
    engine_set_class(slot.engine, !job->large, job->large ? S->large_sms : 0);
    run_job(slot.engine, job);
    const size_t held = engine_device_bytes(slot.engine);
    lock.lock();
    job->t_end = now_s(S);
    if (job->large) --S->n_large;
    if (--S->n_running == 0) S->busy_s += job->t_end - S->busy_since;
    slot.busy = false;
    slot.busy_large = false;
    slot.running = 0;
    slot.held = held;
    S->peak_reserved = std::max(S->peak_reserved, reserved(S));
    if (job->cancel) {
      job->state = RG_JOB_CANCELLED;
      ++S->cancelled;
    } else if (job->status == RG_OK) {
      job->state = RG_JOB_DONE;
      ++S->completed;
      S->latencies_ms.push_back(1e3 * (job->t_end - job->t_submit));
    } else {
      job->state = RG_JOB_FAILED;
      ++S->failed;
    }
    S->cv_done.notify_all();
    S->cv_work.notify_all();
  }
}

uint64_t enqueue(rg_server* S, std::unique_ptr<Job> job) {
  if (job->est > S->budget)
    raise(RG_ERR_INVALID_ARGUMENT, "the request needs about " + std::to_string(job->est >> 20) +
                                       " MiB of device memory, more than the server's budget of " +
                                       std::to_string(S->budget >> 20) + " MiB");
  std::lock_guard<std::mutex> lock(S->mu);
  if (S->stopping) raise(RG_ERR_CANCELLED, "the server is shutting down");
  job->large = job->work >= S->large_work;
  job->id = S->next_id++;
  job->t_submit = now_s(S);
  Job* raw = job.get();
  S->jobs[raw->id] = std::move(job);
  S->queue.push_back(raw);
  ++S->submitted;
  S->cv_work.notify_all();
  return raw->id;
}

Job* find(rg_server* S, uint64_t ticket) {
  auto it = S->jobs.find(ticket);
  if (it == S->jobs.end()) raise(RG_ERR_INVALID_ARGUMENT, "unknown ticket " + std::to_string(ticket));
  return it->second.get();
}

void fill_info(const Job* j, rg_job_info* info) {
  if (!info) return;
  info->state = j->state;
  info->status = j->status;
  info->kind = j->kind;
  info->slot = j->slot;
  info->n_results = j->n_results;
  info->device_bytes = j->est;
  info->submit_s = j->t_submit;
  info->start_s = j->t_start;
  info->end_s = j->t_end;
}

double percentile(std::vector<double> v, double q) {
  if (v.empty()) return 0.0;
  std::sort(v.begin(), v.end());
  const size_t i = (size_t)std::min<double>((double)v.size() - 1, std::ceil(q * (double)v.size()) - 1);
  return v[i];
}

}  // namespace
}  // namespace rg

using namespace rg;

extern "C" int32_t rg_server_create(const rg_server_config* cfg, rg_server** out) {
  RG_TRY({
    if (!out) raise(RG_ERR_INVALID_ARGUMENT, "null output handle");
    *out = nullptr;
    int32_t g = rg_guard_device();
    if (g) return g;
    const int device = cfg ? cfg->device : 0;
    const int n_slots = cfg && cfg->slots > 0 ? cfg->slots : 4;
    if (n_slots > 64) raise(RG_ERR_INVALID_ARGUMENT, "at most 64 slots");
    std::unique_ptr<rg_server> S(new rg_server());
    S->device = device;
    S->t0 = Clock::now();
    cuda_check(cudaSetDevice(device), "cudaSetDevice");
    size_t free_b = 0, total_b = 0;
    cuda_check(cudaMemGetInfo(&free_b, &total_b), "cudaMemGetInfo");
    S->budget = cfg && cfg->device_memory_budget ? (size_t)cfg->device_memory_budget : free_b / 10 * 8;
    S->max_large = cfg && cfg->max_large_slots > 0 ? std::min(cfg->max_large_slots, n_slots)
                                                   : std::max(1, n_slots / 2);
    S->large_work = cfg && cfg->large_work > 0 ? (double)cfg->large_work : 2147483648.0;
    {
      int sms = 0;
      cuda_check(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device), "SM count");
      const int want = cfg ? cfg->large_max_sms : 0;
      S->large_sms = want < 0 ? 0 : (want == 0 ? sms - sms / 3 : std::min(want, sms));
    }
    S->slots.resize(n_slots);
    for (int k = 0; k < n_slots; ++k) {
      int32_t st = rg_engine_create(device, &S->slots[k].engine);
      if (st) {
        for (int i = 0; i < k; ++i) rg_engine_destroy(S->slots[i].engine);
        return st;
      }
    }
    rg_server* raw = S.get();
    for (int k = 0; k < n_slots; ++k) S->workers.emplace_back(worker, raw, k);
    *out = S.release();
  })
}

extern "C" void rg_server_destroy(rg_server* S) {
  if (!S) return;
  {
    std::lock_guard<std::mutex> lock(S->mu);
    for (Job* j : S->queue) {
      j->state = RG_JOB_CANCELLED;
      ++S->cancelled;
    }
    S->queue.clear();
  }
  {
    // let running requests finish, then stop the workers
    std::unique_lock<std::mutex> lock(S->mu);
    S->cv_done.wait(lock, [&] { return S->n_running == 0; });
    S->stopping = true;
    S->cv_work.notify_all();
  }
  for (std::thread& t : S->workers) t.join();
  for (Slot& s : S->slots) rg_engine_destroy(s.engine);
  delete S;
}

extern "C" int32_t rg_server_submit_price(rg_server* S, const rg_price_request* req, const rg_scenario* sc,
                                          int32_t n, uint64_t* ticket) {
  RG_TRY({
    if (!S || !req || !ticket || n < 0 || (n > 0 && !sc)) raise(RG_ERR_INVALID_ARGUMENT, "null argument");
    validate_request(req);
    std::unique_ptr<Job> job(new Job());
    job->kind = RG_JOB_PRICE;
    job->req.copy(*req);
    job->scen.resize(n);
    job->scen_views.resize(n);
    for (int i = 0; i < n; ++i) {
      job->scen[i].market.copy(sc[i].market);
      const int na = sc[i].market.n_assets > 0 ? sc[i].market.n_assets : 0;
      job->scen_views[i].market = job->scen[i].market.m;
      if (sc[i].implied_vol_shift) {
        job->scen[i].shift.assign(sc[i].implied_vol_shift, sc[i].implied_vol_shift + na);
        job->scen_views[i].implied_vol_shift = job->scen[i].shift.data();
      } else {
        job->scen_views[i].implied_vol_shift = nullptr;
      }
    }
    job->n_results = n > 0 ? (uint64_t)n : 1;
    job->results.resize(job->n_results);
    job->est = estimate_price_bytes(&job->req.r, n);
    job->work = (double)req->config.paths * (double)req->trade.steps * (double)job->n_results;
    *ticket = enqueue(S, std::move(job));
  })
}

extern "C" int32_t rg_server_submit_risk(rg_server* S, const rg_price_request* req,
                                         const rg_central_difference_config* cfg, uint64_t* ticket) {
  RG_TRY({
    if (!S || !req || !cfg || !ticket) raise(RG_ERR_INVALID_ARGUMENT, "null argument");
    validate_request(req);
    std::unique_ptr<Job> job(new Job());
    job->kind = RG_JOB_RISK;
    job->req.copy(*req);
    job->risk_cfg = *cfg;
    job->n_results = 0;
    job->est = estimate_price_bytes(&job->req.r, 1 + 4 * req->market.n_assets + 4);
    job->work = (double)req->config.paths * (double)req->trade.steps * (double)(1 + 4 * req->market.n_assets + 4);
    *ticket = enqueue(S, std::move(job));
  })
}

extern "C" int32_t rg_server_submit_book(rg_server* S, const rg_book_request* req, const rg_market_snapshot* sc,
                                         int32_t n, uint64_t* ticket) {
  RG_TRY({
    if (!S || !req || !ticket || n < 0 || (n > 0 && !sc)) raise(RG_ERR_INVALID_ARGUMENT, "null argument");
    std::unique_ptr<Job> job(new Job());
    job->kind = RG_JOB_BOOK;
    job->book.copy(*req);
    job->book_scen.resize(n);
    job->book_scen_views.resize(n);
    for (int i = 0; i < n; ++i) {
      job->book_scen[i].copy(sc[i]);
      job->book_scen_views[i] = job->book_scen[i].m;
    }
    const uint64_t S_ = n > 0 ? (uint64_t)n : 1;
    job->n_results = (uint64_t)(req->n_trades > 0 ? req->n_trades : 0) * S_;
    job->results.resize(job->n_results);
    job->est = estimate_book_bytes(&job->book.r, n);
    double steps = (double)req->universe_steps * (double)req->universe.n_assets;  // the universe generation
    for (int32_t j = 0; j < req->n_trades; ++j) steps += (double)req->trades[j].terms.steps * (double)S_;
    job->work = (double)req->config.paths * steps;
    *ticket = enqueue(S, std::move(job));
  })
}

extern "C" int32_t rg_server_submit_book_trade_bumps(rg_server* S, const rg_book_request* req,
                                                     const rg_book_bumps* sizes, uint64_t* ticket) {
  RG_TRY({
    if (!S || !req || !ticket) raise(RG_ERR_INVALID_ARGUMENT, "null argument");
    std::unique_ptr<Job> job(new Job());
    job->kind = RG_JOB_BOOK_BUMPS;
    job->book.copy(*req);
    if (sizes) {
      job->bumps = *sizes;
      job->has_bumps = true;
    }
    const uint64_t S_ = RG_BOOK_TRADE_SCENARIOS;
    job->n_results = (uint64_t)(req->n_trades > 0 ? req->n_trades : 0) * S_;
    job->results.resize(job->n_results);
    job->est = estimate_book_trade_bumps_bytes(&job->book.r);
    double steps = (double)req->universe_steps * (double)req->universe.n_assets;  // the universe generation
    for (int32_t j = 0; j < req->n_trades; ++j) steps += (double)req->trades[j].terms.steps * (double)S_;
    job->work = (double)req->config.paths * steps;
    *ticket = enqueue(S, std::move(job));
  })
}

extern "C" int32_t rg_server_poll(rg_server* S, uint64_t ticket, rg_job_info* info) {
  RG_TRY({
    if (!S) raise(RG_ERR_INVALID_ARGUMENT, "null server");
    std::lock_guard<std::mutex> lock(S->mu);
    fill_info(find(S, ticket), info);
  })
}

extern "C" int32_t rg_server_wait(rg_server* S, uint64_t ticket, int64_t timeout_ms, rg_job_info* info) {
  RG_TRY({
    if (!S) raise(RG_ERR_INVALID_ARGUMENT, "null server");
    std::unique_lock<std::mutex> lock(S->mu);
    Job* j = find(S, ticket);
    auto done = [&] { return j->state >= RG_JOB_DONE; };
    if (timeout_ms < 0) {
      S->cv_done.wait(lock, done);
    } else if (!S->cv_done.wait_for(lock, std::chrono::milliseconds(timeout_ms), done)) {
      fill_info(j, info);
      raise(RG_ERR_TIMEOUT, "request " + std::to_string(ticket) + " is not finished");
    }
    fill_info(j, info);
    if (j->state == RG_JOB_FAILED) set_last_error(j->error);
  })
}

extern "C" int32_t rg_server_results(rg_server* S, uint64_t ticket, rg_price_result* out, uint64_t capacity) {
  RG_TRY({
    if (!S || !out) raise(RG_ERR_INVALID_ARGUMENT, "null argument");
    std::lock_guard<std::mutex> lock(S->mu);
    Job* j = find(S, ticket);
    if (j->state == RG_JOB_FAILED) raise(j->status, j->error);
    if (j->state == RG_JOB_CANCELLED) raise(RG_ERR_CANCELLED, "request " + std::to_string(ticket) + " was cancelled");
    if (j->state != RG_JOB_DONE) raise(RG_ERR_INVALID_ARGUMENT, "request " + std::to_string(ticket) + " is not finished");
    if (j->kind == RG_JOB_RISK) raise(RG_ERR_INVALID_ARGUMENT, "a risk request has a report, not results");
    if (capacity < j->n_results) raise(RG_ERR_INVALID_ARGUMENT, "output capacity is smaller than n_results");
    std::copy(j->results.begin(), j->results.end(), out);
  })
}

extern "C" int32_t rg_server_risk_report(rg_server* S, uint64_t ticket, rg_batch_risk_report* out) {
  RG_TRY({
    if (!S || !out) raise(RG_ERR_INVALID_ARGUMENT, "null argument");
    std::lock_guard<std::mutex> lock(S->mu);
    Job* j = find(S, ticket);
    if (j->state == RG_JOB_FAILED) raise(j->status, j->error);
    if (j->state == RG_JOB_CANCELLED) raise(RG_ERR_CANCELLED, "request was cancelled");
    if (j->state != RG_JOB_DONE || j->kind != RG_JOB_RISK || !j->report)
      raise(RG_ERR_INVALID_ARGUMENT, "no finished risk report for this ticket");
    *out = *j->report;
  })
}

extern "C" int32_t rg_server_cancel(rg_server* S, uint64_t ticket) {
  RG_TRY({
    if (!S) raise(RG_ERR_INVALID_ARGUMENT, "null server");
    std::lock_guard<std::mutex> lock(S->mu);
    Job* j = find(S, ticket);
    if (j->state == RG_JOB_QUEUED) {
      S->queue.erase(std::remove(S->queue.begin(), S->queue.end(), j), S->queue.end());
      j->state = RG_JOB_CANCELLED;
      j->t_end = now_s(S);
      ++S->cancelled;
      S->cv_done.notify_all();
      S->cv_work.notify_all();
    } else if (j->state == RG_JOB_RUNNING) {
      j->cancel = true;
    }
  })
}

extern "C" int32_t rg_server_release(rg_server* S, uint64_t ticket) {
  RG_TRY({
    if (!S) raise(RG_ERR_INVALID_ARGUMENT, "null server");
    std::lock_guard<std::mutex> lock(S->mu);
    Job* j = find(S, ticket);
    if (j->state < RG_JOB_DONE) raise(RG_ERR_INVALID_ARGUMENT, "request is not finished");
    S->jobs.erase(ticket);
  })
}

extern "C" int32_t rg_server_get_stats(rg_server* S, rg_server_stats* out) {
  RG_TRY({
    if (!S || !out) raise(RG_ERR_INVALID_ARGUMENT, "null argument");
    std::lock_guard<std::mutex> lock(S->mu);
    memset(out, 0, sizeof *out);
    out->submitted = S->submitted;
    out->completed = S->completed;
    out->failed = S->failed;
    out->cancelled = S->cancelled;
    out->queued = S->queue.size();
    out->running = (uint64_t)S->n_running;
    for (const Slot& s : S->slots) out->device_bytes_held += s.held;
    out->device_memory_budget = S->budget;
    out->p50_ms = percentile(S->latencies_ms, 0.50);
    out->p99_ms = percentile(S->latencies_ms, 0.99);
    out->max_ms = S->latencies_ms.empty() ? 0.0 : *std::max_element(S->latencies_ms.begin(), S->latencies_ms.end());
    out->busy_s = S->busy_s + (S->n_running ? now_s(S) - S->busy_since : 0.0);
    out->memory_waits = S->memory_waits;
    out->peak_reserved_bytes = S->peak_reserved;
  })
}
