// rg_book.h — host-side planning and staging of books, shared by the one-shot pipeline
// (book.cu) and resident books (book_resident.cu).
#pragma once

#include "rg_internal.h"

namespace rg {
namespace bk {

enum BookSlot { BK_TABLES = 0, BK_INCR0, BK_INCR1, BK_PARTIAL, BK_SUMS, BK_RECORDS, BK_SCRATCH, BK_SCEN, BK_NSLOTS };
static_assert(BK_NSLOTS <= 8, "engine book buffers");

// Byte budget of one increments buffer of the one-shot pipeline (two are in flight).
constexpr size_t kIncrBudget = size_t(6) << 30;

struct BookPlan {
  int U = 0, S = 0, n_trades = 0;
  int64_t TU = 0;
  double dt = 0;
  DevTrade gen{};
  Prepared br;  // bridge schedule of the universe grid (node_* and stack_max only)
  std::vector<BookTradeDev> trades;
  std::vector<BookScenDev> scen;
  std::vector<BookPair32> pair32;
  std::vector<double> df, dfm;
  std::vector<int32_t> order;
  int group_lo[RG_NMAX], group_n[RG_NMAX];
  // trades in the smallest non-empty underlying-count group
  int min_group() const {
    int m = 0;
    for (int n = 0; n < RG_NMAX; ++n)
      if (group_n[n] > 0 && (m == 0 || group_n[n] < m)) m = group_n[n];
    return m;
  }
};

// The scenarios a book is priced under: a common list of universe markets (n = 0: the base market
// alone), or, with `bumps`, RG_BOOK_TRADE_SCENARIOS bump scenarios on each trade's own underlyings.
struct BookScenarios {
  const rg_market_snapshot* sc = nullptr;
  int n = 0;
  const rg_book_bumps* bumps = nullptr;
  bool per_trade = false;
};
// The bump of scenario k of a trade on n underlyings (the rule documented with rg_book_trade_bump).
rg_book_bump_spec trade_bump(int n, int k, const rg_book_bumps* sizes);

// Request checks (each trade with the reference's own request validation on its slice of the
// universe) and the plan: static tables, then the scenario tables.
void validate_book(const rg_book_request* r, const BookScenarios& sc);
void validate_book_scenarios(const rg_market_snapshot& universe, const BookScenarios& sc);
void plan_book(const rg_book_request* r, const BookScenarios& sc, BookPlan& B);
void plan_book_scenarios(const rg_book_request* r, const BookScenarios& sc, BookPlan& B);

struct BookStaged {
  DevTables tb{};
  BookDev bk{};
  double* L = nullptr;
  float* L32 = nullptr;
};
// QMC tables, bridge schedule, trades, work order and the universe factor (FP64 Cholesky on the
// device, then its FP32 copy) into `tables`, enqueued on `st`.
BookStaged stage_book_static(DevBuf& tables, cudaStream_t st, const rg_book_request* r, const BookPlan& B);

// The scenario tables packed for one H2D copy; point_scenarios aims `bk` at their device copy.
struct ScenarioPack {
  Pack pk;
  size_t o_scen = 0, o_p32 = 0, o_df = 0, o_dfm = 0, o_df_f = 0, o_dfm_f = 0;
};
ScenarioPack pack_book_scenarios(const BookPlan& B);
void point_scenarios(const ScenarioPack& sp, const uint8_t* dev, int S, BookDev& bk);

void* book_buf(rg_engine* E, int slot, size_t bytes);
CUtensorMap increments_map(const float* incr, uint64_t npaths, uint64_t rowlen, int U, int64_t TU, int Pb, int TT);
// One map per underlying count n, with boxes of book_stage_steps(n, sh.TT) steps: maps[n - 1].
void increments_maps(const float* incr, uint64_t npaths, uint64_t rowlen, int U, int64_t TU, const Book32Shape& sh,
                     CUtensorMap* maps);
uint64_t chunk_paths(uint64_t paths, int U, int64_t TU, size_t elem, uint64_t unit);

}  // namespace bk
}  // namespace rg
