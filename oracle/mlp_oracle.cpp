/*
 * mlp_oracle.cpp -- CPU restatement of the reference's MLP local-search path.
 *
 * TEST INFRASTRUCTURE (the checker).  Only tests/, __graft_entry__.smoke() and
 * the CPU-baseline leg of bench.py load this library; the GPU engine never
 * does.  Every function cites the reference file:line it restates.
 *
 * Parity status: pinned.  The known answers of the reference's own tests
 * (K1 MT19937 outputs, K2 berlin52 size 53, K3 cost 494309, K4 cost 367403
 * after one swap pass) are reproduced by tests/test_oracle.py, and ADS buffers
 * and start tours are checked against fixtures produced by the reference's
 * compiled CPU evaluator (oracle/_ref, tests/golden/gen_golden.py).
 *
 * Decisions where the reference is not deterministic:
 *   - Per-block winner: argmin over (delta, ctx); the reference's shared-memory
 *     tree depends on blockDim (source/mlkswap.cu:944-964).
 *   - Sort of candidates: stable on (cost, block index); the reference uses
 *     thrust::sort whose tie order is unspecified (source/mlkernel.cu:256).
 *   - Distances d(a,b) always come from the int32 matrix D (the reference's
 *     ODC kernels recompute them from coordinates with +0 rounding,
 *     source/mlkernel.h:41-49; identical for distRound = false).
 */
#include "mlp_oracle.h"

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <sstream>
#include <string>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

const int32_t kCostInfty32 = 0x7fffffff;          // COST_INFTY, source/mlads.h:24
const int64_t kCostInfty64 = 0x7fffffffffffffffLL;

inline int64_t wrap(int64_t v, int wide) {
  return wide ? v : (int64_t)(int32_t)(uint32_t)(uint64_t)v;
}

/* ------------------------------------------------------------------------ */
/* MT19937 as in source/mtrand.cpp:52-124 and source/mtrand.h:167-195.      */
/* ------------------------------------------------------------------------ */
struct MT {
  uint32_t st[624];
  int p;
  void seed(uint32_t s) {                       // mtrand.cpp:52-61
    st[0] = s;
    for (p = 1; p < 624; ++p) st[p] = 1812433253U * (st[p - 1] ^ (st[p - 1] >> 30)) + (uint32_t)p;
  }
  void gen() {                                  // mtrand.cpp:99-124
    static const uint32_t mag[2] = {0u, 0x9908b0dfU};
    int i;
    uint32_t y;
    for (i = 0; i < 624 - 397; i++) {
      y = (st[i] & 0x80000000U) | (st[i + 1] & 0x7fffffffU);
      st[i] = st[i + 397] ^ (y >> 1) ^ mag[y & 1u];
    }
    for (; i < 623; i++) {
      y = (st[i] & 0x80000000U) | (st[i + 1] & 0x7fffffffU);
      st[i] = st[i + (397 - 624)] ^ (y >> 1) ^ mag[y & 1u];
    }
    y = (st[623] & 0x80000000U) | (st[0] & 0x7fffffffU);
    st[623] = st[396] ^ (y >> 1) ^ mag[y & 1u];
    p = 0;
  }
  uint32_t rand() {                             // mtrand.h:167-179
    if (p >= 624) gen();
    uint32_t x = st[p++];
    x ^= (x >> 11);
    x ^= (x << 7) & 0x9d2c5680U;
    x ^= (x << 15) & 0xefc60000U;
    return x ^ (x >> 18);
  }
  uint32_t rand_max(uint32_t max) {             // mtrand.h:193-195
    return (uint32_t)(((max + 1.0) * rand()) / (4294967295U + 1.0));
  }
};

/* ------------------------------------------------------------------------ */
/* Tour helpers                                                             */
/* ------------------------------------------------------------------------ */
struct Tour {
  int size;
  const int32_t* t;
  int n;
  const int32_t* D;
  inline int64_t d(int a, int b) const { return D[(size_t)t[a] * n + t[b]]; }
};

// update(): w[0] = 0, w[p] = dist(p-1, p)  (source/mlsolution.cpp:216-228)
void weights_of(const Tour& T, std::vector<int64_t>& w) {
  w.assign(T.size + 1, 0);
  for (int p = 1; p < T.size; p++) w[p] = T.d(p - 1, p);
}

inline int move_id_of(int nb) { return nb; }             // SWAP 0, 2OPT 1, OROPTk k+1
inline int oropt_k_of(int id) { return id - 1; }         // MLMI_OROPT_K, mlads.h:27

/* ---------------- faithful reference deltas (ODC kernels) ---------------- */

// mlkswap.cu:770-785
int64_t delta_swap(const Tour& T, const std::vector<int64_t>& w, int i, int j) {
  const int64_t size = T.size;
  int64_t c = (size - i) * (T.d(i - 1, j) - w[i]);
  c += (size - i - 1) * (T.d(j, i + 1) - w[i + 1]);
  c += (size - j) * (T.d(j - 1, i) - w[j]);
  if (j + 1 < size) c += (size - j - 1) * (T.d(i, j + 1) - w[j + 1]);
  return c;
}

// mlk2opt.cu:565-571
int64_t delta_2opt(const Tour& T, const std::vector<int64_t>& w, int i, int j) {
  const int64_t size = T.size;
  int64_t c = (size - i) * (T.d(i - 1, j) - w[i]);
  if (j + 1 < size) c += (size - j - 1) * (T.d(i, j + 1) - w[j + 1]);
  for (int k = 1; k <= j - i; k++) c += (size - i - k) * (w[j - k + 1] - w[i + k]);
  return c;
}

// mlkoropt.cu:704-716 (i < j) and :724-736 (i > j)
int64_t delta_oropt(const Tour& T, const std::vector<int64_t>& w, int k, int i, int j) {
  const int64_t size = T.size;
  int64_t c, s;
  if (i < j) {
    c = (size - i) * (T.d(i - 1, i + k) - w[i]);
    c += (size - j - k) * (T.d(i + k - 1, j + k) - w[j + k]);
    c += (size - j) * T.d(j + k - 1, i) - (size - i - k) * w[i + k];
    s = 0;
    for (int l = i + 1; l < i + k; l++) s += w[l];
    c += (int64_t)(i - j) * s;
    s = 0;
    for (int l = i + k + 1; l < j + k; l++) s += w[l];
    c += (int64_t)k * s;
  } else {
    c = (size - j) * (T.d(j - 1, i) - w[j]);
    c += (size - i - k) * (T.d(i - 1, i + k) - w[i + k]);
    c += (size - j - k) * T.d(i + k - 1, j) - (size - i) * w[i];
    s = 0;
    for (int l = i + 1; l < i + k; l++) s += w[l];
    c += (int64_t)(i - j) * s;
    s = 0;
    for (int l = j + 1; l < i; l++) s += w[l];
    c -= (int64_t)k * s;
  }
  return c;
}

/* ---------------- fast (prefix-sum) deltas, same values ---------------- */
struct Prefix {
  std::vector<int64_t> W;  // W[p] = sum_{q<=p} w[q]
  std::vector<int64_t> Q;  // Q[p] = sum_{q<=p} q*w[q]
  void build(const std::vector<int64_t>& w, int size) {
    W.assign(size + 1, 0);
    Q.assign(size + 1, 0);
    for (int p = 1; p < size; p++) {
      W[p] = W[p - 1] + w[p];
      Q[p] = Q[p - 1] + (int64_t)p * w[p];
    }
  }
  inline int64_t R(int a, int b) const { return a > b ? 0 : W[b] - W[a - 1]; }
};

int64_t fast_2opt(const Tour& T, const std::vector<int64_t>& w, const Prefix& P, int i, int j) {
  const int64_t size = T.size;
  int64_t c = (size - i) * (T.d(i - 1, j) - w[i]);
  if (j + 1 < size) c += (size - j - 1) * (T.d(i, j + 1) - w[j + 1]);
  // sum_{p=i+1}^{j} (2p - i - j - 1) w[p]
  c += 2 * (P.Q[j] - P.Q[i]) - (int64_t)(i + j + 1) * (P.W[j] - P.W[i]);
  return c;
}

int64_t fast_oropt(const Tour& T, const std::vector<int64_t>& w, const Prefix& P, int k, int i, int j) {
  const int64_t size = T.size;
  int64_t c;
  if (i < j) {
    c = (size - i) * (T.d(i - 1, i + k) - w[i]);
    c += (size - j - k) * (T.d(i + k - 1, j + k) - w[j + k]);
    c += (size - j) * T.d(j + k - 1, i) - (size - i - k) * w[i + k];
    c += (int64_t)(i - j) * P.R(i + 1, i + k - 1) + (int64_t)k * P.R(i + k + 1, j + k - 1);
  } else {
    c = (size - j) * (T.d(j - 1, i) - w[j]);
    c += (size - i - k) * (T.d(i - 1, i + k) - w[i + k]);
    c += (size - j - k) * T.d(i + k - 1, j) - (size - i) * w[i];
    c += (int64_t)(i - j) * P.R(i + 1, i + k - 1) - (int64_t)k * P.R(j + 1, i - 1);
  }
  return c;
}

/* ---------------- block -> move mappings of the ODC kernels ---------------- */
const int kTour = 1;  // every reference entry point uses costTour = true

int num_blocks(int nb, int size) {
  if (nb == 0) return ((size + 1) / 2) - 1;                 // mlkswap.cu:1001
  if (nb == 1) return (size + 1) / 2;                       // mlk2opt.cu:680 (GPU_DIVCEIL)
  int k = nb - 1;
  return size + !kTour - k - 2;                             // mlkoropt.cu:842
}

int num_threads(int nb, int size) {
  if (nb == 0) return size - kTour - 3;                     // mlkswap.cu:763
  if (nb == 1) return size - kTour - 2;                     // mlk2opt.cu:559
  int k = nb - 1;
  return size - kTour - k - 1;                              // mlkoropt.cu:699
}

// (block by, thread ctx) -> (i, j)
inline void map_move(int nb, int size, int by, int ctx, int& i, int& j) {
  bool kk = ctx >= by;
  if (nb == 0) {                                            // mlkswap.cu:766-768
    i = kk ? by + 1 : size - kTour - by - 2;
    j = kk ? ctx + 3 : size - kTour - ctx - 1;
  } else if (nb == 1) {                                     // mlk2opt.cu:561-563
    i = kk ? ctx - by + 1 : by - ctx;
    j = kk ? ctx + 2 : size - ctx - kTour - 1;
  } else {                                                  // mlkoropt.cu:701-722
    int k = nb - 1;
    if (kk) {
      i = ctx - by + 1;
      j = ctx + 2;
    } else {
      i = size - ctx - k - kTour;
      j = by - ctx;
    }
  }
}

void eval_block_range(int nb, const Tour& T, const std::vector<int64_t>& w, const Prefix* P,
                      int wide, int faithful, int b0, int b1, int64_t* cost, int32_t* mi,
                      int32_t* mj, int32_t* mctx) {
  const int nthr = num_threads(nb, T.size);
  const int64_t sentinel = wide ? kCostInfty64 : kCostInfty32;
  for (int by = b0; by < b1; by++) {
    int64_t best = sentinel;
    int bi = 0, bj = 0, bc = 0;
    for (int ctx = 0; ctx < nthr; ctx++) {
      int i, j;
      map_move(nb, T.size, by, ctx, i, j);
      int64_t c;
      if (nb == 0)
        c = delta_swap(T, w, i, j);
      else if (nb == 1)
        c = faithful ? delta_2opt(T, w, i, j) : fast_2opt(T, w, *P, i, j);
      else
        c = faithful ? delta_oropt(T, w, nb - 1, i, j) : fast_oropt(T, w, *P, nb - 1, i, j);
      c = wrap(c, wide);
      if (c < best) {  // strict: first (smallest ctx) minimum wins
        best = c;
        bi = i;
        bj = j;
        bc = ctx;
      }
    }
    cost[by] = best;
    mi[by] = bi;
    mj[by] = bj;
    if (mctx) mctx[by] = bc;
  }
}

/* ---------------- merge predicates ---------------- */
inline int iabs(int v) { return v < 0 ? -v : v; }

// f_canSwapMerge, mlkernel.cu:51-54
bool can_swap_same(int i1, int j1, int i2, int j2) {
  return iabs(i1 - i2) > 1 && iabs(i1 - j2) > 1 && iabs(j1 - i2) > 1 && iabs(j1 - j2) > 1;
}
// f_can2OptMerge, mlkernel.cu:56-59
bool can_2opt_same(int i1, int j1, int i2, int j2) {
  return (j1 < i2 - 1) || (i1 > j2 + 1) || (j2 < i1 - 1) || (i2 > j1 + 1);
}
// f_canOrOptMerge, mlkernel.cu:61-71
bool can_oropt_same(int id1, int i1, int j1, int id2, int i2, int j2) {
  int min1 = std::min(i1, j1), max1 = std::max(i1, j1), k1 = oropt_k_of(id1);
  int min2 = std::min(i2, j2), max2 = std::max(i2, j2), k2 = oropt_k_of(id2);
  return (max1 + k1 < min2) || (min1 > max2 + k2);
}

bool can_same(int nb, int id1, int i1, int j1, int id2, int i2, int j2) {
  if (nb == 0) return can_swap_same(i1, j1, i2, j2);
  if (nb == 1) return can_2opt_same(i1, j1, i2, j2);
  return can_oropt_same(id1, i1, j1, id2, i2, j2);
}

// canSwapMerge / can2OptMerge / canOrOptMerge / canMerge, mlkernel.cu:649-729
bool can_merge_swap(int i1, int j1, int id2, int i2, int j2) {
  switch (id2) {
    case 0:
      return can_swap_same(i1, j1, i2, j2);
    case 1:
      return ((i1 < i2 - 1) || (i1 > j2 + 1)) && ((j1 < i2 - 1) || (j1 > j2 + 1));
    default: {
      int min2 = std::min(i2, j2), max2 = std::max(i2, j2), k2 = oropt_k_of(id2);
      return (j1 < min2 - 1) || (i1 > max2 + k2) || ((i1 < min2 - 1) && (j1 > max2 + k2));
    }
  }
}
bool can_merge_2opt(int i1, int j1, int id2, int i2, int j2) {
  switch (id2) {
    case 0:
      return can_merge_swap(i2, j2, 1, i1, j1);
    case 1:
      return can_2opt_same(i1, j1, i2, j2);
    default: {
      int min2 = std::min(i2, j2), max2 = std::max(i2, j2), k2 = oropt_k_of(id2);
      return (i1 > max2 + k2) || (j1 < min2 - 1);
    }
  }
}
bool can_merge_oropt(int id1, int i1, int j1, int id2, int i2, int j2) {
  switch (id2) {
    case 0:
      return can_merge_swap(i2, j2, id1, i1, j1);
    case 1:
      return can_merge_2opt(i2, j2, id1, i1, j1);
    default:
      return can_oropt_same(id1, i1, j1, id2, i2, j2);
  }
}
bool can_merge(int id1, int i1, int j1, int id2, int i2, int j2) {
  switch (id1) {
    case 0:
      return can_merge_swap(i1, j1, id2, i2, j2);
    case 1:
      return can_merge_2opt(i1, j1, id2, i2, j2);
    default:
      return can_merge_oropt(id1, i1, j1, id2, i2, j2);
  }
}

/* ---------------- apply (applyMove of each kernel) ---------------- */
// swap: mlkswap.cu:1070-1078; 2-opt: mlk2opt.cu:737-745; Or-opt: mlkoropt.cu:896-925
void apply_move(int id, int i, int j, int size, int32_t* t) {
  if (id == 0) {
    std::swap(t[i], t[j]);
  } else if (id == 1) {
    while (i < j) {
      std::swap(t[i], t[j]);
      i++;
      j--;
    }
  } else {
    int k = oropt_k_of(id);
    std::vector<int32_t> tmp(t + i, t + i + k);
    if (i < j) {
      int dst = i;
      for (int l = i + k; l < j + k; l++) t[dst++] = t[l];
      for (int l = 0; l < k; l++) t[dst++] = tmp[l];
    } else if (i > j) {
      for (int l = i - 1; l >= j; l--) t[l + k] = t[l];
      for (int l = 0; l < k; l++) t[l + j] = tmp[l];
    }
  }
  (void)size;
}

int64_t cost_of(int size, const int32_t* tour, int n, const int32_t* D, int wide,
                int32_t* w_out) {
  // update(): cost = sum_{i=1}^{size-1} (size - i) * w[i]   (mlsolution.cpp:216-228)
  uint32_t c32 = 0;
  int64_t c64 = 0;
  if (w_out) w_out[0] = 0;
  for (int p = 1; p < size; p++) {
    int32_t wp = D[(size_t)tour[p - 1] * n + tour[p]];
    if (w_out) w_out[p] = wp;
    c32 += (uint32_t)(size - p) * (uint32_t)wp;
    c64 += (int64_t)(size - p) * wp;
  }
  return wide ? c64 : (int64_t)c32;
}

struct Cand {
  int64_t cost;
  int32_t nb, by, id, i, j;
};

/* Stage 2 (per-neighbourhood greedy), mlkernel.cu:73-170 + the sort at :256 */
void merge_same(int nb, int m, const int64_t* cost, const int32_t* mi, const int32_t* mj,
                std::vector<int32_t>& kept) {
  std::vector<int32_t> order;
  for (int b = 0; b < m; b++)
    if (cost[b] < 0) order.push_back(b);
  std::stable_sort(order.begin(), order.end(),
                   [&](int32_t a, int32_t b) { return cost[a] < cost[b]; });
  kept.clear();
  const int id = move_id_of(nb);
  for (int32_t x : order) {
    bool ok = true;
    for (int32_t y : kept)
      if (!can_same(nb, id, mi[y], mj[y], id, mi[x], mj[x])) {
        ok = false;
        break;
      }
    if (ok) kept.push_back(x);
  }
}

/* Stage 3 (cross-neighbourhood greedy), mlkernel.cu:732-864 with a stable sort */
void merge_cross(std::vector<Cand>& list, std::vector<Cand>& sel) {
  std::stable_sort(list.begin(), list.end(),
                   [](const Cand& a, const Cand& b) { return a.cost < b.cost; });
  sel.clear();
  for (const Cand& x : list) {
    if (x.cost >= 0) break;
    bool ok = true;
    for (const Cand& y : sel)
      if (!can_merge(y.id, y.i, y.j, x.id, x.i, x.j)) {
        ok = false;
        break;
      }
    if (ok) sel.push_back(x);
  }
}

void eval_nb(int nb, const Tour& T, const std::vector<int64_t>& w, const Prefix& P, int wide,
             int faithful, int threads, int64_t* cost, int32_t* mi, int32_t* mj, int32_t* mctx) {
  const int nbk = num_blocks(nb, T.size);
#ifdef _OPENMP
  if (threads != 1) {
    int nt = threads > 0 ? threads : omp_get_max_threads();
#pragma omp parallel for schedule(dynamic, 4) num_threads(nt)
    for (int by = 0; by < nbk; by++)
      eval_block_range(nb, T, w, &P, wide, faithful, by, by + 1, cost, mi, mj, mctx);
    return;
  }
#endif
  (void)threads;
  eval_block_range(nb, T, w, &P, wide, faithful, 0, nbk, cost, mi, mj, mctx);
}

}  // namespace

/* ======================================================================== */
extern "C" {

void orc_mt_rand(uint32_t seed, int count, uint32_t* out) {
  MT r;
  r.seed(seed);
  for (int i = 0; i < count; i++) out[i] = r.rand();
}

void orc_mt_rand_max(uint32_t seed, uint32_t max, int count, uint32_t* out) {
  MT r;
  r.seed(seed);
  for (int i = 0; i < count; i++) out[i] = r.rand_max(max);
}

// TSPLibInstance::load + loadNodeCoord + inear (tsplib.cpp:237-240, :455-475);
// only EUC_2D NODE_COORD_SECTION files, as MLProblem::load requires (mlproblem.cpp:94-95).
int orc_tsplib_read(const char* path, int maxn, int32_t* x, int32_t* y) {
  std::ifstream f(path);
  if (!f.is_open()) return -1;
  std::string line;
  int dim = -1;
  bool euc = false;
  while (std::getline(f, line)) {
    std::string key = line, val;
    size_t c = line.find(':');
    if (c != std::string::npos) {
      key = line.substr(0, c);
      val = line.substr(c + 1);
    }
    auto trim = [](std::string s) {
      size_t a = s.find_first_not_of(" \t\r\n"), b = s.find_last_not_of(" \t\r\n");
      return a == std::string::npos ? std::string() : s.substr(a, b - a + 1);
    };
    key = trim(key);
    val = trim(val);
    if (key == "DIMENSION") dim = std::atoi(val.c_str());
    else if (key == "EDGE_WEIGHT_TYPE") euc = (val == "EUC_2D");
    else if (key == "NODE_COORD_SECTION") break;
  }
  if (!euc) return -2;
  if (dim < 0) return -1;
  if (dim > maxn) return -3;
  for (int i = 0; i < dim; i++) {
    int id;
    float fx, fy;
    if (!(f >> id >> fx >> fy)) return -1;
    x[i] = fx >= 0 ? (int)(fx + 0.5F) : (int)(fx - 0.5F);
    y[i] = fy >= 0 ? (int)(fy + 0.5F) : (int)(fy - 0.5F);
  }
  return dim;
}

// mlproblem.cpp:153-166
void orc_dist_from_coords(int n, const int32_t* x, const int32_t* y, int distRound, int32_t* D) {
  const float dr = distRound ? 0.5F : 0.0F;
  for (int i = 0; i < n; i++)
    for (int j = 0; j < n; j++) {
      float s = (float)((x[i] - x[j]) * (x[i] - x[j]) + (y[i] - y[j]) * (y[i] - y[j]));
      D[(size_t)i * n + j] = (int)(sqrtf(s) + dr);
    }
}

// MLSolution::random, mlsolution.cpp:754-874
void orc_random_tour(int n, const int32_t* D, int costTour, uint32_t seed, float alpha,
                     int32_t* tour) {
  MT rng;
  rng.seed(seed);
  const int size = n + (costTour ? 1 : 0);
  std::vector<int32_t> cands;
  for (int c = 1; c < size - (costTour ? 1 : 0); c++) cands.push_back(c % n);
  int len = 0;
  int last = 0;
  tour[len++] = 0;
  uint32_t count = (uint32_t)cands.size();
  while (count > 0) {
    uint32_t rcl, idx;
    if (count > 1) {
      rcl = (uint32_t)std::ceil(alpha * (float)count);
      idx = rcl > 0 ? rng.rand_max(rcl - 1) : 0;
      const int32_t* row = D + (size_t)last * n;
      if (alpha < 0.5f) {
        std::sort(cands.begin(), cands.begin() + count,
                  [row](int32_t a, int32_t b) { return row[a] > row[b]; });
        idx = count - idx - 1;
      } else {
        std::sort(cands.begin(), cands.begin() + count,
                  [row](int32_t a, int32_t b) { return row[a] < row[b]; });
      }
    } else {
      idx = 0;
    }
    int32_t cur = cands[idx];
    tour[len++] = cur;
    last = cur;
    for (uint32_t i = idx; i + 1 < count; i++) cands[i] = cands[i + 1];
    count--;
  }
  if (costTour) tour[len++] = 0;
}

// MLSolution::random (mlsolution.cpp:754-874) with a canonical order of
// equal distances.  Both of the reference's branches pick the candidate of
// ascending rank r = rng.rand(ceil(alpha * count) - 1) by distance to the
// last client added (alpha < 0.5 sorts descending and takes position
// count - r - 1); std::sort leaves the order of equal distances to the
// library, so here the rank is taken in (distance, client id) order.
void orc_random_tour_canonical(int n, const int32_t* D, uint32_t seed, float alpha, int32_t* tour) {
  MT rng;
  rng.seed(seed);
  std::vector<int32_t> cands;
  for (int c = 1; c < n; c++) cands.push_back(c);
  int len = 0, last = 0;
  tour[len++] = 0;
  while (!cands.empty()) {
    const uint32_t count = (uint32_t)cands.size();
    uint32_t r = 0;
    if (count > 1) {
      const uint32_t rcl = (uint32_t)std::ceil(alpha * (float)count);
      r = rcl > 0 ? rng.rand_max(rcl - 1) : 0;
    }
    const int32_t* row = D + (size_t)last * n;
    std::nth_element(cands.begin(), cands.begin() + r, cands.end(), [row](int32_t a, int32_t b) {
      return row[a] != row[b] ? row[a] < row[b] : a < b;
    });
    const int32_t cur = cands[r];
    cands.erase(cands.begin() + r);
    tour[len++] = cur;
    last = cur;
  }
  tour[len++] = 0;
}

int64_t orc_cost(int size, const int32_t* tour, int n, const int32_t* D, int wide,
                 int32_t* w_out) {
  return cost_of(size, tour, n, D, wide, w_out);
}

// MLSolution::ldsUpdate, mlsolution.cpp:420-486 (layout mlads.h:38-74)
void orc_ads_build(int size, const int32_t* tour, int n, const int32_t* D, const int32_t* x,
                   const int32_t* y, int costTour, int distRound, uint32_t* ads) {
  const uint32_t rowElems = (uint32_t)size;
  std::vector<int32_t> w(size);
  uint32_t cost = (uint32_t)cost_of(size, tour, n, D, 0, w.data());
  std::memset(ads, 0, 128);
  ads[0] = 128u + rowElems * (uint32_t)(size + 3) * 4u;
  ads[1] = rowElems;
  ads[2] = (uint32_t)size;
  ads[3] = cost;
  ads[4] = (uint32_t)(costTour != 0);
  ads[5] = (uint32_t)(distRound != 0);
  uint32_t* coords = ads + 32;
  uint32_t* sol = coords + rowElems;
  uint32_t* T = coords + 2 * rowElems;
  uint32_t* C = coords + 3 * rowElems;
  auto pack = [](int32_t h, int32_t l) {
    return ((uint32_t)(uint16_t)h << 16) | (uint32_t)(uint16_t)l;
  };
  coords[0] = pack(x[tour[0]], y[tour[0]]);
  sol[0] = (uint32_t)(uint16_t)tour[0];
  T[0] = 0;
  for (int j = 1; j < size; j++) {
    coords[j] = pack(x[tour[j]], y[tour[j]]);
    sol[j] = pack(tour[j], w[j]);
    T[j] = T[j - 1] + (uint32_t)(uint16_t)w[j];
  }
  for (int i = 0; i < size; i++) {
    uint32_t* row = C + (size_t)rowElems * i;
    row[i] = 0;
    for (int j = i + 1; j < size; j++) row[j] = row[j - 1] + (T[j] - T[i]);
  }
  for (int i = size - 1; i >= 0; i--) {
    uint32_t* row = C + (size_t)rowElems * i;
    for (int j = i - 1; j >= 0; j--) row[j] = row[j + 1] + (T[i] - T[j]);
  }
}

int orc_num_blocks(int nb, int size) { return num_blocks(nb, size); }
int orc_num_threads(int nb, int size) { return num_threads(nb, size); }

void orc_eval(int nb, int size, const int32_t* tour, int n, const int32_t* D, int wide,
              int faithful, int64_t* cost, int32_t* mi, int32_t* mj, int32_t* mctx) {
  Tour T{size, tour, n, D};
  std::vector<int64_t> w;
  weights_of(T, w);
  Prefix P;
  P.build(w, size);
  eval_nb(nb, T, w, P, wide, faithful, 1, cost, mi, mj, mctx);
}

int64_t orc_move_delta(int id, int i, int j, int size, const int32_t* tour, int n,
                       const int32_t* D, int wide) {
  Tour T{size, tour, n, D};
  std::vector<int64_t> w;
  weights_of(T, w);
  int64_t c;
  if (id == 0) c = delta_swap(T, w, i, j);
  else if (id == 1) c = delta_2opt(T, w, i, j);
  else c = delta_oropt(T, w, oropt_k_of(id), i, j);
  return wrap(c, wide);
}

int64_t orc_move_delta_bruteforce(int id, int i, int j, int size, const int32_t* tour, int n,
                                  const int32_t* D, int wide) {
  std::vector<int32_t> t2(tour, tour + size);
  apply_move(id, i, j, size, t2.data());
  int64_t a = cost_of(size, tour, n, D, 1, nullptr);
  int64_t b = cost_of(size, t2.data(), n, D, 1, nullptr);
  return wrap(b - a, wide);
}

int orc_can_merge_same(int nb, int id1, int i1, int j1, int id2, int i2, int j2) {
  return can_same(nb, id1, i1, j1, id2, i2, j2) ? 1 : 0;
}

int orc_can_merge(int id1, int i1, int j1, int id2, int i2, int j2) {
  return can_merge(id1, i1, j1, id2, i2, j2) ? 1 : 0;
}

int orc_merge_same(int nb, int m, const int64_t* cost, const int32_t* mi, const int32_t* mj,
                   int32_t* kept) {
  std::vector<int32_t> k;
  merge_same(nb, m, cost, mi, mj, k);
  for (size_t q = 0; q < k.size(); q++) kept[q] = k[q];
  return (int)k.size();
}

int orc_merge_cross(int m, const int32_t* id, const int32_t* mi, const int32_t* mj,
                    const int64_t* cost, int32_t* kept) {
  std::vector<Cand> list(m);
  for (int q = 0; q < m; q++) list[q] = Cand{cost[q], 0, q, id[q], mi[q], mj[q]};
  std::vector<Cand> sel;
  merge_cross(list, sel);
  for (size_t q = 0; q < sel.size(); q++) kept[q] = sel[q].by;
  return (int)sel.size();
}

void orc_apply(int id, int i, int j, int size, int32_t* tour) { apply_move(id, i, j, size, tour); }

// WAMCAExperiment::runKernel / runGpuGpu, WamcaExperiment.hpp:229-365
int orc_pass(int nb, int size, int32_t* tour, int n, const int32_t* D, int wide, int max_moves,
             int32_t* ids, int32_t* is, int32_t* js, int64_t* costs, int64_t* new_cost) {
  Tour T{size, tour, n, D};
  std::vector<int64_t> w;
  weights_of(T, w);
  Prefix P;
  P.build(w, size);
  const int m = num_blocks(nb, size);
  std::vector<int64_t> c(m);
  std::vector<int32_t> mi(m), mj(m);
  eval_nb(nb, T, w, P, wide, 0, 1, c.data(), mi.data(), mj.data(), nullptr);
  std::vector<int32_t> kept;
  merge_same(nb, m, c.data(), mi.data(), mj.data(), kept);
  int cnt = 0;
  for (int32_t b : kept) {
    apply_move(move_id_of(nb), mi[b], mj[b], size, tour);
    if (cnt < max_moves) {
      ids[cnt] = move_id_of(nb);
      is[cnt] = mi[b];
      js[cnt] = mj[b];
      costs[cnt] = c[b];
    }
    cnt++;
  }
  if (new_cost) *new_cost = cost_of(size, tour, n, D, wide, nullptr);
  return cnt;
}

int64_t orc_sweep(int size, const int32_t* tour, int n, const int32_t* D, int wide, int nb_count,
                  const int32_t* nbs, int threads, int64_t* cost_out, int32_t* i_out,
                  int32_t* j_out) {
  Tour T{size, tour, n, D};
  std::vector<int64_t> w;
  weights_of(T, w);
  Prefix P;
  P.build(w, size);
  int64_t evals = 0;
  size_t off = 0;
  for (int q = 0; q < nb_count; q++) {
    int nb = nbs[q];
    int m = num_blocks(nb, size);
    std::vector<int64_t> c(m);
    std::vector<int32_t> mi(m), mj(m);
    eval_nb(nb, T, w, P, wide, 0, threads, c.data(), mi.data(), mj.data(), nullptr);
    if (cost_out) std::copy(c.begin(), c.end(), cost_out + off);
    if (i_out) std::copy(mi.begin(), mi.end(), i_out + off);
    if (j_out) std::copy(mj.begin(), mj.end(), j_out + off);
    off += m;
    evals += (int64_t)m * num_threads(nb, size);
  }
  return evals;
}

int orc_dvnd(int size, int32_t* tour, int n, const int32_t* D, int wide, int nb_count,
             const int32_t* nbs, int max_iters, int threads, int64_t* final_cost,
             int64_t* evals, int64_t* moves_applied) {
  int it = 0;
  int64_t ev = 0, mv = 0;
  std::vector<int64_t> w;
  Prefix P;
  for (; it < max_iters; it++) {
    Tour T{size, tour, n, D};
    weights_of(T, w);
    P.build(w, size);
    std::vector<Cand> list;
    for (int q = 0; q < nb_count; q++) {
      int nb = nbs[q];
      int m = num_blocks(nb, size);
      std::vector<int64_t> c(m);
      std::vector<int32_t> mi(m), mj(m);
      eval_nb(nb, T, w, P, wide, 0, threads, c.data(), mi.data(), mj.data(), nullptr);
      ev += (int64_t)m * num_threads(nb, size);
      std::vector<int32_t> kept;
      merge_same(nb, m, c.data(), mi.data(), mj.data(), kept);
      for (int32_t b : kept) list.push_back(Cand{c[b], nb, b, move_id_of(nb), mi[b], mj[b]});
    }
    if (list.empty()) break;
    std::vector<Cand> sel;
    merge_cross(list, sel);
    for (const Cand& x : sel) apply_move(x.id, x.i, x.j, size, tour);
    mv += (int64_t)sel.size();
  }
  if (final_cost) *final_cost = cost_of(size, tour, n, D, wide, nullptr);
  if (evals) *evals = ev;
  if (moves_applied) *moves_applied = mv;
  return it;
}

}  // extern "C"

/* ------------------------------------------------------------------------ */
/* TOTAL multi-improvement                                                  */
/* ------------------------------------------------------------------------ */
namespace {

// The TOTAL kernels (kernelSwapTotal mlkswap.cu:334-526, kernel2OptTotal
// mlk2opt.cu:270-447, kernelOrOptTotal mlkoropt.cu:368-612) write one
// candidate per thread instead of one per block (moveElems = grid.y *
// block.x, mlkswap.cu:1022, mlkoropt.cu:851).  mergeGPU sorts them
// (mlkernel.cu:256) and testSwapTotal / test2OptTotal / testOrOptTotal
// (mlkernel.cu:183-250) zero every later move that conflicts with an earlier
// negative one: the greedy independent set in sorted order, which the host
// then applies in that order (WamcaExperiment.hpp:422-542).
// Decisions: a thread evaluates one move (blockDim >= size), so every
// distinct move (i, j) of the neighbourhood -- the moves of the ODC kernels'
// mapping, each once -- is a candidate; ties are sorted by (i, j).
struct TMove {
  int64_t cost;
  int32_t i, j;
};

void total_candidates(int nb, const Tour& T, const std::vector<int64_t>& w, const Prefix& P, int wide,
                      std::vector<TMove>& out, int64_t* evals) {
  const int size = T.size, m = num_blocks(nb, size), nthr = num_threads(nb, size);
  std::vector<uint8_t> seen((size_t)size * size, 0);
  out.clear();
  int64_t ev = 0;
  for (int by = 0; by < m; by++)
    for (int ctx = 0; ctx < nthr; ctx++) {
      int i, j;
      map_move(nb, size, by, ctx, i, j);
      ev++;  // evaluations counted as the kernels' threads (duplicates included)
      uint8_t& s = seen[(size_t)i * size + j];
      if (s) continue;
      s = 1;
      int64_t c;
      if (nb == 0)
        c = delta_swap(T, w, i, j);
      else if (nb == 1)
        c = fast_2opt(T, w, P, i, j);
      else
        c = fast_oropt(T, w, P, nb - 1, i, j);
      c = wrap(c, wide);
      if (c < 0) out.push_back(TMove{c, i, j});
    }
  std::sort(out.begin(), out.end(), [](const TMove& a, const TMove& b) {
    if (a.cost != b.cost) return a.cost < b.cost;
    if (a.i != b.i) return a.i < b.i;
    return a.j < b.j;
  });
  if (evals) *evals += ev;
}

// testSwapTotal / test2OptTotal / testOrOptTotal, mlkernel.cu:183-250
void total_select(int nb, const std::vector<TMove>& cands, std::vector<TMove>& kept) {
  kept.clear();
  const int id = move_id_of(nb);
  for (const TMove& x : cands) {
    bool ok = true;
    for (const TMove& y : kept)
      if (!can_same(nb, id, y.i, y.j, id, x.i, x.j)) {
        ok = false;
        break;
      }
    if (ok) kept.push_back(x);
  }
}

}  // namespace

extern "C" {

int orc_total_select(int nb, int size, const int32_t* tour, int n, const int32_t* D, int wide, int cap,
                     int64_t* cost, int32_t* is, int32_t* js, int64_t* candidates) {
  Tour T{size, tour, n, D};
  std::vector<int64_t> w;
  weights_of(T, w);
  Prefix P;
  P.build(w, size);
  std::vector<TMove> cands, kept;
  total_candidates(nb, T, w, P, wide, cands, nullptr);
  total_select(nb, cands, kept);
  for (size_t q = 0; q < kept.size() && (int)q < cap; q++) {
    cost[q] = kept[q].cost;
    is[q] = kept[q].i;
    js[q] = kept[q].j;
  }
  if (candidates) *candidates = (int64_t)cands.size();
  return (int)kept.size();
}

int orc_total_pass(int nb, int size, int32_t* tour, int n, const int32_t* D, int wide, int max_moves,
                   int32_t* ids, int32_t* is, int32_t* js, int64_t* costs, int64_t* new_cost) {
  std::vector<int64_t> c(size * 2 + 8);
  std::vector<int32_t> ki(c.size()), kj(c.size());
  const int k = orc_total_select(nb, size, tour, n, D, wide, (int)c.size(), c.data(), ki.data(), kj.data(),
                                 nullptr);
  for (int q = 0; q < k; q++) {
    apply_move(move_id_of(nb), ki[q], kj[q], size, tour);
    if (q < max_moves) {
      ids[q] = move_id_of(nb);
      is[q] = ki[q];
      js[q] = kj[q];
      costs[q] = c[q];
    }
  }
  if (new_cost) *new_cost = cost_of(size, tour, n, D, wide, nullptr);
  return k;
}

// DVND with TOTAL candidate sets: per iteration the TOTAL greedy of every
// neighbourhood of `nbs` (ascending) on the same tour, then the cross-
// neighbourhood greedy with canMerge (mlkernel.cu:649-864, stable on the
// neighbourhood order and each neighbourhood's greedy order) and the apply.
int orc_dvnd_total(int size, int32_t* tour, int n, const int32_t* D, int wide, int nb_count,
                   const int32_t* nbs, int max_iters, int64_t* final_cost, int64_t* evals,
                   int64_t* moves_applied) {
  int it = 0;
  int64_t ev = 0, mv = 0;
  std::vector<int64_t> w;
  Prefix P;
  std::vector<TMove> cands, kept;
  for (; it < max_iters; it++) {
    Tour T{size, tour, n, D};
    weights_of(T, w);
    P.build(w, size);
    std::vector<Cand> list;
    for (int q = 0; q < nb_count; q++) {
      const int nb = nbs[q];
      total_candidates(nb, T, w, P, wide, cands, &ev);
      total_select(nb, cands, kept);
      for (size_t r = 0; r < kept.size(); r++)
        list.push_back(Cand{kept[r].cost, nb, (int32_t)r, move_id_of(nb), kept[r].i, kept[r].j});
    }
    if (list.empty()) break;
    std::vector<Cand> sel;
    merge_cross(list, sel);
    for (const Cand& x : sel) apply_move(x.id, x.i, x.j, size, tour);
    mv += (int64_t)sel.size();
  }
  if (final_cost) *final_cost = cost_of(size, tour, n, D, wide, nullptr);
  if (evals) *evals = ev;
  if (moves_applied) *moves_applied = mv;
  return it;
}

// noConflict, dvnd.cu:132-175 (including its typos; the MIN/MAX macros of
// dvnd.cuh and the unsigned k of the Or-opt branches are reproduced).
int orc_legacy_no_conflict(int id1, int i1, int j1, int id2, int i2, int j2) {
  auto K = [](int id) -> unsigned { return id == 2 ? 1u : (id == 3 ? 2u : 3u); };
  auto MN = [](int a, int b) { return a < b ? a : b; };
  auto MX = [](int a, int b) { return a > b ? a : b; };
  if (id1 == 0) {
    if (id2 == 0)
      return iabs(i1 - i2) > 1 && iabs(i1 - j2) > 1 && iabs(j1 - i2) > 1 && iabs(j1 - j2) > 1;
    if (id2 == 1) return ((i1 < i2 - 1) || (i1 > j2 - 1)) && ((j1 < i2 - 1) || (j1 > j2 + 1));
    unsigned k2 = K(id2);
    return (j1 < MN(i2, j2) - 1) || ((unsigned)i1 > (unsigned)MX(i2, j2) + k2) ||
           ((i1 < MN(i2, j2) - 1) && ((unsigned)j1 > (unsigned)MX(i2, j2) + k2));
  } else if (id1 == 1) {
    if (id2 == 0) return ((i2 < i1 - 1) || (i2 > j1 + 1)) && ((j2 < i1 - 1) || (j2 > j1 + 1));
    if (id2 == 1) return (j1 < i2 - 1) || (i1 > j2 + 1) || (j2 > i1 - 1) || (i2 > j1 + 1);
    unsigned k2 = K(id2);
    return ((unsigned)i1 > (unsigned)MX(i2, j2) + k2) || (j1 < MN(i2, j2) - 1);
  } else {
    unsigned k1 = K(id1);
    if (id2 == 0)
      return (j2 < MN(i1, i2) - 1) || ((unsigned)i2 > (unsigned)MX(i1, i2) + k1) ||
             ((i2 < MN(i1, i2) - 1) && ((unsigned)j2 > (unsigned)MX(i1, i2) + k1));
    if (id2 == 1) return (j2 < MN(i1, j1) - 1) || ((unsigned)i2 > (unsigned)MX(i1, j1) + k1);
    unsigned k2 = K(id2);
    return ((unsigned)MX(i1, j1) + k1 < (unsigned)MN(i2, j2)) ||
           ((unsigned)MN(i1, j1) > (unsigned)MX(i2, j2) + k2);
  }
}

// betterNoConflict, dvnd.cu:85-130 (std::sort, unstable, as in the reference)
int orc_legacy_better_no_conflict(int m, const int32_t* ids, const int32_t* is, const int32_t* js,
                                  const int32_t* costs, int32_t* selected, int32_t* imp_value,
                                  int maximize, int melhor_para_pior) {
  struct MI {
    int idx;  // original index into the move arrays
    unsigned index;
  };
  std::vector<MI> v(m);
  for (int q = 0; q < m; q++) v[q] = MI{q, (unsigned)q};
  bool desc = melhor_para_pior ? maximize != 0 : maximize == 0;
  if (desc)
    std::sort(v.begin(), v.end(), [&](const MI& a, const MI& b) { return costs[a.idx] > costs[b.idx]; });
  else
    std::sort(v.begin(), v.end(), [&](const MI& a, const MI& b) { return costs[a.idx] < costs[b.idx]; });
  // MLMove64 stores id:4, i:14, j:14 bit-fields (mlads.h:190-195)
  auto id4 = [](int x) { return x & 0xf; };
  auto f14 = [](int x) { return x & 0x3fff; };
  for (int a = 0; a < m; a++) {
    for (int b = a + 1; b < m; b++) {
      int p = v[a].idx, q = v[b].idx;
      if (!orc_legacy_no_conflict(id4(ids[p]), f14(is[p]), f14(js[p]), id4(ids[q]), f14(is[q]),
                                  f14(js[q]))) {
        if (melhor_para_pior) v[b].index = (unsigned)-1;
        else v[a].index = (unsigned)-1;
        break;
      }
    }
  }
  int len = 0;
  int32_t imp = 0;
  for (int a = 0; a < m; a++)
    if (v[a].index != (unsigned)-1) {
      selected[len++] = (int32_t)v[a].index;
      imp += costs[v[a].idx];
    }
  *imp_value = imp;
  return len;
}

// applyMoves, dvnd.cpp:16-145
uint32_t orc_legacy_apply_moves(int size, int32_t* tour, int n, const int32_t* D, int m,
                                const int32_t* ids, const int32_t* is, const int32_t* js) {
  for (int q = 0; q < m; q++) {
    int id = ids[q];
    if (id == 0 || id == 1) apply_move(0, is[q], js[q], size, tour);   // 2-opt applied as swap
    else if (id > 1 && id < 30) apply_move(id, is[q], js[q], size, tour);  // MLP_MAX_NEIGHBOR = 30
  }
  return (uint32_t)cost_of(size, tour, n, D, 0, nullptr);
}

}  // extern "C"
