/*
 * mlp_gpu.hpp -- the reference's C++ task API (MLProblem, MLSolution,
 * MTRandom, MLKernel and its neighbourhood kernels) as header-only wrappers
 * over the C-ABI of mlp_gpu.h.
 *
 * Shapes follow the reference (source/mlproblem.h:61-151,
 * source/mlsolution.h:62-434, source/mtrand.h:140-196,
 * source/mlkernel.h:104-318, source/mlkswap.h, mlk2opt.h, mlkoropt.h), in
 * namespace wamca.  A caller of the reference switches its includes and adds
 * `using namespace wamca;`; the call sequence of a kernel stays
 *   init(true) -> setSolution -> sendSolution -> defineKernelGrid ->
 *   launchKernel -> sync -> mergeGPU -> recvResult -> applyMove... ->
 *   getSolution -> term.
 * Differences:
 *   - launchKernel() fills moveData with the per-block candidates (one per
 *     reference block); mergeGPU() runs the whole pass on the GPU (greedy
 *     merge and apply) and leaves in moveData the merged moves in
 *     application order, every one improving, so the reference's host loop
 *     "for each move with cost < 0: applyMove(move)" (runGpuGpu,
 *     source/WamcaExperiment.hpp:229-290) brings the host solution to the
 *     GPU's.  recvResult() and sync() have nothing left to do.
 *   - Failures throw std::runtime_error with mlp_last_error().
 *   - MLSolution::random is the reference's constructor on the host (with
 *     std::sort, so equal distances are ordered by the same library as the
 *     reference's); randomDevice builds it on the GPU, with equal distances
 *     in client-id order or (ties = 1) in the reference's own order.
 */
#ifndef MLP_GPU_HPP
#define MLP_GPU_HPP

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <fstream>
#include <stdexcept>
#include <string>
#include <vector>

#include "mlp_gpu.h"

namespace wamca {

inline void check(int status) {
  if (status != MLP_OK) throw std::runtime_error(std::string("mlp: ") + mlp_last_error());
}

/* MT19937 (source/mtrand.cpp:52-124, source/mtrand.h:167-195). */
class MTRandom {
 public:
  MTRandom() { seed(5489u); }
  void seed(uint32_t s) {
    st_[0] = s;
    for (p_ = 1; p_ < kN; ++p_) st_[p_] = 1812433253u * (st_[p_ - 1] ^ (st_[p_ - 1] >> 30)) + (uint32_t)p_;
  }
  uint32_t rand() {
    if (p_ >= kN) gen();
    uint32_t x = st_[p_++];
    x ^= (x >> 11);
    x ^= (x << 7) & 0x9d2c5680u;
    x ^= (x << 15) & 0xefc60000u;
    return x ^ (x >> 18);
  }
  /* uniform in [0, max] */
  uint32_t rand(uint32_t max) { return (uint32_t)(((max + 1.0) * rand()) / (4294967295u + 1.0)); }

 private:
  static const int kN = 624, kM = 397;
  uint32_t st_[kN];
  int p_ = kN;
  void gen() {
    int i = 0;
    uint32_t y;
    for (; i < kN - kM; i++) {
      y = (st_[i] & 0x80000000u) | (st_[i + 1] & 0x7fffffffu);
      st_[i] = st_[i + kM] ^ (y >> 1) ^ ((y & 1u) ? 0x9908b0dfu : 0u);
    }
    for (; i < kN - 1; i++) {
      y = (st_[i] & 0x80000000u) | (st_[i + 1] & 0x7fffffffu);
      st_[i] = st_[i + (kM - kN)] ^ (y >> 1) ^ ((y & 1u) ? 0x9908b0dfu : 0u);
    }
    y = (st_[kN - 1] & 0x80000000u) | (st_[0] & 0x7fffffffu);
    st_[kN - 1] = st_[kM - 1] ^ (y >> 1) ^ ((y & 1u) ? 0x9908b0dfu : 0u);
    p_ = 0;
  }
};

/* MLProblem: the instance, its distance matrix resident on the GPU (a host
 * copy is fetched on first use by the host-side constructor). */
class MLProblem {
 public:
  bool costTour, distRound, coordShift;
  uint32_t size = 0;       // tour length n + 1 (costTour)
  uint32_t maxWeight = 0;  // largest distance
  std::string filename;

  MLProblem(bool _costTour, bool _distRound, bool _coordShift)
      : costTour(_costTour), distRound(_distRound), coordShift(_coordShift) {}
  virtual ~MLProblem() { free(); }
  MLProblem(const MLProblem&) = delete;
  MLProblem& operator=(const MLProblem&) = delete;

  /* TSPLIB EUC_2D file (MLProblem::load, source/mlproblem.cpp:78-207). */
  void load(const char* fname) {
    free();
    check(mlp_problem_load_tsplib(fname, costTour ? 1 : 0, distRound ? 1 : 0, &h_));
    filename = fname;
    info();
  }
  /* Coordinates already in memory (the reference reads them from a file). */
  void loadCoords(int32_t n, const int32_t* x, const int32_t* y) {
    free();
    check(mlp_problem_create_coords(n, x, y, costTour ? 1 : 0, distRound ? 1 : 0, &h_));
    info();
  }
  void free() {
    if (h_) mlp_problem_destroy(h_);
    h_ = nullptr;
    dist_.clear();
    size = 0;
  }
  uint32_t clientCount() const { return n_; }
  /* distance between clients a and b (host copy) */
  int32_t weight(uint32_t a, uint32_t b) const {
    fetch();
    return dist_[(size_t)a * n_ + b];
  }
  mlp_problem_t handle() const { return h_; }

 private:
  mlp_problem_t h_ = nullptr;
  uint32_t n_ = 0;
  mutable std::vector<int32_t> dist_;
  void info() {
    int32_t n = 0, sz = 0, mx = 0;
    check(mlp_problem_info(h_, &n, &sz, &mx));
    n_ = (uint32_t)n;
    size = (uint32_t)sz;
    maxWeight = (uint32_t)mx;
  }
  void fetch() const {
    if (!dist_.empty()) return;
    dist_.resize((size_t)n_ * n_);
    check(mlp_problem_get_dist(h_, dist_.data()));
  }
};

/* MLSolution: the tour (clients), the adjacent weights, the latency cost
 * (uint32, the reference's wrap-around) and, after ldsUpdate(), the
 * reference's ADS buffer. */
class MLSolution {
 public:
  MLProblem& problem;
  uint32_t size;
  uint32_t cost = 0;
  uint32_t clientCount = 0;
  std::vector<uint16_t> clients;  // ushort ids, as the reference's
  std::vector<uint16_t> weights;
  std::vector<uint32_t> ads;      // MLADSData words (source/mlads.h:38-74)

  explicit MLSolution(MLProblem& prob)
      : problem(prob), size(prob.size), clients(prob.size, 0), weights(prob.size, 0) {}
  virtual ~MLSolution() {
    if (s_) mlp_solver_destroy(s_);
  }
  MLSolution(const MLSolution&) = delete;
  MLSolution& operator=(const MLSolution&) = delete;

  void clear() { clientCount = 0; }
  bool add(uint16_t id) {
    if (clientCount >= size) return false;
    clients[clientCount++] = id;
    return true;
  }
  void assign(const MLSolution& sol) {
    size = sol.size;
    cost = sol.cost;
    clientCount = sol.clientCount;
    clients = sol.clients;
    weights = sol.weights;
    ads = sol.ads;
  }

  /* MLSolution::random (source/mlsolution.cpp:754-874) on the host: each
   * step sorts the remaining candidates by distance to the client added last
   * (std::sort; descending for alpha < 0.5) and takes a random one of the
   * first ceil(alpha * count). */
  void random(MTRandom& rng, float alpha) {
    const uint32_t n = problem.clientCount();
    std::vector<uint32_t> cl;
    for (uint32_t c = 1; c < n; c++) cl.push_back(c);
    clear();
    uint32_t last = 0;
    add(0);
    uint32_t count = (uint32_t)cl.size();
    while (count > 0) {
      uint32_t idx = 0;
      if (count > 1) {
        const uint32_t rcl = (uint32_t)std::ceil(alpha * (float)count);
        idx = rcl > 0 ? rng.rand(rcl - 1) : 0;
        const MLProblem& P = problem;
        if (alpha < 0.5f) {
          std::sort(cl.begin(), cl.begin() + count,
                    [&P, last](uint32_t a, uint32_t b) { return P.weight(last, a) > P.weight(last, b); });
          idx = count - idx - 1;
        } else {
          std::sort(cl.begin(), cl.begin() + count,
                    [&P, last](uint32_t a, uint32_t b) { return P.weight(last, a) < P.weight(last, b); });
        }
      }
      const uint32_t cur = cl[idx];
      add((uint16_t)cur);
      last = cur;
      for (uint32_t i = idx; i + 1 < count; i++) cl[i] = cl[i + 1];
      count--;
    }
    if (problem.costTour) add(0);
    update();
  }
  /* The same constructor on the GPU: ties = 0 takes equal distances in
   * client-id order (fast); ties = 1 in the reference's own std::sort order
   * (the same start as random()). */
  void randomDevice(uint32_t seed, float alpha, int32_t ties = 0) {
    std::vector<int32_t> t(size);
    check(mlp_problem_random_tours_ties(problem.handle(), 1, &seed, alpha, ties, t.data()));
    for (uint32_t i = 0; i < size; i++) clients[i] = (uint16_t)t[i];
    clientCount = size;
    update();
  }
  /* weights and cost (MLSolution::update / costCalc, source/mlsolution.cpp:216-245) */
  void update() {
    weights[0] = 0;
    uint32_t c = 0;
    for (uint32_t i = 1; i < clientCount; i++) {
      weights[i] = (uint16_t)problem.weight(clients[i - 1], clients[i]);
      c += (size - i) * (uint32_t)weights[i];
    }
    cost = c;
  }
  uint32_t costCalc() {
    uint32_t c = 0;
    for (uint32_t i = 1; i < clientCount; i++) c += (size - i) * (uint32_t)weights[i];
    return c;
  }
  /* the reference's ADS buffer for this tour, built on the GPU */
  void ldsUpdate() {
    solver();
    check(mlp_solver_set_tour(s_, tour().data(), (int32_t)size));
    ads.assign(32 + (size_t)size * (size + 3), 0);
    check(mlp_solver_ads(s_, ads.data(), (int64_t)ads.size()));
  }
  const uint32_t* adsData() const { return ads.data(); }
  /* MLSolution::save / load text format (source/mlsolution.cpp:685-751) */
  void save(const char* fname) const {
    std::ofstream os(fname);
    os << size << "\n" << cost << "\n";
    for (uint32_t i = 0; i < clientCount; i++) os << clients[i] << (i + 1 < clientCount ? " " : "\n");
  }
  void load(const char* fname) {
    std::ifstream is(fname);
    uint32_t sz = 0, c = 0;
    if (!(is >> sz >> c)) throw std::runtime_error(std::string("cannot read solution file ") + fname);
    clear();
    for (uint32_t i = 0; i < size; i++) {
      uint32_t v;
      if (!(is >> v)) break;
      add((uint16_t)v);
    }
    update();
  }
  std::vector<int32_t> tour() const {
    std::vector<int32_t> t(clientCount);
    for (uint32_t i = 0; i < clientCount; i++) t[i] = clients[i];
    return t;
  }

 private:
  mlp_solver_t s_ = nullptr;
  void solver() {
    if (!s_) check(mlp_solver_create(problem.handle(), 0, &s_));
  }
};

/* MLMove (source/mlads.h:150-215): move id (SWAP 0, 2OPT 1, OROPT-k k+1),
 * positions i, j and the cost delta. */
struct MLMove {
  int id = 0;
  int i = 0, j = 0;
  int cost = 0;
};

/* MLKernel: one neighbourhood on the GPU (source/mlkernel.h:104-318). */
class MLKernel {
 public:
  MLProblem& problem;
  int id;             // move id
  uint32_t tag;       // k of Or-opt-k
  const char* name;
  bool isTotal;
  uint32_t solSize;
  uint32_t moveElems = 0;
  std::vector<MLMove> moveData;
  MLSolution* solution = nullptr;
  bool solDestroy = false;
  uint32_t callCount = 0, mergeCount = 0, imprvCount = 0;

  MLKernel(MLProblem& _problem, bool _isTotal, int kid, uint32_t ktag = 0)
      : problem(_problem), id(kid), tag(ktag), name(""), isTotal(_isTotal), solSize(_problem.size) {}
  virtual ~MLKernel() { term(); }
  MLKernel(const MLKernel&) = delete;
  MLKernel& operator=(const MLKernel&) = delete;

  void init(bool solCreate) {
    term();
    check(mlp_solver_create(problem.handle(), 0, &s_));
    if (isTotal) {
      if (id > MLP_NB_OROPT3) throw std::runtime_error("mlp: TOTAL mode covers swap, 2-opt and Or-opt-1/2/3");
      check(mlp_solver_set_total(s_, 1));
    }
    if (solCreate) {
      solution = new MLSolution(problem);
      solDestroy = true;
    }
  }
  void term() {
    if (solDestroy) delete solution;
    solution = nullptr;
    solDestroy = false;
    if (s_) mlp_solver_destroy(s_);
    s_ = nullptr;
  }
  void resetStats() { callCount = mergeCount = imprvCount = 0; }
  void setSolution(MLSolution* sol) { solution->assign(*sol); }
  void getSolution(MLSolution* sol) { sol->assign(*solution); }
  void sendSolution() { check(mlp_solver_set_tour(s_, solution->tour().data(), (int32_t)solution->clientCount)); }
  void defineKernelGrid() { moveElems = candidates(); }
  /* the per-block candidates (one per reference block) into moveData */
  void launchKernel() {
    const uint32_t m = candidates();
    std::vector<int64_t> c(m);
    std::vector<int32_t> mi(m), mj(m);
    if (oroptK())
      check(mlp_solver_eval_oropt(s_, (int32_t)tag, c.data(), mi.data(), mj.data()));
    else
      check(mlp_solver_eval(s_, id, c.data(), mi.data(), mj.data()));
    moveData.assign(m, MLMove());
    for (uint32_t b = 0; b < m; b++) moveData[b] = MLMove{id, mi[b], mj[b], (int)c[b]};
    moveElems = m;
    callCount++;
  }
  void sync() {}
  /* the pass on the GPU: merged moves in application order into moveData */
  void mergeGPU() {
    const int32_t cap = (int32_t)solSize;
    std::vector<int32_t> ids(cap), mi(cap), mj(cap);
    std::vector<int64_t> c(cap);
    int32_t cnt = 0;
    int64_t nc = 0;
    if (oroptK())
      check(mlp_solver_pass_oropt(s_, (int32_t)tag, cap, mi.data(), mj.data(), c.data(), &cnt, &nc));
    else
      check(mlp_solver_pass(s_, id, cap, ids.data(), mi.data(), mj.data(), c.data(), &cnt, &nc));
    const int32_t k = std::min(cnt, cap);
    moveData.assign(k, MLMove());
    for (int32_t q = 0; q < k; q++) moveData[q] = MLMove{id, mi[q], mj[q], (int)c[q]};
    moveElems = (uint32_t)k;
    mergeCount++;
    if (k > 0) imprvCount++;
  }
  void recvResult() {}
  /* best candidate of the last launch (MLKernel::bestMove) */
  int bestMove(MLMove& move) {
    int b = -1;
    for (uint32_t q = 0; q < moveElems; q++)
      if (b < 0 || moveData[q].cost < moveData[b].cost) b = (int)q;
    if (b >= 0) move = moveData[b];
    return b;
  }
  /* apply one move to the host solution (applyMove of each kernel:
   * mlkswap.cu:1066-1089, mlk2opt.cu:725-755, mlkoropt.cu:886-935) */
  void applyMove(const MLMove& m) {
    std::vector<uint16_t>& t = solution->clients;
    if (m.id == MLP_NB_SWAP) {
      std::swap(t[m.i], t[m.j]);
    } else if (m.id == MLP_NB_2OPT) {
      std::reverse(t.begin() + m.i, t.begin() + m.j + 1);
    } else {
      const int k = m.id - 1;
      if (m.i < m.j)
        std::rotate(t.begin() + m.i, t.begin() + m.i + k, t.begin() + m.j + k);
      else
        std::rotate(t.begin() + m.j, t.begin() + m.i, t.begin() + m.i + k);
    }
    solution->update();
  }
  mlp_solver_t handle() const { return s_; }

 protected:
  mlp_solver_t s_ = nullptr;
  bool oroptK() const { return id > MLP_NB_OROPT3; }
  uint32_t candidates() const {
    if (oroptK()) return solSize - tag - 2;
    int32_t m = 0;
    check(mlp_solver_num_candidates(s_, id, &m));
    return (uint32_t)m;
  }
};

class MLKernelSwap : public MLKernel {
 public:
  explicit MLKernelSwap(MLProblem& p, bool isTotal = false) : MLKernel(p, isTotal, MLP_NB_SWAP) { name = "SWAP"; }
};
class MLKernel2Opt : public MLKernel {
 public:
  explicit MLKernel2Opt(MLProblem& p, bool isTotal = false) : MLKernel(p, isTotal, MLP_NB_2OPT) { name = "2OPT"; }
};
/* Or-opt-k, k in [1, 28] (move id k + 1) */
class MLKernelOrOpt : public MLKernel {
 public:
  MLKernelOrOpt(MLProblem& p, uint32_t k, bool isTotal = false) : MLKernel(p, isTotal, (int)k + 1, k) {
    if (k < 1 || k > 28) throw std::runtime_error("mlp: Or-opt k must lie in [1, 28]");
    name = "OROPT";
  }
};

}  // namespace wamca

#endif  // MLP_GPU_HPP
