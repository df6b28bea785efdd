/*
 * oracle/ref_driver.cpp -- TEST INFRASTRUCTURE ONLY.
 *
 * A thin extern "C" driver over the reference's own CPU evaluator, compiled
 * from the reference sources where they lie (see oracle/Makefile) into
 * oracle/_ref/libmlref.so.  It is used to pin the oracle restatement and to
 * generate the golden fixtures under tests/golden/.  Nothing in the product
 * links or loads it.
 *
 * Reference classes driven here:
 *   MLProblem::load            source/mlproblem.cpp:78-207
 *   MLSolution::random         source/mlsolution.cpp:754-874
 *   MLSolution::update         source/mlsolution.cpp:216-228
 *   MLSolution::costCalc       source/mlsolution.cpp:233-245
 *   MLSolution::ldsUpdate      source/mlsolution.cpp:420-486
 *   MTRandom::seed / rand      source/mtrand.cpp:52-61, source/mtrand.h:167-195
 */
#include <cstring>
#include <cstdint>

#include "mlproblem.h"
#include "mlsolution.h"
#include "mtrand.h"

namespace {

MLProblem* load_problem(const char* path, int costTour, int distRound) {
  MLProblem* p = new MLProblem(costTour != 0, distRound != 0, false);
  p->load(path);
  return p;
}

}  // namespace

extern "C" {

/* First `count` raw outputs of MTRandom seeded with `seed`. */
void ref_mt_rand(uint32_t seed, int count, uint32_t* out) {
  MTRandom rng;
  rng.seed(seed);
  for (int i = 0; i < count; i++) out[i] = rng.rand();
}

/* MTRandom::rand(max) outputs. */
void ref_mt_rand_max(uint32_t seed, uint32_t max, int count, uint32_t* out) {
  MTRandom rng;
  rng.seed(seed);
  for (int i = 0; i < count; i++) out[i] = rng.rand(max);
}

/* problem.size for an instance (dimension + costTour). */
int ref_problem_size(const char* path, int costTour, int distRound) {
  MLProblem* p = load_problem(path, costTour, distRound);
  int s = (int)p->size;
  delete p;
  return s;
}

/* Full size x size weight matrix (row-major) and the clients' coordinates. */
int ref_problem_weights(const char* path, int costTour, int distRound,
                        int32_t* out_w, int32_t* out_x, int32_t* out_y) {
  MLProblem* p = load_problem(path, costTour, distRound);
  int n = (int)p->size;
  for (int i = 0; i < n; i++) {
    if (out_x) out_x[i] = p->clients[i].x;
    if (out_y) out_y[i] = p->clients[i].y;
    if (out_w)
      for (int j = 0; j < n; j++) out_w[(size_t)i * n + j] = p->clients[i].weight[j];
  }
  delete p;
  return n;
}

/*
 * MTRandom(seed) -> MLSolution::random(rng, alpha) -> update() -> ldsUpdate().
 * Writes the tour (problem.size entries) and returns costCalc().
 */
uint32_t ref_random_solution(const char* path, int costTour, int distRound,
                             uint32_t seed, float alpha, int32_t* out_tour) {
  MLProblem* p = load_problem(path, costTour, distRound);
  MLSolution* s = new MLSolution(*p, cudaHostAllocDefault);
  MTRandom rng;
  rng.seed(seed);
  s->random(rng, alpha);
  s->update();
  s->ldsUpdate();
  for (uint32_t i = 0; i < s->clientCount; i++) out_tour[i] = s->clients[i];
  uint32_t c = s->costCalc();
  delete s;
  delete p;
  return c;
}

/* Byte size of the ADS buffer for an instance. */
uint32_t ref_ads_size(const char* path, int costTour, int distRound) {
  MLProblem* p = load_problem(path, costTour, distRound);
  MLSolution* s = new MLSolution(*p, cudaHostAllocDefault);
  uint32_t sz = s->adsDataSize;
  delete s;
  delete p;
  return sz;
}

/*
 * Given a tour, run update() + ldsUpdate() and copy the ADS buffer out.
 * Returns costCalc().
 */
uint32_t ref_lds_update(const char* path, int costTour, int distRound,
                        const int32_t* tour, int tour_len, uint32_t* out_ads) {
  MLProblem* p = load_problem(path, costTour, distRound);
  MLSolution* s = new MLSolution(*p, cudaHostAllocDefault);
  s->clientCount = tour_len;
  for (int i = 0; i < tour_len; i++) s->clients[i] = (ushort)tour[i];
  s->update();
  s->ldsUpdate();
  if (out_ads) std::memcpy(out_ads, s->adsData, s->adsDataSize);
  uint32_t c = s->costCalc();
  delete s;
  delete p;
  return c;
}

}  // extern "C"
