// Exhaustive check of the merge's branch-free cross-neighbourhood conflict
// test (move_shape / shapes_conflict in mlp_common.cuh) against the oracle's
// canMerge restatement (orc_can_merge, mlkernel.cu:649-729), over every pair of
// moves the five neighbourhoods produce on tours of size 6 .. 24:
//   swap (i, j), j >= i + 2; 2-opt (i, j), i < j; Or-opt-k forward (i < j) and
//   backward (i > j), move id k + 1, with the moved block inside the tour.
// Prints the number of pairs checked and exits 0 when all agree.
#include <cstdio>
#include <vector>

#include "mlp_common.cuh"

extern "C" int orc_can_merge(int id1, int i1, int j1, int id2, int i2, int j2);

struct Mv {
  int id, i, j;
};

int main() {
  long long pairs = 0, bad = 0;
  for (int size = 6; size <= 24; size++) {
    std::vector<Mv> mv;
    for (int i = 1; i <= size - 2; i++)
      for (int j = i + 2; j <= size - 2; j++) mv.push_back({0, i, j});
    for (int i = 1; i <= size - 2; i++)
      for (int j = i + 1; j <= size - 2; j++) mv.push_back({1, i, j});
    for (int k = 1; k <= 3; k++)
      for (int r = 1; r <= size - 2; r++)
        for (int c = r + 1; c + k <= size - 1; c++) {
          mv.push_back({k + 1, r, c});
          mv.push_back({k + 1, c, r});
        }
    for (const Mv& a : mv)
      for (const Mv& b : mv) {
        const bool conflict = mlp::shapes_conflict(mlp::move_shape(a.id, a.i, a.j), mlp::move_shape(b.id, b.i, b.j));
        const bool ref = orc_can_merge(a.id, a.i, a.j, b.id, b.i, b.j) == 0;
        pairs++;
        if (conflict != ref && bad++ < 10)
          std::printf("mismatch size %d: (%d,%d,%d) (%d,%d,%d) engine %d oracle %d\n", size, a.id, a.i, a.j, b.id,
                      b.i, b.j, (int)conflict, (int)ref);
      }
  }
  std::printf("%lld pairs, %lld mismatches\n", pairs, bad);
  return bad == 0 ? 0 : 1;
}
