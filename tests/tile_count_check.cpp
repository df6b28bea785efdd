// Host check of the sweep tile-count helpers (mlp_common.cuh): for every tour
// size 4 .. 2048 and every compiled tile shape, sweep_row_tiles / sweep_tiles
// equal a direct enumeration of the tiles' definition (row blocks r0 = 1,
// 1 + tr, ... <= size - 3; diagonals L0 = 1, 1 + tl, ... with
// r0 + L0 <= size - 2), and every position pair (r, c = r + L) with
// 1 <= r <= size - 3, r + 1 <= c <= size - 2 lies in exactly one tile.
#include <cstdio>
#include <vector>

#include "mlp_common.cuh"
#include "mlp_kernels.cuh"

int main() {
  long bad = 0, checked = 0;
  for (int shape = 0; shape < mlp::kNumTileShapes; shape++) {
    const int tl = mlp::kTileShapes[shape].tl, tr = mlp::kTileShapes[shape].tr;
    for (int size = 4; size <= 2048; size++) {
      int total = 0, rb = 0;
      for (int r0 = 1; r0 <= size - 3; r0 += tr, rb++) {
        int row = 0;
        for (int L0 = 1; r0 + L0 <= size - 2; L0 += tl) row++;
        if (row != mlp::sweep_row_tiles(size, r0, tl)) bad++;
        total += row;
      }
      if (rb != mlp::sweep_row_blocks(size, tr)) bad++;
      if (total != mlp::sweep_tiles(size, tl, tr)) bad++;
      if (size <= 300) {  // pair coverage
        std::vector<int> hit((size_t)size * size, 0);
        for (int r0 = 1; r0 <= size - 3; r0 += tr)
          for (int L0 = 1; r0 + L0 <= size - 2; L0 += tl)
            for (int r = r0; r < r0 + tr; r++)
              for (int L = L0; L < L0 + tl; L++)
                if (r <= size - 3 && r + L <= size - 2) hit[(size_t)r * size + r + L]++;
        for (int r = 1; r <= size - 3; r++)
          for (int c = r + 1; c <= size - 2; c++) bad += hit[(size_t)r * size + c] != 1;
      }
      checked++;
    }
  }
  std::printf("%ld cases, %ld mismatches\n", checked, bad);
  return bad != 0;
}
