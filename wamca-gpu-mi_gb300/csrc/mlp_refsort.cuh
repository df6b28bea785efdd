// mlp_refsort.cuh -- the candidate-list sort of MLSolution::random, restated.
//
// MLSolution::random (source/mlsolution.cpp:754-874) keeps one candidate
// array for the whole construction and, at every step, reorders it in place
// with std::sort by distance to the client added last (ClientCompAsc /
// ClientCompDsc, mlsolution.cpp:44-71), then removes the chosen entry by
// shifting.  std::sort is not stable, so which of several equally distant
// candidates lands at a given rank depends on the exact steps of the
// library's sort and on the order the array had before.  The reference is
// built with GCC's libstdc++ (GCC 13 here), whose std::sort is an introsort:
//   1. while a range holds more than 16 elements: unless the depth budget
//      (2 floor(log2 n) levels) is spent, put the median of the elements at
//      first + 1, middle and last - 1 at the front, partition the rest
//      around it without bounds checks (advance from the left past elements
//      ordered before the pivot, from the right past elements the pivot is
//      ordered before, swap, repeat until the two meet), handle the right
//      part the same way and continue with the left part; with the budget
//      spent, heap-sort the range;
//   2. insertion-sort the first 16 elements, then insert every later
//      element without a lower-bound check.
// RefSort below performs these steps, comparison for comparison and move
// for move, on (key, id) pairs ordered by key alone, so the resulting
// permutation equals std::sort's on the same input (checked against the
// library on the host: tests/refsort_check.cpp).  It compiles for the
// device (no recursion: an explicit stack of pending ranges) and the host.
#pragma once

#include <cstdint>

#include "mlp_common.cuh"

namespace mlp {

struct RefSortRange {
  int32_t lo, hi, depth;
};

class RefSort {
 public:
  MLP_HD RefSort(uint32_t* key, int32_t* id, bool desc) : key_(key), id_(id), desc_(desc) {}

  // Orders [0, n).
  MLP_HD void sort(int n) {
    if (n <= 1) return;
    int lg = 0;
    while ((n >> (lg + 1)) != 0) lg++;  // floor(log2 n)
    RefSortRange stack[64];
    int top = 0;
    stack[top++] = RefSortRange{0, n, 2 * lg};
    while (top > 0) {
      RefSortRange r = stack[--top];
      while (r.hi - r.lo > kThreshold) {
        if (r.depth == 0) {
          heap_sort(r.lo, r.hi);
          break;
        }
        r.depth--;
        const int cut = partition_around_median(r.lo, r.hi);
        stack[top++] = RefSortRange{cut, r.hi, r.depth};
        r.hi = cut;
      }
    }
    if (n > kThreshold) {
      insertion(0, kThreshold);
      for (int i = kThreshold; i < n; i++) insert_unbounded(i);
    } else {
      insertion(0, n);
    }
  }

  // Heap sort of [lo, hi) (the sort's fallback once its depth budget is spent).
  MLP_HD void heap_sort(int lo, int hi) {
    const int len = hi - lo;
    if (len >= 2) {
      for (int parent = (len - 2) / 2;; parent--) {
        sift(lo, parent, len, key_[lo + parent], id_[lo + parent]);
        if (parent == 0) break;
      }
    }
    for (int last = hi; last - lo > 1;) {
      last--;
      const uint32_t k = key_[last];
      const int32_t v = id_[last];
      copy_to(last, lo);
      sift(lo, 0, last - lo, k, v);
    }
  }

 private:
  static constexpr int kThreshold = 16;
  uint32_t* key_;
  int32_t* id_;
  bool desc_;

  MLP_HD bool before(uint32_t a, uint32_t b) const { return desc_ ? a > b : a < b; }
  MLP_HD void swap_at(int i, int j) {
    const uint32_t k = key_[i];
    key_[i] = key_[j];
    key_[j] = k;
    const int32_t v = id_[i];
    id_[i] = id_[j];
    id_[j] = v;
  }
  MLP_HD void copy_to(int dst, int src) {
    key_[dst] = key_[src];
    id_[dst] = id_[src];
  }

  // The median of the elements at a, b and c goes to position `to`.
  MLP_HD void median_to(int to, int a, int b, int c) {
    if (before(key_[a], key_[b])) {
      if (before(key_[b], key_[c])) swap_at(to, b);
      else if (before(key_[a], key_[c])) swap_at(to, c);
      else swap_at(to, a);
    } else if (before(key_[a], key_[c])) {
      swap_at(to, a);
    } else if (before(key_[b], key_[c])) {
      swap_at(to, c);
    } else {
      swap_at(to, b);
    }
  }

  // Partition of [lo + 1, hi) around the pivot placed at lo; returns the cut.
  MLP_HD int partition_around_median(int lo, int hi) {
    median_to(lo, lo + 1, lo + (hi - lo) / 2, hi - 1);
    const uint32_t pk = key_[lo];
    int f = lo + 1, l = hi;
    while (true) {
      while (before(key_[f], pk)) f++;
      l--;
      while (before(pk, key_[l])) l--;
      if (!(f < l)) return f;
      swap_at(f, l);
      f++;
    }
  }

  MLP_HD void insertion(int lo, int hi) {
    if (lo == hi) return;
    for (int i = lo + 1; i < hi; i++) {
      if (before(key_[i], key_[lo])) {
        const uint32_t k = key_[i];
        const int32_t v = id_[i];
        for (int j = i; j > lo; j--) copy_to(j, j - 1);
        key_[lo] = k;
        id_[lo] = v;
      } else {
        insert_unbounded(i);
      }
    }
  }

  // Moves the element at i left past every element it is ordered before
  // (an element ordered no later than it stops the walk).
  MLP_HD void insert_unbounded(int i) {
    const uint32_t k = key_[i];
    const int32_t v = id_[i];
    int j = i;
    while (before(k, key_[j - 1])) {
      copy_to(j, j - 1);
      j--;
    }
    key_[j] = k;
    id_[j] = v;
  }

  // Max-heap (under `before`) on [lo, lo + len), children of h at 2h + 1 and
  // 2h + 2 relative to lo: the hole at h sinks along the larger children to
  // the bottom, then (k, v) rises from there back towards h.
  MLP_HD void sift(int lo, int h, int len, uint32_t k, int32_t v) {
    const int top = h;
    int c = h;
    while (c < (len - 1) / 2) {
      c = 2 * (c + 1);
      if (before(key_[lo + c], key_[lo + c - 1])) c--;
      copy_to(lo + h, lo + c);
      h = c;
    }
    if ((len & 1) == 0 && c == (len - 2) / 2) {
      c = 2 * (c + 1);
      copy_to(lo + h, lo + c - 1);
      h = c - 1;
    }
    int parent = (h - 1) / 2;
    while (h > top && before(key_[lo + parent], k)) {
      copy_to(lo + h, lo + parent);
      h = parent;
      parent = (h - 1) / 2;
    }
    key_[lo + h] = k;
    id_[lo + h] = v;
  }
};

}  // namespace mlp
