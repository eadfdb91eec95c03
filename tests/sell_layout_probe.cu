// Host-side check of the sliced operator's slot map (sell_row, sell_slot,
// sell_read_len in lpm_internal.cuh), built and run by
// tests/test_sell_layout_cpu.py.  For seeded row lengths (empty rows, rows
// shorter than a group of four, slices of equal rows, mixed slices, a
// partial last slice) it checks that every slot a row's blocks and read
// padding map to lies inside the row's slice and is used once, that group
// loads start on a multiple of four slots, and that at most three blocks of
// a row sit past the groups.  Prints "ok" and exits 0, else the first
// failure and exits 1.
#include <cstdint>
#include <cstdio>
#include <random>
#include <vector>

#include "lpm_internal.cuh"

using lpm::kSlice;
using lpm::kVec;

static int fail(const char* what, int trial, int j, int k) {
  std::printf("%s: trial %d row %d block %d\n", what, trial, j, k);
  return 1;
}

int main() {
  std::mt19937 rng(20261203u);
  for (int trial = 0; trial < 400; ++trial) {
    const int n = 1 + (int)(rng() % 300);
    std::vector<int> len((size_t)n);
    for (int& l : len) l = (int)(rng() % 70);
    if (trial % 4 == 0)
      for (int& l : len) l = 61;  // interior rows of the simple-cubic lattice
    if (trial % 4 == 1)
      for (int& l : len) l = (int)(rng() % 4);  // slices with no group of four
    // slice sizes as the pattern build sets them: 32 x the longest row
    const int ns = (n + kSlice - 1) / kSlice;
    std::vector<int64_t> sp((size_t)ns + 1, 0);
    for (int s = 0; s < ns; ++s) {
      int mx = 0;
      for (int j = s * kSlice; j < n && j < (s + 1) * kSlice; ++j) mx = len[(size_t)j] > mx ? len[(size_t)j] : mx;
      sp[(size_t)s + 1] = sp[(size_t)s] + (int64_t)mx * kSlice;
    }
    if (sp[(size_t)ns] % kVec != 0) return fail("slot count not a multiple of four", trial, -1, -1);
    std::vector<char> used((size_t)sp[(size_t)ns], 0);
    for (int j = 0; j < n; ++j) {
      const lpm::SellRow r = lpm::sell_row(sp.data(), j);
      const int l = len[(size_t)j];
      if (l - r.g4 > 3) return fail("more than three blocks past the groups", trial, j, l);
      const int rl = lpm::sell_read_len(r, l);
      if (rl < l) return fail("read length shorter than the row", trial, j, rl);
      for (int k = 0; k < rl; ++k) {
        const int64_t s = lpm::sell_slot(r, k);
        if (s < sp[(size_t)(j / kSlice)] || s >= sp[(size_t)(j / kSlice) + 1]) return fail("slot outside its slice", trial, j, k);
        if (used[(size_t)s]) return fail("slot used twice", trial, j, k);
        used[(size_t)s] = 1;
        if (k < r.g4 && k % kVec == 0 && s % kVec != 0) return fail("group not on a multiple of four", trial, j, k);
      }
    }
  }
  std::printf("ok\n");
  return 0;
}
