// Host-only check of the tensor-core GEMM's upper-triangle tile schedule
// (tc::tri_count, tc::tri_coords in fricc_gb300/csrc/gemm_tc.cu) and of the
// rule the (vv|vv) rebuild's triangle epilogue writes by: every needed tile
// enumerated once, in the order of tc::tile_coords restricted to the tiles
// with mt <= 2 nt + 1, and every element of the symmetric output written
// exactly once (elements with row <= column at their place, those with
// row < column also at their mirror).  Exit status 0 when all hold.
#include "../../fricc_gb300/csrc/gemm_tc.cu"

#include <cstdio>
#include <utility>
#include <vector>

int main() {
  using namespace tc;
  int bad = 0;
  for (int tm = 1; tm <= 340; ++tm) {
    for (int tn = (tm + 1) / 2; tn <= (tm + 1) / 2 + 1; ++tn) {
      const int n = tri_count(tm, tn);
      std::vector<std::pair<int, int>> want;
      for (int id = 0; id < tm * tn; ++id) {
        int mt, nt;
        tile_coords(id, tm, tn, mt, nt);
        if (mt <= 2 * nt + 1) want.push_back({mt, nt});
      }
      if ((int)want.size() != n) {
        std::printf("count tm=%d tn=%d: %d, want %zu\n", tm, tn, n, want.size());
        ++bad;
        continue;
      }
      for (int id = 0; id < n; ++id) {
        int mt, nt;
        tri_coords(id, tm, tn, mt, nt);
        if (mt != want[id].first || nt != want[id].second) ++bad;
      }
    }
  }
  for (int v : {9, 10, 12, 16, 17, 23, 31, 40, 45}) {
    const int R = v * v, tm = (R + BM - 1) / BM, tn = (R + 255) / 256;
    std::vector<int> cnt((size_t)R * R, 0);
    for (int id = 0; id < tri_count(tm, tn); ++id) {
      int mt, nt;
      tri_coords(id, tm, tn, mt, nt);
      for (int r1 = mt * BM; r1 < (mt + 1) * BM && r1 < R; ++r1)
        for (int r2 = nt * 256; r2 < (nt + 1) * 256 && r2 < R; ++r2) {
          if (r1 <= r2) ++cnt[(size_t)r1 * R + r2];
          if (r1 < r2) ++cnt[(size_t)r2 * R + r1];
        }
    }
    for (size_t k = 0; k < cnt.size(); ++k)
      if (cnt[k] != 1) ++bad;
  }
  std::printf("%s (%d failures)\n", bad ? "FAIL" : "OK", bad);
  return bad != 0;
}
