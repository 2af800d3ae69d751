// Host check of the inverse z passes' launch-row order (zinv_slot in lh_internal.cuh;
// tests/test_fft_host.py builds and runs it): for every split of nuI u slots and nvI v slots up
// to 160 + 160, the rows map onto the slots one to one, and the levels the staggered
// interpolation reads (v faces q - 1, q for u level q; u levels q, q + 1 for v level q, with
// u slot s at u level s + 1 and v slot s at v level s + 1) were already read by one of the two
// rows before (the second read of a level comes from L2) whenever both slot kinds remain.
// Prints "ok <cases>" or the first failing split.
#include "../rnl_multiblock_nofft_gb300/csrc/lh_internal.cuh"

#include <cstdio>
#include <cstring>
#include <vector>

int main() {
  int cases = 0;
  for (int nu = 0; nu <= 160; ++nu) {
    for (int nv = 0; nv <= 160; ++nv) {
      Geo g;
      std::memset(&g, 0, sizeof(g));
      g.nuI = nu; g.nvI = nv;
      const int n = nu + nv;
      std::vector<int> seen(n, 0);
      for (int y = 0; y < n; ++y) {
        const int s = zinv_slot(g, y);
        if (s < 0 || s >= n || seen[s]++) { std::printf("bad %d %d row %d slot %d\n", nu, nv, y, s); return 1; }
      }
      // neighbour reuse while the rows alternate: row y reads a level of u (or v) that row
      // y - 1 or y - 2 read as well
      const int m = nu < nv ? nu : nv;
      for (int y = 2; y < 2 * m; ++y) {
        const int s = zinv_slot(g, y), p1 = zinv_slot(g, y - 1);
        const bool isU = s < nu;
        const int q = isU ? s + 1 : s - nu + 1;                 // level of this row
        const int qp = p1 < nu ? p1 + 1 : p1 - nu + 1;          // level of the row before
        // u row (level q) reads v faces q - 1 and q; the v row before it (level q - 1) read v at q - 1
        // v row (level q) reads u levels q and q + 1; the u row before it (level q) read u at q
        const bool ok = isU ? (qp == q - 1) : (qp == q);
        if (!ok) { std::printf("reuse %d %d row %d\n", nu, nv, y); return 1; }
      }
      ++cases;
    }
  }
  std::printf("ok %d\n", cases);
  return 0;
}
