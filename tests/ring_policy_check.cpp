// Host check of the grid-rebuild policy (csrc/ring_policy.h): the regrid
// limit is the largest radius whose ring fits the row budget, and a radius
// too wide for the grid forces a rebuild after which its ring has at most
// 2^20 rows.  Built and run by tests/test_ring_policy.py.
#include "ring_policy.h"
#include <cstdio>
#include <random>
int main() {
  using namespace knnsj;
  std::mt19937_64 g(3);
  std::uniform_real_distribution<double> lw(-12.0, 12.0), lr(-6.0, 14.0);
  long bad = 0, n = 0, forced = 0;
  for (uint32_t di = 1; di <= 8; di++) {
    const double div = ring_div_of(di);
    for (int it = 0; it < 200000; it++) {
      const double w = std::exp2(lw(g));
      const double rmax = w * std::exp2(lr(g));
      n++;
      if (it < 2000 && di == 1) {  // one row whatever the radius: no limit
        if (!std::isinf(regrid_limit(w, di))) bad++;
      } else if (it < 2000) {  // the limit: fits, and the next radius up does not
        const double lim = regrid_limit(w, di);
        const double allowed = std::max(std::pow(3.0, (double)di - 1.0), 64.0);
        if (!(ring_rows(lim, w, di) <= allowed && ring_rows(std::nextafter(lim, 1e300), w, di) > allowed)) {
          if (bad < 5) printf("limit di=%u w=%a lim=%a\n", di, w, lim);
          bad++;
        }
      }
      double rgrid = w * 0.5;  // a grid suited to smaller radii than rmax
      const bool due = regrid_due(rgrid, rmax, regrid_limit(w, di), w, div);
      double width = w;
      if (due) width = rgrid * (1.0 + 1.0 / 32768.0);  // the rebuild run_join makes
      if (ring_too_wide(rmax, w, div)) {
        forced++;
        if (!due) bad++;
      }
      // ring cells per dimension of rmax on the grid in use: 2 r / w + 3 at most
      const double per = 2.0 * rmax / width + 3.0;
      const double rows = di > 1 ? std::pow(per, (double)di - 1.0) : 1.0;
      if (due && ring_too_wide(rmax, w, div) && rows > MAX_RING_ROWS * (1.0 + 1e-9)) {
        if (bad < 5) printf("rows di=%u w=%a rmax=%a rows=%g\n", di, w, rmax, rows);
        bad++;
      }
      if (!due && rows > MAX_RING_ROWS * (1.0 + 1e-9)) {
        if (bad < 5) printf("kept di=%u w=%a rmax=%a rows=%g\n", di, w, rmax, rows);
        bad++;
      }
    }
  }
  printf("n=%ld forced=%ld bad=%ld\n", n, forced, bad);
  return bad != 0;
}
