// ring_policy.h -- when the retry loop rebuilds the grid, and for which
// radius: shared by the host loop and the graph's step kernel (join.cu) and
// checked on the host by tests/ring_policy_check.cpp.
#pragma once

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>

#ifndef __CUDACC__  // plain C++ (host tests)
#ifndef __host__
#define __host__
#endif
#ifndef __device__
#define __device__
#endif
#endif

namespace knnsj {

// Cells per dimension a ring of radius r spans on a grid of width w.
inline double ring_rows(double r, double w, uint32_t di) {
  const double per = 2.0 * r / w + 1.0;
  return std::pow(per, (double)(di > 0 ? di - 1 : 0));
}

// A grid of width w is rebuilt before a pass whose largest radius rmax needs
// more ring rows than max(3^(di-1), 64) (and exceeds w).  The row count grows
// with rmax, so the rule is rmax > r_limit: the largest radius that still
// fits, found once per grid by bisection over the ordered bit patterns of
// positive doubles.  The host loop and the graph's step kernel both use it.
// With one indexed dimension a ring is one row whatever its radius: no limit.
inline double regrid_limit(double w, uint32_t di) {
  if (di <= 1) return HUGE_VAL;
  const double allowed = std::max(std::pow(3.0, (double)(di - 1)), 64.0);
  auto over = [&](double r) { return ring_rows(r, w, di) > allowed; };
  uint64_t lo = 0, hi;  // bit patterns: over(lo) false, over(hi) true
  double top = w;
  while (!over(top)) {
    if (!(top < 1e300)) return top;  // (unreachable for di >= 2: the rows grow with r)
    top *= 2.0;
  }
  std::memcpy(&hi, &top, 8);
  while (hi - lo > 1) {
    const uint64_t mid = lo + (hi - lo) / 2;
    double x;
    std::memcpy(&x, &mid, 8);
    if (over(x))
      hi = mid;
    else
      lo = mid;
  }
  double r;
  std::memcpy(&r, &lo, 8);
  return r;
}

// Every ring stays within MAX_RING_ROWS rows, whatever the spread of the
// per-query radii (rows are indexed in 32 bits and each one is visited): a
// grid of width w serves radii up to w * ring_div / 2, whose rings span at
// most ring_div + 3 cells per dimension, and a larger radius forces a
// rebuild sized for it.  A single row (one indexed dimension) needs no cap.
constexpr double MAX_RING_ROWS = 1048576.0;
inline double ring_div_of(uint32_t di) {
  if (di <= 1) return 0.0;
  return std::max(std::pow(MAX_RING_ROWS, 1.0 / (double)(di - 1)) - 3.0, 1.0);
}
__host__ __device__ inline bool ring_too_wide(double rmax, double width, double ring_div) {
  return ring_div > 0.0 && rmax > 0.5 * width * ring_div;
}

// The radius the next grid is sized for and whether a rebuild is due, from
// the radius the grid should suit (rgrid) and the largest radius in flight.
__host__ __device__ inline bool regrid_due(double& rgrid, double rmax, double r_limit, double width,
                                           double ring_div) {
  if (ring_too_wide(rmax, width, ring_div)) {
    const double need = 2.0 * rmax / ring_div;
    if (need > rgrid) rgrid = need;
    return true;
  }
  return rgrid > r_limit && rgrid > width;
}

}  // namespace knnsj
