/*
 * lpg_network.cpp — the radiation migration network on the host, threaded
 * by rows.
 *
 * The reference builds its network once per run (model.py:1244-1256) with
 * laser_core's radiation model (Simini et al., Nature 484, 2012):
 *   out[i][j] = k p_i p_j / ((p_i + s_ij) (p_i + p_j + s_ij)),
 * where s_ij is the population of the nodes k other than i and j with
 * d_ik < d_ij strictly: nodes at the same distance as j are not inside the
 * circle, so the value of s_ij does not depend on how ties are ordered.
 * radiation is migration_method's default (pars.py:55); the reference only
 * ever asks for include_home=False (model.py:1252-1254), and laser_core's
 * diagonal for include_home=True is not known here, so it is rejected.  This
 * follows the package's restatement (core.radiation) operation for
 * operation, so the two agree bit for bit:
 *   - each row orders the nodes by distance from i, ties by index (numpy's
 *     stable argsort), and sums the populations in that order;
 *   - s = the cumulative population before the first node at j's distance,
 *     minus p_i when d_ii < d_ij;
 *   - the product and quotient are evaluated left to right, with no FMA
 *     contraction (-ffp-contract=off).
 */
#include <stdint.h>

#include <algorithm>
#include <atomic>
#include <cmath>
#include <numeric>
#include <thread>
#include <vector>

#include "lpg.h"

/* Per-host-thread error text of the standalone ops (lpg_ops.cu). */
int lpg_ops_fail(int code, const char* fmt, ...);

namespace {

void radiation_rows(int32_t i0, int32_t i1, int32_t n, const double* pops, const double* dist, double k,
                    double* out) {
  std::vector<int32_t> order(n);
  std::vector<double> cum(n);
  for (int32_t i = i0; i < i1; ++i) {
    const double* di = dist + (size_t)i * n;
    std::iota(order.begin(), order.end(), 0);
    std::stable_sort(order.begin(), order.end(), [di](int32_t a, int32_t b) { return di[a] < di[b]; });
    /* cum[r] = populations of ranks before r; before[r] = that sum at the
     * first rank of r's distance */
    double c = 0.0;
    for (int32_t r = 0; r < n; ++r) {
      cum[r] = (r > 0 && di[order[r]] == di[order[r - 1]]) ? cum[r - 1] : c;
      c = c + pops[order[r]];
    }
    double* oi = out + (size_t)i * n;
    for (int32_t j = 0; j < n; ++j) oi[j] = 0.0;
    const double pi = pops[i];
    for (int32_t r = 0; r < n; ++r) {
      const int32_t j = order[r];
      if (j == i) continue;
      const double pj = pops[j];
      const double s = cum[r] - (di[i] < di[j] ? pi : 0.0);
      oi[j] = k * pi * pj / ((pi + s) * (pi + pj + s));
    }
  }
}

}  // namespace

extern "C" int lpg_radiation_network(const double* pops, const double* dist, int32_t n, double k,
                                     int32_t include_home, double* out) {
  if (n < 0 || (n > 0 && (!pops || !dist || !out)))
    return lpg_ops_fail(LPG_ERR_ARG, "radiation_network: bad arguments (n=%d)", n);
  if (include_home)
    return lpg_ops_fail(LPG_ERR_ARG, "radiation_network: include_home=True is not supported (the reference "
                                     "builds its network with include_home=False)");
  for (size_t q = 0; q < (size_t)n * n; ++q)
    if (std::isnan(dist[q])) return lpg_ops_fail(LPG_ERR_ARG, "radiation_network: a distance is NaN");
  std::atomic<bool> failed{false};
  try {
    const unsigned hw = std::max(1u, std::min(16u, std::thread::hardware_concurrency()));
    const int32_t per = std::max<int32_t>(1, (n + (int32_t)hw - 1) / (int32_t)hw);
    std::vector<std::thread> th;
    th.reserve(hw);
    for (int32_t i0 = 0; i0 < n; i0 += per) {
      const int32_t i1 = std::min(n, i0 + per);
      auto job = [=, &failed]() {
        try {
          radiation_rows(i0, i1, n, pops, dist, k, out);
        } catch (...) {
          failed = true;
        }
      };
      try {
        th.emplace_back(job);
      } catch (...) { /* no thread: these rows here */
        job();
      }
    }
    for (auto& t : th) t.join();
  } catch (...) {
    failed = true;
  }
  if (failed) return lpg_ops_fail(LPG_ERR_NOMEM, "radiation_network: out of host resources");
  return LPG_OK;
}
