"""RI timers kept as a base value (csrc/lpg_ri.h) against the reference's
tick-by-tick subtraction (fast_ri, model.py:1825-1854), on the CPU.

For every int16 base, several RI step sizes and first-RI-tick indices, a C
loop subtracts the step on each RI tick exactly as the reference does (int32
difference, eligibility window on it, int16 store) and records the first
eligible tick and the stored values; the closed forms must agree."""

import subprocess
from pathlib import Path

ROOT = Path(__file__).resolve().parent.parent

SRC = r"""
#include <stdio.h>
#include <stdint.h>
#include "lpg_ri.h"

int main(void) {
  const int steps[] = {1, 2, 7, 14, 30, 182, 365};
  const int firsts[] = {1, 2, 3, 9};
  long bad = 0, checked = 0;
  for (int si = 0; si < 7; ++si) {
    const int s = steps[si];
    const int stride = s < 7 ? 61 : 1; /* small steps: long loops, fewer bases */
    for (int fi = 0; fi < 4; ++fi) {
      const int m_lo = firsts[fi];
      for (int u = -32768; u <= 32767; u += stride) {
        int16_t x = (int16_t)u;
        int32_t due = -1;
        const int32_t limit = m_lo + 2 * (65536 / s) + 4;
        for (int32_t m = m_lo; m <= limit; ++m) {
          const int32_t timer = (int32_t)x - s;
          int el = (m == 1) ? (timer <= 0 && timer >= -s) : (timer <= 0 && timer > -s);
          if (el && due < 0) due = m * s;
          x = (int16_t)timer;
          const int32_t n = m - m_lo + 1;
          if (lpg_ri_value((int16_t)u, n, s) != x) ++bad;
          if (lpg_ri_applied(m_lo, m * s, s) != n || lpg_ri_applied(m_lo, m * s + s - 1, s) != n) ++bad;
          if (due >= 0 && m * s > due + 4 * s && n > 8) break;
        }
        if (lpg_ri_applied(m_lo, m_lo * s - 1, s) != 0) ++bad;
        if (due < 0 || lpg_ri_due_tick((int16_t)u, m_lo, s) != due) {
          if (bad < 5) printf("u=%d s=%d m_lo=%d due=%d got=%d\n", u, s, m_lo, due, lpg_ri_due_tick((int16_t)u, m_lo, s));
          ++bad;
        }
        ++checked;
      }
    }
  }
  if (lpg_ri_first(0, -500, 14) != 1 || lpg_ri_first(1, 14, 14) != 1 || lpg_ri_first(1, 15, 14) != 2 ||
      lpg_ri_first(1, 1, 14) != 1)
    ++bad;
  printf("checked %ld bad %ld\n", checked, bad);
  return bad != 0;
}
"""


def test_ri_base_value_closed_forms_match_tick_by_tick(tmp_path):
    src = tmp_path / "ri.c"
    src.write_text(SRC)
    exe = tmp_path / "ri"
    subprocess.run(["gcc", "-O2", f"-I{ROOT / 'laser_polio_gb300' / 'csrc'}", str(src), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True)
    assert out.returncode == 0, out.stdout
    assert "bad 0" in out.stdout


GAP_SRC = r"""
#include <stdio.h>
#include <stdint.h>

/* For every int16 base, step and first RI tick index: the RI ticks between
 * the first two eligibilities of the reference's subtraction loop.  The
 * engine gives each agent one due tick a run, which holds while the run's
 * last RI tick index is below 65536 / step (lpg_check_desc refuses longer
 * runs with RI): that needs every gap to be at least 65536 / step - 1. */
int main(void) {
  const int steps[] = {1, 2, 7, 14, 16, 30, 182, 365};
  long bad = 0;
  for (int si = 0; si < 8; ++si) {
    const int s = steps[si];
    for (int m_lo = 1; m_lo <= 3; ++m_lo)
      for (int u = -32768; u <= 32767; u += (s < 7 ? 7 : 1)) {
        int16_t x = (int16_t)u;
        long m1 = -1, gap = -1;
        const long limit = m_lo + 3L * (65536 / s) + 10;
        for (long m = m_lo; m <= limit && gap < 0; ++m) {
          const int32_t timer = (int32_t)x - s;
          const int el = (m == 1) ? (timer <= 0 && timer >= -s) : (timer <= 0 && timer > -s);
          if (el) {
            if (m1 < 0) m1 = m;
            else gap = m - m1;
          }
          x = (int16_t)timer;
        }
        if (gap < 0 || gap < 65536 / s - 1) {
          if (bad < 5) printf("u=%d s=%d m_lo=%d gap=%ld\n", u, s, m_lo, gap);
          ++bad;
        }
      }
  }
  printf("bad %ld\n", bad);
  return bad != 0;
}
"""


def test_no_agent_is_due_for_ri_twice_within_the_runs_the_engine_accepts(tmp_path):
    src = tmp_path / "gap.c"
    src.write_text(GAP_SRC)
    exe = tmp_path / "gap"
    subprocess.run(["gcc", "-O2", "-o", str(exe), str(src)], check=True)
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout


def test_runs_where_an_ri_timer_comes_round_twice_are_refused():
    """With step 14 the last RI tick index must stay below 65536 // 14 =
    4681: a run of 65533 ticks after tick 0 is accepted, 65534 refused."""
    import pytest

    from laser_polio_gb300 import _lib, synthetic
    from laser_polio_gb300.engine import make_desc

    for dur, ok in ((65533, True), (65534, False)):
        params, _ = synthetic.bundle(kind="zamfara", n_agents=2000, n_nodes=3, dur=dur, seed=1)
        assert params["ri_enabled"] and params["ri_step"] == 14
        desc, _keep = make_desc(params)
        if ok:
            _lib.check_desc(desc)
        else:
            with pytest.raises(ValueError, match="come round twice"):
                _lib.check_desc(desc)
