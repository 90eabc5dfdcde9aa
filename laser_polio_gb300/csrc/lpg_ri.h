/*
 * lpg_ri.h — routine-immunisation timers kept as a base value.
 *
 * The reference (RI_ABM.step and fast_ri, model.py:1805-1854, 1947-1968)
 * subtracts step_size from the int16 ri_timer of every alive, not
 * chronically-missed agent on every RI tick (t = m * step_size, m >= 1; no
 * component runs on tick 0) and vaccinates the agent on the tick where the
 * difference lands in (-step_size, 0], or in [-step_size, 0] on the first RI
 * tick (m = 1).  The difference is stored back wrapped to int16.
 *
 * The engine keeps, in the column, the value before the first subtraction
 * that applies to the agent (its base u) and derives the rest:
 *  - lpg_ri_due_tick: the RI tick on which the agent becomes eligible, from
 *    u and the index m_lo of its first RI tick;
 *  - lpg_ri_value: the reference's value after n subtractions, u - n*step
 *    wrapped to int16 (int16 arithmetic is modular, so one subtraction of
 *    n*step wraps like n subtractions of step);
 *  - lpg_ri_applied: how many RI ticks from m_lo up to a tick.
 * m_lo is 1 for the agents of the initial population.  An agent born on
 * tick tb (>= 1; its date of birth) has the first RI tick at or after tb:
 * births come before the RI step within a tick (model.py:1711-1733).
 */
#ifndef LPG_RI_H
#define LPG_RI_H

#include <stdint.h>

#ifndef LPG_HD
#if defined(__CUDACC__)
#define LPG_HD __host__ __device__ __forceinline__
#else
#define LPG_HD static inline
#endif
#endif

/* Index of the first RI tick of an agent (initial population: 1). */
LPG_HD int32_t lpg_ri_first(int is_newborn, int32_t dob, int32_t step) {
  return is_newborn ? (dob + step - 1) / step : 1;
}

/* The RI tick on which an agent with base u and first RI tick index m_lo
 * becomes eligible: (m_lo + j) * step for the least j >= 0 whose value
 * before the subtraction, u - j*step wrapped to int16, is in (0, step] (or
 * in [0, step] when m_lo + j is the first RI tick of the run).  Before any
 * wrap that is j = ceil(u / step) - 1; a base <= 0 falls to -32768, wraps up
 * by 65536 and comes down again. */
LPG_HD int32_t lpg_ri_due_tick(int16_t u, int32_t m_lo, int32_t step) {
  int32_t j;
  if (m_lo == 1 && u >= 0 && u <= step) {
    j = 0;
  } else if (u > 0) {
    j = ((int32_t)u + step - 1) / step - 1;
  } else {
    j = ((int32_t)u + 65536 + step - 1) / step - 1;
  }
  return (m_lo + j) * step;
}

/* RI ticks m * step with m_lo <= m and m * step <= t_last. */
LPG_HD int32_t lpg_ri_applied(int32_t m_lo, int32_t t_last, int32_t step) {
  if (t_last < 0) return 0;
  const int32_t n = t_last / step - m_lo + 1;
  return n > 0 ? n : 0;
}

/* The reference's ri_timer after n subtractions of step from base u. */
LPG_HD int16_t lpg_ri_value(int16_t u, int32_t n, int32_t step) {
  return (int16_t)(uint16_t)((uint32_t)(int32_t)u - (uint32_t)n * (uint32_t)step);
}

#endif
