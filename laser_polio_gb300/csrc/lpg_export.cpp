/*
 * lpg_export.cpp — the results table of save_sim_results (utils.py:689-786)
 * written as CSV by native code.
 *
 * The reference builds a pandas DataFrame with one row per (timestep, node),
 * timestep-major — timestep, date, node, dot_name, then the result fields —
 * and writes it with DataFrame.to_csv(index=False).  That format is a header
 * of the column names, ',' between fields and '\n' after every row.
 * Integers are written in decimal.  Strings are quoted only when they hold
 * ',', '"', '\n' or '\r', with inner quotes doubled (csv.QUOTE_MINIMAL).
 * After the integer result fields come the summary groupings' string
 * columns (utils.py:1040-1160): per-tick ones (time_period) and then per-node
 * ones (adm0, adm1, adm01, region), in the order pandas appends them.
 * At the Nigeria scale the table has 2555 x 774 = 2.0e6 rows.  Here, blocks
 * of timesteps are formatted in parallel by host threads and written to the
 * file in order.
 */
#include <stdint.h>
#include <stdio.h>
#include <string.h>

#include <algorithm>
#include <string>
#include <thread>
#include <vector>

#include "lpg.h"

/* Per-host-thread error text of the standalone ops (lpg_ops.cu). */
int lpg_ops_fail(int code, const char* fmt, ...);

namespace {

std::string csv_field(const char* s) {
  if (!strpbrk(s, ",\"\n\r")) return std::string(s);
  std::string q = "\"";
  for (const char* p = s; *p; ++p) {
    if (*p == '"') q += '"';
    q += *p;
  }
  q += '"';
  return q;
}

void put_int(std::string& out, int64_t v) {
  char buf[24];
  int n = 0;
  uint64_t u = v < 0 ? (uint64_t)0 - (uint64_t)v : (uint64_t)v;
  do {
    buf[n++] = (char)('0' + (int)(u % 10));
    u /= 10;
  } while (u);
  if (v < 0) out += '-';
  while (n) out += buf[--n];
}

/* String columns by tick ([col][t]) and by node ([col][n]), quoted once. */
struct StrCols {
  int32_t n_tick = 0, n_node = 0;
  std::vector<std::string> tick, node;
};

/* Rows of timesteps [t0, t1) into out. */
void format_rows(std::string& out, int32_t t0, int32_t t1, int32_t n_nodes, const std::vector<std::string>& dates,
                 const std::vector<std::string>& names, int32_t n_fields, const int32_t* const* fields,
                 const StrCols& sc, int32_t nt) {
  for (int32_t t = t0; t < t1; ++t) {
    for (int32_t n = 0; n < n_nodes; ++n) {
      const size_t q = (size_t)t * n_nodes + n;
      put_int(out, t);
      out += ',';
      out += dates[t];
      out += ',';
      put_int(out, n);
      out += ',';
      out += names[n];
      for (int32_t k = 0; k < n_fields; ++k) {
        out += ',';
        put_int(out, fields[k][q]);
      }
      for (int32_t c = 0; c < sc.n_tick; ++c) {
        out += ',';
        out += sc.tick[(size_t)c * nt + t];
      }
      for (int32_t c = 0; c < sc.n_node; ++c) {
        out += ',';
        out += sc.node[(size_t)c * n_nodes + n];
      }
      out += '\n';
    }
  }
}

int write_csv(const char* path, int32_t nt, int32_t n_nodes, const char* const* dates, const char* const* dot_names,
              int32_t n_fields, const char* const* field_names, const int32_t* const* fields, int32_t n_tick_cols,
              const char* const* tick_col_names, const char* const* tick_cols, int32_t n_node_cols,
              const char* const* node_col_names, const char* const* node_cols) {
  if (!path) return lpg_ops_fail(LPG_ERR_ARG, "write_results_csv: null path");
  if (nt < 0 || n_nodes < 0 || n_fields < 0 || n_fields > LPG_EXPORT_MAX_FIELDS)
    return lpg_ops_fail(LPG_ERR_ARG, "write_results_csv: bad sizes nt=%d n_nodes=%d n_fields=%d", nt, n_nodes,
                        n_fields);
  if ((nt > 0 && !dates) || (n_nodes > 0 && !dot_names) || (n_fields > 0 && (!field_names || !fields)))
    return lpg_ops_fail(LPG_ERR_ARG, "write_results_csv: a required array is NULL");
  for (int32_t k = 0; k < n_fields; ++k)
    if (!field_names[k] || (!fields[k] && nt > 0 && n_nodes > 0))
      return lpg_ops_fail(LPG_ERR_ARG, "write_results_csv: field %d is NULL", k);
  if (n_tick_cols < 0 || n_node_cols < 0 || n_tick_cols + n_node_cols > LPG_EXPORT_MAX_FIELDS ||
      (n_tick_cols > 0 && (!tick_col_names || (nt > 0 && !tick_cols))) ||
      (n_node_cols > 0 && (!node_col_names || (n_nodes > 0 && !node_cols))))
    return lpg_ops_fail(LPG_ERR_ARG, "write_results_csv: bad string columns (%d by tick, %d by node)", n_tick_cols,
                        n_node_cols);
  for (int32_t c = 0; c < n_tick_cols; ++c)
    if (!tick_col_names[c]) return lpg_ops_fail(LPG_ERR_ARG, "write_results_csv: a column name is NULL");
  for (int32_t c = 0; c < n_node_cols; ++c)
    if (!node_col_names[c]) return lpg_ops_fail(LPG_ERR_ARG, "write_results_csv: a column name is NULL");
  StrCols sc;
  sc.n_tick = n_tick_cols;
  sc.n_node = n_node_cols;
  sc.tick.resize((size_t)n_tick_cols * nt);
  sc.node.resize((size_t)n_node_cols * n_nodes);
  for (size_t q = 0; q < sc.tick.size(); ++q) {
    if (!tick_cols[q]) return lpg_ops_fail(LPG_ERR_ARG, "write_results_csv: a tick column value is NULL");
    sc.tick[q] = csv_field(tick_cols[q]);
  }
  for (size_t q = 0; q < sc.node.size(); ++q) {
    if (!node_cols[q]) return lpg_ops_fail(LPG_ERR_ARG, "write_results_csv: a node column value is NULL");
    sc.node[q] = csv_field(node_cols[q]);
  }
  std::vector<std::string> ds(nt), nm(n_nodes);
  for (int32_t t = 0; t < nt; ++t) {
    if (!dates[t]) return lpg_ops_fail(LPG_ERR_ARG, "write_results_csv: date %d is NULL", t);
    ds[t] = csv_field(dates[t]);
  }
  for (int32_t n = 0; n < n_nodes; ++n) {
    if (!dot_names[n]) return lpg_ops_fail(LPG_ERR_ARG, "write_results_csv: dot_name %d is NULL", n);
    nm[n] = csv_field(dot_names[n]);
  }
  FILE* f = fopen(path, "wb");
  if (!f) return lpg_ops_fail(LPG_ERR_ARG, "write_results_csv: cannot open %s for writing", path);
  std::string head = "timestep,date,node,dot_name";
  for (int32_t k = 0; k < n_fields; ++k) {
    head += ',';
    head += csv_field(field_names[k]);
  }
  for (int32_t c = 0; c < n_tick_cols; ++c) {
    head += ',';
    head += csv_field(tick_col_names[c]);
  }
  for (int32_t c = 0; c < n_node_cols; ++c) {
    head += ',';
    head += csv_field(node_col_names[c]);
  }
  head += '\n';
  bool ok = fwrite(head.data(), 1, head.size(), f) == head.size();
  /* about 64k rows per block; up to 16 blocks formatted at once */
  const int32_t per = std::max<int32_t>(1, (int32_t)(65536 / std::max<int32_t>(1, n_nodes)));
  const unsigned hw = std::max(1u, std::min(16u, std::thread::hardware_concurrency()));
  std::vector<std::string> bufs(hw);
  std::vector<char> failed(hw, 0);
  for (int32_t t0 = 0; ok && t0 < nt; t0 += per * (int32_t)hw) {
    std::vector<std::thread> th;
    th.reserve(hw);
    int used = 0;
    for (unsigned w = 0; w < hw; ++w) {
      const int32_t a = t0 + (int32_t)w * per, b = std::min<int32_t>(nt, a + per);
      if (a >= nt) break;
      bufs[w].clear();
      auto job = [&, w, a, b]() {
        try {
          format_rows(bufs[w], a, b, n_nodes, ds, nm, n_fields, fields, sc, nt);
        } catch (...) {
          failed[w] = 1;
        }
      };
      try {
        th.emplace_back(job);
      } catch (...) { /* no thread: format this block here */
        job();
      }
      ++used;
    }
    for (auto& x : th) x.join();
    for (int w = 0; w < used; ++w) ok = ok && !failed[w];
    for (int w = 0; ok && w < used; ++w) ok = fwrite(bufs[w].data(), 1, bufs[w].size(), f) == bufs[w].size();
  }
  if (fclose(f) != 0) ok = false;
  if (!ok) return lpg_ops_fail(LPG_ERR_ARG, "write_results_csv: writing %s failed", path);
  return LPG_OK;
}

}  // namespace

extern "C" int lpg_write_results_csv(const char* path, int32_t nt, int32_t n_nodes, const char* const* dates,
                                     const char* const* dot_names, int32_t n_fields, const char* const* field_names,
                                     const int32_t* const* fields, int32_t n_tick_cols,
                                     const char* const* tick_col_names, const char* const* tick_cols,
                                     int32_t n_node_cols, const char* const* node_col_names,
                                     const char* const* node_cols) {
  try {
    return write_csv(path, nt, n_nodes, dates, dot_names, n_fields, field_names, fields, n_tick_cols, tick_col_names,
                     tick_cols, n_node_cols, node_col_names, node_cols);
  } catch (...) { /* allocation or thread creation failed: nothing escapes the C ABI */
    return lpg_ops_fail(LPG_ERR_NOMEM, "write_results_csv: out of host resources");
  }
}
