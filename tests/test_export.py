"""save_sim_results (utils.py:689-786) with the native CSV writer
(lpg_write_results_csv), on the CPU.

The reference's own tests (tests/test_report_saving.py) ask for the columns
below, nt x nodes rows, a round trip through the file, and one dot_name per
node.  The format of pandas' to_csv(index=False) is restated here with the
csv module (',' separator, '\\n' rows, QUOTE_MINIMAL), and the native file
must equal it byte for byte."""

import csv
import datetime
import io
import types

import numpy as np
import pytest

from laser_polio_gb300.core import PropertySet
from laser_polio_gb300.utils import RESULT_TABLE_COLUMNS
from laser_polio_gb300.utils import save_sim_results

COLUMNS = ["timestep", "date", "node", "dot_name"] + [c for c, _ in RESULT_TABLE_COLUMNS]


def _fake_sim(nt, nodes, seed=0, names=None):
    rng = np.random.default_rng(seed)
    start = datetime.date(2019, 1, 1)
    results = types.SimpleNamespace(**{attr: rng.integers(-5, 2_000_000, (nt, nodes)).astype(np.int32)
                                       for _, attr in RESULT_TABLE_COLUMNS})
    if names is None:
        names = [f"AFRO:NIGERIA:STATE_{n % 7}:LGA_{n}" for n in range(nodes)]
    lookup = {n: {"dot_name": names[n]} for n in range(nodes) if names[n] is not None}
    return types.SimpleNamespace(nt=nt, nodes=np.arange(nodes), results=results,
                                 datevec=[start + datetime.timedelta(days=d) for d in range(nt)],
                                 pars=PropertySet({"node_lookup": lookup}))


def _pandas_like_csv(sim):
    nodes = len(sim.nodes)
    lookup = sim.pars.node_lookup
    buf = io.StringIO()
    w = csv.writer(buf, lineterminator="\n", quoting=csv.QUOTE_MINIMAL)
    w.writerow(COLUMNS)
    for t in range(sim.nt):
        for n in range(nodes):
            row = [t, str(sim.datevec[t]), n, lookup.get(n, {}).get("dot_name", "UNKNOWN")]
            row += [int(getattr(sim.results, attr)[t, n]) for _, attr in RESULT_TABLE_COLUMNS]
            w.writerow(row)
    return buf.getvalue().encode()


def test_csv_is_the_pandas_format_byte_for_byte(tmp_path):
    names = ["AFRO:NIGERIA:ZAMFARA:ANKA", 'AFRO:X:"QUOTED":Y', "AFRO:X:A,B:C", None, "AFRO:Z:LINE\nBREAK:W"]
    sim = _fake_sim(7, 5, seed=1, names=names)
    out = tmp_path / "results.csv"
    table = save_sim_results(sim, out)
    assert out.read_bytes() == _pandas_like_csv(sim)
    assert len(table["timestep"]) == sim.nt * 5


def test_many_blocks_and_threads_keep_row_order(tmp_path):
    sim = _fake_sim(400, 300, seed=2)  # 120k rows: several 64k-row blocks formatted by threads
    out = tmp_path / "big.csv"
    save_sim_results(sim, out)
    assert out.read_bytes() == _pandas_like_csv(sim)


def test_round_trip_rows_columns_and_names(tmp_path):
    """The checks of the reference's test_save_sim_results, on the native file."""
    sim = _fake_sim(11, 14, seed=3)
    out = tmp_path / "rt.csv"
    save_sim_results(sim, out)
    with open(out, newline="") as f:
        rows = list(csv.reader(f))
    assert rows[0] == COLUMNS
    body = rows[1:]
    assert len(body) == sim.nt * len(sim.nodes)
    assert max(int(r[0]) for r in body) < sim.nt
    assert len({r[3] for r in body}) == len(sim.nodes)
    for k, (_, attr) in enumerate(RESULT_TABLE_COLUMNS):
        got = np.array([int(r[4 + k]) for r in body]).reshape(sim.nt, -1)
        np.testing.assert_array_equal(got, getattr(sim.results, attr))
    assert [r[1] for r in body[:: len(sim.nodes)]] == [str(d) for d in sim.datevec]


def test_real_sim_object_and_empty_table(tmp_path):
    from laser_polio_gb300 import synthetic

    sim = synthetic.zamfara_like(n_agents=5_000, dur=6, seed=4)
    out = tmp_path / "z.csv"
    save_sim_results(sim, out)
    lines = out.read_text().splitlines()
    assert lines[0] == ",".join(COLUMNS)
    assert len(lines) == 1 + sim.nt * len(sim.nodes)
    empty = _fake_sim(0, 3)
    save_sim_results(empty, tmp_path / "empty.csv")
    assert (tmp_path / "empty.csv").read_text() == ",".join(COLUMNS) + "\n"


def test_errors(tmp_path):
    sim = _fake_sim(3, 2)
    with pytest.raises(ValueError, match="grouping_level"):
        save_sim_results(sim, tmp_path / "x.csv", summary_config={"grouping_level": "adm1"})
    with pytest.raises(ValueError, match="one label more"):
        save_sim_results(sim, tmp_path / "x.csv", summary_config={"time_periods": {"bins": ["2019-01-02"],
                                                                                   "labels": ["a"]}})
    with pytest.raises(OSError, match="cannot open"):
        save_sim_results(sim, tmp_path / "no_such_dir" / "x.csv")
    sim.results.S = sim.results.S[:, :1]
    with pytest.raises(ValueError, match="results.S"):
        save_sim_results(sim, tmp_path / "x.csv")
    # counts are written as int32: a float array or an int64 value beyond int32 is refused, not cut
    sim = _fake_sim(3, 2)
    sim.results.E = sim.results.E.astype(np.float64) + 0.5
    with pytest.raises(TypeError, match="results.E"):
        save_sim_results(sim, tmp_path / "x.csv")
    sim = _fake_sim(3, 2)
    sim.results.I = sim.results.I.astype(np.int64)
    save_sim_results(sim, tmp_path / "ok.csv")  # int64 within range is fine
    sim.results.I[1, 1] = 2**31
    with pytest.raises(ValueError, match="outside int32"):
        save_sim_results(sim, tmp_path / "x.csv")
    try:
        import pandas  # noqa: F401
    except ImportError:
        with pytest.raises(ImportError, match="pandas"):
            save_sim_results(_fake_sim(3, 2), tmp_path / "x.h5")


def test_c_entry_point_rejects_bad_arguments(tmp_path):
    """lpg_write_results_csv's own checks (LPG_ERR_ARG = -1 with a message)."""
    import ctypes as C

    from laser_polio_gb300 import _lib

    lib = _lib.load()
    names = (C.c_char_p * 1)(b"S")
    dates = (C.c_char_p * 1)(b"2019-01-01")
    dots = (C.c_char_p * 1)(b"A:B:C:D")
    field = np.zeros(1, np.int32)
    fields = (C.c_void_p * 1)(field.ctypes.data)
    path = str(tmp_path / "x.csv").encode()
    none = (0, None, None, 0, None, None)
    assert lib.lpg_write_results_csv(None, 1, 1, dates, dots, 1, names, fields, *none) == -1
    assert b"null path" in lib.lpg_op_last_error()
    assert lib.lpg_write_results_csv(path, -1, 1, dates, dots, 1, names, fields, *none) == -1
    assert lib.lpg_write_results_csv(path, 1, 1, dates, dots, 65, names, fields, *none) == -1
    assert b"bad sizes" in lib.lpg_op_last_error()
    assert lib.lpg_write_results_csv(path, 1, 1, None, dots, 1, names, fields, *none) == -1
    assert b"NULL" in lib.lpg_op_last_error()
    assert lib.lpg_write_results_csv(path, 1, 1, dates, dots, 1, names, fields, 1, None, None, 0, None, None) == -1
    assert b"string columns" in lib.lpg_op_last_error()
    assert lib.lpg_write_results_csv(path, 1, 1, dates, dots, 1, names, fields, *none) == 0
    assert (tmp_path / "x.csv").read_text() == "timestep,date,node,dot_name,S\n0,2019-01-01,0,A:B:C:D,0\n"
    tn, tv = (C.c_char_p * 1)(b"time_period"), (C.c_char_p * 1)(b"p,1")
    nn, nv = (C.c_char_p * 1)(b"adm0"), (C.c_char_p * 1)(b"B")
    assert lib.lpg_write_results_csv(path, 1, 1, dates, dots, 1, names, fields, 1, tn, tv, 1, nn, nv) == 0
    assert (tmp_path / "x.csv").read_text() == ("timestep,date,node,dot_name,S,time_period,adm0\n"
                                                '0,2019-01-01,0,A:B:C:D,0,"p,1",B\n')


def _expected_groupings(sim, time_config, level):
    """add_temporal_groupings and add_regional_groupings restated with plain
    loops (utils.py:1040-1160) for the columns a summary_config appends."""
    lookup = sim.pars.node_lookup
    names = [lookup.get(n, {}).get("dot_name", "UNKNOWN") for n in range(len(sim.nodes))]
    cols = {}
    if time_config:
        edges = [datetime.date.fromisoformat(b) for b in time_config["bins"]]
        cols["time_period"] = [time_config["labels"][sum(1 for e in edges if d >= e)] for d in sim.datevec]
    parts = [n.split(":") for n in names]
    adm0 = [p[1] if len(p) > 1 else "" for p in parts]
    adm1 = [p[2] if len(p) > 2 else "" for p in parts]
    adm01 = [a + ":" + b if a and b else "" for a, b in zip(adm0, adm1)]
    region = {"adm0": adm0, "adm01": adm01, "dot_name": names}[level]
    return cols, {"adm0": adm0, "adm1": adm1, "adm01": adm01, "region": region}


def _grouped_csv(sim, tick_cols, node_cols):
    lookup = sim.pars.node_lookup
    buf = io.StringIO()
    w = csv.writer(buf, lineterminator="\n", quoting=csv.QUOTE_MINIMAL)
    w.writerow(COLUMNS + list(tick_cols) + list(node_cols))
    for t in range(sim.nt):
        for n in range(len(sim.nodes)):
            row = [t, str(sim.datevec[t]), n, lookup.get(n, {}).get("dot_name", "UNKNOWN")]
            row += [int(getattr(sim.results, attr)[t, n]) for _, attr in RESULT_TABLE_COLUMNS]
            row += [v[t] for v in tick_cols.values()] + [v[n] for v in node_cols.values()]
            w.writerow(row)
    return buf.getvalue().encode()


@pytest.mark.parametrize("config,level", [
    ({}, "dot_name"),
    ({"admin_level": 1}, "dot_name"),
    ({"grouping_level": "adm0"}, "adm0"),
    ({"time_periods": {"bins": ["2019-01-04", "2019-01-07"], "labels": ["early", "mid", "late"]},
      "grouping_level": "adm01"}, "adm01"),
])
def test_summary_config_groupings(tmp_path, config, level):
    """save_sim_results with a summary_config (run_sim always passes one):
    time_period by date bins closed on the left, adm0/adm1/adm01 from the
    dot name ("" where a field is missing), region at the grouping level."""
    names = ["AFRO:NIGERIA:ZAMFARA:ANKA", "AFRO:NIGERIA:KANO:AJINGI", None, "AFRO:BENIN:ALIBORI"]
    sim = _fake_sim(9, 4, seed=5, names=names)
    out = tmp_path / "g.csv"
    table = save_sim_results(sim, out, summary_config=config)
    tick_cols, node_cols = _expected_groupings(sim, config.get("time_periods"), level)
    assert out.read_bytes() == _grouped_csv(sim, tick_cols, node_cols)
    for col, vals in node_cols.items():
        assert list(table[col][:4]) == vals
    if tick_cols:
        assert list(table["time_period"][::4]) == tick_cols["time_period"]


def test_custom_region_groupings():
    """Custom regions (the regions.yaml structure): a country's nodes whose
    adm01 equals a pattern (adm01 level) or whose dot name contains it take
    the group's name; other countries keep their default region."""
    from laser_polio_gb300.utils import regional_columns

    names = ["AFRO:NIGERIA:KANO:AJINGI", "AFRO:NIGERIA:BORNO:BAMA", "AFRO:NIGERIA:LAGOS:IKEJA",
             "AFRO:BENIN:ALIBORI:KANDI"]
    regions = {"NIGERIA": {"NW_NGA": ["NIGERIA:KANO"], "NE_NGA": ["borno"]}}
    cols = regional_columns(names, ["nigeria", "benin"], "adm01", regions=regions)
    assert cols["region"] == ["NW_NGA", "NE_NGA", "NIGERIA:LAGOS", "BENIN:ALIBORI"]
    cols = regional_columns(names, ["NIGERIA"], "adm0", regions=regions)
    assert cols["region"] == ["NW_NGA", "NE_NGA", "NIGERIA", "BENIN"]


def test_region_groupings_through_save_sim_results(tmp_path):
    """region_groupings with the regions given in the summary_config."""
    names = ["AFRO:NIGERIA:KANO:AJINGI", "AFRO:NIGERIA:BORNO:BAMA"]
    sim = _fake_sim(3, 2, seed=6, names=names)
    cfg = {"region_groupings": ["NIGERIA"], "regions": {"NIGERIA": {"NW_NGA": ["KANO"], "NE_NGA": ["BORNO"]}}}
    table = save_sim_results(sim, tmp_path / "r.csv", summary_config=cfg)
    assert list(table["region"][:2]) == ["NW_NGA", "NE_NGA"]
    assert (tmp_path / "r.csv").read_text().splitlines()[1].endswith(",NIGERIA,KANO,NIGERIA:KANO,NW_NGA")
