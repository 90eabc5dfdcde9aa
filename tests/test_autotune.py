"""The grid-size autotuner (autotune.py): its choice rule and cache on the
CPU with a stand-in handle; on the GPU, a tuned batch of replicates ends
bit-exact with an untuned one (grid sizes change the time, not the results)."""

import numpy as np
import pytest

from laser_polio_gb300 import _abi
from laser_polio_gb300 import autotune


def test_choice_prefers_the_default_within_the_margin():
    assert autotune.choose({304: [10.0, 10.2], 608: [9.9, 10.0]}, default=304, margin=0.03) == 304
    assert autotune.choose({304: [10.0, 10.2], 608: [8.0, 8.1]}, default=304, margin=0.03) == 608
    assert autotune.choose({304: [], 608: [5.0]}, default=304) == 608
    assert autotune.choose({}, default=152) == 152


def test_candidates_hold_the_default_and_respect_the_limit():
    c = autotune.candidates(152, 1216, (1, 2, 8), 1024)
    assert c == sorted(set(c)) and 1216 in c and max(x for x in c if x != 1216) <= 1024 and 152 in c
    assert autotune.candidates(152, 304, (1, 2, 4), None) == [152, 304]


def test_keys_round_to_powers_of_two():
    a = autotune.workload_key("GB300", 152, 64, 10000, 4.0e8)
    b = autotune.workload_key("GB300", 152, 64, 11000, 4.3e8)
    assert a == b and a != autotune.workload_key("GB300", 152, 1, 10000, 4.0e8)


class _Handle:
    """Stand-in: kernel times fall with the grid size up to 4 x SMs."""

    def __init__(self):
        self.grid = {i: 1216 for i, _, _ in _abi.LAUNCH.values()}
        self.prof = {}
        self.steps = 0

    def get_launch(self, which):
        return self.grid[which]

    def set_launch(self, which, blocks):
        self.grid[which] = blocks

    def set_profiling(self, on):
        pass

    def profile(self):
        return {k: tuple(v) for k, v in self.prof.items()}

    def step(self, n):
        self.steps += n
        for name, (idx, _, entries) in _abi.LAUNCH.items():
            g = self.grid[idx]
            ms = 0.01 + abs(g - 608) * 1e-5  # fastest at 608 CTAs
            for e in entries:
                t, c = self.prof.get(e, (0.0, 0))
                self.prof[e] = [t + ms, c + 1]

    def sync(self):
        pass


def test_tune_measures_applies_and_caches(tmp_path):
    path = tmp_path / "cache.json"
    h = _Handle()
    chosen, stepped = autotune.tune(h, "k1", 152, rounds=2, path=path)
    assert stepped == h.steps == 2 * 4
    assert chosen["rounds"] == 608 and chosen["due"] == 608
    # the cooperative round-0 kernel is never tried above its default (all of its CTAs must be resident)
    assert chosen["select"] == 304
    assert h.grid[_abi.LAUNCH["rounds"][0]] == 608
    h2 = _Handle()
    again, stepped2 = autotune.tune(h2, "k1", 152, path=path)
    assert again == chosen and stepped2 == 0 and h2.steps == 0
    assert h2.grid[_abi.LAUNCH["rounds"][0]] == 608


@pytest.mark.gpu
def test_gpu_tuned_batch_equals_untuned(tmp_path, monkeypatch):
    from laser_polio_gb300 import engine
    from laser_polio_gb300 import synthetic

    monkeypatch.setenv("LPG_AUTOTUNE_CACHE", str(tmp_path / "cache.json"))

    def sims():
        return [synthetic.zamfara_like(n_agents=60_000, dur=80, seed=5),
                synthetic.nigeria_like(n_agents=120_000, n_nodes=30, dur=90, seed=6)]

    a, b = sims(), sims()
    assert engine.run_replicates(a) == [None, None]
    assert engine.run_replicates(b, autotune=True) == [None, None]
    assert (tmp_path / "cache.json").exists()
    for x, y in zip(a, b):
        assert (x.t, x.people.count, x.should_stop) == (y.t, y.people.count, y.should_stop)
        for name in ("S", "E", "I", "R", "new_exposed", "births", "deaths", "ri_vaccinated", "sia_vaccinated"):
            np.testing.assert_array_equal(getattr(x.results, name), getattr(y.results, name), err_msg=name)
        for col in ("disease_state", "strain", "date_of_death", "ri_timer"):
            np.testing.assert_array_equal(np.asarray(getattr(x.people, col)), np.asarray(getattr(y.people, col)))
