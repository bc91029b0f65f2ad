"""The batch autotuner's host logic (genpipeline_gb300/autotune.py), with stand-in trials: the
fastest candidate is chosen, the choice is cached per grid class (the multiset of grid shapes),
a candidate the library refuses is skipped, and choices persist in a JSON cache file."""
import json

from genpipeline_gb300.autotune import CANDIDATES, DEFAULT, BatchConfig, BatchTuner, grid_class, summary


def _trial_times(times):
    calls = []

    def trial(cfg):
        calls.append(cfg)
        t = times[cfg]
        if isinstance(t, Exception):
            raise t
        return t

    return trial, calls


def test_grid_class_is_the_multiset_of_shapes():
    a = grid_class([(64, 64, 64), (32, 32, 32), (64, 64, 64)])
    b = grid_class([(32, 32, 32), (64, 64, 64), (64, 64, 64)])
    assert a == b == (((32, 32, 32), 1), ((64, 64, 64), 2))
    assert grid_class([(64, 64, 64)]) != a


def test_fastest_candidate_is_chosen_once_per_class():
    times = {c: 1.0 + i for i, c in enumerate(CANDIDATES)}
    times[CANDIDATES[2]] = 0.5
    trial, calls = _trial_times(times)
    t = BatchTuner(cache_path="")
    grids = [(64, 64, 64)] * 4 + [(32, 32, 32)] * 4
    assert t.tune(grids, trial) == CANDIDATES[2]
    assert calls == list(CANDIDATES)
    assert t.tune(list(reversed(grids)), trial) == CANDIDATES[2]  # same class: cached, no new trials
    assert len(calls) == len(CANDIDATES)
    assert t.choice(grids) == CANDIDATES[2] and t.choice([(16, 16, 16)]) is None
    s = summary(t, grids)
    assert s["choice"] == CANDIDATES[2].label() and len(s["trial_seconds"]) == len(CANDIDATES)


def test_refused_candidates_are_skipped_and_all_refused_keeps_the_default():
    times = {c: RuntimeError("refused") for c in CANDIDATES}
    times[CANDIDATES[4]] = 2.0
    trial, _ = _trial_times(times)
    t = BatchTuner(cache_path="")
    assert t.tune([(24, 24, 24)], trial) == CANDIDATES[4]
    trial, _ = _trial_times({c: RuntimeError("refused") for c in CANDIDATES})
    assert t.tune([(8, 8, 8)], trial) == DEFAULT


def test_choices_persist_in_the_cache_file(tmp_path):
    path = str(tmp_path / "tune.json")
    times = {c: 1.0 for c in CANDIDATES}
    times[CANDIDATES[1]] = 0.1
    trial, _ = _trial_times(times)
    BatchTuner(cache_path=path).tune([(48, 48, 48)] * 3, trial)
    raw = json.load(open(path))
    assert list(raw["choices"].values()) == [{"fused": 1, "batch_share": 1, "batch_group": 0}]
    t2 = BatchTuner(cache_path=path)  # a new process reads the choice back
    assert t2.choice([(48, 48, 48)] * 3) == BatchConfig(1, 1, 0)


def test_labels_name_every_parameter():
    assert "graph loop" in BatchConfig(0, 0, 0).label()
    assert "extent" in BatchConfig(1, 1, 4).label() and "<= 4" in BatchConfig(1, 1, 4).label()
