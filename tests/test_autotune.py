"""The launch-shape autotuner's host side: the coordinate-descent search on a
model of step time, the size buckets and their nearest-bucket lookup, the
JSON cache, and the knob table of the C ABI (a host-side table: setting and
reading it launches nothing, so this runs without a GPU)."""

import pytest

from getm_gb300 import autotune


def _model(opt):
    """A separable step-time model with its minimum at ``opt``."""
    def measure(t):
        return 1.0 + sum(abs(autotune.KNOBS[k][1].index(t[k]) - autotune.KNOBS[k][1].index(opt[k])) * w
                         for w, k in zip((0.3, 0.2, 0.1, 0.05, 0.02, 0.01), autotune.KNOBS))
    return measure


def test_search_finds_the_optimum_of_a_separable_model():
    opt = {"xpass_rows": 2, "ymarch_chunk": 64, "column_rows": 1, "substep_blocks_per_sm": 1, "xpass_vec": 0,
           "column_solve": 1}
    best, t, trials = autotune.search(_model(opt))
    assert best == opt and t == pytest.approx(1.0)
    # coordinate descent: one pass over the candidates of every knob, then a
    # confirming pass; every configuration is timed once
    keys = [tuple(sorted(x.items())) for x, _ in trials]
    assert len(keys) == len(set(keys)) <= 1 + 2 * sum(len(c) - 1 for _, c in autotune.KNOBS.values())
    assert trials[0][0] == autotune.DEFAULTS


def test_search_keeps_the_defaults_when_they_are_best():
    best, t, trials = autotune.search(_model(autotune.DEFAULTS), rounds=3)
    assert best == autotune.DEFAULTS
    assert all(tt >= t for _, tt in trials)


def test_buckets_and_nearest_lookup(tmp_path):
    assert autotune.bucket(400, 300, 40, "mixed") == "mixed/p17/z40"
    assert autotune.bucket(64, 64, 20, "mixed") == "mixed/p12/z20"
    assert autotune.bucket(90, 90, 24, "fp64") == "fp64/p13/z20"
    c = autotune.TileCache()
    small = {"xpass_rows": 2, "ymarch_chunk": 16, "column_rows": 1, "substep_blocks_per_sm": 0}
    big = dict(autotune.DEFAULTS, ymarch_chunk=64)
    c.store(64, 64, 20, "mixed", small, 1.0, 1.2)
    c.store(400, 300, 40, "mixed", big, 4.0, 4.1)
    assert c.lookup(64, 64, 20, "mixed") == small
    assert c.lookup(70, 70, 22, "mixed") == small      # nearest bucket
    assert c.lookup(390, 310, 38, "mixed") == big
    assert c.lookup(64, 64, 20, "fp64") == autotune.DEFAULTS  # no bucket of that precision
    path = tmp_path / "tiles.json"
    c.save(path)
    d = autotune.TileCache.load(path)
    assert d.entries == c.entries
    assert autotune.lookup(64, 64, 20, "mixed", path=path) == small


def test_committed_cache_is_well_formed():
    c = autotune.TileCache.load()
    for key, e in c.entries.items():
        autotune._parse(key)
        assert set(e["tiles"]) <= set(autotune.KNOBS)
        for k, v in e["tiles"].items():
            assert v in autotune.KNOBS[k][1]


def test_knob_table_of_the_c_abi():
    from getm_gb300._lib import GetmError, call

    autotune.apply({"xpass_rows": 4, "column_rows": 2})
    assert autotune.current() == dict(autotune.DEFAULTS, xpass_rows=4, column_rows=2)
    autotune.apply(None)
    assert autotune.current() == autotune.DEFAULTS
    with pytest.raises(GetmError):
        call("getm_tune_set", autotune.KNOBS["ymarch_chunk"][0], 17)
    with pytest.raises(GetmError):
        call("getm_tune_set", 99, 1)
    with pytest.raises(KeyError):
        autotune.apply({"no_such_knob": 1})
    assert autotune.current() == autotune.DEFAULTS


def test_refining_one_knob_from_cached_shapes():
    """A knob added later is searched alone, starting from a bucket's cached
    shapes (``python -m getm_gb300.autotune --knobs column_solve --refine``);
    knobs that only the mixed form's kernels read are not searched for FP64."""
    cached = dict(autotune.DEFAULTS, xpass_rows=2, ymarch_chunk=64)
    opt = dict(cached, column_solve=1, column_rows=1)
    best, t, trials = autotune.search(_model(opt), knobs={"column_solve": autotune.KNOBS["column_solve"]},
                                      start=cached)
    assert best == dict(cached, column_solve=1)
    assert {k for x, _ in trials for k in x if x[k] != cached[k]} == {"column_solve"}
    assert not autotune._applies("fp64", ["column_solve"])
    assert autotune._applies("fp64", ["column_solve", "xpass_rows"]) and autotune._applies("mixed", ["column_solve"])
