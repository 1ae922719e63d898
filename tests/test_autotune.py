"""The autotuner's search and the build's use of its result (CPU only: no
kernel is compiled or timed here)."""
import json

from msplat_gb300 import _build, autotune


def test_coordinate_descent_finds_the_separable_minimum():
    space = {"a": [1, 2, 3], "b": [8, 12, 16], "c": [0, 1]}
    target = {"a": 3, "b": 8, "c": 1}
    calls = []

    def f(s):
        calls.append(dict(s))
        return sum((s[k] - target[k]) ** 2 for k in s)

    best, v, seen = autotune.coordinate_descent(space, {"a": 1, "b": 12, "c": 0}, f, rounds=3)
    assert best == target and v == 0
    assert len(calls) == len(seen)  # every setting evaluated once


def test_defaults_are_in_the_space():
    for k, v in autotune.DEFAULTS.items():
        assert v in autotune.SPACE[k]


def test_build_reads_the_tuning_file(tmp_path):
    p = tmp_path / "tuning.json"
    p.write_text(json.dumps({"defines": {"MSPLAT_FEW_LANES": 16, "MSPLAT_SORT_ITEMS": 8}}))
    d = _build.tuned_defines(str(p))
    assert d == {"MSPLAT_FEW_LANES": 16, "MSPLAT_SORT_ITEMS": 8}
    assert _build.define_flags(d) == ["-DMSPLAT_FEW_LANES=16", "-DMSPLAT_SORT_ITEMS=8"]
    assert _build.tuned_defines(str(tmp_path / "absent.json")) == {}
