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


def test_settings_that_do_not_build_score_infinity():
    logs = []

    def build(setting):
        if setting["b"] == 16:
            raise RuntimeError("nvcc failed for alpha_blending.cu:\nstatic assertion failed")
        return f"lib-{setting['a']}-{setting['b']}"

    def time_lib(lib):
        a, b = (int(x) for x in lib.split("-")[1:])
        return abs(a - 2) + abs(b - 16) * 0.1

    objective = autotune.make_objective(build, time_lib, log=logs.append)
    assert objective({"a": 2, "b": 16}) == float("inf")
    best, v, seen = autotune.coordinate_descent({"a": [1, 2, 3], "b": [8, 12, 16]}, {"a": 1, "b": 8},
                                                objective, rounds=2)
    assert best == {"a": 2, "b": 12} and abs(v - 0.4) < 1e-12
    assert any("does not build" in m for m in logs)


def test_every_space_value_builds_a_distinct_define_set():
    for name, values in autotune.SPACE.items():
        flags = {tuple(_build.define_flags(dict(autotune.DEFAULTS, **{name: v}))) for v in values}
        assert len(flags) == len(values), name


def test_each_workload_keeps_its_own_section(tmp_path):
    """Tuning the batch workload stores its choice beside the frame's, and the
    build applies both (the multi-camera grid's macros are its own)."""
    p = str(tmp_path / "tuning.json")
    autotune.write_tuning(p, "frame", {"MSPLAT_FEW_LANES": 16}, 1.9, {"gaussians": 1, "width": 2, "height": 3}, [])
    autotune.write_tuning(p, "batch", {"MSPLAT_BATCH_BLEND_GATHER_FWD": 2}, 80.0,
                          {"gaussians": 1, "width": 2, "height": 3, "cameras": 16}, [])
    autotune.write_tuning(p, "frame", {"MSPLAT_FEW_LANES": 12}, 1.8, {"gaussians": 1, "width": 2, "height": 3}, [])
    data = json.load(open(p))
    assert data["defines"] == {"MSPLAT_FEW_LANES": 12}
    assert data["workloads"]["batch"]["defines"] == {"MSPLAT_BATCH_BLEND_GATHER_FWD": 2}
    assert _build.tuned_defines(p) == {"MSPLAT_FEW_LANES": 12, "MSPLAT_BATCH_BLEND_GATHER_FWD": 2}
    assert not set(autotune.SPACE) & set(autotune.BATCH_SPACE)
    for k, v in autotune.BATCH_DEFAULTS.items():
        assert v in autotune.BATCH_SPACE[k]


def test_searches_keep_earlier_evaluations(tmp_path):
    """A search of a few parameters adds to the settings earlier searches
    timed; a setting timed again keeps its new time."""
    p = str(tmp_path / "tuning.json")
    shape = {"gaussians": 1, "width": 2, "height": 3}
    autotune.write_tuning(p, "frame", {"MSPLAT_FEW_LANES": 16}, 1.9, shape,
                          [{"defines": {"MSPLAT_FEW_LANES": 16}, "ms": 1.9},
                           {"defines": {"MSPLAT_FEW_LANES": 12}, "ms": 2.0}])
    autotune.write_tuning(p, "frame", {"MSPLAT_FEW_LANES": 16}, 1.85, shape,
                          [{"defines": {"MSPLAT_FEW_LANES": 16}, "ms": 1.85},
                           {"defines": {"MSPLAT_FEW_LANES": 8}, "ms": 2.1}])
    ev = {e["defines"]["MSPLAT_FEW_LANES"]: e["ms"] for e in json.load(open(p))["evaluated"]}
    assert ev == {12: 2.0, 16: 1.85, 8: 2.1}
