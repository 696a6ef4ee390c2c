"""The autotuner's search and cache logic (turns2d_urans_git_gb300/tune.py),
with a fake timing function in place of the GPU.  No GPU."""
import json

from turns2d_urans_git_gb300 import tune
from turns2d_urans_git_gb300.abi import OT2D_FP32_MIXED, OT2D_FP64


def _fake(costs, calls):
    def for_class(jmax, kmax):
        def measure(c):
            calls.append(((jmax, kmax), c))
            return costs(jmax, kmax, c)
        return measure
    return for_class


def test_search_takes_the_fastest_median_and_keeps_order_on_ties():
    seq = iter([5.0, 1.0, 9.0, 2.0, 2.0, 2.0, 2.0, 2.0, 2.0])   # medians: a 5, b 2, c 2
    best, times = tune.search(["a", "b", "c"], lambda c: next(seq))
    assert best == "b" and times == {"a": 5.0, "b": 2.0, "c": 2.0}


def test_tune_searches_each_class_once_then_reads_the_cache(tmp_path):
    path = str(tmp_path / "t.json")
    classes = ((129, 33), (513, 129))
    # a class prefers the wide tile for wide meshes, group 8, no lag
    def costs(jmax, kmax, c):
        shape, group, lag, pipe = c
        return (1.0 + (0.0 if shape == (1 if jmax > 300 else 0) else 0.5) + (0.0 if group == 8 else 0.1) + 0.01 * lag
                + (0.0 if pipe == (1 if jmax > 300 else 0) else 0.05))
    calls = []
    ch, timings = tune.tune(_fake(costs, calls), classes, "GB300", OT2D_FP32_MIXED, cache_path=path)
    assert ch == {(129, 33): (0, 8, 0, 0), (513, 129): (1, 8, 0, 1)}
    assert len(calls) == 2 * 3 * len(tune.CANDIDATES)
    assert all(v is not None for v in timings.values())
    cache = json.load(open(path))
    assert set(cache) == {"GB300|fp32-mixed|129x33", "GB300|fp32-mixed|513x129"}
    # second call: from the cache, no measurement
    calls.clear()
    ch2, timings2 = tune.tune(_fake(costs, calls), classes, "GB300", OT2D_FP32_MIXED, cache_path=path)
    assert ch2 == ch and not calls and all(v is None for v in timings2.values())
    # another precision or GPU is another key; retune measures again
    tune.tune(_fake(costs, calls), classes[:1], "GB300", OT2D_FP64, cache_path=path)
    assert len(calls) == 3 * len(tune.CANDIDATES)
    calls.clear()
    tune.tune(_fake(costs, calls), classes[:1], "GB300", OT2D_FP32_MIXED, cache_path=path, retune=True)
    assert len(calls) == 3 * len(tune.CANDIDATES)
    assert len(json.load(open(path))) == 3


def test_a_corrupt_or_foreign_cache_is_searched_again(tmp_path):
    path = tmp_path / "t.json"
    path.write_text("{not json")
    calls = []
    ch, _ = tune.tune(_fake(lambda j, k, c: float(sum(c)), calls), ((129, 33),), "G", OT2D_FP64, cache_path=str(path))
    assert ch[(129, 33)] == (0, 4, 0, 0) and calls
    # a cached choice outside the candidate set is not trusted
    cache = json.load(open(path))
    cache["G|fp64|129x33"]["choice"] = [7, 3, 99, 0]
    path.write_text(json.dumps(cache))
    calls.clear()
    ch, _ = tune.tune(_fake(lambda j, k, c: float(sum(c)), calls), ((129, 33),), "G", OT2D_FP64, cache_path=str(path))
    assert ch[(129, 33)] == (0, 4, 0, 0) and calls


def test_tuning_table_is_ordered_by_class_and_bounds_array_sizes():
    t = tune.tuning_table({(513, 129): (1, 8, 4, 1), (129, 33): (2, 4, 0, 0), (257, 65): (0, 8, 0, 1)})
    rows = [(e.kd_max, e.jd_max, e.rt_shape, e.lu_group, e.lu_lag, e.pipeline) for e in t]
    assert rows == [(34, 130, 2, 4, 0, 0), (66, 258, 0, 8, 0, 1), (130, 514, 1, 8, 4, 1)]
    assert tune.describe({(129, 33): (2, 4, 0, 1)}) == {"129x33": {"rt_tile": "8x32", "lu_group": 4, "lu_lag": 0,
                                                                   "pipeline": 1}}


def test_the_batch_of_a_search_is_part_of_its_key(tmp_path):
    """Searches at two batch sizes are cached apart; the batch comes from the
    measuring function or is given."""
    path = str(tmp_path / "t.json")
    calls = []
    m = _fake(lambda j, k, c: 1.0 + c[3], calls)
    m.batch = 16
    ch16, _ = tune.tune(m, ((513, 129),), "G", OT2D_FP32_MIXED, cache_path=path)
    m64 = _fake(lambda j, k, c: 1.0 + abs(c[3] - 1), calls)
    ch64, _ = tune.tune(m64, ((513, 129),), "G", OT2D_FP32_MIXED, cache_path=path, batch=64)
    assert ch16[(513, 129)][3] == 0 and ch64[(513, 129)][3] == 1
    assert set(json.load(open(path))) == {"G|fp32-mixed|513x129|b16", "G|fp32-mixed|513x129|b64"}
    calls.clear()
    again, t = tune.tune(None, ((513, 129),), "G", OT2D_FP32_MIXED, cache_path=path, batch=64)
    assert again == ch64 and t[(513, 129)] is None and not calls
