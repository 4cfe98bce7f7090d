"""The autotuner's search on the CPU, with the timing of a step replaced by a
table: it walks the axes one at a time, keeps the fastest value of each with
the best of the others, and skips an axis that changes nothing under the
settings found so far (sort_threads with counted key-sort passes)."""
import pytest

from torpedo_gb300 import autotune


def _tune(cost, axes=autotune.AXES, base=None, monkeypatch=None):
    tried = []

    def fake_time(make_engine, enqueue, stream, settings, frames, warmup):
        tried.append(dict(settings))
        return cost(settings)

    monkeypatch.setattr(autotune, "time_steps", fake_time)
    best, results = autotune.tune(None, None, None, axes=axes, base=base)
    return best, results, tried


def test_keeps_the_fastest_value_of_each_axis(monkeypatch):
    # counted passes fastest; 512-thread depth passes and 8 keys per thread faster
    def cost(s):
        return (1.0 + 0.2 * s["key_sort_lookback"] - 0.05 * (s["depth_sort_threads"] == 512)
                - 0.03 * (s["depth_sort_items"] == 8) + 0.1 * (s["sort_ctas_per_sm"] == 2))

    best, results, tried = _tune(cost, monkeypatch=monkeypatch)
    assert best == {"key_sort_lookback": 0, "sort_threads": 256, "depth_sort_threads": 512,
                    "depth_sort_items": 8, "sort_ctas_per_sm": 0}
    # sort_threads is inert with counted passes: never tried at 512
    assert all(t["sort_threads"] == 256 for t in tried)
    assert len(results) == len(tried)


def test_sort_threads_tried_with_lookback_passes(monkeypatch):
    def cost(s):
        return 1.0 - 0.2 * s["key_sort_lookback"] - 0.1 * (s["sort_threads"] == 512)

    best, _, tried = _tune(cost, monkeypatch=monkeypatch)
    assert best["key_sort_lookback"] == 1 and best["sort_threads"] == 512
    assert any(t["sort_threads"] == 512 for t in tried)


def test_training_axes_keep_the_base_settings(monkeypatch):
    base = {"key_sort_lookback": 0, "sort_ctas_per_sm": 0}

    def cost(s):
        assert {k: s[k] for k in base} == base
        return 1.0 - 0.1 * (s["blend_round"] == 256) - 0.2 * (s["blend_backward_round"] == 32)

    best, _, _ = _tune(cost, axes=autotune.TRAIN_AXES, base=base, monkeypatch=monkeypatch)
    assert best["blend_round"] == 256 and best["blend_backward_round"] == 32 and best["blend_persistent"] == 0
    assert {k: best[k] for k in base} == base


@pytest.mark.parametrize("name,values", autotune.AXES + autotune.TRAIN_AXES)
def test_every_axis_is_an_engine_setting(name, values):
    from torpedo_gb300 import _lib as L

    fields = {f for f, _ in L.Settings._fields_}
    assert name in fields and len(values) >= 2
