"""The batch autotuner's host logic, no GPU: class keys bucket particle counts by
powers of two, untuned lookups return the defaults, a tuned choice is the
fastest candidate, persists in the JSON cache and is reused after a reload
without timing again.  The device name and the timed deposit are stubbed."""
import json

import pytest

import pylians_gb300.autotune as at


@pytest.fixture
def tuner(tmp_path, monkeypatch):
    path = tmp_path / 'cache' / 'autotune.json'
    monkeypatch.setenv('PYL_AUTOTUNE_CACHE', str(path))
    monkeypatch.setattr(at, '_cache', None)
    monkeypatch.setattr(at, '_device_key', lambda: 'GB300_stub')
    timed = []

    def fake_time(dims, n, MAS, interlaced, item, ctas, reps=3, method='atomic'):
        timed.append((item, ctas, method))
        # fastest: the second item candidate, and 8 CTAs per SM
        return abs(item - at.ITEM_CANDIDATES[1]) + abs(ctas - 8)

    monkeypatch.setattr(at, '_time_deposit', fake_time)
    return at, path, timed


def test_class_keys_bucket_by_power_of_two(monkeypatch):
    monkeypatch.setattr(at, '_device_key', lambda: 'dev')
    assert at.class_key(128, 1, 'CIC', False) == 'dev/atomic/128/1024/CIC/0'
    assert at.class_key(128, 1024, 'CIC', False) == 'dev/atomic/128/1024/CIC/0'
    assert at.class_key(128, 1025, 'CIC', True) == 'dev/atomic/128/2048/CIC/1'
    assert at.class_key(256, 1 << 20, 'TSC', True, 'tiled') == 'dev/tiled/256/1048576/TSC/1'


def test_untuned_lookups_return_defaults(tuner):
    at_, path, timed = tuner
    assert at_.item_size(128, 10 ** 6, 'CIC', True, tune=False) == at_.DEFAULT_ITEM
    assert at_.ctas_per_sm(tune=False) == at_.DEFAULT_CTAS
    assert not timed and not path.exists()


def test_tuned_choice_persists_and_is_reused(tuner):
    at_, path, timed = tuner
    assert at_.item_size(128, 10 ** 6, 'CIC', True) == at_.ITEM_CANDIDATES[1]
    assert sorted(t[0] for t in timed) == sorted(at_.ITEM_CANDIDATES)
    assert at_.ctas_per_sm() == 8
    saved = json.loads(path.read_text())
    assert saved['GB300_stub/atomic/128/1048576/CIC/1'] == at_.ITEM_CANDIDATES[1]
    assert saved['GB300_stub/atomic/ctas_per_sm'] == 8
    at_._cache = None                                   # a new process: read back from disk
    timed.clear()
    assert at_.item_size(128, 10 ** 6 + 7, 'CIC', True) == at_.ITEM_CANDIDATES[1]    # same bucket
    assert at_.ctas_per_sm() == 8
    assert not timed


def test_unreadable_cache_starts_empty(tuner):
    at_, path, timed = tuner
    path.parent.mkdir(parents=True)
    path.write_text('{not json')
    assert at_.item_size(64, 5000, 'PCS', False, tune=False) == at_.DEFAULT_ITEM
    assert at_._cache == {}
