"""Placement of whole scenes and stream jobs on GPUs (vedo_gb300.partition): every scene on
exactly one GPU, loads within the greedy bound, the same answer in every process."""
import numpy as np
import pytest

from vedo_gb300 import partition


def test_pack_scenes_places_every_scene_once_and_balances():
    rng = np.random.default_rng(7)
    w = list(np.exp(rng.uniform(np.log(1e3), np.log(5e4), 256)) * 5000)
    for ranks in (1, 2, 3, 4, 8):
        parts = partition.pack_scenes(w, ranks)
        flat = sorted(i for p in parts for i in p)
        assert flat == list(range(256))
        loads = partition.loads(w, parts)
        assert max(loads) <= sum(w) / ranks + max(w) + 1e-6
        if ranks > 1:
            assert max(loads) / min(loads) < 1.05          # 256 scenes: nearly even
        assert all(p == sorted(p) for p in parts)


def test_pack_scenes_is_deterministic_and_ties_go_low():
    parts = partition.pack_scenes([1.0, 1.0, 1.0, 1.0], 2)
    assert parts == [[0, 2], [1, 3]]
    assert partition.pack_scenes([5.0, 1.0, 1.0, 1.0, 1.0, 1.0], 2) == [[0], [1, 2, 3, 4, 5]]
    assert partition.pack_scenes([], 3) == [[], [], []]


def test_dispatch_stream_in_arrival_order():
    assert partition.dispatch_stream([4.0, 1.0, 1.0, 1.0, 1.0, 5.0], 2) == [0, 1, 1, 1, 1, 0]
    r = partition.dispatch_stream([1.0] * 10, 3)
    assert [r.count(k) for k in range(3)] == [4, 3, 3]


def test_bad_arguments_raise():
    with pytest.raises(ValueError):
        partition.pack_scenes([1.0], 0)
    with pytest.raises(ValueError):
        partition.dispatch_stream([float("nan")], 2)
    with pytest.raises(ValueError):
        partition.pack_scenes([-1.0], 2)
