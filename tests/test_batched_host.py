"""Host logic of the ragged batch graph (ctlib_gb300/batched.py) that needs no
GPU: how slices are spread over the parallel graph branches."""

import pytest

from ctlib_gb300.batched import assign_branches


def test_every_slice_once():
    work = [5, 1, 9, 3, 3, 7, 2]
    lanes = assign_branches(work, 3)
    assert sorted(i for lane in lanes for i in lane) == list(range(len(work)))


def test_longest_first_to_least_loaded():
    lanes = assign_branches([10, 1, 1, 8], 2)
    assert lanes == [[0], [3, 1, 2]]  # 10 | 8 + 1 + 1
    loads = [sum([10, 1, 1, 8][i] for i in lane) for lane in lanes]
    assert loads == [10, 10]


def test_more_branches_than_slices():
    lanes = assign_branches([4, 2], 4)
    assert lanes == [[0], [1], [], []]


def test_bad_branch_count():
    with pytest.raises(ValueError):
        assign_branches([1, 2], 0)
