"""The chunk plan of the host-buffer filter call (sep_filter_chunk_plan, the
function sep_filter itself uses): chunks of at most max_pairs pairs; with host
buffers the last chunk splits off a tail so that its output copy is the only
one not overlapped with a filter.  No counterpart in the reference (its
filter.x keeps every state in host memory)."""
import pytest

import semi_empirical_pseudopotentials_gb300 as sep


def test_device_buffers_take_chunks_of_max_pairs():
    assert sep.filter_chunk_plan(32, 64, host_buffers=False) == [32]
    assert sep.filter_chunk_plan(70, 32, host_buffers=False) == [32, 32, 6]


def test_first_host_call_halves_the_last_chunk():
    assert sep.filter_chunk_plan(32, 64) == [16, 8, 4, 4]
    assert sep.filter_chunk_plan(7, 64) == [7]
    assert sep.filter_chunk_plan(11, 64) == [6, 5]


@pytest.mark.parametrize("ratio,plan", [(0.0, [28, 4]), (0.06, [28, 4]), (0.25, [25, 7]),
                                        (1.0, [16, 16]), (5.0, [16, 16])])
def test_measured_ratio_sets_the_tail(ratio, plan):
    """The smallest tail t >= 4 whose filter covers the copy of the rest,
    ratio (32 - t) <= t, at most half the chunk."""
    assert sep.filter_chunk_plan(32, 64, copy_ratio=ratio) == plan
    head, tail = plan
    assert tail >= 4 and (ratio * head <= tail or tail == 16)


def test_memory_limited_chunks_split_only_the_last():
    assert sep.filter_chunk_plan(80, 32, copy_ratio=0.06) == [32, 32, 12, 4]
    assert sep.filter_chunk_plan(80, 32) == [32, 32, 8, 4, 4]
    assert sum(sep.filter_chunk_plan(1000, 33, copy_ratio=0.3)) == 1000


def test_bad_arguments_are_refused():
    with pytest.raises(sep.SepError):
        sep.filter_chunk_plan(0, 32)
    with pytest.raises(sep.SepError):
        sep.filter_chunk_plan(32, 0)
