"""Batched stepping: each member of a batch ends bit-identical to the same
channel stepped alone (the batch graph holds the members' own kernels and
deterministic reductions; co-scheduling changes nothing), for FP64 and the
FP32-mixed form, on uneven grids including an odd ny."""
import numpy as np
import pytest

from tpls_gb300.api import STATE_FIELDS
from tpls_gb300.batch import Batch, Instance, draw_instances, open_instance



def _instances():
    return [Instance(0, 64, 32, 32, 2.0, 1.0, 100.0, 0.05, 11), Instance(1, 32, 19, 48, 7.5, 3.0, 300.0, 0.08, 12),
            Instance(2, 96, 32, 16, 1.3, 5.0, 60.0, 0.02, 13)]


@pytest.mark.gpu
@pytest.mark.parametrize("precision", [0, 1])
def test_batch_members_match_solo_runs(precision):
    insts = _instances()
    solo = []
    for inst in insts:
        g = open_instance(inst, precision)
        assert g.step(5) == 0
        solo.append(g.get_state())
        g.close()
    members = [open_instance(i, precision) for i in insts]
    b = Batch(members)
    assert b.step(2) == 0
    b.step_async(3)
    assert b.step(0) == 0
    for g, ref in zip(members, solo):
        st = g.get_state()
        for k in STATE_FIELDS:
            assert np.array_equal(st[k], ref[k]), k
        assert g.stats()["steps_done"] == 5
    b.close()
    for g in members:
        g.close()


@pytest.mark.gpu
def test_multi_instance_sweeps_match_solo_runs():
    """The batch with its members' FP32 momentum sweeps as multi-instance
    launches (one persistent launch per sweep over every member's tiles):
    each member ends bit-identical to the same channel stepped alone, on
    uneven grids (nx = 33 leaves ragged four-point groups)."""
    insts = [Instance(0, 64, 32, 32, 2.0, 1.0, 100.0, 0.05, 11), Instance(1, 33, 18, 40, 7.5, 3.0, 300.0, 0.08, 12),
             Instance(2, 96, 32, 16, 1.3, 5.0, 60.0, 0.02, 13), Instance(3, 128, 64, 48, 4.0, 2.0, 200.0, 0.06, 14)]
    solo = []
    for inst in insts:
        g = open_instance(inst, 1)
        assert g.step(5) == 0
        solo.append(g.get_state())
        g.close()
    members = [open_instance(i, 1) for i in insts]
    b = Batch(members, multi_sweeps=True)
    assert b.step(2) == 0
    b.step_async(3)
    assert b.step(0) == 0
    for g, ref in zip(members, solo):
        st = g.get_state()
        for k in STATE_FIELDS:
            assert np.array_equal(st[k], ref[k]), k
    b.close()
    for g in members:
        g.close()


@pytest.mark.gpu
def test_multi_instance_sweeps_refuse_ineligible_members():
    """FP64 members, or an odd ny (whose ghost rows need separate exchanges),
    are refused with TPLS_ERR_ARG; the batch then steps as before."""
    from tpls_gb300.api import TplsError
    a = open_instance(_instances()[0], 0)
    with pytest.raises(TplsError):
        Batch([a], multi_sweeps=True)
    c = open_instance(_instances()[1], 1)  # ny = 19
    with pytest.raises(TplsError):
        Batch([c], multi_sweeps=True)
    a.close()
    c.close()


@pytest.mark.gpu
def test_batch_rejects_misaligned_members():
    insts = _instances()[:2]
    a, c = open_instance(insts[0], 1), open_instance(insts[1], 1)
    a.step(1)
    b = Batch([a, c])
    with pytest.raises(Exception):
        b.step(1)
    b.close()
    a.close()
    c.close()


def test_draw_instances_is_seeded_and_in_range():
    a, b = draw_instances(48), draw_instances(48)
    assert [x.__dict__ for x in a] == [x.__dict__ for x in b]
    for x in a:
        assert x.nx in range(64, 257, 32) and x.ny in range(32, 129, 32) and x.nz in range(32, 129, 16)
        assert 1.0 <= x.m <= 20.0 and 50.0 <= x.re <= 500.0 and 0.01 <= x.amp <= 0.1


@pytest.mark.gpu
@pytest.mark.parametrize("precision", [0, 1])
def test_autotuned_tiles_keep_results(precision):
    """The tuner only picks among block shapes with the same per-point
    arithmetic: a tuned context ends bit-identical to an untuned one."""
    inst = _instances()[0]
    a = open_instance(inst, precision)
    b = open_instance(inst, precision, tune=True)
    tiles = b.autotune(reps=3)
    assert set(tiles) == {"jacobi", "sor_even", "sor_odd"}
    b.set_state(a.get_state())
    assert a.step(4) == 0 and b.step(4) == 0
    sa, sb = a.get_state(), b.get_state()
    for k in STATE_FIELDS:
        assert np.array_equal(sa[k], sb[k]), k
    a.close()
    b.close()
