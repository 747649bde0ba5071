"""The device-side time-out path (GPU), without a fault: a step whose waits all
run out is reported on the host and leaves the handle usable.

irr_set_wait_limit(h, limit, withhold_once=1) makes the next step's producers
publish no work, so every consumer's bounded mbarrier wait gives up after the
limit (here 2 ms) and the kernel ends with nothing in flight; the next
synchronising call returns IRR_ERR_DEVICE.  Nothing traps, faults or hangs:
the launch lasts about twice the limit.
"""
import numpy as np
import pytest

from helpers import load_golden

pytestmark = pytest.mark.gpu


def make(irr, c, **cfg):
    h = irr.Handle(irr.default_config(map_idx=irr.IRR_MAP_LJ_MOLDYN,
                                      exec=irr.IRR_EXEC_PARTITIONED, **cfg))
    h.set_params(irr.moldyn_params(float(c["side"]), float(c["cutoff"])))
    h.set_edges(c["edges"])
    h.set_nodes(c["pos"], 24)
    h.init()
    return h


def test_wait_time_out_is_reported_and_recovers(built_lib):
    import irregular_gb300 as irr
    c = load_golden("moldyn_random_2048")
    ref = make(irr, c)
    ref.step()
    expect = ref.get_result(elm_size=12)
    ref.close()

    h = make(irr, c)
    h.set_wait_limit(2000, withhold_once=True)
    h.step()
    with pytest.raises(irr.IrregularError) as ei:
        h.sync()
    assert ei.value.status == irr.IRR_ERR_DEVICE
    # the status was consumed by that report: the next step is normal
    h.step()
    got = h.get_result(elm_size=12)
    assert np.array_equal(got.view(np.uint32), expect.view(np.uint32))
    h.set_wait_limit(0)
    h.step()
    h.sync()
    h.close()


def test_wait_limit_config_field(built_lib):
    """irr_config.wait_limit_us sets the same limit at creation; a negative
    value is rejected."""
    import irregular_gb300 as irr
    c = load_golden("moldyn_random_2048")
    h = make(irr, c, wait_limit_us=5000)
    h.step()
    h.sync()
    h.set_wait_limit(5000, withhold_once=True)
    h.step()
    with pytest.raises(irr.IrregularError) as ei:
        h.get_result(elm_size=12)
    assert ei.value.status == irr.IRR_ERR_DEVICE
    h.close()
    with pytest.raises(irr.IrregularError):
        irr.Handle(irr.default_config(wait_limit_us=-1))
