"""irr_step_pipelined: independent steps whose host copies overlap the
neighbouring steps' reductions must give, step by step, exactly what the
sequential irr_set_nodes / irr_step / irr_get_result calls give."""
import numpy as np
import pytest

import irregular_gb300 as irr
from helpers import random_box

pytestmark = pytest.mark.gpu


def jittered(pos, L, k):
    rng = np.random.Generator(np.random.PCG64(100 + k))
    p = pos + (rng.random(pos.shape, dtype=np.float32) - 0.5) * np.float32(0.05)
    p = np.mod(p, L).astype(np.float32)
    p[p >= L] = 0.0
    return p


@pytest.mark.parametrize("exec_mode", [irr.IRR_EXEC_PARTITIONED, irr.IRR_EXEC_PLAIN])
@pytest.mark.parametrize("pinned", [True, False])
def test_pipelined_equals_sequential(built_lib, oracle_lib, exec_mode, pinned):
    torch = pytest.importorskip("torch")
    O = oracle_lib
    pos, L = random_box(65536, 32.0 / (4.0 / 3.0 * np.pi * 2.5 ** 3), 77)
    edges = O.neighbor_half_list(pos, float(L), np.float32(2.5 * 2.5))
    h = irr.Handle(exec=exec_mode)
    h.set_params(irr.moldyn_params(float(L), 2.5))
    h.set_edges(edges)
    h.set_nodes(pos, 12)
    h.init()
    steps = 5
    inputs = [jittered(pos, L, k) for k in range(steps)]
    want = []
    for p in inputs:
        h.set_nodes(p, 12)
        h.step()
        want.append(h.get_result(elm_size=12).copy())

    def buf(shape):
        if pinned:
            return torch.empty(shape, dtype=torch.float32, pin_memory=True).numpy()
        return np.empty(shape, np.float32)

    ins = []
    for p in inputs:
        b = buf(p.shape)
        b[:] = p
        ins.append(b)
    outs = [buf((pos.shape[0], 3)) for _ in range(steps)]
    for k in range(steps):
        h.step_pipelined(ins[k], outs[k], 12, 12)
    h.pipeline_sync()
    for k in range(steps):
        if exec_mode == irr.IRR_EXEC_PARTITIONED:
            assert np.array_equal(outs[k].view(np.uint32), want[k].view(np.uint32)), k
        else:  # float atomics: order-dependent last bits
            assert np.allclose(outs[k], want[k], rtol=0, atol=1e-5 * np.abs(want[k]).max())
    # a 16-byte input and a 24-byte (double) result format through the same slots
    p4 = np.zeros((pos.shape[0], 4), np.float32)
    p4[:, :3] = inputs[2]
    o24 = np.empty((pos.shape[0], 3), np.float64)
    h.step_pipelined(p4, o24, 16, 24)
    h.pipeline_sync()
    if exec_mode == irr.IRR_EXEC_PARTITIONED:
        assert np.array_equal(o24, want[2].astype(np.float64))
    # and the ordinary calls still see the last step's node data
    h.step()
    last = h.get_result(elm_size=12)
    if exec_mode == irr.IRR_EXEC_PARTITIONED:
        assert np.array_equal(last, want[2])


def test_pipelined_before_init_is_refused(built_lib):
    h = irr.Handle(exec=irr.IRR_EXEC_PARTITIONED)
    with pytest.raises(irr.IrregularError) as e:
        h.step_pipelined(np.zeros((4, 3), np.float32), np.zeros((4, 3), np.float32))
    assert e.value.status == irr.IRR_ERR_STATE


def test_pipelined_step_of_an_empty_graph(built_lib):
    pos = np.random.default_rng(1).random((100, 3)).astype(np.float32) * 10
    h = irr.Handle(exec=irr.IRR_EXEC_PARTITIONED)
    h.set_params(irr.moldyn_params(10.0, 2.5))
    h.set_edges(np.zeros((0, 2), np.int32))
    h.set_nodes(pos, 12)
    h.init()
    out = np.full((100, 3), 7.0, np.float32)
    h.step_pipelined(pos, out, 12, 12)
    h.pipeline_sync()
    assert np.all(out == 0)
