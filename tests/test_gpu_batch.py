"""GPU tests of the batched form: every instance of a batch (uneven sizes, uneven step counts)
must produce exactly the fields and probe series of its serial run, for the autotuned and for
fixed (block size, depth) configurations, across consecutive runs."""
import numpy as np
import pytest

from openems_gb300 import configs
from openems_gb300.batch import BatchEngine
from openems_gb300.engine import Engine_CUDA

from helpers import bits_equal

pytestmark = pytest.mark.gpu


def _instances(n=6, seed0=77):
    out = []
    for k in range(n):
        op, _ = configs.batch_instance(seed0 + k, size_range=(14, 30), steps_range=(60, 200), pml=4)
        steps = 240 + 23 * k         # uneven, some equal to exercise chunking
        out.append((op, steps if k != 3 else 240))
    return out


def _check(serial, batched):
    for a, b in zip(serial, batched):
        for w in (0, 1):
            assert bits_equal(a.read_field(w), b.read_field(w))
        for pid in a.vprobe_ids + a.iprobe_ids:
            assert np.array_equal(a.probe_series(pid), b.probe_series(pid), equal_nan=True)
        assert a.GetNumberOfTimesteps() == b.GetNumberOfTimesteps()


@pytest.mark.parametrize("block,depth", [(0, 0), (256, 1), (128, 4), (512, 2), (256, 0x80000001), (128, 0x80000002), (256, 0xC0000001), (512, 0xC0000002),
                                         (256, 0x20000001), (256, 0x10000001)])
def test_batch_equals_serial(cuda_lib, block, depth):
    inst = _instances()
    total = [2 * s for _, s in inst]
    serial = [Engine_CUDA(op, t) for (op, _), t in zip(inst, total)]
    batched = [Engine_CUDA(op, t) for (op, _), t in zip(inst, total)]
    be = BatchEngine(batched)
    for rnd in range(2):                       # two consecutive runs continue the same state
        for e, (_, s) in zip(serial, inst):
            e.IterateTS(s)
        be.run([s for _, s in inst], block, depth)
        _check(serial, batched)
    cfg = be.config()
    assert cfg["block_size"] in (128, 256, 512)
    if block == 0:
        assert len(cfg["tune_ms"]) == 13 and min(cfg["tune_ms"]) > 0
    be.close()
