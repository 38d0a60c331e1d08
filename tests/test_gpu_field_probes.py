"""GPU: E/H field probes (probe types 2/3, ProcessFieldProbe) against the oracle, bit for bit,
and the reference's own contract (TESTSUITE/probes/fieldprobes.m) on the engine's outputs: each
probe's samples equal the time-domain dump without interpolation at its node, as written to VTK
files by the dump pipeline, within the test's 1e-7 relative bound (float dump, double probe).
"""
import os

import numpy as np
import pytest

from openems_gb300 import configs
from openems_gb300.engine import Engine_CUDA
from openems_gb300.vtkio import read_vtr
from oracle.oracle import OracleEngine

from helpers import compare_engines

pytestmark = pytest.mark.gpu

STEPS = 600


@pytest.mark.parametrize("chunks", [(1, 7, 16, 33), (16,)])
def test_field_probes_bit_exact_and_equal_to_dumps(cuda_lib, tmp_path, chunks):
    op = configs.fieldprobes(steps=STEPS, freqs=(4e8, 7e8))
    g = Engine_CUDA(op, STEPS, dump_path=str(tmp_path))
    done, k = 0, 0
    while done < STEPS:
        n = min(chunks[k % len(chunks)], STEPS - done)
        g.IterateTS(n)
        done += n
        k += 1
    g.flush_dumps()
    r = OracleEngine(op, STEPS)
    r.IterateTS(STEPS)
    res = compare_engines(g, r, check_dumps=False)
    assert all(res.values()), [k for k, v in res.items() if not v]
    assert len(g.fprobe_ids) == 12
    faces = ["xn", "xp", "yn", "yp", "zn", "zp"]
    for j, (pid, p) in enumerate(zip(g.fprobe_ids, op.fprobes)):
        pre = "Et_" if p.field == 0 else "Ht_"
        d = next(d for d in op.td_dumps if d.name == pre + faces[j % 6])
        i = [int(p.pos[a]) - int(d.start[a]) for a in range(3)]
        s = g.probe_series(pid)
        ok = np.nonzero(~np.isnan(s[:, 0]))[0]
        assert ok.size == STEPS // p.interval + 1
        for slot in ok:
            ts = int(slot) * p.interval
            _, _, field = read_vtr(os.path.join(str(tmp_path), f"{d.name}_{ts:08d}.vtr"))
            dump = field[:, i[0], i[1], i[2]].astype(np.float64)
            assert np.all(np.abs(dump - s[slot]) <= 1e-7 * np.abs(dump)), (p.name, ts)


def test_field_probe_api_errors(cuda_lib):
    import ctypes as C
    op = configs.smoke_case()
    g = Engine_CUDA(op, 10)
    pos = (C.c_uint * 3)(1, 1, 1)
    el = (C.c_double * 3)(1e-3, 1e-3, 1e-3)
    pid = C.c_int()
    L = g.lib
    assert L.add_field_probe(g.h, 2, pos, el, 1.0, 1, 0, 0xFFFFFFFF, C.byref(pid)) != 0   # bad field
    assert L.add_field_probe(g.h, 0, pos, el, 1.0, 1, 0, 0xFFFFFFFF, C.byref(pid)) != 0   # after init
