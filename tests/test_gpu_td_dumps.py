"""GPU: time-domain field dumps written by the engine's writer thread as VTK files, against the
oracle's samples, bit for bit.

Covers the ring-and-copy pipeline over uneven chunks (single steps, 16-step graphs and mixes),
a ring of three slots (flushes inside a chunk and the single-step fallback), the file names and
coordinates, and the error path of an unwritable directory.
"""
import ctypes
import os

import numpy as np
import pytest

from openems_gb300 import configs
from openems_gb300.engine import Engine_CUDA, EngineError
from openems_gb300.operator import _dual_line
from openems_gb300.vtkio import read_vtr
from oracle.oracle import OracleEngine

from helpers import bits_equal

pytestmark = pytest.mark.gpu


def _run(op, steps, path, chunks):
    g = Engine_CUDA(op, steps, dump_path=str(path))
    done, k = 0, 0
    while done < steps:
        n = min(chunks[k % len(chunks)], steps - done)
        g.IterateTS(n)
        done += n
        k += 1
    g.flush_dumps()
    return g


def _check(op, g, path, steps):
    r = OracleEngine(op, steps)
    r.IterateTS(steps)
    names = set()
    gl = op.grid.lines
    for did, d in zip(r.td_dump_ids, op.td_dumps):
        ts, smp = r.td_samples(did)
        assert len(ts) > 0
        lines = [(_dual_line(np.asarray(l)) if d.dual else np.asarray(l)) * op.grid.unit for l in gl]
        for t, s in zip(ts, smp):
            fn = os.path.join(str(path), f"{d.name}_{int(t):08d}.vtr")
            names.add(os.path.basename(fn))
            fname, coords, field = read_vtr(fn)
            assert fname == ("E-Field" if d.field == 0 else "H-Field")
            for a in range(3):
                assert np.array_equal(coords[a], lines[a][int(d.start[a]):int(d.stop[a]) + 1])
            assert bits_equal(field, s), (d.name, int(t))
    assert set(os.listdir(str(path))) == names
    # the fields themselves are untouched by the dumps
    assert bits_equal(g.read_field(0), r.read_field(0))


@pytest.mark.parametrize("chunks", [(1,), (16,), (1, 7, 16, 33)])
def test_td_dump_files_bit_exact(cuda_lib, tmp_path, chunks):
    steps = 120
    op = configs.td_dumps(steps=steps)
    g = _run(op, steps, tmp_path, chunks)
    _check(op, g, tmp_path, steps)
    g.close()


def test_small_ring_flushes_inside_chunks(cuda_lib, tmp_path, monkeypatch):
    monkeypatch.setenv("OEMS_CUDA_TD_SLOTS", "3")
    steps = 150
    op = configs.td_dumps(steps=steps)
    # interval 1 on every dump: a 16-step graph would produce 16 samples, more than the ring holds
    for d in op.td_dumps:
        d.interval = 1
    g = _run(op, steps, tmp_path, (40, 3, 64, 43))
    _check(op, g, tmp_path, steps)
    g.close()


def test_unwritable_directory_reports_io_error(cuda_lib, tmp_path):
    op = configs.td_dumps(steps=20)
    g = Engine_CUDA(op, 20, dump_path=str(tmp_path / "missing" / "dir"))
    g.IterateTS(20)
    with pytest.raises(EngineError, match="OEMS_ERR_IO"):
        g.flush_dumps()
    # a time-domain dump has no FD accumulator to read
    buf = np.zeros(16, np.float32)
    assert g.lib.read_fd_dump(g.h, g.td_dump_ids[0], buf.ctypes.data_as(ctypes.POINTER(ctypes.c_float)), 16) != 0
    g.close()
