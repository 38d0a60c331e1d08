"""Frequency-domain dumps written as files (ProcessFieldsFD::DumpFDData, VTK file type).

``oems_cuda_write_fd_dump`` writes, per frequency, the reference's 21 phase snapshots
real(F e^{j 2 pi p/21}), the magnitude and the phase of the accumulated FD field, under the
reference's names (<name>_f=<freq>_p=<deg>.vtr, _abs.vtr, _arg.vtr; Common/processfields_fd.cpp:
114-215).  The test checks the file set, the coordinates, and every value against the engine's
own accumulator (read through the C ABI) transformed in numpy complex64, within float round-off;
the accumulator itself is bit-exact against the oracle in the parity tests.
"""
import math
import os

import numpy as np
import pytest

from openems_gb300 import configs
from openems_gb300.engine import Engine_CUDA
from openems_gb300.vtkio import read_vtr


def _freq_str(f):
    return str(int(f)) if f == int(f) else "%f" % f


@pytest.mark.gpu
def test_fd_dump_files_match_accumulator(cuda_lib, tmp_path):
    op = configs.small_mixed(steps=240)
    g = Engine_CUDA(op, 240, dump_path=str(tmp_path))
    g.IterateTS(240)
    g.sync()
    assert g.dump_ids
    for did, d in zip(g.dump_ids, op.dumps):
        F = g.fd_dump(did).astype(np.complex64)           # [nf][3][sx][sy][sz]
        prefix = os.path.join(str(tmp_path), f"fd{did}")
        g.write_fd_dump(did, prefix)
        scale = float(np.abs(F).max()) or 1.0
        for fi, f in enumerate(d.freqs):
            base = f"{prefix}_f={_freq_str(f)}"
            for p in range(21):
                ang = 2.0 * math.pi * p / 21
                path = f"{base}_p={int(ang * 180 / math.pi):03d}.vtr"
                name, coords, field = read_vtr(path)
                assert name == ("E-Field" if d.field == 0 else "H-Field")
                want = np.real(F[fi] * np.complex64(complex(math.cos(ang), math.sin(ang))))
                assert field.shape == want.shape
                assert np.abs(field - want).max() <= 2e-6 * scale, (did, f, p)
            _, _, mag = read_vtr(base + "_abs.vtr")
            assert np.abs(mag - np.abs(F[fi])).max() <= 2e-6 * scale
            _, _, ph = read_vtr(base + "_arg.vtr")
            big = np.abs(F[fi]) > 1e-3 * scale
            dph = np.angle(np.exp(1j * (ph[big].astype(np.float64) - np.angle(F[fi][big]))))
            assert np.abs(dph).max() <= 1e-5
        # 23 files per frequency
        names = [n for n in os.listdir(str(tmp_path)) if n.startswith(f"fd{did}_f=")]
        assert len(names) == 23 * len(d.freqs)
    # coordinates are the dump's (snapped) mesh lines in metres
    d0 = op.dumps[0]
    _, coords, _ = read_vtr(f"{os.path.join(str(tmp_path), 'fd' + str(g.dump_ids[0]))}_f="
                            f"{_freq_str(d0.freqs[0])}_abs.vtr")
    assert [len(c) for c in coords] == [int(b) - int(a) + 1 for a, b in zip(d0.start, d0.stop)]
    g.close()


@pytest.mark.gpu
def test_fd_dump_file_error_is_reported(cuda_lib, tmp_path):
    op = configs.small_mixed(steps=20)
    g = Engine_CUDA(op, 20, dump_path=str(tmp_path))
    g.IterateTS(20)
    with pytest.raises(Exception, match="write_fd_dump"):
        g.write_fd_dump(g.dump_ids[0], os.path.join(str(tmp_path), "no_such_dir", "x"))
    g.close()
