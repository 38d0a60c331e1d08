"""NF2FF on the device (oems_cuda_nf2ff) against the oracle restatement of nf2ff_calc, on the
FD dumps of a patch-antenna run (UPML, 50 Ohm port, NF2FF box of six faces, three frequencies).
The device sums in a different order (float per chunk of samples, double across chunks, against
the reference's per-thread double sums), so the bound is a relative L2 of 1e-4 on the far
fields and 1e-6 on the radiated power."""
import numpy as np
import pytest

from helpers import rel_l2

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def patch_run(cuda_lib):
    from openems_gb300 import configs
    from openems_gb300.engine import Engine_CUDA
    op = configs.patch(shape=(56, 52, 36), steps=400)
    eng = Engine_CUDA(op, 400)
    eng.IterateTS(400)
    yield eng
    eng.close()


def _oracle(eng, faces, fi, theta, phi, center, radius):
    from oracle.nf2ff_ref import nf2ff
    data = []
    for ie, ih, coords in faces:
        E = eng.fd_dump(ie)[fi]
        H = eng.fd_dump(ih)[fi]
        data.append((coords, E, H))
    d = eng.op.dumps[eng.dump_ids.index(faces[0][0])]
    return nf2ff(data, d.freqs[fi], theta, phi, center=center, radius=radius)


def test_nf2ff_matches_oracle(patch_run):
    from openems_gb300.nf2ff import box_faces, calc_nf2ff
    eng = patch_run
    faces = box_faces(eng)
    assert len(faces) == 6
    theta = np.deg2rad(np.arange(0, 181, 4.0))
    phi = np.deg2rad(np.array([0.0, 45.0, 90.0]))
    center = (0.0, 0.0, 1e-3)
    for fi in range(3):
        r = calc_nf2ff(eng, fi, theta, phi, center=center, radius=1.0)
        o = _oracle(eng, faces, fi, theta, phi, center, 1.0)
        assert rel_l2(r.E_theta, o["E_theta"]) <= 1e-4
        assert rel_l2(r.E_phi, o["E_phi"]) <= 1e-4
        assert r.Prad == pytest.approx(o["Prad"], rel=1e-6)
        assert r.Dmax == pytest.approx(o["Dmax"], rel=1e-4)
        assert r.Prad > 0


def test_nf2ff_rejects_bad_faces(patch_run):
    import ctypes as C
    from openems_gb300.engine import _p
    eng = patch_run
    ids = np.asarray([0], np.int32)
    coords = np.zeros(8)
    th = np.zeros(1)
    c = np.zeros(3)
    out = np.zeros(2)
    rc = eng.lib.nf2ff(eng.h, 1, _p(ids, C.c_int), _p(ids, C.c_int), _p(coords, C.c_double), 0, 1e9, 1,
                       _p(th, C.c_double), 1, _p(th, C.c_double), _p(c, C.c_double), 1.0, 1.0, 1.0,
                       _p(out, C.c_double), _p(out, C.c_double), _p(out, C.c_double), None, None)
    assert rc == 1                                          # an E dump paired with itself
