"""NF2FF oracle (no GPU): the restated transform of nf2ff/nf2ff_calc.cpp is pinned by a known
answer.  The exact time-harmonic fields of a z-directed Hertzian dipole, sampled on the six faces
of a closed box, must give back its far field: E_theta = j eta k Il sin(theta) e^{-jkr}/(4 pi r),
E_phi = 0, radiated power eta (k Il)^2 / (12 pi) and directivity 1.5."""
import numpy as np
import pytest

from oracle.nf2ff_ref import Z0, C0, nf2ff


def dipole_fields(x, y, z, k, il=1e-3):
    """E, H (complex, Cartesian, e^{j w t}) of a z-directed current element Il at the origin."""
    r = np.sqrt(x * x + y * y + z * z)
    st = np.sqrt(x * x + y * y) / r
    ct = z / r
    ph = np.arctan2(y, x)
    jkr = 1j * k * r
    ph_ = np.exp(-jkr)
    Er = Z0 * il * ct / (2 * np.pi * r ** 2) * (1 + 1 / jkr) * ph_
    Et = 1j * Z0 * k * il * st / (4 * np.pi * r) * (1 + 1 / jkr - 1 / (k * r) ** 2) * ph_
    Hp = 1j * k * il * st / (4 * np.pi * r) * (1 + 1 / jkr) * ph_
    # spherical unit vectors in Cartesian components
    rx, ry, rz = st * np.cos(ph), st * np.sin(ph), ct
    tx, ty, tz = ct * np.cos(ph), ct * np.sin(ph), -st
    px, py = -np.sin(ph), np.cos(ph)
    E = np.stack([Er * rx + Et * tx, Er * ry + Et * ty, Er * rz + Et * tz])
    H = np.stack([Hp * px, Hp * py, np.zeros_like(Hp)])
    return E, H


def box_faces(half, n, k):
    faces = []
    line = np.linspace(-half, half, n)
    for ny in range(3):
        for side in (-half, half):
            lines = [line, line, line]
            lines = [l.copy() for l in lines]
            lines[ny] = np.array([side])
            X, Y, Z = np.meshgrid(*lines, indexing="ij")
            E, H = dipole_fields(X, Y, Z, k)
            faces.append((lines, E, H))
    return faces


def test_hertzian_dipole_far_field_known_answer():
    f = 1e9
    k = 2 * np.pi * f / C0
    il = 1e-3
    faces = box_faces(0.2, 81, k)
    theta = np.linspace(10, 170, 17) * np.pi / 180
    phi = np.array([0.0, 0.5 * np.pi, 0.25 * np.pi])
    res = nf2ff(faces, f, theta, phi, radius=1.0)
    ana = 1j * Z0 * k * il * np.sin(theta)[:, None] / (4 * np.pi) * np.exp(-1j * k)
    err = np.abs(res["E_theta"] - ana).max() / np.abs(ana).max()
    assert err < 5e-3, err
    assert np.abs(res["E_phi"]).max() < 5e-3 * np.abs(ana).max()
    p_ana = Z0 * (k * il) ** 2 / (12 * np.pi)
    assert res["Prad"] == pytest.approx(p_ana, rel=5e-3)
    # the directivity over the sampled angles (theta = 90 deg is sampled)
    assert res["Dmax"] == pytest.approx(1.5, rel=1e-2)


def test_face_normal_and_errors():
    from oracle.nf2ff_ref import face_normal
    assert face_normal([np.zeros(4), np.zeros(1), np.zeros(5)]) == 1
    with pytest.raises(ValueError):
        face_normal([np.zeros(1), np.zeros(1), np.zeros(5)])
