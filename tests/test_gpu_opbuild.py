"""The operator numerics on the device (oems_cuda_opbuild_*, Operator.build(device="cuda")):
coefficients, timestep and every extension table bit-identical to the host build, on uniform
and graded meshes with dielectric, lossy, dispersive and metal boxes, lumped ports, UPML, Mur
and PEC/PMC walls."""
import numpy as np
import pytest

from helpers import bits_equal
from openems_gb300 import configs
from openems_gb300.operator import build_device

pytestmark = pytest.mark.gpu

CASES = [
    ("stress", lambda: configs.stress(shape=(60, 52, 44), steps=50, nblocks=24)),
    ("patch_graded", lambda: configs.patch(shape=(56, 52, 36), steps=50)),
    ("mixed", lambda: configs.small_mixed()),
    ("mixed_bc", lambda: configs.small_mixed(bc=(0, 1, 2, 0, 3, 3), seed=3)),
    ("cube", lambda: configs.plain_cube(n=40, steps=50)),
    ("cavity", lambda: configs.cavity(steps=50)),
    ("batch_instance", lambda: configs.batch_instance(7, size_range=(30, 40), steps_range=(50, 60))[0]),
]


def _equal_tables(a, b, path="op"):
    if isinstance(a, np.ndarray):
        assert bits_equal(a, b), path
    elif isinstance(a, (list, tuple)):
        assert len(a) == len(b), path
        for k, (x, y) in enumerate(zip(a, b)):
            _equal_tables(x, y, f"{path}[{k}]")
    elif hasattr(a, "__dataclass_fields__"):
        for f in a.__dataclass_fields__:
            if f in ("excitation", "grid"):
                continue
            _equal_tables(getattr(a, f), getattr(b, f), f"{path}.{f}")
    elif isinstance(a, float):
        assert a == b, path


@pytest.mark.parametrize("name,fn", CASES)
def test_device_build_equals_host_build(cuda_lib, name, fn):
    host = fn()
    with build_device("cuda"):
        dev = fn()
    assert host.dt == dev.dt
    for k in ("vv", "vi", "ii", "iv"):
        assert bits_equal(getattr(host, k), getattr(dev, k)), k
    _equal_tables(host, dev)


def test_device_build_rejects_voxel_materials(cuda_lib):
    case = configs.DesignCase(lines=(26, 26, 20), design=(4, 4, 2), gap=4, steps=10, pml=4)
    with build_device("cuda"):
        with pytest.raises(ValueError, match="voxel"):
            case.build(case.eps0)
