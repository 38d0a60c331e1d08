"""Generate the committed golden fixtures (run from the repository root):

    python tests/golden/make_golden.py

* cavity_contract.json -- the resonance contract of the reference's TESTSUITE/combinedtests/cavity.m
  (analytic TE/TM resonances of the a x b x d PEC cavity and the test's relative limits);
* oracle_small.npz     -- probe series, probe DFTs and field checksums of the CPU oracle on the
  small test geometries (pins the oracle against accidental change; the GPU tests compare the CUDA
  engine to these arrays too).
"""
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from openems_gb300 import configs  # noqa: E402
from oracle.oracle import OracleEngine  # noqa: E402

C0 = 299792458.0

CASES = {
    "smoke": (configs.smoke_case, 60),
    "mixed": (configs.small_mixed, 200),
    "cube24": (lambda: configs.plain_cube(n=24, steps=300), 300),
}


def cavity_contract():
    a, b, d = 5e-2, 2e-2, 6e-2
    k = lambda m, n, l: np.sqrt((m * np.pi / a) ** 2 + (n * np.pi / b) ** 2 + (l * np.pi / d) ** 2)  # noqa: E731
    f_te = [C0 / (2 * np.pi) * k(*mnl) for mnl in ((1, 0, 1), (1, 0, 2), (2, 0, 1), (2, 0, 2))]
    f_tm = [C0 / (2 * np.pi) * k(*mnl) for mnl in ((1, 1, 0), (1, 1, 1))]
    return {
        "source": "TESTSUITE/combinedtests/cavity.m:20-36,150-214",
        "f_start": 1e9, "f_stop": 10e9, "t_start": 7e-10, "steps": 20000,
        "lower_rel_limit": 1.3e-3, "upper_rel_limit": 1.3e-3,
        "lower_rel_limit_TM": 2.5e-3, "upper_rel_limit_TM": 0.0,
        "min_rel_amplitude": 0.6, "min_rel_amplitude_TM": 0.27,
        "outer_rel_limit": 0.02, "max_rel_amplitude": 0.17,
        "f_TE": f_te, "f_TM": f_tm,
    }


def oracle_case(name):
    fn, steps = CASES[name]
    op = fn()
    eng = OracleEngine(op, steps)
    eng.IterateTS(steps)
    out = {}
    for pid, p in zip(eng.vprobe_ids + eng.iprobe_ids, op.vprobes + op.iprobes):
        out[f"{name}_probe{pid}"] = eng.probe_series(pid)
        if p.fd_interval and p.freqs:
            out[f"{name}_dft{pid}"] = eng.probe_dft(pid, len(p.freqs))
    for w in (0, 1):
        f = eng.read_field(w)
        out[f"{name}_field{w}_sum"] = np.array([np.sum(f.astype(np.float64)), np.sum(np.abs(f.astype(np.float64)))])
    eng.close()
    return out


def main():
    with open(os.path.join(HERE, "cavity_contract.json"), "w") as fh:
        json.dump(cavity_contract(), fh, indent=1)
    arrays = {}
    for name in CASES:
        arrays.update(oracle_case(name))
    np.savez_compressed(os.path.join(HERE, "oracle_small.npz"), **arrays)
    print("wrote", sorted(arrays))


if __name__ == "__main__":
    main()
