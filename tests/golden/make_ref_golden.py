"""Generate the reference-engine fixtures (run from the repository root, where the openEMS source
tree is available):

    python tests/golden/make_ref_golden.py [small|c1|c2|c3|all]

Each fixture ``ref_<case>.npz`` holds what openEMS's own multithreaded engine (``Engine_Multithread``
over ``Engine_SSE_Compressed``, compiled unmodified by oracle/refbuild/build_ref.py, denormals kept
as on arm64 hosts) produced for one configuration of ``openems_gb300.configs``:

* ``series_<k>`` / ``dft_<k>``: every probe's time series and DFT, in the order of the operator's
  voltage then current probes;
* ``energy``: Engine_Interface_FDTD::CalcFastEnergy after the last step;
* ``field_sha``: sha256 of the final V and I fields (float32, N-I-J-K) and their per-component L2
  norms ``field_l2``; small cases also keep the full fields;
* ``op_sha``: the digest of the operator inputs (tests/helpers.op_digest), so that a comparison
  knows whether the host it runs on built the same operator bit for bit.

The CUDA tests (tests/test_gpu_ref_parity.py) rebuild each operator, run the GPU engine for the same
steps and compare with these arrays.
"""
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.dirname(HERE))

from openems_gb300 import configs  # noqa: E402
from oracle.refengine import RefEngine  # noqa: E402
from helpers import field_digest, op_digest  # noqa: E402

CASES = {
    # small geometries: full fields kept
    "smoke": (lambda: configs.smoke_case(steps=400), 400, True),
    "mixed": (lambda: configs.small_mixed(steps=600), 600, True),
    "stress_small": (lambda: configs.stress(shape=(40, 36, 30), steps=900, nblocks=12), 900, False),
    "mur_corners": (lambda: configs.mur_corners(steps=1200), 1200, True),
    "patch_small": (lambda: configs.patch(shape=(48, 44, 28), steps=1500, with_nf2ff=False), 1500, False),
    # the benchmark configurations at full size
    "c1_cube_100_10k": (lambda: configs.plain_cube(n=100, steps=10000), 10000, False),
    "c2_patch_160x160x80_20k": (lambda: configs.patch(shape=(160, 160, 80), steps=20000, with_nf2ff=True), 20000,
                                False),
    "c3_stress_512x512x256_1k": (lambda: configs.stress(shape=(512, 512, 256), steps=1000), 1000, False),
}
GROUPS = {"small": ["smoke", "mixed", "stress_small", "mur_corners", "patch_small"],
          "c1": ["c1_cube_100_10k"], "c2": ["c2_patch_160x160x80_20k"], "c3": ["c3_stress_512x512x256_1k"]}
GROUPS["all"] = sum((GROUPS[k] for k in ("small", "c1", "c2", "c3")), [])


def make(name, threads):
    fn, steps, keep = CASES[name]
    if keep:   # small meshes: the per-step barriers of many threads would dominate
        threads = min(threads, 2)
    t0 = time.time()
    op = fn()
    ref = RefEngine(op, steps, kind="multithread", threads=threads)
    t1 = time.time()
    ref.IterateTS(steps)
    t2 = time.time()
    out = {"steps": np.int64(steps), "op_sha": np.array(op_digest(op)), "energy": np.float64(ref.CalcFastEnergy())}
    ids = ref.vprobe_ids + ref.iprobe_ids
    probes = list(op.vprobes) + list(op.iprobes)
    for k, (pid, p) in enumerate(zip(ids, probes)):
        out[f"series_{k}"] = ref.probe_series(pid)
        if p.fd_interval and p.freqs:
            out[f"dft_{k}"] = ref.probe_dft(pid, len(p.freqs))
    sha, l2 = [], []
    for w in (0, 1):
        f = ref.read_field(w)
        sha.append(field_digest(f))
        l2.append([float(np.linalg.norm(f[n].astype(np.float64))) for n in range(3)])
        if keep:
            out[f"field_{w}"] = f
    out["field_sha"] = np.array(sha)
    out["field_l2"] = np.array(l2)
    path = os.path.join(HERE, f"ref_{name}.npz")
    np.savez_compressed(path, **out)
    cells = float(np.prod(op.num_lines))
    print(f"{name}: {steps} steps, setup {t1 - t0:.1f} s, run {t2 - t1:.1f} s "
          f"({cells * steps / (t2 - t1) / 1e6:.0f} MCells/s), {os.path.getsize(path) / 1024:.0f} KB", flush=True)
    ref.close()


if __name__ == "__main__":
    which = sys.argv[1] if len(sys.argv) > 1 else "small"
    threads = int(os.environ.get("OEMS_REF_THREADS", os.cpu_count() or 1))
    for n in GROUPS.get(which, [which]):
        make(n, threads)
