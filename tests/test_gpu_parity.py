"""GPU parity: the CUDA engine (through the C ABI) against the CPU oracle on the same inputs.

Bar: bit-exact fields, probe series, probe DFTs and FD dumps (the engine issues the reference's
separate multiplies and adds without FMA contraction and keeps denormals); energy within a
relative 1e-12 (the device reduction order differs from the sequential sum).  At full sizes the
checks are size-independent properties (power-of-two linearity, snapshot/restore replay) plus a
short bit-exact run against the multithreaded oracle.
"""
import json
import os

import numpy as np
import pytest

from openems_gb300 import configs
from openems_gb300.engine import Engine_CUDA, EngineError
from oracle.oracle import OracleEngine

from helpers import bits_equal, compare_engines, rel_l2

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


def _run_pair(op, steps, chunks=(1,), **kw):
    g = Engine_CUDA(op, steps, **kw)
    r = OracleEngine(op, steps)
    done = 0
    k = 0
    while done < steps:
        n = min(chunks[k % len(chunks)], steps - done)
        g.IterateTS(n)
        r.IterateTS(n)
        done += n
        k += 1
    g.sync()
    return g, r


CASES = [
    ("smoke", configs.smoke_case, 60),
    ("mixed", configs.small_mixed, 200),
    ("mixed_bc2", lambda: configs.small_mixed(bc=(0, 1, 2, 0, 3, 3), seed=3, steps=180), 180),
    ("mixed_mur_all", lambda: configs.small_mixed(bc=(2, 2, 2, 2, 2, 2), seed=5, steps=160), 160),
    ("mur_corners", configs.mur_corners, 600),
    ("mur_corners_lanes", lambda: configs.mur_corners(n=(16, 14, 33), wall_source=False, steps=300), 300),
    ("cube40", lambda: configs.plain_cube(n=40, steps=400), 400),
    ("stress_small", lambda: configs.stress(shape=(40, 36, 30), steps=150, nblocks=16), 150),
    ("patch_small", lambda: configs.patch(shape=(56, 52, 36), steps=250), 250),
    ("plane_wave_upml", lambda: configs.plane_wave(steps=200), 200),
    ("plane_wave_oblique_mur", lambda: configs.plane_wave(bc=(2,) * 6, k_dir=(1.0, 0.5, -0.3), e_dir=(0.0, 0.5, 1.0),
                                                         frequency=10e9, graded=True, dispersive=True,
                                                         box=([0, 6, 5], [20, 23, 19]), steps=220), 220),
    ("plane_wave_sinus", lambda: configs.plane_wave(k_dir=(-0.2, -1.0, 0.4), e_dir=(1.0, 0.0, 0.5), sinus=True,
                                                   steps=200), 200),
    ("lumped_rlc_mur", lambda: configs.lumped_rlc(steps=300), 300),
    ("lumped_rlc_upml_dispersive", lambda: configs.lumped_rlc(bc=(3,) * 6, dispersive=True, steps=240), 240),
    ("coax_cylinders", lambda: configs.coax(steps=150, length=200.0), 150),
    ("conducting_sheet_mur", lambda: configs.conducting_sheet(steps=240), 240),
    ("conducting_sheet_upml_dispersive", lambda: configs.conducting_sheet(bc=(3,) * 6, dispersive=True, steps=200),
     200),
    ("coax_cyl_closed_alpha_mur", lambda: configs.coax_cyl(steps=200, length=400.0), 200),
    ("coax_cyl_closed_alpha_upml", lambda: configs.coax_cyl(steps=200, length=400.0, pml=True), 200),
    ("coax_cyl_lumped_load", lambda: configs.coax_cyl(steps=200, length=400.0, load=30.0), 200),
    ("coax_cyl_rlc_load", lambda: configs.coax_cyl(steps=200, length=400.0, load=30.0, rlc=True), 200),
    ("coax_cyl_conducting_sheet", lambda: configs.coax_cyl(steps=200, length=400.0, shield="sheet"), 200),
    ("cavity_cyl_axis", lambda: configs.cavity_cyl(steps=400), 400),
    ("cavity_cyl_off_axis", lambda: configs.cavity_cyl(steps=300, n_alpha=25, probe_r=10.0), 300),
    ("cavity_cyl_dispersive", lambda: configs.cavity_cyl(steps=300, dispersive=True), 300),
    ("cavity_cyl_field_probes_fd_dumps", lambda: configs.cavity_cyl(steps=300, field_probes=True, fd_dumps=True), 300),
    ("sector_cyl_alpha_upml", lambda: configs.sector_cyl(steps=300), 300),
]


@pytest.mark.parametrize("name,fn,steps", CASES)
def test_bit_exact_against_oracle(cuda_lib, name, fn, steps):
    op = fn()
    g, r = _run_pair(op, steps, chunks=(1, 7, 16, 33))
    res = compare_engines(g, r)
    bad = [k for k, v in res.items() if not v]
    assert not bad, (name, bad)
    eg, er = g.CalcFastEnergy(), r.CalcFastEnergy()
    assert abs(eg - er) <= 1e-12 * abs(er) + 1e-300
    assert g.GetNumberOfTimesteps() == steps


MARCH_CASES = [
    ("cube40", lambda: configs.plain_cube(n=40, steps=300), 300),
    ("cube33_lanes", lambda: configs.plain_cube(n=33, steps=260), 260),
    ("mixed_pec_pmc", lambda: configs.small_mixed(n=(30, 27, 37), bc=(0, 1, 1, 0, 0, 1), pml=0, dispersive=False,
                                                  steps=220), 220),
    ("stress_pec", lambda: configs.stress(shape=(44, 38, 30), steps=160, nblocks=16, bc=(0,) * 6, dispersive=False),
     160),
]


@pytest.mark.parametrize("ty,xchunk", [(None, None), ("1", "4"), ("3", "5"), ("6", "64")])
@pytest.mark.parametrize("name,fn,steps", MARCH_CASES)
def test_march_step_bit_exact_against_oracle(cuda_lib, monkeypatch, name, fn, steps, ty, xchunk):
    """The TMA-staged plane march (OEMS_CUDA_MARCH=1): one kernel per step with I staged by
    cp.async.bulk.tensor, at the default tile and at tiles and x-chunks that leave partial tiles
    and chunks, mixed with single separate-kernel steps by the uneven chunks."""
    monkeypatch.setenv("OEMS_CUDA_MARCH", "1")
    if ty:
        monkeypatch.setenv("OEMS_CUDA_MARCH_TY", ty)
        monkeypatch.setenv("OEMS_CUDA_MARCH_XCHUNK", xchunk)
    op = fn()
    g, r = _run_pair(op, steps, chunks=(1, 7, 16, 33))
    assert g.launches_per_step() == 2                      # march step + processing
    res = compare_engines(g, r)
    bad = [k for k, v in res.items() if not v]
    assert not bad, (name, bad)


@pytest.mark.parametrize("name,fn,steps", [c for c in CASES if c[0] in ("smoke", "mixed", "mixed_mur_all", "mur_corners",
                                                                        "mur_corners_lanes", "stress_small")])
def test_separate_mur_hooks_bit_exact_against_oracle(cuda_lib, monkeypatch, name, fn, steps):
    """The Mur pre/post hooks as separate launches (OEMS_CUDA_MUR_SEPARATE=1) instead of inside
    the voltage update: the same fields, bit for bit, with two more launches per step."""
    op = fn()
    monkeypatch.setenv("OEMS_CUDA_LOR_CARRY", "0")     # separate Mur hooks keep the dispersive apply apart
    monkeypatch.setenv("OEMS_CUDA_SE_SPLIT", "0")      # and the step end in one launch
    fused = Engine_CUDA(op, steps)
    n_fused = fused.launches_per_step()
    fused.close()
    monkeypatch.setenv("OEMS_CUDA_MUR_SEPARATE", "1")
    g, r = _run_pair(op, steps, chunks=(1, 7, 16, 33))
    assert g.launches_per_step() == n_fused + 2
    res = compare_engines(g, r)
    bad = [k for k, v in res.items() if not v]
    assert not bad, (name, bad)


@pytest.mark.parametrize("name,fn,steps", MARCH_CASES[:2])
def test_march_autotune_bit_exact_against_oracle(cuda_lib, monkeypatch, name, fn, steps):
    """Without OEMS_CUDA_MARCH the first long iterate times the plane march against the separate
    kernels and keeps the faster; either way the results equal the oracle's bit for bit."""
    monkeypatch.delenv("OEMS_CUDA_MARCH", raising=False)
    op = fn()
    g, r = _run_pair(op, steps, chunks=(steps - 13, 13))
    assert g.update_kernels()[0] in ("k_step_march", "k_update_v4"), g.update_kernels()
    res = compare_engines(g, r)
    bad = [k for k, v in res.items() if not v]
    assert not bad, (name, bad)


@pytest.mark.parametrize("park", ["1", "0"])
def test_mur_float4_inner_z_walls_bit_exact_against_oracle(cuda_lib, monkeypatch, park):
    """k_update_v4w with z walls away from the row ends (lines 4 / 27 of 30, each with its shift in
    the same group of four): the wall groups sit inside the rows, between streaming groups.  The
    walls are placed by hand, which the oracle models the same way.  park = 1: the direct columns'
    z-wall hooks as k_mur_zsave / k_mur_zpost around the update; park = 0: inside it."""
    import dataclasses
    monkeypatch.setenv("OEMS_CUDA_MUR_PARK", park)
    op = configs.stress(shape=(40, 36, 30), steps=140, nblocks=16)
    walls = []
    for w in op.mur:
        if w.ny == 2:
            lo = w.line_nr < w.line_nr_shift
            w = dataclasses.replace(w, line_nr=4 if lo else 27, line_nr_shift=5 if lo else 26)
        walls.append(w)
    op.mur = walls
    g, r = _run_pair(op, 140, chunks=(1, 7, 16, 33))
    assert g.update_kernels()[0] == ("k_update_v4w<park>" if park == "1" else "k_update_v4w")
    res = compare_engines(g, r)
    bad = [k for k, v in res.items() if not v]
    assert not bad, bad


@pytest.mark.parametrize("seed", [20261204, 3])
@pytest.mark.parametrize("carry", ["1", "0"])
def test_lorentz_carry_bit_exact_against_oracle(cuda_lib, monkeypatch, carry, seed):
    """Inside a captured sequence the dispersive apply of one step and the pre of the next run as
    one launch at the end of the half-step (k_lorentz_carry); OEMS_CUDA_LOR_CARRY=0 keeps them
    apart.  Either way, over mixed chunk lengths, the fields, probes and dumps equal the oracle's
    bit for bit.  The carried form has one launch less per step inside a sequence, except where a
    source edge lies on a dispersive position (seed 20261204: its excitation must follow the
    apply, so the apply keeps its place)."""
    monkeypatch.setenv("OEMS_CUDA_LOR_CARRY", carry)
    op = configs.stress(shape=(40, 36, 30), steps=150, nblocks=16, seed=seed)
    assert len(op.lorentz) == 1
    pos = set(map(tuple, np.asarray(op.lorentz[0].pos).T.tolist()))
    src_on_lor = any(tuple(p) in pos for p in np.asarray(op.exc.volt_index).T.tolist())
    assert src_on_lor == (seed == 20261204)
    g, r = _run_pair(op, 150, chunks=(1, 7, 16, 33))
    res = compare_engines(g, r)
    bad = [k for k, v in res.items() if not v]
    assert not bad, bad
    monkeypatch.setenv("OEMS_CUDA_LOR_CARRY", "0")
    plain = Engine_CUDA(op, 10)
    n_plain = plain.launches_per_step()
    plain.close()
    assert g.launches_per_step() == n_plain - (1 if carry == "1" and not src_on_lor else 0)


@pytest.mark.parametrize("seed", [1, 3])
@pytest.mark.parametrize("vtail", ["1", "0"])
def test_voltage_tail_one_launch_bit_exact_against_oracle(cuda_lib, monkeypatch, vtail, seed):
    """Inside a sequence the Mur apply, the dispersive carry and the excitation of the voltage
    half-step run as one launch (k_vtail) where they touch disjoint values; OEMS_CUDA_VTAIL=0
    keeps three launches.  Both equal the oracle bit for bit over mixed chunk lengths.  Seed 3
    puts a dispersive position on the z = 0 wall line, which keeps the launches apart."""
    monkeypatch.setenv("OEMS_CUDA_VTAIL", vtail)
    op = configs.stress(shape=(40, 36, 30), steps=150, nblocks=16, seed=seed)
    pos = np.asarray(op.lorentz[0].pos)
    on_wall = any(bool(np.any(pos[w.ny] == w.line_nr)) for w in op.mur)
    g, r = _run_pair(op, 150, chunks=(1, 7, 16, 33))
    res = compare_engines(g, r)
    bad = [k for k, v in res.items() if not v]
    assert not bad, bad
    monkeypatch.setenv("OEMS_CUDA_VTAIL", "0")
    sep = Engine_CUDA(op, 10)
    n_sep = sep.launches_per_step()
    sep.close()
    assert on_wall == (seed == 3)
    assert g.launches_per_step() == n_sep - (2 if vtail == "1" and not on_wall else 0), on_wall


def test_probe_range_newest_samples_and_restore(cuda_lib):
    """oems_cuda_read_probe_range over single slots, step by step (the processing-loop pattern the
    engine serves from one pinned fetch per step), equals the full series; after a restore to an
    earlier step and a different field, a read at the same step count returns the new samples."""
    op = configs.small_mixed(steps=60)
    g = Engine_CUDA(op, 60)
    pids = g.vprobe_ids + g.iprobe_ids + g.fprobe_ids
    assert len(pids) >= 2
    got = {p: [] for p in pids}
    blob = None
    for ts in range(1, 41):
        g.IterateTS(1)
        if ts == 20:
            blob = g.snapshot()
        for p in pids:
            got[p].append(g.probe_range(p, ts, 1).copy())
    for p in pids:
        full = g.probe_series(p)
        assert bits_equal(np.concatenate(got[p]).ravel(), np.asarray(full)[1:41].ravel()), p
    g.restore(blob)
    g.IterateTS(1)
    before = {p: g.probe_range(p, 21, 1).copy() for p in pids}     # the same step count as below
    g.restore(blob)
    g.write_field(0, 2.0 * g.read_field(0))
    g.write_field(1, 2.0 * g.read_field(1))
    g.IterateTS(1)
    after = {p: g.probe_range(p, 21, 1).copy() for p in pids}
    assert any(not bits_equal(before[p], after[p]) for p in pids)
    for p in pids:
        assert bits_equal(after[p].ravel(), np.asarray(g.probe_series(p))[21:22].ravel()), p


@pytest.mark.parametrize("split", ["1", "0"])
def test_split_step_end_bit_exact_against_oracle(cuda_lib, monkeypatch, split):
    """Without Mur, TFSF or lumped RLC the step end runs as two parts on a side stream: the
    voltage-side probes and dumps beside the current update, the current side (and the step
    counter) beside the next voltage update.  Probes, FD dumps and fields equal the oracle's bit
    for bit over mixed chunk lengths either way; the split costs one launch more per step."""
    monkeypatch.setenv("OEMS_CUDA_SE_SPLIT", split)
    op = configs.patch(shape=(56, 52, 36), steps=250)
    assert not op.mur and (op.vprobes or op.iprobes)
    g, r = _run_pair(op, 250, chunks=(1, 7, 16, 33))
    res = compare_engines(g, r)
    bad = [k for k, v in res.items() if not v]
    assert not bad, bad
    monkeypatch.setenv("OEMS_CUDA_SE_SPLIT", "0")
    one = Engine_CUDA(op, 10)
    n_one = one.launches_per_step()
    one.close()
    assert g.launches_per_step() == n_one + (1 if split == "1" else 0)


@pytest.mark.parametrize("block", ["256", "128", "64"])
@pytest.mark.parametrize("upml", [False, True])
def test_float4_block_sizes_bit_exact_against_oracle(cuda_lib, monkeypatch, block, upml):
    """The float4 update kernels at 64, 128 and 256 threads per block (OEMS_CUDA_V4_BLOCK,
    _I4_BLOCK, _BOX4_BLOCK, _REG4_BLOCK; the UPML kernels take 128 or 256): the Mur wall blocks
    and the UPML region offsets follow the block size."""
    for k in ("V4", "I4", "BOX4", "REG4"):
        monkeypatch.setenv(f"OEMS_CUDA_{k}_BLOCK", block)
    if upml:
        op = configs.patch(shape=(56, 52, 36), steps=140, with_nf2ff=False)
    else:
        op = configs.stress(shape=(40, 36, 30), steps=140, nblocks=16, seed=1)
    g, r = _run_pair(op, 140, chunks=(1, 7, 16, 33))
    want = ("k_update_reg4+k_update_box4",) * 2 if upml else ("k_update_v4w", "k_update_i4")
    assert g.update_kernels() == want
    res = compare_engines(g, r)
    bad = [k for k, v in res.items() if not v]
    assert not bad, bad


IDX_CASES = [
    ("stress_small", lambda: configs.stress(shape=(40, 36, 30), steps=150, nblocks=16, seed=1), 150),
    ("patch_small", lambda: configs.patch(shape=(56, 52, 36), steps=220), 220),
    ("mixed", configs.small_mixed, 200),
]


@pytest.mark.parametrize("narrow", ["1", "0"])
@pytest.mark.parametrize("name,fn,steps", IDX_CASES)
def test_class_index_widths_bit_exact_against_oracle(cuda_lib, monkeypatch, name, fn, steps, narrow):
    """The operator class index read in 16 bits where every class fits (default) or in 32 bits
    (OEMS_CUDA_IDX16=0): float4, one-cell, UPML and Mur kernels all equal the oracle bit for bit."""
    monkeypatch.setenv("OEMS_CUDA_IDX16", narrow)
    op = fn()
    g, r = _run_pair(op, steps, chunks=(1, 7, 16, 33))
    assert 1 < g.operator_classes() <= 65536
    res = compare_engines(g, r)
    bad = [k for k, v in res.items() if not v]
    assert not bad, (name, bad)


REG4_CASES = [
    ("patch_pml8", lambda: configs.patch(shape=(56, 52, 36), steps=220, with_nf2ff=False), 220),
    ("plane_wave_pml4", lambda: configs.plane_wave(n=(28, 24, 32), pml=4, steps=200), 200),
    ("mixed_upml_pml4", lambda: configs.small_mixed(n=(26, 22, 24), bc=(3, 3, 3, 3, 3, 3), pml=4, dispersive=False,
                                                    steps=180), 180),
]


@pytest.mark.parametrize("name,fn,steps", REG4_CASES)
def test_upml_regions_float4_bit_exact_against_oracle(cuda_lib, name, fn, steps):
    """UPML regions four z cells per thread (k_update_reg4), mixed with single steps: the fields,
    probes and dumps equal the oracle's bit for bit."""
    op = fn()
    g, r = _run_pair(op, steps, chunks=(1, 7, 16, 33))
    assert g.update_kernels()[0].startswith("k_update_reg4"), g.update_kernels()
    res = compare_engines(g, r)
    bad = [k for k, v in res.items() if not v]
    assert not bad, (name, bad)


def test_dense_operator_path_equals_compressed(cuda_lib):
    op = configs.small_mixed(steps=120)
    a = Engine_CUDA(op, 120)
    b = Engine_CUDA(op, 120, max_classes=1)          # forces the dense coefficient arrays
    assert a.operator_classes() > 1 and b.operator_classes() == 0
    a.IterateTS(120)
    b.IterateTS(120)
    for w in (0, 1):
        assert bits_equal(a.read_field(w), b.read_field(w))


def _sse_compressed_tables(op):
    """Build Operator_SSE_Compressed-style tables (lane-strided 4-lane vectors)."""
    Nx, Ny, Nz = (int(v) for v in op.num_lines)
    nv = (Nz + 3) // 4
    cols = []
    for arr in (op.vv, op.vi, op.ii, op.iv):
        for n in range(3):
            lanes = np.zeros((Nx, Ny, nv, 4), np.float32)
            for l in range(4):
                z = np.arange(nv) + l * nv
                ok = z < Nz
                lanes[:, :, ok, l] = arr[n][:, :, z[ok]]
            cols.append(lanes.reshape(-1, 4))
    keys = np.concatenate(cols, axis=1)                 # [(x,y,v), 48]
    uniq, inv = np.unique(keys.view(np.uint32), axis=0, return_inverse=True)
    uniq = uniq.view(np.float32)
    U = uniq.shape[0]
    tabs = []
    for t in range(4):
        tabs.append(np.ascontiguousarray(uniq[:, t * 12:(t + 1) * 12].reshape(U, 3, 4).transpose(1, 0, 2)))
    return U, tabs, inv.reshape(Nx, Ny, nv).astype(np.uint32)


def test_reference_sse_compressed_operator_input(cuda_lib):
    import ctypes as C
    from openems_gb300 import _native
    from openems_gb300.engine import _p
    op = configs.small_mixed(steps=100, n=(14, 12, 11))
    U, tabs, index = _sse_compressed_tables(op)
    ref = Engine_CUDA(op, 100)
    # second engine: same extensions, coefficients through the reference's compressed format
    lib = _native.load_cuda()
    h = C.c_void_p()
    nl = np.ascontiguousarray(op.num_lines, np.uint32)
    assert lib.create(_p(nl, C.c_uint), float(op.dt), 0, C.byref(h)) == 0
    tabs = [np.ascontiguousarray(t) for t in tabs]
    index = np.ascontiguousarray(index)
    assert lib.set_operator_sse_compressed(h, U, *[_p(t, C.c_float) for t in tabs], _p(index, C.c_uint)) == 0
    lib.destroy(h)
    # full engine built from the expanded tables must equal the dense-input engine
    Nz = int(op.num_lines[2])
    nv = (Nz + 3) // 4
    z = np.arange(Nz)
    exp = []
    for t in range(4):
        cls = index[:, :, z % nv]                       # [Nx,Ny,Nz]
        exp.append(np.stack([tabs[t][n][cls, z // nv] for n in range(3)]))
    for a, b in zip(exp, (op.vv, op.vi, op.ii, op.iv)):
        assert bits_equal(a, b)


def test_cavity_reference_contract_on_gpu(cuda_lib):
    from test_oracle import _cavity_check
    with open(os.path.join(GOLDEN, "cavity_contract.json")) as fh:
        c = json.load(fh)
    op = configs.cavity(steps=c["steps"])
    g = Engine_CUDA(op, c["steps"])
    g.IterateTS(c["steps"])
    uy = g.probe_series(g.vprobe_ids[1])
    uz = g.probe_series(g.vprobe_ids[2])
    assert _cavity_check(c, op.dt, uy, uz)
    r = OracleEngine(op, c["steps"])
    r.IterateTS(c["steps"])
    assert bits_equal(uy, r.probe_series(r.vprobe_ids[1]))


def test_coax_reference_contract_on_gpu(cuda_lib):
    """TESTSUITE/combinedtests/Coax.m on the CUDA engine: |U/I| within +3 % / -1 % of the
    analytic Z0 from 0 to 1 GHz."""
    from test_contracts_host import coax_impedance, coax_z0
    op = configs.coax(steps=5000)
    g = Engine_CUDA(op, 5000)
    g.IterateTS(5000)
    g.sync()
    f, Z = coax_impedance(g, op)
    Z0 = coax_z0()
    assert f.size > 50
    assert (Z <= Z0 * 1.03).all() and (Z >= Z0 * 0.99).all(), (Z.min() / Z0, Z.max() / Z0)


def test_cylinder_contracts_on_gpu(cuda_lib):
    """The cylindrical-coordinate contracts on the CUDA engine: the coax example's |U/I| within
    +3/-1 % of Z0, and the pillbox TM010 resonance within -0.25/+0 %, both with probe series
    bit-identical to the multithreaded oracle's."""
    import math
    from openems_gb300.operator import EPS0, MUE0
    for fn, steps in ((configs.coax_cyl, 5000), (configs.cavity_cyl, 20000)):
        op = fn(steps=steps)
        g = Engine_CUDA(op, steps)
        g.IterateTS(steps)
        g.sync()
        r = OracleEngine(op, steps, threads=4)
        r.IterateTS(steps)
        for pid in g.vprobe_ids + g.iprobe_ids:
            assert bits_equal(g.probe_series(pid), r.probe_series(pid)), (fn.__name__, pid)
        u = g.probe_series(g.vprobe_ids[0])
        if fn is configs.coax_cyl:
            i = g.probe_series(g.iprobe_ids[0])
            nfft = 1 << int(math.ceil(math.log2(len(u))))
            f = np.fft.rfftfreq(nfft, op.dt)
            sel = f <= 1e9
            Z = np.abs(np.fft.rfft(u, nfft)[sel] / np.fft.rfft(i, nfft)[sel])
            Z0 = math.sqrt(MUE0 / EPS0) * math.log(230 / 100) / (2 * math.pi)
            assert (Z <= Z0 * 1.03).all() and (Z >= Z0 * 0.99).all()
        else:
            u = u[3000:] - u[3000:].mean()
            nf = 1 << 22
            spec = np.abs(np.fft.rfft(u * np.hanning(len(u)), nf))
            f = np.fft.rfftfreq(nf, op.dt)
            sel = (f > 1e9) & (f < 6e9)
            f010 = 2.404825557695773 * 299792458.0 / (2 * math.pi * 0.05)
            assert -2.5e-3 <= f[sel][np.argmax(spec[sel])] / f010 - 1 <= 0.0


def test_against_committed_fixtures(cuda_lib):
    import sys
    sys.path.insert(0, GOLDEN)
    import make_golden
    gold = np.load(os.path.join(GOLDEN, "oracle_small.npz"))
    for name, (fn, steps) in make_golden.CASES.items():
        op = fn()
        g = Engine_CUDA(op, steps)
        g.IterateTS(steps)
        for pid, p in zip(g.vprobe_ids + g.iprobe_ids, op.vprobes + op.iprobes):
            s = g.probe_series(pid)
            assert rel_l2(s, gold[f"{name}_probe{pid}"]) < 1e-5
            if p.fd_interval and p.freqs:
                d = g.probe_dft(pid, len(p.freqs))
                ref = gold[f"{name}_dft{pid}"]
                assert np.linalg.norm(d - ref) <= 1e-5 * np.linalg.norm(ref)


def test_plain_cube_full_size_bit_exact(cuda_lib):
    """100^3 plain configuration, 400 steps, against the single-thread oracle."""
    op = configs.plain_cube(n=100, steps=400)
    g, r = _run_pair(op, 400, chunks=(100,))
    res = compare_engines(g, r)
    assert all(res.values()), res


def test_stress_full_size_properties(cuda_lib):
    """512x512x256 stress mesh: bit-exact against the multithreaded oracle for a few steps,
    exact power-of-two linearity in the source amplitude, and snapshot/restore replay."""
    op = configs.stress(steps=64)
    g = Engine_CUDA(op, 64)
    r = OracleEngine(op, 64, threads=os.cpu_count() or 4)
    g.IterateTS(3)
    r.IterateTS(3)
    for w in (0, 1):
        assert bits_equal(g.read_field(w), r.read_field(w))
    r.close()
    # linearity: doubling every source amplitude doubles every field exactly
    op.exc.volt_amp = (op.exc.volt_amp * 2).astype(np.float32)
    g2 = Engine_CUDA(op, 64)
    g.IterateTS(29)
    g2.IterateTS(32)
    for w in (0, 1):
        a, b = g.read_field(w), g2.read_field(w)
        # exact except where values underflow into denormals (rounding there is not scale-free)
        assert rel_l2(a * np.float32(2), b) < 1e-7
        assert np.mean(a * np.float32(2) == b) > 0.999
    # snapshot / restore: replaying from a checkpoint reproduces the run bit for bit
    snap = g2.snapshot()
    g2.IterateTS(16)
    f1 = [g2.read_field(w) for w in (0, 1)]
    p1 = g2.probe_series(0) if g2.vprobe_ids else None
    g2.restore(snap)
    assert g2.GetNumberOfTimesteps() == 32
    g2.IterateTS(16)
    for w in (0, 1):
        assert bits_equal(g2.read_field(w), f1[w])
    assert np.isfinite(g2.CalcFastEnergy())


def test_errors_are_status_codes(cuda_lib):
    op = configs.smoke_case()
    g = Engine_CUDA(op, 10)
    with pytest.raises(EngineError):
        g.IterateTS(11)                                  # beyond max_timesteps
    with pytest.raises(EngineError):
        g.GetVolt(3, 0, 0, 0)
    g.IterateTS(10)
    assert g.GetNumberOfTimesteps() == 10
    assert np.isfinite(g.CalcFastEnergy())


def test_launch_accounting(cuda_lib):
    op = configs.small_mixed(steps=20)
    g = Engine_CUDA(op, 20)
    n = g.launches_per_step()
    # lorentz pre+apply (V), update V (+ Mur pre/post), mur apply, excitation V, update I, step_end
    assert n >= 6
    ms, cnt = g.profile(5)
    assert sum(cnt) == 5 * n
    g2 = Engine_CUDA(op, 20)
    g2.IterateTS(5)
    for w in (0, 1):
        assert bits_equal(g.read_field(w), g2.read_field(w))
