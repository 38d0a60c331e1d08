"""Shared comparison helpers for the parity tests."""
import numpy as np


def bits_equal(a, b):
    a = np.ascontiguousarray(a)
    b = np.ascontiguousarray(b)
    if a.shape != b.shape:
        return False
    if a.dtype == np.float32:
        return np.array_equal(a.view(np.uint32), b.view(np.uint32))
    if a.dtype == np.float64:
        return np.array_equal(a.view(np.uint64), b.view(np.uint64))
    if a.dtype == np.complex64:
        return np.array_equal(a.view(np.uint32), b.view(np.uint32))
    if a.dtype == np.complex128:
        return np.array_equal(a.view(np.uint64), b.view(np.uint64))
    return np.array_equal(a, b)


def rel_l2(a, b):
    a = np.asarray(a)
    b = np.asarray(b)
    dt = np.complex128 if (np.iscomplexobj(a) or np.iscomplexobj(b)) else np.float64
    a = a.astype(dt)
    b = b.astype(dt)
    m = np.isfinite(a) & np.isfinite(b)
    den = np.linalg.norm(b[m])
    return np.linalg.norm(a[m] - b[m]) / (den if den > 0 else 1.0)


def compare_engines(ga, gb, check_dumps=True):
    """Bitwise comparison of fields, probe series, probe DFTs and FD dumps of two engines."""
    out = {}
    for w in (0, 1):
        fa, fb = ga.read_field(w), gb.read_field(w)
        out[f"field{w}"] = bits_equal(fa, fb)
    fids = list(getattr(ga, "fprobe_ids", []))
    fps = list(getattr(ga.op, "fprobes", []) or [])
    for pid in ga.vprobe_ids + ga.iprobe_ids + fids:
        sa, sb = ga.probe_series(pid), gb.probe_series(pid)
        out[f"probe{pid}"] = np.array_equal(np.isnan(sa), np.isnan(sb)) and bits_equal(
            np.nan_to_num(sa), np.nan_to_num(sb))
    for pid, p in zip(ga.vprobe_ids + ga.iprobe_ids + fids, ga.op.vprobes + ga.op.iprobes + fps):
        if p.fd_interval and p.freqs:
            out[f"dft{pid}"] = bits_equal(ga.probe_dft(pid, len(p.freqs)), gb.probe_dft(pid, len(p.freqs)))
    if check_dumps:
        for did in ga.dump_ids:
            out[f"dump{did}"] = bits_equal(ga.fd_dump(did), gb.fd_dump(did))
    return out


def op_digest(op):
    """sha256 over every engine input of an OperatorData (coefficients, excitation table and
    signal, UPML/Mur/Lorentz tables, probe definitions).  Two hosts that build the same operator
    bit for bit give the same digest; fixtures record it so that a comparison knows whether its
    inputs were identical."""
    import hashlib
    h = hashlib.sha256()

    def put(a):
        a = np.ascontiguousarray(a)
        h.update(str(a.dtype).encode() + str(a.shape).encode())
        h.update(a.tobytes())

    for k in ("num_lines", "vv", "vi", "ii", "iv"):
        put(getattr(op, k))
    h.update(repr(float(op.dt)).encode())
    ex = op.exc
    for k in ("volt_index", "volt_dir", "volt_amp", "volt_delay", "curr_index", "curr_dir", "curr_amp",
              "curr_delay", "signal_volt", "signal_curr"):
        put(getattr(ex, k))
    h.update(str(int(ex.period)).encode())
    for u in op.upml:
        for k in ("start", "num_lines", "vv", "vvfo", "vvfn", "ii", "iifo", "iifn"):
            put(getattr(u, k))
    for m in op.mur:
        h.update(str((m.ny, m.line_nr, m.line_nr_shift, m.start_ts)).encode())
        put(m.coeff_nyP)
        put(m.coeff_nyPP)
    for o in op.lorentz:
        put(o.pos)
        h.update(str((o.volt_ade_on, o.curr_ade_on, o.volt_lor_on, o.curr_lor_on)).encode())
        for k in ("v_int", "v_ext", "v_lor", "i_int", "i_ext", "i_lor"):
            put(getattr(o, k))
    for p in list(op.vprobes) + list(op.iprobes):
        h.update(repr((list(p.start), list(p.stop), p.weight, p.interval, p.fd_interval, list(p.freqs))).encode())
    return h.hexdigest()


def field_digest(a):
    import hashlib
    return hashlib.sha256(np.ascontiguousarray(a, np.float32).tobytes()).hexdigest()
