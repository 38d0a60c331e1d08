"""ORACLE build recipe (test infrastructure only): compile openEMS's own engine into oracle/_ref/.

The reference's engine-side translation units are compiled unmodified from the openEMS source tree
(``$OEMS_REFERENCE``, default /root/reference) against the declaration-only stand-ins in
``oracle/refbuild/shim`` (CSXCAD, fparser, VTK, Boost.Predef/Program_options/StringAlgo) and the
small functional Boost.Thread stand-in there, then linked with ``harness.cpp`` (the C ABI) and
``link_stubs.cpp`` into two libraries:

- ``liboems_refeng.so``: as the reference runs on this x86-64 host, where its SSE engines set
  flush-to-zero and denormals-are-zero (``Denormal::Disable``, tools/denormal.h);
- ``liboems_refeng_noftz.so``: the same sources with the architecture probe reporting a non-x86
  target, so ``Denormal::Disable`` is the no-op it is on the arm64 hosts of the GPU machines.  This
  is the variant the parity tests compare with: the CUDA engine keeps denormals too.

Flags follow the reference's Release build (``-O3 -DNDEBUG``, no target-specific options); floating
point contraction is off, which is what x86-64 without ``-mfma`` gives anyway.  Nothing here copies
a reference source: objects and libraries go to oracle/_ref/ (git-ignored).  The build needs the
reference tree, so it runs only where that tree exists; it is skipped elsewhere.
"""
import concurrent.futures as cf
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE = os.path.dirname(HERE)
OUT = os.path.join(ORACLE, "_ref")
SHIM = os.path.join(HERE, "shim")
REF = os.environ.get("OEMS_REFERENCE", "/root/reference")

# reference translation units, paths relative to the openEMS source tree
REF_UNITS = [
    "Common/operator_base.cpp", "Common/engine_interface_base.cpp", "Common/processing.cpp",
    "Common/processintegral.cpp", "Common/processvoltage.cpp", "Common/processcurrent.cpp",
    "FDTD/operator.cpp", "FDTD/operator_sse.cpp", "FDTD/operator_sse_compressed.cpp",
    "FDTD/operator_multithread.cpp", "FDTD/operator_cylinder.cpp", "FDTD/operator_cylindermultigrid.cpp",
    "FDTD/engine.cpp", "FDTD/engine_sse.cpp", "FDTD/engine_sse_compressed.cpp", "FDTD/engine_multithread.cpp",
    "FDTD/engine_cylinder.cpp", "FDTD/engine_cylindermultigrid.cpp", "FDTD/engine_interface_fdtd.cpp",
    "FDTD/excitation.cpp",
    "FDTD/extensions/engine_extension.cpp", "FDTD/extensions/operator_extension.cpp",
    "FDTD/extensions/engine_ext_excitation.cpp", "FDTD/extensions/operator_ext_excitation.cpp",
    "FDTD/extensions/engine_ext_upml.cpp", "FDTD/extensions/operator_ext_upml.cpp",
    "FDTD/extensions/engine_ext_mur_abc.cpp", "FDTD/extensions/operator_ext_mur_abc.cpp",
    "FDTD/extensions/engine_ext_dispersive.cpp", "FDTD/extensions/operator_ext_dispersive.cpp",
    "FDTD/extensions/engine_ext_lorentzmaterial.cpp", "FDTD/extensions/operator_ext_lorentzmaterial.cpp",
    "FDTD/extensions/engine_ext_cylinder.cpp", "FDTD/extensions/operator_ext_cylinder.cpp",
    "FDTD/extensions/engine_ext_cylindermultigrid.cpp",
    "tools/useful.cpp", "tools/AdrOp.cpp", "tools/ErrorMsg.cpp", "tools/array_ops.cpp",
]
OWN_UNITS = [os.path.join(HERE, "harness.cpp"), os.path.join(HERE, "link_stubs.cpp")]

VARIANTS = {"liboems_refeng.so": [], "liboems_refeng_noftz.so": ["-DOEMS_SHIM_ARCH_NOT_X86"]}

CXXFLAGS = ["-std=c++17", "-O3", "-DNDEBUG", "-fPIC", "-ffp-contract=off", "-pthread", "-w",
            '-DGIT_VERSION="openEMS-oracle-harness"']


def available() -> bool:
    return os.path.isfile(os.path.join(REF, "FDTD", "engine_sse_compressed.cpp"))


def lib_path(ftz: bool = False) -> str:
    return os.path.join(OUT, "liboems_refeng.so" if ftz else "liboems_refeng_noftz.so")


def _deps():
    own = [os.path.join(HERE, f) for f in ("harness.cpp", "link_stubs.cpp", "build_ref.py")]
    own += [os.path.join(SHIM, r, f) for r, _, fs in os.walk(SHIM) for f in fs]
    return own


def _stale(lib):
    if not os.path.exists(lib):
        return True
    t = os.path.getmtime(lib)
    return any(os.path.getmtime(d) > t for d in _deps())


def _compile(src, obj, extra):
    cmd = ["g++"] + CXXFLAGS + extra + ["-I", SHIM, "-I", REF, "-c", src, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"compiling {src} failed:\n{r.stderr[-4000:]}")
    return obj


def build(force: bool = False) -> list:
    """Build both variants; returns the library paths ([] when the reference tree is absent)."""
    if not available():
        return []
    os.makedirs(OUT, exist_ok=True)
    out = []
    jobs = max(1, min(16, os.cpu_count() or 1))
    for lib, extra in VARIANTS.items():
        path = os.path.join(OUT, lib)
        out.append(path)
        if not force and not _stale(path):
            continue
        odir = os.path.join(OUT, "obj_" + lib.split(".")[0])
        os.makedirs(odir, exist_ok=True)
        srcs = [os.path.join(REF, u) for u in REF_UNITS] + OWN_UNITS
        objs = [os.path.join(odir, os.path.relpath(s, REF if s.startswith(REF) else HERE).replace("/", "_") + ".o")
                for s in srcs]
        with cf.ThreadPoolExecutor(jobs) as ex:
            list(ex.map(lambda a: _compile(a[0], a[1], extra), zip(srcs, objs)))
        cmd = ["g++", "-shared", "-pthread", "-Wl,-z,defs", "-o", path + ".tmp"] + objs
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"linking {lib} failed:\n{r.stderr[-4000:]}")
        os.replace(path + ".tmp", path)
    return out


BINDING_SRC = os.path.join(os.path.dirname(ORACLE), "openems_gb300", "binding", "engine_cuda.cpp")
CUDA_LIB_DIR = os.path.join(os.path.dirname(ORACLE), "openems_gb300", "_build")
INCLUDE = os.path.join(os.path.dirname(ORACLE), "include")


def build_binding() -> str:
    """Compile the openEMS-side binding (openems_gb300/binding/engine_cuda.cpp) against the
    reference's headers and link it with the reference's engine objects and the CUDA engine
    library, every symbol resolved (-z defs): the proof that the drop-in boundary builds inside
    openEMS.  Returns the library path ('' when the reference tree is absent)."""
    if not available():
        return ""
    libs = build()
    odir = os.path.join(OUT, "obj_" + os.path.basename(libs[1]).split(".")[0])
    objs = [os.path.join(odir, f) for f in sorted(os.listdir(odir)) if f.endswith(".o") and not f.startswith("harness")]
    path = os.path.join(OUT, "liboems_engine_cuda_binding.so")
    bobj = os.path.join(OUT, "engine_cuda_binding.o")
    _compile(BINDING_SRC, bobj, ["-I", INCLUDE, "-DOEMS_SHIM_ARCH_NOT_X86"])
    cmd = (["g++", "-shared", "-pthread", "-Wl,-z,defs", "-o", path, bobj] + objs +
           ["-L", CUDA_LIB_DIR, "-loems_cuda", "-Wl,-rpath," + CUDA_LIB_DIR])
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"linking the binding failed:\n{r.stderr[-4000:]}")
    return path


if __name__ == "__main__":
    print(build(force="--force" in sys.argv) or "reference tree not found: nothing built")
