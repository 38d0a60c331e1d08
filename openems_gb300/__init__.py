"""GB300-native EC-FDTD engine: a CUDA (sm_103a) drop-in for openEMS's Engine path.

The engine itself lives in the compiled C-ABI library (``openems_gb300/csrc``); this package
holds the host-side Operator restatement that produces its inputs and a thin ctypes mirror of
openEMS's ``Engine`` / ``Processing`` interface.
"""
