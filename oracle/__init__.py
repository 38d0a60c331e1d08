"""ORACLE -- test infrastructure only.

A plain-C CPU restatement of openEMS's EC-FDTD engine path (``oems_oracle.c``) used as the
checker of the CUDA engine by ``tests/``, by ``__graft_entry__.smoke()`` and by the
CPU-baseline leg of ``bench.py``.  The product package never imports it.
"""
