"""CPU oracle for the XC grid path (test infrastructure only).

The oracle checks the CUDA path: only ``tests/``, ``__graft_entry__.smoke()`` and
the CPU-baseline leg of ``bench.py`` may call it.  The product path in
``graddft_gb300`` never imports it.
"""
from .oracle import *  # noqa: F401,F403
from .ao_numpy import eval_ao_planes  # noqa: F401
