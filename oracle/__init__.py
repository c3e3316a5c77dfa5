"""FP64 CPU restatement of the PhaseShiftGrayCode3D reconstruction path.

TEST INFRASTRUCTURE ONLY: the parity checker used by ``tests/``,
``__graft_entry__.smoke()`` and the CPU-baseline leg of ``bench.py``.  The
shipped library never imports it.  Parity status: unpinned (the reference has
no golden vectors and cannot be compiled without OpenCV); see zim_oracle.c.
"""
from .oracle import *  # noqa: F401,F403
