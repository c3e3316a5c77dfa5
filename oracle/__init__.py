"""FP64 CPU restatement of the PhaseShiftGrayCode3D reconstruction path.

TEST INFRASTRUCTURE ONLY: the parity checker used by ``tests/``,
``__graft_entry__.smoke()`` and the CPU-baseline leg of ``bench.py``.  The
shipped library never imports it.

Parity status: pinned to the reference's own code for every computation the
reference has.  oracle/ref_build.py compiles the reference's decoder V2,
reconstructor V2 and CPU MLS from its sources against a minimal OpenCV
stand-in (oracle/cvshim/) into oracle/_ref/, and tests/test_ref_pin.py
requires this restatement to reproduce it (bit for bit for decode,
rectification, setData, stereoMatch, median, reprojection, radius outlier
filter and the polynomial model; to float rounding of the reference's float
sums for the pixel Gaussian; to one float ulp for MLS against the reference
source evaluated in double).  Still restated from documentation only: the
OpenCV primitives themselves (OpenCV is absent) and the computations the
reference lacks (Gray code, hierarchical unwrapping, SOR, metric Gaussian,
adjoint), which are checked against known answers and independent
implementations.
"""
from .oracle import *  # noqa: F401,F403
