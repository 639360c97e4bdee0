"""Run the undamped Sd-active case of the reference-kernel parity test with
the library given on the command line (the build that divides the Sd ratio
with correct rounding) and save its seismograms.

    python tests/sd_division_run.py <library> <VTI|TTI> <amplitude> <out.npy>

Used by tests/test_gpu_reference_kernels.py in a process of its own, since a
process loads one engine library."""
import os
import sys

sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))

import numpy as np  # noqa: E402

from pseudoacousticmodeling_gb300 import _lib  # noqa: E402

_lib.load(sys.argv[1])

from tests.gpu_cases import engine_for, make_case  # noqa: E402

approx, amp, out = sys.argv[2], float(sys.argv[3]), sys.argv[4]
case = make_case(approx, "cerjan", nshots=2, seed=24, amp=amp)
e = engine_for(case)
e.set_damping(np.ones(case["grid"].N, np.float32))
np.save(out, e.forward(case["sz"], case["sx"]))
e.close()
