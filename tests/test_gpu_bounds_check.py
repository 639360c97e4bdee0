"""Memory safety of the kernels, checked by a build of the library whose
kernels guard every global access of the stepping, CPML-strip, recording,
imaging and gradient kernels against its buffer (-DPAM_BOUNDS_CHECK): a
violation is printed from the device ("PAM_BOUNDS site ...") and redirected
to a scratch array instead of faulting.  tests/bounds_check_run.py runs a set of
edge-case jobs (odd sizes, receivers on the update region's edges, a source
in the border, per-shot spreads, every source-field strategy, both gradients,
the smallest grid) with each build in a process of its own: the checked build
must print no violation and give bitwise the same results."""
import json
import os
import subprocess
import sys

import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _run(lib):
    r = subprocess.run([sys.executable, os.path.join(ROOT, "tests", "bounds_check_run.py"), lib], cwd=ROOT,
                       capture_output=True, text=True, timeout=900)
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-2000:]
    line = [ln for ln in r.stdout.splitlines() if ln.startswith("CHECKSUMS ")]
    assert len(line) == 1, r.stdout[-2000:]
    return r.stdout + r.stderr, json.loads(line[0][len("CHECKSUMS "):])


def test_bounds_checked_build_finds_no_violation_and_changes_nothing():
    from pseudoacousticmodeling_gb300 import build
    normal = build.build()
    checked = build.build_checked()
    log_c, sums_c = _run(checked)
    _, sums_n = _run(normal)
    violations = [ln for ln in log_c.splitlines() if "PAM_BOUNDS" in ln]
    print(f"{len(sums_c)} jobs checked; {len(violations)} guard messages")
    assert not violations, "\n".join(violations[:20])
    assert sums_c == sums_n
