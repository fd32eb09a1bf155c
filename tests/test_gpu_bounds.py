"""The bounds-checked build (libgbdx_bounds.so, -DGBDX_BOUNDS): every kernel
family runs with its buffer indexes checked, reports no index outside its
buffer, and gives results identical to the release build's (the checks
change no arithmetic; parameter gradients, which sum over trajectories in an
order set by the work-stealing queue, to rounding).  The bounds-checked side runs in a child process
(GBDX_BOUNDS=1 selects the library per process); the first run builds it."""
import os
import subprocess
import sys

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))


def test_bounds_build_reports_nothing_and_matches_release(tmp_path):
    import bounds_cases

    out = tmp_path / "bounds.npz"
    env = dict(os.environ, GBDX_BOUNDS="1", PYTHONPATH=os.pathsep.join(
        [os.path.dirname(HERE), HERE, os.environ.get("PYTHONPATH", "")]))
    r = subprocess.run([sys.executable, os.path.join(HERE, "bounds_cases.py"), str(out)],
                       env=env, capture_output=True, text=True, timeout=1800)
    assert r.returncode == 0, r.stdout[-3000:] + r.stderr[-3000:]
    checked = dict(np.load(out))
    release = bounds_cases.run_cases()
    assert set(checked) == set(release)
    for k in release:
        if k in bounds_cases.REDUCED:
            # summed over trajectories in per-CTA partials whose membership
            # follows the work-stealing order: equal to rounding
            a, b = checked[k], release[k]
            assert np.abs(a - b).max() <= 1e-5 * np.abs(b).max(), k
        else:
            assert np.array_equal(checked[k], release[k], equal_nan=True), k
