"""GPU: the whole GPU suite once more on the bounds-checked build of the same sources
(VT_CHECKED=1 loads libvelvet_gb300_checked.so): every data-dependent device index is
range-checked, and any failure makes the sync calls return VT_ERR_STATE, so these
scenarios also show that no kernel reads or writes outside its arrays (the sanitizer
this pool does not offer)."""
import os
import subprocess
import sys
from pathlib import Path

import pytest

pytestmark = pytest.mark.gpu
ROOT = Path(__file__).resolve().parents[1]


def test_gpu_suite_passes_on_the_bounds_checked_build():
    lib = ROOT / "velvet_gb300" / "libvelvet_gb300_checked.so"
    assert lib.exists(), "the bounds-checked library is missing: run __graft_entry__.build()"
    env = dict(os.environ, VT_CHECKED="1")
    r = subprocess.run([sys.executable, "-m", "pytest", str(ROOT / "tests"), "-m", "gpu", "-q", "-x",
                        "-p", "no:cacheprovider", "--ignore", str(Path(__file__)),
                        "--ignore", str(Path(__file__).with_name("test_gpu_fast_build.py"))],
                       cwd=ROOT, env=env, capture_output=True, text=True, timeout=900)
    assert r.returncode == 0, r.stdout[-4000:] + r.stderr[-2000:]
