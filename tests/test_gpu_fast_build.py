"""GPU: the fast build (libvelvet_gb300_fast.so: contracted arithmetic, approximate
division and square root, CUDA's acosf) run through the tests that do not demand bits:
the tolerance suite against the oracle, the exported hash (compiled with the exact flags
in every build, so still exact), the batched and served forms' equality with each cloth
alone (same build on both sides), the bounds and failure checks."""
import os
import subprocess
import sys
from pathlib import Path

import pytest

pytestmark = pytest.mark.gpu
ROOT = Path(__file__).resolve().parents[1]
TESTS = ["test_gpu_tolerance.py", "test_gpu_hash_objects.py", "test_gpu_batch.py", "test_gpu_server.py",
         "test_gpu_ref_golden.py", "test_zz_no_alloc.py"]


def test_fast_build_passes_the_tolerance_and_consistency_suites():
    lib = ROOT / "velvet_gb300" / "libvelvet_gb300_fast.so"
    assert lib.exists(), "the fast library is missing: run __graft_entry__.build()"
    env = dict(os.environ, VT_VARIANT="fast")
    env.pop("VT_CHECKED", None)
    r = subprocess.run([sys.executable, "-m", "pytest", *[str(ROOT / "tests" / t) for t in TESTS], "-m", "gpu",
                        "-q", "-x", "-p", "no:cacheprovider"],
                       cwd=ROOT, env=env, capture_output=True, text=True, timeout=1800)
    assert r.returncode == 0, r.stdout[-4000:] + r.stderr[-2000:]
