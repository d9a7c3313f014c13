"""Host check of the FP32 face clipper: the shared-pool clipper against the local-memory
clipper on seeded random faces (tests/clip_host_check.cu, compiled for the host from the
library's csrc/fia_clip32.cuh).  No GPU: the kernels' clipping code itself, run on the CPU.
The GPU counterpart compares whole steps with the shared path on and off
(test_gpu_fp32.py::test_fp32_clip_shared_pool_matches_local_pool)."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def nvcc():
    for c in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", shutil.which("nvcc")):
        if c and os.path.exists(c):
            return c
    return None


@pytest.fixture(scope="module")
def checker(tmp_path_factory):
    exe = nvcc()
    if exe is None:
        pytest.skip("nvcc not found")
    out = str(tmp_path_factory.mktemp("clip") / "clip_host_check")
    # no contraction on the host: both clippers then round every operation alike
    subprocess.check_call([exe, "-std=c++17", "-O2", "-x", "cu", "-Xcompiler", "-ffp-contract=off",
                           "-I", os.path.join(ROOT, "include"), os.path.join(ROOT, "tests", "clip_host_check.cu"),
                           "-o", out])
    return out


@pytest.mark.parametrize("seed", [1, 2, 3])
def test_shared_pool_clipper_matches_local_clipper(checker, seed):
    r = subprocess.run([checker, "400000", str(seed)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    f = dict(zip(r.stdout.split()[0::2], (int(x) for x in r.stdout.split()[1::2])))
    assert f["mismatches"] == 0
    # the shared pool takes most faces, including non-convex ones clipped from both sides
    assert f["accepted"] > 0.7 * f["faces"]
    assert f["multi"] > 0
    assert f["listed"] > 0
