"""CPU tests of the GPU reference baseline's build recipe (oracle A): the reference's own
project/smokeSimulation.cu, rewritten only where it must build outside its checkout, compiles
for sm_103a with the timing harness appended and exports the harness's entry points.  Nothing
here runs on a GPU; the timing itself is oracle/time_reference_gpu.py."""
import os
import shutil
import subprocess

import pytest

from oracle import build_oracle as B


def _have_reference():
    return os.path.exists(B.REFERENCE_SRC)


def test_gpu_rewrite_keeps_kernels_and_launches():
    if not _have_reference():
        pytest.skip("reference checkout absent")
    text = open(B.REFERENCE_SRC, encoding="utf-8", errors="replace").read()
    out = B.rewrite_reference_gpu(text, "// header")
    assert "num_iterations = ref_num_iterations" in out
    assert "#include <glm/" not in out
    assert '#include "ref_gpu_tail.inc"' in out
    # kernels and launch syntax are left as the reference wrote them
    for k in ("__global__ void divergence", "__global__ void velocityAdvectionU",
              "__global__ void advectSmoke", "__global__ void integrate"):
        assert k in out
    assert out.count("<< <") + out.count("<<<") == text.count("<< <") + text.count("<<<")


def test_gpu_reference_builds_and_exports_harness():
    if not _have_reference() or shutil.which("nvcc") is None:
        pytest.skip("reference checkout or nvcc absent")
    path = B.build_reference_gpu()
    assert path is not None and os.path.exists(path)
    syms = subprocess.run(["nm", "-D", "--defined-only", path], capture_output=True, text=True,
                          check=True).stdout
    for name in ("refg_init", "refg_set_iterations", "refg_set_state", "refg_simulate",
                 "refg_step_timed", "refg_delete", "refg_add_source"):
        assert name in syms, name
