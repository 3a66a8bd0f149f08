"""Build recipe for the oracles (test infrastructure only).

1. The restatement (oracle/smoke_oracle.cpp) -> oracle/_build/libsmoke_oracle.so.
2. The reference's own step built for the host ("oracle B"):
   a. when the reference checkout is present, project/smokeSimulation.cu is rewritten into
      oracle/_ref/ref_step_host.cpp by the text rules below (launch syntax -> host_launch,
      the three solver literals -> variables with the same default values, glm includes
      dropped: glm is unused by the simulation) and the harness oracle/ref_harness_tail.inc is
      appended;
   b. whenever oracle/_ref/ref_step_host.cpp exists, it is compiled with g++/OpenMP against the
      host shim in oracle/ref_shim/ into oracle/_ref/libsmoke_ref_host.so.
   Step 2a only runs where the reference sources are; the generated file is a build
   intermediate under oracle/_ref/ (git-ignored), so a machine without the reference can still
   run step 2b.

Both libraries are compiled without FMA contraction (-ffp-contract=off): the restatement's
float instantiation is then bit-identical to the reference's own arithmetic.

3. The reference's own kernels built for the GPU ("oracle A", a timing baseline only):
   a. when the reference checkout is present, project/smokeSimulation.cu is rewritten into
      oracle/_ref/ref_step_gpu.cu (glm includes dropped, the module header inlined, the
      iteration-count literal read from a variable with the same default) and the harness
      oracle/ref_gpu_tail.inc is appended; kernels and launches are left as they are;
   b. whenever oracle/_ref/ref_step_gpu.cu exists, nvcc compiles it for sm_103a with its
      default floating-point options (as the reference's own CMake build does) into
      oracle/_ref/libsmoke_ref_gpu.so.  Not part of the parity chain (nvcc contracts a*b+c
      into FMAs, so it differs from the host build by rounding).

4. The reference's proxy-plane geometry built for the host (the checker of smk_proxy_planes):
   where the reference checkout is present, the free functions pseudoangle, getMinMaxPoints,
   teselate, sortPoints, rayPlaneIntersection, planeBoxIntersections, duplicate and the member
   BoundingBox::generateProxyGeometry are taken verbatim from project/boundingBox.cpp (whole
   function bodies, found by their signature lines and brace matching) into
   oracle/_ref/ref_proxy_host.cpp between oracle/ref_proxy_prelude.inc (the declarations they
   need; boundingBox.h itself includes OpenGL) and oracle/ref_proxy_tail.inc (a C entry point),
   and compiled with g++ against the checkout's vendored glm (external_src/glm/include) into
   oracle/_ref/libsmoke_ref_proxy.so.  glm is not on machines without the checkout, so this
   build exists only here; tests/golden/make_golden.py records its outputs as fixtures.
"""
from __future__ import annotations

import os
import re
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
REF_OUT = os.path.join(HERE, "_ref")
# The reference checkout: SMOKE_REFERENCE_SRC names its project/smokeSimulation.cu directly;
# otherwise SMOKE_REFERENCE_ROOT names the checkout, by default a directory `reference` beside
# this repository's own checkout.
REFERENCE_ROOT = os.environ.get(
    "SMOKE_REFERENCE_ROOT", os.path.join(os.path.dirname(os.path.dirname(HERE)), "reference"))
REFERENCE_SRC = os.environ.get(
    "SMOKE_REFERENCE_SRC", os.path.join(REFERENCE_ROOT, "project", "smokeSimulation.cu"))

ORACLE_SO = os.path.join(BUILD, "libsmoke_oracle.so")
REF_CPP = os.path.join(REF_OUT, "ref_step_host.cpp")
REF_SO = os.path.join(REF_OUT, "libsmoke_ref_host.so")

CXXFLAGS = ["-O3", "-fopenmp", "-ffp-contract=off", "-fno-fast-math", "-fPIC", "-shared",
            "-std=c++17"]


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("command failed: %s\n%s\n%s" % (" ".join(cmd), r.stdout, r.stderr))


def _stale(out: str, *srcs: str) -> bool:
    if not os.path.exists(out):
        return True
    t = os.path.getmtime(out)
    return any(os.path.getmtime(s) > t for s in srcs if os.path.exists(s))


def build_restatement(force: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    srcs = [os.path.join(HERE, "smoke_oracle.cpp"), os.path.join(HERE, "render_oracle.cpp")]
    if force or any(_stale(ORACLE_SO, s) for s in srcs):
        _run(["g++", *CXXFLAGS, *srcs, "-o", ORACLE_SO])
    return ORACLE_SO


_LAUNCH = re.compile(r"([A-Za-z_][A-Za-z0-9_]*)\s*<<\s*<([^>]*)>>\s*>\s*\(")


def rewrite_reference(text: str, header: str | None) -> str:
    """Text rules applied to project/smokeSimulation.cu (never edited in place); the module's
    header project/smokeSimulation.cuh is inlined where the source includes it."""
    out = []
    for line in text.splitlines():
        s = line.strip()
        if s.startswith("#include <glm/") or s == "using namespace glm;":
            out.append("// (glm include dropped: unused by the simulation)")
            continue
        if s.startswith("#define OVER_RELAXATION"):
            out.append("#define OVER_RELAXATION ref_over_relaxation")
            continue
        if s.startswith("#define MAX_VELOCITY_PER_STEP"):
            out.append("#define MAX_VELOCITY_PER_STEP ref_max_velocity")
            continue
        if s == '#include "smokeSimulation.cuh"' and header is not None:
            out.append("// ---- project/smokeSimulation.cuh (inlined) ----")
            out.extend(header.splitlines())
            continue
        line = line.replace("int num_iterations = 30;", "int num_iterations = ref_num_iterations;")
        line = _LAUNCH.sub(lambda m: "host_launch(%s, %s, " % (m.group(2).strip(), m.group(1)), line)
        out.append(line)
    out.append('#include "ref_harness_tail.inc"')
    return "\n".join(out) + "\n"


def generate_reference_tu() -> bool:
    if not os.path.exists(REFERENCE_SRC):
        return False
    os.makedirs(REF_OUT, exist_ok=True)
    with open(REFERENCE_SRC, "r", encoding="utf-8", errors="replace") as f:
        text = f.read()
    hdr_path = os.path.join(os.path.dirname(REFERENCE_SRC), "smokeSimulation.cuh")
    with open(hdr_path, "r", encoding="utf-8", errors="replace") as f:
        header = f.read()
    new = rewrite_reference(text, header)
    if "<<<" in new.replace(" ", "") or "<< <" in new:
        raise RuntimeError("a kernel launch was left unrewritten")
    old = None
    if os.path.exists(REF_CPP):
        with open(REF_CPP) as f:
            old = f.read()
    if old != new:
        with open(REF_CPP, "w") as f:
            f.write(new)
    return True


def build_reference(force: bool = False) -> str | None:
    generate_reference_tu()
    if not os.path.exists(REF_CPP):
        return None
    deps = [REF_CPP, os.path.join(HERE, "ref_harness_tail.inc"),
            os.path.join(HERE, "ref_shim", "cuda_runtime.h")]
    if force or _stale(REF_SO, *deps):
        _run(["g++", *CXXFLAGS, "-Wno-narrowing", "-w", "-I", os.path.join(HERE, "ref_shim"),
              "-I", HERE, REF_CPP, "-o", REF_SO])
    return REF_SO


REF_GPU_CU = os.path.join(REF_OUT, "ref_step_gpu.cu")
REF_GPU_SO = os.path.join(REF_OUT, "libsmoke_ref_gpu.so")


def rewrite_reference_gpu(text: str, header: str | None) -> str:
    """Text rules for the GPU build: only what the module needs to build outside its checkout
    (glm includes dropped, its header inlined) and the iteration count as a variable."""
    out = ["static int ref_num_iterations = 30;  // num_iterations (smokeSimulation.cu:797)"]
    for line in text.splitlines():
        s = line.strip()
        if s.startswith("#include <glm/") or s == "using namespace glm;":
            out.append("// (glm include dropped: unused by the simulation)")
            continue
        if s == '#include "smokeSimulation.cuh"' and header is not None:
            out.append("// ---- project/smokeSimulation.cuh (inlined) ----")
            out.extend(header.splitlines())
            continue
        out.append(line.replace("int num_iterations = 30;",
                                "int num_iterations = ref_num_iterations;"))
    out.append('#include "ref_gpu_tail.inc"')
    return "\n".join(out) + "\n"


def generate_reference_gpu_tu() -> bool:
    if not os.path.exists(REFERENCE_SRC):
        return False
    os.makedirs(REF_OUT, exist_ok=True)
    with open(REFERENCE_SRC, "r", encoding="utf-8", errors="replace") as f:
        text = f.read()
    with open(os.path.join(os.path.dirname(REFERENCE_SRC), "smokeSimulation.cuh"), "r",
              encoding="utf-8", errors="replace") as f:
        header = f.read()
    new = rewrite_reference_gpu(text, header)
    if "num_iterations = ref_num_iterations" not in new:
        raise RuntimeError("the iteration-count literal was not found")
    old = None
    if os.path.exists(REF_GPU_CU):
        with open(REF_GPU_CU) as f:
            old = f.read()
    if old != new:
        with open(REF_GPU_CU, "w") as f:
            f.write(new)
    return True


def build_reference_gpu(force: bool = False) -> str | None:
    """oracle/_ref/libsmoke_ref_gpu.so, or None when the generated source is absent."""
    generate_reference_gpu_tu()
    if not os.path.exists(REF_GPU_CU):
        return None
    deps = [REF_GPU_CU, os.path.join(HERE, "ref_gpu_tail.inc")]
    if force or _stale(REF_GPU_SO, *deps):
        _run(["nvcc", "-O3", "-gencode", "arch=compute_103a,code=sm_103a", "-Xcompiler", "-fPIC",
              "-shared", "-w", "-I", HERE, REF_GPU_CU, "-o", REF_GPU_SO])
    return REF_GPU_SO


REF_PROXY_CPP = os.path.join(REF_OUT, "ref_proxy_host.cpp")
REF_PROXY_SO = os.path.join(REF_OUT, "libsmoke_ref_proxy.so")
BOUNDING_BOX_SRC = os.path.join(REFERENCE_ROOT, "project", "boundingBox.cpp")
GLM_INCLUDE = os.path.join(REFERENCE_ROOT, "external_src", "glm", "include")
# signature lines (at the start of a line) of the functions taken from boundingBox.cpp
PROXY_FUNCTIONS = [
    "float pseudoangle(float y, float x)",
    "void BoundingBox::generateProxyGeometry(",
    "void getMinMaxPoints(",
    "std::vector<short> teselate(",
    "void sortPoints(",
    "bool rayPlaneIntersection(",
    "std::vector<vec3> planeBoxIntersections(",
    "bool duplicate(",
]


def extract_function(text: str, signature: str) -> str:
    """The whole definition that starts with `signature` at the start of a line: from that line
    to the brace closing its body (the functions contain no braces in strings or comments)."""
    m = re.search(r"^" + re.escape(signature), text, re.M)
    if m is None:
        raise RuntimeError("function not found in boundingBox.cpp: " + signature)
    open_at = text.index("{", m.start())
    depth = 0
    for k in range(open_at, len(text)):
        if text[k] == "{":
            depth += 1
        elif text[k] == "}":
            depth -= 1
            if depth == 0:
                return text[m.start():k + 1]
    raise RuntimeError("unbalanced braces after " + signature)


def generate_reference_proxy_tu() -> bool:
    if not (os.path.exists(BOUNDING_BOX_SRC) and os.path.isdir(GLM_INCLUDE)):
        return False
    os.makedirs(REF_OUT, exist_ok=True)
    with open(BOUNDING_BOX_SRC, "r", encoding="utf-8", errors="replace") as f:
        text = f.read()
    parts = ['#include "ref_proxy_prelude.inc"']
    for sig in PROXY_FUNCTIONS:
        parts.append("// ---- from project/boundingBox.cpp ----")
        parts.append(extract_function(text, sig))
    parts.append('#include "ref_proxy_tail.inc"')
    new = "\n\n".join(parts) + "\n"
    old = None
    if os.path.exists(REF_PROXY_CPP):
        with open(REF_PROXY_CPP) as f:
            old = f.read()
    if old != new:
        with open(REF_PROXY_CPP, "w") as f:
            f.write(new)
    return True


def build_reference_proxy(force: bool = False) -> str | None:
    """oracle/_ref/libsmoke_ref_proxy.so, or None without the reference checkout and its glm."""
    if not generate_reference_proxy_tu():
        return None
    deps = [REF_PROXY_CPP, os.path.join(HERE, "ref_proxy_prelude.inc"), os.path.join(HERE, "ref_proxy_tail.inc")]
    if force or _stale(REF_PROXY_SO, *deps):
        _run(["g++", *CXXFLAGS, "-w", "-I", GLM_INCLUDE, "-I", HERE, REF_PROXY_CPP, "-o", REF_PROXY_SO])
    return REF_PROXY_SO


def build(force: bool = False) -> dict:
    generate_reference_gpu_tu()
    return {"restatement": build_restatement(force), "reference": build_reference(force)}


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
