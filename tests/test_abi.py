"""CPU tests of the C ABI boundary: the library loads, exports every declared symbol, the
reference's C++ signatures link, and argument errors come back as status codes (no GPU
call is made here)."""
import ctypes as C
import os
import re
import subprocess
import tempfile

import pytest

import smoke_simulation_gb300 as smk

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
INCLUDE = os.path.join(ROOT, "include")


def _declared_c_symbols():
    names = set()
    for fn in os.listdir(INCLUDE):
        if not fn.endswith(".h"):
            continue
        text = open(os.path.join(INCLUDE, fn)).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        for m in re.finditer(r"\b(smk_[a-z0-9_]+)\s*\(", text):
            names.add(m.group(1))
    return sorted(names)


def _exported(path):
    out = subprocess.run(["nm", "-D", "--defined-only", path], capture_output=True, text=True,
                         check=True).stdout
    return {line.split()[-1] for line in out.splitlines() if line.strip()}


def test_every_declared_c_symbol_is_exported(smoke_lib):
    declared = _declared_c_symbols()
    assert len(declared) >= 20
    exported = _exported(smk.LIB_PATH)
    missing = [n for n in declared if n not in exported]
    assert not missing, missing
    for n in declared:
        getattr(smoke_lib, n)  # resolvable through ctypes


def test_reference_signatures_link(smoke_lib):
    """A caller written against the reference's header (main.cpp / boundingBox.cpp call
    pattern) links against the library unchanged."""
    src = r'''
#include "smokeSimulation_gb300.cuh"
#include <vector>
int main(int argc, char**) {
    if (argc > 1000) {
        std::vector<float> grid(80 * 80 * 80);
        getGPUProperties();
        initializeVolume(grid.data(), 80, 80, 80);
        int a = addSmokeSource(40, 40, 40, 5);
        addObstacle(60, 10, 60, 0, 0, 0, 13);
        updateObjectPos(a, 41, 40, 40);
        *getGravity() = -9.82f;
        *getBuoyancy() = 2.0f;
        simulate(grid.data(), 0.05f);
        deleteVolume();
    }
    return 0;
}
'''
    with tempfile.TemporaryDirectory() as d:
        cpp = os.path.join(d, "caller.cpp")
        open(cpp, "w").write(src)
        exe = os.path.join(d, "caller")
        r = subprocess.run(["g++", "-std=c++17", "-I", INCLUDE, cpp, "-o", exe,
                            smk.LIB_PATH, "-Wl,-rpath," + os.path.dirname(smk.LIB_PATH)],
                           capture_output=True, text=True)
        assert r.returncode == 0, r.stderr


def test_reference_mangled_symbols_exported(smoke_lib):
    exported = _exported(smk.LIB_PATH)
    for mangled in ("_Z16getGPUPropertiesv", "_Z8simulatePff", "_Z16initializeVolumePfjjj",
                    "_Z12deleteVolumev", "_Z11addObstaclefffffff", "_Z14addSmokeSourceffff",
                    "_Z15updateObjectPosifff", "_Z11getBuoyancyv", "_Z10getGravityv"):
        assert mangled in exported, mangled


def test_default_params_are_the_reference_constants(smoke_lib):
    p = smk.default_params()
    assert p.gravity == pytest.approx(-9.82)       # smokeSimulation.cu:28
    assert p.buoyancy == 2.0                       # :29
    assert p.omega == 1.9                          # :38
    assert p.clamp_const == 3.0                    # :39
    assert p.max_sweeps == 30                      # :797
    assert p.projection == smk.PROJECT_REFERENCE
    assert p.clamp_mode == smk.CLAMP_REFERENCE


def test_invalid_arguments_return_status_codes(smoke_lib):
    L = smoke_lib
    h = C.c_void_p()
    assert L.smk_create(0, 4, 4, None, C.byref(h)) == 1
    assert b"dimensions" in L.smk_last_error()
    p = smk.default_params(projection=7)
    assert L.smk_create(8, 8, 8, C.byref(p), C.byref(h)) == 1
    p = smk.default_params(storage=smk.STORAGE_BF16)   # BF16 needs the pressure scheme
    assert L.smk_create(8, 8, 8, C.byref(p), C.byref(h)) == 1
    p = smk.default_params(projection=1, tol=1e-4, check_every=0)
    assert L.smk_create(8, 8, 8, C.byref(p), C.byref(h)) == 1
    assert L.smk_create(4000, 4000, 4000, None, C.byref(h)) == 1  # 32-bit index limit
    assert L.smk_step(None, 0.1, None) == 1
    assert L.smk_destroy(None) == 1
    assert L.smk_error_string(2) == b"CUDA error"
