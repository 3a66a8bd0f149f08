"""Shared helpers for the parity tests (comparisons, golden access, scene drivers)."""
from __future__ import annotations

import hashlib
import json
import os

import numpy as np

GOLDEN_DIR = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")

# Tolerances for floating-point comparisons that are not bit-exact (stated per quantity):
#  pressure-form projection vs the reference's velocity-form projection, FP32, and
#  FP32 vs the FP64 oracle of the same discretisation.
DENSITY_MAX_ABS = 1e-4
DENSITY_REL_L2 = 1e-5
VELOCITY_MAX_ABS = 1e-3
VELOCITY_REL_L2 = 1e-4


def sha(a: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def golden() -> dict:
    with open(os.path.join(GOLDEN_DIR, "golden.json")) as f:
        return json.load(f)


def state_hashes(st: dict) -> dict:
    out = {"index_now": int(st["index_now"]), "s": sha(st["s"])}
    for k in ("rho", "u", "v", "w"):
        for j in range(2):
            out["%s%d" % (k, j)] = sha(np.asarray(st[k][j], np.float32))
    return out


def oracle_state(o) -> dict:
    return {"rho": o.rho, "u": o.u, "v": o.v, "w": o.w, "s": o.s, "index_now": o.index_now}


def bits_equal(a: np.ndarray, b: np.ndarray) -> bool:
    a = np.ascontiguousarray(a, np.float32)
    b = np.ascontiguousarray(b, np.float32)
    return a.shape == b.shape and np.array_equal(a.view(np.uint32), b.view(np.uint32))


def first_mismatch(a: dict, b: dict) -> str:
    for k in ("rho", "u", "v", "w"):
        for j in range(2):
            x = np.asarray(a[k][j], np.float64)
            y = np.asarray(b[k][j], np.float64)
            if not bits_equal(a[k][j], b[k][j]):
                d = np.abs(x - y)
                idx = np.unravel_index(np.nanargmax(d), d.shape)
                return "%s[%d] differs: max abs %.3g at (z,y,x)=%s" % (k, j, np.nanmax(d), idx)
    if not np.array_equal(a["s"], b["s"]):
        return "mask differs"
    if a["index_now"] != b["index_now"]:
        return "index_now differs"
    return ""


def rel_l2(a, b) -> float:
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    nb = np.linalg.norm(b)
    return float(np.linalg.norm(a - b) / (nb if nb > 0 else 1.0))


def max_abs(a, b) -> float:
    return float(np.max(np.abs(np.asarray(a, np.float64) - np.asarray(b, np.float64))))


def app80_path(step: int):
    """Integer circle for the app80 golden scene (tests/golden/make_golden.py)."""
    ang = 0.3 * step
    return (float(round(40 + 20 * np.cos(ang))), 40.0, float(round(40 + 20 * np.sin(ang))))
