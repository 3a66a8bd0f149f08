"""Generate golden vectors from the reference's own step (host build, oracle/_ref).

Run here, where the reference sources exist:  python tests/golden/make_golden.py
Writes tests/golden/golden.json (SHA-256 of the bit patterns of every state array after the
listed scenes) and tests/golden/tiny_state.npz (one small scene's full final state).  The
GPU machine has no reference checkout; the parity tests there check against these files.

Scenes (all inputs from smoke_simulation_gb300.scenes, integer-valued geometry):
  tiny        12x10x11, every object kind, 5 steps (full arrays kept)
  small_a     20x16x18, 6 steps
  small_b     17x23x19, 2 obstacles (last-wins), 3 sources, 6 steps
  ref80       the 80^3 workload (sphere obstacle, box emitter, noise seed 0, 40 iterations),
              100 steps, density hash every 20 steps
  app80       the reference application's own scene (main.cpp:288-293): source r=5 at the grid
              centre, obstacle r=13 at (60,10,60), one dt=0.01 warm-up step then dt=0.05 steps
              with the default 30 iterations; the source is moved on an integer circle every
              step (updateObjectPos, main.cpp:609-614), gravity/buoyancy changed at step 10
"""
from __future__ import annotations

import hashlib
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import oracle as O  # noqa: E402
from smoke_simulation_gb300 import scenes as S  # noqa: E402


def h(a: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def state_hashes(st: dict) -> dict:
    out = {"index_now": int(st["index_now"]), "s": h(st["s"])}
    for k in ("rho", "u", "v", "w"):
        for j in range(2):
            out["%s%d" % (k, j)] = h(st[k][j])
    return out


def app80_path(step: int):
    ang = 0.3 * step
    return (float(round(40 + 20 * np.cos(ang))), 40.0, float(round(40 + 20 * np.sin(ang))))


def app80_scene() -> S.Scene:
    sc = S.Scene("app80", 80, 80, 80, dt=0.05, steps=20, iterations=30)
    sc.spheres = [(40.0, 40.0, 40.0, 5.0)]
    sc.obstacles = [(60.0, 10.0, 60.0, 0.0, 0.0, 0.0, 13.0)]
    return sc


def main():
    golden = {"generator": "reference project/smokeSimulation.cu, host build (oracle/_ref)",
              "scenes": {}}
    # tiny / small
    for name, sc in (("tiny", S.small_scene(12, 10, 11, steps=5, seed=3)),
                     ("small_a", S.small_scene()),
                     ("small_b", S.small_scene(17, 23, 19, seed=5, obstacles=2, sources=3))):
        ref = O.RefHostSim(sc)
        for _ in range(sc.steps):
            ref.step()
        st = ref.state()
        golden["scenes"][name] = {"steps": sc.steps, "final": state_hashes(st),
                                  "density_out": h(ref.out)}
        if name == "tiny":
            np.savez_compressed(os.path.join(HERE, "tiny_state.npz"),
                                **{"%s%d" % (k, j): st[k][j] for k in ("rho", "u", "v", "w")
                                   for j in range(2)}, s=st["s"], index_now=st["index_now"],
                                density_out=ref.out)
        ref.close()
    # ref80
    sc = S.config_ref80(steps=100)
    ref = O.RefHostSim(sc)
    per = {}
    for k in range(sc.steps):
        ref.step()
        if (k + 1) % 20 == 0:
            per[str(k + 1)] = h(ref.out)
    golden["scenes"]["ref80"] = {"steps": 100, "final": state_hashes(ref.state()),
                                 "density_every_20": per}
    ref.close()
    # app80
    sc = app80_scene()
    ref = O.RefHostSim(sc)
    lib = ref.lib
    per = {}
    ref.step(0.01)
    for k in range(sc.steps):
        if k == 10:
            lib.ref_set_physics(-5.0, 6.0)
        lib.ref_update_pos(0, *app80_path(k))
        ref.step(0.05)
        per[str(k + 1)] = h(ref.out)
    golden["scenes"]["app80"] = {"steps": sc.steps, "final": state_hashes(ref.state()),
                                 "density_each_step": per}
    ref.close()
    with open(os.path.join(HERE, "golden.json"), "w") as f:
        json.dump(golden, f, indent=1, sort_keys=True)
    print("wrote", os.path.join(HERE, "golden.json"))


if __name__ == "__main__":
    main()
