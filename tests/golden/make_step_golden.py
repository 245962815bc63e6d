"""Regenerate tests/golden/step_golden.npz: the oracle's state after a few
steps of three small workloads (3D periodic with a cylinder, 3D channel with
cylinders, 2D with a cylinder).  The fixture guards the oracle against
unintended changes; it is produced by the oracle itself, because the
reference cannot be compiled here (no Fortran compiler, no FFTW).

Usage: python tests/golden/make_step_golden.py
"""
from __future__ import annotations

import ctypes as C
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

from fortran8_gb300 import abi, configs  # noqa: E402
from fortran8_gb300.solver import Solver  # noqa: E402

STEPS = {"c2": 4, "c3": 4, "c1": 6}


def golden_workload(name):
    return {"c2": configs.scaled(configs.c2_3d(), 8, 8, 8),
            "c3": configs.scaled(configs.c3_channel(), 16, 8, 8),
            "c1": configs.scaled(configs.c1_2d(), 16, 16, 1)}[name]


def main():
    lib = C.CDLL(str(ROOT / "oracle" / "liboracle_f8.so"))
    fns = abi.bind(lib, "f8o_")
    out = {}
    for name, n in STEPS.items():
        w = golden_workload(name)
        with Solver(fns, w.grid, w.phys, w.cyls) as s:
            s.load(configs.initial_state(w))
            _, drag = s.step(n)
            st = s.store()
        out[f"{name}_steps"] = np.array(n)
        for f in ("u", "v", "p", "c"):
            out[f"{name}_{f}"] = st[f]
        out[f"{name}_drag"] = drag
    np.savez_compressed(Path(__file__).parent / "step_golden.npz", **out)


if __name__ == "__main__":
    main()
