"""Regenerate tests/golden/koide_rmse.json from the reference's accuracy table.

The reference validates its 2D wall-bounded solver (fenep_2d.f90, method 3:
walls at NY/4 and 3 NY/4 of the 2 pi box, flow_type 2: Fx = 1, Re = 1,
Lp = 55, fenep_2d.f90:4-33, 1080-1143) against Koide's analytic FENE-P
Poiseuille profile (koide_theory, fenep_2d.f90:1385-1437), reporting the RMSE
of U over the channel at steady state for NX = 16, 32, 64, 128
(_theory.py:44-49):

* pattern 1: Re = 1, beta = 1 (Newtonian)
* pattern 2: Re = 1, beta = 0.9, Wi = 1
* pattern 3: Re = 1, beta = 0.9, Wi = 10

This script reads those numbers (as text) into koide_rmse.json, so the tests
run without the reference present.

The FENE-P columns were produced with Lp = 10: the oracle run to steady state
with Lp = 10 reproduces every entry to about 12 significant digits, and no
other value scanned (3 ... 100) does.  The file's header now reads Lp = 55
(fenep_2d.f90:26), a later edit; the Newtonian column does not depend on Lp.
The agreement also needs the reference's wall mode, in which the ghost rows
of C are updated with the polymer step and extrapolated only at the end of
the step (fenep_2d.f90:1371-1374, 1912-1966).

Usage: python tests/golden/make_koide.py <path of the reference checkout>
"""
from __future__ import annotations

import json
import re
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent


def main(ref: Path) -> None:
    txt = (ref / "_theory.py").read_text()
    out = {"source": "_theory.py:44-49 (fenep_dx), koide_theory fenep_2d.f90:1385-1437",
           "nx": [int(v) for v in re.search(r"x = \[(.*?)\]", txt).group(1).split(",")],
           "lp": 10.0, "re": 1.0, "patterns": {}}
    for m in re.finditer(r"if \(pattern == (\d)\): y = \[(.*?)\]\s*#\s*(.*)", txt):
        vals = [float(v) for v in m.group(2).split(",")]
        params = dict(re.findall(r"(\w+)=([\d.]+)", m.group(3)))
        out["patterns"][m.group(1)] = {"rmse": vals, "beta": float(params.get("beta", 1.0)),
                                       "wi": float(params.get("Wi", 1.0))}
    (HERE / "koide_rmse.json").write_text(json.dumps(out, indent=1) + "\n")
    print(json.dumps(out, indent=1))


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit(f"usage: python {Path(__file__).name} <path of the reference checkout>")
    main(Path(sys.argv[1]))
