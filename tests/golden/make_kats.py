"""Regenerate tests/golden/kats.json from the reference's stand-alone check programs.

The reference ships no test suite; its sample*.f90 programs are the only
known-answer checks of the per-cell linear algebra on the hot path.  This
script reads their input literals and expected answers (as text) and writes
them to kats.json so the tests run without the reference present:

* sample.f90:26-28   2x2 symmetric eigenvalues of (8, 2, 5) -> 9, 4
* sample6.f90:38-48  real Thomas solve -> 1, 2, 3, 4
* sample2.f90:142-145 Gauss with pivoting -> 6, 17, 11 (commented case)
* sample2.f90:147-150 singular case ("error occurs") -> the reference's gauss
                      returns the zero vector (fenep.f90:621-625)
* sample2.f90:158-164 6x6 case -> 0.5, 1, 1.5, 2, 2.5, -2.5
* sample5.f90:9      [[2,1,1],[1,2,1],[1,1,2]] eigenvalues 1, 1, 4: the
                      repeated root makes Vieta's discriminant vanish and the
                      reference returns its -100 sentinel (fenep.f90:438-439)

Usage: python tests/golden/make_kats.py <path of the reference checkout>
"""
from __future__ import annotations

import json
import re
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent


def _nums(s: str):
    return [float(x.replace("d", "e")) for x in re.findall(r"-?\d+\.\d*(?:d-?\d+)?", s)]


def main(ref: Path) -> None:
    s1 = (ref / "sample.f90").read_text()
    c = _nums(re.search(r"C\(:\) = \(/(.*?)/\)", s1).group(1))
    s6 = (ref / "sample6.f90").read_text()
    arr = {k: _nums(re.search(rf"^\s*{k} = \[(.*?)\]", s6, re.M).group(1)) for k in "abcd"}
    s2 = (ref / "sample2.f90").read_text()
    # the commented 3x3 case with answer 6, 17, 11
    blk = s2[s2.index("A(1, :) = (/1.0, -2.0, 3.0/)"):]
    rows3 = [_nums(m) for m in re.findall(r"A\(\d, :\) = \(/(.*?)/\)", blk)[:3]]
    b3 = _nums(re.search(r"b\(:\) = \(/(.*?)/\)", blk).group(1))
    blk_s = s2[s2.index("A(1, :) = (/1.0, 1.0, 1.0/)  !"):]
    rows_s = [_nums(m) for m in re.findall(r"A\(\d, :\) = \(/(.*?)/\)", blk_s)[:3]]
    b_s = _nums(re.search(r"b\(:\) = \(/(.*?)/\)", blk_s).group(1))
    blk6 = s2[s2.index("A(1, :) = (/1.0, 1.0, 1.0, 1.0, -1.0, 1.0/)"):]
    rows6 = [_nums(m) for m in re.findall(r"A\(\d, :\) = \(/(.*?)/\)", blk6)[:6]]
    b6 = _nums(re.search(r"b\(:\) = \(/(.*?)/\)", blk6).group(1))
    s5 = (ref / "sample5.f90").read_text()
    a5 = _nums(re.search(r"reshape\(\[(.*?)\]", s5).group(1))
    out = {
        "eig2": {"source": "sample.f90:26-28", "a": c, "expected": [9.0, 4.0]},
        "tdma": {"source": "sample6.f90:38-48", **arr, "expected": [1.0, 2.0, 3.0, 4.0]},
        "gauss3": {"source": "sample2.f90:142-145", "A": rows3, "b": b3, "expected": [6.0, 17.0, 11.0]},
        "gauss3_singular": {"source": "sample2.f90:147-150; fenep.f90:621-625", "A": rows_s, "b": b_s,
                            "expected": [0.0, 0.0, 0.0]},
        "gauss6": {"source": "sample2.f90:158-164", "A": rows6, "b": b6,
                   "expected": [0.5, 1.0, 1.5, 2.0, 2.5, -2.5]},
        "vieta_repeated": {"source": "sample5.f90:9; fenep.f90:438-439",
                           "a": [a5[0], a5[1], a5[2], a5[4], a5[5], a5[8]], "eigenvalues": [1.0, 1.0, 4.0],
                           "expected": -100.0},
    }
    (HERE / "kats.json").write_text(json.dumps(out, indent=1) + "\n")
    print("wrote", HERE / "kats.json")


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit(f"usage: python {Path(__file__).name} <path of the reference checkout>")
    main(Path(sys.argv[1]))
