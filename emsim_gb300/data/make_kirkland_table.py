"""Regenerate ``kirkland_fe_params.csv`` from emsim's parameter asset.

The electron scattering factor fit of Kirkland ("Advanced Computing in Electron
Microscopy", 2nd ed., Appendix C) is published data: 12 parameters per element,
f_e(q) = sum_i a_i / (q^2 + b_i) + c_i exp(-d_i q^2).  emsim ships the table as
``emsim/assets/atom_params.txt`` (parsed at ``emsim/elem.py:312-354`` into float32).
The engine needs exactly the same numbers, so this script re-expresses that table in
a plain CSV (one row per Z: a1..a3, b1..b3, c1..c3, d1..d3), rounded to float32 the
way ``emsim/elem.py:309`` rounds it.

Usage:  python emsim_gb300/data/make_kirkland_table.py path/to/emsim/assets/atom_params.txt
"""
import sys
from pathlib import Path

import numpy as np

OUT = Path(__file__).with_name("kirkland_fe_params.csv")


def main(src: Path) -> None:
    lines = src.read_text().splitlines()
    rows = []
    for z in range(1, 104):
        block = lines[(z - 1) * 4:(z - 1) * 4 + 4]
        head = block[0]
        assert int(head.split(",")[0].split("=")[1]) == z, head
        vals = [float(v) for v in " ".join(block[1:]).split()]
        assert len(vals) == 12
        # asset order per element: a1 b1 a2 b2 / a3 b3 c1 d1 / c2 d2 c3 d3
        a = vals[0:5:2]
        b = vals[1:6:2]
        c = vals[6:11:2]
        d = vals[7:12:2]
        row = np.array(a + b + c + d, dtype=np.float32)
        rows.append((z, row))
    with OUT.open("w") as f:
        f.write("# Kirkland electron scattering factor fit, float32; "
                "columns: Z,a1,a2,a3,b1,b2,b3,c1,c2,c3,d1,d2,d3\n")
        for z, row in rows:
            f.write(str(z) + "," + ",".join(repr(float(v)) for v in row) + "\n")


if __name__ == "__main__":
    if len(sys.argv) != 2:
        raise SystemExit(__doc__)
    main(Path(sys.argv[1]))
