"""Golden Fourier-coefficient tables of the WDM basis, read from cWB's own table.

cWB's WDM filter design (cwb-core/WDM.cc:497-548 getFilter, :550-594
getTDFilter1, :596-636 getTDFilter2) expands the edge of the Meyer-type
basis function in a cosine series whose coefficients it takes from
cwb-core/FourierCoefficients.icc (arrays Cos, Cos2 and SinCos for beta
orders 2..7).  pycwb_gb300.wdm recomputes those coefficients from their
definition by quadrature; this script reads the reference's table as text
and writes it to ``wdm_fourier_tables.npz`` so that the CPU tests can pin
the recomputed coefficients without the reference checkout.

Usage (needs the reference checkout; not used at test time)::

    python tests/golden/make_wdm_golden.py /path/to/pycwb-reference
"""

from __future__ import annotations

import os
import re
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))

_SIZE = re.compile(r"^\s*(Cos|Cos2|SinCos)Size\[(\d)\]\s*=\s*(\d+);")
_VAL = re.compile(r"^\s*(Cos|Cos2|SinCos)\[(\d)\]\[(\d+)\]\s*=\s*([-+0-9.eE]+);")


def read_table(path):
    sizes, vals = {}, {}
    with open(path) as f:
        for line in f:
            m = _SIZE.match(line)
            if m:
                sizes[(m.group(1), int(m.group(2)))] = int(m.group(3))
                continue
            m = _VAL.match(line)
            if m:
                vals[(m.group(1), int(m.group(2)), int(m.group(3)))] = float(m.group(4))
    out = {}
    for (kind, d), n in sizes.items():
        a = np.zeros(n, np.float64)
        for j in range(n):
            a[j] = vals.get((kind, d, j), 0.0)
        out[f"{kind.lower()}_{d}"] = a
    return out


def main(ref_root):
    tables = read_table(os.path.join(ref_root, "cwb-core", "FourierCoefficients.icc"))
    dst = os.path.join(HERE, "wdm_fourier_tables.npz")
    np.savez_compressed(dst, **tables)
    print(dst, {k: v.size for k, v in sorted(tables.items())})


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else os.environ.get("PYCWB_REFERENCE", ""))
