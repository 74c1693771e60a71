#!/usr/bin/env python
"""Parameter file for the distance-Gaussian surface (pes_id 6, 'distgauss')
from a Fortran source that holds the surface as data statements in the form of
pes_malonaldehyde.f90 (shift, imorse / morse, ig1d / g1d, ig2d / g2d,
ig3d / g3d, natoms).  The term tables are read from the caller's own copy of
that file; nothing of it is stored in this repository.

    python distgauss_from_fortran.py path/to/pes_malonaldehyde.f90 params.dat

Output: one number per line, the layout of pes_distgauss (pg_device.cuh):
[natom, shift, nmorse, ng1, ng2, ng3, morse terms (k, re, al, de), 1-D terms
(k, x, a, d, s), 2-D terms (k1, k2, x1, x2, a1, a2, d, s), 3-D terms (k1, k2,
k3, x1, x2, x3, a1, a2, a3, d, s)] with 0-based distance indices k.
"""
import re
import sys


def _data_statements(text):
    """name -> list of values of every 'data name / ... /' statement."""
    out = {}
    # join continuation lines and drop comments
    lines = []
    for ln in text.splitlines():
        ln = ln.split("!")[0]
        lines.append(ln)
    src = " ".join(l.replace("&", " ") for l in lines)
    for m in re.finditer(r"\bdata\s+(\w+)\s*/([^/]*)/", src, flags=re.IGNORECASE):
        name = m.group(1).lower()
        vals = []
        for tok in m.group(2).split(","):
            tok = tok.strip()
            if not tok:
                continue
            if "*" in tok:  # Fortran repeat count n*value
                n, v = tok.split("*", 1)
                vals.extend([float(v.replace("D", "E").replace("d", "e"))] * int(n))
            else:
                vals.append(float(tok.replace("D", "E").replace("d", "e")))
        out[name] = vals
    return out


def parameters(text):
    d = _data_statements(text)
    m = re.search(r"natoms\s*=\s*(\d+)", text)
    if not m:
        raise ValueError("no natoms parameter found")
    natom = int(m.group(1))
    im, mo = d["imorse"], d["morse"]
    i1, g1 = d["ig1d"], d["g1d"]
    i2, g2 = d["ig2d"], d["g2d"]
    i3, g3 = d["ig3d"], d["g3d"]
    nm, n1, n2, n3 = len(im), len(i1), len(i2) // 2, len(i3) // 3
    if len(mo) != 3 * nm or len(g1) != 4 * n1 or len(g2) != 6 * n2 or len(g3) != 8 * n3:
        raise ValueError("term tables of inconsistent length")
    p = [natom, d["shift"][0], nm, n1, n2, n3]
    for t in range(nm):  # v_morse(re, al, de): (k, re, al, de)
        p += [im[t] - 1] + mo[3 * t:3 * t + 3]
    for t in range(n1):  # v_gauss(1, r, x, alpha, d, shift)
        p += [i1[t] - 1] + g1[4 * t:4 * t + 4]
    for t in range(n2):  # g2d(1:2) centres, (3:4) exponents, (5) depth, (6) shift
        p += [i2[2 * t] - 1, i2[2 * t + 1] - 1] + g2[6 * t:6 * t + 6]
    for t in range(n3):  # g3d(1:3), (4:6), (7), (8)
        p += [i3[3 * t] - 1, i3[3 * t + 1] - 1, i3[3 * t + 2] - 1] + g3[8 * t:8 * t + 8]
    return p


def main():
    if len(sys.argv) != 3:
        sys.stderr.write(__doc__)
        return 2
    p = parameters(open(sys.argv[1]).read())
    with open(sys.argv[2], "w") as f:
        f.write("\n".join(repr(float(v)) for v in p) + "\n")
    print("%d parameters (natom %d, %d Morse, %d/%d/%d Gaussians)" % (len(p), p[0], p[2], p[3], p[4], p[5]))
    return 0


if __name__ == "__main__":
    sys.exit(main())
