"""Generate the Partridge-Schwenke water PES tables from the reference's
Fortran source (run once, in the container that has the reference):

    python pyvibdmc_gb300/csrc/gen_ps_pes.py \
        <reference checkout>/pyvibdmc/sample_potentials/FortPots/Partridge_Schwenke_H2O/h2opes_v2.f

The PES (H. Partridge and D. W. Schwenke, J. Chem. Phys. 106, 4618 (1997))
is defined by its fitted coefficients, which are data: this script parses
the DATA statements of ``vibpot`` (h2opes_v2.f:17-392), applies the
first-call scaling of that routine (h2opes_v2.f:420-458: combination of the
c5z/cbasis/ccore/crest sets, cm^-1 -> hartree, Angstrom -> bohr) and writes

* ``gbdmc_ps_pes.cuh`` -- the constants and the three-body polynomial
  sum_j c_j (x1^a x2^b + x2^a x1^b) x3^c as straight-line nested Horner code
  (value and first derivatives) for the CUDA kernels;
* ``oracle/ps_pes_data.npz`` -- the scaled coefficients and exponents, read
  by the CPU oracle, which evaluates the sum term by term as the Fortran does.
"""
import os
import re
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))


def _numbers(text):
    return [float(t.replace("D", "e").replace("d", "e")) for t in re.findall(r"[-+]?\d+\.?\d*[DdEe][-+]?\d+|[-+]?\d+", text)]


def parse(path):
    src = open(path).read()
    # continuation lines of fixed-form Fortran start with a character in column 6
    lines = src.splitlines()
    joined, cur = [], ""
    for ln in lines:
        if ln[:1] in ("c", "C", "*", "!"):
            continue
        if len(ln) > 5 and ln[5] not in (" ", "0") and ln[:5].strip() == "":
            cur += " " + ln[6:]
        else:
            if cur:
                joined.append(cur)
            cur = ln
    joined.append(cur)
    arrays, scalars = {}, {}
    for st in joined:
        m = re.match(r"\s*data\s*\((\w+)\(i(?:,(\d))?\),i=1,245\)\s*/(.*)/\s*$", st)
        if m:
            name, col, body = m.group(1), m.group(2), m.group(3)
            vals = _numbers(body)
            assert len(vals) == 245, (name, len(vals))
            arrays[(name, int(col)) if col else name] = vals
            continue
        m = re.match(r"\s*data\s+([\w,]+)\s*/(.*)/\s*$", st)
        if m:
            names = m.group(1).split(",")
            vals = _numbers(m.group(2))
            if len(names) == len(vals):
                scalars.update(dict(zip(names, vals)))
    idx = np.array([arrays[("idx", k)] for k in (1, 2, 3)], dtype=np.int64).T  # (245, 3), 1-based
    return idx, {k: np.array(arrays[k]) for k in ("c5z", "cbasis", "ccore", "crest")}, scalars


def scale(idx, sets, sc):
    """The first-call block of vibpot (h2opes_v2.f:420-458), in the same order."""
    f5z, fbasis, fcore, frest = sc["f5z"], sc["fbasis"], sc["fcore"], sc["frest"]
    c = np.array([f5z * a + fbasis * b + fcore * cc + frest * r
                  for a, b, cc, r in zip(sets["c5z"], sets["cbasis"], sets["ccore"], sets["crest"])])
    phh1 = sc["phh1"] * f5z
    deoh = sc["deoh"] * f5z
    reoh = sc["reoh"] / 0.529177249
    b1 = sc["b1"] * 0.529177249 * 0.529177249
    c = c * 4.556335e-6
    rad = np.arccos(-1.0) / 1.8e2
    ce = np.cos(sc["thetae"] * rad)
    phh1 = phh1 * np.exp(sc["phh2"])
    phh1 = phh1 * 4.556335e-6
    phh2 = sc["phh2"] * 0.529177249
    deoh = deoh * 4.556335e-6
    roh = sc["roh"] / 0.529177249
    alphaoh = sc["alphaoh"] * 0.529177249
    c[0] = c[0] * 2.0
    return c, dict(reoh=reoh, b1=b1, ce=ce, phh1=phh1, phh2=phh2, deoh=deoh, roh=roh, alphaoh=alphaoh)


def _horner(terms, var):
    """Horner expression text of sum_k coef_k var^k from {k: expr}."""
    if not terms:
        return "0.0"
    top = max(terms)
    expr = terms[top]
    for k in range(top - 1, -1, -1):
        expr = f"fma({var}, {expr}, {terms[k]})" if k in terms else f"({var}) * ({expr})"
    return expr


def poly_code(C, name):
    """Straight-line code for sum_{a,b,c} C[a,b,c] x1^a x2^b x3^c."""
    lines = []
    A, B, K = C.shape
    q = {}
    for c in range(K):
        r = {}
        for a in range(A):
            tb = {b: f"{C[a, b, c]:.17e}" for b in range(B) if C[a, b, c] != 0.0}
            if tb:
                v = f"{name}_r{a}_{c}"
                lines.append(f"  const T {v} = {_horner(tb, 'x2')};")
                r[a] = v
        if r:
            v = f"{name}_q{c}"
            lines.append(f"  const T {v} = {_horner(r, 'x1')};")
            q[c] = v
    lines.append(f"  return {_horner(q, 'x3')};")
    return "\n".join(lines)


def main(path):
    idx, sets, sc = parse(path)
    c, k = scale(idx, sets, sc)
    e = idx - 1  # exponents
    A, B, K = int(e[:, :2].max()) + 1, int(e[:, :2].max()) + 1, int(e[:, 2].max()) + 1
    C = np.zeros((A, B, K))
    for j in range(1, 245):
        a, b, cc = e[j]
        C[a, b, cc] += c[j]
        C[b, a, cc] += c[j]
    # first derivatives of the polynomial
    D1 = np.zeros_like(C)
    D2 = np.zeros_like(C)
    D3 = np.zeros_like(C)
    for a in range(A):
        for b in range(B):
            for cc in range(K):
                if a:
                    D1[a - 1, b, cc] += a * C[a, b, cc]
                if b:
                    D2[a, b - 1, cc] += b * C[a, b, cc]
                if cc:
                    D3[a, b, cc - 1] += cc * C[a, b, cc]
    out = os.path.join(HERE, "gbdmc_ps_pes.cuh")
    with open(out, "w") as f:
        f.write("// Generated by gen_ps_pes.py from the Partridge-Schwenke water PES data\n"
                "// (h2opes_v2.f of the reference's sample potentials).  Do not edit.\n"
                "#pragma once\n\nnamespace gbdmc {\nnamespace ps {\n\n")
        f.write(f"constexpr double kC1 = {c[0]:.17e};  // constant term (c_1, doubled)\n")
        for n, v in k.items():
            f.write(f"constexpr double k_{n} = {v:.17e};\n")
        for nm, T in (("poly", C), ("dpoly1", D1), ("dpoly2", D2), ("dpoly3", D3)):
            f.write(f"\n// sum_(a,b,c) coefficient x1^a x2^b x3^c ({nm})\n"
                    f"template <typename T>\n__device__ __forceinline__ T {nm}(T x1, T x2, T x3) {{\n")
            f.write(poly_code(T, nm) + "\n}\n")
        f.write("\n}  // namespace ps\n}  // namespace gbdmc\n")
    npz = os.path.join(ROOT, "oracle", "ps_pes_data.npz")
    np.savez(npz, c=c, idx=idx, **k)
    print(out, npz, f"{int((C != 0).sum())} nonzero coefficients")


if __name__ == "__main__":
    if len(sys.argv) < 2:
        sys.exit("usage: gen_ps_pes.py <path of the reference's h2opes_v2.f>")
    main(sys.argv[1])
