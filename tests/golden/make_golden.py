"""Generate tests/golden/reference_golden.json from the reference checkout.

Run in a container that has the reference sources (read-only) and g++:
    python tests/golden/make_golden.py <path of the reference checkout>

It records, as small JSON fixtures:
  gauss_1d      the tabulated Gauss-Legendre rules of orders 4, 10, 20
                (src_vie/src_operators/cubatures/gauss_1d.m)
  nearby        the singular-pair tables of nearby_correct.m:5-143 as class
                codes (0 regular, 1 ST, 2 EAc, 3 EAo, 4 VAc, 5 VAo)
  cubature_nop  6x6 face-pair integrals from the reference C++
                (mexcubatures/cubature_nop.cpp) at several offsets
  directfn      the five singular integrals from the reference DIRECTFN C++
                cores (directfn_ws_{st,ea,va}_const.cpp) with the geometry of
                singular_st/ea/va.m, at Np_1D = 20 (the reference default) and
                64, and at Np_1D = 20 for further frequencies
  directfn_tri  single calls of the three cores through the MEX gateways'
                vertex order, on seeded random triangles, Np_1D 8/12/20

The reference C++ is compiled from its own sources by oracle/Makefile into
oracle/_ref/ (outside the repository history).
"""
from __future__ import annotations

import ctypes
import json
import re
import subprocess
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
OUT = Path(__file__).resolve().parent / "reference_golden.json"
FREQ = 298e6
C0 = 299792458.0


def parse_gauss(ref: Path, orders=(4, 10, 20)):
    txt = (ref / "src_vie/src_operators/cubatures/gauss_1d.m").read_text(errors="replace")
    out = {}
    for n in orders:
        m = re.search(r"order == %d \)(.*?)(elseif|else\b)" % n, txt, re.S)
        body = m.group(1)
        xs = dict((int(i), float(v.replace(" ", ""))) for i, v in re.findall(r"xtab\((\d+)\)\s*=\s*([-\s\d.eE+]+);", body))
        ws = dict((int(i), float(v.replace(" ", ""))) for i, v in re.findall(r"weight\((\d+)\)\s*=\s*([-\s\d.eE+]+);", body))
        out[str(n)] = {"x": [xs[i] for i in range(1, n + 1)], "w": [ws[i] for i in range(1, n + 1)]}
    return out


def parse_nearby(ref: Path):
    src = (ref / "src_vie/src_operators/nearby_correct.m").read_text(errors="replace")
    src = "\n".join(l.split("%")[0] for l in src.split("\n"))
    names = {"ST": 1, "EAc": 2, "EAo": 3, "VAc": 4, "VAo": 5}
    out = {}
    for mx, my, mz, body in re.findall(r"isequal\(m,\[(\d),(\d),(\d)\]\)(.*?)(?=elseif|\nend)", src, re.S):
        Cm = re.search(r"C\s*=\s*\[(.*?)\];", body, re.S).group(1)
        Pm = re.search(r"P\s*=\s*\[(.*?)\];", body, re.S).group(1)
        Cr = [r.split() for r in Cm.strip().split("\n")]
        Pr = [[float(x) for x in r.split()] for r in Pm.strip().split("\n")]
        codes = [[0 if Pr[i][j] == 1.0 else names.get(Cr[i][j], -1) for j in range(6)] for i in range(6)]
        out[f"{int(mx) - 1},{int(my) - 1},{int(mz) - 1}"] = codes
    return out


def parse_nearby_kop(ref: Path):
    """The ST entries of the C tables of nearby_correct_kop.m (the only pairs
    that routine changes), as 0/1 matrices per offset."""
    src = (ref / "src_vie/src_operators/cubatures/nearby_correct_kop.m").read_text(errors="replace")
    src = "\n".join(l.split("%")[0] for l in src.split("\n"))
    out = {}
    for mx, my, mz, body in re.findall(r"m == \[(\d),(\d),(\d)\];(.*?)(?=elseif|\nend)", src, re.S):
        Cm = re.search(r"C\s*=\s*\[(.*?)\];", body, re.S).group(1)
        Cr = [r.split() for r in Cm.strip().split("\n")]
        out[f"{int(mx) - 1},{int(my) - 1},{int(mz) - 1}"] = [[1 if Cr[i][j] == "ST" else 0 for j in range(6)]
                                                             for i in range(6)]
    return out


def cubature_kop_cases():
    sys.path.insert(0, str(ROOT))
    from oracle import vie_oracle as vo

    lib = ctypes.CDLL(str(ROOT / "oracle/_ref/libref_cubature_kop.so"))
    cases = []
    for dx in (5e-3, 2e-3):
        ko = 2 * np.pi * FREQ / C0
        Rf = vo.cube_faces(dx, dx, dx)
        Rcol = np.asfortranarray(Rf).reshape(-1, order="F")
        for order in (4, 10):
            Np, w, u, v = vo.gauss_2d(order)
            for m in ((1, 0, 0), (0, 2, 1), (3, 1, 2), (5, 0, 0), (7, 6, 5), (2, 2, 2)):
                r_m = np.array(m, dtype=float) * dx
                out = np.zeros(6)
                lib.ref_cubature_kop(ctypes.c_int(Np), _ptr(w), _ptr(u), _ptr(v), _ptr(r_m), _ptr(np.zeros(3)),
                                     _ptr(Rcol), ctypes.c_double(ko), _ptr(out))
                cases.append({"dx": dx, "ko": ko, "order": order, "m": list(m),
                              "re": out[0::2].tolist(), "im": out[1::2].tolist()})
    return cases


def build_ref(ref: Path):
    subprocess.run(["make", "-C", str(ROOT / "oracle"), f"REF={ref}"], check=True, capture_output=True)


def _ptr(a):
    return np.ascontiguousarray(a, dtype=np.float64).ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def cubature_cases():
    sys.path.insert(0, str(ROOT))
    from oracle import vie_oracle as vo

    lib = ctypes.CDLL(str(ROOT / "oracle/_ref/libref_cubature_nop.so"))
    cases = []
    for dx in (5e-3, 2e-3):
        ko = 2 * np.pi * FREQ / C0
        Rf = vo.cube_faces(dx, dx, dx)
        Rcol = np.asfortranarray(Rf).reshape(-1, order="F")
        for order in (4, 10):
            Np, w, u, v = vo.gauss_2d(order)
            for m in ((1, 0, 0), (0, 2, 1), (3, 1, 2), (5, 0, 0), (7, 6, 5), (2, 2, 2)):
                r_m = np.array(m, dtype=float) * dx
                out = np.zeros(72)
                lib.ref_cubature_nop(ctypes.c_int(Np), _ptr(w), _ptr(u), _ptr(v), _ptr(r_m), _ptr(np.zeros(3)),
                                     _ptr(Rcol), ctypes.c_double(ko), ctypes.c_double(dx), _ptr(out))
                I = out.reshape(6, 6, 2)
                cases.append({"dx": dx, "ko": ko, "order": order, "m": list(m),
                              "re": I[..., 0].tolist(), "im": I[..., 1].tolist()})
    return cases


def directfn_values(ko, dx, Np):
    R = str(ROOT / "oracle/_ref/")
    st = ctypes.CDLL(R + "/libref_directfn_st.so")
    ea = ctypes.CDLL(R + "/libref_directfn_ea.so")
    va = ctypes.CDLL(R + "/libref_directfn_va.so")

    def cst(a, b, c):
        o = np.zeros(2)
        st.ref_directfn_st(_ptr(a), _ptr(b), _ptr(c), ctypes.c_double(ko), ctypes.c_int(Np), _ptr(o))
        return o[0] + 1j * o[1]

    def cea(a, b, c, d):
        o = np.zeros(2)
        ea.ref_directfn_ea(_ptr(a), _ptr(b), _ptr(c), _ptr(d), ctypes.c_double(ko), ctypes.c_int(Np), _ptr(o))
        return o[0] + 1j * o[1]

    def cva(a, b, c, d, e):
        o = np.zeros(2)
        va.ref_directfn_va(_ptr(a), _ptr(b), _ptr(c), _ptr(d), _ptr(e), ctypes.c_double(ko), ctypes.c_int(Np), _ptr(o))
        return o[0] + 1j * o[1]

    A = np.array
    r1, r2, r3, r4 = A([0, 0, 0.]), A([dx, 0, 0.]), A([dx, dx, 0.]), A([0, dx, 0.])
    # singular_st.m:10-22
    ST = cst(r1, r2, r3) + cea(r1, r3, r2, r4) + cea(r1, r3, r4, r2) + cst(r1, r3, r4)
    # singular_ea.m:10-31
    r5, r6, r5o, r6o = A([2 * dx, 0, 0.]), A([2 * dx, dx, 0.]), A([dx, 0, dx]), A([dx, dx, dx])
    EAc = cea(r2, r3, r1, r5) + cva(r3, r1, r2, r5, r6) + cva(r3, r4, r1, r2, r5) + cva(r3, r4, r1, r5, r6)
    EAo = cea(r2, r3, r1, r5o) + cva(r3, r1, r2, r5o, r6o) + cva(r3, r4, r1, r2, r5o) + cva(r3, r4, r1, r5o, r6o)
    # singular_va.m:10-35
    r5, r6, r7 = A([2 * dx, dx, 0.]), A([2 * dx, 2 * dx, 0.]), A([dx, 2 * dx, 0.])
    r5o, r6o, r7o = A([dx, dx, dx]), A([dx, 2 * dx, dx]), A([dx, 2 * dx, 0.])
    VAc = cva(r3, r1, r2, r5, r6) + cva(r3, r1, r2, r6, r7) + cva(r3, r4, r1, r5, r6) + cva(r3, r4, r1, r6, r7)
    VAo = (cva(r3, r1, r2, r5o, r6o) + cva(r3, r1, r2, r6o, r7o) + cva(r3, r4, r1, r5o, r6o)
           + cva(r3, r4, r1, r6o, r7o))
    v = [ST, EAc, EAo, VAc, VAo]
    return {"re": [x.real for x in v], "im": [x.imag for x in v]}


def directfn_tri_cases():
    """Single calls of the three DIRECTFN cores on seeded random vertices
    (gateway argument order: st r1..r3, ea r1..r4, va r1..r5)."""
    R = str(ROOT / "oracle/_ref/")
    libs = {"st": (ctypes.CDLL(R + "/libref_directfn_st.so").ref_directfn_st, 3),
            "ea": (ctypes.CDLL(R + "/libref_directfn_ea.so").ref_directfn_ea, 4),
            "va": (ctypes.CDLL(R + "/libref_directfn_va.so").ref_directfn_va, 5)}
    rng = np.random.default_rng(20240)
    cases = []
    for kind, (fn, nv) in libs.items():
        for Np in (8, 12, 20):
            for _ in range(3):
                r = rng.uniform(-1.0, 1.0, size=(nv, 3)) * rng.choice([1e-3, 5e-3, 0.3])
                ko = float(rng.uniform(0.5, 40.0))
                o = np.zeros(2)
                fn(*[_ptr(v) for v in r], ctypes.c_double(ko), ctypes.c_int(Np), _ptr(o))
                cases.append({"kind": kind, "Np": Np, "ko": ko, "r": r.tolist(), "re": o[0], "im": o[1]})
    return cases


def main(ref: Path):
    build_ref(ref)
    ko = 2 * np.pi * FREQ / C0
    direct = []
    for dx in (5e-3, 2e-3, 3e-3, 1e-2):
        direct.append({"ko": ko, "dx": dx, "Np": 20, **directfn_values(ko, dx, 20)})
    direct.append({"ko": ko, "dx": 5e-3, "Np": 64, **directfn_values(ko, 5e-3, 64)})
    for f in (64e6, 128e6, 447e6, 3e9):
        k = 2 * np.pi * f / C0
        direct.append({"ko": k, "dx": 5e-3, "Np": 20, **directfn_values(k, 5e-3, 20)})
    data = {
        "freq": FREQ,
        "gauss_1d": parse_gauss(ref),
        "nearby": parse_nearby(ref),
        "cubature_nop": cubature_cases(),
        "nearby_kop_st": parse_nearby_kop(ref),
        "cubature_kop": cubature_kop_cases(),
        "directfn": direct,
        "directfn_tri": directfn_tri_cases(),
    }
    OUT.write_text(json.dumps(data, indent=1))
    print(f"wrote {OUT}")


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: make_golden.py <path of the reference checkout>")
    main(Path(sys.argv[1]))
