"""Extract the inputs of the reference's own unit cases into reference_cases.json.

The reference (MEDYAN 5.4.0 inside whwh13/picgo) cannot be compiled here, so
its Catch2 cases that pin this path are re-run against the oracle and the GPU
path from the inputs they hold.  This script reads those test sources as text
and returns the numbers (coordinates, bead sets, constants, CG problem).  The
tests call extract() at run time and skip where the reference tree is absent:
the reference's licence bars redistributing its material, so the values are
not committed.  The cases:

* Mechanics/ForceField/Volume/TestCylinderExclVolume.cpp:13-47   (split-segment scaling)
* Mechanics/ForceField/Volume/TestCylinderExclVolume.cpp:49-101  (integral vs monomer energy)
* Mechanics/ForceField/Volume/TestCylinderExclVolume.cpp:103-166 (energy/force consistency)
* Mechanics/ForceField/Boundary/TestBoundaryBeadRepulsion.cpp:13-96
* Mechanics/Minimizer/TestCGMethod.cpp:9-93

Usage:  python tests/golden/make_reference_fixtures.py [reference_root [out.json]]  (a local copy for inspection)
"""
from __future__ import annotations

import json
import os
import re
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
DEFAULT_ROOT = "/root/reference"
TESTS = "medyan-5.4.0/src/TESTS/Mechanics"


def _nums(s: str):
    out = []
    for tok in re.findall(r"[-+]?(?:\d+\.\d*|\.\d+|\d+)(?:[eE][-+]?\d+)?", s):
        out.append(float(tok))
    return out


def _braced(src: str, start: int) -> tuple[str, int]:
    """Text inside the brace pair opening at or after ``start``."""
    i = src.index("{", start)
    depth = 0
    for j in range(i, len(src)):
        if src[j] == "{":
            depth += 1
        elif src[j] == "}":
            depth -= 1
            if depth == 0:
                return src[i + 1:j], j + 1
    raise ValueError("unbalanced braces")


def _var(src: str, name: str, after: int = 0):
    m = re.compile(r"\b" + re.escape(name) + r"\s*\{").search(src, after)
    if not m:
        raise KeyError(name)
    body, _ = _braced(src, m.start())
    body = re.sub(r"//[^\n]*", "", body)
    return _nums(body)


def exvol_cases(root):
    src = open(os.path.join(root, TESTS, "ForceField/Volume/TestCylinderExclVolume.cpp")).read()
    i_scale = src.index("Cylinder excl volume scaling")
    i_cons = src.index("Cylinder excl volume consistency")
    i_ef = src.index('TEST_CASE("Force field: Cylinder excl volume"')
    scaling = dict(
        coord=_var(src, "coord", i_scale),
        beadSet0=[int(v) for v in _var(src, "beadSet0", i_scale)],
        k0=_var(src, "k0", i_scale), eqLength0=_var(src, "eqLength0", i_scale),
        beadSet1=[int(v) for v in _var(src, "beadSet1", i_scale)],
        k1=_var(src, "k1", i_scale), eqLength1=_var(src, "eqLength1", i_scale),
    )
    seg = src[i_cons:i_ef]
    eqlen = _nums(re.search(r"eqLen\s*=\s*([^;]+);", seg).group(1))[0]
    kvol = _nums(re.search(r"kvol\s*=\s*([^;]+);", seg).group(1))[0]
    nmon = int(_nums(re.search(r"numMon\s*=\s*([^;]+);", seg).group(1))[0])
    # CylinderVolumeEachInteractionInfo initializer: coord indices, monomer range, interval
    info_body, _ = _braced(seg, seg.index("CylinderVolumeEachInteractionInfo iinfo"))
    info_body = re.sub(r"//[^\n]*", "", info_body)
    cyl_bodies = []
    pos = 0
    for _ in range(2):
        b, pos = _braced(info_body, pos)
        cyl_bodies.append(b)
    cyls = []
    for b in cyl_bodies:
        parts = [p.strip() for p in b.split(",") if p.strip()]
        c1, c2 = int(parts[0]), int(parts[1])
        lo = int(eval(parts[2].replace("numMon", str(nmon))))
        hi = int(eval(parts[3].replace("numMon", str(nmon))))
        itv = int(parts[4])
        cyls.append(dict(c1Index=c1, c2Index=c2, monIndexAtMinus=lo, monIndexPastPlus=hi, monInterval=itv,
                         monEqLen=eqlen / nmon))
    consistency = dict(coord=_var(seg, "coord"), beadSet=[int(v) for v in _var(seg, "beadSet")],
                       eqLen=eqlen, kvol=kvol, numMon=nmon, cyl1=cyls[0], cyl2=cyls[1], relEps=1e-2)
    ef = []
    seg = src[i_ef:src.index("if(false)", i_ef)]
    for m in re.finditer(r'testInputs\.push_back\(\{\s*"([^"]+)"', seg):
        body_start = m.end()
        groups = []
        pos = body_start
        for _ in range(4):
            b, pos = _braced(seg, pos)
            groups.append(_nums(re.sub(r"//[^\n]*", "", b)))
        ef.append(dict(name=m.group(1), beadSet=[int(v) for v in groups[0]], k=groups[1], eqLength=groups[2],
                       coord=groups[3]))
    mm = re.search(r"moveMag\s*=.*?:\s*([0-9.eE+-]+)\s*;", src[i_ef:])
    rr = re.search(r"diffDeRelEps\s*=.*?:\s*([0-9.eE+-]+)\s*;", src[i_ef:])
    return dict(scaling=scaling, consistency=consistency, energy_force=ef,
                moveMag=float(mm.group(1)), relEps=float(rr.group(1)), repsTot=10, repsPassReq=9)


def boundary_case(root):
    src = open(os.path.join(root, TESTS, "ForceField/Boundary/TestBoundaryBeadRepulsion.cpp")).read()
    m = re.search(r"PlaneBoundaryElement element1\(\{([^}]*)\},\s*\{([^}]*)\},\s*([^,]+),\s*([^)]+)\)", src)
    point, normal = _nums(m.group(1)), _nums(m.group(2))
    mm = re.search(r"moveMag\s*=.*?:\s*([0-9.eE+-]+)\s*;", src)
    rr = re.search(r"diffDeRelEps\s*=.*?:\s*([0-9.eE+-]+)\s*;", src)
    return dict(point=point, normal=normal, numNeighbors=[int(v) for v in _var(src, "numNeighbors")],
                coords=_var(src, "coords"), kreps=_var(src, "kreps"), slens=_var(src, "slens"),
                beadSet=[int(v) for v in _var(src, "beadSet")], moveMag=float(mm.group(1)),
                relEps=float(rr.group(1)), repsTot=10, repsPassReq=9)


def cg_case(root):
    src = open(os.path.join(root, TESTS, "Minimizer/TestCGMethod.cpp")).read()
    n = int(re.search(r"constexpr int n\s*=\s*(\d+);", src).group(1))
    opt = _var(src, "optCoord")
    w = _var(src, "weight")
    inits_body, _ = _braced(src, src.index("inits"))
    inits = []
    # vector<floatingpoint>(count, value): a vector of `count` copies of `value`;
    # only the first n entries are degrees of freedom.
    m = re.search(r"vector<floatingpoint>\((\d+),\s*n\)", inits_body)
    inits.append([float(n)] * n if m and int(m.group(1)) >= n else None)
    inits.append(list(opt))                      # already at the minimum
    last, _ = _braced(inits_body, inits_body.rindex("vector<floatingpoint>{"))
    inits.append(_nums(last))
    prm = dict(gradTol=float(re.search(r"gradTol\s*=\s*([0-9.eE+-]+);", src).group(1)),
               maxDist=float(re.search(r"maxDist\s*=\s*([0-9.eE+-]+);", src).group(1)),
               lambdaMax=float(re.search(r"lambdaMax\s*=\s*([0-9.eE+-]+);", src).group(1)),
               tryToRecover=0, energyRelTol=1e-9, forceCallLimit=10000)
    return dict(n=n, optCoord=opt, weight=w, inits=inits, params=prm,
                methods=["steepest", "fletcherRieves", "polakRibiere"])


def extract(root: str = DEFAULT_ROOT) -> dict:
    """The inputs of the reference's unit cases, read from its test sources under ``root``."""
    return dict(source="whwh13/picgo medyan-5.4.0 Catch2 cases", exvol=exvol_cases(root),
                boundary=boundary_case(root), cg=cg_case(root))


def available(root: str = DEFAULT_ROOT) -> bool:
    return os.path.isdir(os.path.join(root, TESTS))


def main(argv):
    root = argv[1] if len(argv) > 1 else DEFAULT_ROOT
    path = argv[2] if len(argv) > 2 else os.path.join(HERE, "reference_cases.json")
    with open(path, "w") as fh:
        json.dump(extract(root), fh, indent=1)
    print("wrote", path)


if __name__ == "__main__":
    main(sys.argv)
