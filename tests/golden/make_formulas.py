"""Generates tests/golden/formulas.json: VXA formulas with values computed by the
reference's own evaluator, VX3_MathTree::eval (Voxelyze3/src/Utils/VX3_MathTree.h:50-192),
compiled as host code (oracle/mathtree_harness.cu, `make -C oracle mathtree REF=...`).

Formulas: every stop condition, fitness function, force-field component and
attach condition in the reference's sample worlds (*.vxa under Experiments/,
zoo/ and doc/), and a set written here so that every token of the format
(mtCONST, mtE, mtPI, mtVAR with each variable, the arithmetic, mtPOW, mtSQRT,
the trigonometric functions, mtLOG, mtINT, mtABS, mtNOT, the comparisons,
mtAND, mtOR, mtNORMALCDF) appears.  Token lists come from the restated parser
(oracle/mathtree_ref.py, ParseMathTree's breadth-first, reversed walk).  Each
formula is evaluated on seeded variable sets.

    VX_REFERENCE=<reference project root> python tests/golden/make_formulas.py
"""
import glob
import json
import os
import subprocess
import sys
import xml.etree.ElementTree as ET

import numpy as np

ROOT = os.path.abspath(os.path.join(os.path.dirname(__file__), "..", ".."))
sys.path.insert(0, ROOT)

from oracle.mathtree_ref import TOKENS, parse  # noqa: E402

REF = os.environ.get("VX_REFERENCE", "")
HARNESS = os.path.join(ROOT, "oracle", "_ref", "mathtree_eval")
PATHS = {"stop": "Simulator/StopCondition/StopConditionFormula", "fitness": "Simulator/FitnessFunction",
         "force_x": "Simulator/ForceField/x_forcefield", "force_y": "Simulator/ForceField/y_forcefield",
         "force_z": "Simulator/ForceField/z_forcefield"}
V = lambda n: f"<mtVAR>{n}</mtVAR>"
C = lambda x: f"<mtCONST>{x!r}</mtCONST>"
WRITTEN = {
    "trig": f"<mtADD><mtMUL><mtSIN>{V('x')}</mtSIN><mtCOS>{V('y')}</mtCOS></mtMUL>"
            f"<mtDIV><mtTAN>{V('z')}</mtTAN><mtATAN>{V('t')}</mtATAN></mtDIV></mtADD>",
    "pow_sqrt_log_e": f"<mtSUB><mtPOW><mtABS>{V('x')}</mtABS>{C(1.5)}</mtPOW>"
                      f"<mtSQRT><mtLOG><mtADD>{V('hit')}<mtE></mtE></mtADD></mtLOG></mtSQRT></mtSUB>",
    "int_pi_normalcdf": f"<mtMUL><mtINT><mtMUL>{V('angle')}<mtPI></mtPI></mtMUL></mtINT>"
                        f"<mtNORMALCDF>{V('targetCloseness')}</mtNORMALCDF></mtMUL>",
    "logic": f"<mtOR><mtAND><mtGREATERTHAN>{V('x')}{V('y')}</mtGREATERTHAN>"
             f"<mtLESSTHAN>{V('numClosePairs')}{V('num_voxel')}</mtLESSTHAN></mtAND><mtNOT>{V('hit')}</mtNOT></mtOR>",
    "nested_mixed": f"<mtDIV><mtADD><mtMUL>{V('z')}{C(-2.5)}</mtMUL><mtNORMALCDF><mtSUB>{V('t')}{C(2.0)}</mtSUB>"
                    f"</mtNORMALCDF></mtADD><mtADD><mtABS><mtCOS>{V('angle')}</mtCOS></mtABS>{C(0.25)}</mtADD></mtDIV>",
    "int_ties_away": f"<mtINT><mtMUL>{V('num_voxel')}{C(0.37)}</mtMUL></mtINT>",
}


def reference_formulas():
    out = {}
    files = sorted(glob.glob(os.path.join(REF, "Experiments", "**", "*.vxa"), recursive=True) +
                   glob.glob(os.path.join(REF, "zoo", "**", "*.vxa"), recursive=True) +
                   glob.glob(os.path.join(REF, "doc", "**", "*.vxa"), recursive=True))
    for f in files:
        try:
            root = ET.fromstring(open(f, "rb").read())
        except ET.ParseError:
            continue
        rel = os.path.relpath(f, REF)
        for which, path in PATHS.items():
            el = root.find(path)
            if el is not None and len(el):
                xml = "".join(ET.tostring(c, encoding="unicode") for c in el)
                out.setdefault(xml, f"{rel}:{which}")
        for k in range(5):
            el = root.find(f"Simulator/AttachDetach/AttachCondition/Condition_{k}")
            if el is not None and len(el):
                xml = "".join(ET.tostring(c, encoding="unicode") for c in el)
                out.setdefault(xml, f"{rel}:attach{k}")
    return {name: xml for xml, name in out.items()}


def variable_sets(rng, n=24):
    rows = [[0.0] * 9, [1.0] * 9]
    for _ in range(n):
        rows.append([float(rng.normal(0, 0.05)), float(rng.normal(0, 0.05)), float(rng.normal(0.02, 0.02)),
                     float(rng.integers(0, 6)), float(rng.uniform(0, 5)), float(rng.uniform(-3.1, 3.1)),
                     float(rng.uniform(0, 10)), float(rng.integers(0, 21)), float(rng.integers(1, 1000))])
    return rows


def main():
    if not os.path.isdir(REF):
        sys.exit("set VX_REFERENCE to the reference's project root")
    subprocess.check_call(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "mathtree", f"REF={REF}"])
    rng = np.random.default_rng(17)
    forms = dict(reference_formulas())
    forms.update({f"written:{k}": v for k, v in WRITTEN.items()})
    cases = []
    lines = []
    for name, xml in sorted(forms.items()):
        toks = parse(ET.fromstring(f"<F>{xml}</F>"))
        rows = variable_sets(rng)
        lines.append(" ".join([str(len(toks))] + [f"{TOKENS.index(op)} {v!r}" for op, v in toks] + [str(len(rows))] +
                              [repr(x) for r in rows for x in r]))
        cases.append(dict(name=name, xml=xml, tokens=[[op, v] for op, v in toks], vars=rows))
    res = subprocess.run([HARNESS], input="\n".join(lines) + "\n", capture_output=True, text=True, check=True).stdout.split("\n")
    for c, line in zip(cases, res):
        c["ref"] = [None if x == "error" else float(x) for x in line.split()]
        assert len(c["ref"]) == len(c["vars"]), c["name"]
    used = {op for c in cases for op, _ in c["tokens"]}
    missing = [t for t in TOKENS if t not in used]
    assert not missing, missing
    with open(os.path.join(os.path.dirname(__file__), "formulas.json"), "w") as f:
        json.dump(dict(source="VX3_MathTree::eval (Voxelyze3/src/Utils/VX3_MathTree.h:50-192) compiled as host code",
                       cases=cases), f, indent=0)
    print(f"{len(cases)} formulas, {sum(len(c['vars']) for c in cases)} evaluations")


if __name__ == "__main__":
    main()
