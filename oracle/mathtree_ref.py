"""Test infrastructure: a host restatement of the VXA formula trees (stop condition,
fitness, force field), the checker for the engine's device evaluator.

Parsing follows VX3_SimulationManager::ParseMathTree
(Voxelyze3/src/VX3/VX3_SimulationManager.cu:157-275): the formula's XML subtree
is walked breadth-first, the (tag, text) pairs are pushed on a stack over an
mtEND token, and popping the stack gives the token list (reversed walk, mtEND
last).  Evaluation follows VX3_MathTree::eval
(Voxelyze3/src/Utils/VX3_MathTree.h:50-192): tokens are read in order into a
value queue; an operator consumes the oldest unconsumed values (binary
operators take their left operand from the second one) and appends its result;
mtEND returns the oldest unconsumed value.  Functions use Python's math module
(the C library's); mtINT rounds to nearest, ties to even (rint);
mtNORMALCDF is 0.5*erfc(-x/sqrt(2)).
"""
from __future__ import annotations

import math
import xml.etree.ElementTree as ET
from collections import deque
from typing import List, Optional, Sequence, Tuple

TOKENS = ["mtEND", "mtCONST", "mtE", "mtPI", "mtVAR", "mtADD", "mtSUB", "mtMUL", "mtDIV", "mtPOW", "mtSQRT", "mtSIN",
          "mtCOS", "mtTAN", "mtATAN", "mtLOG", "mtINT", "mtABS", "mtNOT", "mtGREATERTHAN", "mtLESSTHAN", "mtAND", "mtOR",
          "mtNORMALCDF"]
VARS = ["x", "y", "z", "hit", "t", "angle", "targetCloseness", "numClosePairs", "num_voxel"]


def parse(node: Optional[ET.Element]) -> List[Tuple[str, float]]:
    """Token list of a formula element (its children are the formula), as ParseMathTree builds it."""
    if node is None:
        return []
    walk = []
    frontier = deque([node])
    while frontier:
        t = frontier.popleft()
        for c in t:
            walk.append((c.tag.strip(), (c.text or "").rstrip()))
            frontier.append(c)
    out = []
    for tag, text in reversed(walk):
        if tag == "mtVAR":
            out.append((tag, float(VARS.index(text.strip()))))
        elif tag == "mtCONST":
            out.append((tag, float(text.strip())))
        elif tag in TOKENS:
            out.append((tag, 0.0))
        else:
            raise ValueError(f"unknown formula token {tag}")
    out.append(("mtEND", 0.0))
    return out


def _num(v: bool) -> float:
    return 1.0 if v else 0.0


def evaluate(tokens: Sequence[Tuple[str, float]], x, y, z, hit, t, angle, closeness, num_close_pairs, num_voxel) -> float:
    """VX3_MathTree::eval over a token list."""
    var = [x, y, z, hit, t, angle, closeness, float(int(num_close_pairs)), float(int(num_voxel))]
    vals: List[float] = []
    pc = 0
    for op, value in tokens:
        if op == "mtEND":
            return vals[pc]
        if op == "mtCONST":
            r = value
        elif op == "mtE":
            r = 2.71828182845904523536
        elif op == "mtPI":
            r = 3.14159265358979323846
        elif op == "mtVAR":
            r = var[int(value + 0.5)] if value < 8.5 else 0.0
        elif op in ("mtSIN", "mtCOS", "mtTAN", "mtATAN", "mtLOG", "mtINT", "mtNORMALCDF", "mtSQRT", "mtABS", "mtNOT"):
            a = vals[pc]
            pc += 1
            if op == "mtSIN":
                r = math.sin(a)
            elif op == "mtCOS":
                r = math.cos(a)
            elif op == "mtTAN":
                r = math.tan(a)
            elif op == "mtATAN":
                r = math.atan(a)
            elif op == "mtLOG":
                r = math.log(a) if a > 0 else (-math.inf if a == 0 else math.nan)
            elif op == "mtINT":
                r = float(round(a)) if math.isfinite(a) else a
            elif op == "mtNORMALCDF":
                r = 0.5 * math.erfc(-a / math.sqrt(2.0))
            elif op == "mtSQRT":
                r = math.sqrt(a) if a >= 0 else math.nan
            elif op == "mtABS":
                r = abs(a)
            else:
                r = _num(not a)
        else:
            b, a = vals[pc], vals[pc + 1]   # a is the left operand
            pc += 2
            if op == "mtADD":
                r = a + b
            elif op == "mtSUB":
                r = a - b
            elif op == "mtMUL":
                r = a * b
            elif op == "mtDIV":
                r = a / b if b != 0 else (math.copysign(math.inf, a) * math.copysign(1.0, b) if a != 0 else math.nan)
            elif op == "mtPOW":
                try:
                    r = math.pow(a, b)
                except (OverflowError, ValueError):
                    r = math.nan if a < 0 else math.inf
            elif op == "mtGREATERTHAN":
                r = _num(a > b)
            elif op == "mtLESSTHAN":
                r = _num(a < b)
            elif op == "mtAND":
                r = _num(bool(a) and bool(b))
            elif op == "mtOR":
                r = _num(bool(a) or bool(b))
            else:
                raise ValueError(op)
        if pc > len(vals):
            raise ValueError("token sequence error")
        vals.append(r)
    raise ValueError("formula without mtEND")


def formula_of(vxa: str, which: str) -> List[Tuple[str, float]]:
    """Tokens of one formula of a VXA document: 'stop', 'fitness', or 'force_x' / 'force_y' / 'force_z'."""
    root = ET.fromstring(vxa.encode("latin-1") if vxa.lstrip().startswith("<?xml") else vxa)
    path = {"stop": "Simulator/StopCondition/StopConditionFormula", "fitness": "Simulator/FitnessFunction",
            "force_x": "Simulator/ForceField/x_forcefield", "force_y": "Simulator/ForceField/y_forcefield",
            "force_z": "Simulator/ForceField/z_forcefield"}[which]
    return parse(root.find(path))
