"""VXA formula trees (stop condition, fitness, force field, attach conditions) against the
reference's own evaluator, VX3_MathTree::eval (Voxelyze3/src/Utils/VX3_MathTree.h:50-192).

tests/golden/formulas.json holds every formula of the reference's sample worlds and a
set that uses every token of the format, each with values the reference's evaluator
computed on seeded variable sets (tests/golden/make_formulas.py).

* CPU: the host restatement (oracle/mathtree_ref.py) and the engine's host evaluation
  (vx3_inspect_formula) reproduce the reference's values.
* GPU: the evaluator the step kernels run (vx3_eval_formula, on the device) reproduces
  them within 1e-13 relative (the device's sin, cos, tan, atan, log, pow and erfc are
  within a few ulp of the host's); formulas whose value is decided by comparisons,
  rounding and logic (0/1 and integer results) match exactly.
"""
import json
import math
import os

import numpy as np
import pytest

from conftest import GOLDEN
from oracle.mathtree_ref import evaluate

import gpuvoxels_gb300 as g
from gpuvoxels_gb300 import synth

RTOL = 1e-13
CASES = json.load(open(os.path.join(GOLDEN, "formulas.json")))["cases"]


def _vxa_with(xml, which):
    """A one-voxel world whose stop condition, fitness or force field is the formula."""
    base = synth.vxa_document(np.ones((1, 1, 1), np.int32), np.zeros((1, 1, 1)), [synth.PASSIVE])
    if which == "stop":
        return base.replace("</Simulator>", f"<StopCondition><StopConditionFormula>{xml}</StopConditionFormula>"
                                            "</StopCondition></Simulator>")
    if which == "fitness":
        return base.replace("<FitnessFunction><mtVAR>x</mtVAR></FitnessFunction>", f"<FitnessFunction>{xml}</FitnessFunction>")
    return base.replace("</Simulator>", f"<ForceField><{which[-1]}_forcefield>{xml}</{which[-1]}_forcefield></ForceField></Simulator>")


def _close(got, want, exact):
    got, want = np.asarray(got, float), np.asarray([np.nan if w is None else w for w in want], float)
    if exact:
        return np.array_equal(got, want, equal_nan=True)
    same_inf = np.isinf(want) & (got == want)
    ok = np.isclose(got, want, rtol=RTOL, atol=0, equal_nan=True) | same_inf
    return bool(ok.all())


def _exact(case):
    """Formulas made of comparisons, logic, rounding and exact arithmetic only."""
    inexact = {"mtSIN", "mtCOS", "mtTAN", "mtATAN", "mtLOG", "mtPOW", "mtSQRT", "mtNORMALCDF", "mtDIV"}
    return not any(op in inexact for op, _ in case["tokens"])


def test_formula_cases_cover_every_token():
    from oracle.mathtree_ref import TOKENS
    used = {op for c in CASES for op, _ in c["tokens"]}
    assert set(TOKENS) <= used
    assert any(c["name"].startswith("Experiments/") for c in CASES)


@pytest.mark.parametrize("case", CASES, ids=[c["name"] for c in CASES])
def test_restatement_matches_reference_evaluator(case):
    toks = [(op, float(v)) for op, v in case["tokens"]]
    got = [evaluate(toks, *row) for row in case["vars"]]
    assert _close(got, case["ref"], exact=False), case["name"]


@pytest.mark.parametrize("case", CASES, ids=[c["name"] for c in CASES])
def test_engine_host_evaluation_matches_reference(case):
    vxa = _vxa_with(case["xml"], "stop")
    got = [g.eval_formula(vxa, "stop", row) for row in case["vars"]]
    assert _close(got, case["ref"], exact=False), case["name"]


@pytest.mark.gpu
@pytest.mark.parametrize("which", ["stop", "fitness", "force_x"])
def test_device_evaluation_matches_reference(ctx, which):
    for case in CASES:
        vxa = _vxa_with(case["xml"], which)
        got = ctx.eval_formula(vxa, which, np.array(case["vars"]))
        assert _close(got, case["ref"], exact=_exact(case)), (which, case["name"], got, case["ref"])


def test_long_or_malformed_formula_is_refused():
    """Formulas the evaluator cannot hold (more than 63 tokens) or parse are refused with
    VX3_E_PARSE when the world is read, instead of evaluating to NaN."""
    long_xml = "<mtVAR>t</mtVAR>"
    for _ in range(40):
        long_xml = f"<mtADD>{long_xml}<mtCONST>1</mtCONST></mtADD>"
    for xml in (long_xml, "<mtFOO><mtVAR>t</mtVAR></mtFOO>", "<mtVAR>nowhere</mtVAR>"):
        with pytest.raises(g.VX3Error):
            g.inspect_vxa(_vxa_with(xml, "stop"))
    g.inspect_vxa(_vxa_with("<mtSUB><mtVAR>t</mtVAR><mtCONST>1</mtCONST></mtSUB>", "stop"))
