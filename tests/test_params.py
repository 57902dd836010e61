"""
``get_params`` (damping/parameters/loader.py:61-133): the functional table
and the lookup rules of the reference, on the CPU.
"""

from __future__ import annotations

import importlib
from unittest.mock import patch

import pytest

from conftest import package


def params_module():
    return importlib.import_module("tad-dftd4_gb300.parameters")


def test_default_section():
    p = package().get_params(method="d4", variant="bj-eeq-atm", functional=None)
    assert p["s6"] == 1.0 and p["s9"] == 1.0 and p["alp"] == 16.0


@pytest.mark.parametrize("func", ["pbe", "b3lyp", "revpbe", "tpssh"])
def test_functionals(func):
    p = package().get_params(method="d4", variant="bj-eeq-atm", functional=func)
    assert {"a1", "a2", "s8"} <= set(p) and "doi" not in p


def test_tpssh_values_and_default_variant():
    # the values the reference's examples use (examples/d4s.py:35)
    p = package().get_params(method="d4", functional="tpssh")
    assert p == {"s8": 1.85897750, "a1": 0.44286966, "a2": 4.60230534}


def test_doi_kept_on_request():
    p = package().get_params(method="d4", variant="bj-eeq-atm", functional="pbe", keep_doi=True)
    assert "doi" in p


def test_d3_table():
    p = package().get_params(method="d3", functional="pbe")
    assert {"a1", "a2", "s8"} <= set(p)


def test_errors():
    gp = package().get_params
    with pytest.raises(KeyError):
        gp(method="d4", variant="d4-eeq-bj", functional="unknown")
    with pytest.raises(KeyError):
        gp(method="d4", functional="pbe", variant="unknown")
    with pytest.raises(KeyError, match="not found in default parameters"):
        gp(method="d4", functional=None, variant="no-such-variant")
    with pytest.raises(KeyError, match="not found for functional"):
        gp(method="d4", functional="pbe", variant="no-such-variant")
    with pytest.raises(FileNotFoundError, match="missing"):
        gp(method="d5", functional="pbe", variant="x")
    with pytest.raises(ValueError):
        gp(method="d6", functional="pbe")


def test_method_missing_in_functional():
    table = {"default": {"d4": ["bj-eeq-atm"]}, "parameter": {"pbe": {"reference": {}}}}
    mod = params_module()
    with patch.object(mod, "_load", return_value=mod._MethodTable("d4", table)):
        with pytest.raises(KeyError, match="Method"):
            mod.get_params(method="d4", functional="pbe", variant="bj-eeq-atm")


def test_every_lookup_matches_the_reference_loader():
    """Every functional / variant of the reference's d3.toml and d4.toml, and
    the failing lookups, give what the reference's own get_params returned
    (tests/golden/params_golden.json, made by make_params_golden.py)."""
    import json
    from pathlib import Path

    calls = json.loads((Path(__file__).parent / "golden" / "params_golden.json").read_text())
    gp = package().get_params
    assert len(calls) > 700
    for call in calls:
        kw = {k: call[k] for k in ("method", "functional", "variant", "keep_doi")}
        want = call["result"]
        if "ok" in want:
            assert gp(**kw) == want["ok"], kw
        else:
            with pytest.raises(KeyError) as info:
                gp(**kw)
            assert want["error"] == "KeyError", kw
            assert str(info.value) == want["message"], (kw, str(info.value))
