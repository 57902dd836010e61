"""
Generate ``params_golden.json``: what tad-dftd4's own ``get_params``
(``damping/parameters/loader.py:61-133``) returns for every functional and
variant of its ``d3.toml`` / ``d4.toml`` files, plus the outcome of calls that
fail (error type and message).  The product's lookup is checked against this
file by ``tests/test_params.py``.

Run from the repository root (needs the reference source tree)::

    python tests/golden/make_params_golden.py --src <reference>/src
"""

from __future__ import annotations

import argparse
import importlib
import json
import sys
import tomllib
from pathlib import Path

HERE = Path(__file__).resolve().parent
OUT = HERE / "params_golden.json"


def _outcome(fn, **kw):
    try:
        return {"ok": fn(**kw)}
    except Exception as exc:  # the error type and text are part of the behaviour
        return {"error": type(exc).__name__, "message": str(exc)}


def main():
    parser = argparse.ArgumentParser()
    parser.add_argument("--src", type=Path, required=True, help="reference src/ directory")
    parser.add_argument("--out", type=Path, default=OUT)
    args = parser.parse_args()
    sys.path.insert(0, str(HERE / "refstub"))
    sys.path.insert(0, str(args.src))
    sys.modules.setdefault("tomli", tomllib)
    loader = importlib.import_module("tad_dftd4.damping.parameters.loader")
    get_params = loader.get_params
    calls = []
    for method in ("d3", "d4"):
        raw = tomllib.loads((args.src / "tad_dftd4/damping/parameters"
                             / f"{method}.toml").read_text())
        variants = sorted({v for entry in raw["parameter"].values()
                           for v in entry.get(method, {})}
                          | set(raw["default"]["parameter"][method]))
        for functional in [None, "default"]:
            for variant in [None] + variants:
                calls.append({"method": method, "functional": functional,
                              "variant": variant, "keep_doi": False})
        for functional in sorted(raw["parameter"]):
            own = sorted(raw["parameter"][functional].get(method, {}))
            for variant in [None] + own:
                calls.append({"method": method, "functional": functional,
                              "variant": variant, "keep_doi": variant is None})
        calls.append({"method": method, "functional": "pbe", "variant": variants[0],
                      "keep_doi": True})
        for functional in ("PBE", "no-such-functional", "TPSSh"):
            calls.append({"method": method, "functional": functional, "variant": None,
                          "keep_doi": False})
        calls.append({"method": method, "functional": "pbe", "variant": "no-such-variant",
                      "keep_doi": False})
    for call in calls:
        call["result"] = _outcome(get_params, **{k: call[k] for k in
                                                 ("method", "functional", "variant",
                                                  "keep_doi")})
    args.out.write_text(json.dumps(calls, sort_keys=True, separators=(",", ":")))
    print("wrote", args.out, len(calls), "calls")


if __name__ == "__main__":
    main()
