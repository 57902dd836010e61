"""
Build ``damping_params.json``, the functional parameter table of
``get_params``.

tad-dftd4 keeps its damping parameters per density functional in two TOML
files (``damping/parameters/d3.toml``, ``damping/parameters/d4.toml``),
loaded by ``damping/parameters/loader.py:48-58``.  This script parses them
(Python's ``tomllib``) and stores the resulting tables unchanged, keyed by
method, so the package carries the same numbers without a TOML parser or the
reference tree at run time.

Usage::

    python make_params.py --src <tad_dftd4 source dir>
"""

from __future__ import annotations

import argparse
import json
import tomllib
from pathlib import Path

HERE = Path(__file__).resolve().parent
OUT = HERE / "damping_params.json"


def main() -> None:
    ap = argparse.ArgumentParser(description=__doc__.split("\n\n")[0])
    ap.add_argument("--src", required=True, help="tad_dftd4 source package directory")
    args = ap.parse_args()
    src = Path(args.src) / "damping" / "parameters"
    tables = {}
    for method in ("d3", "d4"):
        with (src / f"{method}.toml").open("rb") as fp:
            tables[method] = tomllib.load(fp)
    # TOML dates (publication dates in d3.toml) are stored as ISO text
    OUT.write_text(json.dumps({"source": "damping/parameters/{d3,d4}.toml of tad-dftd4",
                               "tables": tables}, sort_keys=True, separators=(",", ":"),
                              default=lambda v: v.isoformat()))
    print(f"wrote {OUT}")


if __name__ == "__main__":
    main()
