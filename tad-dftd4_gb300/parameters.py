"""
Damping parameters per density functional: ``get_params``, the drop-in for
``tad_dftd4.damping.parameters.get_params``
(``damping/parameters/loader.py:61-133``).

The table is the reference's own (``data/damping_params.json``, built from
its ``d3.toml`` / ``d4.toml`` by ``data/make_params.py``) and the lookup has
the same rules: ``functional=None`` or ``"default"`` takes the method's
default section, otherwise the functional's section (the name is tested as
given and looked up case-folded); the variant defaults to the method's first
default variant; the ``doi`` entry is dropped unless ``keep_doi``; unknown
functionals, methods or variants raise ``KeyError``.  The block is returned
as found, without defaults merged in (``dftd4`` applies those).
"""

from __future__ import annotations

import json
from enum import Enum
from functools import lru_cache
from pathlib import Path

from .damping import Param

__all__ = ["DispersionMethod", "get_params"]

PARAMS_PATH = Path(__file__).resolve().parent / "data" / "damping_params.json"


class DispersionMethod(str, Enum):
    """Dispersion methods with parameter tables (``damping/parameters/base.py``)."""

    d3 = "d3"
    d4 = "d4"
    d5 = "d5"


@lru_cache(maxsize=None)
def _load(method: DispersionMethod) -> dict:
    tables = json.loads(PARAMS_PATH.read_text())["tables"]
    if method.value not in tables:
        raise FileNotFoundError(f"parameter table for method {method.value!r} missing")
    return tables[method.value]


def get_params(*, method: DispersionMethod | str, functional: str | None,
               variant: str | None = None, keep_doi: bool = False) -> Param:
    """Damping parameters of ``functional`` for ``method`` (and ``variant``)."""
    method = DispersionMethod(method)
    table = _load(method)
    if functional in (None, "default"):
        default_section = table["default"]
        variant_section = default_section[method.value]
        if variant not in variant_section:
            raise KeyError(f"Variant '{variant}' not found in default parameters for "
                           f"method={method.value!r}.")
        disp_method_section = default_section["parameter"]
    else:
        func_section = table["parameter"]
        if functional not in func_section:
            raise KeyError(f"Functional '{functional!r}' not found in damping parameters.")
        disp_method_section = func_section[functional.casefold()]
        if method.value not in disp_method_section:
            raise KeyError(f"Method '{method}' not found in damping parameters for "
                           f"'{functional!r}'.")
    if variant is None:
        variant = table["default"][method.value][0]
    variant_section = disp_method_section[method.value]
    if variant not in variant_section:
        raise KeyError(f"Variant '{variant}' not found for functional={functional!r}, "
                       f"method={method.value!r}.")
    out = dict(variant_section[variant])
    if not keep_doi:
        out.pop("doi", None)
    return out  # a Param mapping
