"""
Damping parameters per density functional: ``get_params``, the drop-in for
``tad_dftd4.damping.parameters.get_params``
(``damping/parameters/loader.py:61-133``).

The numbers are the reference's own (``data/damping_params.json``, built from
its ``d3.toml`` / ``d4.toml`` by ``data/make_params.py``).  Each method's file
is turned once into a ``_MethodTable``: the method's default variants, the
default parameter blocks, and per functional the blocks of this method (or
``None`` when the functional has no entry for it).  A lookup is then two
dictionary probes.  Observable behaviour is the reference's:

* ``functional=None`` or ``"default"`` selects the default blocks, and the
  variant must be one of the method's default variants -- so a missing
  ``variant`` is an error there, as in the reference;
* a functional name must appear in the file exactly as given, and its
  blocks are then taken under the case-folded name;
* ``variant=None`` with a functional means the method's first default
  variant;
* the ``doi`` entry is dropped unless ``keep_doi``; the block is returned as
  stored, without defaults merged in (``dftd4`` applies those);
* failures raise ``KeyError`` with the reference's messages, an unknown
  method ``ValueError``, a method without a file ``FileNotFoundError``.
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


class _MethodTable:
    """The parameter file of one dispersion method, indexed for lookups."""

    def __init__(self, method: str, raw: dict):
        self.method = method
        defaults = raw.get("default", {})
        self.default_variants: tuple = tuple(defaults.get(method, ()))
        self.default_blocks: dict = defaults.get("parameter", {}).get(method, {})
        self.functionals: dict = {name: entry.get(method)
                                  for name, entry in raw.get("parameter", {}).items()}

    def blocks(self, functional: str | None, variant: str | None) -> tuple[dict, str]:
        """The variant blocks that apply and the variant to take from them."""
        m = self.method
        if functional is None or functional == "default":
            if variant not in self.default_variants:
                raise KeyError(f"Variant '{variant}' not found in default parameters for "
                               f"method={m!r}.")
            return self.default_blocks, variant
        if functional not in self.functionals:
            raise KeyError(f"Functional '{functional!r}' not found in damping parameters.")
        folded = functional.casefold()
        if folded not in self.functionals:
            raise KeyError(folded)
        blocks = self.functionals[folded]
        if blocks is None:
            raise KeyError(f"Method '{DispersionMethod(m)}' not found in damping parameters "
                           f"for '{functional!r}'.")
        if variant is None:
            variant = self.default_variants[0]
        return blocks, variant


@lru_cache(maxsize=None)
def _load(method: DispersionMethod) -> _MethodTable:
    files = json.loads(PARAMS_PATH.read_text())["tables"]
    if method.value not in files:
        raise FileNotFoundError(f"parameter table for method {method.value!r} missing")
    return _MethodTable(method.value, files[method.value])


def get_params(*, method: DispersionMethod | str, functional: str | None,
               variant: str | None = None, keep_doi: bool = False) -> Param:
    """Damping parameters of ``functional`` for ``method`` (and ``variant``)."""
    method = DispersionMethod(method)
    table = _load(method)
    blocks, variant = table.blocks(functional, variant)
    block = blocks.get(variant)
    if block is None:
        raise KeyError(f"Variant '{variant}' not found for functional={functional!r}, "
                       f"method={method.value!r}.")
    return {k: v for k, v in block.items() if keep_doi or k != "doi"}
