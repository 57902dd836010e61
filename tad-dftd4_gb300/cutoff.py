"""
Real-space cutoffs, the same container as ``tad_dftd4.cutoff.Cutoff``
(``cutoff.py:36-90``; defaults ``defaults.py:26-39``).

As in the reference, ``cn`` is carried but not used by ``dftd4``: the D4
coordination number runs with its own default cutoff (30 Bohr), and only
``cn_eeq`` reaches the charge model (``dispersion/base.py:390, 401-407``).
"""

from __future__ import annotations

import torch

D4_CN_CUTOFF = 30.0
D4_CN_EEQ_CUTOFF = 25.0
D4_CN_EEQ_MAX = 8.0
D4_DISP2_CUTOFF = 60.0
D4_DISP3_CUTOFF = 40.0
D4_KCN = 7.5
D4_K4 = 4.10451
D4_K5 = 19.08857
D4_K6 = 2 * 11.28174**2


class Cutoff:
    """Collection of real-space cutoffs (Bohr)."""

    __slots__ = ("disp2", "disp3", "cn", "cn_eeq", "device", "dtype", "values")

    def __init__(self, disp2=D4_DISP2_CUTOFF, disp3=D4_DISP3_CUTOFF, cn=D4_CN_CUTOFF,
                 cn_eeq=D4_CN_EEQ_CUTOFF, device=None, dtype=None):
        self.device = device
        self.dtype = dtype if dtype is not None else torch.get_default_dtype()
        as_t = lambda v: torch.as_tensor(v, device=device, dtype=self.dtype)  # noqa: E731
        self.disp2 = as_t(disp2)
        self.disp3 = as_t(disp3)
        self.cn = as_t(cn)
        self.cn_eeq = as_t(cn_eeq)
        # the same values as host floats: reading them back from a device
        # tensor would synchronise the stream on every call
        self.values = {k: float(v) for k, v in
                       (("disp2", disp2), ("disp3", disp3), ("cn", cn), ("cn_eeq", cn_eeq))}

    def host_values(self) -> dict:
        """The cutoffs as Python floats (disp2, disp3, cn, cn_eeq)."""
        return dict(self.values)

    def __repr__(self) -> str:
        return (f"Cutoff(disp2={float(self.disp2)}, disp3={float(self.disp3)}, "
                f"cn={float(self.cn)}, cn_eeq={float(self.cn_eeq)})")


# host values of the default cutoffs (``dftd4(cutoff=None)``)
Cutoff.DEFAULTS = {"disp2": D4_DISP2_CUTOFF, "disp3": D4_DISP3_CUTOFF, "cn": D4_CN_CUTOFF,
                   "cn_eeq": D4_CN_EEQ_CUTOFF}
