"""
The C ABI: the library builds, loads without a GPU, exports every function
``include/tad_dftd4_gb300.h`` declares, and the ctypes structures have the
C layout (checked against a small C program compiled with gcc).
"""

from __future__ import annotations

import ctypes
import re
import subprocess

import pytest

from conftest import REPO, package

HEADER = REPO / "include" / "tad_dftd4_gb300.h"


def declared_functions() -> list[str]:
    text = HEADER.read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(d4_[a-z_]+)\s*\(", text)))


def test_library_exports_every_declared_function():
    lib = package()._lib.load()
    names = declared_functions()
    assert len(names) >= 7
    for name in names:
        assert hasattr(lib, name), name
    assert set(names) == set(package()._lib.SIGNATURES)


def test_call_flags_match_the_header():
    """Every D4_FLAG_* of the header has its twin in the ctypes module."""
    text = HEADER.read_text()
    flags = dict(re.findall(r"#define D4_FLAG_([A-Z0-9_]+)\s+(0x[0-9a-fA-F]+|\d+)u", text))
    assert {"GRADIENT", "MIXED", "NO_HOST_WAIT"} <= set(flags)
    lib = package()._lib
    for name, value in flags.items():
        assert getattr(lib, "FLAG_" + name) == int(value, 0), name


def test_abi_version_and_status_strings():
    lib = package()._lib.load()
    assert lib.d4_abi_version() == 2
    assert lib.d4_status_string(0) == b"ok"
    assert b"EEQ" in lib.d4_status_string(5)


def test_workspace_size_is_monotone():
    lib = package()._lib.load()
    small = lib.d4_workspace_size(4, 32, 1, 0)
    grad = lib.d4_workspace_size(4, 32, 1, 1)
    big = lib.d4_workspace_size(8, 64, 1, 1)
    assert 0 < small < grad < big
    assert lib.d4_workspace_size(0, 32, 1, 0) == 0


def test_argument_errors_without_gpu():
    m = package()._lib
    lib = m.load()
    rc = lib.d4_dispersion(None, None, None, None, 0, 1, None, 0, None, None)
    assert rc == 1  # D4_ERR_ARGUMENT, no device touched
    rc = lib.d4_properties(None, None, None, None, None, 0, None, None)
    assert rc == 1


STRUCTS = {
    "d4_tables_t": ("Tables", ["n_ref_elem", "n_elem", "alpha", "refcovcn", "refc", "refq",
                               "gam", "zeff", "r4r2", "cov_d3", "en", "eeq_chi", "eeq_eta",
                               "eeq_kcn", "eeq_rad", "wfpair", "freq_weights"]),
    "d4_model_cfg_t": ("ModelCfg", ["kind", "ga", "gc", "wf"]),
    "d4_params_t": ("Params", ["s6", "s8", "s10", "a1", "a2", "s9", "alp", "has_s8",
                               "has_s10", "cut_disp2", "cut_disp3", "cut_cn", "cut_cn_eeq",
                               "cn_eeq_max", "kcn", "k4", "k5", "k6", "damping", "reserved",
                               "rs6", "rs8", "bet"]),
    "d4_batch_t": ("Batch", ["n_struct", "n_pad", "d_numbers", "d_positions", "d_charge",
                             "d_charges_in", "d_r4r2_in", "d_energy_weights",
                             "d_rvdw_in"]),
    "d4_outputs_t": ("Outputs", ["d_energy", "d_gradient", "d_charges", "d_cn",
                                 "d_param_grad", "d_cn_eeq"]),
    "d4_properties_t": ("Properties", ["d_cn", "d_charges", "d_c6", "d_alpha"]),
}


def test_struct_layout_matches_c(tmp_path):
    lines = ['#include <stdio.h>', '#include <stddef.h>', '#include "tad_dftd4_gb300.h"',
             "int main(void) {"]
    for cname, (_, fields) in STRUCTS.items():
        lines.append(f'printf("{cname} %zu\\n", sizeof({cname}));')
        for f in fields:
            lines.append(f'printf("{cname}.{f} %zu\\n", offsetof({cname}, {f}));')
    lines.append("return 0; }")
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines))
    exe = tmp_path / "layout"
    res = subprocess.run(["gcc", "-I", str(REPO / "include"), str(src), "-o", str(exe)],
                         capture_output=True, text=True)
    if res.returncode != 0:
        pytest.fail(res.stderr)
    out = dict(line.rsplit(" ", 1) for line in
               subprocess.run([str(exe)], capture_output=True, text=True).stdout.splitlines())
    m = package()._lib
    for cname, (pyname, fields) in STRUCTS.items():
        cls = getattr(m, pyname)
        assert int(out[cname]) == ctypes.sizeof(cls), cname
        assert [f for f, _ in cls._fields_] == fields, cname
        for f in fields:
            assert int(out[f"{cname}.{f}"]) == getattr(cls, f).offset, f"{cname}.{f}"
