"""The reference's own known-answer program, unchanged, against both solvers.

native/smoke/abi41_smoke.cpp links directly against an ABI41 library and
checks SDF, self-collision (VV, VT, EE), hard-stretch, tether / bend,
pressure and pin-weight cases, printing one SSBL_ABI41_*_OK marker per case
and exiting non-zero at the first failure.  oracle/build_ref.py compiles it
twice from the reference's sources: linked to the reference solver, and
linked to this repository's library.  Both must print every marker, and the
values each marker prints (positions at 5 decimals, counts, grid sizes) must
equal the reference's golden output recorded on a GB300
(tests/golden/abi41_smoke_reference_gb300.txt), timings excepted.
"""
import os
import re
import subprocess

import pytest

import ref_solver as R

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "abi41_smoke_reference_gb300.txt")

pytestmark = pytest.mark.gpu

MARKERS = ["SSBL_ABI41_SMOKE_START", "SSBL_ABI41_HARD_STRETCH_OK", "SSBL_ABI41_OVERPRESSURE_OK",
           "SSBL_ABI41_TACK_BENDING_OK", "SSBL_ABI41_STATIC_SDF_OK", "SSBL_ABI41_PIN_WEIGHT_OK",
           "SSBL_ABI41_SELF_COLLISION_OK", "SSBL_ABI41_SELF_VT_OK", "SSBL_ABI41_SELF_EE_OK", "SSBL_ABI41_NATIVE_OK"]


@pytest.mark.parametrize("which", ["product", "reference"])
def test_reference_smoke_program(gpu_lib, which):
    exe = R.SMOKE_PRODUCT if which == "product" else R.SMOKE_REF
    if not os.path.exists(exe):
        pytest.skip("reference smoke program not built (oracle/build_ref.py)")
    proc = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    out = proc.stdout + proc.stderr
    print(out[-3000:])
    assert proc.returncode == 0, out[-2000:]
    for m in MARKERS:
        assert re.search(rf"^{m}\b", proc.stdout, re.M), (m, out[-2000:])


def marker_values(text: str) -> dict:
    """{marker: {field: value string}} of the *_OK lines; `a->b` fields split
    into field.0 / field.1; timings dropped."""
    out = {}
    for line in text.splitlines():
        m = re.match(r"^(SSBL_ABI41_\w+_OK)\b(.*)$", line.strip())
        if not m:
            continue
        fields = {}
        for tok in m.group(2).split():
            if "=" not in tok:
                continue
            k, v = tok.split("=", 1)
            if k.endswith("_ms"):
                continue
            if "->" in v:
                a, b = v.split("->", 1)
                fields[k + ".0"], fields[k + ".1"] = a, b
            else:
                fields[k] = v
        out[m.group(1)] = fields
    return out


def test_product_smoke_values_equal_reference_golden(gpu_lib):
    if not os.path.exists(R.SMOKE_PRODUCT):
        pytest.skip("reference smoke program not built (oracle/build_ref.py)")
    proc = subprocess.run([R.SMOKE_PRODUCT], capture_output=True, text=True, timeout=300)
    assert proc.returncode == 0, proc.stderr[-2000:]
    mine = marker_values(proc.stdout)
    with open(GOLDEN) as f:
        golden = marker_values(f.read())
    assert set(golden) <= set(mine), set(golden) - set(mine)
    for marker, fields in golden.items():
        for k, v in fields.items():
            got = mine[marker].get(k)
            assert got is not None, (marker, k)
            try:
                assert abs(float(got) - float(v)) <= 1.0e-5 * max(1.0, abs(float(v))) + 1e-12, (marker, k, got, v)
            except ValueError:
                assert got == v, (marker, k, got, v)
