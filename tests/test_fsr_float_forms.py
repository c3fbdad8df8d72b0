"""The FSR kernels (kittlespt_gb300/csrc/kpt_fsr.cu) replace some of the
reference's double-precision expressions with float forms; this runs the
exhaustive check tests/fsr_float_forms.c, which compares them over every
float input the kernel can see (about 2.2e9 values, a few seconds on 16
threads).  No GPU."""

import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


def test_float_forms_equal_the_double_forms(tmp_path):
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    exe = str(tmp_path / "fsr_float_forms")
    subprocess.run([cc, "-O2", "-ffp-contract=off", "-pthread", os.path.join(HERE, "fsr_float_forms.c"),
                    "-o", exe, "-lm"], check=True)
    out = subprocess.run([exe], check=True, capture_output=True, text=True, timeout=600).stdout.split()
    counts = dict(zip(out[0::2], (int(v) for v in out[1::2])))
    assert counts == {"tap_weight": 0, "one_minus_half_len": 0, "inv_lob": 0}, counts
