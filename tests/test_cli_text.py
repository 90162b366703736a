"""The CLI's number formatting (emida_gb300/cli/text.hpp) gives the bytes of
printf's "%f" and "%llu", which the reference's output lines use
(src/process_files.hpp:244-260): random values over 120 binary orders of
magnitude, offset-like values and their neighbours, exact ties at the 7th
decimal, signed zeros, denormals, the largest doubles, NaN and infinities."""
import os
import subprocess

from tests.conftest import ROOT


def test_put_f_equals_printf(tmp_path):
    exe = str(tmp_path / "text_format_driver")
    subprocess.run(["g++", "-std=c++17", "-O2", os.path.join(ROOT, "tests", "text_format_driver.cpp"),
                    "-o", exe], check=True)
    r = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "0 mismatches" in r.stdout
