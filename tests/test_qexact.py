"""The integer query quantisers (acceles_gb300/csrc/aes_qexact.hpp, used by the device kernel)
against float64 arithmetic on the CPU: random values, near-ties, exact multiples, subnormals and
arbitrary bit patterns.  No GPU."""
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)


def test_integer_quantisers_match_float64(tmp_path):
    exe = str(tmp_path / "qexact")
    subprocess.run(["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-I",
                    os.path.join(REPO, "acceles_gb300", "csrc"),
                    os.path.join(HERE, "cpp", "qexact_main.cpp"), "-o", exe], check=True)
    res = subprocess.run([exe, "1000000"], capture_output=True, text=True)
    assert res.returncode == 0, res.stdout + res.stderr
    assert "mismatches 0" in res.stdout
