"""CPU test of the hex autotuner's persisted table (hephaestus_gb300/csrc/hc_tune_table.h):
appended entries read back, later lines for the same problem win, entries with an
unknown brick shape or an out-of-range CTA count are skipped, and a malformed line
ends the table."""
import os
import subprocess
import tempfile

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_tune_table_round_trip():
    d = tempfile.mkdtemp()
    exe = os.path.join(d, "tune_table_check")
    r = subprocess.run(["g++", "-O1", "-std=c++17", "-I", os.path.join(ROOT, "hephaestus_gb300", "csrc"),
                        os.path.join(ROOT, "tests", "tune_table_check.cpp"), "-o", exe],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    out = subprocess.run([exe, os.path.join(d, "tune.txt")], capture_output=True, text=True, check=True).stdout
    rows = sorted(tuple(int(v) for v in line.split()) for line in out.strip().splitlines())
    assert rows == [(1, 1, 8, 8, 8, 0, 0), (2, 0, 20, 12, 6, 0, 2)], rows
