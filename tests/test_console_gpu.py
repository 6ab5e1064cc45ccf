"""The console command end to end: `python -m rbergomi_gb300.console N M
num_threads path out_file` reads the reference's input files and writes its
result table (rBergomi/main.cpp:83-137)."""
import os
import subprocess
import sys

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_console_end_to_end(tmp_path):
    p = str(tmp_path) + "/"
    for name, text in [("H", "0.07 0.1"), ("eta", "2.2 2.4"), ("rho", "-0.9 -0.85"), ("T", "0.5 1.0"),
                       ("K", "0.8 1.0"), ("xi", "0.07")]:
        with open(p + f".{name}.txt", "w") as f:
            f.write(text + "\n")
    r = subprocess.run([sys.executable, "-m", "rbergomi_gb300.console", "256", "262144", "4", p, "res.txt"], cwd=ROOT,
                       capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    assert r.stdout.startswith("Time elapsed: ")
    lines = open(p + "res.txt").read().splitlines()
    assert lines[0] == "H eta rho T K price iv stat"
    rows = np.array([[float(x) for x in ln.split()] for ln in lines[1:]])
    assert rows.shape == (4, 8)
    np.testing.assert_array_equal(rows[:, :5], [[0.07, 2.2, -0.9, 0.5, 0.8], [0.07, 2.2, -0.9, 1.0, 1.0],
                                                [0.1, 2.4, -0.85, 0.5, 0.8], [0.1, 2.4, -0.85, 1.0, 1.0]])
    # testRBergLib/tests.cpp:16-44 reference prices (N = 256), within 0.005 + stat
    true = np.array([0.2149403, 0.08461882, 0.2157838, 0.07758564])
    assert np.all(np.abs(rows[:, 5] - true) < 0.005 + rows[:, 7])
    assert np.all(rows[:, 6] > 0)
