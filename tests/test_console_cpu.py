"""The reference console's text formats (rBergomi/main.cpp:83-137,
rBergomi/aux.h:82-95) as rbergomi_gb300.console reads and writes them."""
import os
import shutil
import subprocess

import numpy as np
import pytest

from rbergomi_gb300 import console


def write(path, name, text):
    with open(path + f".{name}.txt", "w") as f:
        f.write(text)


def test_read_numbers_stops_like_file2vector(tmp_path):
    p = str(tmp_path) + "/"
    write(p, "H", "0.05 0.2\n\n  0.3\t1e-2 -4.5E+1")
    assert console.read_numbers(p + ".H.txt") == [0.05, 0.2, 0.3, 0.01, -45.0]
    write(p, "eta", "1.5 2.0abc 3.0")      # the stream stops inside "2.0abc"
    assert console.read_numbers(p + ".eta.txt") == [1.5, 2.0]
    write(p, "rho", "x 1 2")
    assert console.read_numbers(p + ".rho.txt") == []
    write(p, "T", ".5 +2")
    assert console.read_numbers(p + ".T.txt") == [0.5, 2.0]


def test_missing_and_empty_inputs_exit_like_the_reference(tmp_path, capsys):
    p = str(tmp_path) + "/"
    assert console.main(["64", "100", "1", p, "out.txt"]) == 27
    assert "Error while opening file" in capsys.readouterr().err
    for name, text in [("H", "0.1"), ("eta", "1.5"), ("rho", "-0.7"), ("T", "1.0"), ("K", ""), ("xi", "0.04")]:
        write(p, name, text)
    assert console.main(["64", "100", "1", p, "out.txt"]) == 17
    assert console.main(["64", "100"]) == 5


class _Res:
    def __init__(self, vals):
        cols = list(zip(*vals))
        self.H, self.eta, self.rho, self.T, self.K, self.price, self.iv, self.stat = cols


ROWS = [(0.05, 1.0, -0.98, 0.05, 1.0, 0.123456789012345, 0.2, 1.5e-5),
        (0.2, 3.0, -0.8, 2.0, 1.3, 2.0 / 3.0, float("nan"), 123456789012.0),
        (1e-7, 100.0, -0.0, 10.0, 0.999999999951, 1e300, 0.1, 7.0)]


def test_written_rows_match_cpp_stream_formatting(tmp_path):
    out = str(tmp_path / "out.txt")
    console.write_results(out, _Res(ROWS))
    lines = open(out).read().splitlines()
    assert lines[0] == "H eta rho T K price iv stat"
    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("no C++ compiler to print the reference format")
    src = tmp_path / "fmt.cpp"
    src.write_text('#include <iostream>\n#include <iomanip>\n#include <cmath>\nint main(){double v[3][8]={' +
                   ",".join("{" + ",".join(repr(x) if x == x else "NAN" for x in r) + "}" for r in ROWS) +
                   '};std::cout<<std::setprecision(10);for(int i=0;i<3;++i){for(int j=0;j<8;++j)'
                   'std::cout<<v[i][j]<<(j<7?" ":"\\n");}}\n')
    exe = tmp_path / "fmt"
    subprocess.run([cxx, "-O1", "-o", str(exe), str(src)], check=True)
    want = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.splitlines()
    assert lines[1:] == want
