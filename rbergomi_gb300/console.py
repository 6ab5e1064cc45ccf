"""The reference console's text formats and command line (rBergomi/main.cpp).

    python -m rbergomi_gb300.console N M num_threads path out_file
    python -m rbergomi_gb300.console            # the built-in debug inputs

Inputs (main.cpp:83-95): the files ``<path>.H.txt``, ``.eta.txt``,
``.rho.txt``, ``.T.txt``, ``.K.txt`` and ``.xi.txt``, each a whitespace
separated list of numbers read until the first token that is not a number
(rBergomi/aux.h:82-95, file2vector); only xi[0] is used.  Output
(main.cpp:121-134): ``<path><out_file>`` with the header line
``H eta rho T K price iv stat`` and one row per output index, every value
printed as a C++ stream prints a double at precision 10 (printf ``%.10g``).
Pricing runs through computeIVRT_tensor on the GPU with a fresh random seed,
as the reference draws its seed words from std::random_device
(main.cpp:103-107).  Exit codes follow the reference: 5 for a wrong argument
count, 27 for an input file that cannot be opened, 17 for an empty parameter
vector.
"""
from __future__ import annotations

import os
import re
import sys
import time

import numpy as np

PARAMS = ("H", "eta", "rho", "T", "K", "xi")
HEADER = "H eta rho T K price iv stat"
# what `file >> double` accepts: optional sign, digits with an optional
# fraction (or a leading-dot fraction), optional exponent; inf / nan spellings
_NUM = re.compile(r"[+-]?(?:(?:\d+\.?\d*|\.\d+)(?:[eE][+-]?\d+)?|inf(?:inity)?|nan)", re.IGNORECASE)

DEFAULTS = dict(N=100, M=100000, num_threads=8, H=[0.05, 0.2], eta=[1.0, 3.0], rho=[-0.98, -0.8], T=[0.05, 2.0],
                K=[1.0, 1.3], xi=[0.04], path="./", out="out.txt")


class ConsoleExit(SystemExit):
    """Raised with the reference console's exit code and message."""

    def __init__(self, code: int, message: str):
        super().__init__(code)
        self.message = message


def read_numbers(fname: str) -> list[float]:
    """file2vector<double> (rBergomi/aux.h:82-95): numbers until the first token
    that does not parse as one."""
    try:
        with open(fname) as f:
            text = f.read()
    except OSError:
        raise ConsoleExit(27, f"\nError while opening file {fname}.\n")
    out = []
    for tok in text.split():
        m = _NUM.match(tok)
        if not m:
            break
        out.append(float(m.group(0)))
        if m.end() != len(tok):  # the stream stops inside this token
            break
    return out


def read_inputs(path: str) -> dict:
    """The six parameter vectors from ``<path>.<name>.txt``."""
    return {name: read_numbers(path + f".{name}.txt") for name in PARAMS}


def format_value(x: float) -> str:
    return "%.10g" % x


def write_results(fname: str, res) -> None:
    """main.cpp:121-134: header, then "H eta rho T K price iv stat" rows."""
    with open(fname, "w") as f:
        f.write(HEADER + "\n")
        for i in range(len(res.H)):
            row = (res.H[i], res.eta[i], res.rho[i], res.T[i], res.K[i], res.price[i], res.iv[i], res.stat[i])
            f.write(" ".join(format_value(float(v)) for v in row) + "\n")


def main(argv: list[str] | None = None) -> int:
    argv = sys.argv[1:] if argv is None else argv
    if len(argv) not in (0, 5):
        sys.stderr.write("Error: Wrong number of arguments.\nUsage: rBergomi N M num_threads path out_file\n")
        return 5
    try:
        if not argv:
            d = dict(DEFAULTS)
            N, M, threads, path, out = d["N"], d["M"], d["num_threads"], d["path"], d["out"]
            vec = {k: d[k] for k in PARAMS}
        else:
            N, M, threads = int(argv[0]), int(argv[1]), int(argv[2])
            path, out = argv[3], argv[4]
            sys.stderr.write(f"N = {N}, M = {M}, num_threads = {threads},\noutfile = {out}\n")
            vec = read_inputs(path)
        if any(len(v) == 0 for v in vec.values()):
            raise ConsoleExit(17, "One or more parameter vectors have size 0.\n")
    except ConsoleExit as e:
        sys.stderr.write(e.message)
        return e.code

    from . import computeIVRT_tensor

    seed = [int(x) for x in np.frombuffer(os.urandom(8 * max(1, threads)), dtype=np.uint64)]
    t0 = time.perf_counter()
    res = computeIVRT_tensor(vec["xi"][0], vec["H"], vec["eta"], vec["rho"], vec["T"], vec["K"], N, M, seed,
                             num_threads=max(1, threads))
    ms = int((time.perf_counter() - t0) * 1000)
    try:
        write_results(path + out, res)
    except OSError:
        sys.stderr.write(f"/nError while opening file {out}./n")
        return 1
    sys.stdout.write(f"Time elapsed: {ms}ms.\n")
    return 0


if __name__ == "__main__":
    sys.exit(main())
