"""C-ABI library checks that need no GPU: exports, host planner, exit codes."""
import ctypes as C
import os
import re
import subprocess
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "rbergomi_gb300.h")


@pytest.fixture(scope="module")
def R():
    import rbergomi_gb300 as R
    if not os.path.exists(R.LIB_PATH):
        from rbergomi_gb300 import build
        build.build()
    R.lib()
    return R


def declared_functions():
    src = open(HEADER).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"^\s*(?:void|int|const char\s*\*|uint64_t|size_t)\s*\**\s*(\w+)\s*\(", src, flags=re.M)))


def test_library_exports_every_declared_symbol(R):
    names = declared_functions()
    assert "computeIVRT_tensor" in names and "computeIVRT_tensor_quadrature" in names
    L = C.CDLL(R.LIB_PATH)
    for n in names:
        assert hasattr(L, n), n
    assert set(names) <= set(R.EXPORTS) | set(names)


def oracle_groups(H, eta, rho, T, K, N):
    """The reference trigger chain (rBergLib/rBergomiMT.cpp:490-507) replayed
    in Python: the (H_vol, H_s, T_s, H_v, eta) state each output sees."""
    O = len(T)
    eps = 1e-10
    states = []
    vol = Hs = Ts = None
    for i in range(len(H) * O):
        h, e, t = H[i // O], eta[i // O], T[i % O]
        ph = H[(i - 1) // O] if i else None
        upd = i == 0 or abs(h - ph) > eps
        if upd:
            vol = h
        upd = upd or abs(t - T[(i - 1) % O]) > eps
        if upd:
            Hs, Ts = h, t
        upd = upd or abs(e - eta[(i - 1) // O]) > eps
        if upd:
            cur = (vol, Hs, Ts, h, e)
        states.append(cur)
    return states


@pytest.mark.parametrize("case", [
    ([0.1], [1.5], [-0.7], [1.0] * 3, [0.9, 1.0, 1.1]),
    ([0.05, 0.1, 0.1, 0.3, 0.1], [1.0, 1.5, 1.5, 2.5, 1.5], [-0.95, -0.7, -0.5, -0.7, -0.3],
     [0.25, 0.25, 0.5, 1.0, 1.0, 2.0], [0.9, 1.1, 1.0, 0.8, 1.3, 2.0]),
    # near-duplicates within the 1e-10 trigger tolerance keep the earlier state
    ([0.1, 0.1 + 5e-11, 0.2], [1.0, 1.0 + 5e-11, 1.0], [-0.5, -0.5, -0.5], [1.0, 1.0 + 5e-11], [1.0, 1.1]),
])
def test_plan_matches_trigger_chain(R, case):
    H, eta, rho, T, K = case
    nv, ng, groups = R.plan_info(0.04, H, eta, rho, T, K, 64)
    states = oracle_groups(H, eta, rho, T, K, 64)
    # outputs share a variance group iff the reference reaches them in the same state
    for a in range(len(states)):
        for b in range(len(states)):
            assert (groups[a] == groups[b]) == (states[a] == states[b])
    assert nv == len({s[0] for s in states})
    assert ng == len(set(states))


def mc_rho_chain(H, eta, rho, T):
    """The plain-MC rho each output prices S with: rho at the last
    H/T/eta/rho trigger (rBergLib/rBergomiMT.cpp:239-262)."""
    O, eps = len(T), 1e-10
    out, cur = [], None
    for i in range(len(H) * O):
        q, t = i // O, i % O
        upd = i == 0 or abs(H[q] - H[(i - 1) // O]) > eps or abs(T[t] - T[(i - 1) % O]) > eps \
            or abs(eta[q] - eta[(i - 1) // O]) > eps or abs(rho[q] - rho[(i - 1) // O]) > eps
        if upd:
            cur = rho[q]
        out.append(cur)
    return out


@pytest.mark.parametrize("case", [
    ([0.1, 0.1], [1.5, 1.5], [-0.7, -0.7 + 5e-11], [1.0], [1.0]),          # stale rho kept
    ([0.1, 0.1], [1.5, 1.5], [-0.7, -0.7 + 5e-11], [1.0, 2.0], [1.0, 1.1]),  # T wrap re-triggers
    ([0.1, 0.1, 0.1], [1.5, 1.5, 1.5], [-0.7, -0.5, -0.5 - 2e-11], [0.5], [1.0]),
])
def test_mc_plan_rho_trigger(R, case):
    H, eta, rho, T, K = case
    _, _, groups, rhos = R.plan_info_mc(0.04, H, eta, rho, T, K, 64)
    np.testing.assert_array_equal(rhos, mc_rho_chain(H, eta, rho, T))
    _, _, groups_rt = R.plan_info(0.04, H, eta, rho, T, K, 64)
    np.testing.assert_array_equal(groups, groups_rt)


def test_unordered_plan_groups():
    """Unordered lists share a Volterra pass per exact H and a variance group
    per exact (H, T, eta) (rBergomi/rBergomiMT.cpp:940-957 recomputes every
    tuple, so equal tuples reach equal states)."""
    import rbergomi_gb300 as R
    rng = np.random.default_rng(5)
    n = 40
    H = rng.choice([0.05, 0.1, 0.3], n)
    eta = rng.choice([1.0, 2.0], n)
    T = rng.choice([0.5, 1.0], n)
    rho = rng.uniform(-0.9, -0.3, n)
    K = rng.uniform(0.8, 1.2, n)
    nv, ng, groups = R.plan_info_unordered(0.04, H, eta, rho, T, K, 64)
    keys = list(zip(H, T, eta))
    assert nv == len(set(H))
    assert ng == len(set(keys))
    for a in range(n):
        for b in range(n):
            assert (groups[a] == groups[b]) == (keys[a] == keys[b])
    with pytest.raises(R.RbgError):
        R.plan_info_unordered(0.04, [1.5], [1.0], [-0.5], [1.0], [1.0], 64)


def test_plan_rejects_bad_input(R):
    with pytest.raises(R.RbgError):
        R.plan_info(0.04, [0.0], [1.0], [-0.5], [1.0], [1.0], 64)
    with pytest.raises(R.RbgError):
        R.plan_info(0.04, [0.1], [1.0], [-0.5], [1.0], [1.0], 0)


def _run(code):
    return subprocess.run([sys.executable, "-c", code], cwd=ROOT, capture_output=True, text=True, timeout=120)


@pytest.mark.parametrize("fn", ["computeIVRT_tensor", "computeIV_tensor"])
def test_dropin_exit_codes(fn):
    """Size mismatch -> exit 17, num_threads < 1 -> exit 21, before any GPU work
    (rBergLib/cinterface.cpp:15-20, 38-42, 54-59)."""
    pre = ("import ctypes as C, numpy as np, rbergomi_gb300 as R\n"
           "L=R.lib(); d=lambda n: (C.c_double*n)(); s=(C.c_uint64*1)(1)\n")
    call = ("L." + fn + "(0.04, d(1), d(1), d(1), 1, d(2), d(2), 2, 8, 16, s, 1, {nt}, "
            "d(2), d(2), d(2), d(2), d(2), d(2), d(2), d(2), {out})\n")
    r = _run(pre + call.format(nt=1, out=3))
    assert r.returncode == 17 and "wrong size" in r.stderr
    r = _run(pre + call.format(nt=0, out=2))
    assert r.returncode == 21 and "positive integer" in r.stderr


@pytest.mark.parametrize("fn", ["computeIVRT_tensor", "computeIV_tensor"])
def test_dropin_empty_grid_returns(fn):
    """par_size * op_size == out_size == 0: the reference's loops run zero
    times and the call returns normally; so does the drop-in, without a GPU."""
    code = ("import ctypes as C, rbergomi_gb300 as R\n"
            "L=R.lib(); d=lambda n: (C.c_double*max(n,1))(); s=(C.c_uint64*1)(1)\n"
            "L." + fn + "(0.04, d(0), d(0), d(0), 0, d(2), d(2), 2, 8, 16, s, 1, 1, "
            "d(0), d(0), d(0), d(0), d(0), d(0), d(0), d(0), 0)\n"
            "L.computeIVRT_tensor_quadrature(0.04, d(1), d(1), d(1), 1, d(0), d(0), 0, 8, 16, d(256), 1, d(0))\n"
            "print('returned')\n")
    r = _run(code)
    assert r.returncode == 0 and "returned" in r.stdout, r.stderr
