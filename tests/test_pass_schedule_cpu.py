"""CPU model of the tensor-core path kernel's pass mode 3 schedule
(rbergomi_gb300/csrc/rbg_mixed.cu: PassPlan<3>, the pass-mode-3 MMA issuers,
mma_chunk_narrow), checked against the direct causal convolution
Y2[j] = sum_{k <= j} W[k] Gamma[j - k] (the hybrid scheme's Volterra sum,
rBergLib/rBergomiMT.cpp:73-109, which the kernel computes as a block-Toeplitz
GEMM).

For 512 < Np <= 1024 the kernel cuts the columns into 256-column passes
(pass 0: n0 chunks of 32, the rest 8) that alternate between two TMEM
buffers.  While pass q's own chunks accumulate into buffer X (thread 0), the
other buffer Y takes the next pass's far-field (thread 1): each own chunk over
all 256 next-pass columns, then the cached chunks 0 .. begin(q) - 1.  The model
replays every MMA with the kernel's arguments (TMEM column, strip row, width,
overwrite flag), reads each chunk's columns where the epilogue reads them, and
checks the invariants the kernel relies on: strip rows below Np + 16, TMEM
columns below 512, cached chunk indices below ncache, a buffer handed from
thread 1 (far-field) to thread 0 (own chunks) only after thread 0's wait for
thread 1's pass, and a release wait before every buffer reuse.

The second model does the same for pass modes 1 and 2 (512-column passes that
draw the earlier chunks again), issued from two threads, one per 256-column
TMEM half: one accumulating thread per column, the chunk's signal from the
thread that owns its columns, and redrawn chunks within their strip window.
"""
import numpy as np
import pytest

KCH, HALF = 32, 256


def plan(Np):
    np2 = (Np + HALF - 1) // HALF
    n0 = (Np - HALF * (np2 - 1)) // KCH
    nc = Np // KCH
    per = HALF // KCH

    def begin(p):
        return 0 if p == 0 else n0 + per * (p - 1)

    def end(p):
        return nc if p + 1 >= np2 else n0 + per * p

    ncache = n0 + per * (np2 - 3) if np2 >= 3 else 0
    return np2, n0, nc, begin, end, ncache


def run_schedule(Np, W_tiles, gamma):
    """Replays the MMAs of every tile; returns the columns the epilogue reads."""
    np2, n0, nc, begin, end, ncache = plan(Np)
    N = len(gamma)
    gpad = np.concatenate([np.zeros(KCH), gamma, np.zeros(Np + 2 * HALF)])  # gpad[KCH + d] = Gamma[d], 0 outside

    def G(d):  # Gamma at lags d (array), zero for d < 0 or d >= N
        d = np.asarray(d)
        out = gpad[np.clip(d, -KCH, Np + 2 * HALF - 1) + KCH]
        return np.where((d >= 0) & (d < N), out, 0.0)

    tmem = np.zeros(2 * HALF)
    writers = {}      # (buffer, pass) -> threads that accumulated into it, in order
    ydone = -1        # thread 0: highest pass whose far-field (thread 1) it waited for
    waited = {0: -10, 1: -10}  # highest pass whose release was waited for, per buffer
    cache = {}
    G_pass = 0
    out = []
    for W in W_tiles:
        cols = np.zeros(Np)

        def mma(thread, G_of_buf, d, tile, jrow, n, overwrite):
            # strip rows jrow + 16 (1 - ks) + [0, n) for K halves ks = 0, 1
            assert 0 <= jrow and jrow + 16 + n - 1 <= Np + 15
            assert 0 <= d and d + n <= 2 * HALF and n % 16 == 0 and 16 <= n <= 256
            buf = d // HALF
            assert (d + n - 1) // HALF == buf  # one buffer per MMA
            seq = writers.setdefault((buf, G_of_buf), [])
            if thread == 1:
                # the far-field of a pass comes first, while the previous pass runs
                assert 0 not in seq and G_of_buf == G_pass + 1, "far-field after the pass's own chunks"
            elif 1 in seq:
                # thread 0 takes over the buffer only after the ydone wait for thread 1's pass
                assert ydone >= G_of_buf - 1, "own chunks before the far-field completed"
            seq.append(thread)
            assert G_of_buf < 2 or waited[buf] >= G_of_buf - 2, "buffer reused before its release"
            i = np.arange(n)[:, None]
            kp = np.arange(KCH)[None, :]
            val = (G(jrow + i - kp) * tile[None, :]).sum(axis=1)
            tmem[d:d + n] = val if overwrite else tmem[d:d + n] + val

        for q in range(np2):
            cb, ce = begin(q), end(q)
            P, Pn = KCH * cb, KCH * ce
            has_y = q + 1 < np2
            k, mC = ce - cb, (cb if has_y else 0)
            xb, yb = (G_pass & 1) * HALF, ((G_pass + 1) & 1) * HALF
            assert Pn - P <= HALF and (not has_y or Pn + HALF <= Np)
            u = 0
            for c in range(cb, ce):
                tile = W[KCH * c:KCH * c + KCH]
                if c == 0 and G_pass >= 2:
                    waited[G_pass & 1] = G_pass - 2
                if c == cb and q > 0:
                    ydone = G_pass - 1
                # thread 0: own chunk into this pass's columns [32 c, Pn)
                mma(0, G_pass, xb + KCH * c - P, tile, 0, Pn - KCH * c, q == 0 and c == 0)
                if c < ncache:
                    cache[c] = tile.copy()
                if has_y:
                    if c == cb and G_pass >= 1:
                        waited[(G_pass + 1) & 1] = G_pass - 1
                    # thread 1: own chunk over all 256 columns of the next pass
                    mma(1, G_pass + 1, yb, tile, Pn - KCH * c, HALF, c == cb)
                    u_end = mC * (c - cb + 1) // k
                    while u < u_end:
                        assert u < ncache and u in cache
                        mma(1, G_pass + 1, yb, cache[u], Pn - KCH * u, HALF, False)
                        u += 1
                # the epilogue reads chunk c's columns of this pass
                cols[KCH * c:KCH * c + KCH] = tmem[xb + KCH * c - P:xb + KCH * c - P + KCH]
            assert u == mC
            G_pass += 1
        out.append(cols)
    return out


@pytest.mark.parametrize("Np", list(range(544, 1025, 32)))
def test_pass_mode_3_schedule_is_the_causal_convolution(Np):
    rng = np.random.default_rng(Np)
    N = Np - (Np // KCH) % 5  # N steps padded to Np = 32 ceil(N / 32): ragged last chunks
    gamma = rng.standard_normal(N) / np.sqrt(1.0 + np.arange(N))
    tiles = [np.concatenate([rng.standard_normal(N), np.zeros(Np - N)]) for _ in range(3)]
    got = run_schedule(Np, tiles, gamma)
    for W, cols in zip(tiles, got):
        ref = np.convolve(W, np.concatenate([gamma, np.zeros(Np - N)]))[:Np]
        np.testing.assert_allclose(cols, ref, rtol=1e-11, atol=1e-11)


def test_pass_mode_3_plan_sizes():
    """Passes, first-pass chunks and cached chunks per CTA at the ends of the range."""
    assert plan(544)[:3] == (3, 1, 17) and plan(544)[5] == 1
    assert plan(768)[:3] == (3, 8, 24) and plan(768)[5] == 8
    assert plan(800)[:3] == (4, 1, 25) and plan(800)[5] == 9
    assert plan(1024)[:3] == (4, 8, 32) and plan(1024)[5] == 16
    # the cache of a CTA holds ncache A tiles of 16 KB: 256 KB per CTA at N = 1024
    assert plan(1024)[5] * 2 * 128 * 32 * 2 == 256 * 1024


def run_redraw_schedule(Np, W, gamma, windowed):
    """Pass modes 1 (Np <= 1024) and 2 (windowed: the strip's first 528 rows
    resident, redrawn chunks read a 528-row window): 512-column passes, pass 0
    n0 = (Np - 512 (np - 1)) / 32 chunks, each later pass first redraws every
    earlier chunk over all its columns, then takes its own 16.  Two issuing
    threads, thread h the MMAs into TMEM columns [256 h, 256 h + 256) of the
    pass; the thread whose half holds a chunk's columns signals them."""
    PASS, WIN = 512, 528
    npass = (Np + PASS - 1) // PASS
    n0 = (Np - PASS * (npass - 1)) // KCH
    nc = Np // KCH
    gpad = np.concatenate([np.zeros(KCH), gamma, np.zeros(2 * Np)])
    N = len(gamma)

    def G(d):
        d = np.asarray(d)
        return np.where((d >= 0) & (d < N), gpad[np.clip(d, -KCH, 2 * Np - 1) + KCH], 0.0)

    tmem = np.zeros(PASS)
    cols = np.zeros(Np)
    for q in range(npass):
        cb = 0 if q == 0 else n0 + 16 * (q - 1)
        ce = nc if q + 1 >= npass else n0 + 16 * q
        toff = KCH * cb
        writer = {}  # TMEM column -> the one thread that accumulates into it this pass
        for c in range(ce):
            redraw = c < cb
            lo, hi = (KCH * cb if redraw else KCH * c), KCH * ce
            tile = W[KCH * c:KCH * c + KCH]
            for me in (0, 1):
                mid = toff + HALF
                plo, phi = (lo, min(hi, mid)) if me == 0 else (max(lo, mid), hi)
                for col0 in range(plo, phi, HALF):
                    n = min(HALF, phi - col0)
                    d = col0 - toff
                    assert 0 <= d and d + n <= PASS and (d < HALF) == (me == 0) and (d + n - 1 < HALF) == (me == 0)
                    if windowed and redraw:
                        # rows of the window copied for this chunk: strip rows lo - 32 c + [0, 528)
                        jrow = col0 - lo
                        assert jrow + 16 + n - 1 < WIN
                    elif windowed:
                        assert col0 - KCH * c + 16 + n - 1 < WIN  # the resident first 528 rows
                    for t in range(d, d + n):
                        assert writer.setdefault(t, me) == me, "two threads accumulate into one column"
                    i = np.arange(n)[:, None]
                    kp = np.arange(KCH)[None, :]
                    val = (G(col0 - KCH * c + i - kp) * tile[None, :]).sum(axis=1)
                    tmem[d:d + n] = val if c == 0 else tmem[d:d + n] + val
            if not redraw:
                owner = 1 if KCH * c - toff >= HALF else 0
                d = KCH * c - toff
                assert all(writer[t] == owner for t in range(d, d + KCH)), "accf from a thread that does not own the columns"
                cols[KCH * c:KCH * c + KCH] = tmem[d:d + KCH]
    return cols


@pytest.mark.parametrize("Np", [544, 800, 1024, 1056, 1536, 2048, 3072, 4096])
def test_redraw_passes_two_thread_split_is_the_causal_convolution(Np):
    rng = np.random.default_rng(Np + 1)
    N = Np - (Np // KCH) % 3
    gamma = rng.standard_normal(N) / np.sqrt(1.0 + np.arange(N))
    W = np.concatenate([rng.standard_normal(N), np.zeros(Np - N)])
    cols = run_redraw_schedule(Np, W, gamma, windowed=Np > 1024)
    ref = np.convolve(W, np.concatenate([gamma, np.zeros(Np - N)]))[:Np]
    np.testing.assert_allclose(cols, ref, rtol=1e-11, atol=1e-11)
