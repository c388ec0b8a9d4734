"""CPU checks of the four-step LDE kernels' index arithmetic (zorch_gb300/
csrc/zc_ntt.cu), restated in Python: the radix-pass member offsets, the
twiddle indexing, the per-thread work mappings of both passes (every word
loaded, scaled and stored exactly once, inside its buffer) and the plan
limits the mappings rely on, for every shape the library accepts."""

from __future__ import annotations

import itertools

import pytest

K_THREADS, K_LOG_THREADS = 512, 9


def pad(i: int) -> int:
    return i + (i >> 5)


def row_stride(m: int) -> int:
    return pad(m) | 1


def passes(logm: int, max_r: int) -> list[tuple[int, int]]:
    """(h0, R) of each balanced pass, as smem_ntt_dif splits the stages."""
    n = (logm + max_r - 1) // max_r
    out, h0 = [], logm - 1
    for q in range(n):
        r = (h0 + 1 + (n - q) - 1) // (n - q)
        out.append((h0, r))
        h0 -= r
    assert h0 == -1
    return out


def plan(log_k: int, log_b: int, tile_log: int = 14) -> dict:
    """plan_lde's four-step split and tile shapes."""
    lk2 = log_k // 2
    lk1 = log_k - lk2
    ti = tile_log - lk2
    if lk2 >= 12 and ti < 3:
        ti = 3
    ti = max(0, min(ti, lk1))
    tt = max(0, min(tile_log - lk1 - log_b, lk2))
    return {"lk1": lk1, "lk2": lk2, "lti": ti, "ltt": tt}


@pytest.mark.parametrize("max_r", [2, 3, 4])
def test_radix_pass_member_offsets_are_shared_by_all_groups(max_r):
    """pad(base + j S) == pad(base) + pad(j S) for every group of every pass
    (the identity dif_pass uses to share member offsets), and the twiddle
    index (off + jm S) << sh == (off << sh) + jm (S << sh)."""
    for logm in range(1, 13):
        for h0, r in passes(logm, max_r):
            ls = h0 - r + 1
            s_ = 1 << ls
            sh0 = logm - 1 - h0
            for g in range(1 << (logm - r)):
                off, blk = g & (s_ - 1), g >> ls
                base = (blk << (h0 + 1)) | off
                for j in range(1 << r):
                    assert pad(base + j * s_) == pad(base) + pad(j * s_), (logm, h0, r, g, j)
                for st in range(r):
                    hb = r - 1 - st
                    for jm in range(1 << hb):
                        pos = off + (jm << ls)
                        assert pos << (sh0 + st) == (off << (sh0 + st)) + jm * (s_ << (sh0 + st))
                        assert pos << (sh0 + st) < max(1, (1 << logm) // 2)


SHAPES = [(lk, lb, tl) for lk in range(13, 25) for lb in range(0, 5) for tl in (13, 14, 15)
          if lk + lb <= 27]


@pytest.mark.parametrize("log_k,log_b,tile", SHAPES)
def test_four_step_plan_limits(log_k, log_b, tile):
    """The mappings assume TI <= kThreads and b*TT rows <= kThreads."""
    p = plan(log_k, log_b, tile)
    assert (1 << p["lti"]) <= K_THREADS
    assert (1 << (log_b + p["ltt"])) <= K_THREADS
    assert p["lti"] <= p["lk1"] and p["ltt"] <= p["lk2"]


def _pass1_words(lk1: int, lk2: int, lti: int):
    ti, k2 = 1 << lti, 1 << lk2
    di = K_THREADS >> lti
    rs = row_stride(k2)
    for t in range(K_THREADS):
        d, i2_0 = t & (ti - 1), t >> lti
        for i2 in range(i2_0, k2, di):
            yield t, d, i2, d * rs + pad(i2)


def _pass2_words(lk1: int, ltt: int, lb: int):
    k1, tt = 1 << lk1, 1 << ltt
    lt = min(lk1, K_LOG_THREADS)
    tpr = 1 << lt
    dt_step = K_THREADS >> lt
    rs = row_stride(k1)
    for t in range(K_THREADS):
        i1_0, dt_0 = t & (tpr - 1), t >> lt
        for i1 in range(i1_0, k1, tpr):
            for s in range(1 << lb):
                for dt in range(dt_0, tt, dt_step):
                    yield t, s, dt, i1, ((s << ltt) + dt) * rs + pad(i1)


# the small shapes exercise both branches of pass 2 (k1 below and above 512)
MAP_SHAPES = [(13, 1), (13, 3), (14, 2), (15, 2), (16, 1), (17, 2), (18, 3), (20, 2)]


@pytest.mark.parametrize("log_k,log_b", MAP_SHAPES)
def test_pass1_mapping_covers_each_word_once(log_k, log_b):
    p = plan(log_k, log_b)
    seen = set()
    ti, k2 = 1 << p["lti"], 1 << p["lk2"]
    for _, d, i2, slot in _pass1_words(p["lk1"], p["lk2"], p["lti"]):
        assert (d, i2) not in seen
        seen.add((d, i2))
        assert slot < ti * row_stride(k2)
    assert len(seen) == ti * k2


@pytest.mark.parametrize("log_k,log_b", MAP_SHAPES)
def test_pass2_mapping_covers_each_word_once(log_k, log_b):
    p = plan(log_k, log_b)
    k1, tt, b = 1 << p["lk1"], 1 << p["ltt"], 1 << log_b
    seen = set()
    for _, s, dt, i1, slot in _pass2_words(p["lk1"], p["ltt"], log_b):
        assert (s, dt, i1) not in seen
        seen.add((s, dt, i1))
        assert slot < (b * tt) * row_stride(k1)
    assert len(seen) == b * tt * k1


@pytest.mark.parametrize("log_k,log_b", MAP_SHAPES)
def test_pass2_output_offsets_stay_in_the_codeword(log_k, log_b):
    """Natural-order store: out[((t2 + dt) << lb) + s + (brev(p) << (lk2 + lb))]
    < n, and distinct for distinct words across every tile; 32-bit offsets."""
    p = plan(log_k, log_b)
    lk1, lk2, ltt = p["lk1"], p["lk2"], p["ltt"]
    n = 1 << (log_k + log_b)
    assert n < 1 << 32
    rows = 1 << (log_b + ltt)
    tiles = 1 << (lk2 - ltt)
    seen = set()
    for tile in (0, tiles - 1) if tiles > 1 else (0,):
        t2_0 = tile << ltt
        for t in range(K_THREADS):
            ri = t & (rows - 1)
            s, dt = ri & ((1 << log_b) - 1), ri >> log_b
            for q in range(t >> (log_b + ltt), 1 << lk1, K_THREADS >> (log_b + ltt)):
                brev = int(format(q, f"0{lk1}b")[::-1], 2)
                off = ((t2_0 + dt) << log_b) + s + (brev << (lk2 + log_b))
                assert 0 <= off < n
                assert off not in seen
                seen.add(off)


def test_running_products_match_direct_powers():
    """The per-thread running products equal the direct powers: pass 1 scales
    word (d, i2) by g^(i1_0 + d + k1 i2) = gi[d] G^i2 reached as G^i2_0 (G^di)^m;
    pass 2 scales (dt, i1) by w^((t2_0 + dt) i1) reached as
    w^((t2_0 + dt_0) i1) (w^(dt_step i1))^m."""
    p_ = 2013265921
    g, w = 31, pow(31, (p_ - 1) >> 10, p_)
    k1, i1_0, ti = 1 << 9, 64, 16
    gk = pow(g, k1, p_)
    for d in range(ti):
        for i2_0 in range(K_THREADS // ti):
            fac = pow(g, i1_0 + d, p_) * pow(gk, i2_0, p_) % p_
            step = pow(gk, K_THREADS // ti, p_)
            for m in range(4):
                i2 = i2_0 + m * (K_THREADS // ti)
                assert fac == pow(g, i1_0 + d + k1 * i2, p_)
                fac = fac * step % p_
    t2_0, dt_step = 8, 1
    for i1, dt_0 in itertools.product(range(0, 1 << 10, 97), range(dt_step)):
        fac = pow(w, (t2_0 + dt_0) * i1, p_)
        step = pow(w, dt_step * i1, p_)
        for m in range(5):
            assert fac == pow(w, (t2_0 + dt_0 + m * dt_step) * i1, p_)
            fac = fac * step % p_
