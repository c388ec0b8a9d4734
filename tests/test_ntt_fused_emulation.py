"""CPU emulation of the fused four-step LDE passes (lde_pass1_fused /
lde_pass2_fused in zorch_gb300/csrc/zc_ntt.cu): every index formula of the
kernels -- the group mappings of the first, middle and last radix passes, the
coalesced global loads with their coset and four-step scale factors, the
shared-memory layout with padded odd-stride rows, the bit-reversed output
positions of both orders -- restated in Python with exact field arithmetic
(canonical values; the Montgomery form is linear, so the words agree), run
over every work item of small shapes and compared with the oracle's LDE.
Each output word is also checked to be written exactly once."""

from __future__ import annotations

import numpy as np
import pytest

P = 2013265921  # BabyBear
GEN = 31


def pad(i: int) -> int:
    return i + (i >> 5)


def row_stride(m: int) -> int:
    return pad(m) | 1


def brev(i: int, bits: int) -> int:
    return int(format(i, f"0{bits}b")[::-1], 2) if bits else 0


def root(log_n: int) -> int:
    return pow(GEN, (P - 1) >> log_n, P)


def passes(logm: int, max_r: int) -> list[tuple[int, int]]:
    n = (logm + max_r - 1) // max_r
    out, h0 = [], logm - 1
    for q in range(n):
        r = (h0 + 1 + (n - q) - 1) // (n - q)
        out.append((h0, r))
        h0 -= r
    return out


def dif_group(v, tw, off, ls, sh0, r_):
    g = 1 << r_
    for r in range(r_):
        hb = r_ - 1 - r
        sh = sh0 + r
        tb, ts = off << sh, 1 << (ls + sh)
        for j in range(g):
            if not j & (1 << hb):
                j2 = j | (1 << hb)
                w = tw[tb + (j & ((1 << hb) - 1)) * ts]
                u, t = v[j], v[j2]
                v[j], v[j2] = (u + t) % P, (u - t) * w % P


def pass1(x, z, c, s, tile, lk1, lk2, lb, lti, h, max_r, writes):
    """lde_pass1_fused for item (coset s, i1 tile, column c)."""
    k1, k2, ti = 1 << lk1, 1 << lk2, 1 << lti
    lk, ln = lk1 + lk2, lk1 + lk2 + lb
    rs = row_stride(k2)
    ps = passes(lk2, max_r)
    ls0 = lk2 - ps[0][1]
    work = [None] * (ti * rs)
    tw = [pow(root(lk2), i, P) for i in range(max(k2 // 2, 1))]
    i1_0 = tile * ti
    gs = h * pow(root(ln), s, P) % P
    big_g = pow(gs, k1, P)
    gi = [pow(gs, i1_0 + i, P) for i in range(ti)]
    gt = [pow(big_g, i, P) for i in range(1 << ls0)]
    gstep = pow(big_g, 1 << ls0, P)
    xs = c * (1 << lk) + i1_0
    zd = (c * (1 << lb) + s) * (1 << lk) + i1_0
    for q, (h0, r_) in enumerate(ps):
        first, last = q == 0, q == len(ps) - 1
        ls = h0 - r_ + 1
        rmask = ti - 1
        for it in range(1 << (lti + lk2 - r_)):
            d, g = it & rmask, it >> lti
            off, blk = g & ((1 << ls) - 1), g >> ls
            base = (blk << (h0 + 1)) | off
            ar = d * rs + pad(base)
            if first:
                assert blk == 0
                src = xs + d + (off << lk1)
                v = [x[src + (j << (ls + lk1))] for j in range(1 << r_)]
                f = gi[d] * gt[off] % P
                for j in range(1 << r_):
                    v[j] = v[j] * f % P
                    f = f * gstep % P
            else:
                v = [work[ar + pad(j << ls)] for j in range(1 << r_)]
                assert None not in v
            dif_group(v, tw, off, ls, lk2 - 1 - h0, r_)
            if last:
                assert ls == 0 and base % (1 << r_) == 0
                zp = zd + d + (brev(base, lk2) << lk1)
                for j in range(1 << r_):
                    pos = zp + (brev(j, r_) << (lk1 + lk2 - r_))
                    assert pos == zd + d + (brev(base + j, lk2) << lk1)
                    z[pos] = v[j]
                    writes[pos] = writes.get(pos, 0) + 1
            else:
                for j in range(1 << r_):
                    work[ar + pad(j << ls)] = v[j]


def pass2(z, out, c, tile, lk1, lk2, lb, ltt, max_r, brev_out, writes):
    """lde_pass2_fused for item (t2 tile, column c)."""
    k1 = 1 << lk1
    lk, ln = lk1 + lk2, lk1 + lk2 + lb
    b = 1 << lb
    lrows = lb + ltt
    rs = row_stride(k1)
    work = [None] * ((1 << lrows) * rs)
    tw = [pow(root(lk1), i, P) for i in range(max(k1 // 2, 1))]
    t2_0 = tile << ltt
    zc = c << ln
    oc = c << ln
    wk = root(lk)
    ps = passes(lk1, max_r)
    if len(ps) > 1 and lk1 - ps[0][1] < 5:  # the smaller radix first (lde_pass2_fused)
        r0 = lk1 // len(ps)
        rest = passes(lk1 - r0, max_r)
        assert len(rest) == len(ps) - 1
        ps = [(lk1 - 1, r0)] + [(h0, r) for h0, r in rest]

    def put(pos, val):
        out[pos] = val
        writes[pos] = writes.get(pos, 0) + 1

    for q, (h0, r_) in enumerate(ps):
        first, last = q == 0, q == len(ps) - 1
        g_ = 1 << r_
        if first:
            ls = h0 - r_ + 1
            for it in range(1 << (ltt + ls)):
                off, dt = it & ((1 << ls) - 1), it >> ls
                t = t2_0 + dt
                f = [pow(wk, t * (off + (j << ls)), P) for j in range(g_)]
                for s in range(b):
                    src = zc + (s << lk) + (t << lk1) + off
                    v = [z[src + (j << ls)] * f[j] % P for j in range(g_)]
                    dif_group(v, tw, off, ls, 0, r_)
                    if last:
                        for j in range(g_):
                            if brev_out:
                                put(oc + (brev(s, lb) << lk) + (brev(t, lk2) << lk1) + j, v[j])
                            else:  # a single pass: r_ == lk1
                                put(oc + (t << lb) + s + (brev(j, r_) << (lk2 + lb)), v[j])
                    else:
                        ar = ((dt << lb) + s) * rs + pad(off)
                        for j in range(g_):
                            work[ar + pad(j << ls)] = v[j]
        elif last:
            for it in range(1 << (lrows + lk1 - r_)):
                r, g = it & ((1 << lrows) - 1), it >> lrows
                s, dt = r & (b - 1), r >> lb
                base = g << r_
                ar = r * rs + pad(base)
                v = [work[ar + pad(j)] for j in range(g_)]
                assert None not in v
                dif_group(v, tw, 0, 0, lk1 - 1 - h0, r_)
                t = t2_0 + dt
                sh = lk2 + lb
                ob = oc + (t << lb) + s + (brev(base, lk1) << sh)
                for j in range(g_):
                    if brev_out:
                        put(oc + (brev(s, lb) << lk) + (brev(t, lk2) << lk1) + base + j, v[j])
                    else:
                        pos = ob + (brev(j, r_) << (lk1 - r_ + sh))
                        assert pos == oc + (t << lb) + s + (brev(base + j, lk1) << sh)
                        put(pos, v[j])
        else:  # dif_pass over all rows
            ls = h0 - r_ + 1
            for gi in range(1 << (lrows + lk1 - r_)):
                row, g = gi & ((1 << lrows) - 1), gi >> lrows
                off, blk = g & ((1 << ls) - 1), g >> ls
                base = (blk << (h0 + 1)) | off
                ar = row * rs + pad(base)
                v = [work[ar + pad(j << ls)] for j in range(g_)]
                assert None not in v
                dif_group(v, tw, off, ls, lk1 - 1 - h0, r_)
                for j in range(g_):
                    work[ar + pad(j << ls)] = v[j]


# (log_k1, log_k2, log_blowup, log_ti, log_tt, max_r, bit-reversed output)
SHAPES = [
    (4, 4, 1, 2, 1, 4, False),   # single-pass rows in both passes
    (5, 4, 2, 3, 0, 2, False),   # 3 + 2 passes
    (5, 5, 1, 5, 2, 4, False),   # 2 passes each, full-row tiles
    (7, 6, 1, 4, 3, 3, False),   # first, middle and last passes
    (6, 6, 2, 3, 2, 4, True),    # bit-reversed output
    (7, 6, 1, 4, 3, 3, True),
    (5, 5, 2, 3, 1, 5, False),   # radix-2^5 (the wide variant): single-pass rows
    (7, 6, 1, 4, 3, 5, False),   # radix-2^5: 4 + 3 and 3 + 3 passes
    (9, 5, 1, 2, 1, 5, False),   # radix-2^5: 5 (pass 1) and 5 + 4 (pass 2)
    (5, 9, 1, 3, 1, 5, True),    # radix-2^5: 5 + 4 (pass 1) and 5, bit-reversed output
]


@pytest.mark.parametrize("shape", SHAPES)
def test_fused_four_step_passes_equal_the_oracle(orc, shape):
    lk1, lk2, lb, lti, ltt, max_r, brev_out = shape
    lk = lk1 + lk2
    k, n, cols = 1 << lk, 1 << (lk + lb), 2
    rng = np.random.default_rng(lk * 31 + lb)
    x = [int(v) for v in rng.integers(0, P, size=cols * k)]
    shift = 31
    z = [None] * (cols * n)
    out = [None] * (cols * n)
    zw, ow = {}, {}
    for c in range(cols):
        for s in range(1 << lb):
            for tile in range(1 << (lk1 - lti)):
                pass1(x, z, c, s, tile, lk1, lk2, lb, lti, shift, max_r, zw)
    assert len(zw) == cols * n and set(zw.values()) == {1}
    for c in range(cols):
        for tile in range(1 << (lk2 - ltt)):
            pass2(z, out, c, tile, lk1, lk2, lb, ltt, max_r, brev_out, ow)
    assert len(ow) == cols * n and set(ow.values()) == {1}
    xm = orc.to_mont(0, np.asarray(x, np.uint32).reshape(cols, k))
    enc = orc.rs_encode_bitrev if brev_out else orc.rs_encode
    want = orc.from_mont(0, enc(0, xm, lb, orc.to_mont(0, np.array([shift], np.uint32))[0]))
    assert np.array_equal(np.asarray(out, np.uint64).reshape(cols, n), want.astype(np.uint64))
