"""The slicing arithmetic of the tensor-core df64 element kernel (feelpp_gb300/csrc/element_tc.cu),
restated step by step in numpy binary32 on the CPU: every slice is an exact bf16 value with an integer
part of at most 256, the exact levels 0..3 of slice products fit binary32 without rounding, and the
product of seven sliced double-float coefficients with seven sliced table columns stays within 3e-14 of
sum_k |c_k T_k| with coefficients three and tables two orders of magnitude apart in a row and column."""
import numpy as np

F32 = np.float32
NS, NEX, NLEV = 7, 4, 8


def _split(x):
    h = F32(x)
    return h, F32(x - np.float64(h))


def _exp_above(x):
    b = int((np.frombuffer(F32(x).tobytes(), np.uint32)[0] >> 23) & 0xFF)
    return -1000 if b == 0 else b - 126


def _two_sum(a, b):
    a, b = F32(a), F32(b)
    s = F32(a + b)
    bb = F32(s - a)
    return s, F32(F32(a - F32(s - bb)) + F32(b - bb))


def _slices(h, l):
    x, y, e = F32(F32(h) * F32(256)), F32(F32(l) * F32(256)), F32(0)
    out = []
    for i in range(NS):
        if i == 3:
            x, e = _two_sum(x, F32(y * F32(16777216.0)))
        elif i == 4:
            x = F32(np.float64(e) * 256.0 + np.float64(x))        # one rounding, as the fused multiply-add
        a = F32(np.rint(x))
        assert abs(a) <= 256
        out.append(F32(a * F32(2.0 ** (-8 * (i + 1)))))
        x = F32(F32(x - a) * F32(256))
    for v in out:                                                # exact bf16: low 16 bits clear
        assert np.frombuffer(F32(v).tobytes(), np.uint32)[0] & 0xFFFF == 0
    return out


def _operand(hi, lo, sig, sign):
    """rows of (hi + lo) 2^(sign * sig_k), scaled by the row exponent and sliced"""
    n = hi.shape[0]
    S = np.zeros((NS, n, 7))
    ex = np.zeros(n)
    for r in range(n):
        p = [F32(2.0 ** (sign * sig[k])) for k in range(7)]
        uh = [F32(hi[r, k] * p[k]) for k in range(7)]
        ul = [F32(lo[r, k] * p[k]) for k in range(7)]
        E = max(_exp_above(u) for u in uh)
        E = 0 if E == -1000 else max(E, -60)
        ex[r] = E
        q = F32(2.0 ** -E)
        for k in range(7):
            for i, v in enumerate(_slices(F32(uh[k] * q), F32(ul[k] * q))):
                S[i, r, k] = v
    return S, ex


def test_sliced_products_match_exact_sums():
    rng = np.random.default_rng(3)
    nrow, ncol, worst = 32, 10, 0.0
    for _ in range(4):
        c = np.concatenate([rng.standard_normal((nrow, 6)) * 10.0 ** rng.uniform(-3, 0, (nrow, 6)),
                            rng.random((nrow, 1)) * 1e-6], axis=1)
        T = np.concatenate([rng.standard_normal((6, ncol)) * 10.0 ** rng.uniform(-2, 0, (6, ncol)),
                            rng.random((1, ncol)) * 1e-2], axis=0)
        ch, cl = np.vectorize(_split)(c)
        th, tl = np.vectorize(_split)(T.T)                       # table columns as rows
        ch, cl, th, tl = (np.asarray(v, np.float32) for v in (ch, cl, th, tl))
        sig = [max(_exp_above(ch[r, k]) for r in range(nrow)) for k in range(7)]
        A, E = _operand(ch, cl, sig, -1)
        B, F = _operand(th, tl, sig, +1)
        D = np.zeros((NEX + 1, nrow, ncol))
        for lv in range(NLEV):
            for i in range(lv + 1):
                j = lv - i
                if i < NS and j < NS:
                    D[min(lv, NEX)] += A[i] @ B[j].T
        for x in range(NEX):                                     # exact in binary32
            assert np.array_equal(D[x].astype(np.float32).astype(np.float64), D[x])
        exact = (ch.astype(np.float64) + cl) @ (th.astype(np.float64) + tl).T
        for r in range(nrow):
            for t in range(ncol):
                s, err = F32(D[0, r, t]), F32(0)
                for x in range(1, NEX):
                    s, e = _two_sum(s, D[x, r, t])
                    err = F32(err + e)
                err = F32(err + F32(D[NEX, r, t]))
                hi = F32(s + err)
                lo = F32(err - F32(hi - s))
                v = (np.float64(hi) + np.float64(lo)) * 2.0 ** (E[r] + F[t])
                scale = np.abs((ch[r].astype(np.float64) + cl[r]) * (th[t].astype(np.float64) + tl[t])).sum()
                worst = max(worst, abs(v - exact[r, t]) / scale)
    assert worst <= 3e-14, worst
