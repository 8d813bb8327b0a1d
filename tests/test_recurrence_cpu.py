"""CPU models of two pieces of the wavefront engine's arithmetic, checked
against plain Gotoh on small random inputs (no GPU needed):

* semi-global row frames: row r is held raised by (r mod R) * ext with the
  profile carrying +ext, the E update becomes max(T + ext - open, E), and every
  R rows (R * ext <= 2048) the carried row drops back -- all in 16-bit
  wrapping arithmetic, as the DPX add-max instructions compute it;
* long records as overlapping windows: window results folded by (score,
  first row, smallest column) equal the whole-record result when windows past
  row 0 start from the fixed-query-start boundary (and, as the counterexample
  shows, not when they start from a free-query-start one).
"""
import numpy as np
import pytest

NEG = -(10 ** 9)


def gotoh_rows(q, r, M, op, ex, ends, local=False, start_row=0, top=None):
    """Row-by-row plain Gotoh; yields (row, H row).  `top` overrides the
    boundary above the first row (query-start rule), as a window uses it."""
    Q = len(q)
    qs, ts = ends & 1, ends & 4
    if top is None:
        top = [0] * Q if (local or qs) else [-(op + ex * j) for j in range(Q)]
    Hp = list(top)
    Ep = [h - op for h in Hp] if not local else [0] * Q
    for i in range(len(r)):
        gi = start_row + i
        Hn, En = [0] * Q, [0] * Q
        left = 0 if (local or ts) else -(op + ex * gi)
        diag_left = 0 if (local or ts or gi == 0) else -(op + ex * (gi - 1))
        F = NEG
        for j in range(Q):
            diag = diag_left if j == 0 else Hp[j - 1]
            En[j] = max(Ep[j] - ex, Hp[j] - op)
            F = max(F - ex, (Hn[j - 1] if j > 0 else left) - op)
            h = max(diag + M[r[i]][q[j]], En[j], F)
            Hn[j] = max(h, 0) if local else h
        Hp, Ep = Hn, En
        yield gi, Hp


def sg_target_end(q, r, M, op, ex, ends, **kw):
    """Semi-global with a free target end: (max over rows of H(i, Q-1), first row)."""
    best, br = NEG, -1
    for i, H in gotoh_rows(q, r, M, op, ex, ends, **kw):
        if H[-1] > best:
            best, br = H[-1], i
    return best, br


def sw_best(q, r, M, op, ex, **kw):
    """Local: (best, first row, smallest column of it in that row)."""
    best, br, bc = 0, -1, 0
    for i, H in gotoh_rows(q, r, M, op, ex, 0, local=True, **kw):
        m = max(H)
        if m > best:
            best, br, bc = m, i, H.index(m)
    return best, br, bc


def w16(x):
    x &= 0xFFFF
    return x - 0x10000 if x >= 0x8000 else x


def frames_sg(q, r, M, op, ex, ends, G=2):
    """The kernel's semi-global recurrence in row frames, G pipeline threads,
    16-bit wrapping add-max."""
    Q = len(q)
    K = (Q + 1 + G - 1) // G
    d = G * K - Q
    R = 1
    while R < (1 << 20) and 2 * R * max(ex, 1) <= 2048:
        R *= 2
    qs, ts = ends & 1, ends & 4
    ppad = 0 if ts else -(op + ex)

    def P(row, col):
        return w16((ppad if col < 0 else int(M[r[row]][q[col]])) + ex)

    def hinit(col):
        return 0 if (col < 0 or qs) else -op - ex * col

    hleft = 0 if ts else -20000
    am = lambda a, b, c: max(w16(a + b), c)  # noqa: E731 -- DPX add-max
    frame = lambda row: (row & (R - 1)) * ex  # noqa: E731
    H = [[w16(hinit(t * K - d + j) - ex) for j in range(K)] for t in range(G)]
    E = [[w16(hinit(t * K - d + j) - op) for j in range(K)] for t in range(G)]
    prevH = [w16((hleft if t == 0 else hinit(t * K - d - 1)) - ex) for t in range(G)]
    outH, outF = [0] * G, [0] * G
    best, brow = -32768, -1
    for step in range(len(r) + G - 1):
        msgH, msgF = [0] + outH[:-1], [0] + outF[:-1]
        newH, newF = list(outH), list(outF)
        for t in range(G):
            row = step - t
            if row < 0 or row >= len(r):
                continue
            col0 = t * K - d
            if row > 0 and (row & (R - 1)) == 0:
                H[t] = [am(x, -R * ex, -32768) for x in H[t]]
                E[t] = [am(x, -R * ex, -32768) for x in E[t]]
                prevH[t] = am(prevH[t], -R * ex, -32768)
            for j in range(K - 1, -1, -1):
                T = am(prevH[t] if j == 0 else H[t][j - 1], P(row, col0 + j), E[t][j])
                E[t][j] = am(T, ex - op, E[t][j])
                H[t][j] = T
            Fs = w16(-20000 + op) if t == 0 else msgF[t]
            for j in range(K):
                T = H[t][j]
                H[t][j] = am(Fs, -op, T)
                Fs = am(Fs, -ex, T)
            prevH[t] = w16(hleft + frame(row)) if t == 0 else msgH[t]
            newH[t], newF[t] = H[t][K - 1], Fs
            if t == G - 1:
                c = am(H[t][K - 1], -frame(row), -32768)
                if c > best:
                    best, brow = c, row
        outH, outF = newH, newF
    return best, brow


def blosum_like(rng, n=20):
    """Symmetric, mostly negative off the diagonal, positive on it."""
    M = rng.integers(-4, 3, (n, n))
    M = np.minimum(M, M.T)
    M[np.arange(n), np.arange(n)] = rng.integers(4, 12, n)
    return M


@pytest.mark.parametrize("ext", [0, 1, 3, 200, 1000])
def test_row_frames_equal_plain_gotoh(ext):
    rng = np.random.default_rng(100 + ext)
    M = blosum_like(rng)
    op = ext + 7
    qlen = 6 if ext >= 1000 else 12
    for trial in range(6):
        q = rng.integers(0, 20, qlen)
        r = rng.integers(0, 20, int(rng.integers(1, 90)))
        for ends in (12, 13, 8, 9):
            for G in (1, 2, 4):
                assert frames_sg(q, r, M, op, ext, ends, G) == sg_target_end(q, r, M, op, ext, ends), \
                    (ext, trial, ends, G)


def window_overlap(Q, mmax, mmin, op, ex, local):
    min_best = 0 if local else Q * min(mmin, 0)
    top = Q * max(mmax, 0) - op - min_best
    return Q + 2 + max(0, -(-top // ex))


def windowed(q, r, M, op, ex, ends, W, O, local, fixed_start_past_row0=True):
    """Fold of window results, windows [k*W - O, (k+1)*W)."""
    Q = len(q)
    res = []
    k = 0
    while k * W < len(r):
        st = 0 if k == 0 else k * W - O
        en = min(len(r), (k + 1) * W)
        top = None
        if st > 0 and not local:
            top = [-(op + ex * j) for j in range(Q)] if fixed_start_past_row0 else None
        sub = r[st:en]
        if local:
            b, i, c = sw_best(q, sub, M, op, ex, start_row=st, top=top)
            res.append((b, i, c))
        else:
            b, i = sg_target_end(q, sub, M, op, ex, ends, start_row=st, top=top)
            res.append((b, i, Q - 1))
        k += 1
    # largest score, then first row, then smallest column; rows of -1 (no
    # improvement) only when every window has the initial score
    best = max(res, key=lambda x: (x[0], -x[1] if x[1] >= 0 else -(10 ** 12), -x[2]))
    return best


@pytest.mark.parametrize("local,ends", [(False, 12), (False, 13), (True, 0)])
def test_window_fold_equals_whole_record(local, ends):
    rng = np.random.default_rng(7 + ends + local)
    M = blosum_like(rng)
    for trial in range(8):
        op, ex = [(10, 1), (5, 2), (30, 10)][trial % 3]
        q = rng.integers(0, 20, 8)
        r = rng.integers(0, 20, int(rng.integers(150, 400)))
        O = window_overlap(len(q), int(M.max()), int(M.min()), op, ex, local)
        W = max(O + 1, 40)
        if local:
            whole = sw_best(q, r, M, op, ex)
        else:
            b, i = sg_target_end(q, r, M, op, ex, ends)
            whole = (b, i, len(q) - 1)
        assert windowed(q, r, M, op, ex, ends, W, O, local) == whole, (trial, op, ex, W, O)


def test_free_query_start_windows_would_invent_alignments():
    # the counterexample behind the fixed-start rule: with a free query start,
    # windows past row 0 that also start freely report scores the whole record
    # does not have (large gap penalties keep the true best small)
    rng = np.random.default_rng(3)
    M = blosum_like(rng)
    op, ex = 207, 200
    found = False
    for _ in range(40):
        q = rng.integers(0, 20, 10)
        r = rng.integers(0, 20, 300)
        O = window_overlap(len(q), int(M.max()), int(M.min()), op, ex, False)
        W = max(O + 1, 40)
        b, i = sg_target_end(q, r, M, op, ex, 13)
        whole = (b, i, len(q) - 1)
        assert windowed(q, r, M, op, ex, 13, W, O, False, fixed_start_past_row0=True) == whole
        if windowed(q, r, M, op, ex, 13, W, O, False, fixed_start_past_row0=False) != whole:
            found = True
    assert found


def sw_matrix(q, r, M, op, ex):
    """All H rows of plain local Gotoh."""
    return [list(H) for _, H in gotoh_rows(q, r, M, op, ex, 0, local=True)]


def sw_reference_end(Hrows):
    """The reference's rule: first row whose maximum strictly beats every
    earlier cell, smallest column of that maximum in that row."""
    best, br, bc = 0, -1, 0
    for i, H in enumerate(Hrows):
        m = max(H)
        if m > best:
            best, br, bc = m, i, H.index(m)
    return (best, br, bc) if best > 0 else (0, -1, 0)


def sw_filtered_end(Hrows, G, K):
    """The wavefront kernel's local-alignment end logic on the same H values:
    thread t owns columns [t*K, (t+1)*K); per row it records its row only when
    its column maximum beats max(its recorded best, the running best of all
    columns to its left for this row), then the threads' (score, row, column)
    are folded left to right with the (score, earlier row, smaller column)
    order."""
    Q = len(Hrows[0]) if Hrows else 0
    best = [0] * G
    row_of = [-1] * G
    saved = [None] * G
    for i, H in enumerate(Hrows):
        left = 0
        for t in range(G):
            cols = H[t * K:min(Q, (t + 1) * K)]
            cm = max(cols) if cols else 0
            thr = max(best[t], left)
            nb = max(thr, cm)
            if cm > thr:
                best[t], row_of[t], saved[t] = cm, i, list(cols)
            left = nb
    acc = None
    for t in range(G):
        b, r = best[t], row_of[t]
        c = 0x7FFF
        if b > 0 and saved[t] is not None:
            c = t * K + saved[t].index(b)
        mine = (b, r, c)
        if acc is not None:
            lb, lr, lc = acc
            if lb > b or (lb == b and (lr < r or (lr == r and lc < c))):
                mine = acc
        acc = mine
    b, r, c = acc
    return (b, r, c) if b > 0 else (0, -1, 0)


@pytest.mark.parametrize("G", [1, 2, 4, 8])
def test_local_end_filter_and_fold_equal_reference_rule(G):
    rng = np.random.default_rng(40 + G)
    for trial in range(150):
        A = 3 if trial % 2 else 6  # small alphabets: many equal maxima
        M = blosum_like(rng, A)
        Q = int(rng.integers(1, 30))
        K = (Q + G - 1) // G
        q = rng.integers(0, A, Q)
        r = rng.integers(0, A, int(rng.integers(0, 60)))
        if trial % 3 == 0 and len(r) > Q:  # a copy of the query: a clear maximum
            pos = int(rng.integers(0, len(r) - Q + 1))
            r[pos:pos + Q] = q
        op, ex = [(3, 1), (5, 2), (2, 1)][trial % 3]
        Hrows = sw_matrix(q, r, M, op, ex)
        assert sw_filtered_end(Hrows, G, K) == sw_reference_end(Hrows), (G, trial)


def sg_kernel_fold(Hrows, Q, G, K, ends, neg_limit):
    """The wavefront kernel's semi-global end logic on plain-Gotoh H rows:
    the target-end running maximum (strict, first row wins), the last-row
    query-end scan split over G threads of K columns (front padding d; each
    thread keeps its first maximum, columns to the left win ties) and the
    combination rule of the two."""
    T = len(Hrows)
    d = G * K - Q
    te, qe = bool(ends & 8), bool(ends & 2)
    best, row_a = neg_limit, -1
    for i, H in enumerate(Hrows):
        if H[Q - 1] > best:
            best, row_a = H[Q - 1], i
    mx = mq = None
    if qe:
        last = Hrows[T - 1]
        for t in range(G):
            b, c = -32768, 0x7FFF
            for j in range(K):
                col = t * K - d + j
                if col >= 0 and last[col] > b:
                    b, c = last[col], col
            if t > 0 and not (b > mx):
                b, c = mx, mq
            mx, mq = b, c
    eq = Q - 1
    if not te and not qe:
        return Hrows[T - 1][Q - 1], eq, T - 1
    score = best if te else neg_limit
    er = row_a if te else -1
    if qe:
        if mx > score:
            score, er, eq = mx, T - 1, mq
        elif mx == score and er == T - 1 and mq < eq:
            eq = mq
    return score, eq, er


@pytest.mark.parametrize("kind", ["actgn", "blosum62"])
def test_semi_global_fold_equals_oracle(kind):
    import oracle as O
    from ish_gb300 import native
    from ish_gb300.scoring import ScoringMatrix

    k = O.ACTGN if kind == "actgn" else O.BLOSUM62
    alpha = 5 if kind == "actgn" else 20
    m = ScoringMatrix(k)
    M = m.values.astype(int)
    rng = np.random.default_rng(91 + alpha)
    for trial in range(12):
        Q = int(rng.integers(1, 25))
        q = rng.integers(0, alpha, Q, dtype=np.uint8)
        recs = [rng.integers(0, alpha, int(rng.integers(1, 50)), dtype=np.uint8) for _ in range(6)]
        op, ex = (3, 1) if kind == "actgn" else (10, 1)
        mx_score = int(m.values[q, q].astype(np.int64).sum())
        buf, off = native.pack_records(recs)
        for ends in range(16):
            om = O.Matcher(O.SEMI_GLOBAL, k, q, mx_score, 0.5, gap_open=op, gap_extend=ex, ends=ends)
            o = om.batch(buf, off, threads=1)
            min_score = int(M.min())
            neg_limit = -32768 + op + 1 if -op < min_score else -32768 - min_score + 1
            for n, r in enumerate(recs):
                Hrows = [list(H) for _, H in gotoh_rows(q, r, M, op, ex, ends)]
                want = (int(o["score"][n]), int(o["qend"][n]), int(o["tend"][n]))
                for G in (1, 2, 4):
                    K = (Q + 1 + G - 1) // G
                    got = sg_kernel_fold(Hrows, Q, G, K, ends, neg_limit)
                    assert got == want, (kind, trial, ends, n, G, got, want)


@pytest.mark.parametrize("kind", ["actgn", "blosum62"])
def test_local_end_logic_equals_oracle(kind):
    import oracle as O
    from ish_gb300 import native
    from ish_gb300.scoring import ScoringMatrix

    k = O.ACTGN if kind == "actgn" else O.BLOSUM62
    alpha = 5 if kind == "actgn" else 20
    m = ScoringMatrix(k)
    M = m.values.astype(int)
    rng = np.random.default_rng(97 + alpha)
    for trial in range(20):
        Q = int(rng.integers(1, 30))
        q = rng.integers(0, alpha, Q, dtype=np.uint8)
        recs = [rng.integers(0, alpha, int(rng.integers(0, 60)), dtype=np.uint8) for _ in range(8)]
        op, ex = (3, 1) if kind == "actgn" else (10, 1)
        mx_score = int(m.values[q, q].astype(np.int64).sum())
        buf, off = native.pack_records(recs)
        o = O.Matcher(O.LOCAL, k, q, mx_score, 0.5, gap_open=op, gap_extend=ex, ends=0).batch(buf, off, threads=1)
        for n, r in enumerate(recs):
            Hrows = sw_matrix(q, r, M, op, ex)
            want = (int(o["score"][n]), int(o["tend"][n]), int(o["qend"][n]))
            for G in (1, 2, 4):
                K = (Q + G - 1) // G
                got = sw_filtered_end(Hrows, G, K) if Hrows else (0, -1, 0)
                assert got == want, (kind, trial, n, G, got, want)
