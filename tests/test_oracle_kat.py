"""Pin the CPU oracle to the reference's own known-answer tests.

Inputs come from tests/golden/kat_inputs.json (string literals of the ish test
functions, extracted as text); expected values are restated from the asserts,
citing tests/<file>:<line> of the ish repository.
"""
import json
import os

import numpy as np
import pytest

import oracle as O

HERE = os.path.dirname(os.path.abspath(__file__))
KAT = json.load(open(os.path.join(HERE, "golden", "kat_inputs.json")))
SG = KAT["test_semi_global.mojo"]
LP = KAT["test_local_and_profile.mojo"]


def lit(table, fn, i):
    return table[fn]["bytes"][i].encode()


def enc(kind, text):
    return O.encode(kind, text)


def ends(qs, qe, ts, te):
    return (O.QS if qs else 0) | (O.QE if qe else 0) | (O.TS if ts else 0) | (O.TE if te else 0)


ALL8 = [(False, False, False, False), (True, False, False, False), (False, True, False, False),
        (False, False, True, False), (False, False, False, True), (True, True, False, False),
        (False, False, True, True), (True, True, True, True)]


# test_semi_global.mojo:86-146 -- exact match, every free-end config scores 8, ends (3, 3).
@pytest.mark.parametrize("cfg", ALL8)
def test_exact_match_striped(cfg):
    q, t = enc(O.ACTGN, lit(SG, "test_exact_match_striped", 0)), enc(O.ACTGN, lit(SG, "test_exact_match_striped", 1))
    assert O.sg_aln(t, q, O.ACTGN, 3, 1, ends(*cfg)) == (8, 3, 3)


# test_semi_global.mojo:204-269
def test_query_substring_striped():
    q = enc(O.ACTGN, lit(SG, "test_query_substring_striped", 0))
    t = enc(O.ACTGN, lit(SG, "test_query_substring_striped", 1))
    assert O.sg_aln(t, q, O.ACTGN, 3, 1, ends(0, 0, 1, 1)) == (8, 5, 3)
    r = O.sg_start_end(t, q, O.ACTGN, 3, 1, ends(0, 0, 1, 1))
    assert (r["score"], r["target_start"], r["target_end"]) == (8, 2, 5)


# test_semi_global.mojo:340-392
def test_target_substring_striped():
    q = enc(O.ACTGN, lit(SG, "test_target_substring_striped", 0))
    t = enc(O.ACTGN, lit(SG, "test_target_substring_striped", 1))
    assert O.sg_aln(t, q, O.ACTGN, 3, 1, ends(1, 1, 0, 0)) == (8, 3, 5)
    r = O.sg_start_end(t, q, O.ACTGN, 3, 1, ends(1, 1, 0, 0))
    assert (r["score"], r["target_start"], r["target_end"]) == (8, 0, 3)


# test_semi_global.mojo:782-829
def test_partial_match_with_mismatch_striped():
    q = enc(O.ACTGN, lit(SG, "test_partial_match_with_mismatch_striped", 0))
    t = enc(O.ACTGN, lit(SG, "test_partial_match_with_mismatch_striped", 1))
    assert O.sg_aln(t, q, O.ACTGN, 3, 1, ends(0, 0, 0, 0))[0] == 4
    assert O.sg_aln(t, q, O.ACTGN, 3, 1, ends(0, 1, 0, 0))[0] == 4


# test_semi_global.mojo:832-902: blosum62 all-ends-free regression (parasail: 172, ends 256/171 1-based).
def test_alignment_striped_regression():
    q = enc(O.BLOSUM62, lit(SG, "test_alignment_striped_regression", 0))
    t = enc(O.BLOSUM62, lit(SG, "test_alignment_striped_regression", 1))
    assert O.sg_aln(t, q, O.BLOSUM62, 3, 1, ends(1, 1, 1, 1)) == (172, 255, 170)


# test_semi_global.mojo:905-958
def test_alignment_with_gap_striped():
    q = enc(O.ACTGN, lit(SG, "test_alignment_with_gap_striped", 0))
    t = enc(O.ACTGN, lit(SG, "test_alignment_with_gap_striped", 1))
    assert O.sg_aln(t, q, O.ACTGN, 3, 1, ends(0, 0, 0, 0))[0] == 5
    assert O.sg_start_end(t, q, O.ACTGN, 3, 1, ends(0, 0, 0, 0))["score"] == 5


# test_semi_global.mojo:961-1004 (the second call uses gap extension 2).
def test_no_match_striped():
    q = enc(O.ACTGN, lit(SG, "test_no_match_striped", 0))
    t = enc(O.ACTGN, lit(SG, "test_no_match_striped", 1))
    assert O.sg_aln(t, q, O.ACTGN, 3, 1, ends(1, 1, 1, 1))[0] == -2
    assert O.sg_aln(t, q, O.ACTGN, 3, 2, ends(0, 0, 0, 0))[0] == -8


# test_semi_global.mojo:1007-1057
def test_empty_sequences_striped():
    nonempty = enc(O.ACTGN, lit(SG, "test_empty_sequences_striped", 1))
    empty = np.zeros(0, np.uint8)
    assert O.sg_aln(nonempty, empty, O.ACTGN, 3, 1, ends(1, 1, 0, 0))[0] == 0
    assert O.sg_aln(empty, empty, O.ACTGN, 3, 1, ends(0, 0, 0, 0))[0] == 0


COMPLEX = [((0, 0, 0, 0), 6), ((1, 0, 0, 0), 10), ((0, 1, 0, 0), 6), ((0, 0, 1, 0), 7),
           ((0, 0, 0, 1), 6), ((1, 1, 0, 0), 10), ((0, 0, 1, 1), 7), ((1, 1, 1, 1), 10)]


# test_semi_global.mojo:1060-1163 (int16 x 8) and 1166-1269 (int8 x 16).
@pytest.mark.parametrize("cfg,score", COMPLEX)
@pytest.mark.parametrize("lanes", [(8, np.int16), (16, np.int8)])
def test_complex_case_striped(cfg, score, lanes):
    W, dt = lanes
    q = enc(O.ACTGN, lit(SG, "test_complex_case_striped", 0))
    t = enc(O.ACTGN, lit(SG, "test_complex_case_striped", 1))
    assert O.sg_aln(t, q, O.ACTGN, 3, 1, ends(*cfg), W=W, dtype=dt)[0] == score
    if cfg == (1, 1, 0, 0) and dt == np.int16:
        r = O.sg_start_end(t, q, O.ACTGN, 3, 1, ends(*cfg), W=W)
        assert r["score"] == score
        assert 0 <= r["target_start"] <= r["target_end"] <= len(t)


# test_semi_global.mojo:1272-1314
def test_reversed_alignment_striped():
    q = enc(O.ACTGN, lit(SG, "test_reversed_alignment_striped", 0))
    t = enc(O.ACTGN, lit(SG, "test_reversed_alignment_striped", 1))
    r = O.sg_start_end(t, q, O.ACTGN, 3, 1, ends(1, 1, 0, 0))
    assert (r["score"], r["target_end"], r["target_start"]) == (8, 3, 0)


# test_semi_global.mojo:1317-1422
def test_biological_example_striped():
    lits = SG["test_biological_example_striped"]["bytes"]
    gene, genome = enc(O.ACTGN, lits[0].encode()), enc(O.ACTGN, lits[1].encode())
    assert O.sg_aln(genome, gene, O.ACTGN, 3, 1, ends(0, 0, 0, 1))[0] == 26
    mid = enc(O.ACTGN, lits[2].encode())
    r = O.sg_start_end(genome, mid, O.ACTGN, 3, 1, ends(0, 0, 1, 1))
    assert (r["score"], r["target_end"], r["target_start"]) == (12, 18, 13)
    tail = enc(O.ACTGN, lits[3].encode())
    r = O.sg_start_end(genome, tail, O.ACTGN, 3, 1, ends(0, 0, 1, 0))
    assert (r["score"], r["target_start"], r["target_end"]) == (10, 18, 22)


# The scalar parasail-style tests on the same pairs assert the same optimal
# scores (test_semi_global.mojo:31-82, 149-201, 395-437, 440-480, 483-521,
# 562-652); the striped oracle agrees on every one.
def test_scalar_kat_scores_agree():
    cases = [
        ("test_no_match", (1, 1, 1, 1), 3, 1, -2),
        ("test_no_match", (0, 0, 0, 0), 3, 1, -8),
        ("test_alignment_with_gap", (0, 0, 0, 0), 3, 1, 5),
        ("test_partial_match_with_mismatch", (0, 0, 0, 0), 3, 1, 4),
        ("test_partial_match_with_mismatch", (0, 1, 0, 0), 3, 1, 4),
        ("test_query_substring", (0, 0, 1, 1), 3, 1, 8),
    ]
    for fn, cfg, go, ge, score in cases:
        q, t = enc(O.ACTGN, lit(SG, fn, 0)), enc(O.ACTGN, lit(SG, fn, 1))
        assert O.sg_aln(t, q, O.ACTGN, go, ge, ends(*cfg))[0] == score, fn


# test_local_and_profile.mojo:19-152 -- striped profile layout and bias.
def test_profile_layout():
    size = 64
    M = np.where(np.eye(size, dtype=bool), 2, -1).astype(np.int8).ravel()
    q = np.arange(size, dtype=np.uint8)
    L = O.lib()
    import ctypes as C
    bias = L.ish_o_sw_bias(M.ctypes.data_as(C.POINTER(C.c_int8)), size)
    assert bias == 1
    p8 = np.zeros(size * 4 * 16, np.uint8)
    p16 = np.zeros(size * 8 * 8, np.uint16)
    L.ish_o_sw_profile_u8(q.ctypes.data_as(C.POINTER(C.c_uint8)), size, M.ctypes.data_as(C.POINTER(C.c_int8)),
                          size, 16, bias, p8.ctypes.data_as(C.POINTER(C.c_uint8)))
    L.ish_o_sw_profile_u16(q.ctypes.data_as(C.POINTER(C.c_uint8)), size, M.ctypes.data_as(C.POINTER(C.c_int8)),
                           size, 8, bias, p16.ctypes.data_as(C.POINTER(C.c_uint16)))
    assert len(p8) // 16 == 256 and len(p16) // 8 == 512
    v8 = p8.reshape(size * 4, 16)
    v16 = p16.reshape(size * 8, 8)
    for c in range(size):
        exp = np.zeros((4, 16), np.uint8)
        exp[c % 4, c // 4] = 3
        assert (v8[c * 4:(c + 1) * 4] == exp).all()
        exp16 = np.zeros((8, 8), np.uint16)
        exp16[c % 8, c // 8] = 3
        assert (v16[c * 8:(c + 1) * 8] == exp16).all()


# test_local_and_profile.mojo:155-280 -- byte SW sanity and the terminate=0 reverse pass.
def test_sw_byte():
    q = np.array([0, 1, 2, 3, 0, 1, 2, 3], np.uint8)
    ref = np.array([3, 0, 1, 2, 3, 0, 1, 2, 3, 0, 1, 2], np.uint8)
    s, r, qe = O.sw(ref, q, O.ACTGN, 3, 1)
    assert s > 10 and r >= 7 and qe == 7
    poor = np.full(9, 3, np.uint8)
    ps = O.sw(poor, q, O.ACTGN, 3, 1)[0]
    assert ps < s
    assert O.sw(poor, q, O.ACTGN, 3, 1, reverse=True, terminate=0)[0] == ps


# test_local_and_profile.mojo:283-386 -- perfect alignment scores 2 * length.
def test_sw_byte_perfect():
    q = np.array([0, 1, 2, 3, 0, 1, 2, 3], np.uint8)
    assert O.sw(q, q, O.ACTGN, 3, 1)[0] == 16


# test_local_and_profile.mojo:389-419 -- KAT against the C SSW library.
def test_compare_vs_c():
    ref = enc(O.ACTGN, lit(LP, "test_compare_vs_c", 0))
    read = enc(O.ACTGN, lit(LP, "test_compare_vs_c", 1))
    assert O.sw(ref, read, O.ACTGN, 3, 1) == (21, 21, 14)


# test_local_and_profile.mojo:422-464
def test_compare_vs_c_ssw_align():
    ref = enc(O.ACTGN, lit(LP, "test_compare_vs_c_ssw_align", 0))
    read = enc(O.ACTGN, lit(LP, "test_compare_vs_c_ssw_align", 1))
    a = O.ssw_align(ref, read, O.ACTGN, 3, 1)
    assert (a["score1"], a["ref_begin1"], a["ref_end1"], a["read_begin1"], a["read_end1"]) == (21, 8, 21, 0, 14)


# test_local_and_profile.mojo:467-565 (align2 and align3 assert the same values).
@pytest.mark.parametrize("fn", ["test_compare_vs_c_ssw_align2", "test_compare_vs_c_ssw_align3"])
def test_compare_vs_c_ssw_align_long(fn):
    ref = enc(O.ACTGN, lit(LP, fn, 0))
    read = enc(O.ACTGN, lit(LP, fn, 1))
    a = O.ssw_align(ref, read, O.ACTGN, 3, 1)
    assert (a["score1"], a["ref_begin1"], a["ref_end1"], a["read_end1"], a["read_begin1"]) == (32, 1, 60, 74, 3)


# tests/matcher/alignment/test_striped_utils.mojo:9-66 -- saturation at the type limits,
# observed through the aligners: a record/query long enough to push int8 lanes past 127.
def test_int8_lane_saturation_is_clamped():
    q = enc(O.ACTGN, b"ACGT" * 20)  # optimal score 160 > int8 max
    s8 = O.sg_aln(q, q, O.ACTGN, 3, 1, ends(1, 1, 1, 1), W=16, dtype=np.int8)[0]
    s16 = O.sg_aln(q, q, O.ACTGN, 3, 1, ends(1, 1, 1, 1), W=8)[0]
    assert s16 == 160 and s8 == 127
