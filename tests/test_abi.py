"""CPU-side checks of the C ABI: the library builds, loads, exports every
entry point include/ish_gpu.h declares, and fails cleanly without a GPU."""
import ctypes as C
import os
import re

import numpy as np
import pytest

import oracle as O
from ish_gb300 import native
from ish_gb300.scoring import ScoringMatrix

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "ish_gpu.h")


def declared_symbols():
    src = open(HEADER).read()
    return sorted(set(re.findall(r"^ISH_API[^(]*?\b(ish_gpu_\w+)\s*\(", src, re.M)))


def test_header_declares_the_binding_surface():
    assert declared_symbols() == sorted(native.EXPORTS)


def test_library_exports_every_declared_symbol():
    lib = native.load(build_if_missing=True)
    for name in declared_symbols():
        assert hasattr(lib, name), name
    assert lib.ish_gpu_abi_version() == 1


def test_open_reports_error_without_device(monkeypatch):
    monkeypatch.setenv("CUDA_VISIBLE_DEVICES", os.environ.get("CUDA_VISIBLE_DEVICES", ""))
    lib = native.load(build_if_missing=True)
    h = C.c_void_p()
    rc = lib.ish_gpu_open(0, C.byref(h))
    try:
        import torch
        has_gpu = torch.cuda.is_available()
    except Exception:
        has_gpu = False
    if has_gpu:
        assert rc == 0
        lib.ish_gpu_close(h)
    else:
        assert rc in (native.ENODEV, native.EDEVICE)
        assert h.value is None
        assert lib.ish_gpu_last_error(None)


def test_null_arguments_are_rejected():
    lib = native.load(build_if_missing=True)
    assert lib.ish_gpu_open(0, None) == native.EINVAL
    assert lib.ish_gpu_set_option(None, native.OPT_KERNEL, 0) == native.EINVAL
    lib.ish_gpu_close(None)  # no-op


@pytest.mark.parametrize("kind", [O.ASCII, O.ACTGN, O.ACTGN0, O.BLOSUM62])
def test_product_matrices_match_oracle(kind):
    vals, size, a2c, c2a = O.matrix(kind)
    m = ScoringMatrix(kind)
    assert m.size == size
    assert (m.values.ravel() == vals).all()
    assert (m.ascii_to_code == a2c).all()
    assert (m.code_to_ascii == c2a).all()
    text = bytes(range(256))
    enc, score = m.encode_and_score(text)
    oenc, oscore = O.encode_and_score(kind, text)
    assert (enc == oenc).all() and score == oscore


def test_output_writer_formats():
    """ish_gb300.output writes what the runners write: decoded records in input
    order, the line runner's tty prefix and colours, the fastx header and
    quality lines (ishlib/parallel_line_search_runner.mojo:113-155,
    ishlib/parallel_fastx_search_runner.mojo:136-177)."""
    from ish_gb300 import output
    from ish_gb300.scoring import ScoringMatrix

    m = ScoringMatrix.from_str("actgn")
    recs = [m.encode(b"acgtNx"), m.encode(b"GGG"), m.encode(b"tta")]
    buf, off = native.pack_records(recs)
    got = []
    output.write_line_matches(got.append, buf, off, [(0, 1, 3), (2, 0, 2)], m.code_to_ascii)
    assert b"".join(got) == b"ACGTNN\nTTA\n"
    got = []
    output.write_line_matches(got.append, buf, off, [(2, 1, 3)], m.code_to_ascii, file_name=b"f.txt",
                              first_line=10, tty=True)
    assert b"".join(got) == (b"\x1b[35mf.txt\x1b[0m:\x1b[32m13\x1b[0m: T\x1b[31mTA\x1b[0m\n")
    got = []
    output.write_fastx_matches(got.append, [b"r0", b"r1", b"r2"], buf, off, [(1, 0, 3)], m.code_to_ascii,
                               quals=[b"!!!!!!", b"III", b"###"])
    assert b"".join(got) == b">r1\nGGG\n+\nIII\n"
    got = []
    output.write_fastx_matches(got.append, [b"r0", b"r1", b"r2"], buf, off, [(0, 2, 4)], m.code_to_ascii, tty=True)
    assert b"".join(got) == b">r0\nAC\x1b[1;31m\x1b[31mGT\x1b[0mNN\n"


def test_caller_output_buffers_are_checked():
    # score_set(out=...) writes into the caller's arrays (e.g. pinned host
    # buffers reused across calls) only when they fit the contract
    import numpy as np

    from ish_gb300 import native

    good = {"score": np.zeros(10, np.int32), "hit_idx": np.zeros(10, np.uint32)}
    out = native.Context._outputs(None, 10, ("score", "hit_idx", "tend"), good)
    assert out["score"] is good["score"] and out["hit_idx"] is good["hit_idx"]
    assert out["tend"].dtype == np.int32 and len(out["tend"]) == 10
    for bad in ({"score": np.zeros(9, np.int32)}, {"score": np.zeros(10, np.int64)},
                {"score": np.zeros(20, np.int32)[::2]}):
        try:
            native.Context._outputs(None, 10, ("score",), bad)
        except ValueError:
            continue
        raise AssertionError(f"accepted {bad}")
