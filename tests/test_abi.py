"""CPU tests of the C ABI boundary: the library loads and exports every
symbol the public header declares; struct layouts match the reference's
records.  No compute call is made (no GPU here)."""
import ctypes as C
import re
from pathlib import Path

from opencuda_gb300 import _lib

ROOT = Path(__file__).resolve().parent.parent


C_HEADERS = ["houghline_gb300.h", "hl_proposal.h", "hl_circle.h"]


def declared_symbols():
    text = "".join((ROOT / "include" / h).read_text() for h in C_HEADERS)
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(hl_[a-z0-9_]+)\s*\(", text)))


def test_library_exports_every_declared_symbol():
    lib = C.CDLL(str(_lib.LIB_PATH))
    syms = declared_symbols()
    assert len(syms) >= 15
    missing = [s for s in syms if not hasattr(lib, s)]
    assert missing == []


def test_binding_covers_header():
    assert sorted(_lib.SIGNATURES) == declared_symbols()


def test_struct_layouts():
    # LineParam is 12 bytes: float angle, int distance, int votes
    # (okano_3_0/HoughLine.h:70-74)
    assert C.sizeof(_lib.hl_line) == 12
    assert _lib.hl_line.distance.offset == 4
    assert C.sizeof(_lib.hl_params) == 32
    # CircleParam: int a, b, radius, votes (okano_3_0/HoughCircle.h:37-44)
    assert C.sizeof(_lib.hl_circle) == 16
    assert C.sizeof(_lib.hl_circle_params) == 20


def test_error_codes_match_reference():
    # okano_3_0/ErrorCode.h:16-56
    assert (_lib.NO_ERROR, _lib.INVALID_DATA, _lib.NULL_POINTER, _lib.OP_OVERFLOW,
            _lib.OUT_OF_MEM, _lib.CUDA_ERROR, _lib.UNIMPLEMENT) == \
        (0, -1, -2, -3, -6, -7, -998)
    hdr = (ROOT / "include" / "houghline_gb300.h").read_text()
    for name, val in [("HL_NO_ERROR", 0), ("HL_INVALID_DATA", -1),
                      ("HL_NULL_POINTER", -2), ("HL_OUT_OF_MEM", -6),
                      ("HL_CUDA_ERROR", -7)]:
        assert re.search(rf"#define {name}\s+{val}\b", hdr)


def test_null_arguments_rejected_without_gpu():
    lib = _lib.load()
    assert lib.hl_create(None, None) == _lib.NULL_POINTER
    assert lib.hl_destroy(None) == _lib.NULL_POINTER
    assert lib.hl_plain(None, None, None, None, None) == _lib.NULL_POINTER
    assert lib.hl_set_vote_shape(None, 0, 0) == _lib.NULL_POINTER


def test_batch_entry_points_reject_null_without_gpu():
    lib = _lib.load()
    assert lib.hl_batch(None, None, 0, None, 0, None, None, None) == _lib.NULL_POINTER
    assert lib.hl_batch_async(None, None, 0, None, 0, None, None, None) == _lib.NULL_POINTER
    assert lib.hl_tiles(None, None, 4, 16, None, None, None) == _lib.NULL_POINTER
    assert lib.hl_circles(None, None, None, None, None, None) == _lib.NULL_POINTER
    assert lib.hl_circle_accumulator(None, None, None, None, None) == _lib.NULL_POINTER
    assert lib.hl_circles_batch(None, None, 0, None, 0, None, None, None) == _lib.NULL_POINTER
    assert lib.hl_set_batch_graph(None, 1) == _lib.NULL_POINTER
    assert lib.hl_autotune(None, None, 0, None, 0, None, None, 0, None, None) == \
        _lib.NULL_POINTER
