"""The output menu's HDF5 format ("Yell 1.0", gen_hdf5_write) through
dgpu_output_write, read back with the oracle's HDF5 reader and compared
with the oracle's restatement of the reference's datasets, bit for bit.

The reader is pinned first on a file assembled here field by field from
the HDF5 file format specification (a two-level group B-tree, a header
continuation, compact and contiguous layouts, big-endian data), a layout
the library's writer does not use.  No GPU: the writer is host code.
"""
import os
import struct
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

from oracle import hdf5 as H  # noqa: E402

from diffusecode_gb300 import output as OUT  # noqa: E402
from diffusecode_gb300.structures import GridData, reciprocal_metric  # noqa: E402


@pytest.fixture(scope="module")
def lib():
    from diffusecode_gb300 import _lib
    try:
        return _lib.load()
    except ImportError as e:
        pytest.skip(str(e))


# ------------------------------------------------------------ reader pin

def _msg(mtype, body, flags=0):
    body = body + b"\0" * (-len(body) % 8)
    return struct.pack("<HHB3x", mtype, len(body), flags) + body


def _header(msgs):
    chunk = b"".join(msgs)
    return struct.pack("<BBHII4x", 1, 0, len(msgs), 1, len(chunk)), chunk


def _handmade():
    """A file with datasets 'a' (compact int32 LE, 2 x 3), 'b' (contiguous
    f32 BE, 4) and 'c' (scalar uint8), the group's symbol table a level-1
    B-tree over two symbol table nodes (leaf K 1: two names per node), the
    root header continued in a second chunk."""
    buf = bytearray(4096)
    eof = [0]

    def put(addr, data):
        buf[addr:addr + len(data)] = data
        eof[0] = max(eof[0], addr + len(data))

    names = ["a", "b", "c"]
    heap_seg = b"\0" * 8 + b"a\0" + b"\0" * 6 + b"b\0" + b"\0" * 6 + b"c\0" + b"\0" * 6
    off = {"a": 8, "b": 16, "c": 24}
    K_NODE = 2
    tree_size = 24 + 2 * K_NODE * 8 + (2 * K_NODE + 1) * 8
    A_ROOT, A_CONT, A_HEAP, A_SEG = 96, 160, 200, 232
    A_T1, A_T0a, A_T0b = 272, 272 + tree_size, 272 + 2 * tree_size
    A_S0, A_S1 = 272 + 3 * tree_size, 272 + 3 * tree_size + 88
    A_DA, A_DB, A_DC, A_RAWB = 1024, 1200, 1400, 1600
    # superblock v0 (leaf K 1, internal K 2)
    sb = H.SIGNATURE + bytes([0, 0, 0, 0, 0, 8, 8, 0]) + struct.pack("<HHI", 1, K_NODE, 0)
    sb += struct.pack("<4Q", 0, H.UNDEF, 0, H.UNDEF)
    sb += struct.pack("<QQI4xQQ", 0, A_ROOT, 1, A_T1, A_HEAP)
    # root header: a continuation into A_CONT, 32 bytes holding the symbol
    # table message and a null message (three messages in all)
    chunk = _msg(0x10, struct.pack("<QQ", A_CONT, 32))
    put(A_ROOT, struct.pack("<BBHII4x", 1, 0, 3, 1, len(chunk)) + chunk)
    put(A_CONT, _msg(0x11, struct.pack("<QQ", A_T1, A_HEAP)) + _msg(0x0, b""))
    put(A_HEAP, b"HEAP" + bytes(4) + struct.pack("<QQQ", len(heap_seg), 1, A_SEG))
    put(A_SEG, heap_seg)

    def tree(level, children, keys):
        t = b"TREE" + bytes([0, level]) + struct.pack("<H", len(children)) + struct.pack("<QQ", H.UNDEF, H.UNDEF)
        for k, ch in enumerate(children):
            t += struct.pack("<QQ", keys[k], ch)
        t += struct.pack("<Q", keys[len(children)])
        return t + bytes(tree_size - len(t))

    put(A_T1, tree(1, [A_T0a, A_T0b], [0, off["b"], off["c"]]))
    put(A_T0a, tree(0, [A_S0], [0, off["b"]]))
    put(A_T0b, tree(0, [A_S1], [off["b"], off["c"]]))

    def snod(entries):
        s = b"SNOD" + bytes([1, 0]) + struct.pack("<H", len(entries))
        for name, hdr in entries:
            s += struct.pack("<QQI4x16x", off[name], hdr, 0)
        return s + bytes(8 + 2 * 40 - len(s))

    put(A_S0, snod([("a", A_DA), ("b", A_DB)]))
    put(A_S1, snod([("c", A_DC)]))
    i32le = bytes([0x10, 0x08, 0, 0]) + struct.pack("<IHH", 4, 0, 32)
    f32be = bytes([0x11, 0x21, 31, 0]) + struct.pack("<IHHBBBBI", 4, 0, 32, 23, 8, 0, 23, 127)
    u8 = bytes([0x10, 0x00, 0, 0]) + struct.pack("<IHH", 1, 0, 8)
    a = np.arange(6, dtype="<i4").reshape(2, 3) - 2
    b = np.array([1.5, -2.25, 3.0e-3, 7.0e5], dtype=">f4")
    space = lambda dims: struct.pack("<BBBB4x", 1, len(dims), 0, 0) + b"".join(struct.pack("<Q", d) for d in dims)
    pre, chunk = _header([_msg(1, space([2, 3])), _msg(3, i32le, 1),
                          _msg(8, struct.pack("<BBH", 3, 0, 24) + a.tobytes())])
    put(A_DA, pre + chunk)
    pre, chunk = _header([_msg(1, space([4])), _msg(3, f32be, 1), _msg(8, struct.pack("<BBQQ", 3, 1, A_RAWB, 16))])
    put(A_DB, pre + chunk)
    put(A_RAWB, b.tobytes())
    pre, chunk = _header([_msg(1, space([])), _msg(3, u8, 1), _msg(8, struct.pack("<BBH", 3, 0, 1) + b"\xc8")])
    put(A_DC, pre + chunk)
    end = eof[0]
    put(0, sb[:40] + struct.pack("<Q", end) + sb[48:])
    return bytes(buf[:end]), a, b


def test_reader_on_a_handmade_file():
    data, a, b = _handmade()
    r = H.read(data)
    assert set(r) == {"a", "b", "c", "__file__"}
    np.testing.assert_array_equal(r["a"][0], a)
    assert r["a"][1] == {"class": "int", "size": 4, "order": "<", "signed": True}
    np.testing.assert_array_equal(r["b"][0], b.astype(np.float64))
    assert r["b"][1]["order"] == ">"
    assert r["c"][0] == 200 and r["c"][1]["signed"] is False


def test_reader_rejects_damaged_files():
    data, _, _ = _handmade()
    with pytest.raises(H.H5Error):
        H.read(data[:-8])                               # shorter than its end-of-file address
    bad = bytearray(data)
    bad[0] = 0
    with pytest.raises(H.H5Error):
        H.read(bytes(bad))


# ------------------------------------------------------------ the writer

RTEN = reciprocal_metric(4.1, 4.3, 5.2, 88, 92, 95)


class Cr:
    icc = (1, 1, 1)
    rten = RTEN


def grid(inc):
    ll = np.array([-2.0, -1.5, 0.25])
    lr = ll + np.array([0.5 * (inc[0] - 1), 0.1 * (inc[0] - 1), 0.0])
    ul = ll + np.array([0.0, 0.25 * (inc[1] - 1), 0.05 * (inc[1] - 1)])
    tl = ll + np.array([0.02 * (inc[2] - 1), 0.0, 0.75 * (inc[2] - 1)])
    return GridData.from_corners(ll, lr, ul, tl, inc=inc)


def check(path, g, v, value, extr, a0, win, valmax, scale):
    r = H.read(open(path, "rb").read())
    want = H.yell(g.inc, g.eck, g.vi, extr, a0, win, value, v.reshape(-1, order="F"), valmax=valmax, scale=scale)
    assert r["__file__"]["eof"] == r["__file__"]["size"]
    assert set(r) - {"__file__"} == set(want)
    got, dt = r["data"]
    assert dt == {"class": "float", "size": 8, "order": "<"} and got.shape == tuple(g.inc)
    np.testing.assert_array_equal(got, want["data"])
    for name in ("lower_limits", "step_sizes", "step_sizes_abs", "step_sizes_ord", "step_sizes_top", "unit_cell"):
        got, dt = r[name]
        assert dt == {"class": "float", "size": 8, "order": ">"}, name
        np.testing.assert_array_equal(got, want[name], err_msg=name)
    assert r["is_direct"][0] == want["is_direct"]
    assert r["is_direct"][1] == {"class": "int", "size": 1, "order": ">", "signed": True}
    assert r["format"][0] == want["format"]
    assert r["format"][1]["class"] == "vlstring" and r["format"][1]["pad"] == 0
    assert r["PROGRAM"][0] == want["PROGRAM"]
    assert r["PROGRAM"][1] == {"class": "string", "size": 9, "pad": 0, "cset": 0}


@pytest.mark.parametrize("inc", [(5, 4, 3), (7, 6, 1), (9, 1, 1), (1, 1, 1)])
@pytest.mark.parametrize("value,valmax,scale", [(1, 0.0, 1.0), (14, 0.0, 2.5), (1, 10000.0, 1.0),
                                                (15, 0.37, 3.0), (2, -1.0, 0.5)])
def test_yell_file(lib, tmp_path, inc, value, valmax, scale):
    g = grid(inc)
    rng = np.random.Generator(np.random.PCG64(sum(inc) * 31 + value))
    v = rng.uniform(-5.0, 50.0, size=inc)
    v.reshape(-1)[::5] *= 1e-7
    extr = (2, 3, 1) if value == 14 else (1, 2, 3)
    a0, win = (4.1, 4.3, 5.2), (88.0, 92.0, 95.0)
    p = str(tmp_path / "out.h5")
    spec = OUT.output_spec("hdf5", g, value=value, extr=extr, cr=Cr(), valmax=valmax, scale=scale, a0=a0, win=win)
    OUT.write(p, spec, v)
    check(p, g, v, value, extr, a0, win, valmax, scale)


def test_yell_cell_from_the_metric_and_negative_maximum(lib, tmp_path):
    """unit_cell from the inverse of cr_rten when a0/win are not given; a
    negative largest value leaves valmax's scaling out (MAXVAL < 0)."""
    g = grid((4, 3, 2))
    v = -np.abs(np.random.Generator(np.random.PCG64(5)).uniform(1.0, 2.0, size=g.inc))
    p = str(tmp_path / "neg.h5")
    OUT.write(p, OUT.output_spec("hdf5", g, cr=Cr(), valmax=100.0), v)
    r = H.read(open(p, "rb").read())
    np.testing.assert_allclose(r["unit_cell"][0], [4.1, 4.3, 5.2, 88.0, 92.0, 95.0], rtol=1e-12)
    np.testing.assert_array_equal(r["data"][0], v)     # data[i, j, k] = qval(i, j, k)


def test_yell_rewrites_an_existing_file_and_reports_io_errors(lib, tmp_path):
    g = grid((3, 3, 1))
    p = tmp_path / "x.h5"
    p.write_bytes(b"x" * 100000)                       # an older, longer file is replaced
    v = np.ones(g.inc)
    OUT.write(str(p), OUT.output_spec("hdf5", g), v)
    r = H.read(p.read_bytes())
    assert r["__file__"]["eof"] == p.stat().st_size
    with pytest.raises(OSError):
        OUT.write(str(tmp_path / "no" / "such" / "dir.h5"), OUT.output_spec("hdf5", g), v)
