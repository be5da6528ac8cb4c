"""Scene-file host code of the library (header parser, body read, writer)
against the oracle's restatement of the reference's PLY layout, and the
oracle's property names against the reference's own
construct_list_of_attributes (tests/golden/ply_attributes.json).  CPU only:
these entry points touch no device."""
import ctypes
import json
import os

import numpy as np
import pytest

import oracle as orc

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden",
                    "ply_attributes.json")


def scene(n, D, seed=0):
    rng = np.random.default_rng(seed)
    K = D - 3
    return {"xyz": rng.standard_normal((n, 3)), "mean": rng.standard_normal((n, K)),
            "rgb": rng.random((n, 3)), "opacity": rng.standard_normal((n, 1)),
            "beta": rng.standard_normal((n, D - 2)), "scale": rng.standard_normal((n, D)),
            "l_triangle": rng.standard_normal((n, D * (D - 1) // 2))}


@pytest.fixture(scope="module")
def lib():
    from ubs import _lib as L
    return L


@pytest.mark.parametrize("D", [6, 7])
def test_oracle_names_match_reference(D):
    want = json.load(open(GOLD))["d%d" % D]
    assert orc.ply_attribute_names(D - 2, D - 3, D, D * (D - 1) // 2) == want
    from ubs.ply import attribute_names
    assert attribute_names({"beta": D - 2, "mean": D - 3, "scale": D,
                            "l_triangle": D * (D - 1) // 2}) == want


@pytest.mark.parametrize("D", [6, 7])
def test_writer_bytes_equal_oracle(lib, tmp_path, D):
    from ubs import ply
    p = scene(257, D)
    names = orc.ply_attribute_names(D - 2, D - 3, D, D * (D - 1) // 2)
    recs = np.frombuffer(orc.ply_bytes(p), np.uint8)
    body = orc.ply_bytes(p)
    hdr_len = body.index(b"end_header\n") + len(b"end_header\n")
    rec = np.frombuffer(body[hdr_len:], "<f4").copy()
    nb = ctypes.create_string_buffer(len(names) * ply.NAME_BYTES)
    for i, nm in enumerate(names):
        ctypes.memmove(ctypes.addressof(nb) + i * ply.NAME_BYTES, nm.encode(), len(nm))
    path = str(tmp_path / "s.ply")
    lib.call("ubs_ply_write", os.fsencode(path), 257, len(names), nb,
             ctypes.c_void_p(rec.ctypes.data))
    assert open(path, "rb").read() == body
    assert len(recs) == len(body)


def test_header_parser_and_body_reader(lib, tmp_path):
    from ubs import ply
    p = scene(100, 6, 1)
    names = orc.ply_attribute_names(4, 3, 6, 15)[::-1] + ["extra_0"]  # any order, extra
    data = orc.ply_bytes(p, names=names, comments=("made by the oracle", "second"))
    path = str(tmp_path / "r.ply")
    open(path, "wb").write(data)
    n, got_names, off = ply.read_header(path)
    assert n == 100 and got_names == names
    assert data[off - len(b"end_header\n"):off] == b"end_header\n"
    buf = np.zeros(100 * len(names), np.float32)
    lib.call("ubs_ply_read_body", os.fsencode(path), off, ctypes.c_void_p(buf.ctypes.data),
             buf.nbytes)
    assert buf.tobytes() == data[off:]
    cmap = ply.column_map(got_names)
    want = orc.ply_parse(data)
    rec = buf.reshape(100, -1)
    for k, cols in cmap.items():
        assert np.array_equal(rec[:, cols], want[k]), k


@pytest.mark.parametrize("header,err", [
    (b"ply\nformat ascii 1.0\nelement vertex 1\nproperty float x\nend_header\n1\n", "format ascii"),
    (b"ply\nformat binary_big_endian 1.0\nelement vertex 1\nproperty float x\nend_header\n",
     "big"),
    (b"ply\nformat binary_little_endian 1.0\nelement vertex 1\nproperty double x\n"
     b"end_header\n", "type double"),
    (b"ply\nformat binary_little_endian 1.0\nelement vertex 2\nproperty float x\n"
     b"end_header\n\0\0\0\0", "truncated"),
    (b"not a ply\n", "not a PLY"),
    (b"ply\nformat binary_little_endian 1.0\nelement face 3\nproperty list uchar int v\n"
     b"element vertex 1\nproperty float x\nend_header\n\0\0\0\0", "face"),
])
def test_header_errors(lib, tmp_path, header, err):
    from ubs import ply
    path = str(tmp_path / "bad.ply")
    open(path, "wb").write(header)
    with pytest.raises(RuntimeError) as e:
        ply.read_header(path)
    assert err in str(e.value)


def test_empty_trailing_element_is_accepted(lib, tmp_path):
    from ubs import ply
    data = (b"ply\nformat binary_little_endian 1.0\nelement vertex 1\nproperty float x\n"
            b"element face 0\nproperty list uchar int vertex_indices\nend_header\n"
            + np.float32(2.5).tobytes())
    path = str(tmp_path / "f.ply")
    open(path, "wb").write(data)
    n, names, off = ply.read_header(path)
    assert (n, names, off) == (1, ["x"], len(data) - 4)
