"""VTK XML PolyData (.vtp) files through the host reader and writer (CPU only).

vtkSurface::CreateFromFile reads .vtp with vtkXMLPolyDataReader and WriteToFile writes
it with vtkXMLPolyDataWriter (Common/vtkSurface.cxx:1993-1998, 2050-2056).  The files
here are built by `_vtp` below from the published layout of VTK's XML formats: ascii,
inline base64 and appended (raw or base64) data arrays; UInt32 or UInt64 block headers;
uncompressed or zlib-compressed in blocks; either byte order; several pieces.  Python's
zlib makes the compressed blocks, so the reader's own DEFLATE decoder is checked against
an independent encoder (stored, fixed-Huffman and dynamic-Huffman blocks).
"""
import base64
import struct
import zlib

import numpy as np
import pytest

import acvd_gb300
from acvd_gb300 import engine as E
from acvd_gb300 import synth

_FMT = {"Float32": "f", "Float64": "d", "Int32": "i", "Int64": "q", "UInt32": "I", "UInt64": "Q",
        "Int16": "h", "UInt16": "H", "Int8": "b", "UInt8": "B"}


def _raw(values, vtype, order):
    return struct.pack(order + str(len(values)) + _FMT[vtype], *values)


def _block(raw, order, header, compress, block_size, level=6, strategy=None):
    h = "I" if header == "UInt32" else "Q"
    if not compress:
        return struct.pack(order + h, len(raw)) + raw, None
    chunks = [raw[i:i + block_size] for i in range(0, len(raw), block_size)] or [b""]
    comp = []
    for c in chunks:
        if strategy is None:
            comp.append(zlib.compress(c, level))
        else:
            o = zlib.compressobj(level, zlib.DEFLATED, 15, 8, strategy)
            comp.append(o.compress(c) + o.flush())
    last = len(chunks[-1]) if len(chunks[-1]) != block_size else 0
    head = struct.pack(order + h * (3 + len(comp)), len(comp), block_size, last, *[len(c) for c in comp])
    return head, b"".join(comp)


def _vtp(pieces, mode="binary", header="UInt64", compress=False, order="<", block_size=1 << 15, ptype="Float32",
         itype="Int64", level=6, strategy=None, appended_encoding="raw"):
    """pieces: [(points (n, 3), polygons: list of vertex lists)]"""
    bo = "LittleEndian" if order == "<" else "BigEndian"
    comp = ' compressor="vtkZLibDataCompressor"' if compress else ""
    xml = [f'<?xml version="1.0"?>\n<VTKFile type="PolyData" version="1.0" byte_order="{bo}" '
           f'header_type="{header}"{comp}>\n  <PolyData>\n']
    appended = b""

    def array(name, vtype, values, ncomp=1):
        nonlocal appended
        attrs = f'type="{vtype}" Name="{name}"' + (f' NumberOfComponents="{ncomp}"' if ncomp > 1 else "")
        if mode == "ascii":
            return f'<DataArray {attrs} format="ascii">\n{" ".join(repr(v) for v in values)}\n</DataArray>\n'
        head, data = _block(_raw(values, vtype, order), order, header, compress, block_size, level, strategy)
        if mode == "binary":
            # VTK encodes a compressed block's header apart from its data
            text = (base64.b64encode(head) + base64.b64encode(data)) if data is not None else base64.b64encode(head)
            return f'<DataArray {attrs} format="binary">\n{text.decode()}\n</DataArray>\n'
        blob = head + (data or b"")
        if appended_encoding == "base64":
            blob = base64.b64encode(head) + (base64.b64encode(data) if data is not None else b"")
        off = len(appended)
        appended += blob
        return f'<DataArray {attrs} format="appended" offset="{off}"/>\n'

    for pts, polys in pieces:
        conn = [int(v) for p in polys for v in p]
        offs = [int(v) for v in np.cumsum([len(p) for p in polys])] if polys else []
        xml.append(f'    <Piece NumberOfPoints="{len(pts)}" NumberOfVerts="0" NumberOfLines="0" '
                   f'NumberOfStrips="0" NumberOfPolys="{len(polys)}">\n      <PointData>\n      </PointData>\n'
                   '      <Points>\n')
        xml.append(array("Points", ptype, [float(v) for v in np.asarray(pts).reshape(-1)], 3))
        xml.append('      </Points>\n      <Polys>\n')
        xml.append(array("connectivity", itype, conn))
        xml.append(array("offsets", itype, offs))
        xml.append('      </Polys>\n    </Piece>\n')
    xml.append("  </PolyData>\n")
    out = "".join(xml).encode()
    if mode == "appended":
        out += f'  <AppendedData encoding="{appended_encoding}">\n   _'.encode() + appended + \
            b"\n  </AppendedData>\n"
    return out + b"</VTKFile>\n"


def _mesh():
    m = synth.torus(24, 12, seed=1)
    return m.points.astype(np.float32).astype(np.float64), m.faces


CASES = {
    "ascii": dict(mode="ascii", ptype="Float64"),
    "binary_u64": dict(mode="binary"),
    "binary_u32_int32": dict(mode="binary", header="UInt32", itype="Int32"),
    "binary_zlib_blocks": dict(mode="binary", compress=True, block_size=1000),
    "binary_zlib_stored": dict(mode="binary", compress=True, level=0),
    "binary_zlib_fixed": dict(mode="binary", compress=True, strategy=zlib.Z_FIXED),
    "appended_raw_zlib": dict(mode="appended", compress=True, header="UInt32", block_size=777),
    "appended_raw": dict(mode="appended"),
    "appended_b64_zlib": dict(mode="appended", compress=True, appended_encoding="base64", block_size=4096),
    "appended_b64": dict(mode="appended", appended_encoding="base64", header="UInt32"),
    "big_endian_zlib": dict(mode="binary", order=">", compress=True, ptype="Float64", itype="UInt32"),
}


@pytest.mark.parametrize("name", sorted(CASES))
def test_vtp_layouts(tmp_path, name):
    pts, faces = _mesh()
    path = tmp_path / "m.vtp"
    path.write_bytes(_vtp([(pts, faces.tolist())], **CASES[name]))
    p2, f2 = E.read_mesh(str(path))
    np.testing.assert_array_equal(p2, pts)
    np.testing.assert_array_equal(f2, faces)


def test_vtp_pieces_are_concatenated(tmp_path):
    pts, faces = _mesh()
    h = synth.heightfield(9, seed=3)
    hp = h.points.astype(np.float32).astype(np.float64)
    path = tmp_path / "two.vtp"
    path.write_bytes(_vtp([(pts, faces.tolist()), (hp, h.faces.tolist())], mode="appended", compress=True))
    p2, f2 = E.read_mesh(str(path))
    np.testing.assert_array_equal(p2, np.vstack([pts, hp]))
    np.testing.assert_array_equal(f2, np.vstack([faces, h.faces + pts.shape[0]]))


def test_vtp_writer_round_trip(tmp_path):
    pts, faces = _mesh()
    path = str(tmp_path / "w.vtp")
    E.write_mesh(path, pts, faces)
    p2, f2 = E.read_mesh(path)
    np.testing.assert_array_equal(p2, pts)
    np.testing.assert_array_equal(f2, faces)
    s = acvd_gb300.Surface.CreateFromFile(path)
    assert s.GetNumberOfPoints() == pts.shape[0] and s.GetNumberOfCells() == faces.shape[0]


def test_large_zlib_array(tmp_path):
    """Dynamic-Huffman blocks with long matches and block boundaries inside one array."""
    m = synth.torus(200, 100, seed=2)
    pts = m.points.astype(np.float32).astype(np.float64)
    path = tmp_path / "big.vtp"
    path.write_bytes(_vtp([(pts, m.faces.tolist())], mode="appended", compress=True, level=9,
                          block_size=1 << 15))
    p2, f2 = E.read_mesh(str(path))
    np.testing.assert_array_equal(p2, pts)
    np.testing.assert_array_equal(f2, m.faces)


def test_vtp_errors(tmp_path):
    pts, faces = _mesh()
    good = _vtp([(pts, faces.tolist())], mode="binary", compress=True)

    def expect(data, code=None):
        path = tmp_path / "bad.vtp"
        path.write_bytes(data)
        with pytest.raises(acvd_gb300.AcvdError) as ei:
            E.read_mesh(str(path))
        if code is not None:
            assert ei.value.code == code

    # a flipped byte inside the compressed data: the DEFLATE stream or its Adler-32 fails
    text = good.decode()
    i = text.index('format="binary">') + 60
    flipped = text[:i] + ("A" if text[i] != "A" else "B") + text[i + 1:]
    expect(flipped.encode())
    # a quad
    expect(_vtp([(pts[:4], [[0, 1, 2, 3]])], mode="ascii"), code=5)
    # other compressors and data sets are refused
    expect(good.replace(b"vtkZLibDataCompressor", b"vtkLZ4DataCompressor"), code=5)
    expect(good.replace(b'type="PolyData"', b'type="UnstructuredGrid"'), code=5)
    expect(good.replace(b'NumberOfStrips="0"', b'NumberOfStrips="2"'), code=5)
    # a face past the points, truncated data, not XML
    expect(_vtp([(pts[:3], [[0, 1, 3]])], mode="ascii"))
    expect(good[: len(good) // 2])
    expect(b"solid nothing\n")
