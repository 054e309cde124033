"""Mesh and cell-data I/O in the VTK formats the reference reads and writes.

* ``read_mesh(path)``: legacy VTK (``.vtk``, ASCII or binary
  UNSTRUCTURED_GRID) or XML VTU (``.vtu``, ascii / base64 binary / raw
  appended data, optionally zlib-compressed), as TNL's mesh readers accept
  them (control.h:20-47, configSetup.h:16-21).  Triangle (VTK type 5),
  tetrahedron (10), quadrilateral (9) and hexahedron (12) cells, and the
  axis-aligned pixel (8) and voxel (11) cells, whose vertices are reordered
  into the quadrilateral / hexahedron order (VTK numbers a pixel's corners
  in lexicographic order, a quadrilateral's counterclockwise).
* Netgen's neutral format (``.ng``, triangles and tetrahedra), the third
  mesh format of configSetup.h:16-21; ``write_netgen`` writes it.
* ``read_cell_data(path, name)``: a cell array from a VTU file, e.g. the
  initial condition ``InitialCondition[Z0]`` (Solver.hpp:296-306).
* ``write_vtu(path, coords, cells, cell_data, ...)``: the snapshot files
  ``data_%05d.vtu`` with cell field ``Z`` (HeatEquationModel.h:164-231).

Points are stored 3D in VTK; 2D meshes drop the z coordinate on reading.
"""
from __future__ import annotations

import base64
import struct
import xml.etree.ElementTree as ET
import zlib
from pathlib import Path

import numpy as np

VTK_TRIANGLE = 5
VTK_TETRA = 10
VTK_PIXEL = 8
VTK_QUAD = 9
VTK_VOXEL = 11
VTK_HEXAHEDRON = 12
# (dimension, vertices per cell, order into the quadrilateral / hexahedron numbering) per cell type
_CELL_TYPES = {VTK_TRIANGLE: (2, 3, None), VTK_TETRA: (3, 4, None), VTK_QUAD: (2, 4, None),
               VTK_HEXAHEDRON: (3, 8, None), VTK_PIXEL: (2, 4, [0, 1, 3, 2]),
               VTK_VOXEL: (3, 8, [0, 1, 3, 2, 4, 5, 7, 6])}
_NP_OF = {"Float32": np.float32, "Float64": np.float64, "Int8": np.int8, "UInt8": np.uint8, "Int16": np.int16,
          "UInt16": np.uint16, "Int32": np.int32, "UInt32": np.uint32, "Int64": np.int64, "UInt64": np.uint64}
_VTK_OF = {np.dtype(v).str[1:]: k for k, v in _NP_OF.items()}


def _cells_of(types: np.ndarray, conn: np.ndarray):
    """Dimension and the [C][nv] cell array of a mesh of one cell kind
    (pixels / voxels reordered into the quadrilateral / hexahedron order)."""
    types = np.asarray(types)
    kinds = set(int(t) for t in np.unique(types))
    if not kinds or not kinds <= set(_CELL_TYPES):
        raise ValueError("supported cells: triangles (VTK 5), tetrahedra (10), quadrilaterals (9), "
                         "hexahedra (12), pixels (8), voxels (11)")
    shapes = {_CELL_TYPES[k][:2] for k in kinds}
    if len(shapes) != 1:
        raise ValueError("mixed cell kinds are not supported")
    dim, nv = shapes.pop()
    conn = np.asarray(conn, np.int64)
    if conn.size != types.size * nv:
        raise ValueError(f"connectivity does not match the cell types ({nv} vertices per cell)")
    cells = conn.reshape(-1, nv).copy()
    for k in kinds:
        order = _CELL_TYPES[k][2]
        if order is not None:
            sel = types == k
            cells[sel] = cells[sel][:, order]
    return dim, cells


def _cell_type(dim: int, nv: int) -> int:
    if nv == dim + 1:
        return VTK_TRIANGLE if dim == 2 else VTK_TETRA
    if nv == 2 ** dim:
        return VTK_QUAD if dim == 2 else VTK_HEXAHEDRON
    raise ValueError(f"no VTK cell with {nv} vertices in {dim}D")


# ---- legacy VTK -------------------------------------------------------------


def _read_legacy(path: Path):
    data = path.read_bytes()
    lines = data.split(b"\n")
    if not lines[0].startswith(b"# vtk DataFile"):
        raise ValueError(f"{path}: not a legacy VTK file")
    binary = lines[2].strip().upper() == b"BINARY"
    pos = len(lines[0]) + len(lines[1]) + len(lines[2]) + 3

    def next_line():
        nonlocal pos
        while True:
            end = data.index(b"\n", pos)
            line = data[pos:end].strip()
            pos = end + 1
            if line:
                return line.decode()

    def read_values(count, dtype_str):
        nonlocal pos
        if binary:
            dt = np.dtype(dtype_str).newbyteorder(">")
            arr = np.frombuffer(data, dtype=dt, count=count, offset=pos).astype(dtype_str)
            pos += count * dt.itemsize
            return arr
        vals = []
        while len(vals) < count:
            vals.extend(next_line().split())
        return np.array(vals[:count], dtype=dtype_str)

    coords = cells = types = None
    vtk_types = {"float": "f4", "double": "f8", "int": "i4", "long": "i8", "vtktypeint64": "i8"}
    while pos < len(data):
        try:
            line = next_line()
        except ValueError:
            break
        key = line.split()
        head = key[0].upper()
        if head == "DATASET" and key[1].upper() != "UNSTRUCTURED_GRID":
            raise ValueError("only UNSTRUCTURED_GRID datasets are supported")
        if head == "POINTS":
            n = int(key[1])
            coords = read_values(3 * n, vtk_types.get(key[2].lower(), "f8")).reshape(n, 3).astype(np.float64)
        elif head == "CELLS":
            ncell, size = int(key[1]), int(key[2])
            raw = read_values(size, "i4").astype(np.int64)
            conn, sizes, q = [], [], 0
            for _ in range(ncell):
                k = int(raw[q])
                conn.append(raw[q + 1:q + 1 + k])
                sizes.append(k)
                q += 1 + k
            if len(set(sizes)) > 1:
                raise ValueError("mixed cell sizes are not supported")
            cells = np.concatenate(conn) if conn else np.zeros(0, np.int64)
        elif head == "CELL_TYPES":
            types = read_values(int(key[1]), "i4")
            break
    if coords is None or cells is None or types is None:
        raise ValueError(f"{path}: POINTS, CELLS or CELL_TYPES missing")
    dim, cells = _cells_of(types, cells)
    return coords[:, :dim].copy(), cells.astype(np.int32)


# ---- VTU ------------------------------------------------------------------------


def _decode_inline(text: str, dtype, compressed: bool, header_dtype):
    raw = base64.b64decode("".join(text.split()))
    hsize = np.dtype(header_dtype).itemsize
    if not compressed:
        n = int(np.frombuffer(raw[:hsize], dtype=header_dtype)[0])
        return np.frombuffer(raw[hsize:hsize + n], dtype=dtype)
    nblocks = int(np.frombuffer(raw[:hsize], dtype=header_dtype)[0])
    # the header itself is base64-encoded separately from the blocks in VTK's
    # compressed format: [nblocks, block size, last size, c1, c2, ...]
    hdr_len = (3 + nblocks) * hsize
    hdr_b64_len = 4 * ((hdr_len + 2) // 3)
    compact = "".join(text.split())
    hdr = np.frombuffer(base64.b64decode(compact[:hdr_b64_len])[:hdr_len], dtype=header_dtype)
    body = base64.b64decode(compact[hdr_b64_len:])
    out, off = [], 0
    for c in hdr[3:3 + nblocks]:
        out.append(zlib.decompress(body[off:off + int(c)]))
        off += int(c)
    return np.frombuffer(b"".join(out), dtype=dtype)


def _decode_appended(buf: bytes, offset: int, dtype, compressed: bool, header_dtype):
    hsize = np.dtype(header_dtype).itemsize
    if not compressed:
        n = int(np.frombuffer(buf[offset:offset + hsize], dtype=header_dtype)[0])
        return np.frombuffer(buf[offset + hsize:offset + hsize + n], dtype=dtype)
    nblocks = int(np.frombuffer(buf[offset:offset + hsize], dtype=header_dtype)[0])
    hdr = np.frombuffer(buf[offset:offset + (3 + nblocks) * hsize], dtype=header_dtype)
    pos = offset + (3 + nblocks) * hsize
    out = []
    for c in hdr[3:3 + nblocks]:
        out.append(zlib.decompress(buf[pos:pos + int(c)]))
        pos += int(c)
    return np.frombuffer(b"".join(out), dtype=dtype)


class _Vtu:
    def __init__(self, path: Path):
        raw = path.read_bytes()
        self.appended = b""
        i = raw.find(b"<AppendedData")
        if i >= 0:
            gt = raw.index(b">", i)
            self.appended = raw[raw.index(b"_", gt) + 1:raw.rfind(b"</AppendedData>")]
            # the grid is closed before <AppendedData>: keep the XML part only
            xml = raw[:gt + 1] + b"</AppendedData></VTKFile>"
        else:
            xml = raw
        self.root = ET.fromstring(xml)
        self.compressed = self.root.get("compressor") is not None
        self.header = np.uint64 if self.root.get("header_type", "UInt32") == "UInt64" else np.uint32
        if self.root.get("byte_order", "LittleEndian") != "LittleEndian":
            raise ValueError("big-endian VTU is not supported")
        self.piece = self.root.find("UnstructuredGrid/Piece")

    def array(self, el):
        dtype = _NP_OF[el.get("type")]
        fmt = el.get("format", "ascii")
        if fmt == "ascii":
            return np.array(el.text.split(), dtype=dtype)
        if fmt == "binary":
            return _decode_inline(el.text, dtype, self.compressed, self.header)
        return _decode_appended(self.appended, int(el.get("offset")), dtype, self.compressed, self.header)

    def named(self, section: str, name: str):
        for el in self.piece.find(section).findall("DataArray"):
            if el.get("Name") == name:
                return self.array(el)
        return None


def _read_vtu(path: Path):
    v = _Vtu(path)
    pts = v.array(v.piece.find("Points/DataArray")).astype(np.float64).reshape(-1, 3)
    conn = v.named("Cells", "connectivity").astype(np.int64)
    offs = v.named("Cells", "offsets").astype(np.int64)
    types = v.named("Cells", "types").astype(np.int64)
    dim, cells = _cells_of(types, conn)
    nv = cells.shape[1]
    if not np.array_equal(offs, np.arange(1, cells.shape[0] + 1) * nv):
        raise ValueError("mixed cell sizes are not supported")
    return pts[:, :dim].copy(), cells.astype(np.int32)


# ---- Netgen ---------------------------------------------------------------------


def _read_netgen(path: Path):
    """Netgen's neutral mesh format (the `ng` mesh-format of configSetup.h:16-21):
    the number of points, one point per line (2 or 3 coordinates), the number
    of elements, one element per line as a material index followed by its
    1-based vertex indices (3 for triangles, 4 for tetrahedra), then
    optionally the boundary elements, which carry no information the solver
    needs (faces and their boundary flags follow from the cells)."""
    tokens = path.read_text().split("\n")
    lines = [ln.split() for ln in tokens if ln.strip()]
    npts = int(lines[0][0])
    pts = np.array([[float(v) for v in ln] for ln in lines[1:1 + npts]], dtype=np.float64)
    if pts.ndim != 2 or pts.shape[1] not in (2, 3):
        raise ValueError(f"{path}: points must have 2 or 3 coordinates")
    ncell = int(lines[1 + npts][0])
    rows = lines[2 + npts:2 + npts + ncell]
    if len(rows) != ncell:
        raise ValueError(f"{path}: expected {ncell} elements")
    cells = np.array([[int(v) for v in ln[1:]] for ln in rows], dtype=np.int64) - 1
    dim = pts.shape[1]
    if cells.shape[1] != dim + 1:
        raise ValueError(f"{path}: {dim}D Netgen meshes hold simplices with {dim + 1} vertices")
    if cells.min(initial=0) < 0 or cells.max(initial=0) >= npts:
        raise ValueError(f"{path}: vertex index out of range")
    return pts, cells.astype(np.int32)


def write_netgen(path, coords: np.ndarray, cells: np.ndarray) -> None:
    """The same neutral format (material 1, no boundary elements)."""
    coords = np.asarray(coords, np.float64)
    with open(path, "w") as fh:
        fh.write(f"{coords.shape[0]}\n")
        np.savetxt(fh, coords, fmt="%.17g")
        fh.write(f"{cells.shape[0]}\n")
        np.savetxt(fh, np.hstack([np.ones((cells.shape[0], 1), np.int64), np.asarray(cells, np.int64) + 1]), fmt="%d")
        fh.write("0\n")


def read_mesh(path, fmt: str = "auto"):
    path = Path(path)
    fmt = path.suffix[1:].lower() if fmt == "auto" else fmt
    if fmt == "vtk":
        return _read_legacy(path)
    if fmt == "vtu":
        return _read_vtu(path)
    if fmt == "ng":
        return _read_netgen(path)
    raise ValueError(f"unsupported mesh format {fmt!r} (vtk, vtu, ng)")


def read_cell_data(path, name: str) -> np.ndarray:
    v = _Vtu(Path(path))
    arr = v.named("CellData", name)
    if arr is None:
        raise KeyError(f"{path}: no cell array named {name!r}")
    return arr.astype(np.float64)


def write_vtu(path, coords: np.ndarray, cells: np.ndarray, cell_data: dict, time: float | None = None,
              cycle: int | None = None, compress: bool = True) -> None:
    """Writes an UnstructuredGrid VTU with raw appended (optionally zlib) data."""
    coords = np.asarray(coords, np.float64)
    cells = np.asarray(cells, np.int64)
    C, nv = cells.shape
    dim = coords.shape[1]
    pts = np.zeros((coords.shape[0], 3))
    pts[:, :dim] = coords
    ctype = _cell_type(dim, nv)
    arrays = []  # (section, name, ncomp, ndarray)
    arrays.append(("Points", "Points", 3, pts.ravel()))
    arrays.append(("Cells", "connectivity", 1, cells.ravel()))
    arrays.append(("Cells", "offsets", 1, np.arange(1, C + 1, dtype=np.int64) * nv))
    arrays.append(("Cells", "types", 1, np.full(C, ctype, np.uint8)))
    for name, arr in cell_data.items():
        arrays.append(("CellData", name, 1, np.ascontiguousarray(arr)))
    blobs, offsets, off = [], [], 0
    for _, _, _, arr in arrays:
        raw = np.ascontiguousarray(arr).tobytes()
        if compress:
            comp = zlib.compress(raw)
            blob = struct.pack("<QQQQ", 1, len(raw), len(raw), len(comp)) + comp
        else:
            blob = struct.pack("<Q", len(raw)) + raw
        blobs.append(blob)
        offsets.append(off)
        off += len(blob)
    comp_attr = ' compressor="vtkZLibDataCompressor"' if compress else ""
    out = [f'<?xml version="1.0"?>\n<VTKFile type="UnstructuredGrid" version="1.0" byte_order="LittleEndian" '
           f'header_type="UInt64"{comp_attr}>\n<UnstructuredGrid>\n']
    if time is not None or cycle is not None:
        out.append("<FieldData>\n")
        if time is not None:
            out.append('<DataArray type="Float64" Name="TIME" NumberOfTuples="1" format="ascii">'
                       f"{time!r}</DataArray>\n")
        if cycle is not None:
            out.append('<DataArray type="Int32" Name="CYCLE" NumberOfTuples="1" format="ascii">'
                       f"{int(cycle)}</DataArray>\n")
        out.append("</FieldData>\n")
    out.append(f'<Piece NumberOfPoints="{pts.shape[0]}" NumberOfCells="{C}">\n')
    sections = {"Points": [], "Cells": [], "CellData": []}
    for (sec, name, ncomp, arr), o in zip(arrays, offsets):
        t = _VTK_OF[np.asarray(arr).dtype.str[1:]]
        sections[sec].append(f'<DataArray type="{t}" Name="{name}" NumberOfComponents="{ncomp}" '
                             f'format="appended" offset="{o}"/>\n')
    out.append("<Points>\n" + "".join(sections["Points"]) + "</Points>\n")
    out.append("<Cells>\n" + "".join(sections["Cells"]) + "</Cells>\n")
    out.append("<CellData>\n" + "".join(sections["CellData"]) + "</CellData>\n")
    out.append("</Piece>\n</UnstructuredGrid>\n<AppendedData encoding=\"raw\">\n_")
    with open(path, "wb") as fh:
        fh.write("".join(out).encode())
        for b in blobs:
            fh.write(b)
        fh.write(b"\n</AppendedData>\n</VTKFile>\n")


def write_legacy_vtk(path, coords: np.ndarray, cells: np.ndarray) -> None:
    """ASCII legacy VTK unstructured grid (mesh only)."""
    coords = np.asarray(coords, np.float64)
    C, nv = cells.shape
    pts = np.zeros((coords.shape[0], 3))
    pts[:, :coords.shape[1]] = coords
    ctype = _cell_type(coords.shape[1], nv)
    with open(path, "w") as fh:
        fh.write("# vtk DataFile Version 2.0\nmhfem mesh\nASCII\nDATASET UNSTRUCTURED_GRID\n")
        fh.write(f"POINTS {pts.shape[0]} double\n")
        np.savetxt(fh, pts, fmt="%.17g")
        fh.write(f"CELLS {C} {C * (nv + 1)}\n")
        np.savetxt(fh, np.hstack([np.full((C, 1), nv), cells]), fmt="%d")
        fh.write(f"CELL_TYPES {C}\n")
        np.savetxt(fh, np.full((C, 1), ctype), fmt="%d")
