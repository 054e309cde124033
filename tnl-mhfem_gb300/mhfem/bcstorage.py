"""Boundary-condition storage: the Python side of the reference's
BoundaryConditionsStorage (BoundaryConditionsStorage.h:9-72) and its tags
(BoundaryConditionsType.h:7-31), with the fields the pytnl binding exposes
(src/pytnl/BoundaryConditionsStorage.h:16-47).

File format.  The reference stores this object with TNL's own binary File
serialization (an object-type string, dofSize, then the three arrays).  TNL
is not available, so this library writes a documented equivalent: the magic
line ``MHFEM-BCS 1\\n``, the serialization type
``TNL::MHFEM::BoundaryConditionsStorage< double >`` as a little-endian int32
length plus bytes, dofSize as int64, then tags (uint8), values and
dirichletValues (float64), each preceded by its int64 element count.  All
arrays are indexed i*F + E.  ``load`` also reads files in the layout the
reference writes through TNL's File (``load_tnl``), e.g. the ``boundary.tnl``
of its examples/HeatEquation/init.py, checked structurally.
"""
from __future__ import annotations

import enum
import struct
from pathlib import Path

import numpy as np

MAGIC = b"MHFEM-BCS 1\n"
SERIALIZATION_TYPE = "TNL::MHFEM::BoundaryConditionsStorage< double >"


class BoundaryConditionsType(enum.IntEnum):
    FixedValue = 0
    FixedFlux = 1
    AdvectiveOutflow = 2
    FixedFluxNoAdvection = 3


class BoundaryConditionsStorage:
    def __init__(self, dofSize: int = 0):
        self.dofSize = int(dofSize)
        self.tags = np.zeros(self.dofSize, np.uint8)
        self.values = np.zeros(self.dofSize)
        self.dirichletValues = np.zeros(self.dofSize)

    def save(self, path) -> None:
        n = self.dofSize
        if not (self.tags.size == self.values.size == self.dirichletValues.size == n):
            raise ValueError("Invalid dofSize in BoundaryConditionsStorage")
        t = SERIALIZATION_TYPE.encode()
        with open(path, "wb") as fh:
            fh.write(MAGIC)
            fh.write(struct.pack("<i", len(t)) + t)
            fh.write(struct.pack("<q", n))
            for arr, dt in ((self.tags, "<u1"), (self.values, "<f8"), (self.dirichletValues, "<f8")):
                fh.write(struct.pack("<q", n))
                fh.write(np.ascontiguousarray(arr, dtype=dt).tobytes())

    @classmethod
    def load(cls, path) -> "BoundaryConditionsStorage":
        """This library's format, or the layout the reference's save() writes
        through TNL's File (detected by its first bytes)."""
        data = Path(path).read_bytes()
        if not data.startswith(MAGIC):
            return cls.load_tnl(path, data)
        pos = len(MAGIC)
        (ln,) = struct.unpack_from("<i", data, pos)
        pos += 4
        typ = data[pos:pos + ln].decode()
        pos += ln
        if typ != SERIALIZATION_TYPE:
            raise ValueError(f"object type does not match (expected {SERIALIZATION_TYPE}, found {typ}).")
        (n,) = struct.unpack_from("<q", data, pos)
        pos += 8
        obj = cls(n)
        for name, dt, size in (("tags", "<u1", 1), ("values", "<f8", 8), ("dirichletValues", "<f8", 8)):
            (m,) = struct.unpack_from("<q", data, pos)
            pos += 8
            if m != n:
                raise ValueError(f"Invalid dofSize in BoundaryConditionsStorage: dofSize = {n}, {name} has {m}")
            setattr(obj, name, np.frombuffer(data, dtype=dt, count=m, offset=pos).copy())
            pos += m * size
        if obj.tags.size and int(obj.tags.max()) > 3:
            raise ValueError("unknown boundary condition tag in file")
        return obj

    @classmethod
    def load_tnl(cls, path, data: bytes | None = None) -> "BoundaryConditionsStorage":
        """The object as BoundaryConditionsStorage::save writes it with TNL's
        File (BoundaryConditionsStorage.h:23-34): saveObjectType (a magic
        number, then the type string as an int32 length and its bytes),
        dofSize as int64, then tags, values and dirichletValues, each an
        Array saved the same way: its object type, its int64 size and the
        raw elements (std::uint8_t tags, BoundaryConditionsType.h:7-9; Real
        values, the Real named in the object type).  The magic number is taken
        from the file's first bytes and the array type strings are not
        compared text for text: TNL's source is not available to pin them.
        The checks are structural: sizes equal to dofSize, the stream fully
        consumed, known tags."""
        data = Path(path).read_bytes() if data is None else data
        pos = 0

        def object_type(where: str) -> str:
            nonlocal pos
            if data[pos:pos + len(magic)] != magic:
                raise ValueError(f"{path}: no object header at {where}")
            pos += len(magic)
            (ln,) = struct.unpack_from("<i", data, pos)
            pos += 4
            if not 0 < ln < 4096 or pos + ln > len(data):
                raise ValueError(f"{path}: bad object type length at {where}")
            typ = data[pos:pos + ln].decode("ascii", "replace")
            pos += ln
            return typ

        head = data.find(b"TNL::MHFEM::BoundaryConditionsStorage")
        if head < 9:
            raise ValueError(f"{path}: neither this library's nor TNL's boundary-conditions format")
        magic = data[:head - 4]
        typ = object_type("the start")
        real = typ[typ.index("<") + 1:typ.rindex(">")].strip() if "<" in typ else "double"
        rsize = {"double": 8, "float": 4}.get(real)
        if rsize is None:
            raise ValueError(f"{path}: unsupported Real type {real!r}")
        (n,) = struct.unpack_from("<q", data, pos)
        pos += 8
        obj = cls(n)
        for name, dt, size in (("tags", "<u1", 1), ("values", f"<f{rsize}", rsize),
                               ("dirichletValues", f"<f{rsize}", rsize)):
            object_type(name)
            (m,) = struct.unpack_from("<q", data, pos)
            pos += 8
            if m != n or pos + m * size > len(data):
                raise ValueError(f"Invalid dofSize in BoundaryConditionsStorage: dofSize = {n}, {name} has {m}")
            arr = np.frombuffer(data, dtype=dt, count=m, offset=pos)
            setattr(obj, name, arr.astype(np.uint8 if size == 1 else np.float64))
            pos += m * size
        if pos != len(data):
            raise ValueError(f"{path}: {len(data) - pos} trailing bytes")
        if obj.tags.size and int(obj.tags.max()) > 3:
            raise ValueError("unknown boundary condition tag in file")
        return obj
