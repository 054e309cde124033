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
arrays are indexed i*F + E.
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
        data = Path(path).read_bytes()
        if not data.startswith(MAGIC):
            raise ValueError(f"{path}: not a boundary-conditions file of this library")
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
