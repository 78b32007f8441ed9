"""Read the VTR pieces this library writes, ASCII or appended binary.

The ASCII pieces are the reference's (CA/src/VtrManager.cpp:186-343); with
``output_format: appended`` in the deck's ``output`` block the same arrays
are written as raw little-endian binary after the XML header (VTK XML,
``header_type="UInt64"``: every array is preceded by its byte count).
``read_vtr`` returns every DataArray by name as a numpy array (cell arrays
in the reference's i-fastest order; a NumberOfComponents > 1 array has
shape (n, components)); coordinate arrays are keyed X_Coordinates,
Y_Coordinates and Z_Coordinates.
"""
from __future__ import annotations

import re

import numpy as np

_DTYPES = {"Int8": "i1", "UInt8": "u1", "Int32": "<i4", "Int64": "<i8", "Float32": "<f4", "Float64": "<f8"}
_TAG = re.compile(rb"<DataArray([^>]*?)(/?)>")
_ATTR = re.compile(rb'(\w+)="([^"]*)"')


def read_vtr(path: str) -> dict:
    data = open(path, "rb").read()
    mark = data.find(b"<AppendedData")
    head = data if mark < 0 else data[:mark]
    blob = None
    if mark >= 0:
        start = data.index(b"_", data.index(b">", mark)) + 1
        blob = memoryview(data)[start:]
    out = {}
    for m in _TAG.finditer(head):
        attrs = {k.decode().lower(): v.decode() for k, v in _ATTR.findall(m.group(1))}
        name = attrs.get("name", "")
        dtype = np.dtype(_DTYPES[attrs["type"]])
        comps = int(attrs.get("numberofcomponents", "1"))
        if attrs.get("format") == "appended":
            off = int(attrs["offset"])
            nbytes = int(np.frombuffer(blob[off:off + 8], "<u8")[0])
            arr = np.frombuffer(blob[off + 8:off + 8 + nbytes], dtype).copy()
        else:
            end = data.index(b"</DataArray>", m.end())
            text = data[m.end():end].split()
            arr = np.array([float(t) for t in text], np.float64).astype(dtype) if dtype.kind == "f" else \
                np.array([int(t) for t in text], dtype)
        out[name] = arr.reshape(-1, comps) if comps > 1 else arr
    return out
