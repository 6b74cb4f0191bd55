"""Reader for the VTK XML PolyData files of the output pipeline (appended raw
data, UInt64 block headers, little endian) — test infrastructure."""
import re
import struct

import numpy as np

_DA = re.compile(r'<DataArray type="(\w+)" Name="([^"]+)"(?: NumberOfComponents="(\d+)")?'
                 r'(?: NumberOfTuples="\d+")? format="appended" offset="(\d+)"/>')


def read_vtp(path):
    """Returns (arrays by name, piece attributes); arrays with several components as (n, c)."""
    data = open(path, "rb").read()
    i = data.index(b'<AppendedData encoding="raw">')
    j = data.index(b"_", i) + 1
    head = data[:i].decode()
    piece = {k: int(v) for k, v in re.findall(r'(Number\w+)="(\d+)"', head)}
    arrays = {}
    for typ, name, comps, off in _DA.findall(head):
        p = j + int(off)
        nbytes = struct.unpack_from("<Q", data, p)[0]
        a = np.frombuffer(data, dtype="<f8" if typ == "Float64" else "<i8", count=nbytes // 8, offset=p + 8)
        c = int(comps) if comps else 1
        arrays[name] = a.reshape(-1, c) if c > 1 else a
    assert data.rstrip().endswith(b"</VTKFile>")
    return arrays, piece


def read_pvd(path):
    """(timestep, part, file) of each DataSet of a .pvd collection."""
    txt = open(path).read()
    return [(float(t), int(p), f) for t, p, f in
            re.findall(r'<DataSet timestep="([^"]+)" part="(\d+)" file="([^"]+)"/>', txt)]
