"""Reader for the VTK XML image files the host mirror's serializer writes (raw
appended Float64 cell arrays with UInt64 size headers) and for its .pvd lists."""
import re
import xml.etree.ElementTree as ET

import numpy as np


def read_vti(path):
    """Returns dict(extent=[6 ints], spacing=[3 floats], arrays={name: [nz, ny, nx]})."""
    data = open(path, "rb").read()
    start = data.index(b"<AppendedData")
    mark = data.index(b"_", data.index(b">", start)) + 1
    head = data[:start].decode() + "</VTKFile>"
    head = head.replace("<AppendedData", "")
    root = ET.fromstring(head)
    assert root.get("type") == "ImageData" and root.get("byte_order") == "LittleEndian"
    assert root.get("header_type") == "UInt64"
    img = root.find("ImageData")
    extent = [int(v) for v in img.get("WholeExtent").split()]
    spacing = [float(v) for v in img.get("Spacing").split()]
    n = [max(extent[2 * a + 1] - extent[2 * a], 1) for a in range(3)]
    arrays = {}
    for da in img.find("Piece").find("CellData").findall("DataArray"):
        assert da.get("type") == "Float64" and da.get("format") == "appended"
        off = mark + int(da.get("offset"))
        nbytes = int(np.frombuffer(data, dtype="<u8", count=1, offset=off)[0])
        assert nbytes == 8 * n[0] * n[1] * n[2]
        arrays[da.get("Name")] = np.frombuffer(data, dtype="<f8", count=nbytes // 8, offset=off + 8).reshape(
            n[2], n[1], n[0])
    return dict(extent=extent, spacing=spacing, arrays=arrays)


def read_pvd(path):
    """[(timestep, file)] of a ParaView collection."""
    text = open(path).read()
    return [(float(t), f) for t, f in re.findall(r'<DataSet timestep="([^"]*)" group="" part="0" file="([^"]*)"',
                                                  text)]
