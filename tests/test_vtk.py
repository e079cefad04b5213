"""Debug output in VTK's XML StructuredGrid format (IO.jl:213-233): the file parses as XML,
declares the reference's six point arrays and the whole ghost-filled extent, and its
appended blocks read back as the Float32 values written (bitwise)."""
import xml.etree.ElementTree as ET

import numpy as np

from flame3d_mhd_gb300 import cases
from flame3d_mhd_gb300.vtk import NAMES, read_vts, write_debug_vts


def test_debug_vts_round_trip(tmp_path):
    c = cases.sod(12, 6, 4)
    Q, x, y, z = c["Q"], c["x"], c["y"], c["z"]
    path = write_debug_vts(str(tmp_path / "debug-0"), Q, x, y, z)
    head = open(path, "rb").read().split(b"<AppendedData")[0].decode() + "</VTKFile>"
    root = ET.fromstring(head.split("?>", 1)[1])
    assert root.get("type") == "StructuredGrid" and root.get("header_type") == "UInt64"
    names = [d.get("Name") for d in root.iter("DataArray")]
    assert names == list(NAMES) + ["Points"]
    r = read_vts(path)
    nz, ny, nx = x.shape
    assert r["extent"] == (nx, ny, nz)
    pts = np.stack([a.astype(np.float32).ravel() for a in (x, y, z)], axis=1)
    assert np.array_equal(r["points"], pts)
    for n, name in enumerate(NAMES):
        assert np.array_equal(r[name], Q[n].astype(np.float32).ravel()), name
