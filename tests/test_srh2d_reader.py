"""The SRH-2D reader (hydrograd_gb.srh2d) on files written here.

The golden fixtures under tests/golden/ are produced by the same reader from
the reference's shipped example cases (make_golden.py); these tests cover the
file formats themselves: continuation lines, the default material zone,
NodeStrings without a BC, and the errors.
"""
import numpy as np
import pytest

from hydrograd_gb import HostMesh
from hydrograd_gb.srh2d import BC_CODES, read_case, read_srhgeom, write_case
from hydrograd_gb.workloads import river_triangles


def _case():
    c = river_triangles(n=8, L=100.0, inlet_q=7.5, pool_center=(20.0, 50.0), pool_radius=15.0)
    # add a third NodeString without a BC (a monitoring line, skipped as a boundary)
    sid = np.append(c["string_ids"], 9).astype(np.int32)
    snodes = np.append(c["string_nodes"], [3, 4, 5]).astype(np.int32)
    off = np.append(c["string_offsets"], c["string_offsets"][-1] + 3).astype(np.int32)
    return dict(node_xyz=c["node_xyz"], cell_nodes=c["cell_nodes"], cell_node_count=c["cell_node_count"],
                string_ids=sid, string_offsets=off, string_nodes=snodes,
                string_bc=np.append(c["string_bc"], -1).astype(np.int32), inlet_q=c["inlet_q"],
                exit_wse=c["exit_wse"], mat_id=c["mat_id"], manning_zones=c["manning_zones"])


def test_round_trip(tmp_path):
    c = _case()
    g, h = str(tmp_path / "reach.srhgeom"), str(tmp_path / "reach.srhhydro")
    write_case(c, g, h)
    r = read_case(g, h)
    for k in ("node_xyz", "cell_nodes", "cell_node_count", "string_ids", "string_offsets", "string_nodes",
              "string_bc", "inlet_q", "exit_wse", "mat_id", "manning_zones"):
        np.testing.assert_array_equal(r[k], c[k], err_msg=k)


def test_mesh_from_files_has_the_boundaries(tmp_path):
    c = _case()
    g, h = str(tmp_path / "reach.srhgeom"), str(tmp_path / "reach.srhhydro")
    write_case(c, g, h)
    m = HostMesh(read_case(g, h))
    assert m.n_cells == 2 * 8 * 8
    assert (m.n_inletq, m.n_exith) == (1, 1)
    assert m.n_wall == 1          # the default wall boundary: the faces in no BC NodeString


def test_cells_in_no_material_are_zone_zero(tmp_path):
    c = _case()
    c["mat_id"] = np.where(np.arange(len(c["mat_id"])) % 3 == 0, 1, 0).astype(np.int32)
    c["manning_zones"] = np.array([0.03, 0.05])
    g, h = str(tmp_path / "a.srhgeom"), str(tmp_path / "a.srhhydro")
    write_case(c, g, h)
    np.testing.assert_array_equal(read_case(g, h)["mat_id"], c["mat_id"])
    mat = tmp_path / "a.srhmat"
    mat.unlink()
    assert read_case(g, h)["mat_id"].max() == 0   # no material file: every cell in the default zone


def test_nodestring_continuation_lines(tmp_path):
    p = tmp_path / "s.srhgeom"
    p.write_text("SRHGEOM 30\nElem 1 1 2 3\nNode 1 0 0 0\nNode 2 1 0 0\nNode 3 0 1 0\n"
                 "NodeString 1 1 2\n3 1\n")
    _, _, _, strings = read_srhgeom(str(p))
    assert strings == {1: [1, 2, 3, 1]}


def test_errors(tmp_path):
    c = _case()
    g, h = str(tmp_path / "e.srhgeom"), str(tmp_path / "e.srhhydro")
    write_case(c, g, h)
    text = open(h).read().replace("EXIT-H", "EXIT-Q")
    open(h, "w").write(text)
    with pytest.raises(ValueError, match="boundary type"):
        read_case(g, h)
    bad = tmp_path / "bad.srhgeom"
    bad.write_text("Elem 1 1 2\nNode 1 0 0 0\nNode 2 1 0 0\n")
    with pytest.raises(ValueError, match="3 to 8"):
        read_srhgeom(str(bad))
    assert set(BC_CODES) == {"wall", "symm", "inlet-q", "exit-h"}
