"""SRH-2D case files -> a case for :class:`SWE2D`.

Reads the three text files a Hydrograd.jl SRH-2D case is made of:

* ``*.srhgeom``  Elem / Node / NodeString records (SRH_2D_SRHGeom.jl:150-219):
  cells as 1-based node lists, node coordinates (x, y, z = bed), and the
  NodeStrings (node chains along the boundary, continued on later lines);
* ``*.srhhydro`` ManningsN / BC / IQParams / EWSParamsC records
  (SRH_2D_SRHHydro.jl:25-96): the Manning n of each material zone, the
  boundary type of each NodeString, inlet discharges and exit water surfaces;
* ``*.srhmat``   Material records (SRH_2D_SRHMat.jl:30-108): the cells of each
  zone; cells listed in no zone belong to zone 0, the default
  (process_SRH_2D_input.jl:136-153).

The result is the dict the mesh builder and the parameter setters take
(node_xyz, cell_nodes, cell_node_count, string_*, mat_id, manning_zones,
inlet_q, exit_wse), with 0-based ids.  A NodeString is a boundary only if the
hydro file gives it a BC; others are skipped (SRH_2D_SRHGeom.jl:306-310).
Initial conditions and run control are the caller's (the reference keeps them
in its run-control JSON).
"""
import os

import numpy as np

BC_CODES = {"wall": 0, "symm": 1, "inlet-q": 2, "exit-h": 3}


def read_srhgeom(path):
    """(node_xyz [n,3], cell_nodes [n,8] 0-based -1-padded, cell_node_count, {string id: 1-based nodes})."""
    elems, nodes, strings = {}, {}, {}
    cur = None
    with open(path) as fh:
        for line in fh:
            parts = line.split()
            if not parts:
                continue
            key = parts[0]
            if key == "Elem":
                elems[int(parts[1])] = [int(p) for p in parts[2:]]
                cur = None
            elif key == "Node":
                nodes[int(parts[1])] = [float(p) for p in parts[2:5]]
                cur = None
            elif key == "NodeString":
                cur = int(parts[1])
                strings[cur] = [int(p) for p in parts[2:]]
            elif key.lower() in ("name", "gridunit") or "srhgeom" in key.lower():
                continue
            elif cur is not None:   # continuation line of the current NodeString
                strings[cur].extend(int(p) for p in parts)
    if not elems or not nodes:
        raise ValueError(f"{path}: no Elem or Node records")
    xyz = np.zeros((max(nodes), 3))
    for k, v in nodes.items():
        xyz[k - 1] = v
    n_cells = max(elems)
    cell_nodes = np.full((n_cells, 8), -1, dtype=np.int32)
    counts = np.zeros(n_cells, dtype=np.int32)
    for k, v in elems.items():
        if not 3 <= len(v) <= 8:
            raise ValueError(f"{path}: Elem {k} has {len(v)} nodes (3 to 8 supported)")
        cell_nodes[k - 1, :len(v)] = np.array(v) - 1
        counts[k - 1] = len(v)
    return xyz, cell_nodes, counts, strings


def read_srhhydro(path):
    """{"ManningsN": {zone: n}, "BC": {string: type}, "IQParams": {string: Q}, "EWSParamsC": {string: WSE}}."""
    out = {"ManningsN": {}, "BC": {}, "IQParams": {}, "EWSParamsC": {}}
    with open(path) as fh:
        for line in fh:
            parts = line.split()
            if len(parts) <= 2:
                continue
            key = parts[0]
            if key == "ManningsN":
                out["ManningsN"][int(parts[1])] = float(parts[2])
            elif key == "BC" and parts[2].upper() != "MONITORING":
                out["BC"][int(parts[1])] = parts[2]
            elif key == "IQParams":
                out["IQParams"][int(parts[1])] = float(parts[2])
            elif key == "EWSParamsC":
                out["EWSParamsC"][int(parts[1])] = float(parts[2])
    return out


def read_srhmat(path, n_cells):
    """Zone of every cell (0 = the default zone)."""
    zones, cur = {}, 0
    with open(path) as fh:
        for line in fh:
            parts = line.split()
            if not parts or parts[0] in ("SRHMAT", "NMaterials", "MatName"):
                continue
            if parts[0] == "Material":
                cur = int(parts[1])
                zones.setdefault(cur, []).extend(int(p) for p in parts[2:])
            elif cur:
                zones[cur].extend(int(p) for p in parts)
    mat = np.zeros(n_cells, dtype=np.int32)
    for k, cells in zones.items():
        for c in cells:
            mat[c - 1] = k
    return mat


def read_case(geom_path, hydro_path, mat_path=None):
    """Mesh, boundaries and parameters of an SRH-2D case.  ``mat_path``
    defaults to the geometry file's name with ``.srhmat``; without a material
    file every cell is in zone 0."""
    xyz, cell_nodes, counts, strings = read_srhgeom(geom_path)
    hydro = read_srhhydro(hydro_path)
    if mat_path is None:
        mat_path = os.path.splitext(geom_path)[0] + ".srhmat"
    mat = read_srhmat(mat_path, len(counts)) if os.path.exists(mat_path) else np.zeros(len(counts), np.int32)
    ids = sorted(strings)
    bc = []
    for i in ids:
        t = hydro["BC"].get(i, "").lower()
        if t and t not in BC_CODES:
            raise ValueError(f"NodeString {i}: boundary type {t!r} is not one of {sorted(BC_CODES)}")
        bc.append(BC_CODES.get(t, -1))
    offsets = np.cumsum([0] + [len(strings[i]) for i in ids]).astype(np.int32)
    snodes = (np.concatenate([np.array(strings[i], dtype=np.int32) - 1 for i in ids]) if ids
              else np.zeros(0, np.int32))
    inlet_ids = [i for i, b in zip(ids, bc) if b == BC_CODES["inlet-q"]]
    exit_ids = [i for i, b in zip(ids, bc) if b == BC_CODES["exit-h"]]
    zones = sorted(hydro["ManningsN"])
    if zones != list(range(len(zones))):
        raise ValueError(f"ManningsN zones {zones} are not 0, 1, ..., n-1")
    if len(zones) and mat.max() >= len(zones):
        raise ValueError(f"cells in material {int(mat.max())} but ManningsN has {len(zones)} zones")
    return dict(node_xyz=xyz, cell_nodes=cell_nodes, cell_node_count=counts,
                string_ids=np.array(ids, dtype=np.int32), string_offsets=offsets, string_nodes=snodes,
                string_bc=np.array(bc, dtype=np.int32),
                inlet_q=np.array([hydro["IQParams"][i] for i in inlet_ids], dtype=float),
                exit_wse=np.array([hydro["EWSParamsC"][i] for i in exit_ids], dtype=float),
                mat_id=mat, manning_zones=np.array([hydro["ManningsN"][k] for k in zones], dtype=float))


def write_case(case, geom_path, hydro_path, mat_path=None):
    """Write a case (as read_case returns) as SRH-2D files, all ids 1-based."""
    xyz, cn, cnt = case["node_xyz"], case["cell_nodes"], case["cell_node_count"]
    names = {v: k.upper() if k != "inlet-q" else "INLET-Q" for k, v in BC_CODES.items()}
    names[BC_CODES["exit-h"]] = "EXIT-H"
    with open(geom_path, "w") as fh:
        fh.write("SRHGEOM 30\nName \"case\"\nGridUnit \"meters\"\n")
        for c in range(len(cnt)):
            fh.write("Elem %d %s\n" % (c + 1, " ".join(str(v + 1) for v in cn[c, :cnt[c]])))
        for i, p in enumerate(xyz):
            fh.write("Node %d %.17g %.17g %.17g\n" % (i + 1, p[0], p[1], p[2]))
        off = case["string_offsets"]
        for s, sid in enumerate(case["string_ids"]):
            nodes = [str(v + 1) for v in case["string_nodes"][off[s]:off[s + 1]]]
            fh.write("NodeString %d %s\n" % (sid, " ".join(nodes[:10])))
            for k in range(10, len(nodes), 10):   # continuation lines
                fh.write(" ".join(nodes[k:k + 10]) + "\n")
    inlet = iter(case["inlet_q"])
    exit_ = iter(case["exit_wse"])
    with open(hydro_path, "w") as fh:
        fh.write("SRHHYDRO 30\n")
        for z, n in enumerate(case["manning_zones"]):
            fh.write("ManningsN %d %.17g\n" % (z, n))
        for sid, b in zip(case["string_ids"], case["string_bc"]):
            if b < 0:
                continue
            fh.write("BC %d %s\n" % (sid, names[int(b)]))
            if b == BC_CODES["inlet-q"]:
                fh.write("IQParams %d %.17g SI CONVEYANCE\n" % (sid, next(inlet)))
            elif b == BC_CODES["exit-h"]:
                fh.write("EWSParamsC %d %.17g SI C\n" % (sid, next(exit_)))
    mat_path = mat_path or os.path.splitext(geom_path)[0] + ".srhmat"
    nz = len(case["manning_zones"])
    with open(mat_path, "w") as fh:
        fh.write("SRHMAT 30\nNMaterials %d\n" % nz)
        for z in range(1, nz):
            cells = [str(c + 1) for c in np.nonzero(case["mat_id"] == z)[0]]
            fh.write("MatName %d zone%d\n" % (z, z))
            fh.write("Material %d %s\n" % (z, " ".join(cells[:10])))
            for k in range(10, len(cells), 10):
                fh.write(" ".join(cells[k:k + 10]) + "\n")
