"""Generate the golden fixtures used to pin the oracle and the CUDA path.

Reads the reference project's shipped example cases (SRH-2D geometry, hydro,
material files, run-control JSON, truth JSON and ManningN sensitivity JSON) and
writes one compressed ``.npz`` per case next to this script.  The fixtures hold
the input mesh, boundary conditions, parameters and initial state, plus the
reference's own outputs:

* ``S0_cells_truth``        bed slope from update_bed_data (process_bed_2D.jl:46-66)
* ``friction_x/y_truth``    Manning friction at the truth state
                            (semi_discretize_swe_2D.jl:544-547, written by
                            process_forward_simulation_results_2D.jl:45-47)
* ``xi_truth``, ``h_truth``, ``u_truth``, ``v_truth``  final state of a Tsit5
                            forward run (swe_2D_forward_simulation.jl:37-39)
* ``sensitivity``           ForwardDiff Jacobian of the final state w.r.t. the
                            zone Manning n (swe_2D_sensitivity.jl:80-94)

Usage:  python tests/golden/make_golden.py [reference_root]
The reference root defaults to /root/reference.  Only this script reads it; the
tests read the generated ``.npz`` files.
"""
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BC_CODES = {"wall": 0, "symm": 1, "inlet-q": 2, "exit-h": 3}


def read_srhgeom(path):
    """Elem / Node / NodeString records (SRH_2D_SRHGeom.jl:150-219)."""
    elems, nodes, strings = {}, {}, {}
    cur = None
    with open(path) as fh:
        for line in fh:
            parts = line.split()
            if not parts:
                continue
            if parts[0] == "Elem":
                elems[int(parts[1])] = [int(p) for p in parts[2:]]
                cur = None
            elif parts[0] == "Node":
                nodes[int(parts[1])] = [float(p) for p in parts[2:5]]
                cur = None
            elif parts[0] == "NodeString":
                cur = int(parts[1])
                strings[cur] = [int(p) for p in parts[2:]]
            elif parts[0].lower() in ("name", "gridunit") or "srhgeom" in parts[0].lower():
                continue
            elif cur is not None:
                strings[cur].extend(int(p) for p in parts)
    n_nodes = max(nodes)
    xyz = np.zeros((n_nodes, 3))
    for k, v in nodes.items():
        xyz[k - 1] = v
    n_cells = max(elems)
    cell_nodes = np.full((n_cells, 8), -1, dtype=np.int32)
    counts = np.zeros(n_cells, dtype=np.int32)
    for k, v in elems.items():
        cell_nodes[k - 1, : len(v)] = np.array(v) - 1
        counts[k - 1] = len(v)
    return xyz, cell_nodes, counts, strings


def read_srhhydro(path):
    """ManningsN / BC / IQParams / EWSParamsC records (SRH_2D_SRHHydro.jl:25-96)."""
    out = {"ManningsN": {}, "BC": {}, "IQParams": {}, "EWSParamsC": {}}
    with open(path) as fh:
        for line in fh:
            parts = line.split()
            if len(parts) <= 1:
                continue
            if parts[0] == "ManningsN":
                out["ManningsN"][int(parts[1])] = float(parts[2])
            elif parts[0] == "BC" and parts[2] != "MONITORING":
                out["BC"][int(parts[1])] = parts[2]
            elif parts[0] == "IQParams":
                out["IQParams"][int(parts[1])] = float(parts[2])
            elif parts[0] == "EWSParamsC":
                out["EWSParamsC"][int(parts[1])] = float(parts[2])
    return out


def read_srhmat(path, n_cells):
    """Material zones -> matID per cell, 0 = default zone (SRH_2D_SRHMat.jl:30-108;
    process_SRH_2D_input.jl:136-153)."""
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


def build_case(case_dir, hydro_name=None):
    ctl = json.load(open(os.path.join(case_dir, "run_control.json")))
    hydro_name = hydro_name or ctl["control_variables"]["srhhydro_file_name"]
    hydro = read_srhhydro(os.path.join(case_dir, hydro_name))
    stem = os.path.splitext(hydro_name)[0]
    geom_file = [f for f in os.listdir(case_dir) if f.endswith(".srhgeom") and f.startswith(stem)]
    geom_file = geom_file[0] if geom_file else [f for f in os.listdir(case_dir) if f.endswith(".srhgeom")][0]
    xyz, cell_nodes, counts, strings = read_srhgeom(os.path.join(case_dir, geom_file))
    mat_file = os.path.join(case_dir, os.path.splitext(geom_file)[0] + ".srhmat")
    mat = read_srhmat(mat_file, len(counts))
    ids = sorted(strings)
    # A NodeString is a boundary when the hydro file gives it a BC
    # (SRH_2D_SRHGeom.jl:306-310); otherwise it is skipped (-1).
    bc = [BC_CODES.get(hydro["BC"].get(i, "").lower(), -1) for i in ids]
    offsets = np.cumsum([0] + [len(strings[i]) for i in ids]).astype(np.int32)
    snodes = np.concatenate([np.array(strings[i], dtype=np.int32) - 1 for i in ids])
    inlet_ids = [i for i in ids if hydro["BC"].get(i, "").lower() == "inlet-q"]
    exit_ids = [i for i in ids if hydro["BC"].get(i, "").lower() == "exit-h"]
    d = dict(
        node_xyz=xyz,
        cell_nodes=cell_nodes,
        cell_node_count=counts,
        string_ids=np.array(ids, dtype=np.int32),
        string_offsets=offsets,
        string_nodes=snodes,
        string_bc=np.array(bc, dtype=np.int32),
        inlet_q=np.array([hydro["IQParams"][i] for i in inlet_ids]),
        exit_wse=np.array([hydro["EWSParamsC"][i] for i in exit_ids]),
        mat_id=mat,
        manning_zones=np.array([hydro["ManningsN"][k] for k in sorted(hydro["ManningsN"])]),
        tspan=np.array(ctl["time_settings"]["tspan"], dtype=float),
    )
    return ctl, d


def initial_state(ctl, case_dir, opts_key, ic_key, file_key):
    opts = ctl[opts_key]
    if opts[ic_key] == "constant":
        wse, wstill, qx, qy = opts[ic_key.replace("_options", "_constant_values")]
        return dict(ic_const=np.array([wse, wstill, qx, qy], dtype=float))
    ic = json.load(open(os.path.join(case_dir, opts[file_key])))
    return dict(ic_wse=np.array(ic["wse"], float), ic_wstill=np.array(ic["wstill"], float),
                ic_qx=np.array(ic["q_x"], float), ic_qy=np.array(ic["q_y"], float))


def forward_case(ref, rel, out_name):
    case_dir = os.path.join(ref, rel)
    ctl, d = build_case(case_dir)
    d.update(initial_state(ctl, case_dir, "forward_simulation_options",
                           "forward_simulation_initial_condition_options",
                           "forward_simulation_initial_condition_file_name"))
    truth = json.load(open(os.path.join(case_dir, "forward_simulation_solution_truth.json")))
    for k in ("xi_truth", "h_truth", "u_truth", "v_truth", "wstill_truth", "hstill_truth", "zb_cell_truth",
              "friction_x_truth", "friction_y_truth", "ManningN_cells_truth"):
        d[k] = np.array(truth[k], dtype=float)
    d["S0_cells_truth"] = np.array(truth["S0_cells_truth"], dtype=float)
    np.savez_compressed(os.path.join(HERE, out_name), source=np.array(rel), **d)


def sensitivity_case(ref, rel, out_name):
    case_dir = os.path.join(ref, rel)
    ctl, d = build_case(case_dir)
    opts = ctl["sensitivity_analysis_options"]
    d.update(initial_state(ctl, case_dir, "sensitivity_analysis_options",
                           "sensitivity_forward_simulation_initial_condition_options",
                           "sensitivity_forward_simulation_initial_condition_file_name"))
    d["manning_zones"] = np.array(opts["sensitivity_ManningN_values"], dtype=float)
    sens = json.load(open(os.path.join(case_dir, "sensitivity_results.json")))
    d["sensitivity"] = np.array(sens["sensitivity_results"], dtype=float)   # column-major (3N x nParams)
    d["sensitivity_params"] = np.array(sens["params_vector"], dtype=float)
    np.savez_compressed(os.path.join(HERE, out_name), source=np.array(rel), **d)


def main():
    ref = sys.argv[1] if len(sys.argv) > 1 else "/root/reference"
    ex = "examples/SWE_2D"
    forward_case(ref, f"{ex}/forward_simulation/oneD_channel_with_bump", "fwd_bump.npz")
    forward_case(ref, f"{ex}/forward_simulation/oneD_channel_uniform_flow", "fwd_uniform.npz")
    forward_case(ref, f"{ex}/forward_simulation/Savannah_River", "fwd_savannah.npz")
    sensitivity_case(ref, f"{ex}/sensitivity_analysis/ManningN/oneD_channel_with_bump", "sens_bump.npz")
    sensitivity_case(ref, f"{ex}/sensitivity_analysis/ManningN/oneD_channel_uniform_flow", "sens_uniform.npz")
    for f in sorted(os.listdir(HERE)):
        if f.endswith(".npz"):
            print(f, os.path.getsize(os.path.join(HERE, f)))


if __name__ == "__main__":
    main()
