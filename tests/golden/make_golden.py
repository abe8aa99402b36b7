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
* cases with a state-dependent Manning n (ManningN_option "variable"):
  ``res_kind`` / ``res_params`` (the function and its parameters, kinds as in
  oracle/hg_oracle.hpp), ``ks_cells`` (roughness height per cell,
  process_SRH_2D_input.jl:158-167), and the truth fields
  ``ManningN_cells_truth``, ``h_ks_cells_truth``, ``friction_factor_cells_truth``,
  ``Re_cells_truth`` computed at the truth state
  (process_forward_simulation_results_2D.jl:26-38)

Usage:  python tests/golden/make_golden.py [reference_root]
The reference root defaults to /root/reference.  Only this script reads it; the
tests read the generated ``.npz`` files.
"""
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(os.path.dirname(os.path.dirname(HERE)), "hydrograd.jl_gb300"))

from hydrograd_gb.srh2d import read_case  # noqa: E402  (the package's SRH-2D reader)


def build_case(case_dir, hydro_name=None):
    ctl = json.load(open(os.path.join(case_dir, "run_control.json")))
    hydro_name = hydro_name or ctl["control_variables"]["srhhydro_file_name"]
    # run-control files name some cases with a different letter case than the
    # file on disk (written on case-insensitive file systems): match without case
    hydro_name = next((f for f in os.listdir(case_dir) if f.lower() == hydro_name.lower()), hydro_name)
    stem = os.path.splitext(hydro_name)[0]
    geom_file = [f for f in os.listdir(case_dir) if f.endswith(".srhgeom") and f.startswith(stem)]
    geom_file = geom_file[0] if geom_file else [f for f in os.listdir(case_dir) if f.endswith(".srhgeom")][0]
    d = read_case(os.path.join(case_dir, geom_file), os.path.join(case_dir, hydro_name))
    d["tspan"] = np.array(ctl["time_settings"]["tspan"], dtype=float)
    return ctl, d


def initial_state(ctl, case_dir, opts_key, ic_key, file_key):
    opts = ctl[opts_key]
    if opts[ic_key] == "constant":
        wse, wstill, qx, qy = opts[ic_key.replace("_options", "_constant_values")]
        return dict(ic_const=np.array([wse, wstill, qx, qy], dtype=float))
    ic = json.load(open(os.path.join(case_dir, opts[file_key])))
    return dict(ic_wse=np.array(ic["wse"], float), ic_wstill=np.array(ic["wstill"], float),
                ic_qx=np.array(ic["q_x"], float), ic_qy=np.array(ic["q_y"], float))


RES_KINDS = {"power_law": 1, "sigmoid": 2, "inverse": 3, "h_Umag_ks": 4}


def forward_case(ref, rel, out_name):
    case_dir = os.path.join(ref, rel)
    ctl, d = build_case(case_dir)
    opts = ctl["forward_simulation_options"]
    d.update(initial_state(ctl, case_dir, "forward_simulation_options",
                           "forward_simulation_initial_condition_options",
                           "forward_simulation_initial_condition_file_name"))
    d["dt"] = np.array(float(ctl["time_settings"]["dt"]))
    truth = json.load(open(os.path.join(case_dir, "forward_simulation_solution_truth.json")))
    for k in ("xi_truth", "h_truth", "u_truth", "v_truth", "wstill_truth", "hstill_truth", "zb_cell_truth",
              "friction_x_truth", "friction_y_truth", "ManningN_cells_truth"):
        d[k] = np.array(truth[k], dtype=float)
    if opts.get("forward_simulation_ManningN_option") == "variable":
        fn = opts["forward_simulation_ManningN_function_type"]
        prm = opts["forward_simulation_ManningN_function_parameters"]
        d["res_kind"] = np.array(RES_KINDS[fn], dtype=np.int32)
        d["res_params"] = np.array([float(prm.get(k, 0.0)) for k in ("n_lower", "n_upper", "k", "h_mid")])
        if "ks" in prm:   # srhmat_ks_dict[iMat - 1] = ks[iMat]: zone id -> ks
            d["ks_cells"] = np.array(prm["ks"], dtype=float)[d["mat_id"]]
        for k in ("h_ks_cells_truth", "friction_factor_cells_truth", "Re_cells_truth"):
            if k in truth:
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
    global HERE
    ref = sys.argv[1] if len(sys.argv) > 1 else "/root/reference"
    if len(sys.argv) > 2:   # write the fixtures elsewhere (to compare with the committed ones)
        HERE = sys.argv[2]
    ex = "examples/SWE_2D"
    forward_case(ref, f"{ex}/forward_simulation/oneD_channel_with_bump", "fwd_bump.npz")
    forward_case(ref, f"{ex}/forward_simulation/oneD_channel_uniform_flow", "fwd_uniform.npz")
    forward_case(ref, f"{ex}/forward_simulation/Savannah_River", "fwd_savannah.npz")
    forward_case(ref, f"{ex}/forward_simulation/oneD_channel_with_bump_ManningN_h", "fwd_bump_nh.npz")
    forward_case(ref, f"{ex}/forward_simulation/Savannah_River_ManningN_ks_h_Umag", "fwd_savannah_nks.npz")
    sensitivity_case(ref, f"{ex}/sensitivity_analysis/ManningN/oneD_channel_with_bump", "sens_bump.npz")
    sensitivity_case(ref, f"{ex}/sensitivity_analysis/ManningN/oneD_channel_uniform_flow", "sens_uniform.npz")
    for f in sorted(os.listdir(HERE)):
        if f.endswith(".npz"):
            print(f, os.path.getsize(os.path.join(HERE, f)))


if __name__ == "__main__":
    main()
