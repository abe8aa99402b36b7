/*
 * hydrograd_gb.h -- C ABI of the GB300 (sm_103a) shallow-water RHS / time-stepping library.
 *
 * The library replaces the hot path of Hydrograd.jl: the ODE right-hand side
 * swe_2d_rhs (src/fvm/discretization/semi_discretize_swe_2D.jl:18-277), its
 * time integration (src/ode_solvers/custom_ODE_solvers.jl:5-95 and the SciML
 * ODEProblem call sites, src/applications/forward_simulation/
 * swe_2D_forward_simulation.jl:24-53), and the reverse-mode gradient that
 * SciMLSensitivity/Zygote compute through it (src/applications/inversion/
 * swe_2D_inversion.jl:247-483).  Julia binds these entry points with ccall;
 * nothing here takes or returns a Julia, PyTorch or CUDA type.
 *
 * Conventions
 *  - Every entry point returns an int status: HG_OK (0) or an HG_ERR_* code;
 *    hg_last_error() gives a message.  No C++ exception crosses this ABI.
 *  - All ids are 0-based.  Node ids index node_x/y/z; cell ids index the cell
 *    arrays in the caller's order (the library renumbers internally and maps
 *    back at this boundary).
 *  - The state is the reference's Q = [xi; q_x; q_y] (3 blocks of n_cells
 *    doubles), xi = wse - wstill (semi_discretize_swe_2D.jl:93-95,
 *    process_ICs_2D.jl:53-57).
 *  - Host buffers are owned by the caller and only read/written during the
 *    call.  Device memory is owned by the context and never exposed.
 *  - One context per host thread; each context runs on its own CUDA stream.
 *  - There is no CPU fallback: hg_create fails with HG_ERR_NO_DEVICE when no
 *    CUDA device is present.
 */
#ifndef HYDROGRAD_GB_H
#define HYDROGRAD_GB_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define HG_ABI_VERSION 1

enum hg_status {
  HG_OK = 0,
  HG_ERR_ARG = 1,        /* bad argument (size, null pointer, id out of range) */
  HG_ERR_MESH = 2,       /* mesh topology/geometry error (clockwise cell, open NodeString, ...) */
  HG_ERR_CUDA = 3,       /* a CUDA call failed */
  HG_ERR_NO_DEVICE = 4,  /* no CUDA device: there is no CPU fallback */
  HG_ERR_STATE = 5,      /* invalid state (initial depth below h_small, NaN/Inf in the result) */
  HG_ERR_INLET = 6,      /* inlet-Q conveyance not positive (bc_2D.jl:679) */
  HG_ERR_UNSUPPORTED = 7 /* option not available in this build */
};

/* Boundary types of a NodeString (src/fvm/boundary_conditions/bc_2D.jl:154-260). */
enum hg_bc { HG_BC_NONE = -1, HG_BC_WALL = 0, HG_BC_SYMM = 1, HG_BC_INLETQ = 2, HG_BC_EXITH = 3 };

/* Arithmetic of the device path. */
enum hg_precision {
  HG_FP64 = 0,  /* plain FP64 everywhere (parity path, within 1e-12 of the FP64 oracle) */
  HG_FP32C = 1  /* FP32 flux/source arithmetic, compensated (hi+lo FP32) state update,
                   FP64-exact wet/dry and positivity decisions, FP64 accumulators */
};

/* Cell renumbering used on the device. */
enum hg_order { HG_ORDER_NONE = 0, HG_ORDER_RCM = 1, HG_ORDER_HILBERT = 2 };

/* Riemann solver (swe_2D_constants.jl:16 RiemannSolver; semi_discretize_swe_2D.jl:352-362):
 * Roe (swe_2D_solvers.jl:4-164), the reference's only working one; HLL -- new:
 * the reference's "HLL" raises an error -- Harten-Lax-van Leer with Einfeldt's
 * wave speeds on the Roe solver's variables and dry/wet/wall branches; HLLC is
 * refused with HG_ERR_UNSUPPORTED, as the reference raises an error for it. */
enum hg_riemann { HG_ROE = 0, HG_HLL = 1, HG_HLLC = 2 };

/*
 * Mesh as an SRH-2D geometry holds it (src/utilities/SRH_2D/SRH_2D_SRHGeom.jl:14-46):
 * nodes, cells as counter-clockwise node lists (<= 8 nodes, rows of 8, unused
 * slots ignored), and NodeStrings.  A NodeString with string_bc = HG_BC_NONE is
 * not a boundary (monitoring line).  Boundary edges on no NodeString form a
 * default wall boundary (SRH_2D_SRHGeom.jl:344-349).  Bed elevation at cells is
 * the mean of node_z (src/fvm/discretization/fvm_schemes_2D.jl:216-224).
 */
typedef struct hg_mesh_desc {
  int32_t n_nodes;
  const double* node_x;
  const double* node_y;
  const double* node_z;
  int32_t n_cells;
  const int32_t* cell_node_count; /* [n_cells] */
  const int32_t* cell_nodes;      /* [n_cells * 8] */
  int32_t n_strings;
  const int32_t* string_ids;      /* [n_strings] NodeString ids (boundary ids) */
  const int32_t* string_offsets;  /* [n_strings + 1] into string_nodes */
  const int32_t* string_nodes;    /* node ids along each NodeString */
  const int32_t* string_bc;       /* [n_strings] hg_bc */
} hg_mesh_desc;

/* Problem constants (src/constants/swe_2D_constants.jl:4-17; solve_swe_2D.jl:51-107). */
typedef struct hg_consts {
  double g;        /* 9.81 (SI) or 32.2 (EN) */
  double k_n;      /* 1.0 (SI) or 1.486 (EN) */
  double h_small;  /* dry threshold, 1e-3 */
  int32_t riemann; /* hg_riemann */
  int32_t order;   /* hg_order (device renumbering) */
} hg_consts;

typedef struct hg_ctx hg_ctx;
typedef struct hg_mesh hg_mesh;

/* ---- diagnostics -------------------------------------------------------- */
/* Message of the last failing call on ctx (ctx may be NULL for hg_create / hg_mesh_build failures). */
int hg_last_error(const hg_ctx* ctx, char* buf, int32_t len);
int hg_abi_version(void);

/* ---- host-only mesh topology (no device needed) -------------------------- */
/* Topology + geometry exactly as initialize_mesh_2D builds it (src/meshes/mesh_2D.jl:75-453). */
int hg_mesh_build(const hg_mesh_desc* desc, hg_mesh** out);
int hg_mesh_free(hg_mesh* mesh);
/* sizes: [n_cells, n_faces, n_ghosts, n_inletq, n_exith, n_wall, n_symm, max_cell_faces] */
int hg_mesh_sizes(const hg_mesh* mesh, int32_t* sizes8);
/* Per cell, per local face slot i (edge node i -> node i+1), in the caller's cell order:
 * neighbour cell id or -1 on a boundary, outward normal, edge length; plus cell areas
 * and centroids (mesh_2D.jl:456-652).  Any output may be NULL. */
int hg_mesh_cell_faces(const hg_mesh* mesh, int32_t* nbr8, double* normals16, double* lengths8, double* areas,
                       double* centroids2);
/* Cell permutation used on the device: perm[new] = old. */
int hg_mesh_order(const hg_mesh* mesh, int32_t order, int32_t* perm);

/* ---- context lifecycle (replaces building SWE2D_Extra_Parameters, application_commons.jl:7-44) */
int hg_create(const hg_mesh_desc* desc, const hg_consts* consts, int32_t precision, int32_t device, hg_ctx** out);
/* Ensembles: many independent problems ("members"), each on one of a set of
 * meshes, stepped together in one context -- one launch per stage over every
 * member's cells.  No counterpart in the reference, which solves one problem
 * per call.  The members' cells are concatenated in member order: member m
 * holds cells [cell_offset[m], cell_offset[m+1]) of every per-cell array and
 * of each of Q's three blocks, and its inlet-Q / exit-H boundaries are
 * [inlet_offset[m], inlet_offset[m+1]) / [exit_offset[m], ...) of the values
 * of hg_set_inlet_q / hg_set_exit_wse and of the inlet-Q gradient.  Every
 * other call (hg_set_*, hg_rhs, hg_integrate, hg_advance, hg_loss_and_grad)
 * applies unchanged to the concatenation.  In CFL stepping each member takes
 * its own step, formed from its own cells (each member is its own problem, as
 * the reference solves one ODEProblem per run,
 * swe_2D_forward_simulation.jl:24-39), and keeps its own time, so a member's
 * trajectory is the one it has alone; a fixed dt applies to every member.
 * hg_integrate's dts_out and hg_elapsed_time report member 0's steps and
 * time; hg_ensemble_steps gives every member's.  The adjoint
 * (hg_loss_and_grad) takes one fixed dt; its loss is the mean over all
 * members' probes. */
typedef struct hg_ensemble_desc {
  int32_t n_meshes;
  const hg_mesh_desc* meshes;   /* [n_meshes] */
  int32_t n_members;
  const int32_t* member_mesh;   /* [n_members] index into meshes */
} hg_ensemble_desc;
int hg_ensemble_create(const hg_ensemble_desc* ensemble, const hg_consts* consts, int32_t precision,
                       int32_t device, hg_ctx** out);
/* n_members; then, where not NULL, the [n_members + 1] offsets (a context made
 * by hg_create is one member). */
int hg_ensemble_layout(const hg_ctx* ctx, int32_t* n_members, int32_t* cell_offset, int32_t* inlet_offset,
                       int32_t* exit_offset);
/* The steps each member took in the steps since the last state upload
 * (dts [nsteps][n_members], may be NULL) and each member's elapsed time
 * (t_elapsed [n_members], may be NULL), of an ensemble context. */
int hg_ensemble_steps(hg_ctx* ctx, int32_t nsteps, double* dts, double* t_elapsed);

/* ---- Tsit5 (the reference's default solver, swe_2D_forward_simulation.jl:37-39)
 * Adaptive Tsitouras 5(4) steps of the RHS from t0 to t1 on the device, Q in/out
 * (caller order).  Error control: weighted RMS norm of the embedded error
 * with scale abstol + reltol max(|Q_old|, |Q_new|), PI step-size controller,
 * step factor in [0.2, 10] with safety 0.9; dt0 <= 0 picks the starting step
 * (Hairer-Norsett-Wanner II.4).  adaptive == 0 takes fixed steps of dt0 > 0
 * with no error control (solve(...; adaptive=false, dt=dt0)).  The n_save
 * ascending times t_save in (t0, t1] are stepped onto and their states
 * written to saves[n_save][3N].  max_steps <= 0: no limit.  stats (may be
 * NULL): accepted steps, rejected steps, RHS evaluations.  No clamp besides
 * the RHS's own, as in the reference's ODE solve. */
int hg_integrate_tsit5(hg_ctx* ctx, double* Q, double t0, double t1, double abstol, double reltol, double dt0,
                       int32_t adaptive, int32_t max_steps, int32_t n_save, const double* t_save, double* saves,
                       int32_t* stats);
/* The step sizes the last hg_integrate_tsit5 call accepted, in order (the
 * adaptive solve's steps, which hg_set_adjoint_steps hands to the gradient
 * calls): the first min(cap, count) into dts, their number into *count (may
 * be NULL).  Returns HG_ERR_ARG (no message) for a null context or dts. */
int hg_tsit5_steps(const hg_ctx* ctx, double* dts, int32_t cap, int32_t* count);
/* The Butcher tableau in use: c[7], a[7][7] (row-major, lower triangle), b[7], btilde[7] = b - bhat. */
int hg_tsit5_tableau(double* c7, double* a49, double* b7, double* btilde7);

int hg_destroy(hg_ctx* ctx);
int hg_sizes(const hg_ctx* ctx, int32_t* sizes8); /* as hg_mesh_sizes */

/* ---- parameters (semi_discretize_swe_2D.jl:112-199; process_ManningN_2D.jl:242-269) */
/* hstill = wstill - zb_cells; hstill is fixed from here on, as in the reference
 * (it is not recomputed when zb changes, process_ICs_2D.jl:55,84). */
int hg_set_still_water(hg_ctx* ctx, const double* wstill_cells);
/* ManningN_cells[i] = n_zone[mat_id[i]] (mat_id 0 = default zone). */
int hg_set_manning_zones(hg_ctx* ctx, const int32_t* mat_id, int32_t n_zones, const double* n_zone);
int hg_set_manning_cells(hg_ctx* ctx, const double* n_cells);
/* Active zb parameter: replaces zb_cells and recomputes zb ghost/face values and
 * the bed slope S0 on the device (process_bed_2D.jl:46-66). */
int hg_set_zb_cells(hg_ctx* ctx, const double* zb_cells);
int hg_set_inlet_q(hg_ctx* ctx, const double* q, int32_t n_inletq);   /* inletQ_TotalQ */
int hg_set_exit_wse(hg_ctx* ctx, const double* wse, int32_t n_exith); /* exitH_WSE */
/* Inlet-Q hydrograph (no counterpart in the reference, whose inlet discharges
 * are constant, bc_2D.jl:192): the discharge of inlet-Q boundary `group`
 * follows the n points (t[i], q[i]), t increasing, linearly interpolated and
 * held at the end values outside them, evaluated at the time of each RHS
 * evaluation: t of hg_rhs; t_n and t_n + dt for the stages of an SSP-RK2 step
 * (t = the simulated time since the last hg_state_upload or hg_integrate);
 * the stage times of hg_integrate_tsit5; s dt and (s + 1) dt for step s of
 * hg_loss_and_grad / hg_final_loss_and_grad, whose inlet-Q gradient is then
 * the derivative w.r.t. a constant shift of the hydrograph.  n = 0 returns the
 * group to its hg_set_inlet_q value. */
int hg_set_inlet_hydrograph(hg_ctx* ctx, int32_t group, int32_t n, const double* t, const double* q);
/* Read back derived data: zb_cells [n], S0 [2n] (x,y interleaved), ManningN_cells [n], hstill [n]. */
int hg_get_bed(hg_ctx* ctx, double* zb_cells, double* S0, double* manning_cells, double* hstill);

/* ---- state-dependent flow resistance
 * Manning's n as a function of the state, ManningN_option "variable"
 * (process_ManningN_2D.jl:102-213, applied at semi_discretize_swe_2D.jl:141-149):
 * every RHS evaluation recomputes n from its own clamped state, with
 * Umag = |q| / h, and uses it for the friction and the inlet-Q conveyance.
 *   HG_RES_POWER_LAW  n = n_lower + (n_upper - n_lower) (h + eps)^(-k)
 *   HG_RES_SIGMOID    n = n_lower + (n_upper - n_lower) / (1 + exp(k (h - h_mid)))
 *   HG_RES_INVERSE    n = n_lower + (n_upper - n_lower) / (1 + k h)
 *   HG_RES_H_UMAG_KS  n from Cheng's (2008) friction factor of Re = Umag h / 1e-6 and h / ks
 * params = {n_lower, n_upper, k[, h_mid]}; ks_cells [n] (caller order) for
 * HG_RES_H_UMAG_KS.  HG_RES_CONSTANT returns to the cells' n
 * (hg_set_manning_zones / _cells).  Gradients (hg_loss_and_grad,
 * hg_final_loss_and_grad, hg_final_vjp) run through these functions: each
 * RHS evaluation's dL/dn is taken back into its state through
 * dn/d(h, qx, qy), so the zb and inlet-Q gradients include it, and into the
 * function's parameters (hg_resistance_grad); the per-cell n gradient is then
 * zero, n not being a parameter.  With a UDE closure (kinds 5-7) they run
 * through the network (hg_ude_grad). */
enum hg_resistance {
  HG_RES_CONSTANT = 0, HG_RES_POWER_LAW = 1, HG_RES_SIGMOID = 2, HG_RES_INVERSE = 3, HG_RES_H_UMAG_KS = 4,
  HG_RES_UDE_MANNING_H = 5,          /* UDE_choice "ManningN_h": n = NN(h) */
  HG_RES_UDE_MANNING_H_UMAG_KS = 6,  /* "ManningN_h_Umag_ks": n = NN(h, Umag, ks) */
  HG_RES_UDE_FLOW_RESISTANCE = 7     /* "FlowResistance": friction = NN(h, |q|) q / |q| */
};
int hg_set_manning_function(hg_ctx* ctx, int32_t kind, const double* params, int32_t n_params,
                            const double* ks_cells);
/* The gradient of the last hg_loss_and_grad / hg_final_loss_and_grad /
 * hg_final_vjp call w.r.t. the parameters {n_lower, n_upper, k, h_mid} of the
 * state-dependent n function (zeros when none was set; h_mid only for the
 * sigmoid; HG_RES_H_UMAG_KS has none). */
int hg_resistance_grad(const hg_ctx* ctx, double* g_params4);
/* UDE closures (process_ManningN_2D.jl:216-273, process_FlowResistance_UDE.jl:3-45)
 * with the network of process_UDE.jl:3-56: per hidden layer Dense(in, w, act)
 * then LayerNorm(w); a linear Dense(w, 1); output lo + (hi - lo) sigmoid(y).
 * Inputs normalised to [-1, 1] by their bounds: h (h_bounds); Umag (u_bounds)
 * and ks (ks_bounds) for ManningN_h_Umag_ks; |q| for FlowResistance with the
 * bounds h_bounds x u_bounds (u_bounds = velocity_magnitude_bounds).
 * params: Lux's flattened order -- per hidden layer the Dense weight (w x in,
 * column-major) and bias, the LayerNorm scale and bias; then the output
 * weight (1 x w) and bias.  LayerNorm: (x - mean) / sqrt(var + 1f-5) * scale +
 * bias, uncorrected variance; layernorm_over_batch = 1 takes mean and variance
 * over the whole (width x cells) array, as Lux's LayerNorm with its default
 * dims = Colon() does; 0 takes them over each cell's features.
 * Gradients (hg_loss_and_grad, hg_final_loss_and_grad, hg_final_vjp) run
 * through the network, as the reference trains it by differentiating the
 * solve (swe_2D_UDE.jl:119,522): each RHS evaluation's dL/dn (dL/dF for
 * FlowResistance) is taken back by reverse mode into the cells' states and
 * into the parameters (hg_ude_grad), through the batch LayerNorm's statistics
 * too; for FlowResistance the inlet conveyance's dL/dn stays a per-cell n
 * gradient. */
enum hg_activation { HG_ACT_RELU = 0, HG_ACT_LEAKYRELU = 1, HG_ACT_SIGMOID = 2, HG_ACT_TANH = 3, HG_ACT_SOFTPLUS = 4 };
typedef struct hg_ude_desc {
  int32_t kind;                  /* HG_RES_UDE_* */
  int32_t n_hidden;              /* 0..4 */
  const int32_t* hidden;         /* [n_hidden] widths, 1..16 */
  const int32_t* activation;     /* [n_hidden] hg_activation */
  const double* params;
  int32_t n_params;
  double output_bounds[2];
  double h_bounds[2];
  double u_bounds[2];
  double ks_bounds[2];
  const double* ks_cells;        /* [n] (HG_RES_UDE_MANNING_H_UMAG_KS) */
  int32_t layernorm_over_batch;
} hg_ude_desc;
int hg_set_ude(hg_ctx* ctx, const hg_ude_desc* ude);
/* dL/dparams of the UDE network from the last hg_loss_and_grad /
 * hg_final_loss_and_grad / hg_final_vjp call, in hg_set_ude's parameter order;
 * n_params must be the closure's count (HG_ERR_ARG otherwise; 0 without a
 * closure). */
int hg_ude_grad(const hg_ctx* ctx, double* g_params, int64_t n_params);

/* Change the Riemann solver (hg_riemann) of a context after hg_create: it
 * applies to every integrator, the RHS and the adjoint. */
int hg_set_riemann_solver(hg_ctx* ctx, int32_t solver);

/* Smallest CFL time step accepted (swe_2D_consts.dt_min, swe_2D_constants.jl:9;
 * the reference sets 0.001 s, solve_swe_2D.jl:83,98, and never reads it).
 * A CFL step below it -- a collapsing state, e.g. a dry front the scheme
 * cannot hold -- makes the stepping call return HG_ERR_STATE (the steps are
 * still taken; the device sets a flag the host reads after them).  Default
 * 0.001 s; 0 turns the check off.  Fixed-dt and Tsit5 steps are not checked. */
int hg_set_dt_min(hg_ctx* ctx, double dt_min);

/* ---- forward ------------------------------------------------------------- */
/* dQdt = swe_2d_rhs(Q, p, t) with host buffers (semi_discretize_swe_2D.jl:18-277). */
int hg_rhs(hg_ctx* ctx, const double* Q, double t, double* dQdt);
/* Check an initial state the way setup_initial_condition does (process_ICs_2D.jl:89-99). */
int hg_check_initial_state(hg_ctx* ctx, const double* Q);
/*
 * Integrate nsteps explicit steps from Q (host, in/out).
 *   method: 0 = SSP-RK2 (Heun) with a depth-positivity clamp after each stage,
 *           1 = forward Euler with the reference's clamp (custom_ODE_solvers.jl:5-33).
 *   dt > 0: fixed step; dt <= 0: CFL step dt = cfl * min_c A_c / sum_f L_f(|u.n_f| + sqrt(g h))
 *           recomputed on the device before every step.
 *   save_every > 0: the state after every save_every-th step is written to saves
 *           (host, [nsteps/save_every][3n]); may be NULL otherwise.
 *   dts_out: the step sizes used ([nsteps], host), may be NULL.
 */
int hg_integrate(hg_ctx* ctx, double* Q, double t0, int32_t nsteps, int32_t method, double dt, double cfl,
                 int32_t save_every, double* saves, double* dts_out);

/* ---- device-resident stepping (the state stays in HBM between calls) ------ */
int hg_state_upload(hg_ctx* ctx, const double* Q);
int hg_state_download(hg_ctx* ctx, double* Q);
/* Enqueue nsteps SSP-RK2 steps on the resident state (no host synchronisation;
 * replays a captured CUDA graph when graph != 0). */
int hg_advance(hg_ctx* ctx, int32_t nsteps, double dt, double cfl, int32_t graph);
int hg_synchronize(hg_ctx* ctx);
/* Sum of the device time steps taken since the last upload. */
int hg_elapsed_time(hg_ctx* ctx, double* t);

/* ---- gradient (replaces Zygote/SciMLSensitivity through the RHS) ----------- */
/*
 * Loss = mean over steps k = 1..nsteps and probes p of (h_p^k - obs[k][p])^2,
 * h = xi + hstill, for nsteps fixed-dt SSP-RK2 steps from Q0.  Gradients by a
 * discrete adjoint with checkpoints every ckpt_every steps (at least; see
 * hg_set_adjoint_tape) and recomputation.  g_manning_cells [n] (dL/dn per
 * cell; zone gradients are sums over a zone's cells), g_zb [n] (dL/dzb_cells
 * through S0, ghost and exit-H values), g_inletq [n_inletq].  Any gradient
 * output may be NULL: the FP32-compensated sweep then skips that gradient's
 * accumulation (the others are unchanged, bit for bit).  Q_final (host, 3n)
 * may be NULL.
 */
int hg_loss_and_grad(hg_ctx* ctx, const double* Q0, int32_t nsteps, double dt, int32_t ckpt_every,
                     const int32_t* probe_cells, const double* obs, int32_t n_probe, double* loss,
                     double* g_manning_cells, double* g_zb, double* g_inletq, double* Q_final);
/* The final-state inversion loss of swe_2D_inversion.jl:383-431 and its
 * gradients, through the same checkpointed adjoint (nsteps SSP-RK2 steps of dt):
 *   WSE term  sum ((h + zb_wse - wse) / (range(wse) + sqrt(eps)))^2 / n
 *   uv term   sum ((qx / (h + sqrt(eps)) - u)^2 + (qy / (h + sqrt(eps)) - v)^2) / max|(u, v)|^2 / n
 * with h = xi + hstill of the final state.  wse may be NULL (no WSE term); u and
 * v both or neither.  zb_wse NULL: WSE_pred uses the context's zb, as with an
 * active zb parameter, and g_zb includes the direct term.  parts[3] = {WSE + uv,
 * WSE, uv}.  The parameter-only regularisers (bound, slope) are the caller's. */
typedef struct hg_final_obs {
  const double* wse;     /* [n] WSE_truth */
  const double* u;       /* [n] u_truth */
  const double* v;       /* [n] v_truth */
  const double* zb_wse;  /* [n] zb_cell_truth, or NULL */
} hg_final_obs;
int hg_final_loss_and_grad(hg_ctx* ctx, const double* Q0, int32_t nsteps, double dt, int32_t ckpt_every,
                           const hg_final_obs* obs, double* parts, double* g_manning_cells, double* g_zb,
                           double* g_inletq, double* Q_final);

/* Memory of the adjoint's stage-state tape.  The forward pass keeps a
 * checkpoint every ckpt_every steps and the stage states of the last segment;
 * the reverse sweep recomputes the other segments.  A longer segment means less
 * recomputation (none when one segment holds all nsteps steps) for 2 states of
 * 24 bytes per cell per step.  bytes < 0 (the default): segments as long as fit
 * in min(half the free device memory, a quarter of the device's), never shorter
 * than ckpt_every; 0: exactly ckpt_every; > 0: as long as fit in that many
 * bytes, never shorter than ckpt_every.  The gradients do not depend on the
 * segment length (the recomputation repeats the forward pass's arithmetic).
 * The call also frees the tape the context holds from earlier gradient calls;
 * the next one allocates what it needs. */
int hg_set_adjoint_tape(hg_ctx* ctx, int64_t bytes);

/* The time stepping the gradient calls (hg_loss_and_grad,
 * hg_final_loss_and_grad, hg_final_vjp) run and differentiate:
 * HG_ADJ_SSPRK2 (the default) -- nsteps SSP-RK2 steps of dt with the
 * depth-positivity clamp after each stage; HG_ADJ_TSIT5 -- nsteps fixed Tsit5
 * steps of dt (hg_integrate_tsit5 with adaptive = 0), the reference's own
 * integrator (swe_2D_forward_simulation.jl:37-39, whose solve its inversion
 * and sensitivity applications differentiate, swe_2D_inversion.jl:304-339,
 * swe_2D_sensitivity.jl:80), with no clamp of the state, as in the reference's
 * ODE solve.  The Tsit5 adjoint is the exact discrete adjoint of the fixed
 * steps: per step, the six stage states recomputed from the step's start
 * state and the stage cotangents taken back through the RHS Jacobian at each
 * (Kbar_i = dt (b_i lam + sum_{k>i} a_ki Ybar_k), Ybar_i = J(Y_i)^T Kbar_i).
 * In an FP32C context the same steps run on FP32 vectors (the states as hi + lo
 * records, as hg_integrate_tsit5 keeps them; the cotangents in FP32) through
 * the FP32 VJP kernels without the clamp masks.  The probe loss is taken at
 * the states after each step, as with SSP-RK2. */
enum hg_adjoint_integrator { HG_ADJ_SSPRK2 = 0, HG_ADJ_TSIT5 = 1 };
int hg_set_adjoint_integrator(hg_ctx* ctx, int32_t integrator);
/* The step sizes the Tsit5 adjoint differentiates (HG_ADJ_TSIT5): with n > 0,
 * the gradient calls take step s of size dts[s] from t_s = dts[0] + ... +
 * dts[s-1] (their dt argument then unused; nsteps <= n, else HG_ERR_ARG) --
 * typically the accepted steps of an adaptive hg_integrate_tsit5 run
 * (hg_tsit5_steps), held fixed as ForwardDiff through the reference's adaptive
 * solve holds them (its step-size control acts on the values, not the
 * derivatives).  n = 0 returns to steps of dt.  The SSP-RK2 adjoint ignores
 * them. */
int hg_set_adjoint_steps(hg_ctx* ctx, const double* dts, int32_t n);

/* Vector-Jacobian product of the final state: with Q_K the state after nsteps
 * SSP-RK2 steps of dt from Q0, the gradients of lambda . Q_K (lambda [3n], the
 * caller's cell order, blocks xi, qx, qy) w.r.t. the per-cell n, zb and the
 * inlet Q, through the same checkpointed adjoint.  One call per cotangent:
 * the rows of the Jacobian dQ_K/dparams that the reference's sensitivity
 * analysis forms with ForwardDiff (swe_2D_sensitivity.jl), or the gradient of
 * any loss of the final state whose dL/dQ_K the caller forms.  Outputs may be
 * NULL as in hg_loss_and_grad. */
int hg_final_vjp(hg_ctx* ctx, const double* Q0, int32_t nsteps, double dt, int32_t ckpt_every, const double* lambda,
                 double* g_manning_cells, double* g_zb, double* g_inletq, double* Q_final);

/* ---- tuning ------------------------------------------------------------------ */
/* The autotuner of the FP32-compensated fused stages (no counterpart in the
 * reference, which has no GPU kernels).  It chooses among kernels and shapes
 * that compute bit-identical results, in one of two families:
 *   family 0: kernel 0 gather (one block per tile) in four shapes: 256-cell
 *             tiles with the register budget of 4 or 3 resident blocks per
 *             SM (variant 0 / 1), 512-cell tiles at 2 per SM (variant 2),
 *             128-cell tiles at 8 per SM (variant 3);
 *             kernel 1 pipe (persistent, the next tile and its halo
 *             prefetched by asynchronous copies); kernel 2 tma (persistent,
 *             bulk-copy prefetch of the next tile);
 *   family 1: kernel 3 face (each wet-wet face evaluated once for both of its
 *             cells), variant 0 / 1 the 256-cell budgets above, where the
 *             mesh has the face tables (degree <= 4).
 *             Family 0 is the default.
 * The two families round differently (the face kernel forms each face's flux
 * once); a context's family is fixed (hg_set_stage_family, HG_STAGE_FAMILY=
 * gather|face), never chosen by timing.  Each usable candidate is timed on the
 * resident state, reps times, and the fastest is kept and stored in a cache
 * file (HG_AUTOTUNE_CACHE, else $XDG_CACHE_HOME/hydrograd_gb/autotune.json,
 * else ~/.cache/hydrograd_gb/autotune.json; HG_AUTOTUNE_CACHE= (empty)
 * disables it) under a key of the GPU, the mesh's face tables, the Riemann
 * solver and the family.  The first RK2 steps of a context take the cached
 * choice, or tune once by themselves and store it.  HG_STAGE_KERNEL=
 * gather|pipe|tma|face and HG_STAGE_VARIANT=0..3 in the environment force a
 * candidate.  kernel (may be NULL) receives the kernel; reps = 0 only
 * reports it. */
int hg_autotune(hg_ctx* ctx, int32_t reps, int32_t* kernel);
/* The current choice: kernel, variant, and where it came from (source: 0 the
 * default, 1 timed, 2 the cache file, 3 forced by the environment).  Any
 * output may be NULL. */
int hg_autotune_info(const hg_ctx* ctx, int32_t* kernel, int32_t* variant, int32_t* source);
/* The autotuner's family: 0 gather / pipe / tma, 1 face (HG_ERR_UNSUPPORTED
 * when the mesh has no face tables).  The next RK2 steps tune within it. */
int hg_set_stage_family(hg_ctx* ctx, int32_t family);

/* ---- measurement support ---------------------------------------------------- */
/* Number of kernel launches this context has enqueued (graph replays count their kernels). */
int hg_launch_count(const hg_ctx* ctx, int64_t* count);
/* Time n launches of the stage kernel alone with CUDA events on the context's stream,
 * flushing L2 between launches when flush_l2 != 0; avg_ms receives the mean duration. */
int hg_time_stage_kernel(hg_ctx* ctx, int32_t n, int32_t flush_l2, double* avg_ms);
/* The same for the FP32C adjoint's interior VJP kernel (boundary faces folded
 * in; one stage-2 VJP of the resident state with a constant cotangent):
 * HG_ERR_UNSUPPORTED for FP64 contexts, a state-dependent resistance, an inlet
 * hydrograph or a mesh the pipelined kernel cannot take. */
int hg_time_vjp_kernel(hg_ctx* ctx, int32_t n, int32_t flush_l2, double* avg_ms);
/* Write a device buffer larger than L2 (used between timed iterations). */
int hg_flush_l2(hg_ctx* ctx);
/* nsteps SSP-RK2 steps on the resident state, each bracketed by CUDA events on
 * the context's stream; when flush_l2 != 0 an L2 flush runs before each step,
 * outside the events.  total_ms receives the summed device time of the steps. */
int hg_advance_timed(hg_ctx* ctx, int32_t nsteps, double dt, double cfl, int32_t flush_l2, double* total_ms);
/* ---- no-allocation RHS ----------------------------------------------------- */
/*
 * No counterpart in the reference.  dQdt = RHS(Q) of an FP64 context for a
 * state that is already in device memory, for callers that cannot allocate
 * device memory once their time loop runs (an integrator inside CUDA.jl's
 * memory pool, or a step being recorded into a CUDA graph, where allocation
 * and device synchronisation are not allowed).  It calls no cudaMalloc or
 * cudaFree: the scratch it needs (inlet-Q conveyance totals and an error-flag
 * word) is a static device array sized for HG_NOALLOC_MAX_INLETQ inlet-Q
 * boundaries; a context with more is rejected with HG_ERR_ARG.  A context
 * with an inlet hydrograph (its inlet Q depends on the time, which this call
 * does not take) or a state-dependent resistance (whose kernels write the
 * context's own per-cell n before every RHS) is rejected with
 * HG_ERR_UNSUPPORTED: use hg_rhs for those.
 *   d_Q, d_dQ: device pointers to 3 n doubles in the device cell order
 *              (perm[device id] = caller id from hg_mesh_order with consts.order).
 *   d_flags:   device int32 that receives the error flags (bit 1: inlet-Q
 *              conveyance not positive), or NULL.  Nothing is checked on the host.
 *   stream:    cudaStream_t to run on, or NULL for the context's stream.
 * The call is asynchronous.  Its first call on a device looks up the scratch
 * array's device address; make that first call before any stream capture.
 * All calls share the scratch array: calls that overlap on the GPU race.
 */
#define HG_NOALLOC_MAX_INLETQ 64
int hg_rhs_device_noalloc(hg_ctx* ctx, const double* d_Q, double* d_dQ, int32_t* d_flags, void* stream);

/* Page-locked host buffers for fast host<->device copies of states. */
int hg_pinned_alloc(int64_t bytes, void** out);
int hg_pinned_free(void* p);

#ifdef __cplusplus
}
#endif
#endif /* HYDROGRAD_GB_H */
