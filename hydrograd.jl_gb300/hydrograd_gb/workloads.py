"""Seeded synthetic workloads (meshes, parameters, initial states).

The reference ships meshes of at most 1,306 cells and publishes no benchmark
data set, so the workloads below are generated: structured grids stored as
unstructured cell lists, with a project-written splitmix64 stream so every
harness (tests, benchmark, oracle) sees the same inputs for the same seed.

* :func:`dam_break`      200x40 quads over 100 m x 20 m, walls, h = 1.0 / 0.5 m.
* :func:`river_triangles` n x n grid split into 2 triangles per quad, nodes
  jittered by +-0.2 dx over 2 km x 2 km; bed = 1e-3 slope + 20 Gaussian bumps;
  5 Voronoi Manning zones; inlet-Q on the west edge, exit-H on the east edge,
  walls elsewhere; a lake at rest with its surface raised 1.5 m in a pool disk
  (dry_land=True: dry except the pool).
* :func:`meander_mixed`  configuration 5: a 10 km reach on a mixed mesh -- a
  core of n_core^2 quads inside a band of jittered triangles (1,600^2 quads +
  1.45 M triangles = 4.0 M cells by default) -- with a meandering channel
  carved 4 m deep into a floodplain of Gaussian bumps, a per-cell Manning n
  field U[0.02, 0.08] smoothed by a 100 m Gaussian, and an inlet hydrograph
  ramping from 200 to 2,000 m^3/s over 3,600 s.

A case is a dict with the mesh arrays of ``hg_mesh_desc`` plus parameters:
mat_id, manning_zones, inlet_q, exit_wse, wstill (per cell) and Q0.
"""
import numpy as np

H_SMALL = 1.0e-3
_GOLD = np.uint64(0x9E3779B97F4A7C15)


def splitmix64(seed, n):
    """n uniform doubles in [0, 1) from the splitmix64 stream of ``seed``."""
    with np.errstate(over="ignore"):
        x = np.uint64(seed) + (np.arange(1, n + 1, dtype=np.uint64) * _GOLD)
        z = x
        z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
        z = z ^ (z >> np.uint64(31))
    return (z >> np.uint64(11)).astype(np.float64) * (1.0 / 9007199254740992.0)


class Stream:
    """Sequential draws from one seed."""

    def __init__(self, seed):
        self.seed = np.uint64(seed)
        self.pos = 0

    def uniform(self, n, lo=0.0, hi=1.0):
        with np.errstate(over="ignore"):
            start = np.uint64(self.seed + np.uint64(self.pos) * _GOLD)
        u = splitmix64(start, n) if n > 0 else np.zeros(0)
        self.pos += n
        return lo + (hi - lo) * u


def _grid_nodes(nx, ny, Lx, Ly):
    xs = np.linspace(0.0, Lx, nx + 1)
    ys = np.linspace(0.0, Ly, ny + 1)
    X, Y = np.meshgrid(xs, ys, indexing="xy")      # node (i, j) -> j*(nx+1) + i
    return X.ravel(), Y.ravel()


def _nid(i, j, nx):
    return j * (nx + 1) + i


def _string(nodes):
    return np.asarray(nodes, dtype=np.int32)


def _pack_strings(strings):
    ids = np.array([s[0] for s in strings], dtype=np.int32)
    bcs = np.array([s[1] for s in strings], dtype=np.int32)
    offs = np.cumsum([0] + [len(s[2]) for s in strings]).astype(np.int32)
    nodes = np.concatenate([s[2] for s in strings]).astype(np.int32) if strings else np.zeros(0, np.int32)
    return ids, offs, nodes, bcs


def initial_xi(h, wstill, zb):
    """xi = h - hstill with hstill = wstill - zb.

    A cell meant to be dry (h == h_small) gets the largest xi whose FP64 depth
    xi + hstill does not exceed h_small, so the RHS clamps it (h <= h_small,
    semi_discretize_swe_2D.jl:104).  Rounding alone would leave about half of
    such cells one ulp above h_small, i.e. a wet film 1e-19 m thick whose
    Manning friction is stiff enough to break any explicit step."""
    hst = wstill - zb
    xi = h - hst
    dry = h <= H_SMALL
    for _ in range(8):
        hi = dry & (xi + hst > h)
        if not hi.any():
            break
        xi[hi] = np.nextafter(xi[hi], -np.inf)
    for _ in range(8):
        lo = ~dry & (xi + hst < h)
        if not lo.any():
            break
        xi[lo] = np.nextafter(xi[lo], np.inf)
    return xi


def cell_centroids(case):
    """Polygon centroids (same formula as the mesh builder)."""
    xyz = case["node_xyz"]
    cn, cnt = case["cell_nodes"], case["cell_node_count"]
    N = len(cnt)
    cx = np.zeros(N)
    cy = np.zeros(N)
    a = np.zeros(N)
    for k in range(cn.shape[1]):
        has = k < cnt
        if not has.any():
            break
        p = cn[:, k]
        q = np.where(k + 1 < cnt, cn[:, (k + 1) % 8], cn[:, 0])
        x1, y1 = xyz[p, 0], xyz[p, 1]
        x2, y2 = xyz[q, 0], xyz[q, 1]
        cr = np.where(has, x1 * y2 - x2 * y1, 0.0)
        cx += np.where(has, (x1 + x2) * cr, 0.0)
        cy += np.where(has, (y1 + y2) * cr, 0.0)
        a += cr
    a = np.abs(a) / 2
    return cx / (6 * a), cy / (6 * a)


def dam_break(nx=200, ny=40, Lx=100.0, Ly=20.0, n=0.03, h_left=1.0, h_right=0.5, x_gate=50.0):
    """Flat-bed dam break, all boundaries walls (the default wall boundary)."""
    X, Y = _grid_nodes(nx, ny, Lx, Ly)
    xyz = np.stack([X, Y, np.zeros_like(X)], axis=1)
    i, j = np.meshgrid(np.arange(nx), np.arange(ny), indexing="xy")
    i, j = i.ravel(), j.ravel()
    cells = np.full((nx * ny, 8), -1, dtype=np.int32)
    cells[:, 0] = _nid(i, j, nx)
    cells[:, 1] = _nid(i + 1, j, nx)
    cells[:, 2] = _nid(i + 1, j + 1, nx)
    cells[:, 3] = _nid(i, j + 1, nx)
    case = dict(node_xyz=xyz, cell_nodes=cells, cell_node_count=np.full(nx * ny, 4, np.int32),
                string_ids=np.zeros(0, np.int32), string_offsets=np.zeros(1, np.int32),
                string_nodes=np.zeros(0, np.int32), string_bc=np.zeros(0, np.int32))
    N = nx * ny
    cx, _ = cell_centroids(case)
    h = np.where(cx < x_gate, h_left, h_right)
    case.update(mat_id=np.zeros(N, np.int32), manning_zones=np.array([n]), inlet_q=np.zeros(0), exit_wse=np.zeros(0),
                wstill=np.zeros(N), Q0=np.concatenate([h, np.zeros(N), np.zeros(N)]),
                name=f"dam_break_{nx}x{ny}")
    return case


def river_triangles(n=708, L=2000.0, seed=0, inlet_q=500.0, exit_wse=None, wstill=None, pool_h=1.5,
                    pool_center=(300.0, 1000.0), pool_radius=350.0, n_bumps=20, n_zones=5, jitter=0.2,
                    dry_land=False):
    """Triangulated reach of 2 n^2 cells.

    dry_land=False (the benchmark state): a lake at rest at wstill (default
    0.3 m above the highest bed cell, so every cell is wet) with the water
    surface raised by pool_h inside the pool disk -- the release sends a bore
    across the reach; exit-H holds the lake level.  dry_land=True: every cell
    outside the pool is dry (h = h_small) and the pool touches the inlet.

    The reference scheme is not robust on a dry bed: at a dry bank its Roe
    wall branch keeps the dry side's xi (swe_2D_solvers.jl:23-53) and pumps
    mass into the wet cell even at rest, and a flooded cell gets the full
    one-sided pressure as momentum while nearly empty.  Dry-bed states are
    therefore used for short parity runs, not for the long benchmark runs.
    """
    rs = Stream(seed)
    dx = L / n
    X, Y = _grid_nodes(n, n, L, L)
    nn = X.size
    jx = rs.uniform(nn, -jitter, jitter) * dx
    jy = rs.uniform(nn, -jitter, jitter) * dx
    ii = np.tile(np.arange(n + 1), n + 1)
    jj = np.repeat(np.arange(n + 1), n + 1)
    interior_x = (ii > 0) & (ii < n)
    interior_y = (jj > 0) & (jj < n)
    X = X + np.where(interior_x, jx, 0.0)      # boundary nodes stay on their edge
    Y = Y + np.where(interior_y, jy, 0.0)
    # Bed: linear slope 1e-3 falling to the east plus Gaussian bumps.
    A = rs.uniform(n_bumps, 0.5, 3.0)
    S = rs.uniform(n_bumps, 20.0, 150.0)
    BX = rs.uniform(n_bumps, 0.0, L)
    BY = rs.uniform(n_bumps, 0.0, L)
    Z = 1e-3 * (L - X)
    for k in range(n_bumps):
        Z = Z + A[k] * np.exp(-((X - BX[k]) ** 2 + (Y - BY[k]) ** 2) / (2 * S[k] ** 2))
    xyz = np.stack([X, Y, Z], axis=1)
    i, j = np.meshgrid(np.arange(n), np.arange(n), indexing="xy")
    i, j = i.ravel(), j.ravel()
    n00, n10, n11, n01 = _nid(i, j, n), _nid(i + 1, j, n), _nid(i + 1, j + 1, n), _nid(i, j + 1, n)
    cells = np.full((2 * n * n, 8), -1, dtype=np.int32)
    cells[0::2, 0], cells[0::2, 1], cells[0::2, 2] = n00, n10, n11
    cells[1::2, 0], cells[1::2, 1], cells[1::2, 2] = n00, n11, n01
    N = 2 * n * n
    west = [_nid(0, jj_, n) for jj_ in range(n, -1, -1)]          # north -> south along x = 0
    east = [_nid(n, jj_, n) for jj_ in range(0, n + 1)]           # south -> north along x = L
    ids, offs, snodes, bcs = _pack_strings([(1, 2, _string(west)), (2, 3, _string(east))])
    case = dict(node_xyz=xyz, cell_nodes=cells, cell_node_count=np.full(N, 3, np.int32), string_ids=ids,
                string_offsets=offs, string_nodes=snodes, string_bc=bcs)
    cx, cy = cell_centroids(case)
    # Orientation check: every triangle counter-clockwise.
    p, q, r = cells[:, 0], cells[:, 1], cells[:, 2]
    area2 = (X[q] - X[p]) * (Y[r] - Y[p]) - (X[r] - X[p]) * (Y[q] - Y[p])
    if not (area2 > 0).all():
        raise RuntimeError("jittered mesh has an inverted triangle; lower the jitter")
    # Manning zones: nearest of n_zones Voronoi seeds.
    SX = rs.uniform(n_zones, 0.0, L)
    SY = rs.uniform(n_zones, 0.0, L)
    zones_n = rs.uniform(n_zones, 0.02, 0.06)
    d2 = (cx[:, None] - SX[None, :]) ** 2 + (cy[:, None] - SY[None, :]) ** 2
    mat = np.argmin(d2, axis=1).astype(np.int32)
    zb = ((Z[cells[:, 0]] + Z[cells[:, 1]]) + Z[cells[:, 2]]) / 3    # mean of node z, in the mesh builder's order
    pool = (cx - pool_center[0]) ** 2 + (cy - pool_center[1]) ** 2 < pool_radius ** 2
    if wstill is None:
        wstill = 2.0 if dry_land else float(np.ceil((zb.max() + 0.3) * 10.0) / 10.0)
    if exit_wse is None:
        exit_wse = 2.0 if dry_land else wstill
    if dry_land:
        h = np.where(pool, pool_h, H_SMALL)
    else:
        h = (wstill - zb) + np.where(pool, pool_h, 0.0)
    xi = initial_xi(h, np.full(N, wstill), zb)
    case.update(mat_id=mat, manning_zones=zones_n, inlet_q=np.array([inlet_q]), exit_wse=np.array([exit_wse]),
                wstill=np.full(N, wstill), Q0=np.concatenate([xi, np.zeros(N), np.zeros(N)]),
                zb_cells=zb, pool_center=tuple(pool_center), pool_radius=float(pool_radius),
                name=f"river_tri_{n}x{n}x2" + ("_dry" if dry_land else ""))
    return case


def probes_and_perturbation(case, n_probe=64, seed=1, zb_sigma=0.05, rim_width=None, inlet_share=0.0):
    """Seeded probe cells and a per-cell bed perturbation drawn in FP32 with
    standard deviation zb_sigma.  The probes are wet cells within rim_width
    (default: 4 mean cell sizes) of the pool's rim, where the released bore
    passes in the first steps, so that a short run's loss sees the flow; a
    fraction inlet_share of them is taken instead from the wet cells within
    rim_width of the west edge (the inlet-Q boundary of river_triangles)."""
    rs = Stream(seed)
    N = len(case["cell_node_count"])
    Q0 = case["Q0"]
    wet = Q0[:N] + case["wstill"] - case["zb_cells"] > 2 * H_SMALL
    cand = np.nonzero(wet)[0]
    cx, cy = cell_centroids(case)
    xyz = case["node_xyz"]
    cell = np.sqrt((np.ptp(xyz[:, 0]) * np.ptp(xyz[:, 1])) / N)
    w = 4.0 * cell if rim_width is None else rim_width
    n_inlet = int(round(n_probe * inlet_share))
    inlet = np.zeros(0, np.int64)
    if n_inlet > 0:
        west = np.nonzero(wet & (cx < xyz[:, 0].min() + w))[0]
        pick = np.unique((rs.uniform(4 * n_inlet) * len(west)).astype(np.int64))[:n_inlet]
        inlet = west[np.sort(pick)]
        n_probe -= len(inlet)
    if "pool_center" in case:
        r = np.hypot(cx - case["pool_center"][0], cy - case["pool_center"][1])
        rim = np.nonzero(wet & (np.abs(r - case["pool_radius"]) < w))[0]
        if len(rim) >= n_probe:
            cand = rim
    pick = np.unique((rs.uniform(4 * n_probe) * len(cand)).astype(np.int64))[:n_probe]
    probes = np.unique(np.concatenate([inlet, cand[np.sort(pick)]])).astype(np.int32)
    # Box-Muller from two uniform draws, rounded to float32.
    u1 = np.maximum(rs.uniform(N), 1e-300)
    u2 = rs.uniform(N)
    dz = (zb_sigma * np.sqrt(-2.0 * np.log(u1)) * np.cos(2 * np.pi * u2)).astype(np.float32)
    return probes, dz.astype(np.float64)


def _gaussian_smooth(field, sigma_cells):
    """Separable Gaussian filter (truncated at 4 sigma, reflecting edges) of a 2D array."""
    r = int(np.ceil(4.0 * sigma_cells))
    x = np.arange(-r, r + 1, dtype=np.float64)
    k = np.exp(-0.5 * (x / sigma_cells) ** 2)
    k /= k.sum()
    out = field
    for axis in (0, 1):
        pad = [(0, 0), (0, 0)]
        pad[axis] = (r, r)
        p = np.pad(out, pad, mode="reflect")
        acc = np.zeros_like(out)
        for i, w in enumerate(k):
            sl = [slice(None), slice(None)]
            sl[axis] = slice(i, i + out.shape[axis])
            acc += w * p[tuple(sl)]
        out = acc
    return out


def meander_mixed(n_core=1600, n_band=106, L=10000.0, seed=7, jitter=0.2, n_bumps=40, depth=4.0,
                  half_width=100.0, q_start=200.0, q_end=2000.0, ramp=3600.0, n_sigma=100.0):
    """Configuration 5.  An (n_core + 2 n_band)^2 grid over L x L: the inner
    n_core^2 squares are quads, the others each split into two triangles; the
    band's interior nodes are jittered by +-jitter dx.  Bed: a 2e-4 slope
    falling to the east, n_bumps Gaussian bumps (A in U[0.2, 1.5] m, sigma in
    U[100, 500] m), and a channel of half-width half_width carved depth m deep
    (cosine profile) along the centreline y = L/2 + a sin(2 pi x / lambda),
    a in U[200, 600] m, lambda in U[1500, 3000] m.  Manning n per cell: U[0.02,
    0.08] per grid square, Gaussian-smoothed (sigma n_sigma m).  Inlet-Q on the
    west edge with the hydrograph (0, q_start), (ramp, q_end); exit-H on the
    east edge at the lake level; walls elsewhere.  Initial state: a lake at
    rest 0.3 m above the highest bed cell (every cell wet)."""
    rs = Stream(seed)
    nc = n_core + 2 * n_band
    dx = L / nc
    X, Y = _grid_nodes(nc, nc, L, L)
    nn = X.size
    ii = np.tile(np.arange(nc + 1), nc + 1)
    jj = np.repeat(np.arange(nc + 1), nc + 1)
    core_node = (ii >= n_band) & (ii <= n_band + n_core) & (jj >= n_band) & (jj <= n_band + n_core)
    inner = (ii > 0) & (ii < nc) & (jj > 0) & (jj < nc)
    jmask = inner & ~core_node
    jx = rs.uniform(nn, -jitter, jitter) * dx
    jy = rs.uniform(nn, -jitter, jitter) * dx
    X = X + np.where(jmask, jx, 0.0)
    Y = Y + np.where(jmask, jy, 0.0)
    A = rs.uniform(n_bumps, 0.2, 1.5)
    S = rs.uniform(n_bumps, 100.0, 500.0)
    BX = rs.uniform(n_bumps, 0.0, L)
    BY = rs.uniform(n_bumps, 0.0, L)
    amp = rs.uniform(1, 200.0, 600.0)[0]
    lam = rs.uniform(1, 1500.0, 3000.0)[0]
    Z = 2e-4 * (L - X)
    for k in range(n_bumps):
        Z = Z + A[k] * np.exp(-((X - BX[k]) ** 2 + (Y - BY[k]) ** 2) / (2 * S[k] ** 2))
    d = np.abs(Y - (0.5 * L + amp * np.sin(2 * np.pi * X / lam)))
    Z = Z - np.where(d < half_width, depth * 0.5 * (1.0 + np.cos(np.pi * d / half_width)), 0.0)
    xyz = np.stack([X, Y, Z], axis=1)
    i, j = np.meshgrid(np.arange(nc), np.arange(nc), indexing="xy")
    i, j = i.ravel(), j.ravel()
    quad = (i >= n_band) & (i < n_band + n_core) & (j >= n_band) & (j < n_band + n_core)
    n00, n10, n11, n01 = _nid(i, j, nc), _nid(i + 1, j, nc), _nid(i + 1, j + 1, nc), _nid(i, j + 1, nc)
    nq = int(quad.sum())
    nt = 2 * int((~quad).sum())
    N = nq + nt
    cells = np.full((N, 8), -1, dtype=np.int32)
    cnt = np.empty(N, np.int32)
    sq = np.empty(N, np.int64)   # grid square of each cell (for the n field)
    # cells in grid-square order: a quad, or the square's two triangles
    per = np.where(quad, 1, 2)
    start = np.concatenate([[0], np.cumsum(per)[:-1]])
    q_idx = start[quad]
    cells[q_idx, 0], cells[q_idx, 1], cells[q_idx, 2], cells[q_idx, 3] = n00[quad], n10[quad], n11[quad], n01[quad]
    cnt[q_idx] = 4
    sq[q_idx] = np.nonzero(quad)[0]
    t_idx = start[~quad]
    nb = ~quad
    cells[t_idx, 0], cells[t_idx, 1], cells[t_idx, 2] = n00[nb], n10[nb], n11[nb]
    cells[t_idx + 1, 0], cells[t_idx + 1, 1], cells[t_idx + 1, 2] = n00[nb], n11[nb], n01[nb]
    cnt[t_idx] = 3
    cnt[t_idx + 1] = 3
    sq[t_idx] = np.nonzero(nb)[0]
    sq[t_idx + 1] = np.nonzero(nb)[0]
    west = [_nid(0, jj_, nc) for jj_ in range(nc, -1, -1)]
    east = [_nid(nc, jj_, nc) for jj_ in range(0, nc + 1)]
    ids, offs, snodes, bcs = _pack_strings([(1, 2, _string(west)), (2, 3, _string(east))])
    case = dict(node_xyz=xyz, cell_nodes=cells, cell_node_count=cnt, string_ids=ids, string_offsets=offs,
                string_nodes=snodes, string_bc=bcs)
    # counter-clockwise check (triangles and quads: the first three nodes)
    p, q, r = cells[:, 0], cells[:, 1], cells[:, 2]
    area2 = (X[q] - X[p]) * (Y[r] - Y[p]) - (X[r] - X[p]) * (Y[q] - Y[p])
    if not (area2 > 0).all():
        raise RuntimeError("jittered mesh has an inverted cell; lower the jitter")
    nf = rs.uniform(nc * nc, 0.02, 0.08).reshape(nc, nc)
    n_cells = _gaussian_smooth(nf, n_sigma / dx).ravel()[sq]
    zsum = Z[cells[:, 0]] + Z[cells[:, 1]]
    zsum = zsum + Z[cells[:, 2]]
    zsum = np.where(cnt == 4, zsum + Z[np.maximum(cells[:, 3], 0)], zsum)
    zb = zsum / cnt
    wstill = float(np.ceil((zb.max() + 0.3) * 10.0) / 10.0)
    h = wstill - zb
    xi = initial_xi(h, np.full(N, wstill), zb)
    case.update(mat_id=np.zeros(N, np.int32), manning_zones=np.array([0.05]), manning_cells=n_cells,
                inlet_q=np.array([q_start]), exit_wse=np.array([wstill]), wstill=np.full(N, wstill),
                Q0=np.concatenate([xi, np.zeros(N), np.zeros(N)]), zb_cells=zb,
                hydrograph=(np.array([0.0, ramp]), np.array([q_start, q_end])),
                name=f"meander_mixed_{n_core}q_{n_band}b")
    return case

