"""The library's host-side mesh build (hg_mesh_build) against the oracle's
independent restatement of mesh_2D.jl / SRH_2D_SRHGeom.jl.  No GPU needed."""
import numpy as np
import pytest

from hydrograd_gb import HostMesh, HgError
from hydrograd_gb.workloads import dam_break, river_triangles
from oracle.oracle import Oracle
from tests.golden_cases import load_fixture


def _cases():
    yield "fwd_bump", load_fixture("fwd_bump")
    yield "fwd_savannah", load_fixture("fwd_savannah")
    yield "dam_break", dam_break(20, 6, 10.0, 3.0)
    yield "river", river_triangles(n=12, L=120.0)


@pytest.mark.parametrize("name,case", list(_cases()), ids=[c[0] for c in _cases()])
def test_topology_and_geometry_match_oracle_bitwise(name, case):
    hm = HostMesh(case)
    o = Oracle(case)
    assert (hm.n_cells, hm.n_faces, hm.n_ghosts) == (o.n_cells, o.n_faces, o.n_ghosts)
    assert (hm.n_inletq, hm.n_exith, hm.n_wall, hm.n_symm) == (o.n_inlet, o.n_exit, o.n_wall, o.n_symm)
    cf = hm.cell_faces()
    om = o.mesh_arrays()
    N = o.n_cells
    cnt = np.asarray(case["cell_node_count"])
    has = np.arange(8)[None, :] < cnt[:, None]
    onb = om["cell_neighbors"].reshape(N, 8)
    fib = om["face_is_boundary"][om["cell_faces"].reshape(N, 8)].astype(bool)
    exp_nbr = np.where(has, np.where(fib, -1, onb), -2)
    assert np.array_equal(cf["nbr"], exp_nbr)
    assert np.array_equal(cf["areas"], om["areas"])
    assert np.array_equal(cf["centroids"].ravel(), om["centroids"])
    on = om["normals"].reshape(N, 8, 2)
    assert np.array_equal(np.where(has[..., None], cf["normals"], 0), np.where(has[..., None], on, 0))
    ol = om["face_lengths"][om["cell_faces"].reshape(N, 8)]
    assert np.array_equal(np.where(has, cf["lengths"], 0), np.where(has, ol, 0))


@pytest.mark.parametrize("order", ["none", "rcm", "hilbert"])
def test_orderings_are_permutations(order):
    hm = HostMesh(river_triangles(n=16, L=160.0))
    p = hm.order(order)
    assert np.array_equal(np.sort(p), np.arange(hm.n_cells))


def test_rcm_reduces_bandwidth():
    case = river_triangles(n=24, L=240.0)
    hm = HostMesh(case)
    nbr = hm.cell_faces()["nbr"]
    def bandwidth(perm):
        inv = np.empty_like(perm); inv[perm] = np.arange(len(perm))
        c = np.repeat(np.arange(len(perm)), 8).reshape(-1, 8)
        ok = nbr >= 0
        return np.abs(inv[c[ok]] - inv[nbr[ok]]).max()
    shuffled = np.random.default_rng(0).permutation(hm.n_cells).astype(np.int32)
    assert bandwidth(hm.order("rcm")) < bandwidth(shuffled) / 10


def test_clockwise_cell_is_rejected():
    case = dam_break(4, 2, 4.0, 2.0)
    case["cell_nodes"][0, :4] = case["cell_nodes"][0, :4][::-1].copy()
    with pytest.raises(HgError) as e:
        HostMesh(case)
    assert e.value.code == 2


def test_nodestring_off_the_boundary_is_rejected():
    case = dam_break(4, 2, 4.0, 2.0)
    case.update(string_ids=np.array([1], np.int32), string_offsets=np.array([0, 2], np.int32),
                string_nodes=np.array([6, 7], np.int32), string_bc=np.array([0], np.int32))
    with pytest.raises(HgError):
        HostMesh(case)
