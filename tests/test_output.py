"""Solution output (output_results, advection_solver.cc:1220-1241): the VTU
writer on host values (no GPU), checked by parsing the file; VTU from a
device vector and the raw state round trip on the GPU."""
import xml.etree.ElementTree as ET

import numpy as np
import pytest

CFG = dict(degree=2, n_cells=(2, 3, 2), mesh_type=1, deformation=0.08)


def read_vtu(path):
    root = ET.parse(path).getroot()
    piece = root.find("UnstructuredGrid/Piece")
    arrays = {}
    for da in root.iter("DataArray"):
        name = da.get("Name") or "points"
        arrays[name] = np.array(da.text.split(), dtype=float)
    return int(piece.get("NumberOfPoints")), int(piece.get("NumberOfCells")), arrays


def test_vtu_from_host_values(adv_lib, oracle_mod, tmp_path):
    cfg = adv_lib.make_config(**CFG)
    o = oracle_mod.Oracle(**CFG)
    vals = np.random.default_rng(0).standard_normal(o.n_dofs)
    path = tmp_path / "solution_000.vtu"
    adv_lib.write_vtu_host(cfg, vals, 0.25, path)
    npts, ncells, a = read_vtu(path)
    k, n = 2, 3
    cells = 2 * 3 * 2
    assert npts == cells * n ** 3 == o.n_dofs
    assert ncells == cells * k ** 3
    assert a["TIME"][0] == 0.25
    # points: the mapped Gauss-Lobatto support points, cell by cell
    np.testing.assert_allclose(a["points"].reshape(-1, 3), o.support_points().reshape(-1, 3), rtol=0, atol=1e-14)
    np.testing.assert_array_equal(a["solution"], vals)
    np.testing.assert_allclose(a["analytic_solution"], o.interpolate(0.25), rtol=0, atol=1e-13)
    conn = a["connectivity"].astype(np.int64).reshape(-1, 8)
    assert conn.min() == 0 and conn.max() == npts - 1
    # every hexahedron stays inside one cell and spans one sub-cell of the node grid
    assert np.all(conn // n ** 3 == conn[:, :1] // n ** 3)
    assert np.array_equal(a["offsets"], 8 * np.arange(1, ncells + 1))
    assert np.all(a["types"] == 12)


@pytest.mark.gpu
def test_vtu_and_state_round_trip_on_device(cuda, adv_lib, tmp_path):
    torch = cuda
    cfg = adv_lib.make_config(**CFG)
    op = adv_lib.AdvectionOperation(cfg)
    u = op.initialize_dof_vector()
    op.project_initial(u)
    op.write_vtu(u, 0.0, tmp_path / "dev.vtu")
    adv_lib.write_vtu_host(cfg, u.cpu().numpy(), 0.0, tmp_path / "host.vtu")
    assert (tmp_path / "dev.vtu").read_text() == (tmp_path / "host.vtu").read_text()
    op.save_state(u, 0.125, tmp_path / "state.bin")
    w = op.initialize_dof_vector()
    assert op.load_state(w, tmp_path / "state.bin") == 0.125
    assert torch.equal(u, w)
    other = adv_lib.AdvectionOperation(adv_lib.make_config(**dict(CFG, degree=3)))
    with pytest.raises(adv_lib.AdvError):
        other.load_state(other.initialize_dof_vector(), tmp_path / "state.bin")
