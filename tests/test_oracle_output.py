"""The oracle's Output_plt_file restatement (mpm_ini.cpp:832-980), the
reference the library's snapshot writer is checked against: the file layout
read back, and its contents against the oracle's own state."""
import numpy as np

from tests.plt_read import read_cell_table, read_particle_plt

NAMES = ["x", "y", "z", "phase", "vx", "vy", "vol", "rho", "P", "tv", "v", "n_neighbor"]


def _state(O, M, cid, grid, steps):
    cs, p, c = M.make_case(cid, grid)
    o = O.Oracle(cs)
    o.upload_particles(p)
    o.upload_cells(c)
    o.advance(steps)
    return cs, o


def test_particle_file_layout_and_values(oracle_mod, tmp_path):
    import pgdg_p2_gb300.mpm as M
    for cid, grid, steps in ((3, (24, 6, 6), 2), (1, (56, 24), 3)):
        cs, o = _state(oracle_mod, M, cid, grid, steps)
        path = tmp_path / f"p{cid}.plt"
        o.output_plt(path, None)
        hdr, data = read_particle_plt(path)
        assert hdr["version"] == (1, 0, 0) and hdr["names"] == NAMES and hdr["zone"] == "grid"
        assert hdr["types"] == [2, 2, 2, 3, 2, 2, 2, 2, 2, 2, 2, 3]
        assert hdr["time"] == o.stats()["time"] > 0
        assert hdr["ranges"] == (-1.0, 1.0) * 12
        p = o.download_particles()
        assert hdr["imax"] == p.n and hdr["jmax"] == hdr["kmax"] == 1
        d = cs.dim
        for k, col in (("x", 0), ("y", 1), ("z", 2)):
            want = p.coord[:, col] if col < d else np.zeros(p.n)
            assert np.array_equal(data[k], want), k
        assert np.array_equal(data["phase"], p.phase)
        assert np.array_equal(data["vx"], p.v[:, 0]) and np.array_equal(data["vy"], p.v[:, 1])
        for k in ("vol", "rho", "P"):
            assert np.array_equal(data[k], getattr(p, k)), k
        assert np.allclose(data["tv"], np.linalg.norm(p.tv[:, :d], axis=1), rtol=1e-15, atol=0)
        assert np.allclose(data["v"], np.linalg.norm(p.v[:, :d], axis=1), rtol=1e-15, atol=0)
        # flag-2 lists: about 4/3 pi 3.2^3 = 137 (3D) or pi 3.2^2 = 32 (2D) in the interior
        nn = data["n_neighbor"]
        assert nn.min() >= 1
        full = 137 if d == 3 else 32
        assert 0.5 * full < np.median(nn) < 1.5 * full, np.median(nn)


def test_cell_table_layout_and_values(oracle_mod, tmp_path):
    import pgdg_p2_gb300.mpm as M
    cs, o = _state(oracle_mod, M, 3, (24, 6, 6), 2)
    path = tmp_path / "c.plt"
    o.output_plt(None, path)
    (h1, h2), rows = read_cell_table(path)
    assert h1 == ('VARIABLES = "x","y","z", "v1","v2", "v","rho0","rho1",        '
                  '"E0","E1","Lim0","Lim1","st", "st1", "P"\n')
    assert h2.startswith('ZONE T="GRID 1",SOLUTIONTIME=')
    assert abs(float(h2.split("=")[-1]) - o.stats()["time"]) <= 1e-5 * o.stats()["time"]
    c = o.download_cells()
    assert rows.shape == (cs.ncells, 15)
    U, B = cs.dim + 2, cs.dim + 1
    idx = np.indices(tuple(cs.ncell[:3])).reshape(3, -1).T
    cen = np.array(cs.box_l[:3]) + np.array(cs.p_size[:3]) * (idx + 0.5)
    want = np.column_stack([cen, c.v[:, 0], c.v[:, 1], np.linalg.norm(c.v[:, :cs.dim], axis=1), c.rho[:, 0],
                            c.rho[:, 1], c.coef[:, 0, 1, 1], c.coef[:, 0, 1, 2], c.lim_u[:, 0, 0], c.lim_u[:, 1, 0],
                            c.alph[:, 0], c.alph[:, 1], c.P])
    # six significant digits
    assert np.allclose(rows, want, rtol=6e-6, atol=1e-300)
    with open(path) as f:
        lines = f.read().split("\n")
    assert all(ln.endswith(" ") for ln in lines[2:-1]) and lines[-1] == ""
