"""pyCATHY-facing files: project folders written and read back, and the
output files (psi, mbeconv) in the layouts pyCATHY's readers parse
(pyCATHY/importers/cathy_outputs.py:480 read_psi, :607 read_mbeconv)."""
import os

import numpy as np
import pytest


def _cases():
    from pycathy_wrapper_gb300.inputs import config0, config2_members, config4_member
    return [config0(tmax=600.0), config2_members(2, tmax=600.0, min_cells=5, max_cells=7)[1],
            config4_member(ncell=5, nstr=4, tmax=600.0)]


@pytest.mark.parametrize("k", [0, 1, 2])
def test_project_round_trip(tmp_path, k):
    from pycathy_wrapper_gb300.project import read_project
    from pycathy_wrapper_gb300.pycathy import write_project
    c = _cases()[k]
    write_project(c, str(tmp_path))
    r = read_project(str(tmp_path))
    np.testing.assert_array_equal(r.dem.dem, c.dem.dem)
    np.testing.assert_array_equal(r.dem.zratio, c.dem.zratio)
    for f in ("delta_x", "delta_y", "base", "ivert", "factor"):
        assert getattr(r.dem, f) == getattr(c.dem, f), f
    for f in ("permx", "permy", "permz", "elstor", "poros", "vgn", "vgrmc", "vgpsat"):
        np.testing.assert_array_equal(getattr(r.soil, f), getattr(c.soil, f))
    for f in ("iopt", "lump", "itmxcg", "ituns", "ituns1", "ituns2", "l2norm", "tetaf",
              "toluns", "tolcg", "deltat", "dtmin", "dtmax", "tmax", "dtmaga", "dtmagm",
              "dtreds", "dtredm"):
        assert getattr(r.parm, f) == getattr(c.parm, f), f
    assert r.bc.indp == c.bc.indp
    np.testing.assert_array_equal(r.bc.atmtim, c.bc.atmtim)
    np.testing.assert_array_equal(np.ravel(r.bc.atminp), np.ravel(c.bc.atminp))
    np.testing.assert_array_equal(np.ravel(r.bc.contp), np.ravel(c.bc.contp))
    np.testing.assert_array_equal(np.ravel(r.bc.presc), np.ravel(c.bc.presc))


def _parse_psi(path):
    """The block parsing of pyCATHY's read_psi."""
    lines = open(path).readlines()
    idx, times = [], []
    for i, ln in enumerate(lines):
        if "TIME" in ln:
            idx.append(i)
            times.append(float(ln.split()[1]))
    idx.append(len(lines))
    blocks = [np.array([float(v) for ln in lines[idx[j] + 1:idx[j + 1]] for v in ln.split()])
              for j in range(len(idx) - 1)]
    return times, blocks


def test_output_files_parse_like_pycathy(tmp_path):
    from pycathy_wrapper_gb300.pycathy import write_mbeconv, write_psi
    rng = np.random.default_rng(0)
    p0, p1 = -rng.uniform(0, 3, 37), -rng.uniform(0, 3, 37)
    write_psi(str(tmp_path / "psi"), [(0, 0.0, p0), (12, 3600.0, p1)])
    times, blocks = _parse_psi(str(tmp_path / "psi"))
    assert times == [0.0, 3600.0]
    np.testing.assert_allclose(blocks[0], p0, rtol=1e-6)
    np.testing.assert_allclose(blocks[1], p1, rtol=1e-6)
    recs = []
    for s in range(1, 4):
        recs.append(dict(nstep=s, iter=3, nitert=7, nback=0, deltat=10.0 * s, time=60.0 * s,
                         store1=1.0 + s, store2=1.0 + s, dstore=-1e-6 * s, cdstor=-2e-6 * s,
                         vin=1e-5, cvin=1e-5 * s, vout=-2e-6, cvout=-2e-6 * s, erras=3e-9,
                         errel=-0.1, cerras=3e-9 * s, caeras=3e-9 * s))
    write_mbeconv(str(tmp_path / "mbeconv"), recs, 1.0)
    a = np.loadtxt(str(tmp_path / "mbeconv"), skiprows=2, usecols=range(19))
    assert a.shape == (3, 19)
    np.testing.assert_array_equal(a[:, 0], [1, 2, 3])
    np.testing.assert_allclose(a[:, 2], [60.0, 120.0, 180.0])
    np.testing.assert_allclose(a[:, 4], 7.0 / 3.0, rtol=1e-3)
    np.testing.assert_allclose(a[:, 13], 1e-5 - 2e-6, rtol=1e-3)


@pytest.mark.gpu
def test_run_ensemble_on_project_folders_matches_api(tmp_path):
    from pycathy_wrapper_gb300.api import Simulation
    from pycathy_wrapper_gb300.inputs import config2_members
    from pycathy_wrapper_gb300.pycathy import run_ensemble, write_project
    cases = config2_members(3, tmax=1800.0, min_cells=6, max_cells=9)
    dirs = []
    for m, c in enumerate(cases):
        d = str(tmp_path / f"cathy_{m + 1}")
        write_project(c, d)
        dirs.append(d)
    res = run_ensemble(dirs, precision=1)
    for c in cases:
        c.parm.precond = 2
    with Simulation(cases, precision=1) as s:
        s.run()
        direct = [s.state(m) for m in range(len(cases))]
    for m, r in enumerate(res):
        assert r["status"] == 1
        np.testing.assert_array_equal(r["pnew"], direct[m][0])
        times, blocks = _parse_psi(os.path.join(dirs[m], "output", "psi"))
        assert times[-1] == pytest.approx(1800.0)
        np.testing.assert_allclose(blocks[-1], r["pnew"], rtol=1e-6, atol=1e-12)
        mb = np.loadtxt(os.path.join(dirs[m], "output", "mbeconv"), skiprows=2, usecols=range(19))
        assert mb[-1, 2] == pytest.approx(1800.0)
