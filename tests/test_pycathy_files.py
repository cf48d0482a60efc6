"""pyCATHY-facing files: project folders written and read back, and the
output files (psi, sw, mbeconv, iter) in the layouts pyCATHY's readers parse
(pyCATHY/importers/cathy_outputs.py:480 read_psi, :418 read_sw,
:607 read_mbeconv) and the reference writes (iter: conver.f:44-45)."""
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


def _parse_sw(path):
    """The block parsing of pyCATHY's read_sw: header lines hold the step and
    the time; the file's first line is the HSPSW marker."""
    lines = open(path).readlines()
    assert lines[0] == "  0   HSPSW\n"
    return _parse_psi(path)


def _parse_iter(path):
    """Fixed-width fields of the reference's iteration lines
    (2I6, 2E10.3, I6, 2E10.2, 2E10.3) and the (NSTEP: ...) step lines."""
    steps, rows = [], []
    for ln in open(path).read().splitlines():
        if "(NSTEP:" in ln:
            w = ln.replace("(", " ").replace(")", " ").split()
            steps.append((int(w[1]), float(w[3]), float(w[5])))
        elif len(ln) == 78 and ln[:6].strip().isdigit():
            cuts = [0, 6, 12, 22, 32, 38, 48, 58, 68, 78]
            f = [ln[a:b] for a, b in zip(cuts[:-1], cuts[1:])]
            rows.append(dict(iter=int(f[0]), niter=int(f[1]), pl2=float(f[2]), pinf=float(f[3]),
                             ikmax=int(f[4]), pnew_ik=float(f[5]), pold_ik=float(f[6]),
                             fl2=float(f[7]), finf=float(f[8])))
    return steps, rows


def test_sw_and_iter_files_from_oracle_records(tmp_path):
    import oracle as O
    from pycathy_wrapper_gb300.inputs import config0
    from pycathy_wrapper_gb300.pycathy import write_iter, write_sw
    case = config0(tmax=3600.0, precond=0)
    o = O.Oracle(case)
    p0 = o.state()[0]
    sw0 = o.vg_nodal(p0)["sw"]
    for _ in range(4):
        o.step()
    p1, t1, _ = o.state()
    sw1 = o.vg_nodal(p1)["sw"]
    write_sw(str(tmp_path / "sw"), [(0, 0.0, sw0), (4, t1, sw1)])
    times, blocks = _parse_sw(str(tmp_path / "sw"))
    assert times == [0.0, pytest.approx(t1, rel=1e-8)]
    np.testing.assert_allclose(blocks[0], sw0, rtol=1e-6)
    np.testing.assert_allclose(blocks[1], sw1, rtol=1e-6)
    its = o.iter_records()
    write_iter(str(tmp_path / "iter"), case.parm, its)
    head = open(str(tmp_path / "iter")).read().splitlines()
    assert head[0] == "     IOPT   (1 PICARD, 2 NEWTON)             =      1"
    assert head[10] == " " + "=" * 77
    steps, rows = _parse_iter(str(tmp_path / "iter"))
    assert len(rows) == len(its)
    assert len(steps) == sum(1 for r in its if r["iter"] == 1)
    for a, b in zip(rows, its):
        assert (a["iter"], a["niter"], a["ikmax"]) == (b["iter"], b["niter"], b["ikmax"])
        for k, rt in (("pl2", 1e-3), ("pinf", 1e-3), ("pnew_ik", 1e-2), ("pold_ik", 1e-2),
                      ("fl2", 1e-3), ("finf", 1e-3)):
            assert a[k] == pytest.approx(b[k], rel=rt, abs=1e-300), k


def test_risul_summary_from_oracle_records(tmp_path):
    """The risul closing summary (cathy_main.f:3880-3950): step statistics
    recomputed from the records, the phase table adding up to the
    nonlinear-scheme total, and the cumulative relative MBE."""
    import re
    import oracle as O
    from pycathy_wrapper_gb300.inputs import config0
    from pycathy_wrapper_gb300.pycathy import write_risul
    case = config0(tmax=3600.0, precond=0)
    o = O.Oracle(case)
    for _ in range(12):
        o.step()
    recs, its = o.step_records(), o.iter_records()
    phases = [0.5, 0.0, 1.25, 0.0, 0.0, 0.0, 3.0, 0.0, 0.25]
    write_risul(str(tmp_path / "risul"), recs, its, phases, 6.0)
    txt = open(str(tmp_path / "risul")).read()
    num = lambda key: float(re.search(re.escape(key) + r"\s*=?\s*(-?[0-9.E+-]+)", txt).group(1))
    assert num("TOTAL NUMBER OF TIME STEPS") == len(recs)
    assert num("TOTAL NUMBER OF NONLINEAR ITERATIONS") == len(its)
    assert num("TOTAL NUMBER OF LINEAR ITERATIONS") == sum(r["niter"] for r in its)
    assert num("TOT CPU FOR NONLINEAR SCHEME") == pytest.approx(5.0)
    assert num("TOT CPU FOR LINEAR SOLVER & RESIDUAL") == pytest.approx(3.0)
    assert num("SMALLEST TIME STEP SIZE") == pytest.approx(min(r["deltat"] for r in recs), rel=1e-3)
    rel = 100.0 * recs[-1]["cerras"] / (recs[-1]["cvin"] + recs[-1]["cvout"])
    assert num("CUMULATIVE (TOTAL) RELATIVE MBE BASED ON CERRAS:") == pytest.approx(rel, rel=1e-4)


def test_mesh_files_match_reference_grid3d(tmp_path):
    """grid3d and xyz from the host mesh builder against the reference's own
    grid3d of the weill example (parsed as pyCATHY's read_grid3d does)."""
    from conftest import GOLDEN, load_golden_case
    from pycathy_wrapper_gb300.pycathy import mesh_gen3d, write_grid3d, write_xyz
    g = np.load(os.path.join(GOLDEN, "weill_grid3d.npz"))
    mesh = mesh_gen3d(load_golden_case("weill"))
    write_grid3d(str(tmp_path / "grid3d"), mesh)
    nnod, n, nt = np.loadtxt(str(tmp_path / "grid3d"), max_rows=1).astype(int)
    assert (nnod, n, nt) == (int(g["nnod"]), g["xyz"].shape[0], g["tetra"].shape[0])
    tet = np.loadtxt(str(tmp_path / "grid3d"), skiprows=1, max_rows=nt).astype(int)
    xyz = np.loadtxt(str(tmp_path / "grid3d"), skiprows=1 + nt)
    np.testing.assert_array_equal(tet, g["tetra"])
    np.testing.assert_allclose(xyz, g["xyz"], rtol=1e-6, atol=1e-6)
    write_xyz(str(tmp_path / "xyz"), mesh)
    a = np.loadtxt(str(tmp_path / "xyz"), skiprows=1)
    assert open(str(tmp_path / "xyz")).readline().split()[:2] == [str(nnod), str(n)]
    np.testing.assert_array_equal(a[:, 0], np.arange(1, n + 1))
    np.testing.assert_allclose(a[:, 1:], g["xyz"], rtol=1e-6, atol=1e-6)


def test_water_table_rules():
    """wtdepth.f's cases on one 3-layer column (nnod = 1, top node first)."""
    from pycathy_wrapper_gb300.pycathy import water_table
    z = np.array([3.0, 2.0, 1.0, 0.0])
    # saturated below 1.5 m: crossing between the nodes at z = 1 (p = 0.5)
    # and z = 2 (p = -0.5), interpolated to z = 1.5
    assert water_table(np.array([-1.5, -0.5, 0.5, 1.5]), z, 1, 3, [1]) == [pytest.approx(1.5)]
    # fully unsaturated: the bottom of the column
    assert water_table(np.array([-4.0, -3.0, -2.0, -1.0]), z, 1, 3, [1]) == [0.0]
    # fully saturated with ponding: surface elevation + surface head
    assert water_table(np.array([0.2, 1.2, 2.2, 3.2]), z, 1, 3, [1]) == [pytest.approx(3.2)]
    # a perched saturated layer above an unsaturated one: the scan from the
    # bottom keeps the lower crossing (z = 0.5 between p = 0.5 and -0.5)
    z5 = np.array([4.0, 3.0, 2.0, 1.0, 0.0])
    p5 = np.array([-0.5, 0.5, -1.0, -0.5, 0.5])
    assert water_table(p5, z5, 1, 4, [1]) == [pytest.approx(0.5)]
    # two columns side by side (nnod = 2): column 2's nodes are 1, 3, 5, 7
    zz = np.repeat(z, 2)
    pp = np.stack([[-1.5, -0.5, 0.5, 1.5], [-4.0, -3.0, -2.0, -1.0]], 1).ravel()
    assert water_table(pp, zz, 2, 3, [1, 2]) == [pytest.approx(1.5), 0.0]


def test_parm_output_controls_round_trip(tmp_path):
    from pycathy_wrapper_gb300.inputs import config0
    from pycathy_wrapper_gb300.project import read_project
    from pycathy_wrapper_gb300.pycathy import write_project
    c = config0(tmax=7200.0)
    c.parm.iprt1, c.parm.timprt, c.parm.nodvp = 3, [1800.0, 3600.0, 7200.0], [5, 17]
    write_project(c, str(tmp_path))
    r = read_project(str(tmp_path))
    assert (r.parm.iprt1, r.parm.timprt, r.parm.nodvp) == (3, [1800.0, 3600.0, 7200.0], [5, 17])


def test_mesh_only_run_writes_grid3d_without_a_gpu(tmp_path):
    """IPRT1 = 3: the mesh files and nothing else (gen3d.f:89-111)."""
    from pycathy_wrapper_gb300.api import build_mesh
    from pycathy_wrapper_gb300.inputs import config0
    from pycathy_wrapper_gb300.pycathy import run_project, write_project
    c = config0(tmax=600.0)
    c.parm.iprt1 = 3
    write_project(c, str(tmp_path))
    res = run_project(str(tmp_path))
    assert res["steps"] == 0
    out = tmp_path / "output"
    assert sorted(os.listdir(out)) == ["grid3d", "xyz"]
    m = build_mesh(c)
    nnod, n, nt = np.loadtxt(str(out / "grid3d"), max_rows=1).astype(int)
    assert (nnod, n, nt) == (m["nnod"], m["n"], m["nt"])


def test_cathy_cli_mesh_only_run(tmp_path):
    """The ``./cathy`` replacement in a project folder (IPRT1 = 3: the mesh
    files, no GPU)."""
    import subprocess
    import sys
    from pycathy_wrapper_gb300.inputs import config0
    from pycathy_wrapper_gb300.pycathy import write_project
    c = config0(tmax=600.0)
    c.parm.iprt1 = 3
    write_project(c, str(tmp_path))
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    env = dict(os.environ, PYTHONPATH=root + os.pathsep + os.environ.get("PYTHONPATH", ""))
    r = subprocess.run([sys.executable, "-m", "pycathy_wrapper_gb300.cathy_cli"],
                       cwd=str(tmp_path), env=env, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    assert "mesh written" in r.stdout
    assert sorted(os.listdir(tmp_path / "output")) == ["grid3d", "xyz"]


def test_parm_lists_continued_on_next_lines(tmp_path):
    """TIMPRT and NODVP are list-directed reads (datin.f:118-119): their
    values may run on over several lines."""
    from pycathy_wrapper_gb300.inputs import config0
    from pycathy_wrapper_gb300.project import read_parm
    from pycathy_wrapper_gb300.pycathy import write_project
    write_project(config0(tmax=7200.0), str(tmp_path))
    path = tmp_path / "input" / "parm"
    ls = open(path).read().splitlines()
    k = next(i for i, ln in enumerate(ls) if "TIMPRT" in ln)
    ls[k] = "4 2 4 600.0 1200.0\tIPRT VTKF NPRT (TIMPRT(I),I=1,NPRT)"
    ls.insert(k + 1, "3600.0")
    ls.insert(k + 2, "7200.0")
    ls[k + 3] = "3 1 2\tNUMVP (NODVP(I),I=1,NUMVP)"
    ls.insert(k + 4, "9")
    open(path, "w").write("\n".join(ls) + "\n")
    p = read_parm(str(path))
    assert p.timprt == [600.0, 1200.0, 3600.0, 7200.0]
    assert p.nodvp == [1, 2, 9]


class _OracleStepper:
    """The oracle behind the calls of drive_outputs (one member)."""

    def __init__(self, case):
        import oracle as O
        self.o, self.tmax = O.Oracle(case), case.parm.tmax

    def _t(self):
        # the time of the last accepted step (the oracle's TIME has already
        # moved on to the next step, as after TIMUPD)
        r = self.o.step_records()
        return r[-1]["time"] if r else 0.0

    def step(self):
        self.o.step()
        return 0 if self._t() >= self.tmax - 1e-9 else 1

    def state(self, m):
        p, _, dt = self.o.state()
        return p, self._t(), dt, 0

    def saturation(self, m):
        return self.o.vg_nodal(self.o.state()[0])["sw"]

    def num_steps(self, m):
        return len(self.o.step_records())


def test_drive_outputs_print_times_and_water_table():
    """Detailed output at TIME = 0 and at the first step reaching each
    TIMPRT, a water-table row per accepted step."""
    from pycathy_wrapper_gb300.api import build_mesh
    from pycathy_wrapper_gb300.inputs import config0
    from pycathy_wrapper_gb300.pycathy import drive_outputs, water_table
    c = config0(tmax=1200.0)
    c.parm.timprt, c.parm.nodvp = [300.0, 1200.0], [1, 7]
    mesh = build_mesh(c)
    mesh["nstr"] = c.dem.nstr
    st = _OracleStepper(c)
    snaps, wt = drive_outputs(st, 1, [c.parm], [mesh])
    recs = st.o.step_records()
    times = [r["time"] for r in recs]
    assert [s[1] for s in snaps[0]] == [0.0, next(t for t in times if t >= 300.0), times[-1]]
    assert snaps[0][-1][1] == pytest.approx(1200.0)
    assert [r[0] for r in wt[0]] == times
    p_end = st.o.state()[0]
    assert wt[0][-1][1] == water_table(p_end, mesh["z"], mesh["nnod"], c.dem.nstr, [1, 7])
    np.testing.assert_array_equal(snaps[0][-1][2], p_end)


class _ScriptedStepper:
    """Two members on a 1-column, 3-layer mesh: member 0 accepts a step of
    100 s per call up to 500 s, member 1 fails after two steps."""

    def __init__(self):
        self.k = [0, 0]
        self.dead = [False, False]

    def step(self):
        for m in (0, 1):
            if self.dead[m] or (m == 0 and self.k[0] == 5):
                continue
            if m == 1 and self.k[1] == 2:
                self.dead[1] = True  # the failed member accepts no more steps
                continue
            self.k[m] += 1
        return sum(1 for m in (0, 1) if not self.dead[m] and not (m == 0 and self.k[0] == 5))

    def state(self, m):
        p = np.array([-1.0, -0.5, 0.5, 1.0]) + 0.01 * self.k[m]
        return p, 100.0 * self.k[m], 100.0, (2 if self.dead[m] else 0)

    def saturation(self, m):
        return np.full(4, 0.5 + 0.01 * self.k[m])

    def num_steps(self, m):
        return self.k[m]


def test_drive_outputs_with_a_failing_member():
    from pycathy_wrapper_gb300.inputs import Parm
    from pycathy_wrapper_gb300.pycathy import drive_outputs
    mesh = dict(z=np.array([3.0, 2.0, 1.0, 0.0]), nnod=1, nstr=3)
    parms = [Parm(timprt=[250.0, 500.0], nodvp=[1]), Parm(timprt=[250.0], nodvp=[1])]
    snaps, wt = drive_outputs(_ScriptedStepper(), 2, parms, [mesh, mesh])
    assert [(k, t) for k, t, _, _ in snaps[0]] == [(0, 0.0), (3, 300.0), (5, 500.0)]
    # the failed member: its start and the last step it accepted
    assert [(k, t) for k, t, _, _ in snaps[1]] == [(0, 0.0), (2, 200.0)]
    assert [t for t, _ in wt[0]] == [100.0, 200.0, 300.0, 400.0, 500.0]
    assert [t for t, _ in wt[1]] == [100.0, 200.0]


@pytest.mark.gpu
def test_saturation_matches_oracle():
    """Sw at the current heads (the sw output's array) against the oracle's
    van Genuchten restatement, FP64 and FP32 paths."""
    import oracle as O
    from pycathy_wrapper_gb300.api import Simulation
    from pycathy_wrapper_gb300.inputs import config0
    for precision in (0, 1):
        case = config0(tmax=3600.0, precond=0 if precision == 0 else 2)
        with Simulation([case], precision=precision) as s:
            for _ in range(5):
                s.step()
            p = s.state(0)[0]
            sw = s.saturation(0)
        ref = O.Oracle(config0(tmax=3600.0, precond=0)).vg_nodal(p)["sw"]
        np.testing.assert_allclose(sw, ref, rtol=1e-12, atol=1e-14)


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
        # the same step-by-step schedule as run_ensemble's output driver
        while s.step() > 0:
            pass
        direct = [s.state(m) for m in range(len(cases))]
        nsteps = [s.num_records(m)[1] for m in range(len(cases))]
    for m, r in enumerate(res):
        assert r["status"] == 1
        np.testing.assert_array_equal(r["pnew"], direct[m][0])
        times, blocks = _parse_psi(os.path.join(dirs[m], "output", "psi"))
        assert times[-1] == pytest.approx(1800.0)
        np.testing.assert_allclose(blocks[-1], r["pnew"], rtol=1e-6, atol=1e-12)
        mb = np.loadtxt(os.path.join(dirs[m], "output", "mbeconv"), skiprows=2, usecols=range(19))
        assert mb[-1, 2] == pytest.approx(1800.0)
        times, sws = _parse_sw(os.path.join(dirs[m], "output", "sw"))
        assert times[-1] == pytest.approx(1800.0)
        assert len(sws[-1]) == len(r["pnew"]) and np.all((sws[-1] > 0.0) & (sws[-1] <= 1.0))
        steps, rows = _parse_iter(os.path.join(dirs[m], "output", "iter"))
        assert rows and steps[-1][2] == pytest.approx(1800.0, rel=1e-4)
        wt = np.loadtxt(os.path.join(dirs[m], "output", "wtdepth"), ndmin=2)
        assert wt.shape[0] == nsteps[m] and wt[-1, 0] == pytest.approx(1800.0)
        assert sorted(os.listdir(os.path.join(dirs[m], "output"))) == [
            "grid3d", "iter", "mbeconv", "psi", "risul", "sw", "wtdepth", "xyz"]


def test_hgsfdet_from_oracle_seepage_records(tmp_path):
    """The seepage-face hydrograph written from a seepage run's step records
    reads back with the reference's layout (one header line, I7 and four
    E17.9 columns) and its volumes are the trapezoids of SFFLW."""
    import oracle as O
    from test_seepage import seepage_case
    from pycathy_wrapper_gb300.pycathy import write_hgsfdet
    o = O.Oracle(seepage_case())
    for _ in range(20):
        assert o.step() == 0
    recs = o.step_records()
    path = str(tmp_path / "hgsfdet")
    write_hgsfdet(path, recs)
    lines = open(path).read().splitlines()
    assert lines[0].startswith("# NSTEP") and lines[0].endswith("NET SEEPFACE FLX")
    assert len(lines) == len(recs) + 1
    assert len(lines[1]) == 7 + 4 * 21
    tab = np.loadtxt(path, skiprows=1)
    prev = np.concatenate([[0.0], [r["sfflw"] for r in recs[:-1]]])
    vol = np.array([(r["sfflw"] + q) * 0.5 * r["deltat"] for r, q in zip(recs, prev)])
    np.testing.assert_array_equal(tab[:, 0], [r["nstep"] for r in recs])
    np.testing.assert_allclose(tab[:, 3], vol, rtol=1e-9, atol=1e-300)
    np.testing.assert_allclose(tab[:, 4], vol / tab[:, 1], rtol=1e-8, atol=1e-300)
    assert (tab[:, 3] < 0).all()
